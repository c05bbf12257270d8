// Median and space-varying median of sprayed panels, exact order
// statistics.
//
// Restates mf_init/boundary/mf and svmf_init/svmf of
// pyseistr/src/sof_cfuns.c:1170-1431 (identical in sof3d_cfuns.c) for the
// only use the filters make of them: the median along the spray axis of one
// trace's panel u[np][n1], with edge replication, of which only the centre
// row c = (np-1)/2 is output.  sf_quantile (:1137-1163) returns the exact
// order statistic q of the window; so do the selection forms here (for
// equal values such as -0.0 and +0.0 they may return the other zero, which
// compares equal):
//   - windows of up to 32 values: a sorting network per thread over the
//     window held in registers (Batcher's odd-even merge sort of 8, 16 or 32
//     elements, the window padded with +inf), then the q-th element;
//   - longer windows: one warp per output sample, the window spread over
//     the lanes, each value's rank counted against all others through warp
//     shuffles; the lane whose value has rank q (values below <= q <
//     values not above) gives it.
// Neither keeps the window in local memory; windows of up to kMaxWin rows
// are accepted.
#pragma once

#include "pwd_common.cuh"

namespace pwd {
namespace {  // internal linkage: included by several translation units

// Longest window (rows of the edge-replicated panel) the filters accept.
constexpr int kMaxWin = 1 << 16;
// Windows up to this length use the per-thread networks.
constexpr int kNetWin = 32;

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

__device__ __forceinline__ void cex(float& a, float& b) {
  const float lo = fminf(a, b), hi = fmaxf(a, b);
  a = lo;
  b = hi;
}

// Batcher's odd-even merge sort of v[0..N) (N a power of two), unrolled.
template <int N>
__device__ __forceinline__ void oddeven_sort(float (&v)[N]) {
#pragma unroll
  for (int p = 1; p < N; p <<= 1)
#pragma unroll
    for (int k = p; k >= 1; k >>= 1)
#pragma unroll
      for (int j = k % p; j + k < N; j += 2 * k)
#pragma unroll
        for (int i = 0; i < k; i++)
          if (i + j + k < N && (i + j) / (2 * p) == (i + j + k) / (2 * p)) cex(v[i + j], v[i + j + k]);
}

// q-th smallest of the window rows start .. start+n-1 (clamped to
// [0, np)) of a panel column col (rows `stride` apart), n <= N.
template <int N>
__device__ __forceinline__ float select_net(const float* col, long stride, int start, int np, int n,
                                            int q) {
  float v[N];
#pragma unroll
  for (int k = 0; k < N; k++)
    v[k] = k < n ? col[(long)clampi(start + k, 0, np - 1) * stride] : __int_as_float(0x7f800000);
  oddeven_sort<N>(v);
  float r = v[0];
#pragma unroll
  for (int k = 1; k < N; k++)
    if (k == q) r = v[k];
  return r;
}

__device__ __forceinline__ float select_thread(const float* col, long stride, int start, int np,
                                               int n, int q) {
  if (n <= 8) return select_net<8>(col, stride, start, np, n, q);
  if (n <= 16) return select_net<16>(col, stride, start, np, n, q);
  return select_net<32>(col, stride, start, np, n, q);
}

// Warp form (any n): every lane of the warp calls it for the same window;
// returns the q-th smallest in every lane.
__device__ __forceinline__ float select_warp(const float* col, long stride, int start, int np, int n,
                                             int q) {
  const int lane = threadIdx.x & 31;
  const int nc = (n + 31) / 32;
  float found = 0.f;
  int have = 0;
  for (int c = 0; c < nc; c++) {
    const int kc = c * 32 + lane;
    const float x = kc < n ? col[(long)clampi(start + kc, 0, np - 1) * stride] : 0.f;
    int lt = 0, le = 0;
    for (int d = 0; d < nc; d++) {
      const int kd = d * 32 + lane;
      const float y = kd < n ? col[(long)clampi(start + kd, 0, np - 1) * stride] : 0.f;
      const int m = min(32, n - d * 32);
      for (int l = 0; l < m; l++) {
        const float z = __shfl_sync(0xffffffffu, y, l);
        lt += z < x;
        le += z <= x;
      }
    }
    if (kc < n && lt <= q && q < le && !have) {
      found = x;
      have = 1;
    }
  }
  // the lowest lane holding the order statistic broadcasts it
  const unsigned who = __ballot_sync(0xffffffffu, have);
  return __shfl_sync(0xffffffffu, found, __ffs(who) - 1);
}

// mf (axis 2, ifbound=1), centre row: window of nmf rows starting at row
// c - m of the edge-replicated panel, m = (nmf-1)/2.  WARP: one warp per
// output sample (windows longer than kNetWin), else one thread.
template <bool WARP>
__global__ void k_median_centre(const float* __restrict__ u, float* __restrict__ out, int n1,
                                int np, long ntr, int nmf) {
  const long t = (blockIdx.x * (long)blockDim.x + threadIdx.x) / (WARP ? 32 : 1);
  if (t >= ntr * n1) return;
  const long tr = t / n1;
  const int i1 = (int)(t % n1);
  const float* col = u + tr * np * (long)n1 + i1;
  const int m = (nmf - 1) / 2, c = (np - 1) / 2;
  const float r = WARP ? select_warp(col, n1, c - m, np, nmf, m)
                       : select_thread(col, n1, c - m, np, nmf, m);
  if (!WARP || (threadIdx.x & 31) == 0) out[tr * n1 + i1] = r;
}

// svmf first pass: median with window nmf+2 of every row (needed for the
// mean absolute value that picks the adaptive windows).
template <bool WARP>
__global__ void k_svmf_pass1(const float* __restrict__ u, float* __restrict__ v2, int n1, int np,
                             long ntr, int nmf) {
  const long t = (blockIdx.x * (long)blockDim.x + threadIdx.x) / (WARP ? 32 : 1);
  if (t >= ntr * np * (long)n1) return;
  const long tr = t / ((long)np * n1);
  const int row = (int)((t / n1) % np);
  const int i1 = (int)(t % n1);
  const float* col = u + tr * np * (long)n1 + i1;
  const int nf = nmf + 2, m = (nf - 1) / 2, m2 = (nmf - 1) / 2;
  const float r = WARP ? select_warp(col, n1, row - m2, np, nf, m)
                       : select_thread(col, n1, row - m2, np, nf, m);
  if (!WARP || (threadIdx.x & 31) == 0) v2[t] = r;
}

// svmf: mean |first-pass median| of each panel, float sum in the
// reference's order (row-major over the panel).
__global__ void k_svmf_avg(const float* __restrict__ v2, float* __restrict__ avg, int n1, int np,
                           long ntr) {
  long tr = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (tr >= ntr) return;
  const float* p = v2 + tr * np * (long)n1;
  float sum = 0.f;
  long m = (long)np * n1;
  for (long i = 0; i < m; i++) sum = __fadd_rn(sum, fabsf(p[i]));
  avg[tr] = __fdiv_rn(sum, (float)(n1 * np));
}

// svmf second pass, centre row, window length from |u| against the mean.
template <bool WARP>
__global__ void k_svmf_pass2(const float* __restrict__ u, const float* __restrict__ avg,
                             float* __restrict__ out, int n1, int np, long ntr, int nmf) {
  const long t = (blockIdx.x * (long)blockDim.x + threadIdx.x) / (WARP ? 32 : 1);
  if (t >= ntr * n1) return;
  const long tr = t / n1;
  const int i1 = (int)(t % n1);
  const float* col = u + tr * np * (long)n1 + i1;
  const int c = (np - 1) / 2;
  const float av = avg[tr];
  const float a = fabsf(col[(long)c * n1]);
  int wl;
  if (a < av)
    wl = (a < __fdiv_rn(av, 2.f)) ? nmf + 2 : nmf;
  else
    wl = (a > __fmul_rn(av, 2.f)) ? nmf - 4 : nmf - 2;
  const int mm2 = (wl - 1) / 2;
  const float r = WARP ? select_warp(col, n1, c - mm2, np, wl, mm2)
                       : select_thread(col, n1, c - mm2, np, wl, mm2);
  if (!WARP || (threadIdx.x & 31) == 0) out[tr * n1 + i1] = r;
}

// Raster-order plain mean of every panel (csomean3d :1523-1537).
__global__ void k_panel_mean(const float* __restrict__ u, float* __restrict__ out, int n1, int np,
                             long ntr) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntr * n1) return;
  long tr = t / n1;
  int i1 = (int)(t % n1);
  const float* panel = u + tr * np * (long)n1 + i1;
  float s = 0.f;
  for (int j = 0; j < np; j++) s = __fadd_rn(s, panel[(long)j * n1]);
  out[t] = __fdiv_rn(s, (float)np);
}

// Launch the median filter of option `option` on panels u[ntr][np][n1].
inline int launch_panel_median(const float* u, float* out, float* v2, float* avg, int n1, int np,
                               long ntr, int nmf, int option, cudaStream_t st) {
  const long nout = ntr * n1;
  const int b = 128;
  // the longest window of the option decides between thread and warp forms
  const bool warp = (option == 1 ? nmf : nmf + 2) > kNetWin;
  const long per = warp ? 32 : 1;
  if (option == 1) {
    if (warp)
      PWD_KERNEL(PWD_FAM_FILTER, st, k_median_centre<true><<<(unsigned)((nout * per + b - 1) / b), b, 0, st>>>(u, out, n1, np, ntr, nmf));
    else
      PWD_KERNEL(PWD_FAM_FILTER, st, k_median_centre<false><<<(unsigned)((nout + b - 1) / b), b, 0, st>>>(u, out, n1, np, ntr, nmf));
  } else {
    const long nv = ntr * np * (long)n1;
    if (warp)
      PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass1<true><<<(unsigned)((nv * per + b - 1) / b), b, 0, st>>>(u, v2, n1, np, ntr, nmf));
    else
      PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass1<false><<<(unsigned)((nv + b - 1) / b), b, 0, st>>>(u, v2, n1, np, ntr, nmf));
    PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_avg<<<(unsigned)((ntr + b - 1) / b), b, 0, st>>>(v2, avg, n1, np, ntr));
    if (warp)
      PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass2<true><<<(unsigned)((nout * per + b - 1) / b), b, 0, st>>>(u, avg, out, n1, np, ntr, nmf));
    else
      PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass2<false><<<(unsigned)((nout + b - 1) / b), b, 0, st>>>(u, avg, out, n1, np, ntr, nmf));
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

// Window lengths the median filters accept.
inline bool median_args_ok(int nmf, int option) {
  if (nmf < 1) return false;
  if (option == 1) return nmf <= kMaxWin;
  return nmf >= 5 && nmf + 2 <= kMaxWin;
}

}  // namespace
}  // namespace pwd
