// Median and space-varying median of sprayed panels, exact order
// statistics.
//
// Restates mf_init/boundary/mf and svmf_init/svmf of
// pyseistr/src/sof_cfuns.c:1170-1431 (identical in sof3d_cfuns.c) for the
// only use the filters make of them: the median along the spray axis of one
// trace's panel u[np][n1], with edge replication, of which only the centre
// row c = (np-1)/2 is output.  sf_quantile (:1137-1163) returns the exact
// order statistic; it is computed here by rank counting, which gives the
// same value (for equal values such as -0.0 and +0.0 it may give the other
// zero, which compares equal).
#pragma once

#include "pwd_common.cuh"

namespace pwd {
namespace {  // internal linkage: included by several translation units

constexpr int kMaxWin = 96;

// q-th smallest of v[0..n)
__device__ __forceinline__ float select_rank(const float* v, int n, int q) {
  for (int c = 0; c < n; c++) {
    float x = v[c];
    int lt = 0, le = 0;
    for (int k = 0; k < n; k++) {
      lt += v[k] < x;
      le += v[k] <= x;
    }
    if (lt <= q && q < le) return x;
  }
  return v[q];
}

__device__ __forceinline__ int clampi(int x, int lo, int hi) { return x < lo ? lo : (x > hi ? hi : x); }

// mf (axis 2, ifbound=1), centre row: window of nmf rows starting at row
// c - m of the edge-replicated panel, m = (nmf-1)/2.
__global__ void k_median_centre(const float* __restrict__ u, float* __restrict__ out, int n1,
                                int np, long ntr, int nmf) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntr * n1) return;
  long tr = t / n1;
  int i1 = (int)(t % n1);
  const float* panel = u + tr * np * (long)n1 + i1;
  const int m = (nmf - 1) / 2, c = (np - 1) / 2;
  float v[kMaxWin];
  for (int k = 0; k < nmf; k++) v[k] = panel[(long)clampi(c + k - m, 0, np - 1) * n1];
  out[tr * n1 + i1] = select_rank(v, nmf, m);
}

// svmf first pass: median with window nmf+2 of every row (needed for the
// mean absolute value that picks the adaptive windows).
__global__ void k_svmf_pass1(const float* __restrict__ u, float* __restrict__ v2, int n1, int np,
                             long ntr, int nmf) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntr * np * (long)n1) return;
  long tr = t / ((long)np * n1);
  int row = (int)((t / n1) % np);
  int i1 = (int)(t % n1);
  const float* panel = u + tr * np * (long)n1 + i1;
  const int nf = nmf + 2, m = (nf - 1) / 2, m2 = (nmf - 1) / 2;
  float v[kMaxWin];
  for (int k = 0; k < nf; k++) v[k] = panel[(long)clampi(row + k - m2, 0, np - 1) * n1];
  v2[t] = select_rank(v, nf, m);
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
__global__ void k_svmf_pass2(const float* __restrict__ u, const float* __restrict__ avg,
                             float* __restrict__ out, int n1, int np, long ntr, int nmf) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= ntr * n1) return;
  long tr = t / n1;
  int i1 = (int)(t % n1);
  const float* panel = u + tr * np * (long)n1 + i1;
  const int c = (np - 1) / 2;
  const float av = avg[tr];
  const float a = fabsf(panel[(long)c * n1]);
  int wl;
  if (a < av)
    wl = (a < __fdiv_rn(av, 2.f)) ? nmf + 2 : nmf;
  else
    wl = (a > __fmul_rn(av, 2.f)) ? nmf - 4 : nmf - 2;
  const int mm2 = (wl - 1) / 2;
  float v[kMaxWin];
  for (int k = 0; k < wl; k++) v[k] = panel[(long)clampi(c + k - mm2, 0, np - 1) * n1];
  out[tr * n1 + i1] = select_rank(v, wl, mm2);
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
  if (option == 1) {
    PWD_KERNEL(PWD_FAM_FILTER, st, k_median_centre<<<(unsigned)((nout + b - 1) / b), b, 0, st>>>(u, out, n1, np, ntr, nmf));
  } else {
    const long nv = ntr * np * (long)n1;
    PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass1<<<(unsigned)((nv + b - 1) / b), b, 0, st>>>(u, v2, n1, np, ntr, nmf));
    PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_avg<<<(unsigned)((ntr + b - 1) / b), b, 0, st>>>(v2, avg, n1, np, ntr));
    PWD_KERNEL(PWD_FAM_FILTER, st, k_svmf_pass2<<<(unsigned)((nout + b - 1) / b), b, 0, st>>>(u, avg, out, n1, np, ntr, nmf));
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
