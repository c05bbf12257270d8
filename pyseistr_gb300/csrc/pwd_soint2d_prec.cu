// Preconditioned 2-D structure-oriented interpolation: the prec = 1
// branches of csoint2d (pyseistr/src/soint2d_cfuns.c:2354-2398, called by
// soint2dc, soint2d.py:92).  The reference solves
//     M P p ~= d   (M the known-sample mask, ps_mask_lop :145-159)
// with ps_solver_prec (:1704-2034, eps = 0) stepped by ps_cgstep (:493-544),
// where P is predict_lop (:1537-1571): the causal integration of a section
// trace by trace along its slopes, tt <- predict_step(tt + x[i2]) (:1422-1449);
// with twoplane, predict2_lop (:1597-1616) chains the integrations along the
// two slope fields.  The result is x = P p.
//
// GPU form: one CTA runs the whole solver of one section (the integration is
// serial over traces, and within a trace the banded solve is serial over
// samples).  The band factors do not change during a call, so a first kernel
// factors every trace once (a thread per trace and plane); the solver
// kernel then streams each trace's taps and LDL' factors into shared memory
// with one bulk copy (cp.async.bulk on an mbarrier, double-buffered so the
// next trace's copy overlaps the current step), applies the filter and its
// adjoint with all threads, and runs the forward and back substitutions on
// one thread per plane.  The CG's vector work and its dot products (FP64
// sums of float products: per thread in float-float, then a fixed block
// tree) use the whole CTA.  Every float operation on a sample is the
// reference's, in its order; only the dot products' summation order
// differs.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <cstdlib>
#include <vector>

#include "pwd_common.cuh"
#include "pwd_gb300.h"
#include "pwd_predict.cuh"

namespace pwd {
namespace {

constexpr int kPrecThreads = 256;
constexpr unsigned long long kStageLimitNs = 50ull * 1000 * 1000;  // one copy: ~1 us
constexpr float kPrecEps = 0.0001f;  // predict_init(n1, n2, 0.0001, nw, 1, false)

struct PrecArgs {
  const float* din;
  const float* mask;
  const float* dip[2];  // pp, qq
  float* out;
  float* fac;    // [plane][trace][blk], the FacLayout of each trace
  float *p, *g, *rr, *gg, *S, *Ss;
  float* vec;    // [plane][3][n1r] trace vectors when they live in global memory
  uint8_t* known;
  int* status;   // set when a bulk copy did not complete in time
  int n1, n2, niter, hasmask, planes;
  long blk;      // floats per trace block (a multiple of 4)
  long cpy;      // floats of a block that a step reads (a multiple of 4)
  int n1r;       // n1 rounded up to a multiple of 4
  int smem_fac;  // factor buffers in shared memory: 0 (read in place), 1 or 2
  int smem_vec;  // trace vectors in shared memory
};

__host__ __device__ inline long round4(long x) { return (x + 3) / 4 * 4; }

// Per-trace factor block (floats, every part 16-byte aligned):
//   taps [NA][n1]        the passfilter taps, unreversed
//   fo   [n1][RS]        row k: o[m][k-m-1] (0 where k-m-1 < 0), the
//                        forward substitution's operands of row k
//   bo   [n1][RS]        row k: o[m][k] (0 beyond the band's end), the back
//                        substitution's operands
//   d    [n1]
// then, in the workspace only, predict_factor's own [NB][n1] + [n1] output.
// A step copies the first part (cpy floats) into shared memory.
__host__ __device__ constexpr int row_stride(int nb) { return nb <= 2 ? 2 : (nb + 3) / 4 * 4; }
struct FacLayout {
  long taps, fo, bo, d, raw, cpy, blk;
};
__host__ __device__ inline FacLayout fac_layout(int order, int n1) {
  const int NA = 2 * order + 1, NB = 2 * order, RS = row_stride(NB);
  FacLayout L;
  L.taps = 0;
  L.fo = round4((long)NA * n1);
  L.bo = L.fo + round4((long)RS * n1);
  L.d = L.bo + round4((long)RS * n1);
  L.cpy = L.d + round4(n1);
  L.raw = L.cpy;
  L.blk = L.raw + round4((long)(NB + 1) * n1);
  return L;
}

// Taps and the reversed filter's LDL' factor (forw = true, the orientation
// predict_lop uses) of every trace of both slope fields, then the factor
// rearranged into the substitutions' row order.
template <int NW>
__global__ void k_prec_factor(const PrecArgs* __restrict__ args, ApCoef c) {
  constexpr int NB = 2 * NW, RS = row_stride(NB);
  const PrecArgs& a = args[blockIdx.y];  // one section per grid row
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= (long)a.planes * a.n2) return;
  const int plane = (int)(t / a.n2), i2 = (int)(t % a.n2), n1 = a.n1;
  const FacLayout L = fac_layout(NW, n1);
  float* base = a.fac + t * a.blk;
  float* raw = base + L.raw;
  PredictFactor F{base + L.taps, nullptr, raw, 1};
  predict_factor<NW>(n1, kPrecEps, kPrecEps, c, a.dip[plane] + (long)i2 * n1, F, 1, true);
  for (int k = 0; k < n1; k++) {
#pragma unroll
    for (int m = 0; m < RS; m++) {
      float vf = 0.f, vb = 0.f;
      if (m < NB) {
        if (k - m - 1 >= 0) vf = raw[(long)m * n1 + (k - m - 1)];
        vb = raw[(long)m * n1 + k];
      }
      base[L.fo + (long)k * RS + m] = vf;
      base[L.bo + (long)k * RS + m] = vb;
    }
    base[L.d + k] = raw[(long)NB * n1 + k];
  }
}

// The per-trace factor of one plane: taps a(j, i) of the reversed filter
// (pwd_define :1075-1082 with adj = forw = true), the substitution rows and
// d.
struct TraceFac {
  const float* taps;
  const float* fo;
  const float* bo;
  const float* d;
  int n1;
  __device__ __forceinline__ float a(int j, int i, int na) const {
    return taps[(long)(na - 1 - j) * n1 + i];
  }
};

// One substitution row: t -= ov[m] * W[m] for m = 0..NB-1 in order, then
// the window of solved values shifts.  Rows whose band is shorter than NB
// carry zero operands against the zero-initialised window, which leaves t
// unchanged (t - 0 * 0 is t, -0 included), so one loop serves every row.
template <int NB>
__device__ __forceinline__ float subst_row(float t, const float (&ov)[NB], float (&W)[NB]) {
#pragma unroll
  for (int m = 0; m < NB; m++) t = __fsub_rn(t, __fmul_rn(ov[m], W[m]));
#pragma unroll
  for (int m = NB - 1; m > 0; m--) W[m] = W[m - 1];
  W[0] = t;
  return t;
}

// ps_banded_solve (:1317-1337) in place on b[plane] for every plane, called
// by all threads: the forward substitution on one thread per plane, then
// b[k] / d[k] by all threads (the back substitution's first operation on
// each row), then the back substitution.  The serial thread takes its rows
// in blocks of kRows: it loads a block's operands and right-hand sides,
// solves the block, then stores it, so that no load waits behind a store
// and only the arithmetic chain of each row is exposed (about 26 cycles a
// row at NB = 4 on the GB300, against 52 with a load and a store per row).
constexpr int kRows = 8;

// Operand access of the substitution thread: generic loads and stores, or,
// when the factor rows and the trace vectors are in shared memory (SH),
// shared-space ones (about a third fewer cycles a row: a generic access
// pays for the address-space check).  The volatile forms keep program
// order, which already loads a block before solving and storing it.
template <bool SH>
struct SubMem {
  const float* base;
  unsigned sbase;
  __device__ __forceinline__ explicit SubMem(const float* p)
      : base(p), sbase(SH ? (unsigned)__cvta_generic_to_shared(p) : 0u) {}
  __device__ __forceinline__ float ld(long k) const {
    if constexpr (SH) {
      float x;
      asm volatile("ld.shared.f32 %0, [%1];" : "=f"(x) : "r"(sbase + (unsigned)k * 4u));
      return x;
    } else {
      return base[k];
    }
  }
  __device__ __forceinline__ float2 ld2(long k) const {
    if constexpr (SH) {
      float2 x;
      asm volatile("ld.shared.v2.f32 {%0, %1}, [%2];" : "=f"(x.x), "=f"(x.y)
                   : "r"(sbase + (unsigned)k * 4u));
      return x;
    } else {
      return *reinterpret_cast<const float2*>(base + k);
    }
  }
  __device__ __forceinline__ float4 ld4(long k) const {
    if constexpr (SH) {
      float4 x;
      asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                   : "=f"(x.x), "=f"(x.y), "=f"(x.z), "=f"(x.w)
                   : "r"(sbase + (unsigned)k * 4u));
      return x;
    } else {
      return *reinterpret_cast<const float4*>(base + k);
    }
  }
  __device__ __forceinline__ void st(long k, float x) const {
    if constexpr (SH) {
      asm volatile("st.shared.f32 [%0], %1;" ::"r"(sbase + (unsigned)k * 4u), "f"(x) : "memory");
    } else {
      const_cast<float*>(base)[k] = x;
    }
  }
};

template <int NB, bool SH>
__device__ __forceinline__ void load_row_m(const SubMem<SH>& m, long k, float (&v)[NB]) {
  if constexpr (NB == 2) {
    const float2 x = m.ld2(k);
    v[0] = x.x;
    v[1] = x.y;
  } else {
#pragma unroll
    for (int q = 0; q < (NB + 3) / 4; q++) {
      const float4 x = m.ld4(k + 4 * q);
      const float xs[4] = {x.x, x.y, x.z, x.w};
#pragma unroll
      for (int e = 0; e < 4; e++)
        if (4 * q + e < NB) v[4 * q + e] = xs[e];
    }
  }
}

template <int NB, bool DOWN, bool SH>
__device__ __forceinline__ void subst_pass(const float* ops_p, float* v_p, int n1) {
  constexpr int RS = row_stride(NB);
  const SubMem<SH> ops(ops_p), v(v_p);
  float W[NB];
#pragma unroll
  for (int m = 0; m < NB; m++) W[m] = 0.f;
  const int nblk = n1 / kRows;
  for (int q = 0; q < nblk; q++) {
    float ov[kRows][NB], t[kRows];
#pragma unroll
    for (int r = 0; r < kRows; r++) {
      const int k = DOWN ? n1 - 1 - (q * kRows + r) : q * kRows + r;
      load_row_m<NB, SH>(ops, (long)k * RS, ov[r]);
      t[r] = v.ld(k);
    }
#pragma unroll
    for (int r = 0; r < kRows; r++) t[r] = subst_row<NB>(t[r], ov[r], W);
#pragma unroll
    for (int r = 0; r < kRows; r++) v.st(DOWN ? n1 - 1 - (q * kRows + r) : q * kRows + r, t[r]);
  }
  for (int j = nblk * kRows; j < n1; j++) {
    const int k = DOWN ? n1 - 1 - j : j;
    float ov[NB];
    load_row_m<NB, SH>(ops, (long)k * RS, ov);
    v.st(k, subst_row<NB>(v.ld(k), ov, W));
  }
}

// sh: the factor rows and the trace vectors are in shared memory.
template <int NB>
__device__ void banded_solve_all(const TraceFac* f, float* const* b, int P, bool sh) {
  const int n1 = f[0].n1;
  const bool solver = (threadIdx.x & 31) == 0 && (int)(threadIdx.x >> 5) < P;
  const int pl = threadIdx.x >> 5;
  if (solver) {
    if (sh)
      subst_pass<NB, false, true>(f[pl].fo, b[pl], n1);
    else
      subst_pass<NB, false, false>(f[pl].fo, b[pl], n1);
  }
  __syncthreads();
  for (int q = 0; q < P; q++)
    for (int k = threadIdx.x; k < n1; k += blockDim.x) b[q][k] = __fdiv_rn(b[q][k], f[q].d[k]);
  __syncthreads();
  if (solver) {
    if (sh)
      subst_pass<NB, true, true>(f[pl].bo, b[pl], n1);
    else
      subst_pass<NB, true, false>(f[pl].bo, b[pl], n1);
  }
}

// pwd_set forward (:1139-1157) into tv: tmp[i] = sum_j a[j][i] tt[i+j-nw]
// for i in [nw, n1-nw) (all threads).
template <int NW>
__device__ __forceinline__ void set_fwd_tmp(const TraceFac& f, const float* tt, float* tv) {
  constexpr int NA = 2 * NW + 1;
  const int n1 = f.n1;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    float s = 0.f;
    if (i >= NW && i < n1 - NW) {
#pragma unroll
      for (int j = 0; j < NA; j++) s = __fadd_rn(s, __fmul_rn(f.a(j, i, NA), tt[i + j - NW]));
    }
    tv[i] = s;
  }
}

// out[i] = sum_j a[j][k] tmp[k] (k = i+j-nw in [nw, n1-nw)), then the eps2
// boundary terms of predict_step (:1437-1442), into rhs (all threads).
template <int NW>
__device__ __forceinline__ void set_fwd_out(const TraceFac& f, const float* tt, const float* tv,
                                            float* rhs) {
  constexpr int NA = 2 * NW + 1;
  const int n1 = f.n1;
  for (int i = threadIdx.x; i < n1; i += blockDim.x) {
    float b = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) {
      const int k = i + j - NW;
      if (k >= NW && k < n1 - NW) b = __fadd_rn(b, __fmul_rn(f.a(j, k, NA), tv[k]));
    }
    if (i == 0) b = __fadd_rn(b, __fmul_rn(kPrecEps, tt[0]));
    if (i == 1) b = __fadd_rn(b, __fmul_rn(kPrecEps, tt[1]));
    if (i == n1 - 2) b = __fadd_rn(b, __fmul_rn(kPrecEps, tt[n1 - 2]));
    if (i == n1 - 1) b = __fadd_rn(b, __fmul_rn(kPrecEps, tt[n1 - 1]));
    rhs[i] = b;
  }
}

// pwd_set adjoint (:1117-1137), first half: tmp[k] = sum over ascending i of
// a[k+nw-i][k] x[i], k in [nw, n1-nw) (all threads).
template <int NW>
__device__ __forceinline__ void set_adj_tmp(const TraceFac& f, const float* x, float* tv) {
  constexpr int NA = 2 * NW + 1;
  const int n1 = f.n1;
  for (int k = threadIdx.x; k < n1; k += blockDim.x) {
    float s = 0.f;
    if (k >= NW && k < n1 - NW) {
#pragma unroll
      for (int j = NA - 1; j >= 0; j--) s = __fadd_rn(s, __fmul_rn(f.a(j, k, NA), x[k + NW - j]));
    }
    tv[k] = s;
  }
}

// Second half, in place on x: x[q] = sum over ascending i in [nw, n1-nw) of
// a[q-i+nw][i] tmp[i], plus the eps2 boundary terms of the solved values
// (each thread reads and writes only its own samples of x).
template <int NW>
__device__ __forceinline__ void set_adj_out(const TraceFac& f, const float* tv, float* x) {
  constexpr int NA = 2 * NW + 1;
  const int n1 = f.n1;
  for (int q = threadIdx.x; q < n1; q += blockDim.x) {
    float o = 0.f;
#pragma unroll
    for (int j = NA - 1; j >= 0; j--) {
      const int i = q + NW - j;
      if (i >= NW && i < n1 - NW) o = __fadd_rn(o, __fmul_rn(f.a(j, i, NA), tv[i]));
    }
    const float t = x[q];
    if (q == 0) o = __fadd_rn(o, __fmul_rn(kPrecEps, t));
    if (q == 1) o = __fadd_rn(o, __fmul_rn(kPrecEps, t));
    if (q == n1 - 2) o = __fadd_rn(o, __fmul_rn(kPrecEps, t));
    if (q == n1 - 1) o = __fadd_rn(o, __fmul_rn(kPrecEps, t));
    x[q] = o;
  }
}

__device__ __forceinline__ void proxy_fence_async() {
  asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
}

// What a scan reads and writes around the integration.
enum ScanIo {
  kAdjMaskRR,  // adjoint: input M rr, output g
  kFwdMaskGG,  // forward: input g, output gg = M x + 0 (0 rr)
  kFwdOut      // forward: input p, output out = x
};

// The solver's CTA state: shared-memory trace vectors and factor buffers,
// and the bulk-copy pipeline over a scan's traces.
struct Cta {
  PrecArgs a;
  float* tt[2];   // the integrated trace of each plane
  float* rhs[2];  // right-hand sides / filter output
  float* tv[2];   // pwd_set intermediate
  float* fb[2];   // factor buffers (planes side by side)
  unsigned long long* bar;
  unsigned phase[2];
  int nbuf;
  int failed_buf;  // the buffer whose copy timed out, -1 if none

  __device__ const float* global_fac(int plane, int i2) const {
    return a.fac + ((long)plane * a.n2 + i2) * a.blk;
  }
  __device__ void issue(int i2, int buf) {
    if (threadIdx.x != 0) return;
    proxy_fence_async();
    const unsigned bytes = (unsigned)(a.cpy * 4);
    mbar_arrive_expect_tx(&bar[buf], bytes * a.planes);
    for (int pl = 0; pl < a.planes; pl++)
      bulk_copy_g2s(fb[buf] + (long)pl * a.cpy, global_fac(pl, i2), bytes, &bar[buf]);
  }
  // Factor of plane `pl` for the step on trace i2 held in buffer `buf`.
  __device__ TraceFac fac(int pl, int i2, int buf) const {
    const float* base = nbuf ? fb[buf] + (long)pl * a.cpy : global_fac(pl, i2);
    return TraceFac{base, nullptr, nullptr, nullptr, a.n1};
  }
  // Waits for buffer buf; false (in every thread) when the copy timed out,
  // the buffer's phase then left pending for a last bounded wait.
  __device__ bool wait(int buf) {
    const bool ok = mbar_wait_bounded(&bar[buf], phase[buf], kStageLimitNs);
    if (__syncthreads_or(!ok)) {
      failed_buf = buf;
      return false;
    }
    phase[buf] ^= 1u;
    return true;
  }
};

template <int NW>
__device__ __forceinline__ TraceFac with_factor(TraceFac f) {
  const FacLayout L = fac_layout(NW, f.n1);
  const float* base = f.taps;
  f.taps = base + L.taps;
  f.fo = base + L.fo;
  f.bo = base + L.bo;
  f.d = base + L.d;
  return f;
}

// One scan: the integration (forward) or its adjoint over the traces of
// the section, for one plane or the chain of two.  Returns false when a
// bulk copy timed out.
template <int NW>
__device__ bool scan(Cta& C, bool adj, ScanIo io, const float* in, float* outv) {
  constexpr int NB = 2 * NW;
  const PrecArgs& a = C.a;
  const int n1 = a.n1, n2 = a.n2, P = a.planes;
  for (int pl = 0; pl < P; pl++)
    for (int i = threadIdx.x; i < n1; i += blockDim.x) C.tt[pl][i] = 0.f;
  __syncthreads();
  for (int k = 0; k < n2; k++) {
    const int i2 = adj ? n2 - 1 - k : k;
    const int buf = C.nbuf == 2 ? (k & 1) : 0;
    if (C.nbuf) {
      if (C.nbuf == 1 || k == 0) C.issue(i2, buf);
      if (!C.wait(buf)) return false;
      if (C.nbuf == 2 && k + 1 < n2) C.issue(adj ? i2 - 1 : i2 + 1, buf ^ 1);
    }
    TraceFac f[2];
    for (int pl = 0; pl < P; pl++) f[pl] = with_factor<NW>(C.fac(pl, i2, buf));
    const long off = (long)i2 * n1;
    if (!adj) {
      // tt1 += x; (two planes: tmp = tt1, tt2 += tmp); y = 0 + tt_last
      for (int i = threadIdx.x; i < n1; i += blockDim.x) {
        float v = __fadd_rn(C.tt[0][i], in[off + i]);
        C.tt[0][i] = v;
        if (P == 2) {
          v = __fadd_rn(C.tt[1][i], __fadd_rn(0.f, v));
          C.tt[1][i] = v;
        }
        float y = __fadd_rn(0.f, v);
        if (io == kFwdMaskGG) {
          y = a.known[off + i] ? __fadd_rn(0.f, y) : 0.f;
          y = __fadd_rn(y, __fmul_rn(0.f, __fmul_rn(0.f, a.rr[off + i])));
        }
        outv[off + i] = y;
      }
      if (k + 1 < n2) {  // the step after the last trace is not used
        __syncthreads();
        for (int pl = 0; pl < P; pl++) set_fwd_tmp<NW>(f[pl], C.tt[pl], C.tv[pl]);
        __syncthreads();
        for (int pl = 0; pl < P; pl++) set_fwd_out<NW>(f[pl], C.tt[pl], C.tv[pl], C.rhs[pl]);
        __syncthreads();
        banded_solve_all<NB>(f, C.rhs, P, C.nbuf > 0 && a.smem_vec);
        // the solved trace is the next step's tt
        for (int pl = 0; pl < P; pl++) {
          float* t = C.tt[pl];
          C.tt[pl] = C.rhs[pl];
          C.rhs[pl] = t;
        }
      }
    } else {
      // tt = predict_step'(tt) per plane, then tt2 += y; tmp = 0 + tt2;
      // tt1 += tmp; x = 0 + tt1 (one plane: tt += y; x = 0 + tt)
      banded_solve_all<NB>(f, C.tt, P, C.nbuf > 0 && a.smem_vec);
      __syncthreads();
      for (int pl = 0; pl < P; pl++) set_adj_tmp<NW>(f[pl], C.tt[pl], C.tv[pl]);
      __syncthreads();
      for (int pl = 0; pl < P; pl++) set_adj_out<NW>(f[pl], C.tv[pl], C.tt[pl]);
      __syncthreads();
      for (int i = threadIdx.x; i < n1; i += blockDim.x) {
        float y = in[off + i];
        if (io == kAdjMaskRR) y = a.known[off + i] ? __fadd_rn(0.f, y) : 0.f;
        float v;
        if (P == 2) {
          const float t2 = __fadd_rn(C.tt[1][i], y);
          C.tt[1][i] = t2;
          v = __fadd_rn(C.tt[0][i], __fadd_rn(0.f, t2));
        } else {
          v = __fadd_rn(C.tt[0][i], y);
        }
        C.tt[0][i] = v;
        outv[off + i] = __fadd_rn(0.f, v);
      }
    }
    __syncthreads();
  }
  return true;
}

// ps_solver_prec + ps_cgstep for one section per CTA.
template <int NW>
__global__ void __launch_bounds__(kPrecThreads) k_soint2d_prec(const PrecArgs* __restrict__ args) {
  const PrecArgs a = args[blockIdx.x];
  extern __shared__ __align__(16) float sm[];
  __shared__ __align__(8) unsigned long long bars[2];
  __shared__ double s_scal[4];  // alfa, beta (as floats), skip, stop
  Cta C;
  C.a = a;
  C.bar = bars;
  C.phase[0] = C.phase[1] = 0u;
  C.nbuf = a.smem_fac;
  C.failed_buf = -1;
  const int n1 = a.n1, P = a.planes;
  const long n = (long)n1 * a.n2;
  {
    float* q = sm;
    for (int b = 0; b < a.smem_fac; b++) {
      C.fb[b] = q;
      q += (long)P * a.cpy;
    }
    float* vbase = a.smem_vec ? q : a.vec;
    for (int pl = 0; pl < 2; pl++) {
      const int pp = pl < P ? pl : 0;
      C.tt[pl] = vbase + (long)(3 * pp + 0) * a.n1r;
      C.rhs[pl] = vbase + (long)(3 * pp + 1) * a.n1r;
      C.tv[pl] = vbase + (long)(3 * pp + 2) * a.n1r;
    }
  }
  if (threadIdx.x == 0 && a.smem_fac) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_fence_init();
  }
  // rr = -dat (dat = din), p = 0; known from the mask or the data
  for (long i = threadIdx.x; i < n; i += blockDim.x) {
    const float di = a.din[i];
    a.rr[i] = -di;
    a.p[i] = 0.f;
    a.S[i] = 0.f;
    a.Ss[i] = 0.f;
    a.known[i] = a.hasmask == 1 ? (a.mask[i] != 0.f) : (di != 0.f);
  }
  __syncthreads();
  if (a.niter == 0) {
    for (long i = threadIdx.x; i < n; i += blockDim.x) a.out[i] = a.din[i];
    return;
  }
  const double TOL = (double)1.e-12f, EPS = (double)1.e-12f;
  double dprr0 = 1., dpgm0 = 1.;
  bool ok = true;
  for (int iter = 0; iter < a.niter && ok; iter++) {
    // g = P' M rr; gg = M P g (+ eps g[nprec:] with eps = 0)
    ok = scan<NW>(C, true, kAdjMaskRR, a.rr, a.g);
    if (!ok) break;
    ok = scan<NW>(C, false, kFwdMaskGG, a.g, a.gg);
    if (!ok) break;
    // snrm2 (float squares, summed here in FP64) and ps_cgstep's dsdot
    ffacc c0, c1, c2, c3, c4;
    double nr = 0., ng = 0.;
    for (long i = threadIdx.x; i < n; i += blockDim.x) {
      const float r = a.rr[i], gv = a.g[i], q = a.gg[i], s = a.Ss[i];
      nr += (double)__fmul_rn(r, r);
      ng += (double)__fmul_rn(gv, gv);
      c0.add_prod(q, q);
      c1.add_prod(s, s);
      c2.add_prod(q, s);
      c3.add_prod(q, r);
      c4.add_prod(s, r);
    }
    dvec<7> acc = {{nr, ng, c0.value(), c1.value(), c2.value(), c3.value(), c4.value()}};
    dvec<7> tot = block_sum<7>(acc);
    if (threadIdx.x == 0) {
      double dprr, dpgm;
      if (iter == 0) {
        dprr0 = (double)(float)tot.v[0];
        dpgm0 = (double)(float)tot.v[1];
        dprr = 1.;
        dpgm = 1.;
      } else {
        dprr = (double)(float)tot.v[0] / dprr0;
        dpgm = (double)(float)tot.v[1] / dpgm0;
      }
      double alfa = 0., beta = 0.;
      bool skip = false;
      const bool stop = dprr < TOL || dpgm < TOL;
      if (!stop) {
        if (iter == 0) {  // the first ps_cgstep call restarts (S = Ss = 0)
          alfa = tot.v[2];
          if (alfa <= 0.) skip = true;
          else alfa = -tot.v[5] / alfa;
        } else {
          const double gdg = tot.v[2], sds = tot.v[3], gds = tot.v[4];
          if (gdg == 0. || sds == 0.) {
            skip = true;
          } else {
            double determ = 1.0 - (gds / gdg) * (gds / sds);
            if (determ > EPS) determ *= gdg * sds;
            else determ = gdg * sds * EPS;
            const double gdr = -tot.v[5], sdr = -tot.v[6];
            alfa = (sds * gdr - gds * sdr) / determ;
            beta = (-gds * gdr + gdg * sdr) / determ;
          }
        }
      }
      s_scal[0] = (double)__double2float_rn(alfa);
      s_scal[1] = (double)__double2float_rn(beta);
      s_scal[2] = skip ? 1. : 0.;
      s_scal[3] = stop ? 1. : 0.;
    }
    __syncthreads();
    if (s_scal[3] != 0.) break;
    if (s_scal[2] == 0.) {
      const float al = (float)s_scal[0], be = (float)s_scal[1];
      for (long i = threadIdx.x; i < n; i += blockDim.x) {
        const float s = __fadd_rn(__fmul_rn(a.S[i], be), __fmul_rn(al, a.g[i]));
        a.S[i] = s;
        a.p[i] = __fadd_rn(a.p[i], s);
        const float s2 = __fadd_rn(__fmul_rn(a.Ss[i], be), __fmul_rn(al, a.gg[i]));
        a.Ss[i] = s2;
        a.rr[i] = __fadd_rn(a.rr[i], s2);
      }
    }
    __syncthreads();
  }
  // x = P p
  if (ok) ok = scan<NW>(C, false, kFwdOut, a.p, a.out);
  if (!ok) {
    if (threadIdx.x == 0) atomicExch(a.status, 1);
    // let the copy in flight land before the CTA exits
    if (C.failed_buf >= 0)
      mbar_wait_bounded(&bars[C.failed_buf], C.phase[C.failed_buf], kStageLimitNs);
  }
}

struct PrecLayout {
  long blk, cpy, fac_floats;
  int n1r, nbuf, smem_vec;
  size_t smem_bytes, total;
};

size_t smem_limit() {
  int dev = 0, v = 0;
  if (cudaGetDevice(&dev) != cudaSuccess ||
      cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev) != cudaSuccess)
    return 48 * 1024;
  return (size_t)v;
}

// An environment knob that can only lower a default (tests run the
// fallbacks of small sections with it).
int env_cap(const char* name, int dflt) {
  const char* v = std::getenv(name);
  if (!v || !*v) return dflt;
  return std::min(dflt, std::max(0, std::atoi(v)));
}

// Factor buffers and trace vectors in shared memory when they fit: two
// factor buffers, else one, else the factors read in place from the
// workspace; the trace vectors likewise.  PWD_PREC_BUFFERS (0, 1) and
// PWD_PREC_VEC (0) lower the choice; the results are the same bits.
PrecLayout prec_layout(int n1, int n2, int order, int planes, size_t smem_cap) {
  PrecLayout L{};
  const FacLayout F = fac_layout(order, n1);
  L.blk = F.blk;
  L.cpy = F.cpy;
  L.n1r = (int)round4(n1);
  L.fac_floats = L.blk * planes * n2;
  const size_t reserve = 4096;  // static shared memory (block sums, barriers)
  const size_t cap = smem_cap > reserve ? smem_cap - reserve : 0;
  const size_t vec = (size_t)3 * planes * L.n1r * 4, fb = (size_t)planes * L.cpy * 4;
  L.smem_vec = vec <= cap ? env_cap("PWD_PREC_VEC", 1) : 0;
  const size_t left = L.smem_vec ? cap - vec : cap;
  L.nbuf = env_cap("PWD_PREC_BUFFERS", 2 * fb <= left ? 2 : (fb <= left ? 1 : 0));
  L.smem_bytes = (L.smem_vec ? vec : 0) + L.nbuf * fb;
  Carver cv(nullptr);
  const long n = (long)n1 * n2;
  cv.take<float>(L.fac_floats);
  for (int k = 0; k < 6; k++) cv.take<float>(n);
  cv.take<float>((size_t)3 * planes * L.n1r);
  cv.take<uint8_t>(n);
  cv.take<int>(1);
  L.total = cv.size();
  return L;
}

// The sections of a call (one for pwd_soint2d_prec) and the shared-memory
// plan of the longest traces, which serves every section.
struct PrecBatch {
  std::vector<pwd_section> secs;
  int planes, order;
  PrecLayout big;  // the plan of the largest n1
};

// Workspace: the per-section argument array, the failure flag, then every
// section's factor store, vectors and scratch.  ws = nullptr only sizes it.
size_t carve_prec(void* ws, const PrecBatch& B, std::vector<PrecArgs>* args, PrecArgs** dargs,
                  int** status) {
  Carver cv(ws);
  const int nsec = (int)B.secs.size();
  PrecArgs* da = cv.take<PrecArgs>(nsec);
  int* st = cv.take<int>(1);
  if (dargs) *dargs = da;
  if (status) *status = st;
  for (int k = 0; k < nsec; k++) {
    const pwd_section& sc = B.secs[k];
    const PrecLayout L = prec_layout(sc.n1, sc.n2, B.order, B.planes, smem_limit());
    const long n = (long)sc.n1 * sc.n2;
    PrecArgs a{};
    a.fac = cv.take<float>(L.fac_floats);
    a.p = cv.take<float>(n);
    a.g = cv.take<float>(n);
    a.rr = cv.take<float>(n);
    a.gg = cv.take<float>(n);
    a.S = cv.take<float>(n);
    a.Ss = cv.take<float>(n);
    a.vec = cv.take<float>((size_t)3 * B.planes * L.n1r);
    a.known = cv.take<uint8_t>(n);
    a.status = st;
    a.n1 = sc.n1;
    a.n2 = sc.n2;
    a.planes = B.planes;
    a.blk = L.blk;
    a.cpy = L.cpy;
    a.n1r = L.n1r;
    a.smem_fac = B.big.nbuf;
    a.smem_vec = B.big.smem_vec;
    if (args) args->push_back(a);
  }
  return cv.size();
}

int prec_batch_make(const pwd_section* sections, int nsec, int order, int twoplane,
                    PrecBatch& B) {
  // (the factor launch takes a grid row per section: at most 65535)
  if (!sections || nsec < 1 || nsec > 65535 || order < 1) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  B.secs.assign(sections, sections + nsec);
  B.planes = twoplane ? 2 : 1;
  B.order = order;
  int n1max = 0, n2max = 0;
  for (const pwd_section& s : B.secs) {
    if (s.n1 < 2 || s.n2 < 1 || s.n3 != 1 || s.offset < 0 || s.out_offset < 0 ||
        (long)s.n1 * s.n2 >= (1L << 31))
      return PWD_EINVAL;
    if (s.n1 > n1max) n1max = s.n1, n2max = s.n2;
  }
  B.big = prec_layout(n1max, n2max, order, B.planes, smem_limit());
  return PWD_OK;
}

template <int NW>
int prec_run(const PrecArgs* dargs, int nsec, int maxtr, const PrecLayout& L,
             cudaStream_t st) {
  const ApCoef c = make_apcoef(NW);
  PWD_KERNEL(PWD_FAM_SOINT, st,
             (k_prec_factor<NW><<<dim3((unsigned)((maxtr + 127) / 128), (unsigned)nsec), 128, 0,
                                  st>>>(dargs, c)));
  int rc = cuda_status(cudaGetLastError());
  if (rc != PWD_OK) return rc;
  rc = cuda_status(cudaFuncSetAttribute(k_soint2d_prec<NW>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize,
                                        (int)L.smem_bytes));
  if (rc != PWD_OK) return rc;
  PWD_KERNEL(PWD_FAM_SOINT, st,
             (k_soint2d_prec<NW><<<(unsigned)nsec, kPrecThreads, L.smem_bytes, st>>>(dargs)));
  return cuda_status(cudaGetLastError());
}

// Enqueues the batch, then reads back the failure flag (synchronising st).
int prec_enqueue(const PrecBatch& B, const float* data, const float* mask, const float* dip1,
                 const float* dip2, float* out, int niter, int hasmask, void* ws, size_t wsb,
                 cudaStream_t st) {
  const size_t need = carve_prec(nullptr, B, nullptr, nullptr, nullptr);
  if (!ws || wsb < need || ((uintptr_t)ws & 255)) return PWD_EWORKSPACE;
  std::vector<PrecArgs> args;
  PrecArgs* dargs = nullptr;
  int* status = nullptr;
  carve_prec(ws, B, &args, &dargs, &status);
  int maxtr = 0;
  for (size_t k = 0; k < args.size(); k++) {
    const pwd_section& s = B.secs[k];
    PrecArgs& a = args[k];
    a.din = data + s.offset;
    a.mask = mask ? mask + s.offset : nullptr;
    a.dip[0] = dip1 + s.out_offset;
    a.dip[1] = (B.planes == 2 ? dip2 : dip1) + s.out_offset;
    a.out = out + s.offset;
    a.niter = niter;
    a.hasmask = hasmask;
    maxtr = std::max(maxtr, a.planes * a.n2);
  }
  int rc = cuda_status(cudaMemcpyAsync(dargs, args.data(), sizeof(PrecArgs) * args.size(),
                                       cudaMemcpyHostToDevice, st));
  if (rc == PWD_OK) rc = cuda_status(cudaMemsetAsync(status, 0, sizeof(int), st));
  if (rc != PWD_OK) return rc;
  const int nsec = (int)args.size();
  switch (B.order) {
    case 1: rc = prec_run<1>(dargs, nsec, maxtr, B.big, st); break;
    case 2: rc = prec_run<2>(dargs, nsec, maxtr, B.big, st); break;
    case 3: rc = prec_run<3>(dargs, nsec, maxtr, B.big, st); break;
    default: rc = prec_run<4>(dargs, nsec, maxtr, B.big, st); break;
  }
  if (rc != PWD_OK) return rc;
  // a bulk copy that timed out leaves a result incomplete: fail loudly (the
  // synchronisation also keeps `args` alive until its copy has run)
  int flag = 0;
  rc = cuda_status(cudaMemcpyAsync(&flag, status, sizeof(int), cudaMemcpyDeviceToHost, st));
  if (rc == PWD_OK) rc = cuda_status(cudaStreamSynchronize(st));
  if (rc != PWD_OK) return rc;
  return flag ? PWD_ECUDA : PWD_OK;
}

}  // namespace
}  // namespace pwd

extern "C" size_t pwd_soint2d_prec_workspace_size(int n1, int n2, int order, int twoplane) {
  pwd_section sec{0, 0, n1, n2, 1};
  pwd::PrecBatch B;
  if (pwd::prec_batch_make(&sec, 1, order, twoplane, B) != PWD_OK) return 0;
  return pwd::carve_prec(nullptr, B, nullptr, nullptr, nullptr);
}

extern "C" int pwd_soint2d_prec(const float* din, const float* mask, const float* dip1,
                                const float* dip2, float* out, int n1, int n2, int order,
                                int niter, int hasmask, int twoplane, void* workspace,
                                size_t workspace_bytes, pwd_stream_t stream) {
  if (!din || !dip1 || !out || niter < 0) return PWD_EINVAL;
  if (hasmask == 1 && !mask) return PWD_EINVAL;
  if (twoplane && !dip2) return PWD_EINVAL;
  pwd_section sec{0, 0, n1, n2, 1};
  pwd::PrecBatch B;
  const int rc = pwd::prec_batch_make(&sec, 1, order, twoplane, B);
  if (rc != PWD_OK) return rc;
  return pwd::prec_enqueue(B, din, mask, dip1, dip2, out, niter, hasmask, workspace,
                           workspace_bytes, (cudaStream_t)stream);
}

extern "C" size_t pwd_soint2d_prec_batch_workspace_size(const pwd_section* sections, int nsec,
                                                        int order, int twoplane) {
  pwd::PrecBatch B;
  if (pwd::prec_batch_make(sections, nsec, order, twoplane, B) != PWD_OK) return 0;
  return pwd::carve_prec(nullptr, B, nullptr, nullptr, nullptr);
}

extern "C" int pwd_soint2d_prec_batch(const float* data, const float* mask, const float* dip1,
                                      const float* dip2, float* out,
                                      const pwd_section* sections, int nsec, int order,
                                      int niter, int hasmask, int twoplane, void* workspace,
                                      size_t workspace_bytes, pwd_stream_t stream) {
  if (!data || !dip1 || !out || niter < 0) return PWD_EINVAL;
  if (hasmask == 1 && !mask) return PWD_EINVAL;
  if (twoplane && !dip2) return PWD_EINVAL;
  pwd::PrecBatch B;
  const int rc = pwd::prec_batch_make(sections, nsec, order, twoplane, B);
  if (rc != PWD_OK) return rc;
  return pwd::prec_enqueue(B, data, mask, dip1, dip2, out, niter, hasmask, workspace,
                           workspace_bytes, (cudaStream_t)stream);
}
