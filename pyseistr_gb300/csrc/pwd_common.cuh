// Shared device code of the GB300 plane-wave-destruction (PWD) library.
//
// Arithmetic contract of the plain FP32 path: every float operation of the
// reference (pyseistr/src/*_cfuns.c) is reproduced in the same order with
// the same rounding.  The library is compiled with -fmad=false so that no
// multiply-add is contracted (the reference is FMA-free x86-64 SSE code);
// FMAs appear only where written explicitly (__fmaf_rn), i.e. inside the
// error-free transformations below.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/pwd_gb300.h"

#ifndef PWD_MAX_ORDER
#define PWD_MAX_ORDER 4
#endif
#define PWD_MAX_NF (2 * PWD_MAX_ORDER)
#define PWD_MAX_NA (2 * PWD_MAX_ORDER + 1)

namespace pwd {

// ---------------------------------------------------------------------------
// All-pass filter constants (apfilt_init, dip_cfuns.c:835-855): b[k] as a
// double and as a float-float pair.
// ---------------------------------------------------------------------------
struct ApCoef {
  int nw, nf;
  double b[PWD_MAX_NA];
  float bh[PWD_MAX_NA], bl[PWD_MAX_NA];
};

inline ApCoef make_apcoef(int nw) {
  ApCoef c;
  c.nw = nw;
  c.nf = 2 * nw;
  for (int k = 0; k <= c.nf; k++) {
    double bk = 1.0;
    for (int j = 0; j < c.nf; j++) {
      if (j < c.nf - k)
        bk *= (k + j + 1.0) / (2 * (2 * j + 1) * (j + 1));
      else
        bk *= 1.0 / (2 * (2 * j + 1));
    }
    c.b[k] = bk;
    c.bh[k] = (float)bk;
    c.bl[k] = (float)(bk - (double)c.bh[k]);
  }
  return c;
}

// ---------------------------------------------------------------------------
// Float-float arithmetic (Dekker 1971, Knuth TAOCP vol. 2 "TwoSum").
// ---------------------------------------------------------------------------
struct ff {
  float h, l;
};
__device__ __forceinline__ ff ff_two_sum(float a, float b) {
  float s = __fadd_rn(a, b);
  float bb = __fsub_rn(s, a);
  float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return {s, e};
}
__device__ __forceinline__ ff ff_mul_f(ff a, float b) {
  float p = __fmul_rn(a.h, b);
  float pl = __fmaf_rn(a.h, b, -p);
  float e = __fmaf_rn(a.l, b, pl);
  float s = __fadd_rn(p, e);
  return {s, __fsub_rn(e, __fsub_rn(s, p))};
}
__device__ __forceinline__ ff ff_mul(ff a, ff b) {
  float p = __fmul_rn(a.h, b.h);
  float pl = __fmaf_rn(a.h, b.h, -p);
  float e = __fmaf_rn(a.h, b.l, __fmaf_rn(a.l, b.h, pl));
  float s = __fadd_rn(p, e);
  return {s, __fsub_rn(e, __fsub_rn(s, p))};
}
__device__ __forceinline__ ff ff_add(ff a, ff b) {
  ff s = ff_two_sum(a.h, b.h);
  float e = __fadd_rn(s.l, __fadd_rn(a.l, b.l));
  return ff_two_sum(s.h, e);
}

// True when rounding the float-float value (h,l) to float could differ from
// rounding the exact value, given an absolute error bound tol of the pair:
// i.e. (h+l) lies within tol of the midpoint between h and its neighbour on
// the side of l.  Also true for zero, tiny or non-finite h (handled exactly).
__device__ __forceinline__ bool ff_near_tie(float h, float l, float tol) {
  uint32_t bits = __float_as_uint(h) & 0x7fffffffu;
  if (bits < (30u << 23) || bits >= 0x7f800000u) return true;
  float ulp = __uint_as_float((bits & 0x7f800000u) - (23u << 23));
  bool toward_zero = (l != 0.f) && ((l < 0.f) != (h < 0.f));
  float half = ((bits & 0x007fffffu) == 0u && toward_zero) ? 0.25f * ulp : 0.5f * ulp;
  return __fsub_rn(half, fabsf(l)) <= tol;
}

// Factor j of tap k: (nf-j-p) or ((p+j)+1), in float as the C expression.
__device__ __forceinline__ float ap_factor(int nf, int k, int j, float p) {
  if (j < nf - k) return __fsub_rn((float)(nf - j), p);
  return __fadd_rn(__fadd_rn(p, (float)j), 1.0f);
}

// passfilter tap k (dip_cfuns.c:863-881): double product rounded to float,
// evaluated in float-float and redone in FP64 only near a rounding tie.
__device__ __forceinline__ float pass_tap(const ApCoef& c, int k, float p) {
  ff a = {c.bh[k], c.bl[k]};
  for (int j = 0; j < c.nf; j++) a = ff_mul_f(a, ap_factor(c.nf, k, j, p));
  if (!ff_near_tie(a.h, a.l, fabsf(a.h) * 0x1p-40f)) return a.h;
  double ak = c.b[k];
  for (int j = 0; j < c.nf; j++) ak = __dmul_rn(ak, (double)ap_factor(c.nf, k, j, p));
  return __double2float_rn(ak);
}

// aderfilter tap k (dip_cfuns.c:883-910), same scheme.
__device__ __forceinline__ float ader_tap(const ApCoef& c, int k, float p) {
  ff s = {0.f, 0.f};
  float sabs = 0.f;
  for (int i = 0; i < c.nf; i++) {
    ff ai = {-1.f, 0.f};
    for (int j = 0; j < c.nf; j++) {
      if (j != i)
        ai = ff_mul_f(ai, ap_factor(c.nf, k, j, p));
      else if (j < c.nf - k)
        ai = {-ai.h, -ai.l};
    }
    s = ff_add(s, ai);
    sabs = __fadd_rn(sabs, fabsf(ai.h));
  }
  ff r = ff_mul(s, ff{c.bh[k], c.bl[k]});
  if (!ff_near_tie(r.h, r.l, sabs * fabsf(c.bh[k]) * 0x1p-38f)) return r.h;
  double ak = 0.0;
  for (int i = 0; i < c.nf; i++) {
    double ai = -1.0;
    for (int j = 0; j < c.nf; j++) {
      if (j != i)
        ai = __dmul_rn(ai, (double)ap_factor(c.nf, k, j, p));
      else if (j < c.nf - k)
        ai = __dmul_rn(ai, -1.0);
    }
    ak = __dadd_rn(ak, ai);
  }
  return __double2float_rn(__dmul_rn(ak, c.b[k]));
}

// Per-thread accumulator of a dot product of floats in float-float: each
// product is split exactly (FMA), sums are error-free (TwoSum) up to the
// low word, about 2^-45 relative over a thread's few terms; converted to
// double for the block and tile sums.  This keeps the double accuracy of
// the reference's dsdot (dip_cfuns.c:122) without per-sample FP64 work.
struct ffacc {
  float h = 0.f, l = 0.f;
  __device__ __forceinline__ void add_prod(float a, float b) {
    float p = __fmul_rn(a, b);
    float pe = __fmaf_rn(a, b, -p);
    ff s = ff_two_sum(h, p);
    h = s.h;
    l = __fadd_rn(l, __fadd_rn(s.l, pe));
  }
  __device__ __forceinline__ double value() const { return (double)h + (double)l; }
};

// (float) (x * s) for a double scale s, as the reference's float*double
// products (dip_cfuns.c:807, :822): float-float product, FP64 near ties.
__device__ __forceinline__ float mul_by_double(float x, float sh, float sl, double s) {
  if (x == 0.f) return __fmul_rn(x, sh);
  float ph = __fmul_rn(x, sh);
  float pl = __fmaf_rn(x, sh, -ph);
  pl = __fmaf_rn(x, sl, pl);
  float h = __fadd_rn(ph, pl);
  float l = __fsub_rn(pl, __fsub_rn(h, ph));
  if (!ff_near_tie(h, l, fabsf(h) * 0x1p-40f)) return h;
  return __double2float_rn(__dmul_rn((double)x, s));
}

// num = r / hypot(d, 1), den = d / hypot(d, 1), each rounded as the
// reference's double computation 1.0/hypot(d,1.0) then float*double
// (dip_cfuns.c:804-808): float-float sqrt and reciprocal, FP64 near ties.
__device__ __forceinline__ void invhypot_scale(float r, float d, float& num, float& den) {
  if (d == 0.f) {  // 1/hypot(0,1) = 1 exactly
    num = __fmul_rn(r, 1.f);
    den = __fmul_rn(d, 1.f);
    return;
  }
  float dh = __fmul_rn(d, d), dl = __fmaf_rn(d, d, -dh);
  ff q = ff_two_sum(1.0f, dh);
  q = ff_two_sum(q.h, __fadd_rn(q.l, dl));
  bool exact = isfinite(q.h);
  float sh = __fsqrt_rn(q.h);
  float t = __fadd_rn(__fmaf_rn(-sh, sh, q.h), q.l);
  float sl = __fdiv_rn(t, __fmul_rn(2.f, sh));
  float ih = __fdiv_rn(1.f, sh);
  float ph = __fmul_rn(sh, ih), pl = __fmaf_rn(sh, ih, -ph);
  float e = __fsub_rn(__fsub_rn(1.f, ph), pl);
  e = __fsub_rn(e, __fmul_rn(sl, ih));
  float il = __fmul_rn(ih, e);
  float out[2];
  const float in[2] = {r, d};
#pragma unroll
  for (int k = 0; k < 2; k++) {
    float x = in[k];
    if (x == 0.f) {
      out[k] = __fmul_rn(x, ih);
      continue;
    }
    float nh = __fmul_rn(x, ih);
    float nl = __fmaf_rn(x, ih, -nh);
    nl = __fmaf_rn(x, il, nl);
    float h = __fadd_rn(nh, nl);
    float l = __fsub_rn(nl, __fsub_rn(h, nh));
    out[k] = h;
    if (ff_near_tie(h, l, fabsf(h) * 0x1p-38f)) exact = false;
  }
  if (exact) {
    num = out[0];
    den = out[1];
    return;
  }
  double nrm = 1.0 / hypot((double)d, 1.0);
  num = __double2float_rn(__dmul_rn((double)r, nrm));
  den = __double2float_rn(__dmul_rn((double)d, nrm));
}

template <int NW>
__device__ __forceinline__ void passfilter(const ApCoef& c, float p, float* a) {
#pragma unroll
  for (int k = 0; k <= 2 * NW; k++) a[k] = pass_tap(c, k, p);
}
// aderfilter, all taps at once: the factors (nf-j-p) and ((p+j)+1) are made
// once, each term prod_{j != i} f_j comes from prefix and suffix products
// (float-float, about 2^-46 relative; the order of the products does not
// matter at that accuracy), and a tap falls back to the exact FP64 replica
// (ader_tap) only near a rounding tie.
template <int NW>
__device__ __forceinline__ void aderfilter(const ApCoef& c, float p, float* a) {
  constexpr int NF = 2 * NW;
  float fa[NF], fb[NF];
#pragma unroll
  for (int j = 0; j < NF; j++) {
    fa[j] = __fsub_rn((float)(NF - j), p);
    fb[j] = __fadd_rn(__fadd_rn(p, (float)j), 1.0f);
  }
#pragma unroll
  for (int k = 0; k <= NF; k++) {
    float f[NF];
#pragma unroll
    for (int j = 0; j < NF; j++) f[j] = j < NF - k ? fa[j] : fb[j];
    ff pre[NF], suf[NF];
    pre[0] = {1.f, 0.f};
#pragma unroll
    for (int i = 1; i < NF; i++) pre[i] = ff_mul_f(pre[i - 1], f[i - 1]);
    suf[NF - 1] = {1.f, 0.f};
#pragma unroll
    for (int i = NF - 2; i >= 0; i--) suf[i] = ff_mul_f(suf[i + 1], f[i + 1]);
    ff sum = {0.f, 0.f};
    float sabs = 0.f;
#pragma unroll
    for (int i = 0; i < NF; i++) {
      ff t = ff_mul(pre[i], suf[i]);
      // ai = -1 * prod_{j != i} f_j, and * -1 once more when i < nf-k
      if (!(i < NF - k)) t = {-t.h, -t.l};
      sum = ff_add(sum, t);
      sabs = __fadd_rn(sabs, fabsf(t.h));
    }
    ff r = ff_mul(sum, ff{c.bh[k], c.bl[k]});
    a[k] = ff_near_tie(r.h, r.l, sabs * fabsf(c.bh[k]) * 0x1p-38f) ? ader_tap(c, k, p) : r.h;
  }
}

// ---------------------------------------------------------------------------
// Mixed-mode filter taps: the same products evaluated directly in FP32
// (relative error a few units of 2^-24 instead of the reference's rounding
// of a double product).  b[k] enters as its float-float pair.
// ---------------------------------------------------------------------------
template <int NW>
__device__ __forceinline__ void passfilter_f32(const ApCoef& c, float p, float* a) {
  constexpr int NF = 2 * NW;
#pragma unroll
  for (int k = 0; k <= NF; k++) {
    float t = 1.f;
#pragma unroll
    for (int j = 0; j < NF; j++)
      t = __fmul_rn(t, j < NF - k ? __fsub_rn((float)(NF - j), p) : __fadd_rn(p, (float)(j + 1)));
    a[k] = __fmaf_rn(c.bl[k], t, __fmul_rn(c.bh[k], t));
  }
}

template <int NW>
__device__ __forceinline__ void aderfilter_f32(const ApCoef& c, float p, float* a) {
  constexpr int NF = 2 * NW;
  float fa[NF], fb[NF];
#pragma unroll
  for (int j = 0; j < NF; j++) {
    fa[j] = __fsub_rn((float)(NF - j), p);
    fb[j] = __fadd_rn(p, (float)(j + 1));
  }
#pragma unroll
  for (int k = 0; k <= NF; k++) {
    float f[NF], pre[NF], suf[NF];
#pragma unroll
    for (int j = 0; j < NF; j++) f[j] = j < NF - k ? fa[j] : fb[j];
    pre[0] = 1.f;
#pragma unroll
    for (int i = 1; i < NF; i++) pre[i] = __fmul_rn(pre[i - 1], f[i - 1]);
    suf[NF - 1] = 1.f;
#pragma unroll
    for (int i = NF - 2; i >= 0; i--) suf[i] = __fmul_rn(suf[i + 1], f[i + 1]);
    // sum_i s_i prod_{j != i} f_j with s_i = +1 where the factor falls with
    // p (i < nf-k) and -1 where it rises, as the reference's sign rule
    float sum = 0.f;
#pragma unroll
    for (int i = 0; i < NF; i++) {
      const float t = __fmul_rn(pre[i], suf[i]);
      sum = i < NF - k ? __fadd_rn(sum, t) : __fsub_rn(sum, t);
    }
    a[k] = __fmaf_rn(c.bl[k], sum, __fmul_rn(c.bh[k], sum));
  }
}

// ---------------------------------------------------------------------------
// Deterministic reductions: per-block partials, summed in a fixed order by
// the last block to finish (no floating-point atomics).
// ---------------------------------------------------------------------------
constexpr int kRedBlock = 256;
constexpr int kRedGridMax = 1184;  // 8 x 148: a fixed, size-independent cap

inline int red_grid(long n) {
  long g = (n + kRedBlock - 1) / kRedBlock;
  if (g > kRedGridMax) g = kRedGridMax;
  if (g < 1) g = 1;
  return (int)g;
}

template <int K>
struct dvec {
  double v[K];
};

template <int K>
__device__ __forceinline__ dvec<K> block_sum(dvec<K> x) {
  __shared__ double sh[K][32];
#pragma unroll
  for (int k = 0; k < K; k++) {
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x.v[k] += __shfl_down_sync(0xffffffffu, x.v[k], o);
  }
  int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  __syncthreads();
  if (lane == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) sh[k][w] = x.v[k];
  }
  __syncthreads();
  int nw = (blockDim.x + 31) >> 5;
  if (w == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) {
      double t = lane < nw ? sh[k][lane] : 0.0;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) t += __shfl_down_sync(0xffffffffu, t, o);
      x.v[k] = t;
    }
  }
  return x;  // valid in thread 0
}

// Publishes this block's partial sums; returns true (in every thread of the
// block) for the last block, which then holds the grid totals in tot.
template <int K>
__device__ __forceinline__ bool grid_sum_last(dvec<K> x, double* partials, unsigned* counter,
                                              dvec<K>& tot) {
  __shared__ bool s_last;
  dvec<K> b = block_sum<K>(x);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) partials[(size_t)k * gridDim.x + blockIdx.x] = b.v[k];
    __threadfence();
    unsigned t = atomicAdd(counter, 1u);
    s_last = (t == gridDim.x - 1);
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  dvec<K> y;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double t = 0.0;
    for (int i = threadIdx.x; i < (int)gridDim.x; i += blockDim.x)
      t += __ldcg(partials + (size_t)k * gridDim.x + i);
    y.v[k] = t;
  }
  tot = block_sum<K>(y);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// ---------------------------------------------------------------------------
// 4-byte asynchronous global-to-shared copies (cp.async): a thread stages
// its own operands a few iterations ahead without holding registers.
// ---------------------------------------------------------------------------
__device__ __forceinline__ void cp_async4(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(d), "l"(src) : "memory");
}
// 8-byte form: both addresses 8-byte aligned
__device__ __forceinline__ void cp_async8(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(d), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() {
  asm volatile("cp.async.commit_group;\n" ::: "memory");
}
template <int N>
__device__ __forceinline__ void cp_async_wait() {
  asm volatile("cp.async.wait_group %0;\n" ::"n"(N) : "memory");
}

// ---------------------------------------------------------------------------
// Bulk copies by the tensor memory accelerator (cp.async.bulk, global to
// shared, completion counted in bytes on an mbarrier).  Addresses and sizes
// are multiples of 16 bytes.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned smem_u32(const void* p) {
  return (unsigned)__cvta_generic_to_shared(p);
}
__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;\n" ::"r"(smem_u32(bar)), "r"(count)
               : "memory");
}
// makes an initialised mbarrier visible to the asynchronous (TMA) proxy
__device__ __forceinline__ void mbar_fence_init() {
  asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
}
__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(smem_u32(bar)),
               "r"(bytes)
               : "memory");
}
__device__ __forceinline__ void bulk_copy_g2s(void* dst, const void* src, unsigned bytes,
                                              unsigned long long* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::
          "r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
  unsigned ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n"
      " selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
// Waits for phase `parity` of the barrier, giving up after `limit_ns`
// nanoseconds of the global timer; true when the phase completed.
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
  const unsigned long long t0 = global_ns();
  while (!mbar_try_wait(bar, parity))
    if (global_ns() - t0 > limit_ns) return false;
  return true;
}

// ---------------------------------------------------------------------------
// Packed FP32 pairs (add / mul / fma .rn.f32x2): two independent IEEE
// operations per instruction, each rounded as its scalar form.  A packed
// multiply whose result feeds a packed add can be contracted into a packed
// FMA by the compiler in spite of the .rn qualifiers and -fmad=false
// (measured: a float-float dot product accumulated on packed pairs came out
// as the FMA-accumulated sum), so these are used only where no product
// feeds an addition directly; the scalar __fmul_rn / __fadd_rn are never
// contracted.
// ---------------------------------------------------------------------------
__device__ __forceinline__ unsigned long long f2_bits(float2 a) {
  return ((unsigned long long)__float_as_uint(a.y) << 32) | __float_as_uint(a.x);
}
__device__ __forceinline__ float2 f2_from(unsigned long long d) {
  return make_float2(__uint_as_float((unsigned)d), __uint_as_float((unsigned)(d >> 32)));
}
__device__ __forceinline__ float2 add2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("add.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 mul2_rn(float2 a, float2 b) {
  unsigned long long d;
  asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)));
  return f2_from(d);
}
__device__ __forceinline__ float2 fma2_rn(float2 a, float2 b, float2 c) {
  unsigned long long d;
  asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(d) : "l"(f2_bits(a)), "l"(f2_bits(b)), "l"(f2_bits(c)));
  return f2_from(d);
}
// ---------------------------------------------------------------------------
// Workspace carving (256-byte aligned slices of the caller's buffer).
// ---------------------------------------------------------------------------
struct Carver {
  char* base;
  size_t off = 0;
  explicit Carver(void* b) : base((char*)b) {}
  template <class T>
  T* take(size_t count) {
    off = (off + 255) & ~(size_t)255;
    T* p = base ? (T*)(base + off) : nullptr;
    off += count * sizeof(T);
    return p;
  }
  size_t size() const { return (off + 255) & ~(size_t)255; }
};

inline int cuda_status(cudaError_t e) { return e == cudaSuccess ? PWD_OK : PWD_ECUDA; }

// Launch accounting (pwd_capi.cu): every kernel launch goes through
// PWD_KERNEL so that it is counted and, while profiling, timed.
void prof_begin(int fam, cudaStream_t st);
void prof_end(int fam, cudaStream_t st);

}  // namespace pwd

#define PWD_KERNEL(fam, st, ...)   \
  do {                             \
    pwd::prof_begin((fam), (st));  \
    __VA_ARGS__;                   \
    pwd::prof_end((fam), (st));    \
  } while (0)

#define PWD_LAUNCH_CHECK()                            \
  do {                                                \
    cudaError_t e_ = cudaGetLastError();              \
    if (e_ != cudaSuccess) return PWD_ECUDA;          \
  } while (0)
