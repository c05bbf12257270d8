// Sparse-data interpolation (csint2d, pyseistr/src/soint2d_cfuns.c:2421-2523,
// called by sint2dc, sint.py:61, and csint3d, soint3d_cfuns.c:2510-2612,
// called by sint3dc, sint.py:97): the shaping-regularised conjugate
// gradients of ps_conjgrad (:888-1012, prec = NULL, given initial model)
// whose operator is the known-sample mask (ps_mask_lop :145-157) and whose
// shaping is the normalised plane-wave smoothing S of csomean2d (pwsmooth_*,
// the spray-weighted mean; in 3-D inline then crossline, below).
//
// The driver below is host code shared by the GPU entry (pwd_sint.cu, whose
// Ops launch the kernels) and by the CPU test harness (whose Ops run the
// same per-sample functions in loops and the oracle's smoothing), so the
// CPU tests check the driver's operation sequence and scalar arithmetic.
// The per-sample functions are the kernels' bodies.
//
// The reference's FP32 CG amplifies any rounding difference by a few times
// per iteration, so every float operation is the reference's, in its order:
// the adjoint smoothing adds its terms into gp one by one as the reference's
// spray adjoint does (not S' gx formed apart and then added), the mask
// products are `0 + x` where the reference zeroes and adds, and the
// scalars alpha, beta and the step are FP64 from FP64 dot products, rounded
// to float where the reference passes them as float.
#pragma once

#include <float.h>
#include <math.h>
#include <stddef.h>

#ifdef __CUDACC__
#define PWD_SINT_HD __host__ __device__ __forceinline__
#else
#define PWD_SINT_HD inline
#endif

namespace pwd {
namespace sint {

struct Vecs {
  const float* din;
  const float* mask;
  float* x;  // the output array: the data, then the interpolated model's image
  float *p, *r, *sp, *gp, *sx, *gx, *sr, *gr;
};

// r = -dat and p = dat before x = S p overwrites x (x holds dat here).
PWD_SINT_HD void init_sample(const Vecs& v, long i) {
  const float d = v.din[i];
  v.r[i] = -d;
  v.p[i] = d;
  v.x[i] = d;
}
// r += M x
PWD_SINT_HD void residual_sample(const Vecs& v, long i) {
  if (v.mask[i] != 0.f) v.r[i] = v.r[i] + v.x[i];
}
// gp = eps p; gx = -eps x; gx += M' r
PWD_SINT_HD void grad_sample(const Vecs& v, long i, float eps) {
  v.gp[i] = eps * v.p[i];
  float g = -eps * v.x[i];
  if (v.mask[i] != 0.f) g = g + v.r[i];
  v.gx[i] = g;
}
// gr = M gx (zeroed, then added where known)
PWD_SINT_HD void mask_sample(const Vecs& v, long i) {
  v.gr[i] = v.mask[i] != 0.f ? 0.f + v.gx[i] : 0.f;
}
// first iteration: s = g
PWD_SINT_HD void first_sample(const Vecs& v, long i) {
  v.sp[i] = v.gp[i];
  v.sx[i] = v.gx[i];
  v.sr[i] = v.gr[i];
}
// later iterations: s = g + a s (saxpy into g, then the two swap)
PWD_SINT_HD void conj_sample(const Vecs& v, long i, float a) {
  v.sp[i] = v.gp[i] + a * v.sp[i];
  v.sx[i] = v.gx[i] + a * v.sx[i];
  v.sr[i] = v.gr[i] + a * v.sr[i];
}
// p += a sp; x += a sx; r += a sr
PWD_SINT_HD void step_sample(const Vecs& v, long i, float a) {
  v.p[i] = v.p[i] + a * v.sp[i];
  v.x[i] = v.x[i] + a * v.sx[i];
  v.r[i] = v.r[i] + a * v.sr[i];
}

// The lambda of csint2d: sqrt(known / n) with `known` summed as the
// reference sums it, adding 1.0f per known sample (exact to 2^24, where
// float addition of 1 stops changing the sum).
inline float lambda_of(unsigned long long known, long n) {
  const float k = known >= 16777216ull ? 16777216.f : (float)known;
  return sqrtf(k / (float)n);
}

// 3-D smoothing of csint3d (pwsmooth3_lop, soint3d_cfuns.c:2157-2300): the
// 2-D smoothing along the inline slope on every (n1, n2) slice, then along
// the crossline slope on every (n1, n3) section of the cube transposed from
// [n3][n2][n1] (index i1 + n1 (i2 + n2 i3)) to [n2][n3][n1] (index
// i1 + n1 (i3 + n3 i2)); the adjoint in reverse, adding into the model.
// Element e of the transposed cube from the cube:
PWD_SINT_HD void to_crossline_sample(const float* c, float* t, int n1, int n2, int n3, long e) {
  const long i1 = e % n1, r = e / n1, i3 = r % n3, i2 = r / n3;
  t[e] = c[i1 + n1 * (i2 + (long)n2 * i3)];
}
// Element e of the cube from the transposed cube; `sum` is the forward's
// final `smooth += xtmp` into a zeroed array (0 + v).
PWD_SINT_HD void from_crossline_sample(const float* t, float* c, int n1, int n2, int n3, long e,
                                       bool sum) {
  const long i1 = e % n1, r = e / n1, i2 = r % n2, i3 = r / n2;
  const float v = t[i1 + n1 * (i3 + (long)n3 * i2)];
  c[e] = sum ? 0.f + v : v;
}

// The sequence of pwsmooth3_lop on primitives P: inline(mode, in, out) and
// crossline(mode, in, out) apply the 2-D smoothing on the cube's slices or
// the transposed cube's sections (mode 0: out = S in; 1: out += S' in; 2:
// out = S' in), to_cross(c, t) and from_cross(t, c, sum) transpose.
template <class P>
int smooth3_forward(P& pr, float* trace, float* smooth, float* itmp, float* itmp2, float* xtmp) {
  int rc;
  if ((rc = pr.inline_(0, trace, itmp))) return rc;
  if ((rc = pr.to_cross(itmp, itmp2))) return rc;
  if ((rc = pr.crossline(0, itmp2, xtmp))) return rc;
  return pr.from_cross(xtmp, smooth, true);
}
template <class P>
int smooth3_adjoint_add(P& pr, float* smooth, float* trace, float* itmp, float* itmp2,
                        float* xtmp) {
  int rc;
  if ((rc = pr.to_cross(smooth, xtmp))) return rc;
  if ((rc = pr.crossline(2, xtmp, itmp2))) return rc;
  if ((rc = pr.from_cross(itmp2, itmp, false))) return rc;
  return pr.inline_(1, itmp, trace);
}

// Vector names the driver passes to Ops.
enum Vec { kP, kR, kSP, kGP, kSX, kGX, kSR, kGR, kX };

// Ops: init(), residual(), grad(eps), mask(), first(), conj(a), step(a),
//      smooth(in, out) (out = S in), smooth_adj_add(in, out) (out += S' in),
//      dot(a, b) (double), each returning 0 or an error status.
template <class Ops>
int conjgrad(Ops& ops, int niter, float lam) {
  const float eps = lam * lam;
  const float tolf = 10 * FLT_EPSILON;  // csint2d: 10 * FLT_EPSILON in float
  const double tol = (double)tolf;
  int rc;
  if ((rc = ops.init())) return rc;
  if ((rc = ops.smooth(kP, kX))) return rc;  // x = S p
  if ((rc = ops.residual())) return rc;
  double r0 = 0.;
  if ((rc = ops.dot(kR, kR, &r0))) return rc;
  if (r0 == 0.) return 0;
  double gn = 0., gnp = 0., g0 = 0.;
  for (int iter = 0; iter < niter; iter++) {
    if ((rc = ops.grad(eps))) return rc;
    if ((rc = ops.smooth_adj_add(kGX, kGP))) return rc;  // gp += S' gx
    if ((rc = ops.smooth(kGP, kGX))) return rc;          // gx = S gp
    if ((rc = ops.mask())) return rc;
    if ((rc = ops.dot(kGP, kGP, &gn))) return rc;
    if (iter == 0) {
      g0 = gn;
      if ((rc = ops.first())) return rc;
    } else {
      const double alpha = gn / gnp, dg = gn / g0;
      if (alpha < tol || dg < tol) break;
      if ((rc = ops.conj((float)alpha))) return rc;
    }
    double srr = 0., spp = 0., sxx = 0.;
    if ((rc = ops.dot(kSR, kSR, &srr)) || (rc = ops.dot(kSP, kSP, &spp)) ||
        (rc = ops.dot(kSX, kSX, &sxx)))
      return rc;
    const double beta = srr + (double)eps * (spp - sxx);
    if ((rc = ops.step((float)(-gn / beta)))) return rc;
    gnp = gn;
  }
  return 0;
}

}  // namespace sint
}  // namespace pwd
