// Test harness: the conjugate-gradient driver, the 3-D smoothing sequence
// and the per-sample code of the sparse-data interpolation
// (pyseistr_gb300/csrc/pwd_sint.cuh) run on the CPU, with the oracle's 2-D
// plane-wave smoothing of one slice standing in for the GPU spray kernels
// (which the GPU tests check against the oracle on their own), so that the
// CPU tests check the driver's operation sequence, scalars and transposes.
// Dot products are summed serially here.  Not part of the library.
#include <vector>

#include "../../oracle/pwd_oracle.cpp"
#include "../../pyseistr_gb300/csrc/pwd_sint.cuh"

namespace {

struct HostOps {
  pwd::sint::Vecs v;
  long n;
  int n1 = 0, n2 = 0, n3 = 1, ns1 = 0, ns2 = 0, order1 = 1, order2 = 1;
  bool three = false;  // csint3d's smoothing
  float eps = 0.f;
  const float* dipi = nullptr;
  std::vector<float> xd, itmp, itmp2, xtmp;
  orc::PwSmooth2<float> S;
  float* vec(int k) {
    using namespace pwd::sint;
    switch (k) {
      case kP: return v.p;
      case kR: return v.r;
      case kSP: return v.sp;
      case kGP: return v.gp;
      case kSX: return v.sx;
      case kGX: return v.gx;
      case kSR: return v.sr;
      case kGR: return v.gr;
      default: return v.x;
    }
  }
  int init() { for (long i = 0; i < n; i++) pwd::sint::init_sample(v, i); return 0; }
  int residual() { for (long i = 0; i < n; i++) pwd::sint::residual_sample(v, i); return 0; }
  int grad(float e) { for (long i = 0; i < n; i++) pwd::sint::grad_sample(v, i, e); return 0; }
  int mask() { for (long i = 0; i < n; i++) pwd::sint::mask_sample(v, i); return 0; }
  int first() { for (long i = 0; i < n; i++) pwd::sint::first_sample(v, i); return 0; }
  int conj(float a) { for (long i = 0; i < n; i++) pwd::sint::conj_sample(v, i, a); return 0; }
  int step(float a) { for (long i = 0; i < n; i++) pwd::sint::step_sample(v, i, a); return 0; }
  // the 2-D smoothing of every slice: mode 0 out = S in, 1 out += S' in, 2 out = S' in
  int slices(int mode, const float* dip, int m1, int m2, int m3, int ns, int order, float* in,
             float* out) {
    const long m12 = (long)m1 * m2;
    orc::PwSmooth2<float> T;
    T.init(ns, m1, m2, order, eps);
    for (int k = 0; k < m3; k++) {
      T.set(dip + k * m12);
      if (mode == 0)
        T.lop(false, false, in + k * m12, out + k * m12);
      else
        T.lop(true, mode == 1, out + k * m12, in + k * m12);
    }
    return 0;
  }
  int inline_(int mode, float* in, float* out) {
    return slices(mode, dipi, n1, n2, n3, ns1, order1, in, out);
  }
  int crossline(int mode, float* in, float* out) {
    return slices(mode, xd.data(), n1, n3, n2, ns2, order2, in, out);
  }
  int to_cross(float* c, float* t) {
    for (long e = 0; e < n; e++) pwd::sint::to_crossline_sample(c, t, n1, n2, n3, e);
    return 0;
  }
  int from_cross(float* t, float* c, bool sum) {
    for (long e = 0; e < n; e++) pwd::sint::from_crossline_sample(t, c, n1, n2, n3, e, sum);
    return 0;
  }
  int smooth(int in, int out) {
    if (!three) {
      S.lop(false, false, vec(in), vec(out));
      return 0;
    }
    return pwd::sint::smooth3_forward(*this, vec(in), vec(out), itmp.data(), itmp2.data(),
                                      xtmp.data());
  }
  int smooth_adj_add(int in, int out) {
    if (!three) {
      S.lop(true, true, vec(out), vec(in));
      return 0;
    }
    return pwd::sint::smooth3_adjoint_add(*this, vec(in), vec(out), itmp.data(), itmp2.data(),
                                          xtmp.data());
  }
  int dot(int a, int b, double* s) {
    const float *x = vec(a), *y = vec(b);
    double t = 0.;
    for (long i = 0; i < n; i++) t += (double)x[i] * (double)y[i];
    *s = t;
    return 0;
  }
};

}  // namespace

extern "C" int emu_sint2d(const float* din, const float* dip, const float* mask, float* out,
                          int n1, int n2, int niter, int ns, int order, float eps) {
  if (n1 < 4 || n2 < 1 || ns < 0 || order < 1 || order > 4 || niter < 0) return 1;
  const long n = (long)n1 * n2;
  std::vector<float> buf(8 * n);
  HostOps ops;
  ops.n = n;
  ops.v.din = din;
  ops.v.mask = mask;
  ops.v.x = out;
  float* b = buf.data();
  ops.v.p = b; ops.v.r = b + n; ops.v.sp = b + 2 * n; ops.v.gp = b + 3 * n;
  ops.v.sx = b + 4 * n; ops.v.gx = b + 5 * n; ops.v.sr = b + 6 * n; ops.v.gr = b + 7 * n;
  unsigned long long known = 0;
  for (long i = 0; i < n; i++) known += mask[i] != 0.f;
  ops.S.init(ns, n1, n2, order, eps);
  ops.S.set(dip);
  return pwd::sint::conjgrad(ops, niter, pwd::sint::lambda_of(known, n));
}

extern "C" int emu_sint3d(const float* din, const float* dipi, const float* dipx,
                          const float* mask, float* out, int n1, int n2, int n3, int niter,
                          int ns1, int ns2, int order1, int order2, float eps) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns1 < 0 || ns2 < 0 || order1 < 1 || order1 > 4 ||
      order2 < 1 || order2 > 4 || niter < 0)
    return 1;
  const long n = (long)n1 * n2 * n3;
  std::vector<float> buf(8 * n);
  HostOps ops;
  ops.n = n;
  ops.n1 = n1;
  ops.n2 = n2;
  ops.n3 = n3;
  ops.three = true;
  ops.ns1 = ns1;
  ops.ns2 = ns2;
  ops.order1 = order1;
  ops.order2 = order2;
  ops.eps = eps;
  ops.dipi = dipi;
  ops.v.din = din;
  ops.v.mask = mask;
  ops.v.x = out;
  float* b = buf.data();
  ops.v.p = b; ops.v.r = b + n; ops.v.sp = b + 2 * n; ops.v.gp = b + 3 * n;
  ops.v.sx = b + 4 * n; ops.v.gx = b + 5 * n; ops.v.sr = b + 6 * n; ops.v.gr = b + 7 * n;
  ops.xd.assign(n, 0.f);
  ops.itmp.assign(n, 0.f);
  ops.itmp2.assign(n, 0.f);
  ops.xtmp.assign(n, 0.f);
  for (long e = 0; e < n; e++) pwd::sint::to_crossline_sample(dipx, ops.xd.data(), n1, n2, n3, e);
  unsigned long long known = 0;
  for (long i = 0; i < n; i++) known += mask[i] != 0.f;
  return pwd::sint::conjgrad(ops, niter, pwd::sint::lambda_of(known, n));
}
