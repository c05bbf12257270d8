// Test harness: the conjugate-gradient driver and per-sample code of the
// sparse-data interpolation (pyseistr_gb300/csrc/pwd_sint.cuh) run on the
// CPU, with the oracle's plane-wave smoothing standing in for the GPU spray
// kernels (which the GPU tests check against the oracle on their own), so
// that the CPU tests check the driver's operation sequence and scalars.
// Dot products are summed serially here.  Not part of the library.
#include <vector>

#include "../../oracle/pwd_oracle.cpp"
#include "../../pyseistr_gb300/csrc/pwd_sint.cuh"

namespace {

struct HostOps {
  pwd::sint::Vecs v;
  long n;
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
  int smooth(int in, int out) { S.lop(false, false, vec(in), vec(out)); return 0; }
  int smooth_adj_add(int in, int out) { S.lop(true, true, vec(out), vec(in)); return 0; }
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
