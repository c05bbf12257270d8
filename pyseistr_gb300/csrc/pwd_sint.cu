// Sparse-data interpolation (csint2d, pyseistr/src/soint2d_cfuns.c:2421-2523,
// called by sint2dc, sint.py:61; csint3d, soint3d_cfuns.c:2510-2612, called
// by sint3dc, sint.py:97): the C entries, their per-sample kernels and the
// GPU operations of the CG driver in pwd_sint.cuh.
//
// Each CG iteration applies the adjoint and the forward plane-wave
// smoothing (the spray kernels of pwd_spray2d.cu, through smooth2_run) and
// a handful of per-sample passes; the dot products are FP64 sums (per
// thread, per block in a fixed tree, then the blocks' partials summed on the
// host in block order: run-to-run deterministic).  The driver needs the dot
// products on the host to take the reference's decisions (the step, the
// conjugate scale and the early stop), so the call synchronises its stream
// twice per iteration.
#include <cuda_runtime.h>

#include <vector>

#include "pwd_common.cuh"
#include "pwd_sint.cuh"

namespace pwd {

size_t smooth2_workspace(int n1, int n2, int n3, int ns, int order);
int smooth2_run(const float* in, const float* dip, float* out, int n1, int n2, int n3, int ns,
                int order, float eps, int mode, void* ws, size_t wsb, cudaStream_t st,
                int reuse);

namespace {

constexpr int kSintThreads = 256;
constexpr int kSintDotBlocks = 512;

enum SintPass { kInit, kResidual, kGrad, kMask, kFirst, kConj, kStep };

__global__ void __launch_bounds__(kSintThreads) k_sint_pass(sint::Vecs v, long n, int pass,
                                                            float a) {
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride) {
    switch (pass) {
      case kInit: sint::init_sample(v, i); break;
      case kResidual: sint::residual_sample(v, i); break;
      case kGrad: sint::grad_sample(v, i, a); break;
      case kMask: sint::mask_sample(v, i); break;
      case kFirst: sint::first_sample(v, i); break;
      case kConj: sint::conj_sample(v, i, a); break;
      default: sint::step_sample(v, i, a); break;
    }
  }
}

// FP64 partial sums of x*y: one per block, in a fixed order.
__global__ void __launch_bounds__(kSintThreads) k_sint_dot(const float* __restrict__ x,
                                                           const float* __restrict__ y, long n,
                                                           double* __restrict__ part) {
  __shared__ double sh[kSintThreads];
  double t = 0.;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    t += (double)x[i] * (double)y[i];
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int h = kSintThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Known samples (mask != 0), one integer per block.
__global__ void __launch_bounds__(kSintThreads) k_sint_count(const float* __restrict__ mask,
                                                             long n,
                                                             unsigned long long* __restrict__ part) {
  __shared__ unsigned long long sh[kSintThreads];
  unsigned long long t = 0;
  const long stride = (long)gridDim.x * blockDim.x;
  for (long i = (long)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += stride)
    t += mask[i] != 0.f;
  sh[threadIdx.x] = t;
  __syncthreads();
  for (int h = kSintThreads / 2; h > 0; h >>= 1) {
    if ((int)threadIdx.x < h) sh[threadIdx.x] += sh[threadIdx.x + h];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = sh[0];
}

// Cube <-> crossline-major transposes (pwsmooth3_lop's index shuffles).
__global__ void __launch_bounds__(kSintThreads) k_sint_cross(const float* __restrict__ a,
                                                             float* __restrict__ b, int n1,
                                                             int n2, int n3, int to, int sum) {
  const long n = (long)n1 * n2 * n3, stride = (long)gridDim.x * blockDim.x;
  for (long e = (long)blockIdx.x * blockDim.x + threadIdx.x; e < n; e += stride) {
    if (to)
      sint::to_crossline_sample(a, b, n1, n2, n3, e);
    else
      sint::from_crossline_sample(a, b, n1, n2, n3, e, sum != 0);
  }
}

struct SintLayout {
  size_t vec_bytes, part_bytes, smooth_bytes, cross_bytes, total;
};

// 8 CG vectors, for csint3d 4 more (itmp, itmp2, xtmp and the transposed
// crossline slope), the dot partials and the smoothing's workspaces: one
// for the inline smoothing and, in 3-D, one for the crossline smoothing, so
// that each keeps the factor store of its own slope field across calls.
SintLayout sint_layout(int n1, int n2, int n3, int ns1, int ns2, int order1, int order2,
                       bool three) {
  SintLayout l{};
  const long n = (long)n1 * n2 * n3;
  l.vec_bytes = ((sizeof(float) * (size_t)n + 255) & ~(size_t)255);
  l.part_bytes = ((sizeof(double) * kSintDotBlocks + 255) & ~(size_t)255);
  l.smooth_bytes = (smooth2_workspace(n1, n2, n3, ns1, order1) + 255) & ~(size_t)255;
  l.cross_bytes = three ? (smooth2_workspace(n1, n3, n2, ns2, order2) + 255) & ~(size_t)255 : 0;
  const bool ok = l.smooth_bytes && (!three || l.cross_bytes);
  const int nvec = three ? 12 : 8;
  l.total = ok ? nvec * l.vec_bytes + l.part_bytes + l.smooth_bytes + l.cross_bytes : 0;
  return l;
}

struct GpuOps {
  sint::Vecs v;
  long n;
  int n1, n2, n3;
  bool three;               // csint3d's smoothing (inline, then crossline)
  const float* dipi;        // inline slopes, cube layout
  const float* xd;          // crossline slopes, crossline-major layout (3-D)
  int ns1, ns2, order1, order2;
  float eps;                // the smoothing's eps (csint2d's / csint3d's eps argument)
  float *itmp, *itmp2, *xtmp;
  void* sws;  // inline smoothing workspace
  size_t swsb;
  void* cws;  // crossline smoothing workspace (3-D)
  size_t cwsb;
  double* part;
  std::vector<double> host;
  cudaStream_t st;
  unsigned grid;

  float* vec(int k) const {
    switch (k) {
      case sint::kP: return v.p;
      case sint::kR: return v.r;
      case sint::kSP: return v.sp;
      case sint::kGP: return v.gp;
      case sint::kSX: return v.sx;
      case sint::kGX: return v.gx;
      case sint::kSR: return v.sr;
      case sint::kGR: return v.gr;
      default: return v.x;
    }
  }
  int pass(int which, float a) {
    PWD_KERNEL(PWD_FAM_CG, st, (k_sint_pass<<<grid, kSintThreads, 0, st>>>(v, n, which, a)));
    return cuda_status(cudaGetLastError());
  }
  int init() { return pass(kInit, 0.f); }
  int residual() { return pass(kResidual, 0.f); }
  int grad(float e) { return pass(kGrad, e); }
  int mask() { return pass(kMask, 0.f); }
  int first() { return pass(kFirst, 0.f); }
  int conj(float a) { return pass(kConj, a); }
  int step(float a) { return pass(kStep, a); }
  // primitives of the 3-D sequence
  // Each smoothing (inline, and crossline in 3-D) always runs on one slope
  // field in its own workspace: after its first call, each call reuses the
  // factor store and w1 the previous one left there.
  bool factored = false, cfactored = false;
  int inline_(int mode, float* in, float* out) {
    const int rc = smooth2_run(in, dipi, out, n1, n2, n3, ns1, order1, eps, mode, sws, swsb, st,
                               factored ? 1 : 0);
    if (rc == PWD_OK) factored = true;
    return rc;
  }
  int crossline(int mode, float* in, float* out) {
    const int rc = smooth2_run(in, xd, out, n1, n3, n2, ns2, order2, eps, mode, cws, cwsb, st,
                               cfactored ? 1 : 0);
    if (rc == PWD_OK) cfactored = true;
    return rc;
  }
  int cross(const float* a, float* b, int to, int sum) {
    PWD_KERNEL(PWD_FAM_CG, st,
               (k_sint_cross<<<grid, kSintThreads, 0, st>>>(a, b, n1, n2, n3, to, sum)));
    return cuda_status(cudaGetLastError());
  }
  int to_cross(float* c, float* t) { return cross(c, t, 1, 0); }
  int from_cross(float* t, float* c, bool sum) { return cross(t, c, 0, sum ? 1 : 0); }
  int smooth(int in, int out) {
    if (!three) return inline_(0, vec(in), vec(out));
    return sint::smooth3_forward(*this, vec(in), vec(out), itmp, itmp2, xtmp);
  }
  int smooth_adj_add(int in, int out) {
    if (!three) return inline_(1, vec(in), vec(out));
    return sint::smooth3_adjoint_add(*this, vec(in), vec(out), itmp, itmp2, xtmp);
  }
  int dot(int a, int b, double* s) {
    PWD_KERNEL(PWD_FAM_CG, st,
               (k_sint_dot<<<kSintDotBlocks, kSintThreads, 0, st>>>(vec(a), vec(b), n, part)));
    int rc = cuda_status(cudaGetLastError());
    if (rc != PWD_OK) return rc;
    rc = cuda_status(cudaMemcpyAsync(host.data(), part, sizeof(double) * kSintDotBlocks,
                                     cudaMemcpyDeviceToHost, st));
    if (rc != PWD_OK) return rc;
    rc = cuda_status(cudaStreamSynchronize(st));
    if (rc != PWD_OK) return rc;
    double t = 0.;
    for (int k = 0; k < kSintDotBlocks; k++) t += host[k];
    *s = t;
    return PWD_OK;
  }
};

bool sint_args_ok(int n1, int n2, int n3, int niter, int ns1, int ns2) {
  return n1 >= 4 && n2 >= 1 && n3 >= 1 && niter >= 0 && ns1 >= 0 && ns2 >= 0 &&
         (long)n1 * n2 * n3 < (1L << 31);
}

// Both entries: three = false is csint2d (n3 = 1; ns2, order2 unused),
// three = true csint3d (for any n3, one included: its crossline pass still
// rounds).
int sint_run(const float* din, const float* dipi, const float* dipx, const float* mask,
             float* out, int n1, int n2, int n3, int niter, int ns1, int ns2, int order1,
             int order2, float eps, bool three, void* workspace, size_t workspace_bytes,
             cudaStream_t st) {
  const SintLayout l = sint_layout(n1, n2, n3, ns1, ns2, order1, order2, three);
  if (!l.total || !workspace || workspace_bytes < l.total || (uintptr_t)workspace % 256)
    return PWD_EWORKSPACE;
  const long n = (long)n1 * n2 * n3;
  char* base = (char*)workspace;
  GpuOps ops;
  ops.n = n;
  ops.n1 = n1;
  ops.n2 = n2;
  ops.n3 = n3;
  ops.three = three;
  ops.dipi = dipi;
  ops.ns1 = ns1;
  ops.ns2 = ns2;
  ops.order1 = order1;
  ops.order2 = order2;
  ops.eps = eps;
  ops.st = st;
  float* f[12];
  const int nvec = three ? 12 : 8;
  for (int k = 0; k < nvec; k++) f[k] = (float*)(base + k * l.vec_bytes);
  ops.v.din = din;
  ops.v.mask = mask;
  ops.v.x = out;
  ops.v.p = f[0];
  ops.v.r = f[1];
  ops.v.sp = f[2];
  ops.v.gp = f[3];
  ops.v.sx = f[4];
  ops.v.gx = f[5];
  ops.v.sr = f[6];
  ops.v.gr = f[7];
  ops.itmp = three ? f[8] : nullptr;
  ops.itmp2 = three ? f[9] : nullptr;
  ops.xtmp = three ? f[10] : nullptr;
  float* xd = three ? f[11] : nullptr;
  ops.xd = xd;
  ops.part = (double*)(base + nvec * l.vec_bytes);
  ops.sws = base + nvec * l.vec_bytes + l.part_bytes;
  ops.swsb = l.smooth_bytes;
  ops.cws = three ? base + nvec * l.vec_bytes + l.part_bytes + l.smooth_bytes : nullptr;
  ops.cwsb = l.cross_bytes;
  ops.host.assign(kSintDotBlocks, 0.);
  const long blocks = (n + kSintThreads - 1) / kSintThreads;
  ops.grid = (unsigned)(blocks < 152L * 8 * 16 ? blocks : 152L * 8 * 16);
  int rc;
  if (three && (rc = ops.cross(dipx, xd, 1, 0))) return rc;
  // the lambda from the number of known samples
  unsigned long long* cpart = (unsigned long long*)ops.part;
  PWD_KERNEL(PWD_FAM_CG, st,
             (k_sint_count<<<kSintDotBlocks, kSintThreads, 0, st>>>(mask, n, cpart)));
  rc = cuda_status(cudaGetLastError());
  if (rc != PWD_OK) return rc;
  std::vector<unsigned long long> cnt(kSintDotBlocks, 0);
  rc = cuda_status(cudaMemcpyAsync(cnt.data(), cpart, sizeof(unsigned long long) * kSintDotBlocks,
                                   cudaMemcpyDeviceToHost, st));
  if (rc == PWD_OK) rc = cuda_status(cudaStreamSynchronize(st));
  if (rc != PWD_OK) return rc;
  unsigned long long known = 0;
  for (unsigned long long c : cnt) known += c;
  return sint::conjgrad(ops, niter, sint::lambda_of(known, n));
}

}  // namespace
}  // namespace pwd

extern "C" size_t pwd_sint2d_workspace_size(int n1, int n2, int ns, int order) {
  if (!pwd::sint_args_ok(n1, n2, 1, 0, ns, 0) || order < 1 || order > PWD_MAX_ORDER) return 0;
  return pwd::sint_layout(n1, n2, 1, ns, 0, order, 1, false).total;
}

extern "C" int pwd_sint2d(const float* din, const float* dip, const float* mask, float* out,
                          int n1, int n2, int niter, int ns, int order, float eps,
                          void* workspace, size_t workspace_bytes, pwd_stream_t stream) {
  if (!din || !dip || !mask || !out || !pwd::sint_args_ok(n1, n2, 1, niter, ns, 0) ||
      order < 1)
    return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  return pwd::sint_run(din, dip, nullptr, mask, out, n1, n2, 1, niter, ns, 0, order, 1, eps,
                       false, workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" size_t pwd_sint3d_workspace_size(int n1, int n2, int n3, int ns1, int ns2, int order1,
                                            int order2) {
  if (!pwd::sint_args_ok(n1, n2, n3, 0, ns1, ns2) || order1 < 1 || order2 < 1 ||
      order1 > PWD_MAX_ORDER || order2 > PWD_MAX_ORDER)
    return 0;
  return pwd::sint_layout(n1, n2, n3, ns1, ns2, order1, order2, true).total;
}

extern "C" int pwd_sint3d(const float* din, const float* dipi, const float* dipx,
                          const float* mask, float* out, int n1, int n2, int n3, int niter,
                          int ns1, int ns2, int order1, int order2, float eps, void* workspace,
                          size_t workspace_bytes, pwd_stream_t stream) {
  if (!din || !dipi || !dipx || !mask || !out || !pwd::sint_args_ok(n1, n2, n3, niter, ns1, ns2) ||
      order1 < 1 || order2 < 1)
    return PWD_EINVAL;
  if (order1 > PWD_MAX_ORDER || order2 > PWD_MAX_ORDER) return PWD_ENOTSUP;
  return pwd::sint_run(din, dipi, dipx, mask, out, n1, n2, n3, niter, ns1, ns2, order1, order2,
                       eps, true, workspace, workspace_bytes, (cudaStream_t)stream);
}
