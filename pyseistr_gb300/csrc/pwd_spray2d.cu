// 2-D plane-wave spray with the structure-oriented mean and median.
//
// Restates csomean2d / csomf2d (pyseistr/src/sof_cfuns.c:1433-1678) with
// pwsmooth_* (:1036-1122) and pwspray_lop (:948-1033).  The spray of a
// section is two independent prediction chains per source trace (towards
// lower and higher trace numbers); every chain is one GPU thread, every
// slice of an n3 > 1 volume is processed in the same launch.
#include <algorithm>

#include "pwd_median.cuh"
#include "pwd_predict.cuh"

namespace pwd {
namespace {

struct Spray2 {
  int n1, n2, n3, ns, np;
  float eps, eps2;
};

// Forward spray (pwspray_lop adj=false): u[tr][np][n1], tr = i3*n2 + i2.
// Thread (i3, source i, dir).  in == nullptr sprays a trace of ones.
template <int NW>
__global__ void k_spray2_chains(const float* __restrict__ in, const float* __restrict__ ones,
                                const float* __restrict__ dip, float* __restrict__ u, Spray2 s,
                                ApCoef c, PredictScratch sc) {
  const long nthr = 2L * s.n2 * s.n3;
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= nthr) return;
  const int dir = (int)(t & 1);
  const long q = t >> 1;
  const int i = (int)(q % s.n2);
  const long i3 = q / s.n2;
  const long n12 = (long)s.n1 * s.n2;
  const float* pp = dip + i3 * n12;
  float* U = u + i3 * s.n2 * (long)s.np * s.n1;
  const float* src = in ? in + i3 * n12 + (long)i * s.n1 : ones;
  PredictScratch my = sc;
  my.o += t;
  my.d += t;
  my.y += t;
  auto slot = [&](int k, int sl) { return U + ((long)k * s.np + sl) * s.n1; };
  if (dir == 0) {
    float* cen = slot(i, s.ns);
    for (int i1 = 0; i1 < s.n1; i1++) cen[i1] = src[i1];
    const float* prev = src;
    for (int is = 0; is < s.ns; is++) {  // predict forward: to trace i-is-1
      int ip = i - is - 1;
      if (ip < 0) break;
      float* out = slot(ip, s.ns - is - 1);
      predict_fwd<NW, false>(s.n1, s.eps, s.eps2, c, prev, pp + (long)ip * s.n1, false, nullptr,
                             nullptr, false, out, my);
      prev = out;
    }
  } else {
    const float* prev = src;
    for (int is = 0; is < s.ns; is++) {  // predict backward: to trace i+is+1
      int ip = i + is + 1;
      if (ip >= s.n2) break;
      float* out = slot(ip, s.ns + is + 1);
      predict_fwd<NW, false>(s.n1, s.eps, s.eps2, c, prev, pp + (long)(ip - 1) * s.n1, true,
                             nullptr, nullptr, false, out, my);
      prev = out;
    }
  }
}

// pwsmooth weights w[is] = ns+1-|is-ns| (pwsmooth_init :1055-1058).
__device__ __forceinline__ float tri_weight(int is, int ns) {
  int a = is - ns;
  return (float)(ns + 1 - (a >= 0 ? a : -a));
}

// pwsmooth_set :1102-1122: w1 = 1 / (weighted spray of ones), 0 where 0.
__global__ void k_norm_weights(const float* __restrict__ u, float* __restrict__ w1, Spray2 s) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = (long)s.n1 * s.n2 * s.n3;
  if (t >= n) return;
  const long tr = t / s.n1;
  const int i1 = (int)(t % s.n1);
  const float* panel = u + tr * s.np * (long)s.n1 + i1;
  float acc = 0.f;
  for (int is = 0; is < s.np; is++)
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(panel[(long)is * s.n1], tri_weight(is, s.ns)), 1.0f));
  w1[t] = (acc != 0.f) ? __double2float_rn(1.0 / (double)acc) : 0.f;
}

// pwsmooth_lop forward :1088-1098: smooth = sum_is u*w[is]*w1.
__global__ void k_weighted_mean(const float* __restrict__ u, const float* __restrict__ w1,
                                float* __restrict__ out, Spray2 s) {
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long n = (long)s.n1 * s.n2 * s.n3;
  if (t >= n) return;
  const long tr = t / s.n1;
  const int i1 = (int)(t % s.n1);
  const float* panel = u + tr * s.np * (long)s.n1 + i1;
  const float ws = w1[t];
  float acc = 0.f;
  for (int is = 0; is < s.np; is++)
    acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(panel[(long)is * s.n1], tri_weight(is, s.ns)), ws));
  out[t] = acc;
}

// Adjoint of the weighted mean (pwsmooth_lop adjoint :1072-1086 with
// pwspray_lop adjoint :957-989).  Thread (i3, output trace i); traces in a
// per-thread contiguous buffer tb[n1].
template <int NW>
__global__ void k_somean2d_adj(const float* __restrict__ x, const float* __restrict__ dip,
                               const float* __restrict__ w1, float* __restrict__ out,
                               float* __restrict__ tbuf, Spray2 s, ApCoef c, PredictScratch sc) {
  const long nthr = (long)s.n2 * s.n3;
  long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (t >= nthr) return;
  const int i = (int)(t % s.n2);
  const long i3 = t / s.n2;
  const long n12 = (long)s.n1 * s.n2;
  const float* pp = dip + i3 * n12;
  const float* X = x + i3 * n12;
  const float* W = w1 + i3 * n12;
  float* tr = tbuf + t * s.n1;
  PredictScratch my = sc;
  my.o += t;
  my.d += t;
  my.y += t;
  float* o = out + i3 * n12 + (long)i * s.n1;
  auto add_slot = [&](int ip, int sl) {
    const float wv = tri_weight(sl, s.ns);
    for (int i1 = 0; i1 < s.n1; i1++) {
      long e = (long)ip * s.n1 + i1;
      tr[i1] = __fadd_rn(tr[i1], __fmul_rn(__fmul_rn(X[e], wv), W[e]));
    }
  };
  for (int i1 = 0; i1 < s.n1; i1++) tr[i1] = 0.f;
  for (int is = s.ns - 1; is >= 0; is--) {
    int ip = i + is + 1;
    if (ip >= s.n2) continue;
    add_slot(ip, s.ns + is + 1);
    predict_adj<NW>(s.n1, s.eps, s.eps2, c, tr, pp + (long)(ip - 1) * s.n1, true, my, my.y);
  }
  for (int i1 = 0; i1 < s.n1; i1++) {
    o[i1] = __fadd_rn(0.f, tr[i1]);
    tr[i1] = 0.f;
  }
  for (int is = s.ns - 1; is >= 0; is--) {
    int ip = i - is - 1;
    if (ip < 0) continue;
    add_slot(ip, s.ns - is - 1);
    predict_adj<NW>(s.n1, s.eps, s.eps2, c, tr, pp + (long)ip * s.n1, false, my, my.y);
  }
  const float wc = tri_weight(s.ns, s.ns);
  for (int i1 = 0; i1 < s.n1; i1++) {
    long e = (long)i * s.n1 + i1;
    float v = __fadd_rn(o[i1], tr[i1]);
    o[i1] = __fadd_rn(v, __fmul_rn(__fmul_rn(X[e], wc), W[e]));
  }
}

struct SprayWork {
  float *u, *w1, *ones, *v2, *avg, *tbuf;
  PredictScratch sc;
};

SprayWork carve_spray2(void* ws, int n1, int n2, int n3, int ns, int order, bool need_w1,
                       bool need_svmf, bool adj, size_t* total) {
  const long n = (long)n1 * n2 * n3;
  const int np = 2 * ns + 1, nb = 2 * order;
  const long nthr = 2L * n2 * n3;
  Carver cv(ws);
  SprayWork w;
  w.u = cv.take<float>(n * np);
  w.w1 = need_w1 ? cv.take<float>(n) : nullptr;
  w.ones = cv.take<float>(n1);
  w.v2 = need_svmf ? cv.take<float>(n * np) : nullptr;
  w.avg = need_svmf ? cv.take<float>((long)n2 * n3) : nullptr;
  w.tbuf = adj ? cv.take<float>(n) : nullptr;
  w.sc.o = cv.take<float>((long)nb * n1 * nthr);
  w.sc.d = cv.take<float>((long)n1 * nthr);
  w.sc.y = cv.take<float>((long)n1 * nthr);
  w.sc.ss = nthr;
  *total = cv.size();
  return w;
}

__global__ void k_fill(float* x, float v, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

template <int NW>
int spray2_forward(const float* in, const float* dip, const SprayWork& w, const Spray2& s,
                   cudaStream_t st) {
  const ApCoef c = make_apcoef(NW);
  const long nthr = 2L * s.n2 * s.n3;
  const int b = 64;
  k_spray2_chains<NW><<<(unsigned)((nthr + b - 1) / b), b, 0, st>>>(in, w.ones, dip, w.u, s, c,
                                                                    w.sc);
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

int spray2_forward_dispatch(int order, const float* in, const float* dip, const SprayWork& w,
                            const Spray2& s, cudaStream_t st) {
  switch (order) {
    case 1: return spray2_forward<1>(in, dip, w, s, st);
    case 2: return spray2_forward<2>(in, dip, w, s, st);
    case 3: return spray2_forward<3>(in, dip, w, s, st);
    case 4: return spray2_forward<4>(in, dip, w, s, st);
  }
  return PWD_ENOTSUP;
}

int somean2d_adj_dispatch(int order, const float* x, const float* dip, float* out,
                          const SprayWork& w, const Spray2& s, cudaStream_t st) {
  const long nthr = (long)s.n2 * s.n3;
  const int b = 64;
  const unsigned g = (unsigned)((nthr + b - 1) / b);
  switch (order) {
    case 1: k_somean2d_adj<1><<<g, b, 0, st>>>(x, dip, w.w1, out, w.tbuf, s, make_apcoef(1), w.sc); break;
    case 2: k_somean2d_adj<2><<<g, b, 0, st>>>(x, dip, w.w1, out, w.tbuf, s, make_apcoef(2), w.sc); break;
    case 3: k_somean2d_adj<3><<<g, b, 0, st>>>(x, dip, w.w1, out, w.tbuf, s, make_apcoef(3), w.sc); break;
    case 4: k_somean2d_adj<4><<<g, b, 0, st>>>(x, dip, w.w1, out, w.tbuf, s, make_apcoef(4), w.sc); break;
    default: return PWD_ENOTSUP;
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

int check2(int n1, int n2, int n3, int ns, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns < 0 || order < 1) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  return PWD_OK;
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_somean2d_workspace_size(int n1, int n2, int n3, int ns, int order) {
  if (check2(n1, n2, n3, ns, order) != PWD_OK) return 0;
  size_t t = 0;
  carve_spray2(nullptr, n1, n2, n3, ns, order, true, false, true, &t);
  return t;
}

extern "C" int pwd_somean2d(const float* data, const float* dip, float* out, int n1, int n2,
                            int n3, int ns, int order, int adj, float eps, void* workspace,
                            size_t workspace_bytes, pwd_stream_t stream) {
  int rc = check2(n1, n2, n3, ns, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip || !out) return PWD_EINVAL;
  size_t need = 0;
  carve_spray2(nullptr, n1, n2, n3, ns, order, true, false, true, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  SprayWork w = carve_spray2(workspace, n1, n2, n3, ns, order, true, false, true, &need);
  cudaStream_t st = (cudaStream_t)stream;
  Spray2 s;
  s.n1 = n1; s.n2 = n2; s.n3 = n3; s.ns = ns; s.np = 2 * ns + 1;
  s.eps = eps * eps;  // pwspray_init :928 predict_init(eps*eps, ...)
  s.eps2 = s.eps;
  const long n = (long)n1 * n2 * n3;
  const int b = 256;
  const unsigned gn = (unsigned)((n + b - 1) / b);
  k_fill<<<(unsigned)((n1 + b - 1) / b), b, 0, st>>>(w.ones, 1.0f, n1);
  // pwsmooth_set: spray of ones and its weighted sum
  if ((rc = spray2_forward_dispatch(order, nullptr, dip, w, s, st)) != PWD_OK) return rc;
  k_norm_weights<<<gn, b, 0, st>>>(w.u, w.w1, s);
  if (adj) {
    rc = somean2d_adj_dispatch(order, data, dip, out, w, s, st);
    if (rc != PWD_OK) return rc;
  } else {
    if ((rc = spray2_forward_dispatch(order, data, dip, w, s, st)) != PWD_OK) return rc;
    k_weighted_mean<<<gn, b, 0, st>>>(w.u, w.w1, out, s);
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

extern "C" size_t pwd_somf2d_workspace_size(int n1, int n2, int n3, int ns, int nmf, int option,
                                            int order) {
  if (check2(n1, n2, n3, ns, order) != PWD_OK || !median_args_ok(nmf, option)) return 0;
  size_t t = 0;
  carve_spray2(nullptr, n1, n2, n3, ns, order, false, option != 1, false, &t);
  return t;
}

extern "C" int pwd_somf2d(const float* data, const float* dip, float* out, int n1, int n2, int n3,
                          int ns, int nmf, int option, int order, float eps, void* workspace,
                          size_t workspace_bytes, pwd_stream_t stream) {
  int rc = check2(n1, n2, n3, ns, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip || !out) return PWD_EINVAL;
  if (!median_args_ok(nmf, option)) return nmf < 1 ? PWD_EINVAL : PWD_ENOTSUP;
  size_t need = 0;
  carve_spray2(nullptr, n1, n2, n3, ns, order, false, option != 1, false, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  SprayWork w = carve_spray2(workspace, n1, n2, n3, ns, order, false, option != 1, false, &need);
  cudaStream_t st = (cudaStream_t)stream;
  Spray2 s;
  s.n1 = n1; s.n2 = n2; s.n3 = n3; s.ns = ns; s.np = 2 * ns + 1;
  s.eps = eps * eps;
  s.eps2 = s.eps;
  if ((rc = spray2_forward_dispatch(order, data, dip, w, s, st)) != PWD_OK) return rc;
  return launch_panel_median(w.u, out, w.v2, w.avg, n1, s.np, (long)n2 * n3, nmf, option, st);
}

extern "C" size_t pwd_panel_median_workspace_size(int n1, int np, long ntr, int nmf, int option) {
  if (n1 < 1 || np < 1 || ntr < 1 || !median_args_ok(nmf, option)) return 0;
  Carver cv(nullptr);
  if (option != 1) {
    cv.take<float>(ntr * np * (long)n1);
    cv.take<float>(ntr);
  } else {
    cv.take<float>(1);
  }
  return cv.size();
}

extern "C" int pwd_panel_median(const float* panels, float* out, int n1, int np, long ntr, int nmf,
                                int option, void* workspace, size_t workspace_bytes,
                                pwd_stream_t stream) {
  if (!panels || !out || n1 < 1 || np < 1 || ntr < 1) return PWD_EINVAL;
  if (!median_args_ok(nmf, option)) return nmf < 1 ? PWD_EINVAL : PWD_ENOTSUP;
  size_t need = pwd_panel_median_workspace_size(n1, np, ntr, nmf, option);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  Carver cv(workspace);
  float* v2 = nullptr;
  float* avg = nullptr;
  if (option != 1) {
    v2 = cv.take<float>(ntr * np * (long)n1);
    avg = cv.take<float>(ntr);
  }
  return launch_panel_median(panels, out, v2, avg, n1, np, ntr, nmf, option, (cudaStream_t)stream);
}
