// Local slope estimation by plane-wave destruction on the GPU.
//
// Restates dipc / dip3 / ps_divne / ps_conjgrad / ps_trianglen_lop of
// pyseistr/src/dip_cfuns.c (:1694-1989, :1619-1691, :796-827, :257-383,
// :672-712) as stream-ordered kernels.  All scalar control (CG convergence,
// line-search acceptance) lives on the device, so a call enqueues a fixed
// launch sequence and never synchronises with the host; kernels after a
// decided exit read a device flag and return at once.
#include <algorithm>
#include <cfloat>
#include <cmath>

#include "pwd_common.cuh"

namespace pwd {
namespace {

constexpr int kBlock = 256;

struct Geo {
  int n1, n2, n3;
  long n;
  long ip;   // neighbour offset: n1 (inline) or n1*n2 (crossline)
  int dip;   // 1 inline, 2 crossline
};

struct DipScalars {
  double usum, usum2, den2, norm2, r0;
  double gn, gnp, g0, alpha, step;
  int zero, cg_done, ls_done, ls_trials, cg_iters;
  unsigned cnt[8];
};

__device__ __forceinline__ bool pwd_valid(const Geo& g, long i, int nw) {
  int i1 = (int)(i % g.n1);
  long r = i / g.n1;
  if (i1 < nw || i1 >= g.n1 - nw) return false;
  if (g.dip == 1) return (int)(r % g.n2) < g.n2 - 1;
  return (int)(r / g.n2) < g.n3 - 1;
}

// allpass1/allpass2 at one sample (dip_cfuns.c:1135-1200, :1399-1465).
template <int NW, bool DER>
__device__ __forceinline__ float pwd_at(const float* __restrict__ u, long i, long ip,
                                        const ApCoef& c, float p) {
  float f[2 * NW + 1];
  if (DER)
    aderfilter<NW>(c, p, f);
  else
    passfilter<NW>(c, p, f);
  float y = 0.f;
#pragma unroll
  for (int iw = 0; iw <= 2 * NW; iw++) {
    int is = iw - NW;
    y = __fadd_rn(y, __fmul_rn(__fsub_rn(u[i + is + ip], u[i - is]), f[iw]));
  }
  return y;
}

template <int NW>
__global__ void k_residual(const float* __restrict__ u, const float* __restrict__ p,
                           float* __restrict__ u2, Geo g, ApCoef c) {
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < g.n;
       i += (long)gridDim.x * blockDim.x)
    u2[i] = pwd_valid(g, i, NW) ? pwd_at<NW, false>(u, i, g.ip, c, p[i]) : 0.f;
}

// One Gauss-Newton linearisation (dip3 :1645-1665 up to ps_divne's first
// normalisation, ps_divne :796-815): derivative filter, residual energy,
// mask, 1/hypot(den,1) scaling and sum of den^2.
template <int NW>
__global__ void k_prep(const float* __restrict__ u, const float* __restrict__ p,
                       float* __restrict__ u2, float* __restrict__ u1, float* __restrict__ p0,
                       const uint8_t* __restrict__ mask, Geo g, ApCoef c, DipScalars* S,
                       double* partials) {
  dvec<2> acc = {{0.0, 0.0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < g.n;
       i += (long)gridDim.x * blockDim.x) {
    float pi = p[i];
    float d = pwd_valid(g, i, NW) ? pwd_at<NW, true>(u, i, g.ip, c, pi) : 0.f;
    float r = u2[i];
    acc.v[0] += (double)r * (double)r;
    p0[i] = pi;
    if (mask && mask[i]) {
      d = 0.f;
      r = 0.f;
    }
    double nrm = 1.0 / hypot((double)d, 1.0);
    float num = __double2float_rn(__dmul_rn((double)r, nrm));
    float den = __double2float_rn(__dmul_rn((double)d, nrm));
    u2[i] = num;
    u1[i] = den;
    acc.v[1] += (double)den * (double)den;
  }
  dvec<2> tot;
  if (grid_sum_last<2>(acc, partials, &S->cnt[0], tot) && threadIdx.x == 0) {
    S->usum = tot.v[0];
    S->den2 = tot.v[1];
    S->zero = (tot.v[1] == 0.0);
    S->norm2 = S->zero ? 0.0 : sqrt((double)g.n / tot.v[1]);
    S->cg_done = S->zero;
    S->ls_done = 0;
    S->ls_trials = 0;
    S->cg_iters = 0;
  }
}

// ps_divne :817-826 second scaling, and ps_conjgrad :267-303 start.
__global__ void k_scale(float* __restrict__ num, float* __restrict__ den, float* __restrict__ r,
                        float* __restrict__ pcg, float* __restrict__ x, long n, DipScalars* S,
                        double* partials) {
  dvec<1> acc = {{0.0}};
  const bool zero = S->zero;
  const double nrm = S->norm2;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    x[i] = 0.f;
    if (zero) continue;
    float a = __double2float_rn(__dmul_rn((double)num[i], nrm));
    float b = __double2float_rn(__dmul_rn((double)den[i], nrm));
    num[i] = a;
    den[i] = b;
    float ri = -a;
    r[i] = ri;
    pcg[i] = 0.f;
    acc.v[0] += (double)ri * (double)ri;
  }
  dvec<1> tot;
  if (grid_sum_last<1>(acc, partials, &S->cnt[1], tot) && threadIdx.x == 0) {
    S->r0 = tot.v[0];
    if (!S->zero && tot.v[0] == 0.0) S->cg_done = 1;
  }
}

// gx = -eps*x + W' r with eps = 1 (ps_conjgrad :306-317); written to tmp.
__global__ void k_cg_grad(const float* __restrict__ x, const float* __restrict__ r,
                          const float* __restrict__ w, float* __restrict__ tmp, long n,
                          const DipScalars* S) {
  if (S->cg_done) return;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x)
    tmp[i] = __fadd_rn(-x[i], __fmul_rn(r[i], w[i]));
}

// gp = eps*p + S' gx; gn = gp.gp; convergence test (:319, :328-345).
__global__ void k_cg_gp(const float* __restrict__ pcg, float* __restrict__ tmp,
                        float* __restrict__ gp, long n, int iter, DipScalars* S,
                        double* partials) {
  if (S->cg_done) return;
  dvec<1> acc = {{0.0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    float v = __fadd_rn(pcg[i], tmp[i]);
    gp[i] = v;
    tmp[i] = v;
    acc.v[0] += (double)v * (double)v;
  }
  dvec<1> tot;
  if (grid_sum_last<1>(acc, partials, &S->cnt[2], tot) && threadIdx.x == 0) {
    double gn = tot.v[0];
    S->gn = gn;
    if (iter == 0) {
      S->g0 = gn;
    } else {
      double alpha = gn / S->gnp;
      double dg = gn / S->g0;
      S->alpha = alpha;
      const double tol = (double)1.e-6f;
      if (alpha < tol || dg < tol) S->cg_done = 1;
    }
  }
}

// gx = S gp (in tmp), gr = W gx, conjugate directions and beta (:320-359).
__global__ void k_cg_update(const float* __restrict__ gp, const float* __restrict__ tmp,
                            const float* __restrict__ w, float* __restrict__ sp,
                            float* __restrict__ sx, float* __restrict__ sr, long n, int iter,
                            DipScalars* S, double* partials) {
  if (S->cg_done) return;
  const float a = __double2float_rn(S->alpha);
  dvec<3> acc = {{0.0, 0.0, 0.0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    float gx = tmp[i];
    float gr = __fadd_rn(0.f, __fmul_rn(gx, w[i]));
    float vp = gp[i], vx = gx, vr = gr;
    if (iter > 0) {
      vp = __fadd_rn(vp, __fmul_rn(a, sp[i]));
      vx = __fadd_rn(vx, __fmul_rn(a, sx[i]));
      vr = __fadd_rn(vr, __fmul_rn(a, sr[i]));
    }
    sp[i] = vp;
    sx[i] = vx;
    sr[i] = vr;
    acc.v[0] += (double)vr * (double)vr;
    acc.v[1] += (double)vp * (double)vp;
    acc.v[2] += (double)vx * (double)vx;
  }
  dvec<3> tot;
  if (grid_sum_last<3>(acc, partials, &S->cnt[3], tot) && threadIdx.x == 0) {
    double beta = tot.v[0] + 1.0 * (tot.v[1] - tot.v[2]);
    S->step = -S->gn / beta;
    S->gnp = S->gn;
    S->cg_iters = iter + 1;
  }
}

// p += alpha sp; x += alpha sx; r += alpha sr (:364-368).
__global__ void k_cg_step(float* __restrict__ pcg, float* __restrict__ x, float* __restrict__ r,
                          const float* __restrict__ sp, const float* __restrict__ sx,
                          const float* __restrict__ sr, long n, const DipScalars* S) {
  if (S->cg_done) return;
  const float a = __double2float_rn(S->step);
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    pcg[i] = __fadd_rn(pcg[i], __fmul_rn(a, sp[i]));
    x[i] = __fadd_rn(x[i], __fmul_rn(a, sx[i]));
    r[i] = __fadd_rn(r[i], __fmul_rn(a, sr[i]));
  }
}

// Triangle smoothing of every line along one axis, in place
// (ps_smooth2 :616-625 = triple2 :564 + doubint2 :508 + fold2 :458), one
// thread per line with its running sums in a line-interleaved scratch.
struct TriAxis {
  int axis, len, nb;
  long nlines, stride;
  int n1, n2;
  float wt, w2;
};

__device__ __forceinline__ long tri_origin(const TriAxis& t, long line) {
  if (t.axis == 0) return line * t.n1;
  if (t.axis == 1) return (line % t.n1) + (line / t.n1) * (long)t.n1 * t.n2;
  return line;
}

__global__ void k_tri_line(float* __restrict__ x, float* __restrict__ scr, TriAxis t,
                           const DipScalars* S) {
  if (S && S->cg_done) return;
  long line = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (line >= t.nlines) return;
  const long o = tri_origin(t, line), d = t.stride, ss = t.nlines;
  const int L = t.len, nb = t.nb, np = L + 2 * nb;
  const float mw = -t.wt, w2 = t.w2;
  float* s = scr + line;
  float acc = 0.f;
  for (int m = 0; m < np; m++) {
    float v = 0.f;
    if (m < L) v = __fadd_rn(v, __fmul_rn(mw, x[o + m * d]));
    int q = m - nb;
    if (q >= 0 && q < L) v = __fadd_rn(v, __fmul_rn(w2, x[o + q * d]));
    q = m - 2 * nb;
    if (q >= 0 && q < L) v = __fadd_rn(v, __fmul_rn(mw, x[o + q * d]));
    acc = __fadd_rn(acc, v);
    s[m * ss] = acc;
  }
  acc = 0.f;
  for (int m = np - 1; m >= 0; m--) {
    acc = __fadd_rn(acc, s[m * ss]);
    s[m * ss] = acc;
  }
  int i, j;
  for (i = 0; i < L; i++) x[o + i * d] = s[(i + nb) * ss];
  for (j = nb + L; j < np; j += L) {
    for (i = 0; i < L && i < np - j; i++)
      x[o + (L - 1 - i) * d] = __fadd_rn(x[o + (L - 1 - i) * d], s[(j + i) * ss]);
    j += L;
    for (i = 0; i < L && i < np - j; i++) x[o + i * d] = __fadd_rn(x[o + i * d], s[(j + i) * ss]);
  }
  for (j = nb; j >= 0; j -= L) {
    for (i = 0; i < L && i < j; i++) x[o + i * d] = __fadd_rn(x[o + i * d], s[(j - 1 - i) * ss]);
    j -= L;
    for (i = 0; i < L && i < j; i++)
      x[o + (L - 1 - i) * d] = __fadd_rn(x[o + (L - 1 - i) * d], s[(j - 1 - i) * ss]);
  }
}

// One backtracking trial of dip3 :1666-1687: p = clip(p0 + lam*dp), new
// residual and its energy; accepted when it decreases.
template <int NW>
__global__ void k_ls_trial(const float* __restrict__ u, const float* __restrict__ p0,
                           const float* __restrict__ dp, float* __restrict__ p,
                           float* __restrict__ u2, Geo g, ApCoef c, int k, DipScalars* S,
                           double* partials) {
  if (S->ls_done) return;
  const float lam = ldexpf(1.0f, -k);
  const float pmin = -FLT_MAX, pmax = FLT_MAX;
  dvec<1> acc = {{0.0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < g.n;
       i += (long)gridDim.x * blockDim.x) {
    float pi = __fadd_rn(p0[i], __fmul_rn(lam, dp[i]));
    if (pi < pmin) pi = pmin;
    if (pi > pmax) pi = pmax;
    p[i] = pi;
    float r = pwd_valid(g, i, NW) ? pwd_at<NW, false>(u, i, g.ip, c, pi) : 0.f;
    u2[i] = r;
    acc.v[0] += (double)r * (double)r;
  }
  dvec<1> tot;
  if (grid_sum_last<1>(acc, partials, &S->cnt[4], tot) && threadIdx.x == 0) {
    S->usum2 = tot.v[0];
    S->ls_trials = k + 1;
    if (tot.v[0] < S->usum) S->ls_done = 1;
  }
}

// mask32 (dip_cfuns.c:914-997, both=false, nj=1): flags samples whose PWD
// stencil touches a zero of the mask data.
__global__ void k_mask32(const float* __restrict__ yy, uint8_t* __restrict__ m0,
                         uint8_t* __restrict__ m1, int n1, int n2, int n3, int nw) {
  long n = (long)n1 * n2 * n3;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    int ix = (int)(i % n1);
    long r = i / n1;
    int iy = (int)(r % n2), iz = (int)(r / n2);
    bool a = false, b = false;
    if (ix >= nw && ix < n1 - nw) {
      if (iy < n2 - 1)
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          a = a || (yy[i - is] == 0.f) || (yy[i + n1 + is] == 0.f);
        }
      if (iz < n3 - 1)
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          b = b || (yy[i - is] == 0.f) || (yy[i + (long)n1 * n2 + is] == 0.f);
        }
    }
    m0[i] = a;
    m1[i] = b;
  }
}

struct DipWork {
  float *u1, *u2, *dp, *p0, *pcg, *r, *gp, *tmp, *sp, *sx, *sr, *tri;
  uint8_t *m0, *m1;
  DipScalars* S;
  double* partials;
};

long tri_scratch_elems(int n1, int n2, int n3, const int rect[3]) {
  long n = (long)n1 * n2 * n3, best = 0;
  const int len[3] = {n1, n2, n3};
  for (int a = 0; a < 3; a++)
    if (rect[a] > 1) {
      long nl = n / len[a];
      long e = nl * (len[a] + 2L * rect[a]);
      if (e > best) best = e;
    }
  return best > 0 ? best : 1;
}

DipWork carve_dip(void* ws, int n1, int n2, int n3, const int rect[3], int has_mask,
                  size_t* total) {
  long n = (long)n1 * n2 * n3;
  Carver cv(ws);
  DipWork w;
  w.u1 = cv.take<float>(n);
  w.u2 = cv.take<float>(n);
  w.dp = cv.take<float>(n);
  w.p0 = cv.take<float>(n);
  w.pcg = cv.take<float>(n);
  w.r = cv.take<float>(n);
  w.gp = cv.take<float>(n);
  w.tmp = cv.take<float>(n);
  w.sp = cv.take<float>(n);
  w.sx = cv.take<float>(n);
  w.sr = cv.take<float>(n);
  w.tri = cv.take<float>(tri_scratch_elems(n1, n2, n3, rect));
  w.m0 = has_mask ? cv.take<uint8_t>(n) : nullptr;
  w.m1 = has_mask ? cv.take<uint8_t>(n) : nullptr;
  w.S = cv.take<DipScalars>(1);
  w.partials = cv.take<double>(4 * (size_t)kRedGridMax);
  *total = cv.size();
  return w;
}

template <int NW>
int dip3_run(const float* u, float* p, const uint8_t* mask, int dip, int n1, int n2, int n3,
             int niter, int liter, const int rect[3], const DipWork& w, cudaStream_t st) {
  Geo g;
  g.n1 = n1;
  g.n2 = n2;
  g.n3 = n3;
  g.n = (long)n1 * n2 * n3;
  g.dip = dip;
  g.ip = dip == 1 ? n1 : (long)n1 * n2;
  const ApCoef c = make_apcoef(NW);
  const int gr = red_grid(g.n);
  const int ge = (int)std::min<long>((g.n + kBlock - 1) / kBlock, 65535L * 8);

  TriAxis ax[3];
  int nax = 0;
  const int len[3] = {n1, n2, n3};
  const long str[3] = {1, n1, (long)n1 * n2};
  for (int a = 0; a < 3; a++) {
    if (rect[a] <= 1) continue;
    TriAxis t;
    t.axis = a;
    t.len = len[a];
    t.nb = rect[a];
    t.nlines = g.n / len[a];
    t.stride = str[a];
    t.n1 = n1;
    t.n2 = n2;
    t.wt = (float)(1.0 / (rect[a] * rect[a]));
    t.w2 = (float)(2. * t.wt);
    ax[nax++] = t;
  }
  auto sweeps = [&]() {
    for (int a = 0; a < nax; a++) {
      int gl = (int)((ax[a].nlines + 127) / 128);
      k_tri_line<<<gl, 128, 0, st>>>(w.tmp, w.tri, ax[a], w.S);
    }
  };

  k_residual<NW><<<ge, kBlock, 0, st>>>(u, p, w.u2, g, c);
  for (int iter = 0; iter < niter; iter++) {
    k_prep<NW><<<gr, kRedBlock, 0, st>>>(u, p, w.u2, w.u1, w.p0, mask, g, c, w.S, w.partials);
    k_scale<<<gr, kRedBlock, 0, st>>>(w.u2, w.u1, w.r, w.pcg, w.dp, g.n, w.S, w.partials);
    for (int it = 0; it < liter; it++) {
      k_cg_grad<<<ge, kBlock, 0, st>>>(w.dp, w.r, w.u1, w.tmp, g.n, w.S);
      sweeps();
      k_cg_gp<<<gr, kRedBlock, 0, st>>>(w.pcg, w.tmp, w.gp, g.n, it, w.S, w.partials);
      sweeps();
      k_cg_update<<<gr, kRedBlock, 0, st>>>(w.gp, w.tmp, w.u1, w.sp, w.sx, w.sr, g.n, it, w.S,
                                            w.partials);
      k_cg_step<<<ge, kBlock, 0, st>>>(w.pcg, w.dp, w.r, w.sp, w.sx, w.sr, g.n, w.S);
    }
    for (int k = 0; k < 8; k++)
      k_ls_trial<NW><<<gr, kRedBlock, 0, st>>>(u, w.p0, w.dp, p, w.u2, g, c, k, w.S, w.partials);
  }
  PWD_LAUNCH_CHECK();
  return PWD_OK;
}

int dip_dispatch(int order, const float* u, float* p, const uint8_t* mask, int dip, int n1,
                 int n2, int n3, int niter, int liter, const int rect[3], const DipWork& w,
                 cudaStream_t st) {
  switch (order) {
    case 1: return dip3_run<1>(u, p, mask, dip, n1, n2, n3, niter, liter, rect, w, st);
    case 2: return dip3_run<2>(u, p, mask, dip, n1, n2, n3, niter, liter, rect, w, st);
    case 3: return dip3_run<3>(u, p, mask, dip, n1, n2, n3, niter, liter, rect, w, st);
    case 4: return dip3_run<4>(u, p, mask, dip, n1, n2, n3, niter, liter, rect, w, st);
  }
  return PWD_ENOTSUP;
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_dip_workspace_size(int n1, int n2, int n3, int order, const int rect[3],
                                         int has_mask) {
  (void)order;
  if (n1 < 1 || n2 < 1 || n3 < 1 || !rect) return 0;
  size_t total = 0;
  carve_dip(nullptr, n1, n2, n3, rect, has_mask, &total);
  return total;
}

extern "C" int pwd_dip(const float* data, const float* mask, float* dip_out, int n1, int n2,
                       int n3, int niter, int liter, int order, const int rect[3],
                       void* workspace, size_t workspace_bytes, pwd_stream_t stream) {
  if (!data || !dip_out || !rect || n1 < 1 || n2 < 1 || n3 < 1 || niter < 0 || liter < 0 ||
      order < 1)
    return PWD_EINVAL;
  for (int a = 0; a < 3; a++)
    if (rect[a] < 0) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  if (2 * order >= n1) return PWD_EINVAL;
  size_t need = 0;
  carve_dip(nullptr, n1, n2, n3, rect, mask != nullptr, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  DipWork w = carve_dip(workspace, n1, n2, n3, rect, mask != nullptr, &need);
  cudaStream_t st = (cudaStream_t)stream;
  const long n = (long)n1 * n2 * n3;
  const bool three = n3 > 1;
  if (cudaMemsetAsync(dip_out, 0, sizeof(float) * n * (three ? 2 : 1), st) != cudaSuccess)
    return PWD_ECUDA;
  if (cudaMemsetAsync(w.S, 0, sizeof(DipScalars), st) != cudaSuccess) return PWD_ECUDA;
  if (mask) {
    int gb = (int)std::min<long>((n + 255) / 256, 65535L * 8);
    k_mask32<<<gb, 256, 0, st>>>(mask, w.m0, w.m1, n1, n2, n3, order);
  }
  int rc = dip_dispatch(order, data, dip_out, w.m0, 1, n1, n2, n3, niter, liter, rect, w, st);
  if (rc != PWD_OK) return rc;
  if (three)
    rc = dip_dispatch(order, data, dip_out + n, w.m1, 2, n1, n2, n3, niter, liter, rect, w, st);
  return rc;
}
