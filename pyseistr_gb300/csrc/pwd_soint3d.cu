// 3-D structure-oriented interpolation: PWD-regularised conjugate gradients.
//
// Restates csoint3d (pyseistr/src/soint3d_cfuns.c:2405-2507): the stacked
// inline/crossline PWD operator allpass3_lop (:625-730) inside ps_solver
// (:894-1175) with the "known" model mask and x0, stepped by ps_cgstep
// (:826-877).  The filter coefficients depend only on the slopes, so they
// are evaluated once per call; the adjoint is computed as a gather that adds
// the contributions to each model sample in the reference's scatter order.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pwd_common.cuh"

namespace pwd {
namespace {

struct Op3 {
  int nx, ny, nz, nw, nj1, nj2;
  long n;
  int drift;
};

struct Coef3 {
  float* f1;    // [na][n] part-1 (inline) taps, 0 where the row is skipped
  float* f2;    // [na][n] part-2 (crossline) taps
  int* id1;     // drift shifts (0 without drift)
  int* id2;
  uint8_t* v1;  // row valid flags
  uint8_t* v2;
};

__device__ __forceinline__ int ps_nint(float x) {
  return (int)(x > 0.0 ? (double)x + 0.5 : (double)x - 0.5);
}

template <int NW>
__global__ void k_ap3_coef(const float* __restrict__ pp, const float* __restrict__ qq, Op3 g,
                           ApCoef c, Coef3 cf) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  const int ix = (int)(i % g.nx);
  const long r = i / g.nx;
  const int iy = (int)(r % g.ny), iz = (int)(r / g.ny);
  for (int part = 0; part < 2; part++) {
    const float* p = part == 0 ? pp : qq;
    const int nj = part == 0 ? g.nj1 : g.nj2;
    bool ok = ix >= NW * nj && ix < g.nx - NW * nj && (part == 0 ? iy < g.ny - 1 : iz < g.nz - 1);
    int id = 0;
    float pi = p[i];
    if (ok && g.drift) {
      // a shift of a trace length or more (or a non-finite slope) always
      // fails the reference's range test; test it before converting
      if (!(fabsf(p[i]) < (float)g.nx)) {
        ok = false;
      } else {
        id = ps_nint(p[i]);
        if (ix - NW * nj - id < 0 || ix + NW * nj - id >= g.nx) ok = false;
        pi = __fsub_rn(p[i], (float)id);
      }
      if (!ok) id = 0;
    }
    float f[2 * NW + 1];
    if (ok) passfilter<NW>(c, pi, f);
    float* dst = part == 0 ? cf.f1 : cf.f2;
    for (int iw = 0; iw <= 2 * NW; iw++) dst[iw * g.n + i] = ok ? f[iw] : 0.f;
    (part == 0 ? cf.id1 : cf.id2)[i] = id;
    (part == 0 ? cf.v1 : cf.v2)[i] = ok;
  }
}

// yy (+)= L xx, yy = [inline residual ; crossline residual].
template <int NW>
__global__ void k_ap3_fwd(const float* __restrict__ xx, float* __restrict__ yy, Op3 g, Coef3 cf,
                          int add, const int* done) {
  if (done && *done) return;
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= g.n) return;
  for (int part = 0; part < 2; part++) {
    float* y = yy + (part == 0 ? 0 : g.n);
    float acc = add ? y[i] : 0.f;
    const uint8_t ok = (part == 0 ? cf.v1 : cf.v2)[i];
    if (ok) {
      const long st = part == 0 ? g.nx : (long)g.nx * g.ny;
      const int nj = part == 0 ? g.nj1 : g.nj2;
      const int id = (part == 0 ? cf.id1 : cf.id2)[i];
      const float* f = part == 0 ? cf.f1 : cf.f2;
#pragma unroll
      for (int iw = 0; iw <= 2 * NW; iw++) {
        int is = (iw - NW) * nj;
        acc = __fadd_rn(acc, __fmul_rn(__fsub_rn(xx[i + st + is], xx[i - is - id]), f[iw * g.n + i]));
      }
    }
    y[i] = acc;
  }
}

// xx = L' yy as a gather: for model sample m, the "+" terms come from rows
// i = m - st - is and the "-" terms from rows i with i - is - id_i = m, all
// added in the reference's scatter order (row i ascending, iw ascending,
// "+" before "-"), part 1 before part 2.
template <int NW>
__device__ __forceinline__ float ap3_adj_part(const float* __restrict__ y, long m, long st, int nj,
                                              const float* __restrict__ f,
                                              const int* __restrict__ idv,
                                              const uint8_t* __restrict__ v, long n, int drift,
                                              int dmax, float acc) {
  constexpr int NA = 2 * NW + 1;
  // "+" list: iw = NA-1 .. 0 gives ascending rows
  long ip[NA];
  int wp[NA];
  int np_ = 0;
  for (int iw = NA - 1; iw >= 0; iw--) {
    long i = m - st - (long)(iw - NW) * nj;
    if (i >= 0 && i < n && v[i]) {
      ip[np_] = i;
      wp[np_] = iw;
      np_++;
    }
  }
  int a = 0;
  auto emit_plus_upto = [&](long ilim, int iwlim, bool strict) {
    while (a < np_ && (ip[a] < ilim || (ip[a] == ilim && (strict ? wp[a] <= iwlim : false)))) {
      acc = __fadd_rn(acc, __fmul_rn(y[ip[a]], f[wp[a] * n + ip[a]]));
      a++;
    }
  };
  if (!drift) {
    for (int iw = 0; iw < NA; iw++) {
      long i = m + (long)(iw - NW) * nj;
      if (i < 0 || i >= n || !v[i]) continue;
      emit_plus_upto(i, iw, true);
      acc = __fsub_rn(acc, __fmul_rn(y[i], f[iw * n + i]));
    }
  } else {
    const long lo = m - (long)NW * nj - dmax, hi = m + (long)NW * nj + dmax;
    for (long i = lo; i <= hi; i++) {
      if (i < 0 || i >= n || !v[i]) continue;
      long q = i - m - idv[i];
      if (q % nj) continue;
      long iw = q / nj + NW;
      if (iw < 0 || iw >= NA) continue;
      emit_plus_upto(i, (int)iw, true);
      acc = __fsub_rn(acc, __fmul_rn(y[i], f[iw * n + i]));
    }
  }
  emit_plus_upto(n, 0, false);
  return acc;
}

template <int NW>
__global__ void k_ap3_adj(float* __restrict__ xx, const float* __restrict__ yy, Op3 g, Coef3 cf,
                          const uint8_t* __restrict__ known, const int* dmax, const int* done,
                          double* partials, unsigned* counter, double* out_sum) {
  if (done && *done) return;
  dvec<1> acc = {{0.0}};
  const int dm = g.drift ? *dmax : 0;
  for (long m = blockIdx.x * (long)blockDim.x + threadIdx.x; m < g.n;
       m += (long)gridDim.x * blockDim.x) {
    float a = 0.f;
    a = ap3_adj_part<NW>(yy, m, g.nx, g.nj1, cf.f1, cf.id1, cf.v1, g.n, g.drift, dm, a);
    a = ap3_adj_part<NW>(yy + g.n, m, (long)g.nx * g.ny, g.nj2, cf.f2, cf.id2, cf.v2, g.n,
                         g.drift, dm, a);
    if (known && known[m]) a = 0.f;
    xx[m] = a;
    acc.v[0] += (double)a * (double)a;
  }
  if (partials) {
    dvec<1> tot;
    if (grid_sum_last<1>(acc, partials, counter, tot) && threadIdx.x == 0) *out_sum = tot.v[0];
  }
}

__global__ void k_max_shift(const int* __restrict__ id1, const int* __restrict__ id2, long n,
                            int* dmax) {
  int best = 0;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < n;
       i += (long)gridDim.x * blockDim.x) {
    best = max(best, abs(id1[i]));
    best = max(best, abs(id2[i]));
  }
  atomicMax(dmax, best);
}

struct SolveScalars {
  double rr0, gsum, g0;
  double dots[6];  // gg.gg, Ss.Ss, gg.Ss, gg.rr, Ss.rr, rr.rr
  float alfa, beta;
  int done, skip, dmax;
  unsigned cnt[4];
};

// gg.gg, Ss.Ss, gg.Ss, gg.rr, Ss.rr, rr.rr over the 2n data space; the last
// block runs the tolerance test of ps_solver (:1086-1100) and ps_cgstep's
// scalar part (:835-866).
__global__ void k_cg3_dots(const float* __restrict__ gg, const float* __restrict__ Ss,
                           const float* __restrict__ rr, long ny, int iter, SolveScalars* S,
                           double* partials) {
  if (S->done) return;
  dvec<6> acc = {{0, 0, 0, 0, 0, 0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ny;
       i += (long)gridDim.x * blockDim.x) {
    double a = gg[i], s = Ss[i], r = rr[i];
    acc.v[0] += a * a;
    acc.v[1] += s * s;
    acc.v[2] += a * s;
    acc.v[3] += a * r;
    acc.v[4] += s * r;
    acc.v[5] += r * r;
  }
  dvec<6> t;
  if (!(grid_sum_last<6>(acc, partials, &S->cnt[1], t) && threadIdx.x == 0)) return;
  const float TOL = 1.e-12f, EPS = 1.e-12f;
  float dpr, dpg;
  if (iter == 0) {
    S->g0 = S->gsum;
    dpr = 1.f;
    dpg = 1.f;
  } else {
    dpr = __fdiv_rn((float)t.v[5], (float)S->rr0);
    dpg = __fdiv_rn((float)S->gsum, (float)S->g0);
  }
  if (dpr < TOL || dpg < TOL) {
    S->done = 1;
    return;
  }
  double alfa, beta;
  S->skip = 0;
  if (iter == 0) {  // the first step of a run restarts (forget)
    beta = 0.0;
    alfa = t.v[0];
    if (alfa <= 0.) {
      S->skip = 1;
      return;
    }
    alfa = -t.v[3] / alfa;
  } else {
    double gdg = t.v[0], sds = t.v[1], gds = t.v[2];
    if (gdg == 0. || sds == 0.) {
      S->skip = 1;
      return;
    }
    double determ = 1.0 - (gds / gdg) * (gds / sds);
    if (determ > (double)EPS)
      determ *= gdg * sds;
    else
      determ = gdg * sds * (double)EPS;
    double gdr = -t.v[3], sdr = -t.v[4];
    alfa = (sds * gdr - gds * sdr) / determ;
    beta = (-gds * gdr + gdg * sdr) / determ;
  }
  S->alfa = __double2float_rn(alfa);
  S->beta = __double2float_rn(beta);
}

__global__ void k_cg3_update(float* __restrict__ x, float* __restrict__ S_, const float* __restrict__ g,
                             float* __restrict__ rr, float* __restrict__ Ss,
                             const float* __restrict__ gg, long nx, int iter, SolveScalars* S) {
  if (S->done || S->skip) return;
  const float a = S->alfa, b = S->beta;
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < 2 * nx;
       i += (long)gridDim.x * blockDim.x) {
    if (i < nx) {
      float s = iter == 0 ? 0.f : S_[i];
      s = __fadd_rn(__fmul_rn(s, b), __fmul_rn(a, g[i]));
      S_[i] = s;
      x[i] = __fadd_rn(x[i], s);
    }
    float s2 = iter == 0 ? 0.f : Ss[i];
    s2 = __fadd_rn(__fmul_rn(s2, b), __fmul_rn(a, gg[i]));
    Ss[i] = s2;
    rr[i] = __fadd_rn(rr[i], s2);
  }
}

// rr = -dd; dd = a*randn (zero without noise)
__global__ void k_init_rr(float* __restrict__ rr, const float* __restrict__ dd, long ny) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < ny) rr[i] = dd ? -dd[i] : -0.0f;
}

__global__ void k_init_x(const float* __restrict__ din, const float* __restrict__ mask,
                         float* __restrict__ x, uint8_t* __restrict__ known, long n, int hasmask) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] = din[i];
  known[i] = hasmask == 1 ? (mask[i] != 0.f) : (din[i] != 0.f);
}

__global__ void k_rr0(const float* __restrict__ rr, long ny, SolveScalars* S, double* partials) {
  dvec<1> acc = {{0.0}};
  for (long i = blockIdx.x * (long)blockDim.x + threadIdx.x; i < ny;
       i += (long)gridDim.x * blockDim.x)
    acc.v[0] += (double)rr[i] * (double)rr[i];
  dvec<1> t;
  if (grid_sum_last<1>(acc, partials, &S->cnt[2], t) && threadIdx.x == 0) S->rr0 = t.v[0];
}

struct Soint3Work {
  float *g, *rr, *gg, *S, *Ss, *dd, *f1, *f2;
  int *id1, *id2;
  uint8_t *v1, *v2, *known;
  SolveScalars* sc;
  double* partials;
};

Soint3Work carve_soint3(void* ws, long n, int order, bool noise, size_t* total) {
  const int na = 2 * order + 1;
  Carver cv(ws);
  Soint3Work w;
  w.g = cv.take<float>(n);
  w.rr = cv.take<float>(2 * n);
  w.gg = cv.take<float>(2 * n);
  w.S = cv.take<float>(n);
  w.Ss = cv.take<float>(2 * n);
  w.dd = noise ? cv.take<float>(2 * n) : nullptr;
  w.f1 = cv.take<float>(na * n);
  w.f2 = cv.take<float>(na * n);
  w.id1 = cv.take<int>(n);
  w.id2 = cv.take<int>(n);
  w.v1 = cv.take<uint8_t>(n);
  w.v2 = cv.take<uint8_t>(n);
  w.known = cv.take<uint8_t>(n);
  w.sc = cv.take<SolveScalars>(1);
  w.partials = cv.take<double>(6 * (size_t)kRedGridMax);
  *total = cv.size();
  return w;
}

// MT19937 (Matsumoto & Nishimura 1998) and the Box-Muller pairs of
// ps_randn_one_bm (:2303-2400), for the optional noise term.
struct Mt {
  uint32_t mt[624];
  int mti;
  explicit Mt(uint32_t s) {
    mt[0] = s;
    for (mti = 1; mti < 624; mti++)
      mt[mti] = 1812433253u * (mt[mti - 1] ^ (mt[mti - 1] >> 30)) + (uint32_t)mti;
  }
  uint32_t next() {
    static const uint32_t mag01[2] = {0u, 0x9908b0dfu};
    uint32_t y;
    if (mti >= 624) {
      int kk;
      for (kk = 0; kk < 624 - 397; kk++) {
        y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + 397] ^ (y >> 1) ^ mag01[y & 1u];
      }
      for (; kk < 623; kk++) {
        y = (mt[kk] & 0x80000000u) | (mt[kk + 1] & 0x7fffffffu);
        mt[kk] = mt[kk + (397 - 624)] ^ (y >> 1) ^ mag01[y & 1u];
      }
      y = (mt[623] & 0x80000000u) | (mt[0] & 0x7fffffffu);
      mt[623] = mt[396] ^ (y >> 1) ^ mag01[y & 1u];
      mti = 0;
    }
    y = mt[mti++];
    y ^= (y >> 11);
    y ^= (y << 7) & 0x9d2c5680u;
    y ^= (y << 15) & 0xefc60000u;
    y ^= (y >> 18);
    return y;
  }
  double real1() { return next() * (1.0 / 4294967295.0); }
};

void make_noise(std::vector<float>& dd, int seed, float var) {
  Mt g((uint32_t)seed);
  const float a = sqrtf(var);
  bool iset = true;
  float vset = 0.f;
  for (size_t i = 0; i < dd.size(); i++) {
    float r;
    if (iset) {
      double x1, x2;
      do {
        x1 = g.real1();
      } while (x1 == 0.0);
      x2 = g.real1();
      double z1 = sqrt(-2.0 * log(x1));
      double z2 = 2.0 * 3.14159265358979323846264338328 * x2;
      vset = (float)(z1 * cos(z2));
      r = (float)(z1 * sin(z2));
      iset = false;
    } else {
      r = vset;
      iset = true;
    }
    dd[i] = a * r;
  }
}

template <int NW>
int soint3_run(const float* data, const float* mask, const float* pp, const float* qq, float* x,
               Op3 g, int niter, int seed, int hasmask, float var, const Soint3Work& w,
               cudaStream_t st) {
  const long n = g.n, ny = 2 * n;
  const int b = 256;
  const unsigned gn = (unsigned)((n + b - 1) / b), g2 = (unsigned)((ny + b - 1) / b);
  const int gr = red_grid(n), gr2 = red_grid(ny);
  Coef3 cf{w.f1, w.f2, w.id1, w.id2, w.v1, w.v2};
  if (cudaMemsetAsync(w.sc, 0, sizeof(SolveScalars), st) != cudaSuccess) return PWD_ECUDA;
  // ps_cgstep's restart zeroes the step vectors (:838-839)
  if (cudaMemsetAsync(w.S, 0, sizeof(float) * n, st) != cudaSuccess) return PWD_ECUDA;
  if (cudaMemsetAsync(w.Ss, 0, sizeof(float) * ny, st) != cudaSuccess) return PWD_ECUDA;
  PWD_KERNEL(PWD_FAM_SOINT, st, k_ap3_coef<NW><<<gn, b, 0, st>>>(pp, qq, g, make_apcoef(NW), cf));
  if (g.drift) PWD_KERNEL(PWD_FAM_SOINT, st, k_max_shift<<<gr, kRedBlock, 0, st>>>(w.id1, w.id2, n, &w.sc->dmax));
  PWD_KERNEL(PWD_FAM_SOINT, st, k_init_x<<<gn, b, 0, st>>>(data, mask, x, w.known, n, hasmask));
  if (var != 0.f) {
    std::vector<float> dd((size_t)ny);
    make_noise(dd, seed, var);
    if (cudaMemcpyAsync(w.dd, dd.data(), sizeof(float) * ny, cudaMemcpyHostToDevice, st) !=
        cudaSuccess)
      return PWD_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PWD_ECUDA;
  }
  PWD_KERNEL(PWD_FAM_SOINT, st, k_init_rr<<<g2, b, 0, st>>>(w.rr, var != 0.f ? w.dd : nullptr, ny));
  PWD_KERNEL(PWD_FAM_SOINT, st, k_ap3_fwd<NW><<<gn, b, 0, st>>>(x, w.rr, g, cf, 1, nullptr));
  PWD_KERNEL(PWD_FAM_SOINT, st, k_rr0<<<gr2, kRedBlock, 0, st>>>(w.rr, ny, w.sc, w.partials));
  for (int iter = 0; iter < niter; iter++) {
    PWD_KERNEL(PWD_FAM_SOINT, st, k_ap3_adj<NW><<<gr, kRedBlock, 0, st>>>(w.g, w.rr, g, cf, w.known, &w.sc->dmax, &w.sc->done,
                                            w.partials, &w.sc->cnt[0], &w.sc->gsum));
    PWD_KERNEL(PWD_FAM_SOINT, st, k_ap3_fwd<NW><<<gn, b, 0, st>>>(w.g, w.gg, g, cf, 0, &w.sc->done));
    PWD_KERNEL(PWD_FAM_SOINT, st, k_cg3_dots<<<gr2, kRedBlock, 0, st>>>(w.gg, w.Ss, w.rr, ny, iter, w.sc, w.partials));
    PWD_KERNEL(PWD_FAM_SOINT, st, k_cg3_update<<<g2, b, 0, st>>>(x, w.S, w.g, w.rr, w.Ss, w.gg, n, iter, w.sc));
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_soint3d_workspace_size(int n1, int n2, int n3, int order) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || order < 1 || order > PWD_MAX_ORDER) return 0;
  size_t t = 0;
  carve_soint3(nullptr, (long)n1 * n2 * n3, order, true, &t);
  return t;
}

extern "C" int pwd_soint3d(const float* data, const float* mask, const float* dip_inline,
                           const float* dip_xline, float* out, int n1, int n2, int n3, int order,
                           int nj1, int nj2, int niter, int drift, int seed, int hasmask,
                           float var, void* workspace, size_t workspace_bytes,
                           pwd_stream_t stream) {
  if (!data || !dip_inline || !dip_xline || !out || n1 < 1 || n2 < 1 || n3 < 1 || order < 1 ||
      nj1 < 1 || nj2 < 1 || niter < 0 || var < 0.f)
    return PWD_EINVAL;
  if (hasmask == 1 && !mask) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  const long n = (long)n1 * n2 * n3;
  size_t need = 0;
  carve_soint3(nullptr, n, order, true, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  Soint3Work w = carve_soint3(workspace, n, order, true, &need);
  Op3 g;
  g.nx = n1; g.ny = n2; g.nz = n3; g.nw = order; g.nj1 = nj1; g.nj2 = nj2; g.n = n;
  g.drift = drift != 0;
  cudaStream_t st = (cudaStream_t)stream;
  switch (order) {
    case 1: return soint3_run<1>(data, mask, dip_inline, dip_xline, out, g, niter, seed, hasmask, var, w, st);
    case 2: return soint3_run<2>(data, mask, dip_inline, dip_xline, out, g, niter, seed, hasmask, var, w, st);
    case 3: return soint3_run<3>(data, mask, dip_inline, dip_xline, out, g, niter, seed, hasmask, var, w, st);
    case 4: return soint3_run<4>(data, mask, dip_inline, dip_xline, out, g, niter, seed, hasmask, var, w, st);
  }
  return PWD_ENOTSUP;
}
