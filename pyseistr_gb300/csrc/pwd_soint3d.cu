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

#include "pwd_batch.cuh"
#include "pwd_common.cuh"

namespace pwd {
namespace {

// Geometry of one patch (section) of the batch.
struct Op3 {
  int nx, ny, nz, nw, nj1, nj2;
  long n;
  int drift;
};

// Per-section solver state.
struct SolveScalars {
  double rr0, gsum, g0;
  float alfa, beta;
  int done, skip, dmax;
  unsigned cnt[4];
};

constexpr int kTile = 8192;  // model samples per tile; tiles never straddle patches
constexpr int kTileThreads = 256;

// The batch: patches packed in data/mask/out at SecDesc::off (n each) and
// their slopes at SecDesc::pout (inline n, then crossline n, the layout of
// pwd_dip_batch's output).  Data-space vectors (2n per patch) live at 2*off,
// filter taps ([na][n] per part) at na*off.
struct SoBatch {
  const SecDesc* secs;
  const int* tile_sec;
  int nsec, ntiles, nw, nj1, nj2, drift, hasmask;
  int xl_after;  // crossline slopes at pp + pout + n (batch layout) instead of qq + pout
  SolveScalars* S;
  double* partials;  // [ntiles][6]
};

struct SoArrays {
  const float *data, *mask, *pp, *qq, *dd;
  float *x, *g, *S, *rr, *gg, *Ss, *f1, *f2;
  int *id1, *id2;
  uint8_t *v1, *v2, *known;
};

struct TileRange {
  int sec;
  long lo, hi;
};
__device__ __forceinline__ TileRange tile_range(const SoBatch& b, int t) {
  TileRange r;
  r.sec = b.tile_sec[t];
  const SecDesc& s = b.secs[r.sec];
  r.lo = (long)(t - s.tile0) * kTile;
  r.hi = min(s.n, r.lo + kTile);
  return r;
}

__device__ __forceinline__ Op3 geometry(const SoBatch& b, const SecDesc& s) {
  Op3 g;
  g.nx = s.n1;
  g.ny = s.n2;
  g.nz = s.n3;
  g.nw = b.nw;
  g.nj1 = b.nj1;
  g.nj2 = b.nj2;
  g.n = s.n;
  g.drift = b.drift;
  return g;
}

// Sum of K doubles over the tiles of one section; true in the block of the
// section's last tile to finish, which receives the totals.
template <int K>
__device__ __forceinline__ bool so_sum_last(dvec<K> x, const SoBatch& b, int t, const SecDesc& s,
                                            unsigned* counter, dvec<K>& tot) {
  __shared__ bool s_last;
  dvec<K> blk = block_sum<K>(x);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) b.partials[(size_t)t * 6 + k] = blk.v[k];
    __threadfence();
    unsigned tk = atomicAdd(counter, 1u);
    s_last = (tk == (unsigned)(s.ntile - 1));
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  dvec<K> y;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double v = 0.0;
    for (int i = threadIdx.x; i < s.ntile; i += blockDim.x)
      v += __ldcg(b.partials + (size_t)(s.tile0 + i) * 6 + k);
    y.v[k] = v;
  }
  tot = block_sum<K>(y);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

__device__ __forceinline__ int ps_nint(float x) {
  return (int)(x > 0.0 ? (double)x + 0.5 : (double)x - 0.5);
}

// allpass3_init's filters (soint3d_cfuns.c:625-660): taps, drift shifts and
// row validity of both parts, once per call.
template <int NW>
__global__ void k_ap3_coef(SoArrays A, SoBatch b, ApCoef c) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const Op3 g = geometry(b, s);
  constexpr int NA = 2 * NW + 1;
  const float* pp = A.pp + s.pout;
  const float* qq = b.xl_after ? pp + s.n : A.qq + s.pout;
  float *f1 = A.f1 + NA * s.off, *f2 = A.f2 + NA * s.off;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
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
      float f[NA];
      if (ok) passfilter<NW>(c, pi, f);
      float* dst = part == 0 ? f1 : f2;
      for (int iw = 0; iw < NA; iw++) dst[iw * g.n + i] = ok ? f[iw] : 0.f;
      (part == 0 ? A.id1 : A.id2)[s.off + i] = id;
      (part == 0 ? A.v1 : A.v2)[s.off + i] = ok;
    }
  }
}

__device__ void cg3_scalars(SolveScalars* S, const dvec<6>& tt, int iter);

// yy (+)= L xx, yy = [inline residual ; crossline residual] (allpass3_lop
// forward, :662-695).  With DOTS (yy = gg = L g inside the CG loop) the
// kernel also accumulates gg.gg, Ss.Ss, gg.Ss, gg.rr, Ss.rr, rr.rr over the
// patch's 2n data space, and the last tile of the patch runs the tolerance
// test of ps_solver (:1086-1100) and ps_cgstep's scalar part (:835-866).
// The dot products are float-float per thread (exact products, ~2^-45 sums),
// double across threads and tiles: no per-sample FP64 arithmetic.
template <int NW, bool DOTS>
__global__ void __launch_bounds__(kTileThreads, 4) k_ap3_fwd(const float* __restrict__ xxb,
                                                          float* __restrict__ yyb, SoArrays A,
                                                          SoBatch b, int add, int use_done,
                                                          int iter) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  if (use_done && b.S[tr.sec].done) return;
  const Op3 g = geometry(b, s);
  constexpr int NA = 2 * NW + 1;
  const float* xx = xxb + s.off;
  float* yy = yyb + 2 * s.off;
  ffacc c0, c1, c2, c3, c4, c5;
  const float *Ssv = A.Ss + 2 * s.off, *rrv = A.rr + 2 * s.off;
  // 32-bit indices within the patch (fewer than 2^31 samples)
  const int n = (int)g.n, hi = (int)tr.hi;
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x) {
    float yo[2];
#pragma unroll 1
    for (int part = 0; part < 2; part++) {
      float* y = yy + (part == 0 ? 0 : n);
      float acc = add ? y[i] : 0.f;
      const uint8_t ok = (part == 0 ? A.v1 : A.v2)[s.off + i];
      const int st = part == 0 ? g.nx : g.nx * g.ny;
      const int nj = part == 0 ? g.nj1 : g.nj2;
      // the shifts are all 0 without drift
      const int id = g.drift ? (part == 0 ? A.id1 : A.id2)[s.off + i] : 0;
      const float* f = (part == 0 ? A.f1 : A.f2) + NA * s.off;
      // operands loaded before the row's validity is known (indices clamped
      // into the patch; a valid row's are in range), added only if valid
      float xa[NA], xb[NA], fv[NA];
#pragma unroll
      for (int iw = 0; iw < NA; iw++) {
        const int is = (iw - NW) * nj;
        const int ia = i + st + is, ib = i - is - id;
        xa[iw] = xx[ia < 0 ? 0 : (ia >= n ? n - 1 : ia)];
        xb[iw] = xx[ib < 0 ? 0 : (ib >= n ? n - 1 : ib)];
        fv[iw] = f[(long)iw * n + i];
      }
      if (ok) {
#pragma unroll
        for (int iw = 0; iw < NA; iw++)
          acc = __fadd_rn(acc, __fmul_rn(__fsub_rn(xa[iw], xb[iw]), fv[iw]));
      }
      y[i] = acc;
      yo[part] = acc;
    }
    if (DOTS) {
#pragma unroll
      for (int part = 0; part < 2; part++) {
        const int k = i + part * n;
        const float a = yo[part], sv = Ssv[k], r = rrv[k];
        c0.add_prod(a, a);
        c1.add_prod(sv, sv);
        c2.add_prod(a, sv);
        c3.add_prod(a, r);
        c4.add_prod(sv, r);
        c5.add_prod(r, r);
      }
    }
  }
  if (DOTS) {
    SolveScalars* S = b.S + tr.sec;
    dvec<6> acc = {{c0.value(), c1.value(), c2.value(), c3.value(), c4.value(), c5.value()}};
    dvec<6> tt;
    if (so_sum_last<6>(acc, b, t, s, &S->cnt[1], tt) && threadIdx.x == 0)
      cg3_scalars(S, tt, iter);
  }
}

// xx = L' yy as a gather: for model sample m, the "+" terms come from rows
// i = m - st - is and the "-" terms from rows i with i - is - id_i = m, all
// added in the reference's scatter order (row i ascending, iw ascending,
// "+" before "-"), part 1 before part 2.
// Indices are 32-bit within a patch (a patch holds fewer than 2^31
// samples); a tap plane is n floats, so plane iw starts at f + iw n (64-bit).
template <int NW>
__device__ __forceinline__ float ap3_adj_part(const float* __restrict__ y, int m, int st, int nj,
                                              const float* __restrict__ f,
                                              const int* __restrict__ idv,
                                              const uint8_t* __restrict__ v, int n, int drift,
                                              int dmax, float acc) {
  constexpr int NA = 2 * NW + 1;
  // "+" list: iw = NA-1 .. 0 gives ascending rows
  int ip[NA];
  int wp[NA];
  int np_ = 0;
  for (int iw = NA - 1; iw >= 0; iw--) {
    const int i = m - st - (iw - NW) * nj;
    if ((unsigned)i < (unsigned)n && v[i]) {
      ip[np_] = i;
      wp[np_] = iw;
      np_++;
    }
  }
  int a = 0;
  auto emit_plus_upto = [&](int ilim, int iwlim, bool strict) {
    while (a < np_ && (ip[a] < ilim || (ip[a] == ilim && (strict ? wp[a] <= iwlim : false)))) {
      acc = __fadd_rn(acc, __fmul_rn(y[ip[a]], f[(long)wp[a] * n + ip[a]]));
      a++;
    }
  };
  if (!drift) {
    for (int iw = 0; iw < NA; iw++) {
      const int i = m + (iw - NW) * nj;
      if ((unsigned)i >= (unsigned)n || !v[i]) continue;
      emit_plus_upto(i, iw, true);
      acc = __fsub_rn(acc, __fmul_rn(y[i], f[(long)iw * n + i]));
    }
  } else {
    const int lo = m - NW * nj - dmax, hi = m + NW * nj + dmax;
    for (int i = lo; i <= hi; i++) {
      if ((unsigned)i >= (unsigned)n || !v[i]) continue;
      const int q = i - m - idv[i];
      if (q % nj) continue;
      const int iw = q / nj + NW;
      if (iw < 0 || iw >= NA) continue;
      emit_plus_upto(i, iw, true);
      acc = __fsub_rn(acc, __fmul_rn(y[i], f[(long)iw * n + i]));
    }
  }
  emit_plus_upto(n, 0, false);
  return acc;
}

// The same without drift: every "+" row (m - st - is) precedes every "-"
// row (m + is), because a valid row has st > 2 NW nj, so the scatter order
// is the "+" terms with iw descending, then the "-" terms with iw ascending.
// All rows' validity, residual and tap are loaded first (indices clamped
// into the patch), then the valid terms are added in that order: the same
// additions as a loop that tests each row before loading it.
template <int NW>
__device__ __forceinline__ float ap3_adj_part_nodrift(const float* __restrict__ y, int m, int st,
                                                      int nj, const float* __restrict__ f,
                                                      const uint8_t* __restrict__ v, int n,
                                                      float acc) {
  constexpr int NA = 2 * NW + 1;
  float yv[2 * NA], fv[2 * NA];
  bool ok[2 * NA];
#pragma unroll
  for (int k = 0; k < 2 * NA; k++) {
    // k < NA: "+" term iw = NA-1-k at row m - st - is; else "-" term iw = k-NA at m + is
    const int iw = k < NA ? NA - 1 - k : k - NA;
    const int is = (iw - NW) * nj;
    const int i = k < NA ? m - st - is : m + is;
    const bool in = (unsigned)i < (unsigned)n;
    const int ic = in ? i : m;
    ok[k] = in && v[ic];
    yv[k] = y[ic];
    fv[k] = f[(long)iw * n + ic];
  }
#pragma unroll
  for (int k = 0; k < NA; k++)
    if (ok[k]) acc = __fadd_rn(acc, __fmul_rn(yv[k], fv[k]));
#pragma unroll
  for (int k = NA; k < 2 * NA; k++)
    if (ok[k]) acc = __fsub_rn(acc, __fmul_rn(yv[k], fv[k]));
  return acc;
}

// g = L' rr with the known samples zeroed (ps_solver :1058-1070) and
// gsum = g.g per patch.
template <int NW, bool DRIFT>
__global__ void __launch_bounds__(kTileThreads, 4) k_ap3_adj(SoArrays A, SoBatch b) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  SolveScalars* S = b.S + tr.sec;
  if (S->done) return;
  const Op3 g = geometry(b, s);
  constexpr int NA = 2 * NW + 1;
  const int dm = g.drift ? S->dmax : 0;
  const float* yy = A.rr + 2 * s.off;
  const float *f1 = A.f1 + NA * s.off, *f2 = A.f2 + NA * s.off;
  const uint8_t *v1 = A.v1 + s.off, *v2 = A.v2 + s.off, *known = A.known + s.off;
  float* gout = A.g + s.off;
  // 32-bit indices within the patch (fewer than 2^31 samples)
  const int n = (int)g.n, st2 = g.nx * g.ny, hi = (int)tr.hi;
  ffacc a0;
  for (int m = (int)tr.lo + threadIdx.x; m < hi; m += blockDim.x) {
    float a = 0.f;
    if (DRIFT) {
      a = ap3_adj_part<NW>(yy, m, g.nx, g.nj1, f1, A.id1 + s.off, v1, n, 1, dm, a);
      a = ap3_adj_part<NW>(yy + n, m, st2, g.nj2, f2, A.id2 + s.off, v2, n, 1, dm, a);
    } else {
      a = ap3_adj_part_nodrift<NW>(yy, m, g.nx, g.nj1, f1, v1, n, a);
      a = ap3_adj_part_nodrift<NW>(yy + n, m, st2, g.nj2, f2, v2, n, a);
    }
    if (known[m]) a = 0.f;
    gout[m] = a;
    a0.add_prod(a, a);
  }
  dvec<1> acc = {{a0.value()}};
  dvec<1> tot;
  if (so_sum_last<1>(acc, b, t, s, &S->cnt[0], tot) && threadIdx.x == 0) S->gsum = tot.v[0];
}

__global__ void k_max_shift(SoArrays A, SoBatch b) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  int best = 0;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    best = max(best, abs(A.id1[s.off + i]));
    best = max(best, abs(A.id2[s.off + i]));
  }
  atomicMax(&b.S[tr.sec].dmax, best);
}

// The tolerance test of ps_solver (:1086-1100) and ps_cgstep's scalar part
// (:835-866) from the patch's six dot products.
__device__ void cg3_scalars(SolveScalars* S, const dvec<6>& tt, int iter) {
  const float TOL = 1.e-12f, EPS = 1.e-12f;
  float dpr, dpg;
  if (iter == 0) {
    S->g0 = S->gsum;
    dpr = 1.f;
    dpg = 1.f;
  } else {
    dpr = __fdiv_rn((float)tt.v[5], (float)S->rr0);
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
    alfa = tt.v[0];
    if (alfa <= 0.) {
      S->skip = 1;
      return;
    }
    alfa = -tt.v[3] / alfa;
  } else {
    double gdg = tt.v[0], sds = tt.v[1], gds = tt.v[2];
    if (gdg == 0. || sds == 0.) {
      S->skip = 1;
      return;
    }
    double determ = 1.0 - (gds / gdg) * (gds / sds);
    if (determ > (double)EPS)
      determ *= gdg * sds;
    else
      determ = gdg * sds * (double)EPS;
    double gdr = -tt.v[3], sdr = -tt.v[4];
    alfa = (sds * gdr - gds * sdr) / determ;
    beta = (-gds * gdr + gdg * sdr) / determ;
  }
  S->alfa = __double2float_rn(alfa);
  S->beta = __double2float_rn(beta);
}

// ps_cgstep's vector part (:867-877).
__global__ void k_cg3_update(SoArrays A, SoBatch b, int iter) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const SolveScalars* S = b.S + tr.sec;
  if (S->done || S->skip) return;
  const float al = S->alfa, be = S->beta;
  float *x = A.x + s.off, *Sv = A.S + s.off, *rr = A.rr + 2 * s.off, *Ss = A.Ss + 2 * s.off;
  const float *g = A.g + s.off, *gg = A.gg + 2 * s.off;
  // 32-bit indices within the patch (fewer than 2^31 samples)
  const int n = (int)s.n, hi = (int)tr.hi;
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x) {
    float sv = iter == 0 ? 0.f : Sv[i];
    sv = __fadd_rn(__fmul_rn(sv, be), __fmul_rn(al, g[i]));
    Sv[i] = sv;
    x[i] = __fadd_rn(x[i], sv);
#pragma unroll
    for (int part = 0; part < 2; part++) {
      const int k = i + part * n;
      float s2 = iter == 0 ? 0.f : Ss[k];
      s2 = __fadd_rn(__fmul_rn(s2, be), __fmul_rn(al, gg[k]));
      Ss[k] = s2;
      rr[k] = __fadd_rn(rr[k], s2);
    }
  }
}

// x = data, known = mask != 0 (or data != 0), rr = -dd (-0 without noise),
// S = Ss = 0 (ps_cgstep's restart, :838-839).
__global__ void k_init(SoArrays A, SoBatch b) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    const long m = s.off + i;
    const float di = A.data[m];
    A.x[m] = di;
    A.known[m] = b.hasmask == 1 ? (A.mask[m] != 0.f) : (di != 0.f);
    A.S[m] = 0.f;
#pragma unroll
    for (int part = 0; part < 2; part++) {
      const long k = 2 * s.off + i + part * s.n;
      A.rr[k] = A.dd ? -A.dd[k] : -0.0f;
      A.Ss[k] = 0.f;
    }
  }
}

// rr0 = rr.rr per patch.
__global__ void k_rr0(SoArrays A, SoBatch b) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  SolveScalars* S = b.S + tr.sec;
  ffacc c0;
  const float* rr = A.rr + 2 * s.off;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x)
#pragma unroll
    for (int part = 0; part < 2; part++) {
      const float r = rr[i + part * s.n];
      c0.add_prod(r, r);
    }
  dvec<1> acc = {{c0.value()}};
  dvec<1> tot;
  if (so_sum_last<1>(acc, b, t, s, &S->cnt[2], tot) && threadIdx.x == 0) S->rr0 = tot.v[0];
}

__global__ void k_tile_map(const SecDesc* secs, int nsec, int ntiles, int* tile_sec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  tile_sec[t] = find_section(nsec, (long)t, [&](int k) { return (long)secs[k].tile0; });
}

struct SoLayout {
  long ntot;  // model samples spanned (data, mask, out)
  int ntiles;
};

SoLayout so_layout(std::vector<SecDesc>& secs) {
  SoLayout L{};
  int tiles = 0;
  for (auto& s : secs) {
    s.n = (long)s.n1 * s.n2 * s.n3;
    s.tile0 = tiles;
    s.ntile = (int)((s.n + kTile - 1) / kTile);
    tiles += s.ntile;
    L.ntot = std::max(L.ntot, s.off + s.n);
  }
  L.ntiles = tiles;
  return L;
}

struct SoWork {
  SoArrays a;
  SecDesc* secs;
  int* tile_sec;
  SolveScalars* S;
  double* partials;
  float* dd;
};

SoWork carve_soint3(void* ws, const SoLayout& L, int nsec, int order, bool noise, size_t* total) {
  const int na = 2 * order + 1;
  const long n = L.ntot;
  Carver cv(ws);
  SoWork w{};
  w.a.g = cv.take<float>(n);
  w.a.rr = cv.take<float>(2 * n);
  w.a.gg = cv.take<float>(2 * n);
  w.a.S = cv.take<float>(n);
  w.a.Ss = cv.take<float>(2 * n);
  w.dd = noise ? cv.take<float>(2 * n) : nullptr;
  w.a.f1 = cv.take<float>(na * n);
  w.a.f2 = cv.take<float>(na * n);
  w.a.id1 = cv.take<int>(n);
  w.a.id2 = cv.take<int>(n);
  w.a.v1 = cv.take<uint8_t>(n);
  w.a.v2 = cv.take<uint8_t>(n);
  w.a.known = cv.take<uint8_t>(n);
  w.secs = cv.take<SecDesc>(nsec);
  w.tile_sec = cv.take<int>(L.ntiles);
  w.S = cv.take<SolveScalars>(nsec);
  w.partials = cv.take<double>((size_t)L.ntiles * 6);
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
int soint3_run(const SoArrays& A, const SoBatch& b, int niter, cudaStream_t st) {
  const unsigned gt = (unsigned)b.ntiles;
  const int bs = kTileThreads;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_tile_map<<<(unsigned)((b.ntiles + 255) / 256), 256, 0, st>>>(
                 b.secs, b.nsec, b.ntiles, const_cast<int*>(b.tile_sec)));
  if (cudaMemsetAsync(b.S, 0, sizeof(SolveScalars) * b.nsec, st) != cudaSuccess) return PWD_ECUDA;
  PWD_KERNEL(PWD_FAM_SOINT, st, k_ap3_coef<NW><<<gt, bs, 0, st>>>(A, b, make_apcoef(NW)));
  if (b.drift) PWD_KERNEL(PWD_FAM_SOINT, st, k_max_shift<<<gt, bs, 0, st>>>(A, b));
  PWD_KERNEL(PWD_FAM_SOINT, st, k_init<<<gt, bs, 0, st>>>(A, b));
  PWD_KERNEL(PWD_FAM_SOINT, st,
             (k_ap3_fwd<NW, false><<<gt, bs, 0, st>>>(A.x, A.rr, A, b, 1, 0, 0)));
  PWD_KERNEL(PWD_FAM_SOINT, st, k_rr0<<<gt, bs, 0, st>>>(A, b));
  for (int iter = 0; iter < niter; iter++) {
    if (b.drift)
      PWD_KERNEL(PWD_FAM_SOINT, st, (k_ap3_adj<NW, true><<<gt, bs, 0, st>>>(A, b)));
    else
      PWD_KERNEL(PWD_FAM_SOINT, st, (k_ap3_adj<NW, false><<<gt, bs, 0, st>>>(A, b)));
    PWD_KERNEL(PWD_FAM_SOINT, st,
               (k_ap3_fwd<NW, true><<<gt, bs, 0, st>>>(A.g, A.gg, A, b, 0, 1, iter)));
    PWD_KERNEL(PWD_FAM_SOINT, st, k_cg3_update<<<gt, bs, 0, st>>>(A, b, iter));
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

int soint3_dispatch(int order, const SoArrays& A, const SoBatch& b, int niter, cudaStream_t st) {
  switch (order) {
    case 1: return soint3_run<1>(A, b, niter, st);
    case 2: return soint3_run<2>(A, b, niter, st);
    case 3: return soint3_run<3>(A, b, niter, st);
    case 4: return soint3_run<4>(A, b, niter, st);
  }
  return PWD_ENOTSUP;
}

// Validates and completes the section table of a batch.
int so_table(const pwd_section* in, int nsec, std::vector<SecDesc>& secs) {
  if (!in || nsec < 1) return PWD_EINVAL;
  secs.assign(nsec, SecDesc{});
  for (int i = 0; i < nsec; i++) {
    if (in[i].n1 < 1 || in[i].n2 < 1 || in[i].n3 < 1 || in[i].offset < 0 || in[i].out_offset < 0 ||
        (long)in[i].n1 * in[i].n2 * in[i].n3 >= (1L << 31))
      return PWD_EINVAL;
    secs[i].off = in[i].offset;
    secs[i].pout = in[i].out_offset;
    secs[i].n1 = in[i].n1;
    secs[i].n2 = in[i].n2;
    secs[i].n3 = in[i].n3;
  }
  return PWD_OK;
}

// Runs a batch: table on the device, noise (single patch only) uploaded.
int so_enqueue(const std::vector<SecDesc>& secs, const SoLayout& L, SoWork& w, const float* data,
               const float* mask, const float* pp, const float* qq, float* out, int order,
               int nj1, int nj2, int niter, int drift, int hasmask, int xl_after,
               const std::vector<float>* noise, cudaStream_t st) {
  const int nsec = (int)secs.size();
  if (cudaMemcpyAsync(w.secs, secs.data(), sizeof(SecDesc) * nsec, cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return PWD_ECUDA;
  if (noise) {
    if (cudaMemcpyAsync(w.dd, noise->data(), sizeof(float) * noise->size(),
                        cudaMemcpyHostToDevice, st) != cudaSuccess)
      return PWD_ECUDA;
    if (cudaStreamSynchronize(st) != cudaSuccess) return PWD_ECUDA;  // noise is a local buffer
  }
  SoArrays A = w.a;
  A.data = data;
  A.mask = mask;
  A.pp = pp;
  A.qq = qq;
  A.dd = noise ? w.dd : nullptr;
  A.x = out;
  SoBatch b{w.secs, w.tile_sec, nsec, L.ntiles, order, nj1, nj2, drift != 0, hasmask, xl_after,
            w.S, w.partials};
  return soint3_dispatch(order, A, b, niter, st);
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_soint3d_workspace_size(int n1, int n2, int n3, int order) {
  if (n1 < 1 || n2 < 1 || n3 < 1 || order < 1 || order > PWD_MAX_ORDER) return 0;
  std::vector<SecDesc> secs(1, SecDesc{});
  secs[0].n1 = n1;
  secs[0].n2 = n2;
  secs[0].n3 = n3;
  SoLayout L = so_layout(secs);
  size_t t = 0;
  carve_soint3(nullptr, L, 1, order, true, &t);
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
  if ((long)n1 * n2 * n3 >= (1L << 31)) return PWD_EINVAL;
  std::vector<SecDesc> secs(1, SecDesc{});
  secs[0].n1 = n1;
  secs[0].n2 = n2;
  secs[0].n3 = n3;
  SoLayout L = so_layout(secs);
  size_t need = 0;
  carve_soint3(nullptr, L, 1, order, true, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  SoWork w = carve_soint3(workspace, L, 1, order, true, &need);
  std::vector<float> dd;
  if (var != 0.f) {
    dd.resize(2 * (size_t)L.ntot);
    make_noise(dd, seed, var);
  }
  return so_enqueue(secs, L, w, data, mask, dip_inline, dip_xline, out, order, nj1, nj2, niter,
                    drift, hasmask, 0, var != 0.f ? &dd : nullptr, (cudaStream_t)stream);
}

extern "C" size_t pwd_soint3d_batch_workspace_size(const pwd_section* sections, int nsec,
                                                   int order) {
  std::vector<SecDesc> secs;
  if (order < 1 || order > PWD_MAX_ORDER || so_table(sections, nsec, secs) != PWD_OK) return 0;
  SoLayout L = so_layout(secs);
  size_t t = 0;
  carve_soint3(nullptr, L, nsec, order, false, &t);
  return t;
}

extern "C" int pwd_soint3d_batch(const float* data, const float* mask, const float* dips,
                                 float* out, const pwd_section* sections, int nsec, int order,
                                 int nj1, int nj2, int niter, int drift, int hasmask,
                                 void* workspace, size_t workspace_bytes, pwd_stream_t stream) {
  if (!data || !dips || !out || order < 1 || nj1 < 1 || nj2 < 1 || niter < 0) return PWD_EINVAL;
  if (hasmask == 1 && !mask) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  std::vector<SecDesc> secs;
  int rc = so_table(sections, nsec, secs);
  if (rc != PWD_OK) return rc;
  SoLayout L = so_layout(secs);
  size_t need = 0;
  carve_soint3(nullptr, L, nsec, order, false, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  SoWork w = carve_soint3(workspace, L, nsec, order, false, &need);
  return so_enqueue(secs, L, w, data, mask, dips, nullptr, out, order, nj1, nj2, niter, drift,
                    hasmask, 1, nullptr, (cudaStream_t)stream);
}
