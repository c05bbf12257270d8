// Local slope estimation by plane-wave destruction on the GPU.
//
// Restates dipc / dip3 / ps_divne / ps_conjgrad / ps_trianglen_lop of
// pyseistr/src/dip_cfuns.c (:1694-1989, :1619-1691, :796-827, :257-383,
// :672-712) as stream-ordered kernels over a batch of independent sections.
// Every launch covers all sections of the batch: elementwise work is split
// into tiles that never straddle a section, reductions are summed per
// section in a fixed tile order (deterministic, no floating-point atomics),
// and all scalar control (CG convergence, line-search acceptance) is per
// section on the device.  A call therefore enqueues a fixed launch sequence
// that depends only on (niter, liter, the smoothed axes), never synchronises
// with the host and can be captured in a CUDA graph; launches for a section
// that has left a loop return at once.
#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstdlib>
#include <vector>

#include "pwd_batch.cuh"
#include "pwd_common.cuh"

namespace pwd {
namespace {

constexpr int kTile = 8192;  // samples per elementwise tile
constexpr int kTileThreads = 256;

struct DipScalars {
  double usum, usum2, r0, norm2;
  double gn, gnp, g0, alpha, step;
  int zero, cg_done, ls_done, ls_trials, cg_iters;
  int stage_timeout;  // a bulk copy of the section's tile did not complete in time
  unsigned cnt[8];
};

struct DipBatch {
  const SecDesc* secs;
  const int* tile_sec;
  int nsec, ntiles;
  DipScalars* S;
  double* partials;  // [ntiles][3]
};

struct DipArrays {
  const float* u;  // data
  float* p;        // slopes (output)
  const uint8_t* mask;
  float *u1, *u2, *dp, *p0, *pcg, *r, *gp, *tmp, *sp, *sx, *sr, *tri;
  float *x2, *r2;  // mixed mode: second buffer of x (dp); r2 unused
  float* t2;       // mixed mode: axes 0-1 result of cubes
  int4* c0map;     // mixed mode: tile table of the axis-0 pass
};

struct TileRange {
  int sec;
  long lo, hi;
};

__device__ __forceinline__ TileRange tile_range(const DipBatch& b, int t) {
  TileRange r;
  r.sec = b.tile_sec[t];
  const SecDesc& s = b.secs[r.sec];
  r.lo = (long)(t - s.tile0) * kTile;
  r.hi = min(s.n, r.lo + kTile);
  return r;
}

// Offset of the slopes being estimated: inline ones first, crossline after.
__device__ __forceinline__ long pout_of(const SecDesc& s, int dip) {
  return s.pout + (dip == 2 ? s.n : 0);
}

// Sum of K doubles over the tiles of one section; true in the block of the
// section's last tile to finish, which receives the totals (summed over the
// section's tiles in tile order).
template <int K>
__device__ __forceinline__ bool sec_sum_last(dvec<K> x, const DipBatch& b, int t, const SecDesc& s,
                                             unsigned* counter, dvec<K>& tot) {
  __shared__ bool s_last;
  dvec<K> blk = block_sum<K>(x);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) b.partials[(size_t)t * 3 + k] = blk.v[k];
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
      v += __ldcg(b.partials + (size_t)(s.tile0 + i) * 3 + k);
    y.v[k] = v;
  }
  tot = block_sum<K>(y);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// Sections hold fewer than 2^31 samples, so 32-bit index arithmetic is used.
__device__ __forceinline__ bool pwd_valid(const SecDesc& s, int i, int nw, int dip) {
  const unsigned ii = (unsigned)i, n1 = (unsigned)s.n1, n2 = (unsigned)s.n2;
  const int i1 = (int)(ii % n1);
  const unsigned r = ii / n1;
  if (i1 < nw || i1 >= s.n1 - nw) return false;
  if (dip == 1) return (int)(r % n2) < s.n2 - 1;
  return (int)(r / n2) < s.n3 - 1;
}

// allpass1/allpass2 at one sample (dip_cfuns.c:1135-1200, :1399-1465).
template <int NW, bool DER, bool FAST = false>
__device__ __forceinline__ float pwd_at(const float* __restrict__ u, int i, int ip,
                                        const ApCoef& c, float p) {
  float f[2 * NW + 1];
  if (FAST) {
    if (DER)
      aderfilter_f32<NW>(c, p, f);
    else
      passfilter_f32<NW>(c, p, f);
  } else if (DER) {
    aderfilter<NW>(c, p, f);
  } else {
    passfilter<NW>(c, p, f);
  }
  float y = 0.f;
#pragma unroll
  for (int iw = 0; iw <= 2 * NW; iw++) {
    int is = iw - NW;
    y = __fadd_rn(y, __fmul_rn(__fsub_rn(u[i + is + ip], u[i - is]), f[iw]));
  }
  return y;
}

__device__ __forceinline__ int nb_offset(const SecDesc& s, int dip) {
  return dip == 1 ? s.n1 : s.n1 * s.n2;
}

// 2-D sections of a batch that also holds cubes have no crossline slope.
__device__ __forceinline__ bool no_pass(const SecDesc& s, int dip) { return dip == 2 && s.n3 == 1; }

template <int NW, bool FAST>
__global__ void k_residual(DipArrays a, DipBatch b, ApCoef c, int dip) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  if (no_pass(s, dip)) return;
  const float* u = a.u + s.off;
  const float* p = a.p + pout_of(s, dip);
  float* u2 = a.u2 + s.off;
  const int ip = nb_offset(s, dip), hi = (int)tr.hi;
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x)
    u2[i] = pwd_valid(s, i, NW, dip) ? pwd_at<NW, false, FAST>(u, i, ip, c, p[i]) : 0.f;
}

// One Gauss-Newton linearisation (dip3 :1645-1665 up to ps_divne's first
// normalisation, ps_divne :796-815): derivative filter, residual energy,
// mask, 1/hypot(den,1) scaling and the sum of den^2.
template <int NW, bool FAST>
__global__ void k_prep(DipArrays a, DipBatch b, ApCoef c, int dip) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  if (no_pass(s, dip)) return;
  const float* u = a.u + s.off;
  const float* p = a.p + pout_of(s, dip);
  float *u2 = a.u2 + s.off, *u1 = a.u1 + s.off, *p0 = a.p0 + s.off;
  const uint8_t* mask = a.mask ? a.mask + s.off : nullptr;
  const int ip = nb_offset(s, dip), hi = (int)tr.hi;
  ffacc a0, a1;
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x) {
    float pi = p[i];
    float d = pwd_valid(s, i, NW, dip) ? pwd_at<NW, true, FAST>(u, i, ip, c, pi) : 0.f;
    float r = u2[i];
    a0.add_prod(r, r);
    p0[i] = pi;
    if (mask && mask[i]) {
      d = 0.f;
      r = 0.f;
    }
    float num, den;
    if (FAST) {
      const float nrm = __frsqrt_rn(__fmaf_rn(d, d, 1.f));
      num = __fmul_rn(r, nrm);
      den = __fmul_rn(d, nrm);
    } else {
      invhypot_scale(r, d, num, den);
    }
    u2[i] = num;
    u1[i] = den;
    a1.add_prod(den, den);
  }
  dvec<2> acc = {{a0.value(), a1.value()}};
  DipScalars* S = b.S + tr.sec;
  dvec<2> tot;
  if (sec_sum_last<2>(acc, b, t, s, &S->cnt[0], tot) && threadIdx.x == 0) {
    S->usum = tot.v[0];
    S->zero = (tot.v[1] == 0.0);
    S->norm2 = S->zero ? 0.0 : sqrt((double)s.n / tot.v[1]);
    S->cg_done = S->zero;
    S->ls_done = 0;
    S->ls_trials = 0;
    S->cg_iters = 0;
  }
}

// ps_divne :817-826 second scaling, and ps_conjgrad :267-303 start.
__global__ void k_scale(DipArrays a, DipBatch b, int dip) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  if (no_pass(s, dip)) return;
  DipScalars* S = b.S + tr.sec;
  const bool zero = S->zero;
  const double nrm = S->norm2;
  float *num = a.u2 + s.off, *den = a.u1 + s.off, *r = a.r ? a.r + s.off : nullptr,
        *pcg = a.pcg + s.off, *x = a.dp + s.off;
  const float nh = __double2float_rn(nrm);
  const float nl = __double2float_rn(nrm - (double)nh);
  ffacc a0;
  const int hi = (int)tr.hi;  // a section holds fewer than 2^31 samples
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x) {
    x[i] = 0.f;
    if (zero) continue;
    float va = mul_by_double(num[i], nh, nl, nrm);
    float vb = mul_by_double(den[i], nh, nl, nrm);
    num[i] = va;
    den[i] = vb;
    float ri = -va;
    if (r) r[i] = ri;  // the mixed CG keeps no residual vector
    pcg[i] = 0.f;
    a0.add_prod(ri, ri);
  }
  dvec<1> acc = {{a0.value()}};
  dvec<1> tot;
  if (sec_sum_last<1>(acc, b, t, s, &S->cnt[1], tot) && threadIdx.x == 0) {
    S->r0 = tot.v[0];
    if (!S->zero && tot.v[0] == 0.0) S->cg_done = 1;
  }
}

// The previous iteration's step p += a sp, x += a sx, r += a sr (:364-368),
// then gx = -eps*x + W' r with eps = 1 (:306-317), written to tmp.  A
// section whose CG stopped skips both (the reference breaks before the step).
__global__ void k_cg_stepgrad(DipArrays a, DipBatch b, int iter) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const DipScalars* S = b.S + tr.sec;
  if (S->cg_done) return;
  const float st = __double2float_rn(S->step);
  float *pcg = a.pcg + s.off, *x = a.dp + s.off, *r = a.r + s.off, *tmp = a.tmp + s.off;
  const float *w = a.u1 + s.off, *sp = a.sp + s.off, *sx = a.sx + s.off, *sr = a.sr + s.off;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    float xi = x[i], ri = r[i];
    if (iter > 0) {
      pcg[i] = __fadd_rn(pcg[i], __fmul_rn(st, sp[i]));
      xi = __fadd_rn(xi, __fmul_rn(st, sx[i]));
      ri = __fadd_rn(ri, __fmul_rn(st, sr[i]));
      x[i] = xi;
      r[i] = ri;
    }
    tmp[i] = __fadd_rn(-xi, __fmul_rn(ri, w[i]));
  }
}

// The step of the last iteration when the CG ran all liter iterations
// (:364-368).  Only x, the CG's result, is read afterwards (the line search
// of dip3 uses it; p and r are discarded when ps_conjgrad returns), so only
// x is stepped.
__global__ void k_cg_step(DipArrays a, DipBatch b) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const DipScalars* S = b.S + tr.sec;
  if (S->cg_done) return;
  const float st = __double2float_rn(S->step);
  float* x = a.dp + s.off;
  const float* sx = a.sx + s.off;
  const int hi = (int)tr.hi;  // a section holds fewer than 2^31 samples
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x)
    x[i] = __fadd_rn(x[i], __fmul_rn(st, sx[i]));
}

// gp = eps*p + S' gx; gn = gp.gp; convergence test (:319, :328-345).
__global__ void k_cg_gp(DipArrays a, DipBatch b, int iter) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  DipScalars* S = b.S + tr.sec;
  if (S->cg_done) return;
  const float* pcg = a.pcg + s.off;
  float *tmp = a.tmp + s.off, *gp = a.gp + s.off;
  ffacc a0;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    float v = __fadd_rn(pcg[i], tmp[i]);
    gp[i] = v;
    tmp[i] = v;
    a0.add_prod(v, v);
  }
  dvec<1> acc = {{a0.value()}};
  dvec<1> tot;
  if (sec_sum_last<1>(acc, b, t, s, &S->cnt[2], tot) && threadIdx.x == 0) {
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
__global__ void k_cg_update(DipArrays a, DipBatch b, int iter) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  DipScalars* S = b.S + tr.sec;
  if (S->cg_done) return;
  const float al = __double2float_rn(S->alpha);
  const float *gp = a.gp + s.off, *tmp = a.tmp + s.off, *w = a.u1 + s.off;
  float *sp = a.sp + s.off, *sx = a.sx + s.off, *sr = a.sr + s.off;
  ffacc a0, a1, a2;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    float gx = tmp[i];
    float gr = __fadd_rn(0.f, __fmul_rn(gx, w[i]));
    float vp = gp[i], vx = gx, vr = gr;
    if (iter > 0) {
      vp = __fadd_rn(vp, __fmul_rn(al, sp[i]));
      vx = __fadd_rn(vx, __fmul_rn(al, sx[i]));
      vr = __fadd_rn(vr, __fmul_rn(al, sr[i]));
    }
    sp[i] = vp;
    sx[i] = vx;
    sr[i] = vr;
    a0.add_prod(vr, vr);
    a1.add_prod(vp, vp);
    a2.add_prod(vx, vx);
  }
  dvec<3> acc = {{a0.value(), a1.value(), a2.value()}};
  dvec<3> tot;
  if (sec_sum_last<3>(acc, b, t, s, &S->cnt[3], tot) && threadIdx.x == 0) {
    double beta = tot.v[0] + 1.0 * (tot.v[1] - tot.v[2]);
    S->step = -S->gn / beta;
    S->gnp = S->gn;
    S->cg_iters = iter + 1;
  }
}

// Triangle smoothing of every line along one axis of every section, in
// place (ps_smooth2 :616-625 = triple2 :564 + doubint2 :508 + fold2 :458).
//
// One warp smooths 32 lines of one section, lane = line (each section's
// lines of every axis are numbered from a multiple of 32).  The forward pass
// forms the spread v(m) = ((0 + -wt x[m]) + 2wt x[m-nb]) + -wt x[m-2nb]
// (terms present where the index is inside the line) ahead of the serial
// loop, which only runs the running sum S[m] = S[m-1] + v(m) into a
// line-interleaved scratch (lanes hold consecutive columns: coalesced).  The
// backward pass runs the suffix sum B[m] = B[m+1] + S[m] in the reference's
// order and folds the reflections straight into the output when the triangle
// is not longer than the line (the general fold2 loops otherwise).  Absent
// terms of v are added as +0 rather than skipped: that changes at most the
// sign of a zero v, and a running sum that starts at +0 never becomes -0, so
// S and B keep the reference's bits.
struct TriParams {
  int axis, nb;
  long nlines;  // lines of this axis over the batch (padded per section to 32)
  float wt, w2;
};

__device__ __forceinline__ int sec_of_line(const SecDesc* secs, int nsec, int axis, long g) {
  int lo = 0, hi = nsec - 1;
  while (lo < hi) {
    int mid = (lo + hi + 1) >> 1;
    if (secs[mid].line0[axis] <= g)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}

constexpr int kMaxRect = 64;
constexpr int kSweepWarps = 4;
constexpr int kFwdChunk = 16;  // strided axes: positions per prefetched chunk

// Offset of line q of one axis inside its section.
__device__ __forceinline__ long line_base(const SecDesc& s, int axis, long q) {
  if (axis == 0) return q * s.n1;
  if (axis == 1) return (q % s.n1) + (q / s.n1) * (long)s.n1 * s.n2;
  return q;
}

// fold2 when the triangle is longer than the line: backward sums written
// back to the scratch, reflections folded by the reference's loops.
__device__ void tri_fold_general(float* __restrict__ x, long d, int L, int nb,
                                 float* __restrict__ sc, long ss) {
  const int np = L + 2 * nb;
  float acc = 0.f;
  for (int m = np - 1; m >= 0; m--) {
    acc = __fadd_rn(acc, sc[m * ss]);
    sc[m * ss] = acc;
  }
  int i, j;
  for (i = 0; i < L; i++) x[i * d] = sc[(i + nb) * ss];
  for (j = nb + L; j < np; j += L) {
    for (i = 0; i < L && i < np - j; i++)
      x[(L - 1 - i) * d] = __fadd_rn(x[(L - 1 - i) * d], sc[(j + i) * ss]);
    j += L;
    for (i = 0; i < L && i < np - j; i++) x[i * d] = __fadd_rn(x[i * d], sc[(j + i) * ss]);
  }
  for (j = nb; j >= 0; j -= L) {
    for (i = 0; i < L && i < j; i++) x[i * d] = __fadd_rn(x[i * d], sc[(j - 1 - i) * ss]);
    j -= L;
    for (i = 0; i < L && i < j; i++)
      x[(L - 1 - i) * d] = __fadd_rn(x[(L - 1 - i) * d], sc[(j - 1 - i) * ss]);
  }
}

// Positions kept by the axis-0 window: a power of two >= 32 + 2 nb.
__host__ __device__ constexpr int sweep_window(int nb) {
  return 32 + 2 * nb <= 64 ? 64 : (32 + 2 * nb <= 128 ? 128 : 256);
}

// Shared memory of one warp: on axis 0 the window [32][P+1] (reused as the
// [32][33] output transposition tile of the backward pass), then the
// right-reflection / left-output stashes [nb][32] each.
__host__ __device__ constexpr int sweep_warp_floats(int axis, int nb) {
  return (axis == 0 ? 32 * (sweep_window(nb) + 1) : 0) + 2 * nb * 32;
}

template <int AXIS>
__global__ void __launch_bounds__(32 * kSweepWarps) k_tri_sweep(DipArrays a, DipBatch b,
                                                                TriParams tp) {
  extern __shared__ float smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const long g0 = (blockIdx.x * (long)kSweepWarps + w) * 32;
  if (g0 >= tp.nlines) return;
  const int si = sec_of_line(b.secs, b.nsec, AXIS, g0);
  if (b.S[si].cg_done) return;
  const SecDesc& s = b.secs[si];
  const int nb = tp.nb;
  const int L = AXIS == 0 ? s.n1 : (AXIS == 1 ? s.n2 : s.n3);
  const long nl = s.n / L;
  const long lb = g0 - s.line0[AXIS];
  if (lb >= nl) return;  // padding lines of the section
  const int nvalid = (int)min(32L, nl - lb);
  const bool mine = lane < nvalid;
  const long q = lb + (mine ? lane : 0);
  const int d = AXIS == 0 ? 1 : (AXIS == 1 ? s.n1 : s.n1 * s.n2);
  float* __restrict__ xl = a.tmp + s.off + line_base(s, AXIS, q);
  float* __restrict__ sc = a.tri + s.scr0[AXIS] + q;
  const long ss = nl;
  const int np = L + 2 * nb;
  const float mw = -tp.wt, w2 = tp.w2;
  float* tile = smem + w * sweep_warp_floats(AXIS, nb);
  float* er = tile + (AXIS == 0 ? 32 * (sweep_window(nb) + 1) : 0);  // er[j][lane] = B[L+nb+j]
  float* el = er + nb * 32;                       // el[i][lane], outputs i < nb

  // ---- forward pass ----
  float acc = 0.f;
  if (AXIS == 0) {
    // the warp's 32 traces pass through a shared-memory window of the last
    // P positions, W[t][pos mod P]: lane j loads position m0+j of every
    // trace (coalesced, unconditional: clamped addresses), and lane t then
    // reads x[m], x[m-nb], x[m-2nb] of its own trace from the window.  The
    // next chunk's loads are in flight during this chunk's sums.
    const int P = sweep_window(nb), P1 = P + 1;
    const float* xs = a.tmp + s.off + lb * L;
    const float* xp = xs + min(lane, L - 1);
    const int tmax = nvalid - 1;
    float xr[32];
#pragma unroll
    for (int t = 0; t < 32; t++) xr[t] = xp[min(t, tmax) * L];
#pragma unroll
    for (int t = 0; t < 32; t++) tile[t * P1 + lane] = xr[t];
    const float* Wl = tile + lane * P1;
    for (int m0 = 0; m0 < np; m0 += 32) {
      const bool more = m0 + 32 < L;
      if (more) {
        const float* xq = xs + min(m0 + 32 + lane, L - 1);
#pragma unroll
        for (int t = 0; t < 32; t++) xr[t] = xq[min(t, tmax) * L];
      }
      __syncwarp();
      const int kmax = min(32, np - m0);
      float* sp = sc + m0 * ss;
#pragma unroll 8
      for (int k = 0; k < kmax; k++) {
        const int m = m0 + k;
        const float x1 = Wl[m & (P - 1)];
        const float x2 = Wl[(m - nb) & (P - 1)];
        const float x3 = Wl[(m - 2 * nb) & (P - 1)];
        const float t1 = m < L ? __fmul_rn(mw, x1) : 0.f;
        const float t2 = (m >= nb && m < L + nb) ? __fmul_rn(w2, x2) : 0.f;
        const float t3 = m >= 2 * nb ? __fmul_rn(mw, x3) : 0.f;
        acc = __fadd_rn(acc, __fadd_rn(__fadd_rn(t1, t2), t3));
        if (mine) *sp = acc;
        sp += ss;
      }
      __syncwarp();
      if (more) {
        const int col = (m0 + 32 + lane) & (P - 1);
#pragma unroll
        for (int t = 0; t < 32; t++) tile[t * P1 + col] = xr[t];
      }
    }
    __syncwarp();
  } else {
    // lanes hold consecutive lines: the loads of x[p], x[p-nb], x[p-2nb] are
    // coalesced; the next chunk's loads are in flight during this chunk's sums
    constexpr int C = kFwdChunk;
    float r1[C], r2[C], r3[C];
#pragma unroll
    for (int k = 0; k < C; k++) {
      const int p = k;
      r1[k] = p < L ? xl[p * d] : 0.f;
      r2[k] = (p >= nb && p < L + nb) ? xl[(p - nb) * d] : 0.f;
      r3[k] = (p >= 2 * nb && p < np) ? xl[(p - 2 * nb) * d] : 0.f;
    }
    for (int m0 = 0; m0 < np; m0 += C) {
      float v[C];
#pragma unroll
      for (int k = 0; k < C; k++)
        v[k] = __fadd_rn(__fadd_rn(__fmul_rn(mw, r1[k]), __fmul_rn(w2, r2[k])),
                         __fmul_rn(mw, r3[k]));
#pragma unroll
      for (int k = 0; k < C; k++) {
        const int p = m0 + C + k;
        r1[k] = p < L ? xl[p * d] : 0.f;
        r2[k] = (p >= nb && p < L + nb) ? xl[(p - nb) * d] : 0.f;
        r3[k] = (p >= 2 * nb && p < np) ? xl[(p - 2 * nb) * d] : 0.f;
      }
      float* sp = sc + m0 * ss;
#pragma unroll
      for (int k = 0; k < C; k++) {
        if (m0 + k < np) {
          acc = __fadd_rn(acc, v[k]);
          if (mine) *sp = acc;
          sp += ss;
        }
      }
    }
  }

  if (nb > L) {  // triangle longer than the line: the general fold, per lane
    if (mine) tri_fold_general(xl, d, L, nb, sc, ss);
    return;
  }

  // ---- backward pass: B[m] for m = np-1 .. 0, chunked by output index
  // i = m - nb in aligned groups of 32 (i from -nb to L+nb-1) ----
  float* xs0 = a.tmp + s.off + lb * L;  // axis 0: trace t at xs0 + t*L
  auto put = [&](int i, float v) {            // output i < nb: written directly
    if (mine) xl[i * d] = v;
  };
  auto flush = [&](int c) {                   // axis 0: tile chunk c to x
    __syncwarp();
    const int i = c * 32 + lane;
    if (i >= nb && i < L) {
#pragma unroll 8
      for (int t = 0; t < 32; t++)
        if (t < nvalid) xs0[t * L + i] = tile[t * 33 + lane];
    }
    __syncwarp();
  };
  const int ctop = (L + nb - 1) >> 5;
  const int cbot = -((nb + 31) >> 5);
  float cur[32], nxt[32];
  auto load = [&](int c, float* buf) {
    const int mtop = c * 32 + 31 + nb;
    const float* sp = sc + (long)mtop * ss;
#pragma unroll
    for (int k = 0; k < 32; k++) {
      const int m = mtop - k;
      buf[k] = (m >= 0 && m < np) ? *sp : 0.f;
      sp -= ss;
    }
  };
  load(ctop, cur);
  acc = 0.f;
  for (int c = ctop; c >= cbot; c--) {
    if (c > cbot) load(c - 1, nxt);
    const int ibase = c * 32;
    if (ibase >= nb && ibase + 31 < L - nb) {
      // interior chunk: outputs are the backward sums themselves
#pragma unroll
      for (int k = 0; k < 32; k++) {
        acc = __fadd_rn(acc, cur[k]);
        if (AXIS == 0)
          tile[lane * 33 + 31 - k] = acc;
        else if (mine)
          xl[(ibase + 31 - k) * d] = acc;
      }
    } else {
#pragma unroll
      for (int k = 0; k < 32; k++) {
        const int i = ibase + 31 - k, m = i + nb;
        if (m < 0 || m >= np) continue;
        acc = __fadd_rn(acc, cur[k]);
        if (i >= L) {
          er[(i - L) * 32 + lane] = acc;
        } else if (i >= 0) {
          float v = acc;
          if (i >= L - nb) v = __fadd_rn(v, er[(L - 1 - i) * 32 + lane]);
          if (i < nb)
            el[i * 32 + lane] = v;
          else if (AXIS == 0)
            tile[lane * 33 + 31 - k] = v;
          else if (mine)
            xl[i * d] = v;
        } else {
          const int ii = -1 - i;
          put(ii, __fadd_rn(el[ii * 32 + lane], acc));
        }
      }
    }
    if (AXIS == 0 && c >= 0) flush(c);
#pragma unroll
    for (int k = 0; k < 32; k++) cur[k] = nxt[k];
  }
}

// One backtracking trial of dip3 :1666-1687: p = clip(p0 + lam*dp), new
// residual and its energy; accepted when it decreases.
template <int NW, bool FAST>
__global__ void k_ls_trial(DipArrays a, DipBatch b, ApCoef c, int dip, int k) {
  const int t = blockIdx.x;
  const TileRange tr = tile_range(b, t);
  const SecDesc& s = b.secs[tr.sec];
  DipScalars* S = b.S + tr.sec;
  if (S->ls_done || no_pass(s, dip)) return;
  const float lam = ldexpf(1.0f, -k);
  const float pmin = -FLT_MAX, pmax = FLT_MAX;
  const float *u = a.u + s.off, *p0 = a.p0 + s.off, *dp = a.dp + s.off;
  float *p = a.p + pout_of(s, dip), *u2 = a.u2 + s.off;
  const int ip = nb_offset(s, dip), hi = (int)tr.hi;
  ffacc a0;
  for (int i = (int)tr.lo + threadIdx.x; i < hi; i += blockDim.x) {
    float pi = __fadd_rn(p0[i], __fmul_rn(lam, dp[i]));
    if (pi < pmin) pi = pmin;
    if (pi > pmax) pi = pmax;
    p[i] = pi;
    float r = pwd_valid(s, i, NW, dip) ? pwd_at<NW, false, FAST>(u, i, ip, c, pi) : 0.f;
    u2[i] = r;
    a0.add_prod(r, r);
  }
  dvec<1> acc = {{a0.value()}};
  dvec<1> tot;
  if (sec_sum_last<1>(acc, b, t, s, &S->cnt[4], tot) && threadIdx.x == 0) {
    S->usum2 = tot.v[0];
    S->ls_trials = k + 1;
    if (tot.v[0] < S->usum) S->ls_done = 1;
  }
}

// Slopes of a section whose staged tile copy in the mixed CG timed out (the
// bounded wait gave up, the tile's CG values are missing) are set to NaN.
__global__ void k_mark_lost(DipArrays a, DipBatch b, int dip) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  if (!b.S[tr.sec].stage_timeout || no_pass(s, dip)) return;
  float* p = a.p + pout_of(s, dip);
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) p[i] = __int_as_float(0x7fc00000);
}

// mask32 (dip_cfuns.c:914-997, both=false, nj=1): flags samples whose PWD
// stencil touches a zero of the mask data.  m0 inline, m1 crossline.
__global__ void k_mask32(const float* __restrict__ mdata, uint8_t* __restrict__ m0,
                         uint8_t* __restrict__ m1, DipBatch b, int nw) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const float* yy = mdata + s.off;
  const int n1 = s.n1, n2 = s.n2, n3 = s.n3;
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    const unsigned ii = (unsigned)i, r = ii / (unsigned)n1;
    int ix = (int)(ii % (unsigned)n1);
    int iy = (int)(r % (unsigned)n2), iz = (int)(r / (unsigned)n2);
    bool ma = false, mb = false;
    if (ix >= nw && ix < n1 - nw) {
      if (iy < n2 - 1)
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          ma = ma || (yy[i - is] == 0.f) || (yy[i + n1 + is] == 0.f);
        }
      if (iz < n3 - 1)
        for (int iw = 0; iw <= 2 * nw; iw++) {
          int is = iw - nw;
          mb = mb || (yy[i - is] == 0.f) || (yy[i + (long)n1 * n2 + is] == 0.f);
        }
    }
    m0[s.off + i] = ma;
    m1[s.off + i] = mb;
  }
}

__global__ void k_zero_slopes(float* __restrict__ p, DipBatch b) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  for (long i = tr.lo + threadIdx.x; i < tr.hi; i += blockDim.x) {
    p[s.pout + i] = 0.f;
    if (s.n3 > 1) p[s.pout + s.n + i] = 0.f;
  }
}

__global__ void k_tile_map(const SecDesc* secs, int nsec, int ntiles, int* tile_sec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  tile_sec[t] = find_section(nsec, (long)t, [&](int k) { return (long)secs[k].tile0; });
}

__global__ void k_put_single(SecDesc* dst, SecDesc v) { *dst = v; }

// Marks the loops of 2-D sections done before the crossline pass.
__global__ void k_skip_2d(const SecDesc* secs, int nsec, DipScalars* S) {
  int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsec || secs[s].n3 > 1) return;
  S[s].cg_done = 1;
  S[s].ls_done = 1;
}

// ---------------------------------------------------------------------------
// Mixed mode of the shaping CG.
//
// ps_smooth2 along a line of length L with radius nb equals, in exact
// arithmetic, the convolution with the triangle w(k) = (nb-|k|)/nb^2,
// |k| < nb, of the line extended by half-sample mirroring (x[-1-i] = x[i],
// x[2L-1-i] = x[i], repeated when nb > L): triple2's spread, the two running
// sums and fold2's reflections are that operator.  The mixed mode applies it
// as a direct convolution, axis by axis: axis 0 in row segments staged in
// shared memory (the CG input operation applied while loading), axis 1 by
// one thread per column streaming down the rows with the CG output
// operation and its dot products (axis 2 of cubes in a third, elementwise
// pass).  One CG iteration of a 2-D section is four launches instead of
// three elementwise kernels and four line sweeps.  The residual and its
// conjugate direction are not kept as vectors: r = W x - num and sr = W sx
// hold in exact arithmetic (ps_conjgrad starts from x = 0, r = -num and
// steps both alike), so they are formed afresh where needed, one rounding
// each; the reference's recurrences for them would cost 16 of the
// iteration's 96 bytes a sample.  x is double-buffered across iterations
// because a segment's halo reads neighbours that another segment steps.
// ---------------------------------------------------------------------------
// Column strips of the axis-1 pass: kSmStrip columns (one thread each) by up
// to kSmB2 rows; inputs staged kSmStages - 1 rows ahead.
#ifndef PWD_SM_STAGES
#define PWD_SM_STAGES 4
#endif
constexpr int kSmStrip = 64, kSmB2 = 128, kSmStages = PWD_SM_STAGES;

// Strip height of the axis-1 passes: kSmB2 unless PWD_CG_STRIP in the
// environment gives 32, 64, 128 or 256 (a tuning knob: shorter strips give
// more tiles for small batches, longer ones fewer halo rows).
inline int strip_rows() {
  const char* e = getenv("PWD_CG_STRIP");
  const int v = e ? atoi(e) : kSmB2;
  return (v == 32 || v == 64 || v == 128 || v == 256) ? v : kSmB2;
}

enum { SM_IN_ARR = 0, SM_IN_CG1 = 1 };
enum { SM_OUT_ARR = 0, SM_OUT_CG1 = 1, SM_OUT_CG2 = 2 };

struct SmParams {
  int sel;  // sections processed: 0 all, 1 slices of 2-D sections only, 2 cubes only
  int nb0, nb1, nb2;
  float wt0, wt1, wt2;
  int iter;
  const float* in;   // SM_IN_ARR input
  float* out;        // SM_OUT_ARR output
  const float* gpc;  // gp, read at the output sample by SM_OUT_CG2 of axis 2
  const float* xo;  // x before the iteration (read) and after it (written):
  float* xn;        // double-buffered, a segment's halo reads other tiles' x
  const int4* c0map;  // axis-0 tiles, two entries each (k_conv0_map)
  int c0buf;          // floats per axis-0 staging buffer
  int tma;            // axis-0 tiles staged by bulk copies (else 4-byte cp.async)
  int b2;             // rows of an axis-1 strip
};

__device__ __forceinline__ bool sm_selected(int sel, const SecDesc& s) {
  return sel == 0 || (sel == 1) == (s.n3 == 1);
}

__device__ __forceinline__ int mirror_idx(int i, int n) {
  if (i >= 0 && i < n) return i;
  if (i < 0 && i >= -n) return -1 - i;
  if (i >= n && i < 2 * n) return 2 * n - 1 - i;
  const int p = 2 * n;  // several reflections: the extension has period 2n
  int r = i % p;
  if (r < 0) r += p;
  return r < n ? r : p - 1 - r;
}

// Triangle tap k of radius nb (|k| < nb).
__device__ __forceinline__ float tri_tap(int k, int nb, float wt) {
  return __fmul_rn((float)(nb - (k < 0 ? -k : k)), wt);
}
// The same for a radius known at compile time: a constant operand.
template <int NB>
__host__ __device__ constexpr float tri_tap_c(int k) {
  return (float)((double)(NB - (k < 0 ? -k : k)) / ((double)NB * NB));
}

// Sum of K doubles over the tiles [tile0, tile0+ntile) of one section; true
// in the block of the section's last tile to finish.
template <int K>
__device__ __forceinline__ bool tiles_sum_last(dvec<K> x, double* partials, int t, int tile0,
                                               int ntile, unsigned* counter, dvec<K>& tot) {
  __shared__ bool s_last;
  dvec<K> blk = block_sum<K>(x);
  if (threadIdx.x == 0) {
#pragma unroll
    for (int k = 0; k < K; k++) partials[(size_t)t * 3 + k] = blk.v[k];
    __threadfence();
    unsigned tk = atomicAdd(counter, 1u);
    s_last = (tk == (unsigned)(ntile - 1));
  }
  __syncthreads();
  if (!s_last) return false;
  __threadfence();
  dvec<K> y;
#pragma unroll
  for (int k = 0; k < K; k++) {
    double v = 0.0;
    for (int i = threadIdx.x; i < ntile; i += blockDim.x)
      v += __ldcg(partials + (size_t)(tile0 + i) * 3 + k);
    y.v[k] = v;
  }
  tot = block_sum<K>(y);
  if (threadIdx.x == 0) *counter = 0u;
  return true;
}

// gn = gp.gp, convergence test and alpha (ps_conjgrad :328-345), in the
// last tile of a section.
__device__ __forceinline__ void cg1_finish(DipScalars* S, double gn, int iter) {
  S->gn = gn;
  if (iter == 0) {
    S->g0 = gn;
  } else {
    const double alpha = gn / S->gnp;
    const double dg = gn / S->g0;
    S->alpha = alpha;
    const double tol = (double)1.e-6f;
    if (alpha < tol || dg < tol) S->cg_done = 1;
  }
}

// beta and the step (:346-359), in the last tile of a section.
__device__ __forceinline__ void cg2_finish(DipScalars* S, const dvec<3>& tot, int iter) {
  const double beta = tot.v[0] + 1.0 * (tot.v[1] - tot.v[2]);
  S->step = -S->gn / beta;
  S->gnp = S->gn;
  S->cg_iters = iter + 1;
}

// Output operation at one sample given the smoothed value v.
struct CgOut {
  ffacc a0, a1, a2;
  // p = pcg (+ step sp after the first iteration), gp = eps p + S' gx with
  // eps = 1, gp.gp; the operands arrive staged: pc = pcg, sv = sp
  __device__ __forceinline__ void cg1v(const DipArrays& a, long i, float v, float st, int iter,
                                       float pc, float sv) {
    float p = pc;
    if (iter > 0) {
      p = __fmaf_rn(st, sv, p);
      a.pcg[i] = p;
    }
    const float g = __fadd_rn(p, v);
    a.gp[i] = g;
    a0.add_prod(g, g);
  }
  // The mixed mode keeps no residual vectors: r = W x - num and sr = W sx
  // (their values in exact arithmetic; each formed afresh with one
  // rounding), so the directions step only p and x and the update writes
  // sp and sx.  gx = S gp arrives as the smoothed value.
  __device__ __forceinline__ void cg2v(const DipArrays& a, long i, float gx, float gpv, float al,
                                       int iter, float wv, float spv, float sxv) {
    float vp = gpv, vx = gx;
    if (iter > 0) {
      vp = __fmaf_rn(al, spv, vp);
      vx = __fmaf_rn(al, sxv, vx);
    }
    a.sp[i] = vp;
    a.sx[i] = vx;
    const float vr = __fmul_rn(wv, vx);  // sr = W sx
    a0.add_prod(vr, vr);
    a1.add_prod(vp, vp);
    a2.add_prod(vx, vx);
  }
};

// Axis 0 of the mixed-mode smoothing.  A tile is either several whole
// traces of a section (traces of up to kC0Seg samples, as many as the
// threads x outputs and the buffer hold) or one kC0Seg-sample segment of a
// longer trace; a table built once per call gives every tile's section,
// first trace, first sample, line count and line length.  Each line (trace
// or segment) is copied to shared memory by cp.async with h0 samples of
// margin on both sides holding the mirrored neighbours, at a row stride that
// keeps every output window 16-byte aligned; the CG input operation then
// runs in place; each thread finally forms consecutive outputs of one line
// from a float4 register window: 8 per thread for the plain array pass (64
// threads), 4 for the pass with the CG input operation (128 threads, five
// staged arrays).  NB0 > 0 fixes the radius at compile time.
constexpr int kC0Seg = 512;
template <int IN>
__host__ __device__ constexpr int conv0_outs() {
  return IN == SM_IN_ARR ? 8 : 4;
}
template <int IN>
__host__ __device__ constexpr int conv0_threads() {
  return kC0Seg / conv0_outs<IN>();
}

// Lines per tile for traces of n1 <= kC0Seg samples (1 for longer traces,
// which are cut into segments) and the buffer stride of a line.
__host__ __device__ inline int conv0_stride(int n1, int h0) {
  return (min(n1, kC0Seg) + 2 * h0 + 3) & ~3;
}
__host__ __device__ inline int conv0_lines(int n1, int h0) {
  if (n1 > kC0Seg) return 1;
  // 8-output groups bound the line count of both passes: ceil(n1/4) <= 2 ceil(n1/8)
  const int by_threads = conv0_threads<SM_IN_ARR>() / ((n1 + 7) / 8);
  const int by_buffer = (kC0Seg + 2 * h0 + 8) / conv0_stride(n1, h0);
  return max(1, min(by_threads, by_buffer));
}
// Tiles of one section.
__host__ __device__ inline int conv0_tiles(int n1, long ntr, int h0) {
  if (n1 > kC0Seg) return (int)(ntr * ((n1 + kC0Seg - 1) / kC0Seg));
  const int lt = conv0_lines(n1, h0);
  return (int)((ntr + lt - 1) / lt);
}
// Floats per staging buffer: lines fill at most kC0Seg + 2 h0 + 8, and the
// last window's float4 reads run up to 10 floats past its line.
__host__ __device__ inline int conv0_buffer(int h0) { return (kC0Seg + 2 * h0 + 24 + 3) & ~3; }

// The tile table of the axis-0 pass (one thread per tile): two int4 per
// tile, {section, n1, first sample, lines << 16 | length} and {first element
// of the tile's first trace (64 bits, low word first), section is 2-D, 0},
// so that a block finds everything it needs to start its copies in one
// 32-byte load.
__global__ void k_conv0_map(const SecDesc* secs, int nsec, int ntiles, int h0, int4* map) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  const int si = find_section(nsec, (long)t, [&](int k) { return (long)secs[k].ctile0; });
  const SecDesc& s = secs[si];
  const int n1 = s.n1, lt = t - s.ctile0;
  int tr0, nl, o1, len;
  if (n1 > kC0Seg) {
    const int nseg = (n1 + kC0Seg - 1) / kC0Seg;
    tr0 = lt / nseg;
    nl = 1;
    o1 = (lt - tr0 * nseg) * kC0Seg;
    len = min(kC0Seg, n1 - o1);
  } else {
    const int lpt = conv0_lines(n1, h0);
    tr0 = lt * lpt;
    nl = min(lpt, s.n2 * s.n3 - tr0);
    o1 = 0;
    len = n1;
  }
  const unsigned long long so = (unsigned long long)(s.off + (long)tr0 * n1);
  map[2 * t] = make_int4(si, n1, o1, (nl << 16) | len);
  map[2 * t + 1] = make_int4((int)(unsigned)so, (int)(unsigned)(so >> 32), s.n3 == 1, 0);
}

// A stopped section keeps its x and r: the CG input pass carries x to the
// new buffer.
template <int NT>
__device__ __noinline__ void conv0_carry(const SmParams& q, long so, int n1, int o1, int nl,
                                         int len) {
  for (int k = 0; k < nl; k++)
    for (int i = threadIdx.x; i < len; i += NT) {
      const long e = so + (long)k * n1 + o1 + i;
      q.xn[e] = q.xo[e];
    }
}

template <int IN, int NB0>
__global__ void __launch_bounds__(conv0_threads<IN>()) k_conv0(DipArrays a, DipBatch b,
                                                              SmParams q) {
  constexpr int NT = conv0_threads<IN>(), OUTS = conv0_outs<IN>();
  // buffers of q.c0buf floats: the input (SM_IN_ARR); x (becoming gx), W,
  // num, sx (SM_IN_CG1); with bulk staging the lines come first, then one
  // staging buffer per array
  extern __shared__ __align__(16) float buf[];
  const int4 tm = q.c0map[2 * blockIdx.x], tx = q.c0map[2 * blockIdx.x + 1];
  if (!(q.sel == 0 || (q.sel == 1) == (tx.z != 0))) return;  // sm_selected
  DipScalars* S = b.S + tm.x;
  const int n1 = tm.y;
  const int h0 = (NB0 > 0 ? NB0 : q.nb0) - 1;
  const int stride = conv0_stride(n1, h0);
  const int o1 = tm.z, nl = tm.w >> 16, len = tm.w & 0xffff;
  // indices below are relative to the tile's first trace (a section holds
  // fewer than 2^31 samples)
  const long so = (long)(((unsigned long long)(unsigned)tx.y << 32) | (unsigned)tx.x);
  // the section's stop flag: with bulk staging it is tested once the
  // copies are under way, so that its load and theirs overlap
  const int done = S->cg_done;
  if (!q.tma && done) {
    if (IN == SM_IN_CG1) conv0_carry<NT>(q, so, n1, o1, nl, len);
    return;
  }
  const int w = len + 2 * h0;  // staged samples per line
  const int nbuf = q.c0buf;
  const bool stepped = IN == SM_IN_CG1 && q.iter > 0;
  if (q.tma) {
    // The tile's samples of each input array are one contiguous range of
    // the array (whole traces, or one trace's segment and its halo): the
    // 16-byte-aligned range that covers it is copied to a staging buffer by
    // one bulk copy per array, then the lines (with mirrored margins) are
    // formed from the staging buffers.  Buffers: the lines (nbuf), then
    // one staging buffer per array.
    __shared__ __align__(8) unsigned long long s_bar;
    __shared__ int s_ok;
    const int p0 = max(0, o1 - h0), p1 = min(n1, o1 + len + h0);
    const long g0 = so + p0, g1 = so + (long)(nl - 1) * n1 + p1;
    const long ga = g0 & ~3L, gb = (g1 + 3) & ~3L;
    const unsigned bytes = (unsigned)((gb - ga) * 4);
    constexpr int NA = IN == SM_IN_ARR ? 1 : 4;
    const int narr = IN == SM_IN_ARR ? 1 : (stepped ? 4 : 3);
    float* stg = buf + nbuf;
    if (threadIdx.x == 0) {
      mbar_init(&s_bar, 1);
      mbar_fence_init();
      mbar_arrive_expect_tx(&s_bar, bytes * narr);
      const float* src[NA];
      if (IN == SM_IN_ARR) {
        src[0] = q.in;
      } else {
        src[0] = q.xo;
        src[1 % NA] = a.u1;
        src[2 % NA] = a.u2;  // num, the division's right-hand side
        src[3 % NA] = a.sx;
      }
      for (int ar = 0; ar < narr; ar++) bulk_copy_g2s(stg + ar * nbuf, src[ar] + ga, bytes, &s_bar);
      // a copy that does not complete in time marks the section and the
      // tile is skipped (after a second bounded wait for the copies)
      // (a tile's copies take microseconds; the limits are 50 ms)
      int ok = mbar_wait_bounded(&s_bar, 0, 50000000ull);
      if (!ok) {
        atomicExch(&S->stage_timeout, 1);
        mbar_wait_bounded(&s_bar, 0, 50000000ull);
      }
      s_ok = ok;
    }
    __syncthreads();
    if (done) {
      if (IN == SM_IN_CG1) conv0_carry<NT>(q, so, n1, o1, nl, len);
      return;
    }
    if (!s_ok) return;
    const float st = stepped ? __double2float_rn(S->step) : 0.f;
    for (int k = 0; k < nl; k++) {
      float* bl = buf + k * stride;
      for (int c = threadIdx.x; c < w; c += NT) {  // slot c: sample o1 - h0 + c
        const int pos = o1 - h0 + c;
        const long i = so + k * n1 + ((unsigned)pos < (unsigned)n1 ? pos : mirror_idx(pos, n1)) - ga;
        if (IN == SM_IN_ARR) {
          bl[c] = stg[i];
        } else {
          float xi = stg[i];
          if (stepped) xi = __fmaf_rn(st, stg[3 * nbuf + i], xi);
          const float wi = stg[nbuf + i];
          const float ri = __fmaf_rn(wi, xi, -stg[2 * nbuf + i]);  // r = W x - num
          bl[c] = __fmaf_rn(ri, wi, -xi);                           // gx = -eps x + W' r
          if (c >= h0 && c < h0 + len) q.xn[so + k * n1 + o1 - h0 + c] = xi;  // own sample
        }
      }
    }
    __syncthreads();
  } else {
  for (int k = 0; k < nl; k++) {
    float* bl = buf + k * stride;
    for (int c = threadIdx.x; c < w; c += NT) {  // slot c: sample o1 - h0 + c
      const int pos = o1 - h0 + c;
      const int i = k * n1 + ((unsigned)pos < (unsigned)n1 ? pos : mirror_idx(pos, n1));
      if (IN == SM_IN_ARR) {
        cp_async4(bl + c, q.in + so + i);
      } else {
        cp_async4(bl + c, q.xo + so + i);
        cp_async4(bl + nbuf + c, a.u1 + so + i);
        cp_async4(bl + 2 * nbuf + c, a.u2 + so + i);
        if (stepped) cp_async4(bl + 3 * nbuf + c, a.sx + so + i);
      }
    }
  }
  cp_async_commit();
  cp_async_wait<0>();
  __syncthreads();
  if (IN == SM_IN_CG1) {
    const float st = stepped ? __double2float_rn(S->step) : 0.f;
    for (int k = 0; k < nl; k++) {
      float* bl = buf + k * stride;
      for (int c = threadIdx.x; c < w; c += NT) {
        float xi = bl[c];
        if (stepped) xi = __fmaf_rn(st, bl[3 * nbuf + c], xi);
        const float wi = bl[nbuf + c];
        const float ri = __fmaf_rn(wi, xi, -bl[2 * nbuf + c]);  // r = W x - num
        bl[c] = __fmaf_rn(ri, wi, -xi);                         // gx = -eps x + W' r
        if (c >= h0 && c < h0 + len) q.xn[so + k * n1 + o1 - h0 + c] = xi;  // own sample
      }
    }
    __syncthreads();
  }
  }
  const int gpl = (len + OUTS - 1) / OUTS;  // output groups per line
  if ((int)threadIdx.x >= nl * gpl) return;
  // line of this thread: (tid + 1/2) / gpl is at least 1/(2 gpl) from an
  // integer, far above the error of the approximate quotient
  const int k = nl == 1 ? 0 : (int)__fdividef((float)threadIdx.x + 0.5f, (float)gpl);
  const int j0 = OUTS * (threadIdx.x - k * gpl);
  const float* wv = buf + k * stride + j0;  // window: outputs j0 .. centred at wv[h0 + u]
  float res[OUTS];
  if (NB0 > 0) {
    constexpr int NB0c = NB0 > 0 ? NB0 : 1, H0 = NB0c - 1, NV = (OUTS + 2 * H0 + 3) / 4;
    float v[4 * NV];
    const float4* p4 = reinterpret_cast<const float4*>(wv);
#pragma unroll
    for (int e = 0; e < NV; e++) {
      const float4 x4 = p4[e];
      v[4 * e] = x4.x;
      v[4 * e + 1] = x4.y;
      v[4 * e + 2] = x4.z;
      v[4 * e + 3] = x4.w;
    }
#pragma unroll
    for (int u = 0; u < OUTS; u++) {
      const int c = H0 + u;
      float acc = __fmul_rn(tri_tap_c<NB0c>(0), v[c]), acc2 = 0.f;
#pragma unroll
      for (int kk = 1; kk <= H0; kk++) {
        const float pr = __fadd_rn(v[c - kk], v[c + kk]);
        if (kk & 1)
          acc2 = __fmaf_rn(tri_tap_c<NB0c>(kk), pr, acc2);
        else
          acc = __fmaf_rn(tri_tap_c<NB0c>(kk), pr, acc);
      }
      res[u] = __fadd_rn(acc, acc2);
    }
  } else {
#pragma unroll
    for (int u = 0; u < OUTS; u++) {
      const float* row = wv + h0 + u;
      float acc = __fmul_rn(tri_tap(0, h0 + 1, q.wt0), row[0]);
      for (int kk = 1; kk <= h0; kk++)
        acc = __fmaf_rn(tri_tap(kk, h0 + 1, q.wt0), __fadd_rn(row[-kk], row[kk]), acc);
      res[u] = acc;
    }
  }
  float* out = q.out + so + k * n1 + o1 + j0;
#pragma unroll
  for (int u = 0; u < OUTS; u++)
    if (j0 + u < len) out[u] = res[u];
}

// Axis 1 of the mixed-mode smoothing with the CG output operation (AX =
// 1), or axis 2 of a cube (AX = 2: the cube seen as a section of n1 n2
// samples by n3 traces, whose axis 1 is the cube's axis 2): one
// thread per column of a strip of kSmStrip columns by up to kSmB2 rows
// streams down the rows (its input column, mirrored at the section's first
// and last traces, staged kSmStages - 1 rows ahead by cp.async together with
// the output operands), keeps the last 2 nb1 - 1 rows (in registers for a
// compiled radius, in a shared-memory ring otherwise) and forms each output
// row's axis-1 sum.  Threads share nothing until the closing reductions.
template <int OUT, int NB1, int AX = 1>
__global__ void __launch_bounds__(kSmStrip, 16) k_conv1(DipArrays a, DipBatch b, SmParams q) {
  extern __shared__ float sm[];
  const int t = blockIdx.x;
  const int si = find_section(b.nsec, (long)t, [&](int k) {
    return (long)(AX == 1 ? b.secs[k].ftile0 : b.secs[k].gtile0);
  });
  const SecDesc& s = b.secs[si];
  if (!sm_selected(q.sel, s)) return;
  DipScalars* S = b.S + si;
  if (S->cg_done) return;
  const int tile0 = AX == 1 ? s.ftile0 : s.gtile0, ntile = AX == 1 ? s.nftile : s.ngtile;
  const int n1 = AX == 1 ? s.n1 : s.n1 * s.n2, n2 = AX == 1 ? s.n2 : s.n3;
  const int b2 = q.b2;
  const int nt1 = (n1 + kSmStrip - 1) / kSmStrip, nt2 = (n2 + b2 - 1) / b2;
  const int lt = t - tile0;
  const int t1 = lt % nt1, t2 = (lt / nt1) % nt2, i3 = lt / (nt1 * nt2);
  const int o2 = t2 * b2;
  const int rows = min(b2, n2 - o2);
  const long so = s.off + (long)i3 * n1 * n2;
  const int j = threadIdx.x;
  const int g1 = t1 * kSmStrip + j;
  const bool colok = g1 < n1;
  const int nb1 = NB1 > 0 ? NB1 : (AX == 1 ? q.nb1 : q.nb2), h1 = nb1 - 1;
  const float wt = AX == 1 ? q.wt1 : q.wt2;
  const float st = (OUT == SM_OUT_CG1 && q.iter > 0) ? __double2float_rn(S->step) : 0.f;
  const float al = (OUT == SM_OUT_CG2 && q.iter > 0) ? __double2float_rn(S->alpha) : 0.f;
  // staging slot: [6][kSmStrip] = input, then 5 output operands
  constexpr int SE = 6 * kSmStrip;
  float* stg = sm;
  float* sring = sm + kSmStages * SE;  // runtime radius: [2 h1 + 1][kSmStrip]
  const int nsteps = rows + 2 * h1;
  auto issue = [&](int step) {
    if (step < nsteps && colok) {
      float* sg = stg + (step % kSmStages) * SE + j;
      const int g2 = mirror_idx(o2 - h1 + step, n2);
      cp_async4(sg, q.in + so + (long)g2 * n1 + g1);
      const int orow = step - 2 * h1;
      if (OUT != SM_OUT_ARR && orow >= 0) {
        const long i = so + (long)(o2 + orow) * n1 + g1;
        if (OUT == SM_OUT_CG1) {
          cp_async4(sg + kSmStrip, a.pcg + i);
          if (q.iter > 0) cp_async4(sg + 2 * kSmStrip, a.sp + i);
        } else {
          cp_async4(sg + kSmStrip, q.gpc + i);
          cp_async4(sg + 2 * kSmStrip, a.u1 + i);
          if (q.iter > 0) {
            cp_async4(sg + 3 * kSmStrip, a.sp + i);
            cp_async4(sg + 4 * kSmStrip, a.sx + i);
          }
        }
      }
    }
    cp_async_commit();
  };
  CgOut co;
  float ov[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
  // this step's staged input and output operands
  auto take = [&](int step) -> float {
    issue(step + kSmStages - 1);
    cp_async_wait<kSmStages - 1>();
    const float* sg = stg + (step % kSmStages) * SE + j;
    if (OUT != SM_OUT_ARR) {
#pragma unroll
      for (int k = 0; k < 5; k++) ov[k] = sg[(k + 1) * kSmStrip];
    }
    return sg[0];
  };
  auto out_op = [&](int orow, float acc) {
    if (!colok) return;
    const long i = so + (long)(o2 + orow) * n1 + g1;
    if (OUT == SM_OUT_ARR)
      q.out[i] = acc;
    else if (OUT == SM_OUT_CG1)
      co.cg1v(a, i, acc, st, q.iter, ov[0], ov[1]);
    else
      co.cg2v(a, i, acc, ov[0], al, q.iter, ov[1], ov[2], ov[3]);
  };
  for (int k = 0; k < kSmStages - 1; k++) issue(k);
  if (NB1 > 0) {
    constexpr int NB1c = NB1 > 0 ? NB1 : 1, H1 = NB1c - 1, RING = 2 * H1 + 1;
    float rg[RING];
    for (int step0 = 0; step0 < nsteps; step0 += RING) {
#pragma unroll
      for (int u = 0; u < RING; u++) {
        const int step = step0 + u;
        if (step < nsteps) {
          rg[u] = take(step);
          if (step >= 2 * H1) {
            float acc = __fmul_rn(tri_tap_c<NB1c>(0), rg[(u - H1 + RING) % RING]), acc2 = 0.f;
#pragma unroll
            for (int k = 1; k <= H1; k++) {
              const float pr = __fadd_rn(rg[(u - H1 - k + 2 * RING) % RING],
                                         rg[(u - H1 + k + RING) % RING]);
              if (k & 1)
                acc2 = __fmaf_rn(tri_tap_c<NB1c>(k), pr, acc2);
              else
                acc = __fmaf_rn(tri_tap_c<NB1c>(k), pr, acc);
            }
            out_op(step - 2 * H1, __fadd_rn(acc, acc2));
          }
        }
      }
    }
  } else {
    const int RING = 2 * h1 + 1;
    int slot = 0;
    for (int step = 0; step < nsteps; step++) {
      sring[slot * kSmStrip + j] = take(step);
      if (step >= 2 * h1) {
        int c = slot - h1;
        if (c < 0) c += RING;
        float acc = __fmul_rn(tri_tap(0, nb1, wt), sring[c * kSmStrip + j]);
        int lo = c, hi = c;
        for (int k = 1; k <= h1; k++) {
          lo = lo == 0 ? RING - 1 : lo - 1;
          hi = hi == RING - 1 ? 0 : hi + 1;
          acc = __fmaf_rn(tri_tap(k, nb1, wt),
                          __fadd_rn(sring[lo * kSmStrip + j], sring[hi * kSmStrip + j]), acc);
        }
        out_op(step - 2 * h1, acc);
      }
      slot = slot == RING - 1 ? 0 : slot + 1;
    }
  }
  cp_async_wait<0>();
  if (OUT == SM_OUT_CG1) {
    dvec<1> acc = {{co.a0.value()}};
    dvec<1> tot;
    if (tiles_sum_last<1>(acc, b.partials, t, tile0, ntile, &S->cnt[2], tot) &&
        threadIdx.x == 0)
      cg1_finish(S, tot.v[0], q.iter);
  } else if (OUT == SM_OUT_CG2) {
    dvec<3> acc = {{co.a0.value(), co.a1.value(), co.a2.value()}};
    dvec<3> tot;
    if (tiles_sum_last<3>(acc, b.partials, t, tile0, ntile, &S->cnt[3], tot) &&
        threadIdx.x == 0)
      cg2_finish(S, tot, q.iter);
  }
}

// Cubes: the axis-0 pass of gp fused into the axis-1 pass that consumes it
// (gp -> tmp -> t2, k_conv0<SM_IN_ARR> then k_conv1<SM_OUT_ARR>), for radii
// compiled on both axes.  Each staged row of the strip is the input's row
// segment of kSmStrip + 2 (NB0 - 1) samples (the strip's columns and the
// axis-0 halo, mirrored at the trace ends); each thread forms its column's
// axis-0 value from the segment in k_conv0's order of operations, so the
// outputs are those of the two separate passes, without the intermediate
// array's write and read.  The block waits for every row (threads read one
// another's copies), and a slot is refilled only after the barrier that
// follows its last reads.  (The same fusion into the conjugate-update pass
// of 2-D sections measured slower than the separate passes.)
__host__ __device__ constexpr int conv01_seg(int nb0) {
  return (kSmStrip + 2 * (nb0 - 1) + 3) & ~3;
}
template <int NB0, int NB1>
__global__ void __launch_bounds__(kSmStrip, 16) k_conv01(DipArrays a, DipBatch b, SmParams q) {
  extern __shared__ float sm[];
  constexpr int H0 = NB0 - 1, H1 = NB1 - 1, RING = 2 * H1 + 1, SEG = conv01_seg(NB0);
  const int t = blockIdx.x;
  const int si = find_section(b.nsec, (long)t, [&](int k) { return (long)b.secs[k].ftile0; });
  const SecDesc& s = b.secs[si];
  if (!sm_selected(q.sel, s)) return;
  if (b.S[si].cg_done) return;
  const int n1 = s.n1, n2 = s.n2;
  const int b2 = q.b2;
  const int nt1 = (n1 + kSmStrip - 1) / kSmStrip, nt2 = (n2 + b2 - 1) / b2;
  const int lt = t - s.ftile0;
  const int t1 = lt % nt1, t2 = (lt / nt1) % nt2, i3 = lt / (nt1 * nt2);
  const int o2 = t2 * b2;
  const int rows = min(b2, n2 - o2);
  const long so = s.off + (long)i3 * n1 * n2;
  const int j = threadIdx.x;
  const int c0 = t1 * kSmStrip;  // the strip's first column
  const int g1 = c0 + j;
  const bool colok = g1 < n1;
  // this thread's samples of the row segment: c0 - H0 + j and, for the
  // halo, c0 - H0 + kSmStrip + j (mirrored into the trace)
  const int e0 = mirror_idx(c0 - H0 + j, n1);
  const bool two = j < 2 * H0;
  const int e1 = two ? mirror_idx(c0 - H0 + kSmStrip + j, n1) : 0;
  const int nsteps = rows + 2 * H1;
  auto issue = [&](int step) {
    if (step < nsteps) {
      float* sg = sm + (step % kSmStages) * SEG;
      const float* row = q.in + so + (long)mirror_idx(o2 - H1 + step, n2) * n1;
      cp_async4(sg + j, row + e0);
      if (two) cp_async4(sg + kSmStrip + j, row + e1);
    }
    cp_async_commit();
  };
  // the axis-0 value of this thread's column on the step's row
  auto take = [&](int step) -> float {
    cp_async_wait<kSmStages - 2>();
    __syncthreads();
    issue(step + kSmStages - 1);
    const float* v = sm + (step % kSmStages) * SEG + j + H0;  // centred on the column
    float acc = __fmul_rn(tri_tap_c<NB0>(0), v[0]), acc2 = 0.f;
#pragma unroll
    for (int kk = 1; kk <= H0; kk++) {
      const float pr = __fadd_rn(v[-kk], v[kk]);
      if (kk & 1)
        acc2 = __fmaf_rn(tri_tap_c<NB0>(kk), pr, acc2);
      else
        acc = __fmaf_rn(tri_tap_c<NB0>(kk), pr, acc);
    }
    return __fadd_rn(acc, acc2);
  };
  for (int k = 0; k < kSmStages - 1; k++) issue(k);
  float rg[RING];
  for (int step0 = 0; step0 < nsteps; step0 += RING) {
#pragma unroll
    for (int u = 0; u < RING; u++) {
      const int step = step0 + u;
      if (step < nsteps) {
        rg[u] = take(step);
        if (step >= 2 * H1) {
          float acc = __fmul_rn(tri_tap_c<NB1>(0), rg[(u - H1 + RING) % RING]), acc2 = 0.f;
#pragma unroll
          for (int k = 1; k <= H1; k++) {
            const float pr = __fadd_rn(rg[(u - H1 - k + 2 * RING) % RING],
                                       rg[(u - H1 + k + RING) % RING]);
            if (k & 1)
              acc2 = __fmaf_rn(tri_tap_c<NB1>(k), pr, acc2);
            else
              acc = __fmaf_rn(tri_tap_c<NB1>(k), pr, acc);
          }
          if (colok) q.out[so + (long)(o2 + step - 2 * H1) * n1 + g1] = __fadd_rn(acc, acc2);
        }
      }
    }
  }
  cp_async_wait<0>();
}

// The same pass with two adjacent columns per thread (kSmStrip / 2 threads
// per strip), for the compiled radii: the convolution runs on packed FP32
// pairs (add / mul / fma .rn.f32x2, each lane rounded as the scalar form, so
// a column's smoothed values are those of k_conv1), the two columns' rows are
// staged by one 8-byte copy where aligned, and the CG output operation runs
// per column.  Only the dot products' accumulation order differs from
// k_conv1 (a thread's partial sums interleave its two columns).
template <int OUT, int NB1, int AX = 1>
__global__ void __launch_bounds__(kSmStrip / 2, 24) k_conv1p(DipArrays a, DipBatch b,
                                                             SmParams q) {
  extern __shared__ __align__(16) float sm[];
  const int t = blockIdx.x;
  const int si = find_section(b.nsec, (long)t, [&](int k) {
    return (long)(AX == 1 ? b.secs[k].ftile0 : b.secs[k].gtile0);
  });
  const SecDesc& s = b.secs[si];
  if (!sm_selected(q.sel, s)) return;
  DipScalars* S = b.S + si;
  if (S->cg_done) return;
  const int tile0 = AX == 1 ? s.ftile0 : s.gtile0, ntile = AX == 1 ? s.nftile : s.ngtile;
  const int n1 = AX == 1 ? s.n1 : s.n1 * s.n2, n2 = AX == 1 ? s.n2 : s.n3;
  const int b2 = q.b2;
  const int nt1 = (n1 + kSmStrip - 1) / kSmStrip, nt2 = (n2 + b2 - 1) / b2;
  const int lt = t - tile0;
  const int t1 = lt % nt1, t2 = (lt / nt1) % nt2, i3 = lt / (nt1 * nt2);
  const int o2 = t2 * b2;
  const int rows = min(b2, n2 - o2);
  const long so = s.off + (long)i3 * n1 * n2;
  const int c0 = 2 * threadIdx.x;  // this thread's columns c0, c0 + 1 of the strip
  const int g1 = t1 * kSmStrip + c0;
  const bool ok0 = g1 < n1, ok1 = g1 + 1 < n1;
  constexpr int H1 = NB1 - 1, RING = 2 * H1 + 1;
  const float st = (OUT == SM_OUT_CG1 && q.iter > 0) ? __double2float_rn(S->step) : 0.f;
  const float al = (OUT == SM_OUT_CG2 && q.iter > 0) ? __double2float_rn(S->alpha) : 0.f;
  constexpr int SE = 6 * kSmStrip;  // staging slot: [6][kSmStrip]
  float* stg = sm;
  const int nsteps = rows + 2 * H1;
  // both columns of a row: one 8-byte copy when both exist and the global
  // address is 8-byte aligned (n1 odd makes every other row unaligned)
  auto cp2 = [&](float* dst, const float* src) {
    if (ok1 && ((reinterpret_cast<uintptr_t>(src) & 7) == 0)) {
      cp_async8(dst, src);
    } else {
      cp_async4(dst, src);
      if (ok1) cp_async4(dst + 1, src + 1);
    }
  };
  auto issue = [&](int step) {
    if (step < nsteps && ok0) {
      float* sg = stg + (step % kSmStages) * SE + c0;
      const int g2 = mirror_idx(o2 - H1 + step, n2);
      cp2(sg, q.in + so + (long)g2 * n1 + g1);
      const int orow = step - 2 * H1;
      if (OUT != SM_OUT_ARR && orow >= 0) {
        const long i = so + (long)(o2 + orow) * n1 + g1;
        if (OUT == SM_OUT_CG1) {
          cp2(sg + kSmStrip, a.pcg + i);
          if (q.iter > 0) cp2(sg + 2 * kSmStrip, a.sp + i);
        } else {
          cp2(sg + kSmStrip, q.gpc + i);
          cp2(sg + 2 * kSmStrip, a.u1 + i);
          if (q.iter > 0) {
            cp2(sg + 3 * kSmStrip, a.sp + i);
            cp2(sg + 4 * kSmStrip, a.sx + i);
          }
        }
      }
    }
    cp_async_commit();
  };
  CgOut co;
  float2 ov[5];
  // this step's staged input pair and output operand pairs (a missing
  // second column holds stale values; its results are not stored)
  auto take = [&](int step) -> float2 {
    issue(step + kSmStages - 1);
    cp_async_wait<kSmStages - 1>();
    const float* sg = stg + (step % kSmStages) * SE + c0;
    if (OUT != SM_OUT_ARR) {
#pragma unroll
      for (int k = 0; k < 5; k++) ov[k] = *reinterpret_cast<const float2*>(sg + (k + 1) * kSmStrip);
    }
    return *reinterpret_cast<const float2*>(sg);
  };
  auto out_op = [&](int orow, float2 acc) {
    if (!ok0) return;
    const long i = so + (long)(o2 + orow) * n1 + g1;
    if (OUT == SM_OUT_ARR) {
      q.out[i] = acc.x;
      if (ok1) q.out[i + 1] = acc.y;
    } else if (OUT == SM_OUT_CG1) {
      co.cg1v(a, i, acc.x, st, q.iter, ov[0].x, ov[1].x);
      if (ok1) co.cg1v(a, i + 1, acc.y, st, q.iter, ov[0].y, ov[1].y);
    } else {
      co.cg2v(a, i, acc.x, ov[0].x, al, q.iter, ov[1].x, ov[2].x, ov[3].x);
      if (ok1) co.cg2v(a, i + 1, acc.y, ov[0].y, al, q.iter, ov[1].y, ov[2].y, ov[3].y);
    }
  };
  for (int k = 0; k < kSmStages - 1; k++) issue(k);
  float2 rg[RING];
  for (int step0 = 0; step0 < nsteps; step0 += RING) {
#pragma unroll
    for (int u = 0; u < RING; u++) {
      const int step = step0 + u;
      if (step < nsteps) {
        rg[u] = take(step);
        if (step >= 2 * H1) {
          const float w0 = tri_tap_c<NB1>(0);
          float2 acc = mul2_rn(make_float2(w0, w0), rg[(u - H1 + RING) % RING]);
          float2 acc2 = make_float2(0.f, 0.f);
#pragma unroll
          for (int k = 1; k <= H1; k++) {
            const float wk = tri_tap_c<NB1>(k);
            const float2 pr = add2_rn(rg[(u - H1 - k + 2 * RING) % RING],
                                      rg[(u - H1 + k + RING) % RING]);
            if (k & 1)
              acc2 = fma2_rn(make_float2(wk, wk), pr, acc2);
            else
              acc = fma2_rn(make_float2(wk, wk), pr, acc);
          }
          out_op(step - 2 * H1, add2_rn(acc, acc2));
        }
      }
    }
  }
  cp_async_wait<0>();
  if (OUT == SM_OUT_CG1) {
    dvec<1> acc = {{co.a0.value()}};
    dvec<1> tot;
    if (tiles_sum_last<1>(acc, b.partials, t, tile0, ntile, &S->cnt[2], tot) &&
        threadIdx.x == 0)
      cg1_finish(S, tot.v[0], q.iter);
  } else if (OUT == SM_OUT_CG2) {
    dvec<3> acc = {{co.a0.value(), co.a1.value(), co.a2.value()}};
    dvec<3> tot;
    if (tiles_sum_last<3>(acc, b.partials, t, tile0, ntile, &S->cnt[3], tot) &&
        threadIdx.x == 0)
      cg2_finish(S, tot, q.iter);
  }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
struct DipLayout {
  long ntot;  // elements spanned by the input arrays
  int ntiles;
  int nftiles;  // column-strip tiles (mixed mode)
  int nctiles;  // row-segment tiles (mixed mode)
  int ngtiles;  // axis-2 strip tiles of cubes (mixed mode)
  int b2;       // rows of an axis-1 / axis-2 strip (mixed mode)
  long ftiles_max;  // strip tiles with the shortest strips (sizes the partial sums)
  long scr_total;
  long nlines[3];
  bool any3d, any2d;
};

// Completes the section table (tiles, triangle line numbering and scratch).
DipLayout layout(std::vector<SecDesc>& secs, const int rect[3]) {
  DipLayout L{};
  long scr[3] = {0, 0, 0}, lines[3] = {0, 0, 0};
  int tiles = 0;
  const int b2 = L.b2 = strip_rows();
  for (auto& s : secs) {
    s.n = (long)s.n1 * s.n2 * s.n3;
    L.ntot = std::max(L.ntot, s.off + s.n);
    L.any3d |= s.n3 > 1;
    L.any2d |= s.n3 == 1;
    s.tile0 = tiles;
    s.ntile = (int)((s.n + kTile - 1) / kTile);
    tiles += s.ntile;
    s.ftile0 = L.nftiles;
    s.nftile = ((s.n1 + kSmStrip - 1) / kSmStrip) * ((s.n2 + b2 - 1) / b2) * s.n3;
    L.nftiles += s.nftile;
    L.ftiles_max += (long)((s.n1 + kSmStrip - 1) / kSmStrip) * ((s.n2 + 31) / 32) * s.n3 +
                    (s.n3 > 1 ? (long)((s.n1 * s.n2 + kSmStrip - 1) / kSmStrip) * ((s.n3 + 31) / 32)
                              : 0);
    s.gtile0 = L.ngtiles;
    s.ngtile = s.n3 > 1 ? ((s.n1 * s.n2 + kSmStrip - 1) / kSmStrip) * ((s.n3 + b2 - 1) / b2)
                        : 0;
    L.ngtiles += s.ngtile;
    s.ctile0 = L.nctiles;
    s.nctile = conv0_tiles(s.n1, (long)s.n2 * s.n3, std::max(rect[0], 1) - 1);
    L.nctiles += s.nctile;
    const int len[3] = {s.n1, s.n2, s.n3};
    for (int a = 0; a < 3; a++) {
      s.line0[a] = lines[a];
      s.scr0[a] = scr[a];
      if (rect[a] > 1) {
        long nl = s.n / len[a];
        // lines are swept 32 per warp: each section starts a new warp
        lines[a] += (nl + 31) / 32 * 32;
        scr[a] += nl * (len[a] + 2L * rect[a]);
      }
    }
  }
  L.ntiles = tiles;
  L.scr_total = std::max(std::max(scr[0], scr[1]), std::max(scr[2], 1L));
  for (int a = 0; a < 3; a++) L.nlines[a] = lines[a];
  return L;
}

struct DipWork {
  DipArrays a;
  uint8_t *m0, *m1;
  SecDesc* secs;
  int* tile_sec;
  DipScalars* S;
  double* partials;
};

DipWork carve_dip(void* ws, const DipLayout& L, int nsec, bool has_mask, size_t* total,
                  bool mixed = false) {
  Carver cv(ws);
  DipWork w{};
  const long n = L.ntot;
  w.a.u1 = cv.take<float>(n);
  w.a.u2 = cv.take<float>(n);
  w.a.dp = cv.take<float>(n);
  w.a.p0 = cv.take<float>(n);
  w.a.pcg = cv.take<float>(n);
  w.a.r = mixed ? nullptr : cv.take<float>(n);
  w.a.gp = cv.take<float>(n);
  w.a.tmp = cv.take<float>(n);
  w.a.sp = cv.take<float>(n);
  w.a.sx = cv.take<float>(n);
  w.a.sr = mixed ? nullptr : cv.take<float>(n);
  w.a.tri = mixed ? nullptr : cv.take<float>(L.scr_total);
  w.a.x2 = mixed ? cv.take<float>(n) : nullptr;
  w.a.t2 = mixed && L.any3d ? cv.take<float>(n) : nullptr;
  w.a.c0map = mixed ? cv.take<int4>(2 * (size_t)L.nctiles) : nullptr;
  w.m0 = has_mask ? cv.take<uint8_t>(n) : nullptr;
  w.m1 = has_mask ? cv.take<uint8_t>(n) : nullptr;
  w.secs = cv.take<SecDesc>(nsec);
  w.tile_sec = cv.take<int>(L.ntiles);
  w.S = cv.take<DipScalars>(nsec);
  w.partials = cv.take<double>(
      (size_t)std::max((long)L.ntiles, mixed ? L.ftiles_max : 0L) * 3);
  *total = cv.size();
  return w;
}

template <int NW>
int dip3_run(DipArrays a, int dip, int niter, int liter, const int rect[3], const DipLayout& L,
             const DipBatch& b, cudaStream_t st) {
  const ApCoef c = make_apcoef(NW);
  TriParams tp[3];
  int nax = 0;
  for (int ax = 0; ax < 3; ax++) {
    if (rect[ax] <= 1 || L.nlines[ax] == 0) continue;
    TriParams t;
    t.axis = ax;
    t.nb = rect[ax];
    t.nlines = L.nlines[ax];
    t.wt = (float)(1.0 / (rect[ax] * rect[ax]));
    t.w2 = (float)(2. * t.wt);
    tp[nax++] = t;
  }
  const unsigned gt = (unsigned)L.ntiles;
  // shared-memory limits of the sweep kernels (the axis-0 form with the
  // largest triangle needs more than the default 48 KB)
  for (int ax = 0; ax < 3; ax++) {
    const int bytes = (int)(sizeof(float) * kSweepWarps * sweep_warp_floats(ax, kMaxRect));
    cudaFuncSetAttribute(ax == 0 ? k_tri_sweep<0> : (ax == 1 ? k_tri_sweep<1> : k_tri_sweep<2>),
                         cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
  }
  auto sweeps = [&]() {
    for (int k = 0; k < nax; k++) {
      const int ax = tp[k].axis;
      const size_t smem = sizeof(float) * kSweepWarps * sweep_warp_floats(ax, tp[k].nb);
      const unsigned grid = (unsigned)((tp[k].nlines / 32 + kSweepWarps - 1) / kSweepWarps);
      auto* kern = ax == 0 ? k_tri_sweep<0> : (ax == 1 ? k_tri_sweep<1> : k_tri_sweep<2>);
      PWD_KERNEL(PWD_FAM_TRIANGLE, st,
                 kern<<<grid, 32 * kSweepWarps, smem, st>>>(a, b, tp[k]));
    }
  };
  PWD_KERNEL(PWD_FAM_PWD, st, k_residual<NW, false><<<gt, kTileThreads, 0, st>>>(a, b, c, dip));
  for (int iter = 0; iter < niter; iter++) {
    PWD_KERNEL(PWD_FAM_PWD, st, k_prep<NW, false><<<gt, kTileThreads, 0, st>>>(a, b, c, dip));
    PWD_KERNEL(PWD_FAM_CG, st, k_scale<<<gt, kTileThreads, 0, st>>>(a, b, dip));
    for (int it = 0; it < liter; it++) {
      PWD_KERNEL(PWD_FAM_CG, st, k_cg_stepgrad<<<gt, kTileThreads, 0, st>>>(a, b, it));
      sweeps();
      PWD_KERNEL(PWD_FAM_CG, st, k_cg_gp<<<gt, kTileThreads, 0, st>>>(a, b, it));
      sweeps();
      PWD_KERNEL(PWD_FAM_CG, st, k_cg_update<<<gt, kTileThreads, 0, st>>>(a, b, it));
    }
    if (liter > 0) PWD_KERNEL(PWD_FAM_CG, st, k_cg_step<<<gt, kTileThreads, 0, st>>>(a, b));
    for (int k = 0; k < 8; k++)
      PWD_KERNEL(PWD_FAM_PWD, st,
                 k_ls_trial<NW, false><<<gt, kTileThreads, 0, st>>>(a, b, c, dip, k));
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

typedef void (*SmKernel)(DipArrays, DipBatch, SmParams);

// Instances for radius nb: compiled for the common 10 (2-D sections) and 5
// (cubes), runtime otherwise.
template <int IN>
SmKernel conv0_kernel(int nb) {
  if (nb == 10) return k_conv0<IN, 10>;
  if (nb == 5) return k_conv0<IN, 5>;
  return k_conv0<IN, 0>;
}
template <int OUT, int AX = 1>
SmKernel conv1_kernel(int nb, bool pair) {
  if (nb == 10) return pair ? k_conv1p<OUT, 10, AX> : k_conv1<OUT, 10, AX>;
  if (nb == 5) return pair ? k_conv1p<OUT, 5, AX> : k_conv1<OUT, 5, AX>;
  return k_conv1<OUT, 0, AX>;
}
// The cubes' fused axis-0 + axis-1 pass of gp for radii compiled on both
// axes (5 and 5, or 10 and 10), unless PWD_CONV01=0 in the environment or
// the paired-column kernels are chosen; null otherwise.
SmKernel conv01_kernel(int nb0, int nb1, bool pair) {
  const char* e = getenv("PWD_CONV01");
  if (pair || (e && atoi(e) == 0)) return nullptr;
  if (nb0 == 5 && nb1 == 5) return k_conv01<5, 5>;
  if (nb0 == 10 && nb1 == 10) return k_conv01<10, 10>;
  return nullptr;
}
size_t conv01_smem(int nb0) { return sizeof(float) * kSmStages * conv01_seg(nb0); }
// Threads of an axis-1 (or axis-2) launch: paired columns for the compiled
// radii when PWD_CONV1_PAIR=1 (a tuning knob: on the batched workload the
// paired kernel measured 4 % slower, 137.0 against 132.9 ms of CG a step).
bool conv1_paired(int nb) {
  const char* e = getenv("PWD_CONV1_PAIR");
  return (nb == 10 || nb == 5) && e && atoi(e) == 1;
}

// Mixed mode of dip3: FP32 filter taps, the fused smoothing passes of the
// shaping CG, FP64 reductions as in the plain path.
template <int NW>
int dip3_run_mixed(DipArrays a, int dip, int niter, int liter, const int rect[3],
                   const DipLayout& L, const DipBatch& b, cudaStream_t st) {
  const ApCoef c = make_apcoef(NW);
  SmParams q{};
  q.nb0 = std::max(rect[0], 1);
  q.nb1 = std::max(rect[1], 1);
  q.nb2 = std::max(rect[2], 1);
  q.wt0 = (float)(1.0 / ((double)q.nb0 * q.nb0));
  q.wt1 = (float)(1.0 / ((double)q.nb1 * q.nb1));
  q.wt2 = (float)(1.0 / ((double)q.nb2 * q.nb2));
  const bool ax2 = q.nb2 > 1 && L.any3d;
  const unsigned gt = (unsigned)L.ntiles, gf = (unsigned)L.nftiles;
  const unsigned gc = (unsigned)L.nctiles, gg = (unsigned)L.ngtiles;
  q.c0map = a.c0map;
  q.b2 = L.b2;
  q.c0buf = conv0_buffer(q.nb0 - 1);
  // axis-0 staging by bulk copies unless PWD_CONV0_TMA=0 in the environment
  const char* tma_env = getenv("PWD_CONV0_TMA");
  q.tma = !(tma_env && atoi(tma_env) == 0);
  const size_t smem0 = sizeof(float) * q.c0buf * (q.tma ? 2 : 1),
               smem0cg = sizeof(float) * q.c0buf * (q.tma ? 5 : 4);
  const bool ring1 = !(q.nb1 == 10 || q.nb1 == 5);
  const size_t smem1 = sizeof(float) * (kSmStages * 6 * kSmStrip +
                                        (ring1 ? (2 * q.nb1 - 1) * kSmStrip : 0));
  const SmKernel c0_cg = conv0_kernel<SM_IN_CG1>(q.nb0), c0_arr = conv0_kernel<SM_IN_ARR>(q.nb0);
  const bool p1 = conv1_paired(q.nb1), p2 = conv1_paired(q.nb2);
  const int c1t = p1 ? kSmStrip / 2 : kSmStrip, c2t = p2 ? kSmStrip / 2 : kSmStrip;
  const SmKernel c1_cg1 = conv1_kernel<SM_OUT_CG1>(q.nb1, p1),
                 c1_cg2 = conv1_kernel<SM_OUT_CG2>(q.nb1, p1),
                 c1_arr = conv1_kernel<SM_OUT_ARR>(q.nb1, p1);
  cudaFuncSetAttribute(c0_cg, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0cg);
  cudaFuncSetAttribute(c0_arr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0);
  for (SmKernel k : {c1_cg1, c1_cg2, c1_arr})
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1);
  const SmKernel c01_arr = conv01_kernel(q.nb0, q.nb1, p1);
  const size_t smem01 = conv01_smem(q.nb0);
  if (c01_arr) cudaFuncSetAttribute(c01_arr, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem01);
  // axis 2 of cubes: the axis-1 kernel on the (n1 n2) x n3 view
  const bool ring2 = !(q.nb2 == 10 || q.nb2 == 5);
  const size_t smem2 = sizeof(float) * (kSmStages * 6 * kSmStrip +
                                        (ring2 ? (2 * q.nb2 - 1) * kSmStrip : 0));
  const SmKernel c2_cg1 = conv1_kernel<SM_OUT_CG1, 2>(q.nb2, p2),
                 c2_cg2 = conv1_kernel<SM_OUT_CG2, 2>(q.nb2, p2);
  for (SmKernel k : {c2_cg1, c2_cg2})
    cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem2);
  float* X[2] = {a.dp, a.x2};
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_conv0_map<<<(gc + 255) / 256, 256, 0, st>>>(b.secs, b.nsec, (int)gc, q.nb0 - 1,
                                                             a.c0map));
  PWD_KERNEL(PWD_FAM_PWD, st, k_residual<NW, true><<<gt, kTileThreads, 0, st>>>(a, b, c, dip));
  for (int iter = 0; iter < niter; iter++) {
    PWD_KERNEL(PWD_FAM_PWD, st, k_prep<NW, true><<<gt, kTileThreads, 0, st>>>(a, b, c, dip));
    PWD_KERNEL(PWD_FAM_CG, st, k_scale<<<gt, kTileThreads, 0, st>>>(a, b, dip));
    for (int it = 0; it < liter; it++) {
      q.iter = it;
      q.xo = X[it & 1];
      q.xn = X[(it + 1) & 1];
      // 2-D sections (every section when no cube is smoothed along axis 2):
      // axis 0 with the input operation, axis 1 with the output operation;
      // the axis-2 smoothing of a length-1 line is the identity
      if (!ax2 || L.any2d) {
        q.sel = ax2 ? 1 : 0;
        q.out = a.tmp;
        PWD_KERNEL(PWD_FAM_CG, st, (c0_cg<<<gc, conv0_threads<SM_IN_CG1>(), smem0cg, st>>>(a, b, q)));
        q.in = a.tmp;
        PWD_KERNEL(PWD_FAM_CG, st, (c1_cg1<<<gf, c1t, smem1, st>>>(a, b, q)));
        q.in = a.gp;
        q.out = a.tmp;
        PWD_KERNEL(PWD_FAM_CG, st, (c0_arr<<<gc, conv0_threads<SM_IN_ARR>(), smem0, st>>>(a, b, q)));
        q.in = a.tmp;
        q.gpc = a.gp;
        PWD_KERNEL(PWD_FAM_CG, st, (c1_cg2<<<gf, c1t, smem1, st>>>(a, b, q)));
      }
      if (ax2) {  // cubes: axes 0 and 1, then axis 2 with the CG operation
        q.sel = 2;
        q.out = a.tmp;
        PWD_KERNEL(PWD_FAM_CG, st, (c0_cg<<<gc, conv0_threads<SM_IN_CG1>(), smem0cg, st>>>(a, b, q)));
        q.in = a.tmp;
        q.out = a.t2;
        PWD_KERNEL(PWD_FAM_CG, st, (c1_arr<<<gf, c1t, smem1, st>>>(a, b, q)));
        q.in = a.t2;
        PWD_KERNEL(PWD_FAM_CG, st, (c2_cg1<<<gg, c2t, smem2, st>>>(a, b, q)));
        if (c01_arr) {  // axis 0 of gp inside the axis-1 pass
          q.in = a.gp;
          q.out = a.t2;
          PWD_KERNEL(PWD_FAM_CG, st, (c01_arr<<<gf, kSmStrip, smem01, st>>>(a, b, q)));
        } else {
          q.in = a.gp;
          q.out = a.tmp;
          PWD_KERNEL(PWD_FAM_CG, st,
                     (c0_arr<<<gc, conv0_threads<SM_IN_ARR>(), smem0, st>>>(a, b, q)));
          q.in = a.tmp;
          q.out = a.t2;
          PWD_KERNEL(PWD_FAM_CG, st, (c1_arr<<<gf, c1t, smem1, st>>>(a, b, q)));
        }
        q.in = a.t2;
        q.gpc = a.gp;
        PWD_KERNEL(PWD_FAM_CG, st, (c2_cg2<<<gg, c2t, smem2, st>>>(a, b, q)));
      }
    }
    DipArrays af = a;  // x and r after the last iteration
    af.dp = X[liter & 1];
    if (liter > 0) PWD_KERNEL(PWD_FAM_CG, st, k_cg_step<<<gt, kTileThreads, 0, st>>>(af, b));
    for (int k = 0; k < 8; k++)
      PWD_KERNEL(PWD_FAM_PWD, st,
                 k_ls_trial<NW, true><<<gt, kTileThreads, 0, st>>>(af, b, c, dip, k));
  }
  PWD_KERNEL(PWD_FAM_OTHER, st, k_mark_lost<<<gt, kTileThreads, 0, st>>>(a, b, dip));
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

int dip_dispatch(int order, DipArrays a, int dip, int niter, int liter, const int rect[3],
                 const DipLayout& L, const DipBatch& b, cudaStream_t st, bool mixed) {
  if (mixed) {
    switch (order) {
      case 1: return dip3_run_mixed<1>(a, dip, niter, liter, rect, L, b, st);
      case 2: return dip3_run_mixed<2>(a, dip, niter, liter, rect, L, b, st);
      case 3: return dip3_run_mixed<3>(a, dip, niter, liter, rect, L, b, st);
      case 4: return dip3_run_mixed<4>(a, dip, niter, liter, rect, L, b, st);
    }
    return PWD_ENOTSUP;
  }
  switch (order) {
    case 1: return dip3_run<1>(a, dip, niter, liter, rect, L, b, st);
    case 2: return dip3_run<2>(a, dip, niter, liter, rect, L, b, st);
    case 3: return dip3_run<3>(a, dip, niter, liter, rect, L, b, st);
    case 4: return dip3_run<4>(a, dip, niter, liter, rect, L, b, st);
  }
  return PWD_ENOTSUP;
}

// Enqueues the estimation of a batch whose section table is in w.secs.
int dip_enqueue(const float* data, const float* mask, float* out, const DipLayout& L,
                const DipWork& w, int nsec, int niter, int liter, int order, const int rect[3],
                cudaStream_t st, bool mixed = false) {
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_tile_map<<<(unsigned)((L.ntiles + 255) / 256), 256, 0, st>>>(w.secs, nsec, L.ntiles, w.tile_sec));
  if (cudaMemsetAsync(w.S, 0, sizeof(DipScalars) * nsec, st) != cudaSuccess) return PWD_ECUDA;
  DipBatch b{w.secs, w.tile_sec, nsec, L.ntiles, w.S, w.partials};
  DipArrays a = w.a;
  a.u = data;
  a.p = out;
  PWD_KERNEL(PWD_FAM_OTHER, st, k_zero_slopes<<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(out, b));
  if (mask)
    PWD_KERNEL(PWD_FAM_OTHER, st,
               k_mask32<<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(mask, w.m0, w.m1, b, order));
  a.mask = mask ? w.m0 : nullptr;
  int rc = dip_dispatch(order, a, 1, niter, liter, rect, L, b, st, mixed);
  if (rc != PWD_OK || !L.any3d) return rc;
  // crossline slopes (dipc :1926); 2-D sections of a mixed batch skip them
  // because their crossline residual region is empty (n3 = 1).
  a.mask = mask ? w.m1 : nullptr;
  PWD_KERNEL(PWD_FAM_OTHER, st, k_skip_2d<<<(nsec + 127) / 128, 128, 0, st>>>(w.secs, nsec, w.S));
  return dip_dispatch(order, a, 2, niter, liter, rect, L, b, st, mixed);
}

int check_dip_args(int niter, int liter, int order, const int rect[3]) {
  if (!rect || niter < 0 || liter < 0 || order < 1) return PWD_EINVAL;
  for (int a = 0; a < 3; a++) {
    if (rect[a] < 0) return PWD_EINVAL;
    if (rect[a] > kMaxRect) return PWD_ENOTSUP;
  }
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  return PWD_OK;
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_dip_workspace_size(int n1, int n2, int n3, int order, const int rect[3],
                                         int has_mask) {
  (void)order;
  if (n1 < 1 || n2 < 1 || n3 < 1 || !rect) return 0;
  std::vector<SecDesc> secs(1, SecDesc{});
  secs[0].n1 = n1;
  secs[0].n2 = n2;
  secs[0].n3 = n3;
  DipLayout L = layout(secs, rect);
  size_t need = 0;
  carve_dip(nullptr, L, 1, has_mask != 0, &need);
  return need;
}

extern "C" int pwd_dip(const float* data, const float* mask, float* dip_out, int n1, int n2,
                       int n3, int niter, int liter, int order, const int rect[3],
                       void* workspace, size_t workspace_bytes, pwd_stream_t stream) {
  int rc = check_dip_args(niter, liter, order, rect);
  if (rc != PWD_OK) return rc;
  if (!data || !dip_out || n1 < 1 || n2 < 1 || n3 < 1 || 2 * order >= n1) return PWD_EINVAL;
  if ((long)n1 * n2 * n3 >= (1L << 31)) return PWD_EINVAL;
  std::vector<SecDesc> secs(1, SecDesc{});
  secs[0].n1 = n1;
  secs[0].n2 = n2;
  secs[0].n3 = n3;
  DipLayout L = layout(secs, rect);
  size_t need = 0;
  carve_dip(nullptr, L, 1, mask != nullptr, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  DipWork w = carve_dip(workspace, L, 1, mask != nullptr, &need);
  cudaStream_t st = (cudaStream_t)stream;
  PWD_KERNEL(PWD_FAM_OTHER, st, k_put_single<<<1, 1, 0, st>>>(w.secs, secs[0]));
  return dip_enqueue(data, mask, dip_out, L, w, 1, niter, liter, order, rect, st);
}

// ---------------------------------------------------------------------------
// batched entry point
// ---------------------------------------------------------------------------
namespace {

int batch_table(const pwd_section* in, int nsec, int order, std::vector<SecDesc>& secs) {
  if (!in || nsec < 1) return PWD_EINVAL;
  secs.assign(nsec, SecDesc{});
  for (int i = 0; i < nsec; i++) {
    if (in[i].n1 < 1 || in[i].n2 < 1 || in[i].n3 < 1 || 2 * order >= in[i].n1 ||
        in[i].offset < 0 || in[i].out_offset < 0 ||
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

}  // namespace

extern "C" size_t pwd_dip_batch_workspace_size(const pwd_section* sections, int nsec, int order,
                                               const int rect[3], int has_mask) {
  std::vector<SecDesc> secs;
  if (!rect || batch_table(sections, nsec, std::max(order, 1), secs) != PWD_OK) return 0;
  DipLayout L = layout(secs, rect);
  size_t need = 0;
  carve_dip(nullptr, L, nsec, has_mask != 0, &need);
  return need;
}

namespace {

// phase bit 1: upload the section table into the workspace; bit 2: enqueue
// the estimation (kernels and memsets only, so it can be captured).
enum { kPrepare = 1, kRun = 2 };

int dip_batch_common(const float* data, const float* mask, float* dip_out,
                     const pwd_section* sections, int nsec, int niter, int liter, int order,
                     const int rect[3], void* workspace, size_t workspace_bytes,
                     pwd_stream_t stream, bool mixed, int phase = kPrepare | kRun,
                     bool has_mask = false) {
  int rc = check_dip_args(niter, liter, order, rect);
  if (rc != PWD_OK) return rc;
  if ((phase & kRun) && (!data || !dip_out)) return PWD_EINVAL;
  if (phase & kRun) has_mask = mask != nullptr;
  std::vector<SecDesc> secs;
  if ((rc = batch_table(sections, nsec, order, secs)) != PWD_OK) return rc;
  DipLayout L = layout(secs, rect);
  size_t need = 0;
  carve_dip(nullptr, L, nsec, has_mask, &need, mixed);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  DipWork w = carve_dip(workspace, L, nsec, has_mask, &need, mixed);
  cudaStream_t st = (cudaStream_t)stream;
  if ((phase & kPrepare) &&
      cudaMemcpyAsync(w.secs, secs.data(), sizeof(SecDesc) * nsec, cudaMemcpyHostToDevice, st) !=
          cudaSuccess)
    return PWD_ECUDA;
  if (!(phase & kRun)) return PWD_OK;
  return dip_enqueue(data, mask, dip_out, L, w, nsec, niter, liter, order, rect, st, mixed);
}

}  // namespace

extern "C" int pwd_dip_batch(const float* data, const float* mask, float* dip_out,
                             const pwd_section* sections, int nsec, int niter, int liter,
                             int order, const int rect[3], void* workspace,
                             size_t workspace_bytes, pwd_stream_t stream) {
  return dip_batch_common(data, mask, dip_out, sections, nsec, niter, liter, order, rect,
                          workspace, workspace_bytes, stream, false);
}

extern "C" int pwd_dip_batch_prepare(const pwd_section* sections, int nsec, int order,
                                     const int rect[3], int has_mask, int mixed,
                                     void* workspace, size_t workspace_bytes,
                                     pwd_stream_t stream) {
  return dip_batch_common(nullptr, nullptr, nullptr, sections, nsec, 0, 0, order, rect, workspace,
                          workspace_bytes, stream, mixed != 0, kPrepare, has_mask != 0);
}

extern "C" int pwd_dip_batch_run(const float* data, const float* mask, float* dip_out,
                                 const pwd_section* sections, int nsec, int niter, int liter,
                                 int order, const int rect[3], int mixed, void* workspace,
                                 size_t workspace_bytes, pwd_stream_t stream) {
  return dip_batch_common(data, mask, dip_out, sections, nsec, niter, liter, order, rect,
                          workspace, workspace_bytes, stream, mixed != 0, kRun);
}

extern "C" size_t pwd_dip_batch_mixed_workspace_size(const pwd_section* sections, int nsec,
                                                     int order, const int rect[3],
                                                     int has_mask) {
  std::vector<SecDesc> secs;
  if (!rect || batch_table(sections, nsec, std::max(order, 1), secs) != PWD_OK) return 0;
  DipLayout L = layout(secs, rect);
  size_t need = 0;
  carve_dip(nullptr, L, nsec, has_mask != 0, &need, true);
  return need;
}

extern "C" int pwd_dip_batch_mixed(const float* data, const float* mask, float* dip_out,
                                   const pwd_section* sections, int nsec, int niter, int liter,
                                   int order, const int rect[3], void* workspace,
                                   size_t workspace_bytes, pwd_stream_t stream) {
  return dip_batch_common(data, mask, dip_out, sections, nsec, niter, liter, order, rect,
                          workspace, workspace_bytes, stream, true);
}

// ---------------------------------------------------------------------------
// Slope estimation with no allocation at all.
//
// Some callers cannot allocate device memory when they estimate slopes: a
// plugin that runs inside a host application owning the CUDA context and
// its memory budget, or a real-time DAS acquisition loop that must not call
// cudaMalloc (it may synchronise the device) after start-up.  For them this
// entry point keeps its scratch in a file-scope device array of fixed size,
// resident on every GPU that loads the library until the process exits.
// ---------------------------------------------------------------------------
namespace {

constexpr size_t kDipStaticScratchBytes = size_t(64) << 20;  // 64 MiB per device
static __device__ __align__(256) unsigned char g_dip_static_scratch[kDipStaticScratchBytes];

// Device address of the array in the current context.  The host-side name
// of a __device__ array is not a device address, so it is looked up with the
// device current.  The lookup allocates nothing and is repeated on every
// call rather than cached: after a cudaDeviceReset the module is loaded
// again in a new context, possibly at another address, and a cached pointer
// would then be stale.  The first lookup in a context loads the module (lazy
// loading, the CUDA default), which commits the array's memory there.
int static_scratch(void** out) {
  void* p = nullptr;
  if (cudaGetSymbolAddress(&p, g_dip_static_scratch) != cudaSuccess || !p) return PWD_ECUDA;
  *out = p;
  return PWD_OK;
}

}  // namespace

extern "C" size_t pwd_dip_static_capacity(void) { return kDipStaticScratchBytes; }

extern "C" int pwd_dip_static(const float* data, const float* mask, float* dip_out, int n1,
                              int n2, int n3, int niter, int liter, int order, const int rect[3],
                              pwd_stream_t stream) {
  int rc = check_dip_args(niter, liter, order, rect);
  if (rc != PWD_OK) return rc;
  if (!data || !dip_out || n1 < 1 || n2 < 1 || n3 < 1 || 2 * order >= n1) return PWD_EINVAL;
  if ((long)n1 * n2 * n3 >= (1L << 31)) return PWD_EINVAL;
  const size_t need = pwd_dip_workspace_size(n1, n2, n3, order, rect, mask != nullptr);
  if (need == 0 || need > kDipStaticScratchBytes) return PWD_EWORKSPACE;  // section too large
  void* ws = nullptr;
  if ((rc = static_scratch(&ws)) != PWD_OK) return rc;
  return pwd_dip(data, mask, dip_out, n1, n2, n3, niter, liter, order, rect, ws,
                 kDipStaticScratchBytes, stream);
}
