// 2-D plane-wave spray with the structure-oriented mean and median.
//
// Restates csomean2d / csomf2d (pyseistr/src/sof_cfuns.c:1433-1678) with
// pwsmooth_* (:1036-1122) and pwspray_lop (:948-1033), for one section or a
// batch of sections of uneven size in one launch.  The spray of a section is
// two independent prediction chains per source trace (towards lower and
// higher trace numbers); every chain is one GPU thread.  For the mean, the
// trace of ones (the normalisation spray of pwsmooth_set) and the data are
// predicted through the same factorisation in the same chain.
#include <algorithm>
#include <cstdlib>
#include <type_traits>
#include <vector>

#include "pwd_batch.cuh"
#include "pwd_median.cuh"
#include "pwd_predict.cuh"

namespace pwd {
namespace {

constexpr int kTile = 2048;
constexpr int kTileThreads = 256;

struct SprayB {
  const SecDesc* secs;
  const int* tile_sec;
  int nsec, ntiles;
  long ntr;  // traces over the batch (n2*n3 per section)
  long ntp;  // the same with each section's traces padded to a multiple of 32
  int ns, np;
  float eps, eps2;
};

struct SprayBufs {
  float* u;     // data panels [trace][np][n1] per section
  float* u1;    // ones panels (mean only)
  float* w1;    // normalisation weights, one per sample (adjoint mean only)
  float* scr;   // factor store and chain scratch
};

// Factor-once form of the forward spray.  The factor store of a section
// (at scr + sc0, 128-byte aligned) holds, for every trace k, the
// passfilter taps of its slopes and the LDL' factors of the predictions
// that use them (forw = false for the chains running towards lower traces,
// true for the others), each element trace-interleaved with the section's
// traces padded to a multiple of 32 (ntp), so that a warp of 32 traces
// reads whole 128-byte lines; then the chains' y scratch, interleaved the
// same way over the 2 ntp chains.
struct FactorLayout {
  float *taps, *f0, *f1, *y, *yb;
  long ntp;
};
__host__ __device__ inline long padded_traces(long ntr) { return (ntr + 31) / 32 * 32; }
template <int NW>
__device__ __forceinline__ FactorLayout factor_layout(const SprayBufs& bf, const SecDesc& s) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  FactorLayout f;
  f.ntp = padded_traces((long)s.n2 * s.n3);
  const long plane = (long)s.n1 * f.ntp;
  f.taps = bf.scr + s.sc0;
  f.f0 = f.taps + NA * plane;
  f.f1 = f.f0 + (NB + 1) * plane;
  f.y = f.f1 + (NB + 1) * plane;
  f.yb = f.y + 2 * plane;
  return f;
}

// The section of padded trace g and its trace q there (q >= n2 n3 is
// padding).  The padded numbering takes the sections longest traces first
// (position k holds section secs[k].cord), so that the long chains start
// in the first waves and the short ones fill the last.
__device__ __forceinline__ const SecDesc& padded_section(const SprayB& b, long g, long& q) {
  const int k = find_section(b.nsec, g, [&](int p) { return b.secs[b.secs[p].cord].tp0; });
  const SecDesc& s = b.secs[b.secs[k].cord];
  q = g - s.tp0;
  return s;
}

// Taps and factors of every trace of the batch.  SPLIT: thread per (padded
// trace, filter orientation), each warp 32 consecutive traces of one
// orientation (batches of few traces, where a thread per trace would leave
// SMs idle); otherwise thread per padded trace with both orientations
// sharing the taps.
template <int NW, bool SPLIT>
__global__ void k_spray2_factor(const float* __restrict__ dip, SprayBufs bf, SprayB b, ApCoef c) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int side = SPLIT ? (int)((t >> 5) & 1) : 0;
  const long g = SPLIT ? (t >> 6) * 32 + (t & 31) : t;
  if (g >= b.ntp) return;
  long q;
  const SecDesc& s = padded_section(b, g, q);
  if (q >= (long)s.n2 * s.n3) return;
  const FactorLayout f = factor_layout<NW>(bf, s);
  PredictFactor F{f.taps + q, f.f0 + q, f.f1 + q, f.ntp};
  if (SPLIT)
    predict_factor<NW>(s.n1, b.eps, b.eps2, c, dip + s.off + q * s.n1, F, side);
  else
    predict_factor_pair<NW>(s.n1, b.eps, b.eps2, c, dip + s.off + q * s.n1, F);
}

// Forward spray with the stored factors.  Chains are numbered so that each
// warp holds 32 consecutive (padded) source traces of one section and one
// direction (whole-line factor and scratch accesses).  MODE 0: data only into u; MODE 1: data and
// the trace of ones together (u and u1); MODE 2: ones only into u1.
template <int NW, int MODE, typename IX = long>
__global__ void __launch_bounds__(64, 10) k_spray2_apply(const float* __restrict__ in, const float* __restrict__ ones,
                               SprayBufs bf, SprayB b) {
  extern __shared__ float apply_ring[];  // kApplyStages x apply_elems(NW) per thread
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int dir = (int)((t >> 5) & 1);
  const long g = (t >> 6) * 32 + (t & 31);
  if (g >= b.ntp) return;
  long q;
  const SecDesc& s = padded_section(b, g, q);
  if (q >= (long)s.n2 * s.n3) return;
  const int n1 = s.n1, n2 = s.n2;
  const int i = (int)(q % n2);
  const long i3 = q / n2;
  const long n12 = (long)n1 * n2;
  const long slice_u = s.u0 + i3 * n2 * (long)b.np * n1;
  float* U = (MODE == 2 ? bf.u1 : bf.u) + slice_u;
  float* U1 = MODE == 1 ? bf.u1 + slice_u : nullptr;
  const float* src = MODE == 2 ? ones : in + s.off + i3 * n12 + (long)i * n1;
  const FactorLayout f = factor_layout<NW>(bf, s);
  const long cl = dir * f.ntp + q, yss = 2 * f.ntp;
  auto slot = [&](float* base, int k, int sl) { return base + ((long)k * b.np + sl) * n1; };
  const int ns = b.ns;
  if (dir == 0) {
    float* cen = slot(U, i, ns);
    for (int i1 = 0; i1 < n1; i1++) cen[i1] = src[i1];
    if (MODE == 1) {
      float* cen1 = slot(U1, i, ns);
      for (int i1 = 0; i1 < n1; i1++) cen1[i1] = 1.0f;
    }
  }
  // the first step reads the source trace (and the ones); later steps read
  // the previous prediction from the chain's interleaved scratch
  const float* prev = src;
  const float* prevb = ones;
  IX ps = 1;
  for (int is = 0; is < ns; is++) {
    // dir 0 predicts forward to trace i-is-1 with its own slopes (forw=false);
    // dir 1 predicts backward to trace i+is+1 with the slopes of ip-1.
    const int ip = dir == 0 ? i - is - 1 : i + is + 1;
    if (ip < 0 || ip >= n2) break;
    const int sl = dir == 0 ? ns - is - 1 : ns + is + 1;
    const long tk = i3 * n2 + (dir == 0 ? ip : ip - 1);
    const float* fac = (dir == 0 ? f.f0 : f.f1) + tk;
    float* out = slot(U, ip, sl);
    if (MODE == 1) {
      float* outb = slot(U1, ip, sl);
      predict_apply<NW, true, IX>(n1, b.eps2, f.taps + tk, fac, (IX)f.ntp, dir == 1, prev, ps,
                                  out, f.y + cl, f.yb + cl, (IX)yss, apply_ring + threadIdx.x,
                                  blockDim.x, prevb, ps, outb);
      prevb = f.yb + cl;
    } else {
      predict_apply<NW, false, IX>(n1, b.eps2, f.taps + tk, fac, (IX)f.ntp, dir == 1, prev, ps,
                                   out, f.y + cl, nullptr, (IX)yss, apply_ring + threadIdx.x,
                                   blockDim.x);
    }
    prev = f.y + cl;
    ps = (IX)yss;
  }
}

// pwsmooth weights w[is] = ns+1-|is-ns| (pwsmooth_init :1055-1058).
__device__ __forceinline__ float tri_weight(int is, int ns) {
  int a = is - ns;
  return (float)(ns + 1 - (a >= 0 ? a : -a));
}

struct TileRange {
  int sec;
  long lo, hi;
};
__device__ __forceinline__ TileRange tile_range(const SprayB& b, int t) {
  TileRange r;
  r.sec = b.tile_sec[t];
  const SecDesc& s = b.secs[r.sec];
  r.lo = (long)(t - s.tile0) * kTile;
  r.hi = min(s.n, r.lo + kTile);
  return r;
}

// pwsmooth_set :1102-1122 and pwsmooth_lop forward :1088-1098: w1 = 1 /
// (weighted spray of ones) (0 where 0), smooth = sum_is u*w[is]*w1.
// store_w1: 0 compute w1, 1 compute and store it, 2 read the stored w1.
__global__ void k_weighted_mean(SprayBufs bf, float* __restrict__ out, SprayB b, int store_w1,
                                int mean) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  for (long j = tr.lo + threadIdx.x; j < tr.hi; j += blockDim.x) {
    const unsigned jj = (unsigned)j;  // sections hold fewer than 2^31 samples
    const long trc = jj / (unsigned)s.n1;
    const int i1 = (int)(jj % (unsigned)s.n1);
    const long po = s.u0 + trc * b.np * (long)s.n1 + i1;
    float ws;
    if (store_w1 == 2) {
      ws = bf.w1[s.off + j];
    } else {
      float acc = 0.f;
      for (int is = 0; is < b.np; is++)
        acc = __fadd_rn(acc, __fmul_rn(__fmul_rn(bf.u1[po + (long)is * s.n1],
                                                 tri_weight(is, b.ns)), 1.0f));
      // 1.0/t in double rounded to float equals the float quotient
      ws = (acc != 0.f) ? __fdiv_rn(1.0f, acc) : 0.f;
      if (store_w1) bf.w1[s.off + j] = ws;
    }
    if (mean) {
      float m = 0.f;
      for (int is = 0; is < b.np; is++)
        m = __fadd_rn(m, __fmul_rn(__fmul_rn(bf.u[po + (long)is * s.n1], tri_weight(is, b.ns)), ws));
      out[s.pout + j] = m;
    }
  }
}

// mf centre row (sof_cfuns.c:1294-1332 via csomf2d :1623-1649).  WARP:
// one warp per output sample (windows longer than kNetWin), else one thread.
template <bool WARP>
__global__ void k_median_tiles(const float* __restrict__ u, float* __restrict__ out, SprayB b,
                               int nmf) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const int m = (nmf - 1) / 2, c = (b.np - 1) / 2;
  const int lane = threadIdx.x & 31;
  const long first = WARP ? (threadIdx.x >> 5) : threadIdx.x;
  const long step = WARP ? (blockDim.x >> 5) : blockDim.x;
  for (long j = tr.lo + first; j < tr.hi; j += step) {
    const unsigned jj = (unsigned)j;
    const long trc = jj / (unsigned)s.n1;
    const int i1 = (int)(jj % (unsigned)s.n1);
    const float* col = u + s.u0 + trc * b.np * (long)s.n1 + i1;
    if (WARP) {
      const float r = select_warp(col, s.n1, c - m, b.np, nmf, m);
      if (lane == 0) out[s.pout + j] = r;
    } else {
      out[s.pout + j] = select_thread(col, s.n1, c - m, b.np, nmf, m);
    }
  }
}

// Adjoint of the weighted mean (pwsmooth_lop adjoint :1072-1086 with
// pwspray_lop adjoint :957-989) on the stored factors.  For output trace i
// the reference runs two chains: over ip = i+ns .. i+1 (slot ns + is + 1,
// the prediction with the slopes of ip - 1, forw = true) and over ip = i-ns
// .. i-1 (slot ns - is - 1, slopes of ip, forw = false), each adding x w[slot]
// w1 of trace ip to its running trace and then applying the adjoint
// prediction.  Here a thread runs one chain (direction 1 the first, 0 the
// second), numbered as the forward chains (a warp holds 32 consecutive traces
// of one direction, so the interleaved factor, trace and scratch accesses are
// whole lines), and leaves its trace in its column of the yb scratch;
// k_somean2d_adj_sum then adds the two and the centre term in the
// reference's order.
template <int NW>
__global__ void __launch_bounds__(64) k_somean2d_adj_chains(const float* __restrict__ x,
                                                            SprayBufs bf, SprayB b) {
  const long t = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const int dir = (int)((t >> 5) & 1);
  const long g = (t >> 6) * 32 + (t & 31);
  if (g >= b.ntp) return;
  long q;
  const SecDesc& s = padded_section(b, g, q);
  if (q >= (long)s.n2 * s.n3) return;
  const int n1 = s.n1, n2 = s.n2;
  const int i = (int)(q % n2);
  const long i3 = q / n2;
  const long n12 = (long)n1 * n2;
  const float* X = x + s.off + i3 * n12;
  const float* W = bf.w1 + s.off + i3 * n12;
  const FactorLayout f = factor_layout<NW>(bf, s);
  const long cl = dir * f.ntp + q, yss = 2 * f.ntp;
  float* tr = f.yb + cl;
  float* ys = f.y + cl;
  for (int i1 = 0; i1 < n1; i1++) tr[(long)i1 * yss] = 0.f;
  for (int is = b.ns - 1; is >= 0; is--) {
    const int ip = dir == 1 ? i + is + 1 : i - is - 1;
    if (ip < 0 || ip >= n2) continue;
    const float wv = tri_weight(dir == 1 ? b.ns + is + 1 : b.ns - is - 1, b.ns);
    for (int i1 = 0; i1 < n1; i1++) {
      const long e = (long)ip * n1 + i1;
      tr[(long)i1 * yss] =
          __fadd_rn(tr[(long)i1 * yss], __fmul_rn(__fmul_rn(X[e], wv), W[e]));
    }
    const long tk = i3 * n2 + (dir == 1 ? ip - 1 : ip);
    predict_adj_stored<NW>(n1, b.eps2, f.taps + tk, (dir == 1 ? f.f1 : f.f0) + tk, f.ntp,
                           dir == 1, tr, ys, yss);
  }
}

// out = ((add ? out : 0) + adjoint of direction 1) + adjoint of direction
// 0, then the centre term x w[ns] w1, per sample (the reference's order).
// add != 0: the terms are added into `out` as it stands (the adjoint with
// add = true, as the sparse-data interpolation's CG applies it,
// soint2d_cfuns.c:2194-2220) instead of into zeros.
template <int NW>
__global__ void k_somean2d_adj_sum(const float* __restrict__ x, float* __restrict__ out,
                                   SprayBufs bf, SprayB b, int add) {
  const TileRange tr = tile_range(b, blockIdx.x);
  const SecDesc& s = b.secs[tr.sec];
  const FactorLayout f = factor_layout<NW>(bf, s);
  const long yss = 2 * f.ntp;
  const float wc = tri_weight(b.ns, b.ns);
  for (long j = tr.lo + threadIdx.x; j < tr.hi; j += blockDim.x) {
    const unsigned jj = (unsigned)j;  // sections hold fewer than 2^31 samples
    const long q = jj / (unsigned)s.n1;
    const int i1 = (int)(jj % (unsigned)s.n1);
    const float t1 = f.yb[(long)i1 * yss + f.ntp + q], t0 = f.yb[(long)i1 * yss + q];
    float* o = out + s.pout + j;
    const float v = __fadd_rn(__fadd_rn(add ? *o : 0.f, t1), t0);
    *o = __fadd_rn(v, __fmul_rn(__fmul_rn(x[s.off + j], wc), bf.w1[s.off + j]));
  }
}

__global__ void k_tile_map(const SecDesc* secs, int nsec, int ntiles, int* tile_sec) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntiles) return;
  tile_sec[t] = find_section(nsec, (long)t, [&](int k) { return (long)secs[k].tile0; });
}

__global__ void k_put_single(SecDesc* dst, SecDesc v) { *dst = v; }

__global__ void k_fill(float* x, float v, long n) {
  long i = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (i < n) x[i] = v;
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
enum Filter { kMean = 1, kMeanAdj = 2, kMedian = 3, kMeanAdjAdd = 4 };

struct SprayLayout {
  int ntiles;
  long ntr, ntp, nu, nscr, n1max, nsamp;
};

SprayLayout layout2(std::vector<SecDesc>& secs, int ns, int order) {
  SprayLayout L{};
  const int np = 2 * ns + 1, nb = 2 * order;
  long u = 0, sc = 0, tr = 0, tp = 0, samp = 0;
  int tiles = 0;
  for (auto& s : secs) {
    s.n = (long)s.n1 * s.n2 * s.n3;
    s.tile0 = tiles;
    s.ntile = (int)((s.n + kTile - 1) / kTile);
    tiles += s.ntile;
    s.tr0 = tr;
    tr += (long)s.n2 * s.n3;
    s.u0 = u;
    u += s.n * np;
    s.sc0 = sc;
    const long pplane = (long)s.n1 * padded_traces((long)s.n2 * s.n3);
    // factor store + chain scratch (padded traces); every section's store
    // starts on a 128-byte boundary
    sc += (long)(2 * order + 1 + 2 * (nb + 1)) * pplane + 4 * pplane;
    sc = (sc + 31) / 32 * 32;
    samp = std::max(samp, s.off + s.n);
    L.n1max = std::max(L.n1max, (long)s.n1);
  }
  // padded chain numbering: sections by decreasing trace length
  std::vector<int> ord(secs.size());
  for (size_t k = 0; k < ord.size(); k++) ord[k] = (int)k;
  std::stable_sort(ord.begin(), ord.end(),
                   [&](int a, int c) { return secs[a].n1 > secs[c].n1; });
  for (size_t k = 0; k < ord.size(); k++) {
    SecDesc& s = secs[ord[k]];
    s.tp0 = tp;
    tp += padded_traces((long)s.n2 * s.n3);
    secs[k].cord = ord[k];
  }
  L.ntiles = tiles;
  L.ntr = tr;
  L.ntp = tp;
  L.nu = u;
  L.nscr = sc;
  L.nsamp = samp;
  return L;
}

struct SprayWork {
  SprayBufs bf;
  float* ones;
  float *v2, *avg;
  SecDesc* secs;
  int* tile_sec;
};

// shared: the layout of the smoothing calls of the sparse-data
// interpolation, the same for the forward and the adjoint mean, so that the
// factor store and the normalisation w1 one call leaves in the workspace
// serve the next calls on the same slopes.
SprayWork carve2(void* ws, const SprayLayout& L, int nsec, int filter, int option,
                 size_t* total, bool shared = false) {
  Carver cv(ws);
  SprayWork w{};
  const bool adj = filter == kMeanAdj || filter == kMeanAdjAdd;
  const bool mean = filter == kMean || adj;
  w.bf.scr = cv.take<float>(std::max(L.nscr, 1L));
  w.bf.w1 = adj || (shared && mean) ? cv.take<float>(L.nsamp) : nullptr;
  w.bf.u = adj && !shared ? nullptr : cv.take<float>(L.nu);
  w.bf.u1 = mean ? cv.take<float>(L.nu) : nullptr;
  w.ones = cv.take<float>(L.n1max);
  const bool svmf = filter == kMedian && option != 1;
  w.v2 = svmf ? cv.take<float>(L.nu) : nullptr;
  w.avg = svmf ? cv.take<float>(L.ntr) : nullptr;
  w.secs = cv.take<SecDesc>(nsec);
  w.tile_sec = cv.take<int>(L.ntiles);
  *total = cv.size();
  return w;
}

// reuse (the shared layout only): bit 0, the factor store is in place (the
// previous call factored the same slopes in this workspace); bit 1, so is
// w1, the normalisation of the mean (1 / the weighted spray of ones).
template <int NW>
int spray2_run(const float* data, const float* dip, float* out, int filter, int option, int nmf,
               const std::vector<SecDesc>& secs, const SprayLayout& L, const SprayWork& w,
               int ns, float eps, cudaStream_t st, int reuse = 0) {
  const int nsec = (int)secs.size();
  const ApCoef c = make_apcoef(NW);
  SprayB b{w.secs, w.tile_sec, nsec, L.ntiles, L.ntr, L.ntp, ns, 2 * ns + 1, eps * eps, eps * eps};
  // tuning knobs (environment): threads per block of the chain kernels
  // (PWD_SPRAY_BLOCK 32 or 64) and the factor kernel's form (PWD_SPRAY_SPLIT
  // 1: a thread per filter orientation, 0: per trace, unset: by the wave count)
  const char* eb = getenv("PWD_SPRAY_BLOCK");
  const int bs = (eb && atoi(eb) == 32) ? 32 : 64;
  const char* esp = getenv("PWD_SPRAY_SPLIT");
  const int split = esp ? (atoi(esp) != 0) : -1;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_tile_map<<<(unsigned)((L.ntiles + 255) / 256), 256, 0, st>>>(w.secs, nsec, L.ntiles, w.tile_sec));
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_fill<<<(unsigned)((L.n1max + 255) / 256), 256, 0, st>>>(w.ones, 1.0f, L.n1max));
  // slots whose source lies outside the section stay 0 (pwspray_lop :995)
  const bool have_w1 = (reuse & 2) && w.bf.w1;
  if (w.bf.u && cudaMemsetAsync(w.bf.u, 0, sizeof(float) * L.nu, st) != cudaSuccess)
    return PWD_ECUDA;
  if (w.bf.u1 && !have_w1 && cudaMemsetAsync(w.bf.u1, 0, sizeof(float) * L.nu, st) != cudaSuccess)
    return PWD_ECUDA;
  const unsigned gap = (unsigned)((2 * L.ntp + bs - 1) / bs);
  const size_t ring = sizeof(float) * kApplyStages * apply_elems(NW) * bs;
  // 32-bit element offsets in the chains when every section's factor store
  // (2 NW + 1 planes of n1 x padded traces, the largest group) allows them
  bool i32 = true;
  for (const SecDesc& s : secs)
    if ((long)(2 * NW + 1) * s.n1 * padded_traces((long)s.n2 * s.n3) >= (1L << 31)) i32 = false;
  auto apply = [&](auto mode) {
    constexpr int M = decltype(mode)::value;
    if (i32)
      PWD_KERNEL(PWD_FAM_SPRAY, st,
                 (k_spray2_apply<NW, M, int><<<gap, bs, ring, st>>>(data, w.ones, w.bf, b)));
    else
      PWD_KERNEL(PWD_FAM_SPRAY, st,
                 (k_spray2_apply<NW, M, long><<<gap, bs, ring, st>>>(data, w.ones, w.bf, b)));
  };
  // a thread per filter orientation when even then the factor launch fills
  // less than one wave (a thread per trace then leaves SMs idle); otherwise
  // a thread per trace, its two factors sharing the taps
  int dev = 0, sms = 1, per = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_spray2_factor<NW, true>, bs, 0);
  if (reuse & 1) {
    // the factor store of the previous call on these slopes is in place
  } else if (split == 1 || (split < 0 && 2 * L.ntp <= (long)sms * per * bs)) {
    PWD_KERNEL(PWD_FAM_SPRAY, st,
               (k_spray2_factor<NW, true><<<(unsigned)((2 * L.ntp + bs - 1) / bs), bs, 0, st>>>(
                   dip, w.bf, b, c)));
  } else {
    PWD_KERNEL(PWD_FAM_SPRAY, st,
               (k_spray2_factor<NW, false><<<(unsigned)((L.ntp + bs - 1) / bs), bs, 0, st>>>(
                   dip, w.bf, b, c)));
  }
  if (filter == kMean && have_w1) {
    // the data alone, normalised by the stored w1
    apply(std::integral_constant<int, 0>());
    PWD_KERNEL(PWD_FAM_FILTER, st,
               k_weighted_mean<<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(w.bf, out, b, 2, 1));
  } else if (filter == kMean) {
    apply(std::integral_constant<int, 1>());
    PWD_KERNEL(PWD_FAM_FILTER, st,
               k_weighted_mean<<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(
                   w.bf, out, b, w.bf.w1 ? 1 : 0, 1));
  } else if (filter == kMeanAdj || filter == kMeanAdjAdd) {
    if (!have_w1) {
      apply(std::integral_constant<int, 2>());
      PWD_KERNEL(PWD_FAM_FILTER, st,
                 k_weighted_mean<<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(w.bf, out, b, 1,
                                                                               0));
    }
    // the adjoint chains on the stored factors, their traces and scratch in
    // the chain scratch of the factor store, then the per-sample sum
    PWD_KERNEL(PWD_FAM_SPRAY, st,
               k_somean2d_adj_chains<NW><<<(unsigned)((2 * L.ntp + 63) / 64), 64, 0, st>>>(
                   data, w.bf, b));
    PWD_KERNEL(PWD_FAM_FILTER, st,
               k_somean2d_adj_sum<NW><<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(
                   data, out, w.bf, b, filter == kMeanAdjAdd ? 1 : 0));
  } else {
    apply(std::integral_constant<int, 0>());
    if (option == 1) {
      if (nmf > kNetWin)
        PWD_KERNEL(PWD_FAM_FILTER, st,
                   k_median_tiles<true><<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(w.bf.u, out, b, nmf));
      else
        PWD_KERNEL(PWD_FAM_FILTER, st,
                   k_median_tiles<false><<<(unsigned)L.ntiles, kTileThreads, 0, st>>>(w.bf.u, out, b, nmf));
    } else {
      for (const SecDesc& s : secs) {  // svmf needs whole-panel means: per section
        int rc = launch_panel_median(w.bf.u + s.u0, out + s.pout, w.v2 + s.u0, w.avg + s.tr0,
                                     s.n1, b.np, (long)s.n2 * s.n3, nmf, option, st);
        if (rc != PWD_OK) return rc;
      }
    }
  }
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

int spray2_dispatch(int order, const float* data, const float* dip, float* out, int filter,
                    int option, int nmf, const std::vector<SecDesc>& secs, const SprayLayout& L,
                    const SprayWork& w, int ns, float eps, cudaStream_t st, int reuse = 0) {
  switch (order) {
    case 1: return spray2_run<1>(data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st, reuse);
    case 2: return spray2_run<2>(data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st, reuse);
    case 3: return spray2_run<3>(data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st, reuse);
    case 4: return spray2_run<4>(data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st, reuse);
  }
  return PWD_ENOTSUP;
}

int check2(int n1, int n2, int n3, int ns, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || ns < 0 || order < 1) return PWD_EINVAL;
  if ((long)n1 * n2 * n3 >= (1L << 31)) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  return PWD_OK;
}

std::vector<SecDesc> single(int n1, int n2, int n3) {
  std::vector<SecDesc> v(1, SecDesc{});
  v[0].n1 = n1;
  v[0].n2 = n2;
  v[0].n3 = n3;
  return v;
}

size_t need_single(int n1, int n2, int n3, int ns, int order, int filter, int option,
                   bool shared = false) {
  std::vector<SecDesc> secs = single(n1, n2, n3);
  SprayLayout L = layout2(secs, ns, order);
  size_t need = 0;
  carve2(nullptr, L, 1, filter, option, &need, shared);
  return need;
}

int run_single(const float* data, const float* dip, float* out, int n1, int n2, int n3, int ns,
               int order, float eps, int filter, int option, int nmf, void* ws, size_t wsb,
               cudaStream_t st, bool shared = false, int reuse = 0) {
  std::vector<SecDesc> secs = single(n1, n2, n3);
  SprayLayout L = layout2(secs, ns, order);
  size_t need = 0;
  carve2(nullptr, L, 1, filter, option, &need, shared);
  if (!ws || wsb < need || ((uintptr_t)ws & 255)) return PWD_EWORKSPACE;
  SprayWork w = carve2(ws, L, 1, filter, option, &need, shared);
  PWD_KERNEL(PWD_FAM_OTHER, st, k_put_single<<<1, 1, 0, st>>>(w.secs, secs[0]));
  return spray2_dispatch(order, data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st,
                         shared ? reuse : 0);
}

int batch_table2(const pwd_section* in, int nsec, std::vector<SecDesc>& secs) {
  if (!in || nsec < 1) return PWD_EINVAL;
  secs.assign(nsec, SecDesc{});
  for (int i = 0; i < nsec; i++) {
    if (check2(in[i].n1, in[i].n2, in[i].n3, 0, 1) != PWD_OK || in[i].offset < 0 ||
        in[i].out_offset < 0)
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

// The 2-D plane-wave smoothing of the n3 (n1, n2) slices of one section for
// the sparse-data interpolation (pwd_sint.cu): mode 0 gives out = S in (the
// weighted spray mean, as pwd_somean2d), mode 1 gives out += S' in, the
// adjoint adding its terms into out in the reference's order, and mode 2
// out = S' in (pwd_somean2d's adjoint).  `in` and `out` must not overlap.
// Every call leaves the slopes' factor store and w1 in the workspace.
size_t smooth2_workspace(int n1, int n2, int n3, int ns, int order) {
  if (check2(n1, n2, n3, ns, order) != PWD_OK) return 0;
  return std::max(need_single(n1, n2, n3, ns, order, kMean, 1, true),
                  need_single(n1, n2, n3, ns, order, kMeanAdjAdd, 1, true));
}

// reuse != 0: the previous smooth2_run call in this workspace was on the
// same slopes and sizes, so its factor store and w1 are used again.
int smooth2_run(const float* in, const float* dip, float* out, int n1, int n2, int n3, int ns,
                int order, float eps, int mode, void* ws, size_t wsb, cudaStream_t st,
                int reuse) {
  int rc = check2(n1, n2, n3, ns, order);
  if (rc != PWD_OK) return rc;
  const int filter = mode == 1 ? kMeanAdjAdd : (mode == 2 ? kMeanAdj : kMean);
  return run_single(in, dip, out, n1, n2, n3, ns, order, eps, filter, 1, 0, ws, wsb, st, true,
                    reuse ? 3 : 0);
}

}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_somean2d_workspace_size(int n1, int n2, int n3, int ns, int order) {
  if (check2(n1, n2, n3, ns, order) != PWD_OK) return 0;
  return std::max(need_single(n1, n2, n3, ns, order, kMean, 1),
                  need_single(n1, n2, n3, ns, order, kMeanAdj, 1));
}

extern "C" int pwd_somean2d(const float* data, const float* dip, float* out, int n1, int n2,
                            int n3, int ns, int order, int adj, float eps, void* workspace,
                            size_t workspace_bytes, pwd_stream_t stream) {
  int rc = check2(n1, n2, n3, ns, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip || !out) return PWD_EINVAL;
  return run_single(data, dip, out, n1, n2, n3, ns, order, eps, adj ? kMeanAdj : kMean, 1, 0,
                    workspace, workspace_bytes, (cudaStream_t)stream);
}

extern "C" size_t pwd_somf2d_workspace_size(int n1, int n2, int n3, int ns, int nmf, int option,
                                            int order) {
  if (check2(n1, n2, n3, ns, order) != PWD_OK || !median_args_ok(nmf, option)) return 0;
  return need_single(n1, n2, n3, ns, order, kMedian, option);
}

extern "C" int pwd_somf2d(const float* data, const float* dip, float* out, int n1, int n2, int n3,
                          int ns, int nmf, int option, int order, float eps, void* workspace,
                          size_t workspace_bytes, pwd_stream_t stream) {
  int rc = check2(n1, n2, n3, ns, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip || !out) return PWD_EINVAL;
  if (!median_args_ok(nmf, option)) return nmf < 1 ? PWD_EINVAL : PWD_ENOTSUP;
  return run_single(data, dip, out, n1, n2, n3, ns, order, eps, kMedian, option, nmf, workspace,
                    workspace_bytes, (cudaStream_t)stream);
}

extern "C" size_t pwd_sofilter2d_batch_workspace_size(const pwd_section* sections, int nsec,
                                                      int ns, int order, int filter, int nmf,
                                                      int option) {
  std::vector<SecDesc> secs;
  if (ns < 0 || order < 1 || order > PWD_MAX_ORDER || filter < 1 || filter > 3) return 0;
  if (filter == kMedian && !median_args_ok(nmf, option)) return 0;
  if (batch_table2(sections, nsec, secs) != PWD_OK) return 0;
  SprayLayout L = layout2(secs, ns, order);
  size_t need = 0;
  carve2(nullptr, L, nsec, filter, option, &need);
  return need;
}

extern "C" int pwd_sofilter2d_batch(const float* data, const float* dip, float* out,
                                    const pwd_section* sections, int nsec, int ns, int order,
                                    int filter, int nmf, int option, float eps, void* workspace,
                                    size_t workspace_bytes, pwd_stream_t stream) {
  if (!data || !dip || !out || ns < 0 || order < 1 || filter < 1 || filter > 3) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER) return PWD_ENOTSUP;
  if (filter == kMedian && !median_args_ok(nmf, option)) return nmf < 1 ? PWD_EINVAL : PWD_ENOTSUP;
  std::vector<SecDesc> secs;
  int rc = batch_table2(sections, nsec, secs);
  if (rc != PWD_OK) return rc;
  SprayLayout L = layout2(secs, ns, order);
  size_t need = 0;
  carve2(nullptr, L, nsec, filter, option, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  SprayWork w = carve2(workspace, L, nsec, filter, option, &need);
  cudaStream_t st = (cudaStream_t)stream;
  if (cudaMemcpyAsync(w.secs, secs.data(), sizeof(SecDesc) * nsec, cudaMemcpyHostToDevice, st) !=
      cudaSuccess)
    return PWD_ECUDA;
  return spray2_dispatch(order, data, dip, out, filter, option, nmf, secs, L, w, ns, eps, st);
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
