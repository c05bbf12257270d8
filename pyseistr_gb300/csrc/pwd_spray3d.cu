// 3-D plane-wave spray over the (2r1+1)x(2r2+1) offset grid with the
// structure-oriented mean and median.
//
// Restates csomean3d / csomf3d (pyseistr/src/sof3d_cfuns.c:1355-1753) with
// update_init/get_update (:980-1056).  Each source trace's spray is a tree
// over the offset grid visited by increasing distance, every cell predicted
// from one or two already-predicted neighbours (predict1_step /
// predict2_step).  A cell's neighbours are strictly closer to the source, so
// the cells of one distance (a level) are independent: a group of lanes runs
// one source's tree, one cell of the current level per lane, the levels in
// order with a warp barrier between them.  The visit table and its levels
// depend only on (r1, r2) and are built on the host and passed by value.
#include <algorithm>
#include <cmath>
#include <vector>

#include "pwd_median.cuh"
#include "pwd_predict.cuh"

namespace pwd {
namespace {

constexpr int kMaxR = 10;
constexpr int kMaxCells = (2 * kMaxR + 1) * (2 * kMaxR + 1);

struct Visit3 {
  int np, np2, np3, ns2, ns3;
  int nlev, maxlev;             // levels of equal distance, largest level
  short jp[kMaxCells];
  unsigned char fl[kMaxCells];  // bits 0-1 update, bit 2 up2, bit 3 up3
  short lev0[kMaxCells + 1];    // first visit index of each level
};

// update_init + get_update, evaluated once per cell.
Visit3 make_visit(int ns2, int ns3) {
  Visit3 v;
  v.ns2 = ns2;
  v.ns3 = ns3;
  v.np2 = 2 * ns2 + 1;
  v.np3 = 2 * ns3 + 1;
  v.np = v.np2 * v.np3;
  std::vector<float> t0(v.np);
  for (int i3 = 0; i3 < v.np3; i3++)
    for (int i2 = 0; i2 < v.np2; i2++)
      t0[i3 * v.np2 + i2] = hypotf((float)(i2 - ns2), (float)(i3 - ns3));
  std::vector<int> visit(v.np);
  for (int i = 0; i < v.np; i++) visit[i] = i;
  // Cells of equal distance never precede one another, so any order
  // sorted by distance gives the same spray.
  std::stable_sort(visit.begin(), visit.end(), [&](int a, int b) { return t0[a] < t0[b]; });
  const int un1 = v.np2, un2 = v.np3;
  for (int i = 0; i < v.np; i++) {
    int j = visit[i];
    float t1 = t0[j];
    int i1 = j % un1, i2 = j / un1;
    int update = 0;
    bool up1 = false, up2 = false;
    if (un1 > 1) {
      int a1 = j - 1, b1 = j + 1;
      up1 = (i1 && (i1 == un1 - 1 || !(t0[a1] > t0[b1])));
      int c1 = up1 ? a1 : b1;
      if (t1 > t0[c1]) update |= 1;
    }
    if (un2 > 1) {
      int a2 = j - un1, b2 = j + un1;
      up2 = (i2 && (i2 == un2 - 1 || !(t0[a2] > t0[b2])));
      int c2 = up2 ? a2 : b2;
      if (t1 > t0[c2]) update |= 2;
    }
    v.jp[i] = (short)j;
    v.fl[i] = (unsigned char)(update | (up1 ? 4 : 0) | (up2 ? 8 : 0));
  }
  // levels: runs of equal distance in the visit order (a neighbour used by
  // get_update is strictly closer, so it lies in an earlier level)
  v.nlev = 0;
  v.maxlev = 0;
  for (int i = 0; i < v.np; i++)
    if (i == 0 || t0[visit[i]] != t0[visit[i - 1]]) v.lev0[v.nlev++] = (short)i;
  v.lev0[v.nlev] = (short)v.np;
  for (int l = 0; l < v.nlev; l++) v.maxlev = std::max(v.maxlev, v.lev0[l + 1] - v.lev0[l]);
  return v;
}

// Lanes per source: the largest level rounded up to a power of two, at
// least 4 (levels hold at most 16 cells for radii up to kMaxR).
int spray3_lanes(const Visit3& v) {
  int l = 4;
  while (l < v.maxlev) l *= 2;
  return l;
}

struct Spray3 {
  int n1, n2, n3;
  float eps, eps2;
};

// Factor once.  A cell of a tree predicts its target trace j from one or
// two neighbours; the band matrix of that prediction (regularization plus
// pwd_define of the filters used) depends only on j and on which
// neighbours, not on the source, so it is factored once per call for every
// target and every variant:
//   0, 1: from the neighbour along axis 2 below / above (slopes p1 of j-1,
//         reversed filter / slopes p1 of j),
//   2, 3: the same along axis 3 (slopes p2 of j-n2 / p2 of j),
//   4 + a + 2b: both, a = 0 below along axis 2, b = 0 below along axis 3.
// The taps of both slope fields are stored once too.  Stores (trace-major,
// contiguous along the trace): taps[dim][trace][NA][n1], factors
// [variant][trace][NB+1][n1] (o[0..NB) then d).
struct Spray3Store {
  float* taps;
  float* fac;
};
__host__ __device__ inline int spray3_variant(int update, bool up2, bool up3) {
  if (update == 1) return up2 ? 0 : 1;
  if (update == 2) return up3 ? 2 : 3;
  return 4 + (up2 ? 0 : 1) + (up3 ? 0 : 2);
}

// passfilter taps of both slope fields: thread per (field, trace, sample).
template <int NW>
__global__ void k_spray3_taps(const float* __restrict__ p1, const float* __restrict__ p2,
                              Spray3Store st, Spray3 s, ApCoef c) {
  constexpr int NA = 2 * NW + 1;
  const long n23 = (long)s.n2 * s.n3, n = (long)s.n1 * n23;
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (g >= 2 * n) return;
  const int dim = g >= n;
  const long e = g - dim * n, tr = e / s.n1;
  const int i = (int)(e - tr * s.n1);
  float t[NA];
  passfilter<NW>(c, (dim ? p2 : p1)[e], t);
  float* dst = st.taps + ((dim * n23 + tr) * NA) * s.n1 + i;
#pragma unroll
  for (int j = 0; j < NA; j++) dst[(long)j * s.n1] = t[j];
}

// Filter column k of a slope trace's stored taps (reversed for forw).
template <int NW>
__device__ __forceinline__ void stored_column(const float* __restrict__ taps, int n1, int k,
                                              bool forw, float* col) {
  constexpr int NA = 2 * NW + 1;
#pragma unroll
  for (int j = 0; j < NA; j++) {
    const float v = taps[(long)j * n1 + k];
    col[forw ? NA - 1 - j : j] = v;
  }
}

// The LDL' factor of one (target, variant): the band and factor steps of
// predict_fwd with the same filters, in the same order.
template <int NW>
__global__ void k_spray3_factor(Spray3Store st, Spray3 s) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  const long n23 = (long)s.n2 * s.n3;
  const long g = blockIdx.x * (long)blockDim.x + threadIdx.x;
  if (g >= 8 * n23) return;
  const int v = (int)(g / n23);
  const long j = g - v * n23;
  const int j2 = (int)(j % s.n2), j3 = (int)(j / s.n2);
  const bool use2 = v <= 1 || v >= 4, use3 = (v >= 2 && v <= 3) || v >= 4;
  const bool up2 = v == 0 || (v >= 4 && ((v - 4) & 1) == 0);
  const bool up3 = v == 2 || (v >= 4 && ((v - 4) & 2) == 0);
  if (use2 && (up2 ? j2 == 0 : j2 == s.n2 - 1)) return;  // never used
  if (use3 && (up3 ? j3 == 0 : j3 == s.n3 - 1)) return;
  const int n1 = s.n1;
  // taps of the first filter (axis 2 if used, else axis 3) and the second
  const long k2 = up2 ? j - 1 : j, k3 = up3 ? j - s.n2 : j;
  const float* ta = use2 ? st.taps + k2 * NA * n1 : st.taps + (n23 + k3) * NA * n1;
  const bool fa = use2 ? up2 : up3;
  const float* tb = st.taps + (n23 + k3) * NA * n1;
  const bool two = v >= 4;
  float* out = st.fac + ((long)v * n23 + j) * (NB + 1) * n1;
  const RegConst rc = reg_const(s.eps, s.eps2);
  FilterWin<NW> w1, w2;
  float O[NB][NB], D[NB];
#pragma unroll
  for (int cc = 0; cc < NA; cc++)
#pragma unroll
    for (int q = 0; q < NA; q++) {
      w1.a[cc][q] = 0.f;
      w2.a[cc][q] = 0.f;
    }
#pragma unroll
  for (int m = 0; m < NB; m++) {
    D[m] = 0.f;
#pragma unroll
    for (int q = 0; q < NB; q++) O[m][q] = 0.f;
  }
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) {
      stored_column<NW>(ta, n1, cc, fa, w1.a[NW + 1 + cc]);
      if (two) stored_column<NW>(tb, n1, cc, up3, w2.a[NW + 1 + cc]);
    }
  for (int i = 0; i < n1; i++) {
    const int cn = i + NW;
    shift_win<NW>(w1);
    if (two) shift_win<NW>(w2);
    if (cn < n1) {
      stored_column<NW>(ta, n1, cn, fa, w1.a[2 * NW]);
      if (two) stored_column<NW>(tb, n1, cn, up3, w2.a[2 * NW]);
    } else {
#pragma unroll
      for (int q = 0; q < NA; q++) {
        w1.a[2 * NW][q] = 0.f;
        w2.a[2 * NW][q] = 0.f;
      }
    }
    float diag, offd[NB];
    reg_row<NB>(i, n1, rc, diag, offd);
    band_add<NW>(w1, i, n1, diag, offd);
    if (two) band_add<NW>(w2, i, n1, diag, offd);
    float dk, ok[NB];
    ldl_row<NB>(i, n1, diag, offd, O, D, dk, ok);
#pragma unroll
    for (int m = 0; m < NB; m++) out[(long)m * n1 + i] = ok[m];
    out[(long)NB * n1 + i] = dk;
#pragma unroll
    for (int m = NB - 1; m > 0; m--) {
      D[m] = D[m - 1];
#pragma unroll
      for (int q = 0; q < NB; q++) O[m][q] = O[m - 1][q];
    }
    D[0] = dk;
#pragma unroll
    for (int q = 0; q < NB; q++) O[0][q] = ok[q];
  }
}

// One cell's prediction (predict1_step / predict2_step) with the stored
// taps and factor: the operations of predict_fwd on the trace without its
// band and factor steps.  ta / tb: the taps of the filters' slope traces
// (reversed for forw), fac: the (target, variant) factor, ys: the lane's y
// scratch (element k at k*ss).
template <int NW, bool TWO>
__device__ void predict_apply3(int n1, float eps2, const float* __restrict__ in1,
                               const float* __restrict__ ta, bool forw1,
                               const float* __restrict__ in2, const float* __restrict__ tb,
                               bool forw2, const float* __restrict__ fac,
                               float* __restrict__ out, float* __restrict__ ys, long ss) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  FilterWin<NW> w1, w2;
  float x1[NA], x2[NA], t1[NA], t2[NA], Y[NB];
#pragma unroll
  for (int cc = 0; cc < NA; cc++) {
    t1[cc] = 0.f;
    t2[cc] = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) {
      w1.a[cc][j] = 0.f;
      if (TWO) w2.a[cc][j] = 0.f;
    }
  }
#pragma unroll
  for (int m = 0; m < NB; m++) Y[m] = 0.f;
#pragma unroll
  for (int cc = 0; cc < NW; cc++)
    if (cc < n1) {
      stored_column<NW>(ta, n1, cc, forw1, w1.a[NW + 1 + cc]);
      if (TWO) stored_column<NW>(tb, n1, cc, forw2, w2.a[NW + 1 + cc]);
    }
#pragma unroll
  for (int q = 0; q < NB; q++) {
    x1[q + 1] = q < n1 ? in1[q] : 0.f;
    if (TWO) x2[q + 1] = q < n1 ? in2[q] : 0.f;
  }
  float b0, b1, b2, b3;  // boundary values t0..t3
  if (TWO) {
    b0 = __fmul_rn(0.5f, __fadd_rn(in1[0], in2[0]));
    b1 = __fmul_rn(0.5f, __fadd_rn(in1[1], in2[1]));
    b2 = __fmul_rn(0.5f, __fadd_rn(in1[n1 - 2], in2[n1 - 2]));
    b3 = __fmul_rn(0.5f, __fadd_rn(in1[n1 - 1], in2[n1 - 1]));
  } else {
    b0 = in1[0];
    b1 = in1[1];
    b2 = in1[n1 - 2];
    b3 = in1[n1 - 1];
  }
  for (int i = 0; i < n1; i++) {
    const int cn = i + NW;
    shift_win<NW>(w1);
    if (TWO) shift_win<NW>(w2);
#pragma unroll
    for (int q = 0; q < NA - 1; q++) {
      x1[q] = x1[q + 1];
      t1[q] = t1[q + 1];
      if (TWO) {
        x2[q] = x2[q + 1];
        t2[q] = t2[q + 1];
      }
    }
    const int ln = i + 2 * NW;
    x1[NA - 1] = ln < n1 ? in1[ln] : 0.f;
    if (TWO) x2[NA - 1] = ln < n1 ? in2[ln] : 0.f;
    if (cn < n1) {
      stored_column<NW>(ta, n1, cn, forw1, w1.a[2 * NW]);
      if (TWO) stored_column<NW>(tb, n1, cn, forw2, w2.a[2 * NW]);
    } else {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        w1.a[2 * NW][j] = 0.f;
        if (TWO) w2.a[2 * NW][j] = 0.f;
      }
    }
    float s1 = 0.f, s2 = 0.f;
    if (cn >= NW && cn < n1 - NW) {
#pragma unroll
      for (int j = 0; j < NA; j++) {
        s1 = __fadd_rn(s1, __fmul_rn(w1.a[2 * NW][j], x1[j]));
        if (TWO) s2 = __fadd_rn(s2, __fmul_rn(w2.a[2 * NW][j], x2[j]));
      }
    }
    t1[NA - 1] = s1;
    if (TWO) t2[NA - 1] = s2;
    float o1 = 0.f, o2 = 0.f;
#pragma unroll
    for (int j = 0; j < NA; j++) {
      const int k = i + j - NW;
      if (k >= NW && k < n1 - NW) {
        o1 = __fadd_rn(o1, __fmul_rn(w1.a[j][j], t1[j]));
        if (TWO) o2 = __fadd_rn(o2, __fmul_rn(w2.a[j][j], t2[j]));
      }
    }
    float b = TWO ? __fadd_rn(o1, o2) : o1;
    if (i == 0) b = __fadd_rn(b, __fmul_rn(eps2, b0));
    if (i == 1) b = __fadd_rn(b, __fmul_rn(eps2, b1));
    if (i == n1 - 2) b = __fadd_rn(b, __fmul_rn(eps2, b2));
    if (i == n1 - 1) b = __fadd_rn(b, __fmul_rn(eps2, b3));
    // forward substitution with o[m][i-1-m] of the stored factor
    float y = b;
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < i) y = __fsub_rn(y, __fmul_rn(fac[(long)m * n1 + (i - 1 - m)], Y[m]));
    ys[(long)i * ss] = y;
#pragma unroll
    for (int m = NB - 1; m > 0; m--) Y[m] = Y[m - 1];
    Y[0] = y;
  }
  // back substitution: x[k] = y[k]/d[k] - sum_m o[m][k] x[k+m+1]
  float X[NB];
#pragma unroll
  for (int m = 0; m < NB; m++) X[m] = 0.f;
  for (int k = n1 - 1; k >= 0; k--) {
    float t = __fdiv_rn(ys[(long)k * ss], fac[(long)NB * n1 + k]);
#pragma unroll
    for (int m = 0; m < NB; m++)
      if (m < n1 - k - 1) t = __fsub_rn(t, __fmul_rn(fac[(long)m * n1 + k], X[m]));
#pragma unroll
    for (int m = NB - 1; m > 0; m--) X[m] = X[m - 1];
    X[0] = t;
    out[k] = t;
  }
}

// One source trace's spray tree (csomean3d :1466-1520) on lps lanes: lane
// k of the group predicts cell k of each level.  Every lane of a warp runs
// every level (lanes without a source or a cell only meet the barriers), so
// a cell's neighbours, predicted by other lanes of the group in earlier
// levels, are complete and visible when it reads them.
template <int NW>
__global__ void __launch_bounds__(128) k_spray3_tree(const float* __restrict__ din,
                                                     float* __restrict__ u, Spray3 s, Visit3 v,
                                                     Spray3Store st, float* __restrict__ ysc,
                                                     long ss, int lps) {
  constexpr int NA = 2 * NW + 1, NB = 2 * NW;
  const long n23 = (long)s.n2 * s.n3;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long i = gt / lps;
  const int lane = (int)(gt - i * lps);
  const bool src_ok = i < n23;
  const int n1 = s.n1, np = v.np, np2 = v.np2;
  float* ys = ysc + gt;  // one y scratch column per lane of the grid
  auto U = [&](long tr, int slot) { return u + (tr * np + slot) * (long)n1; };
  if (src_ok) {
    float* cen = U(i, v.ns3 * np2 + v.ns2);
    for (int j = lane; j < n1; j += lps) cen[j] = din[i * n1 + j];
  }
  __syncwarp();
  const int i2 = src_ok ? (int)(i % s.n2) : 0, i3 = src_ok ? (int)(i / s.n2) : 0;
  for (int lv = 0; lv < v.nlev; lv++) {
    const int ip = v.lev0[lv] + lane;
    if (src_ok && ip < v.lev0[lv + 1]) {
      const int jp = v.jp[ip];
      const int fl = v.fl[ip];
      const int update = fl & 3;
      const bool up2 = (fl & 4) != 0, up3 = (fl & 8) != 0;
      const int k2 = jp % np2, k3 = jp / np2;
      const int j2 = i2 + k2 - v.ns2, j3 = i3 + k3 - v.ns3;
      bool go = update != 0 && j2 >= 0 && j2 < s.n2 && j3 >= 0 && j3 < s.n3;
      const long j = j2 + (long)j3 * s.n2;
      long t2 = 0, t3 = 0;
      int s2 = 0, s3 = 0;
      // taps of the slope traces the filters use (p1 of j-1 or j, p2 of
      // j-n2 or j)
      const float *q2 = nullptr, *q3 = nullptr;
      if (go && (update & 1)) {
        if (up2) {
          if (j2 == 0) go = false;
          t2 = j - 1; q2 = st.taps + t2 * NA * n1; s2 = jp - 1;
        } else {
          if (j2 == s.n2 - 1) go = false;
          t2 = j + 1; q2 = st.taps + j * NA * n1; s2 = jp + 1;
        }
      }
      if (go && (update & 2)) {
        if (up3) {
          if (j3 == 0) go = false;
          t3 = j - s.n2; q3 = st.taps + (n23 + t3) * NA * n1; s3 = jp - np2;
        } else {
          if (j3 == s.n3 - 1) go = false;
          t3 = j + s.n2; q3 = st.taps + (n23 + j) * NA * n1; s3 = jp + np2;
        }
      }
      if (go) {
        float* trace = U(j, jp);
        const float* fac =
            st.fac + ((long)spray3_variant(update, up2, up3) * n23 + j) * (NB + 1) * n1;
        if (update == 1)
          predict_apply3<NW, false>(n1, s.eps2, U(t2, s2), q2, up2, nullptr, nullptr, false, fac,
                                    trace, ys, ss);
        else if (update == 2)
          predict_apply3<NW, false>(n1, s.eps2, U(t3, s3), q3, up3, nullptr, nullptr, false, fac,
                                    trace, ys, ss);
        else
          predict_apply3<NW, true>(n1, s.eps2, U(t2, s2), q2, up2, U(t3, s3), q3, up3, fac,
                                   trace, ys, ss);
      }
    }
    __syncwarp();
  }
}

struct Spray3Work {
  float *u, *v2, *avg;
  Spray3Store st;
  float* ys;  // y scratch of the tree's lanes, lane-interleaved (stride ss)
  long ss;
};

// Threads of the tree launch: LPS lanes per source, blocks of 128.
long spray3_threads(long n23, int lanes) { return (n23 * lanes + 127) / 128 * 128; }

Spray3Work carve_spray3(void* ws, int n1, int n2, int n3, int r1, int r2, int order,
                        bool need_svmf, size_t* total) {
  const long n23 = (long)n2 * n3;
  const int np = (2 * r1 + 1) * (2 * r2 + 1), nb = 2 * order;
  const long nthr = spray3_threads(n23, spray3_lanes(make_visit(r1, r2)));
  Carver cv(ws);
  Spray3Work w;
  w.u = cv.take<float>(n23 * np * n1);
  w.v2 = need_svmf ? cv.take<float>(n23 * np * n1) : nullptr;
  w.avg = need_svmf ? cv.take<float>(n23) : nullptr;
  w.st.taps = cv.take<float>(2L * (nb + 1) * n1 * n23);
  w.st.fac = cv.take<float>(8L * (nb + 1) * n1 * n23);
  w.ys = cv.take<float>((long)n1 * nthr);
  w.ss = nthr;
  *total = cv.size();
  return w;
}

int check3(int n1, int n2, int n3, int r1, int r2, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || r1 < 0 || r2 < 0 || order < 1) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER || r1 > kMaxR || r2 > kMaxR) return PWD_ENOTSUP;
  return PWD_OK;
}

// Taps, factors, then the trees.
template <int NW>
int spray3_run(const float* d, const float* p1, const float* p2, const Spray3Work& w,
               const Spray3& s, const Visit3& v, int lanes, cudaStream_t st) {
  const long n23 = (long)s.n2 * s.n3, n = (long)s.n1 * n23;
  PWD_KERNEL(PWD_FAM_SPRAY, st,
             k_spray3_taps<NW><<<(unsigned)((2 * n + 255) / 256), 256, 0, st>>>(
                 p1, p2, w.st, s, make_apcoef(NW)));
  PWD_KERNEL(PWD_FAM_SPRAY, st,
             k_spray3_factor<NW><<<(unsigned)((8 * n23 + 63) / 64), 64, 0, st>>>(w.st, s));
  const unsigned g = (unsigned)(spray3_threads(n23, lanes) / 128);
  PWD_KERNEL(PWD_FAM_SPRAY, st,
             k_spray3_tree<NW><<<g, 128, 0, st>>>(d, w.u, s, v, w.st, w.ys, w.ss, lanes));
  return PWD_OK;
}

int spray3(const float* d, const float* p1, const float* p2, const Spray3Work& w, int n1, int n2,
           int n3, int r1, int r2, int order, cudaStream_t st) {
  const long n23 = (long)n2 * n3;
  const int np = (2 * r1 + 1) * (2 * r2 + 1);
  if (cudaMemsetAsync(w.u, 0, sizeof(float) * n23 * np * n1, st) != cudaSuccess) return PWD_ECUDA;
  Spray3 s;
  s.n1 = n1; s.n2 = n2; s.n3 = n3;
  s.eps = 0.01f * 0.01f;  // csomean3d/csomf3d force eps=0.01 (:1402, :1586)
  s.eps2 = s.eps;
  const Visit3 v = make_visit(r1, r2);
  const int lanes = spray3_lanes(v);  // 4, 8 or 16: lane groups never straddle warps
  int rc = PWD_OK;
  switch (order) {
    case 1: rc = spray3_run<1>(d, p1, p2, w, s, v, lanes, st); break;
    case 2: rc = spray3_run<2>(d, p1, p2, w, s, v, lanes, st); break;
    case 3: rc = spray3_run<3>(d, p1, p2, w, s, v, lanes, st); break;
    case 4: rc = spray3_run<4>(d, p1, p2, w, s, v, lanes, st); break;
    default: rc = PWD_ENOTSUP;
  }
  if (rc != PWD_OK) return rc;
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_somean3d_workspace_size(int n1, int n2, int n3, int r1, int r2, int order) {
  if (check3(n1, n2, n3, r1, r2, order) != PWD_OK) return 0;
  size_t t = 0;
  carve_spray3(nullptr, n1, n2, n3, r1, r2, order, false, &t);
  return t;
}

extern "C" int pwd_somean3d(const float* data, const float* dip_inline, const float* dip_xline,
                            float* out, int n1, int n2, int n3, int r1, int r2, int order,
                            float eps, void* workspace, size_t workspace_bytes,
                            pwd_stream_t stream) {
  (void)eps;
  int rc = check3(n1, n2, n3, r1, r2, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip_inline || !dip_xline || !out) return PWD_EINVAL;
  size_t need = 0;
  carve_spray3(nullptr, n1, n2, n3, r1, r2, order, false, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  Spray3Work w = carve_spray3(workspace, n1, n2, n3, r1, r2, order, false, &need);
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = spray3(data, dip_inline, dip_xline, w, n1, n2, n3, r1, r2, order, st)) != PWD_OK)
    return rc;
  const long n = (long)n1 * n2 * n3;
  const int np = (2 * r1 + 1) * (2 * r2 + 1);
  PWD_KERNEL(PWD_FAM_FILTER, st, k_panel_mean<<<(unsigned)((n + 255) / 256), 256, 0, st>>>(w.u, out, n1, np, (long)n2 * n3));
  return cudaGetLastError() == cudaSuccess ? PWD_OK : PWD_ECUDA;
}

extern "C" size_t pwd_somf3d_workspace_size(int n1, int n2, int n3, int r1, int r2, int nmf,
                                            int option, int order) {
  if (check3(n1, n2, n3, r1, r2, order) != PWD_OK || !median_args_ok(nmf, option)) return 0;
  size_t t = 0;
  carve_spray3(nullptr, n1, n2, n3, r1, r2, order, option != 1, &t);
  return t;
}

extern "C" int pwd_somf3d(const float* data, const float* dip_inline, const float* dip_xline,
                          float* out, int n1, int n2, int n3, int r1, int r2, int nmf, int option,
                          int order, float eps, void* workspace, size_t workspace_bytes,
                          pwd_stream_t stream) {
  (void)eps;
  int rc = check3(n1, n2, n3, r1, r2, order);
  if (rc != PWD_OK) return rc;
  if (!data || !dip_inline || !dip_xline || !out) return PWD_EINVAL;
  if (!median_args_ok(nmf, option)) return nmf < 1 ? PWD_EINVAL : PWD_ENOTSUP;
  size_t need = 0;
  carve_spray3(nullptr, n1, n2, n3, r1, r2, order, option != 1, &need);
  if (!workspace || workspace_bytes < need || ((uintptr_t)workspace & 255)) return PWD_EWORKSPACE;
  Spray3Work w = carve_spray3(workspace, n1, n2, n3, r1, r2, order, option != 1, &need);
  cudaStream_t st = (cudaStream_t)stream;
  if ((rc = spray3(data, dip_inline, dip_xline, w, n1, n2, n3, r1, r2, order, st)) != PWD_OK)
    return rc;
  const int np = (2 * r1 + 1) * (2 * r2 + 1);
  return launch_panel_median(w.u, out, w.v2, w.avg, n1, np, (long)n2 * n3, nmf, option, st);
}
