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

// One source trace's spray tree (csomean3d :1466-1520) on lps lanes: lane
// k of the group predicts cell k of each level.  Every lane of a warp runs
// every level (lanes without a source or a cell only meet the barriers), so
// a cell's neighbours, predicted by other lanes of the group in earlier
// levels, are complete and visible when it reads them.
template <int NW>
__global__ void __launch_bounds__(128) k_spray3_tree(const float* __restrict__ din,
                                                     const float* __restrict__ p1,
                                                     const float* __restrict__ p2,
                                                     float* __restrict__ u, Spray3 s, Visit3 v,
                                                     ApCoef c, PredictScratch sc, int lps) {
  const long n23 = (long)s.n2 * s.n3;
  const long gt = blockIdx.x * (long)blockDim.x + threadIdx.x;
  const long i = gt / lps;
  const int lane = (int)(gt - i * lps);
  const bool src_ok = i < n23;
  const int n1 = s.n1, np = v.np, np2 = v.np2;
  PredictScratch my = sc;  // one scratch column per lane of the grid
  my.o += gt;
  my.d += gt;
  my.y += gt;
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
      const float *q2 = nullptr, *q3 = nullptr;
      if (go && (update & 1)) {
        if (up2) {
          if (j2 == 0) go = false;
          t2 = j - 1; q2 = p1 + t2 * n1; s2 = jp - 1;
        } else {
          if (j2 == s.n2 - 1) go = false;
          t2 = j + 1; q2 = p1 + j * n1; s2 = jp + 1;
        }
      }
      if (go && (update & 2)) {
        if (up3) {
          if (j3 == 0) go = false;
          t3 = j - s.n2; q3 = p2 + t3 * n1; s3 = jp - np2;
        } else {
          if (j3 == s.n3 - 1) go = false;
          t3 = j + s.n2; q3 = p2 + j * n1; s3 = jp + np2;
        }
      }
      if (go) {
        float* trace = U(j, jp);
        if (update == 1)
          predict_fwd<NW, false>(n1, s.eps, s.eps2, c, U(t2, s2), q2, up2, nullptr, nullptr,
                                 false, trace, my);
        else if (update == 2)
          predict_fwd<NW, false>(n1, s.eps, s.eps2, c, U(t3, s3), q3, up3, nullptr, nullptr,
                                 false, trace, my);
        else
          predict_fwd<NW, true>(n1, s.eps, s.eps2, c, U(t2, s2), q2, up2, U(t3, s3), q3, up3,
                                trace, my);
      }
    }
    __syncwarp();
  }
}

struct Spray3Work {
  float *u, *v2, *avg;
  PredictScratch sc;
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
  w.sc.o = cv.take<float>((long)nb * n1 * nthr);
  w.sc.d = cv.take<float>((long)n1 * nthr);
  w.sc.y = cv.take<float>((long)n1 * nthr);
  w.sc.ss = nthr;
  *total = cv.size();
  return w;
}

int check3(int n1, int n2, int n3, int r1, int r2, int order) {
  if (n1 < 4 || n2 < 1 || n3 < 1 || r1 < 0 || r2 < 0 || order < 1) return PWD_EINVAL;
  if (order > PWD_MAX_ORDER || r1 > kMaxR || r2 > kMaxR) return PWD_ENOTSUP;
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
  const unsigned g = (unsigned)(spray3_threads(n23, lanes) / 128);
  int rc = PWD_OK;
  switch (order) {
    case 1: PWD_KERNEL(PWD_FAM_SPRAY, st, k_spray3_tree<1><<<g, 128, 0, st>>>(d, p1, p2, w.u, s, v, make_apcoef(1), w.sc, lanes)); break;
    case 2: PWD_KERNEL(PWD_FAM_SPRAY, st, k_spray3_tree<2><<<g, 128, 0, st>>>(d, p1, p2, w.u, s, v, make_apcoef(2), w.sc, lanes)); break;
    case 3: PWD_KERNEL(PWD_FAM_SPRAY, st, k_spray3_tree<3><<<g, 128, 0, st>>>(d, p1, p2, w.u, s, v, make_apcoef(3), w.sc, lanes)); break;
    case 4: PWD_KERNEL(PWD_FAM_SPRAY, st, k_spray3_tree<4><<<g, 128, 0, st>>>(d, p1, p2, w.u, s, v, make_apcoef(4), w.sc, lanes)); break;
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
