// Patching: an array of 2 or 3 axes cut into overlapping windows and put
// back together (restates pyseistr/patch.py mode 1: patch2d :64-83, patch3d
// :178-205, patch2d_inv :270-304, patch3d_inv :402-445).
//
// Every axis of length n is padded with zeros to N = n + s - mod(n - l, s)
// when mod(n - l, s) != 0; windows start at 0, s, ... <= N - l on each axis;
// patch id runs over the first axis's starts outermost; a patch is its
// window flattened column-major.  The patch matrix [npatch][l1 l2 l3] is
// therefore a batch of equal sections packed one after another, the layout
// of the library's batched entry points.
//
// Both directions are gathers with no atomics: the forward kernel gives each
// patch element its source sample (0 in the padding); the inverse gives each
// output sample the patches covering it, added in FP64 in increasing patch
// id (the reference's overlap-add order into a float64 array), divided by
// their count (0/0 = NaN where a stride larger than the window leaves a
// sample uncovered) and rounded once to float.  Index arithmetic divides by
// loop-invariant integers through precomputed multipliers.
#include <cuda_runtime.h>
#include <stdint.h>

#include "pwd_common.cuh"

namespace pwd {
namespace {

// Division of n < 2^31 by an invariant d >= 1 (Granlund and Montgomery,
// "Division by invariant integers using multiplication", 1994): with
// 2^(sh-1) < d <= 2^sh and mul = floor(2^32 (2^sh - d) / d) + 1,
// floor(n / d) = (umulhi(mul, n) + n) >> sh.
struct FastDiv {
  unsigned d, mul, sh;
};
FastDiv make_fastdiv(unsigned d) {
  FastDiv f;
  f.d = d;
  f.sh = 0;
  while ((1ull << f.sh) < d) f.sh++;
  f.mul = (unsigned)((((1ull << 32) * ((1ull << f.sh) - d)) / d) + 1);
  return f;
}
__device__ __forceinline__ unsigned fdiv(unsigned n, const FastDiv& f) {
  return (__umulhi(f.mul, n) + n) >> f.sh;
}

struct PatchGeom {
  int n[3], l[3], s[3], np[3];  // sizes, windows, strides, window starts per axis
  unsigned L, npatch;           // elements per patch, patches
  FastDiv dl1, dl2, dl3, dnp2, dnp3, ds[3];
};

long padded_len(long n, long l, long s) {
  const long t = ((n - l) % s + s) % s;  // Python's mod for a positive s
  return t ? n + s - t : n;
}

// Geometry; false when a size is invalid or the index arithmetic would not
// fit 31 bits.
bool make_geom(const int n[3], const int l[3], const int s[3], PatchGeom& g) {
  long npatch = 1, L = 1, ntot = 1;
  for (int a = 0; a < 3; a++) {
    if (n[a] < 1 || l[a] < 1 || s[a] < 1) return false;
    g.n[a] = n[a];
    g.l[a] = l[a];
    g.s[a] = s[a];
    const long N = padded_len(n[a], l[a], s[a]);
    const long np = (N - l[a]) / s[a] + 1;
    if (np < 1) return false;
    g.np[a] = (int)np;
    npatch *= np;
    L *= l[a];
    ntot *= n[a];
  }
  if (npatch * L >= (1L << 31) || ntot >= (1L << 31)) return false;
  g.L = (unsigned)L;
  g.npatch = (unsigned)npatch;
  g.dl1 = make_fastdiv((unsigned)l[0]);
  g.dl2 = make_fastdiv((unsigned)l[1]);
  g.dl3 = make_fastdiv((unsigned)l[2]);
  g.dnp2 = make_fastdiv((unsigned)g.np[1]);
  g.dnp3 = make_fastdiv((unsigned)g.np[2]);
  for (int a = 0; a < 3; a++) g.ds[a] = make_fastdiv((unsigned)s[a]);
  return true;
}

// x[e], e = id L + k1 + l1 (k2 + l2 k3): the sample at (p s + k) per axis.
__global__ void k_patch(const float* __restrict__ a, float* __restrict__ x, PatchGeom g) {
  const unsigned total = g.npatch * g.L;
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    // e = ((id l3 + k3) l2 + k2) l1 + k1, id = (p1 np2 + p2) np3 + p3
    const unsigned r = fdiv(e, g.dl1);
    const unsigned k1 = e - r * (unsigned)g.l[0];
    const unsigned t = fdiv(r, g.dl2);
    const unsigned k2 = r - t * (unsigned)g.l[1];
    const unsigned id = fdiv(t, g.dl3);
    const unsigned k3 = t - id * (unsigned)g.l[2];
    const unsigned q = fdiv(id, g.dnp3);
    const unsigned p3 = id - q * (unsigned)g.np[2];
    const unsigned p1 = fdiv(q, g.dnp2);
    const unsigned p2 = q - p1 * (unsigned)g.np[1];
    const unsigned i1 = p1 * g.s[0] + k1, i2 = p2 * g.s[1] + k2, i3 = p3 * g.s[2] + k3;
    float v = 0.f;
    if (i1 < (unsigned)g.n[0] && i2 < (unsigned)g.n[1] && i3 < (unsigned)g.n[2])
      v = a[i1 + (size_t)g.n[0] * (i2 + (size_t)g.n[1] * i3)];
    x[e] = v;
  }
}

// Window starts along one axis covering sample i: [lo, hi].
__device__ __forceinline__ void cover(unsigned i, int l, int np, const FastDiv& ds,
                                      unsigned& lo, unsigned& hi) {
  hi = min(fdiv(i, ds), (unsigned)np - 1);
  lo = i >= (unsigned)l ? fdiv(i - (unsigned)l, ds) + 1 : 0u;
}

__global__ void k_patch_inv(const float* __restrict__ x, float* __restrict__ a, PatchGeom g,
                            FastDiv dn1, FastDiv dn2) {
  const unsigned total = (unsigned)g.n[0] * g.n[1] * g.n[2];
  for (unsigned e = blockIdx.x * blockDim.x + threadIdx.x; e < total;
       e += gridDim.x * blockDim.x) {
    const unsigned r = fdiv(e, dn1);
    const unsigned i1 = e - r * (unsigned)g.n[0];
    const unsigned i3 = fdiv(r, dn2);
    const unsigned i2 = r - i3 * (unsigned)g.n[1];
    unsigned lo1, hi1, lo2, hi2, lo3, hi3;
    cover(i1, g.l[0], g.np[0], g.ds[0], lo1, hi1);
    cover(i2, g.l[1], g.np[1], g.ds[1], lo2, hi2);
    cover(i3, g.l[2], g.np[2], g.ds[2], lo3, hi3);
    // GB300's FP64 rate is small: the count is an integer, the first term
    // enters without an addition (0.0 + v is v, except that a zero becomes
    // +0), and a power-of-two count divides by its exact reciprocal (the
    // same double as the division)
    double sum = 0.0;
    unsigned cnt = 0;
    for (unsigned p1 = lo1; p1 <= hi1; p1++)
      for (unsigned p2 = lo2; p2 <= hi2; p2++)
        for (unsigned p3 = lo3; p3 <= hi3; p3++) {
          const unsigned id = (p1 * (unsigned)g.np[1] + p2) * (unsigned)g.np[2] + p3;
          const unsigned k = (i1 - p1 * g.s[0]) +
                             (unsigned)g.l[0] * ((i2 - p2 * g.s[1]) +
                                                 (unsigned)g.l[1] * (i3 - p3 * g.s[2]));
          const double v = (double)x[(size_t)id * g.L + k];
          sum = cnt == 0 ? (v == 0.0 ? 0.0 : v) : __dadd_rn(sum, v);
          cnt++;
        }
    double q;
    if (cnt == 0)
      q = __ddiv_rn(0.0, 0.0);  // no window covers the sample: NaN as 0/0
    else if ((cnt & (cnt - 1)) == 0)
      q = __dmul_rn(sum, 1.0 / (double)cnt);
    else
      q = __ddiv_rn(sum, (double)cnt);
    a[e] = __double2float_rn(q);
  }
}

int launch_grid(long work) {
  const long b = (work + 255) / 256;
  return (int)(b < 152L * 32 ? (b > 0 ? b : 1) : 152L * 32);
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" size_t pwd_patch_count(int n1, int n2, int n3, int l1, int l2, int l3, int s1,
                                  int s2, int s3) {
  const int n[3] = {n1, n2, n3}, l[3] = {l1, l2, l3}, s[3] = {s1, s2, s3};
  PatchGeom g;
  return make_geom(n, l, s, g) ? (size_t)g.npatch : 0;
}

extern "C" int pwd_patch(const float* a, float* x, int n1, int n2, int n3, int l1, int l2,
                         int l3, int s1, int s2, int s3, pwd_stream_t stream) {
  const int n[3] = {n1, n2, n3}, l[3] = {l1, l2, l3}, s[3] = {s1, s2, s3};
  PatchGeom g;
  if (!a || !x || !make_geom(n, l, s, g)) return PWD_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_patch<<<launch_grid((long)g.npatch * g.L), 256, 0, st>>>(a, x, g));
  return cuda_status(cudaGetLastError());
}

extern "C" int pwd_patch_inv(const float* x, float* a, int n1, int n2, int n3, int l1, int l2,
                             int l3, int s1, int s2, int s3, pwd_stream_t stream) {
  const int n[3] = {n1, n2, n3}, l[3] = {l1, l2, l3}, s[3] = {s1, s2, s3};
  PatchGeom g;
  if (!a || !x || !make_geom(n, l, s, g)) return PWD_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             k_patch_inv<<<launch_grid((long)n1 * n2 * n3), 256, 0, st>>>(
                 x, a, g, make_fastdiv((unsigned)n1), make_fastdiv((unsigned)n2)));
  return cuda_status(cudaGetLastError());
}
