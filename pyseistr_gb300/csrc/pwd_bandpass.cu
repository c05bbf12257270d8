// Band-pass: Butterworth low-cut and high-cut filters along each trace
// (restates pyseistr/src/bp_cfuns.c: sf_butter_init :422-464, sf_butter_apply
// :471-507, cbp :524-645, called by bandpassc, bp.py:128-181).
//
// A filter of nn poles is a cascade of nn/2 second-order sections after a
// first-order one when nn is odd; each section is a recurrence along the
// trace, and zero phase runs the whole cascade once more from the trace's
// end.  The low-cut filter goes first (forward, then backward), the
// high-cut one second.  Every operation is the reference's, in float, in
// its order, with no contraction: outputs are bit-identical to it.
//
// The recurrences are serial along a trace, so the parallelism is the trace
// count: one thread per trace, a warp per 32 traces.  A warp walks its
// traces in chunks of 32 samples: a 32 x 32 chunk comes in coalesced (lane =
// sample) by cp.async into a shared-memory ring a few chunks ahead, each
// thread runs its trace's samples through all sections of the pass (fusing
// the sections of one direction changes nothing: section k at sample i
// needs only section k-1 at samples <= i), and the chunk goes back out
// coalesced.  A backward pass walks the chunks, and the samples in each, in
// reverse.  Passes after the first read the output array back, which for a
// record of tens of MB is still in L2.
#include <cuda_runtime.h>
#include <math.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "pwd_common.cuh"

namespace pwd {
namespace {

constexpr int kBpSec = 3;     // second-order sections per pass
constexpr int kBpPass = 8;    // passes per launch
constexpr int kBpStages = 4;  // chunks per warp in flight

struct BpPass {
  int back, low, first, ns2;
  float fc0, fc2;                // the first-order section (when first)
  float c0[kBpSec], c2[kBpSec];  // second-order sections
  float mid;                     // their common middle feedback tap
};
struct BpPlan {
  int npass;
  BpPass p[kBpPass];
};

typedef float BpRing[kBpStages][32][33];

// One pass of a cascade over the warp's 32 traces.
template <bool LOW, bool FIRST, int NS2>
__device__ void bp_pass(const float* src, float* dst, long n1, long t0, long ntr,
                        const BpPass& P, BpRing& ring) {
  const int lane = threadIdx.x & 31;
  const int nch = (int)((n1 + 31) / 32);
  const bool back = P.back;
  const float fc0 = P.fc0, fc2 = P.fc2, mid = P.mid;
  float c0[NS2 > 0 ? NS2 : 1], c2[NS2 > 0 ? NS2 : 1];
#pragma unroll
  for (int k = 0; k < NS2; k++) {
    c0[k] = P.c0[k];
    c2[k] = P.c2[k];
  }
  float fx1 = 0.f, fy1 = 0.f;
  float x1[NS2 > 0 ? NS2 : 1], x2[NS2 > 0 ? NS2 : 1], y1[NS2 > 0 ? NS2 : 1],
      y2[NS2 > 0 ? NS2 : 1];
#pragma unroll
  for (int k = 0; k < NS2; k++) x1[k] = x2[k] = y1[k] = y2[k] = 0.f;

  // the sample through every section: first order
  //   y = ((x0 +- x1) - c2 y1) c0,
  // second order
  //   y = ((((x0 +- 2 x1) + x2) - mid y1) - c2 y2) c0,
  // + for the low-pass (high-cut) filter, - for the high-pass one
  auto step = [&](float v) -> float {
    if (FIRST) {
      const float s = LOW ? __fadd_rn(v, fx1) : __fsub_rn(v, fx1);
      fx1 = v;
      fy1 = __fmul_rn(__fsub_rn(s, __fmul_rn(fc2, fy1)), fc0);
      v = fy1;
    }
#pragma unroll
    for (int k = 0; k < NS2; k++) {
      const float tx = __fmul_rn(2.f, x1[k]);
      const float s = __fadd_rn(LOW ? __fadd_rn(v, tx) : __fsub_rn(v, tx), x2[k]);
      const float y = __fmul_rn(
          __fsub_rn(__fsub_rn(s, __fmul_rn(mid, y1[k])), __fmul_rn(c2[k], y2[k])), c0[k]);
      x2[k] = x1[k];
      x1[k] = v;
      y2[k] = y1[k];
      y1[k] = y;
      v = y;
    }
    return v;
  };

  const long ntw = ntr - t0 < 32 ? ntr - t0 : 32;  // traces of this warp
  auto load = [&](int q) {
    if (q < nch) {
      const long i = (long)(back ? nch - 1 - q : q) * 32 + lane;
      if (i < n1) {
        const float* s = src + t0 * n1 + i;
#pragma unroll 8
        for (int j = 0; j < ntw; j++) cp_async4(&ring[q % kBpStages][j][lane], s + j * n1);
      }
    }
    cp_async_commit();
  };

#pragma unroll
  for (int q = 0; q < kBpStages - 1; q++) load(q);
  for (int q = 0; q < nch; q++) {
    load(q + kBpStages - 1);
    cp_async_wait<kBpStages - 1>();
    __syncwarp();
    float* row = ring[q % kBpStages][lane];
    const int c = back ? nch - 1 - q : q;
    const long len = n1 - (long)c * 32 < 32 ? n1 - (long)c * 32 : 32;
    if (len == 32) {
      if (back) {
#pragma unroll
        for (int i = 31; i >= 0; i--) row[i] = step(row[i]);
      } else {
#pragma unroll
        for (int i = 0; i < 32; i++) row[i] = step(row[i]);
      }
    } else if (back) {
      for (int i = (int)len - 1; i >= 0; i--) row[i] = step(row[i]);
    } else {
      for (int i = 0; i < (int)len; i++) row[i] = step(row[i]);
    }
    __syncwarp();
    const long i = (long)c * 32 + lane;
    if (i < n1) {
      float* d = dst + t0 * n1 + i;
#pragma unroll 8
      for (int j = 0; j < ntw; j++) d[j * n1] = ring[q % kBpStages][j][lane];
    }
    __syncwarp();
  }
}

// One warp per 32 traces, the plan's passes in order; the first reads `in`
// (which may be `out`), the others read `out` back.  Each lane reads back
// only the samples it stored itself.
__global__ void __launch_bounds__(32) k_bandpass(const float* in, float* out, long n1, long ntr,
                                                 BpPlan plan) {
  __shared__ __align__(16) BpRing ring;
  const long t0 = (long)blockIdx.x * 32;
  for (int p = 0; p < plan.npass; p++) {
    const BpPass& P = plan.p[p];
    const float* src = p == 0 ? in : out;
    const int code = (P.low ? 8 : 0) + (P.first ? 4 : 0) + P.ns2;
    switch (code) {
#define BP_CASE(L, F, N)                                         \
  case (L ? 8 : 0) + (F ? 4 : 0) + N:                            \
    bp_pass<L, F, N>(src, out, n1, t0, ntr, P, ring);            \
    break;
      BP_CASE(false, false, 1) BP_CASE(false, false, 2) BP_CASE(false, false, 3)
      BP_CASE(false, true, 0) BP_CASE(false, true, 1) BP_CASE(false, true, 2)
      BP_CASE(false, true, 3) BP_CASE(true, false, 1) BP_CASE(true, false, 2)
      BP_CASE(true, false, 3) BP_CASE(true, true, 0) BP_CASE(true, true, 1)
      BP_CASE(true, true, 2) BP_CASE(true, true, 3)
#undef BP_CASE
      default:
        break;
    }
    __syncwarp();
    __threadfence_block();
  }
}

// ---------------------------------------------------------------------------
// Host: coefficients and the pass plan.
// ---------------------------------------------------------------------------

// Butterworth sections of `nn` poles at `cutoff` cycles per sample, each
// expression typed as the reference's C (sf_butter_init): a float combined
// with a double constant is evaluated in double and stored as float; the
// sines and cosines are the C library's float ones.
struct Butter {
  bool low;
  int nn;
  float fc0, fc2;              // first-order section (nn odd)
  std::vector<float> c0, c2;   // nn/2 second-order sections
  float mid;
};

Butter butter(bool low, float cutoff, int nn) {
  const double pi = 3.14159265358979323846264338328;
  Butter b;
  b.low = low;
  b.nn = nn;
  b.fc0 = b.fc2 = 0.f;
  const float arg = (float)(2. * pi * (double)cutoff);
  const float sw = sinf(arg), cw = cosf(arg);
  if (nn % 2) {
    if (low) {
      const float f = (float)((1. + (double)cw) / (double)sw);
      b.fc0 = (float)(1. / (1. + (double)f));
      b.fc2 = (float)(1. - (double)f);
    } else {
      const float f = (float)((double)sw / (1. + (double)cw));
      b.fc0 = (float)(1. / ((double)f + 1.));
      b.fc2 = (float)((double)f - 1.);
    }
  }
  float g = low ? sinf((float)(0.5 * (double)arg)) : cosf((float)(0.5 * (double)arg));
  g = g * g;
  for (int j = 0; j < nn / 2; j++) {
    const float ss = sinf((float)(pi * (double)(2 * j + 1) / (double)(2 * nn))) * sw;
    b.c0.push_back((float)((double)g / (1. + (double)ss)));
    b.c2.push_back((float)((1. - (double)ss) / (double)g));
  }
  b.mid = (float)(-2. * (double)cw / (double)g);
  return b;
}

// The cascade of `b` in one direction as passes of at most kBpSec
// second-order sections, the first-order section leading the first one.
void add_passes(const Butter& b, bool back, std::vector<BpPass>& out) {
  const int ns = b.nn / 2;
  int k = 0;
  bool first = b.nn % 2;
  do {
    BpPass p;
    memset(&p, 0, sizeof p);
    p.back = back;
    p.low = b.low;
    p.first = first;
    p.fc0 = b.fc0;
    p.fc2 = b.fc2;
    p.mid = b.mid;
    while (p.ns2 < kBpSec && k < ns) {
      p.c0[p.ns2] = b.c0[k];
      p.c2[p.ns2] = b.c2[k];
      p.ns2++;
      k++;
    }
    out.push_back(p);
    first = false;
  } while (k < ns);
}

}  // namespace
}  // namespace pwd

using namespace pwd;

extern "C" int pwd_bandpass(const float* in, float* out, int n1, int n2, int n3, float d1,
                            float flo, float fhi, int nplo, int nphi, int phase,
                            pwd_stream_t stream) {
  if (!in || !out || n1 < 1 || n2 < 1 || n3 < 1) return PWD_EINVAL;
  const long ntr = (long)n2 * n3;
  if (ntr > (1L << 36)) return PWD_EINVAL;
  cudaStream_t st = (cudaStream_t)stream;
  // cbp's parameter handling (bp_cfuns.c:555-596): cut-offs in cycles per
  // sample unless negative, poles at least 1 and halved for zero phase
  const float eps = 0.0001f;
  if (!(flo < 0.f)) flo = flo * d1;
  if (!(fhi < 0.f)) fhi = fhi * d1;
  if (nplo < 1) nplo = 1;
  if (nplo > 1 && !phase) nplo /= 2;
  if (nphi < 1) nphi = 1;
  if (nphi > 1 && !phase) nphi /= 2;
  std::vector<BpPass> passes;
  if (flo > eps) {
    const Butter b = butter(false, flo, nplo);
    add_passes(b, false, passes);
    if (!phase) add_passes(b, true, passes);
  }
  if ((double)fhi < 0.5 - (double)eps) {
    const Butter b = butter(true, fhi, nphi);
    add_passes(b, false, passes);
    if (!phase) add_passes(b, true, passes);
  }
  if (passes.empty()) {
    if (in == out) return PWD_OK;
    return cuda_status(cudaMemcpyAsync(out, in, sizeof(float) * (size_t)n1 * ntr,
                                       cudaMemcpyDeviceToDevice, st));
  }
  const unsigned grid = (unsigned)((ntr + 31) / 32);
  for (size_t p0 = 0; p0 < passes.size(); p0 += kBpPass) {
    BpPlan plan;
    memset(&plan, 0, sizeof plan);
    plan.npass = (int)std::min(passes.size() - p0, (size_t)kBpPass);
    for (int k = 0; k < plan.npass; k++) plan.p[k] = passes[p0 + k];
    PWD_KERNEL(PWD_FAM_OTHER, st,
               k_bandpass<<<grid, 32, 0, st>>>(p0 == 0 ? in : out, out, (long)n1, ntr, plan));
    const int rc = cuda_status(cudaGetLastError());
    if (rc != PWD_OK) return rc;
  }
  return PWD_OK;
}
