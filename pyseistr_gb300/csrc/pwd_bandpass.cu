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
// count: one thread per trace, a warp per 32 traces, and with a few
// thousand traces one warp per SM; the time is the instructions each
// thread issues per sample, so data movement is kept to a few instructions
// per 4 samples.  A warp walks its traces in chunks of 32 samples: a 32 x 32
// chunk comes in coalesced by cp.async into a shared-memory ring a few
// chunks ahead (16-byte copies, 8 lanes per trace, when traces start on
// 16-byte boundaries; else 4-byte copies, lane = sample), each thread runs
// its trace's samples through all sections of the pass reading and writing
// 4 samples per shared-memory access (fusing the sections of one direction
// changes nothing: section k at sample i needs only section k-1 at samples
// <= i), and the chunk goes back out coalesced.  A backward pass walks the
// chunks, and the samples in each, in reverse.  Passes after the first read
// the output array back, which for a record of tens of MB is still in L2.
#include <cuda_runtime.h>
#include <math.h>
#include <stdint.h>
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

// rows of 36 floats: 16-byte aligned, and a quarter-warp's 16-byte accesses
// to 8 rows (row stride 36 = 4 mod 32 banks) or to 8 consecutive quads of one
// row fall in distinct banks
constexpr int kBpPitch = 36;
typedef float BpRing[kBpStages][32][kBpPitch];

__device__ __forceinline__ void cp_async16(float* dst, const float* src) {
  const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;\n" ::"r"(d), "l"(src) : "memory");
}

// One pass of a cascade over the warp's 32 traces.
template <bool VEC, bool LOW, bool FIRST, int NS2>
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
  // VEC: lane -> trace lane / 8 + 4 m (m < 8), samples 4 (lane % 8) .. + 3
  const int vq = 4 * (lane & 7), vj = lane >> 3;
  auto load = [&](int q) {
    if (q < nch) {
      const long c0 = (long)(back ? nch - 1 - q : q) * 32;
      float(*buf)[kBpPitch] = ring[q % kBpStages];
      if (VEC) {
        if (c0 + vq < n1) {
          const float* s = src + (t0 + vj) * n1 + c0 + vq;
#pragma unroll
          for (int m = 0; m < 8; m++)
            if (vj + 4 * m < ntw) cp_async16(&buf[vj + 4 * m][vq], s + 4 * m * n1);
        }
      } else if (c0 + lane < n1) {
        const float* s = src + t0 * n1 + c0 + lane;
#pragma unroll 8
        for (int j = 0; j < ntw; j++) cp_async4(&buf[j][lane], s + j * n1);
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
      float4* r4 = reinterpret_cast<float4*>(row);
      if (back) {
#pragma unroll
        for (int g = 7; g >= 0; g--) {
          float4 v = r4[g];
          v.w = step(v.w);
          v.z = step(v.z);
          v.y = step(v.y);
          v.x = step(v.x);
          r4[g] = v;
        }
      } else {
#pragma unroll
        for (int g = 0; g < 8; g++) {
          float4 v = r4[g];
          v.x = step(v.x);
          v.y = step(v.y);
          v.z = step(v.z);
          v.w = step(v.w);
          r4[g] = v;
        }
      }
    } else if (back) {
      for (int i = (int)len - 1; i >= 0; i--) row[i] = step(row[i]);
    } else {
      for (int i = 0; i < (int)len; i++) row[i] = step(row[i]);
    }
    __syncwarp();
    float(*buf)[kBpPitch] = ring[q % kBpStages];
    const long c0 = (long)c * 32;
    if (VEC) {
      if (c0 + vq < n1) {
        float* d = dst + (t0 + vj) * n1 + c0 + vq;
#pragma unroll
        for (int m = 0; m < 8; m++)
          if (vj + 4 * m < ntw)
            *reinterpret_cast<float4*>(d + 4 * m * n1) =
                *reinterpret_cast<const float4*>(&buf[vj + 4 * m][vq]);
      }
    } else if (c0 + lane < n1) {
      float* d = dst + t0 * n1 + c0 + lane;
#pragma unroll 8
      for (int j = 0; j < ntw; j++) d[j * n1] = buf[j][lane];
    }
    __syncwarp();
  }
}

// One warp per 32 traces, the plan's passes in order; the first reads `in`
// (which may be `out`), the others read `out` back.  Each lane reads back
// only the samples it stored itself.
template <bool VEC>
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
    bp_pass<VEC, L, F, N>(src, out, n1, t0, ntr, P, ring);       \
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
  // 16-byte copies when every trace starts on a 16-byte boundary
  const bool vec = n1 % 4 == 0 && (uintptr_t)in % 16 == 0 && (uintptr_t)out % 16 == 0;
  for (size_t p0 = 0; p0 < passes.size(); p0 += kBpPass) {
    BpPlan plan;
    memset(&plan, 0, sizeof plan);
    plan.npass = (int)std::min(passes.size() - p0, (size_t)kBpPass);
    for (int k = 0; k < plan.npass; k++) plan.p[k] = passes[p0 + k];
    const float* src = p0 == 0 ? in : out;
    if (vec)
      PWD_KERNEL(PWD_FAM_OTHER, st,
                 k_bandpass<true><<<grid, 32, 0, st>>>(src, out, (long)n1, ntr, plan));
    else
      PWD_KERNEL(PWD_FAM_OTHER, st,
                 k_bandpass<false><<<grid, 32, 0, st>>>(src, out, (long)n1, ntr, plan));
    const int rc = cuda_status(cudaGetLastError());
    if (rc != PWD_OK) return rc;
  }
  return PWD_OK;
}
