// Radon coherence along linear, parabolic and hyperbolic curves: the work of
// one GPU thread, shared by the kernels of pwd_coh.cu and by the CPU test
// that runs this same code for every thread index (the header compiles as
// plain C++ without nvcc).
//
// Restates coh (pyseistr/src/coh_cfuns.c:181-225) as set up by coh_init2
// (:158-179) and driven by cohc_fb (:415-545), which cohc (das.py:92) calls.
// Model m[iv][itau] (nt x nv), data d[ih][it] (nt x nh), flat column-major.
// The curve of model sample (itau, iv) crosses trace ih at sample
// it = floor(t / dt) + 1 with
//   linear      t = itau dt + h[ih] v[iv]
//   parabolic   t = itau dt + h[ih]^2 v[iv] / hmax / hmax
//   hyperbolic  t = sqrt(tau^2 + (h[ih] / v[iv])^2), tau = itau dt,
// every operation in float, in that order; samples with 0 <= it <= nt take
// part.  it = nt is, in the flat data array, the next trace's first sample
// (on the last trace, one past the end of the array).
//
// Adjoint (forw = -1): num and den, the stack and energy of the data along
// the curve, summed over ih in increasing order, and
// m = num^2 / (nh den + 1e-16) in double, rounded to float.  A curve that
// reaches past the end of the data array (sample nt of the last trace)
// makes the reference read whatever follows its array, an undefined value
// (NaN or garbage in practice); here that sample reads as 0, so the model
// sample is the coherence of the curve's other terms.
//
// Forward (forw = 1): d[ih][it] += m[iv][itau] in the reference's loop order
// (itau, then ih, then iv).  One thread owns an output trace: it walks itau
// and, at each, first the previous trace's curves that reach sample nt
// (they land on this trace's first sample), then its own, so every output
// sample receives its terms in the reference's order and the results are
// bit-identical.  The past-the-end sample of the last trace is dropped.
#pragma once

#include <math.h>

#ifdef __CUDACC__
#define PWD_COH_HD __host__ __device__ __forceinline__
#else
#define PWD_COH_HD inline
#endif

namespace pwd {
namespace coh {

struct CohParams {
  const float* in;  // model (forward) or data (adjoint)
  const float* v;   // nv curve parameters
  const float* h;   // nh offsets
  float* out;       // data (forward) or model (adjoint)
  int typ;          // 1 linear, 2 parabolic, 3 hyperbolic (others: linear)
  int nt, nv, nh;
  float dt;
  float hmax;  // parabolic normaliser (the reference's file-scope static)
};

// Index returned for a curve value with no usable sample index (NaN, or a
// magnitude of at least 2e9 samples): it fails the 0 <= it test, so the
// term is skipped.  Callers refuse such inputs beforehand.
constexpr int kNoIndex = -1;

PWD_COH_HD int curve_index(const CohParams& q, int itau, int ih, int iv) {
  const float hh = q.h[ih], vv = q.v[iv];
  float t;
  if (q.typ == 2) {
    t = (float)itau * q.dt + hh * hh * vv / q.hmax / q.hmax;
  } else if (q.typ == 3) {
    const float tau = (float)itau * q.dt, hv = hh / vv;
    t = sqrtf(tau * tau + hv * hv);
  } else {
    t = (float)itau * q.dt + hh * vv;
  }
  const float fl = floorf(t / q.dt) + 1.f;
  if (!(fabsf(fl) < 2.0e9f)) return kNoIndex;
  return (int)fl;
}

// Adjoint: model sample k = iv * nt + itau (consecutive threads take
// consecutive itau, so their data reads along a curve are consecutive).
PWD_COH_HD float adjoint_sample(const CohParams& q, long k) {
  const int iv = (int)(k / q.nt), itau = (int)(k - (long)iv * q.nt);
  const long ndata = (long)q.nt * q.nh;
  float num = 0.f, den = 0.f;
  for (int ih = 0; ih < q.nh; ih++) {
    const int it = curve_index(q, itau, ih, iv);
    if (it < 0 || it > q.nt) continue;
    const long id = (long)ih * q.nt + it;
    if (id >= ndata) continue;  // past the end: a zero term (num + 0 = num)
    const float y = q.in[id];
    num = num + y;
    den = den + y * y;
  }
  const float nn = num * num, nd = (float)q.nh * den;
  return (float)((double)nn / ((double)nd + 0.0000000000000001));
}

// Forward: the whole output trace ih (out[ih * nt .. ih * nt + nt)).
PWD_COH_HD void forward_trace(const CohParams& q, int ih) {
  float* o = q.out + (long)ih * q.nt;
  for (int it = 0; it < q.nt; it++) o[it] = 0.f;
  for (int itau = 0; itau < q.nt; itau++) {
    if (ih > 0)
      for (int iv = 0; iv < q.nv; iv++)
        if (curve_index(q, itau, ih - 1, iv) == q.nt) o[0] += q.in[(long)iv * q.nt + itau];
    for (int iv = 0; iv < q.nv; iv++) {
      const int it = curve_index(q, itau, ih, iv);
      if (it >= 0 && it < q.nt) o[it] += q.in[(long)iv * q.nt + itau];
    }
  }
}

// Stacked windows: element g of nwin windows' models (adjoint) or trace g
// of their data (forward), window g / (nt nv) or g / nh.
PWD_COH_HD void adjoint_item(const CohParams& q, long g) {
  const long nmod = (long)q.nt * q.nv, w = g / nmod;
  CohParams p = q;
  p.in = q.in + w * (long)q.nt * q.nh;
  p.out = q.out + w * nmod;
  const long k = g - w * nmod;
  p.out[k] = adjoint_sample(p, k);
}
PWD_COH_HD void forward_item(const CohParams& q, long g) {
  const long w = g / q.nh;
  CohParams p = q;
  p.in = q.in + w * (long)q.nt * q.nv;
  p.out = q.out + w * (long)q.nt * q.nh;
  forward_trace(p, (int)(g - w * q.nh));
}

}  // namespace coh
}  // namespace pwd
