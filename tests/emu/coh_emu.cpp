// Test harness: the per-thread code of the coherence kernels
// (pyseistr_gb300/csrc/pwd_coh.cuh) run on the CPU for every thread index of
// the kernels' grids, so that the CPU tests check the kernels' own index
// arithmetic and float operations against the oracle.  Not part of the
// library.
#include "../../pyseistr_gb300/csrc/pwd_coh.cuh"

extern "C" int emu_coherence_batch(const float* in, const float* v, const float* h, int typ,
                                   int nt, int nv, int nh, int nwin, float dt, int forw,
                                   float hmax, float* out) {
  if (nt < 1 || nv < 1 || nh < 1 || nwin < 1 || (forw != 1 && forw != -1)) return 1;
  if (typ != 1 && typ != 2 && typ != 3) typ = 1;
  pwd::coh::CohParams q;
  q.in = in;
  q.v = v;
  q.h = h;
  q.out = out;
  q.typ = typ;
  q.nt = nt;
  q.nv = nv;
  q.nh = nh;
  q.dt = dt;
  q.hmax = hmax;
  if (forw == -1) {
    const long n = (long)nt * nv * nwin;
    for (long g = 0; g < n; g++) pwd::coh::adjoint_item(q, g);
  } else {
    for (long g = 0; g < (long)nh * nwin; g++) pwd::coh::forward_item(q, g);
  }
  return 0;
}

extern "C" int emu_coherence(const float* in, const float* v, const float* h, int typ, int nt,
                             int nv, int nh, float dt, int forw, float hmax, float* out) {
  return emu_coherence_batch(in, v, h, typ, nt, nv, nh, 1, dt, forw, hmax, out);
}
