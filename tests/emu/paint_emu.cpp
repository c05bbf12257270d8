// Test harness: the per-thread code of the painting kernel
// (pyseistr_gb300/csrc/pwd_paint.cuh) run on the CPU for both threads of a
// section, with the entry point's parameter set-up, so that the CPU tests
// check the kernel's own arithmetic against the oracle.  Not part of the
// library.
#include <vector>

#include "../../pyseistr_gb300/csrc/pwd_paint.cuh"

extern "C" int emu_paint2d_batch(const float* dip, const float* seed, float* out, int n1,
                                 int n2, int nsec, int order, int i0, float eps) {
  if (n1 < 4 || n2 < 1 || nsec < 1 || order < 1 || order > pwd::paint::kMaxNw || i0 < 0 ||
      i0 >= n2)
    return 1;
  std::vector<float> ws(2 * nsec * pwd::paint::slice_floats(n1, order), 12345.f);
  pwd::paint::PaintParams q;
  q.dip = dip;
  q.seed = seed;
  q.out = out;
  q.ws = ws.data();
  q.n1 = n1;
  q.n2 = n2;
  q.nw = order;
  q.i0 = i0;
  q.eps = eps * eps;
  for (int k = 0; k < pwd::paint::kMaxNa; k++) q.b[k] = 0.;
  pwd::paint::filter_constants(order, q.b);
  for (long g = 2L * nsec - 1; g >= 0; g--) pwd::paint::paint_item(q, g);  // any thread order
  return 0;
}

extern "C" int emu_paint2d(const float* dip, const float* seed, float* out, int n1, int n2,
                           int order, int i0, float eps) {
  return emu_paint2d_batch(dip, seed, out, n1, n2, 1, order, i0, eps);
}
