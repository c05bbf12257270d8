// Plane-wave painting (cpaint2d, pyseistr/src/paint_cfuns.c:1861-1940,
// called by pwpaintc and rgt, rgt.py:4-87): the C entry and its kernel.  The
// arithmetic of one thread is in pwd_paint.cuh.
//
// The painting is a chain of trace predictions from the seed trace outward,
// each a banded LDL' factorisation and two substitutions along the trace:
// serial work, so one thread paints one side of a section (two threads per
// section) and the time is the chain's length times a step's latency.  The
// GPU pays off when the section is already on the device (slopes estimated
// there) or when many sections are painted at once; a single section is no
// faster than the reference's C.  pwd_paint2d_batch paints many sections
// of one size in one launch (two threads per section).
#include <cuda_runtime.h>

#include "pwd_common.cuh"
#include "pwd_paint.cuh"

namespace pwd {
namespace {

// nsec stacked sections, two threads each.
__global__ void __launch_bounds__(64) k_paint2d(paint::PaintParams q, int nsec) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < 2L * nsec) paint::paint_item(q, g);
}

}  // namespace
}  // namespace pwd

extern "C" size_t pwd_paint2d_batch_workspace_size(int n1, int nsec, int order) {
  if (n1 < 4 || nsec < 1 || order < 1 || order > pwd::paint::kMaxNw) return 0;
  const size_t bytes =
      sizeof(float) * 2 * (size_t)nsec * (size_t)pwd::paint::slice_floats(n1, order);
  return (bytes + 255) & ~(size_t)255;
}

extern "C" size_t pwd_paint2d_workspace_size(int n1, int order) {
  return pwd_paint2d_batch_workspace_size(n1, 1, order);
}

extern "C" int pwd_paint2d_batch(const float* dip, const float* seed, float* out, int n1, int n2,
                                 int nsec, int order, int i0, float eps, void* workspace,
                                 size_t workspace_bytes, pwd_stream_t stream) {
  if (!dip || !seed || !out || n1 < 4 || n2 < 1 || nsec < 1 || order < 1 || i0 < 0 || i0 >= n2)
    return PWD_EINVAL;
  if (order > pwd::paint::kMaxNw) return PWD_ENOTSUP;
  if ((long)n1 * n2 * nsec > (1L << 40)) return PWD_EINVAL;
  const size_t need = pwd_paint2d_batch_workspace_size(n1, nsec, order);
  if (!workspace || workspace_bytes < need || (uintptr_t)workspace % 256) return PWD_EWORKSPACE;
  pwd::paint::PaintParams q;
  q.dip = dip;
  q.seed = seed;
  q.out = out;
  q.ws = (float*)workspace;
  q.n1 = n1;
  q.n2 = n2;
  q.nw = order;
  q.i0 = i0;
  q.eps = eps * eps;  // predict_init(n1, n2, eps*eps, order, 1, false)
  for (int k = 0; k < pwd::paint::kMaxNa; k++) q.b[k] = 0.;
  pwd::paint::filter_constants(order, q.b);
  cudaStream_t st = (cudaStream_t)stream;
  const unsigned grid = (unsigned)((2L * nsec + 63) / 64);
  PWD_KERNEL(PWD_FAM_OTHER, st, (pwd::k_paint2d<<<grid, 64, 0, st>>>(q, nsec)));
  return pwd::cuda_status(cudaGetLastError());
}

extern "C" int pwd_paint2d(const float* dip, const float* seed, float* out, int n1, int n2,
                           int order, int i0, float eps, void* workspace,
                           size_t workspace_bytes, pwd_stream_t stream) {
  return pwd_paint2d_batch(dip, seed, out, n1, n2, 1, order, i0, eps, workspace,
                           workspace_bytes, stream);
}
