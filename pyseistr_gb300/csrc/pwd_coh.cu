// Radon coherence (cohc_fb, pyseistr/src/coh_cfuns.c:415-545, called by
// cohc, das.py:92): the C entry and its two kernels.  The arithmetic of one
// thread is in pwd_coh.cuh.
//
// Adjoint: one thread per model sample, a gather along its curve over all
// traces.  The data section of a DAS window (3000 x 860 floats, 10 MB) stays
// in L2, and consecutive threads read consecutive samples of each trace, so
// the kernel is bound by the curve-index arithmetic (an IEEE division per
// term), not by HBM: nt nv nh terms per call.
//
// Forward: one thread per output trace, which adds the model along the
// curves in the reference's order (bit-identical output); the parallelism
// is the trace count.  The batch entry stacks the windows of a record (the
// DAS detection loop, demos/test_pyseistr_das_massive.py:190-203) in one
// launch, which multiplies that parallelism.
#include <cuda_runtime.h>

#include "pwd_coh.cuh"
#include "pwd_common.cuh"

namespace pwd {
namespace {

// nwin windows stacked one after another in `in` and `out` (one window:
// nwin = 1).
__global__ void __launch_bounds__(256) k_coh_adjoint(coh::CohParams q, int nwin) {
  const long stride = (long)gridDim.x * blockDim.x, n = (long)q.nt * q.nv * nwin;
  for (long g = (long)blockIdx.x * blockDim.x + threadIdx.x; g < n; g += stride)
    coh::adjoint_item(q, g);
}

__global__ void __launch_bounds__(32) k_coh_forward(coh::CohParams q, int nwin) {
  const long g = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (g < (long)q.nh * nwin) coh::forward_item(q, g);
}

}  // namespace
}  // namespace pwd

extern "C" int pwd_coherence_batch(const float* in, const float* v, const float* h, int typ,
                                   int nt, int nv, int nh, int nwin, float dt, int forw,
                                   float hmax, float* out, pwd_stream_t stream) {
  if (!in || !v || !h || !out || nt < 1 || nv < 1 || nh < 1 || nwin < 1) return PWD_EINVAL;
  if (forw != 1 && forw != -1) return PWD_EINVAL;
  const long nmod = (long)nt * nv, ndata = (long)nt * nh;
  if (nmod * nwin > (1L << 40) || ndata * nwin > (1L << 40)) return PWD_EINVAL;
  if (typ != 1 && typ != 2 && typ != 3) typ = 1;  // coh_init2 :169
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
  cudaStream_t st = (cudaStream_t)stream;
  if (forw == -1) {
    // a grid of at most 32 waves of 152 SMs x 8 blocks; the loop strides
    // over the rest
    const long blocks = (nmod * nwin + 255) / 256;
    const unsigned grid = (unsigned)(blocks < 152L * 8 * 32 ? blocks : 152L * 8 * 32);
    PWD_KERNEL(PWD_FAM_OTHER, st, (pwd::k_coh_adjoint<<<grid, 256, 0, st>>>(q, nwin)));
  } else {
    const unsigned grid = (unsigned)(((long)nh * nwin + 31) / 32);
    PWD_KERNEL(PWD_FAM_OTHER, st, (pwd::k_coh_forward<<<grid, 32, 0, st>>>(q, nwin)));
  }
  return pwd::cuda_status(cudaGetLastError());
}

extern "C" int pwd_coherence(const float* in, const float* v, const float* h, int typ, int nt,
                             int nv, int nh, float dt, int forw, float hmax, float* out,
                             pwd_stream_t stream) {
  return pwd_coherence_batch(in, v, h, typ, nt, nv, nh, 1, dt, forw, hmax, out, stream);
}
