// FK dip filter (fkdip, pyseistr/fk.py:2-68): the C entries and their
// kernels; the arithmetic of each thread is in pwd_fk.cuh.
//
// Every pass is a grid-stride loop over the elements (or butterflies) of
// the whole section, reading one workspace buffer and writing another: the
// time FFT of all traces, a transpose to frequency rows, the space FFT of
// all rows, the cone mask (and the promotion to complex128), the inverse
// space FFT, the rebuild of the full spectrum of the output traces, the
// inverse time FFT and the real part.  The FFTs are radix-2 Stockham passes
// (log2 N launches per transform batch, each moving the batch once through
// HBM); the complex128 half runs on the FP64 pipe.
#include <cuda_runtime.h>
#include <math.h>

#include <cstdlib>
#include <vector>

#include "pwd_common.cuh"
#include "pwd_fk.cuh"

namespace pwd {
namespace {

constexpr int kFkThreads = 256;
// one transform per block in shared memory while its two buffers fit
constexpr int kFkSmemThreads = 512;
constexpr size_t kFkSmemMax = 200 * 1024;

unsigned fk_grid(long n) {
  const long b = (n + kFkThreads - 1) / kFkThreads;
  return (unsigned)(b < 152L * 8 * 16 ? b : 152L * 8 * 16);
}

#define PWD_FK_LOOP(n) \
  for (long idx = (long)blockIdx.x * blockDim.x + threadIdx.x; idx < (n); \
       idx += (long)gridDim.x * blockDim.x)

template <class R, class T>
__global__ void __launch_bounds__(kFkThreads) k_fk_load(const T* d, fk::Cx<R>* a, int n1, int nf,
                                                        long n) {
  PWD_FK_LOOP(n) fk::load_trace_sample<R, T>(d, a, n1, nf, idx);
}

template <class R>
__global__ void __launch_bounds__(kFkThreads) k_fk_pass(const fk::Cx<R>* x, fk::Cx<R>* y, int len,
                                                        int ns, long nbf, const fk::Cx<R>* tw,
                                                        int inverse) {
  PWD_FK_LOOP(nbf) fk::stockham_pass<R>(x, y, len, ns, idx, tw, inverse != 0);
}

template <class R>
__global__ void __launch_bounds__(kFkThreads) k_fk_rows(const fk::Cx<R>* a, fk::Cx<R>* b, int n2,
                                                        int nf, int nk, long n) {
  PWD_FK_LOOP(n) fk::rows_sample<R>(a, b, n2, nf, nk, idx);
}

template <class R>
__global__ void __launch_bounds__(kFkThreads) k_fk_mask(const fk::Cx<R>* b, fk::Cx<double>* c,
                                                        int nrow, int nk, double w, long n) {
  PWD_FK_LOOP(n) fk::mask_sample<R>(b, c, nrow, nk, w, idx);
}

__global__ void __launch_bounds__(kFkThreads) k_fk_full(const fk::Cx<double>* c,
                                                        fk::Cx<double>* dd, int nf, int nk,
                                                        int nrow, double inv_nk, long n) {
  PWD_FK_LOOP(n) fk::full_sample(c, dd, nf, nk, nrow, idx, inv_nk);
}

__global__ void __launch_bounds__(kFkThreads) k_fk_out(const fk::Cx<double>* dd, double* out,
                                                       int n1, int nf, double inv_nf, long n) {
  PWD_FK_LOOP(n) fk::out_sample(dd, out, n1, nf, idx, inv_nf);
}

// All log2(len) Stockham passes of one transform per block in shared
// memory (two buffers of len elements): the transform crosses HBM once each
// way instead of once per pass, with the same butterflies in the same
// order as the per-pass kernel, so the same results.
template <class R>
__global__ void __launch_bounds__(kFkSmemThreads) k_fk_fft_smem(const fk::Cx<R>* x,
                                                                fk::Cx<R>* y, int len,
                                                                const fk::Cx<R>* tw,
                                                                int inverse) {
  extern __shared__ __align__(16) unsigned char fk_sm[];
  fk::Cx<R>* a = reinterpret_cast<fk::Cx<R>*>(fk_sm);
  fk::Cx<R>* b = a + len;
  const fk::Cx<R>* xg = x + (long)blockIdx.x * len;
  for (int i = threadIdx.x; i < len; i += blockDim.x) a[i] = xg[i];
  __syncthreads();
  for (int ns = 1; ns < len; ns *= 2) {
    for (int j = threadIdx.x; j < len / 2; j += blockDim.x)
      fk::stockham_pass<R>(a, b, len, ns, j, tw, inverse != 0);
    __syncthreads();
    fk::Cx<R>* t = a;
    a = b;
    b = t;
  }
  fk::Cx<R>* yg = y + (long)blockIdx.x * len;
  for (int i = threadIdx.x; i < len; i += blockDim.x) yg[i] = a[i];
}

// log2(len) Stockham passes over `batch` transforms; returns the buffer
// holding the result (x or y).  Transforms whose two buffers fit in shared
// memory run in one launch (k_fk_fft_smem), longer ones pass by pass.
template <class R>
fk::Cx<R>* fft_batch(fk::Cx<R>* x, fk::Cx<R>* y, int len, long batch, const fk::Cx<R>* tw,
                     bool inverse, cudaStream_t st, int* rc) {
  const size_t smem = 2 * sizeof(fk::Cx<R>) * (size_t)len;
  const char* env = getenv("PWD_FK_SMEM");  // 0: every transform pass by pass
  const bool allow = !(env && atoi(env) == 0);
  if (allow && len >= 2 && smem <= kFkSmemMax && batch <= 0x7fffffffL) {
    *rc = cuda_status(cudaFuncSetAttribute(k_fk_fft_smem<R>,
                                           cudaFuncAttributeMaxDynamicSharedMemorySize,
                                           (int)smem));
    if (*rc != PWD_OK) return x;
    const int threads = len / 2 < kFkSmemThreads ? len / 2 : kFkSmemThreads;
    PWD_KERNEL(PWD_FAM_OTHER, st,
               (k_fk_fft_smem<R><<<(unsigned)batch, threads, smem, st>>>(x, y, len, tw,
                                                                          inverse ? 1 : 0)));
    *rc = cuda_status(cudaGetLastError());
    return y;
  }
  const long nbf = batch * (len / 2);
  for (int ns = 1; ns < len; ns *= 2) {
    PWD_KERNEL(PWD_FAM_OTHER, st,
               (k_fk_pass<R><<<fk_grid(nbf), kFkThreads, 0, st>>>(x, y, len, ns, nbf, tw,
                                                                  inverse ? 1 : 0)));
    fk::Cx<R>* t = x;
    x = y;
    y = t;
  }
  *rc = cuda_status(cudaGetLastError());
  return x;
}

struct FkLayout {
  int nf, nk, nrow;
  size_t a, b, c, d, tw_r, tw_d, total;
};

size_t up256(size_t v) { return (v + 255) & ~(size_t)255; }

FkLayout fk_layout(int n1, int n2, size_t in_real) {
  FkLayout l{};
  l.nf = fk::pow2_at_least(n1);
  l.nk = fk::pow2_at_least(n2);
  l.nrow = l.nf / 2 + 1;
  const size_t cr = 2 * in_real, cd = 2 * sizeof(double);
  l.a = up256(cr * (size_t)n2 * l.nf);                   // time spectra, each of 2 buffers
  l.b = up256(cr * (size_t)l.nrow * l.nk);               // FK rows, input precision
  l.c = up256(cd * (size_t)l.nrow * l.nk);               // FK rows, complex128
  l.d = up256(cd * (size_t)n2 * l.nf);                   // full spectra of the output traces
  l.tw_r = up256(cr * (size_t)(l.nf / 2 + l.nk / 2 + 2));
  l.tw_d = up256(cd * (size_t)(l.nf / 2 + l.nk / 2 + 2));
  l.total = 2 * (l.a + l.b + l.c + l.d) + l.tw_r + l.tw_d;
  return l;
}

// exp(-2 pi i m / n), m < n/2, in double.
void twiddles(int n, std::vector<double>& re, std::vector<double>& im) {
  re.clear();
  im.clear();
  for (int m = 0; m < n / 2; m++) {
    const double a = 2.0 * 3.14159265358979323846 * (double)m / (double)n;
    re.push_back(cos(a));
    im.push_back(-sin(a));
  }
}

bool fk_args_ok(int n1, int n2, double w) {
  return n1 >= 1 && n2 >= 1 && n1 <= (1 << 20) && n2 <= (1 << 20) && w != 0.0 &&
         (double)fk::pow2_at_least(n1) * fk::pow2_at_least(n2) < 4.0e9;
}

template <class R, class T>
int fk_run(const T* d, double* out, int n1, int n2, double w, void* ws, size_t wsb,
           cudaStream_t st) {
  if (!d || !out || !fk_args_ok(n1, n2, w)) return PWD_EINVAL;
  const FkLayout l = fk_layout(n1, n2, sizeof(R));
  if (!ws || wsb < l.total || (uintptr_t)ws % 256) return PWD_EWORKSPACE;
  char* p = (char*)ws;
  fk::Cx<R>* a0 = (fk::Cx<R>*)p;
  fk::Cx<R>* a1 = (fk::Cx<R>*)(p += l.a);
  fk::Cx<R>* b0 = (fk::Cx<R>*)(p += l.a);
  fk::Cx<R>* b1 = (fk::Cx<R>*)(p += l.b);
  fk::Cx<double>* c0 = (fk::Cx<double>*)(p += l.b);
  fk::Cx<double>* c1 = (fk::Cx<double>*)(p += l.c);
  fk::Cx<double>* d0 = (fk::Cx<double>*)(p += l.c);
  fk::Cx<double>* d1 = (fk::Cx<double>*)(p += l.d);
  fk::Cx<R>* twr = (fk::Cx<R>*)(p += l.d);
  fk::Cx<double>* twd = (fk::Cx<double>*)(p += l.tw_r);
  const int nf = l.nf, nk = l.nk, nrow = l.nrow;
  // twiddle tables: [time (nf/2)][space (nk/2)], in the input precision and in double
  std::vector<double> tre, tim, kre, kim;
  twiddles(nf, tre, tim);
  twiddles(nk, kre, kim);
  std::vector<fk::Cx<R>> hr;
  std::vector<fk::Cx<double>> hd;
  for (size_t m = 0; m < tre.size(); m++) {
    hr.push_back(fk::Cx<R>{(R)tre[m], (R)tim[m]});
    hd.push_back(fk::Cx<double>{tre[m], tim[m]});
  }
  for (size_t m = 0; m < kre.size(); m++) {
    hr.push_back(fk::Cx<R>{(R)kre[m], (R)kim[m]});
    hd.push_back(fk::Cx<double>{kre[m], kim[m]});
  }
  hr.push_back(fk::Cx<R>{(R)1, (R)0});  // keeps both tables non-empty
  hd.push_back(fk::Cx<double>{1., 0.});
  int rc = cuda_status(cudaMemcpyAsync(twr, hr.data(), sizeof(fk::Cx<R>) * hr.size(),
                                       cudaMemcpyHostToDevice, st));
  if (rc == PWD_OK)
    rc = cuda_status(cudaMemcpyAsync(twd, hd.data(), sizeof(fk::Cx<double>) * hd.size(),
                                     cudaMemcpyHostToDevice, st));
  if (rc != PWD_OK) return rc;
  const fk::Cx<R>* tw_t = twr;
  const fk::Cx<R>* tw_k = twr + nf / 2;
  const fk::Cx<double>* twd_k = twd + nf / 2;
  const fk::Cx<double>* twd_t = twd;
  // 1. time FFT of every trace
  const long na = (long)n2 * nf;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             (k_fk_load<R, T><<<fk_grid(na), kFkThreads, 0, st>>>(d, a0, n1, nf, na)));
  fk::Cx<R>* a = fft_batch<R>(a0, a1, nf, n2, tw_t, false, st, &rc);
  if (rc != PWD_OK) return rc;
  // 2. rows 0 .. nf/2, FFT along space
  const long nb = (long)nrow * nk;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             (k_fk_rows<R><<<fk_grid(nb), kFkThreads, 0, st>>>(a, b0, n2, nf, nk, nb)));
  fk::Cx<R>* b = fft_batch<R>(b0, b1, nk, nrow, tw_k, false, st, &rc);
  if (rc != PWD_OK) return rc;
  // 3. cone mask, complex128
  PWD_KERNEL(PWD_FAM_OTHER, st,
             (k_fk_mask<R><<<fk_grid(nb), kFkThreads, 0, st>>>(b, c0, nrow, nk, w, nb)));
  // 4. inverse FFT along space
  fk::Cx<double>* c = fft_batch<double>(c0, c1, nk, nrow, twd_k, true, st, &rc);
  if (rc != PWD_OK) return rc;
  // 5. full spectra of the output traces, inverse FFT along time, real part
  PWD_KERNEL(PWD_FAM_OTHER, st,
             (k_fk_full<<<fk_grid(na), kFkThreads, 0, st>>>(c, d0, nf, nk, nrow,
                                                            1.0 / (double)nk, na)));
  fk::Cx<double>* dd = fft_batch<double>(d0, d1, nf, n2, twd_t, true, st, &rc);
  if (rc != PWD_OK) return rc;
  const long no = (long)n1 * n2;
  PWD_KERNEL(PWD_FAM_OTHER, st,
             (k_fk_out<<<fk_grid(no), kFkThreads, 0, st>>>(dd, out, n1, nf, 1.0 / (double)nf,
                                                           no)));
  return cuda_status(cudaGetLastError());
}

}  // namespace
}  // namespace pwd

extern "C" size_t pwd_fkdip_workspace_size(int n1, int n2, int f64) {
  if (!pwd::fk_args_ok(n1, n2, 1.0)) return 0;
  return pwd::fk_layout(n1, n2, f64 ? sizeof(double) : sizeof(float)).total;
}

extern "C" int pwd_fkdip(const float* d, double* out, int n1, int n2, double w, void* workspace,
                         size_t workspace_bytes, pwd_stream_t stream) {
  return pwd::fk_run<float, float>(d, out, n1, n2, w, workspace, workspace_bytes,
                                   (cudaStream_t)stream);
}

extern "C" int pwd_fkdip_f64(const double* d, double* out, int n1, int n2, double w,
                             void* workspace, size_t workspace_bytes, pwd_stream_t stream) {
  return pwd::fk_run<double, double>(d, out, n1, n2, w, workspace, workspace_bytes,
                                     (cudaStream_t)stream);
}
