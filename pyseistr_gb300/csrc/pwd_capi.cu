// Library-wide entry points of the C ABI: version, status strings, launch
// accounting and kernel-family timing with CUDA events.
#include <atomic>
#include <mutex>
#include <vector>

#include "pwd_common.cuh"

namespace pwd {
namespace {

std::atomic<unsigned long long> g_launches{0};

struct Rec {
  int fam;
  cudaEvent_t a, b;
};

struct Profiler {
  std::mutex mu;
  bool on = false;
  std::vector<Rec> recs;
  std::vector<cudaEvent_t> pool;
  cudaEvent_t get() {
    if (!pool.empty()) {
      cudaEvent_t e = pool.back();
      pool.pop_back();
      return e;
    }
    cudaEvent_t e = nullptr;
    cudaEventCreate(&e);
    return e;
  }
};

Profiler& prof() {
  static Profiler p;
  return p;
}

thread_local cudaEvent_t t_pending = nullptr;

}  // namespace

void prof_begin(int fam, cudaStream_t st) {
  (void)fam;
  g_launches.fetch_add(1, std::memory_order_relaxed);
  Profiler& p = prof();
  if (!p.on) return;
  std::lock_guard<std::mutex> lk(p.mu);
  t_pending = p.get();
  cudaEventRecord(t_pending, st);
}

void prof_end(int fam, cudaStream_t st) {
  Profiler& p = prof();
  if (!p.on || !t_pending) return;
  std::lock_guard<std::mutex> lk(p.mu);
  cudaEvent_t b = p.get();
  cudaEventRecord(b, st);
  p.recs.push_back({fam, t_pending, b});
  t_pending = nullptr;
}

}  // namespace pwd

extern "C" int pwd_version(void) { return 100; }  // 0.1.0

extern "C" const char* pwd_status_string(int status) {
  switch (status) {
    case PWD_OK: return "ok";
    case PWD_EINVAL: return "invalid size or parameter";
    case PWD_EWORKSPACE: return "workspace missing, too small or not 256-byte aligned";
    case PWD_ECUDA: return "CUDA launch or runtime error";
    case PWD_ENOTSUP: return "parameter outside what this build supports";
  }
  return "unknown status";
}

extern "C" unsigned long long pwd_launch_count(void) { return pwd::g_launches.load(); }

extern "C" void pwd_profile_start(void) {
  pwd::Profiler& p = pwd::prof();
  std::lock_guard<std::mutex> lk(p.mu);
  p.on = true;
}

extern "C" int pwd_profile_stop(double* ms, int* launches, int nfam) {
  pwd::Profiler& p = pwd::prof();
  std::lock_guard<std::mutex> lk(p.mu);
  p.on = false;
  for (int f = 0; f < nfam; f++) {
    if (ms) ms[f] = 0.0;
    if (launches) launches[f] = 0;
  }
  int n = 0;
  for (auto& r : p.recs) {
    cudaEventSynchronize(r.b);
    float t = 0.f;
    cudaEventElapsedTime(&t, r.a, r.b);
    if (r.fam >= 0 && r.fam < nfam) {
      if (ms) ms[r.fam] += t;
      if (launches) launches[r.fam] += 1;
    }
    p.pool.push_back(r.a);
    p.pool.push_back(r.b);
    n++;
  }
  p.recs.clear();
  return n;
}

// FP32 FMA throughput probe: every thread runs 8 independent FMA chains for
// `iters` steps (16 flops a step) and folds them into out[thread], so the
// timed launch measures the CUDA-core FP32 peak that the latency-bound
// spray kernels are compared with.
namespace {
__global__ void k_fma_probe(float* out, int iters, float x, float y) {
  float a[8];
#pragma unroll
  for (int k = 0; k < 8; k++) a[k] = (float)(threadIdx.x + k);
  for (int it = 0; it < iters; it++) {
#pragma unroll
    for (int k = 0; k < 8; k++) a[k] = __fmaf_rn(a[k], x, y);
  }
  float s = 0.f;
#pragma unroll
  for (int k = 0; k < 8; k++) s = __fadd_rn(s, a[k]);
  out[blockIdx.x * (size_t)blockDim.x + threadIdx.x] = s;
}
}  // namespace

extern "C" int pwd_fp32_fma_probe(float* out, int blocks, int threads, int iters,
                                  pwd_stream_t stream) {
  if (!out || blocks < 1 || threads < 32 || threads > 1024 || iters < 1) return PWD_EINVAL;
  k_fma_probe<<<blocks, threads, 0, (cudaStream_t)stream>>>(out, iters, 0.999999f, 1e-7f);
  return pwd::cuda_status(cudaGetLastError());
}
