// trace.cu - kernel tracing with CUDA events and the issue-rate
// micro-benchmarks used as roofline denominators.
#include <cuda_runtime.h>
#include <string.h>

#include <algorithm>
#include <vector>

#include "ztm_internal.cuh"

static cudaEvent_t prof_event(ztm_ctx* c) {
  if (!c->prof_pool.empty()) {
    cudaEvent_t e = c->prof_pool.back();
    c->prof_pool.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

ZtmProf::ZtmProf(ztm_ctx* ctx, const char* name, cudaStream_t stream)
    : c(ctx), s(stream ? stream : ctx->stream) {
  if (!c->prof) return;
  cudaStreamCaptureStatus st = cudaStreamCaptureStatusNone;
  cudaStreamIsCapturing(s, &st);
  if (st != cudaStreamCaptureStatusNone) return;  // no events inside a graph capture
  ZtmProfRec r;
  r.name = name;
  r.a = prof_event(c);
  r.b = prof_event(c);
  cudaEventRecord(r.a, s);
  b = r.b;
  c->prof_recs.push_back(r);
}

ZtmProf::~ZtmProf() {
  if (b) cudaEventRecord(b, s);
}

namespace {

// FMA chains: 8 independent chains per thread, many warps per SM.
template <typename T>
__global__ void fma_peak_kernel(T* out, int iters, T a, T b) {
  T x0 = (T)threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4, x5 = x0 + 5,
    x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = fma(x0, a, b); x1 = fma(x1, a, b); x2 = fma(x2, a, b); x3 = fma(x3, a, b);
      x4 = fma(x4, a, b); x5 = fma(x5, a, b); x6 = fma(x6, a, b); x7 = fma(x7, a, b);
    }
  }
  T s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == (T)-1.2345) out[blockIdx.x] = s;  // keeps the chains alive
}

__global__ void rsqrt_peak_kernel(float* out, int iters) {
  float x0 = 1.f + threadIdx.x, x1 = x0 + 1, x2 = x0 + 2, x3 = x0 + 3, x4 = x0 + 4,
        x5 = x0 + 5, x6 = x0 + 6, x7 = x0 + 7;
  for (int i = 0; i < iters; i++) {
#pragma unroll
    for (int u = 0; u < 16; u++) {
      x0 = rsqrtf(x0); x1 = rsqrtf(x1); x2 = rsqrtf(x2); x3 = rsqrtf(x3);
      x4 = rsqrtf(x4); x5 = rsqrtf(x5); x6 = rsqrtf(x6); x7 = rsqrtf(x7);
    }
  }
  float s = x0 + x1 + x2 + x3 + x4 + x5 + x6 + x7;
  if (s == -1.2345f) out[blockIdx.x] = s;
}

}  // namespace

extern "C" int ztm_ctx_profile(ztm_ctx* c, int enable) {
  if (!c) return ZTM_ERR_ARG;
  c->prof = enable != 0;
  return ZTM_OK;
}

extern "C" int ztm_ctx_profile_read(ztm_ctx* c, const char* name, double* ms, long long* count) {
  if (!c || !ms || !count) return ZTM_ERR_ARG;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device) cudaSetDevice(c->device);
  int rc = ztm_cuda_check(c, cudaStreamSynchronize(c->stream), "profile read");
  double tot = 0.0;
  long long n = 0;
  std::vector<ZtmProfRec> keep;
  for (auto& r : c->prof_recs) {
    if (!name || !*name || strstr(r.name, name)) {
      float t = 0.f;
      if (!rc && cudaEventElapsedTime(&t, r.a, r.b) == cudaSuccess) {
        tot += t;
        n++;
      } else {
        cudaGetLastError();
      }
      c->prof_pool.push_back(r.a);
      c->prof_pool.push_back(r.b);
    } else {
      keep.push_back(r);
    }
  }
  c->prof_recs.swap(keep);
  *ms = tot;
  *count = n;
  if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
  return rc;
}

extern "C" int ztm_measure_peak(ztm_ctx* c, int kind, double* value) {
  if (!c || !value || kind < 0 || kind > 2) return ZTM_ERR_ARG;
  int prev = -1;
  cudaGetDevice(&prev);
  if (prev != c->device) cudaSetDevice(c->device);
  const int threads = 256;
  const int blocks = 8 * std::max(c->num_sms, 1);
  const int iters = kind == 1 ? 64 : 2048;
  void* out = nullptr;
  int rc = ztm_cuda_check(c, cudaMalloc(&out, blocks * 8), "peak buffer");
  cudaEvent_t e0 = nullptr, e1 = nullptr;
  if (!rc) {
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    for (int rep = 0; rep < 3 && !rc; rep++) {
      cudaEventRecord(e0, c->stream);
      if (kind == 0)
        fma_peak_kernel<float><<<blocks, threads, 0, c->stream>>>((float*)out, iters, 0.999f, 1e-3f);
      else if (kind == 1)
        fma_peak_kernel<double><<<blocks, threads, 0, c->stream>>>((double*)out, iters, 0.999, 1e-3);
      else
        rsqrt_peak_kernel<<<blocks, threads, 0, c->stream>>>((float*)out, iters);
      cudaEventRecord(e1, c->stream);
      rc = ztm_cuda_check(c, cudaEventSynchronize(e1), "peak kernel");
    }
    float ms = 0.f;
    if (!rc) cudaEventElapsedTime(&ms, e0, e1);
    const double ops = (double)blocks * threads * iters * 16 * 8;
    if (!rc && ms > 0) *value = (kind == 2 ? ops / 1e9 : 2.0 * ops / 1e12) / (ms * 1e-3);
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
  }
  if (prev >= 0 && prev != c->device) cudaSetDevice(prev);
  return rc;
}
