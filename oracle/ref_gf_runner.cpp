// ref_gf_runner.cpp - loads the reference GF kernel (compiled unchanged from
// GFM_GPU.cu into oracle/_ref/gf_ref.cubin) with the CUDA driver API and runs
// it the way GFM_GPU.cu:28-32 does: zeroed g, one launch of GF<<<N/ii, ii>>>
// with ii = (di-1)*fh+1.  Test and baseline infrastructure only.
#include <cuda.h>
#include <stdio.h>
#include <string.h>

extern "C" int ref_gf_run(const char* image_path, int bfr, int di, int dj, int dk, int fh,
                          int fv, const float* h_rho, long long n_rho, const float* h_s,
                          float* h_g, int reps, float* ms_per_launch) {
  CUresult r;
  CUdevice dev;
  CUcontext ctx;
  CUmodule mod;
  CUfunction fn;
  if ((r = cuInit(0)) != CUDA_SUCCESS) return 1;
  if ((r = cuDeviceGet(&dev, 0)) != CUDA_SUCCESS) return 2;
  if ((r = cuDevicePrimaryCtxRetain(&ctx, dev)) != CUDA_SUCCESS) return 3;
  if ((r = cuCtxPushCurrent(ctx)) != CUDA_SUCCESS) return 4;
  int rc = 0;
  CUdeviceptr d_r = 0, d_g = 0, d_s = 0;
  CUevent e0 = nullptr, e1 = nullptr;
  int ii = (di - 1) * fh + 1;
  long long N = n_rho;
  size_t M = (size_t)di * dj;
  if (cuModuleLoad(&mod, image_path) != CUDA_SUCCESS) { rc = 5; goto out_ctx; }
  if (cuModuleGetFunction(&fn, mod, "_Z2GFiiiiiiPfS_S_") != CUDA_SUCCESS) { rc = 6; goto out_mod; }
  if (cuMemAlloc(&d_r, 4 * N) || cuMemAlloc(&d_g, 4 * M) || cuMemAlloc(&d_s, 4 * M)) {
    rc = 7;
    goto out_mem;
  }
  cuMemcpyHtoD(d_r, h_rho, 4 * N);
  cuMemcpyHtoD(d_s, h_s, 4 * M);
  cuEventCreate(&e0, 0);
  cuEventCreate(&e1, 0);
  {
    void* args[] = {&bfr, &di, &dj, &dk, &fh, &fv, &d_g, &d_r, &d_s};
    unsigned grid = (unsigned)(N / ii);
    float total = 0.f;
    for (int it = 0; it < (reps > 0 ? reps : 1); it++) {
      cuMemsetD32(d_g, 0, M);
      cuEventRecord(e0, 0);
      if (cuLaunchKernel(fn, grid, 1, 1, ii, 1, 1, 0, 0, args, nullptr) != CUDA_SUCCESS) {
        rc = 8;
        goto out_mem;
      }
      cuEventRecord(e1, 0);
      if (cuEventSynchronize(e1) != CUDA_SUCCESS) { rc = 9; goto out_mem; }
      float ms = 0.f;
      cuEventElapsedTime(&ms, e0, e1);
      if (it > 0 || reps <= 1) total += ms;
    }
    if (ms_per_launch) *ms_per_launch = total / (reps > 1 ? reps - 1 : 1);
  }
  cuMemcpyDtoH(h_g, d_g, 4 * M);
out_mem:
  if (e0) cuEventDestroy(e0);
  if (e1) cuEventDestroy(e1);
  if (d_r) cuMemFree(d_r);
  if (d_g) cuMemFree(d_g);
  if (d_s) cuMemFree(d_s);
out_mod:
  cuModuleUnload(mod);
out_ctx:
  cuCtxPopCurrent(&ctx);
  cuDevicePrimaryCtxRelease(dev);
  return rc;
}
