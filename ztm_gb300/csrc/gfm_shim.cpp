// gfm_shim.cpp - drop-in for the reference's ./GFM executable.
//
// TFM.cpp:90-94 writes /dev/shm/R.dat (float32 drho, fine grid) and
// /dev/shm/S.dat (float32 station heights, di*dj), runs ./GFM, and reads
// /dev/shm/G.dat (float32, di*dj, mGal).  GFM_GPU.cu:24-34 does that with
// hard-coded dimensions.  This program keeps the file contract and runs the
// sum through libztmgrav.so.  Dimensions come from ZTM_GFM_DIMS
// ("di,dj,dk,fh,fv,bfr"), else from <dir>/GFM.cfg (same six integers), else
// the reference defaults 61,61,35,1,2,10 (GFM_GPU.cu:24).  <dir> is
// ZTM_GFM_DIR or /dev/shm.  ZTM_GFM_PRECISION=fp64 selects the double
// kernel (default fp32, the reference's arithmetic).  Nodes are selected by
// GF's own test on the float values of R.dat, fabs(rho) > .001f
// (GFM_GPU.cu:19), in both precisions, so that a node at exactly 0.001f is
// left out as the reference leaves it out.  A short R.dat is zero-filled (the
// reference leaves that tail uninitialised).  Exit status:
// 0 on success, 1 on a file error, 2 on a library error.
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <string>
#include <vector>

#include "ztm_grav.h"

static bool parse_dims(const char* s, int* d) {
  return s && sscanf(s, "%d,%d,%d,%d,%d,%d", &d[0], &d[1], &d[2], &d[3], &d[4], &d[5]) == 6;
}

int main() {
  const char* envdir = getenv("ZTM_GFM_DIR");
  std::string dir = envdir ? envdir : "/dev/shm";
  int d[6] = {61, 61, 35, 1, 2, 10};
  if (!parse_dims(getenv("ZTM_GFM_DIMS"), d)) {
    FILE* cfg = fopen((dir + "/GFM.cfg").c_str(), "r");
    if (cfg) {
      int t[6];
      if (fscanf(cfg, "%d %d %d %d %d %d", &t[0], &t[1], &t[2], &t[3], &t[4], &t[5]) == 6 ||
          (rewind(cfg), fscanf(cfg, "%d,%d,%d,%d,%d,%d", &t[0], &t[1], &t[2], &t[3], &t[4], &t[5]) == 6))
        memcpy(d, t, sizeof t);
      fclose(cfg);
    }
  }
  ztm_grid g;
  g.di = d[0]; g.dj = d[1]; g.dk = d[2]; g.fh = d[3]; g.fv = d[4]; g.bfr = d[5];
  g.threshold = 0.001;
  g.scale = 1.0;
  if (g.di < 1 || g.dj < 1 || g.dk < 1 || g.fh < 1 || g.fv < 1 || g.bfr < 0) {
    fprintf(stderr, "GFM: bad dimensions\n");
    return 1;
  }
  const long long ii = (long long)(g.di - 1) * g.fh + 1, jj = (long long)(g.dj - 1) * g.fh + 1,
                  kk = (long long)(g.dk - 1) * g.fv + 1;
  const long long N = ii * jj * kk, M = (long long)g.di * g.dj;
  std::vector<float> r32(N, 0.f), s32(M, 0.f), g32(M, 0.f);
  FILE* fr = fopen((dir + "/R.dat").c_str(), "rb");
  FILE* fs = fopen((dir + "/S.dat").c_str(), "rb");
  if (!fr || !fs) {
    fprintf(stderr, "GFM: cannot open %s/R.dat or S.dat\n", dir.c_str());
    if (fr) fclose(fr);
    if (fs) fclose(fs);
    return 1;
  }
  size_t nr = fread(r32.data(), 4, N, fr);
  size_t ns = fread(s32.data(), 4, M, fs);
  fclose(fr);
  fclose(fs);
  (void)nr;
  if ((long long)ns != M) {
    fprintf(stderr, "GFM: S.dat holds %zu of %lld values\n", ns, M);
    return 1;
  }
  std::vector<double> drho(r32.begin(), r32.end()), surf(s32.begin(), s32.end()), G(M);
  std::vector<int> nn;  // GF's selection, GFM_GPU.cu:19, on the float values
  for (long long n = 0; n < N; n++)
    if (fabsf(r32[n]) > .001f) nn.push_back((int)n);
  const char* prec = getenv("ZTM_GFM_PRECISION");
  int p = (prec && !strcmp(prec, "fp64")) ? ZTM_PREC_FP64 : ZTM_PREC_FP32;
  ztm_ctx* ctx = nullptr;
  int rc = ztm_ctx_create(0, &ctx);
  if (rc != ZTM_OK) {
    fprintf(stderr, "GFM: no CUDA device (status %d)\n", rc);
    return 2;
  }
  rc = ztm_gfm_pointmass(ctx, &g, drho.data(), nn.data(), (long long)nn.size(), surf.data(),
                         G.data(), p, 0);
  if (rc != ZTM_OK) {
    fprintf(stderr, "GFM: %s\n", ztm_last_error(ctx));
    ztm_ctx_destroy(ctx);
    return 2;
  }
  ztm_ctx_destroy(ctx);
  for (long long m = 0; m < M; m++) g32[m] = (float)G[m];
  FILE* fg = fopen((dir + "/G.dat").c_str(), "wb");
  if (!fg || fwrite(g32.data(), 4, M, fg) != (size_t)M) {
    fprintf(stderr, "GFM: cannot write %s/G.dat\n", dir.c_str());
    if (fg) fclose(fg);
    return 1;
  }
  fclose(fg);
  return 0;
}
