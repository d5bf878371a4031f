// ztm_grav.hpp - C++ convenience layer over ztm_grav.h for ZTM's own types.
// zmath's vec is std::vector<double> (zmath.cpp:19), so the gravity block of
// FM::FM (TFM.cpp:90-99) becomes one call of ztm::gfm(drho, surf, G, ...);
// on a non-zero status the caller keeps its CPU lambda (TFM.cpp:95-99).
#pragma once
#include <cstddef>
#include <vector>

#include "ztm_grav.h"

namespace ztm {

// One context per thread, created on first use and kept for the process
// (replaces the per-call process spawn and context creation of
// TFM.cpp:93 / GFM_GPU.cu:28-30).
inline ztm_ctx* thread_ctx() {
  thread_local struct Holder {
    ztm_ctx* c = nullptr;
    int rc = ztm_ctx_create(0, &c);
    ~Holder() { ztm_ctx_destroy(c); }
  } h;
  return h.rc == ZTM_OK ? h.c : nullptr;
}

// G (di*dj, mGal) from drho (fine grid, g/cc) and surf (di*dj grid-unit
// heights), over the nodes in nn (the list TFM.cpp:89 builds).
inline int gfm(const std::vector<double>& drho, const std::vector<double>& surf,
               std::vector<double>& G, const std::vector<int>& nn, int di, int dj, int dk,
               int fh = 1, int fv = 2, int bfr = 10, int precision = ZTM_PREC_FP64) {
  ztm_ctx* c = thread_ctx();
  if (!c) return ZTM_ERR_NODEV;
  ztm_grid g{di, dj, dk, fh, fv, bfr, 0.001, 1.0};
  G.assign((std::size_t)di * dj, 0.0);
  return ztm_gfm_pointmass(c, &g, drho.data(), nn.data(), (long long)nn.size(), surf.data(),
                           G.data(), precision, 0);
}

}  // namespace ztm
