// temporary: adjoint and interface launchers
#include "ztm_internal.cuh"
size_t ztm_adjoint_ws(const MeshDesc&, int, int, int) { return 0; }
int ztm_launch_adjoint(ztm_ctx* c, const MeshDesc&, int, const double*, const double*, double*,
                       double, int, const ztm_opts*, WsCarver&) {
  return ztm_fail(c, ZTM_ERR_ARG, "not built yet");
}
size_t ztm_iface_ws(const IMeshDesc&, int, int, int) { return 0; }
int ztm_launch_iface_fwd(ztm_ctx* c, const IMeshDesc&, const double*, const double*, int,
                         const double*, double*, double, int, const ztm_opts*, WsCarver&) {
  return ztm_fail(c, ZTM_ERR_ARG, "not built yet");
}
int ztm_launch_iface_adj(ztm_ctx* c, const IMeshDesc&, const double*, const double*, int,
                         const double*, const double*, double*, double*, double, int,
                         const ztm_opts*, WsCarver&) {
  return ztm_fail(c, ZTM_ERR_ARG, "not built yet");
}
extern "C" int ztm_gfm_interface_misfit(ztm_ctx* c, const ztm_imesh*, const double*, const double*,
                                        int, const double*, const double*, double*, double*,
                                        double*, double*, const ztm_opts*) {
  return ztm_fail(c, ZTM_ERR_ARG, "not built yet");
}
extern "C" int ztm_gfm_batch(ztm_ctx* c, const ztm_job*, int, const ztm_opts*) {
  return ztm_fail(c, ZTM_ERR_ARG, "not built yet");
}
