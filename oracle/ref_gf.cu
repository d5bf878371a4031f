// Compiles the reference GF kernel (GFM_GPU.cu:16-22) UNCHANGED from the
// reference sources, for timing and golden vectors only.  The reference's
// host main() is renamed so that only the kernel is used.  Built by
// oracle/build.py into oracle/_ref/ (never committed, never shipped).
#define main ztm_ref_gfm_main
#include ZTM_REF_GFM
