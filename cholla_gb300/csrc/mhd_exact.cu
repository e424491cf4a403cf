// mhd_exact.cu -- the ideal-MHD VL step in the reference's arithmetic, bit-identical to the
// reference build (this file is compiled with -fmad=false).  Body: mhd_body.cuh.
#define CGB_MHD_NS mx
#define CGB_MHD_STEP mhd_exact_step
#define CGB_MHD_REDUCTIONS 1
#define CGB_MHD_FAST 0
#include "mhd_body.cuh"
