// mhd_fast.cu -- the ideal-MHD VL step in fast FP64: the same source as the exact form with
// multiply-adds contracted into FMAs (fewer FP64 instructions; results within rounding of
// the reference's).  Body: mhd_body.cuh.
#define CGB_MHD_NS mxf
#define CGB_MHD_STEP mhd_fast_step
#define CGB_MHD_REDUCTIONS 0
#include "mhd_body.cuh"
