// mhd_fast.cu -- the ideal-MHD VL step in fast FP64: the same source as the exact form with
// quotients as reciprocal products, square roots from FP32 seeds with Newton steps, minima,
// maxima and sign tests on the integer pipe, and multiply-adds contracted into FMAs (fewer
// FP64 instructions; within rounding of the reference's results).  Body: mhd_body.cuh.
#define CGB_MHD_NS mxf
#define CGB_MHD_STEP mhd_fast_step
#define CGB_MHD_REDUCTIONS 0
#define CGB_MHD_FAST 1
#include "mhd_body.cuh"
