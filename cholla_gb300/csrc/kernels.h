// kernels.h -- host-side entry points of the CUDA kernels (internal to libchollagb).
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"

namespace cgb
{
// FP64 hydro VL step in the reference's operation order (hydro_exact.cu).  Runs the
// predictor, the corrector and the finalize pass (DE select/sync, temperature floor when
// temp_floor != 0, and the CFL reduction into sc.dti when do_dt != 0).
// dt_dev != nullptr: the kernels read the time step from device memory (engine path).
// marks != nullptr: four events recorded before the predictor, after it, after the
// corrector and after the finalize pass (per-kernel timing).
cudaError_t hydro_exact_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                             const double *dt_dev, double U_floor, int temp_floor, int do_dt, cudaStream_t s,
                             cudaEvent_t *marks = nullptr);
// The VL step of a 2D box (nz = 1) in exact FP64, predictor and corrector (hydro_2d.cu); the caller
// runs the finalize pass.  sc.W holds the predictor's fluxes for the PCM corrector (2 nf fields).
cudaError_t hydro_2d_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                          const double *dt_dev, cudaStream_t s);
// dt_t[0] = C_cfl / max_dti (clamped so that t does not pass t_end when t_end > 0), dt_t[1] += dt_t[0]
cudaError_t cfl_dt(const unsigned long long *dti, double *dt_t, double c_cfl, double t_end, cudaStream_t s);
// Fast FP64 (mixed = 0) or mixed-precision (mixed = 1) step (hydro_fast.cu).  sc.W holds the
// primitives of Uⁿ and of U½: 2 * (nf + 1) fields of 8 bytes cover both element types.
// carry != 0 (3D boxes a caller steps repeatedly on the same state: the engine, batches): the
// finalize also writes the next step's primitives of the real cells and sets sc.status[1], after
// which a step forms only the ghost cells' primitives; the caller clears sc.status[1] whenever
// the state may have changed outside the steps.
cudaError_t hydro_fast_step(const Box &b, int recon, int solver, int mixed, double *U, const Scratch &sc, double dt,
                            const double *dt_dev, double U_floor, int temp_floor, int do_dt, cudaStream_t s,
                            cudaEvent_t *marks = nullptr, int carry = 0);
// TMA staging of the fast forms' 3D corrector sweeps (on by default; off: plain loads, same results)
void set_sweep_tma(int enable);
int sweep_tma();
// Average_Cell_Single_Field of the density for real cells left with negative density
cudaError_t negative_density_average(const Box &b, double *U, cudaStream_t s);
cudaError_t hydro_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s);
cudaError_t hydro_temperature_floor(const Box &b, double *U, double U_floor, cudaStream_t s);

// MHD (mhd_exact.cu): the VL step with HLLD and constrained transport, FP64 in the reference's
// operation order.  scratch holds mhd_scratch_doubles(b) doubles and must start zeroed.
size_t mhd_scratch_doubles(const Box &b);
// fields of that scratch: U½ (nf), 6 interface-state and 3 flux arrays (nf - 1 each), the 3 edge
// EMFs and the 3 cell-centred electric fields of the CT slopes
inline size_t mhd_scratch_fields(int nf) { return (size_t)nf + 9 * (size_t)(nf - 1) + 6; }
// dt_dev != null: dt is read on the device (the box engine keeps it there)
cudaError_t mhd_exact_step(const Box &b, int recon, double *U, double *scratch, double dt, const double *dt_dev,
                           cudaStream_t s);
// the same step with multiply-adds contracted (fast FP64 form of MHD)
cudaError_t mhd_fast_step(const Box &b, int recon, double *U, double *scratch, double dt, const double *dt_dev,
                          cudaStream_t s);
inline cudaError_t mhd_step(const Box &b, int recon, int precision, double *U, double *scratch, double dt,
                            const double *dt_dev, cudaStream_t s)
{
  return precision == 2 ? mhd_fast_step(b, recon, U, scratch, dt, dt_dev, s)
                        : mhd_exact_step(b, recon, U, scratch, dt, dt_dev, s);
}
// max inverse crossing time with the fast magnetosonic speed into *dti (cleared first)
cudaError_t mhd_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s);
// max |div B| over the real cells into *out (as the bits of a non-negative double; cleared first)
cudaError_t mhd_max_divb(const Box &b, const double *U, unsigned long long *out, cudaStream_t s);

// ---- batches: many 3D boxes of one scheme, stepped together ----
// One launch carries up to BATCH_CHUNK jobs in its parameter space (__grid_constant__), so the
// tile code reads a job's geometry and pointers from the constant bank, as the single-box
// kernels read their Box.  A batch of more jobs runs one chain of launches per chunk of jobs.
constexpr int BATCH_CHUNK    = 16;
constexpr int BATCH_MAX_JOBS = 256;
struct BatchJob {
  Box b;
  double *U;                 // state (caller-owned)
  void *W;                   // fast-path primitives: 2 * nslot * n * 8 bytes
  double *GEp, *Epre;        // dual-energy partial update, pre-sync energy
  unsigned long long *dti;   // max inverse crossing time (ordered double bits)
  int *status;               // bad-cell flags
  double *dt_t;              // [dt, t]
  double t_end;              // clamp of t (<= 0: none)
  int flags[6];              // boundary flags (ghost fill)
};
// tile kinds: cells of the padded box (256 per tile), predictor tiles (8 x 8 x 4), corrector
// sweep tiles of the chunk's tile set, real cells (256 per tile)
enum BatchKind { BK_CELLS = 0, BK_PRED, BK_SWX, BK_SWY, BK_SWZ, BK_REAL, BK_NUM };
struct BatchChunk {
  int njobs;
  int total[BK_NUM];                  // tiles of all the chunk's jobs per kind (= the grids)
  int off[BK_NUM][BATCH_CHUNK + 1];   // first tile of each job per kind
  BatchJob jobs[BATCH_CHUNK];
};
// kernel parameters may take up to 32 764 bytes (CUDA 12.1 and later, Volta and later GPUs)
static_assert(sizeof(BatchChunk) <= 32764, "a chunk must fit the kernel parameter space");
// tiles of a box per kind (the tiling the batched kernels decode) with sweep tile set `set` (0 / 1)
void batch_tiles(const Box &b, int tiles[BK_NUM], int set);
// W bytes a job needs
size_t batch_w_bytes(const Box &b);
// Launch one step of every job of chunk C on stream s (all jobs share the scheme): ghost fill,
// dt = c_cfl / max_dti (clamped to t_end), primitives, predictor, x/y/z sweeps, negative-density
// repair, finalize with the CFL reduction for the next step; one block per tile.
cudaError_t batch_chunk_step(const BatchChunk &C, int recon, int solver, int mixed, int de, int ns, double c_cfl,
                             double U_floor, int temp_floor, int set, cudaStream_t s);

// dispatch on the arithmetic: 0 = FP64 in the reference's order, 1 = mixed, 2 = fast FP64
inline cudaError_t hydro_step(const Box &b, int recon, int solver, int precision, double *U, const Scratch &sc,
                              double dt, const double *dt_dev, double U_floor, int temp_floor, int do_dt,
                              cudaStream_t s, cudaEvent_t *marks = nullptr, int carry = 0)
{
  if (precision == 0)
    return hydro_exact_step(b, recon, solver, U, sc, dt, dt_dev, U_floor, temp_floor, do_dt, s, marks);
  return hydro_fast_step(b, recon, solver, precision == 1 ? 1 : 0, U, sc, dt, dt_dev, U_floor, temp_floor,
                         do_dt, s, marks, carry);
}

// ghost-cell fill of all six faces in one launch (boundaries.cu)
cudaError_t set_boundaries(const Box &b, double *U, const int flags[6], cudaStream_t s);
}  // namespace cgb
