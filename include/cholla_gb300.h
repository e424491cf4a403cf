/*
 * cholla_gb300.h -- C ABI of libchollagb, the GB300 (sm_103a) replacement for Cholla's
 * single-GPU VL hydro/MHD step.
 *
 * The entry points mirror the reference interface of the path they replace (cited per
 * function, paths relative to the cholla-hydro/cholla source tree).  Differences from the
 * reference, all at the boundary:
 *   - every function returns an int status (CGB_OK or an error code; cgb_last_error()
 *     gives the message) instead of aborting the process through GPU_Error_Check/chexit;
 *   - the scheme (reconstruction, Riemann solver, dual energy, floors, adiabatic index),
 *     which the reference fixes with compile-time macros and the global `gama`, is set at
 *     run time with cgb_set_scheme();
 *   - work is queued on the stream given to cgb_set_stream() (default: the legacy stream 0,
 *     as in the reference) and the step itself never synchronises with the host.
 * Pointers named d_* are device pointers; the state is updated in place in the
 * reference's field-major layout U[f*n_cells + i + j*nx + k*nx*ny].
 */
#ifndef CHOLLA_GB300_H
#define CHOLLA_GB300_H

#ifdef __cplusplus
extern "C" {
#endif

/* status codes */
#define CGB_OK              0
#define CGB_ERR_CUDA        1  /* a CUDA call failed (message from cudaGetErrorString) */
#define CGB_ERR_ARGS        2  /* invalid sizes, pointers or options */
#define CGB_ERR_NOMEM       3  /* device allocation of scratch failed */
#define CGB_ERR_NONFINITE   4  /* the step produced non-finite or negative density */
#define CGB_ERR_TIMEOUT     5  /* a bounded device wait ran out */
#define CGB_ERR_UNSUPPORTED 6  /* option combination not built */

/* bits of the device status word a step leaves (cgb_check_status, cgb_box_check_status,
   cgb_batch_job_status) */
#define CGB_STATUS_NEG_DENSITY 1 /* an update gave a real cell density <= 0; the step repaired it by averaging
                                    the six neighbours (hydro_cuda.cu:296 Average_Cell_Single_Field) */
#define CGB_STATUS_NONFINITE   2 /* a real cell holds non-finite density or total energy, or density <= 0
                                    after that repair: the state is unusable */
#define CGB_STATUS_TIMEOUT     4 /* a bounded device wait (a TMA copy into shared memory) ran out and its
                                    tile was left undone: the state is unusable (CGB_ERR_TIMEOUT) */
/* largest |div B| cgb_check_magnetic_divergence accepts (src/mhd/magnetic_divergence.cu:105) */
#define CGB_MAX_DIVB 1.0e-9

/* reconstruction (builds/make.type.*: -DPCM / -DPLMC / -DPPMC / -DPLMP / -DPPMP; PLMP and PPMP are
   the primitive-limited forms of src/reconstruction/plmp_cuda.cu and ppmp_cuda.cu; every
   reconstruction is built in all three arithmetic forms) */
#define CGB_PCM  0
#define CGB_PLMC 1
#define CGB_PPMC 2
#define CGB_PLMP 3
#define CGB_PPMP 4
/* Riemann solver (-DHLLC / -DROE / -DHLLD / -DHLL / -DEXACT; the hydro solvers are built in every
   arithmetic form; HLL, src/riemann_solvers/hll_cuda.cu, not in 1D or 2D, where the reference's
   VL_1D and VL_2D integrators have no HLL branch) */
#define CGB_HLLC  0
#define CGB_ROE   1
#define CGB_HLLD  2
#define CGB_HLL   3
#define CGB_EXACT 4
/* arithmetic */
#define CGB_FP64      0 /* FP64 in the reference's operation order: bit-exact with its -fmad=false build */
#define CGB_MIXED     1 /* FP32 reconstruction and fluxes, FP64 state accumulation, energy recovery and dt */
#define CGB_FP64_FAST 2 /* FP64 with reciprocal forms, per-cell primitives and FMA (not bit-exact) */

typedef struct {
  int reconstruction;    /* CGB_PCM / CGB_PLMC / CGB_PPMC / CGB_PLMP / CGB_PPMP */
  int riemann_solver;    /* CGB_HLLC / CGB_ROE / CGB_HLLD / CGB_HLL / CGB_EXACT */
  int dual_energy;       /* -DDE: GasEnergy is the last field */
  int mhd;               /* -DMHD: face-centred Bx, By, Bz follow the scalars; needs CGB_HLLD */
  int n_scalars;         /* -DSCALAR: passive scalars after Energy (0..2) */
  int density_floor;     /* -DDENSITY_FLOOR */
  int temperature_floor; /* -DTEMPERATURE_FLOOR: applied after the step, before the CFL reduction */
  int precision;         /* CGB_FP64, CGB_MIXED or CGB_FP64_FAST */
  double gamma;          /* adiabatic index: the reference's global `gama` (global.h:147) */
  double U_floor;        /* specific internal-energy floor used by the temperature floor */
} cgb_scheme;

/* Scheme for the drop-in entry points below (replaces the make.type macros and `gama`). */
int cgb_set_scheme(const cgb_scheme *scheme);
int cgb_get_scheme(cgb_scheme *scheme);
/* Stream for subsequent calls (a cudaStream_t; NULL = legacy default stream). */
int cgb_set_stream(void *stream);
const char *cgb_last_error(void);
/* Library version string. */
const char *cgb_version(void);

/* One VL step of the padded box in place.
 * Replaces VL_Algorithm_3D_CUDA (src/integrators/VL_3D_cuda.h:9-11, VL_3D_cuda.cu:38-360).
 * Same arguments and meaning; d_grav_potential, x/y/z_off, x/y/zbound, custom_grav and
 * host_grav_potential belong to the gravity build (out of scope) and must be NULL / 0
 * (non-zero custom_grav or a non-NULL potential returns CGB_ERR_UNSUPPORTED).
 * Scratch is allocated on the current device on the first call for a box shape and kept
 * until cgb_free_memory_vl_3d(); a call with a new shape, or on another device, reallocates
 * it (one scratch per process, as the reference's file-scope scratch). */
int cgb_vl_algorithm_3d(double *d_conserved, double *d_grav_potential, int nx, int ny, int nz, int x_off, int y_off,
                        int z_off, int n_ghost, double dx, double dy, double dz, double xbound, double ybound,
                        double zbound, double dt, int n_fields, int custom_grav, double density_floor,
                        double *host_grav_potential);

/* The step of cgb_vl_algorithm_3d without any device allocation (no counterpart in the
 * reference).  For callers that cannot let the library allocate device memory: a host
 * program that has handed the device's memory to its own pool before stepping, and one that
 * overlaps the step with work on other streams and cannot take the device-wide
 * synchronisation that a first-call cudaMalloc, or the cudaFree of a shape change, implies.
 * Scratch comes from a 24 MiB file-scope __device__ array of the library, which the CUDA driver
 * maps with the module's static data (under lazy module loading: on first use, so the first
 * call on a device is when those 24 MiB leave the free pool).  Its address is looked up once
 * per device (cudaGetSymbolAddress, with that device current) on the first call there, so
 * make that first call before capturing any stream that will contain this call.
 * Limit: a box whose scratch exceeds the pool is rejected with CGB_ERR_ARGS and a message.  With
 * n padded cells and f fields the scratch is (f + 2) * 8 * n bytes with CGB_FP64 and
 * (2 f + 4) * 8 * n bytes with CGB_FP64_FAST or CGB_MIXED, each array rounded up to 256 bytes,
 * plus 512 bytes: with 6 fields, fewer than 393,216 padded cells (e.g. 73^3) in FP64 and fewer
 * than 196,608 (e.g. 58^3) in the fast forms.  The FP64 form has no room for the sweeps'
 * accumulator here, so it runs the corrector as one fused tile per 8 x 8 x 4 cells: the same
 * result bit for bit as cgb_vl_algorithm_3d, at about 0.8x its speed.  Each call clears the
 * pool's status word on the stream before the step; nothing else in the pool needs to start at
 * zero.  There is one pool per device: calls that can overlap in time (from several host
 * threads, or queued on streams that run concurrently) race on it and corrupt each other's
 * results, so serialise them.  The pool's address is cached per device ordinal for the life of
 * the process: after cudaDeviceReset (or any teardown of the device's primary context) do not
 * call this entry point again in that process. */
int cgb_vl_algorithm_3d_static(double *d_conserved, double *d_grav_potential, int nx, int ny, int nz, int x_off,
                               int y_off, int z_off, int n_ghost, double dx, double dy, double dz, double xbound,
                               double ybound, double zbound, double dt, int n_fields, int custom_grav,
                               double density_floor, double *host_grav_potential);

/* Bad-cell report of the drop-in steps (cgb_vl_algorithm_3d, cgb_vl_algorithm_1d): the status
 * bits (CGB_STATUS_*) their steps collected since the last call, which clears them; synchronises
 * the library's stream.  Returns CGB_ERR_NONFINITE (message in cgb_last_error) when
 * CGB_STATUS_NONFINITE is set.  The reference prints such cells from the device and carries on
 * (src/hydro/hydro_cuda.cu:381-389); this library counts them on the device and reports on request,
 * so the step itself never synchronises. */
int cgb_check_status(int *flags);

/* Replaces VL_Algorithm_1D_CUDA (src/integrators/VL_1D_cuda.h, VL_1D_cuda.cu:30-146). */
int cgb_vl_algorithm_1d(double *d_conserved, int nx, int x_off, int n_ghost, double dx, double xbound, double dt,
                        int n_fields, int custom_grav);

/* Replaces VL_Algorithm_2D_CUDA (src/integrators/VL_2D_cuda.h:9-10, VL_2D_cuda.cu:25-174): one VL step of
 * an nx x ny padded box (one cell deep), in place.  As the reference's 2D integrator: no density floor,
 * no HLL solver, and with PCM the corrector reuses the predictor's fluxes of Uⁿ.  Exact FP64 form only;
 * custom_grav must be 0.  Scratch is shared with cgb_vl_algorithm_3d (same rules). */
int cgb_vl_algorithm_2d(double *d_conserved, int nx, int ny, int x_off, int y_off, int n_ghost, double dx, double dy,
                        double xbound, double ybound, double dt, int n_fields, int custom_grav);

/* Replaces Free_Memory_VL_3D (VL_3D_cuda.cu:362-377).  Frees the library's scratch only,
 * on the device that owns it whatever the current device: unlike the reference it does not
 * free the caller's d_conserved. */
int cgb_free_memory_vl_3d(void);

/* Replaces Calc_dt_GPU (src/hydro/hydro_cuda.h:69-70, hydro_cuda.cu:562-597): writes the
 * maximum inverse crossing time over the real cells to *max_dti (host).  As in the
 * reference this synchronises the stream; dt = C_cfl / max_dti. */
int cgb_calc_dt_gpu(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx,
                    double dy, double dz, double gamma, double *max_dti);

/* Replaces Apply_Temperature_Floor (src/hydro/hydro_cuda.cu:1103-1115). */
int cgb_apply_temperature_floor(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                double U_floor);

/* Ghost-cell fill of all faces of a single-GPU machine.  Replaces Grid3D::Set_Boundaries for
 * flags 1 periodic, 2 reflective, 3 transmissive (with the hydro inflow diode), 4 custom
 * (left untouched) (src/grid/boundary_conditions.cpp:165-417, cuda_boundaries.cu:71-300).
 * flags[6] = {x-lower, x-upper, y-lower, y-upper, z-lower, z-upper}. */
int cgb_set_boundaries(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, const int flags[6]);

/* Maximum |div B| (MHD) over the cells with x, y, z >= 2 of the whole box, upper ghost layers
 * included, as the reference's thread guard has it: fill the ghost cells first.  Replaces
 * calculateMagneticDivergence / checkMagneticDivergence (src/mhd/magnetic_divergence.cu:33-105);
 * writes the value to *max_divb (host).  n_ghost is checked like every entry point's but does
 * not change the range. */
int cgb_max_magnetic_divergence(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                double dx, double dy, double dz, double *max_divb);
/* The reference's checkMagneticDivergence (src/mhd/magnetic_divergence.cu:92-120): the same maximum
 * into *max_divb, and CGB_ERR_NONFINITE (instead of the reference's process exit) when it exceeds
 * CGB_MAX_DIVB or is negative or NaN. */
int cgb_check_magnetic_divergence(const double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields,
                                  double dx, double dy, double dz, double *max_divb);

/* ---- box handles: device-resident stepping of many boxes (no counterpart in the reference,
 * which can hold one box shape per process: its scratch is file-scope globals) ---- */
typedef struct cgb_box cgb_box;

/* Create a box of padded size nx*ny*nz (ny = nz = 1 for 1D) with its own scratch.
 * flags[6]: boundary flags as in cgb_set_boundaries, applied before every step. */
int cgb_box_create(cgb_box **box, int nx, int ny, int nz, int n_ghost, double dx, double dy, double dz,
                   const cgb_scheme *scheme, const int flags[6]);
int cgb_box_destroy(cgb_box *box);
int cgb_box_n_fields(const cgb_box *box);
/* Set the simulation time and the end time dt is clamped to (t_end <= 0: no clamp). */
int cgb_box_set_time(cgb_box *box, double t, double t_end);
/* Replay each step from a captured CUDA graph (needs a non-default stream). */
int cgb_box_use_graph(cgb_box *box, int enable);
/* Record per-kernel times with events on the launching stream (no extra synchronisation;
 * graph replay is off while timing). */
int cgb_box_enable_timing(cgb_box *box, int enable);
/* Summed predictor / corrector / finalize milliseconds and the number of timed steps. */
int cgb_box_kernel_times(cgb_box *box, double ms[3], long long *steps);
/* Advance n_steps: ghost fill, dt = c_cfl / max inverse crossing time of the current state
 * (clamped to t_end), VL step, temperature floor, CFL reduction for the next step.  The time
 * step never leaves the device; nothing synchronises with the host. */
int cgb_box_advance(cgb_box *box, double *d_conserved, int n_steps, double c_cfl, void *stream);
/* Current time and last dt (synchronises the last stream used with the box).  Returns
 * CGB_ERR_NONFINITE, with t and dt_last filled in, while the box's status word records a bad cell. */
int cgb_box_get_time(cgb_box *box, double *t, double *dt_last);
/* Status bits (CGB_STATUS_*) of the box's steps since the last call, which clears them (synchronises
 * the box's last stream); CGB_ERR_NONFINITE when CGB_STATUS_NONFINITE is set. */
int cgb_box_check_status(cgb_box *box, int *flags);
const char *cgb_box_last_error(void);

/* ---- batches: many independent 3D boxes of one scheme advanced together (no counterpart in
 * the reference).  Every job keeps its own state (caller-owned, device resident), scratch, dt
 * and time; one step of the batch is one chain of launches per 16 jobs over the tiles of all
 * of them, and one chain of the single-box step per large job (the chains run side by side),
 * replayed from a captured CUDA graph.  Jobs join and
 * leave between steps (the graph is captured again at the next step).  Fast FP64 or mixed
 * precision, hydro. ---- */
typedef struct cgb_batch cgb_batch;


/* stream: the batch's own cudaStream_t (required); c_cfl: CFL number of every job. */
int cgb_batch_create(cgb_batch **batch, const cgb_scheme *scheme, double c_cfl, void *stream);
int cgb_batch_destroy(cgb_batch *batch);
/* Library scratch (bytes) a job of padded size nx*ny*nz takes, for admission by free memory. */
long long cgb_batch_job_bytes(const cgb_batch *batch, int nx, int ny, int nz);
/* Add a box (ghosts refilled every step with flags[6], t_end <= 0: no end time); its first dt
 * comes from a CFL reduction of d_conserved queued now. */
int cgb_batch_add(cgb_batch *batch, double *d_conserved, int nx, int ny, int nz, int n_ghost, double dx, double dy,
                  double dz, const int flags[6], double t_end, int *job_id);
int cgb_batch_remove(cgb_batch *batch, int job_id);
int cgb_batch_n_jobs(const cgb_batch *batch);
/* Hold a job out of the steps (hold = 1) or release it (0); a held job keeps its state, time and
 * pending dt and resumes where it stopped.  Takes effect at the next step. */
int cgb_batch_hold(cgb_batch *batch, int job_id, int hold);
/* Jobs of at least `cells` padded cells (default 2^21) run solo: a chain of the single-box step
 * of their own (the box engine's kernels), the others share the batched kernels.  Same results
 * for a job whatever shares the batch; takes effect at the next step. */
int cgb_batch_set_solo_cells(cgb_batch *batch, long long cells);
/* Spread the jobs over at least `chains` parallel chains of launches (default 1; a chain holds
 * at most 16 jobs), balanced by cells.  Same results bit for bit; takes effect at the next step. */
int cgb_batch_set_chains(cgb_batch *batch, int chains);
/* Sweep tile set (0 or 1) of the jobs that share the batched kernels: two compiled tile shapes of the
 * corrector sweeps, for the autotuner to pick between per size mix; takes effect at the next step.
 * The two agree to rounding (the compiler contracts a few products differently in each). */
int cgb_batch_set_tiles(cgb_batch *batch, int set);
/* Advance every job by n_steps on the batch stream (no host synchronisation). */
int cgb_batch_step(cgb_batch *batch, int n_steps);
/* Time and last dt of one job (synchronises the batch stream).  Returns CGB_ERR_NONFINITE, with t and
 * dt_last filled in, while the job's status word records a bad cell (the other jobs are unaffected). */
int cgb_batch_job_time(cgb_batch *batch, int job_id, double *t, double *dt_last);
/* Status bits (CGB_STATUS_*) of one job's steps so far (not cleared; synchronises the batch stream);
 * CGB_ERR_NONFINITE when CGB_STATUS_NONFINITE is set. */
int cgb_batch_job_status(cgb_batch *batch, int job_id, int *flags);
const char *cgb_batch_last_error(void);

/* ---- self-check: the integer-pipe binary64 <-> binary32 conversions of the mixed form against
 * the hardware conversions, on the n doubles at d_values (and the binary32 in each low word);
 * mismatches[0] (narrowing) and [1] (widening) receive the counts.  Synchronises `stream`. ---- */
int cgb_selftest_conversions(const double *d_values, long long n, unsigned long long *mismatches, void *stream);
/* ---- self-check: the fast FP64 form's reciprocal and square root (an FP32 estimate refined in FP64)
 * beside CUDA's correctly rounded ones, on the n doubles at d_values: d_out[0..n) the fast
 * 1/x, [n..2n) CUDA's 1/x, [2n..3n) the fast sqrt(|x|), [3n..4n) CUDA's sqrt(|x|).  Synchronises
 * `stream`. ---- */
int cgb_selftest_fast_math(const double *d_values, long long n, double *d_out, void *stream);
/* FP64 fused multiply-adds per second of the whole GPU (8 blocks per SM of 256 threads, each 8
 * independent FMA chains of `iters` steps), timed with events on `stream`: the FP64-pipe ceiling
 * that the FP64 forms' kernels are measured against. */
int cgb_selftest_fp64_rate(int iters, double *fma_per_s, void *stream);
/* ---- self-check of the bounded waits: a kernel whose mbarrier expects bytes that no copy delivers
 * waits `limit` polls, gives up, and writes CGB_STATUS_TIMEOUT to *d_status (device int); no copy is
 * ever issued, so nothing is left in flight.  Synchronises `stream`. ---- */
int cgb_selftest_tma_timeout(int *d_status, unsigned limit, void *stream);
/* ---- TMA staging of the fast forms' 3D corrector sweeps: on (1, default) or off (0: every thread
 * loads its share of the tile).  The two are separate kernels of the same tile code and agree to
 * rounding (the code generator contracts a few products differently in each). ---- */
int cgb_set_tma(int enable);

/* ---- fault injection for tests (no counterpart in the reference): the n-th device allocation the
 * library makes from now on (1 = the next; 0 = off) reports out-of-memory without calling CUDA, so
 * each entry point's CGB_ERR_NOMEM path can be exercised on the host.  Nothing runs on the GPU. ---- */
int cgb_debug_fail_alloc(int n);

/* ---- initial conditions on the device (the serving workload's problems) ---- */
/* Blast: uniform density rho and pressure p, plus thermal energy `energy` spread uniformly
 * over the cells whose centre lies within `radius` of (cx, cy, cz) (box coordinates of the real
 * region, origin at its lower corner).  Zero velocity.  GasEnergy (dual_energy) consistent. */
int cgb_ic_blast(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx, double dy,
                 double dz, double cx, double cy, double cz, double radius, double energy, double rho, double p,
                 double gamma, int dual_energy, void *stream);
/* Shock tube along the unit normal (nxv, nyv, nzv) through (cx, cy, cz): (rho_l, p_l) where
 * (r - c).n < 0, (rho_r, p_r) elsewhere, zero velocity. */
int cgb_ic_shock_tube(double *d_conserved, int nx, int ny, int nz, int n_ghost, int n_fields, double dx, double dy,
                      double dz, double cx, double cy, double cz, double nxv, double nyv, double nzv, double rho_l,
                      double p_l, double rho_r, double p_r, double gamma, int dual_energy, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* CHOLLA_GB300_H */
