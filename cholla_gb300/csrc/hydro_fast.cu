// hydro_fast.cu -- the fast forms' single-box and batch steps: primitives, the per-solver
// predictor and corrector sweeps (hydro_fast_hllc.cu, hydro_fast_roe.cu, hydro_fast_hll.cu,
// hydro_fast_exact.cu: one translation unit per Riemann solver, so that they compile in
// parallel), the negative-density repair and the FP64 finalize (dual-energy select/sync,
// temperature floor, CFL reduction).
#include "hydro_fast_body.cuh"

namespace cgb
{
#ifndef CGB_SWEEP_TMA
#define CGB_SWEEP_TMA 1  // stage the 3D sweeps' tiles with the TMA unit where W½ allows a tensor map
#endif
namespace
{
int g_sweep_tma = CGB_SWEEP_TMA;  // run-time switch (cgb_set_tma)

// ------------------------------------------------------------------------------------------
// finalize (FP64): DE select/sync, temperature floor, CFL reduction
// ------------------------------------------------------------------------------------------
__device__ __forceinline__ void block_max_to(double v, unsigned long long *dst)
{
  __shared__ double red[32];
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = hf::max_ord(v, __shfl_down_sync(0xffffffffu, v, o));
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = v;
  __syncthreads();
  if (warp == 0) {
    int const nw = (blockDim.x + 31) >> 5;
    v            = (lane < nw) ? red[lane] : -1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v = hf::max_ord(v, __shfl_down_sync(0xffffffffu, v, o));
    if (lane == 0 && v >= 0.0) atomicMax(dst, (unsigned long long)__double_as_longlong(v));
  }
}

// MIX: the mixed-precision form takes the reciprocal of the density with one Newton step and each
// cell's crossing rate in FP32; the total-minus-kinetic energy, the selection, sync, floor and the
// maximum over the box stay FP64 (maxima compare bit patterns on the integer pipe).
// Wout != null: also write the primitives of the updated real cells (the next step's Wⁿ, in the
// compute type) and set status[1], which tells the next step's k_fprims to form only the ghosts'.
template <bool MIX>
__device__ __forceinline__ void ffinalize_block(const Box &b, double *__restrict__ U, const double *__restrict__ Epre,
                                                unsigned long long *__restrict__ dti, int *__restrict__ status,
                                                double U_floor, int temp_floor, int do_dt, double idx, double idy,
                                                double idz, long long blk, void *__restrict__ Wout = nullptr)
{
  int const ng = b.ng;
  bool const one_d = (b.ny == 1 && b.nz == 1);
  int const rx = b.nx - 2 * ng, ry = one_d ? 1 : b.ny - 2 * ng, rz = one_d ? 1 : b.nz - 2 * ng;
  long long const nreal = (long long)rx * ry * rz;
  long long const r     = blk * blockDim.x + threadIdx.x;
  // binary32 1/dx, 1/dy, 1/dz of the mixed form's crossing rate, converted once per block
  __shared__ float sid[3];
  if (MIX && do_dt) {
    if (threadIdx.x == 0) sid[0] = (float)idx, sid[1] = (float)idy, sid[2] = (float)idz;
    __syncthreads();
  }
  double m = -1.0;
  if (r < nreal) {
    int x, y, z;
    real_xyz(r, rx, ry, x, y, z);
    x += ng;
    y = one_d ? 0 : y + ng;
    z = one_d ? 0 : z + ng;
    long long const n = b.n, id = b.id(x, y, z);
    double const d = U[id], d_inv = inv_density<MIX>(d);
    double const mx = U[n + id], my = U[2 * n + id], mz = U[3 * n + id];
    double const ke = kinetic(mx, my, mz, d_inv);
    double E        = U[4 * n + id];
    double ge       = 0.0;  // GasEnergy after the sync and the floor (dual energy)
    if (b.de) {
      long long const fge = (long long)(b.nf - 1) * n;
      // the maxima run on the integer pipe (max_ord), which the FP64-bound finalize leaves idle
      double Emax;
      if (one_d) {
        Emax = hf::max_ord(hf::max_ord(Epre[max(x - 1, ng)], E), Epre[min(x + 1, b.nx - ng - 1)]);
      } else {
        Emax = hf::max_ord(Epre[b.id(max(x - 1, ng), y, z)], E);
        Emax = hf::max_ord(Emax, Epre[b.id(min(x + 1, b.nx - ng - 1), y, z)]);
        Emax = hf::max_ord(Emax, Epre[b.id(x, max(y - 1, ng), z)]);
        Emax = hf::max_ord(Emax, Epre[b.id(x, min(y + 1, b.ny - ng - 1), z)]);
        Emax = hf::max_ord(Emax, Epre[b.id(x, y, max(z - 1, ng))]);
        Emax = hf::max_ord(Emax, Epre[b.id(x, y, min(z + 1, b.nz - ng - 1))]);
      }
      double const ut = E - ke;
      // Select_Internal_Energy_3D (hydro_cuda.cu:949-1016): U/E > eta1 or U/Emax > eta2
      double Ui   = (hf::ratio_gt(ut, E, ETA_1) || hf::ratio_gt(ut, Emax, ETA_2)) ? ut : U[fge + id];
      Ui          = hf::max_pos(Ui, TINY);
      U[fge + id] = Ui;
      ge          = Ui;
      E           = ke + Ui;  // Sync_Energies_3D (hydro_cuda.cu:1070-1099)
      U[4 * n + id] = E;
    }
    if (temp_floor) {  // Temperature_Floor_Kernel (hydro_cuda.cu:1117-1153)
      if (E - ke < U_floor * d) {
        E             = ke + d * U_floor;
        U[4 * n + id] = E;
      }
      if (b.de && ge < U_floor * d) {
        ge                                 = d * U_floor;
        U[(long long)(b.nf - 1) * n + id] = ge;
      }
    }
    if (bad_cell(d, E)) atomicOr(status, STATUS_NONFINITE);
    if (Wout) {  // the next step's primitives, from the values just stored
      using T = typename std::conditional<MIX, float, double>::type;
      double q[NSLOT];
      q[0] = d, q[1] = mx, q[2] = my, q[3] = mz, q[4] = E, q[5] = ge;
#pragma unroll
      for (int k = 0; k < NS_MAX; k++) q[6 + k] = k < b.ns ? U[(long long)(5 + k) * n + id] : 0.0;
      T w[NSLOT];
      prim_from_cons<T>(q, b, w);
#pragma unroll
      for (int sl = 0; sl < NSLOT; sl++)
        if (live(sl, b)) static_cast<T *>(Wout)[(long long)sl * n + id] = w[sl];
    }
    if (do_dt && MIX) {
      // the crossing rate of the cell in FP32 from its FP64 thermal energy (E - ke); the maximum
      // over the box, which sets dt, stays FP64
      float const idf = hf::to_f32(d_inv), g = b.gf;
      float const c2  = g * (g - 1.0f) * hf::to_f32(E - ke) * idf;
      float const cs  = sqrtf(fmaxf(c2, 0.0f));
      float const ax  = fabsf(hf::to_f32(mx) * idf) + cs;
      float mf;
      if (one_d) {
        mf = ax * sid[0];
      } else {
        float const ay = fabsf(hf::to_f32(my) * idf) + cs, az = fabsf(hf::to_f32(mz) * idf) + cs;
        mf = fmaxf(fmaxf(ax * sid[0], ay * sid[1]), az * sid[2]);
      }
      m = hf::to_f64(mf);
    } else if (do_dt) {  // hydroInverseCrossingTime (hydro_cuda.cu:404-419)
      double const c2 = b.gamma * (E - ke) * (b.gamma - 1.0) * d_inv;
      double const cs = hf::sqrtT(hf::max_pos(c2, 0.0));
      double const ax = fabs(mx * d_inv) + cs;
      if (one_d) {
        m = ax * idx;
      } else {  // non-negative terms: max_pos orders them by their bits
        double const ay = fabs(my * d_inv) + cs, az = fabs(mz * d_inv) + cs;
        m = hf::max_pos(hf::max_pos(ax * idx, ay * idy), hf::max_pos(az * idz, 0.0));
      }
    }
  }
  if (Wout && blk == 0 && threadIdx.x == 0) status[1] = 1;
  if (do_dt) block_max_to(m, dti);
}

template <bool MIX>
__global__ void __launch_bounds__(256) k_ffinalize(Box b, double *__restrict__ U, const double *__restrict__ Epre,
                                                   unsigned long long *__restrict__ dti, int *__restrict__ status,
                                                   double U_floor, int temp_floor, int do_dt, double idx, double idy,
                                                   double idz, void *__restrict__ Wout)
{
  ffinalize_block<MIX>(b, U, Epre, dti, status, U_floor, temp_floor, do_dt, idx, idy, idz, blockIdx.x, Wout);
}

// ==========================================================================================
// batch kernels of the steps around the solver's predictor and sweeps
// ==========================================================================================
__global__ void __launch_bounds__(256) kb_ghost(const __grid_constant__ BatchChunk C)
{
  int const tile     = blockIdx.x;
  int const j        = find_job(C, BK_CELLS, tile);
  BatchJob const &J  = C.jobs[j];
  long long const id = (long long)(tile - C.off[BK_CELLS][j]) * 256 + threadIdx.x;
  if (id < J.b.n) ghost_cell(J.b, J.U, *reinterpret_cast<const Flags *>(J.flags), id);
}

// dt = c_cfl / max_dti clamped to t_end (as k_cfl_dt), then the reduction word is cleared for
// this step's finalize
__global__ void kb_cfl(const __grid_constant__ BatchChunk C, double c_cfl)
{
  int const j = threadIdx.x;
  if (j >= C.njobs) return;
  BatchJob const &J = C.jobs[j];
  double const m    = __longlong_as_double((long long)*J.dti);
  double dt         = c_cfl / m;
  double const t    = J.dt_t[1];
  if (J.t_end > 0.0 && t + dt > J.t_end) dt = J.t_end - t;
  J.dt_t[0] = dt;
  J.dt_t[1] = t + dt;
  *J.dti    = 0ULL;
}

// Average_Cell_Single_Field of the density for real cells left with non-positive density
__global__ void __launch_bounds__(256) kb_negavg(const __grid_constant__ BatchChunk C)
{
  int const tile    = blockIdx.x;
  int const j       = find_job(C, BK_REAL, tile);
  BatchJob const &J = C.jobs[j];
  Box const &b      = J.b;
  if (!b.floor_on) return;
  long long const r = (long long)(tile - C.off[BK_REAL][j]) * 256 + threadIdx.x;
  int const ng = b.ng, rx = b.nx - 2 * ng, ry = b.ny - 2 * ng;
  if (r >= real_cells(b)) return;
  int const x = (int)(r % rx) + ng, y = (int)((r / rx) % ry) + ng, z = (int)(r / ((long long)rx * ry)) + ng;
  double *U          = J.U;
  long long const id = b.id(x, y, z);
  if (U[id] < b.density_floor && !(U[id] > 0)) {
    U[id] = (U[b.id(x - 1, y, z)] + U[b.id(x + 1, y, z)] + U[b.id(x, y - 1, z)] + U[b.id(x, y + 1, z)] +
             U[b.id(x, y, z - 1)] + U[b.id(x, y, z + 1)]) /
            6;
  }
}

template <bool MIX>
__global__ void __launch_bounds__(256)
    kb_final(const __grid_constant__ BatchChunk C, double U_floor, int temp_floor, int do_dt)
{
  int const tile    = blockIdx.x;
  int const j       = find_job(C, BK_REAL, tile);
  BatchJob const &J = C.jobs[j];
  ffinalize_block<MIX>(J.b, J.U, J.Epre, J.dti, J.status, U_floor, temp_floor, do_dt, J.b.idx, J.b.idy, J.b.idz,
                       tile - C.off[BK_REAL][j], MIX ? J.W : nullptr);
}

}  // namespace

template <int SET>
void batch_tiles_set(const Box &b, int tiles[BK_NUM])
{
  using TS = TileSet<SET>;
  int a, c, d;
  tiles[BK_CELLS] = (int)((b.n + 255) / 256);
  pred_grid(b, a, c, d);
  tiles[BK_PRED] = a * c * d;
  sweep_grid<0, TS::XL, TS::XA, TS::XB>(b, a, c, d);
  tiles[BK_SWX] = a * c * d;
  sweep_grid<1, TS::YL, TS::YA, TS::YB>(b, a, c, d);
  tiles[BK_SWY] = a * c * d;
  sweep_grid<2, TS::YL, TS::YA, TS::YB>(b, a, c, d);
  tiles[BK_SWZ] = a * c * d;
  tiles[BK_REAL] = (int)((real_cells(b) + 255) / 256);
}

void batch_tiles(const Box &b, int tiles[BK_NUM], int set)
{
  if (set == 1)
    batch_tiles_set<1>(b, tiles);
  else
    batch_tiles_set<0>(b, tiles);
}

size_t batch_w_bytes(const Box &b) { return 2 * (size_t)nslot(b) * (size_t)b.n * sizeof(double); }

cudaError_t batch_chunk_step(const BatchChunk &C, int recon, int solver, int mixed, int de, int ns, double c_cfl,
                             double U_floor, int temp_floor, int set, cudaStream_t s)
{
  if (C.njobs <= 0) return cudaSuccess;
  int const nsl = ns > 0 ? 6 + ns : 5 + (de ? 1 : 0);
  kb_ghost<<<C.total[BK_CELLS], 256, 0, s>>>(C);
  kb_cfl<<<1, BATCH_CHUNK, 0, s>>>(C, c_cfl);
  if (mixed)
    kb_prims<float><<<C.total[BK_CELLS], 256, 0, s>>>(C);
  else
    kb_prims<double><<<C.total[BK_CELLS], 256, 0, s>>>(C);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  switch (solver) {
    case SOLVER_ROE: e = batch_solver_roe(C, recon, mixed, set, nsl, s); break;
    case SOLVER_HLL: e = batch_solver_hll(C, recon, mixed, set, nsl, s); break;
    case SOLVER_EXACT: e = batch_solver_exact(C, recon, mixed, set, nsl, s); break;
    default: e = batch_solver_hllc(C, recon, mixed, set, nsl, s); break;
  }
  if (e != cudaSuccess) return e;
  kb_negavg<<<C.total[BK_REAL], 256, 0, s>>>(C);
  if (mixed)
    kb_final<true><<<C.total[BK_REAL], 256, 0, s>>>(C, U_floor, temp_floor, 1);
  else
    kb_final<false><<<C.total[BK_REAL], 256, 0, s>>>(C, U_floor, temp_floor, 1);
  return cudaGetLastError();
}

void set_sweep_tma(int enable) { g_sweep_tma = enable ? 1 : 0; }
int sweep_tma() { return g_sweep_tma; }

// bytes of W scratch the fast paths need: primitives of Uⁿ and of U½ (8 bytes covers both types)
size_t fast_scratch_bytes(const Box &b) { return 2 * (size_t)nslot(b) * (size_t)b.n * sizeof(double); }

cudaError_t hydro_fast_step(const Box &box, int recon, int solver, int mixed, double *U, const Scratch &sc, double dt,
                            const double *dt_dev, double U_floor, int temp_floor, int do_dt, cudaStream_t s,
                            cudaEvent_t *marks, int carry)
{
  Box const b = with_inverses(box);
  bool const one_d = (b.ny == 1 && b.nz == 1);
  if (b.nz < 2 * b.ng + 1) temp_floor = 0;  // the reference's temperature floor acts in 3D only
  // Primitives carried from the finalize to the next step: mixed form, 3D boxes whose finalize runs.
  // The finalize already holds 1/d and the kinetic energy, so the carry saves the U loads and the
  // FP64 work of a separate primitives pass over the real cells (256^3 mixed: 5.73 -> 5.63 ms per
  // step).  In the fast FP64 form the primitives' own FP64 products dominate, and moving them into
  // the FP64-bound finalize measured no gain (107.9 -> 108.5 ms), so that form keeps k_fprims.
  carry = carry && mixed && !one_d && b.nz >= 2 * b.ng + 1 && (b.de || temp_floor || do_dt);
  int const *cf = carry ? sc.status + 1 : nullptr;
  cudaError_t e;
  if (marks) cudaEventRecord(marks[0], s);
  {
    long long blocks = (b.n + 255) / 256;
    if (blocks > 152 * 16) blocks = 152 * 16;
    if (mixed)
      k_fprims<float><<<(unsigned)blocks, 256, 0, s>>>(b, U, (float *)sc.W, cf);
    else
      k_fprims<double><<<(unsigned)blocks, 256, 0, s>>>(b, U, (double *)sc.W, cf);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  switch (solver) {
    case SOLVER_ROE: e = fast_solver_roe(b, recon, mixed, U, sc, dt, dt_dev, s, marks); break;
    case SOLVER_HLL: e = fast_solver_hll(b, recon, mixed, U, sc, dt, dt_dev, s, marks); break;
    case SOLVER_EXACT: e = fast_solver_exact(b, recon, mixed, U, sc, dt, dt_dev, s, marks); break;
    default: e = fast_solver_hllc(b, recon, mixed, U, sc, dt, dt_dev, s, marks); break;
  }
  if (e != cudaSuccess) return e;
  if (b.floor_on && !one_d) {
    if ((e = negative_density_average(b, U, s)) != cudaSuccess) return e;
  }
  if (b.de || temp_floor || do_dt) {
    if (do_dt && (e = cudaMemsetAsync(sc.dti, 0, sizeof(unsigned long long), s)) != cudaSuccess) return e;
    int const ng = b.ng;
    long long const nreal =
        (long long)(b.nx - 2 * ng) * (one_d ? 1 : b.ny - 2 * ng) * (one_d ? 1 : b.nz - 2 * ng);
    unsigned const grid = (unsigned)((nreal + 255) / 256);
    void *const wout = carry ? sc.W : nullptr;
    if (mixed) {
      k_ffinalize<true><<<grid, 256, 0, s>>>(b, U, sc.Epre, sc.dti, sc.status, U_floor, temp_floor, do_dt, b.idx,
                                              b.idy, b.idz, wout);
    } else {
      k_ffinalize<false><<<grid, 256, 0, s>>>(b, U, sc.Epre, sc.dti, sc.status, U_floor, temp_floor, do_dt, b.idx,
                                               b.idy, b.idz, wout);
    }
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (marks) cudaEventRecord(marks[3], s);
  return cudaSuccess;
}


}  // namespace cgb
