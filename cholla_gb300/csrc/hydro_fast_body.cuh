// hydro_fast_body.cuh -- throughput forms of the fused VL hydro step: fast FP64 (T = double) and
// mixed precision (T = float: reconstruction and fluxes in FP32; conserved accumulation,
// total-minus-kinetic energy, dual-energy selection and the CFL reduction in FP64).
//
//   prims      Uⁿ (FP64) -> Wⁿ: primitives in T, once per cell, pressure recovered in FP64
//   predictor  Wⁿ tile -> PCM + Riemann (T) -> half update in FP64 -> primitives of U½ (T)
//              written as W½; GasEnergy pdV partial update (FP64)
//   corrector  W½ -> x, y, z sweeps of reconstruction + Riemann (T) into register
//              accumulators -> Uⁿ⁺¹ = Uⁿ + ΔU in FP64, in place
//   finalize   dual-energy select/sync, temperature floor, CFL reduction (FP64)
//
// Quantities travel in fixed slots: 0 d, 1-3 velocity / momentum, 4 p / E, 5 GasEnergy,
// 6.. passive scalars, so every register-array index is a compile-time constant.
//
// This header holds the kernels and launchers as templates.  hydro_fast.cu runs the steps around
// the Riemann solver (primitives, negative-density repair, finalize); the predictor and the
// sweeps are instantiated once per solver in hydro_fast_hllc.cu, hydro_fast_roe.cu,
// hydro_fast_hll.cu and hydro_fast_exact.cu, which compile in parallel.
#pragma once
#include <type_traits>

#include "common.cuh"
#include "ghost.cuh"
#include "hydro_fast.cuh"
#include "hydro_math.cuh"
#include "kernels.h"
#include "tma.cuh"

namespace cgb
{
// The predictor and the corrector's three sweeps of one box (after the primitives, before the
// negative-density repair and the finalize) and of one batch chunk, for one Riemann solver; each
// pair is defined in that solver's translation unit.
cudaError_t fast_solver_hllc(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                             const double *dtp, cudaStream_t s, cudaEvent_t *marks);
cudaError_t fast_solver_roe(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                            const double *dtp, cudaStream_t s, cudaEvent_t *marks);
cudaError_t fast_solver_hll(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                            const double *dtp, cudaStream_t s, cudaEvent_t *marks);
cudaError_t batch_solver_hllc(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s);
cudaError_t batch_solver_roe(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s);
cudaError_t batch_solver_hll(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s);
cudaError_t fast_solver_exact(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                              const double *dtp, cudaStream_t s, cudaEvent_t *marks);
cudaError_t batch_solver_exact(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s);

namespace
{

constexpr int NSLOT = 6 + NS_MAX;
// tiles of the 3D step (single boxes and batches alike): predictor 8 x 8 x 4 cells; corrector
// sweeps along x over 30 x 2 x 4 cells, along y and z over 30 x 8 x 1.  Measured at 256^3 on
// GB300 (PPMC + HLLC, dual energy): against 64 x 2 x 2 / 32 x 8 x 1 the sweeps take 1 % less in
// the mixed form and 2 % less in the fast FP64 form; 6 / 3 resident blocks target 1 % less than
// 5 / 2 in the mixed form.
constexpr int PTX = 8, PTY = 8, PTZ = 4;
constexpr int PRED_SIDEQ = 6;  // direction-free Riemann side quantities per cell in the predictor tile
template <typename T>
constexpr bool pred_sideq()
{
  return sizeof(T) == 8;
}
// (compile-time tunables: the tile shapes and the resident blocks per SM the sweeps' register
// budget targets, FP32 and FP64 compute)
#ifndef CGB_SWEEP_XL  // x sweep: cells per pencil, pencils along y and along z
#define CGB_SWEEP_XL 30
#define CGB_SWEEP_XA 2
#define CGB_SWEEP_XB 4
#endif
#ifndef CGB_SWEEP_YL  // y and z sweeps: cells per pencil, x-adjacent pencils, pencils across
#define CGB_SWEEP_YL 30
#define CGB_SWEEP_YA 8
#define CGB_SWEEP_YB 1
#endif
#ifndef CGB_SWEEP_MINB_F32
#define CGB_SWEEP_MINB_F32 6
#endif
#ifndef CGB_SWEEP_MINB_F64
#define CGB_SWEEP_MINB_F64 3
#endif
constexpr int SXL = CGB_SWEEP_XL, SXA = CGB_SWEEP_XA, SXB = CGB_SWEEP_XB;
constexpr int SYL = CGB_SWEEP_YL, SYA = CGB_SWEEP_YA, SYB = CGB_SWEEP_YB;
// the batches' second tile set (cgb_batch_set_tiles; the autotuner picks between the two)
#ifndef CGB_SWEEP_ALT_XL
#define CGB_SWEEP_ALT_XL 64
#define CGB_SWEEP_ALT_XA 2
#define CGB_SWEEP_ALT_XB 2
#define CGB_SWEEP_ALT_YL 32
#define CGB_SWEEP_ALT_YA 8
#define CGB_SWEEP_ALT_YB 1
#endif
template <int SET>
struct TileSet {
  static constexpr int XL = SXL, XA = SXA, XB = SXB, YL = SYL, YA = SYA, YB = SYB;
};
template <>
struct TileSet<1> {
  static constexpr int XL = CGB_SWEEP_ALT_XL, XA = CGB_SWEEP_ALT_XA, XB = CGB_SWEEP_ALT_XB;
  static constexpr int YL = CGB_SWEEP_ALT_YL, YA = CGB_SWEEP_ALT_YA, YB = CGB_SWEEP_ALT_YB;
};

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// q = n / d and r = n % d for 0 <= n < 2^22 and d >= 1 from an FP32 reciprocal (relative error
// below 2^-22, so the estimate is off by at most one and one correction makes it exact); larger
// n take the integer division
__device__ __forceinline__ int divmod(int n, int d, int &r)
{
  int q;
  if (n < (1 << 22)) {
    q = __float2int_rz(__int2float_rn(n) * __frcp_rn(__int2float_rn(d)));
    r = n - q * d;
    if (r < 0) {
      q -= 1, r += d;
    } else if (r >= d) {
      q += 1, r -= d;
    }
  } else {
    q = n / d, r = n - q * d;
  }
  return q;
}

// real-cell coordinates of the linear real index i (x fastest) in 32-bit arithmetic when i fits
__device__ __forceinline__ void real_xyz(long long i, int rx, int ry, int &x, int &y, int &z)
{
  if (i < 0x7fffffffLL) {
    unsigned const u = (unsigned)i, q = u / (unsigned)rx;
    x = (int)(u - q * (unsigned)rx), y = (int)(q % (unsigned)ry), z = (int)(q / (unsigned)ry);
  } else {
    long long const q = i / rx;
    x = (int)(i - q * rx), y = (int)(q % ry), z = (int)(q / ry);
  }
}

// number of slots a box carries and which of them are live
__host__ __device__ __forceinline__ int nslot(const Box &b) { return b.ns > 0 ? 6 + b.ns : 5 + b.de; }
__device__ __forceinline__ bool live(int s, const Box &b)
{
  return s < 5 || (s == 5 && b.de) || (s >= 6 && s - 6 < b.ns);
}
// state field of slot s (unrotated)
__device__ __forceinline__ long long field(int s, const Box &b) { return s < 5 ? s : s == 5 ? b.nf - 1 : s - 1; }
// slot of the rotated quantity q for a sweep with momenta (o1, o2, o3)
__device__ __forceinline__ int rot(int q, int o1, int o2, int o3)
{
  return q == 1 ? o1 : q == 2 ? o2 : q == 3 ? o3 : q;
}

// 1/d in FP64 from an FP32 estimate and `steps` Newton steps (2 FP64 FMAs each)
template <int steps>
__device__ __forceinline__ double rcp_nr(double d)
{
  double r = hf::to_f64(__frcp_rn(hf::to_f32(d)));
#pragma unroll
  for (int i = 0; i < steps; i++) r = fma(r, fma(-d, r, 1.0), r);
  return r;
}

// FP64 value to the compute type and back (integer-pipe conversions in the mixed form)
template <typename T>
__device__ __forceinline__ T narrow(double x)
{
  if constexpr (std::is_same<T, float>::value)
    return hf::to_f32(x);
  else
    return x;
}
template <typename T>
__device__ __forceinline__ double widen(T a)
{
  if constexpr (std::is_same<T, float>::value)
    return hf::to_f64(a);
  else
    return a;
}

// gamma and 1/(gamma - 1) in the compute type
template <typename T>
__device__ __forceinline__ T gamma_of(const Box &b)
{
  if constexpr (std::is_same<T, float>::value)
    return b.gf;
  else
    return b.gamma;
}
template <typename T>
__device__ __forceinline__ T ig1_of(const Box &b)
{
  if constexpr (std::is_same<T, float>::value)
    return b.ig1f;
  else
    return b.ig1;
}

// 1/d of a cell: an FP32 estimate refined by one Newton step in the mixed form (whose primitives
// are rounded to FP32) and by two (hf::rcp) in the fast FP64 form
template <bool MIX>
__device__ __forceinline__ double inv_density(double d)
{
  if constexpr (MIX)
    return rcp_nr<1>(d);
  else
    return hf::rcp(d);
}
// kinetic energy (mx^2 + my^2 + mz^2) / 2d from 1/d, every FP64 operation explicitly rounded:
// the primitives of a cell then come out bit for bit alike in every kernel that forms them (the
// finalize writes the next step's primitives of the real cells, k_fprims those of the ghosts)
__device__ __forceinline__ double kinetic(double mx, double my, double mz, double id)
{
  return __dmul_rn(__dmul_rn(0.5, __fma_rn(mz, mz, __fma_rn(my, my, __dmul_rn(mx, mx)))), id);
}

// Primitives (T) of one cell from its FP64 conserved state q (slots), pressure recovered in
// FP64 (Load_Data, reconstruction.h:139-212; Get_Pressure_From_DE, hydro_utilities.h:136-151).
template <typename T>
__device__ __forceinline__ void prim_from_cons(const double *q, const Box &b, T *w)
{
  constexpr bool mix = std::is_same<T, float>::value;
  double const d     = q[0];
  double const id    = inv_density<mix>(d);
  double const eth   = __dsub_rn(q[4], kinetic(q[1], q[2], q[3], id));
  double p           = eth;
  if (b.de) {
    p = hf::ratio_gt(eth, q[4], ETA_1) ? eth : q[5];
    if constexpr (mix) {  // the thermal energy is selected in FP64; its scalings need not be
      w[5] = hf::to_f32(q[5]) * hf::to_f32(id);
    } else {
      p    = hf::max_pos(__dmul_rn(p, __dsub_rn(b.gamma, 1.0)), TINY);
      w[5] = __dmul_rn(q[5], id);
    }
  } else {
    if constexpr (!mix) p = hf::max_pos(__dmul_rn(__dsub_rn(b.gamma, 1.0), eth), TINY);
    w[5] = T(0);
  }
  w[0] = narrow<T>(d);
  if constexpr (mix) {
    float const idf = hf::to_f32(id);
    w[1] = hf::to_f32(q[1]) * idf;
    w[2] = hf::to_f32(q[2]) * idf;
    w[3] = hf::to_f32(q[3]) * idf;
    // p holds the FP64 thermal energy (the DE selection or E - ke): the pressure in FP32, floored
    // at TINY (a NaN stays NaN, for the bad-cell checks downstream)
    float const pf = hf::to_f32(p) * b.gm1f;
    w[4]           = pf < (float)TINY ? (float)TINY : pf;
  } else {
    w[1] = __dmul_rn(q[1], id);
    w[2] = __dmul_rn(q[2], id);
    w[3] = __dmul_rn(q[3], id);
    w[4] = p;
  }
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) {
    if constexpr (mix)
      w[6 + k] = (k < b.ns) ? hf::to_f32(q[6 + k]) * hf::to_f32(id) : 0.f;
    else
      w[6 + k] = (k < b.ns) ? __dmul_rn(q[6 + k], id) : 0.0;
  }
}

template <typename T>
__device__ __forceinline__ hf::Prim<T> prim_at(const T *P, int stride, int i, const Box &b)
{
  hf::Prim<T> s;
  s.d   = P[0 * stride + i];
  s.vn  = P[1 * stride + i];
  s.vt1 = P[2 * stride + i];
  s.vt2 = P[3 * stride + i];
  s.p   = P[4 * stride + i];
  s.ge  = b.de ? P[5 * stride + i] : T(0);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) s.sc[k] = (k < b.ns) ? P[(6 + k) * stride + i] : T(0);
  return s;
}

// the same with the sides' direction-free quantities formed beforehand (hf::side_q)
// Exact Riemann solver (exact_cuda.cu:19-334) from primitive interface states, f in the slots of
// hf::hllc_q.  The pressures are the ones the other solvers use (the DE selection, floored at TINY);
// the star state (Newton iteration on the pressure, at most 21 passes) and its sample at x/t = 0 run
// in FP64 in both forms, with the single-precision powf of the reference, and the flux follows
// exact_cuda.cu: mass flux ds vs, transverse velocities and passive quantities upwind by vs.
template <typename T>
__device__ __forceinline__ void exact_q(const hf::Prim<T> &l, const hf::Prim<T> &r, const hf::SideQ<T> &Ql,
                                        const hf::SideQ<T> &Qr, T *f, const Box &b)
{
  double const g  = b.gamma;
  double const dl = widen(l.d), vl = widen(l.vn), pl = widen(Ql.p);
  double const dr = widen(r.d), vr = widen(r.vn), pr = widen(Qr.p);
  double const cl = hf::sqrtT(g * pl * hf::rcp(dl)), cr = hf::sqrtT(g * pr * hf::rcp(dr));
  double pm = 0, vm = 0, ds = 0, vs = 0, ps = 0;
  hx::exact_star(pm, vm, dl, vl, pl, cl, dr, vr, pr, cr, g);
  hx::exact_sample(pm, vm, ds, vs, ps, dl, vl, pl, cl, dr, vr, pr, cr, g);
  bool const left = vs >= 0;
  double const vy = widen(left ? l.vt1 : r.vt1), vz = widen(left ? l.vt2 : r.vt2);
  double const m  = ds * vs;
  f[0] = narrow<T>(m);
  f[1] = narrow<T>(m * vs + ps);
  f[2] = narrow<T>(m * vy);
  f[3] = narrow<T>(m * vz);
  f[4] = narrow<T>((ps * b.ig1 + 0.5 * ds * (vs * vs + vy * vy + vz * vz) + ps) * vs);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < b.ns) f[6 + k] = narrow<T>(m * widen(left ? l.sc[k] : r.sc[k]));
  if (b.de) f[5] = narrow<T>(m * widen(left ? l.ge : r.ge));
}

template <typename T, int SOLVER>
__device__ __forceinline__ void riemann_q(const hf::Prim<T> &L, const hf::Prim<T> &R, const hf::SideQ<T> &QL,
                                          const hf::SideQ<T> &QR, T *f, const Box &b)
{
  if constexpr (SOLVER == SOLVER_ROE)
    hf::roe_q(L, R, QL, QR, f, b.ns, b.de, gamma_of<T>(b));
  else if constexpr (SOLVER == SOLVER_HLL)
    hf::hll_q(L, R, QL, QR, f, b.ns, b.de);
  else if constexpr (SOLVER == SOLVER_EXACT)
    exact_q(L, R, QL, QR, f, b);
  else
    hf::hllc_q(L, R, QL, QR, f, b.ns, b.de, gamma_of<T>(b));
}

template <typename T, int SOLVER>
__device__ __forceinline__ void riemann(const hf::Prim<T> &L, const hf::Prim<T> &R, T *f, const Box &b)
{
  if constexpr (SOLVER == SOLVER_ROE)
    hf::roe(L, R, f, b.ns, b.de, gamma_of<T>(b), ig1_of<T>(b));
  else if constexpr (SOLVER == SOLVER_HLL)
    hf::hll(L, R, f, b.ns, b.de, gamma_of<T>(b), ig1_of<T>(b));
  else if constexpr (SOLVER == SOLVER_EXACT)
    exact_q(L, R, hf::side_q<T, false>(L, b.de, gamma_of<T>(b), ig1_of<T>(b)),
            hf::side_q<T, false>(R, b.de, gamma_of<T>(b), ig1_of<T>(b)), f, b);
  else
    hf::hllc(L, R, f, b.ns, b.de, gamma_of<T>(b), ig1_of<T>(b));
}

// ------------------------------------------------------------------------------------------
// primitives of every cell of the padded box
template <typename T>
__device__ __forceinline__ void fprims_cell(const Box &b, const double *__restrict__ U, T *__restrict__ Wn, long long i)
{
  long long const n = b.n;
  double q[NSLOT];
#pragma unroll
  for (int s = 0; s < NSLOT; s++) q[s] = live(s, b) ? U[field(s, b) * n + i] : 0.0;
  T w[NSLOT];
  prim_from_cons<T>(q, b, w);
#pragma unroll
  for (int s = 0; s < NSLOT; s++)
    if (live(s, b)) Wn[(long long)s * n + i] = w[s];
}

// real cells of a 3D box and the i-th of its ghost cells (0 <= i < n - real): the two z slabs,
// then the two y slabs between them, then the two x slabs of the remaining rows
__host__ __device__ __forceinline__ long long real_count(const Box &b)
{
  return (long long)(b.nx - 2 * b.ng) * (b.ny - 2 * b.ng) * (b.nz - 2 * b.ng);
}
__device__ __forceinline__ long long ghost_cell(const Box &b, long long i)
{
  long long const nx = b.nx, ny = b.ny, ng = b.ng, plane = nx * ny;
  if (i < 2 * ng * plane) {
    long long z = i / plane;
    if (z >= ng) z += b.nz - 2 * ng;
    return z * plane + (i - (i / plane) * plane);
  }
  i -= 2 * ng * plane;
  long long const band = 2 * ng * nx;  // the two y slabs of one z plane
  if (i < band * (b.nz - 2 * ng)) {
    long long const z = i / band, r = i - z * band, yy = r / nx;
    long long const y = yy >= ng ? yy + ny - 2 * ng : yy;
    return (r - yy * nx) + nx * y + plane * (z + ng);
  }
  i -= band * (b.nz - 2 * ng);
  long long const row = i / (2 * ng), xx = i - row * 2 * ng, my = ny - 2 * ng;
  long long const x = xx >= ng ? xx + nx - 2 * ng : xx;
  return x + nx * (row % my + ng) + plane * (row / my + ng);
}

// carry != null and *carry != 0: the previous step's finalize wrote the primitives of the real
// cells (3D boxes stepped by the engine or a batch), so only the ghost shell is formed here
template <typename T>
__global__ void __launch_bounds__(256) k_fprims(Box b, const double *__restrict__ U, T *__restrict__ Wn,
                                                const int *__restrict__ carry)
{
  bool const ghosts     = carry && *carry;
  long long const count = ghosts ? b.n - real_count(b) : b.n;
  for (long long i = (long long)blockIdx.x * blockDim.x + threadIdx.x; i < count; i += (long long)gridDim.x * blockDim.x)
    fprims_cell(b, U, Wn, ghosts ? ghost_cell(b, i) : i);
}

// ------------------------------------------------------------------------------------------
// one TX x TY x TZ tile (block coordinates bx, by, bz) of the predictor
template <typename T, int TX, int TY, int TZ, int SOLVER>
__device__ __forceinline__ void fpred_tile(const Box &b, const double *__restrict__ U, const T *__restrict__ Wn,
                                           T *__restrict__ W, double *__restrict__ GEp, double dt,
                                           const double *__restrict__ dtp, int bx_, int by_, int bz_)
{
  if (dtp) dt = *dtp;
  constexpr int HY = TY > 1 ? 1 : 0, HZ = TZ > 1 ? 1 : 0;
  constexpr int BX = TX + 2, BY = TY + 2 * HY, BZ = TZ + 2 * HZ;
  constexpr int NB  = BX * BY * BZ;
  constexpr int NFX = (TX + 1) * TY * TZ;
  constexpr int NFY = HY ? TX * (TY + 1) * TZ : 0;
  constexpr int NFZ = HZ ? TX * TY * (TZ + 1) : 0;
  constexpr int NT  = TX * TY * TZ;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int const ns_ = nslot(b);
  constexpr bool PRE = pred_sideq<T>();      // side quantities formed once per cell (FP64 only)
  T *Ps  = reinterpret_cast<T *>(smem_raw);  // [slot][NB] primitives of the box
  T *Qs  = Ps + ns_ * NB;                    // [PRED_SIDEQ][NB] the cells' Riemann side quantities
  T *Fxs = Qs + (PRE ? PRED_SIDEQ * NB : 0); // [slot][faces] fluxes, conserved orientation
  T *Fys = Fxs + ns_ * NFX;
  T *Fzs = Fys + ns_ * NFY;

  int const x0 = 1 + bx_ * TX;
  int const y0 = HY ? 1 + by_ * TY : 0;
  int const z0 = HZ ? 1 + bz_ * TZ : 0;
  long long const n = b.n;
  // dt/2dx, dt/2dy, dt/2dz: formed once per block (FP64 products)
  __shared__ T sdt[3];
  if (threadIdx.x == 0) {
    sdt[0] = narrow<T>(0.5 * dt * b.idx), sdt[1] = narrow<T>(0.5 * dt * b.idy), sdt[2] = narrow<T>(0.5 * dt * b.idz);
  }

  for (int t = threadIdx.x; t < NB; t += NT) {
    int const bx = t % BX, by = (t / BX) % BY, bz = t / (BX * BY);
    long long const gid =
        b.id(clampi(x0 - 1 + bx, 0, b.nx - 1), clampi(y0 - HY + by, 0, b.ny - 1), clampi(z0 - HZ + bz, 0, b.nz - 1));
    for (int s = 0; s < ns_; s++) Ps[s * NB + t] = Wn[(long long)s * n + gid];
  }
  __syncthreads();
  // The PCM interface states are the cells: each cell's direction-free side quantities (energy,
  // used pressure, 1/d, sqrt(d), sound speed, enthalpy) are formed once here for the up to six
  // faces that read them (edge and corner cells of the halo feed no face and are skipped).  This
  // takes 30% of the fast FP64 predictor's FP64 work away; the mixed predictor, whose Riemann
  // work is FP32 and whose time goes to its FP64 half update, measured slower with the extra pass
  // (1.62 -> 1.94 ms at 256^3) and forms them per face.
  for (int t = threadIdx.x; PRE && t < NB; t += NT) {
    int const bx = t % BX, by = (t / BX) % BY, bz = t / (BX * BY);
    int const halo = (bx == 0 || bx == BX - 1) + (HY && (by == 0 || by == BY - 1)) + (HZ && (bz == 0 || bz == BZ - 1));
    if (halo > 1) continue;
    hf::SideQ<T> const q =
        hf::side_q<T, SOLVER == SOLVER_HLLC || SOLVER == SOLVER_HLL>(prim_at(Ps, NB, t, b), b.de, gamma_of<T>(b),
                                                                     ig1_of<T>(b));
    Qs[0 * NB + t] = q.E, Qs[1 * NB + t] = q.p, Qs[2 * NB + t] = q.id;
    Qs[3 * NB + t] = q.sq, Qs[4 * NB + t] = q.c, Qs[5 * NB + t] = q.h;
  }
  if (PRE) __syncthreads();

  int const nfaces = NFX + NFY + NFZ;
  for (int t = threadIdx.x; t < nfaces; t += NT) {
    int dir, i, j, k, nfd, fidx;
    T *Fd;
    if (t < NFX) {
      dir = 0, nfd = NFX, Fd = Fxs, fidx = t;
      i = t % (TX + 1), j = (t / (TX + 1)) % TY, k = t / ((TX + 1) * TY);
    } else if (t < NFX + NFY) {
      dir = 1, nfd = NFY, Fd = Fys, fidx = t - NFX;
      i = fidx % TX, j = (fidx / TX) % (TY + 1), k = fidx / (TX * (TY + 1));
    } else {
      dir = 2, nfd = NFZ, Fd = Fzs, fidx = t - NFX - NFY;
      i = fidx % TX, j = (fidx / TX) % TY, k = fidx / (TX * TY);
    }
    int const lx = (dir == 0) ? i : i + 1, ly = (dir == 1) ? j : j + HY, lz = (dir == 2) ? k : k + HZ;
    int const cl = lx + BX * (ly + BY * lz);
    int const cr = cl + (dir == 0 ? 1 : dir == 1 ? BX : BX * BY);
    int const o1 = dir + 1, o2 = (dir + 1) % 3 + 1, o3 = (dir + 2) % 3 + 1;
    hf::Prim<T> L = prim_at(Ps, NB, cl, b), R = prim_at(Ps, NB, cr, b);
    // rotate the velocities into (normal, t1, t2) with selects (a runtime-indexed array would
    // live in local memory)
    auto pick = [](T x, T y, T z, int k) { return k == 1 ? x : (k == 2 ? y : z); };
    T const ua = L.vn, ub = L.vt1, uc = L.vt2, va = R.vn, vb = R.vt1, vc = R.vt2;
    L.vn = pick(ua, ub, uc, o1), L.vt1 = pick(ua, ub, uc, o2), L.vt2 = pick(ua, ub, uc, o3);
    R.vn = pick(va, vb, vc, o1), R.vt1 = pick(va, vb, vc, o2), R.vt2 = pick(va, vb, vc, o3);
    auto sq = [&](int c) {
      hf::SideQ<T> q;
      q.E = Qs[0 * NB + c], q.p = Qs[1 * NB + c], q.id = Qs[2 * NB + c];
      q.sq = Qs[3 * NB + c], q.c = Qs[4 * NB + c], q.h = Qs[5 * NB + c];
      return q;
    };
    T f[NSLOT];
    if constexpr (PRE)
      riemann_q<T, SOLVER>(L, R, sq(cl), sq(cr), f, b);
    else
      riemann<T, SOLVER>(L, R, f, b);
#pragma unroll
    for (int q = 0; q < NSLOT; q++)
      if (live(q, b)) Fd[rot(q, o1, o2, o3) * nfd + fidx] = f[q];
  }
  __syncthreads();

  int const t = threadIdx.x;
  int const i = t % TX, j = (t / TX) % TY, k = t / (TX * TY);
  int const gx = x0 + i, gy = y0 + j, gz = z0 + k;
  bool const one_d = (b.ny == 1 && b.nz == 1);
  bool valid = gx > 0 && gx < b.nx - 1;
  if (!one_d) valid = valid && gy > 0 && gy < b.ny - 1 && gz > 0 && gz < b.nz - 1;
  if (!valid) return;
  long long const gid = b.id(gx, gy, gz);
  int const c  = (i + 1) + BX * ((j + HY) + BY * (k + HZ));
  int const fx = i + (TX + 1) * (j + TY * k);
  int const fy = i + TX * (j + (TY + 1) * k);
  int const fz = i + TX * (j + TY * k);
  T const dtodx = sdt[0], dtody = sdt[1], dtodz = sdt[2];
  double q[NSLOT];
#pragma unroll
  for (int s = 0; s < NSLOT; s++) {
    q[s] = 0.0;
    if (live(s, b)) {
      T a = dtodx * (Fxs[s * NFX + fx] - Fxs[s * NFX + fx + 1]);
      if (!one_d) {
        a += dtody * (Fys[s * NFY + fy] - Fys[s * NFY + fy + TX]);
        a += dtodz * (Fzs[s * NFZ + fz] - Fzs[s * NFZ + fz + TX * TY]);
      }
      q[s] = U[field(s, b) * n + gid] + widen(a);
    }
  }
  if (b.de) {
    // pdV source from the neighbours' cell-centred velocities of Uⁿ (hydro_cuda.cu:178-202);
    // the 1D half step takes the plain total-minus-kinetic pressure (VL_1D_cuda.cu:180-187)
    T const P = Ps[4 * NB + c];
    T Ph      = P;
    if (one_d) {
      double const d = U[gid], id = 1.0 / d;
      double const mx = U[n + gid], my = U[2 * n + gid], mz = U[3 * n + gid];
      Ph = narrow<T>((U[4 * n + gid] - 0.5 * (mx * mx + my * my + mz * mz) * id) * (b.gamma - 1.0));
    }
    T div = dtodx * (Ps[NB + c - 1] - Ps[NB + c + 1]);
    if (!one_d)
      div += dtody * (Ps[2 * NB + c - BX] - Ps[2 * NB + c + BX]) +
             dtodz * (Ps[3 * NB + c - BX * BY] - Ps[3 * NB + c + BX * BY]);
    q[5] += widen(T(0.5) * Ph * div);
    int const ng = b.ng;
    bool real    = gx >= ng && gx < b.nx - ng;
    if (!one_d) real = real && gy >= ng && gy < b.ny - ng && gz >= ng && gz < b.nz - ng;
    // full-dt partial update (hydro_cuda.cu:754-833): twice the half-step pdV term
    if (real) GEp[gid] = U[(long long)(b.nf - 1) * n + gid] + widen(P * div);
  }
  if (b.floor_on && !one_d && q[0] < b.density_floor) {
    double const s = b.density_floor / q[0];
    q[0]           = b.density_floor;
    q[1] *= s, q[2] *= s, q[3] *= s, q[4] *= s;
    if (b.de) q[5] *= s;
  }
  T w[NSLOT];
  prim_from_cons<T>(q, b, w);
#pragma unroll
  for (int s = 0; s < NSLOT; s++)
    if (live(s, b)) W[(long long)s * n + gid] = w[s];
}

#ifndef CGB_PRED_MINB_F32
#define CGB_PRED_MINB_F32 2  // resident predictor blocks per SM the FP32 register budget targets
#endif
#ifndef CGB_PRED_MINB_F64
#define CGB_PRED_MINB_F64 2  // the same for FP64 compute
#endif
template <typename T, int TX, int TY, int TZ, int SOLVER>
__global__ void __launch_bounds__(TX *TY *TZ, sizeof(T) == 4 ? CGB_PRED_MINB_F32 : CGB_PRED_MINB_F64)
    k_fpred(Box b, const double *__restrict__ U, const T *__restrict__ Wn, T *__restrict__ W, double *__restrict__ GEp,
            double dt, const double *__restrict__ dtp)
{
  fpred_tile<T, TX, TY, TZ, SOLVER>(b, U, Wn, W, GEp, dt, dtp, blockIdx.x, blockIdx.y, blockIdx.z);
}

// ------------------------------------------------------------------------------------------
// corrector: one sweep kernel per direction over long pencils
// ------------------------------------------------------------------------------------------
template <int RECON>
struct FHalo {
  static constexpr int H = (RECON == RECON_PPMC || RECON == RECON_PPMP)   ? 3
                          : (RECON == RECON_PLMC || RECON == RECON_PLMP) ? 2
                                                                         : 1;
};

// A sweep block: CS = WA * WB pencils of L cells along the sweep direction DIR.  Arrays in
// shared memory are [slot][pencil position, pencil]; along x the position is fastest (the x
// pencils are contiguous in HBM), along y and z the pencil index is (WA consecutive x cells).
// Threads of a sweep block: one per reconstructed cell (L + 2 per pencil; PCM: one per face,
// L + 1), rounded up to whole warps, so that the reconstruction and Riemann phases each take one
// pass; the update phase uses the first L * CS of them, one per updated cell.
__host__ __device__ constexpr int sweep_threads(int L, int CS, int recon)
{
  return ((recon == RECON_PCM ? L + 1 : L + 2) * CS + 31) / 32 * 32;
}

template <int DIR, int L, int WA, int WB, int RECON>
struct Sweep {
  static constexpr int H  = FHalo<RECON>::H;
  static constexpr int CS = WA * WB;
  static constexpr int NU = L * CS;  // updated cells
  static constexpr int NT = sweep_threads(L, CS, RECON);
  static constexpr int LA = L + 2 * H, LR = L + 2, LF = L + 1;
  static constexpr int NP = LA * CS, NR = LR * CS, NF = LF * CS;
  // P (loaded primitives), QL and QR (face states); the fluxes reuse P once it is consumed
  // (PCM has no face states: its fluxes follow P)
  static constexpr int PER_Q = RECON == RECON_PCM ? NP + NF : NP + 2 * NR;
  static constexpr int STRIDE = DIR == 0 ? 1 : CS;
  __device__ static int at(int a, int c, int len) { return DIR == 0 ? a + len * c : c + CS * a; }
  // TMA staging of P (y and z sweeps need WB == 1): the box of one slot lands as rows along x,
  // padded so that its first x can be rounded down to a 16-byte boundary (offset 0 .. E - 1):
  // x sweep CS rows of LAP cells, y and z sweeps LA rows of WAP cells
  template <typename T>
  struct Tma {
    static constexpr int E   = 16 / (int)sizeof(T);
    static constexpr int LAP = (LA + 2 * E - 2) / E * E;
    static constexpr int WAP = (WA + 2 * E - 2) / E * E;
    static constexpr int NPT = DIR == 0 ? LAP * CS : WAP * LA;
    static constexpr int ROW = DIR == 0 ? LAP : WAP;
    static constexpr int NPS = ((NPT > NP ? NPT : NP) + 31) / 32 * 32;  // slot stride, whole 128 bytes
    static constexpr int PER_Q = RECON == RECON_PCM ? NPS + NF : NPS + 2 * NR;
    static constexpr bool ok = DIR == 0 || WB == 1;
  };
  __device__ static void split(int i, int len, int &a, int &c)
  {
    if (DIR == 0) {
      a = i % len, c = i / len;
    } else {
      c = i % CS, a = i / CS;
    }
  }
};

// resident blocks per SM the sweeps' register budget targets: the tunables above, except for the
// exact solver, whose FP64 Newton iteration needs more registers than 6 FP32 blocks leave (it
// spilled about 1.5 KB a thread there) and targets 2
template <typename T, int SOLVER>
__host__ __device__ constexpr int sweep_min_blocks()
{
  return SOLVER == SOLVER_EXACT ? 2 : (sizeof(T) == 4 ? CGB_SWEEP_MINB_F32 : CGB_SWEEP_MINB_F64);
}

// W scratch of the fast forms: 2 * nslot * n * 8 bytes.  The first half holds Wⁿ (T) and then
// the corrector's FP64 accumulator; W½ (T) starts at the second half.
template <typename T>
__host__ __device__ __forceinline__ T *half_prims(T *Wn, const Box &b)
{
  return reinterpret_cast<T *>(reinterpret_cast<unsigned char *>(Wn) + (size_t)nslot(b) * (size_t)b.n * sizeof(double));
}

// Corrector accumulator of one field: FP64 in the fast FP64 form; in the mixed form an FP32
// pair (hi, lo) whose exact sum carries the value (Knuth's error-free TwoSum), so the sums stay
// on the FP32 pipe.  Every operation is an explicitly
// rounded intrinsic: no contraction or reassociation may change them.
template <typename T>
struct Acc;
template <>
struct Acc<double> {
  double v;
};
template <>
struct __align__(8) Acc<float> {
  float hi, lo;
};

// s + e == a + b exactly (TwoSum)
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
  s              = __fadd_rn(a, b);
  float const bb = __fsub_rn(s, a);
  e              = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
}

// the increment k * fl - k * fr of a cell from its two faces; each product is rounded once, as
// the face's other cell rounds it
// a face's flux times dt/dx, rounded once (no contraction into a later sum)
__device__ __forceinline__ double scaled_flux(double k, double f) { return __dmul_rn(k, f); }
__device__ __forceinline__ float scaled_flux(float k, float f) { return __fmul_rn(k, f); }
// a cell's increment from its low and high faces' scaled fluxes: their difference, rounded once
// in the fast FP64 form, kept error-free as an FP32 (hi, lo) pair in the mixed form
__device__ __forceinline__ Acc<double> scaled_diff(double fl, double fr) { return {__dsub_rn(fl, fr)}; }
__device__ __forceinline__ Acc<float> scaled_diff(float fl, float fr)
{
  Acc<float> r;
  two_sum(fl, -fr, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ Acc<double> acc_add(Acc<double> a, Acc<double> b) { return {__dadd_rn(a.v, b.v)}; }
__device__ __forceinline__ Acc<float> acc_add(Acc<float> a, Acc<float> b)
{
  float s, e;
  two_sum(a.hi, b.hi, s, e);
  float const t = __fadd_rn(e, __fadd_rn(a.lo, b.lo));
  Acc<float> r;  // renormalise; TwoSum, since cancellation in hi can leave |t| > |s|
  two_sum(s, t, r.hi, r.lo);
  return r;
}
__device__ __forceinline__ double acc_value(Acc<double> a) { return a.v; }
__device__ __forceinline__ double acc_value(Acc<float> a) { return __dadd_rn(hf::to_f64(a.hi), hf::to_f64(a.lo)); }

// Uⁿ⁺¹ = Uⁿ + acc in FP64 (GasEnergy from its pdV partial update), the density floor, and the
// pre-sync total energy for the dual-energy selection
__device__ __forceinline__ void final_update(const Box &b, long long gid, const double *acc, double *__restrict__ U,
                                             const double *__restrict__ GEp, double *__restrict__ Epre,
                                             int *__restrict__ status)
{
  long long const n = b.n;
  bool const one_d  = (b.ny == 1 && b.nz == 1);
  double v[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; q++) {
    v[q] = 0.0;
    if (live(q, b)) v[q] = (q == 5 ? GEp[gid] : U[field(q, b) * n + gid]) + acc[q];
  }
  if (b.floor_on && !one_d && v[0] < b.density_floor) {
    if (v[0] > 0) {
      double const sc = b.density_floor / v[0];
      v[0]            = b.density_floor;
      v[1] *= sc, v[2] *= sc, v[3] *= sc, v[4] *= sc;
      if (b.de) v[5] *= sc;
    } else {
      atomicOr(status, STATUS_NEG_DENSITY);
    }
  }
  if (not_finite(v[0]) || not_finite(v[4])) atomicOr(status, STATUS_NONFINITE);
#pragma unroll
  for (int q = 0; q < NSLOT; q++)
    if (live(q, b)) U[field(q, b) * n + gid] = v[q];
  if (b.de) Epre[gid] = v[4];
}

// Sweep DIR of the corrector: reconstruction + Riemann solve on the pencils of W½, flux
// difference dt/dx (F(i-1/2) - F(i+1/2)) per cell.  Not FINAL: the difference is added to the
// accumulator dU (the x sweep starts it).  FINAL (the last sweep): Uⁿ⁺¹ = Uⁿ + (dU + the
// difference) in FP64 in place, density floor, Epre = pre-sync total energy.
// With TMA (single boxes): the P boxes are copied by the Tensor Memory Accelerator from the tensor
// map `map` of W (4D: x, y, z, slot), one copy per slot issued by thread 0 and counted on an
// mbarrier; without, every thread loads its share of the P array.
template <typename T, int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL, bool TMA = false>
__device__ __forceinline__ void fsweep_tile(const Box &b, const T *__restrict__ W, T *__restrict__ dU,
                                            double *__restrict__ U, const double *__restrict__ GEp,
                                            double *__restrict__ Epre, int *__restrict__ status, double dt,
                                            const double *__restrict__ dtp, int bx_, int by_, int bz_,
                                            const CUtensorMap *map = nullptr)
{
  using S  = Sweep<DIR, L, WA, WB, RECON>;
  using TM = typename S::template Tma<T>;
  static_assert(!TMA || TM::ok, "TMA staging of the y and z sweeps needs WB == 1");
  constexpr int H  = S::H;
  constexpr int NT = S::NT;
  constexpr int PS = TMA ? TM::NPS : S::NP;  // P elements per slot
  constexpr int o1 = DIR + 1, o2 = (DIR + 1) % 3 + 1, o3 = (DIR + 2) % 3 + 1;
  // dt / dx of the sweep, formed once per block (an FP64 product) before the first barrier
  __shared__ T sdtod;
  if (threadIdx.x == 0) sdtod = narrow<T>((dtp ? *dtp : dt) * (DIR == 0 ? b.idx : DIR == 1 ? b.idy : b.idz));
  extern __shared__ __align__(16) unsigned char smem_raw[];
  int const ns_ = nslot(b);
  // a TMA tile copy writes to a 128-byte-aligned shared address: the P slots start at the first
  // 128-byte boundary of the dynamic shared memory (its launch adds 128 bytes for this), and every
  // slot spans whole 128 bytes (Tma::NPS)
  unsigned const pad = TMA ? (128u - (smem_u32(smem_raw) & 127u)) & 127u : 0u;
  T *Ps  = reinterpret_cast<T *>(smem_raw + pad);
  T *QLs = Ps + ns_ * PS;
  T *QRs = QLs + ns_ * S::NR;
  T *Fs  = RECON == RECON_PCM ? QLs : Ps;

  int const ng     = b.ng;
  bool const one_d = (b.ny == 1 && b.nz == 1);
  long long const n = b.n;
  int const a0 = bx_ * L, ca0 = by_ * WA, cb0 = bz_ * WB;
  // global cell of sweep position a (real-cell coordinates, may lie in the ghosts) on pencil c
  auto cell = [&](int a, int c, int &gx, int &gy, int &gz) {
    int const ca = ca0 + c % WA + ng, cb = cb0 + c / WA + ng, g = a0 + a + ng;
    if (DIR == 0) {
      gx = g, gy = one_d ? 0 : ca, gz = one_d ? 0 : cb;
    } else if (DIR == 1) {
      gy = g, gx = ca, gz = cb;
    } else {
      gz = g, gx = ca, gy = cb;
    }
  };

  // A partial tile (the box's real extent is not a multiple of the tile) skips the interface
  // states and fluxes that no real cell needs: lim = real cells of the tile along the sweep,
  // pencil_in(c) = pencil c lies inside the box.
  int const ry = b.ny - 2 * ng, rz = b.nz - 2 * ng, rx = b.nx - 2 * ng;
  int const lim = (DIR == 0 ? rx : DIR == 1 ? ry : rz) - a0;
  auto pencil_in = [&](int c) {
    return one_d || (ca0 + c % WA < (DIR == 0 ? ry : rx) && cb0 + c / WA < (DIR == 2 ? ry : rz));
  };

  int const t = threadIdx.x;
  // P index of sweep position a on pencil c, and the step between neighbouring positions
  int off = 0;  // TMA: the box's first x lies `off` cells before the block's first needed x
  auto pidx = [&](int a, int c) -> int {
    if constexpr (TMA) return DIR == 0 ? (a + off) + TM::ROW * c : (c + off) + TM::ROW * a;
    return S::at(a, c, S::LA);
  };
  constexpr int STR = TMA ? (DIR == 0 ? 1 : TM::ROW) : S::STRIDE;
  if constexpr (TMA) {
    // Every position a used face needs lies in 1 .. n-2 whatever the tile, so the unclamped boxes
    // give those positions exactly what the plain load gives them; positions past the array (a
    // partial tile) read zeros and feed only faces the tile skips.
    __shared__ uint64_t bar;
    __shared__ int aligned;
    int const xs = DIR == 0 ? a0 + ng - H : ca0 + ng;  // first needed x
    off          = (xs % TM::E + TM::E) % TM::E;  // 0 .. E - 1 (the box may start left of x = 0)
    if (t == 0) {
      // self-check before any copy: destinations on 128 bytes, the box's x on 16 bytes, the
      // mbarrier on 8; a failure skips the tile and records it instead of issuing the copy
      aligned = (smem_u32(Ps) & 127u) == 0 && ((PS * (int)sizeof(T)) & 127) == 0 && (xs - off) % TM::E == 0 &&
                (smem_u32(&bar) & 7u) == 0;
      if (aligned) {
        mbar_init(&bar, 1);
        fence_mbar_init();
      } else {
        atomicOr(status, STATUS_TMA_TIMEOUT);
      }
    }
    __syncthreads();
    if (!aligned) return;  // block-uniform
    if (t == 0) {
      mbar_arrive_expect_tx(&bar, (unsigned)(ns_ * TM::NPT * (int)sizeof(T)));
      int const xa = xs - off, s0 = a0 + ng - H;
      for (int q = 0; q < ns_; q++) {
        int const w = rot(q, o1, o2, o3);
        if (DIR == 0)
          tma_load_4d(Ps + q * PS, map, &bar, xa, ca0 + ng, cb0 + ng, w);
        else if (DIR == 1)
          tma_load_4d(Ps + q * PS, map, &bar, xa, s0, cb0 + ng, w);
        else
          tma_load_4d(Ps + q * PS, map, &bar, xa, cb0 + ng, s0, w);
      }
    }
    bool const ok = __syncthreads_and(mbar_wait(&bar, 0));
    if (!ok) {  // a copy never completed: leave the tile undone, reported through the status word
      if (t == 0) {
        atomicOr(status, STATUS_TMA_TIMEOUT);
        mbar_wait(&bar, 0);  // bounded: let a late copy land before the block's shared memory goes
      }
      return;
    }
  } else {
    // Positions past the box (a partial tile) read the nearest cell the predictor wrote (1 .. n-2;
    // the outermost layer of W½ stays zero), so their discarded states stay physical and off the
    // slow paths.  No real cell's stencil reaches the outermost layer.
    for (int p = t; p < S::NP; p += NT) {
      int a, c, gx, gy, gz;
      S::split(p, S::LA, a, c);
      cell(a - H, c, gx, gy, gz);
      long long const gid = b.id(clampi(gx, 1, b.nx - 2), one_d ? 0 : clampi(gy, 1, b.ny - 2),
                                 one_d ? 0 : clampi(gz, 1, b.nz - 2));
      for (int q = 0; q < ns_; q++) Ps[q * S::NP + p] = W[(long long)rot(q, o1, o2, o3) * n + gid];
    }
    __syncthreads();
  }
  if (RECON != RECON_PCM) {
    for (int r = t; r < S::NR; r += NT) {
      int a, c;
      S::split(r, S::LR, a, c);
      if (a > lim + 1 || !pencil_in(c)) continue;  // cell a0 + a - 1 feeds no real face
      int const base = pidx(a - 1 + H, c);
      // the stencil is read from shared memory variable by variable and each face value written
      // back as soon as it is known (a handful of live registers instead of five whole cells)
      auto ld  = [&](int j, int q) { return Ps[q * PS + base + j * STR]; };
      auto out = [&](int q, T l, T rr) {
        QLs[q * S::NR + r] = l;
        QRs[q * S::NR + r] = rr;
      };
      if constexpr (RECON == RECON_PPMC)
        hf::ppmc_cell<T>(ld, out, b.ns, b.de, gamma_of<T>(b));
      else if constexpr (RECON == RECON_PLMC)
        hf::plmc_cell<T>(ld, out, b.ns, b.de, gamma_of<T>(b));
      else if constexpr (RECON == RECON_PPMP)
        hf::ppmp_cell<T>(ld, out, b.ns, b.de);
      else
        hf::plmp_cell<T>(ld, out, b.ns, b.de);
    }
    __syncthreads();
  }
  // Conservation: each face's flux is scaled once, dtod * F rounded as one uncontracted product
  // that both of its cells read, and a cell's increment is the difference of its two faces'
  // scaled fluxes, summed over the three sweeps in an accumulator of at least 48 significant bits
  // (W^n's space, 8 bytes per field): FP64 in the fast FP64 form, an FP32 (hi, lo) pair built
  // with error-free sums in the mixed form.  So the updates telescope to accumulation roundoff.
  T const dtod = sdtod;
  for (int f = t; f < S::NF; f += NT) {
    int a, c;
    S::split(f, S::LF, a, c);  // face a lies between sweep positions a - 1 and a
    if (a > lim || !pencil_in(c)) continue;
    hf::Prim<T> Lf, Rf;
    if (RECON == RECON_PCM) {
      int const pl = pidx(a - 1 + H, c);
      Lf = prim_at(Ps, PS, pl, b);
      Rf = prim_at(Ps, PS, pl + STR, b);
    } else {
      Lf = prim_at(QLs, S::NR, S::at(a, c, S::LR), b);
      Rf = prim_at(QRs, S::NR, S::at(a + 1, c, S::LR), b);
    }
    T fl[NSLOT];
    riemann<T, SOLVER>(Lf, Rf, fl, b);
#pragma unroll
    for (int q = 0; q < NSLOT; q++)
      if (live(q, b)) Fs[q * S::NF + f] = scaled_flux(dtod, fl[q]);
  }
  __syncthreads();

  if (t >= S::NU) return;  // the threads beyond the updated cells only reconstructed and solved
  int a, c, gx, gy, gz;
  S::split(t, L, a, c);
  cell(a, c, gx, gy, gz);
  bool real = gx < b.nx - ng;
  if (!one_d) real = real && gy < b.ny - ng && gz < b.nz - ng;
  if (!real) return;
  long long const gid = b.id(gx, gy, gz);
  int const fm        = S::at(a, c, S::LF);
  Acc<T> acc[NSLOT];
#pragma unroll
  for (int q = 0; q < NSLOT; q++) {
    int const qq = q == 1 ? o1 : q == 2 ? o2 : q == 3 ? o3 : q;  // rotated momenta back to x, y, z
    if (live(q, b)) acc[qq] = scaled_diff(Fs[q * S::NF + fm], Fs[q * S::NF + fm + S::STRIDE]);
  }
  Acc<T> *__restrict__ dA = reinterpret_cast<Acc<T> *>(dU);
  if (!FIRST) {
#pragma unroll
    for (int q = 0; q < NSLOT; q++)
      if (live(q, b)) acc[q] = acc_add(dA[(long long)q * n + gid], acc[q]);
  }
  if constexpr (!FINAL) {
#pragma unroll
    for (int q = 0; q < NSLOT; q++)
      if (live(q, b)) dA[(long long)q * n + gid] = acc[q];
  } else {
    double inc[NSLOT];
#pragma unroll
    for (int q = 0; q < NSLOT; q++) inc[q] = live(q, b) ? acc_value(acc[q]) : 0.0;
    final_update(b, gid, inc, U, GEp, Epre, status);
  }
}

// Mixed-precision sweeps are latency-bound (FP32 reconstruction chains): more resident blocks
// per SM hide more of it (CGB_SWEEP_MINB_F32); the FP64 sweeps are FP64-pipe bound.
template <typename T, int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL>
__global__ void __launch_bounds__(sweep_threads(L, WA *WB, RECON), sweep_min_blocks<T, SOLVER>())
    k_fsweep(Box b, const T *__restrict__ W, T *__restrict__ dU, double *__restrict__ U,
             const double *__restrict__ GEp, double *__restrict__ Epre, int *__restrict__ status, double dt,
             const double *__restrict__ dtp)
{
  fsweep_tile<T, DIR, L, WA, WB, RECON, SOLVER, FIRST, FINAL>(b, W, dU, U, GEp, Epre, status, dt, dtp, blockIdx.x,
                                                              blockIdx.y, blockIdx.z);
}

// the same sweep with its P boxes staged by the TMA unit from the tensor map of W½
template <typename T, int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL>
__global__ void __launch_bounds__(sweep_threads(L, WA *WB, RECON), sweep_min_blocks<T, SOLVER>())
    k_fsweep_tma(Box b, const T *__restrict__ W, T *__restrict__ dU, double *__restrict__ U,
                 const double *__restrict__ GEp, double *__restrict__ Epre, int *__restrict__ status, double dt,
                 const double *__restrict__ dtp, const __grid_constant__ CUtensorMap map)
{
  fsweep_tile<T, DIR, L, WA, WB, RECON, SOLVER, FIRST, FINAL, true>(b, W, dU, U, GEp, Epre, status, dt, dtp,
                                                                    blockIdx.x, blockIdx.y, blockIdx.z, &map);
}

template <typename T, int DIR, int L, int WA, int WB, int SOLVER, bool FIRST, bool FINAL>
cudaError_t launch_sweep_tma(const Box &b, int recon, const T *Wh, T *dU, double *U, const Scratch &sc, double dt,
                             const double *dtp, cudaStream_t s, bool &launched)
{
  launched = false;
  if (!sweep_tma() || (DIR != 0 && WB != 1)) return cudaSuccess;
  int const rx = b.nx - 2 * b.ng, ry = b.ny - 2 * b.ng, rz = b.nz - 2 * b.ng;
  int const ra = DIR == 0 ? rx : DIR == 1 ? ry : rz, rb = DIR == 0 ? ry : rx, rc = DIR == 2 ? ry : rz;
  dim3 grid((ra + L - 1) / L, (rb + WA - 1) / WA, (rc + WB - 1) / WB);
  void (*k)(Box, const T *, T *, double *, const double *, double *, int *, double, const double *, CUtensorMap);
  size_t per_q;
  int bx, by, bz;
#define CGB_PICK(R)                                                                                        \
  {                                                                                                        \
    using TM = typename Sweep<DIR, L, WA, WB, R>::template Tma<T>;                                         \
    per_q    = TM::PER_Q;                                                                                  \
    bx       = DIR == 0 ? TM::LAP : TM::WAP;                                                               \
    by       = DIR == 0 ? WA : DIR == 1 ? Sweep<DIR, L, WA, WB, R>::LA : 1;                                \
    bz       = DIR == 0 ? WB : DIR == 1 ? 1 : Sweep<DIR, L, WA, WB, R>::LA;                                \
    k        = k_fsweep_tma<T, DIR, L, WA, WB, R, SOLVER, FIRST, FINAL>;                                   \
  }
  if (recon == RECON_PPMC) {
    CGB_PICK(RECON_PPMC)
  } else if (recon == RECON_PLMC) {
    CGB_PICK(RECON_PLMC)
  } else if (recon == RECON_PPMP) {
    CGB_PICK(RECON_PPMP)
  } else if (recon == RECON_PLMP) {
    CGB_PICK(RECON_PLMP)
  } else {
    CGB_PICK(RECON_PCM)
  }
#undef CGB_PICK
  CUtensorMap map;
  if (!tma_encode_4d(&map, Wh, (int)sizeof(T), b.nx, b.ny, b.nz, nslot(b), bx, by, bz)) return cudaSuccess;
  size_t const sm = sizeof(T) * (size_t)nslot(b) * per_q + 128;  // + room to start P on 128 bytes
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, sweep_threads(L, WA * WB, recon), sm, s>>>(b, Wh, dU, U, sc.GEp, sc.Epre, sc.status, dt, dtp, map);
  launched = true;
  return cudaGetLastError();
}

template <typename T, int DIR, int L, int WA, int WB, int SOLVER, bool FIRST, bool FINAL>
cudaError_t launch_sweep(const Box &b, int recon, const T *Wh, T *dU, double *U, const Scratch &sc, double dt,
                         const double *dtp, cudaStream_t s)
{
  if (!(b.ny == 1 && b.nz == 1)) {
    bool launched = false;
    cudaError_t const e =
        launch_sweep_tma<T, DIR, L, WA, WB, SOLVER, FIRST, FINAL>(b, recon, Wh, dU, U, sc, dt, dtp, s, launched);
    if (e != cudaSuccess || launched) return e;
  }
  // real cells along the sweep (ra) and across it (rb: the WA axis, rc: the WB axis)
  bool const one_d = (b.ny == 1 && b.nz == 1);
  int const rx = b.nx - 2 * b.ng, ry = one_d ? 1 : b.ny - 2 * b.ng, rz = one_d ? 1 : b.nz - 2 * b.ng;
  int const ra = DIR == 0 ? rx : DIR == 1 ? ry : rz;
  int const rb = DIR == 0 ? ry : rx;
  int const rc = DIR == 2 ? ry : rz;
  dim3 grid((ra + L - 1) / L, (rb + WA - 1) / WA, (rc + WB - 1) / WB);
  void (*k)(Box, const T *, T *, double *, const double *, double *, int *, double, const double *);
  size_t per_q;
#define CGB_PICK(R)                                                                                        \
  per_q = Sweep<DIR, L, WA, WB, R>::PER_Q;                                                                \
  k     = k_fsweep<T, DIR, L, WA, WB, R, SOLVER, FIRST, FINAL>;
  if (recon == RECON_PPMC) {
    CGB_PICK(RECON_PPMC)
  } else if (recon == RECON_PLMC) {
    CGB_PICK(RECON_PLMC)
  } else if (recon == RECON_PPMP) {
    CGB_PICK(RECON_PPMP)
  } else if (recon == RECON_PLMP) {
    CGB_PICK(RECON_PLMP)
  } else {
    CGB_PICK(RECON_PCM)
  }
#undef CGB_PICK
  size_t const sm = sizeof(T) * (size_t)nslot(b) * per_q;
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, sweep_threads(L, WA * WB, recon), sm, s>>>(b, Wh, dU, U, sc.GEp, sc.Epre, sc.status, dt, dtp);
  return cudaGetLastError();
}

// ------------------------------------------------------------------------------------------
template <typename T, int TX, int TY, int TZ>
size_t fpred_smem(const Box &b)
{
  constexpr int HY = TY > 1, HZ = TZ > 1;
  constexpr int NB = (TX + 2) * (TY + 2 * HY) * (TZ + 2 * HZ);
  constexpr int NF = (TX + 1) * TY * TZ + (HY ? TX * (TY + 1) * TZ : 0) + (HZ ? TX * TY * (TZ + 1) : 0);
  return sizeof(T) * ((size_t)nslot(b) * (NB + NF) + (pred_sideq<T>() ? (size_t)PRED_SIDEQ * NB : 0));
}

// predictor and the x, y, z sweeps of one box whose primitives Wⁿ are current
template <typename T, int TX, int TY, int TZ, int SOLVER>
cudaError_t pred_sweeps(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                        cudaStream_t s, cudaEvent_t *marks)
{
  T *Wn = (T *)sc.W;
  T *Wh = half_prims(Wn, b);
  cudaError_t e;
  {
    size_t const sm = fpred_smem<T, TX, TY, TZ>(b);
    dim3 grid((b.nx - 2 + TX - 1) / TX, TY > 1 ? (b.ny - 2 + TY - 1) / TY : 1, TZ > 1 ? (b.nz - 2 + TZ - 1) / TZ : 1);
    auto k = k_fpred<T, TX, TY, TZ, SOLVER>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess) return e;
    k<<<grid, TX * TY * TZ, sm, s>>>(b, U, Wn, Wh, sc.GEp, dt, dtp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  if (marks) cudaEventRecord(marks[1], s);
  // corrector: x, y, z sweeps; W^n is dead after the predictor and holds the accumulator
  if (b.ny == 1 && b.nz == 1) {
    e = launch_sweep<T, 0, 128, 1, 1, SOLVER, true, true>(b, recon, Wh, Wn, U, sc, dt, dtp, s);
  } else {
    e = launch_sweep<T, 0, SXL, SXA, SXB, SOLVER, true, false>(b, recon, Wh, Wn, U, sc, dt, dtp, s);
    if (e == cudaSuccess) e = launch_sweep<T, 1, SYL, SYA, SYB, SOLVER, false, false>(b, recon, Wh, Wn, U, sc, dt, dtp, s);
    if (e == cudaSuccess) e = launch_sweep<T, 2, SYL, SYA, SYB, SOLVER, false, true>(b, recon, Wh, Wn, U, sc, dt, dtp, s);
  }
  if (e != cudaSuccess) return e;
  if (marks) cudaEventRecord(marks[2], s);
  return cudaSuccess;
}

// the same for a box of either form: 3D tiles, or the 1D step's pencils of 128 cells (the
// reference's 1D integrator has no HLL branch, so no 1D HLL kernels are built)
template <int SOLVER>
cudaError_t fast_solver(const Box &b, int recon, int mixed, double *U, const Scratch &sc, double dt,
                        const double *dtp, cudaStream_t s, cudaEvent_t *marks)
{
  if (b.ny == 1 && b.nz == 1) {
    if constexpr (SOLVER == SOLVER_HLL) {
      return cudaErrorNotSupported;
    } else {
      return mixed ? pred_sweeps<float, 128, 1, 1, SOLVER>(b, recon, U, sc, dt, dtp, s, marks)
                   : pred_sweeps<double, 128, 1, 1, SOLVER>(b, recon, U, sc, dt, dtp, s, marks);
    }
  }
  return mixed ? pred_sweeps<float, PTX, PTY, PTZ, SOLVER>(b, recon, U, sc, dt, dtp, s, marks)
               : pred_sweeps<double, PTX, PTY, PTZ, SOLVER>(b, recon, U, sc, dt, dtp, s, marks);
}

}  // namespace

// ==========================================================================================
// batches: one chunk of jobs per launch, one block per tile.  The chunk (job geometry, pointers
// and per-kind tile offsets) is the kernel's __grid_constant__ parameter: a block finds its
// job by binary search over the chunk's offsets and runs the single-box tile code on it, with
// the job's fields read from the constant bank.
// ==========================================================================================
namespace
{

__host__ __device__ inline void pred_grid(const Box &b, int &gx, int &gy, int &gz)
{
  gx = (b.nx - 2 + PTX - 1) / PTX, gy = (b.ny - 2 + PTY - 1) / PTY, gz = (b.nz - 2 + PTZ - 1) / PTZ;
}
template <int DIR, int L, int WA, int WB>
__host__ __device__ inline void sweep_grid(const Box &b, int &ga, int &gb, int &gc)
{
  int const rx = b.nx - 2 * b.ng, ry = b.ny - 2 * b.ng, rz = b.nz - 2 * b.ng;
  int const ra = DIR == 0 ? rx : DIR == 1 ? ry : rz;
  int const rb = DIR == 0 ? ry : rx;
  int const rc = DIR == 2 ? ry : rz;
  ga = (ra + L - 1) / L, gb = (rb + WA - 1) / WA, gc = (rc + WB - 1) / WB;
}
__host__ __device__ inline long long real_cells(const Box &b)
{
  return (long long)(b.nx - 2 * b.ng) * (b.ny - 2 * b.ng) * (b.nz - 2 * b.ng);
}

// job j of the chunk with off[kind][j] <= tile < off[kind][j + 1]
__device__ __forceinline__ int find_job(const BatchChunk &C, int kind, int tile)
{
  int lo = 0, hi = C.njobs - 1;
  while (lo < hi) {
    int const mid = (lo + hi + 1) >> 1;
    if (C.off[kind][mid] <= tile)
      lo = mid;
    else
      hi = mid - 1;
  }
  return lo;
}


template <typename T>
__global__ void __launch_bounds__(256) kb_prims(const __grid_constant__ BatchChunk C)
{
  int const tile     = blockIdx.x;
  int const j        = find_job(C, BK_CELLS, tile);
  BatchJob const &J  = C.jobs[j];
  long long const id = (long long)(tile - C.off[BK_CELLS][j]) * 256 + threadIdx.x;
  if (J.status[1]) {  // the real cells' primitives are current: the ghost shell only
    if (id < J.b.n - real_count(J.b)) fprims_cell<T>(J.b, J.U, (T *)J.W, ghost_cell(J.b, id));
  } else if (id < J.b.n) {
    fprims_cell<T>(J.b, J.U, (T *)J.W, id);
  }
}

// FP32 tiles: four resident blocks per SM (64 registers), the single-box predictor's occupancy
template <typename T, int SOLVER>
__global__ void __launch_bounds__(PTX *PTY *PTZ, sizeof(T) == 4 ? 4 : 2)
    kb_pred(const __grid_constant__ BatchChunk C)
{
  int const tile    = blockIdx.x;
  int const j       = find_job(C, BK_PRED, tile);
  BatchJob const &J = C.jobs[j];
  int gx, gy, gz;
  pred_grid(J.b, gx, gy, gz);
  int tx, ty;
  int const tz = divmod(divmod(tile - C.off[BK_PRED][j], gx, tx), gy, ty);
  T *Wn        = (T *)J.W;
  T *Wh        = half_prims(Wn, J.b);
  (void)gz;
  fpred_tile<T, PTX, PTY, PTZ, SOLVER>(J.b, J.U, Wn, Wh, J.GEp, 0.0, J.dt_t, tx, ty, tz);
}

template <typename T, int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL>
__global__ void __launch_bounds__(sweep_threads(L, WA *WB, RECON), sweep_min_blocks<T, SOLVER>())
    kb_sweep(const __grid_constant__ BatchChunk C)
{
  int const kind    = BK_SWX + DIR;
  int const tile    = blockIdx.x;
  int const j       = find_job(C, kind, tile);
  BatchJob const &J = C.jobs[j];
  int ga, gb, gc;
  sweep_grid<DIR, L, WA, WB>(J.b, ga, gb, gc);
  int ta, tb;
  int const tc = divmod(divmod(tile - C.off[kind][j], ga, ta), gb, tb);
  T *Wn        = (T *)J.W;  // holds the accumulator dU once the predictor has run
  T *Wh        = half_prims(Wn, J.b);
  (void)gc;
  fsweep_tile<T, DIR, L, WA, WB, RECON, SOLVER, FIRST, FINAL>(J.b, Wh, Wn, J.U, J.GEp, J.Epre, J.status, 0.0, J.dt_t,
                                                              ta, tb, tc);
}


template <typename T, int DIR, int L, int WA, int WB, int SOLVER, bool FIRST, bool FINAL>
cudaError_t launch_batch_sweep(const BatchChunk &C, int recon, int nsl, cudaStream_t s)
{
  void (*k)(BatchChunk);
  size_t per_q;
#define CGB_PICK(R)                                                                                        \
  per_q = Sweep<DIR, L, WA, WB, R>::PER_Q;                                                                \
  k     = kb_sweep<T, DIR, L, WA, WB, R, SOLVER, FIRST, FINAL>;
  if (recon == RECON_PPMC) {
    CGB_PICK(RECON_PPMC)
  } else if (recon == RECON_PLMC) {
    CGB_PICK(RECON_PLMC)
  } else if (recon == RECON_PPMP) {
    CGB_PICK(RECON_PPMP)
  } else if (recon == RECON_PLMP) {
    CGB_PICK(RECON_PLMP)
  } else {
    CGB_PICK(RECON_PCM)
  }
#undef CGB_PICK
  size_t const sm = sizeof(T) * (size_t)nsl * per_q;
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<C.total[BK_SWX + DIR], sweep_threads(L, WA * WB, recon), sm, s>>>(C);
  return cudaGetLastError();
}

// predictor and x/y/z sweeps of one chunk whose primitives are current
template <typename T, int SET, int SOLVER>
cudaError_t batch_pred_sweeps(const BatchChunk &C, int recon, int nsl, cudaStream_t s)
{
  cudaError_t e;
  {
    constexpr int NB = (PTX + 2) * (PTY + 2) * (PTZ + 2);
    constexpr int NF = (PTX + 1) * PTY * PTZ + PTX * (PTY + 1) * PTZ + PTX * PTY * (PTZ + 1);
    size_t const sm  = sizeof(T) * ((size_t)nsl * (NB + NF) + (pred_sideq<T>() ? (size_t)PRED_SIDEQ * NB : 0));
    auto k           = kb_pred<T, SOLVER>;
    if ((e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm)) != cudaSuccess) return e;
    k<<<C.total[BK_PRED], PTX * PTY * PTZ, sm, s>>>(C);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  using TS = TileSet<SET>;
  if ((e = launch_batch_sweep<T, 0, TS::XL, TS::XA, TS::XB, SOLVER, true, false>(C, recon, nsl, s)) != cudaSuccess)
    return e;
  if ((e = launch_batch_sweep<T, 1, TS::YL, TS::YA, TS::YB, SOLVER, false, false>(C, recon, nsl, s)) != cudaSuccess)
    return e;
  return launch_batch_sweep<T, 2, TS::YL, TS::YA, TS::YB, SOLVER, false, true>(C, recon, nsl, s);
}

template <int SOLVER>
cudaError_t batch_solver(const BatchChunk &C, int recon, int mixed, int set, int nsl, cudaStream_t s)
{
  if (set == 1)
    return mixed ? batch_pred_sweeps<float, 1, SOLVER>(C, recon, nsl, s)
                 : batch_pred_sweeps<double, 1, SOLVER>(C, recon, nsl, s);
  return mixed ? batch_pred_sweeps<float, 0, SOLVER>(C, recon, nsl, s)
               : batch_pred_sweeps<double, 0, SOLVER>(C, recon, nsl, s);
}

}  // namespace

}  // namespace cgb
