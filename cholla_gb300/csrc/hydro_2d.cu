// hydro_2d.cu -- the VL step on a 2D box (nz = 1), exact FP64 in the reference's operation order
// (built with -fmad=false): VL_Algorithm_2D_CUDA (src/integrators/VL_2D_cuda.cu:25-174) with the
// 2D kernels it calls (VL_2D_cuda.cu:176-258, hydro_cuda.cu:87-170, 725-752).
//
//   predictor  Uⁿ -> U½       per 16 x 16 tile: PCM interface states and fluxes of the x and y
//                             faces in shared memory, the half update (no density floor in 2D),
//                             and the full-dt pdV partial update of GasEnergy from Uⁿ (GEp)
//   corrector  U½ -> Uⁿ⁺¹     per tile: reconstruction (PLMC / PPMC / PLMP / PPMP) of U½ along x
//                             and y, the Riemann fluxes, U += dt/dx ΔFx + dt/dy ΔFy in place and the
//                             pre-sync energy.  With PCM the reference's 2D integrator reuses the
//                             predictor's interface states of Uⁿ, so the corrector takes the
//                             predictor's fluxes, which the predictor stores for it.
//   finalize   (hydro_exact.cu) dual-energy select over the four face neighbours and sync, CFL
//
// The interface states and fluxes of the reconstructing schemes live in shared memory only.
#include "common.cuh"
#include "hydro_math.cuh"
#include "kernels.h"

namespace cgb
{
namespace
{
constexpr int T2 = 16;  // tile edge

__device__ __forceinline__ int field_of_q2(int q, const Box &b) { return (q < 5 + b.ns) ? q : b.nf - 1; }
__device__ __forceinline__ int clamp2(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// predictor: (T2 + 2)^2 cells of Uⁿ in shared memory, the x and y faces of the tile's cells, the
// half update, GEp; with store_flux, the face fluxes go to Fst for the PCM corrector:
// Fst[f * n + id] = flux at the high x face of cell id, Fst[(nf + f) * n + id] at its high y face
template <int SOLVER>
__global__ void __launch_bounds__(T2 *T2) k2_pred(Box b, const double *__restrict__ U, double *__restrict__ Uh,
                                                  double *__restrict__ GEp, double *__restrict__ Fst, double dt,
                                                  const double *__restrict__ dtp)
{
  if (dtp) dt = *dtp;
  constexpr int B = T2 + 2, NB = B * B, NFX = (T2 + 1) * T2, NFY = T2 * (T2 + 1), NT = T2 * T2;
  extern __shared__ double smem2[];
  int const nq = b.nq();
  double *Us  = smem2;           // [nq][NB] canonical order
  double *Fxs = Us + nq * NB;    // [nq][NFX] canonical order
  double *Fys = Fxs + nq * NFX;  // [nq][NFY]
  int const x0 = 1 + blockIdx.x * T2, y0 = 1 + blockIdx.y * T2;
  long long const n = b.n;
  for (int t = threadIdx.x; t < NB; t += NT) {
    int const gx = clamp2(x0 - 1 + t % B, 0, b.nx - 1), gy = clamp2(y0 - 1 + t / B, 0, b.ny - 1);
    long long const gid = b.id(gx, gy, 0);
    for (int q = 0; q < nq; q++) Us[q * NB + t] = U[(long long)field_of_q2(q, b) * n + gid];
  }
  __syncthreads();
  for (int t = threadIdx.x; t < NFX + NFY; t += NT) {
    int const dir = t < NFX ? 0 : 1;
    int const u   = dir == 0 ? t : t - NFX;
    int i, j, cl, cr;
    if (dir == 0) {  // face between box cells (i, j+1) and (i+1, j+1)
      i = u % (T2 + 1), j = u / (T2 + 1);
      cl = i + B * (j + 1), cr = cl + 1;
    } else {         // face between (i+1, j) and (i+1, j+1)
      i = u % T2, j = u / T2;
      cl = (i + 1) + B * j, cr = cl + B;
    }
    int const o1 = dir + 1, o2 = (dir + 1) % 3 + 1, o3 = (dir + 2) % 3 + 1;
    double qL[NQ_MAX], qR[NQ_MAX], f[NQ_MAX];
#pragma unroll
    for (int q = 0; q < NQ_MAX; q++) {
      if (q < nq) {
        int const s = (q == 1) ? o1 : (q == 2) ? o2 : (q == 3) ? o3 : q;
        qL[q] = Us[s * NB + cl];
        qR[q] = Us[s * NB + cr];
      }
    }
    hx::riemann<SOLVER>(qL, qR, f, b.ns, b.de, b.gamma);
    double *Fd    = dir == 0 ? Fxs : Fys;
    int const nfd = dir == 0 ? NFX : NFY;
#pragma unroll
    for (int q = 0; q < NQ_MAX; q++) {
      if (q < nq) {
        int const s = (q == 1) ? o1 : (q == 2) ? o2 : (q == 3) ? o3 : q;
        Fd[s * nfd + u] = f[q];
        if (Fst) {  // the face's low-side cell owns it; the tile's last face only at the box's end
          int const gx = dir == 0 ? x0 - 1 + i : x0 + i, gy = dir == 0 ? y0 + j : y0 - 1 + j;
          bool const own = dir == 0 ? (i < T2 || blockIdx.x == gridDim.x - 1) : (j < T2 || blockIdx.y == gridDim.y - 1);
          if (own && gx < b.nx && gy < b.ny)
            Fst[((long long)(dir * b.nf) + field_of_q2(s, b)) * n + b.id(gx, gy, 0)] = f[q];
        }
      }
    }
  }
  __syncthreads();
  int const t = threadIdx.x, i = t % T2, j = t / T2;
  int const gx = x0 + i, gy = y0 + j;
  if (!(gx > 0 && gx < b.nx - 1 && gy > 0 && gy < b.ny - 1)) return;
  long long const gid = b.id(gx, gy, 0);
  int const c = (i + 1) + B * (j + 1), fx = i + (T2 + 1) * j, fy = i + T2 * j;
  double const hdt = 0.5 * dt, dtodx = hdt / b.dx, dtody = hdt / b.dy;
  // Update_Conserved_Variables_2D_half (VL_2D_cuda.cu:176-258)
  double out[NQ_MAX];
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++)
    if (q < nq)
      out[q] = Us[q * NB + c] + dtodx * (Fxs[q * NFX + fx] - Fxs[q * NFX + fx + 1]) +
               dtody * (Fys[q * NFY + fy] - Fys[q * NFY + fy + T2]);
  int const qge = 5 + b.ns;
  if (b.de) {
    double const d = Us[c], d_inv = 1.0 / d;
    double const vx = Us[NB + c] * d_inv, vy = Us[2 * NB + c] * d_inv, vz = Us[3 * NB + c] * d_inv;
    double const E      = Us[4 * NB + c];
    double const vx_imo = Us[NB + c - 1] / Us[c - 1], vx_ipo = Us[NB + c + 1] / Us[c + 1];
    double const vy_jmo = Us[2 * NB + c - B] / Us[c - B], vy_jpo = Us[2 * NB + c + B] / Us[c + B];
    // the half step's pdV term uses the plain total-minus-kinetic pressure
    double const P = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (b.gamma - 1.0);
    out[qge]       = out[qge] + 0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo));
    // Partial_Update_Advected_Internal_Energy_2D (hydro_cuda.cu:725-752), full dt, real cells
    int const ng = b.ng;
    if (gx > ng - 1 && gx < b.nx - ng && gy > ng - 1 && gy < b.ny - ng) {
      double const GE   = Us[qge * NB + c];
      double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double const Pp   = fmax(hx::pressure_de(E, E - Ekin, GE, b.gamma), TINY);
      double const fdx = dt / b.dx, fdy = dt / b.dy;
      GEp[gid]          = GE + 0.5 * Pp * (fdx * (vx_imo - vx_ipo) + fdy * (vy_jmo - vy_jpo));
    }
  }
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++)
    if (q < nq) Uh[(long long)field_of_q2(q, b) * n + gid] = out[q];
}

// corrector tile sizes: U½ with a halo of H cells on all sides (a 2D tile's corners are few)
template <int RECON>
struct C2 {
  static constexpr int H  = (RECON == RECON_PPMC || RECON == RECON_PPMP) ? 3 : 2;
  static constexpr int B  = T2 + 2 * H, NB = B * B;
  static constexpr int NR = (T2 + 2) * T2;  // reconstructed cells per direction
  static constexpr int NF = (T2 + 1) * T2;  // faces per direction
};

template <int RECON, int SOLVER>
__global__ void __launch_bounds__(T2 *T2) k2_corr(Box b, const double *__restrict__ Uh, double *__restrict__ U,
                                                  const double *__restrict__ GEp, const double *__restrict__ Fst,
                                                  double *__restrict__ Epre, int *__restrict__ status, double dt,
                                                  const double *__restrict__ dtp)
{
  if (dtp) dt = *dtp;
  constexpr int NT = T2 * T2;
  int const ng = b.ng, nq = b.nq();
  int const x0 = ng + blockIdx.x * T2, y0 = ng + blockIdx.y * T2;
  long long const n = b.n;
  int const t = threadIdx.x, ti = t % T2, tj = t / T2;
  int const gx = x0 + ti, gy = y0 + tj;
  bool const real = gx < b.nx - ng && gy < b.ny - ng;
  double dX[NQ_MAX], dY[NQ_MAX];  // dt/dx (F(i-1/2) - F(i+1/2)) per canonical field
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++) dX[q] = dY[q] = 0.0;
  double const dtodx = dt / b.dx, dtody = dt / b.dy;
  if (RECON == RECON_PCM) {
    // the predictor's fluxes of Uⁿ (VL_2D_cuda.cu:97-122 reconstructs nothing for PCM)
    if (real) {
      long long const gid = b.id(gx, gy, 0), imo = b.id(gx - 1, gy, 0), jmo = b.id(gx, gy - 1, 0);
#pragma unroll
      for (int q = 0; q < NQ_MAX; q++) {
        if (q < nq) {
          long long const f = field_of_q2(q, b);
          dX[q] = dtodx * (Fst[f * n + imo] - Fst[f * n + gid]);
          dY[q] = dtody * (Fst[(b.nf + f) * n + jmo] - Fst[(b.nf + f) * n + gid]);
        }
      }
    }
  } else {
    using S = C2<RECON>;
    constexpr int H = S::H, B = S::B;
    extern __shared__ double smem2[];
    double *Ps  = smem2;            // [nq][NB] primitives, rotated for the current sweep
    double *QLs = Ps + nq * S::NB;  // [nq][NR] rotated conserved states of one direction
    double *QRs = QLs + nq * S::NR;
    double *Fs  = QRs + nq * S::NR;  // [nq][NF]
#pragma unroll
    for (int dir = 0; dir < 2; dir++) {
      int const st = dir == 0 ? 1 : B;
      int const o1 = dir + 1, o2 = (dir + 1) % 3 + 1, o3 = (dir + 2) % 3 + 1;
      // U½ -> primitives in this sweep's rotated order (the reference's reconstruction kernels
      // load them per direction, and the kinetic energy's rounding depends on the order)
      for (int p = t; p < S::NB; p += NT) {
        int const cx = clamp2(x0 - H + p % B, 1, b.nx - 2), cy = clamp2(y0 - H + p / B, 1, b.ny - 2);
        long long const gid = b.id(cx, cy, 0);
        double q[NQ_MAX];
#pragma unroll
        for (int k = 0; k < NQ_MAX; k++) {
          if (k < nq) {
            int const src = k == 1 ? o1 : k == 2 ? o2 : k == 3 ? o3 : field_of_q2(k, b);
            q[k]          = Uh[(long long)src * n + gid];
          }
        }
        hx::Prim const P = (RECON == RECON_PLMP || RECON == RECON_PPMP) ? hx::load_prim_plm(q, b.ns, b.de, b.gamma)
                                                                        : hx::load_prim(q, b.ns, b.de, b.gamma);
        Ps[0 * S::NB + p] = P.d;
        Ps[1 * S::NB + p] = P.vn;
        Ps[2 * S::NB + p] = P.vt1;
        Ps[3 * S::NB + p] = P.vt2;
        Ps[4 * S::NB + p] = P.p;
#pragma unroll
        for (int k = 0; k < NS_MAX; k++)
          if (k < b.ns) Ps[(5 + k) * S::NB + p] = P.sc[k];
        if (b.de) Ps[(5 + b.ns) * S::NB + p] = P.ge;
      }
      __syncthreads();
      // reconstructed cell r: position a = -1 .. T2 along the sweep, line l across it
      for (int r = t; r < S::NR; r += NT) {
        int const a = r % (T2 + 2) - 1, l = r / (T2 + 2);
        int const base = dir == 0 ? (a + H) + B * (l + H) : (l + H) + B * (a + H);
        auto prim_at = [&](int off) {
          int const pi = base + off * st;
          hx::Prim P;
          P.d   = Ps[pi];
          P.vn  = Ps[S::NB + pi];
          P.vt1 = Ps[2 * S::NB + pi];
          P.vt2 = Ps[3 * S::NB + pi];
          P.p   = Ps[4 * S::NB + pi];
#pragma unroll
          for (int k = 0; k < NS_MAX; k++) P.sc[k] = (k < b.ns) ? Ps[(5 + k) * S::NB + pi] : 0.0;
          P.ge = b.de ? Ps[(5 + b.ns) * S::NB + pi] : 0.0;
          return P;
        };
        double qLv[NQ_MAX], qRv[NQ_MAX];
        if (RECON == RECON_PPMC || RECON == RECON_PLMC) {
          hx::Prim Lp, Rp;
          if (RECON == RECON_PPMC)
            hx::ppmc_cell(prim_at(-2), prim_at(-1), prim_at(0), prim_at(1), prim_at(2), b.ns, b.de, b.gamma, Lp, Rp);
          else
            hx::plmc_cell(prim_at(-1), prim_at(0), prim_at(1), b.ns, b.de, b.gamma, Lp, Rp);
          hx::prim_to_q(Lp, qLv, b.ns, b.de, b.gamma);
          hx::prim_to_q(Rp, qRv, b.ns, b.de, b.gamma);
        } else if (RECON == RECON_PLMP) {
          hx::Prim const c[3] = {prim_at(-1), prim_at(0), prim_at(1)};
          hx::plmp_ppmp_cell<1>(c, b.ns, b.de, b.gamma, qLv, qRv);
        } else {
          hx::Prim const c[5] = {prim_at(-2), prim_at(-1), prim_at(0), prim_at(1), prim_at(2)};
          hx::plmp_ppmp_cell<2>(c, b.ns, b.de, b.gamma, qLv, qRv);
        }
#pragma unroll
        for (int k = 0; k < NQ_MAX; k++) {
          if (k < nq) {
            QLs[k * S::NR + r] = qLv[k];
            QRs[k * S::NR + r] = qRv[k];
          }
        }
      }
      __syncthreads();
      // face f: position a = 0 .. T2 (between reconstructed cells a - 1 and a), line l
      for (int f = t; f < S::NF; f += NT) {
        int const a = f % (T2 + 1), l = f / (T2 + 1);
        int const rl = a + (T2 + 2) * l, rr = rl + 1;
        double qL[NQ_MAX], qR[NQ_MAX], fl[NQ_MAX];
#pragma unroll
        for (int k = 0; k < NQ_MAX; k++) {
          if (k < nq) {
            qL[k] = QLs[k * S::NR + rl];
            qR[k] = QRs[k * S::NR + rr];
          }
        }
        hx::riemann<SOLVER>(qL, qR, fl, b.ns, b.de, b.gamma);
#pragma unroll
        for (int k = 0; k < NQ_MAX; k++)
          if (k < nq) Fs[k * S::NF + f] = fl[k];
      }
      __syncthreads();
      {
        int const a = dir == 0 ? ti : tj, l = dir == 0 ? tj : ti;
        int const fm = a + (T2 + 1) * l;
        double const k = dir == 0 ? dtodx : dtody;
#pragma unroll
        for (int q = 0; q < NQ_MAX; q++) {
          if (q < nq) {
            int const cf   = q == 1 ? o1 : q == 2 ? o2 : q == 3 ? o3 : q;  // rotated slot -> canonical slot
            double const v = k * (Fs[q * S::NF + fm] - Fs[q * S::NF + fm + 1]);
#pragma unroll
            for (int c = 0; c < NQ_MAX; c++) {
              if (c == cf) {
                if (dir == 0)
                  dX[c] = v;
                else
                  dY[c] = v;
              }
            }
          }
        }
      }
      __syncthreads();  // QLs / Fs are reused by the next direction
    }
  }
  if (!real) return;
  long long const gid = b.id(gx, gy, 0);
  // Update_Conserved_Variables_2D (hydro_cuda.cu:87-170): U += dX + dY, after the pdV partial update
  double v[NQ_MAX];
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++) {
    if (q < nq) {
      double const u0 = (b.de && q == nq - 1) ? GEp[gid] : U[(long long)field_of_q2(q, b) * n + gid];
      v[q]            = u0 + (dX[q] + dY[q]);
    }
  }
  if (not_finite(v[0]) || not_finite(v[4])) atomicOr(status, STATUS_NONFINITE);
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++)
    if (q < nq) U[(long long)field_of_q2(q, b) * n + gid] = v[q];
  if (b.de) Epre[gid] = v[4];
}

template <int SOLVER>
cudaError_t step2d(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp, cudaStream_t s)
{
  double *Fst = recon == RECON_PCM ? static_cast<double *>(sc.W) : nullptr;
  int const nq = b.nq();
  {
    size_t const sm = sizeof(double) * nq * ((T2 + 2) * (T2 + 2) + 2 * (T2 + 1) * T2);
    auto k          = k2_pred<SOLVER>;
    cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
    if (e != cudaSuccess) return e;
    dim3 grid((b.nx - 2 + T2 - 1) / T2, (b.ny - 2 + T2 - 1) / T2);
    k<<<grid, T2 * T2, sm, s>>>(b, U, sc.Uh, sc.GEp, Fst, dt, dtp);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
  }
  dim3 grid((b.nx - 2 * b.ng + T2 - 1) / T2, (b.ny - 2 * b.ng + T2 - 1) / T2);
  void (*k)(Box, const double *, double *, const double *, const double *, double *, int *, double, const double *);
  size_t sm = 0;
#define CGB_2D(R)                                                                                          \
  k  = k2_corr<R, SOLVER>;                                                                                 \
  sm = R == RECON_PCM ? 0 : sizeof(double) * nq * (C2<R>::NB + 2 * C2<R>::NR + C2<R>::NF);
  switch (recon) {
    case RECON_PPMC: CGB_2D(RECON_PPMC) break;
    case RECON_PLMC: CGB_2D(RECON_PLMC) break;
    case RECON_PLMP: CGB_2D(RECON_PLMP) break;
    case RECON_PPMP: CGB_2D(RECON_PPMP) break;
    default: CGB_2D(RECON_PCM) break;
  }
#undef CGB_2D
  cudaError_t e = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  k<<<grid, T2 * T2, sm, s>>>(b, sc.Uh, U, sc.GEp, Fst, sc.Epre, sc.status, dt, dtp);
  return cudaGetLastError();
}
}  // namespace

cudaError_t hydro_2d_step(const Box &b, int recon, int solver, double *U, const Scratch &sc, double dt,
                          const double *dt_dev, cudaStream_t s)
{
  switch (solver) {
    case SOLVER_ROE: return step2d<SOLVER_ROE>(b, recon, U, sc, dt, dt_dev, s);
    case SOLVER_EXACT: return step2d<SOLVER_EXACT>(b, recon, U, sc, dt, dt_dev, s);
    case SOLVER_HLLC: return step2d<SOLVER_HLLC>(b, recon, U, sc, dt, dt_dev, s);
    default: return cudaErrorInvalidValue;  // the reference's 2D integrator has no HLL branch
  }
}

}  // namespace cgb
