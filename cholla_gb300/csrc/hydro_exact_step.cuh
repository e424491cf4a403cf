// hydro_exact_step.cuh -- the predictor and corrector kernels of the exact FP64 hydro step,
// templated on reconstruction and Riemann solver.  Each hydro_exact_<solver>.cu translation unit
// (built with -fmad=false, so every operation keeps the reference's rounding) includes this file
// and instantiates the step for its solver only, which keeps the build parallel.
//
//   predictor  Uⁿ  -> U½     PCM + Riemann + half update, per 3D tile; the 3 face fluxes
//                            of every cell live in shared memory (VL_3D_cuda.cu:138-212)
//                            + the full-dt pdV partial update of GasEnergy (hydro_cuda.cu:754-833)
//   corrector  U½ -> Uⁿ⁺¹    x, y, z sweeps of reconstruction + Riemann into an accumulator,
//                            then the conserved update in place (VL_3D_cuda.cu:224-339,
//                            hydro_cuda.cu:172-402); or, without room for the accumulator, the
//                            same per fused tile
#pragma once
#include "common.cuh"
#include "hydro_math.cuh"
#include "kernels.h"
namespace cgb
{

namespace
{

__device__ __forceinline__ int field_of_q(int q, const Box &b)
{
  return (q < 5 + b.ns) ? q : b.nf - 1;  // the last carried quantity is GasEnergy
}

// rotation of the three momenta for a sweep direction: (o1, o2, o3) of hllc_cuda.cu:54-70
__device__ __forceinline__ void rot(int dir, int &o1, int &o2, int &o3)
{
  o1 = dir + 1;
  o2 = (dir + 1) % 3 + 1;
  o3 = (dir + 2) % 3 + 1;
}

__device__ __forceinline__ int clampi(int v, int lo, int hi) { return v < lo ? lo : (v > hi ? hi : v); }

// ------------------------------------------------------------------------------------------
// predictor
// ------------------------------------------------------------------------------------------
template <int TX, int TY, int TZ, int SOLVER>
__global__ void __launch_bounds__(TX *TY *TZ) k_predictor(Box b, const double *__restrict__ U, double *__restrict__ Uh,
                                                          double *__restrict__ GEp, double dt,
                                                          const double *__restrict__ dtp)
{
  if (dtp) dt = *dtp;  // time step kept on the device (engine path)
  constexpr int HY = TY > 1 ? 1 : 0, HZ = TZ > 1 ? 1 : 0;
  constexpr int BX = TX + 2, BY = TY + 2 * HY, BZ = TZ + 2 * HZ;
  constexpr int NB  = BX * BY * BZ;
  constexpr int NFX = (TX + 1) * TY * TZ;
  constexpr int NFY = HY ? TX * (TY + 1) * TZ : 0;
  constexpr int NFZ = HZ ? TX * TY * (TZ + 1) : 0;
  constexpr int NT  = TX * TY * TZ;
  extern __shared__ double smem[];
  int const nq = b.nq();
  double *Us   = smem;            // [nq][NB] canonical fields
  double *Fxs  = Us + nq * NB;    // [nq][NFX]
  double *Fys  = Fxs + nq * NFX;  // [nq][NFY]
  double *Fzs  = Fys + nq * NFY;  // [nq][NFZ]

  int const x0 = 1 + blockIdx.x * TX;
  int const y0 = HY ? 1 + blockIdx.y * TY : 0;
  int const z0 = HZ ? 1 + blockIdx.z * TZ : 0;

  for (int t = threadIdx.x; t < NB; t += NT) {
    int const bx = t % BX, by = (t / BX) % BY, bz = t / (BX * BY);
    int const gx = clampi(x0 - 1 + bx, 0, b.nx - 1);
    int const gy = clampi(y0 - HY + by, 0, b.ny - 1);
    int const gz = clampi(z0 - HZ + bz, 0, b.nz - 1);
    long long const gid = b.id(gx, gy, gz);
    for (int q = 0; q < nq; q++) Us[q * NB + t] = U[(long long)field_of_q(q, b) * b.n + gid];
  }
  __syncthreads();

  // face fluxes: x faces first, then y, then z (each thread takes a strided share)
  int const nfaces = NFX + NFY + NFZ;
  for (int t = threadIdx.x; t < nfaces; t += NT) {
    int dir, i, j, k, nfd;
    double *Fd;
    if (t < NFX) {
      dir = 0, nfd = NFX, Fd = Fxs;
      int const u = t;
      i = u % (TX + 1), j = (u / (TX + 1)) % TY, k = u / ((TX + 1) * TY);
    } else if (t < NFX + NFY) {
      dir = 1, nfd = NFY, Fd = Fys;
      int const u = t - NFX;
      i = u % TX, j = (u / TX) % (TY + 1), k = u / (TX * (TY + 1));
    } else {
      dir = 2, nfd = NFZ, Fd = Fzs;
      int const u = t - NFX - NFY;
      i = u % TX, j = (u / TX) % TY, k = u / (TX * TY);
    }
    // left and right box cells of this face
    int lx = i + 1, ly = j + HY, lz = k + HZ;
    if (dir == 0) lx = i;
    if (dir == 1) ly = j;
    if (dir == 2) lz = k;
    int const rx = lx + (dir == 0), ry = ly + (dir == 1), rz = lz + (dir == 2);
    int const cl = lx + BX * (ly + BY * lz), cr = rx + BX * (ry + BY * rz);
    int o1, o2, o3;
    rot(dir, o1, o2, o3);
    double qL[NQ_MAX], qR[NQ_MAX], f[NQ_MAX];
#pragma unroll
    for (int q = 0; q < NQ_MAX; q++) {
      if (q < nq) {
        int const src = (q == 1) ? o1 : (q == 2) ? o2 : (q == 3) ? o3 : q;
        qL[q]         = Us[src * NB + cl];
        qR[q]         = Us[src * NB + cr];
      }
    }
    hx::riemann<SOLVER>(qL, qR, f, b.ns, b.de, b.gamma);
    int const fidx = t - (dir == 0 ? 0 : dir == 1 ? NFX : NFX + NFY);
#pragma unroll
    for (int q = 0; q < NQ_MAX; q++) {
      if (q < nq) {
        int const dst        = (q == 1) ? o1 : (q == 2) ? o2 : (q == 3) ? o3 : q;
        Fd[dst * nfd + fidx] = f[q];
      }
    }
  }
  __syncthreads();

  // half update (VL_3D_cuda.cu:379-495; VL_1D_cuda.cu:158-215 when ny = nz = 1)
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
  double const dth   = 0.5 * dt;
  double const dtodx = dth / b.dx, dtody = dth / b.dy, dtodz = dth / b.dz;
  int const fge      = b.nf - 1;

  double P = 0.0, Pp = 0.0, vx_imo = 0, vx_ipo = 0, vy_jmo = 0, vy_jpo = 0, vz_kmo = 0, vz_kpo = 0;
  int const qge = 5 + b.ns;
  if (b.de) {
    double const d = Us[c], d_inv = 1.0 / d;
    double const vx = Us[NB + c] * d_inv, vy = Us[2 * NB + c] * d_inv, vz = Us[3 * NB + c] * d_inv;
    double const E = Us[4 * NB + c], GE = Us[qge * NB + c];
    if (one_d) {
      // VL_1D_cuda.cu:180-187: plain total-minus-kinetic pressure, no floor
      P = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (b.gamma - 1.0);
      // hydro_cuda.cu:705-752 (1D partial update) uses the dual-energy pressure
      double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      Pp                 = fmax(hx::pressure_de(E, E - E_kin, GE, b.gamma), TINY);
    } else {
      double const E_kin = 0.5 * d * hx::sqmag(vx, vy, vz);
      P                  = hx::pressure_de(E, E - E_kin, GE, b.gamma);
      P                  = fmax(P, TINY);
      Pp                 = P;
    }
    vx_imo = Us[NB + c - 1] / Us[c - 1];
    vx_ipo = Us[NB + c + 1] / Us[c + 1];
    if (!one_d) {
      vy_jmo = Us[2 * NB + c - BX] / Us[c - BX];
      vy_jpo = Us[2 * NB + c + BX] / Us[c + BX];
      vz_kmo = Us[3 * NB + c - BX * BY] / Us[c - BX * BY];
      vz_kpo = Us[3 * NB + c + BX * BY] / Us[c + BX * BY];
    }
  }
  double out[NQ_MAX];
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++) {
    if (q < nq) {
      double v = Us[q * NB + c] + dtodx * (Fxs[q * NFX + fx] - Fxs[q * NFX + fx + 1]);
      if (!one_d) {
        v = v + dtody * (Fys[q * NFY + fy] - Fys[q * NFY + fy + TX]);
        v = v + dtodz * (Fzs[q * NFZ + fz] - Fzs[q * NFZ + fz + TX * TY]);
      }
      out[q] = v;
    }
  }
  if (b.de) {
    double const pdv = one_d ? 0.5 * P * (dtodx * (vx_imo - vx_ipo))
                             : 0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo) +
                                          dtodz * (vz_kmo - vz_kpo));
    out[qge] = out[qge] + pdv;
  }
  if (b.floor_on && !one_d) {
    double const floor = b.density_floor;
    if (out[0] < floor) {
      double const dens_0 = out[0];
      out[0]              = floor;
      out[1] *= (floor / dens_0);
      out[2] *= (floor / dens_0);
      out[3] *= (floor / dens_0);
      out[4] *= (floor / dens_0);
      if (b.de) out[qge] *= (floor / dens_0);
    }
  }
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++)
    if (q < nq) Uh[(long long)field_of_q(q, b) * b.n + gid] = out[q];

  // pdV partial update of GasEnergy with the full dt, on real cells (hydro_cuda.cu:754-833)
  if (b.de) {
    int const ng = b.ng;
    bool real    = gx >= ng && gx < b.nx - ng;
    if (!one_d) real = real && gy >= ng && gy < b.ny - ng && gz >= ng && gz < b.nz - ng;
    if (real) {
      double const fdx = dt / b.dx, fdy = dt / b.dy, fdz = dt / b.dz;
      double const GE  = Us[qge * NB + c];
      double const term =
          one_d ? 0.5 * Pp * (fdx * (vx_imo - vx_ipo))
                : 0.5 * Pp * (fdx * (vx_imo - vx_ipo) + fdy * (vy_jmo - vy_jpo) + fdz * (vz_kmo - vz_kpo));
      GEp[gid] = GE + term;
    }
  }
  (void)fge;
}

// ------------------------------------------------------------------------------------------
// corrector
// ------------------------------------------------------------------------------------------
// cells of U½ each side of a tile that its interface states need: PPM stencils 3, PLM 2, PCM 1
template <int RECON>
struct Halo {
  static constexpr int H = (RECON == RECON_PPMC || RECON == RECON_PPMP) ? 3
                           : (RECON == RECON_PLMC || RECON == RECON_PLMP) ? 2
                                                                           : 1;
};
// the primitive-limited reconstructions load their primitives their own way
template <int RECON>
__device__ __forceinline__ hx::Prim load_recon_prim(const double *q, const Box &b)
{
  if (RECON == RECON_PLMP || RECON == RECON_PPMP) return hx::load_prim_plm(q, b.ns, b.de, b.gamma);
  return hx::load_prim(q, b.ns, b.de, b.gamma);
}
// interface states of one cell (rotated conserved): qL at its high face, qR at its low face;
// prim_at(k) = the primitives k cells along the sweep from it
template <int RECON, typename F>
__device__ __forceinline__ void recon_cell(const Box &b, F prim_at, double *qLv, double *qRv)
{
  if (RECON == RECON_PPMC || RECON == RECON_PLMC) {
    hx::Prim Lp, Rp;
    if (RECON == RECON_PPMC) {
      hx::ppmc_cell(prim_at(-2), prim_at(-1), prim_at(0), prim_at(1), prim_at(2), b.ns, b.de, b.gamma, Lp, Rp);
    } else {
      hx::plmc_cell(prim_at(-1), prim_at(0), prim_at(1), b.ns, b.de, b.gamma, Lp, Rp);
    }
    hx::prim_to_q(Lp, qLv, b.ns, b.de, b.gamma);
    hx::prim_to_q(Rp, qRv, b.ns, b.de, b.gamma);
  } else if (RECON == RECON_PLMP) {
    hx::Prim const c[3] = {prim_at(-1), prim_at(0), prim_at(1)};
    hx::plmp_ppmp_cell<1>(c, b.ns, b.de, b.gamma, qLv, qRv);
  } else {
    hx::Prim const c[5] = {prim_at(-2), prim_at(-1), prim_at(0), prim_at(1), prim_at(2)};
    hx::plmp_ppmp_cell<2>(c, b.ns, b.de, b.gamma, qLv, qRv);
  }
}

template <int TX, int TY, int TZ, int RECON>
struct CorrSizes {
  static constexpr int H   = Halo<RECON>::H;
  static constexpr int HY  = TY > 1, HZ = TZ > 1;
  static constexpr int PX  = (TX + 2 * H) * TY * TZ;
  static constexpr int PY  = HY ? TX * (TY + 2 * H) * TZ : 0;
  static constexpr int PZ  = HZ ? TX * TY * (TZ + 2 * H) : 0;
  static constexpr int PM  = PX > PY ? (PX > PZ ? PX : PZ) : (PY > PZ ? PY : PZ);
  static constexpr int RX  = (TX + 2) * TY * TZ;
  static constexpr int RY  = HY ? TX * (TY + 2) * TZ : 0;
  static constexpr int RZ  = HZ ? TX * TY * (TZ + 2) : 0;
  static constexpr int RM  = RX > RY ? (RX > RZ ? RX : RZ) : (RY > RZ ? RY : RZ);
  static constexpr int FX  = (TX + 1) * TY * TZ;
  static constexpr int FY  = HY ? TX * (TY + 1) * TZ : 0;
  static constexpr int FZ  = HZ ? TX * TY * (TZ + 1) : 0;
  static constexpr int FM  = FX > FY ? (FX > FZ ? FX : FZ) : (FY > FZ ? FY : FZ);
  // shared doubles per carried quantity: pencil (primitives / conserved), QL, QR, F
  static constexpr int PER_Q = PM + (RECON == RECON_PCM ? 0 : 2 * RM) + FM;
};

// Two resident blocks per SM (128 registers, some spilled to L1) instead of the one that 164
// registers allow: 256^3 corrector 274 -> 241 ms; three blocks spill more and lose (249 ms).
template <int TX, int TY, int TZ, int RECON, int SOLVER>
__global__ void __launch_bounds__(TX *TY *TZ, 2) k_corrector(Box b, const double *__restrict__ Uh, double *__restrict__ U,
                                                          const double *__restrict__ GEp, double *__restrict__ Epre,
                                                          int *__restrict__ status, double dt,
                                                          const double *__restrict__ dtp)
{
  if (dtp) dt = *dtp;
  using S         = CorrSizes<TX, TY, TZ, RECON>;
  constexpr int H = S::H;
  constexpr int NT = TX * TY * TZ;
  extern __shared__ double smem[];
  int const nq = b.nq();
  double *Ps   = smem;             // [nq][PM]  primitives in rotated order (conserved for PCM)
  double *QLs  = Ps + nq * S::PM;  // [nq][RM]
  double *QRs  = (RECON == RECON_PCM) ? QLs : QLs + nq * S::RM;
  double *Fs   = (RECON == RECON_PCM) ? QLs : QRs + nq * S::RM;  // [nq][FM]

  int const ng = b.ng;
  int const x0 = ng + blockIdx.x * TX;
  int const y0 = S::HY ? ng + blockIdx.y * TY : 0;
  int const z0 = S::HZ ? ng + blockIdx.z * TZ : 0;
  bool const one_d = (b.ny == 1 && b.nz == 1);

  int const t  = threadIdx.x;
  int const ti = t % TX, tj = (t / TX) % TY, tk = t / (TX * TY);
  double acc[NQ_MAX];
#pragma unroll
  for (int q = 0; q < NQ_MAX; q++) acc[q] = 0.0;

  int const ndir = one_d ? 1 : 3;
  for (int dir = 0; dir < ndir; dir++) {
    int o1, o2, o3;
    rot(dir, o1, o2, o3);
    // extents of the pencil along (a = sweep axis, u, w = the other two tile axes)
    int const TA = dir == 0 ? TX : dir == 1 ? TY : TZ;
    int const TU = dir == 0 ? TY : dir == 1 ? TZ : TX;  // (y,z), (z,x), (x,y) ordering for u,w
    int const TW = dir == 0 ? TZ : dir == 1 ? TX : TY;
    int const LA = TA + 2 * H;
    int const np = LA * TU * TW;
    // 1. pencil of U½ -> primitives (Load_Data) for this direction
    for (int p = t; p < np; p += NT) {
      int const a = p % LA - H, u = (p / LA) % TU, w = p / (LA * TU);
      int gx, gy, gz;
      if (dir == 0) {
        gx = x0 + a, gy = y0 + u, gz = z0 + w;
      } else if (dir == 1) {
        gy = y0 + a, gz = z0 + u, gx = x0 + w;
      } else {
        gz = z0 + a, gx = x0 + u, gy = y0 + w;
      }
      gx = clampi(gx, 0, b.nx - 1);
      gy = clampi(gy, 0, b.ny - 1);
      gz = clampi(gz, 0, b.nz - 1);
      long long const gid = b.id(gx, gy, gz);
      double q[NQ_MAX];
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++) {
        if (qq < nq) {
          int const src = (qq == 1) ? o1 : (qq == 2) ? o2 : (qq == 3) ? o3 : field_of_q(qq, b);
          q[qq]         = Uh[(long long)src * b.n + gid];
        }
      }
      if (RECON == RECON_PCM) {
#pragma unroll
        for (int qq = 0; qq < NQ_MAX; qq++)
          if (qq < nq) Ps[qq * S::PM + p] = q[qq];
      } else {
        hx::Prim const P = load_recon_prim<RECON>(q, b);
        Ps[0 * S::PM + p] = P.d;
        Ps[1 * S::PM + p] = P.vn;
        Ps[2 * S::PM + p] = P.vt1;
        Ps[3 * S::PM + p] = P.vt2;
        Ps[4 * S::PM + p] = P.p;
#pragma unroll
        for (int k = 0; k < NS_MAX; k++)
          if (k < b.ns) Ps[(5 + k) * S::PM + p] = P.sc[k];
        if (b.de) Ps[(5 + b.ns) * S::PM + p] = P.ge;
      }
    }
    __syncthreads();
    // 2. reconstruct cells a = -1 .. TA along the sweep -> QL (at a+1/2), QR (at a-1/2)
    int const LR = TA + 2;
    if (RECON != RECON_PCM) {
      int const nr = LR * TU * TW;
      for (int r = t; r < nr; r += NT) {
        int const a = r % LR - 1, uw = r / LR;
        int const base = (a + H) + LA * uw;  // pencil index of the centre cell
        auto prim_at = [&](int off) {
          hx::Prim P;
          int const pi = base + off;
          P.d   = Ps[0 * S::PM + pi];
          P.vn  = Ps[1 * S::PM + pi];
          P.vt1 = Ps[2 * S::PM + pi];
          P.vt2 = Ps[3 * S::PM + pi];
          P.p   = Ps[4 * S::PM + pi];
#pragma unroll
          for (int k = 0; k < NS_MAX; k++) P.sc[k] = (k < b.ns) ? Ps[(5 + k) * S::PM + pi] : 0.0;
          P.ge = b.de ? Ps[(5 + b.ns) * S::PM + pi] : 0.0;
          return P;
        };
        double qLv[NQ_MAX], qRv[NQ_MAX];
        recon_cell<RECON>(b, prim_at, qLv, qRv);
#pragma unroll
        for (int qq = 0; qq < NQ_MAX; qq++) {
          if (qq < nq) {
            QLs[qq * S::RM + r] = qLv[qq];
            QRs[qq * S::RM + r] = qRv[qq];
          }
        }
      }
      __syncthreads();
    }
    // 3. Riemann problems at faces between a and a+1, a = -1 .. TA-1 (face index a+1)
    int const LF = TA + 1;
    int const nfc = LF * TU * TW;
    // PCM keeps the conserved pencil in Ps; fluxes go to a separate slice to avoid aliasing
    double *Fd = (RECON == RECON_PCM) ? QLs : Fs;
    for (int fi = t; fi < nfc; fi += NT) {
      int const a = fi % LF - 1, uw = fi / LF;
      double qL[NQ_MAX], qR[NQ_MAX], f[NQ_MAX];
      if (RECON == RECON_PCM) {
        int const pl = (a + H) + LA * uw, pr = pl + 1;
#pragma unroll
        for (int qq = 0; qq < NQ_MAX; qq++) {
          if (qq < nq) {
            qL[qq] = Ps[qq * S::PM + pl];
            qR[qq] = Ps[qq * S::PM + pr];
          }
        }
      } else {
        int const rl = (a + 1) + LR * uw, rr = rl + 1;
#pragma unroll
        for (int qq = 0; qq < NQ_MAX; qq++) {
          if (qq < nq) {
            qL[qq] = QLs[qq * S::RM + rl];
            qR[qq] = QRs[qq * S::RM + rr];
          }
        }
      }
      hx::riemann<SOLVER>(qL, qR, f, b.ns, b.de, b.gamma);
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++)
        if (qq < nq) Fd[qq * S::FM + fi] = f[qq];
    }
    __syncthreads();
    // 4. flux difference for this thread's cell, back in canonical field order
    {
      int a, u, w;
      if (dir == 0) {
        a = ti, u = tj, w = tk;
      } else if (dir == 1) {
        a = tj, u = tk, w = ti;
      } else {
        a = tk, u = ti, w = tj;
      }
      int const fm = a + LF * (u + TU * w);  // face a-1/2
      double const dtod = dt / (dir == 0 ? b.dx : dir == 1 ? b.dy : b.dz);
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++) {
        if (qq < nq) {
          int const dst  = (qq == 1) ? o1 : (qq == 2) ? o2 : (qq == 3) ? o3 : qq;
          double const d = dtod * (Fd[qq * S::FM + fm] - Fd[qq * S::FM + fm + 1]);
          // acc[dst] += d, written without a runtime-indexed register array
#pragma unroll
          for (int c = 0; c < NQ_MAX; c++)
            if (c == dst) acc[c] = (dir == 0) ? d : acc[c] + d;
        }
      }
    }
    __syncthreads();
  }

  // conserved update of real cells (hydro_cuda.cu:172-402; 1D: :20-82), in place
  int const gx = x0 + ti, gy = y0 + tj, gz = z0 + tk;
  bool real = gx < b.nx - ng;
  if (!one_d) real = real && gy < b.ny - ng && gz < b.nz - ng;
  if (!real) return;
  long long const gid = b.id(gx, gy, gz);
  double v[NQ_MAX];
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++) {
    if (qq < nq) {
      int const f     = field_of_q(qq, b);
      double const u0 = (b.de && qq == nq - 1) ? GEp[gid] : U[(long long)f * b.n + gid];
      v[qq]           = u0 + acc[qq];
    }
  }
  if (b.floor_on && !one_d) {
    double const floor = b.density_floor;
    if (v[0] < floor) {
      if (v[0] > 0) {
        double const dens_0 = v[0];
        v[0]                = floor;
        v[1] *= (floor / dens_0);
        v[2] *= (floor / dens_0);
        v[3] *= (floor / dens_0);
        v[4] *= (floor / dens_0);
        if (b.de) v[nq - 1] *= (floor / dens_0);
      } else {
        atomicOr(status, STATUS_NEG_DENSITY);  // negative density: averaged by the finalize kernel
      }
    }
  }
  if (not_finite(v[0]) || not_finite(v[4])) atomicOr(status, STATUS_NONFINITE);
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++)
    if (qq < nq) U[(long long)field_of_q(qq, b) * b.n + gid] = v[qq];
  if (b.de) Epre[gid] = v[4];
}

// ------------------------------------------------------------------------------------------
// The exact corrector as one sweep per direction over long pencils (x: 64 x 2 x 2 cells per
// block, y and z: 32 x 8 x 1), for boxes whose scratch has room for an FP64 accumulator: the
// fused 8 x 8 x 4 tile recomputes a third of its interface states in halos, these about 6%.
// Every operation and its order are the fused corrector's: primitives from U½ (Load_Data),
// PPMC / PLMC, the Riemann solver, d = dtod * (F(a-1/2) - F(a+1/2)); the x sweep stores d, the
// y sweep adds its own (acc + d), the z sweep adds its own and writes U + acc with the floor
// and the pre-sync energy, exactly as the fused kernel's register accumulator does.
// ------------------------------------------------------------------------------------------
// exact sweeps' tiles (compile-time tunables): x sweep cells per pencil and pencils along y and
// z, y and z sweeps cells per pencil and x-adjacent pencils
#ifndef CGB_XSWEEP_XL
#define CGB_XSWEEP_XL 64
#define CGB_XSWEEP_XA 2
#define CGB_XSWEEP_XB 2
#define CGB_XSWEEP_YL 32
#define CGB_XSWEEP_YA 8
#endif
constexpr int XSW_XL = CGB_XSWEEP_XL, XSW_XA = CGB_XSWEEP_XA, XSW_XB = CGB_XSWEEP_XB;
constexpr int XSW_YL = CGB_XSWEEP_YL, XSW_YA = CGB_XSWEEP_YA;

template <int DIR, int L, int WA, int WB, int RECON>
struct XSweep {
  static constexpr int H  = Halo<RECON>::H;
  static constexpr int CS = WA * WB;
  static constexpr int NT = L * CS;
  static constexpr int LA = L + 2 * H, LR = L + 2, LF = L + 1;
  static constexpr int NP = LA * CS, NR = LR * CS, NF = LF * CS;
  // the pencil (primitives, or conserved for PCM), QL, QR; the fluxes reuse the pencil once it
  // is consumed (PCM: they follow it)
  static constexpr int PER_Q  = RECON == RECON_PCM ? NP + NF : NP + 2 * NR;
  static constexpr int STRIDE = DIR == 0 ? 1 : CS;
  // position a of pencil c in an array of row length len: x sweeps keep a fastest, y and z
  // sweeps the pencil index (x), so that neighbouring threads touch neighbouring x
  __device__ static int at(int a, int c, int len) { return DIR == 0 ? a + len * c : c + CS * a; }
  __device__ static void split(int i, int len, int &a, int &c)
  {
    if (DIR == 0) {
      a = i % len, c = i / len;
    } else {
      c = i % CS, a = i / CS;
    }
  }
};

template <int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL>
__global__ void __launch_bounds__(L *WA *WB, 2)
    k_xsweep(Box b, const double *__restrict__ Uh, double *__restrict__ A, double *__restrict__ U,
             const double *__restrict__ GEp, double *__restrict__ Epre, int *__restrict__ status, double dt,
             const double *__restrict__ dtp)
{
  if (dtp) dt = *dtp;
  using S            = XSweep<DIR, L, WA, WB, RECON>;
  constexpr int H    = S::H;
  constexpr int NT   = S::NT;
  constexpr int ST   = S::STRIDE;
  extern __shared__ double smem[];
  int const nq = b.nq();
  double *Ps   = smem;
  double *QLs  = Ps + nq * S::NP;
  double *QRs  = QLs + nq * S::NR;
  double *Fs   = (RECON == RECON_PCM) ? QLs : Ps;
  int o1, o2, o3;
  rot(DIR, o1, o2, o3);
  int const ng      = b.ng;
  long long const n = b.n;
  int const a0 = blockIdx.x * L, ca0 = blockIdx.y * WA, cb0 = blockIdx.z * WB;
  int const rx = b.nx - 2 * ng, ry = b.ny - 2 * ng, rz = b.nz - 2 * ng;
  // partial tiles skip the interface states and fluxes no real cell needs
  int const lim  = (DIR == 0 ? rx : DIR == 1 ? ry : rz) - a0;
  auto pencil_in = [&](int c) { return ca0 + c % WA < (DIR == 0 ? ry : rx) && cb0 + c / WA < (DIR == 2 ? ry : rz); };
  auto cell      = [&](int a, int c, int &gx, int &gy, int &gz) {
    int const ca = ca0 + c % WA + ng, cb = cb0 + c / WA + ng, g = a0 + a + ng;
    if (DIR == 0) {
      gx = g, gy = ca, gz = cb;
    } else if (DIR == 1) {
      gy = g, gx = ca, gz = cb;
    } else {
      gz = g, gx = ca, gy = cb;
    }
  };
  int const t = threadIdx.x;
  // 1. pencils of U½ -> primitives (Load_Data); positions past the box read the nearest cell
  //    the predictor wrote (1 .. n-2) and feed only skipped interfaces
  for (int p = t; p < S::NP; p += NT) {
    int a, c, gx, gy, gz;
    S::split(p, S::LA, a, c);
    cell(a - H, c, gx, gy, gz);
    long long const gid = b.id(clampi(gx, 1, b.nx - 2), clampi(gy, 1, b.ny - 2), clampi(gz, 1, b.nz - 2));
    double q[NQ_MAX];
#pragma unroll
    for (int qq = 0; qq < NQ_MAX; qq++) {
      if (qq < nq) {
        int const src = (qq == 1) ? o1 : (qq == 2) ? o2 : (qq == 3) ? o3 : field_of_q(qq, b);
        q[qq]         = Uh[(long long)src * n + gid];
      }
    }
    if (RECON == RECON_PCM) {
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++)
        if (qq < nq) Ps[qq * S::NP + p] = q[qq];
    } else {
      hx::Prim const P = load_recon_prim<RECON>(q, b);
      Ps[0 * S::NP + p] = P.d;
      Ps[1 * S::NP + p] = P.vn;
      Ps[2 * S::NP + p] = P.vt1;
      Ps[3 * S::NP + p] = P.vt2;
      Ps[4 * S::NP + p] = P.p;
#pragma unroll
      for (int k = 0; k < NS_MAX; k++)
        if (k < b.ns) Ps[(5 + k) * S::NP + p] = P.sc[k];
      if (b.de) Ps[(5 + b.ns) * S::NP + p] = P.ge;
    }
  }
  __syncthreads();
  // 2. reconstruction: recon position a holds cell a - 1 (QL at its right face, QR at its left)
  if (RECON != RECON_PCM) {
    for (int r = t; r < S::NR; r += NT) {
      int a, c;
      S::split(r, S::LR, a, c);
      if (a > lim + 1 || !pencil_in(c)) continue;
      int const base = S::at(a - 1 + H, c, S::LA);
      auto prim_at   = [&](int off) {
        hx::Prim P;
        int const pi = base + off * ST;
        P.d          = Ps[0 * S::NP + pi];
        P.vn         = Ps[1 * S::NP + pi];
        P.vt1        = Ps[2 * S::NP + pi];
        P.vt2        = Ps[3 * S::NP + pi];
        P.p          = Ps[4 * S::NP + pi];
#pragma unroll
        for (int k = 0; k < NS_MAX; k++) P.sc[k] = (k < b.ns) ? Ps[(5 + k) * S::NP + pi] : 0.0;
        P.ge = b.de ? Ps[(5 + b.ns) * S::NP + pi] : 0.0;
        return P;
      };
      double qLv[NQ_MAX], qRv[NQ_MAX];
      recon_cell<RECON>(b, prim_at, qLv, qRv);
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++) {
        if (qq < nq) {
          QLs[qq * S::NR + r] = qLv[qq];
          QRs[qq * S::NR + r] = qRv[qq];
        }
      }
    }
    __syncthreads();
  }
  // 3. Riemann problems: face a lies between cells a - 1 and a
  for (int f = t; f < S::NF; f += NT) {
    int a, c;
    S::split(f, S::LF, a, c);
    if (a > lim || !pencil_in(c)) continue;
    double qL[NQ_MAX], qR[NQ_MAX], fl[NQ_MAX];
    if (RECON == RECON_PCM) {
      int const pl = S::at(a - 1 + H, c, S::LA), pr = pl + ST;
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++) {
        if (qq < nq) {
          qL[qq] = Ps[qq * S::NP + pl];
          qR[qq] = Ps[qq * S::NP + pr];
        }
      }
    } else {
      int const rl = S::at(a, c, S::LR), rr = rl + ST;
#pragma unroll
      for (int qq = 0; qq < NQ_MAX; qq++) {
        if (qq < nq) {
          qL[qq] = QLs[qq * S::NR + rl];
          qR[qq] = QRs[qq * S::NR + rr];
        }
      }
    }
    hx::riemann<SOLVER>(qL, qR, fl, b.ns, b.de, b.gamma);
#pragma unroll
    for (int qq = 0; qq < NQ_MAX; qq++)
      if (qq < nq) Fs[qq * S::NF + f] = fl[qq];
  }
  __syncthreads();
  // 4. this thread's cell: the flux difference of the sweep added to the accumulator
  int a, c, gx, gy, gz;
  S::split(t, L, a, c);
  cell(a, c, gx, gy, gz);
  if (!(gx < b.nx - ng && gy < b.ny - ng && gz < b.nz - ng)) return;
  long long const gid = b.id(gx, gy, gz);
  int const fm        = S::at(a, c, S::LF);
  double const dtod   = dt / (DIR == 0 ? b.dx : DIR == 1 ? b.dy : b.dz);
  double acc[NQ_MAX];
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++) acc[qq] = 0.0;
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++) {
    if (qq < nq) {
      int const dst  = (qq == 1) ? o1 : (qq == 2) ? o2 : (qq == 3) ? o3 : qq;
      double const d = dtod * (Fs[qq * S::NF + fm] - Fs[qq * S::NF + fm + ST]);
#pragma unroll
      for (int cc = 0; cc < NQ_MAX; cc++)
        if (cc == dst) acc[cc] = FIRST ? d : A[(long long)cc * n + gid] + d;
    }
  }
  if constexpr (!FINAL) {
#pragma unroll
    for (int qq = 0; qq < NQ_MAX; qq++)
      if (qq < nq) A[(long long)qq * n + gid] = acc[qq];
    return;
  }
  // conserved update of real cells (hydro_cuda.cu:172-402), in place, as in k_corrector
  double v[NQ_MAX];
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++) {
    if (qq < nq) {
      int const f     = field_of_q(qq, b);
      double const u0 = (b.de && qq == nq - 1) ? GEp[gid] : U[(long long)f * n + gid];
      v[qq]           = u0 + acc[qq];
    }
  }
  if (b.floor_on) {
    double const floor = b.density_floor;
    if (v[0] < floor) {
      if (v[0] > 0) {
        double const dens_0 = v[0];
        v[0]                = floor;
        v[1] *= (floor / dens_0);
        v[2] *= (floor / dens_0);
        v[3] *= (floor / dens_0);
        v[4] *= (floor / dens_0);
        if (b.de) v[nq - 1] *= (floor / dens_0);
      } else {
        atomicOr(status, STATUS_NEG_DENSITY);  // negative density: averaged by the finalize kernel
      }
    }
  }
  if (not_finite(v[0]) || not_finite(v[4])) atomicOr(status, STATUS_NONFINITE);
#pragma unroll
  for (int qq = 0; qq < NQ_MAX; qq++)
    if (qq < nq) U[(long long)field_of_q(qq, b) * n + gid] = v[qq];
  if (b.de) Epre[gid] = v[4];
}

template <int DIR, int L, int WA, int WB, int RECON, int SOLVER, bool FIRST, bool FINAL>
cudaError_t launch_xsweep(const Box &b, const double *Uh, double *A, double *U, const Scratch &sc, double dt,
                          const double *dtp, cudaStream_t s)
{
  using S         = XSweep<DIR, L, WA, WB, RECON>;
  size_t const sm = sizeof(double) * (size_t)b.nq() * S::PER_Q;
  auto k          = k_xsweep<DIR, L, WA, WB, RECON, SOLVER, FIRST, FINAL>;
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int const rx = b.nx - 2 * b.ng, ry = b.ny - 2 * b.ng, rz = b.nz - 2 * b.ng;
  int const ra = DIR == 0 ? rx : DIR == 1 ? ry : rz, rb = DIR == 0 ? ry : rx, rc = DIR == 2 ? ry : rz;
  dim3 grid((ra + L - 1) / L, (rb + WA - 1) / WA, (rc + WB - 1) / WB);
  k<<<grid, L * WA * WB, sm, s>>>(b, Uh, A, U, sc.GEp, sc.Epre, sc.status, dt, dtp);
  return cudaGetLastError();
}

// the three exact sweeps of one recon / solver pair
template <int RECON, int SOLVER>
cudaError_t launch_xsweeps(const Box &b, double *U, const Scratch &sc, double dt, const double *dtp, cudaStream_t s)
{
  double *A     = static_cast<double *>(sc.W);
  cudaError_t e = launch_xsweep<0, XSW_XL, XSW_XA, XSW_XB, RECON, SOLVER, true, false>(b, sc.Uh, A, U, sc, dt, dtp, s);
  if (e == cudaSuccess)
    e = launch_xsweep<1, XSW_YL, XSW_YA, 1, RECON, SOLVER, false, false>(b, sc.Uh, A, U, sc, dt, dtp, s);
  if (e == cudaSuccess)
    e = launch_xsweep<2, XSW_YL, XSW_YA, 1, RECON, SOLVER, false, true>(b, sc.Uh, A, U, sc, dt, dtp, s);
  return e;
}

template <int TX, int TY, int TZ, int SOLVER>
size_t predictor_smem(const Box &b)
{
  constexpr int HY = TY > 1 ? 1 : 0, HZ = TZ > 1 ? 1 : 0;
  constexpr int NB  = (TX + 2) * (TY + 2 * HY) * (TZ + 2 * HZ);
  constexpr int NFX = (TX + 1) * TY * TZ;
  constexpr int NFY = HY ? TX * (TY + 1) * TZ : 0;
  constexpr int NFZ = HZ ? TX * TY * (TZ + 1) : 0;
  return sizeof(double) * (size_t)b.nq() * (NB + NFX + NFY + NFZ);
}

template <int TX, int TY, int TZ, int RECON, int SOLVER>
size_t corrector_smem(const Box &b)
{
  return sizeof(double) * (size_t)b.nq() * CorrSizes<TX, TY, TZ, RECON>::PER_Q;
}

template <int TX, int TY, int TZ, int SOLVER>
cudaError_t launch_predictor(const Box &b, const double *U, double *Uh, double *GEp, double dt, const double *dtp,
                             cudaStream_t s)
{
  size_t const sm = predictor_smem<TX, TY, TZ, SOLVER>(b);
  auto k          = k_predictor<TX, TY, TZ, SOLVER>;
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  dim3 grid((b.nx - 2 + TX - 1) / TX, TY > 1 ? (b.ny - 2 + TY - 1) / TY : 1, TZ > 1 ? (b.nz - 2 + TZ - 1) / TZ : 1);
  k<<<grid, TX * TY * TZ, sm, s>>>(b, U, Uh, GEp, dt, dtp);
  return cudaGetLastError();
}

template <int TX, int TY, int TZ, int RECON, int SOLVER>
cudaError_t launch_corrector(const Box &b, const double *Uh, double *U, const double *GEp, double *Epre, int *status,
                             double dt, const double *dtp, cudaStream_t s)
{
  size_t const sm = corrector_smem<TX, TY, TZ, RECON, SOLVER>(b);
  auto k          = k_corrector<TX, TY, TZ, RECON, SOLVER>;
  cudaError_t e   = cudaFuncSetAttribute(k, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)sm);
  if (e != cudaSuccess) return e;
  int const rx = b.nx - 2 * b.ng, ry = b.ny - 2 * b.ng, rz = b.nz - 2 * b.ng;
  dim3 grid((rx + TX - 1) / TX, TY > 1 ? (ry + TY - 1) / TY : 1, TZ > 1 ? (rz + TZ - 1) / TZ : 1);
  k<<<grid, TX * TY * TZ, sm, s>>>(b, Uh, U, GEp, Epre, status, dt, dtp);
  return cudaGetLastError();
}

template <int TX, int TY, int TZ, int SOLVER>
cudaError_t dispatch_step(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                          cudaStream_t s, cudaEvent_t *marks)
{
  cudaError_t e;
  if (marks) cudaEventRecord(marks[0], s);
  e = launch_predictor<TX, TY, TZ, SOLVER>(b, U, sc.Uh, sc.GEp, dt, dtp, s);
  if (e != cudaSuccess) return e;
  if (marks) cudaEventRecord(marks[1], s);
  // 3D with an accumulator in the scratch: the three sweeps; else the fused tile corrector
  bool const sweeps = TY > 1 && sc.W != nullptr;
#define CGB_CORR(R)                                                                                       \
  (sweeps ? launch_xsweeps<R, SOLVER>(b, U, sc, dt, dtp, s)                                               \
          : launch_corrector<TX, TY, TZ, R, SOLVER>(b, sc.Uh, U, sc.GEp, sc.Epre, sc.status, dt, dtp, s))
  switch (recon) {
    case RECON_PPMC: e = CGB_CORR(RECON_PPMC); break;
    case RECON_PLMC: e = CGB_CORR(RECON_PLMC); break;
    case RECON_PLMP: e = CGB_CORR(RECON_PLMP); break;
    case RECON_PPMP: e = CGB_CORR(RECON_PPMP); break;
    default: e = CGB_CORR(RECON_PCM); break;
  }
#undef CGB_CORR
  if (marks) cudaEventRecord(marks[2], s);
  return e;
}
}  // namespace

// one exact FP64 predictor + corrector with the solver SOLVER (1D boxes: TY = TZ = 1)
template <int SOLVER>
cudaError_t exact_solver_step(const Box &b, int recon, double *U, const Scratch &sc, double dt, const double *dtp,
                              cudaStream_t s, cudaEvent_t *marks)
{
  bool const one_d = (b.ny == 1 && b.nz == 1);
  return one_d ? dispatch_step<128, 1, 1, SOLVER>(b, recon, U, sc, dt, dtp, s, marks)
               : dispatch_step<8, 8, 4, SOLVER>(b, recon, U, sc, dt, dtp, s, marks);
}

}  // namespace cgb
