// mhd_body.cuh -- the VL step of ideal MHD with constrained transport in FP64, written in the
// reference's operation order.  Compiled twice: mhd_exact.cu (-fmad=false, the reference's own
// operations: bit-identical to the reference build) and mhd_fast.cu (the fast FP64 form: the
// helpers mdiv, msqrt, mmin, ... below switch to reciprocal, Newton and integer-pipe forms,
// and multiply-adds are contracted into FMAs).  The includer defines CGB_MHD_NS (kernel
// namespace), CGB_MHD_STEP (the step's name), CGB_MHD_FAST and CGB_MHD_REDUCTIONS (1: also
// define the scratch size, CFL and div B entry points).
//
// Stages of VL_Algorithm_3D_CUDA with MHD (src/integrators/VL_3D_cuda.cu:38-360), one kernel
// each, interface states and fluxes in HBM as the reference keeps them (the step is bound by the
// FP64 pipe, not by this traffic):
//   PCM (cell-centred B) -> HLLD x/y/z -> CT edge EMFs -> half update + face-B half update
//   PLMC / PPMC on U½ (MHD characteristic projection) -> HLLD -> CT EMFs -> full update,
//   face-B update, density floor.
// State layout: fields d, mx, my, mz, E, [scalars], Bx, By, Bz (face-centred at +1/2).  The
// interface and flux arrays hold nf - 1 fields: the hydro ones, then the two transverse B
// components of the sweep (By, Bz in the rotated frame) at 5 + ns and 6 + ns.
#include "common.cuh"
#include "hydro_math.cuh"
#include "kernels.h"
#if CGB_MHD_FAST
#include "hydro_fast.cuh"
#endif

namespace cgb
{
namespace CGB_MHD_NS
{

constexpr double HLLD_SMALL = 1.0e-8;  // src/riemann_solvers/hlld_cuda.h:56

// The arithmetic that the two builds do differently.  Exact (CGB_MHD_FAST 0): the reference's
// operations themselves.  Fast: quotients as products with a reciprocal (FP32 seed + two
// Newton steps, shared where a denominator repeats: mdivr with minv), square roots and
// reciprocal square roots from FP32 seeds with Newton steps, and minima, maxima and sign tests
// on the integer pipe (the step is bound by the FP64 pipe).  Each fast form is within an ulp
// or two of the exact one.
#if CGB_MHD_FAST
__device__ __forceinline__ double mdiv(double a, double b) { return a * hf::rcp(b); }
__device__ __forceinline__ double minv(double b) { return hf::rcp(b); }
__device__ __forceinline__ double mdivr(double a, double, double rb) { return a * rb; }
__device__ __forceinline__ double msqrt(double x) { return hf::sqrtT(x); }
__device__ __forceinline__ double mrsqrt(double x) { return hf::rcp(hf::sqrtT(x)); }
__device__ __forceinline__ double mmin(double a, double b) { return hf::min_ord(a, b); }
__device__ __forceinline__ double mmax(double a, double b) { return hf::max_ord(a, b); }
__device__ __forceinline__ bool mpos(double l, double r) { return hf::prod_pos(l, r); }  // l * r > 0
__device__ __forceinline__ bool mgt0(double x) { return hf::is_pos(x); }                  // x > 0
__device__ __forceinline__ bool mlt0(double x) { return hf::is_neg(x); }                  // x < 0
#else
__device__ __forceinline__ double mdiv(double a, double b) { return a / b; }
__device__ __forceinline__ double minv(double) { return 0.0; }  // unused by mdivr
__device__ __forceinline__ double mdivr(double a, double b, double) { return a / b; }
__device__ __forceinline__ double msqrt(double x) { return sqrt(x); }
__device__ __forceinline__ double mrsqrt(double x) { return rsqrt(x); }
__device__ __forceinline__ double mmin(double a, double b) { return fmin(a, b); }
__device__ __forceinline__ double mmax(double a, double b) { return fmax(a, b); }
__device__ __forceinline__ bool mpos(double l, double r) { return l * r > 0.0; }
__device__ __forceinline__ bool mgt0(double x) { return x > 0.0; }
__device__ __forceinline__ bool mlt0(double x) { return x < 0.0; }
#endif

__device__ __forceinline__ double dot3(double a1, double a2, double a3, double b1, double b2, double b3)
{
  return a1 * b1 + ((a2 * b2) + (a3 * b3));  // math_utilities.h dotProduct
}
__device__ __forceinline__ double sqm(double a, double b, double c) { return dot3(a, b, c, a, b, c); }
__device__ __forceinline__ double magE(double bx, double by, double bz) { return 0.5 * sqm(bx, by, bz); }

// mhd_utilities.h:205-237 cellCenteredMagneticFields
__device__ __forceinline__ void cc_b(const Box &b, const double *U, int x, int y, int z, double &bx, double &by,
                                     double &bz)
{
  long long const id = b.id(x, y, z), n = b.n;
  const double *Bx = U + (long long)b.fB() * n, *By = Bx + n, *Bz = By + n;
  bx = (x > 0) ? 0.5 * (Bx[id] + Bx[b.id(x - 1, y, z)]) : Bx[id];
  by = (y > 0) ? 0.5 * (By[id] + By[b.id(x, y - 1, z)]) : By[id];
  bz = (z > 0) ? 0.5 * (Bz[id] + Bz[b.id(x, y, z - 1)]) : Bz[id];
}

// mhd_utilities.h:38-59 _magnetosonicSpeed
__device__ __forceinline__ double magnetosonic(double d, double p, double bx, double by, double bz, double gamma,
                                               double choice)
{
  double const bXSquared = bx * bx;
  double const bSquared  = bXSquared + ((by * by) + (bz * bz));
  double const term1     = gamma * p + bSquared;
  double term2           = (term1 * term1) - 4. * gamma * p * bXSquared;
  term2                  = msqrt(term2);
  return msqrt(mdiv(term1 + choice * term2, 2.0 * mmax(d, TINY)));
}
__device__ __forceinline__ double cfast(double d, double p, double bx, double by, double bz, double g)
{
  return magnetosonic(d, p, bx, by, bz, g, 1.0);
}
__device__ __forceinline__ double cslow(double d, double p, double bx, double by, double bz, double g)
{
  return magnetosonic(d, p, bx, by, bz, g, -1.0);
}

struct MPrim {
  double d, vx, vy, vz, p, bx, by, bz;
  double sc[NS_MAX];
};
struct Chr {
  double a[7];
};
struct Eig {
  double cf, cs, af, as, by, bz, nfs, sign, qf, qs, Af, As, qpf, qps, Apf, Aps;
};

// reconstruction.h:139-212 Load_Data (MHD, no dual energy), rotated to sweep o1
__device__ __forceinline__ MPrim load_data(const Box &b, const double *U, int x, int y, int z, int o1, int o2, int o3)
{
  long long const id = b.id(x, y, z), n = b.n;
  MPrim P;
  P.d  = U[id];
  double const rd = minv(P.d);
  P.vx = mdivr(U[o1 * n + id], P.d, rd);
  P.vy = mdivr(U[o2 * n + id], P.d, rd);
  P.vz = mdivr(U[o3 * n + id], P.d, rd);
  double cbx, cby, cbz;
  cc_b(b, U, x, y, z, cbx, cby, cbz);
  if (o1 == 1) {
    P.bx = cbx, P.by = cby, P.bz = cbz;
  } else if (o1 == 2) {
    P.bx = cby, P.by = cbz, P.bz = cbx;
  } else {
    P.bx = cbz, P.by = cbx, P.bz = cby;
  }
  // hydro_utilities.h:34-45 Calc_Pressure_Primitive
  double pressure = U[4 * n + id] - 0.5 * P.d * sqm(P.vx, P.vy, P.vz);
  pressure -= magE(P.bx, P.by, P.bz);
  P.p = mmax((b.gamma - 1.) * pressure, TINY);
#pragma unroll
  for (int s = 0; s < NS_MAX; s++) P.sc[s] = s < b.ns ? mdivr(U[(long long)(5 + s) * n + id], P.d, rd) : 0.0;
  return P;
}

// reconstruction.h:310-361 Compute_Eigenvectors
__device__ __forceinline__ Eig eigenvectors(const MPrim &p, double cs, double cs2, double gamma)
{
  Eig e;
  e.cf = cfast(p.d, p.p, p.bx, p.by, p.bz, gamma);
  e.cs = cslow(p.d, p.p, p.bx, p.by, p.bz, gamma);
  double const cf2 = e.cf * e.cf, css2 = e.cs * e.cs;
  double const denom = (cf2 - css2), num2 = (cf2 - cs2);
  if (denom <= 0.0 or num2 <= 0.0) {
    e.af = 1.0;
    e.as = 0.0;
  } else {
    double const num1 = (cs2 - css2);
    if (num1 <= 0.0) {
      e.af = 0.0;
      e.as = 1.0;
    } else {
      double const rden = minv(denom);
      e.af = msqrt(mdivr(num1, denom, rden));
      e.as = msqrt(mdivr(num2, denom, rden));
    }
  }
  double const bd = rhypot(p.by, p.bz);
  e.by            = isfinite(bd) ? p.by * bd : 1.0;
  e.bz            = isfinite(bd) ? p.bz * bd : 0.0;
  e.sign          = copysign(1.0, p.bx);
  e.nfs           = mdiv(0.5, cs2);
  e.qpf           = e.sign * e.nfs * e.af * e.cf;
  e.qps           = e.sign * e.nfs * e.as * e.cs;
  e.qf            = e.sign * e.af * e.cf;
  e.qs            = e.sign * e.as * e.cs;
  double const sd = msqrt(p.d), rcsd = minv(cs * sd);
  e.Af            = e.af * cs * sd;
  e.As            = e.as * cs * sd;
  e.Apf           = mdivr(0.5 * e.af, cs * sd, rcsd);
  e.Aps           = mdivr(0.5 * e.as, cs * sd, rcsd);
  return e;
}

// reconstruction.h:378-437 Primitive_To_Characteristic (MHD)
__device__ __forceinline__ Chr prim_to_char(const MPrim &p, const MPrim &s, const Eig &e, double cs2, double rd,
                                            double rcs2)
{
  Chr o;
  double const isd = mrsqrt(p.d);
  double const pd  = mdivr(s.p, p.d, rd);
  o.a[0] = e.nfs * e.af * (pd - e.cf * s.vx) + e.qps * (e.by * s.vy + e.bz * s.vz) +
           e.Aps * (e.by * s.by + e.bz * s.bz);
  o.a[1] = 0.5 * (e.by * (s.bz * e.sign * isd + s.vz) - e.bz * (s.by * e.sign * isd + s.vy));
  o.a[2] = e.nfs * e.as * (pd - e.cs * s.vx) - e.qpf * (e.by * s.vy + e.bz * s.vz) -
           e.Apf * (e.by * s.by + e.bz * s.bz);
  o.a[3] = s.d - mdivr(s.p, cs2, rcs2);
  o.a[4] = e.nfs * e.as * (pd + e.cs * s.vx) + e.qpf * (e.by * s.vy + e.bz * s.vz) -
           e.Apf * (e.by * s.by + e.bz * s.bz);
  o.a[5] = 0.5 * (e.by * (s.bz * e.sign * isd - s.vz) - e.bz * (s.by * e.sign * isd - s.vy));
  o.a[6] = e.nfs * e.af * (pd + e.cf * s.vx) - e.qps * (e.by * s.vy + e.bz * s.vz) +
           e.Aps * (e.by * s.by + e.bz * s.bz);
  return o;
}

// reconstruction.h:453-491 Characteristic_To_Primitive (MHD)
__device__ __forceinline__ MPrim char_to_prim(const MPrim &p, const Chr &c, const Eig &e, double cs2)
{
  MPrim o;
  const double *a = c.a;
  o.d  = p.d * (e.af * (a[0] + a[6]) + e.as * (a[2] + a[4])) + a[3];
  o.vx = e.cf * e.af * (a[6] - a[0]) + e.cs * e.as * (a[4] - a[2]);
  o.vy = e.by * (e.qs * (a[0] - a[6]) + e.qf * (a[4] - a[2])) + e.bz * (a[5] - a[1]);
  o.vz = e.bz * (e.qs * (a[0] - a[6]) + e.qf * (a[4] - a[2])) + e.by * (a[1] - a[5]);
  o.p  = p.d * cs2 * (e.af * (a[0] + a[6]) + e.as * (a[2] + a[4]));
  o.bx = 0.0;
  double const sd = msqrt(p.d);
  o.by = e.by * (e.As * (a[0] + a[6]) - e.Af * (a[2] + a[4])) - e.bz * e.sign * sd * (a[5] + a[1]);
  o.bz = e.bz * (e.As * (a[0] + a[6]) - e.Af * (a[2] + a[4])) + e.by * e.sign * sd * (a[5] + a[1]);
#pragma unroll
  for (int s = 0; s < NS_MAX; s++) o.sc[s] = 0.0;
  return o;
}

// reconstruction.h:918-968 Write_Data (MHD): conserved interface state of the sweep's frame
__device__ __forceinline__ void write_data(const Box &b, const MPrim &s, double *Q, const double *U, long long id,
                                           int o1, int o2, int o3)
{
  long long const n = b.n;
  Q[id]          = s.d;
  Q[o1 * n + id] = s.d * s.vx;
  Q[o2 * n + id] = s.d * s.vy;
  Q[o3 * n + id] = s.d * s.vz;
  Q[(long long)b.fB() * n + id]       = s.by;
  Q[(long long)(b.fB() + 1) * n + id] = s.bz;
  double const bx = U[(long long)(b.fB() + (o1 - 1)) * n + id];
  // hydro_utilities.h:106-118 Calc_Energy_Primitive
  double energy = mdiv(mmax(s.p, TINY), b.gamma - 1.) + 0.5 * s.d * sqm(s.vx, s.vy, s.vz);
  energy += magE(bx, s.by, s.bz);
  Q[4 * n + id] = energy;
  for (int k = 0; k < b.ns; k++) Q[(long long)(5 + k) * n + id] = s.d * s.sc[k];
}

__device__ __forceinline__ void perm(int dir, int &o1, int &o2, int &o3)
{
  o1 = dir == 0 ? 1 : dir == 1 ? 2 : 3;
  o2 = dir == 0 ? 2 : dir == 1 ? 3 : 1;
  o3 = dir == 0 ? 3 : dir == 1 ? 1 : 2;
}

// reconstruction.h:95-119 Thread_Guard (true = skip)
template <int order>
__device__ __forceinline__ bool guard(const Box &b, int x, int y, int z)
{
  bool out = x < order - 1 or x >= b.nx - order;
  if (b.ny > 1) out = y < order - 1 or y >= b.ny - order or out;
  if (b.nz > 1) {
    out = z < order - 1 or z >= b.nz - order or out;
  } else {
    out = z >= b.nz or out;
  }
  return out;
}

__device__ __forceinline__ void xyz(const Box &b, long long t, int &x, int &y, int &z)
{
  z = (int)(t / ((long long)b.nx * b.ny));
  y = (int)((t - (long long)z * b.nx * b.ny) / b.nx);
  x = (int)(t - (long long)z * b.nx * b.ny - (long long)y * b.nx);
}

#define CGB_CELLS(t) \
  for (long long t = (long long)blockIdx.x * blockDim.x + threadIdx.x; t < b.n; t += (long long)gridDim.x * blockDim.x)

// ------------------------------------------------------------------------------------------
// reconstruction
// ------------------------------------------------------------------------------------------
// pcm_cuda.cu:256-424 PCM_Reconstruction_3D (MHD): cell-centred B, transverse components
__global__ void k_pcm(Box b, const double *__restrict__ U, double *QLx, double *QRx, double *QLy, double *QRy,
                      double *QLz, double *QRz)
{
  long long const n = b.n;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    double const d = U[id], mxv = U[n + id], myv = U[2 * n + id], mzv = U[3 * n + id], E = U[4 * n + id];
    double cbx, cby, cbz;
    cc_b(b, U, x, y, z, cbx, cby, cbz);
    double const bb[3] = {cbx, cby, cbz};
    auto put = [&](double *Q, long long at, int dir) {
      Q[at]         = d;
      Q[n + at]     = mxv;
      Q[2 * n + at] = myv;
      Q[3 * n + at] = mzv;
      Q[4 * n + at] = E;
      for (int s = 0; s < b.ns; s++) Q[(long long)(5 + s) * n + at] = U[(long long)(5 + s) * n + id];
      Q[(long long)b.fB() * n + at]       = bb[(dir + 1) % 3];
      Q[(long long)(b.fB() + 1) * n + at] = bb[(dir + 2) % 3];
    };
    put(QLx, id, 0);
    put(QLy, id, 1);
    put(QLz, id, 2);
    if (x > 0) put(QRx, b.id(x - 1, y, z), 0);
    if (y > 0) put(QRy, b.id(x, y - 1, z), 1);
    if (z > 0) put(QRz, b.id(x, y, z - 1), 2);
  }
}

// ppmc_cuda.cu:540-695 PPMC_VL with the MHD characteristic projection (7 waves)
__global__ void k_ppmc(Box b, const double *__restrict__ U, double *QL, double *QR, int dir)
{
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  int const sx = dir == 0, sy = dir == 1, sz = dir == 2;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    if (guard<3>(b, x, y, z)) continue;
    MPrim const ci   = load_data(b, U, x, y, z, o1, o2, o3);
    MPrim const cim1 = load_data(b, U, x - sx, y - sy, z - sz, o1, o2, o3);
    MPrim const cip1 = load_data(b, U, x + sx, y + sy, z + sz, o1, o2, o3);
    MPrim const cim2 = load_data(b, U, x - 2 * sx, y - 2 * sy, z - 2 * sz, o1, o2, o3);
    MPrim const cip2 = load_data(b, U, x + 2 * sx, y + 2 * sy, z + 2 * sz, o1, o2, o3);
    double const rd  = minv(ci.d);
    double const cs  = msqrt(mdivr(b.gamma * ci.p, ci.d, rd));  // hydro_utilities.h:209 Calc_Sound_Speed
    double const cs2 = cs * cs, rcs2 = minv(cs2);
    Eig const e      = eigenvectors(ci, cs, cs2, b.gamma);
    Chr const ai = prim_to_char(ci, ci, e, cs2, rd, rcs2), aim1 = prim_to_char(ci, cim1, e, cs2, rd, rcs2),
              aim2 = prim_to_char(ci, cim2, e, cs2, rd, rcs2), aip1 = prim_to_char(ci, cip1, e, cs2, rd, rcs2),
              aip2 = prim_to_char(ci, cip2, e, cs2, rd, rcs2);
    Chr aR, aL;
#pragma unroll
    for (int k = 0; k < 7; k++) hx::ppm1(aim2.a[k], aim1.a[k], ai.a[k], aip1.a[k], aip2.a[k], aL.a[k], aR.a[k]);
    MPrim L = char_to_prim(ci, aL, e, cs2);
    MPrim R = char_to_prim(ci, aR, e, cs2);
    for (int s = 0; s < b.ns; s++) hx::ppm1(cim2.sc[s], cim1.sc[s], ci.sc[s], cip1.sc[s], cip2.sc[s], L.sc[s], R.sc[s]);
    R.d = mmax(R.d, TINY);
    L.d = mmax(L.d, TINY);
    R.p = mmax(R.p, TINY);
    L.p = mmax(L.p, TINY);
    write_data(b, L, QL, U, id, o1, o2, o3);
    write_data(b, R, QR, U, b.id(x - sx, y - sy, z - sz), o1, o2, o3);
  }
}

// plmc_cuda.cu:24-300 PLMC_cuda with the MHD characteristic projection
__global__ void k_plmc(Box b, const double *__restrict__ U, double *QL, double *QR, int dir)
{
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  int const sx = dir == 0, sy = dir == 1, sz = dir == 2;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    if (guard<2>(b, x, y, z)) continue;
    MPrim const ci   = load_data(b, U, x, y, z, o1, o2, o3);
    MPrim const cimo = load_data(b, U, x - sx, y - sy, z - sz, o1, o2, o3);
    MPrim const cipo = load_data(b, U, x + sx, y + sy, z + sz, o1, o2, o3);
    double const rd  = minv(ci.d);
    double const cs  = msqrt(mdivr(b.gamma * ci.p, ci.d, rd));
    double const cs2 = cs * cs, rcs2 = minv(cs2);
    Eig const e      = eigenvectors(ci, cs, cs2, b.gamma);
    // reconstruction.h:224-296 Compute_Slope / Van_Leer_Slope
    auto slope = [&](const MPrim &l, const MPrim &r, double coef) {
      MPrim s;
      s.d  = coef * (r.d - l.d);
      s.vx = coef * (r.vx - l.vx);
      s.vy = coef * (r.vy - l.vy);
      s.vz = coef * (r.vz - l.vz);
      s.p  = coef * (r.p - l.p);
      s.bx = 0.0;
      s.by = coef * (r.by - l.by);
      s.bz = coef * (r.bz - l.bz);
#pragma unroll
      for (int k = 0; k < NS_MAX; k++) s.sc[k] = k < b.ns ? coef * (r.sc[k] - l.sc[k]) : 0.0;
      return s;
    };
    auto vl = [](double l, double r) -> double { return mpos(l, r) ? mdiv(2.0 * l * r, l + r) : 0.0; };
    MPrim const dL = slope(cimo, ci, 1.0);
    MPrim const dR = slope(ci, cipo, 1.0);
    MPrim const dC = slope(cimo, cipo, 0.5);
    MPrim dG;
    dG.d  = vl(dL.d, dR.d);
    dG.vx = vl(dL.vx, dR.vx);
    dG.vy = vl(dL.vy, dR.vy);
    dG.vz = vl(dL.vz, dR.vz);
    dG.p  = vl(dL.p, dR.p);
    dG.bx = 0.0;
    dG.by = vl(dL.by, dR.by);
    dG.bz = vl(dL.bz, dR.bz);
#pragma unroll
    for (int k = 0; k < NS_MAX; k++) dG.sc[k] = k < b.ns ? vl(dL.sc[k], dR.sc[k]) : 0.0;
    Chr const aL = prim_to_char(ci, dL, e, cs2, rd, rcs2), aR = prim_to_char(ci, dR, e, cs2, rd, rcs2),
              aC = prim_to_char(ci, dC, e, cs2, rd, rcs2), aG = prim_to_char(ci, dG, e, cs2, rd, rcs2);
    // reconstruction.h:512-559 Monotonize_Characteristic_Return_Primitive
    auto mono = [](double l, double r, double cc, double vg) -> double {
      if (mpos(l, r)) {
        double const la = 2.0 * mmin(fabs(l), fabs(r));
        double const lb = mmin(fabs(cc), fabs(vg));
        return copysign(mmin(la, lb), cc);
      }
      return 0.0;
    };
    Chr am;
#pragma unroll
    for (int k = 0; k < 7; k++) am.a[k] = mono(aL.a[k], aR.a[k], aC.a[k], aG.a[k]);
    MPrim dm = char_to_prim(ci, am, e, cs2);
#pragma unroll
    for (int k = 0; k < NS_MAX; k++) dm.sc[k] = k < b.ns ? mono(dL.sc[k], dR.sc[k], dC.sc[k], dG.sc[k]) : 0.0;
    // reconstruction.h:645-673 Calc_Interface_Linear
    auto lin = [&](double sign) {
      MPrim o;
      auto f = [&sign](double st, double sl) -> double { return st + sign * 0.5 * sl; };
      o.d  = f(ci.d, dm.d);
      o.vx = f(ci.vx, dm.vx);
      o.vy = f(ci.vy, dm.vy);
      o.vz = f(ci.vz, dm.vz);
      o.p  = f(ci.p, dm.p);
      o.bx = 0.0;
      o.by = f(ci.by, dm.by);
      o.bz = f(ci.bz, dm.bz);
#pragma unroll
      for (int k = 0; k < NS_MAX; k++) o.sc[k] = k < b.ns ? f(ci.sc[k], dm.sc[k]) : 0.0;
      return o;
    };
    MPrim L = lin(1.0);
    MPrim R = lin(-1.0);
    // reconstruction.h:686-723 Plm_Limit_Interfaces
    auto lim = [](double &l, double &r, double vm, double vi, double vp) {
      r = mmax(mmin(vi, vm), r);
      r = mmin(mmax(vi, vm), r);
      l = mmax(mmin(vi, vp), l);
      l = mmin(mmax(vi, vp), l);
    };
    lim(L.d, R.d, cimo.d, ci.d, cipo.d);
    lim(L.vx, R.vx, cimo.vx, ci.vx, cipo.vx);
    lim(L.vy, R.vy, cimo.vy, ci.vy, cipo.vy);
    lim(L.vz, R.vz, cimo.vz, ci.vz, cipo.vz);
    lim(L.p, R.p, cimo.p, ci.p, cipo.p);
    lim(L.by, R.by, cimo.by, ci.by, cipo.by);
    lim(L.bz, R.bz, cimo.bz, ci.bz, cipo.bz);
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < b.ns) lim(L.sc[k], R.sc[k], cimo.sc[k], ci.sc[k], cipo.sc[k]);
    R.d = mmax(R.d, TINY);
    L.d = mmax(L.d, TINY);
    R.p = mmax(R.p, TINY);
    L.p = mmax(L.p, TINY);
    write_data(b, L, QL, U, id, o1, o2, o3);
    write_data(b, R, QR, U, b.id(x - sx, y - sy, z - sz), o1, o2, o3);
  }
}

// ------------------------------------------------------------------------------------------
// HLLD (hlld_cuda.cu:31-508, mhd::Calculate_HLLD_Fluxes_CUDA and mhd::internal)
// ------------------------------------------------------------------------------------------
struct HState {
  double d, vx, vy, vz, E, by, bz, p, pt;
  double sc[NS_MAX];
};
struct HStar {
  double d, vy, vz, E, by, bz;
};
struct HDStar {
  double vy, vz, by, bz, EL, ER;
};
struct HFlux {
  double d, mx, my, mz, E, by, bz;
};

__device__ __forceinline__ HState hlld_load(const Box &b, const double *Q, double bx, long long t, int o1, int o2,
                                            int o3)
{
  long long const n = b.n;
  HState s;
  s.d  = Q[t];
  s.d  = mmax(s.d, TINY);
  double const rd = minv(s.d);
  s.vx = mdivr(Q[t + n * o1], s.d, rd);
  s.vy = mdivr(Q[t + n * o2], s.d, rd);
  s.vz = mdivr(Q[t + n * o3], s.d, rd);
  s.E  = Q[t + n * 4];
  s.E  = mmax(s.E, TINY);
  s.by = Q[t + n * b.fB()];
  s.bz = Q[t + n * (b.fB() + 1)];
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) s.sc[k] = k < b.ns ? mdivr(Q[t + n * (5 + k)], s.d, rd) : 0.0;
  double pressure = s.E - 0.5 * s.d * sqm(s.vx, s.vy, s.vz);
  pressure -= magE(bx, s.by, s.bz);
  s.p = mmax((b.gamma - 1.) * pressure, TINY);
  double const pt = s.p + magE(bx, s.by, s.bz);  // mhd_utilities.h computeTotalPressure
  s.pt            = mmax(pt, TINY);
  return s;
}
__device__ __forceinline__ HFlux hlld_nonstar(const HState &s, double bx)
{
  HFlux f;
  f.d  = s.d * s.vx;
  f.mx = f.d * s.vx + s.pt - bx * bx;
  f.my = f.d * s.vy - bx * s.by;
  f.mz = f.d * s.vz - bx * s.bz;
  f.by = s.by * s.vx - bx * s.vy;
  f.bz = s.bz * s.vx - bx * s.vz;
  f.E  = s.vx * (s.E + s.pt) - bx * (s.vx * bx + ((s.vy * s.by) + (s.vz * s.bz)));
  return f;
}
__device__ __forceinline__ HStar hlld_star(const HState &s, double SM, double S, double bx, double ptStar)
{
  HStar st;
  double const rsm = minv(S - SM);
  st.d = mdivr(s.d * (S - s.vx), S - SM, rsm);
  if (fabs(s.d * (S - s.vx) * (S - SM) - (bx * bx)) < ptStar * HLLD_SMALL) {
    st.vy = s.vy;
    st.vz = s.vz;
    st.by = s.by;
    st.bz = s.bz;
  } else {
    double const denom = s.d * (S - s.vx) * (S - SM) - (bx * bx);
    double const rden  = minv(denom);
    double coef        = mdivr(bx * (SM - s.vx), denom, rden);
    st.vy              = s.vy - s.by * coef;
    st.vz              = s.vz - s.bz * coef;
    double tp          = (S - s.vx);
    tp                 = tp * tp;
    coef               = mdivr(s.d * tp - (bx * bx), denom, rden);
    st.by              = s.by * coef;
    st.bz              = s.bz * coef;
  }
  st.E = mdivr(s.E * (S - s.vx) - s.pt * s.vx + ptStar * SM +
                   bx * (dot3(s.vx, s.vy, s.vz, bx, s.by, s.bz) - dot3(SM, st.vy, st.vz, bx, st.by, st.bz)),
               S - SM, rsm);
  return st;
}
__device__ __forceinline__ HFlux hlld_starflux(const HStar &st, const HState &s, const HFlux &f, double SM, double S)
{
  HFlux o;
  o.d  = f.d + S * (st.d - s.d);
  o.mx = f.mx + S * (st.d * SM - s.d * s.vx);
  o.my = f.my + S * (st.d * st.vy - s.d * s.vy);
  o.mz = f.mz + S * (st.d * st.vz - s.d * s.vz);
  o.E  = f.E + S * (st.E - s.E);
  o.by = f.by + S * (st.by - s.by);
  o.bz = f.bz + S * (st.bz - s.bz);
  return o;
}
__device__ __forceinline__ HDStar hlld_dstar(const HStar &L, const HStar &R, double bx, double ptStar, double SM)
{
  HDStar o;
  o.EL = 0.0, o.ER = 0.0;
  if (0.5 * (bx * bx) < HLLD_SMALL * ptStar) {
    if (SM >= 0.0) {
      o.vy = L.vy, o.vz = L.vz, o.by = L.by, o.bz = L.bz, o.EL = L.E;
    } else {
      o.vy = R.vy, o.vz = R.vz, o.by = R.by, o.bz = R.bz, o.ER = R.E;
    }
  } else {
    double const sqrtDL = msqrt(L.d), sqrtDR = msqrt(R.d);
    double const inv    = mdiv(1.0, sqrtDL + sqrtDR);
    double const sgnb   = copysign(1.0, bx);
    o.vy = inv * (sqrtDL * L.vy + sqrtDR * R.vy + sgnb * (R.by - L.by));
    o.vz = inv * (sqrtDL * L.vz + sqrtDR * R.vz + sgnb * (R.bz - L.bz));
    o.by = inv * (sqrtDL * R.by + sqrtDR * L.by + sgnb * (sqrtDL * sqrtDR) * (R.vy - L.vy));
    o.bz = inv * (sqrtDL * R.bz + sqrtDR * L.bz + sgnb * (sqrtDL * sqrtDR) * (R.vz - L.vz));
    double const vdb = dot3(SM, o.vy, o.vz, bx, o.by, o.bz);
    o.EL = L.E - sqrtDL * sgnb * (dot3(SM, L.vy, L.vz, bx, L.by, L.bz) - vdb);
    o.ER = R.E + sqrtDR * sgnb * (dot3(SM, R.vy, R.vz, bx, R.by, R.bz) - vdb);
  }
  return o;
}
__device__ __forceinline__ HFlux hlld_dstarflux(const HDStar &ds, double dsE, const HStar &st, const HState &s,
                                                const HFlux &f, double SM, double S, double SStar)
{
  HFlux o;
  double const sd = SStar - S;
  o.d  = f.d - S * s.d - sd * st.d + SStar * st.d;
  o.mx = f.mx - S * (s.d * s.vx) - sd * (st.d * SM) + SStar * (st.d * SM);
  o.my = f.my - S * (s.d * s.vy) - sd * (st.d * st.vy) + SStar * (st.d * ds.vy);
  o.mz = f.mz - S * (s.d * s.vz) - sd * (st.d * st.vz) + SStar * (st.d * ds.vz);
  o.E  = f.E - S * s.E - sd * st.E + SStar * dsE;
  o.by = f.by - S * s.by - sd * st.by + SStar * ds.by;
  o.bz = f.bz - S * s.bz - sd * st.bz + SStar * ds.bz;
  return o;
}

__global__ void k_hlld(Box b, const double *__restrict__ QL, const double *__restrict__ QR,
                       const double *__restrict__ Bface, double *__restrict__ F, int dir)
{
  long long const n = b.n;
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  CGB_CELLS(t)
  {
    double const bx = Bface[t];
    HState const sL = hlld_load(b, QL, bx, t, o1, o2, o3);
    HState const sR = hlld_load(b, QR, bx, t, o1, o2, o3);
    auto ret = [&](const HFlux &f, const HState &s) {
      F[t]                    = f.d;
      F[t + n * o1]           = f.mx;
      F[t + n * o2]           = f.my;
      F[t + n * o3]           = f.mz;
      F[t + n * 4]            = f.E;
      F[t + n * b.fB()]       = f.by;
      F[t + n * (b.fB() + 1)] = f.bz;
      for (int k = 0; k < b.ns; k++) F[t + n * (5 + k)] = s.sc[k] * f.d;
    };
    double const cL = cfast(sL.d, sL.p, bx, sL.by, sL.bz, b.gamma);
    double const cR = cfast(sR.d, sR.p, bx, sR.by, sR.bz, b.gamma);
    double const cmax = mmax(cL, cR);
    double const SL = mmin(sL.vx, sR.vx) - cmax;
    double const SR = mmax(sL.vx, sR.vx) + cmax;
    HFlux const fL = hlld_nonstar(sL, bx);
    if (mgt0(SL)) {
      ret(fL, sL);
      continue;
    }
    HFlux const fR = hlld_nonstar(sR, bx);
    if (mlt0(SR)) {
      ret(fR, sR);
      continue;
    }
    double SM;
    {
      double const rd = SR - sR.vx, ld = SL - sL.vx;
      SM = mdiv(rd * sR.d * sR.vx - ld * sL.d * sL.vx - sR.pt + sL.pt, rd * sR.d - ld * sL.d);
    }
    double const ptStar = mdiv(sR.d * sL.pt * (SR - sR.vx) - sL.d * sR.pt * (SL - sL.vx) +
                                   sL.d * sR.d * (SR - sR.vx) * (SL - sL.vx) * (sR.vx - sL.vx),
                               sR.d * (SR - sR.vx) - sL.d * (SL - sL.vx));
    HStar const stL = hlld_star(sL, SM, SL, bx, ptStar);
    double const SLStar = SM + -1 * mdiv(fabs(bx), msqrt(mmax(stL.d, TINY)));
    if (SLStar > 0.0 and SL <= 0.0) {
      ret(hlld_starflux(stL, sL, fL, SM, SL), sL);
      continue;
    }
    HStar const stR = hlld_star(sR, SM, SR, bx, ptStar);
    double const SRStar = SM + 1 * mdiv(fabs(bx), msqrt(mmax(stR.d, TINY)));
    if (SRStar <= 0.0 and SR >= 0.0) {
      ret(hlld_starflux(stR, sR, fR, SM, SR), sR);
      continue;
    }
    HDStar const ds = hlld_dstar(stL, stR, bx, ptStar, SM);
    if (SM > 0.0 and SLStar <= 0.0) {
      ret(hlld_dstarflux(ds, ds.EL, stL, sL, fL, SM, SL, SLStar), sL);
      continue;
    }
    if (SRStar > 0.0 and SM <= 0.0) {
      ret(hlld_dstarflux(ds, ds.ER, stR, sR, fR, SM, SR, SRStar), sR);
      continue;
    }
  }
}

// ------------------------------------------------------------------------------------------
// constrained transport
// ------------------------------------------------------------------------------------------
// The cell-centred electric field that _ctSlope (ct_electric_fields.h:66-118) subtracts from a face
// flux: at cell i for CT direction d, (M3 B2c - M2 B3c) / density with (m1, m2) = (d + 1, d + 2)
// mod 3 and B2c, B3c the cell's face fields averaged with the faces below it.  It depends on the
// cell and d alone, and each cell's three values feed 24 slope evaluations of its neighbours' edges,
// so k_ct_centred forms them once per cell (the same operations, so the same bits) into ec[d][i].
// Cells whose lower neighbour along m1 or m2 lies before the array's first element get 0: only
// edges of the outermost ghost layer would read them.
__global__ void k_ct_centred(Box b, const double *__restrict__ U, double *__restrict__ ec)
{
  long long const n = b.n;
  int const fB      = b.fB();
  CGB_CELLS(t)
  {
    double const density = U[t];
#pragma unroll
    for (int d = 0; d < 3; d++) {
      int const m1 = (d + 1) % 3, m2 = (d + 2) % 3;
      long long const s1 = m1 == 0 ? 1 : m1 == 1 ? (long long)b.nx : (long long)b.nx * b.ny;
      long long const s2 = m2 == 0 ? 1 : m2 == 1 ? (long long)b.nx : (long long)b.nx * b.ny;
      if (t < s1 || t < s2) {
        ec[d * n + t] = 0.0;
        continue;
      }
      double const M2  = U[t + (long long)(m1 + 1) * n];
      double const M3  = U[t + (long long)(m2 + 1) * n];
      double const B2c = 0.5 * (U[t + (long long)(m1 + fB) * n] + U[t - s1 + (long long)(m1 + fB) * n]);
      double const B3c = 0.5 * (U[t + (long long)(m2 + fB) * n] + U[t - s2 + (long long)(m2 + fB) * n]);
      ec[d * n + t]    = mdiv(M3 * B2c - M2 * B3c, density);
    }
  }
}

// ct_electric_fields.h:66-118 _ctSlope, with the cell-centred field read from ec
__device__ __forceinline__ double ct_slope(const Box &b, const double *flux, const double *ec, double fluxSign,
                                           int ctDir, int cq1, int cq2, int fq1, int fq2, int x, int y, int z)
{
  long long const n = b.n;
  int const xc = x - int(cq1 == 0) - int(cq2 == 0);
  int const yc = y - int(cq1 == 1) - int(cq2 == 1);
  int const zc = z - int(cq1 == 2) - int(cq2 == 2);
  long long const ic    = b.id(xc, yc, zc);
  long long const iflux = b.id(x - int(fq1 == 0) - int(fq2 == 0), y - int(fq1 == 1) - int(fq2 == 1),
                               z - int(fq1 == 2) - int(fq2 == 2));
  int const fB    = b.fB();
  double const ef = fluxSign * flux[iflux + (long long)(int(fluxSign == 1) + fB) * n];
  return ef - ec[(long long)ctDir * n + ic];
}

// ct_electric_fields.cu:20-279 Calculate_CT_Electric_Fields
__global__ void k_ct(Box b, const double *__restrict__ Fx, const double *__restrict__ Fy,
                     const double *__restrict__ Fz, const double *__restrict__ ec, double *__restrict__ emf)
{
  long long const n = b.n;
  int const fB      = b.fB();
  // flux field positions of the magnetic fluxes (grid_enum.h:95-100)
  int const fxBz = fB, fxBy = fB + 1, fyBx = fB, fyBz = fB + 1, fzBy = fB, fzBx = fB + 1;
  CGB_CELLS(t)
  {
    int x, y, z;
    xyz(b, t, x, y, z);
    if (!(x > 0 and y > 0 and z > 0 and x < b.nx and y < b.ny and z < b.nz)) continue;
    // the upwind slope: only the side the mass flux selects is evaluated (both when it is zero)
    auto S = [&](const double *fl, double sg, int cd, int a, int c, int cc, int d) {
      return [=, &b] { return ct_slope(b, fl, ec, sg, cd, a, c, cc, d, x, y, z); };
    };
    auto pick = [](double sgnUp, auto pos, auto neg) {
      if (mgt0(sgnUp)) return pos();
      if (mlt0(sgnUp)) return neg();
      return 0.5 * (pos() + neg());
    };
    double syp, syn, szp, szn, sxp, sxn, fyp, fyn, fzp, fzn, fxp, fxn;
    // X electric field
    syp = pick(Fz[b.id(x, y, z - 1)], S(Fy, -1, 0, 2, -1, 1, 2), S(Fy, -1, 0, -1, -1, 1, -1));
    syn = pick(Fz[b.id(x, y - 1, z - 1)], S(Fy, -1, 0, 1, 2, 1, 2), S(Fy, -1, 0, 1, -1, 1, -1));
    szp = pick(Fy[b.id(x, y - 1, z)], S(Fz, 1, 0, 1, -1, 1, 2), S(Fz, 1, 0, -1, -1, 2, -1));
    szn = pick(Fy[b.id(x, y - 1, z - 1)], S(Fz, 1, 0, 1, 2, 1, 2), S(Fz, 1, 0, 2, -1, -1, 2));
    fyp = +Fz[b.id(x, y, z - 1) + (long long)fzBx * n];
    fyn = +Fz[b.id(x, y - 1, z - 1) + (long long)fzBx * n];
    fzp = -Fy[b.id(x, y - 1, z) + (long long)fyBx * n];
    fzn = -Fy[b.id(x, y - 1, z - 1) + (long long)fyBx * n];
    emf[t + 0 * n] = 0.25 * (+fyp + fyn + fzp + fzn + syp + syn + szp + szn);
    // Y electric field
    sxp = pick(Fz[b.id(x, y, z - 1)], S(Fx, 1, 1, 2, -1, 0, 2), S(Fx, 1, 1, -1, -1, 0, -1));
    sxn = pick(Fz[b.id(x - 1, y, z - 1)], S(Fx, 1, 1, 0, 2, 0, 2), S(Fx, 1, 1, 0, -1, 0, -1));
    szp = pick(Fx[b.id(x - 1, y, z)], S(Fz, -1, 1, 0, -1, 0, 2), S(Fz, -1, 1, -1, -1, 2, -1));
    szn = pick(Fx[b.id(x - 1, y, z - 1)], S(Fz, -1, 1, 0, 2, 0, 2), S(Fz, -1, 1, 2, -1, 2, -1));
    fxp = -Fz[b.id(x, y, z - 1) + (long long)fzBy * n];
    fxn = -Fz[b.id(x - 1, y, z - 1) + (long long)fzBy * n];
    fzp = +Fx[b.id(x - 1, y, z) + (long long)fxBy * n];
    fzn = +Fx[b.id(x - 1, y, z - 1) + (long long)fxBy * n];
    emf[t + 1 * n] = 0.25 * (+fxp + fxn + fzp + fzn + sxp + sxn + szp + szn);
    // Z electric field
    syp = pick(Fx[b.id(x - 1, y, z)], S(Fy, 1, 2, 0, -1, 0, 1), S(Fy, 1, 2, -1, -1, 1, -1));
    syn = pick(Fx[b.id(x - 1, y - 1, z)], S(Fy, 1, 2, 0, 1, 0, 1), S(Fy, 1, 2, 1, -1, 1, -1));
    sxp = pick(Fy[b.id(x, y - 1, z)], S(Fx, -1, 2, 1, -1, 0, 1), S(Fx, -1, 2, -1, -1, 0, -1));
    sxn = pick(Fy[b.id(x - 1, y - 1, z)], S(Fx, -1, 2, 0, 1, 0, 1), S(Fx, -1, 2, 0, -1, 0, -1));
    fxp = +Fy[b.id(x, y - 1, z) + (long long)fyBz * n];
    fxn = +Fy[b.id(x - 1, y - 1, z) + (long long)fyBz * n];
    fyp = -Fx[b.id(x - 1, y, z) + (long long)fxBz * n];
    fyn = -Fx[b.id(x - 1, y - 1, z) + (long long)fxBz * n];
    emf[t + 2 * n] = 0.25 * (+fxp + fxn + fyp + fyn + sxp + sxn + syp + syn);
  }
}

// magnetic_update.cu:21-81 Update_Magnetic_Field_3D
__global__ void k_bupdate(Box b, const double *src, double *dst, const double *__restrict__ emf, double dt,
                          const double *__restrict__ dtp, double scale)
{
  long long const n = b.n;
  dt                 = (dtp ? *dtp : dt) * scale;
  double const dtodx = dt / b.dx, dtody = dt / b.dy, dtodz = dt / b.dz;
  CGB_CELLS(t)
  {
    int x, y, z;
    xyz(b, t, x, y, z);
    if (!(x > 0 and y > 0 and z > 0 and x < b.nx - 1 and y < b.ny - 1 and z < b.nz - 1)) continue;
    double const ex1 = emf[b.id(x, y + 1, z) + 0 * n], ex2 = emf[b.id(x, y, z + 1) + 0 * n],
                 ex3 = emf[b.id(x, y + 1, z + 1) + 0 * n];
    double const ey1 = emf[b.id(x + 1, y, z) + 1 * n], ey2 = emf[b.id(x, y, z + 1) + 1 * n],
                 ey3 = emf[b.id(x + 1, y, z + 1) + 1 * n];
    double const ez1 = emf[b.id(x + 1, y, z) + 2 * n], ez2 = emf[b.id(x, y + 1, z) + 2 * n],
                 ez3 = emf[b.id(x + 1, y + 1, z) + 2 * n];
    long long const bx = t + (long long)b.fB() * n, by = bx + n, bz = by + n;
    dst[bx] = src[bx] + dtodz * (ey3 - ey1) + dtody * (ez1 - ez3);
    dst[by] = src[by] + dtodx * (ez3 - ez2) + dtodz * (ex1 - ex3);
    dst[bz] = src[bz] + dtody * (ex3 - ex2) + dtodx * (ey2 - ey3);
  }
}

// ------------------------------------------------------------------------------------------
// conserved updates
// ------------------------------------------------------------------------------------------
// VL_3D_cuda.cu:379-495 Update_Conserved_Variables_3D_half (MHD: hydro fields and scalars)
__global__ void k_update_half(Box b, const double *__restrict__ U, double *__restrict__ Uh,
                              const double *__restrict__ Fx, const double *__restrict__ Fy,
                              const double *__restrict__ Fz, double dt, const double *__restrict__ dtp, double scale)
{
  long long const n = b.n;
  dt                 = (dtp ? *dtp : dt) * scale;
  double const dtodx = dt / b.dx, dtody = dt / b.dy, dtodz = dt / b.dz;
  double const floor = b.density_floor;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    if (!(x > 0 && x < b.nx - 1 && y > 0 && y < b.ny - 1 && z > 0 && z < b.nz - 1)) continue;
    long long const imo = b.id(x - 1, y, z), jmo = b.id(x, y - 1, z), kmo = b.id(x, y, z - 1);
    auto upd = [&](int f) {
      long long const o = (long long)f * n;
      return U[o + id] + dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]) +
             dtodz * (Fz[o + kmo] - Fz[o + id]);
    };
    for (int f = 0; f < 5; f++) Uh[(long long)f * n + id] = upd(f);
    for (int s = 0; s < b.ns; s++) Uh[(long long)(5 + s) * n + id] = upd(5 + s);
    if (b.floor_on) {
      if (Uh[id] < floor) {
        double const dens_0 = Uh[id];
        Uh[id]              = floor;
        Uh[1 * n + id] *= (floor / dens_0);
        Uh[2 * n + id] *= (floor / dens_0);
        Uh[3 * n + id] *= (floor / dens_0);
        Uh[4 * n + id] *= (floor / dens_0);
      }
    }
  }
}

// hydro_cuda.cu:172-402 Update_Conserved_Variables_3D (MHD: hydro fields and scalars; B by CT)
__global__ void k_update_full(Box b, double *__restrict__ U, const double *__restrict__ Fx,
                              const double *__restrict__ Fy, const double *__restrict__ Fz, double dt,
                              const double *__restrict__ dtp)
{
  long long const n = b.n;
  int const ng      = b.ng;
  if (dtp) dt = *dtp;
  double const dtodx = dt / b.dx, dtody = dt / b.dy, dtodz = dt / b.dz;
  double const floor = b.density_floor;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    if (!(x > ng - 1 && x < b.nx - ng && y > ng - 1 && y < b.ny - ng && z > ng - 1 && z < b.nz - ng)) continue;
    long long const imo = b.id(x - 1, y, z), jmo = b.id(x, y - 1, z), kmo = b.id(x, y, z - 1);
    auto upd = [&](int f) {
      long long const o = (long long)f * n;
      U[o + id] += dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]) +
                   dtodz * (Fz[o + kmo] - Fz[o + id]);
    };
    for (int f = 0; f < 5; f++) upd(f);
    for (int s = 0; s < b.ns; s++) upd(5 + s);
    if (b.floor_on && U[id] < floor && U[id] > 0) {
      double const dens_0 = U[id];
      U[id]               = floor;
      U[1 * n + id] *= (floor / dens_0);
      U[2 * n + id] *= (floor / dens_0);
      U[3 * n + id] *= (floor / dens_0);
      U[4 * n + id] *= (floor / dens_0);
    }
  }
}

// hydro_cuda.cu:437-471 Calc_dt_3D (MHD branch): max over real cells of (|v| + c_fast)/dx
__global__ void k_calc_dt(Box b, const double *__restrict__ U, unsigned long long *__restrict__ dti)
{
  long long const n = b.n;
  int const ng      = b.ng;
  __shared__ double red[32];
  double m = -1.0;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    if (!(x > ng - 1 && x < b.nx - ng && y > ng - 1 && y < b.ny - ng && z > ng - 1 && z < b.nz - ng)) continue;
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E = U[4 * n + id];
    double bx, by, bz;
    cc_b(b, U, x, y, z, bx, by, bz);
    double pressure = E - 0.5 * d * sqm(vx, vy, vz);
    pressure -= magE(bx, by, bz);
    double const gasP = fmax((b.gamma - 1.) * pressure, TINY);
    double const cf   = cfast(d, gasP, bx, by, bz, b.gamma);
    double cm         = fmax((fabs(vx) + cf) / b.dx, (fabs(vy) + cf) / b.dy);
    cm                = fmax(cm, (fabs(vz) + cf) / b.dz);
    cm                = fmax(cm, 0.0);
    m                 = fmax(m, cm);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = m;
  __syncthreads();
  if (warp == 0) {
    m = (lane < (int)((blockDim.x + 31) >> 5)) ? red[lane] : -1.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0 && m >= 0.0) atomicMax(dti, (unsigned long long)__double_as_longlong(m));
  }
}

// magnetic_divergence.cu:33-76 calculateMagneticDivergence: max |div B| over the real cells
__global__ void k_max_divb(Box b, const double *__restrict__ U, unsigned long long *__restrict__ out)
{
  long long const n = b.n;
  __shared__ double red[32];
  double m = 0.0;
  CGB_CELLS(id)
  {
    int x, y, z;
    xyz(b, id, x, y, z);
    // the reference's thread guard: every cell from index 2 up, the upper ghost layers included
    if (!(x > 1 && y > 1 && z > 1)) continue;
    long long const fB = b.fB();
    double const div = fabs((U[fB * n + id] - U[fB * n + b.id(x - 1, y, z)]) / b.dx +
                            (U[(fB + 1) * n + id] - U[(fB + 1) * n + b.id(x, y - 1, z)]) / b.dy +
                            (U[(fB + 2) * n + id] - U[(fB + 2) * n + b.id(x, y, z - 1)]) / b.dz);
    m = fmax(m, div);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  int const lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  if (lane == 0) red[warp] = m;
  __syncthreads();
  if (warp == 0) {
    m = (lane < (int)((blockDim.x + 31) >> 5)) ? red[lane] : 0.0;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
    if (lane == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
  }
}

#undef CGB_CELLS

unsigned grid_for(long long n)
{
  long long blocks = (n + 255) / 256;
  if (blocks > 152LL * 32) blocks = 152LL * 32;
  return (unsigned)blocks;
}

}  // namespace CGB_MHD_NS

#if CGB_MHD_REDUCTIONS
size_t mhd_scratch_doubles(const Box &b) { return mhd_scratch_fields(b.nf) * (size_t)b.n; }
#endif

cudaError_t CGB_MHD_STEP(const Box &b, int recon, double *U, double *scratch, double dt, const double *dt_dev,
                         cudaStream_t s)
{
  using namespace CGB_MHD_NS;
  size_t const n = (size_t)b.n, nif = (size_t)(b.nf - 1) * n;
  double *Uh = scratch, *QLx = Uh + (size_t)b.nf * n, *QRx = QLx + nif, *QLy = QRx + nif, *QRy = QLy + nif,
         *QLz = QRy + nif, *QRz = QLz + nif, *Fx = QRz + nif, *Fy = Fx + nif, *Fz = Fy + nif, *emf = Fz + nif,
         *ec = emf + 3 * n;
  unsigned const g = grid_for(b.n);
  long long const fB = b.fB();
  auto face = [&](const double *src, int d) { return src + (fB + d) * (long long)n; };
  auto riemann = [&](const double *Ub) {
    k_hlld<<<g, 256, 0, s>>>(b, QLx, QRx, face(Ub, 0), Fx, 0);
    k_hlld<<<g, 256, 0, s>>>(b, QLy, QRy, face(Ub, 1), Fy, 1);
    k_hlld<<<g, 256, 0, s>>>(b, QLz, QRz, face(Ub, 2), Fz, 2);
  };
  // predictor: PCM, HLLD, CT, half updates with 0.5 dt
  k_pcm<<<g, 256, 0, s>>>(b, U, QLx, QRx, QLy, QRy, QLz, QRz);
  riemann(U);
  k_ct_centred<<<g, 256, 0, s>>>(b, U, ec);
  k_ct<<<g, 256, 0, s>>>(b, Fx, Fy, Fz, ec, emf);
  // the half step uses dt * 0.5 on the device (the same product as 0.5 * dt on the host)
  k_update_half<<<g, 256, 0, s>>>(b, U, Uh, Fx, Fy, Fz, dt, dt_dev, 0.5);
  k_bupdate<<<g, 256, 0, s>>>(b, U, Uh, emf, dt, dt_dev, 0.5);
  // corrector: reconstruction of U½, HLLD, CT, full updates with dt
  if (recon == RECON_PPMC) {
    for (int d = 0; d < 3; d++)
      k_ppmc<<<g, 256, 0, s>>>(b, Uh, d == 0 ? QLx : d == 1 ? QLy : QLz, d == 0 ? QRx : d == 1 ? QRy : QRz, d);
  } else if (recon == RECON_PLMC) {
    for (int d = 0; d < 3; d++)
      k_plmc<<<g, 256, 0, s>>>(b, Uh, d == 0 ? QLx : d == 1 ? QLy : QLz, d == 0 ? QRx : d == 1 ? QRy : QRz, d);
  } else {
    k_pcm<<<g, 256, 0, s>>>(b, Uh, QLx, QRx, QLy, QRy, QLz, QRz);
  }
  riemann(Uh);
  k_ct_centred<<<g, 256, 0, s>>>(b, Uh, ec);
  k_ct<<<g, 256, 0, s>>>(b, Fx, Fy, Fz, ec, emf);
  k_update_full<<<g, 256, 0, s>>>(b, U, Fx, Fy, Fz, dt, dt_dev);
  k_bupdate<<<g, 256, 0, s>>>(b, U, U, emf, dt, dt_dev, 1.0);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  if (b.floor_on) return negative_density_average(b, U, s);
  return cudaSuccess;
}

#if CGB_MHD_REDUCTIONS
cudaError_t mhd_calc_dt(const Box &b, const double *U, unsigned long long *dti, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(dti, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  CGB_MHD_NS::k_calc_dt<<<CGB_MHD_NS::grid_for(b.n), 256, 0, s>>>(b, U, dti);
  return cudaGetLastError();
}

cudaError_t mhd_max_divb(const Box &b, const double *U, unsigned long long *out, cudaStream_t s)
{
  cudaError_t e = cudaMemsetAsync(out, 0, sizeof(unsigned long long), s);
  if (e != cudaSuccess) return e;
  CGB_MHD_NS::k_max_divb<<<CGB_MHD_NS::grid_for(b.n), 256, 0, s>>>(b, U, out);
  return cudaGetLastError();
}
#endif

}  // namespace cgb
