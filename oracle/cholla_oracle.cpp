/*
 * cholla_oracle.cpp -- FP64 CPU restatement of Cholla's VL hydro/MHD step.
 *
 * TEST INFRASTRUCTURE ONLY (parity checker and CPU baseline); see cholla_oracle.h.
 * Compiled with -O2 -ffp-contract=off so that no multiply-add is fused, matching the
 * reference's -fmad=false build (Makefile:148).  Every arithmetic expression keeps the
 * reference's evaluation order: that is what makes the oracle reproduce the reference
 * to the last bit, so the order is part of the specification being restated.
 *
 * Paths below are relative to the cholla-hydro/cholla source tree.
 */
#include "cholla_oracle.h"

#include <cfloat>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>
#ifdef _OPENMP
  #include <omp.h>
#endif

namespace
{
// src/global/global.h:25, 62-73
constexpr double TINY  = 1.0e-20;
constexpr double ETA_1 = 0.001;
constexpr double ETA_2 = 0.035;
// src/riemann_solvers/hlld_cuda.h:56
constexpr double HLLD_SMALL = 1.0e-8;
constexpr int MAXS          = 8;

int g_threads = 0;

inline double SIGN(double a) { return (a < 0.) ? -1. : 1.; }  // global.h:144
inline int sgn_int(double x) { return (x < 0) ? -1 : 1; }     // global_cuda.h:41-48

// math_utilities.h: dotProduct = a1*b1 + ((a2*b2) + (a3*b3))
inline double dot3(double a1, double a2, double a3, double b1, double b2, double b3)
{
  return a1 * b1 + ((a2 * b2) + (a3 * b3));
}
inline double sqmag(double a, double b, double c) { return dot3(a, b, c, a, b, c); }

// hydro_utilities.h:136-151
inline double pressure_from_de(double E, double U_total, double U_advected, double gamma)
{
  double U;
  if (U_total / E > ETA_1) {
    U = U_total;
  } else {
    U = U_advected;
  }
  double P = U * (gamma - 1.0);
  return fmax(P, TINY);
}

// Geometry and field bookkeeping for one padded grid.
struct Grid {
  int nx, ny, nz;
  size_t n;  // n_cells
  int ng, nf, ns;
  bool de, mhd;
  int fB;    // index of magnetic_x (mhd)
  int fGE;   // index of GasEnergy (de)
  int nif;   // number of fields in interface / flux arrays
  double gamma;
  explicit Grid(const orc_config *c)
  {
    nx    = c->nx;
    ny    = c->ny;
    nz    = c->nz;
    n     = (size_t)nx * ny * nz;
    ng    = c->n_ghost;
    nf    = c->n_fields;
    ns    = c->n_scalars;
    de    = c->de != 0;
    mhd   = c->mhd != 0;
    fB    = 5 + ns;
    fGE   = nf - 1;
    nif   = mhd ? nf - 1 : nf;
    gamma = c->gamma;
  }
  size_t id(int x, int y, int z) const { return (size_t)x + (size_t)y * nx + (size_t)z * nx * ny; }
  void xyz(size_t i, int &x, int &y, int &z) const
  {
    z = (int)(i / ((size_t)nx * ny));
    y = (int)((i - (size_t)z * nx * ny) / nx);
    x = (int)(i - (size_t)z * nx * ny - (size_t)y * nx);
  }
};

inline void perm(int dir, int &o1, int &o2, int &o3)
{
  if (dir == 0) {
    o1 = 1, o2 = 2, o3 = 3;
  } else if (dir == 1) {
    o1 = 2, o2 = 3, o3 = 1;
  } else {
    o1 = 3, o2 = 1, o3 = 2;
  }
}

// mhd_utilities.h:205-237 cellCenteredMagneticFields
inline void cc_b_strided(const double *U, size_t n_cells, int nx, int ny, int fB, size_t id, int x, int y, int z,
                         double &bx, double &by, double &bz)
{
  const double *Bx = U + (size_t)fB * n_cells, *By = U + (size_t)(fB + 1) * n_cells, *Bz = U + (size_t)(fB + 2) * n_cells;
  bx = (x > 0) ? 0.5 * (Bx[id] + Bx[id - 1]) : Bx[id];
  by = (y > 0) ? 0.5 * (By[id] + By[id - (size_t)nx]) : By[id];
  bz = (z > 0) ? 0.5 * (Bz[id] + Bz[id - (size_t)nx * ny]) : Bz[id];
}
inline void cc_b(const Grid &g, const double *U, int x, int y, int z, double &bx, double &by, double &bz)
{
  cc_b_strided(U, g.n, g.nx, g.ny, g.fB, g.id(x, y, z), x, y, z, bx, by, bz);
}

// mhd_utilities.h:38-59 _magnetosonicSpeed
inline double magnetosonic(double d, double p, double bx, double by, double bz, double gamma, double choice)
{
  double bXSquared = bx * bx;
  double bSquared  = bXSquared + ((by * by) + (bz * bz));
  double term1     = gamma * p + bSquared;
  double term2     = (term1 * term1) - 4. * gamma * p * bXSquared;
  term2            = sqrt(term2);
  return sqrt((term1 + choice * term2) / (2.0 * fmax(d, TINY)));
}
inline double cfast(double d, double p, double bx, double by, double bz, double gamma)
{
  return magnetosonic(d, p, bx, by, bz, gamma, 1.0);
}
inline double cslow(double d, double p, double bx, double by, double bz, double gamma)
{
  return magnetosonic(d, p, bx, by, bz, gamma, -1.0);
}
inline double magE(double bx, double by, double bz) { return 0.5 * sqmag(bx, by, bz); }  // mhd_utilities.h:84
// hydro_utilities.h:162-166 Calc_Kinetic_Energy_From_Velocity
inline double kinetic_energy(double d, double vx, double vy, double vz) { return 0.5 * d * sqmag(vx, vy, vz); }
// hydro_utilities.h:34-45 Calc_Pressure_Primitive: gas pressure from total energy, floored at TINY
inline double pressure_primitive(double E, double d, double vx, double vy, double vz, double gamma, bool mhd,
                                 double bx, double by, double bz)
{
  double pressure = E - kinetic_energy(d, vx, vy, vz);
  if (mhd) pressure -= magE(bx, by, bz);
  return fmax((gamma - 1.) * pressure, TINY);
}
// hydro_utilities.h:106-118 Calc_Energy_Primitive: total energy from a (floored) pressure
inline double energy_primitive(double P, double d, double vx, double vy, double vz, double gamma, bool mhd,
                               double bx, double by, double bz)
{
  double energy = (fmax(P, TINY) / (gamma - 1.)) + kinetic_energy(d, vx, vy, vz);
  if (mhd) energy += magE(bx, by, bz);
  return energy;
}
// mhd_utilities.h:117-124 computeTotalPressure: gas plus magnetic pressure, floored at TINY
inline double total_pressure(double p, double bx, double by, double bz) { return fmax(p + magE(bx, by, bz), TINY); }
// mhd_utilities.h:176-180 alfvenSpeed
inline double alfven_speed(double bx, double d) { return fabs(bx) / sqrt(fmax(d, TINY)); }

// ============================================================================================
// Reconstruction (src/reconstruction/reconstruction.h)
// ============================================================================================
struct Prim {
  double d, vx, vy, vz, p, bx, by, bz, ge;
  double sc[MAXS];
};
struct Chr {
  double a[7];
};
struct Eig {
  double cf, cs, cf2, cs2, af, as, by, bz, nfs, sign, qf, qs, Af, As, qpf, qps, Apf, Aps;
};

// reconstruction.h:139-212 Load_Data
Prim load_data(const Grid &g, const double *U, int x, int y, int z, int o1, int o2, int o3)
{
  size_t const id = g.id(x, y, z);
  size_t const n  = g.n;
  Prim P;
  P.d  = U[id];
  P.vx = U[o1 * n + id] / P.d;
  P.vy = U[o2 * n + id] / P.d;
  P.vz = U[o3 * n + id] / P.d;
  double cbx = 0, cby = 0, cbz = 0;
  P.bx = P.by = P.bz = 0;
  if (g.mhd) {
    cc_b(g, U, x, y, z, cbx, cby, cbz);
    if (o1 == 1) {
      P.bx = cbx, P.by = cby, P.bz = cbz;
    } else if (o1 == 2) {
      P.bx = cby, P.by = cbz, P.bz = cbx;
    } else {
      P.bx = cbz, P.by = cbx, P.bz = cby;
    }
  }
  P.ge = 0;
  if (g.de) {
    double const E  = U[4 * n + id];
    double const GE = U[(size_t)g.fGE * n + id];
    double Ent      = 0.5 * P.d * sqmag(P.vx, P.vy, P.vz);
    if (g.mhd) Ent += magE(cbx, cby, cbz);
    P.p  = pressure_from_de(E, E - Ent, GE, g.gamma);
    P.ge = GE / P.d;
  } else {
    // hydro_utilities.h:34-45 Calc_Pressure_Primitive
    P.p = pressure_primitive(U[4 * n + id], P.d, P.vx, P.vy, P.vz, g.gamma, g.mhd, P.bx, P.by, P.bz);
  }
  for (int s = 0; s < g.ns; s++) P.sc[s] = U[(size_t)(5 + s) * n + id] / P.d;
  return P;
}

// reconstruction.h:310-361 Compute_Eigenvectors (MHD)
Eig eigenvectors(const Prim &p, double cs, double cs2, double gamma)
{
  Eig e;
  e.cf  = cfast(p.d, p.p, p.bx, p.by, p.bz, gamma);
  e.cs  = cslow(p.d, p.p, p.bx, p.by, p.bz, gamma);
  e.cf2 = e.cf * e.cf;
  e.cs2 = e.cs * e.cs;
  double const denom = (e.cf2 - e.cs2), num2 = (e.cf2 - cs2);
  if (denom <= 0.0 or num2 <= 0.0) {
    e.af = 1.0;
    e.as = 0.0;
  } else if (double const num1 = (cs2 - e.cs2); num1 <= 0.0) {
    e.af = 0.0;
    e.as = 1.0;
  } else {
    e.af = sqrt(num1 / denom);
    e.as = sqrt(num2 / denom);
  }
  double const bd = 1.0 / hypot(p.by, p.bz);  // rhypot
  e.by            = std::isfinite(bd) ? p.by * bd : 1.0;
  e.bz            = std::isfinite(bd) ? p.bz * bd : 0.0;
  e.sign          = copysign(1.0, p.bx);
  e.nfs           = 0.5 / cs2;
  e.qpf           = e.sign * e.nfs * e.af * e.cf;
  e.qps           = e.sign * e.nfs * e.as * e.cs;
  e.qf            = e.sign * e.af * e.cf;
  e.qs            = e.sign * e.as * e.cs;
  e.Af            = e.af * cs * sqrt(p.d);
  e.As            = e.as * cs * sqrt(p.d);
  e.Apf           = 0.5 * e.af / (cs * sqrt(p.d));
  e.Aps           = 0.5 * e.as / (cs * sqrt(p.d));
  return e;
}

// reconstruction.h:378-437 Primitive_To_Characteristic
Chr prim_to_char(bool mhd, const Prim &p, const Prim &s, const Eig &e, double cs, double cs2)
{
  Chr o;
  if (mhd) {
    double const isd = 1.0 / sqrt(p.d);  // rsqrt
    o.a[0] = e.nfs * e.af * (s.p / p.d - e.cf * s.vx) + e.qps * (e.by * s.vy + e.bz * s.vz) +
             e.Aps * (e.by * s.by + e.bz * s.bz);
    o.a[1] = 0.5 * (e.by * (s.bz * e.sign * isd + s.vz) - e.bz * (s.by * e.sign * isd + s.vy));
    o.a[2] = e.nfs * e.as * (s.p / p.d - e.cs * s.vx) - e.qpf * (e.by * s.vy + e.bz * s.vz) -
             e.Apf * (e.by * s.by + e.bz * s.bz);
    o.a[3] = s.d - s.p / cs2;
    o.a[4] = e.nfs * e.as * (s.p / p.d + e.cs * s.vx) + e.qpf * (e.by * s.vy + e.bz * s.vz) -
             e.Apf * (e.by * s.by + e.bz * s.bz);
    o.a[5] = 0.5 * (e.by * (s.bz * e.sign * isd - s.vz) - e.bz * (s.by * e.sign * isd - s.vy));
    o.a[6] = e.nfs * e.af * (s.p / p.d + e.cf * s.vx) - e.qps * (e.by * s.vy + e.bz * s.vz) +
             e.Aps * (e.by * s.by + e.bz * s.bz);
  } else {
    o.a[0] = -p.d * s.vx / (2.0 * cs) + s.p / (2.0 * cs2);
    o.a[1] = s.d - s.p / (cs2);
    o.a[2] = s.vy;
    o.a[3] = s.vz;
    o.a[4] = p.d * s.vx / (2.0 * cs) + s.p / (2.0 * cs2);
    o.a[5] = o.a[6] = 0.0;
  }
  return o;
}

// reconstruction.h:453-491 Characteristic_To_Primitive
Prim char_to_prim(bool mhd, const Prim &p, const Chr &c, const Eig &e, double cs, double cs2)
{
  Prim o;
  std::memset(&o, 0, sizeof(o));
  const double *a = c.a;
  if (mhd) {
    o.d  = p.d * (e.af * (a[0] + a[6]) + e.as * (a[2] + a[4])) + a[3];
    o.vx = e.cf * e.af * (a[6] - a[0]) + e.cs * e.as * (a[4] - a[2]);
    o.vy = e.by * (e.qs * (a[0] - a[6]) + e.qf * (a[4] - a[2])) + e.bz * (a[5] - a[1]);
    o.vz = e.bz * (e.qs * (a[0] - a[6]) + e.qf * (a[4] - a[2])) + e.by * (a[1] - a[5]);
    o.p  = p.d * cs2 * (e.af * (a[0] + a[6]) + e.as * (a[2] + a[4]));
    o.by = e.by * (e.As * (a[0] + a[6]) - e.Af * (a[2] + a[4])) - e.bz * e.sign * sqrt(p.d) * (a[5] + a[1]);
    o.bz = e.bz * (e.As * (a[0] + a[6]) - e.Af * (a[2] + a[4])) + e.by * e.sign * sqrt(p.d) * (a[5] + a[1]);
  } else {
    o.d  = a[0] + a[1] + a[4];
    o.vx = cs / p.d * (a[4] - a[0]);
    o.vy = a[2];
    o.vz = a[3];
    o.p  = cs2 * (a[0] + a[4]);
  }
  return o;
}

// reconstruction.h:794-901 PPM_Single_Variable
void ppm1(double im2, double im1, double i, double ip1, double ip2, double &L_iph, double &R_imh)
{
  double const C2 = 1.25;
  auto limit      = [&C2](double const &ci, double const &cim1, double const &iface, double const &s2i,
                     double const &s2im1) -> double {
    double s2c = 3.0 * (cim1 + ci - 2.0 * iface);
    double lim = 0.0;
    if (SIGN(s2c) == SIGN(s2im1) and SIGN(s2c) == SIGN(s2i)) {
      lim = SIGN(s2c) * fmin(C2 * fabs(s2im1), fmin(C2 * fabs(s2i), fabs(s2c)));
    }
    double const dl = iface - cim1;
    double const dr = ci - iface;
    if (dl * dr < 0.0) {
      return 0.5 * (cim1 + ci) - lim / 6.0;
    } else {
      return iface;
    }
  };
  double const sl   = (i - im1);
  double const sr   = (ip1 - i);
  double const sim1 = 0.5 * sl + 0.5 * (im1 - im2);
  double const si   = 0.5 * sr + 0.5 * sl;
  double const sip1 = 0.5 * (ip2 - ip1) + 0.5 * sr;
  R_imh             = 0.5 * (im1 + i) + (sim1 - si) / 6.0;
  L_iph             = 0.5 * (i + ip1) + (si - sip1) / 6.0;
  double const d2im1 = im2 + i - 2.0 * im1;
  double const d2i   = im1 + ip1 - 2.0 * i;
  double const d2ip1 = i + ip2 - 2.0 * ip1;
  R_imh              = limit(i, im1, R_imh, d2i, d2im1);
  L_iph              = limit(ip1, i, L_iph, d2ip1, d2i);
  double d2f         = 6.0 * (R_imh + L_iph - 2.0 * i);
  double d2lim       = 0.0;
  if (SIGN(d2im1) == SIGN(d2i) and SIGN(d2im1) == SIGN(d2ip1) and SIGN(d2im1) == SIGN(d2f)) {
    d2lim = SIGN(d2f) * fmin(fmin(C2 * fabs(d2im1), C2 * fabs(d2i)), fmin(C2 * fabs(d2ip1), fabs(d2f)));
  }
  double cmax       = fmax(fabs(im2), fabs(im1));
  cmax              = fmax(cmax, fabs(i));
  cmax              = fmax(cmax, fabs(ip1));
  cmax              = fmax(cmax, fabs(ip2));
  double const rho  = (fabs(d2f) > (1.0e-12) * cmax) ? d2lim / d2f : 0.0;
  double const sfl  = i - R_imh;
  double const sfr  = L_iph - i;
  if ((sfl * sfr) <= 0.0 or ((ip1 - i) * (i - im1)) <= 0.0) {
    if (rho <= (1.0 - (1.0e-12))) {
      R_imh = i - rho * sfl;
      L_iph = i + rho * sfr;
    }
  } else {
    if (fabs(sfl) >= 2.0 * fabs(sfr)) R_imh = i - 2.0 * sfr;
    if (fabs(sfr) >= 2.0 * fabs(sfl)) L_iph = i + 2.0 * sfl;
  }
}

// reconstruction.h:918-968 Write_Data
void write_data(const Grid &g, const Prim &s, double *Q, const double *U, size_t id, int o1, int o2, int o3)
{
  size_t const n = g.n;
  Q[id]          = s.d;
  Q[o1 * n + id] = s.d * s.vx;
  Q[o2 * n + id] = s.d * s.vy;
  Q[o3 * n + id] = s.d * s.vz;
  if (g.mhd) {
    double bx;
    Q[(size_t)g.fB * n + id]       = s.by;
    Q[(size_t)(g.fB + 1) * n + id] = s.bz;
    bx                             = U[(size_t)(g.fB + (o1 - 1)) * n + id];
    // hydro_utilities.h:106-118 Calc_Energy_Primitive
    Q[4 * n + id] = energy_primitive(s.p, s.d, s.vx, s.vy, s.vz, g.gamma, true, bx, s.by, s.bz);
  } else {
    Q[4 * n + id] = energy_primitive(s.p, s.d, s.vx, s.vy, s.vz, g.gamma, false, 0.0, 0.0, 0.0);
  }
  if (g.de) Q[(size_t)g.fGE * n + id] = s.d * s.ge;
  for (int k = 0; k < g.ns; k++) Q[(size_t)(5 + k) * n + id] = s.d * s.sc[k];
}

// reconstruction.h:95-119 Thread_Guard (true = skip)
template <int order>
bool guard(const Grid &g, int x, int y, int z)
{
  bool out = x < order - 1 or x >= g.nx - order;
  if (g.ny > 1) out = y < order - 1 or y >= g.ny - order or out;
  if (g.nz > 1) {
    out = z < order - 1 or z >= g.nz - order or out;
  } else {
    out = z >= g.nz or out;
  }
  return out;
}

// reconstruction.h:224-247 Compute_Slope: coef * (right - left) per primitive field
Prim compute_slope(const Grid &g, const Prim &l, const Prim &r, double coef)
{
  Prim s;
  std::memset(&s, 0, sizeof(s));
  s.d  = coef * (r.d - l.d);
  s.vx = coef * (r.vx - l.vx);
  s.vy = coef * (r.vy - l.vy);
  s.vz = coef * (r.vz - l.vz);
  s.p  = coef * (r.p - l.p);
  if (g.mhd) {
    s.by = coef * (r.by - l.by);
    s.bz = coef * (r.bz - l.bz);
  }
  if (g.de) s.ge = coef * (r.ge - l.ge);
  for (int k = 0; k < g.ns; k++) s.sc[k] = coef * (r.sc[k] - l.sc[k]);
  return s;
}

// reconstruction.h:258-296 Van_Leer_Slope: harmonic mean where the one-sided slopes agree in sign
inline double van_leer(double l, double r)
{
  if (l * r > 0.0) {
    return 2.0 * l * r / (l + r);
  } else {
    return 0.0;
  }
}
Prim van_leer_slope(const Grid &g, const Prim &dL, const Prim &dR)
{
  Prim dG;
  std::memset(&dG, 0, sizeof(dG));
  dG.d  = van_leer(dL.d, dR.d);
  dG.vx = van_leer(dL.vx, dR.vx);
  dG.vy = van_leer(dL.vy, dR.vy);
  dG.vz = van_leer(dL.vz, dR.vz);
  dG.p  = van_leer(dL.p, dR.p);
  if (g.mhd) {
    dG.by = van_leer(dL.by, dR.by);
    dG.bz = van_leer(dL.bz, dR.bz);
  }
  if (g.de) dG.ge = van_leer(dL.ge, dR.ge);
  for (int k = 0; k < g.ns; k++) dG.sc[k] = van_leer(dL.sc[k], dR.sc[k]);
  return dG;
}

// reconstruction.h:512-559 Monotonize_Characteristic_Return_Primitive
inline double monotonize(double l, double r, double cc, double vg)
{
  if (l * r > 0.0) {
    double const la = 2.0 * fmin(fabs(l), fabs(r));
    double const lb = fmin(fabs(cc), fabs(vg));
    return copysign(fmin(la, lb), cc);
  } else {
    return 0.0;
  }
}
Prim monotonize_characteristic(const Grid &g, const Prim &p, const Prim &dL, const Prim &dR, const Prim &dC,
                               const Prim &dG, const Chr &aL, const Chr &aR, const Chr &aC, const Chr &aG,
                               const Eig &e, double cs, double cs2)
{
  Chr am;
  int const nchar = g.mhd ? 7 : 5;
  for (int k = 0; k < 7; k++) am.a[k] = 0.0;
  for (int k = 0; k < nchar; k++) am.a[k] = monotonize(aL.a[k], aR.a[k], aC.a[k], aG.a[k]);
  Prim dm = char_to_prim(g.mhd, p, am, e, cs, cs2);
  if (g.de) dm.ge = monotonize(dL.ge, dR.ge, dC.ge, dG.ge);
  for (int k = 0; k < g.ns; k++) dm.sc[k] = monotonize(dL.sc[k], dR.sc[k], dC.sc[k], dG.sc[k]);
  return dm;
}

// reconstruction.h:645-673 Calc_Interface_Linear: cell + sign * slope / 2
Prim calc_interface_linear(const Grid &g, const Prim &c, const Prim &dm, double sign)
{
  Prim o;
  std::memset(&o, 0, sizeof(o));
  auto f = [&sign](double st, double sl) -> double { return st + sign * 0.5 * sl; };
  o.d  = f(c.d, dm.d);
  o.vx = f(c.vx, dm.vx);
  o.vy = f(c.vy, dm.vy);
  o.vz = f(c.vz, dm.vz);
  o.p  = f(c.p, dm.p);
  if (g.mhd) {
    o.by = f(c.by, dm.by);
    o.bz = f(c.bz, dm.bz);
  }
  if (g.de) o.ge = f(c.ge, dm.ge);
  for (int k = 0; k < g.ns; k++) o.sc[k] = f(c.sc[k], dm.sc[k]);
  return o;
}

// reconstruction.h:686-723 Plm_Limit_Interfaces: each interface value within its two cells' range
inline void plm_limit(double &l, double &r, double vm, double vi, double vp)
{
  r = fmax(fmin(vi, vm), r);
  r = fmin(fmax(vi, vm), r);
  l = fmax(fmin(vi, vp), l);
  l = fmin(fmax(vi, vp), l);
}
void plm_limit_interfaces(const Grid &g, Prim &L, Prim &R, const Prim &cm, const Prim &ci, const Prim &cp)
{
  plm_limit(L.d, R.d, cm.d, ci.d, cp.d);
  plm_limit(L.vx, R.vx, cm.vx, ci.vx, cp.vx);
  plm_limit(L.vy, R.vy, cm.vy, ci.vy, cp.vy);
  plm_limit(L.vz, R.vz, cm.vz, ci.vz, cp.vz);
  plm_limit(L.p, R.p, cm.p, ci.p, cp.p);
  if (g.mhd) {
    plm_limit(L.by, R.by, cm.by, ci.by, cp.by);
    plm_limit(L.bz, R.bz, cm.bz, ci.bz, cp.bz);
  }
  if (g.de) plm_limit(L.ge, R.ge, cm.ge, ci.ge, cp.ge);
  for (int k = 0; k < g.ns; k++) plm_limit(L.sc[k], R.sc[k], cm.sc[k], ci.sc[k], cp.sc[k]);
}

template <typename F>
void par_cells(const Grid &g, F f)
{
  long long const n = (long long)g.n;
#pragma omp parallel for schedule(static) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (long long i = 0; i < n; i++) f((size_t)i);
}

}  // namespace

#ifndef _OPENMP
static int omp_get_max_threads() { return 1; }
#endif

extern "C" {

void orc_set_threads(int n) { g_threads = n; }

void orc_mt19937_uniform(unsigned long long seed, double a, double b, size_t n, double *out)
{
  std::mt19937_64 prng(seed);
  std::uniform_real_distribution<double> dist(a, b);
  for (size_t i = 0; i < n; i++) out[i] = dist(prng);
}
void orc_mt19937_32_uniform(unsigned long seed, double a, double b, size_t n, double *out)
{
  std::mt19937 prng(seed);
  std::uniform_real_distribution<double> dist(a, b);
  for (size_t i = 0; i < n; i++) out[i] = dist(prng);
}
int orc_get_threads(void) { return g_threads > 0 ? g_threads : omp_get_max_threads(); }

void orc_ppm_single_variable(double im2, double im1, double i, double ip1, double ip2, double *L_iph, double *R_imh)
{
  ppm1(im2, im1, i, ip1, ip2, *L_iph, *R_imh);
}

// ---- reconstruction building blocks, one call each, for the reference's helper unit tests
// (src/reconstruction/reconstruction_tests.cu).  A primitive state travels as 9 doubles
// (density, vx, vy, vz, pressure, Bx, By, Bz, gas energy), a characteristic one as 7, the MHD
// eigenvector set as the 18 members of reconstruction::EigenVecs in declaration order.
}  // extern "C"
namespace
{
Prim unpack_prim(const double *v)
{
  Prim p;
  std::memset(&p, 0, sizeof(p));
  p.d = v[0], p.vx = v[1], p.vy = v[2], p.vz = v[3], p.p = v[4], p.bx = v[5], p.by = v[6], p.bz = v[7], p.ge = v[8];
  return p;
}
void pack_prim(const Prim &p, double *v)
{
  v[0] = p.d, v[1] = p.vx, v[2] = p.vy, v[3] = p.vz, v[4] = p.p, v[5] = p.bx, v[6] = p.by, v[7] = p.bz, v[8] = p.ge;
}
Chr unpack_chr(const double *v)
{
  Chr a;
  for (int k = 0; k < 7; k++) a.a[k] = v[k];
  return a;
}
Eig unpack_eig(const double *v)
{
  Eig e;
  static_assert(sizeof(Eig) == 18 * sizeof(double), "EigenVecs has 18 members");
  std::memcpy(&e, v, sizeof(e));
  return e;
}
}  // namespace
extern "C" {

// ---- hydro / MHD utilities on the path (src/utils/hydro_utilities.h, mhd_utilities.h) ----
double orc_t_pressure_primitive(double E, double d, double vx, double vy, double vz, double gamma, int mhd, double bx,
                                double by, double bz)
{
  return pressure_primitive(E, d, vx, vy, vz, gamma, mhd != 0, bx, by, bz);
}
double orc_t_energy_primitive(double P, double d, double vx, double vy, double vz, double gamma, int mhd, double bx,
                              double by, double bz)
{
  return energy_primitive(P, d, vx, vy, vz, gamma, mhd != 0, bx, by, bz);
}
double orc_t_pressure_from_de(double E, double U_total, double U_advected, double gamma)
{
  return pressure_from_de(E, U_total, U_advected, gamma);
}
double orc_t_kinetic_energy(double d, double vx, double vy, double vz) { return kinetic_energy(d, vx, vy, vz); }
double orc_t_magnetic_energy(double bx, double by, double bz) { return magE(bx, by, bz); }
double orc_t_total_pressure(double p, double bx, double by, double bz) { return total_pressure(p, bx, by, bz); }
double orc_t_fast_magnetosonic(double d, double p, double bx, double by, double bz, double gamma)
{
  return cfast(d, p, bx, by, bz, gamma);
}
double orc_t_slow_magnetosonic(double d, double p, double bx, double by, double bz, double gamma)
{
  return cslow(d, p, bx, by, bz, gamma);
}
double orc_t_alfven_speed(double bx, double d) { return alfven_speed(bx, d); }
void orc_t_cell_centered_b(const double *U, size_t id, int x, int y, int z, size_t n_cells, int nx, int ny, int fB,
                           double *out)
{
  cc_b_strided(U, n_cells, nx, ny, fB, id, x, y, z, out[0], out[1], out[2]);
}

int orc_t_thread_guard(const orc_config *c, int order, int x, int y, int z)
{
  Grid g(c);
  return order == 2 ? guard<2>(g, x, y, z) : guard<3>(g, x, y, z);
}

void orc_t_load_data(const orc_config *c, const double *U, int x, int y, int z, int dir, double *out)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  pack_prim(load_data(g, U, x, y, z, o1, o2, o3), out);
}

void orc_t_write_data(const orc_config *c, const double *state, double *Q, const double *U, size_t id, int dir)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  write_data(g, unpack_prim(state), Q, U, id, o1, o2, o3);
}

void orc_t_compute_slope(const orc_config *c, const double *left, const double *right, double coef, double *out)
{
  Grid g(c);
  pack_prim(compute_slope(g, unpack_prim(left), unpack_prim(right), coef), out);
}

void orc_t_van_leer_slope(const orc_config *c, const double *left, const double *right, double *out)
{
  Grid g(c);
  pack_prim(van_leer_slope(g, unpack_prim(left), unpack_prim(right)), out);
}

void orc_t_eigenvectors(const double *prim, double cs, double cs2, double gamma, double *out)
{
  Eig const e = eigenvectors(unpack_prim(prim), cs, cs2, gamma);
  std::memcpy(out, &e, sizeof(e));
}

void orc_t_prim_to_char(int mhd, const double *prim, const double *slope, const double *eig, double cs, double cs2,
                        double *out)
{
  Chr const a = prim_to_char(mhd != 0, unpack_prim(prim), unpack_prim(slope), unpack_eig(eig), cs, cs2);
  for (int k = 0; k < 7; k++) out[k] = a.a[k];
}

void orc_t_char_to_prim(int mhd, const double *prim, const double *chr, const double *eig, double cs, double cs2,
                        double *out)
{
  pack_prim(char_to_prim(mhd != 0, unpack_prim(prim), unpack_chr(chr), unpack_eig(eig), cs, cs2), out);
}

void orc_t_monotonize_characteristic(const orc_config *c, const double *prim, const double *const del[4],
                                     const double *const del_a[4], const double *eig, double cs, double cs2,
                                     double *out)
{
  Grid g(c);
  Prim const d0 = unpack_prim(del[0]), d1 = unpack_prim(del[1]), d2 = unpack_prim(del[2]), d3 = unpack_prim(del[3]);
  Chr const a0 = unpack_chr(del_a[0]), a1 = unpack_chr(del_a[1]), a2 = unpack_chr(del_a[2]), a3 = unpack_chr(del_a[3]);
  pack_prim(monotonize_characteristic(g, unpack_prim(prim), d0, d1, d2, d3, a0, a1, a2, a3, unpack_eig(eig), cs, cs2),
            out);
}

void orc_t_calc_interface_linear(const orc_config *c, const double *cell, const double *slope, double sign,
                                 double *out)
{
  Grid g(c);
  pack_prim(calc_interface_linear(g, unpack_prim(cell), unpack_prim(slope), sign), out);
}

void orc_t_plm_limit_interfaces(const orc_config *c, double *l_iph, double *r_imh, const double *cell_im1,
                                const double *cell_i, const double *cell_ip1)
{
  Grid g(c);
  Prim L = unpack_prim(l_iph), R = unpack_prim(r_imh);
  plm_limit_interfaces(g, L, R, unpack_prim(cell_im1), unpack_prim(cell_i), unpack_prim(cell_ip1));
  pack_prim(L, l_iph);
  pack_prim(R, r_imh);
}

// src/reconstruction/pcm_cuda.cu:256-424 PCM_Reconstruction_3D (and :13-121 for 1D)
void orc_pcm_3d(const orc_config *c, const double *U, double *QLx, double *QRx, double *QLy, double *QRy, double *QLz,
                double *QRz)
{
  Grid g(c);
  size_t const n = g.n;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    double v[16];
    int nv = 0;
    double const d = U[id], mx = U[n + id], my = U[2 * n + id], mz = U[3 * n + id], E = U[4 * n + id];
    double cbx = 0, cby = 0, cbz = 0;
    if (g.mhd) cc_b(g, U, x, y, z, cbx, cby, cbz);
    (void)v;
    (void)nv;
    auto put = [&](double *Q, size_t at, int dir) {
      Q[at]         = d;
      Q[n + at]     = mx;
      Q[2 * n + at] = my;
      Q[3 * n + at] = mz;
      Q[4 * n + at] = E;
      for (int s = 0; s < g.ns; s++) Q[(size_t)(5 + s) * n + at] = U[(size_t)(5 + s) * n + id];
      if (g.mhd) {
        double const b[3] = {cbx, cby, cbz};
        Q[(size_t)g.fB * n + at]       = b[(dir + 1) % 3];
        Q[(size_t)(g.fB + 1) * n + at] = b[(dir + 2) % 3];
      }
      if (g.de) Q[(size_t)g.fGE * n + at] = U[(size_t)g.fGE * n + id];
    };
    put(QLx, id, 0);
    put(QLy, id, 1);
    put(QLz, id, 2);
    if (x > 0) put(QRx, g.id(x - 1, y, z), 0);
    if (y > 0) put(QRy, g.id(x, y - 1, z), 1);
    if (z > 0) put(QRz, g.id(x, y, z - 1), 2);
  });
}

// src/reconstruction/ppmc_cuda.cu:540-695 PPMC_VL
void orc_ppmc_vl(const orc_config *c, const double *U, double *QL, double *QR, int dir)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  int const sx = dir == 0, sy = dir == 1, sz = dir == 2;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (guard<3>(g, x, y, z)) return;
    Prim const ci   = load_data(g, U, x, y, z, o1, o2, o3);
    Prim const cim1 = load_data(g, U, x - sx, y - sy, z - sz, o1, o2, o3);
    Prim const cip1 = load_data(g, U, x + sx, y + sy, z + sz, o1, o2, o3);
    Prim const cim2 = load_data(g, U, x - 2 * sx, y - 2 * sy, z - 2 * sz, o1, o2, o3);
    Prim const cip2 = load_data(g, U, x + 2 * sx, y + 2 * sy, z + 2 * sz, o1, o2, o3);
    double const cs  = sqrt(g.gamma * ci.p / ci.d);  // hydro_utilities.h:209 Calc_Sound_Speed
    double const cs2 = cs * cs;
    Eig e;
    std::memset(&e, 0, sizeof(e));
    if (g.mhd) e = eigenvectors(ci, cs, cs2, g.gamma);
    Chr const ai   = prim_to_char(g.mhd, ci, ci, e, cs, cs2);
    Chr const aim1 = prim_to_char(g.mhd, ci, cim1, e, cs, cs2);
    Chr const aim2 = prim_to_char(g.mhd, ci, cim2, e, cs, cs2);
    Chr const aip1 = prim_to_char(g.mhd, ci, cip1, e, cs, cs2);
    Chr const aip2 = prim_to_char(g.mhd, ci, cip2, e, cs, cs2);
    Chr aR, aL;
    int const nchar = g.mhd ? 7 : 5;
    for (int k = 0; k < 7; k++) aR.a[k] = aL.a[k] = 0.0;
    for (int k = 0; k < nchar; k++) ppm1(aim2.a[k], aim1.a[k], ai.a[k], aip1.a[k], aip2.a[k], aL.a[k], aR.a[k]);
    Prim L = char_to_prim(g.mhd, ci, aL, e, cs, cs2);
    Prim R = char_to_prim(g.mhd, ci, aR, e, cs, cs2);
    if (g.de) ppm1(cim2.ge, cim1.ge, ci.ge, cip1.ge, cip2.ge, L.ge, R.ge);
    for (int s = 0; s < g.ns; s++) ppm1(cim2.sc[s], cim1.sc[s], ci.sc[s], cip1.sc[s], cip2.sc[s], L.sc[s], R.sc[s]);
    R.d = fmax(R.d, TINY);
    L.d = fmax(L.d, TINY);
    R.p = fmax(R.p, TINY);
    L.p = fmax(L.p, TINY);
    write_data(g, L, QL, U, id, o1, o2, o3);
    write_data(g, R, QR, U, g.id(x - sx, y - sy, z - sz), o1, o2, o3);
  });
}

// src/reconstruction/plmc_cuda.cu:24-300 PLMC_cuda (VL: no characteristic tracing)
void orc_plmc(const orc_config *c, const double *U, double *QL, double *QR, int dir)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  int const sx = dir == 0, sy = dir == 1, sz = dir == 2;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (guard<2>(g, x, y, z)) return;
    Prim const ci   = load_data(g, U, x, y, z, o1, o2, o3);
    Prim const cimo = load_data(g, U, x - sx, y - sy, z - sz, o1, o2, o3);
    Prim const cipo = load_data(g, U, x + sx, y + sy, z + sz, o1, o2, o3);
    double const cs  = sqrt(g.gamma * ci.p / ci.d);
    double const cs2 = cs * cs;
    Eig e;
    std::memset(&e, 0, sizeof(e));
    if (g.mhd) e = eigenvectors(ci, cs, cs2, g.gamma);
    Prim const dL = compute_slope(g, cimo, ci, 1.0);
    Prim const dR = compute_slope(g, ci, cipo, 1.0);
    Prim const dC = compute_slope(g, cimo, cipo, 0.5);
    Prim const dG = van_leer_slope(g, dL, dR);
    Chr const aL  = prim_to_char(g.mhd, ci, dL, e, cs, cs2);
    Chr const aR  = prim_to_char(g.mhd, ci, dR, e, cs, cs2);
    Chr const aC  = prim_to_char(g.mhd, ci, dC, e, cs, cs2);
    Chr const aG  = prim_to_char(g.mhd, ci, dG, e, cs, cs2);
    Prim const dm = monotonize_characteristic(g, ci, dL, dR, dC, dG, aL, aR, aC, aG, e, cs, cs2);
    Prim L        = calc_interface_linear(g, ci, dm, 1.0);
    Prim R        = calc_interface_linear(g, ci, dm, -1.0);
    plm_limit_interfaces(g, L, R, cimo, ci, cipo);
    R.d = fmax(R.d, TINY);
    L.d = fmax(L.d, TINY);
    R.p = fmax(R.p, TINY);
    L.p = fmax(L.p, TINY);
    write_data(g, L, QL, U, id, o1, o2, o3);
    write_data(g, R, QR, U, g.id(x - sx, y - sy, z - sz), o1, o2, o3);
  });
}

}  // extern "C"

// ---- primitive-limited reconstructions: PLMP and PPMP ----
// src/reconstruction/plmp_cuda.cu:21-328 PLMP_cuda and ppmp_cuda.cu:28-683 PPMP_cuda as the VL
// build compiles them (no half-step tracing, no flattening or steepening macros): every
// primitive (density, the three velocities, pressure, scalars and GasEnergy per unit mass) is
// limited on its own, with no characteristic projection.
namespace
{
// One cell's primitives as both kernels load them (plmp_cuda.cu:108-133, ppmp_cuda.cu:155-180):
// velocities by division, pressure from the total energy (dual energy: the select of
// Get_Pressure_From_DE) floored at TINY; q = {d, v1, v2, v3, p, scalars..., ge}.
struct PrimQ {
  double q[5 + MAXS + 1];
};

PrimQ load_prim_q(const Grid &g, const double *U, size_t id, int o1, int o2, int o3)
{
  PrimQ s;
  size_t const n = g.n;
  double const d = U[id];
  double const vx = U[(size_t)o1 * n + id] / d, vy = U[(size_t)o2 * n + id] / d, vz = U[(size_t)o3 * n + id] / d;
  double p;
  if (g.de) {
    double const E    = U[4 * n + id];
    double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
    double const dge  = U[(size_t)g.fGE * n + id];
    p                 = pressure_from_de(E, E - Ekin, dge, g.gamma);
    s.q[5 + g.ns]     = dge / d;
  } else {
    p = (U[4 * n + id] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (g.gamma - 1.0);
  }
  s.q[0] = d, s.q[1] = vx, s.q[2] = vy, s.q[3] = vz, s.q[4] = fmax(p, TINY);
  for (int k = 0; k < g.ns; k++) s.q[5 + k] = U[(size_t)(5 + k) * n + id] / d;
  return s;
}

// Van Leer-limited slope of a three-point stencil (plmp_cuda.cu:330-365 Interface_Values_PLM,
// ppmp_cuda.cu:687-720 Calculate_Slope): monotonised central difference with the harmonic mean.
inline double limited_slope(double qm, double q, double qp)
{
  double const dl = q - qm, dr = qp - q, dc = 0.5 * (qp - qm);
  double const dg = (dl * dr > 0.0) ? 2.0 * dl * dr / (dl + dr) : 0.0;
  double const a = fmin(fabs(dl), fabs(dr)), b = fmin(fabs(dc), fabs(dg));
  return sgn_int(dc) * fmin(2.0 * a, b);
}

// Fryxell et al. (2000) parabola through cell i with the monotonicity constraints
// (ppmp_cuda.cu:727-752 Interface_Values_PPM).
void ppm_parabola(double qm, double q, double qp, double sm, double s0, double sp, double &L, double &R)
{
  L = 0.5 * (q + qm) - (1.0 / 6.0) * (s0 - sm);
  R = 0.5 * (qp + q) - (1.0 / 6.0) * (sp - s0);
  if ((R - q) * (q - L) <= 0) L = R = q;
  if (6.0 * (R - L) * (q - 0.5 * (L + R)) > (R - L) * (R - L)) L = 3.0 * q - 2.0 * R;
  if (6.0 * (R - L) * (q - 0.5 * (L + R)) < -(R - L) * (R - L)) R = 3.0 * q - 2.0 * L;
  L = fmax(fmin(q, qm), L);
  L = fmin(fmax(q, qm), L);
  R = fmax(fmin(q, qp), R);
  R = fmin(fmax(q, qp), R);
}

// order 1: PLMP (cells 1 .. n-3 along dir), order 2: PPMP (cells 2 .. n-4).  Writes the state on
// the low side of cell i into QR at i-1 and the state on its high side into QL at i, as conserved
// variables (plmp_cuda.cu:290-326, ppmp_cuda.cu:645-681).
template <int order>
void recon_primitive(const orc_config *c, const double *U, double *QL, double *QR, int dir)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  int const ext   = dir == 0 ? g.nx : dir == 1 ? g.ny : g.nz;
  size_t const st = dir == 0 ? 1 : dir == 1 ? (size_t)g.nx : (size_t)g.nx * g.ny;
  int const nq    = 5 + g.ns + (g.de ? 1 : 0);
  size_t const n  = g.n;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    int const a = dir == 0 ? x : dir == 1 ? y : z;
    if (a < order || a >= ext - order - 1) return;
    PrimQ s[2 * order + 1];
    for (int j = 0; j <= 2 * order; j++) s[j] = load_prim_q(g, U, id - order * st + j * st, o1, o2, o3);
    double lo[5 + MAXS + 1], hi[5 + MAXS + 1];
    for (int k = 0; k < nq; k++) {
      if (order == 1) {
        double const dm = limited_slope(s[0].q[k], s[1].q[k], s[2].q[k]);
        lo[k]           = s[1].q[k] - 0.5 * dm;
        hi[k]           = s[1].q[k] + 0.5 * dm;
      } else {
        double const sm = limited_slope(s[0].q[k], s[1].q[k], s[2].q[k]);
        double const s0 = limited_slope(s[1].q[k], s[2].q[k], s[3].q[k]);
        double const sp = limited_slope(s[2].q[k], s[3].q[k], s[4].q[k]);
        ppm_parabola(s[1].q[k], s[2].q[k], s[3].q[k], sm, s0, sp, lo[k], hi[k]);
      }
    }
    lo[0] = fmax(lo[0], TINY), hi[0] = fmax(hi[0], TINY);
    lo[4] = fmax(lo[4], TINY), hi[4] = fmax(hi[4], TINY);
    auto put = [&](double *Q, size_t at, const double *v) {
      double const d        = v[0];
      Q[at]                 = d;
      Q[(size_t)o1 * n + at] = d * v[1];
      Q[(size_t)o2 * n + at] = d * v[2];
      Q[(size_t)o3 * n + at] = d * v[3];
      Q[4 * n + at]         = v[4] / (g.gamma - 1.0) + 0.5 * d * (v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
      for (int k = 0; k < g.ns; k++) Q[(size_t)(5 + k) * n + at] = d * v[5 + k];
      if (g.de) Q[(size_t)g.fGE * n + at] = d * v[5 + g.ns];
    };
    put(QR, id - st, lo);
    put(QL, id, hi);
  });
}
}  // namespace

void orc_plmp(const orc_config *c, const double *U, double *QL, double *QR, int dir)
{
  recon_primitive<1>(c, U, QL, QR, dir);
}

void orc_ppmp(const orc_config *c, const double *U, double *QL, double *QR, int dir)
{
  recon_primitive<2>(c, U, QL, QR, dir);
}

extern "C" {

// src/riemann_solvers/hllc_cuda.cu:19-307 Calculate_HLLC_Fluxes_CUDA
void orc_hllc(const orc_config *c, const double *QL, const double *QR, double *F, int dir)
{
  Grid g(c);
  size_t const n = g.n;
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  double const gamma = g.gamma;
  par_cells(g, [&](size_t tid) {
    double const g1 = gamma - 1.0;
    double const etah = 0;
    double dl = QL[tid], mxl = QL[o1 * n + tid], myl = QL[o2 * n + tid], mzl = QL[o3 * n + tid], El = QL[4 * n + tid];
    double dr = QR[tid], mxr = QR[o1 * n + tid], myr = QR[o2 * n + tid], mzr = QR[o3 * n + tid], Er = QR[4 * n + tid];
    double dscl[MAXS], dscr[MAXS], scl[MAXS], scr[MAXS];
    for (int s = 0; s < g.ns; s++) {
      dscl[s] = QL[(size_t)(5 + s) * n + tid];
      dscr[s] = QR[(size_t)(5 + s) * n + tid];
    }
    double dgel = 0, dger = 0, gel = 0, ger = 0;
    if (g.de) {
      dgel = QL[(size_t)g.fGE * n + tid];
      dger = QR[(size_t)g.fGE * n + tid];
    }
    double vxl = mxl / dl, vyl = myl / dl, vzl = mzl / dl, pl;
    if (g.de) {
      double const E_kin = 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl);
      pl                 = pressure_from_de(El, El - E_kin, dgel, gamma);
    } else {
      pl = (El - 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl)) * (gamma - 1.0);
    }
    pl = fmax(pl, TINY);
    for (int s = 0; s < g.ns; s++) scl[s] = dscl[s] / dl;
    if (g.de) gel = dgel / dl;
    double vxr = mxr / dr, vyr = myr / dr, vzr = mzr / dr, pr;
    if (g.de) {
      double const E_kin = 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr);
      pr                 = pressure_from_de(Er, Er - E_kin, dger, gamma);
    } else {
      pr = (Er - 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr)) * (gamma - 1.0);
    }
    pr = fmax(pr, TINY);
    for (int s = 0; s < g.ns; s++) scr[s] = dscr[s] / dr;
    if (g.de) ger = dger / dr;
    double const Hl = (El + pl) / dl;
    double const Hr = (Er + pr) / dr;
    double const sqrtdl = sqrt(dl);
    double const sqrtdr = sqrt(dr);
    double const vx     = (sqrtdl * vxl + sqrtdr * vxr) / (sqrtdl + sqrtdr);
    double const vy     = (sqrtdl * vyl + sqrtdr * vyr) / (sqrtdl + sqrtdr);
    double const vz     = (sqrtdl * vzl + sqrtdr * vzr) / (sqrtdl + sqrtdr);
    double const H      = (sqrtdl * Hl + sqrtdr * Hr) / (sqrtdl + sqrtdr);
    double const vsq    = (vx * vx + vy * vy + vz * vz);
    double const asq    = g1 * (H - 0.5 * vsq);
    double const a      = sqrt(asq);
    double const lambda_m = vx - a;
    double const lambda_p = vx + a;
    double const cfl      = sqrt(gamma * pl / dl);
    double const cfr      = sqrt(gamma * pr / dr);
    double Sl             = fmin(lambda_m, vxl - cfl);
    double Sr             = fmax(lambda_p, vxr + cfr);
    Sl                    = sgn_int(Sl) * fmax(fabs(Sl), etah);
    Sr                    = sgn_int(Sr) * fmax(fabs(Sr), etah);
    double const f_d_l = mxl, f_mx_l = mxl * vxl + pl, f_my_l = myl * vxl, f_mz_l = mzl * vxl,
                 f_E_l = (El + pl) * vxl;
    double const f_d_r = mxr, f_mx_r = mxr * vxr + pr, f_my_r = myr * vxr, f_mz_r = mzr * vxr,
                 f_E_r = (Er + pr) * vxr;
    double const f_ge_l = dgel * vxl, f_ge_r = dger * vxr;
    auto out = [&](double fd, double fmx, double fmy, double fmz, double fE) {
      F[tid]          = fd;
      F[o1 * n + tid] = fmx;
      F[o2 * n + tid] = fmy;
      F[o3 * n + tid] = fmz;
      F[4 * n + tid]  = fE;
    };
    if (Sl > 0.0) {
      out(f_d_l, f_mx_l, f_my_l, f_mz_l, f_E_l);
      for (int s = 0; s < g.ns; s++) F[(size_t)(5 + s) * n + tid] = dscl[s] * vxl;
      if (g.de) F[(size_t)g.fGE * n + tid] = f_ge_l;
      return;
    } else if (Sr < 0.0) {
      out(f_d_r, f_mx_r, f_my_r, f_mz_r, f_E_r);
      for (int s = 0; s < g.ns; s++) F[(size_t)(5 + s) * n + tid] = dscr[s] * vxr;
      if (g.de) F[(size_t)g.fGE * n + tid] = f_ge_r;
      return;
    }
    double const Sm = (dr * vxr * (Sr - vxr) - dl * vxl * (Sl - vxl) + pl - pr) / (dr * (Sr - vxr) - dl * (Sl - vxl));
    double const ps = dl * (vxl - Sl) * (vxl - Sm) + pl;
    double const dls  = dl * (Sl - vxl) / (Sl - Sm);
    double const mxls = (mxl * (Sl - vxl) + ps - pl) / (Sl - Sm);
    double const myls = dls * vyl;
    double const mzls = dls * vzl;
    double const Els  = (El * (Sl - vxl) - pl * vxl + ps * Sm) / (Sl - Sm);
    double const gels = dls * gel;
    double const drs  = dr * (Sr - vxr) / (Sr - Sm);
    double const mxrs = (mxr * (Sr - vxr) + ps - pr) / (Sr - Sm);
    double const myrs = drs * vyr;
    double const mzrs = drs * vzr;
    double const Ers  = (Er * (Sr - vxr) - pr * vxr + ps * Sm) / (Sr - Sm);
    double const gers = drs * ger;
    double const f_d  = 0.5 * (f_d_l + f_d_r + (Sr - fabs(Sm)) * drs + (Sl + fabs(Sm)) * dls - Sl * dl - Sr * dr);
    double const f_mx =
        0.5 * (f_mx_l + f_mx_r + (Sr - fabs(Sm)) * mxrs + (Sl + fabs(Sm)) * mxls - Sl * mxl - Sr * mxr);
    double const f_my =
        0.5 * (f_my_l + f_my_r + (Sr - fabs(Sm)) * myrs + (Sl + fabs(Sm)) * myls - Sl * myl - Sr * myr);
    double const f_mz =
        0.5 * (f_mz_l + f_mz_r + (Sr - fabs(Sm)) * mzrs + (Sl + fabs(Sm)) * mzls - Sl * mzl - Sr * mzr);
    double const f_E = 0.5 * (f_E_l + f_E_r + (Sr - fabs(Sm)) * Ers + (Sl + fabs(Sm)) * Els - Sl * El - Sr * Er);
    out(f_d, f_mx, f_my, f_mz, f_E);
    for (int s = 0; s < g.ns; s++) {
      double const scls = dls * scl[s], scrs = drs * scr[s];
      double const fl = dscl[s] * vxl, fr = dscr[s] * vxr;
      F[(size_t)(5 + s) * n + tid] =
          0.5 * (fl + fr + (Sr - fabs(Sm)) * scrs + (Sl + fabs(Sm)) * scls - Sl * dscl[s] - Sr * dscr[s]);
    }
    if (g.de) {
      F[(size_t)g.fGE * n + tid] =
          0.5 * (f_ge_l + f_ge_r + (Sr - fabs(Sm)) * gers + (Sl + fabs(Sm)) * gels - Sl * dgel - Sr * dger);
    }
  });
}

// src/riemann_solvers/roe_cuda.cu:19-400 Calculate_Roe_Fluxes_CUDA
void orc_roe(const orc_config *c, const double *QL, const double *QR, double *F, int dir)
{
  Grid g(c);
  size_t const n = g.n;
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  double const gamma = g.gamma;
  par_cells(g, [&](size_t tid) {
    double const etah = 0.0;
    double const g1   = gamma - 1.0;
    double dl = QL[tid], mxl = QL[o1 * n + tid], myl = QL[o2 * n + tid], mzl = QL[o3 * n + tid], El = QL[4 * n + tid];
    double dr = QR[tid], mxr = QR[o1 * n + tid], myr = QR[o2 * n + tid], mzr = QR[o3 * n + tid], Er = QR[4 * n + tid];
    double dscl[MAXS], dscr[MAXS], scl[MAXS], scr[MAXS], fscl[MAXS], fscr[MAXS];
    for (int s = 0; s < g.ns; s++) {
      dscl[s] = QL[(size_t)(5 + s) * n + tid];
      dscr[s] = QR[(size_t)(5 + s) * n + tid];
    }
    double dgel = 0, dger = 0, gel = 0, ger = 0, f_ge_l = 0, f_ge_r = 0;
    if (g.de) {
      dgel = QL[(size_t)g.fGE * n + tid];
      dger = QR[(size_t)g.fGE * n + tid];
    }
    double vxl = mxl / dl, vyl = myl / dl, vzl = mzl / dl, pl;
    if (g.de) {
      double const E_kin = 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl);
      pl                 = pressure_from_de(El, El - E_kin, dgel, gamma);
    } else {
      pl = (El - 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl)) * (gamma - 1.0);
    }
    pl = fmax(pl, TINY);
    for (int s = 0; s < g.ns; s++) scl[s] = dscl[s] / dl;
    if (g.de) gel = dgel / dl;
    double vxr = mxr / dr, vyr = myr / dr, vzr = mzr / dr, pr;
    if (g.de) {
      double const E_kin = 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr);
      pr                 = pressure_from_de(Er, Er - E_kin, dger, gamma);
    } else {
      pr = (Er - 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr)) * (gamma - 1.0);
    }
    pr = fmax(pr, TINY);
    for (int s = 0; s < g.ns; s++) scr[s] = dscr[s] / dr;
    if (g.de) ger = dger / dr;
    double const Hl = (El + pl) / dl, Hr = (Er + pr) / dr;
    double const sqrtdl = sqrt(dl), sqrtdr = sqrt(dr);
    double const vx  = (sqrtdl * vxl + sqrtdr * vxr) / (sqrtdl + sqrtdr);
    double const vy  = (sqrtdl * vyl + sqrtdr * vyr) / (sqrtdl + sqrtdr);
    double const vz  = (sqrtdl * vzl + sqrtdr * vzr) / (sqrtdl + sqrtdr);
    double const H   = (sqrtdl * Hl + sqrtdr * Hr) / (sqrtdl + sqrtdr);
    double const vsq = (vx * vx + vy * vy + vz * vz);
    double const asq = g1 * fmax((H - 0.5 * vsq), TINY);
    double const a   = sqrt(asq);
    double const lambda_m = vx - a, lambda_0 = vx, lambda_p = vx + a;
    double f_d_l = mxl, f_mx_l = mxl * vxl + pl, f_my_l = mxl * vyl, f_mz_l = mxl * vzl, f_E_l = (El + pl) * vxl;
    double f_d_r = mxr, f_mx_r = mxr * vxr + pr, f_my_r = mxr * vyr, f_mz_r = mxr * vzr, f_E_r = (Er + pr) * vxr;
    if (g.de) {
      f_ge_l = mxl * gel;
      f_ge_r = mxr * ger;
    }
    for (int s = 0; s < g.ns; s++) {
      fscl[s] = mxl * scl[s];
      fscr[s] = mxr * scr[s];
    }
    auto out = [&](double fd, double fmx, double fmy, double fmz, double fE) {
      F[tid]          = fd;
      F[o1 * n + tid] = fmx;
      F[o2 * n + tid] = fmy;
      F[o3 * n + tid] = fmz;
      F[4 * n + tid]  = fE;
    };
    if (lambda_m >= 0.0) {
      out(f_d_l, f_mx_l, f_my_l, f_mz_l, f_E_l);
      for (int s = 0; s < g.ns; s++) F[(size_t)(5 + s) * n + tid] = fscl[s];
      if (g.de) F[(size_t)g.fGE * n + tid] = f_ge_l;
      return;
    } else if (lambda_p <= 0.0) {
      out(f_d_r, f_mx_r, f_my_r, f_mz_r, f_E_r);
      for (int s = 0; s < g.ns; s++) F[(size_t)(5 + s) * n + tid] = fscr[s];
      if (g.de) F[(size_t)g.fGE * n + tid] = f_ge_r;
      return;
    }
    double sum_0 = 0, sum_1 = 0, sum_2 = 0, sum_3 = 0, sum_4 = 0;
    double const del_d = dr - dl, del_mx = mxr - mxl, del_my = myr - myl, del_mz = mzr - mzl, del_E = Er - El;
    double const Na = 0.5 / asq;
    double coeff    = 0.0;
    double const a0 = del_d * Na * (0.5 * g1 * vsq + vx * a) - del_mx * Na * (g1 * vx + a) - del_my * Na * g1 * vy -
                      del_mz * Na * g1 * vz + del_E * Na * g1;
    coeff = a0 * fmax(fabs(lambda_m), etah);
    sum_0 += coeff;
    sum_1 += coeff * (vx - a);
    sum_2 += coeff * vy;
    sum_3 += coeff * vz;
    sum_4 += coeff * (H - vx * a);
    double const a1 = -del_d * vy + del_my;
    coeff           = a1 * fmax(fabs(lambda_0), etah);
    sum_2 += coeff;
    sum_4 += coeff * vy;
    double const a2 = -del_d * vz + del_mz;
    coeff           = a2 * fmax(fabs(lambda_0), etah);
    sum_3 += coeff;
    sum_4 += coeff * vz;
    double const a3 = del_d * (1.0 - Na * g1 * vsq) + del_mx * g1 * vx / asq + del_my * g1 * vy / asq +
                      del_mz * g1 * vz / asq - del_E * g1 / asq;
    coeff = a3 * fmax(fabs(lambda_0), etah);
    sum_0 += coeff;
    sum_1 += coeff * vx;
    sum_2 += coeff * vy;
    sum_3 += coeff * vz;
    sum_4 += coeff * 0.5 * vsq;
    double const a4 = del_d * Na * (0.5 * g1 * vsq - vx * a) - del_mx * Na * (g1 * vx - a) - del_my * Na * g1 * vy -
                      del_mz * Na * g1 * vz + del_E * Na * g1;
    coeff = a4 * fmax(fabs(lambda_p), etah);
    sum_0 += coeff;
    sum_1 += coeff * (vx + a);
    sum_2 += coeff * vy;
    sum_3 += coeff * vz;
    sum_4 += coeff * (H + vx * a);
    int hlle_flag = 0;
    double test0 = dl + a0, test1 = mxl + a0 * (vx - a), test2 = myl + a0 * vy, test3 = mzl + a0 * vz,
           test4 = El + a0 * (H - vx * a);
    if (lambda_0 > lambda_m) {
      if (test0 <= 0.0) hlle_flag = 1;
      if (test4 - 0.5 * (test1 * test1 + test2 * test2 + test3 * test3) / test0 < 0.0) hlle_flag = 2;
    }
    test0 += a3 + a4;
    test1 += a3 * vx;
    test2 += a1 + a3 * vy;
    test3 += a2 + a3 * vz;
    test4 += a1 * vy + a2 * vz + a3 * 0.5 * vsq;
    if (lambda_p > lambda_0) {
      if (test0 <= 0.0) hlle_flag = 1;
      if (test4 - 0.5 * (test1 * test1 + test2 * test2 + test3 * test3) / test0 < 0.0) hlle_flag = 2;
    }
    if (hlle_flag != 0) {
      double const cfl = sqrt(gamma * pl / dl);
      double const cfr = sqrt(gamma * pr / dr);
      double const bm  = fmin(fmin(lambda_m, vxl - cfl), 0.0);
      double const bp  = fmax(fmax(lambda_p, vxr + cfr), 0.0);
      f_d_l            = mxl - bm * dl;
      f_d_r            = mxr - bp * dr;
      f_mx_l           = mxl * (vxl - bm) + pl;
      f_mx_r           = mxr * (vxr - bp) + pr;
      f_my_l           = myl * (vxl - bm);
      f_my_r           = myr * (vxr - bp);
      f_mz_l           = mzl * (vxl - bm);
      f_mz_r           = mzr * (vxr - bp);
      f_E_l            = El * (vxl - bm) + pl * vxl;
      f_E_r            = Er * (vxr - bp) + pr * vxr;
      if (g.de) {
        f_ge_l = dgel * (vxl - bm);
        f_ge_r = dger * (vxr - bp);
      }
      for (int s = 0; s < g.ns; s++) {
        fscl[s] = dscl[s] * (vxl - bm);
        fscr[s] = dscr[s] * (vxr - bp);
      }
      double const tmp = 0.5 * (bp + bm) / (bp - bm);
      out(0.5 * (f_d_l + f_d_r) + (f_d_l - f_d_r) * tmp, 0.5 * (f_mx_l + f_mx_r) + (f_mx_l - f_mx_r) * tmp,
          0.5 * (f_my_l + f_my_r) + (f_my_l - f_my_r) * tmp, 0.5 * (f_mz_l + f_mz_r) + (f_mz_l - f_mz_r) * tmp,
          0.5 * (f_E_l + f_E_r) + (f_E_l - f_E_r) * tmp);
      for (int s = 0; s < g.ns; s++)
        F[(size_t)(5 + s) * n + tid] = 0.5 * (fscl[s] + fscr[s]) + (fscl[s] - fscr[s]) * tmp;
      if (g.de) F[(size_t)g.fGE * n + tid] = 0.5 * (f_ge_l + f_ge_r) + (f_ge_l - f_ge_r) * tmp;
      return;
    }
    out(0.5 * (f_d_l + f_d_r - sum_0), 0.5 * (f_mx_l + f_mx_r - sum_1), 0.5 * (f_my_l + f_my_r - sum_2),
        0.5 * (f_mz_l + f_mz_r - sum_3), 0.5 * (f_E_l + f_E_r - sum_4));
    for (int s = 0; s < g.ns; s++)
      F[(size_t)(5 + s) * n + tid] = (F[tid] >= 0.0) ? F[tid] * scl[s] : F[tid] * scr[s];
    if (g.de) F[(size_t)g.fGE * n + tid] = (F[tid] >= 0.0) ? F[tid] * gel : F[tid] * ger;
  });
}

// src/riemann_solvers/hll_cuda.cu:19-268 Calculate_HLL_Fluxes_CUDA: the two-wave flux with
// Davis's wave-speed estimates (the slower of the two left-going and the faster of the two
// right-going acoustic speeds).  Interface states are conserved; every cell is computed.
void orc_hll(const orc_config *c, const double *QL, const double *QR, double *F, int dir)
{
  Grid g(c);
  size_t const n = g.n;
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  double const gamma = g.gamma;
  par_cells(g, [&](size_t tid) {
    int const nq = 5 + g.ns + (g.de ? 1 : 0);
    double ql[5 + MAXS + 1], qr[5 + MAXS + 1], fl[5 + MAXS + 1], fr[5 + MAXS + 1];
    size_t idx[5 + MAXS + 1];
    idx[0] = 0, idx[1] = (size_t)o1, idx[2] = (size_t)o2, idx[3] = (size_t)o3, idx[4] = 4;
    for (int s = 0; s < g.ns; s++) idx[5 + s] = (size_t)(5 + s);
    if (g.de) idx[nq - 1] = (size_t)g.fGE;
    for (int k = 0; k < nq; k++) ql[k] = QL[idx[k] * n + tid], qr[k] = QR[idx[k] * n + tid];
    auto side = [&](const double *q, double *f, double &vx, double &p) {
      double const d = q[0];
      vx             = q[1] / d;
      double const vy = q[2] / d, vz = q[3] / d;
      if (g.de) {
        double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
        p                  = pressure_from_de(q[4], q[4] - E_kin, q[nq - 1], gamma);
      } else {
        p = (q[4] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
      }
      p    = fmax(p, TINY);
      f[0] = q[1];
      f[1] = q[1] * vx + p;
      f[2] = q[2] * vx;
      f[3] = q[3] * vx;
      f[4] = (q[4] + p) * vx;
      for (int k = 5; k < nq; k++) f[k] = q[k] * vx;  // scalars and the thermal energy advect
    };
    double vxl, pl, vxr, pr;
    side(ql, fl, vxl, pl);
    side(qr, fr, vxr, pr);
    double const cfl = sqrt(gamma * pl / ql[0]), cfr = sqrt(gamma * pr / qr[0]);
    double const Sl = fmin(vxr - cfr, vxl - cfl);
    double const Sr = fmax(vxl + cfl, vxr + cfr);
    for (int k = 0; k < nq; k++) {
      double out;
      if (Sl > 0.0) {
        out = fl[k];
      } else if (Sr < 0.0) {
        out = fr[k];
      } else {
        out = ((Sr * fl[k]) - (Sl * fr[k]) + Sl * Sr * (qr[k] - ql[k])) / (Sr - Sl);
      }
      F[idx[k] * n + tid] = out;
    }
  });
}

// src/riemann_solvers/exact_cuda.cu:19-334 Calculate_Exact_Fluxes_CUDA: the exact Riemann
// solution (Toro 2009, ch. 4) sampled on the interface, x/t = 0.  Star pressure from the
// primitive-variable guess (two-shock correction when it is not positive), then Newton with a
// relative tolerance of 1e-6 and at most 21 passes.  The reference evaluates its fractional
// powers in single precision (powf), so this restatement does too: its results agree with the
// reference's to single-precision rounding of those powers, not bit for bit.  (The reference's
// VL integrator itself does not compile with this solver selected: VL_3D_cuda.cu:149.)
namespace
{
inline double fpow(double a, double b) { return (double)powf((float)a, (float)b); }

void exact_pressure_function(double &f, double &fd, double p, double dk, double pk, double ck, double g)
{
  if (p <= pk) {  // rarefaction branch
    f  = (2.0 / (g - 1.0)) * ck * (fpow(p / pk, (g - 1.0) / (2.0 * g)) - 1.0);
    fd = (1.0 / (dk * ck)) * fpow(p / pk, -((g + 1.0) / (2.0 * g)));
  } else {  // shock branch
    double const bk = ((g - 1.0) / (g + 1.0)) * pk;
    double const q  = sqrt(((2.0 / (g + 1.0)) / dk) / (bk + p));
    f  = (p - pk) * q;
    fd = (1.0 - 0.5 * (p - pk) / (bk + p)) * q;
  }
}

void exact_star(double &pm, double &vm, double dl, double vl, double pl, double cl, double dr, double vr, double pr,
                double cr, double g)
{
  double const tol = 1.0e-6;
  double ppv       = 0.5 * (pl + pr) + 0.125 * (vl - vr) * (dl + dr) * (cl + cr);
  if (ppv < 0.0) ppv = 0.0;
  double const gl = sqrt((2.0 / ((g + 1.0) * dl)) / (((g - 1.0) / (g + 1.0)) * pl + ppv));
  double const gr = sqrt((2.0 / ((g + 1.0) * dr)) / (((g - 1.0) / (g + 1.0)) * pr + ppv));
  double pold     = (gl * pl + gr * pr - (vr - vl)) / (gl + gr);
  if (pold < 0.0) pold = tol;
  double fl = 0, fld = 0, fr = 0, frd = 0;
  for (int it = 0; it <= 20; it++) {
    exact_pressure_function(fl, fld, pold, dl, pl, cl, g);
    exact_pressure_function(fr, frd, pold, dr, pr, cr, g);
    pm                  = pold - (fl + fr + vr - vl) / (fld + frd);
    double const change = 2.0 * fabs((pm - pold) / (pm + pold));
    if (change <= tol) break;
    if (pm < 0.0) pm = tol;
    pold = pm;
  }
  vm = 0.5 * (vl + vr + fr - fl);
}

// the state on x/t = 0 of the wave pattern with star pressure pm and contact speed vm
void exact_sample(double pm, double vm, double &d, double &v, double &p, double dl, double vl, double pl, double cl,
                  double dr, double vr, double pr, double cr, double g)
{
  double const gm = (g - 1.0) / (g + 1.0);
  if (vm >= 0) {  // left of the contact
    if (pm <= pl) {  // left rarefaction
      if (vl - cl >= 0) {
        d = dl, v = vl, p = pl;
      } else if (vm - cl * fpow(pm / pl, (g - 1.0) / (2.0 * g)) < 0) {
        d = dl * fpow(pm / pl, 1.0 / g), v = vm, p = pm;
      } else {  // inside the fan
        double const c = (2.0 / (g + 1.0)) * (cl + ((g - 1.0) / 2.0) * vl);
        v = c;
        d = dl * fpow(c / cl, 2.0 / (g - 1.0));
        p = pl * fpow(c / cl, 2.0 * g / (g - 1.0));
      }
    } else {  // left shock
      double const sl = vl - cl * sqrt(((g + 1.0) / (2.0 * g)) * (pm / pl) + ((g - 1.0) / (2.0 * g)));
      if (sl >= 0) {
        d = dl, v = vl, p = pl;
      } else {
        d = dl * (pm / pl + gm) / ((pm / pl) * gm + 1.0), v = vm, p = pm;
      }
    }
  } else {  // right of the contact
    if (pm > pr) {  // right shock
      double const sr = vr + cr * sqrt(((g + 1.0) / (2.0 * g)) * (pm / pr) + ((g - 1.0) / (2.0 * g)));
      if (sr <= 0) {
        d = dr, v = vr, p = pr;
      } else {
        d = dr * (pm / pr + gm) / ((pm / pr) * gm + 1.0), v = vm, p = pm;
      }
    } else {  // right rarefaction
      if (vr + cr <= 0) {
        d = dr, v = vr, p = pr;
      } else if (vm + cr * fpow(pm / pr, (g - 1.0) / (2.0 * g)) >= 0) {
        d = dr * fpow(pm / pr, 1.0 / g), v = vm, p = pm;
      } else {  // inside the fan
        double const c = (2.0 / (g + 1.0)) * (cr - ((g - 1.0) / 2.0) * vr);
        v = -c;
        d = dr * fpow(c / cr, 2.0 / (g - 1.0));
        p = pr * fpow(c / cr, 2.0 * g / (g - 1.0));
      }
    }
  }
}
}  // namespace

void orc_exact(const orc_config *c, const double *QL, const double *QR, double *F, int dir)
{
  Grid g(c);
  size_t const n = g.n;
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  double const gamma = g.gamma;
  par_cells(g, [&](size_t tid) {
    auto load = [&](const double *Q, double &d, double &vx, double &vy, double &vz, double &p, double &ge,
                    double *sc) {
      d  = Q[tid];
      vx = Q[(size_t)o1 * n + tid] / d;
      vy = Q[(size_t)o2 * n + tid] / d;
      vz = Q[(size_t)o3 * n + tid] / d;
      double const E = Q[4 * n + tid];
      ge             = 0.0;
      if (g.de) {
        double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
        double const dge   = Q[(size_t)g.fGE * n + tid];
        p                  = pressure_from_de(E, E - E_kin, dge, gamma);
        ge                 = dge / d;
      } else {
        p = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
      }
      p = fmax(p, TINY);
      for (int s = 0; s < g.ns; s++) sc[s] = Q[(size_t)(5 + s) * n + tid] / d;
    };
    double dl, vxl, vyl, vzl, pl, gel, scl[MAXS];
    double dr, vxr, vyr, vzr, pr, ger, scr[MAXS];
    load(QL, dl, vxl, vyl, vzl, pl, gel, scl);
    load(QR, dr, vxr, vyr, vzr, pr, ger, scr);
    double const cl = sqrt(gamma * pl / dl), cr = sqrt(gamma * pr / dr);
    double pm = 0, vm = 0, ds = 0, vs = 0, ps = 0;
    exact_star(pm, vm, dl, vxl, pl, cl, dr, vxr, pr, cr, gamma);
    exact_sample(pm, vm, ds, vs, ps, dl, vxl, pl, cl, dr, vxr, pr, cr, gamma);
    F[tid]                  = ds * vs;
    F[(size_t)o1 * n + tid] = ds * vs * vs + ps;
    bool const left         = vs >= 0;  // the transverse velocities and passive quantities advect upwind
    double const vy = left ? vyl : vyr, vz = left ? vzl : vzr;
    F[(size_t)o2 * n + tid] = ds * vs * vy;
    F[(size_t)o3 * n + tid] = ds * vs * vz;
    for (int s = 0; s < g.ns; s++) F[(size_t)(5 + s) * n + tid] = ds * vs * (left ? scl[s] : scr[s]);
    if (g.de) F[(size_t)g.fGE * n + tid] = ds * vs * (left ? gel : ger);
    double const Es = (ps / (gamma - 1.0)) + 0.5 * ds * (vs * vs + vy * vy + vz * vz);
    F[4 * n + tid]  = (Es + ps) * vs;
  });
}

// src/riemann_solvers/hlld_cuda.cu:31-508 (mhd::Calculate_HLLD_Fluxes_CUDA and mhd::internal)
namespace
{
struct HState {
  double d, vx, vy, vz, E, by, bz, p, pt;
  double sc[MAXS];
  double ge;
};
struct HStar {
  double d, vy, vz, E, by, bz;
};
struct HDStar {
  double vy, vz, by, bz, EL = 0.0, ER = 0.0;
};
struct HFlux {
  double d, mx, my, mz, E, by, bz;
};
struct HSpeeds {
  double L, LStar, M, RStar, R;
};

HState hlld_load(const Grid &g, const double *Q, double bx, size_t t, int o1, int o2, int o3)
{
  size_t const n = g.n;
  HState s;
  s.d  = Q[t];
  s.d  = fmax(s.d, TINY);
  s.vx = Q[t + n * o1] / s.d;
  s.vy = Q[t + n * o2] / s.d;
  s.vz = Q[t + n * o3] / s.d;
  s.E  = Q[t + n * 4];
  s.E  = fmax(s.E, TINY);
  s.by = Q[t + n * g.fB];
  s.bz = Q[t + n * (g.fB + 1)];
  for (int k = 0; k < g.ns; k++) s.sc[k] = Q[t + n * (5 + k)] / s.d;
  s.ge = 0;
  if (g.de) {
    s.ge         = Q[t + n * g.fGE] / s.d;
    double const Ent = 0.5 * s.d * sqmag(s.vx, s.vy, s.vz) + magE(bx, s.by, s.bz);
    s.p          = fmax(pressure_from_de(s.E, s.E - Ent, s.ge * s.d, g.gamma), TINY);
  } else {
    s.p = pressure_primitive(s.E, s.d, s.vx, s.vy, s.vz, g.gamma, true, bx, s.by, s.bz);
  }
  s.pt = total_pressure(s.p, bx, s.by, s.bz);
  return s;
}
HFlux hlld_nonstar(const HState &s, double bx)
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
HStar hlld_star(const HState &s, const HSpeeds &sp, double S, double bx, double ptStar)
{
  HStar st;
  st.d = s.d * (S - s.vx) / (S - sp.M);
  if (fabs(s.d * (S - s.vx) * (S - sp.M) - (bx * bx)) < ptStar * HLLD_SMALL) {
    st.vy = s.vy;
    st.vz = s.vz;
    st.by = s.by;
    st.bz = s.bz;
  } else {
    double const denom = s.d * (S - s.vx) * (S - sp.M) - (bx * bx);
    double coef        = bx * (sp.M - s.vx) / denom;
    st.vy              = s.vy - s.by * coef;
    st.vz              = s.vz - s.bz * coef;
    double tp          = (S - s.vx);
    tp                 = tp * tp;
    coef               = (s.d * tp - (bx * bx)) / denom;
    st.by              = s.by * coef;
    st.bz              = s.bz * coef;
  }
  st.E = (s.E * (S - s.vx) - s.pt * s.vx + ptStar * sp.M +
          bx * (dot3(s.vx, s.vy, s.vz, bx, s.by, s.bz) - dot3(sp.M, st.vy, st.vz, bx, st.by, st.bz))) /
         (S - sp.M);
  return st;
}
HFlux hlld_starflux(const HStar &st, const HState &s, const HFlux &f, const HSpeeds &sp, double S)
{
  HFlux o;
  o.d  = f.d + S * (st.d - s.d);
  o.mx = f.mx + S * (st.d * sp.M - s.d * s.vx);
  o.my = f.my + S * (st.d * st.vy - s.d * s.vy);
  o.mz = f.mz + S * (st.d * st.vz - s.d * s.vz);
  o.E  = f.E + S * (st.E - s.E);
  o.by = f.by + S * (st.by - s.by);
  o.bz = f.bz + S * (st.bz - s.bz);
  return o;
}
HDStar hlld_dstar(const HStar &L, const HStar &R, double bx, double ptStar, const HSpeeds &sp)
{
  HDStar o;
  if (0.5 * (bx * bx) < HLLD_SMALL * ptStar) {
    if (sp.M >= 0.0) {
      o.vy = L.vy, o.vz = L.vz, o.by = L.by, o.bz = L.bz, o.EL = L.E;
    } else {
      o.vy = R.vy, o.vz = R.vz, o.by = R.by, o.bz = R.bz, o.ER = R.E;
    }
  } else {
    double const sqrtDL = sqrt(L.d), sqrtDR = sqrt(R.d);
    double const inv    = 1.0 / (sqrtDL + sqrtDR);
    double const sgnb   = copysign(1.0, bx);
    o.vy = inv * (sqrtDL * L.vy + sqrtDR * R.vy + sgnb * (R.by - L.by));
    o.vz = inv * (sqrtDL * L.vz + sqrtDR * R.vz + sgnb * (R.bz - L.bz));
    o.by = inv * (sqrtDL * R.by + sqrtDR * L.by + sgnb * (sqrtDL * sqrtDR) * (R.vy - L.vy));
    o.bz = inv * (sqrtDL * R.bz + sqrtDR * L.bz + sgnb * (sqrtDL * sqrtDR) * (R.vz - L.vz));
    double const vdb = dot3(sp.M, o.vy, o.vz, bx, o.by, o.bz);
    o.EL = L.E - sqrtDL * sgnb * (dot3(sp.M, L.vy, L.vz, bx, L.by, L.bz) - vdb);
    o.ER = R.E + sqrtDR * sgnb * (dot3(sp.M, R.vy, R.vz, bx, R.by, R.bz) - vdb);
  }
  return o;
}
HFlux hlld_dstarflux(const HDStar &ds, double dsE, const HStar &st, const HState &s, const HFlux &f,
                     const HSpeeds &sp, double S, double SStar)
{
  HFlux o;
  double const sd = SStar - S;
  o.d  = f.d - S * s.d - sd * st.d + SStar * st.d;
  o.mx = f.mx - S * (s.d * s.vx) - sd * (st.d * sp.M) + SStar * (st.d * sp.M);
  o.my = f.my - S * (s.d * s.vy) - sd * (st.d * st.vy) + SStar * (st.d * ds.vy);
  o.mz = f.mz - S * (s.d * s.vz) - sd * (st.d * st.vz) + SStar * (st.d * ds.vz);
  o.E  = f.E - S * s.E - sd * st.E + SStar * dsE;
  o.by = f.by - S * s.by - sd * st.by + SStar * ds.by;
  o.bz = f.bz - S * s.bz - sd * st.bz + SStar * ds.bz;
  return o;
}
// hlld_cuda.cu approximateLRWaveSpeeds: outermost signal speeds from the larger fast speed
void hlld_lr_speeds(const HState &sL, const HState &sR, double bx, double gamma, HSpeeds &sp)
{
  double const cL   = cfast(sL.d, sL.p, bx, sL.by, sL.bz, gamma);
  double const cR   = cfast(sR.d, sR.p, bx, sR.by, sR.bz, gamma);
  double const cmax = fmax(cL, cR);
  sp.L              = fmin(sL.vx, sR.vx) - cmax;
  sp.R              = fmax(sL.vx, sR.vx) + cmax;
}
// hlld_cuda.cu approximateMiddleWaveSpeed: the contact speed
double hlld_middle_speed(const HState &sL, const HState &sR, const HSpeeds &sp)
{
  double const rd = sp.R - sR.vx, ld = sp.L - sL.vx;
  return (rd * sR.d * sR.vx - ld * sL.d * sL.vx - sR.pt + sL.pt) / (rd * sR.d - ld * sL.d);
}
// hlld_cuda.cu approximateStarWaveSpeed: the Alfven wave bounding one star region (side -1 / +1)
double hlld_star_speed(const HStar &st, const HSpeeds &sp, double bx, double side)
{
  return sp.M + side * alfven_speed(bx, st.d);
}
// hlld_cuda.cu starTotalPressure: total pressure in the star regions
double hlld_pt_star(const HState &sL, const HState &sR, const HSpeeds &sp)
{
  return (sR.d * sL.pt * (sp.R - sR.vx) - sL.d * sR.pt * (sp.L - sL.vx) +
          sL.d * sR.d * (sp.R - sR.vx) * (sp.L - sL.vx) * (sR.vx - sL.vx)) /
         (sR.d * (sp.R - sR.vx) - sL.d * (sp.L - sL.vx));
}
// hlld_cuda.cu returnFluxes: the flux of one interface into the permuted flux fields; passive
// scalars and the thermal energy are advected with the density flux of the upwind state
void hlld_return(const Grid &g, double *F, size_t t, int o1, int o2, int o3, const HFlux &f, const HState &s)
{
  size_t const n = g.n;
  F[t]                  = f.d;
  F[t + n * o1]         = f.mx;
  F[t + n * o2]         = f.my;
  F[t + n * o3]         = f.mz;
  F[t + n * 4]          = f.E;
  F[t + n * g.fB]       = f.by;
  F[t + n * (g.fB + 1)] = f.bz;
  for (int k = 0; k < g.ns; k++) F[t + n * (5 + k)] = s.sc[k] * f.d;
  if (g.de) F[t + n * g.fGE] = s.ge * f.d;
}
}  // namespace

void orc_hlld(const orc_config *c, const double *QL, const double *QR, const double *Bface, double *F, int dir)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  par_cells(g, [&](size_t t) {
    double const bx = Bface[t];
    HState const sL = hlld_load(g, QL, bx, t, o1, o2, o3);
    HState const sR = hlld_load(g, QR, bx, t, o1, o2, o3);
    auto ret        = [&](const HFlux &f, const HState &s) { hlld_return(g, F, t, o1, o2, o3, f, s); };
    HSpeeds sp;
    hlld_lr_speeds(sL, sR, bx, g.gamma, sp);
    HFlux fL = hlld_nonstar(sL, bx);
    if (sp.L > 0.0) {
      ret(fL, sL);
      return;
    }
    HFlux fR = hlld_nonstar(sR, bx);
    if (sp.R < 0.0) {
      ret(fR, sR);
      return;
    }
    sp.M                = hlld_middle_speed(sL, sR, sp);
    double const ptStar = hlld_pt_star(sL, sR, sp);
    HStar const stL     = hlld_star(sL, sp, sp.L, bx, ptStar);
    sp.LStar            = hlld_star_speed(stL, sp, bx, -1);
    if (sp.LStar > 0.0 and sp.L <= 0.0) {
      ret(hlld_starflux(stL, sL, fL, sp, sp.L), sL);
      return;
    }
    HStar const stR = hlld_star(sR, sp, sp.R, bx, ptStar);
    sp.RStar        = hlld_star_speed(stR, sp, bx, 1);
    if (sp.RStar <= 0.0 and sp.R >= 0.0) {
      ret(hlld_starflux(stR, sR, fR, sp, sp.R), sR);
      return;
    }
    HDStar const ds = hlld_dstar(stL, stR, bx, ptStar, sp);
    if (sp.M > 0.0 and sp.LStar <= 0.0) {
      ret(hlld_dstarflux(ds, ds.EL, stL, sL, fL, sp, sp.L, sp.LStar), sL);
      return;
    }
    if (sp.RStar > 0.0 and sp.M <= 0.0) {
      ret(hlld_dstarflux(ds, ds.ER, stR, sR, fR, sp, sp.R, sp.RStar), sR);
      return;
    }
  });
}

// ---- HLLD building blocks, one call each, for the reference's HLLD-internal unit tests
// (src/riemann_solvers/hlld_cuda_tests.cu:1877-2400).  States travel packed in the member order
// of mhd::internal::State (9), StarState (6), DoubleStarState (6), Flux (7) and Speeds (5).
}  // extern "C"
namespace
{
HState unpack_hstate(const double *v)
{
  HState s;
  std::memset(&s, 0, sizeof(s));
  s.d = v[0], s.vx = v[1], s.vy = v[2], s.vz = v[3], s.E = v[4], s.by = v[5], s.bz = v[6], s.p = v[7], s.pt = v[8];
  return s;
}
void pack_hstate(const HState &s, double *v)
{
  v[0] = s.d, v[1] = s.vx, v[2] = s.vy, v[3] = s.vz, v[4] = s.E, v[5] = s.by, v[6] = s.bz, v[7] = s.p, v[8] = s.pt;
}
HStar unpack_hstar(const double *v) { return HStar{v[0], v[1], v[2], v[3], v[4], v[5]}; }
void pack_hstar(const HStar &s, double *v) { v[0] = s.d, v[1] = s.vy, v[2] = s.vz, v[3] = s.E, v[4] = s.by, v[5] = s.bz; }
HFlux unpack_hflux(const double *v) { return HFlux{v[0], v[1], v[2], v[3], v[4], v[5], v[6]}; }
void pack_hflux(const HFlux &f, double *v)
{
  v[0] = f.d, v[1] = f.mx, v[2] = f.my, v[3] = f.mz, v[4] = f.E, v[5] = f.by, v[6] = f.bz;
}
HSpeeds unpack_speeds(const double *v) { return HSpeeds{v[0], v[1], v[2], v[3], v[4]}; }
HDStar unpack_hdstar(const double *v)
{
  HDStar d;
  d.vy = v[0], d.vz = v[1], d.by = v[2], d.bz = v[3], d.EL = v[4], d.ER = v[5];
  return d;
}
}  // namespace
extern "C" {

void orc_t_hlld_load_state(const orc_config *c, const double *Q, double bx, size_t t, int dir, double *out)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  pack_hstate(hlld_load(g, Q, bx, t, o1, o2, o3), out);
}

void orc_t_hlld_return_fluxes(const orc_config *c, size_t t, int dir, double *F, const double *flux,
                              const double *state)
{
  Grid g(c);
  int o1, o2, o3;
  perm(dir, o1, o2, o3);
  hlld_return(g, F, t, o1, o2, o3, unpack_hflux(flux), unpack_hstate(state));
}

void orc_t_hlld_lr_speeds(const double *stateL, const double *stateR, double bx, double gamma, double *speeds)
{
  HSpeeds sp{0, 0, 0, 0, 0};
  hlld_lr_speeds(unpack_hstate(stateL), unpack_hstate(stateR), bx, gamma, sp);
  speeds[0] = sp.L, speeds[1] = sp.LStar, speeds[2] = sp.M, speeds[3] = sp.RStar, speeds[4] = sp.R;
}

double orc_t_hlld_middle_speed(const double *stateL, const double *stateR, const double *speeds)
{
  return hlld_middle_speed(unpack_hstate(stateL), unpack_hstate(stateR), unpack_speeds(speeds));
}

double orc_t_hlld_star_speed(const double *star, const double *speeds, double bx, double side)
{
  return hlld_star_speed(unpack_hstar(star), unpack_speeds(speeds), bx, side);
}

double orc_t_hlld_star_total_pressure(const double *stateL, const double *stateR, const double *speeds)
{
  return hlld_pt_star(unpack_hstate(stateL), unpack_hstate(stateR), unpack_speeds(speeds));
}

void orc_t_hlld_nonstar_fluxes(const double *state, double bx, double *flux)
{
  pack_hflux(hlld_nonstar(unpack_hstate(state), bx), flux);
}

void orc_t_hlld_star_state(const double *state, const double *speeds, double S, double bx, double pt_star,
                           double *star)
{
  pack_hstar(hlld_star(unpack_hstate(state), unpack_speeds(speeds), S, bx, pt_star), star);
}

void orc_t_hlld_star_fluxes(const double *star, const double *state, const double *flux, const double *speeds,
                            double S, double *out)
{
  pack_hflux(hlld_starflux(unpack_hstar(star), unpack_hstate(state), unpack_hflux(flux), unpack_speeds(speeds), S),
             out);
}

void orc_t_hlld_double_star_state(const double *starL, const double *starR, double bx, double pt_star,
                                  const double *speeds, double *out)
{
  HDStar const d = hlld_dstar(unpack_hstar(starL), unpack_hstar(starR), bx, pt_star, unpack_speeds(speeds));
  out[0] = d.vy, out[1] = d.vz, out[2] = d.by, out[3] = d.bz, out[4] = d.EL, out[5] = d.ER;
}

void orc_t_hlld_double_star_fluxes(const double *dstar, double dstar_energy, const double *star, const double *state,
                                   const double *flux, const double *speeds, double S, double S_star, double *out)
{
  pack_hflux(hlld_dstarflux(unpack_hdstar(dstar), dstar_energy, unpack_hstar(star), unpack_hstate(state),
                            unpack_hflux(flux), unpack_speeds(speeds), S, S_star),
             out);
}

// src/mhd/ct_electric_fields.h:66-118 _ctSlope and ct_electric_fields.cu:20-279
namespace
{
inline double ct_slope(const Grid &g, const double *flux, const double *U, double fluxSign, int ctDir, int cq1,
                       int cq2, int fq1, int fq2, int x, int y, int z)
{
  size_t const n = g.n;
  int const m1   = (ctDir + 1) % 3;
  int const m2   = (ctDir + 2) % 3;
  int const xc   = x - int(cq1 == 0) - int(cq2 == 0);
  int const yc   = y - int(cq1 == 1) - int(cq2 == 1);
  int const zc   = z - int(cq1 == 2) - int(cq2 == 2);
  size_t const ic = g.id(xc, yc, zc);
  size_t const iflux = g.id(x - int(fq1 == 0) - int(fq2 == 0), y - int(fq1 == 1) - int(fq2 == 1),
                            z - int(fq1 == 2) - int(fq2 == 2));
  size_t const iB2 = g.id(xc - int(m1 == 0), yc - int(m1 == 1), zc - int(m1 == 2));
  size_t const iB3 = g.id(xc - int(m2 == 0), yc - int(m2 == 1), zc - int(m2 == 2));
  double const density = U[ic];
  double const M2      = U[ic + (size_t)(m1 + 1) * n];
  double const M3      = U[ic + (size_t)(m2 + 1) * n];
  double const B2c     = 0.5 * (U[ic + (size_t)(m1 + g.fB) * n] + U[iB2 + (size_t)(m1 + g.fB) * n]);
  double const B3c     = 0.5 * (U[ic + (size_t)(m2 + g.fB) * n] + U[iB3 + (size_t)(m2 + g.fB) * n]);
  double const ec      = (M3 * B2c - M2 * B3c) / density;
  double const ef      = fluxSign * flux[iflux + (size_t)(int(fluxSign == 1) + g.fB) * n];
  return ef - ec;
}
}  // namespace

double orc_ct_slope(const orc_config *c, const double *flux, const double *U, double flux_sign, int ct_dir, int cq1,
                    int cq2, int fq1, int fq2, int x, int y, int z)
{
  Grid g(c);
  return ct_slope(g, flux, U, flux_sign, ct_dir, cq1, cq2, fq1, fq2, x, y, z);
}

void orc_ct_electric_fields(const orc_config *c, const double *Fx, const double *Fy, const double *Fz,
                            const double *U, double *emf)
{
  Grid g(c);
  size_t const n = g.n;
  int const fB   = g.fB;
  // flux field positions of the magnetic fluxes (grid_enum.h:95-100)
  int const fxBz = fB, fxBy = fB + 1, fyBx = fB, fyBz = fB + 1, fzBy = fB, fzBx = fB + 1;
  par_cells(g, [&](size_t t) {
    int x, y, z;
    g.xyz(t, x, y, z);
    if (!(x > 0 and y > 0 and z > 0 and x < g.nx and y < g.ny and z < g.nz)) return;
    auto S = [&](const double *fl, double sgn, int cd, int a, int b, int cc, int d) {
      return ct_slope(g, fl, U, sgn, cd, a, b, cc, d, x, y, z);
    };
    auto pick = [](double sgnUp, double pos, double neg) {
      if (sgnUp > 0.0) return pos;
      if (sgnUp < 0.0) return neg;
      return 0.5 * (pos + neg);
    };
    double syp, syn, szp, szn, sxp, sxn, fyp, fyn, fzp, fzn, fxp, fxn;
    // X electric field
    syp = pick(Fz[g.id(x, y, z - 1)], S(Fy, -1, 0, 2, -1, 1, 2), S(Fy, -1, 0, -1, -1, 1, -1));
    syn = pick(Fz[g.id(x, y - 1, z - 1)], S(Fy, -1, 0, 1, 2, 1, 2), S(Fy, -1, 0, 1, -1, 1, -1));
    szp = pick(Fy[g.id(x, y - 1, z)], S(Fz, 1, 0, 1, -1, 1, 2), S(Fz, 1, 0, -1, -1, 2, -1));
    szn = pick(Fy[g.id(x, y - 1, z - 1)], S(Fz, 1, 0, 1, 2, 1, 2), S(Fz, 1, 0, 2, -1, -1, 2));
    fyp = +Fz[g.id(x, y, z - 1) + (size_t)fzBx * n];
    fyn = +Fz[g.id(x, y - 1, z - 1) + (size_t)fzBx * n];
    fzp = -Fy[g.id(x, y - 1, z) + (size_t)fyBx * n];
    fzn = -Fy[g.id(x, y - 1, z - 1) + (size_t)fyBx * n];
    emf[t + 0 * n] = 0.25 * (+fyp + fyn + fzp + fzn + syp + syn + szp + szn);
    // Y electric field
    sxp = pick(Fz[g.id(x, y, z - 1)], S(Fx, 1, 1, 2, -1, 0, 2), S(Fx, 1, 1, -1, -1, 0, -1));
    sxn = pick(Fz[g.id(x - 1, y, z - 1)], S(Fx, 1, 1, 0, 2, 0, 2), S(Fx, 1, 1, 0, -1, 0, -1));
    szp = pick(Fx[g.id(x - 1, y, z)], S(Fz, -1, 1, 0, -1, 0, 2), S(Fz, -1, 1, -1, -1, 2, -1));
    szn = pick(Fx[g.id(x - 1, y, z - 1)], S(Fz, -1, 1, 0, 2, 0, 2), S(Fz, -1, 1, 2, -1, 2, -1));
    fxp = -Fz[g.id(x, y, z - 1) + (size_t)fzBy * n];
    fxn = -Fz[g.id(x - 1, y, z - 1) + (size_t)fzBy * n];
    fzp = +Fx[g.id(x - 1, y, z) + (size_t)fxBy * n];
    fzn = +Fx[g.id(x - 1, y, z - 1) + (size_t)fxBy * n];
    emf[t + 1 * n] = 0.25 * (+fxp + fxn + fzp + fzn + sxp + sxn + szp + szn);
    // Z electric field
    syp = pick(Fx[g.id(x - 1, y, z)], S(Fy, 1, 2, 0, -1, 0, 1), S(Fy, 1, 2, -1, -1, 1, -1));
    syn = pick(Fx[g.id(x - 1, y - 1, z)], S(Fy, 1, 2, 0, 1, 0, 1), S(Fy, 1, 2, 1, -1, 1, -1));
    sxp = pick(Fy[g.id(x, y - 1, z)], S(Fx, -1, 2, 1, -1, 0, 1), S(Fx, -1, 2, -1, -1, 0, -1));
    sxn = pick(Fy[g.id(x - 1, y - 1, z)], S(Fx, -1, 2, 0, 1, 0, 1), S(Fx, -1, 2, 0, -1, 0, -1));
    fxp = +Fy[g.id(x, y - 1, z) + (size_t)fyBz * n];
    fxn = +Fy[g.id(x - 1, y - 1, z) + (size_t)fyBz * n];
    fyp = -Fx[g.id(x - 1, y, z) + (size_t)fxBz * n];
    fyn = -Fx[g.id(x - 1, y - 1, z) + (size_t)fxBz * n];
    emf[t + 2 * n] = 0.25 * (+fxp + fxn + fyp + fyn + sxp + sxn + syp + syn);
  });
}

// src/mhd/magnetic_update.cu:21-81 Update_Magnetic_Field_3D
void orc_update_magnetic(const orc_config *c, const double *src, double *dst, const double *emf, double dt)
{
  Grid g(c);
  size_t const n = g.n;
  double const dtodx = dt / c->dx, dtody = dt / c->dy, dtodz = dt / c->dz;
  par_cells(g, [&](size_t t) {
    int x, y, z;
    g.xyz(t, x, y, z);
    if (!(x > 0 and y > 0 and z > 0 and x < g.nx - 1 and y < g.ny - 1 and z < g.nz - 1)) return;
    double const ex1 = emf[g.id(x, y + 1, z) + 0 * n], ex2 = emf[g.id(x, y, z + 1) + 0 * n],
                 ex3 = emf[g.id(x, y + 1, z + 1) + 0 * n];
    double const ey1 = emf[g.id(x + 1, y, z) + 1 * n], ey2 = emf[g.id(x, y, z + 1) + 1 * n],
                 ey3 = emf[g.id(x + 1, y, z + 1) + 1 * n];
    double const ez1 = emf[g.id(x + 1, y, z) + 2 * n], ez2 = emf[g.id(x, y + 1, z) + 2 * n],
                 ez3 = emf[g.id(x + 1, y + 1, z) + 2 * n];
    size_t const bx = t + (size_t)g.fB * n, by = t + (size_t)(g.fB + 1) * n, bz = t + (size_t)(g.fB + 2) * n;
    dst[bx] = src[bx] + dtodz * (ey3 - ey1) + dtody * (ez1 - ez3);
    dst[by] = src[by] + dtodx * (ez3 - ez2) + dtodz * (ex1 - ex3);
    dst[bz] = src[bz] + dtody * (ex3 - ex2) + dtodx * (ey2 - ey3);
  });
}

// src/integrators/VL_3D_cuda.cu:379-495 Update_Conserved_Variables_3D_half
void orc_update_half(const orc_config *c, const double *U, double *Uh, const double *Fx, const double *Fy,
                     const double *Fz, double dt)
{
  Grid g(c);
  size_t const n = g.n;
  double const dtodx = dt / c->dx, dtody = dt / c->dy, dtodz = dt / c->dz;
  double const gamma = g.gamma, floor = c->density_floor;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (!(x > 0 && x < g.nx - 1 && y > 0 && y < g.ny - 1 && z > 0 && z < g.nz - 1)) return;
    size_t const imo = g.id(x - 1, y, z), jmo = g.id(x, y - 1, z), kmo = g.id(x, y, z - 1);
    double P = 0, vx_imo = 0, vx_ipo = 0, vy_jmo = 0, vy_jpo = 0, vz_kmo = 0, vz_kpo = 0;
    if (g.de) {
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const E = U[4 * n + id], GE = U[(size_t)g.fGE * n + id];
      double E_kin   = 0.5 * d * sqmag(vx, vy, vz);
      if (g.mhd) {
        double bx, by, bz;
        cc_b(g, U, x, y, z, bx, by, bz);
        E_kin += magE(bx, by, bz);
      }
      P = pressure_from_de(E, E - E_kin, GE, gamma);
      P = fmax(P, TINY);
      size_t const ipo = g.id(x + 1, y, z), jpo = g.id(x, y + 1, z), kpo = g.id(x, y, z + 1);
      vx_imo = U[n + imo] / U[imo];
      vx_ipo = U[n + ipo] / U[ipo];
      vy_jmo = U[2 * n + jmo] / U[jmo];
      vy_jpo = U[2 * n + jpo] / U[jpo];
      vz_kmo = U[3 * n + kmo] / U[kmo];
      vz_kpo = U[3 * n + kpo] / U[kpo];
    }
    auto upd = [&](int f) {
      size_t const o = (size_t)f * n;
      return U[o + id] + dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]) +
             dtodz * (Fz[o + kmo] - Fz[o + id]);
    };
    for (int f = 0; f < 5; f++) Uh[(size_t)f * n + id] = upd(f);
    for (int s = 0; s < g.ns; s++) Uh[(size_t)(5 + s) * n + id] = upd(5 + s);
    if (g.de) {
      size_t const o = (size_t)g.fGE * n;
      Uh[o + id] = U[o + id] + dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]) +
                   dtodz * (Fz[o + kmo] - Fz[o + id]) +
                   0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo) + dtodz * (vz_kmo - vz_kpo));
    }
    if (c->density_floor_on) {
      if (Uh[id] < floor) {
        double const dens_0 = Uh[id];
        Uh[id]              = floor;
        Uh[1 * n + id] *= (floor / dens_0);
        Uh[2 * n + id] *= (floor / dens_0);
        Uh[3 * n + id] *= (floor / dens_0);
        Uh[4 * n + id] *= (floor / dens_0);
        if (g.de) Uh[(size_t)g.fGE * n + id] *= (floor / dens_0);
      }
    }
  });
}

// src/hydro/hydro_cuda.cu:754-833 Partial_Update_Advected_Internal_Energy_3D (and :705-752 for 1D)
void orc_de_partial_update(const orc_config *c, double *U, double dt)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  double const dtodx = dt / c->dx, dtody = dt / c->dy, dtodz = dt / c->dz;
  bool const one_d = g.ny == 1 && g.nz == 1;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (one_d) {
      if (!(x > ng - 1 && x < g.nx - ng)) return;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const E = U[4 * n + id], GE = U[(size_t)g.fGE * n + id];
      double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double P           = pressure_from_de(E, E - E_kin, GE, g.gamma);
      P                  = fmax(P, TINY);
      double const vx_imo = U[n + id - 1] / U[id - 1], vx_ipo = U[n + id + 1] / U[id + 1];
      U[(size_t)g.fGE * n + id] += 0.5 * P * (dtodx * (vx_imo - vx_ipo));
      return;
    }
    if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) return;
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E = U[4 * n + id], GE = U[(size_t)g.fGE * n + id];
    double E_kin   = 0.5 * d * sqmag(vx, vy, vz);
    if (g.mhd) {
      double bx, by, bz;
      cc_b(g, U, x, y, z, bx, by, bz);
      E_kin += magE(bx, by, bz);
    }
    double P = pressure_from_de(E, E - E_kin, GE, g.gamma);
    P        = fmax(P, TINY);
    size_t const imo = g.id(x - 1, y, z), jmo = g.id(x, y - 1, z), kmo = g.id(x, y, z - 1);
    size_t const ipo = g.id(x + 1, y, z), jpo = g.id(x, y + 1, z), kpo = g.id(x, y, z + 1);
    double const vx_imo = U[n + imo] / U[imo], vx_ipo = U[n + ipo] / U[ipo];
    double const vy_jmo = U[2 * n + jmo] / U[jmo], vy_jpo = U[2 * n + jpo] / U[jpo];
    double const vz_kmo = U[3 * n + kmo] / U[kmo], vz_kpo = U[3 * n + kpo] / U[kpo];
    U[(size_t)g.fGE * n + id] +=
        0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo) + dtodz * (vz_kmo - vz_kpo));
  });
}

// src/hydro/hydro_cuda.cu:172-402 Update_Conserved_Variables_3D (DENSITY_FLOOR and TEMPERATURE_FLOOR on)
void orc_update_full(const orc_config *c, double *U, const double *Fx, const double *Fy, const double *Fz, double dt)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  double const dtodx = dt / c->dx, dtody = dt / c->dy, dtodz = dt / c->dz;
  double const floor = c->density_floor;
  std::vector<unsigned char> negative(c->density_floor_on ? g.n : 0, 0);
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) return;
    size_t const imo = g.id(x - 1, y, z), jmo = g.id(x, y - 1, z), kmo = g.id(x, y, z - 1);
    auto upd = [&](int f) {
      size_t const o = (size_t)f * n;
      U[o + id] += dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]) +
                   dtodz * (Fz[o + kmo] - Fz[o + id]);
    };
    for (int f = 0; f < 5; f++) upd(f);
    for (int s = 0; s < g.ns; s++) upd(5 + s);
    if (g.de) upd(g.fGE);
    if (c->density_floor_on) {
      if (U[id] < floor) {
        if (U[id] > 0) {
          double const dens_0 = U[id];
          U[id]               = floor;
          U[1 * n + id] *= (floor / dens_0);
          U[2 * n + id] *= (floor / dens_0);
          U[3 * n + id] *= (floor / dens_0);
          U[4 * n + id] *= (floor / dens_0);
          if (g.de) U[(size_t)g.fGE * n + id] *= (floor / dens_0);
        } else {
          negative[id] = 1;
        }
      }
    }
  });
  // hydro_cuda.cu:1155-1177 Average_Cell_Single_Field(density).  The reference averages the six
  // neighbours while they are being updated by other threads; here the average is taken over the
  // updated neighbours, after the whole update, which is the outcome once every thread has finished.
  if (c->density_floor_on) {
    for (size_t id = 0; id < g.n; id++) {
      if (!negative[id]) continue;
      int x, y, z;
      g.xyz(id, x, y, z);
      double const v = (U[g.id(x - 1, y, z)] + U[g.id(x + 1, y, z)] + U[g.id(x, y - 1, z)] + U[g.id(x, y + 1, z)] +
                        U[g.id(x, y, z - 1)] + U[g.id(x, y, z + 1)]) /
                       6;
      U[id] = v;
    }
  }
}

// src/hydro/hydro_cuda.cu:20-82 Update_Conserved_Variables_1D
static void update_full_1d(const Grid &g, double *U, const double *F, double dx, double dt)
{
  size_t const n     = g.n;
  double const dtodx = dt / dx;
  for (size_t id = g.ng; id < n - g.ng; id++) {
    for (int f = 0; f < 5; f++) U[(size_t)f * n + id] += dtodx * (F[(size_t)f * n + id - 1] - F[(size_t)f * n + id]);
    for (int s = 0; s < g.ns; s++)
      U[(size_t)(5 + s) * n + id] += dtodx * (F[(size_t)(5 + s) * n + id - 1] - F[(size_t)(5 + s) * n + id]);
    if (g.de) U[(size_t)g.fGE * n + id] += dtodx * (F[(size_t)g.fGE * n + id - 1] - F[(size_t)g.fGE * n + id]);
  }
}

// src/hydro/hydro_cuda.cu:949-1016 Select_Internal_Energy_3D (and :835-885 for 1D)
void orc_de_select(const orc_config *c, double *U)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  bool const one_d = g.ny == 1 && g.nz == 1;
  // every read is of E or of the cell's own fields, and only GasEnergy is written
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    double Emax;
    double const d = U[id], d_inv = 1.0 / d;
    if (one_d) {
      if (!(x > ng - 1 && x < g.nx - ng)) return;
      int const imo = std::max(x - 1, ng), ipo = std::min(x + 1, g.nx - ng - 1);
      double const E = U[4 * n + id];
      Emax           = fmax(U[4 * n + imo], E);
      Emax           = fmax(Emax, U[4 * n + ipo]);
    } else {
      if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) return;
      size_t const imo = g.id(std::max(x - 1, ng), y, z), ipo = g.id(std::min(x + 1, g.nx - ng - 1), y, z);
      size_t const jmo = g.id(x, std::max(y - 1, ng), z), jpo = g.id(x, std::min(y + 1, g.ny - ng - 1), z);
      size_t const kmo = g.id(x, y, std::max(z - 1, ng)), kpo = g.id(x, y, std::min(z + 1, g.nz - ng - 1));
      double const E = U[4 * n + id];
      Emax           = fmax(U[4 * n + imo], E);
      Emax           = fmax(Emax, U[4 * n + ipo]);
      Emax           = fmax(Emax, U[4 * n + jmo]);
      Emax           = fmax(Emax, U[4 * n + jpo]);
      Emax           = fmax(Emax, U[4 * n + kmo]);
      Emax           = fmax(Emax, U[4 * n + kpo]);
    }
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E          = U[4 * n + id];
    double const U_advected = U[(size_t)g.fGE * n + id];
    double const U_total    = E - 0.5 * d * (vx * vx + vy * vy + vz * vz);
    double Ui;
    if ((U_total / E > ETA_1) or (U_total / Emax > ETA_2)) {
      Ui = U_total;
    } else {
      Ui = U_advected;
    }
    Ui                        = fmax(Ui, TINY);
    U[(size_t)g.fGE * n + id] = Ui;
  });
}

// src/hydro/hydro_cuda.cu:1070-1099 Sync_Energies_3D (and :1018-1041 for 1D)
void orc_de_sync(const orc_config *c, double *U)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  bool const one_d = g.ny == 1 && g.nz == 1;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (one_d) {
      if (!(x > ng - 1 && x < g.nx - ng)) return;
    } else if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) {
      return;
    }
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const Ui = U[(size_t)g.fGE * n + id];
    U[4 * n + id]   = 0.5 * d * (vx * vx + vy * vy + vz * vz) + Ui;
  });
}

// src/hydro/hydro_cuda.cu:1117-1153 Temperature_Floor_Kernel
void orc_temperature_floor(const orc_config *c, double *U, double U_floor)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) return;
    double const d = U[id], d_inv = 1.0 / d;
    double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
    double const E = U[4 * n + id];
    double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
    double Ui = (E - Ekin) / d;
    if (Ui < U_floor) U[4 * n + id] = Ekin + d * U_floor;
    if (g.de) {
      Ui = U[(size_t)g.fGE * n + id] / d;
      if (Ui < U_floor) U[(size_t)g.fGE * n + id] = d * U_floor;
    }
  });
}

// src/hydro/hydro_cuda.cu:404-435, 437-471, 514-560: Calc_dt_{1D,3D}; returns max inverse time step
double orc_calc_dt(const orc_config *c, const double *U)
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  double const gamma = g.gamma, dx = c->dx, dy = c->dy, dz = c->dz;
  bool const one_d = g.ny == 1 && g.nz == 1;
  double result = -DBL_MAX;
  long long const N = (long long)n;
#pragma omp parallel for reduction(max : result) num_threads(g_threads > 0 ? g_threads : omp_get_max_threads())
  for (long long ii = 0; ii < N; ii++) {
    size_t const id = (size_t)ii;
    int x, y, z;
    g.xyz(id, x, y, z);
    double m = -DBL_MAX;
    if (one_d) {
      if (!(id > (size_t)ng - 1 && id < n - ng)) continue;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double P = (U[4 * n + id] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
      P        = fmax(P, TINY);
      double const cs = sqrt(d_inv * gamma * P);
      m               = fmax(m, (fabs(vx) + cs) / dx);
    } else if (g.nz == 1) {  // hydro_cuda.cu:473-512 Calc_dt_2D
      if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng)) continue;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double P = (U[4 * n + id] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
      P        = fmax(P, TINY);
      double const cs = sqrt(d_inv * gamma * P);
      m               = fmax(m, fmax((fabs(vx) + cs) / dx, (fabs(vy) + cs) / dy));
    } else {
      if (!(x > ng - 1 && x < g.nx - ng && y > ng - 1 && y < g.ny - ng && z > ng - 1 && z < g.nz - ng)) continue;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const E = U[4 * n + id];
      double cm;
      if (g.mhd) {
        double bx, by, bz;
        cc_b(g, U, x, y, z, bx, by, bz);
        double pressure = E - 0.5 * d * sqmag(vx, vy, vz);
        pressure -= magE(bx, by, bz);
        double const gasP = fmax((gamma - 1.) * pressure, TINY);
        double const cf   = cfast(d, gasP, bx, by, bz, gamma);
        cm = fmax((fabs(vx) + cf) / dx, (fabs(vy) + cf) / dy);
        cm = fmax(cm, (fabs(vz) + cf) / dz);
        cm = fmax(cm, 0.0);
      } else {
        double const P  = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
        double const cs = sqrt(d_inv * gamma * P);
        cm = fmax((fabs(vx) + cs) / dx, (fabs(vy) + cs) / dy);
        cm = fmax(cm, (fabs(vz) + cs) / dz);
        cm = fmax(cm, 0.0);
      }
      m = fmax(m, cm);
    }
    result = fmax(result, m);
  }
  return result;
}

// src/mhd/magnetic_divergence.cu:33-76 calculateMagneticDivergence: max |div B| over the cells that
// its thread guard (:50) admits, x, y, z > 1 up to the last cell, so the upper ghost layers count
double orc_max_divB(const orc_config *c, const double *U)
{
  Grid g(c);
  size_t const n = g.n;
  double const dx = c->dx, dy = c->dy, dz = c->dz;
  double result = 0.0;
  for (int z = 2; z < g.nz; z++)
    for (int y = 2; y < g.ny; y++)
      for (int x = 2; x < g.nx; x++) {
        size_t const id = g.id(x, y, z);
        double const div =
            fabs((U[(size_t)g.fB * n + id] - U[(size_t)g.fB * n + g.id(x - 1, y, z)]) / dx +
                 (U[(size_t)(g.fB + 1) * n + id] - U[(size_t)(g.fB + 1) * n + g.id(x, y - 1, z)]) / dy +
                 (U[(size_t)(g.fB + 2) * n + id] - U[(size_t)(g.fB + 2) * n + g.id(x, y, z - 1)]) / dz);
        result = fmax(result, div);
      }
  return result;
}

// src/grid/cuda_boundaries.cu:71-300 SetGhostCellsKernel / SetBoundaryMapping / FindIndex and
// src/grid/boundary_conditions.cpp:54-131, 412-500 (the six faces, in order, with their extents)
namespace
{
int find_index(int ig, int nx, int flag, int face, int ng, double *a)
{
  if (face == 0) {
    switch (flag) {
      case 1: return ig + nx - 2 * ng;
      case 2: *a = -1.0; return 2 * ng - ig - 1;
      case 3: return ng;
      case 4: return -1;
      case 5: return ig;
      default: return ig + nx - 2 * ng;
    }
  } else {
    switch (flag) {
      case 1: return ig - nx + 2 * ng;
      case 2: *a = -1.0; return 2 * (nx - ng) - ig - 1;
      case 3: return nx - ng - 1;
      case 4: return -1;
      case 5: return ig;
      default: return ig - nx + 2 * ng;
    }
  }
}
long long boundary_mapping(int ig, int jg, int kg, double *a, const int *flags, int nx, int ny, int nz, int ng)
{
  long long idx = 0;
  int ir = 0, jr = 0, kr = 0;
  if (nx > 1) {
    if (ig < ng) {
      ir = find_index(ig, nx, flags[0], 0, ng, &a[0]);
    } else if (ig >= nx - ng) {
      ir = find_index(ig, nx, flags[1], 1, ng, &a[0]);
    } else {
      ir = ig;
    }
    if (ir < 0) return -1;
    idx += ir;
  }
  if (ny > 1) {
    if (jg < ng) {
      jr = find_index(jg, ny, flags[2], 0, ng, &a[1]);
    } else if (jg >= ny - ng) {
      jr = find_index(jg, ny, flags[3], 1, ng, &a[1]);
    } else {
      jr = jg;
    }
    if (jr < 0) return -1;
    idx += (long long)nx * jr;
  }
  if (nz > 1) {
    if (kg < ng) {
      kr = find_index(kg, nz, flags[4], 0, ng, &a[2]);
    } else if (kg >= nz - ng) {
      kr = find_index(kg, nz, flags[5], 1, ng, &a[2]);
    } else {
      kr = kg;
    }
    if (kr < 0) return -1;
    idx += (long long)nx * ny * kr;
  }
  return idx;
}
}  // namespace

void orc_set_boundaries(const orc_config *c, double *U, const int flags_in[6])
{
  Grid g(c);
  size_t const n = g.n;
  int const ng   = g.ng;
  int flags[6]   = {0, 0, 0, 0, 0, 0};
  if (g.nx > 1) flags[0] = flags_in[0], flags[1] = flags_in[1];
  if (g.ny > 1) flags[2] = flags_in[2], flags[3] = flags_in[3];
  if (g.nz > 1) flags[4] = flags_in[4], flags[5] = flags_in[5];
  for (int dir = 0; dir < 6; dir++) {
    if ((dir < 2 && g.nx <= 1) || (dir >= 2 && dir < 4 && g.ny <= 1) || (dir >= 4 && g.nz <= 1)) continue;
    if (flags[dir] == 4 || flags[dir] == 5) continue;
    // boundary_conditions.cpp Set_Boundary_Extents
    int imin[3] = {0, 0, 0}, imax[3] = {0, 0, 0};
    int jl = 0, ju = g.ny, kl = 0, ku = g.nz;
    if (g.ny > 1) jl = ng, ju = g.ny - ng;
    if (g.nz > 1) kl = ng, ku = g.nz - ng;
    if (dir == 0) imin[0] = 0, imax[0] = ng, imin[1] = jl, imax[1] = ju, imin[2] = kl, imax[2] = ku;
    if (dir == 1) imin[0] = g.nx - ng, imax[0] = g.nx, imin[1] = jl, imax[1] = ju, imin[2] = kl, imax[2] = ku;
    if (dir == 2) imin[0] = 0, imax[0] = g.nx, imin[1] = 0, imax[1] = ng, imin[2] = kl, imax[2] = ku;
    if (dir == 3) imin[0] = 0, imax[0] = g.nx, imin[1] = g.ny - ng, imax[1] = g.ny, imin[2] = kl, imax[2] = ku;
    if (dir == 4) imin[0] = 0, imax[0] = g.nx, imin[1] = 0, imax[1] = g.ny, imin[2] = 0, imax[2] = ng;
    if (dir == 5) imin[0] = 0, imax[0] = g.nx, imin[1] = 0, imax[1] = g.ny, imin[2] = g.nz - ng, imax[2] = g.nz;
    for (int k = imin[2]; k < imax[2]; k++)
      for (int j = imin[1]; j < imax[1]; j++)
        for (int i = imin[0]; i < imax[0]; i++) {
          size_t const gidx = g.id(i, j, k);
          double a[3]       = {1., 1., 1.};
          long long const idx = boundary_mapping(i, j, k, a, flags, g.nx, g.ny, g.nz, ng);
          if (idx < 0) continue;
          for (int f = 0; f < g.nf; f++) U[gidx + (size_t)f * n] = U[(size_t)idx + (size_t)f * n];
          if (flags[0] == 2 || flags[1] == 2) U[gidx + n] *= a[0];
          if (flags[2] == 2 || flags[3] == 2) U[gidx + 2 * n] *= a[1];
          if (flags[4] == 2 || flags[5] == 2) U[gidx + 3 * n] *= a[2];
          if (!g.mhd && flags[dir] == 3) {
            size_t const momdex = gidx + (size_t)(dir / 2 + 1) * n;
            if (dir % 2 == 0) {
              if (U[momdex] > 0.0) {
                U[gidx + 4 * n] -= 0.5 * (U[momdex] * U[momdex]) / U[gidx];
                U[momdex] = 0.0;
              }
            } else {
              if (U[momdex] < 0.0) {
                U[gidx + 4 * n] -= 0.5 * (U[momdex] * U[momdex]) / U[gidx];
                U[momdex] = 0.0;
              }
            }
          }
        }
  }
}

// src/integrators/VL_3D_cuda.cu:38-360 VL_Algorithm_3D_CUDA
int orc_vl_step_3d(const orc_config *c, double *U, double dt)
{
  Grid g(c);
  if (g.mhd && g.de) return -1;  // the reference's MHD+DE flux indexing is out of bounds
  if (g.mhd && c->solver != ORC_HLLD) return -1;
  if (!g.mhd && c->solver == ORC_HLLD) return -1;
  if (g.mhd && (c->recon == ORC_PLMP || c->recon == ORC_PPMP)) return -1;  // hydro-only kernels
  if (g.ns > MAXS) return -1;
  size_t const n = g.n;
  std::vector<double> Uh((size_t)g.nf * n, 0.0);
  std::vector<double> QLx((size_t)g.nf * n, 0.0), QRx((size_t)g.nf * n, 0.0), QLy((size_t)g.nf * n, 0.0),
      QRy((size_t)g.nf * n, 0.0), QLz((size_t)g.nf * n, 0.0), QRz((size_t)g.nf * n, 0.0);
  std::vector<double> Fx((size_t)g.nf * n, 0.0), Fy((size_t)g.nf * n, 0.0), Fz((size_t)g.nf * n, 0.0);
  std::vector<double> emf(g.mhd ? 3 * n : 0, 0.0);
  auto riemann = [&](const double *Ub) {
    if (c->solver == ORC_HLLC) {
      orc_hllc(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_hllc(c, QLy.data(), QRy.data(), Fy.data(), 1);
      orc_hllc(c, QLz.data(), QRz.data(), Fz.data(), 2);
    } else if (c->solver == ORC_ROE) {
      orc_roe(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_roe(c, QLy.data(), QRy.data(), Fy.data(), 1);
      orc_roe(c, QLz.data(), QRz.data(), Fz.data(), 2);
    } else if (c->solver == ORC_HLL) {
      orc_hll(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_hll(c, QLy.data(), QRy.data(), Fy.data(), 1);
      orc_hll(c, QLz.data(), QRz.data(), Fz.data(), 2);
    } else if (c->solver == ORC_EXACT) {
      orc_exact(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_exact(c, QLy.data(), QRy.data(), Fy.data(), 1);
      orc_exact(c, QLz.data(), QRz.data(), Fz.data(), 2);
    } else {
      orc_hlld(c, QLx.data(), QRx.data(), Ub + (size_t)g.fB * n, Fx.data(), 0);
      orc_hlld(c, QLy.data(), QRy.data(), Ub + (size_t)(g.fB + 1) * n, Fy.data(), 1);
      orc_hlld(c, QLz.data(), QRz.data(), Ub + (size_t)(g.fB + 2) * n, Fz.data(), 2);
    }
  };
  // predictor
  orc_pcm_3d(c, U, QLx.data(), QRx.data(), QLy.data(), QRy.data(), QLz.data(), QRz.data());
  riemann(U);
  if (g.mhd) orc_ct_electric_fields(c, Fx.data(), Fy.data(), Fz.data(), U, emf.data());
  orc_update_half(c, U, Uh.data(), Fx.data(), Fy.data(), Fz.data(), 0.5 * dt);
  if (g.mhd) orc_update_magnetic(c, U, Uh.data(), emf.data(), 0.5 * dt);
  // corrector
  if (c->recon == ORC_PCM) {
    orc_pcm_3d(c, Uh.data(), QLx.data(), QRx.data(), QLy.data(), QRy.data(), QLz.data(), QRz.data());
  } else if (c->recon == ORC_PLMC) {
    orc_plmc(c, Uh.data(), QLx.data(), QRx.data(), 0);
    orc_plmc(c, Uh.data(), QLy.data(), QRy.data(), 1);
    orc_plmc(c, Uh.data(), QLz.data(), QRz.data(), 2);
  } else if (c->recon == ORC_PLMP) {
    orc_plmp(c, Uh.data(), QLx.data(), QRx.data(), 0);
    orc_plmp(c, Uh.data(), QLy.data(), QRy.data(), 1);
    orc_plmp(c, Uh.data(), QLz.data(), QRz.data(), 2);
  } else if (c->recon == ORC_PPMP) {
    orc_ppmp(c, Uh.data(), QLx.data(), QRx.data(), 0);
    orc_ppmp(c, Uh.data(), QLy.data(), QRy.data(), 1);
    orc_ppmp(c, Uh.data(), QLz.data(), QRz.data(), 2);
  } else {
    orc_ppmc_vl(c, Uh.data(), QLx.data(), QRx.data(), 0);
    orc_ppmc_vl(c, Uh.data(), QLy.data(), QRy.data(), 1);
    orc_ppmc_vl(c, Uh.data(), QLz.data(), QRz.data(), 2);
  }
  riemann(Uh.data());
  if (g.de) orc_de_partial_update(c, U, dt);
  if (g.mhd) orc_ct_electric_fields(c, Fx.data(), Fy.data(), Fz.data(), Uh.data(), emf.data());
  orc_update_full(c, U, Fx.data(), Fy.data(), Fz.data(), dt);
  if (g.mhd) orc_update_magnetic(c, U, U, emf.data(), dt);
  if (g.de) {
    orc_de_select(c, U);
    orc_de_sync(c, U);
  }
  return 0;
}

// src/integrators/VL_1D_cuda.cu:30-146 VL_Algorithm_1D_CUDA and :158-215 Update_Conserved_Variables_1D_half
int orc_vl_step_1d(const orc_config *c, double *U, double dt)
{
  Grid g(c);
  if (g.mhd || g.ny != 1 || g.nz != 1 || c->solver == ORC_HLLD) return -1;
  // VL_1D_cuda.cu:69-80 and :112-123 have Riemann branches for the exact solver, Roe and HLLC
  // only: built with HLL, the 1D integrator computes no fluxes.
  if (c->solver == ORC_HLL) return -1;
  size_t const n = g.n;
  std::vector<double> Uh((size_t)g.nf * n, 0.0), QL((size_t)g.nf * n, 0.0), QR((size_t)g.nf * n, 0.0),
      F((size_t)g.nf * n, 0.0);
  auto pcm1 = [&](const double *Ub) {  // pcm_cuda.cu:13-121 PCM_Reconstruction_1D
    for (size_t x = 0; x + 1 < n; x++)
      for (int f = 0; f < g.nf; f++) {
        QL[(size_t)f * n + x] = Ub[(size_t)f * n + x];
        QR[(size_t)f * n + x] = Ub[(size_t)f * n + x + 1];
      }
  };
  auto riemann = [&]() {
    if (c->solver == ORC_ROE) {
      orc_roe(c, QL.data(), QR.data(), F.data(), 0);
    } else if (c->solver == ORC_EXACT) {
      orc_exact(c, QL.data(), QR.data(), F.data(), 0);
    } else {
      orc_hllc(c, QL.data(), QR.data(), F.data(), 0);
    }
  };
  pcm1(U);
  riemann();
  {
    double const dtodx = (0.5 * dt) / c->dx;
    for (size_t id = 1; id + 1 < n; id++) {
      size_t const imo = id - 1;
      double P = 0, vx_imo = 0, vx_ipo = 0;
      if (g.de) {
        double const d = U[id], d_inv = 1.0 / d;
        double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
        P      = (U[4 * n + id] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (g.gamma - 1.0);
        vx_imo = U[n + imo] / U[imo];
        vx_ipo = U[n + id + 1] / U[id + 1];
      }
      for (int f = 0; f < 5 + g.ns; f++)
        Uh[(size_t)f * n + id] = U[(size_t)f * n + id] + dtodx * (F[(size_t)f * n + imo] - F[(size_t)f * n + id]);
      if (g.de) {
        size_t const o = (size_t)g.fGE * n;
        Uh[o + id]     = U[o + id] + dtodx * (F[o + imo] - F[o + id]) + 0.5 * P * (dtodx * (vx_imo - vx_ipo));
      }
    }
  }
  if (c->recon == ORC_PCM) {
    pcm1(Uh.data());
  } else if (c->recon == ORC_PLMC) {
    orc_plmc(c, Uh.data(), QL.data(), QR.data(), 0);
  } else if (c->recon == ORC_PLMP) {
    orc_plmp(c, Uh.data(), QL.data(), QR.data(), 0);
  } else if (c->recon == ORC_PPMP) {
    orc_ppmp(c, Uh.data(), QL.data(), QR.data(), 0);
  } else {
    orc_ppmc_vl(c, Uh.data(), QL.data(), QR.data(), 0);
  }
  riemann();
  if (g.de) orc_de_partial_update(c, U, dt);
  update_full_1d(g, U, F.data(), c->dx, dt);
  if (g.de) {
    orc_de_select(c, U);
    orc_de_sync(c, U);
  }
  return 0;
}

// ---- the 2D VL step ----
// src/integrators/VL_2D_cuda.cu:25-174 VL_Algorithm_2D_CUDA on an nx x ny grid (nz = 1), with
// the 2D kernels of VL_2D_cuda.cu:176-258 and hydro_cuda.cu (Update_Conserved_Variables_2D,
// the 2D dual-energy kernels).  The 2D integrator has no density floor and no HLL branch.
int orc_vl_step_2d(const orc_config *c, double *U, double dt)
{
  Grid g(c);
  if (g.mhd || g.nz != 1 || g.ny < 2 || g.ns > MAXS) return -1;
  if (c->solver == ORC_HLLD || c->solver == ORC_HLL) return -1;
  size_t const n = g.n;
  int const nx = g.nx, ny = g.ny, ng = g.ng;
  std::vector<double> Uh((size_t)g.nf * n, 0.0);
  std::vector<double> QLx((size_t)g.nf * n, 0.0), QRx((size_t)g.nf * n, 0.0), QLy((size_t)g.nf * n, 0.0),
      QRy((size_t)g.nf * n, 0.0), Qz((size_t)g.nf * n, 0.0);
  std::vector<double> Fx((size_t)g.nf * n, 0.0), Fy((size_t)g.nf * n, 0.0);
  auto riemann = [&]() {
    if (c->solver == ORC_ROE) {
      orc_roe(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_roe(c, QLy.data(), QRy.data(), Fy.data(), 1);
    } else if (c->solver == ORC_EXACT) {
      orc_exact(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_exact(c, QLy.data(), QRy.data(), Fy.data(), 1);
    } else {
      orc_hllc(c, QLx.data(), QRx.data(), Fx.data(), 0);
      orc_hllc(c, QLy.data(), QRy.data(), Fy.data(), 1);
    }
  };
  auto interior = [&](int x, int y) { return x > ng - 1 && x < nx - ng && y > ng - 1 && y < ny - ng; };
  // pcm_cuda.cu:123-254 PCM_Reconstruction_2D: the 3D form's x and y faces on a one-cell-deep grid
  orc_pcm_3d(c, U, QLx.data(), QRx.data(), QLy.data(), QRy.data(), Qz.data(), Qz.data());
  riemann();
  {  // VL_2D_cuda.cu:176-258 Update_Conserved_Variables_2D_half
    double const hdt = 0.5 * dt, dtodx = hdt / c->dx, dtody = hdt / c->dy;
    par_cells(g, [&](size_t id) {
      int x, y, z;
      g.xyz(id, x, y, z);
      if (!(x > 0 && x < nx - 1 && y > 0 && y < ny - 1)) return;
      size_t const imo = id - 1, jmo = id - nx, ipo = id + 1, jpo = id + nx;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const P  = (U[4 * n + id] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (g.gamma - 1.0);
      auto upd        = [&](size_t f) {
        return U[f * n + id] + dtodx * (Fx[f * n + imo] - Fx[f * n + id]) + dtody * (Fy[f * n + jmo] - Fy[f * n + id]);
      };
      for (int f = 0; f < 5 + g.ns; f++) Uh[(size_t)f * n + id] = upd((size_t)f);
      if (g.de) {
        double const vx_imo = U[n + imo] / U[imo], vx_ipo = U[n + ipo] / U[ipo];
        double const vy_jmo = U[2 * n + jmo] / U[jmo], vy_jpo = U[2 * n + jpo] / U[jpo];
        Uh[(size_t)g.fGE * n + id] =
            upd((size_t)g.fGE) + 0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo));
      }
    });
  }
  // VL_2D_cuda.cu:97-122 reconstructs U-half only for PLMP, PLMC, PPMP and PPMC: with PCM the
  // corrector's Riemann solve reads the predictor's interface states of Un again.
  if (c->recon != ORC_PCM) {
    void (*recon)(const orc_config *, const double *, double *, double *, int) =
        c->recon == ORC_PLMC ? orc_plmc : c->recon == ORC_PLMP ? orc_plmp : c->recon == ORC_PPMP ? orc_ppmp : orc_ppmc_vl;
    recon(c, Uh.data(), QLx.data(), QRx.data(), 0);
    recon(c, Uh.data(), QLy.data(), QRy.data(), 1);
  }
  riemann();
  double const dtodx = dt / c->dx, dtody = dt / c->dy;
  if (g.de) {  // hydro_cuda.cu:725-752 Partial_Update_Advected_Internal_Energy_2D (reads U only)
    par_cells(g, [&](size_t id) {
      int x, y, z;
      g.xyz(id, x, y, z);
      if (!interior(x, y)) return;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const E = U[4 * n + id], GE = U[(size_t)g.fGE * n + id];
      double const Ekin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double const P    = fmax(pressure_from_de(E, E - Ekin, GE, g.gamma), TINY);
      size_t const imo = id - 1, ipo = id + 1, jmo = id - nx, jpo = id + nx;
      double const vx_imo = U[n + imo] / U[imo], vx_ipo = U[n + ipo] / U[ipo];
      double const vy_jmo = U[2 * n + jmo] / U[jmo], vy_jpo = U[2 * n + jpo] / U[jpo];
      U[(size_t)g.fGE * n + id] += 0.5 * P * (dtodx * (vx_imo - vx_ipo) + dtody * (vy_jmo - vy_jpo));
    });
  }
  // hydro_cuda.cu:87-170 Update_Conserved_Variables_2D: U += (x difference + y difference)
  par_cells(g, [&](size_t id) {
    int x, y, z;
    g.xyz(id, x, y, z);
    if (!interior(x, y)) return;
    size_t const imo = id - 1, jmo = id - nx;
    for (int f = 0; f < g.nf; f++) {
      size_t const o = (size_t)f * n;
      U[o + id] += dtodx * (Fx[o + imo] - Fx[o + id]) + dtody * (Fy[o + jmo] - Fy[o + id]);
    }
  });
  if (g.de) {
    // hydro_cuda.cu:880-933 Select_Internal_Energy_2D: neighbour maximum of E over the four
    // face neighbours, indices clamped to the real cells
    std::vector<double> GEsel(n, 0.0);
    par_cells(g, [&](size_t id) {
      int x, y, z;
      g.xyz(id, x, y, z);
      if (!interior(x, y)) return;
      size_t const imo = (size_t)std::max(x - 1, ng) + (size_t)y * nx;
      size_t const ipo = (size_t)std::min(x + 1, nx - ng - 1) + (size_t)y * nx;
      size_t const jmo = (size_t)x + (size_t)std::max(y - 1, ng) * nx;
      size_t const jpo = (size_t)x + (size_t)std::min(y + 1, ny - ng - 1) * nx;
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      double const E   = U[4 * n + id];
      double const Uad = U[(size_t)g.fGE * n + id];
      double const Utot = E - 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double Emax       = fmax(U[4 * n + imo], E);
      Emax              = fmax(Emax, U[4 * n + ipo]);
      Emax              = fmax(Emax, U[4 * n + jmo]);
      Emax              = fmax(Emax, U[4 * n + jpo]);
      double const Usel = (Utot / E > ETA_1 || Utot / Emax > ETA_2) ? Utot : Uad;
      GEsel[id]         = fmax(Usel, TINY);
    });
    // hydro_cuda.cu:1035-1068 Sync_Energies_2D: E = kinetic + selected internal energy
    par_cells(g, [&](size_t id) {
      int x, y, z;
      g.xyz(id, x, y, z);
      if (!interior(x, y)) return;
      U[(size_t)g.fGE * n + id] = GEsel[id];
      double const d = U[id], d_inv = 1.0 / d;
      double const vx = U[n + id] * d_inv, vy = U[2 * n + id] * d_inv, vz = U[3 * n + id] * d_inv;
      U[4 * n + id] = 0.5 * d * (vx * vx + vy * vy + vz * vz) + GEsel[id];
    });
  }
  return 0;
}

}  // extern "C"
