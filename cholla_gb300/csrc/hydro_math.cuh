// hydro_math.cuh -- per-cell and per-face hydro arithmetic of the VL step, FP64.
//
// These device functions keep the operation order of the reference kernels they
// replace (file:line beside each).  Compiled in a translation unit built with
// -fmad=false, they reproduce the reference's FP64 results bit for bit; the fused
// kernels around them only change where intermediate values live (registers and
// shared memory instead of full-grid interface and flux arrays in HBM).
//
// States are "rotated" for the sweep direction: q[0]=d, q[1]=m_normal, q[2]=m_t1,
// q[3]=m_t2, q[4]=E, q[5..5+ns)=scalars, q[5+ns]=GasEnergy (when DE is on), with
// (normal, t1, t2) = (x,y,z), (y,z,x), (z,x,y) for sweeps in x, y, z
// (the o1/o2/o3 permutation of src/riemann_solvers/hllc_cuda.cu:54-70).
#pragma once
#include "common.cuh"

namespace cgb
{
namespace hx  // exact FP64 hydro
{

__device__ __forceinline__ double sqmag(double a, double b, double c)  // math_utilities.h dotProduct
{
  return a * a + ((b * b) + (c * c));
}

__device__ __forceinline__ double sgn(double a) { return (a < 0.) ? -1. : 1.; }  // global.h SIGN

// hydro_utilities.h:136-151 Get_Pressure_From_DE
__device__ __forceinline__ double pressure_de(double E, double U_total, double U_adv, double gamma)
{
  double U = (U_total / E > ETA_1) ? U_total : U_adv;
  double P = U * (gamma - 1.0);
  return fmax(P, TINY);
}

struct Prim {
  double d, vn, vt1, vt2, p, ge;
  double sc[NS_MAX];
};

// reconstruction.h:139-212 Load_Data, hydro part, from a rotated conserved state.
__device__ __forceinline__ Prim load_prim(const double *q, int ns, int de, double gamma)
{
  Prim P;
  P.d   = q[0];
  P.vn  = q[1] / P.d;
  P.vt1 = q[2] / P.d;
  P.vt2 = q[3] / P.d;
  P.ge  = 0.0;
  if (de) {
    double const E   = q[4];
    double const GE  = q[5 + ns];
    double const Ent = 0.5 * P.d * sqmag(P.vn, P.vt1, P.vt2);
    P.p              = pressure_de(E, E - Ent, GE, gamma);
    P.ge             = GE / P.d;
  } else {
    double const pressure = q[4] - 0.5 * P.d * sqmag(P.vn, P.vt1, P.vt2);
    P.p                   = fmax((gamma - 1.) * pressure, TINY);
  }
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) P.sc[k] = (k < ns) ? q[5 + k] / P.d : 0.0;
  return P;
}

// reconstruction.h:918-968 Write_Data (hydro): primitive interface state -> rotated conserved.
__device__ __forceinline__ void prim_to_q(const Prim &s, double *q, int ns, int de, double gamma)
{
  q[0] = s.d;
  q[1] = s.d * s.vn;
  q[2] = s.d * s.vt1;
  q[3] = s.d * s.vt2;
  // hydro_utilities.h:106-118 Calc_Energy_Primitive
  q[4] = (fmax(s.p, TINY) / (gamma - 1.)) + 0.5 * s.d * sqmag(s.vn, s.vt1, s.vt2);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) q[5 + k] = s.d * s.sc[k];
  if (de) q[5 + ns] = s.d * s.ge;
}

// reconstruction.h:794-901 PPM_Single_Variable
__device__ __forceinline__ void ppm1(double im2, double im1, double i, double ip1, double ip2, double &L_iph,
                                     double &R_imh)
{
  double const C2 = 1.25;
  auto limit = [&C2](double ci, double cim1, double iface, double s2i, double s2im1) -> double {
    double s2c = 3.0 * (cim1 + ci - 2.0 * iface);
    double lim = 0.0;
    if (sgn(s2c) == sgn(s2im1) and sgn(s2c) == sgn(s2i)) {
      lim = sgn(s2c) * fmin(C2 * fabs(s2im1), fmin(C2 * fabs(s2i), fabs(s2c)));
    }
    double const dl = iface - cim1;
    double const dr = ci - iface;
    return (dl * dr < 0.0) ? 0.5 * (cim1 + ci) - lim / 6.0 : iface;
  };
  double const sl    = (i - im1);
  double const sr    = (ip1 - i);
  double const sim1  = 0.5 * sl + 0.5 * (im1 - im2);
  double const si    = 0.5 * sr + 0.5 * sl;
  double const sip1  = 0.5 * (ip2 - ip1) + 0.5 * sr;
  double R           = 0.5 * (im1 + i) + (sim1 - si) / 6.0;
  double L           = 0.5 * (i + ip1) + (si - sip1) / 6.0;
  double const d2im1 = im2 + i - 2.0 * im1;
  double const d2i   = im1 + ip1 - 2.0 * i;
  double const d2ip1 = i + ip2 - 2.0 * ip1;
  R                  = limit(i, im1, R, d2i, d2im1);
  L                  = limit(ip1, i, L, d2ip1, d2i);
  double const d2f   = 6.0 * (R + L - 2.0 * i);
  double d2lim       = 0.0;
  if (sgn(d2im1) == sgn(d2i) and sgn(d2im1) == sgn(d2ip1) and sgn(d2im1) == sgn(d2f)) {
    d2lim = sgn(d2f) * fmin(fmin(C2 * fabs(d2im1), C2 * fabs(d2i)), fmin(C2 * fabs(d2ip1), fabs(d2f)));
  }
  double cmax      = fmax(fabs(im2), fabs(im1));
  cmax             = fmax(cmax, fabs(i));
  cmax             = fmax(cmax, fabs(ip1));
  cmax             = fmax(cmax, fabs(ip2));
  double const rho = (fabs(d2f) > (1.0e-12) * cmax) ? d2lim / d2f : 0.0;
  double const sfl = i - R;
  double const sfr = L - i;
  if ((sfl * sfr) <= 0.0 or ((ip1 - i) * (i - im1)) <= 0.0) {
    if (rho <= (1.0 - (1.0e-12))) {
      R = i - rho * sfl;
      L = i + rho * sfr;
    }
  } else {
    if (fabs(sfl) >= 2.0 * fabs(sfr)) R = i - 2.0 * sfr;
    if (fabs(sfr) >= 2.0 * fabs(sfl)) L = i + 2.0 * sfl;
  }
  L_iph = L;
  R_imh = R;
}

// ppmc_cuda.cu:540-695 PPMC_VL for one cell (hydro): 5-cell stencil of primitives ->
// left state at i+1/2 and right state at i-1/2, limited in the characteristic variables.
__device__ __forceinline__ void ppmc_cell(const Prim &cm2, const Prim &cm1, const Prim &c, const Prim &cp1,
                                          const Prim &cp2, int ns, int de, double gamma, Prim &L, Prim &R)
{
  double const cs  = sqrt(gamma * c.p / c.d);  // hydro_utilities.h:209 Calc_Sound_Speed
  double const cs2 = cs * cs;
  // reconstruction.h:378-437 Primitive_To_Characteristic (hydro)
  auto a0 = [&](const Prim &s) { return -c.d * s.vn / (2.0 * cs) + s.p / (2.0 * cs2); };
  auto a1 = [&](const Prim &s) { return s.d - s.p / (cs2); };
  auto a4 = [&](const Prim &s) { return c.d * s.vn / (2.0 * cs) + s.p / (2.0 * cs2); };
  double l0, r0, l1, r1, l2, r2, l3, r3, l4, r4;
  ppm1(a0(cm2), a0(cm1), a0(c), a0(cp1), a0(cp2), l0, r0);
  ppm1(a1(cm2), a1(cm1), a1(c), a1(cp1), a1(cp2), l1, r1);
  ppm1(cm2.vt1, cm1.vt1, c.vt1, cp1.vt1, cp2.vt1, l2, r2);
  ppm1(cm2.vt2, cm1.vt2, c.vt2, cp1.vt2, cp2.vt2, l3, r3);
  ppm1(a4(cm2), a4(cm1), a4(c), a4(cp1), a4(cp2), l4, r4);
  // reconstruction.h:453-491 Characteristic_To_Primitive (hydro)
  L.d   = l0 + l1 + l4;
  L.vn  = cs / c.d * (l4 - l0);
  L.vt1 = l2;
  L.vt2 = l3;
  L.p   = cs2 * (l0 + l4);
  R.d   = r0 + r1 + r4;
  R.vn  = cs / c.d * (r4 - r0);
  R.vt1 = r2;
  R.vt2 = r3;
  R.p   = cs2 * (r0 + r4);
  L.ge = R.ge = 0.0;
  if (de) ppm1(cm2.ge, cm1.ge, c.ge, cp1.ge, cp2.ge, L.ge, R.ge);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) {
    L.sc[k] = R.sc[k] = 0.0;
    if (k < ns) ppm1(cm2.sc[k], cm1.sc[k], c.sc[k], cp1.sc[k], cp2.sc[k], L.sc[k], R.sc[k]);
  }
  R.d = fmax(R.d, TINY);
  L.d = fmax(L.d, TINY);
  R.p = fmax(R.p, TINY);
  L.p = fmax(L.p, TINY);
}

// plmc_cuda.cu:24-300 PLMC_cuda for one cell (hydro, VL: no characteristic tracing).
__device__ __forceinline__ void plmc_cell(const Prim &cm, const Prim &c, const Prim &cp, int ns, int de,
                                          double gamma, Prim &L, Prim &R)
{
  double const cs  = sqrt(gamma * c.p / c.d);
  double const cs2 = cs * cs;
  auto vl = [](double l, double r) -> double { return (l * r > 0.0) ? 2.0 * l * r / (l + r) : 0.0; };
  // reconstruction.h:512-559 Monotonize
  auto mono = [](double l, double r, double cc, double vg) -> double {
    if (l * r > 0.0) {
      double const la = 2.0 * fmin(fabs(l), fabs(r));
      double const lb = fmin(fabs(cc), fabs(vg));
      return copysign(fmin(la, lb), cc);
    }
    return 0.0;
  };
  // slopes (reconstruction.h:224-296)
  double const dLd = 1.0 * (c.d - cm.d), dRd = 1.0 * (cp.d - c.d), dCd = 0.5 * (cp.d - cm.d);
  double const dLn = 1.0 * (c.vn - cm.vn), dRn = 1.0 * (cp.vn - c.vn), dCn = 0.5 * (cp.vn - cm.vn);
  double const dL1 = 1.0 * (c.vt1 - cm.vt1), dR1 = 1.0 * (cp.vt1 - c.vt1), dC1 = 0.5 * (cp.vt1 - cm.vt1);
  double const dL2 = 1.0 * (c.vt2 - cm.vt2), dR2 = 1.0 * (cp.vt2 - c.vt2), dC2 = 0.5 * (cp.vt2 - cm.vt2);
  double const dLp = 1.0 * (c.p - cm.p), dRp = 1.0 * (cp.p - c.p), dCp = 0.5 * (cp.p - cm.p);
  double const dGd = vl(dLd, dRd), dGn = vl(dLn, dRn), dG1 = vl(dL1, dR1), dG2 = vl(dL2, dR2), dGp = vl(dLp, dRp);
  // characteristic projections (hydro)
  auto a0 = [&](double sd, double sn, double sp) {
    (void)sd;
    return -c.d * sn / (2.0 * cs) + sp / (2.0 * cs2);
  };
  auto a1 = [&](double sd, double sn, double sp) {
    (void)sn;
    return sd - sp / (cs2);
  };
  auto a4 = [&](double sd, double sn, double sp) {
    (void)sd;
    return c.d * sn / (2.0 * cs) + sp / (2.0 * cs2);
  };
  double const m0 = mono(a0(dLd, dLn, dLp), a0(dRd, dRn, dRp), a0(dCd, dCn, dCp), a0(dGd, dGn, dGp));
  double const m1 = mono(a1(dLd, dLn, dLp), a1(dRd, dRn, dRp), a1(dCd, dCn, dCp), a1(dGd, dGn, dGp));
  double const m2 = mono(dL1, dR1, dC1, dG1);
  double const m3 = mono(dL2, dR2, dC2, dG2);
  double const m4 = mono(a4(dLd, dLn, dLp), a4(dRd, dRn, dRp), a4(dCd, dCn, dCp), a4(dGd, dGn, dGp));
  // back to primitive slopes
  double const sd = m0 + m1 + m4;
  double const sn = cs / c.d * (m4 - m0);
  double const s1 = m2;
  double const s2 = m3;
  double const sp = cs2 * (m0 + m4);
  auto lin = [](double st, double sl, double sign) { return st + sign * 0.5 * sl; };
  L.d   = lin(c.d, sd, 1.0);
  L.vn  = lin(c.vn, sn, 1.0);
  L.vt1 = lin(c.vt1, s1, 1.0);
  L.vt2 = lin(c.vt2, s2, 1.0);
  L.p   = lin(c.p, sp, 1.0);
  R.d   = lin(c.d, sd, -1.0);
  R.vn  = lin(c.vn, sn, -1.0);
  R.vt1 = lin(c.vt1, s1, -1.0);
  R.vt2 = lin(c.vt2, s2, -1.0);
  R.p   = lin(c.p, sp, -1.0);
  // reconstruction.h:686-723 Plm_Limit_Interfaces
  auto lim = [](double &l, double &r, double vm, double vi, double vp) {
    r = fmax(fmin(vi, vm), r);
    r = fmin(fmax(vi, vm), r);
    l = fmax(fmin(vi, vp), l);
    l = fmin(fmax(vi, vp), l);
  };
  lim(L.d, R.d, cm.d, c.d, cp.d);
  lim(L.vn, R.vn, cm.vn, c.vn, cp.vn);
  lim(L.vt1, R.vt1, cm.vt1, c.vt1, cp.vt1);
  lim(L.vt2, R.vt2, cm.vt2, c.vt2, cp.vt2);
  lim(L.p, R.p, cm.p, c.p, cp.p);
  L.ge = R.ge = 0.0;
  if (de) {
    double const dL = 1.0 * (c.ge - cm.ge), dR = 1.0 * (cp.ge - c.ge), dC = 0.5 * (cp.ge - cm.ge);
    double const s  = mono(dL, dR, dC, vl(dL, dR));
    L.ge            = lin(c.ge, s, 1.0);
    R.ge            = lin(c.ge, s, -1.0);
    lim(L.ge, R.ge, cm.ge, c.ge, cp.ge);
  }
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) {
    L.sc[k] = R.sc[k] = 0.0;
    if (k < ns) {
      double const dL = 1.0 * (c.sc[k] - cm.sc[k]), dR = 1.0 * (cp.sc[k] - c.sc[k]),
                   dC = 0.5 * (cp.sc[k] - cm.sc[k]);
      double const s  = mono(dL, dR, dC, vl(dL, dR));
      L.sc[k]         = lin(c.sc[k], s, 1.0);
      R.sc[k]         = lin(c.sc[k], s, -1.0);
      lim(L.sc[k], R.sc[k], cm.sc[k], c.sc[k], cp.sc[k]);
    }
  }
  R.d = fmax(R.d, TINY);
  L.d = fmax(L.d, TINY);
  R.p = fmax(R.p, TINY);
  L.p = fmax(L.p, TINY);
}

// hllc_cuda.cu:19-307 Calculate_HLLC_Fluxes_CUDA for one face, rotated conserved states.
__device__ __forceinline__ void hllc(const double *qL, const double *qR, double *f, int ns, int de, double gamma)
{
  double const g1 = gamma - 1.0;
  double const dl = qL[0], mxl = qL[1], myl = qL[2], mzl = qL[3], El = qL[4];
  double const dr = qR[0], mxr = qR[1], myr = qR[2], mzr = qR[3], Er = qR[4];
  double const dgel = de ? qL[5 + ns] : 0.0, dger = de ? qR[5 + ns] : 0.0;
  double const vxl = mxl / dl, vyl = myl / dl, vzl = mzl / dl;
  double pl;
  if (de) {
    double const E_kin = 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl);
    pl                 = pressure_de(El, El - E_kin, dgel, gamma);
  } else {
    pl = (El - 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl)) * (gamma - 1.0);
  }
  pl = fmax(pl, TINY);
  double const gel = de ? dgel / dl : 0.0;
  double const vxr = mxr / dr, vyr = myr / dr, vzr = mzr / dr;
  double pr;
  if (de) {
    double const E_kin = 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr);
    pr                 = pressure_de(Er, Er - E_kin, dger, gamma);
  } else {
    pr = (Er - 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr)) * (gamma - 1.0);
  }
  pr = fmax(pr, TINY);
  double const ger    = de ? dger / dr : 0.0;
  double const Hl     = (El + pl) / dl;
  double const Hr     = (Er + pr) / dr;
  double const sqrtdl = sqrt(dl);
  double const sqrtdr = sqrt(dr);
  double const vx     = (sqrtdl * vxl + sqrtdr * vxr) / (sqrtdl + sqrtdr);
  double const vy     = (sqrtdl * vyl + sqrtdr * vyr) / (sqrtdl + sqrtdr);
  double const vz     = (sqrtdl * vzl + sqrtdr * vzr) / (sqrtdl + sqrtdr);
  double const H      = (sqrtdl * Hl + sqrtdr * Hr) / (sqrtdl + sqrtdr);
  double const vsq    = (vx * vx + vy * vy + vz * vz);
  double const asq    = g1 * (H - 0.5 * vsq);
  double const a      = sqrt(asq);
  double const cfl    = sqrt(gamma * pl / dl);
  double const cfr    = sqrt(gamma * pr / dr);
  double Sl           = fmin(vx - a, vxl - cfl);
  double Sr           = fmax(vx + a, vxr + cfr);
  // h-correction with etah = 0 (hllc_cuda.cu:52, 181-183)
  Sl = ((Sl < 0) ? -1 : 1) * fmax(fabs(Sl), 0.0);
  Sr = ((Sr < 0) ? -1 : 1) * fmax(fabs(Sr), 0.0);
  if (Sl > 0.0) {
    f[0] = mxl;
    f[1] = mxl * vxl + pl;
    f[2] = myl * vxl;
    f[3] = mzl * vxl;
    f[4] = (El + pl) * vxl;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[5 + k] = qL[5 + k] * vxl;
    if (de) f[5 + ns] = dgel * vxl;
    return;
  }
  if (Sr < 0.0) {
    f[0] = mxr;
    f[1] = mxr * vxr + pr;
    f[2] = myr * vxr;
    f[3] = mzr * vxr;
    f[4] = (Er + pr) * vxr;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[5 + k] = qR[5 + k] * vxr;
    if (de) f[5 + ns] = dger * vxr;
    return;
  }
  double const f_d_l = mxl, f_mx_l = mxl * vxl + pl, f_my_l = myl * vxl, f_mz_l = mzl * vxl, f_E_l = (El + pl) * vxl;
  double const f_d_r = mxr, f_mx_r = mxr * vxr + pr, f_my_r = myr * vxr, f_mz_r = mzr * vxr, f_E_r = (Er + pr) * vxr;
  double const Sm   = (dr * vxr * (Sr - vxr) - dl * vxl * (Sl - vxl) + pl - pr) / (dr * (Sr - vxr) - dl * (Sl - vxl));
  double const ps   = dl * (vxl - Sl) * (vxl - Sm) + pl;
  double const dls  = dl * (Sl - vxl) / (Sl - Sm);
  double const mxls = (mxl * (Sl - vxl) + ps - pl) / (Sl - Sm);
  double const myls = dls * vyl;
  double const mzls = dls * vzl;
  double const Els  = (El * (Sl - vxl) - pl * vxl + ps * Sm) / (Sl - Sm);
  double const drs  = dr * (Sr - vxr) / (Sr - Sm);
  double const mxrs = (mxr * (Sr - vxr) + ps - pr) / (Sr - Sm);
  double const myrs = drs * vyr;
  double const mzrs = drs * vzr;
  double const Ers  = (Er * (Sr - vxr) - pr * vxr + ps * Sm) / (Sr - Sm);
  double const aSm  = fabs(Sm);
  f[0] = 0.5 * (f_d_l + f_d_r + (Sr - aSm) * drs + (Sl + aSm) * dls - Sl * dl - Sr * dr);
  f[1] = 0.5 * (f_mx_l + f_mx_r + (Sr - aSm) * mxrs + (Sl + aSm) * mxls - Sl * mxl - Sr * mxr);
  f[2] = 0.5 * (f_my_l + f_my_r + (Sr - aSm) * myrs + (Sl + aSm) * myls - Sl * myl - Sr * myr);
  f[3] = 0.5 * (f_mz_l + f_mz_r + (Sr - aSm) * mzrs + (Sl + aSm) * mzls - Sl * mzl - Sr * mzr);
  f[4] = 0.5 * (f_E_l + f_E_r + (Sr - aSm) * Ers + (Sl + aSm) * Els - Sl * El - Sr * Er);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) {
    if (k < ns) {
      double const dscl = qL[5 + k], dscr = qR[5 + k];
      double const scls = dls * (dscl / dl), scrs = drs * (dscr / dr);
      f[5 + k] = 0.5 * (dscl * vxl + dscr * vxr + (Sr - aSm) * scrs + (Sl + aSm) * scls - Sl * dscl - Sr * dscr);
    }
  }
  if (de) {
    double const gels = dls * gel, gers = drs * ger;
    f[5 + ns] = 0.5 * (dgel * vxl + dger * vxr + (Sr - aSm) * gers + (Sl + aSm) * gels - Sl * dgel - Sr * dger);
  }
}

// roe_cuda.cu:19-400 Calculate_Roe_Fluxes_CUDA for one face, with its HLLE fallback.
__device__ __forceinline__ void roe(const double *qL, const double *qR, double *f, int ns, int de, double gamma)
{
  double const etah = 0.0;
  double const g1   = gamma - 1.0;
  double const dl = qL[0], mxl = qL[1], myl = qL[2], mzl = qL[3], El = qL[4];
  double const dr = qR[0], mxr = qR[1], myr = qR[2], mzr = qR[3], Er = qR[4];
  double const dgel = de ? qL[5 + ns] : 0.0, dger = de ? qR[5 + ns] : 0.0;
  double const vxl = mxl / dl, vyl = myl / dl, vzl = mzl / dl;
  double pl;
  if (de) {
    double const E_kin = 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl);
    pl                 = pressure_de(El, El - E_kin, dgel, gamma);
  } else {
    pl = (El - 0.5 * dl * (vxl * vxl + vyl * vyl + vzl * vzl)) * (gamma - 1.0);
  }
  pl = fmax(pl, TINY);
  double scl[NS_MAX], scr[NS_MAX];
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) scl[k] = (k < ns) ? qL[5 + k] / dl : 0.0;
  double const gel = de ? dgel / dl : 0.0;
  double const vxr = mxr / dr, vyr = myr / dr, vzr = mzr / dr;
  double pr;
  if (de) {
    double const E_kin = 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr);
    pr                 = pressure_de(Er, Er - E_kin, dger, gamma);
  } else {
    pr = (Er - 0.5 * dr * (vxr * vxr + vyr * vyr + vzr * vzr)) * (gamma - 1.0);
  }
  pr = fmax(pr, TINY);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) scr[k] = (k < ns) ? qR[5 + k] / dr : 0.0;
  double const ger      = de ? dger / dr : 0.0;
  double const Hl       = (El + pl) / dl;
  double const Hr       = (Er + pr) / dr;
  double const sqrtdl   = sqrt(dl);
  double const sqrtdr   = sqrt(dr);
  double const vx       = (sqrtdl * vxl + sqrtdr * vxr) / (sqrtdl + sqrtdr);
  double const vy       = (sqrtdl * vyl + sqrtdr * vyr) / (sqrtdl + sqrtdr);
  double const vz       = (sqrtdl * vzl + sqrtdr * vzr) / (sqrtdl + sqrtdr);
  double const H        = (sqrtdl * Hl + sqrtdr * Hr) / (sqrtdl + sqrtdr);
  double const vsq      = (vx * vx + vy * vy + vz * vz);
  double const asq      = g1 * fmax((H - 0.5 * vsq), TINY);
  double const a        = sqrt(asq);
  double const lambda_m = vx - a, lambda_0 = vx, lambda_p = vx + a;
  double f_d_l = mxl, f_mx_l = mxl * vxl + pl, f_my_l = mxl * vyl, f_mz_l = mxl * vzl, f_E_l = (El + pl) * vxl;
  double f_d_r = mxr, f_mx_r = mxr * vxr + pr, f_my_r = mxr * vyr, f_mz_r = mxr * vzr, f_E_r = (Er + pr) * vxr;
  double f_ge_l = mxl * gel, f_ge_r = mxr * ger;
  if (lambda_m >= 0.0) {
    f[0] = f_d_l, f[1] = f_mx_l, f[2] = f_my_l, f[3] = f_mz_l, f[4] = f_E_l;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[5 + k] = mxl * scl[k];
    if (de) f[5 + ns] = f_ge_l;
    return;
  }
  if (lambda_p <= 0.0) {
    f[0] = f_d_r, f[1] = f_mx_r, f[2] = f_my_r, f[3] = f_mz_r, f[4] = f_E_r;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[5 + k] = mxr * scr[k];
    if (de) f[5 + ns] = f_ge_r;
    return;
  }
  double sum_0 = 0.0, sum_1 = 0.0, sum_2 = 0.0, sum_3 = 0.0, sum_4 = 0.0;
  double const del_d = dr - dl, del_mx = mxr - mxl, del_my = myr - myl, del_mz = mzr - mzl, del_E = Er - El;
  double const Na = 0.5 / asq;
  double coeff;
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
    f_ge_l           = dgel * (vxl - bm);
    f_ge_r           = dger * (vxr - bp);
    double const tmp = 0.5 * (bp + bm) / (bp - bm);
    f[0]             = 0.5 * (f_d_l + f_d_r) + (f_d_l - f_d_r) * tmp;
    f[1]             = 0.5 * (f_mx_l + f_mx_r) + (f_mx_l - f_mx_r) * tmp;
    f[2]             = 0.5 * (f_my_l + f_my_r) + (f_my_l - f_my_r) * tmp;
    f[3]             = 0.5 * (f_mz_l + f_mz_r) + (f_mz_l - f_mz_r) * tmp;
    f[4]             = 0.5 * (f_E_l + f_E_r) + (f_E_l - f_E_r) * tmp;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++) {
      if (k < ns) {
        double const fl = qL[5 + k] * (vxl - bm), fr = qR[5 + k] * (vxr - bp);
        f[5 + k]        = 0.5 * (fl + fr) + (fl - fr) * tmp;
      }
    }
    if (de) f[5 + ns] = 0.5 * (f_ge_l + f_ge_r) + (f_ge_l - f_ge_r) * tmp;
    return;
  }
  f[0] = 0.5 * (f_d_l + f_d_r - sum_0);
  f[1] = 0.5 * (f_mx_l + f_mx_r - sum_1);
  f[2] = 0.5 * (f_my_l + f_my_r - sum_2);
  f[3] = 0.5 * (f_mz_l + f_mz_r - sum_3);
  f[4] = 0.5 * (f_E_l + f_E_r - sum_4);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) f[5 + k] = (f[0] >= 0.0) ? f[0] * scl[k] : f[0] * scr[k];
  if (de) f[5 + ns] = (f[0] >= 0.0) ? f[0] * gel : f[0] * ger;
}

// ---- primitive-limited reconstructions (the VL build of plmp_cuda.cu:21-328 and
// ppmp_cuda.cu:28-683: no half-step tracing, no flattening or steepening): every primitive is
// limited on its own, with no characteristic projection ----

__device__ __forceinline__ int sgn_int(double x) { return (x < 0) ? -1 : 1; }  // global_cuda.h:41-48

// One cell's primitives as PLMP_cuda / PPMP_cuda load them (plmp_cuda.cu:108-133,
// ppmp_cuda.cu:155-180) from a rotated conserved state: velocities by division, the kinetic
// energy summed in the sweep's order, pressure from the total energy (dual energy: the select of
// Get_Pressure_From_DE) floored at TINY, scalars and GasEnergy per unit mass.
__device__ __forceinline__ Prim load_prim_plm(const double *q, int ns, int de, double gamma)
{
  Prim P;
  P.d   = q[0];
  P.vn  = q[1] / P.d;
  P.vt1 = q[2] / P.d;
  P.vt2 = q[3] / P.d;
  P.ge  = 0.0;
  double p;
  if (de) {
    double const E    = q[4];
    double const Ekin = 0.5 * P.d * (P.vn * P.vn + P.vt1 * P.vt1 + P.vt2 * P.vt2);
    double const dge  = q[5 + ns];
    p                 = pressure_de(E, E - Ekin, dge, gamma);
    P.ge              = dge / P.d;
  } else {
    p = (q[4] - 0.5 * P.d * (P.vn * P.vn + P.vt1 * P.vt1 + P.vt2 * P.vt2)) * (gamma - 1.0);
  }
  P.p = fmax(p, TINY);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++) P.sc[k] = (k < ns) ? q[5 + k] / P.d : 0.0;
  return P;
}

// Van Leer-limited slope of a three-point stencil (plmp_cuda.cu:330-365 Interface_Values_PLM,
// ppmp_cuda.cu:687-720 Calculate_Slope): monotonised central difference with the harmonic mean.
__device__ __forceinline__ double limited_slope(double qm, double q, double qp)
{
  double const dl = q - qm, dr = qp - q, dc = 0.5 * (qp - qm);
  double const dg = (dl * dr > 0.0) ? 2.0 * dl * dr / (dl + dr) : 0.0;
  double const a = fmin(fabs(dl), fabs(dr)), b = fmin(fabs(dc), fabs(dg));
  return sgn_int(dc) * fmin(2.0 * a, b);
}

// Fryxell et al. (2000) parabola through cell i with its monotonicity constraints
// (ppmp_cuda.cu:727-752 Interface_Values_PPM): L at the cell's low face, R at its high face.
__device__ __forceinline__ void ppm_parabola(double qm, double q, double qp, double sm, double s0, double sp,
                                             double &L, double &R)
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

// the primitive slots of a Prim as one indexable list: 0 d, 1 vn, 2 vt1, 3 vt2, 4 p, 5.. scalars, last ge
__device__ __forceinline__ double prim_slot(const Prim &s, int k, int ns)
{
  if (k == 0) return s.d;
  if (k == 1) return s.vn;
  if (k == 2) return s.vt1;
  if (k == 3) return s.vt2;
  if (k == 4) return s.p;
#pragma unroll
  for (int j = 0; j < NS_MAX; j++)
    if (k == 5 + j && j < ns) return s.sc[j];
  return s.ge;
}

// Interface primitives (v: d, v1, v2, v3, p, scalars, ge) -> rotated conserved state, as
// plmp_cuda.cu:290-326 / ppmp_cuda.cu:645-681 write them.
__device__ __forceinline__ void plm_put(const double *v, double *q, int ns, int de, double gamma)
{
  double const d = v[0];
  q[0]           = d;
  q[1]           = d * v[1];
  q[2]           = d * v[2];
  q[3]           = d * v[3];
  q[4]           = v[4] / (gamma - 1.0) + 0.5 * d * (v[1] * v[1] + v[2] * v[2] + v[3] * v[3]);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) q[5 + k] = d * v[5 + k];
  if (de) q[5 + ns] = d * v[5 + ns];
}

// PLMP (ORDER 1, stencil c[0..2], centre c[1]) or PPMP (ORDER 2, stencil c[0..4], centre c[2])
// for one cell: qL = the state at its high face, qR = the state at its low face (rotated conserved).
template <int ORDER>
__device__ __forceinline__ void plmp_ppmp_cell(const Prim *c, int ns, int de, double gamma, double *qL, double *qR)
{
  int const nq = 5 + ns + (de ? 1 : 0);
  double lo[NQ_MAX], hi[NQ_MAX];
#pragma unroll
  for (int k = 0; k < NQ_MAX; k++) {
    lo[k] = hi[k] = 0.0;
    if (k < nq) {
      if (ORDER == 1) {
        double const q  = prim_slot(c[1], k, ns);
        double const dm = limited_slope(prim_slot(c[0], k, ns), q, prim_slot(c[2], k, ns));
        lo[k]           = q - 0.5 * dm;
        hi[k]           = q + 0.5 * dm;
      } else {
        double const q0 = prim_slot(c[0], k, ns), q1 = prim_slot(c[1], k, ns), q2 = prim_slot(c[2], k, ns);
        double const q3 = prim_slot(c[3], k, ns), q4 = prim_slot(c[4], k, ns);
        double const sm = limited_slope(q0, q1, q2);
        double const s0 = limited_slope(q1, q2, q3);
        double const sp = limited_slope(q2, q3, q4);
        ppm_parabola(q1, q2, q3, sm, s0, sp, lo[k], hi[k]);
      }
    }
  }
  lo[0] = fmax(lo[0], TINY), hi[0] = fmax(hi[0], TINY);
  lo[4] = fmax(lo[4], TINY), hi[4] = fmax(hi[4], TINY);
  plm_put(hi, qL, ns, de, gamma);
  plm_put(lo, qR, ns, de, gamma);
}

// hll_cuda.cu:19-268 Calculate_HLL_Fluxes_CUDA: two-wave flux with Davis's wave speeds, from
// rotated conserved interface states.
__device__ __forceinline__ void hll(const double *qL, const double *qR, double *f, int ns, int de, double gamma)
{
  int const nq = 5 + ns + (de ? 1 : 0);
  double fl[NQ_MAX], fr[NQ_MAX];
  auto side = [&](const double *q, double *fo, double &vx, double &p) {
    double const d  = q[0];
    vx              = q[1] / d;
    double const vy = q[2] / d, vz = q[3] / d;
    if (de) {
      double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      p                  = pressure_de(q[4], q[4] - E_kin, q[5 + ns], gamma);
    } else {
      p = (q[4] - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
    }
    p     = fmax(p, TINY);
    fo[0] = q[1];
    fo[1] = q[1] * vx + p;
    fo[2] = q[2] * vx;
    fo[3] = q[3] * vx;
    fo[4] = (q[4] + p) * vx;
#pragma unroll
    for (int k = 5; k < NQ_MAX; k++) fo[k] = (k < nq) ? q[k] * vx : 0.0;  // scalars, thermal energy advect
  };
  double vxl, pl, vxr, pr;
  side(qL, fl, vxl, pl);
  side(qR, fr, vxr, pr);
  double const cfl = sqrt(gamma * pl / qL[0]), cfr = sqrt(gamma * pr / qR[0]);
  double const Sl = fmin(vxr - cfr, vxl - cfl);
  double const Sr = fmax(vxl + cfl, vxr + cfr);
#pragma unroll
  for (int k = 0; k < NQ_MAX; k++) {
    if (k < nq) {
      if (Sl > 0.0) {
        f[k] = fl[k];
      } else if (Sr < 0.0) {
        f[k] = fr[k];
      } else {
        f[k] = ((Sr * fl[k]) - (Sl * fr[k]) + Sl * Sr * (qR[k] - qL[k])) / (Sr - Sl);
      }
    }
  }
}

// ---- exact_cuda.cu:19-334 Calculate_Exact_Fluxes_CUDA: the exact Riemann solution (Toro ch. 4)
// sampled at x/t = 0, star pressure by Newton from the primitive-variable guess.  The reference
// evaluates its fractional powers in single precision (powf on double arguments); so does this.
__device__ __forceinline__ double fpow(double a, double b) { return (double)powf((float)a, (float)b); }

__device__ __forceinline__ void exact_pressure_function(double &f, double &fd, double p, double dk, double pk,
                                                        double ck, double g)
{
  if (p <= pk) {  // rarefaction
    f  = (2.0 / (g - 1.0)) * ck * (fpow(p / pk, (g - 1.0) / (2.0 * g)) - 1.0);
    fd = (1.0 / (dk * ck)) * fpow(p / pk, -((g + 1.0) / (2.0 * g)));
  } else {  // shock
    double const bk = ((g - 1.0) / (g + 1.0)) * pk;
    double const q  = sqrt(((2.0 / (g + 1.0)) / dk) / (bk + p));
    f  = (p - pk) * q;
    fd = (1.0 - 0.5 * (p - pk) / (bk + p)) * q;
  }
}

__device__ __forceinline__ void exact_star(double &pm, double &vm, double dl, double vl, double pl, double cl,
                                           double dr, double vr, double pr, double cr, double g)
{
  double const tol = 1.0e-6;
  double ppv       = 0.5 * (pl + pr) + 0.125 * (vl - vr) * (dl + dr) * (cl + cr);
  if (ppv < 0.0) ppv = 0.0;
  double const gl = sqrt((2.0 / ((g + 1.0) * dl)) / (((g - 1.0) / (g + 1.0)) * pl + ppv));
  double const gr = sqrt((2.0 / ((g + 1.0) * dr)) / (((g - 1.0) / (g + 1.0)) * pr + ppv));
  double pold     = (gl * pl + gr * pr - (vr - vl)) / (gl + gr);
  if (pold < 0.0) pold = tol;
  double fl = 0, fld = 0, fr = 0, frd = 0;
  for (int it = 0; it <= 20; it++) {  // at most 21 Newton passes: the loop always ends
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

__device__ __forceinline__ void exact_sample(double pm, double vm, double &d, double &v, double &p, double dl,
                                             double vl, double pl, double cl, double dr, double vr, double pr,
                                             double cr, double g)
{
  double const gm = (g - 1.0) / (g + 1.0);
  if (vm >= 0) {
    if (pm <= pl) {  // left rarefaction
      if (vl - cl >= 0) {
        d = dl, v = vl, p = pl;
      } else if (vm - cl * fpow(pm / pl, (g - 1.0) / (2.0 * g)) < 0) {
        d = dl * fpow(pm / pl, 1.0 / g), v = vm, p = pm;
      } else {
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
  } else {
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
      } else {
        double const c = (2.0 / (g + 1.0)) * (cr - ((g - 1.0) / 2.0) * vr);
        v = -c;
        d = dr * fpow(c / cr, 2.0 / (g - 1.0));
        p = pr * fpow(c / cr, 2.0 * g / (g - 1.0));
      }
    }
  }
}

__device__ __forceinline__ void exact(const double *qL, const double *qR, double *f, int ns, int de, double gamma)
{
  auto load = [&](const double *q, double &d, double &vx, double &vy, double &vz, double &p, double &ge,
                  double *sc) {
    d  = q[0];
    vx = q[1] / d;
    vy = q[2] / d;
    vz = q[3] / d;
    double const E = q[4];
    ge             = 0.0;
    if (de) {
      double const E_kin = 0.5 * d * (vx * vx + vy * vy + vz * vz);
      double const dge   = q[5 + ns];
      p                  = pressure_de(E, E - E_kin, dge, gamma);
      ge                 = dge / d;
    } else {
      p = (E - 0.5 * d * (vx * vx + vy * vy + vz * vz)) * (gamma - 1.0);
    }
    p = fmax(p, TINY);
#pragma unroll
    for (int k = 0; k < NS_MAX; k++) sc[k] = (k < ns) ? q[5 + k] / d : 0.0;
  };
  double dl, vxl, vyl, vzl, pl, gel, scl[NS_MAX];
  double dr, vxr, vyr, vzr, pr, ger, scr[NS_MAX];
  load(qL, dl, vxl, vyl, vzl, pl, gel, scl);
  load(qR, dr, vxr, vyr, vzr, pr, ger, scr);
  double const cl = sqrt(gamma * pl / dl), cr = sqrt(gamma * pr / dr);
  double pm = 0, vm = 0, ds = 0, vs = 0, ps = 0;
  exact_star(pm, vm, dl, vxl, pl, cl, dr, vxr, pr, cr, gamma);
  exact_sample(pm, vm, ds, vs, ps, dl, vxl, pl, cl, dr, vxr, pr, cr, gamma);
  f[0]            = ds * vs;
  f[1]            = ds * vs * vs + ps;
  bool const left = vs >= 0;  // transverse velocities and passive quantities advect upwind
  double const vy = left ? vyl : vyr, vz = left ? vzl : vzr;
  f[2] = ds * vs * vy;
  f[3] = ds * vs * vz;
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) f[5 + k] = ds * vs * (left ? scl[k] : scr[k]);
  if (de) f[5 + ns] = ds * vs * (left ? gel : ger);
  double const Es = (ps / (gamma - 1.0)) + 0.5 * ds * (vs * vs + vy * vy + vz * vz);
  f[4]            = (Es + ps) * vs;
}

// flux of one face with the scheme's solver (SOLVER_* of common.cuh)
template <int SOLVER>
__device__ __forceinline__ void riemann(const double *qL, const double *qR, double *f, int ns, int de, double gamma)
{
  if (SOLVER == SOLVER_ROE) {
    roe(qL, qR, f, ns, de, gamma);
  } else if (SOLVER == SOLVER_HLL) {
    hll(qL, qR, f, ns, de, gamma);
  } else if (SOLVER == SOLVER_EXACT) {
    exact(qL, qR, f, ns, de, gamma);
  } else {
    hllc(qL, qR, f, ns, de, gamma);
  }
}

}  // namespace hx
}  // namespace cgb
