// hydro_fast.cuh -- the VL hydro arithmetic reformulated for GB300's ALU balance.
//
// Same scheme as hydro_math.cuh (PPMC / PLMC / PPMP / PLMP / PCM, HLLC / Roe / HLL, dual
// energy; the exact solver's fast form is in hydro_fast_body.cuh), same limiter
// decisions, but written for throughput: every quotient by a shared denominator becomes one
// reciprocal and multiplies, primitives are computed once per cell instead of once per
// stencil use, constant divisions are multiplications, the Riemann solvers take primitive
// interface states directly (no round trip through conserved variables), and fused
// multiply-adds are allowed.  T is the compute type: double for the fast FP64 path (agrees
// with the reference to ~1e-14 relative per step), float for the mixed-precision path.
#pragma once
#include <type_traits>

#include "common.cuh"

namespace cgb
{
namespace hf
{

template <typename T>
struct Prim {
  T d, vn, vt1, vt2, p, ge;
  T sc[NS_MAX];
};

// binary64 <-> binary32 conversions on the integer pipe.  The hardware conversions issue on the
// FP64 pipe, which bounds the mixed form's FP64 stages (half of their FP64 instructions were
// conversions); these reproduce them bit for bit from the IEEE 754 formats: a binary32 in
// the normal range widens exactly (exponent rebased by 1023 - 127, fraction shifted by 29
// bits); a binary64 narrows by truncating the fraction to 23 bits and rounding to nearest,
// ties to even (up when the 29 dropped bits exceed half an ulp, or equal it with an odd kept
// fraction; a carry into the exponent is the correct result, up to infinity).  Signed zeros
// are formed on the integer pipe too.  Subnormals, infinities, NaNs and results outside the
// binary32 normal range take the hardware conversion, out of line: inline, its predicated
// conversion took an FP64-pipe issue slot in every thread although no thread needed it, while
// a call is made only by the threads whose value does.
static __device__ __noinline__ double to_f64_hw(float f) { return (double)f; }
static __device__ __noinline__ float to_f32_hw(double x) { return (float)x; }
__device__ __forceinline__ double to_f64(float f)
{
  unsigned const u = __float_as_uint(f);
  unsigned const e = (u >> 23) & 0xffu;
  if (e - 1u < 254u)
    return __hiloint2double((int)((u & 0x80000000u) | ((e + 896u) << 20) | ((u & 0x7fffffu) >> 3)), (int)(u << 29));
  if ((u & 0x7fffffffu) == 0u) return __hiloint2double((int)(u & 0x80000000u), 0);
  return to_f64_hw(f);
}
__device__ __forceinline__ float to_f32(double x)
{
  unsigned const hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  unsigned const e = (hi >> 20) & 0x7ffu;
  if (e - 897u < 254u) {
    unsigned const m    = ((hi & 0xfffffu) << 3) | (lo >> 29);
    unsigned const rest = lo & 0x1fffffffu, half = 0x10000000u;
    unsigned const r    = ((hi & 0x80000000u) | ((e - 896u) << 23)) + m;
    return __uint_as_float(r + ((rest > half) | ((rest == half) & (m & 1u))));
  }
  if (((hi & 0x7fffffffu) | lo) == 0u) return __uint_as_float(hi & 0x80000000u);
  return to_f32_hw(x);
}

// Seeds of the FP64 reciprocal and square root: the same conversions for operands already known
// to lie well inside the binary32 normal range (the callers check the binary64 exponent first), so
// with no fallback at all; narrowing truncates (the refinement that follows absorbs the extra half
// ulp).  Measured at 256^3 in the fast FP64 form: the hardware fallback of the general conversions,
// although never taken there, still cost 3% of the step, and a general all-integer conversion (with
// zeros, subnormals, infinities and NaNs on the integer pipe) slowed the mixed form and the MHD
// kernels.
__device__ __forceinline__ float seed_f32(double x)
{
  unsigned const hi = (unsigned)__double2hiint(x), lo = (unsigned)__double2loint(x);
  unsigned const e  = (hi >> 20) & 0x7ffu;
  return __uint_as_float((hi & 0x80000000u) | ((e - 896u) << 23) | ((hi & 0xfffffu) << 3) | (lo >> 29));
}
__device__ __forceinline__ double seed_f64(float f)
{
  unsigned const u = __float_as_uint(f);
  return __hiloint2double((int)((u & 0x80000000u) | ((((u >> 23) & 0xffu) + 896u) << 20) | ((u & 0x7fffffu) >> 3)),
                          (int)(u << 29));
}
// |x| in [2^-99, 2^99): the range where the seeds and their refinements stay far from overflow
// and underflow (an exponent test on the integer pipe)
__device__ __forceinline__ bool seed_range(double x)
{
  return ((((unsigned)__double2hiint(x) >> 20) & 0x7ffu) - 924u) < 198u;
}

// Comparisons of the limiters.  For double they run on the integer pipes, on the IEEE bit
// patterns: the step is bound by the FP64 pipe, where every compare and min/max is a full-rate
// FP64 instruction (DSETP), while the integer pipes sit idle.  Results equal the FP64
// comparisons for finite inputs (-0 and +0 compare equal).  Sign tests of a product (a*b > 0)
// read the operands' signs, which differs from the rounded product only if it underflows to
// zero (|a*b| < 5e-324).  The float overloads are the plain FP32 operations.
__device__ __forceinline__ bool is_pos(double x) { return __double_as_longlong(x) > 0; }  // x > 0
__device__ __forceinline__ bool is_neg(double x)                                          // x < 0
{
  return (__double_as_longlong(x) ^ (long long)0x8000000000000000ULL) > 0;
}
__device__ __forceinline__ unsigned long long mag_bits(double x)
{
  return (unsigned long long)__double_as_longlong(x) & 0x7fffffffffffffffULL;
}
__device__ __forceinline__ bool mag_lt(double a, double b) { return mag_bits(a) < mag_bits(b); }  // |a| < |b|
__device__ __forceinline__ bool is_zero(double x) { return mag_bits(x) == 0; }
__device__ __forceinline__ double mag_min(double a, double b)                                      // min(|a|, |b|)
{
  unsigned long long const x = mag_bits(a), y = mag_bits(b);
  return __longlong_as_double((long long)(x < y ? x : y));
}
__device__ __forceinline__ double mag_max(double a, double b)  // max(|a|, |b|)
{
  unsigned long long const x = mag_bits(a), y = mag_bits(b);
  return __longlong_as_double((long long)(x > y ? x : y));
}
// fmax(x, c) for a constant c > 0: as signed 64-bit integers, every negative double (and -0)
// orders below every non-negative one, and non-negative doubles order by magnitude
__device__ __forceinline__ double max_pos(double x, double c)
{
  return __double_as_longlong(x) < __double_as_longlong(c) ? c : x;
}
// max(a, b) of finite doubles of either sign on the integer pipe: the bit pattern with the
// magnitude bits flipped for negatives orders as a signed integer in the order of the values
__device__ __forceinline__ long long ordered_key(double a)
{
  long long const k = __double_as_longlong(a);
  return k ^ ((k >> 63) & 0x7fffffffffffffffLL);
}
__device__ __forceinline__ double max_ord(double a, double b) { return ordered_key(a) < ordered_key(b) ? b : a; }
__device__ __forceinline__ double min_ord(double a, double b) { return ordered_key(b) < ordered_key(a) ? b : a; }
// min / max of the compute type: FP32 instructions for float; for double the ordered bit patterns
// on the integer pipe (finite inputs), which the FP64-bound forms leave idle
__device__ __forceinline__ float tmin(float a, float b) { return fminf(a, b); }
__device__ __forceinline__ float tmax(float a, float b) { return fmaxf(a, b); }
__device__ __forceinline__ double tmin(double a, double b) { return min_ord(a, b); }
__device__ __forceinline__ double tmax(double a, double b) { return max_ord(a, b); }
// a > b of the compute type (for double on the integer pipe, finite inputs; -0 orders below +0,
// which changes no comparison below, whose sides are never a -0 / +0 pair of opposite meaning)
__device__ __forceinline__ bool tgt(double a, double b) { return ordered_key(a) > ordered_key(b); }
__device__ __forceinline__ bool tgt(float a, float b) { return a > b; }
__device__ __forceinline__ bool is_pos(float x) { return x > 0.f; }
__device__ __forceinline__ bool is_neg(float x) { return x < 0.f; }
__device__ __forceinline__ bool mag_lt(float a, float b) { return fabsf(a) < fabsf(b); }
__device__ __forceinline__ bool is_zero(float x) { return x == 0.f; }
__device__ __forceinline__ float mag_min(float a, float b) { return fminf(fabsf(a), fabsf(b)); }
__device__ __forceinline__ float mag_max(float a, float b) { return fmaxf(fabsf(a), fabsf(b)); }
__device__ __forceinline__ float max_pos(float x, float c) { return fmaxf(x, c); }
__device__ __forceinline__ bool prod_pos(double a, double b)  // a * b > 0
{
  return is_pos(a) ? is_pos(b) : (is_neg(a) && is_neg(b));
}
__device__ __forceinline__ bool prod_neg(double a, double b)  // a * b < 0
{
  return is_pos(a) ? is_neg(b) : (is_neg(a) && is_pos(b));
}
__device__ __forceinline__ bool prod_pos(float a, float b) { return a * b > 0.f; }
__device__ __forceinline__ bool prod_neg(float a, float b) { return a * b < 0.f; }

template <typename T>
struct Eps;
template <>
struct Eps<double> {
  static constexpr double roundoff = 1.0e-12;  // reconstruction.h:869-879 thresholds
};
template <>
struct Eps<float> {
  static constexpr float roundoff = 1.0e-6f;  // same test scaled to single precision
};

// Reciprocal and square root.  FP64: an FP32 estimate refined in FP64 (3 and 7 FP64
// instructions instead of a ~12-instruction divide or square-root sequence).  rcp: with the
// estimate's relative error e = 1 - d r (one FMA, exact up to one rounding), the third-order
// iteration r (1 + e + e^2) leaves a relative error of order e^3 ~ 2^-69 (the cubically convergent
// reciprocal iteration; J.-M. Muller et al., "Handbook of Floating-Point Arithmetic", 2nd ed.,
// Birkhauser 2018, ch. 4 on Newton-Raphson-based division).  sqrtT: one Newton-Raphson step on the
// inverse square root, y <- y (3/2 - x y^2 / 2), takes the FP32 estimate from ~2^-22 to ~2^-42
// relative error; the square root s = x y is then corrected once with its own residual,
// s + (x - s^2) y / 2 (Karp and Markstein, "High-precision division and square root", ACM TOMS
// 23(4), 1997), which squares that error.  Both stay within 1 ulp of the correctly rounded result,
// which cgb_selftest_fast_math measures against CUDA's 1 / x and sqrt over the FP32 exponent
// range.  Outside |x| in [2^-99, 2^99) (and for x <= 0 in the square root) a true divide / square
// root is used.  FP32: the hardware approximations (about 1 ulp).
__device__ __forceinline__ double rcp(double d)
{
  if (!seed_range(d)) return 1.0 / d;
  double const r = seed_f64(__frcp_rn(seed_f32(d)));
  double const e = fma(-d, r, 1.0);
  return fma(r, fma(e, e, e), r);
}
__device__ __forceinline__ float rcp(float d) { return __frcp_rn(d); }

__device__ __forceinline__ double sqrtT(double x)
{
  if (!(seed_range(x) && is_pos(x))) return sqrt(x);
  double y       = seed_f64(rsqrtf(seed_f32(x)));
  double const h = 0.5 * x;
  y              = y * fma(-h * y, y, 1.5);
  double const s = x * y;
  return fma(fma(-s, s, x), 0.5 * y, s);  // Karp-Markstein correction of the square root
}
__device__ __forceinline__ float sqrtT(float x) { return __fsqrt_rn(x); }

// PPM_Single_Variable (reconstruction.h:794-901), reciprocal-multiply form, with the stencil's
// one-sided differences formed once: the second differences are differences of neighbouring
// slopes; the parabolic face value midpoint + (centred slope left - centred slope right) / 6 is
// midpoint + (outer one-sided slope - inner one) / 12 (the centred slopes' shared term cancels);
// the limiter's face midpoint and its curvature 3 (a_{k-1} + a_k - 2 face) = 6 (midpoint - face)
// reuse that midpoint (algebraically the reference's expressions; they round differently only in
// the last bits).
template <typename T>
__device__ __forceinline__ void ppm1(T im2, T im1, T i, T ip1, T ip2, T &L_iph, T &R_imh)
{
  T const C2      = T(1.25);
  T const sixth   = T(1.0 / 6.0);
  T const twelfth = T(1.0 / 12.0);
  auto limit      = [&](T ci, T cim1, T mid, T iface, T s2i, T s2im1) -> T {
    T const s2c = T(6) * (mid - iface);
    T lim       = T(0);
    bool const n = is_neg(s2c);
    // sgn(s2c) min(C2 |s2im1|, C2 |s2i|, |s2c|); C2 * min(|a|, |b|) == min(C2 |a|, C2 |b|)
    if (n == is_neg(s2im1) && n == is_neg(s2i)) lim = copysign(mag_min(C2 * mag_min(s2im1, s2i), s2c), s2c);
    T const dl = iface - cim1, dr = ci - iface;
    return prod_neg(dl, dr) ? mid - lim * sixth : iface;
  };
  T const sm    = im1 - im2;
  T const sl    = i - im1;
  T const sr    = ip1 - i;
  T const sp    = ip2 - ip1;
  T const mR    = T(0.5) * (im1 + i);
  T const mL    = T(0.5) * (i + ip1);
  T R           = mR + (sm - sr) * twelfth;
  T L           = mL + (sl - sp) * twelfth;
  T const d2im1 = sl - sm;
  T const d2i   = sr - sl;
  T const d2ip1 = sp - sr;
  R             = limit(i, im1, mR, R, d2i, d2im1);
  L             = limit(ip1, i, mL, L, d2ip1, d2i);
  T const sfl   = i - R;
  T const sfr   = L - i;
  bool const extremum = !prod_pos(sfl, sfr) || !prod_pos(sr, sl);
  // Both paths, then a select: the lanes of a warp do not split on the local extremum test (the
  // split left about 40% of the FP64 sweeps' issue slots idle; with the select, fast FP64 256^3
  // 86.8 -> 83.6 ms per step).
  T const d2f  = T(6) * (R + L - T(2) * i);
  T const cmax = mag_max(mag_max(mag_max(im2, im1), mag_max(i, ip1)), ip2);
  T d2lim      = T(0);
  bool const nn = is_neg(d2im1);
  if (nn == is_neg(d2i) && nn == is_neg(d2ip1) && nn == is_neg(d2f))
    d2lim = copysign(mag_min(C2 * mag_min(mag_min(d2im1, d2i), d2ip1), d2f), d2f);
  // d2lim / d2f as a reciprocal product: |d2lim| <= |d2f|, so rho is in [0, 1]; the product is
  // kept there when the reciprocal of a subnormal d2f overflows (0 * inf, or a subnormal d2lim
  // times inf), where the quotient itself would be 0 or at most 1
  bool const big = mag_lt(Eps<T>::roundoff * cmax, d2f) && !is_zero(d2lim);
  T const rho    = big ? mag_min(d2lim * rcp(d2f), T(1)) : T(0);
  bool const sc  = !mag_lt(T(1) - Eps<T>::roundoff, rho);
  T const RA = sc ? i - rho * sfl : R, LA = sc ? i + rho * sfr : L;
  T const RB = !mag_lt(sfl, T(2) * sfr) ? i - T(2) * sfr : R;
  T const LB = !mag_lt(sfr, T(2) * sfl) ? i + T(2) * sfl : L;
  R = extremum ? RA : RB;
  L = extremum ? LA : LB;
  L_iph = L;
  R_imh = R;
}

// FP32 path: evaluate the characteristic part of a reconstruction in FP64 where it is
// ill-conditioned in FP32 (see ppmc_cell).
constexpr bool kWideFallback = true;

// Characteristic part of PPMC_VL (ppmc_cuda.cu:540-695): density, normal velocity and pressure
// at the cell's right (L*) and left (R*) faces from PPM on the projected variables
// a0 = p/(2cs^2) - d (vn - vref)/(2cs), a1 = d - p/cs^2, a4 = p/(2cs^2) + d (vn - vref)/(2cs),
// taken with the centre cell's (index 2) density and sound speed.  vref shifts the frame; PPM
// is equivariant under a common shift of its five inputs, so the result does not depend on it
// beyond rounding, but vref = centre velocity removes the bulk-flow part of the cancellation.
template <typename T>
__device__ __forceinline__ void ppmc_char(const T (&d)[5], const T (&vn)[5], const T (&p)[5], T gamma, T vref, T &Ld,
                                          T &Lvn, T &Lp, T &Rd, T &Rvn, T &Rp)
{
  T const id   = rcp(d[2]);
  T const cs   = sqrtT(gamma * p[2] * id);
  T const cs2  = cs * cs;
  T const rcs  = rcp(cs);
  T const h2c2 = T(0.5) * rcs * rcs;  // 1 / (2 cs^2)
  T const dh2c = d[2] * T(0.5) * rcs;  // d / (2 cs)
  T a0[5], a1[5], a4[5];
#pragma unroll
  for (int k = 0; k < 5; k++) {
    a0[k] = p[k] * h2c2 - dh2c * (vn[k] - vref);
    a1[k] = d[k] - T(2) * p[k] * h2c2;
    a4[k] = p[k] * h2c2 + dh2c * (vn[k] - vref);
  }
  T l0, r0, l1, r1, l4, r4;
  ppm1(a0[0], a0[1], a0[2], a0[3], a0[4], l0, r0);
  ppm1(a1[0], a1[1], a1[2], a1[3], a1[4], l1, r1);
  ppm1(a4[0], a4[1], a4[2], a4[3], a4[4], l4, r4);
  T const csid = cs * id;
  Ld  = l0 + l1 + l4;
  Lvn = csid * (l4 - l0) + vref;
  Lp  = cs2 * (l0 + l4);
  Rd  = r0 + r1 + r4;
  Rvn = csid * (r4 - r0) + vref;
  Rp  = cs2 * (r0 + r4);
}

// PPMC_VL for one cell: characteristic PPM of (d, vn, p), plain PPM of the transverse
// velocities, GasEnergy and scalars, then the density and pressure floors.  In FP32 the
// projection is taken in the frame of the centre cell's normal velocity; where the normal-velocity
// differences across the stencil still exceed 32 sound speeds (cold or near-vacuum gas) the
// projected variables' +-d dv/(2cs) terms would cancel away most FP32 digits, so that cell's
// characteristic part is evaluated in FP64 from the same FP32 inputs.
// Streamed: ld(j, s) returns slot s (0 d, 1 vn, 2 vt1, 3 vt2, 4 p, 5 GasEnergy, 6.. scalars) of
// the stencil cell j (-2 .. 2) and st(s, L, R) takes the cell's high-face (L) and low-face (R)
// values of slot s, one variable at a time, so that no more than one variable's stencil is live.
template <typename T, typename LD, typename ST>
__device__ __forceinline__ void ppmc_cell(LD ld, ST st, int ns, int de, T gamma)
{
  T const tiny = T(TINY);
  {
    T const d[5] = {ld(-2, 0), ld(-1, 0), ld(0, 0), ld(1, 0), ld(2, 0)};
    T const v[5] = {ld(-2, 1), ld(-1, 1), ld(0, 1), ld(1, 1), ld(2, 1)};
    T const p[5] = {ld(-2, 4), ld(-1, 4), ld(0, 4), ld(1, 4), ld(2, 4)};
    T Ld, Lvn, Lp, Rd, Rvn, Rp;
    if constexpr (std::is_same<T, float>::value) {
      float const cs = sqrtT(gamma * p[2] * rcp(d[2]));
      float const dv = fmax(fmax(fabs(v[0] - v[2]), fabs(v[1] - v[2])), fmax(fabs(v[3] - v[2]), fabs(v[4] - v[2])));
      if (kWideFallback && !(dv <= 32.0f * cs)) {
        double const dw[5] = {d[0], d[1], d[2], d[3], d[4]};
        double const vw[5] = {v[0], v[1], v[2], v[3], v[4]};
        double const pw[5] = {p[0], p[1], p[2], p[3], p[4]};
        double a, b, c, e, f, g;
        ppmc_char<double>(dw, vw, pw, (double)gamma, 0.0, a, b, c, e, f, g);
        Ld = (float)a, Lvn = (float)b, Lp = (float)c, Rd = (float)e, Rvn = (float)f, Rp = (float)g;
      } else {
        ppmc_char<float>(d, v, p, gamma, v[2], Ld, Lvn, Lp, Rd, Rvn, Rp);
      }
    } else {
      ppmc_char<T>(d, v, p, gamma, T(0), Ld, Lvn, Lp, Rd, Rvn, Rp);
    }
    st(0, max_pos(Ld, tiny), max_pos(Rd, tiny));
    st(1, Lvn, Rvn);
    st(4, max_pos(Lp, tiny), max_pos(Rp, tiny));
  }
  auto plain = [&](int s) {
    T L, R;
    ppm1(ld(-2, s), ld(-1, s), ld(0, s), ld(1, s), ld(2, s), L, R);
    st(s, L, R);
  };
  plain(2);
  plain(3);
  if (de) plain(5);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) plain(6 + k);
}

template <typename T>
__device__ __forceinline__ T plm_vl(T l, T r)  // van Leer average of two slopes
{
  return prod_pos(l, r) ? T(2) * l * r / (l + r) : T(0);
}
template <typename T>
__device__ __forceinline__ T plm_mono(T l, T r, T cc, T vg)  // monotonised slope
{
  if (prod_pos(l, r)) return copysign(mag_min(T(2) * mag_min(l, r), mag_min(cc, vg)), cc);
  return T(0);
}

// Characteristic part of PLMC_cuda (plmc_cuda.cu:24-300): the half-slopes hd, hn, hp of density,
// normal velocity and pressure from the monotonised slopes of the projected variables
// a0 = p/(2cs^2) - d vn/(2cs), a1 = d - p/cs^2, a4 = p/(2cs^2) + d vn/(2cs) (centre cell index 1).
template <typename T>
__device__ __forceinline__ void plmc_char(const T (&d)[3], const T (&vn)[3], const T (&p)[3], T gamma, T &hd, T &hn,
                                          T &hp)
{
  T const id   = rcp(d[1]);
  T const cs   = sqrtT(gamma * p[1] * id);
  T const cs2  = cs * cs;
  T const rcs  = rcp(cs);
  T const h2c2 = T(0.5) * rcs * rcs;
  T const dh2c = d[1] * T(0.5) * rcs;
  auto chr = [&](T sd, T sn, T sp, T &b0, T &b1, T &b4) {
    b0 = sp * h2c2 - dh2c * sn;
    b1 = sd - T(2) * sp * h2c2;
    b4 = sp * h2c2 + dh2c * sn;
  };
  T const dLd = d[1] - d[0], dRd = d[2] - d[1], dCd = T(0.5) * (d[2] - d[0]);
  T const dLn = vn[1] - vn[0], dRn = vn[2] - vn[1], dCn = T(0.5) * (vn[2] - vn[0]);
  T const dLp = p[1] - p[0], dRp = p[2] - p[1], dCp = T(0.5) * (p[2] - p[0]);
  T L0, L1, L4, R0, R1, R4, C0, C1, C4, G0, G1, G4;
  chr(dLd, dLn, dLp, L0, L1, L4);
  chr(dRd, dRn, dRp, R0, R1, R4);
  chr(dCd, dCn, dCp, C0, C1, C4);
  chr(plm_vl(dLd, dRd), plm_vl(dLn, dRn), plm_vl(dLp, dRp), G0, G1, G4);
  T const m0 = plm_mono(L0, R0, C0, G0), m1 = plm_mono(L1, R1, C1, G1), m4 = plm_mono(L4, R4, C4, G4);
  hd = T(0.5) * (m0 + m1 + m4);
  hn = T(0.5) * cs * id * (m4 - m0);
  hp = T(0.5) * cs2 * (m0 + m4);
}

// PLMC_cuda for one cell (VL, no characteristic tracing).  In FP32 a cell whose normal-velocity
// differences exceed 32 sound speeds takes its characteristic part in FP64 (see ppmc_cell).
// Streamed like ppmc_cell: ld(j, s) for the stencil cells j = -1 .. 1, st(s, L, R) per variable.
template <typename T, typename LD, typename ST>
__device__ __forceinline__ void plmc_cell(LD ld, ST st, int ns, int de, T gamma)
{
  // each interface value within the range of its two cells (Plm_Limit_Interfaces)
  auto lim = [](T &l, T &r, T vm, T vi, T vp) {
    r = tmin(tmax(vi, vm), tmax(tmin(vi, vm), r));
    l = tmin(tmax(vi, vp), tmax(tmin(vi, vp), l));
  };
  T const tiny = T(TINY);
  {
    T const d[3] = {ld(-1, 0), ld(0, 0), ld(1, 0)}, v[3] = {ld(-1, 1), ld(0, 1), ld(1, 1)};
    T const p[3] = {ld(-1, 4), ld(0, 4), ld(1, 4)};
    T hd, hn, hp;
    if constexpr (std::is_same<T, float>::value) {
      float const cs = sqrtT(gamma * p[1] * rcp(d[1]));
      if (kWideFallback && !(fmax(fabs(v[1] - v[0]), fabs(v[2] - v[1])) <= 32.0f * cs)) {
        double const dw[3] = {d[0], d[1], d[2]}, vw[3] = {v[0], v[1], v[2]}, pw[3] = {p[0], p[1], p[2]};
        double a, b, e;
        plmc_char<double>(dw, vw, pw, (double)gamma, a, b, e);
        hd = (float)a, hn = (float)b, hp = (float)e;
      } else {
        plmc_char<float>(d, v, p, gamma, hd, hn, hp);
      }
    } else {
      plmc_char<T>(d, v, p, gamma, hd, hn, hp);
    }
    T Ld = d[1] + hd, Rd = d[1] - hd, Lv = v[1] + hn, Rv = v[1] - hn, Lp = p[1] + hp, Rp = p[1] - hp;
    lim(Ld, Rd, d[0], d[1], d[2]);
    lim(Lv, Rv, v[0], v[1], v[2]);
    lim(Lp, Rp, p[0], p[1], p[2]);
    st(0, max_pos(Ld, tiny), max_pos(Rd, tiny));
    st(1, Lv, Rv);
    st(4, max_pos(Lp, tiny), max_pos(Rp, tiny));
  }
  // monotonised slopes of the other variables, each on its own
  auto plain = [&](int s) {
    T const cm = ld(-1, s), c = ld(0, s), cp = ld(1, s);
    T const dL = c - cm, dR = cp - c;
    T const h  = T(0.5) * plm_mono(dL, dR, T(0.5) * (cp - cm), plm_vl(dL, dR));
    T L = c + h, R = c - h;
    lim(L, R, cm, c, cp);
    st(s, L, R);
  };
  plain(2);
  plain(3);
  if (de) plain(5);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) plain(6 + k);
}

// Van Leer-limited slope of a three-point stencil (plmp_cuda.cu:330-365 Interface_Values_PLM,
// ppmp_cuda.cu:687-720 Calculate_Slope): sgn(centred) min(2 min(|dl|, |dr|), |centred|, |harmonic|),
// the harmonic mean 2 dl dr / (dl + dr) taken where dl and dr have one sign.
template <typename T>
__device__ __forceinline__ T prim_slope(T qm, T q, T qp)
{
  T const dl = q - qm, dr = qp - q, dc = T(0.5) * (qp - qm);
  T const dg = prod_pos(dl, dr) ? T(2) * dl * dr * rcp(dl + dr) : T(0);
  T const m  = mag_min(T(2) * mag_min(dl, dr), mag_min(dc, dg));
  return is_neg(dc) ? -m : m;
}

// PLMP_cuda for one cell under VL (plmp_cuda.cu, no half-step evolution): every primitive on its
// own, faces at the centre value plus and minus half its limited slope, density and pressure
// floored at TINY.  Streamed as plmc_cell: ld(j, s) for j = -1 .. 1, st(s, high face, low face).
template <typename T, typename LD, typename ST>
__device__ __forceinline__ void plmp_cell(LD ld, ST st, int ns, int de)
{
  auto one = [&](int s, bool floor) {
    T const c = ld(0, s);
    T const h = T(0.5) * prim_slope(ld(-1, s), c, ld(1, s));
    T L = c + h, R = c - h;
    if (floor) L = max_pos(L, T(TINY)), R = max_pos(R, T(TINY));
    st(s, L, R);
  };
  one(0, true);
  one(1, false);
  one(2, false);
  one(3, false);
  one(4, true);
  if (de) one(5, false);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) one(6 + k, false);
}

// PPMP_cuda for one cell under VL (ppmp_cuda.cu:727-752 Interface_Values_PPM, Fryxell et al. 2000,
// without flattening or steepening, as the reference builds it): the parabola through the cell
// from its neighbours' limited slopes, then its monotonicity constraints.  The two overshoot
// corrections are selects on one evaluation of the test: the second cannot hold after the first
// has moved the low face (then 6 (R - L)(q - (L + R)/2) = 9 (R - q)^2 >= 0 > -(R - L)^2).
// Streamed as ppmc_cell: ld(j, s) for j = -2 .. 2, st(s, high face, low face).
template <typename T, typename LD, typename ST>
__device__ __forceinline__ void ppmp_cell(LD ld, ST st, int ns, int de)
{
  T const sixth = T(1.0 / 6.0);
  auto one      = [&](int s, bool floor) {
    T const q0 = ld(-2, s), qm = ld(-1, s), q = ld(0, s), qp = ld(1, s), q4 = ld(2, s);
    T const sm = prim_slope(q0, qm, q), s0 = prim_slope(qm, q, qp), sp = prim_slope(q, qp, q4);
    T L = T(0.5) * (q + qm) - sixth * (s0 - sm);
    T R = T(0.5) * (qp + q) - sixth * (sp - s0);
    bool const flat = !prod_pos(R - q, q - L);  // (R - q)(q - L) <= 0: a local extremum
    L = flat ? q : L;
    R = flat ? q : R;
    T const dRL = R - L, lhs = T(6) * dRL * (q - T(0.5) * (L + R)), sq = dRL * dRL;
    bool const lo = tgt(lhs, sq), hi = !lo && tgt(-sq, lhs);
    T const Lc = lo ? T(3) * q - T(2) * R : L;
    T const Rc = hi ? T(3) * q - T(2) * L : R;
    L = tmin(tmax(q, qm), tmax(tmin(q, qm), Lc));
    R = tmin(tmax(q, qp), tmax(tmin(q, qp), Rc));
    if (floor) L = max_pos(L, T(TINY)), R = max_pos(R, T(TINY));
    st(s, R, L);
  };
  one(0, true);
  one(1, false);
  one(2, false);
  one(3, false);
  one(4, true);
  if (de) one(5, false);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) one(6 + k, false);
}

// u / e > eta without the division, keeping the quotient's sign behaviour: the total energy
// e of an updated cell can be negative, and then the reference's ratio test selects u when
// u < eta * e.  e == 0 gives +inf (u > 0) or NaN (u == 0) in the quotient.
template <typename T>
__device__ __forceinline__ bool ratio_gt(T u, T e, T eta)
{
  return e > T(0) ? u > eta * e : (e < T(0) ? u < eta * e : u > T(0));
}
// The FP64 form with every comparison on the integer pipe (ordered bit patterns, see ordered_key):
// one FP64 multiply instead of a multiply and up to four FP64 compares.  It differs from the
// quotient test only when u is +0 and eta * e is -0 (e negative and below 2e-305 in size).
__device__ __forceinline__ bool ratio_gt(double u, double e, double eta)
{
  if (is_pos(e)) return ordered_key(u) > ordered_key(eta * e);
  if (is_neg(e)) return ordered_key(u) < ordered_key(eta * e);
  return is_pos(u);
}

// Pressure a Riemann solver uses for an interface state: with dual energy the reference
// recomputes it from the interface's conserved E and GasEnergy with Get_Pressure_From_DE
// (hydro_utilities.h:136-151): the total-minus-kinetic pressure unless the thermal fraction
// of E is below eta_1, then (gamma-1) * GasEnergy.
template <typename T>
__device__ __forceinline__ T pressure_used(const Prim<T> &s, T E, T ig1, T g1, int de)
{
  if (!de) return max_pos(s.p, T(TINY));
  T const eth = s.p * ig1;
  T const p   = ratio_gt(eth, E, T(ETA_1)) ? s.p : s.d * s.ge * g1;
  return max_pos(p, T(TINY));
}

// The quantities of one side of a Riemann problem that depend on that state alone and not on the
// direction: total energy, the pressure the solver uses, 1/d, sqrt(d), the sound speed of the used
// pressure (HLLC only) and the specific enthalpy (E + p) / d.  The predictor's PCM interface states
// are the cells themselves, so it forms these once per cell for the six faces that use them.
template <typename T>
struct SideQ {
  T E, p, id, sq, c, h;
};
template <typename T, bool SOUND>
__device__ __forceinline__ SideQ<T> side_q(const Prim<T> &s, int de, T gamma, T ig1)
{
  SideQ<T> q;
  q.E  = s.p * ig1 + T(0.5) * s.d * (s.vn * s.vn + s.vt1 * s.vt1 + s.vt2 * s.vt2);
  q.p  = pressure_used(s, q.E, ig1, gamma - T(1), de);
  q.id = rcp(s.d);
  q.sq = sqrtT(s.d);
  q.c  = SOUND ? sqrtT(gamma * q.p * q.id) : T(0);
  q.h  = (q.E + q.p) * q.id;
  return q;
}

// HLLC flux (hllc_cuda.cu:19-307) from primitive interface states; f in rotated order
// in fixed slots: 0 d, 1 m_n, 2 m_t1, 3 m_t2, 4 E, 5 GasEnergy, 6.. scalars.  Fixed slots keep
// every register-array index a compile-time constant (no local memory).
template <typename T>
__device__ __forceinline__ void hllc_q(const Prim<T> &l, const Prim<T> &r, const SideQ<T> &Ql, const SideQ<T> &Qr,
                                       T *f, int ns, int de, T gamma)
{
  T const g1  = gamma - T(1);
  T const El = Ql.E, Er = Qr.E, pl = Ql.p, pr = Qr.p;
  T const sqrtdl = Ql.sq, sqrtdr = Qr.sq;
  T const isum   = rcp(sqrtdl + sqrtdr);
  T const wl = sqrtdl * isum, wr = sqrtdr * isum;
  T const vx  = wl * l.vn + wr * r.vn;
  T const vy  = wl * l.vt1 + wr * r.vt1;
  T const vz  = wl * l.vt2 + wr * r.vt2;
  T const H   = wl * Ql.h + wr * Qr.h;
  T const asq = g1 * (H - T(0.5) * (vx * vx + vy * vy + vz * vz));
  T const a   = sqrtT(asq);
  T const cfl = Ql.c;
  T const cfr = Qr.c;
  // outer wave speeds relative to each side's own velocity, kept apart from the velocity so a
  // cold side's sound speed is not rounded away (FP32: cf ~1e-10 against v ~1)
  T dSl, dSr, Sl, Sr;
  if constexpr (std::is_same<T, float>::value) {
    dSl = fmin((vx - a) - l.vn, -cfl), dSr = fmax((vx + a) - r.vn, cfr);
    Sl = l.vn + dSl, Sr = r.vn + dSr;
  } else {
    Sl = tmin(vx - a, l.vn - cfl), Sr = tmax(vx + a, r.vn + cfr);
    dSl = Sl - l.vn, dSr = Sr - r.vn;
  }
  T const ql = l.d * dSl, qr = r.d * dSr;  // mass fluxes relative to the outer waves
  T const Sm  = (qr * r.vn - ql * l.vn + pl - pr) * rcp(qr - ql);
  {
    // The flux in the one-sided form F*K = FK + SK (U*K - UK) (K = L when Sm >= 0, else R;
    // the reference's symmetric sum (Batten eq. 27) equals it exactly), with U*K - UK written
    // without cancellation as k (1, SK, vt1, vt2, (EK + pK)/dK + (SK - vK) Sm, ...),
    // k = SK (Sm - vK) / (SK - Sm).  Only the upwind star state is formed, and the symmetric
    // sum's subtraction of terms of the size of the wave speeds (~1e9 next to a near-vacuum
    // interface state, density floored at TINY) is avoided: in FP32 that cancellation costs
    // every significant digit, in FP64 about nine.  The supersonic cases (Sl > 0: FL; Sr < 0: FR)
    // take the same instructions with SK = 0, which makes k = 0 and the flux FK, so the lanes of
    // a warp do not split on the local Mach number.
    bool const sup = is_pos(Sl) || is_neg(Sr);
    bool const lft = is_pos(Sl) || (!is_neg(Sr) && !is_neg(Sm));
    // field-by-field selects (a reference to l or r would put both states in local memory)
    T const Kd = lft ? l.d : r.d, Kv = lft ? l.vn : r.vn, Kt1 = lft ? l.vt1 : r.vt1, Kt2 = lft ? l.vt2 : r.vt2;
    T const SK = sup ? T(0) : (lft ? Sl : Sr), EK = lft ? El : Er, pK = lft ? pl : pr;
    // SK - Sm from the separated parts; it is negative on the left and positive on the right,
    // and only rounding of a degenerate (both sides cold) interface can bring it to zero
    T const gap = (sup ? -Kv : (lft ? dSl : dSr)) - (Sm - Kv);
    T const den = lft ? tmin(gap, T(-1e-30)) : tmax(gap, T(1e-30));
    T const k   = SK * (Sm - Kv) * rcp(den);
    T const vk  = Kv + k;
    f[0] = Kd * vk;
    f[1] = Kd * (Kv * Kv + k * SK) + pK;
    f[2] = Kd * Kt1 * vk;
    f[3] = Kd * Kt2 * vk;
    f[4] = (EK + pK) * vk + k * Kd * (SK - Kv) * Sm;
#pragma unroll
    for (int q = 0; q < NS_MAX; q++)
      if (q < ns) f[6 + q] = Kd * (lft ? l.sc[q] : r.sc[q]) * vk;
    if (de) f[5] = Kd * (lft ? l.ge : r.ge) * vk;
  }
}

template <typename T>
__device__ __forceinline__ void hllc(const Prim<T> &l, const Prim<T> &r, T *f, int ns, int de, T gamma, T ig1)
{
  hllc_q(l, r, side_q<T, true>(l, de, gamma, ig1), side_q<T, true>(r, de, gamma, ig1), f, ns, de, gamma);
}

// HLL flux (hll_cuda.cu:19-268) from primitive interface states; f in the slots of hllc_q.  The
// outer wave speeds are Davis's, Sl = min(vL - cL, vR - cR) and Sr = max(vL + cL, vR + cR), from
// each side's velocity and sound speed of its used pressure (hll_cuda.cu:162-174).  The two-wave
// flux F = (Sr FL - Sl FR + Sl Sr (UR - UL)) / (Sr - Sl) of a quantity X carried with the mass
// (1, the velocities, GasEnergy and the scalars per unit mass: flux dK vK XK, state dK XK) is
//   F = dL bL XL + dR bR XR,  bL = Sr (vL - Sl) / (Sr - Sl),  bR = Sl (Sr - vR) / (Sr - Sl),
// plus wL pL + wR pR in the normal momentum and bL EL + bR ER + wL pL vL + wR pR vR in the energy,
// with wL = Sr / (Sr - Sl) and wR = -Sl / (Sr - Sl) (expand the products to check).  vL - Sl >= cL
// and Sr - vR >= cR come from the separated parts, as in hllc_q, so no difference of wave-speed
// sized terms is formed.  Supersonic faces (Sl > 0: FL; Sr < 0: FR) take the same instructions
// with the weights selected (wL = 1, bL = vL, wR = bR = 0, or the mirror image), so the lanes of
// a warp do not split on the local Mach number.
template <typename T>
__device__ __forceinline__ void hll_q(const Prim<T> &l, const Prim<T> &r, const SideQ<T> &Ql, const SideQ<T> &Qr,
                                      T *f, int ns, int de)
{
  T const cl = Ql.c, cr = Qr.c;
  T Sl, Sr, dSl, dSr;  // dSl = Sl - vL <= -cL, dSr = Sr - vR >= cR
  if constexpr (std::is_same<T, float>::value) {
    dSl = tmin((r.vn - cr) - l.vn, -cl), dSr = tmax((l.vn + cl) - r.vn, cr);
    Sl = l.vn + dSl, Sr = r.vn + dSr;
  } else {
    Sl = tmin(r.vn - cr, l.vn - cl), Sr = tmax(l.vn + cl, r.vn + cr);
    dSl = Sl - l.vn, dSr = Sr - r.vn;
  }
  T const inv  = rcp(tmax(Sr - Sl, T(1e-30)));  // Sr - Sl >= cL + cR > 0 but for rounding
  bool const upl = is_pos(Sl), upr = !upl && is_neg(Sr);
  T const wl   = upl ? T(1) : (upr ? T(0) : Sr * inv);
  T const wr   = upl ? T(0) : (upr ? T(1) : -Sl * inv);
  T const bl   = upl ? l.vn : (upr ? T(0) : -(Sr * dSl) * inv);
  T const br   = upl ? T(0) : (upr ? r.vn : (Sl * dSr) * inv);
  T const al = l.d * bl, ar = r.d * br;
  f[0] = al + ar;
  f[1] = al * l.vn + ar * r.vn + (wl * Ql.p + wr * Qr.p);
  f[2] = al * l.vt1 + ar * r.vt1;
  f[3] = al * l.vt2 + ar * r.vt2;
  f[4] = bl * Ql.E + br * Qr.E + (wl * Ql.p * l.vn + wr * Qr.p * r.vn);
#pragma unroll
  for (int q = 0; q < NS_MAX; q++)
    if (q < ns) f[6 + q] = al * l.sc[q] + ar * r.sc[q];
  if (de) f[5] = al * l.ge + ar * r.ge;
}

template <typename T>
__device__ __forceinline__ void hll(const Prim<T> &l, const Prim<T> &r, T *f, int ns, int de, T gamma, T ig1)
{
  hll_q(l, r, side_q<T, true>(l, de, gamma, ig1), side_q<T, true>(r, de, gamma, ig1), f, ns, de);
}

// Roe flux with the HLLE fallback (roe_cuda.cu:19-400) from primitive interface states.
template <typename T>
__device__ __forceinline__ void roe_q(const Prim<T> &l, const Prim<T> &r, const SideQ<T> &Ql, const SideQ<T> &Qr,
                                      T *f, int ns, int de, T gamma)
{
  T const g1  = gamma - T(1);
  T const dl = l.d, dr = r.d, vxl = l.vn, vyl = l.vt1, vzl = l.vt2, vxr = r.vn, vyr = r.vt1, vzr = r.vt2;
  T const mxl = dl * vxl, myl = dl * vyl, mzl = dl * vzl, mxr = dr * vxr, myr = dr * vyr, mzr = dr * vzr;
  T const El = Ql.E, Er = Qr.E, pl = Ql.p, pr = Qr.p, idl = Ql.id, idr = Qr.id;
  T const sqrtdl = Ql.sq, sqrtdr = Qr.sq;
  T const isum   = rcp(sqrtdl + sqrtdr);
  T const wl = sqrtdl * isum, wr = sqrtdr * isum;
  T const vx = wl * vxl + wr * vxr, vy = wl * vyl + wr * vyr, vz = wl * vzl + wr * vzr;
  T const H   = wl * Ql.h + wr * Qr.h;
  T const vsq = vx * vx + vy * vy + vz * vz;
  T const asq = g1 * max_pos(H - T(0.5) * vsq, T(TINY));
  T const a   = sqrtT(asq);
  T const lm = vx - a, l0 = vx, lp = vx + a;
  T fdl = mxl, fmxl = mxl * vxl + pl, fmyl = mxl * vyl, fmzl = mxl * vzl, fEl = (El + pl) * vxl;
  T fdr = mxr, fmxr = mxr * vxr + pr, fmyr = mxr * vyr, fmzr = mxr * vzr, fEr = (Er + pr) * vxr;
  if (lm >= T(0)) {
    f[0] = fdl, f[1] = fmxl, f[2] = fmyl, f[3] = fmzl, f[4] = fEl;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[6 + k] = mxl * l.sc[k];
    if (de) f[5] = mxl * l.ge;
    return;
  }
  if (lp <= T(0)) {
    f[0] = fdr, f[1] = fmxr, f[2] = fmyr, f[3] = fmzr, f[4] = fEr;
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[6 + k] = mxr * r.sc[k];
    if (de) f[5] = mxr * r.ge;
    return;
  }
  T const dd = dr - dl, dmx = mxr - mxl, dmy = myr - myl, dmz = mzr - mzl, dE = Er - El;
  T const iasq = rcp(asq);
  T const Na   = T(0.5) * iasq;
  T const a0 = Na * (dd * (T(0.5) * g1 * vsq + vx * a) - dmx * (g1 * vx + a) - g1 * (dmy * vy + dmz * vz) + dE * g1);
  T const a1 = dmy - dd * vy;
  T const a2 = dmz - dd * vz;
  T const a3 = dd * (T(1) - Na * g1 * vsq) + g1 * iasq * (dmx * vx + dmy * vy + dmz * vz - dE);
  T const a4 = Na * (dd * (T(0.5) * g1 * vsq - vx * a) - dmx * (g1 * vx - a) - g1 * (dmy * vy + dmz * vz) + dE * g1);
  T const c0 = a0 * fabs(lm), c1 = a1 * fabs(l0), c2 = a2 * fabs(l0), c3 = a3 * fabs(l0), c4 = a4 * fabs(lp);
  T const s0 = c0 + c3 + c4;
  T const s1 = c0 * (vx - a) + c3 * vx + c4 * (vx + a);
  T const s2 = c0 * vy + c1 + c3 * vy + c4 * vy;
  T const s3 = c0 * vz + c2 + c3 * vz + c4 * vz;
  T const s4 = c0 * (H - vx * a) + c1 * vy + c2 * vz + c3 * T(0.5) * vsq + c4 * (H + vx * a);
  bool hlle = false;
  T t0 = dl + a0, t1 = mxl + a0 * (vx - a), t2 = myl + a0 * vy, t3 = mzl + a0 * vz, t4 = El + a0 * (H - vx * a);
  if (l0 > lm) {
    if (t0 <= T(0)) hlle = true;
    if (t4 - T(0.5) * (t1 * t1 + t2 * t2 + t3 * t3) / t0 < T(0)) hlle = true;
  }
  t0 += a3 + a4;
  t1 += a3 * vx;
  t2 += a1 + a3 * vy;
  t3 += a2 + a3 * vz;
  t4 += a1 * vy + a2 * vz + a3 * T(0.5) * vsq;
  if (lp > l0) {
    if (t0 <= T(0)) hlle = true;
    if (t4 - T(0.5) * (t1 * t1 + t2 * t2 + t3 * t3) / t0 < T(0)) hlle = true;
  }
  if (hlle) {
    T const cfl = sqrtT(gamma * pl * idl), cfr = sqrtT(gamma * pr * idr);
    T const bm = tmin(tmin(lm, vxl - cfl), T(0)), bp = tmax(tmax(lp, vxr + cfr), T(0));
    T const tmp = T(0.5) * (bp + bm) / (bp - bm);
    auto hl = [&](T fl, T fr) { return T(0.5) * (fl + fr) + (fl - fr) * tmp; };
    f[0] = hl(mxl - bm * dl, mxr - bp * dr);
    f[1] = hl(mxl * (vxl - bm) + pl, mxr * (vxr - bp) + pr);
    f[2] = hl(myl * (vxl - bm), myr * (vxr - bp));
    f[3] = hl(mzl * (vxl - bm), mzr * (vxr - bp));
    f[4] = hl(El * (vxl - bm) + pl * vxl, Er * (vxr - bp) + pr * vxr);
#pragma unroll
    for (int k = 0; k < NS_MAX; k++)
      if (k < ns) f[6 + k] = hl(dl * l.sc[k] * (vxl - bm), dr * r.sc[k] * (vxr - bp));
    if (de) f[5] = hl(dl * l.ge * (vxl - bm), dr * r.ge * (vxr - bp));
    return;
  }
  f[0] = T(0.5) * (fdl + fdr - s0);
  f[1] = T(0.5) * (fmxl + fmxr - s1);
  f[2] = T(0.5) * (fmyl + fmyr - s2);
  f[3] = T(0.5) * (fmzl + fmzr - s3);
  f[4] = T(0.5) * (fEl + fEr - s4);
#pragma unroll
  for (int k = 0; k < NS_MAX; k++)
    if (k < ns) f[6 + k] = f[0] * ((f[0] >= T(0)) ? l.sc[k] : r.sc[k]);
  if (de) f[5] = f[0] * ((f[0] >= T(0)) ? l.ge : r.ge);
}
template <typename T>
__device__ __forceinline__ void roe(const Prim<T> &l, const Prim<T> &r, T *f, int ns, int de, T gamma, T ig1)
{
  roe_q(l, r, side_q<T, false>(l, de, gamma, ig1), side_q<T, false>(r, de, gamma, ig1), f, ns, de, gamma);
}

}  // namespace hf
}  // namespace cgb
