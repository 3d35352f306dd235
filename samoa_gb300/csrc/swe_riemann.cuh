// Device-side edge fluxes of the SWE step: the GeoClaw double-precision Riemann
// solvers and the Lax-Friedrichs fluxes, evaluated per edge in FP64.
//
// Bit-for-bit agreement with the CPU restatement needs the same rounding at
// every operation: this file is compiled with --fmad=false (no contraction)
// and keeps the reference's left-to-right evaluation order of each expression.
// Sums written in the reference as dot_product/matmul start from +0.0; that
// first addition only turns a -0.0 into +0.0, which z0() does with integer
// instructions instead of spending an FP64 add.
#pragma once

// The kernels are compiled twice: in namespace swe with strict IEEE rounding
// (no contraction) and in namespace swe_fma with FMA contraction (SWE_KNS).
#ifndef SWE_KNS
#define SWE_KNS swe
#endif
namespace swe {}

#include <stdint.h>

namespace SWE_KNS {
using namespace ::swe;

constexpr double kG = 9.80665;  // src/SWE/SWE_data_types.f90:34

enum Solver : int { FWAVE = 1, AUG_RIEMANN = 3, LF = 10, LF_BATH = 11, LLF = 12, LLF_BATH = 13 };
enum Boundary : int { BC_OUTFLOW = 0, BC_SLIP = 1, BC_NOSLIP = 2 };

struct State {
    double h, p1, p2, b;  // surface elevation, momentum, bathymetry
};
struct Update {
    double h, p1, p2, s;  // net update (or flux) and maximum wave speed
};

// Bit casts the compiler cannot see through: tests on the bit pattern of a double
// stay integer instructions (with the plain casts the compiler may turn a test
// such as "bits << 1 == 0" back into an FP64 comparison, on the FP64 pipe).
__device__ __forceinline__ long long dbits(double x) {
    long long r;
    asm("mov.b64 %0, %1;" : "=l"(r) : "d"(x));
    return r;
}
__device__ __forceinline__ double bitsd(long long v) {
    double r;
    asm("mov.b64 %0, %1;" : "=d"(r) : "l"(v));
    return r;
}

__device__ __forceinline__ double z0(double x) {
    long long v = dbits(x);
    return bitsd(v == (long long)0x8000000000000000ULL ? 0LL : v);
}
// The step's products, named by where they are taken (the solver's, the edge
// rotations', the cell update's): plain FP64 multiplies. Moving them to the
// integer pipe was measured slower (see the design notes of the FP64 diet).
__device__ __forceinline__ double prod(double a, double b) { return a * b; }
__device__ __forceinline__ double prod_rot(double a, double b) { return a * b; }
__device__ __forceinline__ double prod_cell(double a, double b) { return a * b; }

__device__ __forceinline__ double dmn(double a, double b) { return (a < b) ? a : b; }
__device__ __forceinline__ double dmx(double a, double b) { return (a > b) ? a : b; }

// IEEE predicates on the integer pipe (bit patterns), exact for every input
// including +-0, infinities and NaN; the FP64 pipe is the step's bottleneck.
__device__ __forceinline__ long long abs_bits(double x) { return dbits(x) & 0x7fffffffffffffffLL; }
__device__ __forceinline__ bool not_nan(long long a) { return a <= 0x7ff0000000000000LL; }  // a = abs_bits
__device__ __forceinline__ bool is_finite(double x) { return abs_bits(x) < 0x7ff0000000000000LL; }
__device__ __forceinline__ bool lt0(double x) {  // x < 0.0
    const long long b = dbits(x);
    const long long a = b & 0x7fffffffffffffffLL;
    return b < 0 && a != 0 && not_nan(a);
}
__device__ __forceinline__ bool gt0(double x) {  // x > 0.0
    const long long b = dbits(x);
    return b > 0 && b <= 0x7ff0000000000000LL;
}
__device__ __forceinline__ bool is_nan(double x) { return abs_bits(x) > 0x7ff0000000000000LL; }
// A key that orders like the value for non-NaN doubles, with -0 equal to +0.
__device__ __forceinline__ long long ord_key(double x) {
    long long b = dbits(x);
    b = (b == (long long)0x8000000000000000ULL) ? 0LL : b;
    return b >= 0 ? b : (b ^ 0x7fffffffffffffffLL);
}
__device__ __forceinline__ bool lt(double a, double b) {  // a < b
    return !is_nan(a) && !is_nan(b) && ord_key(a) < ord_key(b);
}
__device__ __forceinline__ double imin(double a, double b) { return lt(a, b) ? a : b; }  // dmn on the integer pipe
__device__ __forceinline__ double imax(double a, double b) { return lt(b, a) ? a : b; }  // dmx on the integer pipe
// x with its sign flipped when `neg` (exact, like multiplying by -1)
__device__ __forceinline__ double flip(double x, bool neg) {
    return bitsd(dbits(x) ^ (neg ? (long long)0x8000000000000000ULL : 0LL));
}
// An FP64 multiply the compiler keeps inside the branch it is written in.
__device__ __forceinline__ double mul_here(double a, double b) {
    double r;
    asm volatile("mul.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(a), "d"(b));
    return r;
}
// x + z for z = +-0, as IEEE addition gives it: x itself, except that a zero x
// takes +0 unless both are -0; a NaN x takes the FP64 add.
__device__ __forceinline__ double add_zero(double x, double z) {
    const long long b = dbits(x);
    if ((b << 1) == 0) return bitsd(b & dbits(z));  // -0 only when both are -0
    if (abs_bits(x) > 0x7ff0000000000000LL) {
        double r;
        asm volatile("add.rn.f64 %0, %1, %2;" : "=d"(r) : "d"(x), "d"(z));
        return r;
    }
    return x;
}
// RN(x * p) for p = 2^k: while x and the result are normal numbers the product
// is exact and only the exponent field moves (an integer add on the bit
// pattern); +-0 stays itself; a subnormal, infinite or NaN operand and an
// under- or overflowing result take the FP64 multiply.
__device__ __forceinline__ double scale_pow2(double x, int k, double p) {
    const long long b = dbits(x);
    const int e = (int)((b >> 52) & 0x7ff);
    if ((unsigned)(e - 1) <= 2045u && (unsigned)(e + k - 1) <= 2045u) return bitsd(b + ((long long)k << 52));
    if ((b << 1) == 0) return x;
    return mul_here(x, p);
}

// ---------------------------------------------------------------------------
// Correctly rounded division with a shared reciprocal.
// Several quotients in the step share a divisor (a cell's depth divides its
// edges' normal and tangential momenta; the two f-wave coefficients share
// s2 - s1). recip_rn computes y = RN(1/b) once: two Newton-Raphson steps from
// the hardware approximation bring y within one ulp of 1/b, and a third step
// with an exact residual e = 1 - b y rounds it correctly unless b's significand
// is all ones (Markstein's reciprocal theorem). div_rn then gets RN(a/b) from y:
// q0 = RN(a y) is within 1.5 ulp of a/b, one correction q1 = RN(q0 + (a - b q0) y)
// brings it well inside one ulp, and a second correction is Markstein's
// division theorem: if y = RN(1/b) and q is within one ulp of a/b, then
// r = a - b q is exact and RN(q + r y) = RN(a/b) (P. Markstein, IBM J. Res.
// Dev. 34(1), 1990; M. Cornea-Hasegan, R. Golliver, P. Markstein, ARITH-14,
// 1999). The exponents of a and b are kept within [-500, 500], where no
// intermediate result under- or overflows; outside that range, for a zero
// divisor and for the all-ones significand, plain IEEE division is used. All
// tests are integer operations, so the FP64 pipe only sees the arithmetic.
// swe_division_check compares the results with IEEE division on the device.
__device__ __forceinline__ double rcp_approx(double b) {
    double y;
    asm("rcp.approx.ftz.f64 %0, %1;" : "=d"(y) : "d"(b));
    return y;
}

struct Recip {
    double b, y;
    bool fast;
};

// 1/b to about one ulp (two Newton-Raphson steps from the hardware
// approximation), for cotangents, which need no correct rounding; b must be
// a normal number.
__device__ __forceinline__ double rcp_nr(double b) {
    double y = rcp_approx(b);
    double e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    return fma(y, e, y);
}

__device__ __forceinline__ bool exp_in(double x, int lo, int hi) {
    const int e = (int)((dbits(x) >> 52) & 0x7ff) - 1023;
    return e >= lo && e <= hi;
}

__device__ __forceinline__ bool recip_fast(double b) {
    const long long bits = dbits(b);
    return exp_in(b, -500, 500) && ((bits & 0x000fffffffffffffLL) != 0x000fffffffffffffLL);
}

__device__ __forceinline__ Recip recip_rn(double b) {
    Recip r;
    r.b = b;
    r.fast = recip_fast(b);
    double y = rcp_approx(b);
    double e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    y = fma(y, e, y);
    e = fma(-b, y, 1.0);
    r.y = fma(y, e, y);
    return r;
}

__device__ __forceinline__ double div_rn(double a, const Recip& r) {
    if (!r.fast) return a / r.b;
    if ((dbits(a) << 1) == 0) return a * r.y;  // +-0 with the IEEE sign
    if (!exp_in(a, -500, 500)) return a / r.b;
    double q = prod(a, r.y);
    double res = fma(-r.b, q, a);
    q = fma(res, r.y, q);
    res = fma(-r.b, q, a);
    return fma(res, r.y, q);
}


// Non-strict comparisons on the integer pipe with IEEE semantics (false if either is NaN).
__device__ __forceinline__ bool le(double a, double b) {  // a <= b
    return !is_nan(a) && !is_nan(b) && ord_key(a) <= ord_key(b);
}
__device__ __forceinline__ double iabs(double x) { return bitsd(abs_bits(x)); }  // fabs

// RN(1 / h) from a precomputed reciprocal y when it is known to be correctly
// rounded (recip_rn's fast range), else the IEEE division.
__device__ __forceinline__ double inv_of(double h, double y, bool y_ok) { return y_ok ? y : 1.0 / h; }

// The branch decisions of one augmented-solver evaluation, for its reverse
// (the discrete adjoint re-evaluates the values; the decisions fix the branch).
struct AugRec {
    int8_t rs;        // riemanntype: 0 a side at most dry, 1 two rarefactions, 2 two shocks, 3 one of each
    bool lowR, highR;  // h_min resp. h_max is hR
    bool lhigh;        // one of each: hL > hR
    bool t_pos;        // two rarefactions: t = -delu + 2 (sqL + sqR) kept (not the 0)
    bool l0_sE1, l2_sE2, hst_pos, hbar_pos, tilde_x, sonic;
    int8_t dcase;      // deldelh bounds: 0 none, 1 both speeds apart, 2 sE1 >= ct, 3 sE2 <= -ct
    bool dd_min_first, dd_max_first;  // each bound kept the running value
    bool ph_mx_pl, ph_min_first, ph_mn_pl, ph_max_first;  // deldelphi bounds
    double s1m, s2m;   // riemanntype's speeds
};

// Riemann structure with one Newton step, src/geoclaw/riemannsolvers.f:507-618.
// sqL / sqR are sqrt(g * hL) and sqrt(g * hR) (the caller's, the same operands
// and so the same bits as computing them here); yL / yR are RN(1 / hL) and
// RN(1 / hR) where yL_ok / yR_ok, else the divisions are done here.
template <bool REC>
__device__ __forceinline__ void riemann_structure_rec(double hL, double hR, double uL, double uR, double drytol,
                                                     double sqL, double sqR, double yL, double yR, bool yL_ok,
                                                     bool yR_ok, double& hm, double& s1m, double& s2m,
                                                     AugRec* rec) {
    const double g = kG;
    const bool r_lower = lt(hR, hL);  // h_min = dmn(hR, hL) is hR
    const double h_min = r_lower ? hR : hL, sq_min = r_lower ? sqR : sqL;
    const bool r_higher = lt(hL, hR);  // h_max = dmx(hR, hL) is hR
    const double h_max = r_higher ? hR : hL, sq_max = r_higher ? sqR : sqL;
    if (REC) {
        rec->lowR = r_lower;
        rec->highR = r_higher;
    }
    double delu = uR - uL;
    if (le(h_min, drytol)) {
        if (REC) rec->rs = 0;
        hm = 0.0;
        double t = ((uR + uL) - scale_pow2(sqR, 1, 2.0)) + scale_pow2(sqL, 1, 2.0);
        s1m = t;
        s2m = t;
        return;
    }
    double F_min = delu + scale_pow2(sq_min - sq_max, 1, 2.0);
    double F_max = 0.0;  // needed only when F_min <= 0
    if (!gt0(F_min)) F_max = delu + (h_max - h_min) * sqrt(((0.5 * g) * (h_max + h_min)) / (h_max * h_min));
    if (gt0(F_min)) {  // two rarefactions
        const double t0 = -delu + scale_pow2(sqL + sqR, 1, 2.0);
        double t = imax(0.0, t0);
        if (REC) {
            rec->rs = 1;
            rec->t_pos = !lt(t0, 0.0);
        }
        hm = (1.0 / (16.0 * g)) * (t * t);
        const double sqm = sqrt(g * hm);
        s1m = (uL + scale_pow2(sqL, 1, 2.0)) - 3.0 * sqm;
        s2m = (uR - scale_pow2(sqR, 1, 2.0)) + 3.0 * sqm;
    } else if (le(F_max, 0.0)) {  // two shocks: one Newton step on sqrt(h)
        if (REC) rec->rs = 2;
        double h0 = h_max;
        const double i0 = r_higher ? inv_of(hR, yR, yR_ok) : inv_of(hL, yL, yL_ok);
        const double iL = inv_of(hL, yL, yL_ok), iR = inv_of(hR, yR, yR_ok);
        double gL = sqrt((0.5 * g) * (i0 + iL));
        double gR = sqrt((0.5 * g) * (i0 + iR));
        double F0 = (delu + (h0 - hL) * gL) + (h0 - hR) * gR;
        double dfdh = ((gL - (g * (h0 - hL)) / ((4.0 * (h0 * h0)) * gL)) + gR) -
                      (g * (h0 - hR)) / ((4.0 * (h0 * h0)) * gR);
        const double sq0 = sqrt(h0);
        double slope = scale_pow2(sq0, 1, 2.0) * dfdh;
        double t = sq0 - F0 / slope;
        hm = t * t;
        const double im = 1.0 / hm;
        double u1m = uL - (hm - hL) * sqrt((0.5 * g) * (im + iL));
        double u2m = uR + (hm - hR) * sqrt((0.5 * g) * (im + iR));
        const double sqm = sqrt(g * hm);
        s1m = u1m - sqm;
        s2m = u2m + sqm;
    } else {  // one shock, one rarefaction
        if (REC) {
            rec->rs = 3;
            rec->lhigh = lt(hR, hL);
        }
        double h0 = h_min;
        const double i0 = r_lower ? inv_of(hR, yR, yR_ok) : inv_of(hL, yL, yL_ok);
        double F0 = (delu + scale_pow2(sq_min - sq_max, 1, 2.0)) + (h0 - h_min) * sqrt((0.5 * g) * (i0 + i0));
        double slope = (F_max - F0) / (h_max - h_min);
        hm = h0 - F0 / slope;
        const double sqm = sqrt(g * hm);
        if (lt(hR, hL)) {
            s1m = (uL + scale_pow2(sqL, 1, 2.0)) - 3.0 * sqm;
            s2m = (uL + scale_pow2(sqL, 1, 2.0)) - sqm;
        } else {
            s2m = (uR - scale_pow2(sqR, 1, 2.0)) + 3.0 * sqm;
            s1m = (uR - scale_pow2(sqR, 1, 2.0)) + sqm;
        }
    }
}

__device__ __forceinline__ void riemann_structure_core(double hL, double hR, double uL, double uR, double drytol,
                                                      double sqL, double sqR, double yL, double yR, bool yL_ok,
                                                      bool yR_ok, double& hm, double& s1m, double& s2m) {
    riemann_structure_rec<false>(hL, hR, uL, uR, drytol, sqL, sqR, yL, yR, yL_ok, yR_ok, hm, s1m, s2m, nullptr);
}

// The same with sqrt(g * h) and the reciprocals computed here (the wet/dry
// edges' wall test; a call, so the callers keep their registers).
static __device__ __noinline__ void riemann_structure(double hL, double hR, double uL, double uR, double drytol,
                                                      double& hm, double& s1m, double& s2m) {
    riemann_structure_core(hL, hR, uL, uR, drytol, sqrt(kG * hL), sqrt(kG * hR), 0.0, 0.0, false, false, hm, s1m,
                           s2m);
}

__device__ __forceinline__ double det3(double a00, double a01, double a02, double a10, double a11, double a12,
                                       double a20, double a21, double a22) {
    double d1 = a00 * (a11 * a22 - a12 * a21);
    double d2 = a01 * (a10 * a22 - a12 * a20);
    double d3 = a02 * (a10 * a21 - a11 * a20);
    return (d1 - d2) + d3;
}

// RN(0 * x): a zero with x's sign for finite x (0 * inf and 0 * NaN are NaN).
__device__ __forceinline__ double mul0(double x) {
    return is_finite(x) ? bitsd(dbits(x) & (long long)0x8000000000000000ULL) : x * 0.0;
}
// |x| < 2^300 (or zero): products of three such numbers neither overflow nor are infinite
__device__ __forceinline__ bool moderate(double x) { return abs_bits(x) < 0x52b0000000000000LL; }

// Augmented solver (George 2008) with maxiter = 1, src/geoclaw/riemannsolvers.f:2-258.
// The entropy corrector is off in the source; with one iteration the star
// states after the Cramer solve never reach the outputs.
// sqL / sqR: sqrt(g * h) of the (fixed-up) depths; yL / yR: RN(1 / h) where yL_ok / yR_ok.
//
// The 3x3 Cramer solve has the eigenvector matrix R = [[1, 0, 1], [l0, 0, l2],
// [l0^2, 1, l2^2]] with constant 0 and 1 entries. Evaluated in the source's
// order, a product by 1 is its other factor and a product by 0 a signed zero,
// and subtracting or adding a zero leaves a nonzero value unchanged, so for
// finite operands the four determinants have the values
//   det(R) = RN(l0 - l2), the numerators RN(e1 - RN(e0 l2)), the full
//   expression for beta1, and RN(RN(e0 l0) - e1)
// with at most a different sign of a zero result. Such a zero only reaches the
// f-waves, whose zeros the net-update accumulation turns into +0, except as a
// divisor: a zero determinant, and operands that are not finite or so large
// that a product could overflow, take the source's full expressions.
template <bool REC>
__device__ __forceinline__ void riemann_aug_rec(double hL, double hR, double huL, double huR, double bL, double bR,
                                               double uL, double uR, double vL, double vR, double delphi,
                                               double sE1, double sE2, double sqL, double sqR, double yL,
                                               double yR, bool yL_ok, bool yR_ok, double drytol, double sw[3],
                                               double fw[3][3], AugRec* rec) {
    const double g = kG;
    double delh = hR - hL;
    double delhu = huR - huL;
    double delb = bR - bL;
    double hm, s1m, s2m;
    riemann_structure_rec<REC>(hL, hR, uL, uR, drytol, sqL, sqR, yL, yR, yL_ok, yR_ok, hm, s1m, s2m, rec);
    double l0 = imin(sE1, s2m);
    double l2 = imax(sE2, s1m);
    if (REC) {
        rec->l0_sE1 = lt(sE1, s2m);
        rec->l2_sE2 = lt(s1m, sE2);
        rec->s1m = s1m;
        rec->s2m = s2m;
    }
    sE1 = l0;
    sE2 = l2;
    // sE2 - sE1 = -(l0 - l2) exactly (round to nearest is symmetric): one
    // reciprocal serves hstarHLL's divisor and the Cramer determinant
    const double dsp = sE2 - sE1;
    const Recip rsp = recip_rn(dsp);
    const double hq = div_rn(((huL - huR) + sE2 * hR) - sE1 * hL, rsp);
    double hstarHLL = imax(hq, 0.0);
    double l1 = scale_pow2(l0 + l2, -1, 0.5);
    if (lt(iabs(l1), 1e-20)) l1 = 0.0;
    const double r20 = l0 * l0, r22 = l2 * l2;

    const double ct = 1e-6;
    const double hhalf = scale_pow2(hL + hR, -1, 0.5);
    double hbar = imax(hhalf, 0.0);
    double su = uL + uR;
    const double ghbar = g * hbar;
    double s1s2bar = scale_pow2(su * su, -2, 0.25) - ghbar;
    const double uLR = uL * uR;
    double s1s2tilde = imax(0.0, uLR) - ghbar;
    bool sonic = le(iabs(s1s2bar), ct);
    sonic |= le(s1s2bar * s1s2tilde, ct);
    sonic |= le((s1s2bar * sE1) * sE2, ct);
    sonic |= lt(imin(iabs(sE1), iabs(sE2)), ct);
    sonic |= lt0(sE1) && gt0(s1m);
    sonic |= gt0(sE2) && lt0(s2m);
    sonic |= lt0((uL + sqL) * (uR + sqR));  // sqrt(g * h) of the fixed-up depths
    sonic |= lt0((uL - sqL) * (uR - sqR));
    if (REC) {
        rec->hst_pos = lt(0.0, hq);
        rec->hbar_pos = lt(0.0, hhalf);
        rec->tilde_x = !lt(uLR, 0.0);
        rec->sonic = sonic;
        rec->dcase = 0;
    }

    double deldelh, deldelphi;
    const double dgh = (delb * g) * hbar;
    if (sonic) {
        deldelh = flip(delb, true);
        deldelphi = flip(ghbar * delb, true);
    } else {
        const Recip rb = recip_rn(s1s2bar);
        deldelh = div_rn(dgh, rb);
        deldelphi = flip(div_rn(dgh * s1s2tilde, rb), true);
    }
    const double hsd = hstarHLL * dsp;
    int dcase = 0;
    double lo = 0.0, hi = 0.0;  // the two bounds of the case
    if (lt(sE1, -ct) && lt(ct, sE2)) {
        dcase = 1;
        hi = hsd / sE2;
        lo = hsd / sE1;
    } else if (le(ct, sE1)) {
        dcase = 2;
        hi = hsd / sE1;
        lo = flip(hL, true);
    } else if (le(sE2, -ct)) {
        dcase = 3;
        hi = hR;
        lo = hsd / sE2;
    }
    if (dcase) {
        const double x1 = imin(deldelh, hi);
        if (REC) {
            rec->dcase = (int8_t)dcase;
            rec->dd_min_first = lt(deldelh, hi);
            rec->dd_max_first = lt(lo, x1);
        }
        deldelh = imax(x1, lo);
    }
    const double pl = flip(hL * delb, true), pr = flip(hR * delb, true);
    const double gmx = g * imax(pl, pr), gmn = g * imin(pl, pr);
    const double y1 = imin(deldelphi, gmx);
    if (REC) {
        rec->ph_mx_pl = lt(pr, pl);
        rec->ph_min_first = lt(deldelphi, gmx);
        rec->ph_mn_pl = lt(pl, pr);
        rec->ph_max_first = lt(gmn, y1);
    }
    deldelphi = imax(y1, gmn);
    double d0 = delh - deldelh, d1 = delhu, d2 = delphi - deldelphi;

    double beta0, beta1, beta2;
    const double det = l0 - l2;
    const bool quick = moderate(l0) && moderate(l2) && moderate(d0) && moderate(d1) && moderate(d2) &&
                       (dbits(det) << 1) != 0;
    // beta1's numerator, the source's expression with the products by 1 dropped
    const double n1 = ((d1 * r22 - l2 * d2) - d0 * (l0 * r22 - l2 * r20)) + (l0 * d2 - d1 * r20);
    if (quick) {
        const Recip rd{det, flip(rsp.y, true), rsp.fast};  // RN(1 / det) = -RN(1 / (sE2 - sE1))
        beta0 = div_rn(d1 - d0 * l2, rd);
        beta1 = div_rn(n1, rd);
        beta2 = div_rn(d0 * l0 - d1, rd);
    } else {
        const double r00 = 1.0, r01 = 0.0, r02 = 1.0, r10 = l0, r11 = 0.0, r12 = l2, r21 = 1.0;
        const double dt = det3(r00, r01, r02, r10, r11, r12, r20, r21, r22);
        beta0 = det3(d0, r01, r02, d1, r11, r12, d2, r21, r22) / dt;
        beta1 = det3(r00, d0, r02, r10, d1, r12, r20, d2, r22) / dt;
        beta2 = det3(r00, r01, d0, r10, r11, d1, r20, r21, d2) / dt;
    }

    sw[0] = l0;
    sw[1] = l1;
    sw[2] = l2;
    // f-waves: beta times rows 2 and 3 of R (r11 = 0, r21 = 1)
    fw[0][0] = beta0 * l0; fw[1][0] = beta0 * r20; fw[2][0] = (beta0 * l0) * vL;
    fw[0][1] = mul0(beta1); fw[1][1] = beta1;
    fw[0][2] = beta2 * l2; fw[1][2] = beta2 * r22; fw[2][2] = (beta2 * l2) * vR;
    fw[2][1] = ((((hR * uR) * vR) - ((hL * uL) * vL)) - fw[2][0]) - fw[2][2];
}

static __device__ __noinline__ void riemann_aug(double hL, double hR, double huL, double huR, double bL, double bR,
                                                double uL, double uR, double vL, double vR, double delphi,
                                                double sE1, double sE2, double sqL, double sqR, double yL,
                                                double yR, bool yL_ok, bool yR_ok, double drytol, double sw[3],
                                                double fw[3][3]) {
    riemann_aug_rec<false>(hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, sqL, sqR, yL, yR, yL_ok,
                           yR_ok, drytol, sw, fw, nullptr);
}

// Wet/dry handling, wave speeds and net updates of c_bind_geoclaw_solver_dp
// (src/geoclaw/c_bind_riemannsolvers.f90:16-176) with the f-wave
// (src/geoclaw/riemannsolvers.f:446-500) or augmented solver. netL/netR are
// the left/right net updates of (h, hu, hv) in the edge frame.
// sqL0 / sqR0 are sqrt(g * depth) of the two cells, computed once per cell by the
// caller; they are used only where the reference evaluates sqrt(g * h) on an
// unmodified wet depth (the same operands, so the same bits).
// yL0 / yR0 are RN(1 / depth) of the two cells (read only for wet sides).
// Branch-frozen evaluation (FZ, the f-wave only): FZ = 1 records the decisions
// of the edge into *fz, FZ = 2 takes them from *fz instead of the comparisons
// (a forward run whose every branch is that of a recorded run, for checking the
// discrete adjoint by finite differences). Bits: 0 both sides dry, 1 right wet,
// 2 left wet, 3 right wall, 4 right bottom lowered, 5 left wall, 6 left bottom
// lowered, 7 sE1 = sL, 8 sE2 = sR, 9 + 2w / 10 + 2w wave w's speed < 0 / > 0.
template <int FZ>
__device__ __forceinline__ bool fzb(uint16_t* fz, int bit, bool v) {
    if (FZ == 2) return (*fz >> bit) & 1u;
    if (FZ == 1 && v) *fz |= (uint16_t)(1u << bit);
    return v;
}

template <int SOLVER, int FZ = 0>
__device__ __forceinline__ void geoclaw_solver(double hL, double hR, double huL, double huR, double hvL,
                                               double hvR, double bL, double bR, double sqL0, double sqR0,
                                               double yL0, double yR0, double drytol, double netL[3],
                                               double netR[3], double& maxspeed, uint16_t* fz = nullptr) {
    const double g = kG;
    netL[0] = netL[1] = netL[2] = 0.0;
    netR[0] = netR[1] = netR[2] = 0.0;
    maxspeed = 0.0;
    if (FZ == 1) *fz = 0;
    const bool wetR0 = fzb<FZ>(fz, 1, lt(drytol, hR)), wetL0 = fzb<FZ>(fz, 2, lt(drytol, hL));  // h > drytol
    if (fzb<FZ>(fz, 0, !wetL0 && !wetR0 && !is_nan(hL) && !is_nan(hR) && !is_nan(drytol))) return;  // both dry
    if (FZ == 2) {  // a recorded wet side is wet here, whatever its current depth
        if (wetL0) sqL0 = sqrt(g * hL);
        if (wetR0) sqR0 = sqrt(g * hR);
    }
    double uL, uR, vL, vR;
    if (wetR0) {
        if (FZ == 2) {
            uR = huR / hR;
            vR = hvR / hR;
        } else {
            const Recip r{hR, yR0, recip_fast(hR)};
            uR = div_rn(huR, r);
            vR = div_rn(hvR, r);
        }
    } else {
        hR = 0.0; huR = 0.0; hvR = 0.0; uR = 0.0; vR = 0.0;
    }
    if (wetL0) {
        if (FZ == 2) {
            uL = huL / hL;
            vL = hvL / hL;
        } else {
            const Recip r{hL, yL0, recip_fast(hL)};
            uL = div_rn(huL, r);
            vL = div_rn(hvL, r);
        }
    } else {
        hL = 0.0; huL = 0.0; hvL = 0.0; uL = 0.0; vL = 0.0;
    }
    bool wall_l = false, wall_r = false;  // wall(1) = 0 resp. wall(3) = 0 (wall(2) = 0 with either)
    if (!wetR0) {  // hR is now 0.0, and 0.0 <= drytol
        double hstar = 0.0, s1m, s2m;
        if (FZ != 2) riemann_structure(hL, hL, uL, -uL, drytol, hstar, s1m, s2m);  // a rare edge: sqrt here
        double hstartest = dmx(hL, hstar);
        if (fzb<FZ>(fz, 3, hstartest + bL < bR)) {
            wall_r = true;
            hR = hL; huR = -huL; bR = bL; uR = -uL; vR = vL;
        } else if (fzb<FZ>(fz, 4, hL + bL < bR)) {
            bR = hL + bL;
        }
    } else if (!wetL0) {
        double hstar = 0.0, s1m, s2m;
        if (FZ != 2) riemann_structure(hR, hR, -uR, uR, drytol, hstar, s1m, s2m);  // a rare edge: sqrt here
        double hstartest = dmx(hR, hstar);
        if (fzb<FZ>(fz, 5, hstartest + bR < bL)) {
            wall_l = true;
            hL = hR; huL = -huR; bL = bR; uL = -uR; vL = vR;
        } else if (fzb<FZ>(fz, 6, hR + bR < bL)) {
            bL = hR + bR;
        }
    }
    const double hsum = hR + hL;
    const double ghalf_h = prod(g * 0.5, hsum);  // (0.5 * g) * (hR + hL): delphi, chat, the f-wave's deldelphi
    double delphi = ((prod(huR - huL, uL + uR) - prod(prod(uL, uR), hR - hL)) +
                     prod(prod(0.5 * g, ((bR + hR) - bL) - hL), hsum)) -
                    prod(ghalf_h, bR - bL);
    // sqrt(g * h) after the wet/dry fix-ups: a wet side keeps its depth, a dry one
    // has depth 0, and a wall mirrors the wet side's depth
    // a dry side has h = 0 <= drytol now, a wet one is unchanged, a wall mirrors the wet side
    const bool wetL = wetL0 || wall_l, wetR = wetR0 || wall_r;
    double sqL = wetL ? (wall_l ? sqR0 : sqL0) : 0.0;
    double sqR = wetR ? (wall_r ? sqL0 : sqR0) : 0.0;
    double sL = uL - sqL;
    double sR = uR + sqR;
    // one division with its own divisor: the IEEE division (correctly rounded, as
    // recip_rn + div_rn is) needs fewer FP64 instructions than a private reciprocal
    double uhat = (prod(sqL, uL) + prod(sqR, uR)) / (sqR + sqL);
    double chat = sqrt(ghalf_h);
    const double r1 = uhat - chat, r2 = uhat + chat;
    double sE1 = fzb<FZ>(fz, 7, lt(sL, r1)) ? sL : r1;  // imin(sL, r1)
    double sE2 = fzb<FZ>(fz, 8, lt(r2, sR)) ? sR : r2;  // imax(sR, r2)

    double sw[3], fw[3][3];
    if (SOLVER == AUG_RIEMANN) {
        // RN(1 / h) of the fixed-up depths: a wet side's own, a wall's mirrored one
        const double yLf = wall_l ? yR0 : yL0, yRf = wall_r ? yL0 : yR0;
        const bool okL = wetL && recip_fast(hL), okR = wetR && recip_fast(hR);
        riemann_aug(hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, sqL, sqR, yLf, yRf, okL, okR,
                    drytol, sw, fw);
    } else {
        double delhu = huR - huL;
        double delb = bR - bL;
        double deldelphi = -prod(ghalf_h, delb);
        double dpd = delphi - deldelphi;
        const Recip rD = recip_rn(sE2 - sE1);
        double beta1 = div_rn(prod(sE2, delhu) - dpd, rD);
        double beta2 = div_rn(dpd - prod(sE1, delhu), rD);
        sw[0] = sE1; sw[1] = scale_pow2(sE1 + sE2, -1, 0.5); sw[2] = sE2;
        fw[0][0] = beta1; fw[1][0] = prod(beta1, sE1); fw[2][0] = prod(beta1, vL);
        fw[0][2] = beta2; fw[1][2] = prod(beta2, sE2); fw[2][2] = prod(beta2, vR);
        fw[0][1] = 0.0; fw[1][1] = 0.0;
        fw[2][1] = ((prod(huR, vR) - prod(huL, vL)) - fw[2][0]) - fw[2][2];
    }
    // eliminate ghost fluxes of a wall (multiplication by 0 keeps the sign of zero)
    auto zero_wave = [&](const int w) {
        sw[w] = sw[w] * 0.0;
        fw[0][w] = fw[0][w] * 0.0;
        fw[1][w] = fw[1][w] * 0.0;
        fw[2][w] = fw[2][w] * 0.0;
    };
    if (wall_l) {
        zero_wave(0);
        zero_wave(1);
    } else if (wall_r) {
        zero_wave(1);
        zero_wave(2);
    }
    // net updates: each accumulator starts at +0 and takes its waves in wave order;
    // +0 + x is z0(x), and the f-wave's wave 2 carries exact +0 in h and hu,
    // which leaves an accumulator unchanged (it is never -0)
    bool tL[3] = {false, false, false}, tR[3] = {false, false, false};
    auto acc = [](double& a, bool& t, double c) {
        a = t ? a + c : z0(c);
        t = true;
    };
#pragma unroll
    for (int w = 0; w < 3; ++w) {
        const bool neg = fzb<FZ>(fz, 9 + 2 * w, lt0(sw[w])), pos = fzb<FZ>(fz, 10 + 2 * w, gt0(sw[w]));
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            if (SOLVER != AUG_RIEMANN && w == 1 && e < 2) continue;
            const double f = fw[e][w];
            if (neg) {
                acc(netL[e], tL[e], f);
            } else if (pos) {
                acc(netR[e], tR[e], f);
            } else {
                const double hf = 0.5 * f;
                acc(netL[e], tL[e], hf);
                acc(netR[e], tR[e], hf);
            }
        }
    }
    // m = |s1|; if (|s2| > m) m = |s2|; if (|s3| > m) m = |s3|, on the bit
    // patterns (non-negative values order like them; a NaN candidate never wins)
    long long m = abs_bits(sw[0]);
    const long long a1 = abs_bits(sw[1]), a2 = abs_bits(sw[2]);
    if (a1 > m && not_nan(a1)) m = a1;
    if (a2 > m && not_nan(a2)) m = a2;
    maxspeed = bitsd(m);
}

// compute_geoclaw_flux, src/SWE/SWE_euler_timestep.f90:449-481.
// axis: 0 = any normal; 1 = n = (+-1, +0); 2 = n = (+0, +-1). For an
// axis-aligned normal each component of T p and of net(2:3) T is one exact
// product plus a signed zero, i.e. the other momentum with its sign flipped
// and -0 mapped to +0, which integer instructions give bit for bit while the
// operands are finite (0 * inf would be NaN). For a diagonal normal
// (|n1| = |n2| = c) the four products of each rotation are +-RN(c p1) and
// +-RN(c p2), since RN(-x) = -RN(x): two products per side, the signs set on
// the bit patterns. Otherwise the general form runs.
template <int SOLVER, int FZ = 0>
__device__ __forceinline__ void geoclaw_flux(double n1, double n2, const State& QL, const State& QR, double dL,
                                             double dR, double sqL, double sqR, double yL, double yR,
                                             double drytol, Update& fL, Update& fR, int axis = 0,
                                             uint16_t* fz = nullptr) {
    // both sides dry: the solver returns zero net updates and speed, and their
    // rotation back is +0 in every component, so neither rotation is needed
    const bool dry2 = FZ == 2 ? ((*fz & 1u) != 0)
                              : (!lt(drytol, dL) && !lt(drytol, dR) && !is_nan(dL) && !is_nan(dR) && !is_nan(drytol));
    if (dry2) {
        if (FZ == 1) *fz = 1;
        fL = Update{0.0, 0.0, 0.0, 0.0};
        fR = Update{0.0, 0.0, 0.0, 0.0};
        return;
    }
    if (SOLVER == FWAVE && FZ == 0) {
        // Water at rest on both sides under one surface (lake at rest): every
        // momentum is +-0, both sides are wet and the c-binding's surface
        // difference ((bR + hR) - bL) - hL is +-0. Then in the f-wave path the
        // velocities, uhat and the momentum jump are signed zeros; delphi is
        // +-0 - X with X = RN(ghalf_h (bR - bL)) and deldelphi is -X, so
        // delphi - deldelphi is a zero (x - x = +0), both f-wave coefficients
        // divide a zero, and every f-wave component is a signed zero. The net
        // updates start at +0 and add zeros, so they are +0, and rotating them
        // back gives +0 in every component. The speeds are sL = -sqL,
        // sR = sqR, Roe uhat -+ chat = -+chat with chat = sqrt(ghalf_h), so
        // |sE1| = max(sqL, chat), |sE2| = max(sqR, chat), and the middle wave's
        // |RN(sE1 + sE2) / 2| (sE1 <= 0 <= sE2) exceeds neither: the maximum
        // speed is the largest of sqL, sqR and chat. And chat never exceeds
        // the larger of sqL, sqR: with h the larger depth, RN(hR + hL) <= 2h,
        // so ghalf_h = RN(RN(g / 2) RN(hR + hL)) <= RN((g / 2) 2h) = RN(g h)
        // (g / 2 is exact, and RN, the product by a positive factor and sqrt
        // are monotone), hence chat <= RN(sqrt(RN(g h))), the cell's own
        // sqrt(g h). So the maximum speed is max(sqL, sqR), both positive. The
        // same bits as the full evaluation, without its FP64 arithmetic.
        // The surface difference x - hL, x = RN(RN(bR + hR) - bL), rounds to a
        // zero exactly when x equals hL and both are finite (gradual underflow:
        // the difference of two distinct finite doubles is not rounded to zero;
        // inf - inf is NaN). hL > drytol >= 0 is positive, so equal values have
        // equal bit patterns: one FP64 addition fewer per edge.
        const bool still = ((dbits(QL.p1) | dbits(QL.p2) | dbits(QR.p1) | dbits(QR.p2)) << 1) == 0;
        if (still && lt(drytol, dL) && lt(drytol, dR)) {
            const double x = (QR.b + dR) - QL.b;
            if (dbits(x) == dbits(dL) && is_finite(dL)) {
                const long long m = dbits(sqL) > dbits(sqR) ? dbits(sqL) : dbits(sqR);
                const double ms = bitsd(m);
                fL = Update{0.0, 0.0, 0.0, ms};
                fR = Update{0.0, 0.0, 0.0, ms};
                return;
            }
        }
    }
    const bool fin = is_finite(QL.p1) && is_finite(QL.p2) && is_finite(QR.p1) && is_finite(QR.p2);
    const bool fast = axis != 0 && fin;
    const bool diag = axis == 0 && fin && abs_bits(n1) == abs_bits(n2);
    const bool sn = axis == 1 ? lt0(n1) : lt0(n2);  // sign of the nonzero component
    const bool g1 = dbits(n1) < 0, g2 = dbits(n2) < 0;  // sign bits of the normal
    const double c = bitsd(abs_bits(n1));
    double pL1, pL2, pR1, pR2;
    if (diag) {
        // RN(n1 p1) = +-a1, RN(n2 p2) = +-a2, RN(-n2 p1) = -+a1, RN(n1 p2) = +-a2
        const double aL1 = prod_rot(c, QL.p1), aL2 = prod_rot(c, QL.p2);
        const double aR1 = prod_rot(c, QR.p1), aR2 = prod_rot(c, QR.p2);
        pL1 = z0(flip(aL1, g1)) + flip(aL2, g2);
        pL2 = z0(flip(aL1, !g2)) + flip(aL2, g1);
        pR1 = z0(flip(aR1, g1)) + flip(aR2, g2);
        pR2 = z0(flip(aR1, !g2)) + flip(aR2, g1);
    } else if (fast) {
        if (axis == 1) {
            pL1 = z0(flip(QL.p1, sn)); pL2 = z0(flip(QL.p2, sn));
            pR1 = z0(flip(QR.p1, sn)); pR2 = z0(flip(QR.p2, sn));
        } else {
            pL1 = z0(flip(QL.p2, sn)); pL2 = z0(flip(QL.p1, !sn));
            pR1 = z0(flip(QR.p2, sn)); pR2 = z0(flip(QR.p1, !sn));
        }
    } else {
        // T = [[n1, n2], [-n2, n1]]; p_edge = T p
        pL1 = z0(prod_rot(n1, QL.p1)) + prod_rot(n2, QL.p2);
        pL2 = z0(prod_rot(-n2, QL.p1)) + prod_rot(n1, QL.p2);
        pR1 = z0(prod_rot(n1, QR.p1)) + prod_rot(n2, QR.p2);
        pR2 = z0(prod_rot(-n2, QR.p1)) + prod_rot(n1, QR.p2);
    }
    double netL[3], netR[3], ms;
    geoclaw_solver<SOLVER, FZ>(dL, dR, pL1, pR1, pL2, pR2, QL.b, QR.b, sqL, sqR, yL, yR, drytol, netL, netR, ms,
                               fz);
    fL.h = netL[0];
    fL.s = ms;
    fR.h = netR[0];
    fR.s = ms;
    const bool nfin = is_finite(netL[1]) && is_finite(netL[2]) && is_finite(netR[1]) && is_finite(netR[2]);
    if (diag && nfin) {
        // RN(m1 n1) = +-b1, RN(m2 (-n2)) = -+b2, RN(m1 n2) = +-b1, RN(m2 n1) = +-b2
        const double bL1 = prod_rot(netL[1], c), bL2 = prod_rot(netL[2], c);
        const double bR1 = prod_rot(netR[1], c), bR2 = prod_rot(netR[2], c);
        fL.p1 = z0(flip(bL1, g1)) + flip(bL2, !g2);
        fL.p2 = z0(flip(bL1, g2)) + flip(bL2, g1);
        fR.p1 = z0(flip(bR1, g1)) + flip(bR2, !g2);
        fR.p2 = z0(flip(bR1, g2)) + flip(bR2, g1);
    } else if (fast && nfin) {
        if (axis == 1) {
            fL.p1 = z0(flip(netL[1], sn)); fL.p2 = z0(flip(netL[2], sn));
            fR.p1 = z0(flip(netR[1], sn)); fR.p2 = z0(flip(netR[2], sn));
        } else {
            fL.p1 = z0(flip(netL[2], !sn)); fL.p2 = z0(flip(netL[1], sn));
            fR.p1 = z0(flip(netR[2], !sn)); fR.p2 = z0(flip(netR[1], sn));
        }
    } else {
        // p = net(2:3) T
        fL.p1 = z0(prod_rot(netL[1], n1)) + prod_rot(netL[2], -n2);
        fL.p2 = z0(prod_rot(netL[1], n2)) + prod_rot(netL[2], n1);
        fR.p1 = z0(prod_rot(netR[1], n1)) + prod_rot(netR[2], -n2);
        fR.p2 = z0(prod_rot(netR[1], n2)) + prod_rot(netR[2], n1);
    }
}

__device__ __forceinline__ double normal_velocity(double n1, double n2, double p1, double p2, double d) {
    return z0(n1 * (p1 / d)) + n2 * (p2 / d);
}
// The same with the quotients from r = {d, RN(1 / d)} (div_rn: IEEE results).
__device__ __forceinline__ double normal_velocity(double n1, double n2, double p1, double p2, const Recip& r) {
    return z0(n1 * div_rn(p1, r)) + n2 * div_rn(p2, r);
}

// compute_lf_flux, src/SWE/SWE_euler_timestep.f90:359-446
// yL / yR: RN(1 / depth) of the two states where the depth is above the dry
// tolerance (else not read).
template <int SOLVER>
__device__ __forceinline__ void lf_flux(double n1, double n2, const State& QL, const State& QR, double dL,
                                        double dR, double drytol, Update& fL, Update& fR, double yL, double yR) {
    const double g = kG;
    if (SOLVER == LF_BATH || SOLVER == LLF_BATH) {
        const Recip rL{dL, yL, lt(drytol, dL) && recip_fast(dL)}, rR{dR, yR, lt(drytol, dR) && recip_fast(dR)};
        if (dL < drytol || dR < drytol) {
            fL = Update{0.0, 0.0, 0.0, 0.0};
            fR = Update{0.0, 0.0, 0.0, 0.0};
            if (dL < drytol && dR < drytol) {
            } else if (dL < drytol) {
                double hR = dmx(dR, 0.0);
                double vR = normal_velocity(n1, n2, QR.p1, QR.p2, rR);
                fR.s = sqrt(g * hR) + fabs(vR);
                double pr = ((0.5 * g) * hR) * hR;
                fR.p1 = (-((0.5 * vR) * QR.p1) - pr * n1) + (0.5 * fR.s) * QR.p1;
                fR.p2 = (-((0.5 * vR) * QR.p2) - pr * n2) + (0.5 * fR.s) * QR.p2;
            } else {
                double hL = dmx(dL, 0.0);
                double vL = normal_velocity(n1, n2, QL.p1, QL.p2, rL);
                fL.s = sqrt(g * hL) + fabs(vL);
                double pr = ((0.5 * g) * hL) * hL;
                fL.p1 = ((0.5 * vL) * QL.p1 + pr * n1) + (0.5 * fL.s) * QL.p1;
                fL.p2 = ((0.5 * vL) * QL.p2 + pr * n2) + (0.5 * fL.s) * QL.p2;
            }
            return;
        }
        double hL = dmx(dL, 0.0), hR = dmx(dR, 0.0);
        double vL = normal_velocity(n1, n2, QL.p1, QL.p2, rL);
        double vR = normal_velocity(n1, n2, QR.p1, QR.p2, rR);
        fL.s = sqrt(g * hL) + fabs(vL);
        fR.s = sqrt(g * hR) + fabs(vR);
        double alpha = (SOLVER == LLF_BATH) ? dmx(fL.s, fR.s) : 100.0;
        fL.h = 0.5 * ((hL * vL + hR * vR) + alpha * (QL.h - QR.h));
        fR.h = -fL.h;
        double pr = (0.5 * g) * (hL * hL + hR * hR);
        fL.p1 = 0.5 * (((QL.p1 * vL + QR.p1 * vR) + pr * n1) + alpha * (QL.p1 - QR.p1));
        fL.p2 = 0.5 * (((QL.p2 * vL + QR.p2 * vR) + pr * n2) + alpha * (QL.p2 - QR.p2));
        fR.p1 = -fL.p1;
        fR.p2 = -fL.p2;
        double src = ((0.25 * g) * (hL + hR)) * (QR.b - QL.b);
        fL.p1 = fL.p1 + src * n1;
        fL.p2 = fL.p2 + src * n2;
        fR.p1 = fR.p1 + src * n1;
        fR.p2 = fR.p2 + src * n2;
    } else {
        dL = QL.h - 0.0;
        dR = QR.h - 0.0;
        double hL = dmx(dL, 0.0), hR = dmx(dR, 0.0);
        double vL = normal_velocity(n1, n2, QL.p1, QL.p2, dL);
        double vR = normal_velocity(n1, n2, QR.p1, QR.p2, dR);
        fL.s = sqrt(g * dL) + fabs(vL);
        fR.s = sqrt(g * dR) + fabs(vR);
        double alpha = (SOLVER == LLF) ? dmx(fL.s, fR.s) : 100.0;
        fL.h = 0.5 * ((vL * hL + vR * hR) + alpha * (QL.h - QR.h));
        fR.h = -fL.h;
        double sc = (vL * vL) * hL + (vR * vR) * hR;
        double pr = (0.5 * g) * (hL * hL + hR * hR);
        fL.p1 = 0.5 * ((sc + pr * n1) + alpha * (QL.p1 - QR.p1));
        fL.p2 = 0.5 * ((sc + pr * n2) + alpha * (QL.p2 - QR.p2));
        fR.p1 = -fL.p1;
        fR.p2 = -fL.p2;
    }
}

// One edge: dL/dR are the depths h - b of the two states, sqL/sqR their
// sqrt(g * depth) and yL/yR RN(1 / depth) (only read for depths above the dry
// tolerance).
template <int SOLVER, int FZ = 0>
__device__ __forceinline__ void edge_flux(double n1, double n2, const State& QL, const State& QR, double dL,
                                          double dR, double sqL, double sqR, double yL, double yR, double drytol,
                                          Update& fL, Update& fR, int axis = 0, uint16_t* fz = nullptr) {
    if (SOLVER == FWAVE || SOLVER == AUG_RIEMANN)
        geoclaw_flux<SOLVER, FZ>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, drytol, fL, fR, axis, fz);
    else
        lf_flux<SOLVER>(n1, n2, QL, QR, dL, dR, drytol, fL, fR, yL, yR);
}

// depth, sqrt(g * depth) and RN(1 / depth) of a state, as the edge code needs them
__device__ __forceinline__ void depth_terms(const State& Q, double drytol, double& d, double& sq) {
    d = Q.h - Q.b;
    sq = d > drytol ? sqrt(kG * d) : 0.0;
}

__device__ __forceinline__ void depth_terms(const State& Q, double drytol, double& d, double& sq, double& y) {
    d = Q.h - Q.b;
    const bool wet = lt(drytol, d);
    sq = wet ? sqrt(kG * d) : 0.0;
    y = wet ? recip_rn(d).y : 0.0;
}

// Ghost state of bnd_skeleton_scalar_op, src/SWE/SWE_euler_timestep.f90:231-255.
template <int BC>
__device__ __forceinline__ State boundary_ghost(double n1, double n2, const State& Q) {
    State g = Q;
    if (BC == BC_SLIP) {
        double d = z0(Q.p1 * n1) + Q.p2 * n2;
        g.p1 = Q.p1 - d * n1;
        g.p2 = Q.p2 - d * n2;
    } else if (BC == BC_NOSLIP) {
        g.p1 = -Q.p1;
        g.p2 = -Q.p2;
    }
    return g;
}

}  // namespace SWE_KNS
