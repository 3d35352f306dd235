// Discrete adjoint of the SWE step (f-wave and augmented solvers, the four
// Lax-Friedrichs fluxes), hand-written reverse mode.
//
// The step x' = F(x, b; dt) is differentiated on the branches its forward
// evaluation takes (wet/dry fix-ups, wall reconstruction, the Einfeldt
// min/max, the wave-speed signs that split the net updates, the augmented
// solver's Riemann structure, sonic tests and bounds, the LF fluxes' maxima,
// the cell's wetting and drying clamps). dt is frozen (it enters as a
// constant), so the CFL reduction is not differentiated.
//
// Per edge, geoclaw_vjp / lf_vjp re-evaluate the forward flux (the same
// expressions, so the same branches as the forward step) and pull the
// cotangents of the two net updates back to (h, hu, hv, b) of both cells. The reverse-step kernel mirrors the forward kernel: a CTA stages a
// segment, evaluates each edge task's VJP once and writes each side's result
// into a per-(cell, local edge) slot in shared memory (no atomics), then each
// cell sums its slots and its own direct term.
#pragma once

#include "swe_kernel.cuh"

namespace swe {

struct Grad4 {
    double h, hu, hv, b;
};

// ---------------------------------------------------------------------------
// Reverse of the augmented solver (riemann_aug_JCP with riemanntype,
// src/geoclaw/riemannsolvers.f:2-258,507-618). The exact forward (riemann_aug_rec)
// records its branch decisions; the reverse re-evaluates the values it needs in
// plain arithmetic under those decisions and pulls the cotangents of the
// f-waves back to the solver's inputs (the fixed-up depths, momenta,
// bathymetries, velocities, delphi, the Einfeldt speeds and sqrt(g h)).

// d sqrt(x) / dx times b (0 where the root is 0, as the reference gradient has it)
__device__ __forceinline__ double dsqrt(double root, double b) { return gt0(root) ? b * 0.5 / root : 0.0; }

// Cotangents of riemanntype's inputs.
struct RsCot {
    double hL, hR, uL, uR, sqL, sqR;
};
// a / b for cotangents: the reciprocal to about one ulp (rcp_nr) for a normal divisor, else IEEE
__device__ __forceinline__ double cdiv(double a, double b) {
    return exp_in(b, -1000, 1000) ? a * rcp_nr(b) : a / b;
}

__device__ __forceinline__ void rs_rev(const AugRec& r, double hL, double hR, double uL, double uR, double sqL,
                                       double sqR, double b1, double b2, RsCot& c) {
    const double g = kG;
    const double delu = uR - uL;
    double b_delu = 0.0;
    if (r.rs == 0) {  // s1m = s2m = ((uR + uL) - 2 sqR) + 2 sqL
        const double bt = b1 + b2;
        c.uR += bt;
        c.uL += bt;
        c.sqR -= 2.0 * bt;
        c.sqL += 2.0 * bt;
        return;
    }
    if (r.rs == 1) {  // two rarefactions
        const double t = r.t_pos ? -delu + 2.0 * (sqL + sqR) : 0.0;
        const double hm = (1.0 / (16.0 * g)) * (t * t);
        const double sqm = sqrt(g * hm);
        c.uL += b1;
        c.sqL += 2.0 * b1;
        c.uR += b2;
        c.sqR -= 2.0 * b2;
        const double b_sqm = 3.0 * (b2 - b1);
        const double b_hm = dsqrt(sqm, b_sqm * g);
        const double b_t = b_hm * t * ((1.0 / (8.0 * g)));
        if (r.t_pos) {
            b_delu -= b_t;
            c.sqL += 2.0 * b_t;
            c.sqR += 2.0 * b_t;
        }
    } else if (r.rs == 2) {  // two shocks: one Newton step
        const double h0 = r.highR ? hR : hL;
        const double i0 = cdiv(1.0, h0), iL = cdiv(1.0, hL), iR = cdiv(1.0, hR);
        const double gL = sqrt((0.5 * g) * (i0 + iL)), gR = sqrt((0.5 * g) * (i0 + iR));
        const double F0 = (delu + (h0 - hL) * gL) + (h0 - hR) * gR;
        const double kk = 4.0 * (h0 * h0);
        const double eL = cdiv((g * (h0 - hL)), (kk * gL)), eR = cdiv((g * (h0 - hR)), (kk * gR));
        const double dfdh = ((gL - eL) + gR) - eR;
        const double sq0 = sqrt(h0);
        const double slope = 2.0 * sq0 * dfdh;
        const double tt = sq0 - cdiv(F0, slope);
        const double hm = tt * tt, im = cdiv(1.0, hm);
        const double cL = sqrt((0.5 * g) * (im + iL)), cR = sqrt((0.5 * g) * (im + iR));
        const double sqm = sqrt(g * hm);
        // s1m = u1m - sqm, s2m = u2m + sqm
        double b_hm = dsqrt(sqm, (b2 - b1) * g);
        // u2m = uR + (hm - hR) cR, u1m = uL - (hm - hL) cL
        c.uR += b2;
        b_hm = fma(b2, cR, b_hm);
        double b_hR = -b2 * cR;
        const double b_cR = b2 * (hm - hR);
        c.uL += b1;
        b_hm = fma(-b1, cL, b_hm);
        double b_hL = b1 * cL;
        const double b_cL = -b1 * (hm - hL);
        double b_im = 0.0, b_iL = 0.0, b_iR = 0.0, b_i0 = 0.0, b_h0 = 0.0;
        const double aL = dsqrt(cL, b_cL * (0.5 * g)), aR = dsqrt(cR, b_cR * (0.5 * g));
        b_im += aL + aR;
        b_iL += aL;
        b_iR += aR;
        b_hm = fma(-b_im, im * im, b_hm);
        const double b_tt = 2.0 * tt * b_hm;
        // tt = sq0 - F0 / slope, slope = 2 sq0 dfdh
        double b_sq0 = b_tt;
        const double b_F0 = -cdiv(b_tt, slope);
        const double b_slope = b_tt * cdiv(F0, (slope * slope));
        b_sq0 = fma(b_slope, 2.0 * dfdh, b_sq0);
        const double b_dfdh = b_slope * 2.0 * sq0;
        b_h0 += dsqrt(sq0, b_sq0);
        // dfdh = ((gL - eL) + gR) - eR
        double b_gL = b_dfdh, b_gR = b_dfdh;
        const double b_eL = -b_dfdh, b_eR = -b_dfdh;
        double b_kk = 0.0;
        {
            const double q = cdiv(g, (kk * gL));
            b_h0 = fma(b_eL, q, b_h0);
            b_hL = fma(-b_eL, q, b_hL);
            b_kk = fma(-b_eL, cdiv(eL, kk), b_kk);
            b_gL = fma(-b_eL, cdiv(eL, gL), b_gL);
        }
        {
            const double q = cdiv(g, (kk * gR));
            b_h0 = fma(b_eR, q, b_h0);
            b_hR = fma(-b_eR, q, b_hR);
            b_kk = fma(-b_eR, cdiv(eR, kk), b_kk);
            b_gR = fma(-b_eR, cdiv(eR, gR), b_gR);
        }
        b_h0 = fma(b_kk, 8.0 * h0, b_h0);
        // F0 = (delu + (h0 - hL) gL) + (h0 - hR) gR
        b_delu += b_F0;
        b_h0 = fma(b_F0, gL + gR, b_h0);
        b_hL = fma(-b_F0, gL, b_hL);
        b_hR = fma(-b_F0, gR, b_hR);
        b_gL = fma(b_F0, h0 - hL, b_gL);
        b_gR = fma(b_F0, h0 - hR, b_gR);
        // gL = sqrt(0.5 g (i0 + iL)), gR = sqrt(0.5 g (i0 + iR))
        const double bgl = dsqrt(gL, b_gL * (0.5 * g)), bgr = dsqrt(gR, b_gR * (0.5 * g));
        b_i0 += bgl + bgr;
        b_iL += bgl;
        b_iR += bgr;
        b_h0 = fma(-b_i0, i0 * i0, b_h0);
        b_hL = fma(-b_iL, iL * iL, b_hL);
        b_hR = fma(-b_iR, iR * iR, b_hR);
        if (r.highR) b_hR += b_h0;
        else b_hL += b_h0;
        c.hL += b_hL;
        c.hR += b_hR;
    } else {  // one shock, one rarefaction
        const double hmn = r.lowR ? hR : hL, hmx = r.highR ? hR : hL;
        const double sqmn = r.lowR ? sqR : sqL, sqmx = r.highR ? sqR : sqL;
        const double F0 = delu + 2.0 * (sqmn - sqmx);
        const double P = cdiv(((0.5 * g) * (hmx + hmn)), (hmx * hmn));
        const double W = sqrt(P);
        const double Fmax = delu + (hmx - hmn) * W;
        const double den = hmx - hmn;
        const double slope = cdiv((Fmax - F0), den);
        const double hm = hmn - cdiv(F0, slope);
        const double sqm = sqrt(g * hm);
        double b_sqm;
        if (r.lhigh) {
            const double bb = b1 + b2;
            c.uL += bb;
            c.sqL += 2.0 * bb;
            b_sqm = -3.0 * b1 - b2;
        } else {
            const double bb = b1 + b2;
            c.uR += bb;
            c.sqR -= 2.0 * bb;
            b_sqm = 3.0 * b2 + b1;
        }
        const double b_hm = dsqrt(sqm, b_sqm * g);
        // hm = hmn - F0 / slope; slope = (Fmax - F0) / den
        double b_hmn = b_hm, b_hmx = 0.0;
        double b_F0 = -cdiv(b_hm, slope);
        const double b_slope = b_hm * cdiv(F0, (slope * slope));
        const double b_Fmax = cdiv(b_slope, den);
        b_F0 -= cdiv(b_slope, den);
        const double b_den = -b_slope * cdiv(slope, den);
        b_hmx += b_den;
        b_hmn -= b_den;
        // Fmax = delu + (hmx - hmn) W, W = sqrt(P), P = 0.5 g (1 / hmn + 1 / hmx)
        b_delu += b_Fmax;
        b_hmx = fma(b_Fmax, W, b_hmx);
        b_hmn = fma(-b_Fmax, W, b_hmn);
        const double b_P = dsqrt(W, b_Fmax * (hmx - hmn));
        b_hmx = fma(-b_P * (0.5 * g), cdiv(1.0, (hmx * hmx)), b_hmx);
        b_hmn = fma(-b_P * (0.5 * g), cdiv(1.0, (hmn * hmn)), b_hmn);
        // F0 = delu + 2 (sq_min - sq_max)
        b_delu += b_F0;
        if (r.lowR) c.sqR += 2.0 * b_F0;
        else c.sqL += 2.0 * b_F0;
        if (r.highR) c.sqR -= 2.0 * b_F0;
        else c.sqL -= 2.0 * b_F0;
        if (r.lowR) c.hR += b_hmn;
        else c.hL += b_hmn;
        if (r.highR) c.hR += b_hmx;
        else c.hL += b_hmx;
    }
    c.uR += b_delu;
    c.uL -= b_delu;
}

// Cotangents of the augmented solver's inputs.
struct AugCot {
    double hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, sqL, sqR;
};

__device__ __forceinline__ void aug_rev(const AugRec& r, const double F[3][3], double hL, double hR, double huL,
                                        double huR, double bL, double bR, double uL, double uR, double vL, double vR,
                                        double delphi, double sE1in, double sE2in, double sqL, double sqR,
                                        AugCot& c) {
    const double g = kG;
    // ---- forward values on the recorded branches
    const double s1m = r.s1m, s2m = r.s2m;
    const double delh = hR - hL, delhu = huR - huL, delb = bR - bL;
    const double l0 = r.l0_sE1 ? sE1in : s2m, l2 = r.l2_sE2 ? sE2in : s1m;
    const double dsp = l2 - l0;
    const double q = (((huL - huR) + l2 * hR) - l0 * hL) / dsp;
    const double hstar = r.hst_pos ? q : 0.0;
    const double hbar = r.hbar_pos ? 0.5 * (hL + hR) : 0.0;
    const double su = uL + uR;
    const double s1s2bar = 0.25 * (su * su) - g * hbar;
    const double s1s2tilde = (r.tilde_x ? uL * uR : 0.0) - g * hbar;
    const double dgh = (delb * g) * hbar;
    const double ddh0 = r.sonic ? -delb : cdiv(dgh, s1s2bar);
    const double hsd = hstar * dsp;
    double hi = 0.0, lo = 0.0;
    if (r.dcase == 1) {
        hi = cdiv(hsd, l2);
        lo = cdiv(hsd, l0);
    } else if (r.dcase == 2) {
        hi = cdiv(hsd, l0);
        lo = -hL;
    } else if (r.dcase == 3) {
        hi = hR;
        lo = cdiv(hsd, l2);
    }
    const double x1 = r.dd_min_first ? ddh0 : hi;
    const double deldelh = r.dcase ? (r.dd_max_first ? x1 : lo) : ddh0;
    // (deldelphi and d2 = delphi - deldelphi enter beta1 only, linearly: their values are not needed)
    const double d0 = delh - deldelh, d1 = delhu;
    const double det = l0 - l2, id = cdiv(1.0, det);
    const double beta0 = (d1 - l2 * d0) * id, beta2 = (l0 * d0 - d1) * id;
    // ---- reverse
    // fw(3,2) = (((hR uR) vR - (hL uL) vL) - fw(3,1)) - fw(3,3)
    const double F21 = F[2][1];
    c.hR = fma(F21, uR * vR, c.hR);
    c.uR = fma(F21, hR * vR, c.uR);
    c.vR = fma(F21, hR * uR, c.vR);
    c.hL = fma(-F21, uL * vL, c.hL);
    c.uL = fma(-F21, hL * vL, c.uL);
    c.vL = fma(-F21, hL * uL, c.vL);
    const double G20 = F[2][0] - F21, G22 = F[2][2] - F21;
    // fw(1..3, 1) = beta0 (l0, l0^2, l0 vL), fw(2, 2) = beta1, fw(1..3, 3) = beta2 (l2, l2^2, l2 vR)
    double b_b0 = fma(F[0][0], l0, fma(F[1][0], l0 * l0, G20 * l0 * vL));
    double b_l0 = fma(F[0][0], beta0, fma(F[1][0], 2.0 * l0 * beta0, G20 * beta0 * vL));
    c.vL = fma(G20, beta0 * l0, c.vL);
    const double b_b1 = F[1][1];
    double b_b2 = fma(F[0][2], l2, fma(F[1][2], l2 * l2, G22 * l2 * vR));
    double b_l2 = fma(F[0][2], beta2, fma(F[1][2], 2.0 * l2 * beta2, G22 * beta2 * vR));
    c.vR = fma(G22, beta2 * l2, c.vR);
    // beta1 = d2 - l0^2 beta0 - l2^2 beta2
    double b_d2 = b_b1;
    b_b0 = fma(-b_b1, l0 * l0, b_b0);
    b_b2 = fma(-b_b1, l2 * l2, b_b2);
    b_l0 = fma(-b_b1, 2.0 * l0 * beta0, b_l0);
    b_l2 = fma(-b_b1, 2.0 * l2 * beta2, b_l2);
    // beta0 = (d1 - l2 d0) / det, beta2 = (l0 d0 - d1) / det, det = l0 - l2
    double b_d1 = (b_b0 - b_b2) * id;
    double b_d0 = fma(l0, b_b2, -l2 * b_b0) * id;
    b_l2 = fma(-d0 * b_b0, id, b_l2);
    b_l0 = fma(d0 * b_b2, id, b_l0);
    const double b_det = -fma(b_b0, beta0, b_b2 * beta2) * id;
    b_l0 += b_det;
    b_l2 -= b_det;
    // d0 = delh - deldelh, d1 = delhu, d2 = delphi - deldelphi
    double b_delh = b_d0, b_delhu = b_d1, b_delb = 0.0;
    const double b_ddh = -b_d0;
    c.delphi += b_d2;
    const double b_ddphi = -b_d2;
    double b_hbar = 0.0, b_dgh = 0.0, b_sb = 0.0, b_st = 0.0, b_hsd = 0.0;
    // deldelphi = max(y1, g mn), y1 = min(ddp0, g mx)
    double b_pl = 0.0, b_pr = 0.0, b_y1 = 0.0, b_ddp0 = 0.0;
    if (r.ph_max_first) b_y1 = b_ddphi;
    else if (r.ph_mn_pl) b_pl += g * b_ddphi;
    else b_pr += g * b_ddphi;
    if (r.ph_min_first) b_ddp0 = b_y1;
    else if (r.ph_mx_pl) b_pl += g * b_y1;
    else b_pr += g * b_y1;
    // pl = -(hL delb), pr = -(hR delb)
    c.hL = fma(-b_pl, delb, c.hL);
    c.hR = fma(-b_pr, delb, c.hR);
    b_delb = fma(-b_pl, hL, fma(-b_pr, hR, b_delb));
    if (r.sonic) {  // -((g hbar) delb)
        b_hbar = fma(-b_ddp0, g * delb, b_hbar);
        b_delb = fma(-b_ddp0, g * hbar, b_delb);
    } else {  // -((dgh s1s2tilde) / s1s2bar)
        b_dgh = fma(-b_ddp0, cdiv(s1s2tilde, s1s2bar), b_dgh);
        b_st = fma(-b_ddp0, cdiv(dgh, s1s2bar), b_st);
        b_sb = fma(b_ddp0, dgh * cdiv(s1s2tilde, (s1s2bar * s1s2bar)), b_sb);
    }
    // deldelh = max(min(ddh0, hi), lo) in the recorded case
    double b_ddh0 = 0.0;
    if (r.dcase) {
        double b_x1 = 0.0, b_lo = 0.0, b_hi = 0.0;
        if (r.dd_max_first) b_x1 = b_ddh;
        else b_lo = b_ddh;
        if (r.dd_min_first) b_ddh0 = b_x1;
        else b_hi = b_x1;
        if (r.dcase == 1) {  // hi = hsd / l2, lo = hsd / l0
            b_hsd = fma(b_hi, cdiv(1.0, l2), fma(b_lo, cdiv(1.0, l0), b_hsd));
            b_l2 = fma(-b_hi, cdiv(hsd, (l2 * l2)), b_l2);
            b_l0 = fma(-b_lo, cdiv(hsd, (l0 * l0)), b_l0);
        } else if (r.dcase == 2) {  // hi = hsd / l0, lo = -hL
            b_hsd = fma(b_hi, cdiv(1.0, l0), b_hsd);
            b_l0 = fma(-b_hi, cdiv(hsd, (l0 * l0)), b_l0);
            c.hL -= b_lo;
        } else {  // hi = hR, lo = hsd / l2
            c.hR += b_hi;
            b_hsd = fma(b_lo, cdiv(1.0, l2), b_hsd);
            b_l2 = fma(-b_lo, cdiv(hsd, (l2 * l2)), b_l2);
        }
    } else {
        b_ddh0 = b_ddh;
    }
    if (r.sonic) {  // -delb
        b_delb -= b_ddh0;
    } else {  // dgh / s1s2bar
        b_dgh = fma(b_ddh0, cdiv(1.0, s1s2bar), b_dgh);
        b_sb = fma(-b_ddh0, cdiv(dgh, (s1s2bar * s1s2bar)), b_sb);
    }
    // hsd = hstar dsp
    double b_hstar = b_hsd * dsp;
    double b_dsp = b_hsd * hstar;
    // dgh = (delb g) hbar
    b_delb = fma(b_dgh, g * hbar, b_delb);
    b_hbar = fma(b_dgh, g * delb, b_hbar);
    // s1s2tilde = max(0, uL uR) - g hbar, s1s2bar = 0.25 su^2 - g hbar, su = uL + uR
    b_hbar = fma(-(b_st + b_sb), g, b_hbar);
    if (r.tilde_x) {
        c.uL = fma(b_st, uR, c.uL);
        c.uR = fma(b_st, uL, c.uR);
    }
    const double b_su = b_sb * 0.5 * su;
    c.uL += b_su;
    c.uR += b_su;
    if (r.hbar_pos) {
        c.hL += 0.5 * b_hbar;
        c.hR += 0.5 * b_hbar;
    }
    // hstar = max(q, 0), q = (((huL - huR) + l2 hR) - l0 hL) / dsp
    if (r.hst_pos) {
        const double bq = cdiv(b_hstar, dsp);
        c.huL += bq;
        c.huR -= bq;
        b_l2 = fma(bq, hR, b_l2);
        c.hR = fma(bq, l2, c.hR);
        b_l0 = fma(-bq, hL, b_l0);
        c.hL = fma(-bq, l0, c.hL);
        b_dsp = fma(-bq, q, b_dsp);
    }
    // dsp = l2 - l0
    b_l2 += b_dsp;
    b_l0 -= b_dsp;
    // l0 = min(sE1, s2m), l2 = max(sE2, s1m)
    double b_s1m = 0.0, b_s2m = 0.0;
    if (r.l0_sE1) c.sE1 += b_l0;
    else b_s2m += b_l0;
    if (r.l2_sE2) c.sE2 += b_l2;
    else b_s1m += b_l2;
    // delh = hR - hL, delhu = huR - huL, delb = bR - bL
    c.hR += b_delh;
    c.hL -= b_delh;
    c.huR += b_delhu;
    c.huL -= b_delhu;
    c.bR += b_delb;
    c.bL -= b_delb;
    RsCot rc{0.0, 0.0, 0.0, 0.0, 0.0, 0.0};
    rs_rev(r, hL, hR, uL, uR, sqL, sqR, b_s1m, b_s2m, rc);
    c.hL += rc.hL;
    c.hR += rc.hR;
    c.uL += rc.uL;
    c.uR += rc.uR;
    c.sqL += rc.sqL;
    c.sqR += rc.sqR;
}

// VJP of the f-wave edge flux: given the cotangents gL / gR of the left/right
// net updates (h, hu, hv, world frame), add the cotangents of the inputs to
// outL / outR. QL / QR are the states (h = surface), dL / dR their depths,
// sqL0 / sqR0 their sqrt(g * depth) as in the forward step.
// axis: the normal's direction as in geoclaw_flux (0 diagonal, 1 along x, 2 along y).
// SOLVER: FWAVE or AUG_RIEMANN (the solver core between the shared wet/dry
// handling, Einfeldt speeds and net-update split of c_bind_geoclaw_solver_dp).
template <int SOLVER>
__device__ __forceinline__ void geoclaw_vjp(double n1, double n2, const State& QL, const State& QR, double dL0,
                                            double dR0, double sqL0, double sqR0, double yL0, double yR0,
                                            double drytol, const double gL[3], const double gR[3], Grad4& outL,
                                            Grad4& outR, int axis = 0) {
    const double g = kG;
    const double c = 0.5 * g;
    if (SOLVER == FWAVE) {
        // Water at rest on both sides under one surface (the forward step's
        // lake-at-rest path: every momentum +-0, both sides wet, the surface
        // difference ((bR + dR) - bL) - dL a zero). There beta1 = beta2 = 0 and
        // every velocity is 0, so to first order only the coefficients move:
        // d beta1 = (sE2 d delhu - d dpd) / D, d beta2 = (d dpd - sE1 d delhu) / D
        // (D = sE2 - sE1; the derivatives through sE1, sE2 and D multiply a zero),
        // d dpd = ghalf_h (d hR' - d hL') with h' the surfaces (the surface
        // difference multiplies the zero, and b cancels between delphi and
        // deldelphi), d delhu = n . (d pR - d pL). The left net update is
        // beta1 (1, sE1 n) (sE1 < 0), the right one beta2 (1, sE2 n) (sE2 > 0);
        // the middle wave's components are products of two zeros.
        const bool still = ((dbits(QL.p1) | dbits(QL.p2) | dbits(QR.p1) | dbits(QR.p2)) << 1) == 0;
        // (the surface difference x - dL0 is a zero exactly when x = RN(RN(bR + dR0) - bL) equals dL0 > 0 and
        // both are finite, as in the forward step's test)
        if (still && lt(drytol, dL0) && lt(drytol, dR0) && dbits((QR.b + dR0) - QL.b) == dbits(dL0) &&
            is_finite(dL0)) {
            const double ghalf = c * (dR0 + dL0);
            const double chat = sqrt(ghalf);
            const double sE1 = -imax(sqL0, chat), sE2 = imax(sqR0, chat);
            const double rD = rcp_nr(sE2 - sE1);
            // n . (g1, g2) of each side's cotangent: a signed component for the
            // axis-aligned normals (1, 0) and (0, 1) up to sign, whose other
            // component is a zero; the cotangents need no bit-exact rounding, so
            // products are fused
            const bool ax = axis != 0;
            const int k = axis == 2 ? 2 : 1;
            const bool sg = axis == 2 ? lt0(n2) : lt0(n1);
            const double nL = ax ? flip(gL[k], sg) : fma(n1, gL[1], n2 * gL[2]);
            const double nR = ax ? flip(gR[k], sg) : fma(n1, gR[1], n2 * gR[2]);
            const double gb1 = fma(sE1, nL, gL[0]);
            const double gb2 = fma(sE2, nR, gR[0]);
            const double g_du = fma(sE2, gb1, -(sE1 * gb2)) * rD;  // cotangent of delhu
            const double g_dh = ghalf * ((gb2 - gb1) * rD);          // of hR' (minus it for hL')
            outL.h -= g_dh;
            outR.h += g_dh;
            if (ax) {
                const double t = flip(g_du, sg);
                if (k == 1) {
                    outL.hu -= t;
                    outR.hu += t;
                } else {
                    outL.hv -= t;
                    outR.hv += t;
                }
            } else {
                outL.hu = fma(-g_du, n1, outL.hu);
                outL.hv = fma(-g_du, n2, outL.hv);
                outR.hu = fma(g_du, n1, outR.hu);
                outR.hv = fma(g_du, n2, outR.hv);
            }
            return;
        }
    }
    // ---------------- forward (geoclaw_flux<SOLVER>, the same values)
    const bool fin = is_finite(QL.p1) && is_finite(QL.p2) && is_finite(QR.p1) && is_finite(QR.p2);
    const bool fast = axis != 0 && fin;
    const bool sn = axis == 1 ? lt0(n1) : lt0(n2);
    double pL1, pL2, pR1, pR2;
    if (axis == 0 && fin && abs_bits(n1) == abs_bits(n2)) {  // diagonal: two products per side
        const bool g1 = dbits(n1) < 0, g2 = dbits(n2) < 0;
        const double cn = bitsd(abs_bits(n1));
        const double aL1 = cn * QL.p1, aL2 = cn * QL.p2, aR1 = cn * QR.p1, aR2 = cn * QR.p2;
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
        pL1 = z0(n1 * QL.p1) + n2 * QL.p2;
        pL2 = z0(-n2 * QL.p1) + n1 * QL.p2;
        pR1 = z0(n1 * QR.p1) + n2 * QR.p2;
        pR2 = z0(-n2 * QR.p1) + n1 * QR.p2;
    }
    double hL = dL0, hR = dR0, bL = QL.b, bR = QR.b;
    const bool wetR = lt(drytol, hR), wetL = lt(drytol, hL);
    if (!wetL && !wetR && !is_nan(hL) && !is_nan(hR)) return;  // no flux, no derivative
    double huL, huR, uL, uR, vL, vR;
    // a wet cell whose reciprocal was left for the edges that need it (f-wave, zero momenta)
    if (SOLVER == FWAVE && wetR && dbits(yR0) == 0) yR0 = recip_rn(hR).y;
    if (SOLVER == FWAVE && wetL && dbits(yL0) == 0) yL0 = recip_rn(hL).y;
    if (wetR) {
        const Recip r{hR, yR0, recip_fast(hR)};
        huR = pR1; uR = div_rn(pR1, r); vR = div_rn(pR2, r);
    } else {
        hR = 0.0; huR = 0.0; uR = 0.0; vR = 0.0;
    }
    if (wetL) {
        const Recip r{hL, yL0, recip_fast(hL)};
        huL = pL1; uL = div_rn(pL1, r); vL = div_rn(pL2, r);
    } else {
        hL = 0.0; huL = 0.0; uL = 0.0; vL = 0.0;
    }
    bool wall_l = false, wall_r = false, lower_l = false, lower_r = false;
    if (!wetR) {
        double hstar, s1m, s2m;
        riemann_structure(hL, hL, uL, -uL, drytol, hstar, s1m, s2m);
        if (dmx(hL, hstar) + bL < bR) {
            wall_r = true;
            hR = hL; huR = -huL; bR = bL; uR = -uL; vR = vL;
        } else if (hL + bL < bR) {
            lower_r = true;
            bR = hL + bL;
        }
    } else if (!wetL) {
        double hstar, s1m, s2m;
        riemann_structure(hR, hR, -uR, uR, drytol, hstar, s1m, s2m);
        if (dmx(hR, hstar) + bR < bL) {
            wall_l = true;
            hL = hR; huL = -huR; bL = bR; uL = -uR; vL = vR;
        } else if (hR + bR < bL) {
            lower_l = true;
            bL = hR + bR;
        }
    }
    const double X = ((bR + hR) - bL) - hL;
    const double Hs = hR + hL;
    const double dB = bR - bL;
    const double sqL = (wetL || wall_l) ? (wall_l ? sqR0 : sqL0) : 0.0;
    const double sqR = (wetR || wall_r) ? (wall_r ? sqL0 : sqR0) : 0.0;
    const double sL = uL - sqL, sR = uR + sqR;
    const double A = sqL * uL + sqR * uR, B = sqR + sqL;
    const Recip rB = recip_rn(B);
    const double uhat = div_rn(A, rB);
    const double chat = sqrt((g * 0.5) * Hs);
    const double r1 = uhat - chat, r2 = uhat + chat;
    const bool e1_is_sL = lt(sL, r1), e2_is_sR = lt(r2, sR);
    const double sE1 = e1_is_sL ? sL : r1, sE2 = e2_is_sR ? sR : r2;
    const double delphi = ((((huR - huL) * (uL + uR)) - ((uL * uR) * (hR - hL))) + ((c * X) * Hs)) - ((c * Hs) * dB);
    const double delhu = huR - huL;
    const double K = (g * 0.5) * Hs;
    double beta1 = 0.0, beta2 = 0.0, sw[3];
    Recip rD{1.0, 1.0, false};
    AugRec rec{};
    if (SOLVER == FWAVE) {
        const double ddp = -(K * dB);
        const double dpd = delphi - ddp;
        const double D = sE2 - sE1;
        rD = recip_rn(D);
        beta1 = div_rn(sE2 * delhu - dpd, rD);
        beta2 = div_rn(dpd - sE1 * delhu, rD);
        sw[0] = sE1;
        sw[1] = 0.5 * (sE1 + sE2);
        sw[2] = sE2;
    } else {  // the same call as geoclaw_solver's, recording the branch decisions
        const double yLf = wall_l ? yR0 : yL0, yRf = wall_r ? yL0 : yR0;
        const bool okL = (wetL || wall_l) && recip_fast(hL), okR = (wetR || wall_r) && recip_fast(hR);
        double fwa[3][3];
        riemann_aug_rec<true>(hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, sqL, sqR, yLf, yRf, okL,
                              okR, drytol, sw, fwa, &rec);
    }
    // ---------------- reverse (cotangents: products fused into FMAs where they feed a sum; they
    // need no bit-exact agreement, only the forward recompute above does)
    // back-rotation p = net(2:3) T (for an axis-aligned normal: signed selections)
    double nL[3], nR[3];
    nL[0] = gL[0];
    nR[0] = gR[0];
    if (axis == 1) {
        nL[1] = flip(gL[1], sn); nL[2] = flip(gL[2], sn);
        nR[1] = flip(gR[1], sn); nR[2] = flip(gR[2], sn);
    } else if (axis == 2) {
        nL[1] = flip(gL[2], sn); nL[2] = flip(gL[1], !sn);
        nR[1] = flip(gR[2], sn); nR[2] = flip(gR[1], !sn);
    } else {
        nL[1] = fma(gL[1], n1, gL[2] * n2); nL[2] = fma(-gL[1], n2, gL[2] * n1);
        nR[1] = fma(gR[1], n1, gR[2] * n2); nR[2] = fma(-gR[1], n2, gR[2] * n1);
    }
    // net-update split by wave-speed sign; walls remove waves
    double F[3][3];
#pragma unroll
    for (int w = 0; w < 3; ++w) {
        const bool zeroed = (wall_l && w < 2) || (wall_r && w > 0);
        const bool neg = lt0(sw[w]), pos = gt0(sw[w]);
#pragma unroll
        for (int e = 0; e < 3; ++e) {
            double f = neg ? nL[e] : (pos ? nR[e] : 0.5 * (nL[e] + nR[e]));
            F[e][w] = zeroed ? 0.0 : f;
        }
    }
    double b_huR, b_vR, b_huL, b_vL, b_sE1, b_sE2, b_delphi, b_dB, b_Hs;
    // the solver core's cotangents of hL, hR, bL, bR, uL, uR, sqrt(g h) (the f-wave has
    // them through delphi, K and the Einfeldt speeds only)
    double k_hL = 0.0, k_hR = 0.0, k_bL = 0.0, k_bR = 0.0, k_uL = 0.0, k_uR = 0.0, k_sqL = 0.0, k_sqR = 0.0;
    if (SOLVER == FWAVE) {
        // fw(3,2) = ((huR vR - huL vL) - fw(3,1)) - fw(3,3); wave 2 carries no h / hu
        b_huR = F[2][1] * vR;
        b_vR = F[2][1] * huR;
        b_huL = -F[2][1] * vL;
        b_vL = -F[2][1] * huL;
        const double F30 = F[2][0] - F[2][1], F32 = F[2][2] - F[2][1];
        double b_beta1 = fma(F30, vL, fma(F[1][0], sE1, F[0][0]));
        double b_beta2 = fma(F32, vR, fma(F[1][2], sE2, F[0][2]));
        b_sE1 = F[1][0] * beta1;
        b_sE2 = F[1][2] * beta2;
        b_vL = fma(F30, beta1, b_vL);
        b_vR = fma(F32, beta2, b_vR);
        // beta1 = (sE2 delhu - dpd) / D, beta2 = (dpd - sE1 delhu) / D, D = sE2 - sE1
        const double N1b = b_beta1 * rD.y, N2b = b_beta2 * rD.y;
        const double b_D = -fma(b_beta1, beta1, b_beta2 * beta2) * rD.y;
        b_sE2 += fma(N1b, delhu, b_D);
        b_sE1 -= fma(N2b, delhu, b_D);
        double b_delhu = fma(N1b, sE2, -(N2b * sE1));
        const double b_dpd = N2b - N1b;
        // dpd = delphi - ddp, ddp = -(K dB), K = c Hs
        b_delphi = b_dpd;
        const double b_ddp = -b_dpd;
        double b_K = -b_ddp * dB;
        b_dB = -b_ddp * K;
        b_Hs = b_K * c;
        // delhu = huR - huL
        b_huR += b_delhu;
        b_huL -= b_delhu;
    } else {
        AugCot ac{};
        aug_rev(rec, F, hL, hR, huL, huR, bL, bR, uL, uR, vL, vR, delphi, sE1, sE2, sqL, sqR, ac);
        b_huR = ac.huR;
        b_huL = ac.huL;
        b_vR = ac.vR;
        b_vL = ac.vL;
        b_sE1 = ac.sE1;
        b_sE2 = ac.sE2;
        b_delphi = ac.delphi;
        b_dB = 0.0;
        b_Hs = 0.0;
        k_hL = ac.hL;
        k_hR = ac.hR;
        k_bL = ac.bL;
        k_bR = ac.bR;
        k_uL = ac.uL;
        k_uR = ac.uR;
        k_sqL = ac.sqL;
        k_sqR = ac.sqR;
    }
    // Einfeldt speeds
    double b_sL = e1_is_sL ? b_sE1 : 0.0, b_r1 = e1_is_sL ? 0.0 : b_sE1;
    double b_sR = e2_is_sR ? b_sE2 : 0.0, b_r2 = e2_is_sR ? 0.0 : b_sE2;
    const double b_uhat = b_r1 + b_r2;
    const double b_chat = b_r2 - b_r1;
    if (chat > 0.0) b_Hs = fma(b_chat * (0.5 * rcp_nr(chat)), g * 0.5, b_Hs);
    double b_uL = b_sL + k_uL, b_uR = b_sR + k_uR;
    double b_sqL = k_sqL - b_sL, b_sqR = b_sR + k_sqR;
    const double b_A = b_uhat * rB.y, b_B = -b_uhat * uhat * rB.y;
    b_sqL += fma(b_A, uL, b_B);
    b_sqR += fma(b_A, uR, b_B);
    b_uL = fma(b_A, sqL, b_uL);
    b_uR = fma(b_A, sqR, b_uR);
    // delphi = ((T1 - T2) + T3) - T4
    {
        const double d = b_delphi;
        const double su = uL + uR, dhu = huR - huL, uu = uL * uR, dh = hR - hL;
        const double dsu = d * su;
        b_huR += dsu;
        b_huL -= dsu;
        b_uL += fma(d, dhu, -(d * uR * dh));
        b_uR += fma(d, dhu, -(d * uL * dh));
        double b_hR = fma(-d, uu, k_hR), b_hL = fma(d, uu, k_hL);
        const double b_X = d * c * Hs;
        b_Hs += fma(d, c * X, -(d * c * dB));
        b_dB = fma(-d, c * Hs, b_dB);
        // X = ((bR + hR) - bL) - hL
        double b_bR = b_X + k_bR, b_bL = k_bL - b_X;
        b_hR += b_X;
        b_hL -= b_X;
        // Hs = hR + hL, dB = bR - bL
        b_hR += b_Hs;
        b_hL += b_Hs;
        b_bR += b_dB;
        b_bL -= b_dB;
        // sqrt(g h) of the fixed-up depths
        if (sqL > 0.0) b_hL = fma(b_sqL, 0.5 * g * rcp_nr(sqL), b_hL);
        if (sqR > 0.0) b_hR = fma(b_sqR, 0.5 * g * rcp_nr(sqR), b_hR);
        // undo the wall / lowering fix-ups: map the cotangents back to the original sides
        double b_hL0 = 0.0, b_hR0 = 0.0, b_bL0 = 0.0, b_bR0 = 0.0;
        if (wall_r) {  // hR = hL, huR = -huL, bR = bL, uR = -uL, vR = vL
            b_hL += b_hR; b_hR = 0.0;
            b_huL -= b_huR; b_huR = 0.0;
            b_bL += b_bR; b_bR = 0.0;
            b_uL -= b_uR; b_uR = 0.0;
            b_vL += b_vR; b_vR = 0.0;
        } else if (lower_r) {  // bR = hL + bL
            b_hL += b_bR;
            b_bL += b_bR;
            b_bR = 0.0;
        }
        if (wall_l) {
            b_hR += b_hL; b_hL = 0.0;
            b_huR -= b_huL; b_huL = 0.0;
            b_bR += b_bL; b_bL = 0.0;
            b_uR -= b_uL; b_uL = 0.0;
            b_vR += b_vL; b_vL = 0.0;
        } else if (lower_l) {
            b_hR += b_bL;
            b_bR += b_bL;
            b_bL = 0.0;
        }
        b_bL0 = b_bL;
        b_bR0 = b_bR;
        // wet extraction: u = hu / h, v = hv / h on wet sides; dry sides are constants
        double b_pL1 = 0.0, b_pL2 = 0.0, b_pR1 = 0.0, b_pR2 = 0.0;
        if (wetR) {
            b_pR1 += fma(b_uR, yR0, b_huR);
            b_pR2 = fma(b_vR, yR0, b_pR2);
            b_hR0 = fma(-fma(b_uR, uR, b_vR * vR), yR0, b_hR);
        }
        if (wetL) {
            b_pL1 += fma(b_uL, yL0, b_huL);
            b_pL2 = fma(b_vL, yL0, b_pL2);
            b_hL0 = fma(-fma(b_uL, uL, b_vL * vL), yL0, b_hL);
        }
        // depths h - b, rotations p_edge = T p
        outL.h += b_hL0;
        outL.b += b_bL0 - b_hL0;
        outR.h += b_hR0;
        outR.b += b_bR0 - b_hR0;
        if (axis == 1) {
            outL.hu += flip(b_pL1, sn); outL.hv += flip(b_pL2, sn);
            outR.hu += flip(b_pR1, sn); outR.hv += flip(b_pR2, sn);
        } else if (axis == 2) {
            outL.hu += flip(b_pL2, !sn); outL.hv += flip(b_pL1, sn);
            outR.hu += flip(b_pR2, !sn); outR.hv += flip(b_pR1, sn);
        } else {
            outL.hu += fma(b_pL1, n1, -(b_pL2 * n2));
            outL.hv += fma(b_pL1, n2, b_pL2 * n1);
            outR.hu += fma(b_pR1, n1, -(b_pR2 * n2));
            outR.hv += fma(b_pR1, n2, b_pR2 * n1);
        }
    }
}

// VJP of the Lax-Friedrichs fluxes (compute_lf_flux, src/SWE/SWE_euler_timestep.f90:359-446):
// with the cotangents gL / gR of the left/right (h, hu, hv) updates, add the
// cotangents of the two states (h = surface, hu, hv, b) to outL / outR. Every
// max, |v| and the dry-side tests are differentiated on the branch taken; the
// maximum wave speed matters where it enters the flux (the dry-side momentum
// flux and the local LF alpha).
__device__ __forceinline__ double sgn(double x) { return lt0(x) ? -1.0 : (gt0(x) ? 1.0 : 0.0); }

// Normal velocity v = n1 (p1 / d) + n2 (p2 / d): adds its cotangent bv to p1, p2 and d.
__device__ __forceinline__ void nv_vjp(double n1, double n2, double v, double d, double bv, double& bp1,
                                       double& bp2, double& bd) {
    const double r = cdiv(1.0, d);
    bp1 = fma(bv * n1, r, bp1);
    bp2 = fma(bv * n2, r, bp2);
    bd = fma(-bv * v, r, bd);
}

// d sqrt(g h) / dh times bs (0 where h = 0, as the reference gradient has it)
__device__ __forceinline__ double sqrt_g_vjp(double h, double bs) {
    return gt0(h) ? cdiv(bs * (0.5 * kG), sqrt(kG * h)) : 0.0;
}

template <int SOLVER>
__device__ __forceinline__ void lf_vjp(double n1, double n2, const State& QL, const State& QR, double dL0,
                                       double dR0, double drytol, const double gL[3], const double gR[3],
                                       Grad4& outL, Grad4& outR) {
    const double g = kG;
    if (SOLVER == LF_BATH || SOLVER == LLF_BATH) {
        const double dL = dL0, dR = dR0;
        const bool dryL = dL < drytol, dryR = dR < drytol;
        if (dryL || dryR) {
            if (dryL && dryR) return;
            // one wet side W: f_W.p = s_W (+-0.5 v_W p - pr n) + 0.5 sp p, f_W.h = 0
            const bool right = dryL;
            const State& Q = right ? QR : QL;
            const double d = right ? dR : dL;
            const double* gg = right ? gR : gL;
            const double sgw = right ? -1.0 : 1.0;  // fR: -(0.5 v p) - pr n; fL: +(0.5 v p) + pr n
            const double hw = dmx(d, 0.0);
            const double v = normal_velocity(n1, n2, Q.p1, Q.p2, d);
            const double sp = sqrt(g * hw) + fabs(v);
            double b_v = sgw * 0.5 * fma(gg[1], Q.p1, gg[2] * Q.p2);
            const double b_pr = sgw * fma(gg[1], n1, gg[2] * n2);
            const double b_sp = 0.5 * fma(gg[1], Q.p1, gg[2] * Q.p2);
            const double k = fma(sgw * 0.5, v, 0.5 * sp);
            double b_p1 = gg[1] * k, b_p2 = gg[2] * k;
            double b_h = b_pr * (g * hw) + sqrt_g_vjp(hw, b_sp);
            b_v = fma(b_sp, sgn(v), b_v);
            double b_d = gt0(d) ? b_h : 0.0;
            nv_vjp(n1, n2, v, d, b_v, b_p1, b_p2, b_d);
            Grad4& o = right ? outR : outL;
            o.h += b_d;
            o.hu += b_p1;
            o.hv += b_p2;
            o.b -= b_d;
            return;
        }
        const double hL = dmx(dL, 0.0), hR = dmx(dR, 0.0);
        const double vL = normal_velocity(n1, n2, QL.p1, QL.p2, dL);
        const double vR = normal_velocity(n1, n2, QR.p1, QR.p2, dR);
        const double sL = sqrt(g * hL) + fabs(vL), sR = sqrt(g * hR) + fabs(vR);
        const bool left_max = sL > sR;
        const double alpha = (SOLVER == LLF_BATH) ? (left_max ? sL : sR) : 100.0;
        // fL = (F_h, F_p1 + src n1, F_p2 + src n2), fR = (-F_h, -F_p1 + src n1, -F_p2 + src n2)
        const double bFh = gL[0] - gR[0], bF1 = gL[1] - gR[1], bF2 = gL[2] - gR[2];
        const double b_src = fma(gL[1] + gR[1], n1, (gL[2] + gR[2]) * n2);
        double b_hL = 0.5 * bFh * vL, b_hR = 0.5 * bFh * vR;
        double b_vL = 0.5 * fma(bFh, hL, fma(bF1, QL.p1, bF2 * QL.p2));
        double b_vR = 0.5 * fma(bFh, hR, fma(bF1, QR.p1, bF2 * QR.p2));
        const double b_alpha = 0.5 * fma(bFh, QL.h - QR.h, fma(bF1, QL.p1 - QR.p1, bF2 * (QL.p2 - QR.p2)));
        double b_hsL = 0.5 * bFh * alpha, b_hsR = -0.5 * bFh * alpha;
        double b_pL1 = 0.5 * bF1 * (vL + alpha), b_pR1 = 0.5 * bF1 * (vR - alpha);
        double b_pL2 = 0.5 * bF2 * (vL + alpha), b_pR2 = 0.5 * bF2 * (vR - alpha);
        const double b_pr = 0.5 * fma(bF1, n1, bF2 * n2);
        b_hL = fma(b_pr * g, hL, b_hL);
        b_hR = fma(b_pr * g, hR, b_hR);
        const double cs = (0.25 * g) * (QR.b - QL.b), ch = (0.25 * g) * (hL + hR);
        b_hL = fma(b_src, cs, b_hL);
        b_hR = fma(b_src, cs, b_hR);
        double b_bR = b_src * ch, b_bL = -b_src * ch;
        double b_sL = 0.0, b_sR = 0.0;
        if (SOLVER == LLF_BATH) {
            if (left_max) b_sL = b_alpha;
            else b_sR = b_alpha;
        }
        b_hL += sqrt_g_vjp(hL, b_sL);
        b_hR += sqrt_g_vjp(hR, b_sR);
        b_vL = fma(b_sL, sgn(vL), b_vL);
        b_vR = fma(b_sR, sgn(vR), b_vR);
        double b_dL = gt0(dL) ? b_hL : 0.0, b_dR = gt0(dR) ? b_hR : 0.0;
        nv_vjp(n1, n2, vL, dL, b_vL, b_pL1, b_pL2, b_dL);
        nv_vjp(n1, n2, vR, dR, b_vR, b_pR1, b_pR2, b_dR);
        outL.h += b_hsL + b_dL;
        outL.hu += b_pL1;
        outL.hv += b_pL2;
        outL.b += b_bL - b_dL;
        outR.h += b_hsR + b_dR;
        outR.hu += b_pR1;
        outR.hv += b_pR2;
        outR.b += b_bR - b_dR;
    } else {
        // no bathymetry: depth = surface
        const double dL = QL.h - 0.0, dR = QR.h - 0.0;
        const double hL = dmx(dL, 0.0), hR = dmx(dR, 0.0);
        const double vL = normal_velocity(n1, n2, QL.p1, QL.p2, dL);
        const double vR = normal_velocity(n1, n2, QR.p1, QR.p2, dR);
        const double sL = sqrt(g * dL) + fabs(vL), sR = sqrt(g * dR) + fabs(vR);
        const bool left_max = sL > sR;
        const double alpha = (SOLVER == LLF) ? (left_max ? sL : sR) : 100.0;
        const double bFh = gL[0] - gR[0], bF1 = gL[1] - gR[1], bF2 = gL[2] - gR[2];
        const double b_sc = 0.5 * (bF1 + bF2);
        const double b_pr = 0.5 * fma(bF1, n1, bF2 * n2);
        const double b_alpha = 0.5 * fma(bFh, QL.h - QR.h, fma(bF1, QL.p1 - QR.p1, bF2 * (QL.p2 - QR.p2)));
        double b_hsL = 0.5 * bFh * alpha, b_hsR = -0.5 * bFh * alpha;
        double b_pL1 = 0.5 * bF1 * alpha, b_pR1 = -0.5 * bF1 * alpha;
        double b_pL2 = 0.5 * bF2 * alpha, b_pR2 = -0.5 * bF2 * alpha;
        double b_vL = fma(0.5 * bFh, hL, b_sc * 2.0 * vL * hL), b_vR = fma(0.5 * bFh, hR, b_sc * 2.0 * vR * hR);
        double b_hL = fma(0.5 * bFh, vL, fma(b_sc, vL * vL, b_pr * g * hL));
        double b_hR = fma(0.5 * bFh, vR, fma(b_sc, vR * vR, b_pr * g * hR));
        double b_sL = 0.0, b_sR = 0.0;
        if (SOLVER == LLF) {
            if (left_max) b_sL = b_alpha;
            else b_sR = b_alpha;
        }
        b_vL = fma(b_sL, sgn(vL), b_vL);
        b_vR = fma(b_sR, sgn(vR), b_vR);
        double b_dL = (gt0(dL) ? b_hL : 0.0) + sqrt_g_vjp(dL, b_sL);
        double b_dR = (gt0(dR) ? b_hR : 0.0) + sqrt_g_vjp(dR, b_sR);
        nv_vjp(n1, n2, vL, dL, b_vL, b_pL1, b_pL2, b_dL);
        nv_vjp(n1, n2, vR, dR, b_vR, b_pR1, b_pR2, b_dR);
        outL.h += b_hsL + b_dL;
        outL.hu += b_pL1;
        outL.hv += b_pL2;
        outR.h += b_hsR + b_dR;
        outR.hu += b_pR1;
        outR.hv += b_pR2;
    }
}

// Cotangent of a boundary ghost state pulled back to the cell (the ghost of
// bnd_skeleton_scalar_op is a linear function of the cell state).
template <int BC>
__device__ __forceinline__ void boundary_ghost_vjp(double n1, double n2, const Grad4& gg, Grad4& out) {
    out.h += gg.h;
    out.b += gg.b;
    if (BC == BC_SLIP) {  // p - (p . n) n
        const double d = gg.hu * n1 + gg.hv * n2;
        out.hu += gg.hu - d * n1;
        out.hv += gg.hv - d * n2;
    } else if (BC == BC_NOSLIP) {
        out.hu -= gg.hu;
        out.hv -= gg.hv;
    } else {
        out.hu += gg.hu;
        out.hv += gg.hv;
    }
}

struct AdjointArgs {
    const double* h;          // x_t (state before the step)
    const double* hu;
    const double* hv;
    const double* b;
    const int8_t* depth;
    const uint8_t* branch;    // per cell: bit 0 wetting fix fired, bit 1 drying clamp fired (forward step t)
    const double* lam_h;      // cotangent of x_{t+1}
    const double* lam_hu;
    const double* lam_hv;
    double* out_h;            // cotangent of x_t
    double* out_hu;
    double* out_hv;
    double* bbar;             // += cotangent of b
    const int4* tasks;
    const long long* seg_ptr;
    const int4* seg_info;
    InstParams P;
    double dt;
    int32_t n_seg, seg_cells, n_cells_total, parity;
    unsigned int* error;
    double2* memo;            // per cell (d, sqrt(g d)) shared with the forward step, or null
    // per depth d: -dt / volume(d) and scaling * sqrt(0.5)^(d - 1) (edge lengths: the
    // hypotenuse of a depth-d cell is len[d], its legs len[d + 1]), computed on the host
    // with the same operations the cells would do, once per launch
    double ndv_tab[kMaxDepth + 1];
    double len_tab[kMaxDepth + 2];
};

// mu = -dt / volume * lambda' where the drying clamp did not fire: the
// cotangent of the (length-weighted) sum of a cell's edge updates
__device__ __forceinline__ void cell_mu(const AdjointArgs& A, int c, double ndv, double& m0, double& m1, double& m2) {
    if (A.branch[c] & 2u) {
        m0 = m1 = m2 = 0.0;
    } else {
        m0 = ndv * A.lam_h[c];
        m1 = ndv * A.lam_hu[c];
        m2 = ndv * A.lam_hv[c];
    }
}

// The edge VJP of the step's flux for each solver.
template <int SOLVER>
__device__ __forceinline__ void edge_vjp(double n1, double n2, const State& QL, const State& QR, double dL,
                                         double dR, double sqL, double sqR, double yL, double yR, double drytol,
                                         const double gL[3], const double gR[3], Grad4& oL, Grad4& oR, int axis) {
    if (SOLVER == FWAVE || SOLVER == AUG_RIEMANN)
        geoclaw_vjp<SOLVER>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, drytol, gL, gR, oL, oR, axis);
    else
        lf_vjp<SOLVER>(n1, n2, QL, QR, dL, dR, drytol, gL, gR, oL, oR);
}

// Launch bounds of the reverse kernel: at most 256 threads; with SWE_ADJ_MIN_BLOCKS
// defined, also that many resident CTAs of 256 threads (registers capped at
// 65536 / (256 * SWE_ADJ_MIN_BLOCKS)). Undefined: the compiler's own register choice.
#ifdef SWE_ADJ_MIN_BLOCKS
#define SWE_ADJ_BOUNDS __launch_bounds__(256, SWE_ADJ_MIN_BLOCKS)
#else
#define SWE_ADJ_BOUNDS __launch_bounds__(256)
#endif

template <int SOLVER>
__global__ void SWE_ADJ_BOUNDS adjoint_kernel(const AdjointArgs A) {
    extern __shared__ __align__(16) unsigned char smem_raw[];
    const int T = A.seg_cells;
    double* sh_h = reinterpret_cast<double*>(smem_raw);
    double* sh_hu = sh_h + T;
    double* sh_hv = sh_hu + T;
    double* sh_b = sh_hv + T;
    double* sh_rh = sh_b + T;          // RN(1 / depth) where wet
    double* sh_sq = sh_rh + T;
    double* sh_mu = sh_sq + T;         // [3][T]
    double* slot = sh_mu + 3 * T;      // [4 quantities][3 local edges][T]
    const InstParams& P = A.P;
    const int tid = threadIdx.x;
    const int odd = A.parity & 1;

    for (int seg = blockIdx.x; seg < A.n_seg; seg += gridDim.x) {
        const int4 si = __ldg(&A.seg_info[seg]);
        const int c0 = si.x, cn = si.y;
        if (tid == 0 && seg + (int)gridDim.x < A.n_seg) {
            // this CTA's next segment (the deal is static) is on its way to L2
            // while the CTA works on this one: its state, cotangents, bathymetry
            // cotangent, memo entries, depths, branch records and edge tasks
            const int nx = seg + (int)gridDim.x;
            const int4 sn = __ldg(&A.seg_info[nx]);
            const size_t bytes = (size_t)sn.y * 8u;
            prefetch_l2(A.h + sn.x, bytes);
            prefetch_l2(A.hu + sn.x, bytes);
            prefetch_l2(A.hv + sn.x, bytes);
            prefetch_l2(A.b + sn.x, bytes);
            prefetch_l2(A.lam_h + sn.x, bytes);
            prefetch_l2(A.lam_hu + sn.x, bytes);
            prefetch_l2(A.lam_hv + sn.x, bytes);
            prefetch_l2(A.bbar + sn.x, bytes);
            if (A.memo) prefetch_l2(A.memo + sn.x, (size_t)sn.y * 16u);
            prefetch_l2(A.depth + sn.x, (size_t)sn.y);
            prefetch_l2(A.branch + sn.x, (size_t)sn.y);
            const long long a = __ldg(&A.seg_ptr[nx]), e = __ldg(&A.seg_ptr[nx + 1]);
            prefetch_l2(A.tasks + a, (size_t)(e - a) * 16u);
        }
        for (int i = tid; i < cn; i += blockDim.x) {
            const int cc = c0 + i;
            const double h = A.h[cc], b = A.b[cc];
            sh_h[i] = h;
            sh_hu[i] = A.hu[cc];
            sh_hv[i] = A.hv[cc];
            sh_b[i] = b;
            // sqrt(g d) from the step's memo when the depth has the same bits (a
            // pair (d, sqrt(g d)) either way, so a hit is the root's value; a miss
            // is written back by this CTA, which owns the cell). The f-wave's
            // RN(1 / d) is left to the VJP of an edge that takes the general path
            // (0 here) when the cell's momenta are +-0, since its edges may all be
            // at rest; a cell with momentum has general edges and gets it here.
            const double d = h - b;
            const bool wet = lt(P.drytol, d);
            double sq = 0.0;
            bool miss = wet;
            if (wet && A.memo) {
                const double2 m = A.memo[cc];
                if (dbits(m.x) == dbits(d)) {
                    sq = m.y;
                    miss = false;
                }
            }
            if (miss) {
                sq = sqrt(kG * d);
                if (A.memo) A.memo[cc] = make_double2(d, sq);
            }
            const bool still = ((dbits(sh_hu[i]) | dbits(sh_hv[i])) << 1) == 0;
            sh_rh[i] = (wet && (SOLVER != FWAVE || !still)) ? recip_rn(d).y : 0.0;
            sh_sq[i] = sq;
            const int dd = A.depth[cc];
            double m0, m1, m2;
            cell_mu(A, cc, A.ndv_tab[dd], m0, m1, m2);
            sh_mu[i] = m0;
            sh_mu[T + i] = m1;
            sh_mu[2 * T + i] = m2;
            for (int k = 0; k < 12; ++k) slot[k * T + i] = 0.0;
        }
        __syncthreads();

        const long long t0 = A.seg_ptr[seg], t1 = A.seg_ptr[seg + 1];
        for (long long t = t0 + tid; t < t1; t += blockDim.x) {
            const int4 tk = __ldg(&A.tasks[t]);
            const uint32_t meta = (uint32_t)tk.z;
            const bool bnd = (meta >> 14) & 1u;
            int L, R, iL, iR, pL;
            if (bnd || !odd) {
                L = tk.x; iL = meta & 3u; pL = (meta >> 4) & 31u;
                R = tk.y; iR = (meta >> 2) & 3u;
            } else {
                L = tk.y; iL = (meta >> 2) & 3u; pL = (meta >> 9) & 31u;
                R = tk.x; iR = meta & 3u;
            }
            if ((unsigned)L >= (unsigned)A.n_cells_total || (!bnd && (unsigned)R >= (unsigned)A.n_cells_total) ||
                iL > 2 || iR > 2 || pL > 16) {
                atomicOr(A.error, 1u);
                continue;
            }
            const double n1 = c_normal[pL][iL][0], n2 = c_normal[pL][iL][1];
            const int sl = L - c0, sr = R - c0;
            const bool lin = (unsigned)sl < (unsigned)cn;
            const bool rin = !bnd && (unsigned)sr < (unsigned)cn;
            State QL, QR;
            double dL, dR, sqL, sqR, yL, yR, mL[3], mR[3] = {0.0, 0.0, 0.0};
            int depL, depR = 0;
            if (lin) {
                QL = State{sh_h[sl], sh_hu[sl], sh_hv[sl], sh_b[sl]};
                dL = QL.h - QL.b;
                sqL = sh_sq[sl];
                yL = sh_rh[sl];
                mL[0] = sh_mu[sl]; mL[1] = sh_mu[T + sl]; mL[2] = sh_mu[2 * T + sl];
            } else {
                QL = State{A.h[L], A.hu[L], A.hv[L], A.b[L]};
                depth_terms(QL, P.drytol, dL, sqL, yL);
                const int dd = A.depth[L];
                cell_mu(A, L, A.ndv_tab[dd], mL[0], mL[1], mL[2]);
            }
            depL = A.depth[L];
            if (bnd) {
                if (P.bc == BC_SLIP) QR = boundary_ghost<BC_SLIP>(n1, n2, QL);
                else if (P.bc == BC_NOSLIP) QR = boundary_ghost<BC_NOSLIP>(n1, n2, QL);
                else QR = QL;
                dR = dL;
                sqR = sqL;
                yR = yL;
            } else {
                if (rin) {
                    QR = State{sh_h[sr], sh_hu[sr], sh_hv[sr], sh_b[sr]};
                    dR = QR.h - QR.b;
                    sqR = sh_sq[sr];
                    yR = sh_rh[sr];
                    mR[0] = sh_mu[sr]; mR[1] = sh_mu[T + sr]; mR[2] = sh_mu[2 * T + sr];
                } else {
                    QR = State{A.h[R], A.hu[R], A.hv[R], A.b[R]};
                    depth_terms(QR, P.drytol, dR, sqR, yR);
                    const int dd = A.depth[R];
                    cell_mu(A, R, A.ndv_tab[dd], mR[0], mR[1], mR[2]);
                }
                depR = A.depth[R];
            }
            // the edge's length in each cell: hypotenuse for local edge 2, else a leg
            const double lenL = A.len_tab[iL == 1 ? depL : depL + 1];
            const double gL[3] = {lenL * mL[0], lenL * mL[1], lenL * mL[2]};
            double gR[3] = {0.0, 0.0, 0.0};
            if (!bnd) {
                const double lenR = A.len_tab[iR == 1 ? depR : depR + 1];
                gR[0] = lenR * mR[0];
                gR[1] = lenR * mR[1];
                gR[2] = lenR * mR[2];
            }
            Grad4 oL{0.0, 0.0, 0.0, 0.0}, oR{0.0, 0.0, 0.0, 0.0};
            // The VJP is linear in the cotangents of the edge's updates: where they are
            // all zero (no gauge's cotangent has reached either cell yet) its outputs
            // are zeros, and the edge needs no evaluation.
            const long long gz = (dbits(gL[0]) | dbits(gL[1]) | dbits(gL[2]) | dbits(gR[0]) | dbits(gR[1]) |
                                  dbits(gR[2])) << 1;
            if (gz != 0)
                edge_vjp<SOLVER>(n1, n2, QL, QR, dL, dR, sqL, sqR, yL, yR, P.drytol, gL, gR, oL, oR,
                                 (int)((meta >> 15) & 3u));
            if (bnd) {  // the ghost's cotangent goes back to the cell
                if (P.bc == BC_SLIP) boundary_ghost_vjp<BC_SLIP>(n1, n2, oR, oL);
                else if (P.bc == BC_NOSLIP) boundary_ghost_vjp<BC_NOSLIP>(n1, n2, oR, oL);
                else boundary_ghost_vjp<BC_OUTFLOW>(n1, n2, oR, oL);
            }
            if (lin) {
                slot[(0 * 3 + iL) * T + sl] = oL.h;
                slot[(1 * 3 + iL) * T + sl] = oL.hu;
                slot[(2 * 3 + iL) * T + sl] = oL.hv;
                slot[(3 * 3 + iL) * T + sl] = oL.b;
            }
            if (rin) {
                slot[(0 * 3 + iR) * T + sr] = oR.h;
                slot[(1 * 3 + iR) * T + sr] = oR.hu;
                slot[(2 * 3 + iR) * T + sr] = oR.hv;
                slot[(3 * 3 + iR) * T + sr] = oR.b;
            }
        }
        __syncthreads();

        for (int i = tid; i < cn; i += blockDim.x) {
            const int cc = c0 + i;
            const uint8_t br = A.branch[cc];
            const double lh = A.lam_h[cc], lu = A.lam_hu[cc], lv = A.lam_hv[cc];
            double gh = 0.0, gu = 0.0, gv = 0.0, gb = 0.0;
            if (br & 2u) {  // drying clamp: h' = min(b, 0), p' = 0
                if (sh_b[i] < 0.0) gb += lh;
            } else if (br & 1u) {  // wetting fix: h~ = b + drytol, p~ = 0
                gb += lh;
            } else {
                gh = lh;
                gu = lu;
                gv = lv;
            }
#pragma unroll
            for (int k = 0; k < 3; ++k) {
                gh += slot[(0 * 3 + k) * T + i];
                gu += slot[(1 * 3 + k) * T + i];
                gv += slot[(2 * 3 + k) * T + i];
                gb += slot[(3 * 3 + k) * T + i];
            }
            A.out_h[cc] = gh;
            A.out_hu[cc] = gu;
            A.out_hv[cc] = gv;
            A.bbar[cc] += gb;
        }
        __syncthreads();
    }
}

}  // namespace swe
