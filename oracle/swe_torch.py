"""FP64 torch restatement of the SWE step for the reference gradient (test infrastructure only).

A vectorised, differentiable copy of the oracle's Jacobi-form step for the
f-wave solver (src/geoclaw/riemannsolvers.f:446-500 inside
c_bind_geoclaw_solver_dp, src/geoclaw/c_bind_riemannsolvers.f90:16-176; cell
update src/SWE/SWE_euler_timestep.f90:257-355) on the C-ABI mesh layout. Its
forward values equal the C oracle's bit for bit (tests check this); its
gradient through torch.autograd, with the dt sequence frozen and every branch
(wet/dry, wave-speed signs, min/max) differentiated on the side taken, is the
FP64 CPU reference for the GPU's hand-written discrete adjoint.

The f-wave solver, the augmented solver (riemann_aug_JCP with riemanntype,
src/geoclaw/riemannsolvers.f:2-258,507-618) and the four Lax-Friedrichs fluxes
(compute_lf_flux, src/SWE/SWE_euler_timestep.f90:359-446) are restated, with OUTFLOW, SLIP or
NOSLIP walls; wall reconstruction at wet/dry edges (the riemanntype branch) is
covered: its condition is evaluated like the solver does and its value changes
are differentiated.
"""
import math

import numpy as np
import torch

G = 9.80665


class _ExactSqrt(torch.autograd.Function):
    """Correctly rounded square root (numpy's IEEE sqrt): torch's vectorised CPU
    sqrt is not correctly rounded on every build, and the restatement has to
    match the oracle bit for bit."""

    @staticmethod
    def forward(ctx, x):
        y = torch.from_numpy(np.sqrt(x.detach().cpu().numpy())).to(x.device)
        ctx.save_for_backward(y)
        return y

    @staticmethod
    def backward(ctx, gy):
        (y,) = ctx.saved_tensors
        safe = torch.where(y > 0, y, torch.ones_like(y))
        return torch.where(y > 0, gy * 0.5 / safe, torch.zeros_like(gy))


def _sqrt(x):
    return _ExactSqrt.apply(x)


class BranchTape:
    """Records the outcome of every branch of the flux in evaluation order and
    replays it: with a replayed tape the step is the branch-frozen function
    whose derivative the adjoint computes, so finite differences of it do not
    straddle the kinks of min/max and sign switches."""

    def __init__(self):
        self.items = []
        self.pos = 0
        self.replay = False

    def start(self, replay):
        self.replay = replay
        self.pos = 0
        if not replay:
            self.items = []

    def cmp(self, value):
        if self.replay:
            v = self.items[self.pos]
            self.pos += 1
            return v
        self.items.append(value)
        return value


_NOTAPE = None


def _cmp(tape, value):
    return value if tape is None else tape.cmp(value)


def _where(c, a, b):
    return torch.where(c, a, b)


def _dmn(a, b):
    return torch.where(a < b, a, b)


def _dmx(a, b):
    return torch.where(a > b, a, b)


def _riemann_structure_hstar(hL, hR, uL, uR, drytol):
    """hm of riemanntype (src/geoclaw/riemannsolvers.f:507-618), values only (it
    decides the wall branch; no derivative flows through the condition)."""
    g = G
    hL, hR, uL, uR = (x.detach() for x in (hL, hR, uL, uR))
    h_min = _dmn(hR, hL)
    h_max = _dmx(hR, hL)
    delu = uR - uL
    safe = lambda x: torch.where(x > 0, x, torch.ones_like(x))
    F_min = delu + 2.0 * (_sqrt(g * h_min) - _sqrt(g * h_max))
    F_max = delu + (h_max - h_min) * _sqrt(((0.5 * g) * (h_max + h_min)) / safe(h_max * h_min))
    t = _dmx(torch.zeros_like(delu), -delu + 2.0 * (_sqrt(g * hL) + _sqrt(g * hR)))
    hm_rare = (1.0 / (16.0 * g)) * (t * t)
    h0 = h_max
    gL = _sqrt((0.5 * g) * (1.0 / safe(h0) + 1.0 / safe(hL)))
    gR = _sqrt((0.5 * g) * (1.0 / safe(h0) + 1.0 / safe(hR)))
    F0 = (delu + (h0 - hL) * gL) + (h0 - hR) * gR
    dfdh = ((gL - (g * (h0 - hL)) / ((4.0 * (h0 * h0)) * gL)) + gR) - (g * (h0 - hR)) / ((4.0 * (h0 * h0)) * gR)
    slope = (2.0 * _sqrt(h0)) * dfdh
    tt = _sqrt(h0) - F0 / torch.where(slope != 0, slope, torch.ones_like(slope))
    hm_shock = tt * tt
    h0 = h_min
    F0b = (delu + 2.0 * (_sqrt(g * h0) - _sqrt(g * h_max))) + (h0 - h_min) * _sqrt(
        (0.5 * g) * (1.0 / safe(h0) + 1.0 / safe(h_min)))
    den = h_max - h_min
    slope_b = (F_max - F0b) / torch.where(den != 0, den, torch.ones_like(den))
    hm_mix = h0 - F0b / torch.where(slope_b != 0, slope_b, torch.ones_like(slope_b))
    hm = torch.where(F_min > 0.0, hm_rare, torch.where(F_max <= 0.0, hm_shock, hm_mix))
    return torch.where(h_min <= drytol, torch.zeros_like(hm), hm)


def _fwave_core(v, tape):
    """riemann_fwave (src/geoclaw/riemannsolvers.f:446-500): speeds and f-waves
    from the wrapper's values v (a dict)."""
    g = G
    zero, one = v["zero"], v["one"]
    hL, hR, huL, huR, bL, bR = v["hL"], v["hR"], v["huL"], v["huR"], v["bL"], v["bR"]
    vL, vR, sE1, sE2, delphi = v["vL"], v["vR"], v["sE1"], v["sE2"], v["delphi"]
    delhu = huR - huL
    delb = bR - bL
    deldelphi = -(((g * 0.5) * (hR + hL)) * delb)
    dpd = delphi - deldelphi
    ds = sE2 - sE1
    ds = _where(ds != 0, ds, one)
    beta1 = (sE2 * delhu - dpd) / ds
    beta2 = (dpd - sE1 * delhu) / ds
    sw = [sE1, 0.5 * (sE1 + sE2), sE2]
    fw = [[beta1, zero, beta2], [beta1 * sE1, zero, beta2 * sE2], [beta1 * vL, None, beta2 * vR]]
    fw[2][1] = ((huR * vR - huL * vL) - fw[2][0]) - fw[2][2]
    return sw, fw


def _tmin(tape, a, b):  # dmn(a, b) = (a < b) ? a : b, the comparison on the tape
    return torch.where(_cmp(tape, a < b), a, b)


def _tmax(tape, a, b):  # dmx(a, b) = (a > b) ? a : b
    return torch.where(_cmp(tape, a > b), a, b)


def _riemann_structure(hL, hR, uL, uR, sqL, sqR, drytol, tape, one):
    """riemanntype (src/geoclaw/riemannsolvers.f:507-618) with one Newton step,
    differentiable: every branch is evaluated on safe operands where it is not
    taken and the taken one selected. sqL / sqR are sqrt(g h) of hL / hR.
    Returns (s1m, s2m)."""
    g = G
    lowR = _cmp(tape, hR < hL)    # h_min = dmn(hR, hL) is hR
    highR = _cmp(tape, hR > hL)   # h_max = dmx(hR, hL) is hR
    h_min, h_max = _where(lowR, hR, hL), _where(highR, hR, hL)
    sq_min, sq_max = _where(lowR, sqR, sqL), _where(highR, sqR, sqL)
    delu = uR - uL
    dry = _cmp(tape, h_min <= drytol)
    t_dry = ((uR + uL) - 2.0 * sqR) + 2.0 * sqL
    hmn, hmx = _where(dry, one, h_min), _where(dry, one, h_max)
    hLs, hRs = _where(dry, one, hL), _where(dry, one, hR)
    F_min = delu + 2.0 * (sq_min - sq_max)
    F_max = delu + (hmx - hmn) * _sqrt(((0.5 * g) * (hmx + hmn)) / (hmx * hmn))
    rare = _cmp(tape, F_min > 0.0)
    shock = _cmp(tape, F_max <= 0.0)
    # two rarefactions
    t = _tmax(tape, torch.zeros_like(delu), -delu + 2.0 * (sqL + sqR))
    hm_r = (1.0 / (16.0 * g)) * (t * t)
    sqm_r = _sqrt(g * hm_r)
    s1_r = (uL + 2.0 * sqL) - 3.0 * sqm_r
    s2_r = (uR - 2.0 * sqR) + 3.0 * sqm_r
    # two shocks: one Newton step on sqrt(h)
    h0 = hmx
    gL = _sqrt((0.5 * g) * (1.0 / h0 + 1.0 / hLs))
    gR = _sqrt((0.5 * g) * (1.0 / h0 + 1.0 / hRs))
    F0 = (delu + (h0 - hLs) * gL) + (h0 - hRs) * gR
    dfdh = ((gL - (g * (h0 - hLs)) / ((4.0 * (h0 * h0)) * gL)) + gR) - (g * (h0 - hRs)) / ((4.0 * (h0 * h0)) * gR)
    slope = (2.0 * _sqrt(h0)) * dfdh
    tt = _sqrt(h0) - F0 / _where(slope != 0, slope, one)
    hm_s = tt * tt
    hms = _where(hm_s > 0, hm_s, one)
    u1m = uL - (hm_s - hLs) * _sqrt((0.5 * g) * (1.0 / hms + 1.0 / hLs))
    u2m = uR + (hm_s - hRs) * _sqrt((0.5 * g) * (1.0 / hms + 1.0 / hRs))
    sqm_s = _sqrt(g * hm_s)
    s1_s, s2_s = u1m - sqm_s, u2m + sqm_s
    # one shock, one rarefaction
    h0 = hmn
    F0m = (delu + 2.0 * (sq_min - sq_max)) + (h0 - hmn) * _sqrt((0.5 * g) * (1.0 / h0 + 1.0 / hmn))
    den = hmx - hmn
    slope_m = (F_max - F0m) / _where(den != 0, den, one)
    hm_m = h0 - F0m / _where(slope_m != 0, slope_m, one)
    sqm_m = _sqrt(g * _where(hm_m >= 0, hm_m, one))
    lhigh = _cmp(tape, hL > hR)
    s1_m = _where(lhigh, (uL + 2.0 * sqL) - 3.0 * sqm_m, (uR - 2.0 * sqR) + sqm_m)
    s2_m = _where(lhigh, (uL + 2.0 * sqL) - sqm_m, (uR - 2.0 * sqR) + 3.0 * sqm_m)
    s1m = _where(dry, t_dry, _where(rare, s1_r, _where(shock, s1_s, s1_m)))
    s2m = _where(dry, t_dry, _where(rare, s2_r, _where(shock, s2_s, s2_m)))
    return s1m, s2m


def _det3(a00, a01, a02, a10, a11, a12, a20, a21, a22):
    d1 = a00 * (a11 * a22 - a12 * a21)
    d2 = a01 * (a10 * a22 - a12 * a20)
    d3 = a02 * (a10 * a21 - a11 * a20)
    return (d1 - d2) + d3


def _aug_core(v, tape):
    """riemann_aug_JCP (src/geoclaw/riemannsolvers.f:2-258) with maxiter = 1 and
    the entropy corrector off, the oracle's expressions."""
    g = G
    zero, one = v["zero"], v["one"]
    hL, hR, huL, huR, bL, bR = v["hL"], v["hR"], v["huL"], v["huR"], v["bL"], v["bR"]
    uL, uR, vL, vR, delphi, sqL, sqR = v["uL"], v["uR"], v["vL"], v["vR"], v["delphi"], v["sqL"], v["sqR"]
    delh, delhu, delb = hR - hL, huR - huL, bR - bL
    s1m, s2m = _riemann_structure(hL, hR, uL, uR, sqL, sqR, v["drytol"], tape, one)
    l0 = _tmin(tape, v["sE1"], s2m)
    l2 = _tmax(tape, v["sE2"], s1m)
    sE1, sE2 = l0, l2
    dsp = sE2 - sE1
    hstar = _tmax(tape, (((huL - huR) + sE2 * hR) - sE1 * hL) / _where(dsp != 0, dsp, one), zero)
    l1 = 0.5 * (l0 + l2)
    l1 = _where(_cmp(tape, torch.abs(l1) < 1e-20), zero, l1)
    r10, r12, r20, r22 = l0, l2, l0 * l0, l2 * l2
    ct = 1e-6
    hbar = _tmax(tape, 0.5 * (hL + hR), zero)
    su = uL + uR
    s1s2bar = 0.25 * (su * su) - g * hbar
    s1s2tilde = _tmax(tape, zero, uL * uR) - g * hbar
    sonic = ((torch.abs(s1s2bar) <= ct) | (s1s2bar * s1s2tilde <= ct) | ((s1s2bar * sE1) * sE2 <= ct) |
             (torch.minimum(torch.abs(sE1), torch.abs(sE2)) < ct) | ((sE1 < 0.0) & (s1m > 0.0)) |
             ((sE2 > 0.0) & (s2m < 0.0)) | ((uL + sqL) * (uR + sqR) < 0.0) | ((uL - sqL) * (uR - sqR) < 0.0))
    sonic = _cmp(tape, sonic)
    sbs = _where(sonic | (s1s2bar == 0), one, s1s2bar)
    deldelh = _where(sonic, -delb, ((delb * g) * hbar) / sbs)
    caseA = _cmp(tape, (sE1 < -ct) & (sE2 > ct))
    caseB = _cmp(tape, (~caseA) & (sE1 >= ct))
    caseC = _cmp(tape, (~caseA) & (~caseB) & (sE2 <= -ct))
    hsd = hstar * (sE2 - sE1)
    l0s, l2s = _where(l0 != 0, l0, one), _where(l2 != 0, l2, one)
    dA = _tmax(tape, _tmin(tape, deldelh, hsd / l2s), hsd / l0s)
    dB = _tmax(tape, _tmin(tape, deldelh, hsd / l0s), -hL)
    dC = _tmax(tape, _tmin(tape, deldelh, hR), hsd / l2s)
    deldelh = _where(caseA, dA, _where(caseB, dB, _where(caseC, dC, deldelh)))
    deldelphi = _where(sonic, -((g * hbar) * delb), -((((delb * g) * hbar) * s1s2tilde) / sbs))
    pl, pr = -(hL * delb), -(hR * delb)
    deldelphi = _tmin(tape, deldelphi, g * _tmax(tape, pl, pr))
    deldelphi = _tmax(tape, deldelphi, g * _tmin(tape, pl, pr))
    d0, d1, d2 = delh - deldelh, delhu, delphi - deldelphi
    r00, r01, r02, r11, r21 = one, zero, one, zero, one
    det = _det3(r00, r01, r02, r10, r11, r12, r20, r21, r22)
    dets = _where(det != 0, det, one)
    beta0 = _det3(d0, r01, r02, d1, r11, r12, d2, r21, r22) / dets
    beta1 = _det3(r00, d0, r02, r10, d1, r12, r20, d2, r22) / dets
    beta2 = _det3(r00, r01, d0, r10, r11, d1, r20, r21, d2) / dets
    fw = [[beta0 * r10, beta1 * r11, beta2 * r12], [beta0 * r20, beta1 * r21, beta2 * r22],
          [(beta0 * r10) * vL, None, (beta2 * r12) * vR]]
    fw[2][1] = ((((hR * uR) * vR) - ((hL * uL) * vL)) - fw[2][0]) - fw[2][2]
    return [l0, l1, l2], fw


def aug_flux(n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape=None):
    """compute_geoclaw_flux with the augmented solver, vectorised over edges."""
    return geoclaw_flux(_aug_core, n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape)


def fwave_flux(n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape=None):
    """compute_geoclaw_flux with the f-wave solver, vectorised over edges.
    Returns the left and right net updates (h, hu, hv) in world coordinates."""
    return geoclaw_flux(_fwave_core, n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape)


def geoclaw_flux(core, n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape=None):
    """compute_geoclaw_flux (src/SWE/SWE_euler_timestep.f90:449-481) around
    c_bind_geoclaw_solver_dp's wet/dry handling (c_bind_riemannsolvers.f90:16-176)
    with the solver `core`, vectorised over edges."""
    g = G
    zero = torch.zeros_like(hsL)
    one = torch.ones_like(hsL)
    pL1 = n1 * pxL + n2 * pyL
    pL2 = -n2 * pxL + n1 * pyL
    pR1 = n1 * pxR + n2 * pyR
    pR2 = -n2 * pxR + n1 * pyR
    hL = hsL - bL
    hR = hsR - bR
    active = _cmp(tape, ~((hL <= drytol) & (hR <= drytol)))
    wetR = _cmp(tape, hR > drytol)
    wetL = _cmp(tape, hL > drytol)
    hRs = _where(wetR, hR, one)
    hLs = _where(wetL, hL, one)
    uR = _where(wetR, pR1 / hRs, zero)
    vR = _where(wetR, pR2 / hRs, zero)
    huR = _where(wetR, pR1, zero)
    hvR = _where(wetR, pR2, zero)
    hR = _where(wetR, hR, zero)
    uL = _where(wetL, pL1 / hLs, zero)
    vL = _where(wetL, pL2 / hLs, zero)
    huL = _where(wetL, pL1, zero)
    hvL = _where(wetL, pL2, zero)
    hL = _where(wetL, hL, zero)
    # wet/dry walls (c_bind_riemannsolvers.f90:87-115)
    rdry = ~wetR
    ldry = (~rdry) & (~wetL)
    hst_r = _riemann_structure_hstar(hL, hL, uL, -uL, drytol)
    wall_r = _cmp(tape, rdry & (_dmx(hL.detach(), hst_r) + bL < bR))
    lower_r = _cmp(tape, rdry & (~wall_r) & (hL + bL < bR))
    hst_l = _riemann_structure_hstar(hR, hR, -uR, uR, drytol)
    wall_l = _cmp(tape, ldry & (_dmx(hR.detach(), hst_l) + bR < bL))
    lower_l = _cmp(tape, ldry & (~wall_l) & (hR + bR < bL))
    hR_, huR_, bR_, uR_, vR_ = (_where(wall_r, hL, hR), _where(wall_r, -huL, huR), _where(wall_r, bL, bR),
                                _where(wall_r, -uL, uR), _where(wall_r, vL, vR))
    bR_ = _where(lower_r, hL + bL, bR_)
    hL_, huL_, bL_, uL_, vL_ = (_where(wall_l, hR, hL), _where(wall_l, -huR, huL), _where(wall_l, bR, bL),
                                _where(wall_l, -uR, uL), _where(wall_l, vR, vL))
    bL_ = _where(lower_l, hR + bR, bL_)
    hR, huR, bR, uR, vR = hR_, huR_, bR_, uR_, vR_
    hL, huL, bL, uL, vL = hL_, huL_, bL_, uL_, vL_

    delphi = ((((huR - huL) * (uL + uR)) - ((uL * uR) * (hR - hL))) +
              (((0.5 * g) * (((bR + hR) - bL) - hL)) * (hR + hL))) - (((0.5 * g) * (hR + hL)) * (bR - bL))
    sq_in_L = g * hL
    sq_in_R = g * hR
    sqL = _sqrt(_where(sq_in_L > 0, sq_in_L, one)) * (sq_in_L > 0)
    sqR = _sqrt(_where(sq_in_R > 0, sq_in_R, one)) * (sq_in_R > 0)
    sL = uL - sqL
    sR = uR + sqR
    den = sqR + sqL
    uhat = (sqL * uL + sqR * uR) / _where(den > 0, den, one)
    ch_in = (g * 0.5) * (hR + hL)
    chat = _sqrt(_where(ch_in > 0, ch_in, one)) * (ch_in > 0)
    r1, r2 = uhat - chat, uhat + chat
    sE1 = _where(_cmp(tape, sL < r1), sL, r1)
    sE2 = _where(_cmp(tape, sR > r2), sR, r2)
    sw, fw = core(dict(zero=zero, one=one, hL=hL, hR=hR, huL=huL, huR=huR, bL=bL, bR=bR, uL=uL, uR=uR, vL=vL,
                       vR=vR, sE1=sE1, sE2=sE2, delphi=delphi, sqL=sqL, sqR=sqR, drytol=drytol), tape)
    walls = [wall_l, wall_l | wall_r, wall_r]
    for w in range(3):
        sw[w] = _where(walls[w], sw[w] * 0.0, sw[w])
        for e in range(3):
            fw[e][w] = _where(walls[w], fw[e][w] * 0.0, fw[e][w])
    netL = [zero, zero, zero]
    netR = [zero, zero, zero]
    signs = [(_cmp(tape, sw[w] < 0.0), _cmp(tape, sw[w] > 0.0)) for w in range(3)]
    for e in range(3):
        for w in range(3):
            neg, pos = signs[w]
            f = fw[e][w]
            netL[e] = _where(neg, netL[e] + f, _where(pos, netL[e], netL[e] + 0.5 * f))
            netR[e] = _where(pos, netR[e] + f, _where(neg, netR[e], netR[e] + 0.5 * f))
    netL = [_where(active, x, zero) for x in netL]
    netR = [_where(active, x, zero) for x in netR]
    fL = (netL[0], netL[1] * n1 + netL[2] * -n2, netL[1] * n2 + netL[2] * n1)
    fR = (netR[0], netR[1] * n1 + netR[2] * -n2, netR[1] * n2 + netR[2] * n1)
    return fL, fR


FWAVE, AUG_RIEMANN, LF, LF_BATH, LLF, LLF_BATH = 1, 3, 10, 11, 12, 13
SOLVERS = {"fwave": FWAVE, "hlle": FWAVE, "aug_riemann": AUG_RIEMANN, "lf": LF, "lfbath": LF_BATH, "llf": LLF,
           "llfbath": LLF_BATH}


def lf_flux(solver, n1, n2, hsL, pxL, pyL, bL, hsR, pxR, pyR, bR, drytol, tape=None):
    """compute_lf_flux (src/SWE/SWE_euler_timestep.f90:359-446), vectorised over
    edges, the same expressions as the oracle's: LF / LLF with or without the
    well-balanced bathymetry terms, the dry-side fluxes of the bathymetry
    variants. Returns the left and right fluxes (h, hu, hv)."""
    g = G
    zero = torch.zeros_like(hsL)
    one = torch.ones_like(hsL)

    def nv(px, py, d):  # z0(n1 * (p1 / d)) + n2 * (p2 / d): the +0 start changes no value
        return n1 * (px / d) + n2 * (py / d)

    local = solver in (LLF, LLF_BATH)
    if solver in (LF_BATH, LLF_BATH):
        dL, dR = hsL - bL, hsR - bR
        dryL = _cmp(tape, dL < drytol)
        dryR = _cmp(tape, dR < drytol)
        dLs, dRs = _where(dryL, one, dL), _where(dryR, one, dR)  # a dry side's values are not used
        hL, hR = _dmx(dL, zero), _dmx(dR, zero)
        vL, vR = nv(pxL, pyL, dLs), nv(pxR, pyR, dRs)
        sL = _sqrt(g * hL) + torch.abs(vL)
        sR = _sqrt(g * hR) + torch.abs(vR)
        alpha = _where(_cmp(tape, sL > sR), sL, sR) if local else 100.0 * one
        Fh = 0.5 * ((hL * vL + hR * vR) + alpha * (hsL - hsR))
        pr = (0.5 * g) * (hL * hL + hR * hR)
        Fp1 = 0.5 * (((pxL * vL + pxR * vR) + pr * n1) + alpha * (pxL - pxR))
        Fp2 = 0.5 * (((pyL * vL + pyR * vR) + pr * n2) + alpha * (pyL - pyR))
        src = ((0.25 * g) * (hL + hR)) * (bR - bL)
        wetL = (Fh, Fp1 + src * n1, Fp2 + src * n2)
        wetR = (-Fh, -Fp1 + src * n1, -Fp2 + src * n2)
        prR, prL = ((0.5 * g) * hR) * hR, ((0.5 * g) * hL) * hL
        onlyR = (zero, (-((0.5 * vR) * pxR) - prR * n1) + (0.5 * sR) * pxR,
                 (-((0.5 * vR) * pyR) - prR * n2) + (0.5 * sR) * pyR)
        onlyL = (zero, ((0.5 * vL) * pxL + prL * n1) + (0.5 * sL) * pxL,
                 ((0.5 * vL) * pyL + prL * n2) + (0.5 * sL) * pyL)
        both = dryL & dryR
        fL = tuple(_where(dryL | dryR, _where(dryL, zero, a), w) for a, w in zip(onlyL, wetL))
        fR = tuple(_where(dryL | dryR, _where(both | dryR, zero, a), w) for a, w in zip(onlyR, wetR))
        return fL, fR
    dL, dR = hsL - 0.0, hsR - 0.0
    hL, hR = _dmx(dL, zero), _dmx(dR, zero)
    vL, vR = nv(pxL, pyL, dL), nv(pxR, pyR, dR)
    sL = _sqrt(g * dL) + torch.abs(vL)
    sR = _sqrt(g * dR) + torch.abs(vR)
    alpha = _where(_cmp(tape, sL > sR), sL, sR) if local else 100.0 * one
    Fh = 0.5 * ((vL * hL + vR * hR) + alpha * (hsL - hsR))
    sc = (vL * vL) * hL + (vR * vR) * hR
    pr = (0.5 * g) * (hL * hL + hR * hR)
    Fp1 = 0.5 * ((sc + pr * n1) + alpha * (pxL - pxR))
    Fp2 = 0.5 * ((sc + pr * n2) + alpha * (pyL - pyR))
    return (Fh, Fp1, Fp2), (-Fh, -Fp1, -Fp2)


class TorchStep:
    """The step on a fixed mesh (C-ABI layout), f-wave or a Lax-Friedrichs flux, differentiable.

    Edges are oriented by the step parity exactly like the GPU kernel; ``step``
    applies one Euler step with a given dt to (h, hu, hv) for bathymetry b.
    """

    def __init__(self, mesh, scaling=1.0, drytol=0.01, bc="outflow", solver="fwave"):
        from oracle import oracle as O
        sid = SOLVERS[solver] if isinstance(solver, str) else int(solver)
        if sid == FWAVE:
            self.flux = fwave_flux
        elif sid == AUG_RIEMANN:
            self.flux = aug_flux
        elif sid in (LF, LF_BATH, LLF, LLF_BATH):
            self.flux = lambda *a, **k: lf_flux(sid, *a, **k)
        else:
            raise ValueError("solver %r is not restated here" % (solver,))
        self.n = mesh.n_cells
        self.drytol = drytol
        self.bc = bc
        ec = torch.as_tensor(np.asarray(mesh.edge_cells, np.int64))
        el = torch.as_tensor(np.asarray(mesh.edge_local, np.int64)) - 1
        self.ea, self.eb = ec[:, 0], ec[:, 1]
        self.la, self.lb = el[:, 0], el[:, 1]
        self.bcell = torch.as_tensor(np.asarray(mesh.bnd_cell, np.int64))
        self.bloc = torch.as_tensor(np.asarray(mesh.bnd_local, np.int64)) - 1
        table = np.zeros((17, 3, 2))
        for p in range(-8, 9):
            if p:
                for e in range(3):
                    table[p + 8, e] = O.normal(p, e + 1)
        table = torch.as_tensor(table)
        pl = torch.as_tensor(np.asarray(mesh.plotter, np.int64)) + 8
        self.nA = table[pl[self.ea], self.la]
        self.nB = table[pl[self.eb], self.lb]
        self.nBnd = table[pl[self.bcell], self.bloc]
        d = torch.as_tensor(np.asarray(mesh.depth, np.int64))
        leg = torch.as_tensor([O.leg_size(i) for i in range(-1, 61)], dtype=torch.float64)
        vol = torch.as_tensor([O.cell_volume(i) for i in range(0, 61)], dtype=torch.float64)
        self.leg = scaling * leg[d + 1]
        self.hyp = scaling * leg[d]
        self.vol = (scaling * scaling) * vol[d]

    def step(self, h, hu, hv, b, dt, parity, tape=None):
        n = self.n
        odd = parity & 1
        if odd:
            L, R, iL, iR, nn = self.eb, self.ea, self.lb, self.la, self.nB
        else:
            L, R, iL, iR, nn = self.ea, self.eb, self.la, self.lb, self.nA
        fL, fR = self.flux(nn[:, 0], nn[:, 1], h[L], hu[L], hv[L], b[L], h[R], hu[R], hv[R], b[R], self.drytol,
                           tape)
        c = self.bcell
        n1, n2 = self.nBnd[:, 0], self.nBnd[:, 1]
        gp1, gp2 = hu[c], hv[c]
        if self.bc == "slip":
            dd = hu[c] * n1 + hv[c] * n2
            gp1, gp2 = hu[c] - dd * n1, hv[c] - dd * n2
        elif self.bc == "noslip":
            gp1, gp2 = -hu[c], -hv[c]
        fB, _ = self.flux(n1, n2, h[c], hu[c], hv[c], b[c], h[c], gp1, gp2, b[c], self.drytol, tape)
        # slot values [cell, local edge]
        slots = []
        for q in range(3):
            s = torch.zeros(n, 3, dtype=h.dtype)
            s = s.index_put((L, iL), fL[q], accumulate=True)
            s = s.index_put((R, iR), fR[q], accumulate=True)
            s = s.index_put((c, self.bloc), fB[q], accumulate=True)
            slots.append(s)
        k0, k2 = (2, 0) if odd else (0, 2)
        sc = -dt / self.vol
        d = []
        for q in range(3):
            s = slots[q]
            d.append((self.leg * s[:, k0] + self.hyp * s[:, 1]) + self.leg * s[:, k2])
        dh, dp1, dp2 = (sc * x for x in d)
        wet_fix = _cmp(tape, (h < b + self.drytol) & (dh > 0.0))
        h1 = _where(wet_fix, b + self.drytol, h)
        p1 = _where(wet_fix, torch.zeros_like(hu), hu)
        p2 = _where(wet_fix, torch.zeros_like(hv), hv)
        h1 = h1 + dh
        p1 = p1 + dp1
        p2 = p2 + dp2
        dry = _cmp(tape, h1 < b + self.drytol)
        h1 = _where(dry, _dmn(b, torch.zeros_like(b)), h1)
        p1 = _where(dry, torch.zeros_like(p1), p1)
        p2 = _where(dry, torch.zeros_like(p2), p2)
        return h1, p1, p2


def gauge_objective_frozen(tstep, h0, hu0, hv0, b, dts, gauges, obs, tapes, replay):
    """J with every step's branches recorded into (replay=False) or replayed
    from (replay=True) the per-step tapes."""
    x = (h0, hu0, hv0)
    J = 0.0
    with torch.no_grad():
        for t, dt in enumerate(dts):
            tapes[t].start(replay)
            x = tstep.step(*x, b, float(dt), t, tapes[t])
            J += float(((x[0][gauges] - obs[t]) ** 2).sum())
    return J


def gauge_objective_and_grad(tstep, h0, hu0, hv0, b, dts, gauges, obs, parity0=0, need_grad=True):
    """J = sum_t sum_g (h_t[gauge] - obs[t, g])^2 over len(dts) steps and its
    gradient with respect to h0 and b, by reverse accumulation one step at a
    time (states kept on the host; each step re-run under autograd)."""
    states = [(h0, hu0, hv0)]
    J = 0.0
    with torch.no_grad():
        for t, dt in enumerate(dts):
            h, hu, hv = tstep.step(*states[-1], b, float(dt), parity0 + t)
            states.append((h, hu, hv))
            J += float(((h[gauges] - obs[t]) ** 2).sum())
    if not need_grad:
        return J, None, None
    lam = [torch.zeros_like(h0), torch.zeros_like(h0), torch.zeros_like(h0)]
    gb = torch.zeros_like(b)
    for t in range(len(dts) - 1, -1, -1):
        hT = states[t + 1][0]
        lam[0] = lam[0].index_add(0, gauges, 2.0 * (hT[gauges] - obs[t]))
        x = [s.clone().requires_grad_(True) for s in states[t]]
        bb = b.clone().requires_grad_(True)
        out = tstep.step(*x, bb, float(dts[t]), parity0 + t)
        grads = torch.autograd.grad(out, x + [bb], grad_outputs=lam, allow_unused=True)
        lam = [g if g is not None else torch.zeros_like(h0) for g in grads[:3]]
        gb = gb + (grads[3] if grads[3] is not None else 0.0)
    return J, lam[0], gb
