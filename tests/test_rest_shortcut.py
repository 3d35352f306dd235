"""The f-wave step's exact lake-at-rest path (geoclaw_flux in
samoa_gb300/csrc/swe_riemann.cuh) against the oracle's full evaluation, on the
CPU: wherever both sides are wet, every momentum is +-0 and the c-binding
surface difference ((bR + hR) - bL) - hL rounds to a zero, the full f-wave
solver (src/geoclaw/riemannsolvers.f:446-500 with
src/geoclaw/c_bind_riemannsolvers.f90:50-176, as the oracle restates them)
returns +0 net updates on both sides and the maximum wave speed
max(sqrt(g hL), sqrt(g hR)), which is what the kernel's shortcut returns
without the solver's arithmetic. The proof's key step, that
chat = sqrt(RN(g/2 RN(hL + hR))) never exceeds the larger side's
sqrt(RN(g h)), is checked on its own over random and adversarial depth pairs.
"""
import math
import struct

import numpy as np

from oracle import oracle as O

G = 9.80665


def _bits(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def test_roe_speed_never_exceeds_the_larger_side():
    rng = np.random.default_rng(11)
    pairs = [(float(2.0 ** rng.uniform(-20, 40)), float(2.0 ** rng.uniform(-20, 40))) for _ in range(50000)]
    for _ in range(20000):  # neighbours one or a few ulps apart
        h = float(2.0 ** rng.uniform(-20, 40))
        k = int(rng.integers(0, 4))
        h2 = h
        for _ in range(k):
            h2 = float(np.nextafter(h2, np.inf))
        pairs.append((h, h2))
    for hL, hR in pairs:
        chat = math.sqrt((0.5 * G) * (hR + hL))
        m = max(math.sqrt(G * hL), math.sqrt(G * hR))
        assert chat <= m, (hL, hR, chat, m)


def test_full_fwave_evaluation_on_rest_edges_is_the_shortcut():
    rng = np.random.default_rng(12)
    drytol = 1e-3
    normals = [O.normal(p, e) for p in range(1, 17) for e in range(3)]
    checked = 0
    for _ in range(4000):
        bL = -float(rng.uniform(0.01, 5000.0))
        bR = -float(rng.uniform(0.01, 5000.0)) if rng.random() < 0.8 else bL
        s = float(rng.choice([0.0, rng.uniform(-1e-3, 1e-3), rng.uniform(-1.0, 1.0)]))
        hL, hR = s, s
        dL, dR = hL - bL, hR - bR
        if not (dL > drytol and dR > drytol):
            continue
        surf = ((bR + dR) - bL) - dL
        if surf != 0.0:
            continue  # not on the exact path: the full solver runs there
        pu = [(-0.0 if rng.random() < 0.5 else 0.0) for _ in range(4)]
        n = normals[int(rng.integers(0, len(normals)))]
        ul, ur = O.edge_flux(O.FWAVE, n, [hL, pu[0], pu[1], bL], [hR, pu[2], pu[3], bR], drytol)
        ms = max(math.sqrt(G * dL), math.sqrt(G * dR))
        for side in (ul, ur):
            assert all(_bits(float(v)) == 0 for v in side[:3]), (side, dL, dR)  # +0, not -0
            assert _bits(float(side[3])) == _bits(ms), (side[3], ms)
        checked += 1
    assert checked > 1000
