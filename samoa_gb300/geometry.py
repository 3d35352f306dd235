"""Geometry tables of Sierpinski cells (src/SFC_data_types.f90:509-587), host side.

``leg_sizes()[i + 1] = sqrt(0.5)**i`` for i = -1..60, folded the way a Fortran
compiler folds the PARAMETER arrays: the double fl(sqrt(0.5)) raised to the
integer power exactly, then rounded once. ``volumes()[i] = 0.5**(i + 1)``.
"""
import functools
import math
from fractions import Fraction

import numpy as np

MAX_DEPTH = 60


@functools.lru_cache(maxsize=None)
def leg_sizes():
    x = Fraction(math.sqrt(0.5))
    out = [float(1 / x)] + [float(x ** i) for i in range(0, MAX_DEPTH + 1)]
    return np.array(out, np.float64)


@functools.lru_cache(maxsize=None)
def volumes():
    return np.array([math.ldexp(1.0, -(i + 1)) for i in range(MAX_DEPTH + 1)], np.float64)
