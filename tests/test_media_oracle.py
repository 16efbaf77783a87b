"""CPU checks of the medium restatement against analytic transmittance."""
import ctypes as C
import math

import numpy as np
import pytest

from kiraray_gb300 import scenes
from oracle import pyoracle as O


def _pt_with_medium(medium):
    sc = scenes.cornell_box(8, 8)
    sc.media = [medium]
    return O.PathTracer(sc)


def _transmittance(pt, o, d, tmax, n=20000, seed=7):
    lib = O.load()
    lib.oracle_medium_transmittance.restype = C.c_double
    lib.oracle_medium_transmittance.argtypes = [C.c_void_p, C.c_void_p, C.c_void_p, C.c_float,
                                                C.c_int, C.c_uint32]
    o = np.asarray(o, np.float32)
    d = np.asarray(d, np.float32)
    return lib.oracle_medium_transmittance(pt._h, o.ctypes.data, d.ctypes.data, tmax, n, seed)


@pytest.mark.parametrize("sigma,length", [(0.5, 1.0), (2.0, 1.0), (1.0, 3.0)])
def test_homogeneous_transmittance_is_exponential(oracle_lib, sigma, length):
    med = scenes.Medium(None, (0, 0, 0), (1, 1, 1), sigma_t=(sigma,) * 3, albedo=(0.5,) * 3)
    pt = _pt_with_medium(med)
    n = 40000
    t = _transmittance(pt, [0, 0, 0], [1, 0, 0], length, n)
    want = math.exp(-sigma * length)
    sd = math.sqrt(want * (1 - want) / n)
    assert abs(t - want) < 5 * sd + 1e-4, (t, want)


def _optical_depth(med, o, d, tmax, steps=20000):
    """Numerical optical depth of the trilinear density along o + t d."""
    dens = med.density.astype(np.float64)
    nz, ny, nx = dens.shape
    lo, hi = np.array(med.bounds_min), np.array(med.bounds_max)
    t = (np.arange(steps) + 0.5) / steps * tmax
    p = np.asarray(o)[None] + t[:, None] * np.asarray(d)[None]
    f = (p - lo) / (hi - lo) * np.array([nx, ny, nz]) - 0.5
    i0 = np.floor(f).astype(int)
    w = f - i0
    val = np.zeros(steps)
    for a in (0, 1):
        for b in (0, 1):
            for c in (0, 1):
                x, y, z = i0[:, 0] + a, i0[:, 1] + b, i0[:, 2] + c
                ok = (x >= 0) & (y >= 0) & (z >= 0) & (x < nx) & (y < ny) & (z < nz)
                v = np.where(ok, dens[np.clip(z, 0, nz - 1), np.clip(y, 0, ny - 1), np.clip(x, 0, nx - 1)], 0)
                wt = (w[:, 0] if a else 1 - w[:, 0]) * (w[:, 1] if b else 1 - w[:, 1]) * \
                     (w[:, 2] if c else 1 - w[:, 2])
                val += wt * v
    inside = np.all((p >= lo) & (p <= hi), axis=1)
    return med.scale * med.sigma_t[1] * (val * inside).sum() * tmax * np.linalg.norm(d) / steps


@pytest.mark.parametrize("case", ["constant", "layered"])
def test_grid_medium_transmittance(oracle_lib, case):
    if case == "constant":
        dens = np.ones((8, 8, 8), np.float16)
        med = scenes.Medium(dens, (0, 0, 0), (2, 2, 2), sigma_t=(1, 1, 1), albedo=(0.9,) * 3,
                            scale=1.5, majorant_res=(4, 4, 4))
        o, d, tmax = [-1.0, 1.0, 1.0], [1, 0, 0], 5.0
    else:
        dens = np.full((16, 16, 16), 0.5, np.float16)
        dens[:2] = 1.0   # raises the majorant of the first cells along z
        med = scenes.Medium(dens, (0, 0, 0), (1, 1, 1), sigma_t=(2, 2, 2), albedo=(0.9,) * 3,
                            scale=1.0, majorant_res=(2, 2, 2))
        o, d, tmax = [0.5, 0.5, -0.5], [0, 0, 1], 2.0
    pt = _pt_with_medium(med)
    n = 100000
    t = _transmittance(pt, o, d, tmax, n)
    want = math.exp(-_optical_depth(med, o, d, tmax))
    assert abs(t - want) < 5 * math.sqrt(want * (1 - want) / n) + 2e-4, (t, want)
