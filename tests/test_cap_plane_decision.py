"""The cap plane's FP32 decision against the reference's FP64 rounding (CPU).

The plane of bin (fdx, fdy) of an angle with specular offset (fxm0, fym0) is
round(sqrt(r^2 - fd^2) - fzm0), fzm0 = sqrt(r^2 - fxm0^2 - fym0^2)
(Reconstruction/src/fonctions.cpp:893-921, FP64).  k_cap_cols computes it in
FP32, using the correctly rounded float sqrt of the exact integer r^2 - fd^2,
fzm0 rounded to float, one subtraction, + 0.5 and floor.  Within 1e-3 of a
rounding boundary it falls back to FP64.  numpy's float32 arithmetic rounds
as the kernel's does, so this restatement is exact.  For every bin of every
angle the FP32 decision outside the guard must equal the FP64 rounding, so
the cap indices are bit-exact.
"""
from __future__ import annotations

import math

import numpy as np
import pytest

from mtd_transmission_gb300 import Geometry, api
from tests import simul


def _round_away(x):
    return np.sign(x) * np.floor(np.abs(x) + 0.5)


def _check(acq, offsets):
    rayon = api.derive(Geometry.from_acquisition(acq))["rayon"]
    N = acq.nxmax
    r2 = rayon * rayon
    assert r2 == int(r2) and r2 < 2 ** 24  # the kernels' exact-integer float path
    coef = float(np.float32(acq.coef_na_obj_limit))
    disc_thr = int(min(math.ceil(coef * N * N), 2 * N * N + 1))
    fd = np.arange(-N, N)
    fdx, fdy = np.meshgrid(fd, fd)
    fd2 = (fdx * fdx + fdy * fdy)[fdx * fdx + fdy * fdy < disc_thr]
    sf = np.sqrt((int(r2) - fd2).astype(np.float32))          # __fsqrt_rn((float)(r2i - fd^2))
    s64 = np.sqrt(r2 - fd2.astype(np.float64))                 # the reference's sqrt in double
    guarded = total = 0
    for tx, ty in offsets:
        c = r2 - float(tx) * tx - float(ty) * ty
        if _round_away(c) < 0:
            continue                                           # skipped angle (fzm0 < 0)
        fz = math.sqrt(c)
        fzf = np.float32(fz)
        d = sf - fzf
        fr = d - np.floor(d)
        take = np.abs(fr - np.float32(0.5)) > np.float32(1e-3)
        assert d.dtype == np.float32 and fr.dtype == np.float32
        k32 = np.floor(d + np.float32(0.5))
        ref = _round_away(s64 - fz)
        bad = np.flatnonzero(take & (k32 != ref))
        assert bad.size == 0, (tx, ty, fd2[bad[:3]], d[bad[:3]], (s64 - fz)[bad[:3]])
        guarded += int((~take).sum())
        total += take.size
    return guarded, total


@pytest.mark.parametrize("name", ["plain_512_born", "rytov_1024", "large_2048"])
def test_fp32_plane_decision_on_workload_tilts(name):
    acq, _, _ = simul.workload(name)
    guarded, total = _check(acq, simul.spiral_tilts(acq.nb_holo, acq.nxmax))
    assert guarded < 0.005 * total  # the FP64 fallback is rare


def test_fp32_plane_decision_on_random_offsets():
    """Integer specular offsets anywhere in the NA disc, not only the spiral's."""
    acq, _, _ = simul.workload("rytov_1024")
    rng = np.random.default_rng(7)
    N = acq.nxmax
    off = rng.integers(-N, N, size=(2000, 2))
    off = off[(off ** 2).sum(1) < N * N]
    guarded, total = _check(acq, off)
    assert guarded < 0.005 * total
