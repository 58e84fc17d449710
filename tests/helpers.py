"""Shared helpers: workloads, oracle configuration, error metrics."""
from __future__ import annotations

from dataclasses import replace

import numpy as np

import oracle
from tests import simul

ORACLE_KEYS = ("ccd_roix", "nxmax", "circle_cx", "circle_cy", "dim_final", "na", "n0", "lambda0", "f_tube", "f_obj",
               "tpcam", "rf", "born", "c_aber", "deroul", "volkov", "coef_na_obj_limit")


def oracle_cfg(acq) -> oracle.Config:
    return oracle.Config(**{k: getattr(acq, k) for k in ORACLE_KEYS})


def rel_l2(a, b) -> float:
    a = np.asarray(a, np.complex128 if np.iscomplexobj(a) or np.iscomplexobj(b) else np.float64)
    b = np.asarray(b, a.dtype)
    den = np.linalg.norm(b.ravel())
    return float(np.linalg.norm((a - b).ravel()) / (den if den > 0 else 1.0))


def small_case(name="plain_512_born", M=8, seed=None, **over):
    """A small stack of a named workload; returns (acq, phantom, data dict)."""
    acq, ph, s = simul.workload(name)
    acq = replace(acq, nb_holo=M, **over)
    d = simul.holograms(acq, ph, M=M, seed=s if seed is None else seed)
    return acq, ph, {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in d.items()}


def c64(a: np.ndarray) -> np.ndarray:
    return np.ascontiguousarray(a, np.complex64)


def planted_ties(F: int, M: int, rng) -> np.ndarray:
    """Random complex64 spectra with near ties planted at the top: FP32
    magnitudes tie or round across where the reference's FP64 ones do not
    (five kinds, cycled over the M spectra)."""
    s = (rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))).astype(np.complex64)
    s *= np.float32(0.25)
    out = []
    for a in range(M):
        sp = s[a].ravel().copy()
        m = np.float32(4.0)  # above every random magnitude; m^2 exact
        p = int(rng.integers(1, F * F - 8))
        kind = a % 5
        if kind == 0:    # FP32 tie, FP64 larger at the later bin
            sp[p] = m
            sp[p + 3] = np.complex64(m + 1j * m * np.float32(2.0 ** -15))
        elif kind == 1:  # exact tie: the first bin wins
            sp[p] = m
            sp[p + 5] = m
        elif kind == 2:  # index 0 compared by |z|^2: (2, 0) ties with |z| = 4
            sp[0] = np.float32(2.0)
            sp[p] = m
        elif kind == 3:  # index 0 larger in FP64 only: |z0|^2 = 4 (1 + 2^-30) against 4
            sp[0] = np.complex64(2.0 + 1j * 2.0 * np.float32(2.0 ** -15))
            sp[p] = m
        else:            # the same at a value that is not a power of two: FP32 ties, FP64 larger later
            sp[p] = np.complex64(m * np.float32(1.0 + 2.0 ** -23))
            sp[p + 2] = np.complex64(m * np.float32(1.0 + 2.0 ** -23) + 1j * m * np.float32(2.0 ** -16))
        out.append(sp.reshape(F, F))
    return np.stack(out)
