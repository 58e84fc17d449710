"""Shared helpers: workloads, oracle configuration, error metrics."""
from __future__ import annotations

from dataclasses import replace

import numpy as np

import oracle
from mtd_transmission_gb300 import simul

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
