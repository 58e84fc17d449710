"""ctypes wrapper of the reference's own functions, built from its sources
by oracle/ref/build_ref.py into oracle/_ref/ (test infrastructure only).

Used by the CPU tests to pin the oracle's restatement on the reference's
code: extraction, specular search, field recentring, Volkov unwrapping, the
reconstruction's parameters (its manip class) and the whole volume stage
(per-field spectra, retroPropag_Born, normalisation, shifts, 3D inverse
FFT, index conversion).  Available only where the reference's sources were
present at build time.
"""
from __future__ import annotations

import ctypes
import os
import struct
import tempfile

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_DIR = os.path.join(_HERE, "_ref")
_pre = _rec = None


def build() -> list[str]:
    import importlib.util
    spec = importlib.util.spec_from_file_location("build_ref", os.path.join(_HERE, "ref", "build_ref.py"))
    m = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(m)
    return m.build()


def available() -> bool:
    return all(os.path.exists(os.path.join(_DIR, n)) for n in ("libref_pretraitement.so", "libref_reconstruction.so"))


def _libs():
    global _pre, _rec
    if _pre is None:
        P, I, Dd = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
        _pre = ctypes.CDLL(os.path.join(_DIR, "libref_pretraitement.so"))
        _pre.ref_pre_tukey2d.argtypes = [I, ctypes.c_float, P]
        _pre.ref_pre_extract.argtypes = [P, I, I, I, I, P]
        _pre.ref_pre_coord_spec.argtypes = [P, I]
        _pre.ref_pre_field.argtypes = [P, I, I, I, P, P]
        _pre.ref_pre_volkov.argtypes = [P, I, P]
        _pre.ref_pre_herraez.argtypes = [P, I, I, P]
        _rec = ctypes.CDLL(os.path.join(_DIR, "libref_reconstruction.so"))
        _rec.ref_rec_manip.argtypes = [ctypes.c_char_p, P]
        _rec.ref_rec_volume.argtypes = [ctypes.c_char_p, P, P, I, P, P, P]
        del Dd
    return _pre, _rec


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def tukey2d(n: int, alpha: float) -> np.ndarray:
    out = np.empty((n, n), np.float64)
    _libs()[0].ref_pre_tukey2d(n, alpha, _p(out))
    return out


def extract(holo: np.ndarray, nxmax: int, cx: int, cy: int) -> np.ndarray:
    h = np.ascontiguousarray(holo, np.float64)
    out = np.empty((2 * nxmax, 2 * nxmax), np.complex128)
    _libs()[0].ref_pre_extract(_p(h), h.shape[0], nxmax, cx, cy, _p(out))
    return out


def coord_spec(spec: np.ndarray) -> int:
    s = np.ascontiguousarray(spec, np.complex128)
    return int(_libs()[0].ref_pre_coord_spec(_p(s), s.shape[0]))


def field(spec: np.ndarray, px: int, py: int):
    """calc_Uborn2 and calcPhase_mpi_pi_atan2: (field, wrapped phase)."""
    s = np.ascontiguousarray(spec, np.complex128)
    f = np.empty_like(s)
    ph = np.empty(s.shape, np.float64)
    _libs()[0].ref_pre_field(_p(s), s.shape[0], px, py, _p(f), _p(ph))
    return f, ph


def volkov(phase: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(phase, np.float64)
    out = np.empty_like(p)
    _libs()[0].ref_pre_volkov(_p(p), p.shape[0], _p(out))
    return out


def herraez(phase: np.ndarray, angle: int = 0) -> np.ndarray:
    p = np.ascontiguousarray(phase, np.float64)
    out = np.empty_like(p)
    _libs()[0].ref_pre_herraez(_p(p), p.shape[0], angle, _p(out))
    return out


def config_tree(cfg, n_angles: int, root: str) -> str:
    """A configuration tree the reference's manip class reads: $HOME/.config/
    gui_tomo.conf naming the config and result folders, recon.txt,
    config_manip.txt and the preprocessing's parametres.raw (NXMAX, angles,
    rayon, CCD_ROIX, tailleTheoPixelHolo).  Returns the HOME to use."""
    from oracle import derive
    home = os.path.join(root, "home")
    conf, res = os.path.join(root, "config"), os.path.join(root, "result")
    for d in (os.path.join(home, ".config"), conf, res):
        os.makedirs(d, exist_ok=True)
    with open(os.path.join(home, ".config", "gui_tomo.conf"), "w") as f:
        f.write(f"CHEMIN_CONFIG {conf}\nCHEMIN_RESULT {res}\nCHEMIN_ACQUIS {root}\nCHEMIN_CONFIG_PC_ACQUIS {conf}\n")
    with open(os.path.join(conf, "config_manip.txt"), "w") as f:
        f.write(f"NA {cfg.na}\nN0 {cfg.n0}\nLAMBDA {cfg.lambda0:.12g}\nF_TUBE {cfg.f_tube}\nF_OBJ {cfg.f_obj}\n"
                f"TPCAM {cfg.tpcam:.12g}\nRF {cfg.rf}\nNXMAX {cfg.nxmax}\nCIRCLE_CX {cfg.circle_cx}\n"
                f"CIRCLE_CY {cfg.circle_cy}\nDIM_ROI {cfg.ccd_roix}\nNB_HOLO {n_angles}\n")
    with open(os.path.join(conf, "recon.txt"), "w") as f:
        f.write(f"CCD_ROIX {cfg.ccd_roix}\nDEROUL {cfg.deroul}\nVOLKOV {cfg.volkov}\nC_ABER {cfg.c_aber}\n"
                f"BORN {cfg.born}\nNB_THREADS 1\nPREMIER_ANGLE 0\nDIM_FINAL {cfg.dim_final}\nEXPORT_OTF 1\n"
                f"COEF_NA_OBJ_LIMIT {cfg.coef_na_obj_limit}\n")
    d = derive(cfg)
    with open(os.path.join(res, "parametres.raw"), "wb") as f:
        f.write(struct.pack("<5d", cfg.nxmax, n_angles, d["rayon"], cfg.ccd_roix, d["tp_holo"]))
    return home


MANIP_KEYS = ("rayon", "tp_holo", "tp_uborn", "delta_f", "tp_tomo", "n0", "lambda0", "na", "coef_na_obj_limit",
              "dim_final", "nxmax")


def manip(cfg, n_angles: int = 1) -> dict:
    with tempfile.TemporaryDirectory() as root:
        home = config_tree(cfg, n_angles, root)
        out = np.empty(len(MANIP_KEYS), np.float64)
        _libs()[1].ref_rec_manip(home.encode(), _p(out))
    return dict(zip(MANIP_KEYS, out.tolist()))


def reconstruction(fields: np.ndarray, posspec: np.ndarray, cfg) -> dict:
    f = np.ascontiguousarray(fields, np.complex128)
    p = np.ascontiguousarray(posspec, np.float64)
    n, D = f.shape[0], cfg.dim_final
    ind = np.empty((D, D, D), np.complex128)
    cnt = np.empty((D, D, D), np.float64)
    otf = np.empty((D, D, D), np.float64)
    with tempfile.TemporaryDirectory() as root:
        home = config_tree(cfg, n, root)
        _libs()[1].ref_rec_volume(home.encode(), _p(f), _p(p), n, _p(ind), _p(cnt), _p(otf))
    return {"indice": ind, "counts": cnt, "otf": otf}
