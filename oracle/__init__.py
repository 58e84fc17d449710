"""ctypes wrapper of the FP64 CPU oracle (``tdm_oracle.cpp``).

Test infrastructure only: imported by ``tests/``, ``__graft_entry__.smoke()``
and the CPU-baseline leg of ``bench.py``, to produce reference values.  The
restatement follows the reference functions (cited file:line in the C++) and
is pinned on them: ``oracle.reference_build`` runs the reference's own source
files, compiled into ``oracle/_ref/``, on the same inputs
(``tests/test_oracle_pinned.py``).
"""
from __future__ import annotations

import ctypes
import os
import subprocess
from dataclasses import dataclass

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
_LIB_PATH = os.path.join(_HERE, "liboracle_tdm.so")
_lib = None


def build(force: bool = False) -> str:
    """Compile liboracle_tdm.so with the Makefile beside this file."""
    if force or not os.path.exists(_LIB_PATH) or (
        os.path.getmtime(_LIB_PATH) < os.path.getmtime(os.path.join(_HERE, "tdm_oracle.cpp"))
    ):
        subprocess.run(["make", "-C", _HERE, "-s", "-B" if force else "all"], check=True)
    return _LIB_PATH


class OrcCfg(ctypes.Structure):
    _fields_ = [
        ("n0", ctypes.c_double), ("na", ctypes.c_double), ("lambda0", ctypes.c_double),
        ("f_tube", ctypes.c_double), ("f_obj", ctypes.c_double), ("tpcam", ctypes.c_double),
        ("rf", ctypes.c_double), ("coef_na_obj_limit", ctypes.c_double),
        ("ccd_roix", ctypes.c_int), ("nxmax", ctypes.c_int), ("circle_cx", ctypes.c_int),
        ("circle_cy", ctypes.c_int), ("dim_final", ctypes.c_int),
        ("born", ctypes.c_int), ("c_aber", ctypes.c_int), ("deroul", ctypes.c_int), ("volkov", ctypes.c_int),
    ]


class OrcDerived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rayon", "tp_holo", "tp_uborn", "tp_tomo", "delta_f")]


def lib():
    global _lib
    if _lib is None:
        build()
        L = ctypes.CDLL(_LIB_PATH)
        P = ctypes.c_void_p
        L.orc_derive.argtypes = [ctypes.POINTER(OrcCfg), ctypes.POINTER(OrcDerived)]
        L.orc_tukey2d.argtypes = [ctypes.c_int, ctypes.c_float, P]
        L.orc_fft2d.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_fft3d.argtypes = [P, ctypes.c_int, ctypes.c_int]
        L.orc_extract.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_coord_spec.argtypes = [P, ctypes.c_int]
        L.orc_calc_uborn2.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.c_int, P]
        L.orc_volkov.argtypes = [P, ctypes.c_int, P]
        L.orc_herraez.argtypes = [P, ctypes.c_int, ctypes.c_int, P, P]
        L.orc_crand.argtypes = [ctypes.c_longlong, ctypes.c_int, P]
        L.orc_aber_surface.argtypes = [P, ctypes.c_int, P, P]
        L.orc_fields.argtypes = [P, ctypes.c_int, ctypes.c_int, ctypes.POINTER(OrcCfg), P, P, P, P, P, P, P, P]
        L.orc_reconstruction.argtypes = [P, P, ctypes.c_int, ctypes.POINTER(OrcCfg), P, P, P, P, P]
        L.orc_set_threads.argtypes = [ctypes.c_int]
        _lib = L
    return _lib


def _p(a):
    return None if a is None else a.ctypes.data_as(ctypes.c_void_p)


def _f32(v) -> float:
    """extract_val returns float: keys are rounded to single precision."""
    return float(np.float32(v))


@dataclass
class Config:
    """Keys of config_manip.txt / recon.txt used on the path."""
    ccd_roix: int = 512
    nxmax: int = 64
    circle_cx: int = 128
    circle_cy: int = 128
    dim_final: int = 256
    na: float = 1.40
    n0: float = 1.515
    lambda0: float = 633e-9
    f_tube: float = 0.15
    f_obj: float = 0.002
    tpcam: float = 5.5e-6
    rf: float = 0.75
    born: int = 1
    c_aber: int = 1
    deroul: int = 1
    volkov: int = 1
    coef_na_obj_limit: float = 1.0

    def cstruct(self) -> OrcCfg:
        return OrcCfg(
            n0=_f32(self.n0), na=_f32(self.na), lambda0=_f32(self.lambda0), f_tube=_f32(self.f_tube),
            f_obj=_f32(self.f_obj), tpcam=_f32(self.tpcam), rf=_f32(self.rf),
            coef_na_obj_limit=_f32(self.coef_na_obj_limit), ccd_roix=self.ccd_roix, nxmax=self.nxmax,
            circle_cx=self.circle_cx, circle_cy=self.circle_cy, dim_final=self.dim_final,
            born=int(self.born), c_aber=int(self.c_aber), deroul=int(self.deroul), volkov=int(self.volkov))


def derive(cfg: Config) -> dict:
    d = OrcDerived()
    c = cfg.cstruct()
    lib().orc_derive(ctypes.byref(c), ctypes.byref(d))
    return {n: getattr(d, n) for n, _ in OrcDerived._fields_}


def tukey2d(n: int, alpha: float) -> np.ndarray:
    out = np.empty((n, n), np.float64)
    lib().orc_tukey2d(n, alpha, _p(out))
    return out


def fft2d(a: np.ndarray, sign: int = -1) -> np.ndarray:
    x = np.ascontiguousarray(a, np.complex128).copy()
    assert lib().orc_fft2d(_p(x), x.shape[0], sign) == 0
    return x


def fft3d(a: np.ndarray, sign: int = -1) -> np.ndarray:
    x = np.ascontiguousarray(a, np.complex128).copy()
    assert lib().orc_fft3d(_p(x), x.shape[0], sign) == 0
    return x


def extract(holo: np.ndarray, cfg: Config) -> np.ndarray:
    """holo2TF_UBorn for one hologram (H x H samples) -> F x F complex crop."""
    H = holo.shape[0]
    tk = tukey2d(H, 0.05)
    h = np.ascontiguousarray(holo, np.float64)
    F = 2 * cfg.nxmax
    out = np.empty((F, F), np.complex128)
    rc = lib().orc_extract(_p(h), H, cfg.nxmax, cfg.circle_cx, cfg.circle_cy, _p(tk), _p(out))
    if rc != 0:
        raise ValueError(f"orc_extract failed rc={rc}")
    return out


def reference_amplitude(intensity: np.ndarray) -> np.ndarray:
    """initRef (pretraitement_hors_axe_CPU/fonctions.cpp:46-61): sqrt of the
    reference intensity, 1 where the intensity is 0."""
    i = np.asarray(intensity, np.float64)
    return np.where(i != 0, np.sqrt(np.where(i != 0, i, 1.0)), 1.0)


def extract_stack(holos: np.ndarray, cfg: Config, ref_intensity: np.ndarray | None = None) -> np.ndarray:
    """holo2TF_UBorn per hologram; with ref_intensity each hologram is first
    divided by the reference amplitude (main.cpp:147, commented out in the
    reference's own run)."""
    if ref_intensity is not None:
        amp = reference_amplitude(ref_intensity)
        return np.stack([extract(np.asarray(h, np.float64) / amp, cfg) for h in holos])
    return np.stack([extract(h, cfg) for h in holos])


def coord_spec(spec: np.ndarray) -> int:
    s = np.ascontiguousarray(spec, np.complex128)
    return int(lib().orc_coord_spec(_p(s), s.shape[0]))


def calc_uborn2(spec: np.ndarray, px: int, py: int) -> np.ndarray:
    s = np.ascontiguousarray(spec, np.complex128)
    out = np.empty_like(s)
    lib().orc_calc_uborn2(_p(s), s.shape[0], px, py, _p(out))
    return out


def volkov(phase: np.ndarray) -> np.ndarray:
    p = np.ascontiguousarray(phase, np.float64)
    out = np.empty_like(p)
    lib().orc_volkov(_p(p), p.shape[0], _p(out))
    return out


def herraez(phase: np.ndarray, angle: int = 0):
    """Herraez unwrapping of a square wrapped phase as the angle of index
    `angle` of the stack: (unwrapped phase, 2 pi count per pixel)."""
    p = np.ascontiguousarray(phase, np.float64)
    out = np.empty_like(p)
    inc = np.empty(p.shape, np.int32)
    lib().orc_herraez(_p(p), p.shape[0], angle, _p(out), _p(inc))
    return out, inc


def crand(skip: int, n: int) -> np.ndarray:
    """n outputs of the C library's rand() after `skip` draws (oracle's restatement)."""
    out = np.empty(n, np.int32)
    lib().orc_crand(skip, n, _p(out))
    return out


def aber_surface(img: np.ndarray, mask: np.ndarray | None = None):
    im = np.ascontiguousarray(img, np.float64)
    F = im.shape[0]
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    out = np.empty_like(im)
    n = lib().orc_aber_surface(_p(m), F, _p(im), _p(out))
    if n < 0:
        raise ValueError("aberration fit undefined (<= 9 background samples)")
    return out


def fields(spectra: np.ndarray, cfg: Config, mask: np.ndarray | None = None, debug: bool = False):
    """Second loop of tomo_pretraitement: returns (fields, tabPosSpec[, dbg])."""
    s = np.ascontiguousarray(spectra, np.complex128)
    M, F, _ = s.shape
    out = np.empty_like(s)
    pos = np.empty(2 * M, np.float64)
    m = None if mask is None else np.ascontiguousarray(mask, np.uint8)
    dbg = {k: np.empty((M, F, F), np.float64) for k in ("phase", "unwrap", "amp", "phase_corr", "amp_corr")} if debug else {}
    c = cfg.cstruct()
    rc = lib().orc_fields(_p(s), M, cfg.nxmax, ctypes.byref(c), _p(m), _p(out), _p(pos),
                          _p(dbg.get("phase")), _p(dbg.get("unwrap")), _p(dbg.get("amp")),
                          _p(dbg.get("phase_corr")), _p(dbg.get("amp_corr")))
    if rc != 0:
        raise ValueError(f"orc_fields failed rc={rc}")
    return (out, pos, dbg) if debug else (out, pos)


def reconstruction(fields_: np.ndarray, posspec: np.ndarray, cfg: Config, want_counts=True, want_otf=True,
                   want_spectrum=False, want_indice=True):
    f = np.ascontiguousarray(fields_, np.complex128)
    p = np.ascontiguousarray(posspec, np.float64)
    M = f.shape[0]
    D = cfg.dim_final
    ind = np.empty((D, D, D), np.complex128)
    secs = np.zeros(2, np.float64)
    cnt = np.empty((D, D, D), np.float64) if want_counts else None
    otf = np.empty((D, D, D), np.float64) if want_otf else None
    spc = np.empty((D, D, D), np.complex128) if want_spectrum else None
    c = cfg.cstruct()
    rc = lib().orc_reconstruction(_p(f), _p(p), M, ctypes.byref(c), _p(ind), _p(cnt), _p(otf), _p(spc), _p(secs))
    if rc != 0:
        raise ValueError(f"orc_reconstruction failed rc={rc}")
    return {"indice": ind, "counts": cnt, "otf": otf, "spectrum": spc, "seconds": secs}


def set_threads(n: int) -> int:
    return int(lib().orc_set_threads(n))


# ---------------------------------------------------------------- forward operator and adjoint
# The volume stage of the reconstruction is x = T(V) = s shift3(IFFT3(shift3(V)))
# with s = delta_f^3 * (-1 / (2 n0 k_v^2)) (Reconstruction/main.cpp:282-352) and
# IFFT3 unnormalised.  The forward operator samples G(x) = T^-1(x) at every
# angle's cap cells, the cells retroPropag_Born accumulates
# (Reconstruction/src/fonctions.cpp:903-925); cap values are indexed by the
# per-field FFT bin (kx, ky), the bin of cell fd being ((fd + N) - posSpec) mod F.

def _round_half_away(v):
    return np.sign(v) * np.floor(np.abs(v) + 0.5)


def volume_scale(cfg: Config) -> float:
    dv = derive(cfg)
    k_v = 2 * np.pi / float(np.float32(cfg.lambda0))
    return dv["delta_f"] ** 3 * (-1.0 / (2 * float(np.float32(cfg.n0)) * k_v * k_v))


def cap_cells(posspec: np.ndarray, cfg: Config):
    """Per angle: (mask over the F x F bins [ky][kx], Z, Y, X cell indices) or None when skipped."""
    N, D = cfg.nxmax, cfg.dim_final
    F, dec = 2 * N, D // 2
    rayon = derive(cfg)["rayon"]
    M = len(posspec) // 2
    ky, kx = np.meshgrid(np.arange(F), np.arange(F), indexing="ij")
    coef = float(np.float32(cfg.coef_na_obj_limit))
    out = []
    for a in range(M):
        px, py = int(posspec[a]), int(posspec[M + a])
        fxm0, fym0 = px - N, py - N
        c = rayon * rayon - fxm0 * fxm0 - fym0 * fym0
        if _round_half_away(c) < 0:
            out.append(None)
            continue
        fzm0 = np.sqrt(c)
        fdx = ((kx + px) % F) - N
        fdy = ((ky + py) % F) - N
        inside = fdx * fdx + fdy * fdy < coef * N * N
        s2 = np.where(inside, rayon * rayon - fdx * fdx - fdy * fdy, 0.0)
        koz = _round_half_away(np.sqrt(s2) - fzm0)
        X = -fxm0 + fdx + dec
        Y = -fym0 + fdy + dec
        Z = (koz + dec).astype(np.int64)
        out.append((inside, Z[inside], Y[inside], X[inside]))
    return out


def _shift3(v):
    return np.fft.fftshift(v)


def forward_caps(index: np.ndarray, absorption: np.ndarray | None, posspec: np.ndarray, cfg: Config) -> np.ndarray:
    """Cap values S G(index + i absorption), n x F x F complex in FFT-bin order."""
    D, F = cfg.dim_final, 2 * cfg.nxmax
    x = index.astype(np.complex128)
    if absorption is not None:
        x = x + 1j * absorption
    G = _shift3(np.fft.fftn(_shift3(x))) / (volume_scale(cfg) * D ** 3)
    cells = cap_cells(posspec, cfg)
    caps = np.zeros((len(cells), F, F), np.complex128)
    for a, cell in enumerate(cells):
        if cell is None:
            continue
        inside, Z, Y, X = cell
        caps[a][inside] = G[Z, Y, X]
    return caps


def adjoint_caps(caps: np.ndarray, posspec: np.ndarray, cfg: Config) -> np.ndarray:
    """G^H S^H caps as a complex volume (index = real part, absorption = imaginary part)."""
    D = cfg.dim_final
    V = np.zeros((D, D, D), np.complex128)
    for a, cell in enumerate(cap_cells(posspec, cfg)):
        if cell is None:
            continue
        inside, Z, Y, X = cell
        np.add.at(V, (Z, Y, X), caps[a][inside])
    return _shift3(np.fft.ifftn(_shift3(V)) * D ** 3) / (volume_scale(cfg) * D ** 3)
