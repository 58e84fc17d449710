"""Python mirror of the C ABI in include/tdm.h (ctypes over libtdm.so).

The library is the product: every call goes to the sm_103a kernels.  There is
no CPU fallback; importing works without a GPU, but creating a context needs
the CUDA device and a built libtdm.so (``mtd_transmission_gb300.build``).

Array arguments may be numpy arrays (host memory) or contiguous torch tensors
(host or CUDA memory); the library detects device pointers itself.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

_HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(_HERE, "libtdm.so")

TDM_OK = 0
STATUS = {-1: "TDM_EINVAL", -2: "TDM_EUNSUPPORTED", -3: "TDM_ECUDA", -4: "TDM_ENOMEM", -5: "TDM_EDATA", -6: "TDM_EIO"}
STATUS_CODES = {v: k for k, v in STATUS.items()}

# Exported symbols declared in include/tdm.h.
EXPORTS = (
    "tdm_create", "tdm_destroy", "tdm_last_error", "tdm_get_derived", "tdm_derive", "tdm_set_mask", "tdm_extract",
    "tdm_fields", "tdm_fields_debug", "tdm_reconstruct", "tdm_pipeline", "tdm_synchronize", "tdm_stream",
    "tdm_launch_count", "tdm_stage_ms", "tdm_extract_val", "tdm_extract_string", "tdm_read_geom", "tdm_read_pgm",
    "tdm_pgm_info", "tdm_write_tiff_f32", "tdm_profile", "tdm_profile_count", "tdm_profile_read",
    "tdm_extract_noalloc", "tdm_pipeline_async", "tdm_cap_planes", "tdm_forward", "tdm_adjoint",
    "tdm_tv_reconstruct", "tdm_batch_create", "tdm_batch_launch", "tdm_batch_destroy", "tdm_autotune",
    "tdm_join", "tdm_set_schedule", "tdm_set_reference_intensity", "tdm_set_wait_limit",
    "tdm_write_hdf5_complex",
)


class TdmError(RuntimeError):
    def __init__(self, status: int, message: str):
        super().__init__(f"{STATUS.get(status, status)}: {message}")
        self.status = status


class Geometry(ctypes.Structure):
    """tdm_geom: keys of recon.txt / config_manip.txt (real keys float-rounded)."""
    _fields_ = [
        ("ccd_roix", ctypes.c_int), ("nxmax", ctypes.c_int), ("circle_cx", ctypes.c_int),
        ("circle_cy", ctypes.c_int), ("dim_final", ctypes.c_int), ("born", ctypes.c_int),
        ("c_aber", ctypes.c_int), ("deroul", ctypes.c_int), ("volkov", ctypes.c_int),
        ("na", ctypes.c_double), ("n0", ctypes.c_double), ("lambda0", ctypes.c_double),
        ("f_tube", ctypes.c_double), ("f_obj", ctypes.c_double), ("tpcam", ctypes.c_double),
        ("rf", ctypes.c_double), ("coef_na_obj_limit", ctypes.c_double),
    ]

    @classmethod
    def from_acquisition(cls, acq) -> "Geometry":
        f = lambda v: float(np.float32(v))  # noqa: E731  extract_val returns float
        return cls(ccd_roix=acq.ccd_roix, nxmax=acq.nxmax, circle_cx=acq.circle_cx, circle_cy=acq.circle_cy,
                   dim_final=acq.dim_final, born=int(acq.born), c_aber=int(acq.c_aber), deroul=int(acq.deroul),
                   volkov=int(acq.volkov), na=f(acq.na), n0=f(acq.n0), lambda0=f(acq.lambda0),
                   f_tube=f(acq.f_tube), f_obj=f(acq.f_obj), tpcam=f(acq.tpcam), rf=f(acq.rf),
                   coef_na_obj_limit=f(acq.coef_na_obj_limit))


class Derived(ctypes.Structure):
    _fields_ = [(n, ctypes.c_double) for n in ("rayon", "tp_holo", "tp_uborn", "tp_tomo", "delta_f")]


_lib = None


class TvOpts(ctypes.Structure):
    """tdm_tv_opts."""
    _fields_ = [("iterations", ctypes.c_int), ("init", ctypes.c_int), ("step", ctypes.c_float),
                ("tv_weight", ctypes.c_float), ("tv_eps", ctypes.c_float), ("index_min", ctypes.c_float),
                ("index_max", ctypes.c_float), ("absorption_min", ctypes.c_float),
                ("absorption_max", ctypes.c_float)]


class TvReport(ctypes.Structure):
    """tdm_tv_report."""
    _fields_ = [("iterations", ctypes.c_int), ("misfit_first", ctypes.c_double), ("misfit_last", ctypes.c_double),
                ("seconds", ctypes.c_double)]


def lib():
    """Loads libtdm.so; raises when it has not been built."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: build it with `python -m mtd_transmission_gb300.build`")
    L = ctypes.CDLL(LIB_PATH)
    P, I, D = ctypes.c_void_p, ctypes.c_int, ctypes.c_double
    L.tdm_create.argtypes = [ctypes.POINTER(Geometry), I, ctypes.POINTER(P)]
    L.tdm_destroy.argtypes = [P]
    L.tdm_last_error.argtypes = [P]
    L.tdm_last_error.restype = ctypes.c_char_p
    L.tdm_get_derived.argtypes = [P, ctypes.POINTER(Derived)]
    L.tdm_derive.argtypes = [ctypes.POINTER(Geometry), ctypes.POINTER(Derived)]
    L.tdm_set_mask.argtypes = [P, P]
    L.tdm_extract.argtypes = [P, P, I, I, P]
    L.tdm_fields.argtypes = [P, P, I, P, P]
    L.tdm_fields_debug.argtypes = [P, P, I, P, P, P, P, P]
    L.tdm_reconstruct.argtypes = [P, P, P, I, P, P, P, P]
    L.tdm_pipeline.argtypes = [P, P, I, I, P, P, P, P, P]
    L.tdm_pipeline_async.argtypes = [P, P, I, I, P, P, P, P]
    L.tdm_forward.argtypes = [P, P, P, I, P, P]
    L.tdm_batch_create.argtypes = [I, P, P, P, P, P, P, P, ctypes.POINTER(ctypes.c_void_p)]
    L.tdm_batch_launch.argtypes = [P, P]
    L.tdm_autotune.argtypes = [P, P, I, I, ctypes.POINTER(I)]
    L.tdm_set_schedule.argtypes = [P, I, I]
    L.tdm_set_wait_limit.argtypes = [P, ctypes.c_longlong]
    L.tdm_set_reference_intensity.argtypes = [P, P]
    L.tdm_join.argtypes = [P]
    L.tdm_batch_destroy.argtypes = [P]
    L.tdm_adjoint.argtypes = [P, P, I, P, P, P]
    L.tdm_tv_reconstruct.argtypes = [P, P, I, P, ctypes.POINTER(TvOpts), P, P, ctypes.POINTER(TvReport)]
    L.tdm_cap_planes.argtypes = [P, ctypes.POINTER(I), ctypes.POINTER(I)]
    L.tdm_synchronize.argtypes = [P]
    L.tdm_stream.argtypes = [P]
    L.tdm_stream.restype = P
    L.tdm_launch_count.argtypes = [P]
    L.tdm_launch_count.restype = ctypes.c_uint64
    L.tdm_stage_ms.argtypes = [P, ctypes.c_char_p]
    L.tdm_stage_ms.restype = D
    L.tdm_extract_val.argtypes = [ctypes.c_char_p, ctypes.c_char_p, D, ctypes.POINTER(D)]
    L.tdm_extract_string.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p, ctypes.c_size_t]
    L.tdm_read_geom.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.POINTER(Geometry)]
    L.tdm_read_pgm.argtypes = [ctypes.c_char_p, I, P, ctypes.POINTER(I)]
    L.tdm_pgm_info.argtypes = [ctypes.c_char_p, ctypes.POINTER(I), ctypes.POINTER(I), ctypes.POINTER(I)]
    L.tdm_write_tiff_f32.argtypes = [ctypes.c_char_p, P, I, I, I, D, I]
    L.tdm_write_hdf5_complex.argtypes = [ctypes.c_char_p, P, P, I, I, I]
    L.tdm_extract_noalloc.argtypes = [ctypes.POINTER(Geometry), P, I, I, P, P]
    L.tdm_profile.argtypes = [P, I]
    L.tdm_profile_count.argtypes = []
    L.tdm_profile_read.argtypes = [P, I, ctypes.POINTER(ctypes.c_char_p), ctypes.POINTER(D), ctypes.POINTER(I)]
    _lib = L
    return L


def ptr(a):
    """Address of a numpy array or contiguous torch tensor (None -> NULL)."""
    if a is None:
        return None
    if isinstance(a, np.ndarray):
        if not a.flags["C_CONTIGUOUS"]:
            raise ValueError("array must be C-contiguous")
        return ctypes.c_void_p(a.ctypes.data)
    if hasattr(a, "data_ptr"):
        if not a.is_contiguous():
            raise ValueError("tensor must be contiguous")
        return ctypes.c_void_p(a.data_ptr())
    raise TypeError(f"unsupported array type {type(a)}")


def derive(geom: Geometry) -> dict:
    d = Derived()
    lib().tdm_derive(ctypes.byref(geom), ctypes.byref(d))
    return {n: getattr(d, n) for n, _ in Derived._fields_}


class Context:
    """One reconstruction context (device buffers, tables, stream) on the current GPU."""

    def __init__(self, geom: Geometry, max_angles: int):
        self.geom = geom
        self.max_angles = max_angles
        h = ctypes.c_void_p()
        rc = lib().tdm_create(ctypes.byref(geom), max_angles, ctypes.byref(h))
        if rc != TDM_OK:
            raise TdmError(rc, "tdm_create failed")
        self._h = h
        self.F = 2 * geom.nxmax
        self.D = geom.dim_final

    def _check(self, rc: int, what: str):
        if rc != TDM_OK:
            raise TdmError(rc, f"{what}: {lib().tdm_last_error(self._h).decode()}")

    def close(self):
        if getattr(self, "_h", None):
            lib().tdm_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def stream(self) -> int:
        return int(lib().tdm_stream(self._h) or 0)

    @property
    def launch_count(self) -> int:
        return int(lib().tdm_launch_count(self._h))

    def stage_ms(self, name: str) -> float:
        return float(lib().tdm_stage_ms(self._h, name.encode()))

    def profile(self, enable: bool = True):
        """Starts (or stops) per-kernel event timing; clears previous records."""
        self._check(lib().tdm_profile(self._h, int(enable)), "tdm_profile")

    def profile_read(self) -> dict:
        """{kernel name: (total device ms, launches)} since the last profile() call."""
        out = {}
        for i in range(lib().tdm_profile_count()):
            nm, t, n = ctypes.c_char_p(), ctypes.c_double(), ctypes.c_int()
            self._check(lib().tdm_profile_read(self._h, i, ctypes.byref(nm), ctypes.byref(t), ctypes.byref(n)),
                        "tdm_profile_read")
            if n.value:
                out[nm.value.decode()] = (t.value, n.value)
        return out

    def derived(self) -> dict:
        d = Derived()
        self._check(lib().tdm_get_derived(self._h, ctypes.byref(d)), "tdm_get_derived")
        return {n: getattr(d, n) for n, _ in Derived._fields_}

    def synchronize(self):
        self._check(lib().tdm_synchronize(self._h), "tdm_synchronize")

    def join(self):
        """tdm_join: orders the context stream after the queued volume stages."""
        self._check(lib().tdm_join(self._h), "tdm_join")

    def set_mask(self, mask=None):
        self._check(lib().tdm_set_mask(self._h, ptr(mask)), "tdm_set_mask")

    def set_reference_intensity(self, intensity=None):
        """tdm_set_reference_intensity: H x H float32 Intensite_ref image (holograms are
        divided by its square root before extraction), or None to clear it."""
        if intensity is not None and isinstance(intensity, np.ndarray):
            intensity = np.ascontiguousarray(intensity, np.float32)
        self._check(lib().tdm_set_reference_intensity(self._h, ptr(intensity)), "tdm_set_reference_intensity")

    @staticmethod
    def _bits(holos) -> int:
        dt = str(getattr(holos, "dtype", ""))
        if "uint16" in dt:
            return 16
        if "uint8" in dt:
            return 8
        raise TypeError("holograms must be uint8 or uint16")

    def extract(self, holos, n=None, spectra_out=None):
        n = holos.shape[0] if n is None else n
        self._check(lib().tdm_extract(self._h, ptr(holos), self._bits(holos), n, ptr(spectra_out)), "tdm_extract")
        return spectra_out

    def fields(self, spectra=None, n=None, fields_out=None, posspec_out=None):
        n = spectra.shape[0] if n is None else n
        self._check(lib().tdm_fields(self._h, ptr(spectra), n, ptr(fields_out), ptr(posspec_out)), "tdm_fields")
        return fields_out, posspec_out

    def fields_debug(self, spectra=None, n=None, fields_out=None, posspec_out=None, phase=None, unwrapped=None,
                     amp=None):
        n = spectra.shape[0] if n is None else n
        self._check(lib().tdm_fields_debug(self._h, ptr(spectra), n, ptr(fields_out), ptr(posspec_out), ptr(phase),
                                           ptr(unwrapped), ptr(amp)), "tdm_fields_debug")

    def reconstruct(self, fields=None, posspec=None, n=None, indice=None, absorption=None, otf=None, counts=None):
        n = fields.shape[0] if n is None else n
        self._check(lib().tdm_reconstruct(self._h, ptr(fields), ptr(posspec), n, ptr(indice), ptr(absorption),
                                          ptr(otf), ptr(counts)), "tdm_reconstruct")

    def pipeline(self, holos, indice=None, absorption=None, otf=None, counts=None, posspec=None, n=None):
        n = holos.shape[0] if n is None else n
        self._check(lib().tdm_pipeline(self._h, ptr(holos), self._bits(holos), n, ptr(indice), ptr(absorption),
                                       ptr(otf), ptr(counts), ptr(posspec)), "tdm_pipeline")

    def forward(self, index, absorption=None, n=None, posspec=None, caps_out=None):
        """tdm_forward: cap values S G(index + i absorption) (n x F x F complex, FFT-bin order)."""
        F = 2 * self.geom.nxmax
        if caps_out is None:
            caps_out = np.zeros((n, F, F), np.complex64)
        n = caps_out.shape[0] if n is None else n
        self._check(lib().tdm_forward(self._h, ptr(index), ptr(absorption), n, ptr(posspec), ptr(caps_out)),
                    "tdm_forward")
        return caps_out

    def adjoint(self, caps, n=None, posspec=None, index_out=None, absorption_out=None):
        """tdm_adjoint: index_out + i absorption_out = G^H S^H caps."""
        n = caps.shape[0] if n is None else n
        D = self.geom.dim_final
        if index_out is None:
            index_out = np.zeros((D, D, D), np.float32)
        self._check(lib().tdm_adjoint(self._h, ptr(caps), n, ptr(posspec), ptr(index_out), ptr(absorption_out)),
                    "tdm_adjoint")
        return index_out, absorption_out

    def tv_reconstruct(self, index_io, absorption_io=None, caps=None, n=None, posspec=None, iterations=50,
                       init=1, step=1.0, tv_weight=1e-3, tv_eps=1e-4, index_min=0.0, index_max=float("inf"),
                       absorption_min=0.0, absorption_max=float("inf")):
        """tdm_tv_reconstruct: projected-gradient TV reconstruction; returns the report as a dict."""
        n = (caps.shape[0] if caps is not None else self.max_angles) if n is None else n
        o = TvOpts(iterations=iterations, init=init, step=step, tv_weight=tv_weight, tv_eps=tv_eps,
                   index_min=index_min, index_max=index_max, absorption_min=absorption_min,
                   absorption_max=absorption_max)
        r = TvReport()
        self._check(lib().tdm_tv_reconstruct(self._h, ptr(caps), n, ptr(posspec), ctypes.byref(o), ptr(index_io),
                                             ptr(absorption_io), ctypes.byref(r)), "tdm_tv_reconstruct")
        return {f: getattr(r, f) for f, _ in TvReport._fields_}

    def set_schedule(self, chunk: int, lanes: int):
        """tdm_set_schedule: angles per chunk and chunks in flight of the per-angle stages."""
        self._check(lib().tdm_set_schedule(self._h, chunk, lanes), "tdm_set_schedule")

    def set_wait_limit(self, polls: int):
        """tdm_set_wait_limit: polls of the extraction's first bounded wait on each bulk copy (-1: default)."""
        self._check(lib().tdm_set_wait_limit(self._h, polls), "tdm_set_wait_limit")

    def autotune(self, holos, n=None) -> int:
        """tdm_autotune: picks the fastest schedule (chunk, lanes) on this stack; returns its chunk."""
        n = holos.shape[0] if n is None else n
        out = ctypes.c_int()
        self._check(lib().tdm_autotune(self._h, ptr(holos), self._bits(holos), n, ctypes.byref(out)), "tdm_autotune")
        return out.value

    @property
    def cap_planes(self):
        """(zmin, band): the spectrum planes the Ewald caps can reach (tdm_cap_planes)."""
        z, b = ctypes.c_int(), ctypes.c_int()
        self._check(lib().tdm_cap_planes(self._h, ctypes.byref(z), ctypes.byref(b)), "tdm_cap_planes")
        return z.value, b.value

    def pipeline_async(self, holos, indice=None, absorption=None, otf=None, counts=None, n=None):
        """tdm_pipeline_async: queues one volume and returns; outputs are complete after synchronize().
        Host buffers should be pinned and must stay untouched until then."""
        n = holos.shape[0] if n is None else n
        self._check(lib().tdm_pipeline_async(self._h, ptr(holos), self._bits(holos), n, ptr(indice),
                                             ptr(absorption), ptr(otf), ptr(counts)), "tdm_pipeline_async")


def extract_noalloc(geom: Geometry, holos, spectra_out, stream: int = 0, n=None) -> int:
    """tdm_extract_noalloc: extraction without any GPU allocation (device buffers only).

    For callers that cannot allocate GPU memory (an acquisition loop that must
    not stall on cudaMalloc, or an application whose memory pool owns the
    device).  Returns the TDM status; the work is queued on `stream`.

    The library cannot see buffer sizes, so the arrays are checked here:
    holos a contiguous CUDA tensor of at least n uint8/uint16 H x H images,
    spectra_out a contiguous CUDA tensor holding at least n F x F complex
    values (complex64, or float32 with a trailing 2)."""
    import torch
    H, F = geom.ccd_roix, 2 * geom.nxmax
    n = holos.shape[0] if n is None else n
    for name, t in (("holos", holos), ("spectra_out", spectra_out)):
        if not isinstance(t, torch.Tensor) or not t.is_cuda or not t.is_contiguous():
            raise ValueError(f"extract_noalloc: {name} must be a contiguous CUDA tensor")
    if holos.dtype not in (torch.uint8, torch.uint16, torch.int16) or tuple(holos.shape[1:]) != (H, H):
        raise ValueError(f"extract_noalloc: holos must be (n, {H}, {H}) uint8 or uint16")
    if not 0 < n <= holos.shape[0]:
        raise ValueError(f"extract_noalloc: n={n} outside [1, {holos.shape[0]}]")
    if spectra_out.device != holos.device:
        raise ValueError("extract_noalloc: holos and spectra_out must be on the same device")
    if spectra_out.dtype == torch.complex64:
        ok = spectra_out.dim() == 3 and tuple(spectra_out.shape[1:]) == (F, F)
    else:
        ok = (spectra_out.dtype == torch.float32 and spectra_out.dim() == 4
              and tuple(spectra_out.shape[1:]) == (F, F, 2))
    if not ok or spectra_out.shape[0] < n:
        raise ValueError(f"extract_noalloc: spectra_out must hold at least n={n} complex64 ({F}, {F}) spectra")
    return int(lib().tdm_extract_noalloc(ctypes.byref(geom), ptr(holos), Context._bits(holos), n, ptr(spectra_out),
                                         ctypes.c_void_p(stream)))


# ---- host-side file helpers -------------------------------------------------

def extract_val(path: str, key: str, default: float = 0.0):
    out = ctypes.c_double()
    rc = lib().tdm_extract_val(path.encode(), key.encode(), default, ctypes.byref(out))
    if rc < 0:
        raise TdmError(rc, f"cannot read {path}")
    return out.value, bool(rc)


def extract_string(path: str, key: str) -> str | None:
    buf = ctypes.create_string_buffer(4096)
    rc = lib().tdm_extract_string(path.encode(), key.encode(), buf, len(buf))
    if rc < 0:
        raise TdmError(rc, f"cannot read {path}")
    return buf.value.decode() if rc else None


def read_geom(recon_txt: str, config_manip_txt: str) -> Geometry:
    g = Geometry()
    rc = lib().tdm_read_geom(recon_txt.encode(), config_manip_txt.encode(), ctypes.byref(g))
    if rc != TDM_OK:
        raise TdmError(rc, "tdm_read_geom")
    return g


def read_pgm(path: str, roi: int) -> np.ndarray:
    w, h, mx = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    rc = lib().tdm_pgm_info(path.encode(), ctypes.byref(w), ctypes.byref(h), ctypes.byref(mx))
    if rc != TDM_OK:
        raise TdmError(rc, f"cannot read {path}")
    out = np.empty((roi, roi), np.uint8 if mx.value < 256 else np.uint16)
    bits = ctypes.c_int()
    rc = lib().tdm_read_pgm(path.encode(), roi, ptr(out), ctypes.byref(bits))
    if rc != TDM_OK:
        raise TdmError(rc, f"cannot read {path}")
    return out


def write_tiff(path: str, vol: np.ndarray, pixel_size: float, orientation: int = 4):
    v = np.ascontiguousarray(vol, np.float32)
    if v.ndim == 2:
        v = v[None]
    pages, hgt, wdt = v.shape
    rc = lib().tdm_write_tiff_f32(path.encode(), ptr(v), wdt, hgt, pages, pixel_size, orientation)
    if rc != TDM_OK:
        raise TdmError(rc, f"cannot write {path}")


def write_hdf5_complex(path: str, re: np.ndarray, im: np.ndarray):
    """tdm_write_hdf5_complex: /indice_complexe/{Re,Im} float32 (nz, ny, nx)."""
    r = np.ascontiguousarray(re, np.float32)
    i = np.ascontiguousarray(im, np.float32)
    nz, ny, nx = r.shape
    rc = lib().tdm_write_hdf5_complex(path.encode(), ptr(r), ptr(i), nx, ny, nz)
    if rc != TDM_OK:
        raise TdmError(rc, f"cannot write {path}")


class Batch:
    """tdm_batch: several stacks (one Context each) in one CUDA-graph launch.

    stacks: list of (context, holos, indice, absorption, otf) with device
    buffers (otf / absorption may be None); the buffers are bound at creation."""

    def __init__(self, stacks):
        k = len(stacks)
        arr = lambda vals: (ctypes.c_void_p * k)(*[None if v is None else ptr(v).value for v in vals])
        ctxs = (ctypes.c_void_p * k)(*[st[0]._h.value for st in stacks])
        holos = arr([st[1] for st in stacks])
        bits = (ctypes.c_int * k)(*[st[0]._bits(st[1]) for st in stacks])
        n = (ctypes.c_int * k)(*[int(st[1].shape[0]) for st in stacks])
        h = ctypes.c_void_p()
        rc = lib().tdm_batch_create(k, ctxs, holos, bits, n, arr([st[2] for st in stacks]),
                                    arr([st[3] for st in stacks]), arr([st[4] for st in stacks]), ctypes.byref(h))
        if rc != TDM_OK:
            raise TdmError(rc, "tdm_batch_create: " + lib().tdm_last_error(stacks[0][0]._h).decode())
        self._h = h
        self._stacks = stacks  # keep the buffers alive

    def launch(self, stream: int = 0):
        rc = lib().tdm_batch_launch(self._h, ctypes.c_void_p(stream))
        if rc != TDM_OK:
            raise TdmError(rc, "tdm_batch_launch failed")

    def close(self):
        if getattr(self, "_h", None):
            lib().tdm_batch_destroy(self._h)
            self._h = None

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def __del__(self):
        self.close()

