"""The allocation-free extraction entry point (tdm_extract_noalloc).

Callers that cannot allocate GPU memory -- an acquisition loop that must not
stall on cudaMalloc between bursts of frames, or an application whose memory
pool already owns the device -- call tdm_extract_noalloc with their own device
buffers; its scratch is a fixed 4 MiB array inside the library.  These checks
call it through the C ABI twice in a row (two geometries, so the second call
reuses scratch the first one filled) and compare each result with tdm_extract
on a context, within the parity tolerance of the other tests.  This file is
collected last so that a failure here does not hide the other tests.
"""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

from mtd_transmission_gb300 import Context, Geometry, api
from tests.helpers import rel_l2, small_case

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _case(name, M, **over):
    import torch
    acq, _, d = small_case(name, M=M, **over)
    holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
    return acq, holos


def _with_context(acq, holos):
    import torch
    F = 2 * acq.nxmax
    ref = torch.zeros((holos.shape[0], F, F, 2), dtype=torch.float32, device="cuda")
    with Context(Geometry.from_acquisition(acq), holos.shape[0]) as ctx:
        ctx.extract(holos, spectra_out=ref)
        ctx.synchronize()
    return ref


def test_noalloc_extract_matches_context_twice():
    import torch
    stream = torch.cuda.current_stream().cuda_stream
    cases = [_case("plain_512_born", 6),                                   # 512^2, 128^2 crops
             _case("rytov_1024", 5, ccd_roix=1024, nxmax=128, circle_cx=256, circle_cy=256)]  # 1024^2, 256^2
    for acq, holos in cases:
        F = 2 * acq.nxmax
        out = torch.full((holos.shape[0], F, F, 2), float("nan"), dtype=torch.float32, device="cuda")
        rc = api.extract_noalloc(Geometry.from_acquisition(acq), holos, out, stream)
        assert rc == 0
        torch.cuda.synchronize()
        ref = _with_context(acq, holos)
        o, r = out.cpu().numpy(), ref.cpu().numpy()
        for a in range(holos.shape[0]):
            c_o = o[a, ..., 0] + 1j * o[a, ..., 1]
            c_r = r[a, ..., 0] + 1j * r[a, ..., 1]
            assert rel_l2(c_o, c_r) <= TOL, a


def _raw(geom, holos_ptr, n, out_ptr):
    """The C entry point itself, without the Python wrapper's buffer checks."""
    return api.lib().tdm_extract_noalloc(ctypes.byref(geom), holos_ptr, 16, n, out_ptr, None)


def test_noalloc_extract_rejections():
    import torch
    acq, holos = _case("plain_512_born", 1)
    F = 2 * acq.nxmax
    g = Geometry.from_acquisition(acq)
    out = torch.zeros((1, F, F, 2), dtype=torch.float32, device="cuda")
    einval, eunsup = api.STATUS_CODES["TDM_EINVAL"], api.STATUS_CODES["TDM_EUNSUPPORTED"]
    # holograms in host memory: the entry point takes device buffers only
    assert _raw(g, api.ptr(holos.cpu()), 1, api.ptr(out)) == einval
    # spectra not 8-byte aligned, 16-bit holograms not 2-byte aligned: refused before any launch
    wide = torch.zeros(2 * F * F + 2, dtype=torch.float32, device="cuda")
    assert _raw(g, api.ptr(holos), 1, ctypes.c_void_p(wide.data_ptr() + 4)) == einval
    hb = torch.zeros(holos.numel() + 1, dtype=torch.uint16, device="cuda")
    assert _raw(g, ctypes.c_void_p(hb.data_ptr() + 1), 1, api.ptr(out)) == einval
    # a 2048^2 hologram with 512^2 crops needs 8 MiB of scratch, beyond the fixed 4 MiB
    big = Geometry.from_acquisition(acq)
    big.ccd_roix, big.nxmax, big.circle_cx, big.circle_cy = 2048, 256, 512, 512
    assert _raw(big, api.ptr(holos), 1, api.ptr(out)) == eunsup
    # the wrapper refuses buffers too small for n before calling the library
    with pytest.raises(ValueError):
        api.extract_noalloc(g, holos, out, n=2)
