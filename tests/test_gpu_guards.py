"""Decisions near rounding boundaries and bounded device waits.

Specular search: the reference's coordSpec (pretraitement_hors_axe_CPU/fonctions.cpp:88-101)
compares FP64 magnitudes (|z|^2 at index 0, |z| elsewhere, first maximum
wins).  The GPU compares in FP32 and re-decides in FP64 when the runner-up is
within the guard of the winner.  Planted near ties, which FP32 alone decides
differently from FP64, must give the oracle's positions.

Bounded waits: with the extraction's first bulk-copy wait limited to zero
polls every wait gives up at once; the call must report TDM_ECUDA with its
message, the data must still be right (the warp waited for its copy under
the full bound), and the next call with the default bound must be clean.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import Context, Geometry, TdmError, api
from tests.helpers import c64, planted_ties, small_case

pytestmark = pytest.mark.gpu


def _fp32_decision(spec: np.ndarray) -> int:
    """coordSpec with FP32 magnitudes (the GPU's first decision)."""
    s = spec.astype(np.complex64).ravel()
    sq = (s.real * s.real + s.imag * s.imag).astype(np.float32)
    v = np.sqrt(sq).astype(np.float32)
    v[0] = sq[0]
    return int(np.argmax(v))  # first maximum


def test_specular_near_ties_match_fp64():
    acq, _, _ = small_case("plain_512_born", M=1)
    F = 2 * acq.nxmax
    M = 10
    rng = np.random.default_rng(7)
    spec = planted_ties(F, M, rng)
    ref = [oracle.coord_spec(spec[a].astype(np.complex128)) for a in range(M)]
    fp32 = [_fp32_decision(spec[a]) for a in range(M)]
    assert fp32 != ref  # the planted ties do separate FP32 from FP64
    from dataclasses import replace
    acq = replace(acq, c_aber=0)  # positions only: no fit needed on random spectra
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        pos = np.zeros(2 * M, np.int32)
        ctx.fields(c64(spec), posspec_out=pos)
    got = [int(pos[M + a]) * F + int(pos[a]) for a in range(M)]
    assert got == ref


def test_bounded_wait_reports_without_a_fault():
    import torch
    acq, _, d = small_case("plain_512_born", M=4)
    F = 2 * acq.nxmax
    holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
    with Context(Geometry.from_acquisition(acq), 4) as ctx:
        ref = torch.zeros((4, F, F), dtype=torch.complex64, device="cuda")
        ctx.extract(holos, spectra_out=ref)
        ctx.synchronize()
        ctx.set_wait_limit(0)
        out = torch.zeros_like(ref)
        ctx.extract(holos, spectra_out=out)
        with pytest.raises(TdmError) as e:
            ctx.synchronize()
        assert e.value.status == api.STATUS_CODES["TDM_ECUDA"]
        assert "bulk copy" in str(e.value)
        assert torch.equal(out, ref)  # each warp waited for its copy under the full bound
        ctx.set_wait_limit(-1)
        out.zero_()
        ctx.extract(holos, spectra_out=out)
        ctx.synchronize()  # clean
        assert torch.equal(out, ref)
