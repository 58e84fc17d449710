"""Herraez unwrapping (VOLKOV 0) on the GPU against the oracle.

The oracle's restatement of phaseUnwrapping_Mat is pinned bit for bit on
the reference's own compiled unwrapper (tests/test_oracle_pinned.py).  Given
the GPU's own wrapped phase, the GPU's unwrapped phase must equal the
oracle's bit for bit: the reliabilities, the edge order of the reference's
merge sort, the border pixels' rand() draws (which depend on the angle's
index in the stack) and the group merging are integer or exactly rounded
float work.  The fields and the volume from holograms are then compared
with the oracle's VOLKOV 0 path at the path's usual tolerance.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import Context, Geometry
from tests.helpers import c64, oracle_cfg, rel_l2, small_case

pytestmark = pytest.mark.gpu

TOL = 1e-4
# (workload, overrides): 128-point fields, the reference's own 250-point
# geometry (mixed-radix passes), 256-point and 512-point fields, Rytov and
# Born
CASES = {
    "rytov_128": ("rytov_1024", dict(ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128, dim_final=256)),
    "born_128": ("plain_512_born", dict()),
    "rytov_250": ("tomo_config_1024", dict()),
    "rytov_256": ("rytov_1024", dict()),
    "born_512": ("large_2048", dict()),  # 512-point fields: the forest in global memory
}


def _run(key, M):
    name, over = CASES[key]
    acq, _, d = small_case(name, M=M, volkov=0, **over)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    F = 2 * acq.nxmax
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        if F <= 256:  # the 1024^3 phantom leaves no background on the fit's grid: unit mask
            ctx.set_mask(np.ascontiguousarray(d["mask"]))
        fo = np.zeros((M, F, F), np.complex64)
        po = np.zeros(2 * M, np.int32)
        ph = np.zeros((M, F, F), np.float32)
        un = np.zeros((M, F, F), np.float32)
        ctx.fields_debug(c64(spec), fields_out=fo, posspec_out=po, phase=ph, unwrapped=un)
    return acq, cfg, d, spec, fo, po, ph, un


@pytest.mark.parametrize("key", list(CASES))
def test_unwrap_bit_exact_on_the_gpu_phase(key):
    """Each angle's unwrapped phase equals the oracle's Herraez unwrap of the
    GPU's own wrapped phase, bit for bit, for angles 0 .. M-1 of the stack
    (so later angles draw their border reliabilities further down the C
    library's rand() sequence)."""
    M = 5
    _, _, _, _, _, _, ph, un = _run(key, M)
    wraps = 0
    for a in range(M):
        ref, inc = oracle.herraez(ph[a].astype(np.float64), a)
        np.testing.assert_array_equal(un[a], ref.astype(np.float32), err_msg=f"angle {a}")
        wraps += int(np.count_nonzero(inc))
    if key.startswith("rytov"):
        assert wraps > 0  # the Rytov phases (tens of radians) do wrap


@pytest.mark.parametrize("key", ["rytov_128", "born_128", "rytov_250"])
def test_fields_and_volume_against_the_oracle(key):
    """Holograms to fields (VOLKOV 0) and the volume, against the oracle's
    VOLKOV 0 path from the same holograms: positions exactly, fields and
    volume within the path's 1e-4 rel-L2."""
    M = 6
    acq, cfg, d, spec, fo, po, _, _ = _run(key, M)
    fields, pos = oracle.fields(spec, cfg, d["mask"])
    np.testing.assert_array_equal(po, pos.astype(np.int32))
    for a in range(M):
        assert rel_l2(fo[a], fields[a]) <= TOL, (a, rel_l2(fo[a], fields[a]))
    ref = oracle.reconstruction(fields, pos, cfg)
    D = acq.dim_final
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros((D, D, D), np.float32)
        cnt = np.zeros((D, D, D), np.uint32)
        ctx.pipeline(np.ascontiguousarray(d["holos"]), indice=re, absorption=im, counts=cnt)
    np.testing.assert_array_equal(cnt, ref["counts"].astype(np.uint32))
    assert rel_l2(re, ref["indice"].real) <= TOL and rel_l2(im, ref["indice"].imag) <= TOL
