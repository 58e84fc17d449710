"""The reference's own configuration on the GPU.

Tomo_config/config_manip.txt and recon.txt of the reference (NXMAX 125,
CIRCLE_CX 247, CIRCLE_CY 777, CCD_ROIX 1024, DIM_FINAL 512, Rytov, Volkov,
aberration correction) give 250 x 250 fields, a 500 x 500 Volkov mirror and
DIM_FINAL != 4 NXMAX.  The geometry comes from
tests/golden/tomo_config_geometry.json, which tdm_read_geom parsed from
those files (checked on the CPU where the reference tree exists).  A small
synthetic stack at that geometry against the FP64 oracle: specular
positions and hit counts bit for bit, spectra, fields and the volume within
rel-L2 1e-4.
"""
from __future__ import annotations

import json
import os
from dataclasses import replace

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import Context, Geometry
from tests import simul
from tests.helpers import c64, oracle_cfg, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _golden_geometry() -> Geometry:
    with open(os.path.join(os.path.dirname(__file__), "golden", "tomo_config_geometry.json")) as f:
        return Geometry(**json.load(f))


@pytest.fixture(scope="module", params=["rytov", "born_no_aber"])
def case(request):
    acq, ph, seed = simul.workload("tomo_config_1024")
    over = dict(nb_holo=8) if request.param == "rytov" else dict(nb_holo=8, born=1, c_aber=0)
    acq = replace(acq, **over)
    d = simul.holograms(acq, ph, M=acq.nb_holo, seed=seed)
    d = {k: (v.numpy() if hasattr(v, "numpy") else v) for k, v in d.items()}
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    g = _golden_geometry()
    g.born, g.c_aber = acq.born, acq.c_aber
    return acq, g, cfg, d, spec, fields, pos, dbg


def test_stages_and_volume(case):
    acq, g, cfg, d, spec, fields, pos, dbg = case
    M, F, D = acq.nb_holo, 2 * acq.nxmax, acq.dim_final
    assert (F, D) == (250, 512)
    with Context(g, M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        sp = np.zeros((M, F, F), np.complex64)
        ctx.extract(np.ascontiguousarray(d["holos"]), spectra_out=sp)
        for a in range(M):
            assert rel_l2(sp[a], spec[a]) <= TOL, a
        fo = np.zeros((M, F, F), np.complex64)
        po = np.zeros(2 * M, np.int32)
        ctx.fields(c64(spec), fields_out=fo, posspec_out=po)
        np.testing.assert_array_equal(po, pos.astype(np.int32))
        for a in range(M):
            assert rel_l2(fo[a], fields[a]) <= TOL, a
        if acq.c_aber:
            un = np.zeros((M, F, F), np.float32)
            ctx.fields_debug(c64(spec), unwrapped=un)
            for a in range(M):
                assert rel_l2(un[a], dbg["unwrap"][a]) <= TOL, a
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros_like(re)
        cnt = np.zeros((D, D, D), np.uint32)
        pp = np.zeros(2 * M, np.int32)
        ctx.pipeline(np.ascontiguousarray(d["holos"]), indice=re, absorption=im, counts=cnt, posspec=pp)
    np.testing.assert_array_equal(pp, pos.astype(np.int32))
    ref = oracle.reconstruction(fields, pos, cfg, want_otf=False)
    np.testing.assert_array_equal(cnt, ref["counts"].astype(np.uint32))
    assert rel_l2(re, ref["indice"].real) <= TOL
    assert rel_l2(im, ref["indice"].imag) <= TOL
