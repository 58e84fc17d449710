"""bench.py's byte accounting for the stage rooflines (no GPU).

The per-unit figures are the path's algorithmic bytes per stage: extraction
H^2 2 + F^2 8 per hologram, fields 2 F^2 8 per angle, cap mapping
F^2 8 + hits (8 + 4) 2 per angle, volume 32 D^3 per volume.
"""
from __future__ import annotations

import numpy as np
import pytest

import bench
from tests import simul


def _hits(nxmax):
    a = np.arange(-nxmax, nxmax)
    return int((a[:, None] ** 2 + a[None, :] ** 2 < nxmax ** 2).sum())


@pytest.mark.parametrize("name,per_holo,per_field,per_cap,hits,volume,total", [
    ("plain_512_born", 655_360, 262_144, 439_448, 12_849, 536_870_912, 0.673e9),
    ("rytov_1024", 2_621_440, 1_048_576, 1_758_584, 51_429, 4_294_967_296, 7.552e9),
    ("large_2048", 10_485_760, 4_194_304, 7_037_720, 205_857, 34_359_738_368, 56.08e9),
])
def test_stage_bytes(name, per_holo, per_field, per_cap, hits, volume, total):
    acq, _, _ = simul.workload(name)
    assert _hits(acq.nxmax) == hits
    b = bench.stage_bytes(acq, hits)
    M = acq.nb_holo
    assert b["extraction"] == M * per_holo
    assert b["fields"] == M * per_field
    assert b["cap_mapping"] == M * per_cap
    assert b["volume"] == volume
    assert abs(sum(b.values()) - total) / total < 1e-3


def test_stage_roofline_arithmetic():
    acq, _, _ = simul.workload("rytov_1024")
    hits = _hits(acq.nxmax)
    kern = {"extract_rows": 1.0, "extract_cols": 0.5, "field_rows": 0.25, "volkov_cols": 0.75,
            "cap_rows": 0.5, "cap_cols": 0.5, "gather": 0.75, "ypass": 0.5, "xpass": 0.5}
    r = bench.stage_roofline(acq, hits, kern, 5.0, 6787.6)
    b = bench.stage_bytes(acq, hits)
    for st, t in (("extraction", 1.5), ("fields", 1.0), ("cap_mapping", 1.0), ("volume", 1.75)):
        assert r[st]["ms_per_step"] == t
        assert r[st]["achieved_gbs"] == pytest.approx(b[st] / (t * 1e-3) / 1e9, abs=0.05)
        assert r[st]["frac"] == pytest.approx(r[st]["achieved_gbs"] / 6787.6, abs=1e-4)
    assert r["whole_path_live"]["bytes_per_step"] == int(sum(b.values()))
    assert r["whole_path_live"]["achieved_gbs"] == pytest.approx(sum(b.values()) / 5e-3 / 1e9, abs=0.05)
    # stages without timed kernels are left out
    assert "fields" not in bench.stage_roofline(acq, hits, {"extract_rows": 1.0}, 5.0, 6787.6)
