"""The oracle pinned on the reference's own code.

oracle/ref/build_ref.py compiles the reference's preprocessing and
reconstruction sources (Tomo_prog/pretraitement_hors_axe_CPU,
Tomo_prog/Reconstruction) against stand-in FFTW/OpenCV/libtiff headers into
oracle/_ref/.  These CPU tests run the reference functions on the same
inputs as the oracle's restatement and compare: window and hit counts bit
for bit, specular positions exactly, everything else at FP64 round-off
(the two builds use different FFT implementations).  The one difference
kept by policy is the Volkov zero frequency: the reference reads one element
past its spectrum there (src/deroulement_volkov4.cpp:189), which adds a
constant piston to the unwrapped phase, so that comparison removes the
piston.  Skipped where the reference's sources were not available to build.
"""
from __future__ import annotations

import numpy as np
import pytest

import oracle
from oracle import reference_build as rb
from tests.helpers import oracle_cfg, planted_ties, rel_l2, small_case

pytestmark = pytest.mark.skipif(not rb.available(), reason="reference build (oracle/_ref) not available")

ROUNDOFF = 1e-12


@pytest.fixture(scope="module")
def born():
    acq, _, d = small_case("plain_512_born", M=4)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    return acq, cfg, d, spec, fields, pos, dbg


@pytest.fixture(scope="module")
def rytov():
    acq, _, d = small_case("rytov_1024", M=4, ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128, dim_final=256)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    return acq, cfg, d, spec, fields, pos, dbg


@pytest.mark.parametrize("n", [64, 128, 250, 256, 500, 512, 1024])
@pytest.mark.parametrize("alpha", [0.05, 0.1])
def test_tukey_window_bit_exact(n, alpha):
    np.testing.assert_array_equal(oracle.tukey2d(n, alpha), rb.tukey2d(n, alpha))


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_extraction(case, request):
    acq, cfg, d, spec, *_ = request.getfixturevalue(case)
    for a in range(len(spec)):
        ref = rb.extract(d["holos"][a].astype(np.float64), acq.nxmax, acq.circle_cx, acq.circle_cy)
        assert rel_l2(spec[a], ref) <= ROUNDOFF, a


def test_extraction_off_centre_crop():
    """A crop window away from the centre, as the reference's own
    configuration places it (CIRCLE_CX 247, CIRCLE_CY 777 on 1024^2)."""
    acq, _, d = small_case("plain_512_born", M=1)
    h = d["holos"][0].astype(np.float64)
    cfg = oracle_cfg(acq)
    cfg.circle_cx, cfg.circle_cy = 100, 380
    assert rel_l2(oracle.extract(h, cfg), rb.extract(h, cfg.nxmax, 100, 380)) <= ROUNDOFF


def test_specular_search(born):
    *_, spec, _, pos, _ = born
    M, F = len(spec), spec.shape[1]
    for a in range(M):
        got = rb.coord_spec(spec[a])
        assert got == oracle.coord_spec(spec[a])
        assert (got % F, got // F) == (int(pos[a]), int(pos[M + a]))
    ties = planted_ties(F, 10, np.random.default_rng(7)).astype(np.complex128)
    assert [rb.coord_spec(s) for s in ties] == [oracle.coord_spec(s) for s in ties]


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_recentred_field_and_phase(case, request):
    acq, cfg, d, spec, fields, pos, dbg = request.getfixturevalue(case)
    M, F = len(spec), spec.shape[1]
    for a in range(M):
        px, py = int(pos[a]), int(pos[M + a])
        f_ref, ph_ref = rb.field(spec[a], px, py)
        assert rel_l2(oracle.calc_uborn2(spec[a], px, py), f_ref) <= ROUNDOFF
        dph = np.angle(np.exp(1j * (dbg["phase"][a] - ph_ref)))
        assert np.abs(dph).max() <= 1e-9, a


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_volkov_unwrap_up_to_the_zero_frequency_piston(case, request):
    *_, dbg = request.getfixturevalue(case)
    for a in range(len(dbg["phase"])):
        ph = dbg["phase"][a]
        diff = oracle.volkov(ph) - rb.volkov(ph)
        assert np.abs(diff - diff.mean()).max() <= 1e-10, a


def _herraez_phase(F, sigma, seed):
    rng = np.random.default_rng(seed)
    y, x = np.mgrid[0:F, 0:F] / F
    true = 25 * np.exp(-((x - .5) ** 2 + (y - .45) ** 2) / 0.04) - 6 * y
    return np.angle(np.exp(1j * (true + rng.normal(0, sigma, (F, F)))))


@pytest.mark.parametrize("F", [64, 250, 256])
@pytest.mark.parametrize("sigma", [0.0, 1.2])
@pytest.mark.parametrize("angle", [0, 3])
def test_herraez_unwrap_bit_exact(F, sigma, angle):
    """phaseUnwrapping_Mat (deroulement_herraez.cpp:32-74): the restatement
    gives the reference's unwrapped phase bit for bit, on smooth phases and on
    noisy ones whose residues make the result depend on the edge order, for
    the first angle of a stack and a later one (the border pixels'
    reliabilities come from rand(), whose earlier draws are skipped)."""
    wrapped = _herraez_phase(F, sigma, seed=F + int(10 * sigma))
    got, inc = oracle.herraez(wrapped, angle)
    np.testing.assert_array_equal(got, rb.herraez(wrapped, angle))
    assert inc.min() < 0 or inc.max() > 0


def test_reconstruction_parameters():
    from tests import simul
    for name in ("plain_512_born", "rytov_1024", "large_2048"):
        acq, _, _ = simul.workload(name)
        cfg = oracle_cfg(acq)
        got = rb.manip(cfg, 7)
        ref = oracle.derive(cfg)
        for k in ("rayon", "tp_holo", "tp_uborn", "delta_f", "tp_tomo"):
            assert got[k] == ref[k], (name, k)
        assert got["dim_final"] == acq.dim_final and got["nxmax"] == acq.nxmax


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_volume_stage(case, request):
    acq, cfg, d, spec, fields, pos, dbg = request.getfixturevalue(case)
    ref = rb.reconstruction(fields, pos, cfg)
    got = oracle.reconstruction(fields, pos, cfg)
    np.testing.assert_array_equal(got["counts"], ref["counts"])
    np.testing.assert_array_equal(got["otf"], ref["otf"])
    assert rel_l2(got["indice"], ref["indice"]) <= ROUNDOFF


def test_shipped_geometry():
    """The reference's own configuration (Tomo_config: CCD_ROIX 1024, NXMAX 125,
    CIRCLE_CX 247, CIRCLE_CY 777, DIM_FINAL 512): 250^2 fields and a 500^2
    Volkov mirror, through extraction, specular search, recentring and
    unwrapping."""
    acq, _, d = small_case("plain_512_born", M=1, ccd_roix=1024, nxmax=125, circle_cx=247, circle_cy=777,
                           dim_final=512)
    cfg = oracle_cfg(acq)
    h = d["holos"][0].astype(np.float64)
    spec = oracle.extract(h, cfg)
    assert rel_l2(spec, rb.extract(h, 125, 247, 777)) <= ROUNDOFF
    c = oracle.coord_spec(spec)
    assert c == rb.coord_spec(spec)
    F = 250
    f_ref, ph = rb.field(spec, c % F, c // F)
    assert rel_l2(oracle.calc_uborn2(spec, c % F, c // F), f_ref) <= ROUNDOFF
    diff = oracle.volkov(ph) - rb.volkov(ph)
    assert np.abs(diff - diff.mean()).max() <= 1e-10
