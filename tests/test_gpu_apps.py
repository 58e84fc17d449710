"""The drop-in executables on the reference's file contract, checked against
the oracle: tomo_pretraitement -> tomo_reconstruction, and tomo_pipeline."""
from __future__ import annotations

import os
import subprocess
from dataclasses import replace

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import build as tdm_build
from tests import simul
from tests.helpers import oracle_cfg, rel_l2, small_case
from tests.test_host_io import _read_hdf5, _read_tiff, _write_pgm

pytestmark = pytest.mark.gpu
BIN = tdm_build.BIN


@pytest.fixture(scope="module")
def acquisition(tmp_path_factory):
    root = tmp_path_factory.mktemp("tomo")
    home, cfgd, acq_d, res_d = root / "home", root / "config", root / "acquis", root / "result"
    for d in (home / ".config", cfgd, acq_d, res_d):
        d.mkdir(parents=True)
    acq, ph, d = small_case("plain_512_born", M=7, ccd_roix=256, nxmax=32, circle_cx=64, circle_cy=64,
                            dim_final=128)
    (home / ".config" / "gui_tomo.conf").write_text(
        f"CHEMIN_RESULT {res_d}\nCHEMIN_ACQUIS {acq_d}\nCHEMIN_CONFIG {cfgd}\n")
    (cfgd / "recon.txt").write_text(acq.recon_txt())
    (cfgd / "config_manip.txt").write_text(acq.config_manip_txt())
    kept = [a for a in range(7) if a != 3]          # i003.pgm is missing: skipped and compacted
    for a in kept:
        _write_pgm(acq_d / f"i{a:03d}.pgm", d["holos"][a], 4095)
    _write_pgm(acq_d / "Image_mask.pgm", d["mask"], 255)
    env = dict(os.environ, HOME=str(home))
    holos = d["holos"][kept]
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(holos.astype(np.float64), cfg)
    fields, pos = oracle.fields(spec, cfg, d["mask"])
    ref = oracle.reconstruction(fields, pos, cfg)
    return dict(acq=acq, env=env, res=res_d, fields=fields, pos=pos, ref=ref, M=len(kept))


def _run(exe, env, *args):
    r = subprocess.run([os.path.join(BIN, exe), *args], env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stdout + r.stderr
    return r.stdout


def test_pretraitement_files(acquisition):
    A = acquisition
    out = _run("tomo_pretraitement", A["env"])
    assert "fichier 3 inexistant" in out
    M, F = A["M"], 2 * A["acq"].nxmax
    dim = f"{F}x{F}x{M}"
    re = np.fromfile(A["res"] / f"UBornfinal_Re{dim}.raw", "<f8").reshape(M, F, F)
    im = np.fromfile(A["res"] / f"UBornfinal_Im{dim}.raw", "<f8").reshape(M, F, F)
    for a in range(M):
        assert rel_l2(re[a] + 1j * im[a], A["fields"][a]) <= 1e-4
    np.testing.assert_array_equal(np.fromfile(A["res"] / "tab_posSpec.raw", "<f8"), A["pos"])
    par = np.fromfile(A["res"] / "parametres.raw", "<f8")
    d = oracle.derive(oracle_cfg(A["acq"]))
    np.testing.assert_array_equal(par, [A["acq"].nxmax, M, d["rayon"], A["acq"].ccd_roix, d["tp_holo"]])


def test_reconstruction_files(acquisition):
    A = acquisition
    _run("tomo_reconstruction", A["env"])
    D = A["acq"].dim_final
    ind = np.stack([p[1] for p in _read_tiff(A["res"] / "indice.tif")])
    ab = np.stack([p[1] for p in _read_tiff(A["res"] / "absorption.tif")])
    otf = np.stack([p[1] for p in _read_tiff(A["res"] / "OTF3D.tif")])
    assert ind.shape == (D, D, D)
    assert rel_l2(ind, A["ref"]["indice"].real) <= 1e-4
    assert rel_l2(ab, A["ref"]["indice"].imag) <= 1e-4
    np.testing.assert_array_equal(otf, A["ref"]["otf"].astype(np.float32))


def test_pipeline_matches_two_programs(acquisition):
    A = acquisition
    res = A["res"]
    two = np.stack([p[1] for p in _read_tiff(res / "indice.tif")])
    _run("tomo_pipeline", A["env"])
    one = np.stack([p[1] for p in _read_tiff(res / "indice.tif")])
    assert rel_l2(one, A["ref"]["indice"].real) <= 1e-4
    assert rel_l2(one, two) <= 1e-5


STATES = ("/LC/polar0/", "/LC/polar90/", "/RC/polar0/", "/RC/polar90/")


@pytest.fixture(scope="module")
def polarisation(tmp_path_factory):
    """A polarisation acquisition: four states of uneven size under
    CHEMIN_RACINE/demosaic<state>, the mask at CHEMIN_RACINE/Image_mask.pgm,
    $HOME/.config/gui_tomo_polar.conf (pretraitement_hors_axe_CPU/main.cpp:63-80)."""
    root = tmp_path_factory.mktemp("polar")
    home, cfgd, racine = root / "home", root / "config", root / "racine"
    for d in (home / ".config", cfgd, racine):
        d.mkdir(parents=True)
    (home / ".config" / "gui_tomo_polar.conf").write_text(
        f"CHEMIN_CONFIG {cfgd}\nCHEMIN_RACINE {racine}\nCHEMIN_RESULT {root}\nCHEMIN_ACQUIS {root}\n")
    acq, ph, _ = small_case("plain_512_born", M=1, ccd_roix=256, nxmax=32, circle_cx=64, circle_cy=64,
                            dim_final=128)
    sizes = (5, 7, 4, 6)
    acq = replace(acq, nb_holo=max(sizes))
    (cfgd / "recon.txt").write_text(acq.recon_txt())
    (cfgd / "config_manip.txt").write_text(acq.config_manip_txt())
    cfg = oracle_cfg(acq)
    refs, mask = {}, None
    for k, (state, M) in enumerate(zip(STATES, sizes)):
        d = simul.holograms(replace(acq, nb_holo=M), ph, M=M, seed=20 + k)
        holos = d["holos"].numpy()
        mask = d["mask"].numpy() if mask is None else mask
        sd = racine / "demosaic" / state.strip("/")
        (sd / "UBorn").mkdir(parents=True)
        for a in range(M):
            _write_pgm(sd / f"i{a:03d}.pgm", holos[a], 4095)
        # tomo_reconstruction -polar reads its configuration in the state's UBorn folder
        (sd / "UBorn" / "recon.txt").write_text(acq.recon_txt())
        (sd / "UBorn" / "config_manip.txt").write_text(acq.config_manip_txt())
        spec = oracle.extract_stack(holos.astype(np.float64), cfg)
        fields, pos = oracle.fields(spec, cfg, mask)
        refs[state] = (sd / "UBorn", oracle.reconstruction(fields, pos, cfg, want_otf=False, want_counts=False))
    _write_pgm(racine / "Image_mask.pgm", mask, 255)
    return dict(env=dict(os.environ, HOME=str(home)), refs=refs)


def test_polarisation_one_state(polarisation):
    """tomo_pretraitement -polar -etat S then tomo_reconstruction -polar -etat S:
    the state's volume in its UBorn folder as HDF5 (/indice_complexe/Re, Im)."""
    A = polarisation
    state = STATES[1]
    _run("tomo_pretraitement", A["env"], "-polar", "-etat", state)
    _run("tomo_reconstruction", A["env"], "-polar", "-etat", state)
    res, ref = A["refs"][state]
    vol = _read_hdf5(res / "indice_cplx_hdf5.hdf")["indice_complexe"]
    assert rel_l2(vol["Re"], ref["indice"].real) <= 1e-4
    assert rel_l2(vol["Im"], ref["indice"].imag) <= 1e-4


def test_polarisation_four_states_in_one_graph(polarisation):
    """tomo_pipeline -polar: the four states of uneven size as one CUDA-graph
    launch, each state's volume against the oracle."""
    A = polarisation
    for state in STATES:
        f = A["refs"][state][0] / "indice_cplx_hdf5.hdf"
        if f.exists():
            f.unlink()
    out = _run("tomo_pipeline", A["env"], "-polar")
    for state in STATES:
        assert state in out
        res, ref = A["refs"][state]
        vol = _read_hdf5(res / "indice_cplx_hdf5.hdf")["indice_complexe"]
        assert rel_l2(vol["Re"], ref["indice"].real) <= 1e-4, state
        assert rel_l2(vol["Im"], ref["indice"].imag) <= 1e-4, state
