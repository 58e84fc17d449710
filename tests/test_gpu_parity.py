"""GPU parity against the FP64 oracle, stage by stage and end to end.

Bars: bit-exact specular positions, hit counts and OTF masks; rel-L2 <= 1e-4
on spectra, fields and volumes (FP32 FFTs vs the FP64 oracle).
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import Context, Geometry, TdmError
from tests.helpers import c64, oracle_cfg, rel_l2, small_case

pytestmark = pytest.mark.gpu
TOL = 1e-4


def _wrap(d):
    return np.angle(np.exp(1j * d))


@pytest.fixture(scope="module")
def born():
    acq, ph, d = small_case("plain_512_born", M=8)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    return acq, cfg, d, spec, fields, pos, dbg


@pytest.fixture(scope="module")
def rytov():
    acq, ph, d = small_case("rytov_1024", M=8, ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128,
                            dim_final=256)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos, dbg = oracle.fields(spec, cfg, d["mask"], debug=True)
    return acq, cfg, d, spec, fields, pos, dbg


def test_extract_parity(born):
    acq, cfg, d, spec, *_ = born
    F = 2 * acq.nxmax
    with Context(Geometry.from_acquisition(acq), 8) as ctx:
        out = np.zeros((8, F, F), np.complex64)
        ctx.extract(np.ascontiguousarray(d["holos"]), spectra_out=out)
    for a in range(8):
        assert rel_l2(out[a], spec[a]) <= TOL, a


def test_extract_8bit():
    acq, ph, d = small_case("plain_512_born", M=3)
    h8 = np.ascontiguousarray((d["holos"] >> 4).astype(np.uint8))
    cfg = oracle_cfg(acq)
    ref = oracle.extract_stack(h8.astype(np.float64), cfg)
    F = 2 * acq.nxmax
    with Context(Geometry.from_acquisition(acq), 3) as ctx:
        out = np.zeros((3, F, F), np.complex64)
        ctx.extract(h8, spectra_out=out)
    for a in range(3):
        assert rel_l2(out[a], ref[a]) <= TOL


@pytest.mark.parametrize("roix,nxmax", [(256, 128), (512, 128), (1024, 256)])
def test_extract_wide_band(roix, nxmax):
    """Crops wider than one round of the row pass's output tile (64 band
    columns per round for 256- and 512-pixel holograms, 128 above): the
    context path against the oracle, and the allocation-free entry point
    bit for bit against the context path."""
    import torch
    from mtd_transmission_gb300 import api
    acq, ph, d = small_case("plain_512_born", M=2, ccd_roix=roix, nxmax=nxmax, circle_cx=roix // 2,
                            circle_cy=roix // 2, dim_final=max(4 * nxmax, 128))
    ref = oracle.extract_stack(d["holos"].astype(np.float64), oracle_cfg(acq))
    F = 2 * acq.nxmax
    holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
    out = torch.zeros((2, F, F), dtype=torch.complex64, device="cuda")
    with Context(Geometry.from_acquisition(acq), 2) as ctx:
        ctx.extract(holos, spectra_out=out)
        ctx.synchronize()
    na = torch.full((2, F, F), complex("nan"), dtype=torch.complex64, device="cuda")
    assert api.extract_noalloc(Geometry.from_acquisition(acq), holos, na, torch.cuda.current_stream().cuda_stream) == 0
    torch.cuda.synchronize()
    assert torch.equal(na, out)
    o = out.cpu().numpy()
    for a in range(2):
        assert rel_l2(o[a], ref[a]) <= TOL, a


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_fields_parity(case, request):
    acq, cfg, d, spec, fields, pos, dbg = request.getfixturevalue(case)
    F, M = 2 * acq.nxmax, spec.shape[0]
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        fo = np.zeros((M, F, F), np.complex64)
        po = np.zeros(2 * M, np.int32)
        ph = np.zeros((M, F, F), np.float32)
        un = np.zeros((M, F, F), np.float32)
        am = np.zeros((M, F, F), np.float32)
        ctx.fields_debug(c64(spec), fields_out=fo, posspec_out=po, phase=ph, unwrapped=un, amp=am)
    np.testing.assert_array_equal(po, pos.astype(np.int32))
    for a in range(M):
        assert rel_l2(am[a], dbg["amp"][a]) <= TOL, ("amp", a)
        big = dbg["amp"][a] > 1e-3 * dbg["amp"][a].max()
        assert np.abs(_wrap(ph[a] - dbg["phase"][a]))[big].max() < 1e-3, ("phase", a)
        assert rel_l2(un[a], dbg["unwrap"][a]) <= TOL, ("unwrap", a)
        assert rel_l2(fo[a], fields[a]) <= TOL, ("field", a)


@pytest.mark.parametrize("over", [dict(c_aber=0), dict(deroul=0)])
def test_fields_options(over):
    acq, ph, d = small_case("plain_512_born", M=4, **over)
    cfg = oracle_cfg(acq)
    spec = oracle.extract_stack(d["holos"].astype(np.float64), cfg)
    fields, pos = oracle.fields(spec, cfg, d["mask"])
    F = 2 * acq.nxmax
    with Context(Geometry.from_acquisition(acq), 4) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        fo = np.zeros((4, F, F), np.complex64)
        po = np.zeros(8, np.int32)
        ctx.fields(c64(spec), fields_out=fo, posspec_out=po)
    np.testing.assert_array_equal(po, pos.astype(np.int32))
    for a in range(4):
        assert rel_l2(fo[a], fields[a]) <= TOL, a


@pytest.mark.parametrize("case", ["born", "rytov"])
def test_reconstruct_parity(case, request):
    acq, cfg, d, spec, fields, pos, dbg = request.getfixturevalue(case)
    D, M = acq.dim_final, spec.shape[0]
    ref = oracle.reconstruction(fields, pos, cfg)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros((D, D, D), np.float32)
        otf = np.zeros((D, D, D), np.uint8)
        cnt = np.zeros((D, D, D), np.uint32)
        ctx.reconstruct(c64(fields), pos.astype(np.int32), indice=re, absorption=im, otf=otf, counts=cnt)
    np.testing.assert_array_equal(cnt, ref["counts"].astype(np.uint32))
    np.testing.assert_array_equal(otf, ref["otf"].astype(np.uint8))
    assert rel_l2(re, ref["indice"].real) <= TOL
    assert rel_l2(im, ref["indice"].imag) <= TOL


def test_pipeline_end_to_end(born):
    acq, cfg, d, spec, fields, pos, dbg = born
    D, M = acq.dim_final, spec.shape[0]
    ref = oracle.reconstruction(fields, pos, cfg)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros((D, D, D), np.float32)
        cnt = np.zeros((D, D, D), np.uint32)
        po = np.zeros(2 * M, np.int32)
        ctx.pipeline(np.ascontiguousarray(d["holos"]), indice=re, absorption=im, counts=cnt, posspec=po)
        assert ctx.launch_count > 0
    np.testing.assert_array_equal(po, pos.astype(np.int32))
    np.testing.assert_array_equal(cnt, ref["counts"].astype(np.uint32))
    assert rel_l2(re, ref["indice"].real) <= TOL
    assert rel_l2(im, ref["indice"].imag) <= TOL


def test_pipeline_async_sequence(born):
    """tdm_pipeline_async: three volumes queued back to back with pinned host
    buffers (uploads, kernels and downloads of consecutive calls overlap) give
    the synchronous pipeline's outputs once tdm_synchronize returns."""
    import torch
    acq, cfg, d, spec, fields, pos, dbg = born
    D, M = acq.dim_final, spec.shape[0]
    holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).pin_memory()
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        re0 = np.zeros((D, D, D), np.float32)
        im0 = np.zeros((D, D, D), np.float32)
        otf0 = np.zeros((D, D, D), np.uint8)
        ctx.pipeline(holos, indice=re0, absorption=im0, otf=otf0)
        outs = [(torch.full((D, D, D), float("nan")).pin_memory(), torch.full((D, D, D), float("nan")).pin_memory(),
                 torch.zeros((D, D, D), dtype=torch.uint8).pin_memory()) for _ in range(3)]
        for re, im, otf in outs:
            ctx.pipeline_async(holos, indice=re, absorption=im, otf=otf)
        ctx.synchronize()
    for re, im, otf in outs:
        np.testing.assert_array_equal(re.numpy(), re0)
        np.testing.assert_array_equal(im.numpy(), im0)
        np.testing.assert_array_equal(otf.numpy(), otf0)


def test_reconstruct_edge_positions():
    """Specular positions at the crop edges and corners (corner angles fall
    outside the Ewald sphere and are skipped by the reference)."""
    acq, ph, d = small_case("plain_512_born", M=1)
    N, F, D = acq.nxmax, 2 * acq.nxmax, acq.dim_final
    rng = np.random.default_rng(5)
    pos_xy = [(0, 0), (F - 1, F - 1), (0, N), (N, F - 1), (N, N), (F - 1, 0), (N + 10, N - 33)]
    M = len(pos_xy)
    f = (rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))) * 0.1
    pos = np.array([p[0] for p in pos_xy] + [p[1] for p in pos_xy], np.float64)
    cfg = oracle_cfg(acq)
    ref = oracle.reconstruction(f, pos, cfg)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        re = np.zeros((D, D, D), np.float32)
        im = np.zeros((D, D, D), np.float32)
        cnt = np.zeros((D, D, D), np.uint32)
        ctx.reconstruct(c64(f), pos.astype(np.int32), indice=re, absorption=im, counts=cnt)
    np.testing.assert_array_equal(cnt, ref["counts"].astype(np.uint32))
    assert rel_l2(re, ref["indice"].real) <= TOL
    assert rel_l2(im, ref["indice"].imag) <= TOL


def test_single_angle_counts():
    """One angle: every in-disc cap pixel is hit exactly once."""
    acq, ph, d = small_case("plain_512_born", M=1)
    N, F, D = acq.nxmax, 2 * acq.nxmax, acq.dim_final
    f = np.ones((1, F, F), np.complex64)
    with Context(Geometry.from_acquisition(acq), 1) as ctx:
        cnt = np.zeros((D, D, D), np.uint32)
        ctx.reconstruct(f, np.array([N + 3, N - 5], np.int32), counts=cnt)
    fd = np.arange(-N, N)
    disc = (fd[:, None] ** 2 + fd[None, :] ** 2) < N * N
    assert cnt.sum() == disc.sum() and cnt.max() == 1


def test_device_buffers_match_host():
    """Device (torch CUDA) inputs and outputs give the same volume as host buffers."""
    import torch
    acq, ph, d = small_case("plain_512_born", M=4)
    D = acq.dim_final
    with Context(Geometry.from_acquisition(acq), 4) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        re_h = np.zeros((D, D, D), np.float32)
        ctx.pipeline(np.ascontiguousarray(d["holos"]), indice=re_h)
        h_dev = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
        re_d = torch.zeros((D, D, D), dtype=torch.float32, device="cuda")
        ctx.pipeline(h_dev, indice=re_d)
        ctx.synchronize()
    np.testing.assert_array_equal(re_d.cpu().numpy(), re_h)


def test_invalid_geometry():
    acq, ph, d = small_case("plain_512_born", M=1)
    for over in (dict(dim_final=128), dict(nxmax=60), dict(circle_cx=10), dict(ccd_roix=500)):
        with pytest.raises(TdmError):
            Context(Geometry.from_acquisition(replace(acq, **over)), 1)


def test_mask_without_background():
    acq, ph, d = small_case("plain_512_born", M=1)
    F = 2 * acq.nxmax
    with Context(Geometry.from_acquisition(acq), 1) as ctx:
        with pytest.raises(TdmError):
            ctx.set_mask(np.zeros((F, F), np.uint8))


def test_batch_graph_matches_one_by_one():
    """Three stacks of different geometries in one CUDA-graph launch
    (tdm_batch) give, bit for bit, the volumes of one tdm_pipeline call each."""
    import torch
    from mtd_transmission_gb300 import Batch
    cases = [small_case("plain_512_born", M=5),
             small_case("rytov_1024", M=4, ccd_roix=512, nxmax=64, circle_cx=128, circle_cy=128, dim_final=256),
             small_case("plain_512_born", M=3, ccd_roix=256, nxmax=32, circle_cx=64, circle_cy=64, dim_final=128)]
    ctxs, stacks, refs = [], [], []
    try:
        for acq, _, d in cases:
            D, M = acq.dim_final, acq.nb_holo
            ctx = Context(Geometry.from_acquisition(acq), M)
            ctxs.append(ctx)
            ctx.set_mask(np.ascontiguousarray(d["mask"]))
            holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
            re = torch.zeros((D, D, D), device="cuda")
            im = torch.zeros_like(re)
            otf = torch.zeros((D, D, D), dtype=torch.uint8, device="cuda")
            ctx.pipeline(holos, indice=re, absorption=im, otf=otf)
            ctx.synchronize()
            refs.append((re.clone(), im.clone(), otf.clone()))
            re.zero_()
            im.zero_()
            otf.zero_()
            stacks.append((ctx, holos, re, im, otf))
        with Batch(stacks) as b:
            for _ in range(2):  # replays reuse the bound buffers
                b.launch(torch.cuda.current_stream().cuda_stream)
            torch.cuda.synchronize()
        for (ctx, holos, re, im, otf), (r0, i0, o0) in zip(stacks, refs):
            assert torch.equal(re, r0) and torch.equal(im, i0) and torch.equal(otf, o0)
    finally:
        for ctx in ctxs:
            ctx.close()


def test_autotune_keeps_results():
    """tdm_autotune picks a schedule (8, 12, 16 or 32 angles per chunk); the volume does not
    depend on the chunking (every per-angle kernel sees only its own angle)."""
    import torch
    acq, _, d = small_case("plain_512_born", M=40)
    D = acq.dim_final
    holos = torch.from_numpy(np.ascontiguousarray(d["holos"])).cuda()
    with Context(Geometry.from_acquisition(acq), 40) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        re0 = torch.zeros((D, D, D), device="cuda")
        im0 = torch.zeros_like(re0)
        ctx.pipeline(holos, indice=re0, absorption=im0)
        chunk = ctx.autotune(holos)
        assert chunk in (8, 12, 16, 32)
        re = torch.zeros_like(re0)
        im = torch.zeros_like(re0)
        ctx.pipeline(holos, indice=re, absorption=im)
        ctx.synchronize()
        assert torch.equal(re, re0) and torch.equal(im, im0), chunk


def test_schedules_keep_results():
    """Every schedule (angles per chunk x chunks in flight, each chunk on its
    own stream and scratch slots) gives the same volume bit for bit, from
    device holograms and from host holograms (uploaded several chunks per
    copy into the staging ring, the last group partial), 16-bit and 8-bit;
    schedules beyond the buffers' capacity are refused."""
    import torch
    from mtd_transmission_gb300.api import TdmError
    acq, _, d = small_case("plain_512_born", M=40)
    D = acq.dim_final
    stacks = []
    for h in (np.ascontiguousarray(d["holos"]), np.ascontiguousarray((d["holos"] >> 4).astype(np.uint8))):
        h_holos = torch.from_numpy(h).pin_memory()
        stacks.append((h_holos.cuda(), h_holos))
    with Context(Geometry.from_acquisition(acq), 40) as ctx:
        ctx.set_mask(np.ascontiguousarray(d["mask"]))
        for holos, h_holos in stacks:
            ctx.set_schedule(16, 1)
            re0 = torch.zeros((D, D, D), device="cuda")
            im0 = torch.zeros_like(re0)
            ctx.pipeline(holos, indice=re0, absorption=im0)
            ctx.synchronize()
            for chunk, lanes in ((4, 4), (8, 3), (8, 4), (16, 2), (32, 1), (5, 2), (3, 2)):
                ctx.set_schedule(chunk, lanes)
                for src in (holos, h_holos):
                    re = torch.zeros_like(re0)
                    im = torch.zeros_like(re0)
                    ctx.pipeline(src, indice=re, absorption=im)
                    ctx.synchronize()
                    assert torch.equal(re, re0) and torch.equal(im, im0), (chunk, lanes, src.is_cuda, src.dtype)
        for chunk, lanes in ((64, 3), (8, 9), (0, 1), (129, 1)):
            with pytest.raises(TdmError):
                ctx.set_schedule(chunk, lanes)


def test_reference_intensity():
    """tdm_set_reference_intensity divides every pixel by sqrt(I_ref) (1 where
    I_ref is 0) before the extraction, as initRef and main.cpp:147 of the
    reference; clearing it gives the plain extraction back bit for bit, and a
    negative intensity is refused."""
    acq, ph, d = small_case("plain_512_born", M=3)
    H, F = acq.ccd_roix, 2 * acq.nxmax
    rng = np.random.default_rng(5)
    iref = rng.uniform(500.0, 3000.0, (H, H)).astype(np.float32)
    iref[rng.random((H, H)) < 0.01] = 0.0
    cfg = oracle_cfg(acq)
    ref = oracle.extract_stack(d["holos"].astype(np.float64), cfg, ref_intensity=iref)
    holos = np.ascontiguousarray(d["holos"])
    with Context(Geometry.from_acquisition(acq), 3) as ctx:
        plain = np.zeros((3, F, F), np.complex64)
        ctx.extract(holos, spectra_out=plain)
        ctx.set_reference_intensity(iref)
        out = np.zeros_like(plain)
        ctx.extract(holos, spectra_out=out)
        for a in range(3):
            assert rel_l2(out[a], ref[a]) <= TOL, a
        ctx.set_reference_intensity(None)
        again = np.zeros_like(plain)
        ctx.extract(holos, spectra_out=again)
        assert np.array_equal(again, plain)
        with pytest.raises(TdmError):
            ctx.set_reference_intensity(-iref)


def test_too_many_angles_refused():
    """Hit counts are gathered in 16 bits per voxel: more than 65535 angles is refused at creation."""
    acq, ph, d = small_case("plain_512_born", M=1)
    with pytest.raises(TdmError):
        Context(Geometry.from_acquisition(acq), 65536)
