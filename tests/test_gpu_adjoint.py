"""Forward cap operator, its adjoint and the regularised reconstruction.

The forward operator samples G(x) = M_in FFT3(M_out x) / (s D^3) (the exact
inverse of the reconstruction's volume stage) at every angle's Ewald-cap
cells; the adjoint is the unnormalised scatter followed by G^H.  Checked
against the FP64 oracle restatement, by the dot-product test, by central
finite differences (eps = 1e-3 on 32 random voxels), through the
torch.autograd binding, and by the TV-regularised reconstruction of a
missing-cone phantom against the single-pass reconstruction.
"""
from __future__ import annotations

from dataclasses import replace

import numpy as np
import pytest

import oracle
from mtd_transmission_gb300 import Context, Geometry
from tests import simul
from tests.helpers import oracle_cfg, rel_l2

pytestmark = pytest.mark.gpu
TOL = 1e-5


def geometry(M=12, seed=3):
    """256^2 holograms, 64^2 fields (NXMAX 32), 128^3 volume; M specular positions inside the NA disc."""
    acq, _, _ = simul.workload("plain_512_born")
    acq = replace(acq, ccd_roix=256, nxmax=32, circle_cx=64, circle_cy=64, dim_final=128, nb_holo=M)
    rng = np.random.default_rng(seed)
    N = acq.nxmax
    r = 0.7 * N * np.sqrt(rng.uniform(0, 1, M))
    t = rng.uniform(0, 2 * np.pi, M)
    pos = np.concatenate([np.round(N + r * np.cos(t)), np.round(N + r * np.sin(t))]).astype(np.int32)
    return acq, pos


def phantom(D, dn=0.03):
    """Two touching spherical cells of index step dn."""
    z, y, x = np.meshgrid(*(np.arange(D) - D / 2,) * 3, indexing="ij")
    v = np.zeros((D, D, D), np.float32)
    for cx in (-0.12 * D, 0.12 * D):
        v[(x - cx) ** 2 + y ** 2 + (z / 0.8) ** 2 < (0.12 * D) ** 2] = dn
    return v


def caps_np(c):
    return c[..., 0] + 1j * c[..., 1]


def test_forward_and_adjoint_match_oracle():
    acq, pos = geometry()
    cfg = oracle_cfg(acq)
    D, F, M = acq.dim_final, 2 * acq.nxmax, acq.nb_holo
    rng = np.random.default_rng(1)
    xn = rng.standard_normal((D, D, D)).astype(np.float32)
    xk = rng.standard_normal((D, D, D)).astype(np.float32)
    y = (rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))).astype(np.complex64)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        caps = ctx.forward(xn, xk, n=M, posspec=pos)
        an, ak = ctx.adjoint(y, n=M, posspec=pos, absorption_out=np.zeros((D, D, D), np.float32))
    ref_f = oracle.forward_caps(xn.astype(np.float64), xk.astype(np.float64), pos.astype(np.float64), cfg)
    ref_a = oracle.adjoint_caps(y.astype(np.complex128), pos.astype(np.float64), cfg)
    assert np.array_equal(caps != 0, ref_f != 0)  # same cap cells
    assert rel_l2(caps, ref_f) <= TOL
    assert rel_l2(an, ref_a.real) <= TOL
    assert rel_l2(ak, ref_a.imag) <= TOL


def test_dot_product():
    acq, pos = geometry(M=16, seed=7)
    D, F, M = acq.dim_final, 2 * acq.nxmax, acq.nb_holo
    rng = np.random.default_rng(2)
    xn = rng.standard_normal((D, D, D)).astype(np.float32)
    xk = rng.standard_normal((D, D, D)).astype(np.float32)
    y = (rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))).astype(np.complex64)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        ax = ctx.forward(xn, xk, n=M, posspec=pos).astype(np.complex128)
        an, ak = ctx.adjoint(y, n=M, posspec=pos, absorption_out=np.zeros((D, D, D), np.float32))
    lhs = np.vdot(y.astype(np.complex128), ax)                       # <y, A x>
    rhs = np.vdot((an + 1j * ak).astype(np.complex128), xn + 1j * xk.astype(np.float64))  # <A^H y, x>
    assert abs(lhs - rhs) / abs(lhs) <= TOL


def test_finite_differences_32_voxels():
    """f(x) = 1/2 |A x - y|^2: central differences with eps = 1e-3 at 32
    voxels against the gradient A^H (A x - y) from the adjoint."""
    acq, pos = geometry(M=12, seed=11)
    D, M = acq.dim_final, acq.nb_holo
    rng = np.random.default_rng(4)
    x0 = np.zeros((D, D, D), np.float32)   # sparse iterate: the FP32 forward stays exact at the eps scale
    idx = rng.integers(0, D, (64, 3))
    x0[idx[:, 0], idx[:, 1], idx[:, 2]] = 0.02 * rng.standard_normal(64)
    xt = np.zeros_like(x0)
    idt = rng.integers(0, D, (64, 3))
    xt[idt[:, 0], idt[:, 1], idt[:, 2]] = 0.02 * rng.standard_normal(64)
    eps = 1e-3
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        y = ctx.forward(xt, None, n=M, posspec=pos).astype(np.complex128)

        def f(x):
            r = ctx.forward(x, None, n=M, posspec=pos).astype(np.complex128) - y
            return 0.5 * float(np.vdot(r, r).real)

        r0 = (ctx.forward(x0, None, n=M, posspec=pos).astype(np.complex128) - y).astype(np.complex64)
        g, _ = ctx.adjoint(r0, n=M, posspec=pos)
        vox = rng.integers(0, D, (32, 3))
        fd, an = [], []
        for v in vox:
            xp = x0.copy()
            xm = x0.copy()
            xp[tuple(v)] += eps
            xm[tuple(v)] -= eps
            fd.append((f(xp) - f(xm)) / (2 * eps))
            an.append(float(g[tuple(v)]))
    fd, an = np.array(fd), np.array(an)
    assert np.abs(fd - an).max() <= 1e-3 * np.abs(an).max()


def test_autograd_binding():
    torch = pytest.importorskip("torch")
    from mtd_transmission_gb300.autograd import cap_forward
    acq, pos = geometry(M=8, seed=5)
    D, F, M = acq.dim_final, 2 * acq.nxmax, acq.nb_holo
    rng = np.random.default_rng(6)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        p = torch.from_numpy(pos).cuda()
        x = torch.from_numpy(rng.standard_normal((D, D, D)).astype(np.float32)).cuda().requires_grad_(True)
        k = torch.from_numpy(rng.standard_normal((D, D, D)).astype(np.float32)).cuda().requires_grad_(True)
        y = torch.from_numpy(rng.standard_normal((M, F, F, 2)).astype(np.float32)).cuda()
        loss = 0.5 * ((cap_forward(x, k, ctx, M, p) - y) ** 2).sum()
        loss.backward()
        r = (cap_forward(x.detach(), k.detach(), ctx, M, p) - y).contiguous()
        gn = torch.empty_like(x)
        gk = torch.empty_like(k)
        ctx.adjoint(r, n=M, posspec=p, index_out=gn, absorption_out=gk)
        ctx.synchronize()
        assert rel_l2(x.grad.cpu().numpy(), gn.cpu().numpy()) <= 1e-6
        assert rel_l2(k.grad.cpu().numpy(), gk.cpu().numpy()) <= 1e-6


def test_tv_reconstruction_beats_single_pass_and_resumes():
    """Missing-cone phantom: the TV-regularised reconstruction with positivity
    is closer to the phantom than the single-pass reconstruction from the same
    cap values, stays inside its box, and a run split in two halves (the
    first half's iterate saved and passed back) equals one run."""
    acq, pos = geometry(M=24, seed=9)
    D, M = acq.dim_final, acq.nb_holo
    truth = phantom(D)
    opts = dict(step=1.0, tv_weight=2e-3, tv_eps=1e-3, index_min=0.0, index_max=0.05)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        caps = ctx.forward(truth, None, n=M, posspec=pos)
        born = np.zeros((D, D, D), np.float32)
        ctx.tv_reconstruct(born, caps=caps, n=M, posspec=pos, iterations=0, init=1)
        full = np.zeros_like(born)
        rep = ctx.tv_reconstruct(full, caps=caps, n=M, posspec=pos, iterations=20, init=1, **opts)
        half = np.zeros_like(born)
        ctx.tv_reconstruct(half, caps=caps, n=M, posspec=pos, iterations=10, init=1, **opts)
        ctx.tv_reconstruct(half, caps=caps, n=M, posspec=pos, iterations=10, init=0, **opts)
    e_born, e_tv = rel_l2(born, truth), rel_l2(full, truth)
    assert e_tv < 0.8 * e_born, (e_born, e_tv)
    assert rep["misfit_last"] < rep["misfit_first"]
    assert full.min() >= 0.0 and full.max() <= 0.05
    np.testing.assert_array_equal(half, full)


def geometry_stated(M=400):
    """The regularised-reconstruction workload at its stated size: a 256^3
    index volume and 400 Ewald caps of 128^2 (NXMAX 64), specular positions
    on the Fermat spiral out to 0.9 NXMAX."""
    acq, _, _ = simul.workload("plain_512_born")
    acq = replace(acq, nb_holo=M)
    N = acq.nxmax
    t = simul.spiral_tilts(M, N)
    pos = np.concatenate([N + t[:, 0], N + t[:, 1]]).astype(np.int32)
    return acq, pos


def test_operator_pair_at_stated_size():
    """256^3 -> 400 caps of 128^2: forward and adjoint against the FP64
    oracle, the dot-product test, and central differences with eps = 1e-3 on
    32 random voxels against A^H (A x - y)."""
    import torch
    acq, pos = geometry_stated()
    cfg = oracle_cfg(acq)
    D, F, M = acq.dim_final, 2 * acq.nxmax, acq.nb_holo
    assert (D, F, M) == (256, 128, 400)
    rng = np.random.default_rng(12)
    xn = rng.standard_normal((D, D, D)).astype(np.float32)
    xk = rng.standard_normal((D, D, D)).astype(np.float32)
    y = (rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))).astype(np.complex64)
    with Context(Geometry.from_acquisition(acq), M) as ctx:
        caps = ctx.forward(xn, xk, n=M, posspec=pos)
        an, ak = ctx.adjoint(y, n=M, posspec=pos, absorption_out=np.zeros((D, D, D), np.float32))
        ref_f = oracle.forward_caps(xn.astype(np.float64), xk.astype(np.float64), pos.astype(np.float64), cfg)
        assert np.array_equal(caps != 0, ref_f != 0)
        assert rel_l2(caps, ref_f) <= TOL
        del ref_f
        ref_a = oracle.adjoint_caps(y.astype(np.complex128), pos.astype(np.float64), cfg)
        assert rel_l2(an, ref_a.real) <= TOL
        assert rel_l2(ak, ref_a.imag) <= TOL
        del ref_a
        lhs = np.vdot(y.astype(np.complex128), caps.astype(np.complex128))
        rhs = np.vdot((an + 1j * ak).astype(np.complex128), xn + 1j * xk.astype(np.float64))
        assert abs(lhs - rhs) / abs(lhs) <= TOL
        # finite differences on device buffers (f in FP64 from the FP32 caps)
        p = torch.from_numpy(pos).cuda()
        x0 = torch.zeros((D, D, D), device="cuda")
        xt = torch.zeros_like(x0)
        for v in (x0, xt):
            idx = torch.from_numpy(rng.integers(0, D, (64, 3))).cuda()
            v[idx[:, 0], idx[:, 1], idx[:, 2]] = torch.from_numpy(0.02 * rng.standard_normal(64)).float().cuda()
        out = torch.empty((M, F, F), dtype=torch.complex64, device="cuda")

        def fwd(x):
            ctx.forward(x, None, n=M, posspec=p, caps_out=out)
            ctx.synchronize()
            return out.to(torch.complex128)

        yt = fwd(xt)

        def f(x):
            r = fwd(x) - yt
            return 0.5 * float(torch.vdot(r.flatten(), r.flatten()).real)

        r0 = (fwd(x0) - yt).to(torch.complex64).contiguous()
        g = torch.empty_like(x0)
        ctx.adjoint(r0, n=M, posspec=p, index_out=g)
        ctx.synchronize()
        eps = 1e-3
        fd, ga = [], []
        for v in rng.integers(0, D, (32, 3)):
            v = tuple(int(c) for c in v)
            xp, xm = x0.clone(), x0.clone()
            xp[v] += eps
            xm[v] -= eps
            fd.append((f(xp) - f(xm)) / (2 * eps))
            ga.append(float(g[v]))
    fd, ga = np.array(fd), np.array(ga)
    assert np.abs(fd - ga).max() <= 1e-3 * np.abs(ga).max()
