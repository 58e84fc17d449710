"""Pins the FP64 oracle: independent restatements of each reference step in
numpy (FFTs vs numpy.fft, float-typed Tukey arithmetic, shifts vs np.roll,
cap indices vs a direct Python loop) and known-answer cases."""
from __future__ import annotations

import math

import numpy as np
import pytest

import oracle
from tests.helpers import oracle_cfg, rel_l2, small_case


@pytest.mark.parametrize("n", [64, 128, 256, 512, 250, 500, 200, 6])
def test_fft2d_matches_numpy(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n)) + 1j * rng.standard_normal((n, n))
    assert np.abs(oracle.fft2d(a, -1) - np.fft.fft2(a)).max() <= 1e-12 * np.abs(np.fft.fft2(a)).max()
    assert np.abs(oracle.fft2d(a, +1) - np.fft.ifft2(a) * a.size).max() <= 1e-12 * n * n * np.abs(a).max()


@pytest.mark.parametrize("n", [32, 64])
def test_fft3d_matches_numpy(n):
    rng = np.random.default_rng(n)
    a = rng.standard_normal((n, n, n)) + 1j * rng.standard_normal((n, n, n))
    ref = np.fft.ifftn(a) * a.size
    assert np.abs(oracle.fft3d(a, +1) - ref).max() <= 1e-12 * np.abs(ref).max()


def _tukey_numpy(n: int, alpha: float) -> np.ndarray:
    """tukey2D re-derived with numpy float32 scalars for the float sub-expressions."""
    f32 = np.float32
    a = f32(alpha)
    b1 = int(np.round(a * f32(n - 1) / f32(2)))
    b2 = int(np.round(f32(n - 1) * (f32(1) - a / f32(2))))
    t = np.zeros(n)
    for i in range(n):
        if i <= b1:
            arg = f32(2 * i) / (a * f32(n - 1)) - f32(1)
            t[i] = 0.5 * (1 + math.cos(3.1415 * float(arg)))
        elif i <= b2:
            t[i] = 1.0
        else:
            arg = f32(2 * i) / (a * f32(n - 1)) - f32(2) / a + f32(1)
            t[i] = 0.5 * (1 + math.cos(3.1415 * float(arg)))
    return np.outer(t, t)


@pytest.mark.parametrize("n,alpha", [(128, 0.1), (256, 0.1), (512, 0.05), (1024, 0.05)])
def test_tukey_float_semantics(n, alpha):
    np.testing.assert_array_equal(oracle.tukey2d(n, alpha), _tukey_numpy(n, alpha))


@pytest.mark.parametrize("n", [256, 512, 1024, 2048])
def test_hologram_window_flat_where_the_row_pass_skips_it(n):
    """The extraction's row pass reads the hologram window only for the first
    and last K of each lane's E elements (x = j + T n1, T = n / E; K = 2 at
    2048 points, else 1) and takes it as exactly 1 elsewhere; the window of
    tukey2D (alpha 0.05) is exactly 1 on that whole middle."""
    e = 64 if n >= 2048 else 32 if n >= 512 else 16
    t_lanes, k = n // e, (2 if n >= 2048 else 1)
    t = _tukey_numpy(n, 0.05)[n // 2]
    assert np.all(t[t_lanes * k:n - t_lanes * k] == 1.0)
    assert t[0] != 1.0 and t[-1] != 1.0


def test_crand_is_the_c_library_generator():
    """The oracle's restatement of the C library's rand() (glibc's default
    generator), which Herraez unwrapping draws its border reliabilities from,
    against the C library itself, from the start and after 102,000 draws."""
    import ctypes
    try:
        libc = ctypes.CDLL("libc.so.6")
    except OSError:
        pytest.skip("no glibc")
    libc.srand(1)
    first = np.array([libc.rand() for _ in range(2000)], np.int32)
    np.testing.assert_array_equal(oracle.crand(0, 2000), first)
    for _ in range(100000):
        libc.rand()
    np.testing.assert_array_equal(oracle.crand(102000, 100), np.array([libc.rand() for _ in range(100)], np.int32))


def test_coord_spec_quirk():
    F = 16
    s = np.zeros((F, F), np.complex128)
    s[3, 5] = 2.5                     # |z| = 2.5
    s[0, 0] = 1.7                     # |z|^2 = 2.89 > 2.5 although |z| < 2.5
    assert oracle.coord_spec(s) == 0
    s[0, 0] = 1.5                     # 2.25 < 2.5
    assert oracle.coord_spec(s) == 3 * F + 5
    s[7, 1] = 2.5                     # tie: the first maximum wins
    assert oracle.coord_spec(s) == 3 * F + 5


def test_calc_uborn2_matches_roll():
    rng = np.random.default_rng(1)
    F = 32
    s = rng.standard_normal((F, F)) + 1j * rng.standard_normal((F, F))
    px, py = 7, 23
    ref = np.roll(np.fft.ifft2(np.roll(s, (-py, -px), (0, 1))) * F * F, (F // 2, F // 2), (0, 1))
    assert rel_l2(oracle.calc_uborn2(s, px, py), ref) < 1e-13


def test_volkov_unwraps_known_phase():
    F = 128
    y, x = np.mgrid[0:F, 0:F] / F
    true = 14 * np.exp(-((x - 0.45) ** 2 + (y - 0.55) ** 2) / 0.05) + 3 * x - 2 * y
    wrapped = np.angle(np.exp(1j * true))
    assert np.abs(wrapped - true).max() > 6  # really wrapped
    un = oracle.volkov(wrapped)
    d = un - true
    assert np.abs(d - d.mean()).max() < 0.05


def test_aberration_fit_is_least_squares():
    F = 64
    rng = np.random.default_rng(3)
    y, x = np.mgrid[0:F, 0:F].astype(float)
    img = 3 + 0.02 * x - 0.01 * y + 1e-4 * x * y - 2e-6 * x ** 3 + 0.05 * rng.standard_normal((F, F))
    mask = np.full((F, F), 255, np.uint8)
    mask[20:40, 25:45] = 0
    surf = oracle.aber_surface(img, mask)
    samp = (y % 5 == 0) & (x % 5 == 0) & (mask > 45)
    u, v = (x - 31.5) / 31.5, (y - 31.5) / 31.5
    B = np.stack([u ** px * v ** py for px in range(5) for py in range(5 - px)], -1)
    c, *_ = np.linalg.lstsq(B[samp], img[samp], rcond=None)
    assert np.abs(surf - B @ c).max() < 1e-9


def _cap_counts_python(posspec, M, N, D, rayon, coef=1.0):
    """retroPropag_Born index arithmetic restated directly (hit counts only)."""
    cnt = np.zeros(D * D * D, np.int64)
    dec = D // 2
    for a in range(M):
        px, py = int(posspec[a]), int(posspec[M + a])
        fxm0, fym0 = px - N, py - N
        c = rayon * rayon - fxm0 * fxm0 - fym0 * fym0
        if round(c) < 0:
            continue
        fzm0 = math.sqrt(c)
        for fdy in range(-N, N):
            for fdx in range(-N, N):
                if fdx * fdx + fdy * fdy < coef * N * N:
                    koz = math.floor(math.sqrt(rayon * rayon - fdx * fdx - fdy * fdy) - fzm0 + 0.5)
                    cnt[(-fxm0 + fdx + dec) + (-fym0 + fdy + dec) * D + (koz + dec) * D * D] += 1
    return cnt.reshape(D, D, D)


def test_cap_counts_independent():
    acq, ph, d = small_case("plain_512_born", M=1, nxmax=32, circle_cx=64, circle_cy=64, dim_final=128,
                            ccd_roix=256)
    N, F, D = 32, 64, 128
    cfg = oracle_cfg(acq)
    rng = np.random.default_rng(0)
    pos = np.array([40, 10, 32, 0, 63, 22, 5, 32, 50, 63], np.float64)  # 5 angles: x then y
    M = 5
    f = rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))
    r = oracle.reconstruction(f, pos, cfg)
    rayon = oracle.derive(cfg)["rayon"]
    np.testing.assert_array_equal(r["counts"], _cap_counts_python(pos, M, N, D, rayon))
    assert (r["otf"] == (r["counts"] > 0)).all()


def test_extraction_of_a_plane_wave():
    """A pure carrier lands at (CIRCLE_CX + t) in the fftshifted spectrum."""
    acq, ph, d = small_case("plain_512_born", M=1)
    H, N = acq.ccd_roix, acq.nxmax
    y, x = np.mgrid[0:H, 0:H]
    tx, ty = 9, -14
    fx, fy = acq.circle_cx - H // 2 + tx, acq.circle_cy - H // 2 + ty
    holo = 1000 + 500 * np.cos(2 * np.pi * (fx * x + fy * y) / H)
    spec = oracle.extract(holo, oracle_cfg(acq))
    k = oracle.coord_spec(spec)
    assert (k % (2 * N), k // (2 * N)) == (N + tx, N + ty)


def test_oracle_forward_adjoint_pair():
    """The oracle's cap forward operator and adjoint are adjoint (dot-product
    test in FP64) and sample exactly the cells the reconstruction counts."""
    cfg = oracle.Config()
    cfg.ccd_roix, cfg.nxmax, cfg.circle_cx, cfg.circle_cy, cfg.dim_final = 256, 16, 64, 64, 64
    rng = np.random.default_rng(0)
    M, F, D = 5, 32, 64
    pos = np.concatenate([rng.integers(6, F - 6, M), rng.integers(6, F - 6, M)]).astype(np.float64)
    xn, xk = rng.standard_normal((D, D, D)), rng.standard_normal((D, D, D))
    y = rng.standard_normal((M, F, F)) + 1j * rng.standard_normal((M, F, F))
    ax = oracle.forward_caps(xn, xk, pos, cfg)
    ahy = oracle.adjoint_caps(y, pos, cfg)
    lhs, rhs = np.vdot(y, ax), np.vdot(ahy, xn + 1j * xk)
    assert abs(lhs - rhs) <= 1e-12 * abs(lhs)
    # the cells are the reconstruction's: scattering ones gives its hit counts
    counts = np.zeros((D, D, D))
    for a, cell in enumerate(oracle.cap_cells(pos, cfg)):
        np.add.at(counts, cell[1:], 1.0)
    ref = oracle.reconstruction(np.zeros((M, F, F), np.complex128), pos, cfg, want_otf=False, want_indice=False)
    np.testing.assert_array_equal(counts, ref["counts"])


def test_reference_amplitude_rule():
    """initRef (fonctions.cpp:46-61): sqrt of the intensity, 1 where it is 0;
    a unit reference leaves the extraction unchanged."""
    i = np.array([[0.0, 4.0], [9.0, 2.0]])
    np.testing.assert_array_equal(oracle.reference_amplitude(i), [[1.0, 2.0], [3.0, np.sqrt(2.0)]])
    acq, ph, d = small_case("plain_512_born", M=1)
    cfg = oracle_cfg(acq)
    h = d["holos"].astype(np.float64)
    ones = np.ones((acq.ccd_roix, acq.ccd_roix))
    np.testing.assert_array_equal(oracle.extract_stack(h, cfg, ref_intensity=ones), oracle.extract_stack(h, cfg))
