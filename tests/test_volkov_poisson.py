"""The Volkov unwrap's Poisson solve as the kernels compute it, restated in
numpy on the CPU (no GPU), against integ_grad4's form on the 2F x 2F mirror
(src/deroulement_volkov4.cpp:162-191, then cut_quad4 :247-276):

    tampon = -i (kappa_x FFT2(gx) + kappa_y FFT2(gy)) / (2 pi |kappa|^2) / L^2,
    tampon(0, 0) = 0,  IntM = Re IFFT2(tampon) on the quadrant,

with the reference's kappa (init_kvect_shift: k/L below L/2, (k - L)/L from
L/2 up, so -1/2 at the Nyquist bin).  gx is odd and gy even about the
mirror's vertical axis (and the other way about the horizontal one), so the
kernels fold the 2F-point transforms into F-point DCT-II / DST-II forward
transforms, P = -4/L^2 (kappa_x A + kappa_y B) / |kappa|^2, and DCT-III
inverses (k_fields.cu: column_dct_dst in k_volkov_cols, k_volkov_integ_rows
and k_volkov_integ_cols; k_generic.cu the same on the mixed-radix engine).
The emulation below follows their pairing of bins k and F - k, their
permutation of the samples and their packing of two real sequences per
complex transform.  The last test checks the identity that lets the kernels
drop the wrapped phase's own gradient and add its mean instead.
"""
from __future__ import annotations

import numpy as np
import pytest


def perm(n):
    m = np.arange(n)
    return np.where(m < n // 2, 2 * m, 2 * (n - 1 - m) + 1)


def mirror(q, sx, sy):
    """2F x 2F mirror of the quadrant q (rows F + y, columns F + x), with sign
    sx across the vertical axis and sy across the horizontal one."""
    F = q.shape[0]
    m = np.zeros((2 * F, 2 * F))
    m[F:, F:] = q
    m[F:, :F] = sx * q[:, ::-1]
    m[:F, F:] = sy * q[::-1, :]
    m[:F, :F] = sx * sy * q[::-1, ::-1]
    return m


def reference_form(qx, qy):
    """2 pi IntM on the quadrant from the 2F x 2F transforms."""
    F = qx.shape[0]
    L = 2 * F
    gx, gy = mirror(qx, -1, 1), mirror(qy, 1, -1)
    k = np.arange(L)
    kap = np.where(k < L // 2, k, k - L) / L
    kx, ky = kap[None, :], kap[:, None]
    k2 = kx ** 2 + ky ** 2
    k2[0, 0] = 1.0
    tam = -1j * (kx * np.fft.fft2(gx) + ky * np.fft.fft2(gy)) / (2 * np.pi * k2) / (L * L)
    tam[0, 0] = 0.0
    return 2 * np.pi * np.real(np.fft.ifft2(tam) * L * L)[F:, F:]


def kernel_form(qx, qy):
    """2 pi IntM as the three kernels compute it."""
    F = qx.shape[0]
    L = 2 * F
    P = perm(F)
    k = np.arange(F)
    wk = np.exp(-1j * np.pi * k / (2 * F))
    part = (F - k) % F
    sg = (-1.0) ** np.arange(F)
    # column pass: one transform of gx + i (-1)^y gy per column
    c = np.zeros((F, F), complex)
    for x in range(F):
        V = np.fft.fft((qx[:, x] + 1j * sg * qy[:, x])[P])
        a, b = wk * V, np.conj(wk) * V[part]
        c[:, x] = 0.5 * (a.real + b.real) + 0.5j * (a.real - b.real)
    # row pass, two rows per inverse transform
    U = np.zeros((F, F))
    kx = k / L
    for r0 in range(0, F, 2):
        rows = []
        for r in (r0, r0 + 1):
            V = np.fft.fft((sg * c[r].real + 1j * c[r].imag)[P])
            Vm = V[part]
            e = wk * (V + np.conj(Vm))          # 2 qu
            d = wk * (V - np.conj(Vm))          # 2i qv
            kyv = r / L
            den = kx ** 2 + kyv ** 2
            num = 0.5 * (-4.0 / (L * L)) * (kyv * d.imag - kx * e.imag)
            rows.append(np.where(den > 0, num / np.where(den > 0, den, 1.0), 0.0))
        X = rows[0] + 1j * rows[1]
        Xm = np.where(k == 0, 0.0, X[part])
        v = np.fft.ifft(np.conj(wk) * (X - 1j * Xm)) * F
        U[r0, P], U[r0 + 1, P] = v.real, v.imag
    # column pass, two columns per inverse transform
    out = np.zeros((F, F))
    for x0 in range(0, F, 2):
        X = U[:, x0] + 1j * U[:, x0 + 1]
        Xm = np.where(k == 0, 0.0, X[part])
        v = np.fft.ifft(np.conj(wk) * (X - 1j * Xm)) * F
        out[P, x0], out[P, x0 + 1] = v.real, v.imag
    return out


@pytest.mark.parametrize("F", [8, 16, 250, 256])
def test_folded_poisson_solve_matches_the_mirror_form(F):
    rng = np.random.default_rng(F)
    qx, qy = rng.standard_normal((F, F)), rng.standard_normal((F, F))
    ref = reference_form(qx, qy)
    assert np.abs(kernel_form(qx, qy) - ref).max() <= 1e-10 * np.abs(ref).max()


def test_nyquist_terms_cancel():
    """The reference's -1/2 at the Nyquist bin does not reach the quadrant:
    the same solve with +1/2 there gives the same IntM."""
    F = 16
    L = 2 * F
    rng = np.random.default_rng(3)
    qx, qy = rng.standard_normal((F, F)), rng.standard_normal((F, F))
    gx, gy = mirror(qx, -1, 1), mirror(qy, 1, -1)
    k = np.arange(L)
    out = []
    for nyq in (-0.5, 0.5):
        kap = np.where(k < L // 2, k, k - L) / L
        kap[L // 2] = nyq
        kx, ky = kap[None, :], kap[:, None]
        k2 = kx ** 2 + ky ** 2
        k2[0, 0] = 1.0
        tam = -1j * (kx * np.fft.fft2(gx) + ky * np.fft.fft2(gy)) / (2 * np.pi * k2)
        tam[0, 0] = 0.0
        out.append(np.real(np.fft.ifft2(tam))[F:, F:])
    assert np.abs(out[0] - out[1]).max() <= 1e-12 * np.abs(out[0]).max()


def test_phase_gradient_term_is_the_phase_less_its_mean():
    """deroul_volkov4_total_sym_paire forms gx = (Re(-i dZ/dx / Z) - dphi/dx) / 2pi
    (and gy alike) on the even mirror, solves, and adds phi back.  The
    solve inverts the spectral gradient exactly except at zero frequency,
    which it sets to 0, so the phi terms contribute -(phi - mean phi): the
    kernels solve for the phasor's gradient alone and add mean(phi)."""
    F = 16
    L = 2 * F
    rng = np.random.default_rng(5)
    true = np.cumsum(np.cumsum(rng.standard_normal((F, F)) * 0.8, 0), 1)
    phi = np.angle(np.exp(1j * true))

    def even(q):
        return mirror(q, 1, 1)

    k = np.arange(L)
    kap = np.where(k < L // 2, k, k - L) / L

    def dx(m):  # gradient_fft4 along x
        return np.fft.ifft(np.fft.fft(m, axis=1) * 2j * np.pi * kap[None, :], axis=1)

    def dy(m):
        return np.fft.ifft(np.fft.fft(m, axis=0) * 2j * np.pi * kap[:, None], axis=0)

    def solve(gx, gy):
        kx, ky = kap[None, :], kap[:, None]
        k2 = kx ** 2 + ky ** 2
        k2[0, 0] = 1.0
        t = -1j * (kx * np.fft.fft2(gx) + ky * np.fft.fft2(gy)) / (2 * np.pi * k2)
        t[0, 0] = 0.0
        return np.real(np.fft.ifft2(t))

    Z = even(np.cos(phi)) + 1j * even(np.sin(phi))
    pm = even(phi)
    gxz, gyz = np.real(-1j * dx(Z) / Z) / (2 * np.pi), np.real(-1j * dy(Z) / Z) / (2 * np.pi)
    gxp, gyp = np.real(dx(pm)) / (2 * np.pi), np.real(dy(pm)) / (2 * np.pi)
    reference = pm + 2 * np.pi * solve(gxz - gxp, gyz - gyp)
    kernels = pm.mean() + 2 * np.pi * solve(gxz, gyz)
    assert np.abs(reference - kernels).max() <= 1e-12 * np.abs(reference).max()
    assert abs(pm.mean() - phi.mean()) <= 1e-15 * F * F  # the mirror's mean is the quadrant's
