"""The algebra of the warp-resident FFT engine and of the half-length Volkov
transforms, restated in numpy on the CPU (no GPU).

- fft_warp_regs: lane j of a transform holds elements j + T n1 on entry; an
  E-point DFT per lane, the twiddles W_N^(j k1), the transposing exchange and
  E/T DFTs of T points leave bin (j + q T) + E k2 in register q T + k2.
- The holder of bin N - k (used to pair bins k and -k by a lane shuffle).
- mirror_derivative: the spectral derivative of the 2F-point even mirror of a
  row from two F-point transforms of the row permuted by mirror_pos.
- column_dct_dst: a column's DCT-II of gx and DST-II of gy from one F-point
  transform of gx + i (-1)^y gy permuted by mirror_pos.
"""
from __future__ import annotations

import numpy as np
import pytest


def warp_fft_e(n):
    return 64 if n >= 2048 else 32 if n >= 512 else 16 if n >= 128 else 8


def mirror_pos(m, F):
    return np.where(m < F // 2, 2 * m, 2 * (F - 1 - m) + 1)


def warp_fft_regs(x, N):
    """Emulates fft_warp_regs<N, -1> on one transform: returns reg[j][r]."""
    E = warp_fft_e(N)
    T = N // E
    lanes = np.array([[x[j + T * n1] for n1 in range(E)] for j in range(T)])      # [j][n1]
    k1 = np.arange(E)
    stage1 = lanes @ np.exp(-2j * np.pi * np.outer(np.arange(E), k1) / E)        # E-point DFT per lane
    stage1 *= np.exp(-2j * np.pi * np.outer(np.arange(T), k1) / N)              # W_N^(j k1)
    reg = np.empty((T, E), complex)
    for j in range(T):
        for q in range(E // T):
            col = stage1[:, j + q * T]                                          # lane n2's value at k1 = j + qT
            reg[j, q * T:(q + 1) * T] = col @ np.exp(-2j * np.pi * np.outer(np.arange(T), np.arange(T)) / T)
    return reg


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048])
def test_warp_fft_output_order(N):
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    ref = np.fft.fft(x)
    E = warp_fft_e(N)
    T = N // E
    reg = warp_fft_regs(x, N)
    for j in range(T):
        for q in range(E // T):
            for k2 in range(T):
                k = (j + q * T) + E * k2
                assert abs(reg[j, q * T + k2] - ref[k]) <= 1e-9 * np.abs(ref).max()
                # warp_out_pos: position of that bin in the padded array
                pos = j + q * T + E * k2 + q + (E // T) * k2
                assert pos == k + k // T


@pytest.mark.parametrize("N", [64, 128, 256, 512, 1024, 2048])
def test_partner_bin_holder(N):
    E = warp_fft_e(N)
    T = N // E
    where = {}
    for j in range(T):
        for q in range(E // T):
            for k2 in range(T):
                where[(j + q * T) + E * k2] = (j, q * T + k2)
    for j in range(T):
        for q in range(E // T):
            for k2 in range(T):
                k = (j + q * T) + E * k2
                if j > 0:
                    holder = ((T - j) % T, (E // T - 1 - q) * T + (T - 1 - k2))
                else:
                    holder = (0, (T - k2) % T if q == 0 else (E // T - q) * T + T - 1 - k2)
                assert where[(N - k) % N] == holder, (k, holder)


def _mirror(z):
    F = z.size
    X = np.arange(2 * F)
    return np.where(X >= F, z[np.clip(X - F, 0, F - 1)], z[np.clip(F - 1 - X, 0, F - 1)])


@pytest.mark.parametrize("F", [64, 128, 256, 512])
def test_mirror_derivative(F):
    rng = np.random.default_rng(F + 1)
    z = rng.standard_normal(F) + 1j * rng.standard_normal(F)
    L = 2 * F
    k = np.arange(L)
    kappa = np.where(k < L // 2, k, k - L) / L
    # the 2F-point filter on the mirror: FFT, x i 2 pi kappa / 2F, unnormalised inverse
    ref = np.fft.ifft(np.fft.fft(_mirror(z)) * 1j * 2 * np.pi * kappa / L) * L
    m = np.arange(F)
    V = np.fft.fft(z[mirror_pos(m, F)])
    kk = np.arange(F)
    W = 1j * (np.pi / (2 * F)) * (np.exp(1j * np.pi * kk / F) * V[(F - kk) % F] - (1 - 2 * kk / F) * V)
    W[0] = 0
    w = np.fft.ifft(W) * F                    # unnormalised inverse F-point transform
    got = np.empty(F, complex)
    got[mirror_pos(m, F)] = np.where(m < F // 2, w, -w)
    assert np.abs(got - ref[F:]).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("F", [64, 128, 250, 256, 512])
def test_column_dct_dst(F):
    rng = np.random.default_rng(F + 2)
    a, b = rng.standard_normal(F), rng.standard_normal(F)
    y = np.arange(F)
    k = np.arange(F)[:, None]
    dct = (a[None, :] * np.cos(np.pi * k * (2 * y + 1) / (2 * F))).sum(1)
    dst = (b[None, :] * np.sin(np.pi * k * (2 * y + 1) / (2 * F))).sum(1)
    m = np.arange(F)
    V = np.fft.fft((a + 1j * ((-1.0) ** y) * b)[mirror_pos(m, F)])
    kk = np.arange(F)
    w = np.exp(-1j * np.pi * kk / (2 * F))
    A, B = w * V, np.conj(w) * V[(F - kk) % F]
    ck, cf = 0.5 * (A.real + B.real), 0.5 * (A.real - B.real)
    scale = np.abs(a).sum() + np.abs(b).sum()
    assert np.abs(ck - dct).max() <= 1e-12 * scale
    assert np.abs(cf - dst).max() <= 1e-12 * scale
