"""The mixed-radix engine and the generic Volkov passes, restated in numpy on
the CPU (no GPU), with the index arithmetic of fft_generic.cuh and
k_generic.cu:

- gfft: the radix plan (4 first, then 2, 3, 5, 7) and the Stockham passes
  (read b + k N/R, twiddle W_(S R)^((b mod S) k), R-point DFT, write
  (b / S) S R + (b mod S) + m S) against numpy.fft, both signs;
- gmirror_derivative: the 2F-point even mirror's spectral derivative at
  X = F + x from F-point transforms, the partner bin F - k read at index
  (k ? F - k : 0);
- the column pass's 2F-point FFT of Q from one F-point transform, with bins
  [0, F) in the column's array and bin F + j at index j of the pair's array.
"""
from __future__ import annotations

import numpy as np
import pytest


def gfft_radix(m):
    for r in (4, 2, 3, 5, 7):
        if m % r == 0:
            return r
    return m


def gfft(x, sign):
    """Emulates gfft<N, sign>: the Stockham passes of fft_generic.cuh."""
    N = len(x)
    a = np.asarray(x, complex).copy()
    S = 1
    while S < N:
        R = gfft_radix(N // S)
        NB = N // R
        out = np.empty(N, complex)
        for b in range(NB):
            p = b % S
            v = np.array([a[b + k * NB] for k in range(R)])
            v = v * np.exp(sign * 2j * np.pi * p * np.arange(R) / (S * R))
            y = np.array([np.sum(v * np.exp(sign * 2j * np.pi * np.arange(R) * m / R)) for m in range(R)])
            base = (b // S) * S * R + p
            for m in range(R):
                out[base + m * S] = y[m]
        a = out
        S *= R
    return a


@pytest.mark.parametrize("N", [250, 500, 200, 300, 112, 6])
def test_gfft_matches_numpy(N):
    rng = np.random.default_rng(N)
    x = rng.standard_normal(N) + 1j * rng.standard_normal(N)
    assert np.abs(gfft(x, -1) - np.fft.fft(x)).max() <= 1e-10 * np.abs(x).sum()
    assert np.abs(gfft(x, +1) - np.fft.ifft(x) * N).max() <= 1e-10 * np.abs(x).sum()


def mirror_pos(m, F):
    return np.where(m < F // 2, 2 * m, 2 * (F - 1 - m) + 1)


def gslot(y, F):
    return np.where(y & 1, F - 1 - (y >> 1), y >> 1)


def gmirror_derivative(z):
    """Emulates gmirror_derivative<F> on a row z (complex): returns d[x], the
    derivative of the even mirror at X = F + x."""
    F = len(z)
    m = np.arange(F)
    a = z[mirror_pos(m, F)]
    V = np.fft.fft(a)
    k = np.arange(F)
    vm = V[np.where(k > 0, F - k, 0)]
    e = np.exp(1j * np.pi * k / F)
    t = e * vm - (1 - 2 * k / F) * V
    W = 1j * (np.pi / (2 * F)) * t
    W[0] = 0
    w = np.fft.ifft(W) * F
    d = np.empty(F, complex)
    d[mirror_pos(m, F)] = np.where(m < F // 2, w, -w)
    return d


def mirror_derivative_direct(z):
    """gradient_fft4 on the mirror, restricted to one row: FFT of the 2F-point
    even mirror, x 2 pi i kappa / 2F with kappa the signed bin (the Nyquist bin
    of the mirror is zero), inverse; the right half X = F + x."""
    F = len(z)
    L = 2 * F
    mir = np.concatenate([z[::-1], z])
    k = np.arange(L)
    kap = np.where(k < L // 2, k, k - L) / L
    g = np.fft.ifft(np.fft.fft(mir) * 2j * np.pi * kap)
    return g[F:]


@pytest.mark.parametrize("F", [250, 200, 64])
def test_generic_mirror_derivative(F):
    rng = np.random.default_rng(F)
    z = rng.standard_normal(F) + 1j * rng.standard_normal(F)
    ref = mirror_derivative_direct(z)
    assert np.abs(gmirror_derivative(z) - ref).max() <= 1e-10 * np.abs(ref).max()


@pytest.mark.parametrize("F", [250, 200, 64])
def test_generic_column_fft_of_q(F):
    """The bins the column pass stores: [0, F) in the column's array, bin F + j
    at index j of the pair's array, from one F-point transform."""
    rng = np.random.default_rng(F + 1)
    L = 2 * F
    gx = rng.standard_normal(F)
    gy = rng.standard_normal(F)
    Q = np.empty(L, complex)
    Q[F:] = gx + 1j * gy                         # Y = F + y
    Q[:F] = np.conj(Q[F:][::-1])                 # Q[L-1-Y] = conj(Q[Y])
    ref = np.fft.fft(Q)
    y = np.arange(F)
    u = gx + 1j * np.where(y & 1, -gy, gy)       # gx + i (-1)^y gy
    inp = np.empty(F, complex)
    inp[gslot(y, F)] = u                         # element gslot(y) holds row y
    V = np.fft.fft(inp)
    lo = np.empty(F, complex)
    hi = np.empty(F, complex)
    for k in range(F):
        wk = np.exp(-1j * np.pi * k / L)
        va, vb = wk * V[k], np.conj(wk) * V[F - k if k else 0]
        ck, cf = 0.5 * (va.real + vb.real), 0.5 * (va.real - vb.real)
        sg = -2.0 if k & 1 else 2.0
        if k == 0:
            lo[0] = 2 * ck
            hi[0] = 1j * (va.imag + vb.imag)
        else:
            r1, r2 = sg * (ck + cf), -sg * (cf - ck)
            lo[k] = r1 * np.conj(wk)
            hi[F - k] = r2 * wk
    got = np.concatenate([lo, hi])
    assert np.abs(got - ref).max() <= 1e-10 * np.abs(ref).max()
