"""The mixed-radix engine and the generic Volkov passes, restated in numpy on
the CPU (no GPU), with the index arithmetic of fft_generic.cuh and
k_generic.cu:

- gfft: the radix plan (10 while it divides, then 4, 2, 3, 5, 7), the
  Stockham passes (read b + k N/R, twiddle W_(S R)^((b mod S) k) formed as
  W^(k/2) W^(k - k/2) from W^1, R-point DFT, write
  (b / S) S R + (b mod S) + m S) and the radix-10 DFT's 2 x 5 register
  decomposition against numpy.fft, both signs;
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
    for r in (10, 4, 2, 3, 5, 7):
        if m % r == 0:
            return r
    return m


def dft(v, sign):
    R = len(v)
    return np.array([np.sum(v * np.exp(sign * 2j * np.pi * np.arange(R) * m / R)) for m in range(R)])


def dft_composite(x, R1, R2, sign):
    """Emulates dft_composite<R1, R2>: k = R2 k1 + k2, m = m1 + R1 m2."""
    R = R1 * R2
    y = np.empty(R, complex)  # y[m1 R2 + k2]
    for k2 in range(R2):
        v = dft(np.array([x[R2 * k1 + k2] for k1 in range(R1)]), sign)
        for m1 in range(R1):
            y[m1 * R2 + k2] = v[m1] * np.exp(sign * 2j * np.pi * ((k2 * m1) % R) / R)
    out = np.empty(R, complex)
    for m1 in range(R1):
        u = dft(y[m1 * R2:(m1 + 1) * R2], sign)
        for m2 in range(R2):
            out[m1 + R1 * m2] = u[m2]
    return out


def twiddle_powers(w1, R):
    """W^k for k < R from W^1 as gfft_pass forms them."""
    t = [1.0 + 0j, w1]
    for k in range(2, R):
        t.append(t[k >> 1] * t[k - (k >> 1)])
    return np.array(t[:R])


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
            v = v * twiddle_powers(np.exp(sign * 2j * np.pi * p / (S * R)), R)
            y = dft_composite(v, 2, 5, sign) if R == 10 else dft(v, sign)
            base = (b // S) * S * R + p
            for m in range(R):
                out[base + m * S] = y[m]
        a = out
        S *= R
    return a


def test_radix_plan():
    def passes(n):
        out = []
        while n > 1:
            r = gfft_radix(n)
            out.append(r)
            n //= r
        return out
    assert passes(250) == [10, 5, 5] and passes(500) == [10, 10, 5]


@pytest.mark.parametrize("sign", [-1, 1])
def test_radix10_register_decomposition(sign):
    rng = np.random.default_rng(10)
    x = rng.standard_normal(10) + 1j * rng.standard_normal(10)
    assert np.abs(dft_composite(x, 2, 5, sign) - dft(x, sign)).max() <= 1e-12


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
