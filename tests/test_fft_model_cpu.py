"""CPU model of the specialised passes' four-step line transform (no GPU).

fft_method_test_gb300/csrc/fft_fast.cuh transforms a line of N = R1 * R2
points with TPL threads: stage A (owners a = t + TPL j) does DFT-R1 over
x[R2 i + a], multiplies by W_N^(S a k) and stores Y[k][a] at line position
k (RB + 1) + a; stage B (owners k) does DFT-R2 over Y[k][.] and produces
X[k + R1 m].  The inverse swaps the radices.  Radix 12 and 20 are
prime-factor DFTs (4 x 3, 4 x 5).  The splits are read from the header, so
the model checks the table the kernels are built from: every owner index,
every line position inside the padded line, and the transform itself against
numpy's FFT, for every specialised edge and both directions.
"""
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "fft_method_test_gb300", "csrc", "fft_fast.cuh")


def _splits():
    src = open(HEADER).read()
    out = {}
    for n, r1, r2, tpl in re.findall(
            r"struct Split<(\d+)>\s*{\s*static constexpr int R1 = (\d+), R2 = (\d+), TPL = (\d+);", src):
        out[int(n)] = (int(r1), int(r2), int(tpl))
    return out


def _dft(v, sign):
    r = len(v)
    k = np.arange(r)
    return np.exp(sign * 2j * np.pi * np.outer(k, k) / r) @ v


def _dft_pfa(v, p, q, sign):
    """Prime-factor DFT as the kernel's dft_pfa<P, Q>: input (Q n1 + P n2) mod R
    to a[n1][n2], DFT-Q along n2, DFT-P along n1, output k from a[k % P][k % Q]."""
    r = p * q
    a = np.array([[v[(q * n1 + p * n2) % r] for n2 in range(q)] for n1 in range(p)])
    a = np.array([_dft(row, sign) for row in a])
    a = np.array([_dft(a[:, n2], sign) for n2 in range(q)]).T
    return np.array([a[k % p, k % q] for k in range(r)])


def _dft_nat(v, sign):
    r = len(v)
    if r == 12:
        return _dft_pfa(v, 4, 3, sign)
    if r == 20:
        return _dft_pfa(v, 4, 5, sign)
    return _dft(v, sign)


def _four_step(x, ra, rb, tpl, sign, span):
    """Stage A then stage B on one line, with the kernel's owner loops and
    line layout; returns the output and the largest line position used."""
    n = ra * rb
    tw = np.exp(-2j * np.pi * np.arange(n) / n)
    line = np.full(span, np.nan + 0j)
    maxpos = 0
    for t in range(tpl):
        for j in range(rb // tpl):
            a = t + tpl * j
            v = _dft_nat(np.array([x[rb * i + a] for i in range(ra)]), sign)
            for k in range(ra):
                w = tw[a * k] if sign < 0 else np.conj(tw[a * k])
                pos = k * (rb + 1) + a
                maxpos = max(maxpos, pos)
                line[pos] = v[k] * w if k else v[k]
    out = np.full(n, np.nan + 0j)
    for t in range(tpl):
        for j in range(ra // tpl):
            k = t + tpl * j
            y = _dft_nat(np.array([line[k * (rb + 1) + a] for a in range(rb)]), sign)
            for m in range(rb):
                out[k + ra * m] = y[m]
    return out, maxpos


def test_header_lists_every_specialised_edge():
    assert sorted(_splits()) == [32, 48, 64, 80, 96, 128, 160, 256]


@pytest.mark.parametrize("n", [32, 48, 64, 80, 96, 128, 160, 256])
def test_four_step_line_matches_numpy(n):
    r1, r2, tpl = _splits()[n]
    assert r1 * r2 == n and r1 >= r2
    assert r1 % tpl == 0 and r2 % tpl == 0  # whole owners per thread
    span = n + r1  # line_span<N>() in the header
    x = np.random.default_rng(n).standard_normal(n) + 1j * np.random.default_rng(n + 1).standard_normal(n)
    fwd, m1 = _four_step(x, r1, r2, tpl, -1, span)
    assert m1 < span
    np.testing.assert_allclose(fwd, np.fft.fft(x), rtol=0, atol=1e-10 * np.abs(x).sum())
    # the inverse runs the radices swapped; unnormalised
    inv, m2 = _four_step(fwd, r2, r1, tpl, +1, span)
    assert m2 < span
    np.testing.assert_allclose(inv / n, x, rtol=0, atol=1e-12 * np.abs(x).sum())


@pytest.mark.parametrize("p,q", [(4, 3), (4, 5)])
def test_prime_factor_dft(p, q):
    v = np.random.default_rng(p * q).standard_normal(p * q) + 0.5j
    np.testing.assert_allclose(_dft_pfa(v, p, q, -1), np.fft.fft(v), atol=1e-12)
    np.testing.assert_allclose(_dft_pfa(v, p, q, +1), p * q * np.fft.ifft(v), atol=1e-12)


@pytest.mark.parametrize("n", [32, 48, 80, 160, 256])
def test_two_real_lines_separation_and_reconstruction(n):
    """k_fx_fwd: one complex FFT of z = a + i b gives both half spectra,
    A[k] = (Z[k] + conj Z[-k]) / 2 and B[k] = (Z[k] - conj Z[-k]) / (2i), for
    k = 0 .. N/2 + 1 (the last lands in the row padding).  k_fx_inv: Z[k] =
    A[k] + i B[k] below N/2 + 1 and conj A[N-k] + i conj B[N-k] above, with
    the DC and Nyquist imaginary parts dropped; the inverse FFT returns a and
    b as its real and imaginary parts."""
    rng = np.random.default_rng(n)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    Z = np.fft.fft(a + 1j * b)
    nh = n // 2 + 1
    A = np.empty(nh + 1, complex)
    B = np.empty(nh + 1, complex)
    for k in range(nh + 1):  # the kernel's pairs run to k = NH (even count)
        zk, zn = Z[k], Z[0 if k == 0 else n - k]
        A[k] = complex(0.5 * (zk.real + zn.real), 0.5 * (zk.imag - zn.imag))
        B[k] = complex(0.5 * (zk.imag + zn.imag), 0.5 * (zn.real - zk.real))
    np.testing.assert_allclose(A[:nh], np.fft.rfft(a), atol=1e-10)
    np.testing.assert_allclose(B[:nh], np.fft.rfft(b), atol=1e-10)
    # reconstruction from the stored half spectra (positions 0 .. N/2 only)
    Zr = np.empty(n, complex)
    for k in range(n):
        lo = k < nh
        kk = k if lo else n - k
        Ak, Bk = complex(A[kk]), complex(B[kk])
        if kk == 0 or 2 * kk == n:
            Ak, Bk = complex(Ak.real, 0.0), complex(Bk.real, 0.0)
        if not lo:
            Ak, Bk = Ak.conjugate(), Bk.conjugate()
        Zr[k] = complex(Ak.real - Bk.imag, Ak.imag + Bk.real)
    z = np.fft.ifft(Zr)
    np.testing.assert_allclose(z.real, a, atol=1e-12)
    np.testing.assert_allclose(z.imag, b, atol=1e-12)
