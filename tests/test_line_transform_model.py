"""CPU model of the register line transform's index algebra, checked against
the transform definitions (scipy) in double precision.

The CUDA line kernels (`csrc/poisson_impl.cuh`, `csrc/regfft.cuh`) transform
two real lines at once as one complex sequence z = a + i b. This file
restates, in numpy, the steps those kernels take, with the same index maps:

* the half-length DCT-I input step (`dct_half_pre`): length N + 1 lines become
  y_m = s_m / 2 - sin(pi m / N) d_m with s_m = x_m + x_{N-m},
  d_m = x_m - x_{N-m}, and the partial X_1 = sum d_m cos(pi m / N). Each
  thread forms sin / cos(pi m / N) from its angle pi t / N and pi n1 / N1
  by the angle-addition formulas;
* the four-step FFT of length L = N1 N2 (`reg_fft_core`):
  1. thread t holds x[n1] = z[n1 N2 + t];
  2. a length-N1 DFT runs on the radix-2 / radix-3 recursion (`RegDft`);
  3. the twiddles W_L^(t k1) are applied;
  4. a padded transpose follows;
  5. length-N2 DFTs leave register r N2 + k2 of thread t holding
     Z[t + r N2 + N1 k2];
* the output step (`dct_half_output`):
  - the mirror Z_{N-k} is taken from lane N2 - t;
  - the even outputs are X_{2k} = Z_k + Z_{N-k};
  - the odd increments are D_k = i (Z_k - Z_{N-k});
  - a blocked running sum goes over C = N1 / 2 values per lane, with an
    exclusive scan of the block totals across the lanes.
* the real-DFT pair (periodic axes):
  - the forward store splits the pair's spectrum into FFTW's half-complex
    order;
  - the inverse rebuilds Z_k = A_k + i B_k from two half-complex lines
    (`reg_input`) and runs the sign +1 transform as conj(FFT(conj z));
  - the fused z sweep scales each line's spectrum by its 1/lambda row
    pairwise in (m, L - m) (`reg_eig_row`).

The kernels are checked against the oracle on the GPU. This model checks the
algorithm and its index maps for every register shape the library builds,
with no GPU. That includes the 384- and 768-point shapes on the radix-3
base, whose DCT-I lines are config 5's 769 points.
"""
import os
import subprocess
import sys

import numpy as np
import pytest

from conftest import PKG

scipy_fft = pytest.importorskip("scipy.fft")

# (N1, N2) register shapes of the library's line kernels (MIFGPU_REG_SHAPES)
SHAPES = [(8, 8), (16, 8), (16, 16), (32, 16), (32, 32), (48, 8), (48, 16)]


def reg_dft(x):
    """Forward DFT along the last axis by the kernels' recursion: radix-2
    splits down to a 2- or 3-point base (`RegDft`, sign -1)."""
    n = x.shape[-1]
    if n == 2:
        return np.stack([x[..., 0] + x[..., 1], x[..., 0] - x[..., 1]], axis=-1)
    if n == 3:
        c, s = -0.5, -np.sin(2 * np.pi / 3)
        a, b, d = x[..., 0], x[..., 1], x[..., 2]
        sm, df = b + d, b - d
        mid = a + c * sm
        # x1 = mid + i s (b - d), x2 = mid - i s (b - d)
        return np.stack([a + sm, mid + 1j * s * df, mid - 1j * s * df], axis=-1)
    e = reg_dft(x[..., 0::2])
    o = reg_dft(x[..., 1::2])
    w = np.exp(-2j * np.pi * np.arange(n // 2) / n)
    return np.concatenate([e + w * o, e - w * o], axis=-1)


def four_step(z, n1, n2):
    """`reg_fft_core` without the store: returns regs[t, r*N2 + k2]."""
    L = n1 * n2
    t = np.arange(n2)
    x = np.stack([z[k * n2 + t] for k in range(n1)], axis=1)  # x[t, n1]
    x = reg_dft(x)
    x = x * np.exp(-2j * np.pi * np.outer(t, np.arange(n1)) / L)  # W_L^(t k1)
    R = n1 // n2
    regs = np.empty((n2, n1), dtype=complex)
    for tt in range(n2):
        for r in range(R):
            k1 = tt + r * n2
            # the transpose: row[k1 (N2+1) + n2] read back by thread tt
            regs[tt, r * n2:(r + 1) * n2] = reg_dft(x[:, k1])
    return regs


def dct1_pair(a, b, n1, n2):
    """DCT-I (REDFT00, unnormalised) of the two length N+1 lines a, b by
    the kernels' half-length algorithm; returns (X_a, X_b)."""
    N = n1 * n2
    m = np.arange(N)
    xm, xn = a[m] + 1j * b[m], a[N - m] + 1j * b[N - m]
    # per thread t, n1: sin / cos(pi m / N) by angle addition
    t, k1 = m % n2, m // n2
    st, ct = np.sin(np.pi * t / N), np.cos(np.pi * t / N)
    sp, cp = np.sin(np.pi * k1 / n1), np.cos(np.pi * k1 / n1)
    sn, cs = st * cp + ct * sp, ct * cp - st * sp
    # packed on the pair: both lines take the same real arithmetic
    sm, d = xm + xn, xm - xn
    v = 0.5 * sm - sn * d
    x1 = np.sum(cs * d)  # per-thread partials reduced across the lanes
    regs = four_step(v, n1, n2)

    C, R = n1 // 2, n1 // n2

    def reg(c):
        return (c % R) * n2 + c // R

    ev = np.empty((n2, C), dtype=complex)
    scratch = np.empty(N // 2, dtype=complex)
    for tt in range(n2):
        partner = (n2 - tt) % n2
        for c in range(C):
            zk = regs[tt, reg(c)]
            zn = regs[partner, reg(n1 - 1 - c)]
            if tt == 0:
                zn = zk if c == 0 else regs[0, reg(n1 - c)]
            ev[tt, c] = zk + zn
            d_k = 0j if (c == 0 and tt == 0) else 1j * (zk - zn)
            scratch[c * n2 + tt] = d_k
    # blocked running sums over k = t C + c, then the block offsets
    blocks = scratch.reshape(n2, C)
    run = np.cumsum(blocks, axis=1)
    incl = np.cumsum(run[:, -1])
    excl = np.concatenate([[0j], incl[:-1]])
    odd = (x1 + excl[:, None] + run).reshape(-1)  # X_{2k+1}, k = 0..N/2-1
    out = np.empty(N + 1, dtype=complex)
    for tt in range(n2):
        for c in range(C):
            k = c * n2 + tt
            out[2 * k] = ev[tt, c]
            out[2 * k + 1] = odd[k]
    out[N] = 2 * regs[0, reg(C)]  # Z_{N/2} on lane 0
    return out.real, out.imag


def natural(regs, n1, n2):
    """`reg_fft_core`'s store: row[t + r N2 + N1 k2] = regs[t, r N2 + k2]."""
    out = np.empty(n1 * n2, dtype=complex)
    for t in range(n2):
        for r in range(n1 // n2):
            for k2 in range(n2):
                out[t + r * n2 + n1 * k2] = regs[t, r * n2 + k2]
    return out


def r2hc_pair(a, b, n1, n2):
    """Forward real DFT of the pair in FFTW's half-complex order: the
    spectrum X of a + i b split on the way out (the line kernel's store for
    a forward real-DFT sweep)."""
    L = n1 * n2
    x = natural(four_step(a + 1j * b, n1, n2), n1, n2)
    m = np.arange(L)
    xm, xn = x[m], x[np.where(m == 0, 0, L - m)]
    low = 2 * m <= L
    ha = np.where(low, (xm.real + xn.real) / 2, (xn.imag - xm.imag) / 2)
    hb = np.where(low, (xm.imag + xn.imag) / 2, (xm.real - xn.real) / 2)
    return ha, hb


def merge_pair(ha, hb):
    """`reg_input` for HC2R: Z_m = A_m + i B_m from two half-complex lines."""
    L = ha.size
    h = ha + 1j * hb  # row[m] = (a_hc[m], b_hc[m])
    z = h.copy()
    for m in range(1, L):
        if 2 * m == L:
            continue
        if 2 * m < L:
            hk, hm = h[m], h[L - m]
            z[m] = (hk.real - hm.imag) + 1j * (hm.real + hk.imag)
        else:
            hk, hm = h[L - m], h[m]
            z[m] = (hk.real + hm.imag) + 1j * (hk.imag - hm.real)
    return z


def inverse_pair(z, n1, n2, scale):
    """The sign +1 transform as conj(FFT(conj z)), scaled on the store."""
    x = natural(four_step(np.conj(z), n1, n2), n1, n2)
    x = np.conj(x) * scale
    return x.real, x.imag


def eig_pair(x, ea, eb):
    """`reg_eig_row`: eig_a A_m + i eig_b B_m on the natural-order spectrum X
    of the pair, with A = (X_m + conj X_-m)/2, B = (X_m - conj X_-m)/(2i)."""
    L = x.size
    out = np.empty_like(x)
    for m in range(L // 2 + 1):
        mn = 0 if m == 0 else L - m
        xm, xn = x[m], x[mn]
        for i, j, p, q in ((m, m, xm, xn), (mn, mn, xn, xm)):
            ga, gb = ea[j] / 2, eb[j] / 2
            out[i] = (ga * (p.real + q.real) + gb * (p.real - q.real)) + 1j * (
                ga * (p.imag - q.imag) + gb * (p.imag + q.imag))
    return out


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_four_step_register_map_is_the_dft(n1, n2):
    rng = np.random.default_rng(1000 + n1 * n2)
    L = n1 * n2
    z = rng.standard_normal(L) + 1j * rng.standard_normal(L)
    got = natural(four_step(z, n1, n2), n1, n2)
    ref = np.fft.fft(z)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def halfcomplex(x):
    """R2HC by its definition: r_0..r_{n/2}, i_{(n+1)/2-1}..i_1 of the DFT
    with exponent sign -1."""
    n = x.size
    X = np.fft.fft(x)
    hc = np.empty(n)
    for m in range(n):
        hc[m] = X[m].real if 2 * m <= n else X[n - m].imag
    return hc


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_real_dft_pair_matches_r2hc_and_inverts(n1, n2):
    rng = np.random.default_rng(4000 + n1 * n2)
    L = n1 * n2
    a, b = rng.standard_normal(L), rng.standard_normal(L)
    ha, hb = r2hc_pair(a, b, n1, n2)
    for h, x in ((ha, a), (hb, b)):
        ref = halfcomplex(x)
        assert np.abs(h - ref).max() <= 1e-12 * np.abs(ref).max()
    # HC2R of the half-complex pair, normalised by 1/L as the inverse sweeps do
    ra, rb = inverse_pair(merge_pair(ha, hb), n1, n2, 1.0 / L)
    assert np.abs(ra - a).max() <= 1e-12 and np.abs(rb - b).max() <= 1e-12


@pytest.mark.parametrize("n1,n2", [(16, 8), (32, 16)])
def test_periodic_forward_eig_inverse_pair(n1, n2):
    """The fused z sweep on a periodic axis: forward, each line's 1/lambda
    row (even in m, as the periodic eigenvalues are), inverse; per line the
    circular solve ifft(e * fft(x))."""
    rng = np.random.default_rng(5000 + n1 * n2)
    L = n1 * n2
    a, b = rng.standard_normal(L), rng.standard_normal(L)
    m = np.arange(L)
    lam = 2 * (np.cos(2 * np.pi * np.minimum(m, L - m) / L) - 1)  # exactly even in m
    ea = np.where(m == 0, 0.0, 1.0 / np.where(m == 0, 1.0, lam))  # zero mode: 0
    eb = 1.0 / (lam - 1.25)
    x = natural(four_step(a + 1j * b, n1, n2), n1, n2)
    ra, rb = inverse_pair(eig_pair(x, ea, eb), n1, n2, 1.0 / L)
    for r, line, e in ((ra, a, ea), (rb, b, eb)):
        ref = np.fft.ifft(e * np.fft.fft(line)).real
        assert np.abs(r - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n1,n2", SHAPES)
def test_half_length_dct1_pair_matches_redft00(n1, n2):
    rng = np.random.default_rng(2000 + n1 * n2)
    N = n1 * n2
    a = rng.standard_normal(N + 1)
    b = rng.standard_normal(N + 1)
    xa, xb = dct1_pair(a, b, n1, n2)
    for x, ref in ((xa, scipy_fft.dct(a, type=1)), (xb, scipy_fft.dct(b, type=1))):
        assert np.abs(x - ref).max() <= 1e-12 * np.abs(ref).max()


@pytest.mark.parametrize("n1,n2", [(16, 16), (48, 16)])
def test_half_length_dct1_pair_inverts(n1, n2):
    """REDFT00 is its own inverse up to the factor 2N, the normalisation of
    the inverse sweeps."""
    rng = np.random.default_rng(3000 + n1 * n2)
    N = n1 * n2
    a = rng.standard_normal(N + 1)
    b = rng.standard_normal(N + 1)
    xa, xb = dct1_pair(a, b, n1, n2)
    ra, rb = dct1_pair(xa, xb, n1, n2)
    assert np.abs(ra / (2 * N) - a).max() <= 1e-12
    assert np.abs(rb / (2 * N) - b).max() <= 1e-12


def test_twiddle_header_matches_its_generator():
    """`twiddle192.cuh` is the committed output of `gen_twiddle192.py`."""
    pytest.importorskip("mpmath")
    csrc = os.path.join(PKG, "csrc")
    out = subprocess.run([sys.executable, os.path.join(csrc, "gen_twiddle192.py")], check=True,
                         capture_output=True, text=True).stdout
    with open(os.path.join(csrc, "twiddle192.cuh")) as f:
        assert f.read() == out
