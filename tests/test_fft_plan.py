"""The spectral solve's transform plan (msc-thesis_gb300/csrc/pic_fft_dev.cuh,
pic_spectral.cu) restated in numpy and checked against numpy's FFT on the
CPU: the radix plan, the per-thread butterfly mapping, the padded
shared-memory slots (every slot written once per pass), the per-pass
twiddle tables, the split of a packed pair of real rows and the Hermitian
extension of the inverse rows.  The GPU kernels themselves are checked in
test_gpu_spectral.py."""
import numpy as np
import pytest

E = 16  # elements per thread


def pass_lgr(lgn, lgns):
    return 4 if lgn - lgns >= 4 else lgn - lgns


def passes(lgn):
    out, lgns = [], 0
    while lgns < lgn:
        out.append((lgns, pass_lgr(lgn, lgns)))
        lgns += pass_lgr(lgn, lgns)
    return out


def twiddle_tables(lgn):
    """Per-pass tables as the host builds them: pass (lgns, lgr), lgns > 0,
    holds W_(Ns R)^(r m) at r Ns + m."""
    t = []
    for lgns, lgr in passes(lgn):
        if lgns == 0:
            continue
        R, Ns = 1 << lgr, 1 << lgns
        r, m = np.meshgrid(np.arange(R), np.arange(Ns), indexing="ij")
        t.append(np.exp(-2j * np.pi * (r * m).ravel() / (Ns * R)))
    return np.concatenate(t) if t else np.zeros(0, complex)


def pad(i):
    return i + (i >> 4)


def transform(x, inv=False):
    """One transform as the device runs it: thread t of n/16 holds 16
    elements; pass (lgns, lgr) gives thread t the butterflies j = t + b n/16,
    b < 16/R, with inputs j + r n/R; outputs go to (j / Ns) Ns R + (j mod Ns)
    + r Ns through padded slots."""
    n = len(x)
    lgn = n.bit_length() - 1
    tp = n >> 4
    tw = twiddle_tables(lgn)
    if inv:
        tw = np.conj(tw)
    buf = np.full(n + (n >> 4) + 8, np.nan, complex)
    # first pass inputs straight from the source: element t + k tp
    v = np.array([[x[t + k * tp] for k in range(E)] for t in range(tp)])
    off = 0
    plan = passes(lgn)
    for p, (lgns, lgr) in enumerate(plan):
        R, Ns = 1 << lgr, 1 << lgns
        if p > 0:
            v = np.array([[buf[pad(t + (k >> lgr) * tp + (k & (R - 1)) * (n >> lgr))]
                           for k in range(E)] for t in range(tp)])
        for t in range(tp):
            for b in range(E // R):
                j = t + b * tp
                u = v[t, b * R:(b + 1) * R].copy()
                if lgns > 0:
                    u = u * tw[off + np.arange(R) * Ns + (j & (Ns - 1))]
                u = np.fft.ifft(u) * R if inv else np.fft.fft(u)
                v[t, b * R:(b + 1) * R] = u
        if lgns > 0:
            off += R * Ns
        if p == len(plan) - 1:
            break
        buf[:] = np.nan
        written = set()
        for t in range(tp):
            for k in range(E):
                j, r = t + (k >> lgr) * tp, k & (R - 1)
                d = ((j >> lgns) << (lgns + lgr)) + (j & (Ns - 1)) + (r << lgns)
                assert pad(d) not in written
                written.add(pad(d))
                buf[pad(d)] = v[t, k]
        assert len(written) == n
    # result_index: t + (k / R) tp + (k mod R) n / R for the last pass's R
    lgr = plan[-1][1]
    out = np.empty(n, complex)
    for t in range(tp):
        for k in range(E):
            out[t + (k >> lgr) * tp + (k & ((1 << lgr) - 1)) * (n >> lgr)] = v[t, k]
    return out


def test_twiddle_table_lengths():
    # fft::twiddle_len: the tables of the passes after the first, back to back
    expect = {4: 0, 5: 32, 6: 64, 7: 128, 8: 256, 9: 256 + 512, 10: 256 + 1024,
              11: 256 + 2048, 12: 256 + 4096}
    for lgn, n in expect.items():
        assert len(twiddle_tables(lgn)) == n


@pytest.mark.parametrize("lgn", range(4, 13))
def test_transform_plan_matches_numpy(lgn):
    n = 1 << lgn
    rng = np.random.default_rng(lgn)
    x = rng.standard_normal(n) + 1j * rng.standard_normal(n)
    ref = np.fft.fft(x)
    assert np.abs(transform(x) - ref).max() < 1e-9 * np.abs(ref).max()
    ref_inv = np.fft.ifft(x) * n
    assert np.abs(transform(x, inv=True) - ref_inv).max() < 1e-9 * np.abs(ref_inv).max()


def test_packed_rows_and_hermitian_rows():
    """Forward rows: z = a + i b transformed once gives A_k = (Z_k + conj
    Z_-k)/2 and B_k = (Z_k - conj Z_-k)/2i; inverse rows: X + iY extended by
    Hermitian symmetry (imaginary parts at 0 and n/2 dropped) inverts to
    x + i y."""
    n = 64
    rng = np.random.default_rng(5)
    a, b = rng.standard_normal(n), rng.standard_normal(n)
    Z = transform(a + 1j * b)
    k = np.arange(n // 2 + 1)
    m = Z[(n - k) % n]
    A = 0.5 * (Z[k].real + m.real) + 0.5j * (Z[k].imag - m.imag)
    B = 0.5 * (Z[k].imag + m.imag) + 0.5j * (m.real - Z[k].real)
    assert np.allclose(A, np.fft.rfft(a)) and np.allclose(B, np.fft.rfft(b))
    X, Y = A.copy(), B.copy()
    for V in (X, Y):
        V[0], V[n // 2] = V[0].real, V[n // 2].real
    W = np.empty(n, complex)
    W[:n // 2 + 1] = X + 1j * Y
    kk = np.arange(1, n // 2)
    W[n - kk] = np.conj(X[kk]) + 1j * np.conj(Y[kk])
    z = transform(W, inv=True) / n
    assert np.allclose(z.real, a) and np.allclose(z.imag, b)
