"""The index arithmetic of the cluster plane passes, restated in numpy (CPU):
the 128 x 128 pass splits each plane into four 64 x 64 quadrants with
parity-major k-space axes (kernels_mixed128.cu), the 96 x 64 pass into three
32-column slabs with residue-major x (kernels_mixed96.cu); both close the
long transforms with one radix-2 / radix-3 step between CTAs.  The 32-point
transform of four threads (mix_core.cuh fft32_group) and the factor tables'
position orders are checked the same way.  Exact against numpy's FFT to
rounding."""
import numpy as np

rng = np.random.default_rng(0)


def test_parity_major_quadrants_invert_and_round_trip():
    X = rng.standard_normal((128, 128)) + 1j * rng.standard_normal((128, 128))  # [ky][kx]
    P = lambda k: (k % 2) * 64 + k // 2
    S = np.zeros_like(X)
    for ky in range(128):
        S[P(ky), [P(kx) for kx in range(128)]] = X[ky]
    tw = np.exp(-2j * np.pi * np.arange(128) / 128)
    Q = {(rx, ry): S[64 * ry:64 * ry + 64, 64 * rx:64 * rx + 64] for rx in (0, 1) for ry in (0, 1)}
    A = {q: np.fft.ifft(Q[q], axis=0) * 64 for q in Q}
    w = np.conj(tw[:64])
    T = {(rx, ry): (A[(rx, 0)] + w[:, None] * A[(rx, 1)]) if ry == 0 else (A[(rx, 0)] - w[:, None] * A[(rx, 1)])
         for (rx, ry) in Q}
    B = {q: np.fft.ifft(T[q], axis=1) * 64 for q in T}
    R = {(rx, ry): (B[(0, ry)] + w[None, :] * B[(1, ry)]) if rx == 0 else (B[(0, ry)] - w[None, :] * B[(1, ry)])
         for (rx, ry) in Q}
    full = np.block([[R[(0, 0)], R[(1, 0)]], [R[(0, 1)], R[(1, 1)]]])
    ref = np.fft.ifft2(X) * 128 * 128
    assert np.abs(full - ref).max() <= 1e-12 * np.abs(ref).max()
    # forward: decimation in frequency along x, then y
    F = {(rx, ry): (R[(0, ry)] + R[(1, ry)]) if rx == 0 else (R[(0, ry)] - R[(1, ry)]) * tw[:64][None, :]
         for (rx, ry) in R}
    F = {q: np.fft.fft(F[q], axis=1) for q in F}
    G = {(rx, ry): (F[(rx, 0)] + F[(rx, 1)]) if ry == 0 else (F[(rx, 0)] - F[(rx, 1)]) * tw[:64][:, None]
         for (rx, ry) in F}
    G = {q: np.fft.fft(G[q], axis=0) for q in G}
    S2 = np.block([[G[(0, 0)], G[(1, 0)]], [G[(0, 1)], G[(1, 1)]]])
    np.testing.assert_allclose(S2, S * 128 * 128, rtol=0, atol=1e-9 * np.abs(S).max() * 128 * 128)


def test_residue_major_slabs_invert_and_round_trip():
    X = rng.standard_normal((64, 96)) + 1j * rng.standard_normal((64, 96))  # [ky][kx]
    P = lambda k: (k % 3) * 32 + k // 3
    S = np.zeros_like(X)
    S[:, [P(k) for k in range(96)]] = X
    w96 = np.exp(-2j * np.pi * np.arange(96) / 96)
    C = {q: np.fft.ifft(np.fft.ifft(S[:, 32 * q:32 * q + 32], axis=0) * 64, axis=1) * 32 for q in range(3)}
    n = lambda i: 32 * i + np.arange(32)
    R = {i: sum(np.conj(w96[(n(i) * r) % 96])[None, :] * C[r] for r in range(3)) for i in range(3)}
    ref = np.fft.ifft2(X) * 64 * 96
    assert np.abs(np.hstack([R[0], R[1], R[2]]) - ref).max() <= 1e-12 * np.abs(ref).max()
    D = {q: np.fft.fft(sum(w96[(n(i) * q) % 96][None, :] * R[i] for i in range(3)), axis=1) for q in range(3)}
    S2 = np.hstack([np.fft.fft(D[q], axis=0) for q in range(3)])
    np.testing.assert_allclose(S2, S * 64 * 96, rtol=0, atol=1e-9 * np.abs(S).max() * 64 * 96)


def test_fft32_of_four_threads():
    x = rng.standard_normal(32) + 1j * rng.standard_normal(32)
    w32 = np.exp(-2j * np.pi * np.arange(32) / 32)
    Y = np.array([np.fft.fft(x[t::4]) * w32[(t * np.arange(8)) % 32] for t in range(4)])  # thread t: x[t + 4a]
    out = np.zeros(32, complex)
    for t in range(4):
        for c in (t, t + 4):
            out[c + 8 * np.arange(4)] = np.fft.fft(Y[:, c])
    np.testing.assert_allclose(out, np.fft.fft(x), atol=1e-12)


def test_factor_table_orders():
    """axis_h_table positions: parity-major (128) and residue-major (96)."""
    for n, r in ((128, 2), (96, 3)):
        h = n // r
        ks = [r * (pos % h) + pos // h for pos in range(n)]
        assert sorted(ks) == list(range(n))
        assert all((k % r) * h + k // r == pos for pos, k in enumerate(ks))


def test_fft48_of_four_threads():
    """fft48_group (mix_core.cuh): a DFT12 in registers (DFT4, twiddle
    w12^(n1 k2), DFT3), twiddle w48^(t c), exchange, three DFT4 per thread;
    thread t holds x[t + 4a] before and X[t + 4j] after."""
    tw48 = np.exp(-2j * np.pi * np.arange(48) / 48)

    def dft12(v):
        u = [np.fft.fft([v[n1 + 3 * n2] for n2 in range(4)]) for n1 in range(3)]
        for n1 in (1, 2):
            for k2 in (1, 2, 3):
                u[n1][k2] *= tw48[4 * n1 * k2]
        out = np.zeros(12, complex)
        for k2 in range(4):
            out[k2 + 4 * np.arange(3)] = np.fft.fft([u[0][k2], u[1][k2], u[2][k2]])
        return out

    x = rng.standard_normal(48) + 1j * rng.standard_normal(48)
    Y = np.array([dft12(x[t::4]) * tw48[(t * np.arange(12)) % 48] for t in range(4)])
    out = np.zeros(48, complex)
    for t in range(4):
        v = np.zeros(12, complex)
        for e in range(3):
            p = np.fft.fft(Y[:, t + 4 * e])
            v[e + 3 * np.arange(4)] = p
        out[t + 4 * np.arange(12)] = v
    np.testing.assert_allclose(out, np.fft.fft(x), atol=1e-12)
