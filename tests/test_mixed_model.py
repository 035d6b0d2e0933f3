"""The mixed form's arithmetic contract, modelled in numpy on the CPU.

The mixed form advances q and qdag together as one FP32 complex field
z = q + i qdag with FP32 transforms, applies the bond factor as z - h z with
h = 1 - gx gy gz built from per-axis tables, carries each step's mean in FP64
(the k = 0 term dropped from the FP32 transform and added back) and rescales
every step by a power of two from that mean, folding the exponents into the
FP64 density sums and Q.  This file restates that scheme in numpy (complex64
FFTs) and checks it against the FP64 restatement of the reference
(oracle/scft_oracle.py: diblock_discrete, integrate_diblock_discrete): the
scheme, not only the CUDA kernels that implement it, has to meet the FP32
bar, including a case whose Q (~1e53) is far outside the FP32 range, which
only the rescaling makes representable.  The CUDA kernels themselves are
checked against the FP64 method on the GPU (test_gpu_mixed.py).
"""
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for _p in (ROOT, os.path.join(ROOT, "oracle"), os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

MODEL_TOL = 1e-4  # relative, Q and densities (FP32 transforms, N <= 200 steps)


def mixed_sweep_model(s, wa, wb, rescale=True):
    """Q, rho_A, rho_B of a diblock from smeared fields wa, wb (real), by the
    mixed form's scheme with FP32 storage and transforms."""
    g, N, Na = s.g, s.N, s.Nda
    hd = [(-np.expm1(-k * k / 6.0)).astype(np.float32) for k in (g.kvec_1d(d) for d in range(3))]
    hx, hy, hz = hd[0][None, None, :], hd[1][None, :, None], hd[2][:, None, None]
    hxy = hx + hy - hx * hy
    h = (hxy + hz - hxy * hz).astype(np.float32)
    EA = np.exp(-wa).astype(np.float32)
    EB = np.exp(-wb).astype(np.float32)
    z, K = [], np.zeros((2, N), int)
    for n in range(N):
        Eq = EA if (Na > 0 and n < Na) else EB
        Ed = EB if n <= N - Na - 1 else EA
        if n == 0:
            z.append((Eq + 1j * Ed).astype(np.complex64))
            continue
        prev = z[-1]
        mq, md = prev.real.astype(np.float64).mean(), prev.imag.astype(np.float64).mean()
        eq = int(np.frexp(mq)[1]) if rescale else 0
        ed = int(np.frexp(md)[1]) if rescale else 0
        Z = np.fft.fftn(prev)
        assert Z.dtype == np.complex64
        Z[0, 0, 0] = 0  # the mean goes around the FP32 transform in FP64
        Z = (Z - (h * Z).astype(np.complex64)).astype(np.complex64)
        v = np.fft.ifftn(Z).astype(np.complex64)
        qr = ((v.real.astype(np.float64) + mq) * Eq * 2.0 ** -eq).astype(np.float32)
        qi = ((v.imag.astype(np.float64) + md) * Ed * 2.0 ** -ed).astype(np.float32)
        z.append((qr + 1j * qi).astype(np.complex64))
        K[0, n], K[1, n] = K[0, n - 1] + eq, K[1, n - 1] + ed
    Q = z[N - 1].real.astype(np.float64).mean() * 2.0 ** K[0, N - 1]
    ra, rb = np.zeros(g.shape), np.zeros(g.shape)
    for j in range(N):
        t = z[j].real.astype(np.float64) * z[N - 1 - j].imag.astype(np.float64) * 2.0 ** (K[0, j] + K[1, N - 1 - j])
        if Na > 0 and j < Na:
            ra += t
        else:
            rb += t
    f = s.nD / Q / g.V
    return Q, ra * np.exp(wa) * f, rb * np.exp(wb) * f


def reference_case(grid, N, shift):
    import scft_oracle as O
    from ref_case import case_from_params
    from scft.workloads import plate_params, seeded_fields

    p = plate_params(10.0, N=N, grid=grid)
    c = case_from_params(p, seeded_fields(p, 7))
    s = O.System.from_case(c)
    o = O.calc_poly_density(s, O.State.from_fields(s.g, c.fields))
    wa = (o["smwa"] + s.tables["shellU"]).real - shift
    wb = o["smwb"].real - shift
    Qd, q, qd = O.diblock_discrete(s, wa.astype(np.complex128), wb.astype(np.complex128))
    ra, rb = O.integrate_diblock_discrete(s, q, qd, Qd, s.nD, wa, wb)
    return s, wa, wb, Qd.real, ra.real, rb.real


@pytest.mark.parametrize("grid,N,shift", [((32, 32, 32), 32, 0.0), ((24, 24, 24), 100, 0.0),
                                          ((24, 24, 24), 200, 0.6)])
def test_mixed_scheme_meets_the_fp32_bar(grid, N, shift):
    s, wa, wb, Q64, ra64, rb64 = reference_case(grid, N, shift)
    Q, ra, rb = mixed_sweep_model(s, wa, wb)
    peak = np.abs(ra64 + rb64).max()
    assert abs(Q - Q64) <= MODEL_TOL * abs(Q64), (Q, Q64)
    assert np.abs(ra - ra64).max() <= MODEL_TOL * peak
    assert np.abs(rb - rb64).max() <= MODEL_TOL * peak


def test_power_of_two_rescaling_keeps_a_huge_q_in_range():
    # a uniform shift of -0.6 per segment multiplies Q by e^{0.6 N} (~1e53 at N = 200)
    s, wa, wb, Q64, _, _ = reference_case((24, 24, 24), 200, 0.6)
    assert Q64 > 1e50
    with np.errstate(all="ignore"):
        Q_plain, _, _ = mixed_sweep_model(s, wa, wb, rescale=False)
    assert not np.isfinite(Q_plain)  # FP32 alone overflows
    Q, _, _ = mixed_sweep_model(s, wa, wb)
    assert abs(Q - Q64) <= MODEL_TOL * Q64
