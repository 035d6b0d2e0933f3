"""dH/d(separation) against the reference's own converged separation sweep.

The fixture (tests/golden/separation_sweep_16x16x32_N16.npz, make_golden.py
--separation) holds H after the reference converged each separation of two
coplanar discs independently from one seeded field (16 x 16 x 32 grid,
N = 16; H changes by ~1e-11 per iteration at the end): d = 0.36 .. 0.52 of
L_z in steps of 0.04, and 0.44 -+ 0.002, 0.001, 0.0005.  The reference has no
derivative; its sweeps (particle-separation/) difference converged H the
same way.

On this coarse grid H(d) carries a ripple of period 1/16 of L_z in d (the
plate centres move by d/2 against a 1/32 grid), so differences need a small
step: the central difference at h = 0.0005 and 0.001 is extrapolated
(Richardson) to h -> 0.

* The FP64 method runs the same iterations from the same field and must land
  on the reference's converged H (1e-9 relative).
* At a converged saddle point dH/dd from scft_grad_geom is the total
  derivative of H(d) (envelope theorem): against the reference's
  extrapolated central difference at d = 0.44 (1e-4 relative, both forms),
  and, integrated (Simpson) over 17 separations the GPU converged between
  0.40 and 0.44, against the reference's H(0.44) - H(0.40) (1e-4 of the
  integral of |dH/dd|).
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FIXTURE = "separation_sweep_16x16x32_N16.npz"


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def converge(S, ds, prec, iters):
    """Converged H and dH/dd (per unit of d, fractions of L_z) of each d."""
    sys.path.insert(0, GOLDEN)
    from make_golden import separation_fields, separation_params

    ps = [separation_params(d, prec) for d in ds]
    with S.Context(ps) as c:
        for k, p in enumerate(ps):
            c.set_fields(k, separation_fields(p))
        c.calc_poly_density()
        c.update_1s(iters)
        H = c.calc_H()[:, 0].copy()
        g = c.grad_geom()
    Lz = ps[0].L[2]
    return H, Lz * (g[:, 1, 3] - g[:, 0, 3]) / 2


def reference_derivative(z, d0=0.44):
    """Richardson-extrapolated central difference of the reference's H."""
    ds = [round(float(d), 6) for d in z["d"]]
    H = dict(zip(ds, z["H"]))

    def cd(h):
        return (H[round(d0 + h, 6)] - H[round(d0 - h, 6)]) / (2 * h)

    return (4 * cd(0.0005) - cd(0.001)) / 3, cd(0.0005), cd(0.002)


def simpson(f, h):
    return h / 3 * (f[0] + f[-1] + 4 * f[1:-1:2].sum() + 2 * f[2:-1:2].sum())


@pytest.mark.parametrize("prec", [0, 1])
def test_separation_derivative_against_reference_sweep(S, prec):
    z = np.load(os.path.join(GOLDEN, FIXTURE))
    iters = int(z["iters"])
    ds = [float(d) for d in z["d"]]
    H, dHdd = converge(S, ds, prec, iters)
    if prec == 0:
        assert np.abs(H - z["H"]).max() <= 1e-9 * np.abs(z["H"]).max(), H - z["H"]
    D, D5, D20 = reference_derivative(z)
    g44 = dHdd[ds.index(0.44)]
    assert abs(g44 - D) <= 1e-4 * abs(D), (g44, D, D5, D20)


def test_integrated_derivative_matches_reference_delta_h(S):
    z = np.load(os.path.join(GOLDEN, FIXTURE))
    Href = dict(zip([round(float(d), 6) for d in z["d"]], z["H"]))
    fine = 0.40 + 0.0025 * np.arange(17)
    _, dHdd = converge(S, list(fine), 0, int(z["iters"]))
    integral = simpson(dHdd, 0.0025)
    dH = Href[0.44] - Href[0.4]
    scale = simpson(np.abs(dHdd), 0.0025)
    assert abs(integral - dH) <= 1e-4 * scale, (integral, dH, scale)
