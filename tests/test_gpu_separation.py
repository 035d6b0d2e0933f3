"""dH/d(separation) against the reference's own converged separation sweep.

The fixture (tests/golden/separation_sweep_16x16x32_N16.npz, make_golden.py
--separation) holds H after the reference converged each of seven
separations of two coplanar grafted-free discs independently from one seeded
field (16 x 16 x 32 grid, N = 16; H changes by ~1e-11 per iteration at the
end): d = 0.36 .. 0.52 of L_z in steps of 0.04, and 0.44 -+ 0.002.  The
reference has no derivative; its sweeps (particle-separation/) difference
converged H the same way.

* The FP64 method runs the same iterations from the same field and must land
  on the reference's converged H (1e-9 relative).
* At a converged saddle point dH/dd from scft_grad_geom is the total
  derivative of H(d) (envelope theorem): against the reference's central
  difference at d = 0.44 (h = 0.002 of L_z, 1e-4 relative), and its Simpson
  integral over 0.36 .. 0.52 against the reference's H(0.52) - H(0.36).
* The mixed form converged the same way gives the same derivative within its
  FP32 bar (1e-4 of the central difference).
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def converged_sweep(S, prec):
    sys.path.insert(0, GOLDEN)
    from make_golden import separation_fields, separation_params

    z = np.load(os.path.join(GOLDEN, "separation_sweep_16x16x32_N16.npz"))
    ds = [float(d) for d in z["d"]]
    ps = [separation_params(d, prec) for d in ds]
    with S.Context(ps) as c:
        for k, p in enumerate(ps):
            c.set_fields(k, separation_fields(p))
        c.calc_poly_density()
        c.update_1s(int(z["iters"]))
        H = c.calc_H()[:, 0].copy()
        g = c.grad_geom()
    Lz = ps[0].L[2]
    dHdd = Lz * (g[:, 1, 3] - g[:, 0, 3]) / 2  # per unit of d (fractions of L_z)
    return z, ds, H, dHdd


def simpson(f, h):
    return h / 3 * (f[0] + 4 * f[1] + 2 * f[2] + 4 * f[3] + f[4])


def test_fp64_separation_derivative_against_reference_sweep(S):
    z, ds, H, dHdd = converged_sweep(S, S.PREC_FP64)
    Href = z["H"]
    assert np.abs(H - Href).max() <= 1e-9 * np.abs(Href).max(), H - Href
    i44, im, ip = ds.index(0.44), ds.index(0.438), ds.index(0.442)
    fd = (Href[ip] - Href[im]) / (ds[ip] - ds[im])
    assert abs(dHdd[i44] - fd) <= 1e-4 * abs(fd), (dHdd[i44], fd)
    dH_ref = Href[ds.index(0.52)] - Href[ds.index(0.36)]
    integral = simpson(dHdd[:5], 0.04)
    assert abs(integral - dH_ref) <= 1e-3 * np.abs(dHdd[:5]).max() * 0.16, (integral, dH_ref)


def test_mixed_separation_derivative_against_reference_sweep(S):
    z, ds, H, dHdd = converged_sweep(S, S.PREC_MIXED)
    Href = z["H"]
    im, ip = ds.index(0.438), ds.index(0.442)
    fd = (Href[ip] - Href[im]) / (ds[ip] - ds[im])
    assert abs(dHdd[ds.index(0.44)] - fd) <= 1e-4 * abs(fd), (dHdd[ds.index(0.44)], fd)
