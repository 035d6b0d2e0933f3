"""The headline accuracy bar at full size: the batched mixed form against the
plain FP64 method at 64^3, N=100 (the 15-angle sweep's grid and chain), and
the geometric derivatives against finite differences at config-1 and config-3
sizes.

* |dH| / |H| <= 1e-6 between the two forms after the same 25 iterations from
  the same near-saddle fields (500 mixed-form iterations from the seeded
  start; the bench's own protocol), for three angles in one batch.
* dH/dtheta, dH/dc of the mixed form within 1e-4 (relative to the largest
  component) of the FP64 method's, and of a central difference of the FP64
  H at fixed fields (h = 1e-3 rad; 1e-4 of the plate spacing).
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DH_REL = 1e-6
GRAD_REL = 1e-4


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def relaxed(S, params_mixed, fields, iters=500):
    with S.Context(params_mixed) as c:
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        c.update_1s(iters)
        return [c.get_fields(k) for k in range(len(fields))]


def run(S, params, fields, iters):
    with S.Context(params) as c:
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        if iters:
            c.update_1s(iters)
        H = c.calc_H()[:, 0].copy()
        g = c.grad_geom()
        out = [c.get_fields(k) for k in range(len(fields))]
    return H, g, out


def test_mixed_form_meets_the_headline_bar_at_64cubed_N100(S):
    from scft.workloads import plate_params, seeded_fields

    thetas = (0.0, 10.0, 45.0)
    pm = [plate_params(t, precision=S.PREC_MIXED) for t in thetas]
    p64 = [plate_params(t, precision=S.PREC_FP64) for t in thetas]
    fields = relaxed(S, pm, [seeded_fields(p, 1000 + k) for k, p in enumerate(pm)])
    Hm, gm, _ = run(S, pm, fields, 25)
    H64, g64, f64 = run(S, p64, fields, 25)
    dH = np.abs(Hm - H64) / np.abs(H64)
    assert dH.max() <= DH_REL, dH
    for k in range(len(thetas)):
        a, b = gm[k, 0], g64[k, 0]
        assert np.abs(a - b).max() <= GRAD_REL * np.abs(b).max(), (k, a, b)
    # dH/dtheta of the mixed form against a central difference of the FP64
    # H at fixed fields (the FP64 method's fields after the 25 iterations)
    k, h = 1, 1e-3
    Hp, _, _ = run(S, [plate_params(thetas[k] + math.degrees(h), precision=S.PREC_FP64)], [f64[k]], 0)
    Hmn, _, _ = run(S, [plate_params(thetas[k] - math.degrees(h), precision=S.PREC_FP64)], [f64[k]], 0)
    _, g0, _ = run(S, [plate_params(thetas[k], precision=S.PREC_MIXED)], [f64[k]], 0)
    fd = (Hp[0] - Hmn[0]) / (2 * h)
    assert abs(g0[0, 0, 0] - fd) <= GRAD_REL * max(abs(fd), np.abs(g0[0, 0]).max()), (g0[0, 0, 0], fd)


def test_separation_derivative_at_config3_size(S):
    """Config 3's geometry (two plates, 64 x 64 x 128, N=100, separation
    along z): dH/dd of the mixed form against a central difference of the
    FP64 H at fixed near-saddle fields, h = 1e-4 of L_z."""
    from scft.workloads import plate_params, seeded_fields

    def two(d, prec):
        return plate_params(0.0, grid=(64, 64, 128), box_rg=(6.4, 6.4, 12.8), precision=prec,
                            centers=((0.5, 0.5, 0.5 - d / 2), (0.5, 0.5, 0.5 + d / 2)))

    d, h = 0.30, 1e-4
    f = relaxed(S, [two(d, S.PREC_MIXED)], [seeded_fields(two(d, S.PREC_MIXED), 1004)], 300)
    _, gm, _ = run(S, [two(d, S.PREC_MIXED)], f, 0)
    _, g64, _ = run(S, [two(d, S.PREC_FP64)], f, 0)
    Hp, _, _ = run(S, [two(d + h, S.PREC_FP64)], f, 0)
    Hn, _, _ = run(S, [two(d - h, S.PREC_FP64)], f, 0)
    fd = (Hp[0] - Hn[0]) / (2 * h)  # per unit of d (fractions of L_z)
    Lz = two(d, S.PREC_FP64).L[2]
    an_m = Lz * (gm[0, 1, 3] - gm[0, 0, 3]) / 2
    an_64 = Lz * (g64[0, 1, 3] - g64[0, 0, 3]) / 2
    assert abs(an_64 - fd) <= GRAD_REL * abs(fd), (an_64, fd)
    assert abs(an_m - fd) <= GRAD_REL * abs(fd), (an_m, fd)
