"""Plain FP64 method against the reference at the benchmark configurations'
full sizes: config 1 (one plate, 64^3, N=100), config 2's non-64^3 grids
(96 x 64 x 64 and 48^3, N=100, from the mixed-size sweep), config 3 (two
plates at d = 0.30 L_z, 64 x 64 x 128, N=100) and config 4 (two grafted
plates, 128 x 128 x 256, N=200, Ng=20).

The fixtures (tests/golden/config*_*.npz, make_golden.py --large) hold what
the compiled reference wrote after set-up and after a few update_1s() calls
from the seeded fields of the bench workloads: H and Q per iteration at full
precision, and digests (sum, sum of |.|^2, 512 sampled points) of the initial
and final densities, fields and smeared fields.  The test regenerates the
same seeded fields (checked against the fixture's digest of them), runs the
same iterations through the C ABI, and compares at the plain method's bars:
densities, fields and smeared fields 1e-10 relative, H 1e-9 relative.
"""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

RHO_TOL = 1e-10
H_TOL = 1e-9

LARGE = ["config1_plate64_N100", "config2_96x64x64_N100", "config2_48cubed_N100", "config3_sep030_64x64x128_N100",
         "config4_graft_128x128x256_N200"]


def digest_close(a, ref, tol, M):
    """A digest (make_golden.digest) against the reference's, each part on
    its own scale: the sampled points relative to the largest sampled value,
    sum |.|^2 relative, and the sum to tol * sqrt(M * sum |.|^2) (the sum of
    a field with zero mean is itself near zero)."""
    a, ref = np.asarray(a), np.asarray(ref)
    s_ok = abs(a[0] - ref[0]) <= tol * np.sqrt(M * abs(ref[1]))
    q_ok = abs(a[1] - ref[1]) <= tol * abs(ref[1])
    p_ok = np.abs(a[2:] - ref[2:]).max() <= tol * np.abs(ref[2:]).max()
    return bool(s_ok and q_ok and p_ok), (abs(a[0] - ref[0]), abs(a[1] - ref[1]) / abs(ref[1]),
                                          np.abs(a[2:] - ref[2:]).max() / np.abs(ref[2:]).max())


@pytest.fixture(scope="module")
def scft():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    S.load()
    return S


@pytest.mark.parametrize("name", LARGE)
def test_fp64_matches_reference_at_full_size(scft, name):
    import sys

    sys.path.insert(0, GOLDEN)
    from make_golden import digest, large_case

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    p, c, iters = large_case(name)
    ns = int(z["samples"])
    M = c.M
    # the regenerated seeded input is the one the reference ran on
    assert np.array_equal(digest(c.fields["wabm"], ns), z["digest_in_wabm"])
    tr = z["trace"]
    assert tr.shape[0] == iters + 1
    graft = c.sigma > 0 and c.n_exp_nr > 0
    with scft.Context(p) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        rows = [ctx.calc_H()[0].copy()]
        got = {}
        got["rhoda0"], got["rhodb0"], rg0 = ctx.density(0)
        got["smwa0"], got["smwb0"], _ = ctx.smeared(0)
        if graft:
            got["rhog_exp0"] = rg0
        for _ in range(iters):
            ctx.update_1s(1)
            rows.append(ctx.calc_H()[0].copy())
        f = ctx.get_fields(0)
        got["wpl"], got["wabp"], got["wabm"] = f["wpl"], f["wabp"], f["wabm"]
        got["rhoda"], got["rhodb"], rg = ctx.density(0)
        got["smwa"], got["smwb"], _ = ctx.smeared(0)
        if graft:
            got["rhog_exp"] = rg
    rows = np.array(rows)
    # H (Re and Im) and Q of the diblock after every iteration
    for col_ours, col_ref in ((0, 1), (2, 3)):
        err = np.abs(rows[:, col_ours] - tr[:, col_ref]) / np.abs(tr[:, col_ref])
        assert err.max() <= H_TOL, (name, col_ref, err)
    if graft:
        # Qga before the first update is 0 on both sides (the set-up's
        # density build does not form it)
        d = np.abs(rows[:, 4] - tr[:, 5])
        assert (d <= H_TOL * np.abs(tr[:, 5])).all(), (name, "Qga", rows[:, 4], tr[:, 5])
    for k, a in got.items():
        ok, parts = digest_close(digest(a, ns), z["digest_" + k], RHO_TOL, M)
        assert ok, (name, k, parts)
