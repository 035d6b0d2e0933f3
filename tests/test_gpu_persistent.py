"""The persistent sweep (scft_set_persistent: one launch per sweep of a group
of 64 x 64 x 64 instances, CTAs taking plane and z-column tasks from a
counter) against the per-step launches (two launches per propagator step).

Each instance's arithmetic is the same in both schedules, so H, Q and the
densities must agree bit for bit: uneven chain lengths in one launch (the
instances active at step n are a prefix of the job order), odd and tiny N, a
single-block chain, two concurrent persistent groups, and the 64^3 group of a
batch of mixed grids.  The bounded dependency waits are checked by lowering
their limit to zero: the sweep stops, the call returns SCFT_ERR_CUDA, and the
context computes correctly again once its fields are set anew.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def batch(S, Ns, thetas=None, fA=0.5, grids=None):
    from scft.workloads import plate_params, seeded_fields

    thetas = thetas or [10.0 * k for k in range(len(Ns))]
    grids = grids or [(64, 64, 64)] * len(Ns)
    ps = [plate_params(t, N=N, fA=fA, grid=g, box_rg=tuple(6.4 * n / 64 for n in g), precision=S.PREC_MIXED)
          for t, N, g in zip(thetas, Ns, grids)]
    return ps, [seeded_fields(p, 60 + k) for k, p in enumerate(ps)]


def run(S, ps, fields, persistent, groups=1, iters=3):
    with S.Context(ps) as c:
        c.set_sweep_groups(groups, 1)
        c.set_persistent(persistent)
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        H0 = c.calc_H().copy()
        c.update_1s(iters)
        H = c.calc_H().copy()
        rho = [c.density(k)[:2] for k in range(len(ps))]
        sched = c.schedule()
        launches = c.launch_count()
    return H0, H, rho, sched, launches


@pytest.mark.parametrize("Ns,groups", [([16, 12, 12, 7], 1), ([2], 1), ([3, 2], 1), ([9, 9, 9], 2)])
def test_persistent_sweep_is_bit_identical(S, Ns, groups):
    ps, fields = batch(S, Ns)
    a = run(S, ps, fields, False, groups)
    b = run(S, ps, fields, True, groups)
    assert b[3]["persistent"] and not a[3]["persistent"]
    np.testing.assert_array_equal(a[0], b[0])
    np.testing.assert_array_equal(a[1], b[1])
    for (ra, rb), (qa, qb) in zip(a[2], b[2]):
        np.testing.assert_array_equal(ra, qa)
        np.testing.assert_array_equal(rb, qb)
    # one sweep launch per group and iteration instead of about two per step
    assert b[4] < a[4]


def test_persistent_single_block_chain(S):
    ps, fields = batch(S, [8, 8], fA=1.0)
    a = run(S, ps, fields, False)
    b = run(S, ps, fields, True)
    np.testing.assert_array_equal(a[1], b[1])


def test_persistent_group_of_a_mixed_grid_batch(S):
    ps, fields = batch(S, [10, 10, 8], grids=[(64, 64, 64), (64, 64, 64), (48, 48, 48)])
    a = run(S, ps, fields, False, groups=2)
    b = run(S, ps, fields, True, groups=2)
    np.testing.assert_array_equal(a[1], b[1])


def test_dependency_wait_that_runs_out_stops_the_sweep(S):
    ps, fields = batch(S, [12, 12])
    ref = run(S, ps, fields, True, iters=0)
    with S.Context(ps) as c:
        c.set_sweep_groups(1, 1)
        c.set_persistent(True)
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        c.update_1s(1)
        c.set_wait_limit(0)
        with pytest.raises(S.ScftError) as e:
            c.update_1s(1)
        assert e.value.code == S.ERR_CUDA and "ran out" in str(e.value)
        c.set_wait_limit(-1)
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        H = c.calc_H()
    np.testing.assert_array_equal(H, ref[0])


@pytest.mark.parametrize("case", ["uneven", "nz128", "single_block"])
def test_warp_local_plane_form_is_bit_identical(S, case):
    """The two forms of the 64-point plane pass (block-barrier exchanges and
    warp-local columns over the swizzled, asynchronously loaded plane) do the
    same arithmetic in the same order."""
    from scft.workloads import plate_params, seeded_fields

    if case == "uneven":
        ps, fields = batch(S, [14, 11, 11, 6])
    elif case == "single_block":
        ps, fields = batch(S, [8, 8], fA=1.0)
    else:
        ps = [plate_params(0.0, N=9, grid=(64, 64, 128), box_rg=(6.4, 6.4, 12.8), precision=S.PREC_MIXED,
                           centers=((0.5, 0.5, 0.4), (0.5, 0.5, 0.6)))]
        fields = [seeded_fields(ps[0], 71)]
    res = []
    for form in (0, 1):
        with S.Context(ps) as c:
            c.set_sweep_groups(2 if len(ps) > 1 else 1, 1)
            c.set_persistent(False)
            c.set_plane_form(form)
            for k, f in enumerate(fields):
                c.set_fields(k, f)
            c.calc_poly_density()
            c.update_1s(3)
            assert c.schedule()["plane_form"] == form
            res.append((c.calc_H().copy(), [c.density(k)[:2] for k in range(len(ps))]))
    np.testing.assert_array_equal(res[0][0], res[1][0])
    for (ra, rb), (qa, qb) in zip(res[0][1], res[1][1]):
        np.testing.assert_array_equal(ra, qa)
        np.testing.assert_array_equal(rb, qb)
