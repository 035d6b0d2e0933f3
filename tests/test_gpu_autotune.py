"""The autotuner (scft_autotune): launch schedule (groups, phases, z-pass
columns, persistent sweep) and the stage order of the generic FFTs per axis
length.  Whatever it picks must leave the results within the mixed form's
FP32 bar of the FP64 method (2e-5 relative in H on these small grids), and
every FFT plan it reports must be a factorisation of its axis length into
the supported radices.
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


def test_autotuned_schedule_and_fft_plans_keep_results(S):
    from scft.workloads import plate_params, seeded_fields

    grids = [(64, 64, 64), (48, 48, 48), (40, 24, 30), (96, 64, 64)]
    Ns = [12, 10, 8, 6]

    def batch(prec):
        return [plate_params(10.0 * k, N=N, grid=g, box_rg=tuple(6.4 * n / 64 for n in g), precision=prec)
                for k, (g, N) in enumerate(zip(grids, Ns))]

    fields = [seeded_fields(p, 80 + k) for k, p in enumerate(batch(S.PREC_FP64))]
    with S.Context(batch(S.PREC_FP64)) as c:
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        c.update_1s(2)
        H64 = c.calc_H()[:, 0].copy()
    with S.Context(batch(S.PREC_MIXED)) as c:
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        sched = c.autotune(2)
        assert sched["groups"] >= 1 and sched["phases"] >= 1 and sched["ms_per_sweep"] > 0
        for k, g in enumerate(grids):
            for d in range(3):
                plan = c.fft_plan(k, d)
                assert int(np.prod(plan)) == g[d], (g, d, plan)
                assert set(plan) <= {2, 3, 4, 5, 8} and plan.count(2) <= 1 or plan == [2], plan
        for k, f in enumerate(fields):
            c.set_fields(k, f)
        c.calc_poly_density()
        c.update_1s(2)
        Hm = c.calc_H()[:, 0]
    assert np.abs(Hm - H64).max() <= 2e-5 * np.abs(H64).max(), (Hm, H64)
