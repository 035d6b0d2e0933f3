"""Failure detection through the C ABI on the GPU, without a GPU fault.

* H = NaN: a NaN in a host field buffer runs through the sweep (no index or
  loop bound depends on a value) and scft_calc_H returns SCFT_ERR_NAN, where
  the reference exits 1 (code/calc_h.cpp:38-61).
* q_g[Ng-1] <= 0 at 5 or more points: SCFT_ERR_QNONPOS, where the reference
  exits 4 (code/grafted_nanoparticle.cpp:82-107).  tests/test_failures.py runs
  the compiled reference on the same two inputs and sees those exits.
* A bounded mbarrier wait of the mixed plane pass that runs out: the first
  wait's poll limit is lowered to 0 (scft_set_wait_limit), so every such wait
  runs out at once; each CTA then waits, bounded, for its copies to land and
  finishes, and the call returns SCFT_ERR_CUDA.  With the limit restored the
  same context runs on and matches a context that never timed out.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def scft():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    S.load()
    return S


@pytest.mark.parametrize("mixed", [False, True])
def test_nan_field_gives_err_nan(scft, mixed):
    from test_failures import nan_case

    c = nan_case()
    p = scft.params_from_case(c, precision=scft.PREC_MIXED if mixed else scft.PREC_FP64)
    with scft.Context(p) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        H = ctx.calc_H()
        assert ctx.last_status == scft.ERR_NAN
        assert np.isnan(H[0, 0])
        # the context still answers
        ctx.set_fields(0, {k: np.nan_to_num(v) for k, v in c.fields.items()})
        ctx.calc_poly_density()
        H = ctx.calc_H()
        assert ctx.last_status == scft.OK and np.isfinite(H[0, 0])


def test_nonpositive_graft_propagator_gives_err_qnonpos(scft):
    from test_failures import qnonpos_case

    c = qnonpos_case()
    with scft.Context(scft.params_from_case(c)) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        with pytest.raises(scft.ScftError) as e:
            ctx.calc_H()
        assert e.value.code == scft.ERR_QNONPOS
        assert "q_g" in str(e.value)


def _sweep_case(scft):
    from scft.workloads import plate_params, seeded_fields

    ps = [plate_params(t, N=16, precision=scft.PREC_MIXED) for t in (10.0, 45.0)]
    return ps, [seeded_fields(p, 40 + k) for k, p in enumerate(ps)]


def test_mbarrier_wait_that_runs_out_returns_err_cuda(scft):
    """With the per-step launches (the persistent sweep's own waits are in
    tests/test_gpu_persistent.py)."""
    ps, fields = _sweep_case(scft)
    with scft.Context(ps) as ref:
        ref.set_persistent(False)
        for k in range(2):
            ref.set_fields(k, fields[k])
        ref.calc_poly_density()
        ref.update_1s(3)
        H_ref = ref.calc_H()[:, 0].copy()
    with scft.Context(ps) as ctx:
        ctx.set_persistent(False)
        for k in range(2):
            ctx.set_fields(k, fields[k])
        ctx.calc_poly_density()
        ctx.update_1s(1)
        ctx.set_wait_limit(0)
        with pytest.raises(scft.ScftError) as e:
            ctx.update_1s(1)
        assert e.value.code == scft.ERR_CUDA
        assert "ran out" in str(e.value)
        ctx.set_wait_limit(-1)
        ctx.update_1s(1)
        H = ctx.calc_H()[:, 0]
    # every CTA finished its work after the timeout: the state is the same
    np.testing.assert_array_equal(H, H_ref)
