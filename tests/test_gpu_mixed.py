"""The mixed-precision form (FP32 packed propagators, FP64 k-space fields,
reductions, log Q and H) against the plain FP64 method on the same inputs.

Tolerances written here are the measured FP32 floor of this form on small
grids (N <= 64): H relative 2e-5, Q relative 2e-5, densities 2e-5 (max over
the grid).  The error is coherent: the per-step FP32 rounding of the dominant
low-k modes repeats every step, so log Q drifts by ~N * 1e-7 (an FP32
transform in numpy shows the same ~1e-6 at N = 32).
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

H_TOL = 2e-5
RHO_TOL = 2e-5
Q_TOL = 2e-5


@pytest.fixture(scope="module")
def scft():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    assert S.mixed_available()
    return S


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


def run_pair(S, params, fields, iters):
    out = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        ps = []
        for p in params:
            q = S.Params.from_buffer_copy(p)
            q.precision = prec
            ps.append(q)
        with S.Context(ps) as ctx:
            for k, f in enumerate(fields):
                ctx.set_fields(k, f)
            ctx.calc_poly_density()
            H = [ctx.calc_H()]
            for _ in range(iters):
                ctx.update_1s(1)
                H.append(ctx.calc_H())
            dens = [ctx.density(k) for k in range(len(params))]
            flds = [ctx.get_fields(k) for k in range(len(params))]
        out[prec] = (np.array(H), dens, flds)
    return out[S.PREC_FP64], out[S.PREC_MIXED]


def test_mixed_matches_fp64_single_plate(scft):
    from scft.workloads import plate_params, seeded_fields

    p = plate_params(10.0, N=32, grid=(32, 32, 32))
    (H64, d64, _), (H32, d32, _) = run_pair(scft, [p], [seeded_fields(p, 3)], 10)
    assert np.abs(H32[:, 0, 0] - H64[:, 0, 0]).max() <= H_TOL * np.abs(H64[:, 0, 0]).max()
    assert np.abs(H32[:, 0, 2] - H64[:, 0, 2]).max() <= Q_TOL * np.abs(H64[:, 0, 2]).max()
    assert rel(d32[0][0].real, d64[0][0].real) < RHO_TOL
    assert rel(d32[0][1].real, d64[0][1].real) < RHO_TOL


def test_mixed_uneven_batch_matches_fp64(scft):
    """Different grids (incl. 5 and 3 factors), N odd and even, one plate or none."""
    from scft.workloads import plate_params, seeded_fields

    params = [plate_params(0.0, N=21, grid=(24, 20, 16)),
              plate_params(30.0, N=32, grid=(32, 32, 32)),
              plate_params(90.0, N=16, grid=(16, 24, 30), centers=())]
    fields = [seeded_fields(p, 10 + k) for k, p in enumerate(params)]
    (H64, d64, _), (H32, d32, _) = run_pair(scft, params, fields, 6)
    for k in range(len(params)):
        assert np.abs(H32[:, k, 0] - H64[:, k, 0]).max() <= H_TOL * np.abs(H64[:, k, 0]).max()
        assert rel(d32[k][0].real, d64[k][0].real) < RHO_TOL
        assert rel(d32[k][1].real, d64[k][1].real) < RHO_TOL


def test_mixed_field_round_trip_and_fields_match(scft):
    from scft.workloads import plate_params, seeded_fields

    p = plate_params(10.0, N=16, grid=(16, 16, 16))
    f = seeded_fields(p, 4)
    q = scft.Params.from_buffer_copy(p)
    q.precision = scft.PREC_MIXED
    with scft.Context(q) as ctx:
        ctx.set_fields(0, f)
        g = ctx.get_fields(0)
    assert rel(g["wabm"], f["wabm"]) < 1e-13
    assert np.abs(g["wpl"]).max() < 1e-14
    (_, _, f64), (_, _, f32) = run_pair(scft, [p], [f], 5)
    for name in ("wpl", "wabp", "wabm"):
        assert rel(f32[0][name], f64[0][name]) < 5e-5, name


def test_mixed_rejects_complex_fields(scft):
    from scft.workloads import plate_params

    p = plate_params(0.0, N=8, grid=(8, 8, 8), precision=scft.PREC_MIXED)
    rng = np.random.default_rng(0)
    with scft.Context(p) as ctx:
        bad = {"wabm": rng.standard_normal((8, 8, 8)) + 0.1j * rng.standard_normal((8, 8, 8))}
        with pytest.raises(scft.ScftError) as e:
            ctx.set_fields(0, bad)
        assert e.value.code == scft.ERR_COMPLEX


def test_mixed_range_normalisation_long_chain(scft):
    """N=200 on a resolved grid (dx ~ 0.5 b) with fields strong enough that Q
    is ~1e53, far outside FP32's range: the power-of-two rescaling keeps the
    FP32 sweep in range.  Bars for this extreme case: Q 1e-4 (on the same
    fields), H 1e-5 relative."""
    from scft.workloads import plate_params, seeded_fields

    p = plate_params(20.0, N=200, fA=0.4, chiN=30.0, grid=(32, 32, 32), box_rg=(2.8, 2.8, 2.8),
                     lam_pl=0.001, lam_mi=0.0002)
    f = seeded_fields(p, 5)
    f["wabm"] = f["wabm"] * 10.0
    (H64, d64, _), (H32, d32, _) = run_pair(scft, [p], [f], 1)
    assert np.isfinite(H64).all() and H64[0, 0, 2] > 1e45
    assert abs(H32[0, 0, 2] - H64[0, 0, 2]) <= 1e-4 * abs(H64[0, 0, 2])  # same fields
    assert np.abs(H32[:, 0, 0] - H64[:, 0, 0]).max() <= 1e-5 * np.abs(H64[:, 0, 0]).max()
    assert rel(d32[0][0].real, d64[0][0].real) < 1e-3


@pytest.mark.parametrize("nz", [64, 32, 128])
def test_mixed_64cubed_specialised_kernels_match_fp64(scft, nz):
    """Batches of 64 x 64 xy planes take the specialised 64-point plane pass
    (and, for nz = 64, the 64-point z pass); uneven N."""
    from scft.workloads import plate_params, seeded_fields

    box = (6.4, 6.4, 6.4 * nz / 64)
    params = [plate_params(10.0, N=20, grid=(64, 64, nz), box_rg=box),
              plate_params(45.0, N=13, grid=(64, 64, nz), box_rg=box)]
    fields = [seeded_fields(p, 20 + k) for k, p in enumerate(params)]
    (H64, d64, _), (H32, d32, _) = run_pair(scft, params, fields, 3)
    for k in range(len(params)):
        assert np.abs(H32[:, k, 0] - H64[:, k, 0]).max() <= H_TOL * np.abs(H64[:, k, 0]).max()
        assert np.abs(H32[:, k, 2] - H64[:, k, 2]).max() <= Q_TOL * np.abs(H64[:, k, 2]).max()
        assert rel(d32[k][0].real, d64[k][0].real) < RHO_TOL
        assert rel(d32[k][1].real, d64[k][1].real) < RHO_TOL


@pytest.mark.parametrize("grids", [((64, 64, 64),) * 5, ((48, 48, 48), (32, 32, 32), (48, 48, 48)),
                                   ((48, 48, 48), (64, 64, 64), (32, 32, 32), (64, 64, 64))])
def test_sweep_schedule_does_not_change_results(scft, grids):
    """Sweep groups and z-pass tile widths only regroup independent work:
    every schedule gives bit-identical H, Q and densities.  The autotuner
    reports a valid choice; it also picks the generic FFTs' stage orders,
    which changes FP32 rounding, so its result agrees to the FP32 bar."""
    from scft.workloads import plate_params, seeded_fields

    params = [plate_params(5.0 * k, N=24 + 4 * k, grid=g, box_rg=(4.0, 4.0, 4.0), precision=scft.PREC_MIXED)
              for k, g in enumerate(grids)]
    fields = [seeded_fields(p, 40 + k) for k, p in enumerate(params)]
    res = []
    for mode in ("g1", "g3", "g2p2", "tuned"):
        with scft.Context(params) as ctx:
            for k, f in enumerate(fields):
                ctx.set_fields(k, f)
            ctx.calc_poly_density()
            if mode == "g1":
                ctx.set_sweep_groups(1)
            elif mode == "g3":
                ctx.set_sweep_groups(3)
            elif mode == "g2p2":
                ctx.set_sweep_groups(2, 2)
            else:
                t = ctx.autotune(2)
                assert 1 <= t["groups"] <= len(params) and t["ms_per_sweep"] > 0
                assert t["col_tile"] in ((8, 16, 32) if (64, 64, 64) in grids else (0,))
            ctx.update_1s(3)
            res.append((ctx.calc_H(), [ctx.density(k)[0] for k in range(len(params))]))
    for H, d in res[1:3]:
        assert np.array_equal(H, res[0][0])
        for a, b in zip(d, res[0][1]):
            assert np.array_equal(a, b)
    H, d = res[3]
    assert np.abs(H[:, 0] - res[0][0][:, 0]).max() <= 2e-5 * np.abs(res[0][0][:, 0]).max()
    for a, b in zip(d, res[0][1]):
        assert np.abs(a - b).max() <= 1e-4 * np.abs(b).max()


def test_mixed_grid_batch_runs_64cubed_on_the_64_point_kernels(scft):
    """In a batch of mixed grids the 64^3 instances run the 64-point plane and
    z kernels and the others the generic ones, and the batch matches the FP64
    method.  The 64-point kernels have one launch shape, so a 64^3 instance's
    H, Q and densities are bit-identical to those of a context holding it
    alone; the generic kernels size their blocks for the largest grid of the
    batch, which reorders FP32 plane sums, so the others agree to the FP32
    tolerance."""
    from scft.workloads import plate_params, seeded_fields

    params = [plate_params(0.0, N=21, grid=(48, 48, 48), box_rg=(4.8, 4.8, 4.8)),
              plate_params(30.0, N=24, grid=(64, 64, 64)),
              plate_params(90.0, N=16, grid=(32, 32, 32), box_rg=(4.0, 4.0, 4.0)),
              plate_params(60.0, N=13, grid=(64, 64, 64))]
    fields = [seeded_fields(p, 60 + k) for k, p in enumerate(params)]
    (H64, d64, _), (H32, d32, _) = run_pair(scft, params, fields, 4)
    for k in range(len(params)):
        assert np.abs(H32[:, k, 0] - H64[:, k, 0]).max() <= H_TOL * np.abs(H64[:, k, 0]).max()
        assert np.abs(H32[:, k, 2] - H64[:, k, 2]).max() <= Q_TOL * np.abs(H64[:, k, 2]).max()
        assert rel(d32[k][0].real, d64[k][0].real) < RHO_TOL
        assert rel(d32[k][1].real, d64[k][1].real) < RHO_TOL
    for k, p in enumerate(params):
        (_, _, _), (H1, d1, _) = run_pair(scft, [p], [fields[k]], 4)
        if tuple(p.Nx) == (64, 64, 64):
            assert np.array_equal(H1[:, 0], H32[:, k])
            assert np.array_equal(d1[0][0], d32[k][0])
            assert np.array_equal(d1[0][1], d32[k][1])
        else:
            assert np.abs(H1[:, 0, 0] - H32[:, k, 0]).max() <= H_TOL * np.abs(H32[:, k, 0]).max()
            assert rel(d1[0][0].real, d32[k][0].real) < RHO_TOL


GRAFT_GEOMS = {
    "two_plates_32": dict(grid=(32, 32, 32), box_rg=(4.0, 4.0, 4.0),
                          centers=((0.5, 0.5, 0.375), (0.5, 0.5, 0.625))),
    # 128 x 128 planes: the in-place plane passes with 1024 threads
    "one_plate_128x128x16": dict(grid=(128, 128, 16), box_rg=(4.0, 4.0, 2.0), centers=((0.5, 0.5, 0.5),)),
}


def grafted_params(scft, prec, theta=20.0, geom="two_plates_32"):
    """Config 4's chemistry at a small size: rotated plates grafted with
    chains of the A-like species C (chi_AC = 0, chi_BC = chi_AB)."""
    from scft.workloads import plate_params, rg

    N = 32
    p = plate_params(theta, N=N, fA=0.4, chiN=30.0, precision=prec, thickness_rg=0.3, radius_rg=0.8, xi_rg=0.2,
                     sigma=0.5 / rg(N) ** 2, Ng=8, lam_pl=0.002, lam_mi=0.001, **GRAFT_GEOMS[geom])
    p.chi_bc = p.chi_ab
    return p


@pytest.mark.parametrize("geom", sorted(GRAFT_GEOMS))
def test_mixed_grafted_plates_match_fp64(scft, geom):
    from scft.workloads import seeded_fields

    f = seeded_fields(grafted_params(scft, scft.PREC_FP64, geom=geom), 21)
    out = {}
    for prec in (scft.PREC_FP64, scft.PREC_MIXED):
        with scft.Context(grafted_params(scft, prec, geom=geom)) as ctx:
            assert ctx.info(0)["phiG"] > 0
            ctx.set_fields(0, f)
            ctx.calc_poly_density()
            H = [ctx.calc_H()[0]]
            for _ in range(4):
                ctx.update_1s(1)
                H.append(ctx.calc_H()[0])
            out[prec] = (np.array(H), ctx.density(0), ctx.get_fields(0))
    (H64, d64, f64), (H32, d32, f32) = out[scft.PREC_FP64], out[scft.PREC_MIXED]
    assert np.abs(H32[:, 0] - H64[:, 0]).max() <= H_TOL * np.abs(H64[:, 0]).max()
    assert np.abs(H32[:, 4] - H64[:, 4]).max() <= Q_TOL * np.abs(H64[:, 4]).max()  # Re Qga
    for a, b in zip(d32, d64):
        assert rel(a, b) < RHO_TOL
    for k in ("wpl", "wbcp", "wbcm"):
        assert rel(f32[k], f64[k]) < RHO_TOL, k


def test_complex_langevin_is_fp64_only(scft):
    p = scft.make_params(precision=scft.PREC_MIXED, do_cl=1, cl_seed=3)
    with pytest.raises(scft.ScftError):
        scft.Context(p)


def test_set_fields_all_matches_per_instance_calls(scft):
    """scft_set_fields_all is the per-instance call for every instance at once:
    identical densities and H; a complex field is reported with its instance."""
    import torch

    from scft.workloads import plate_params, seeded_fields

    params = [plate_params(t, N=16, grid=(32, 32, 32), box_rg=(4.0, 4.0, 4.0), precision=scft.PREC_MIXED)
              for t in (0.0, 30.0, 60.0)]
    fields = [seeded_fields(p, 60 + k) for k, p in enumerate(params)]
    bufs = []
    for f in fields:
        arr = np.stack([np.asarray(f.get(n, np.zeros((32, 32, 32))), np.complex128) for n in scft.FIELD_NAMES])
        t = torch.zeros(arr.size * 2, dtype=torch.float64, pin_memory=True)
        t.numpy()[:] = arr.view(np.float64).ravel()
        bufs.append(t)
    res = []
    for batched in (False, True):
        with scft.Context(params) as ctx:
            if batched:
                ctx.set_fields_all_raw([b.data_ptr() for b in bufs])
            else:
                for k, f in enumerate(fields):
                    ctx.set_fields(k, f)
            ctx.update_1s(2)
            res.append((ctx.calc_H(), [ctx.density(k)[0] for k in range(3)]))
    assert np.array_equal(res[0][0], res[1][0])
    for a, b in zip(res[0][1], res[1][1]):
        assert np.array_equal(a, b)
    bad = bufs[1].numpy().copy()
    bad[0] = 0.5  # real part of w+ at one point: w_A, w_B get an imaginary part
    bt = torch.from_numpy(bad).pin_memory()
    with scft.Context(params) as ctx:
        with pytest.raises(scft.ScftError, match="instance 1"):
            ctx.set_fields_all_raw([bufs[0].data_ptr(), bt.data_ptr(), bufs[2].data_ptr()])
