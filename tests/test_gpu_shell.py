"""The A-attractive shell potential (an extension with no counterpart in the
reference): U_A = Lambda * sum_j [rho_p(L + 2w, R + w) - rho_p(L, R)] on A
segments, the potential of the single-plate workload's plate surface.

There is no reference output for it, so the FP64 method is checked against
the numpy restatement extended the same way (oracle/scft_oracle.py, pinned to
the reference without the shell) at the plain method's bars (densities 1e-10,
H 1e-9 relative), the mixed form against the FP64 method at its FP32 floor
(2e-5), and the geometric derivatives, which gain Lambda int rho_A dU/dg,
against central differences (1e-5 relative).
"""
import dataclasses
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

LAM, WIDTH = -0.3, 0.4


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    return scft


def tiny_plate_case():
    import json

    from ref_case import Case

    z = np.load(os.path.join(GOLDEN, "tiny_plate.npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    c.fields = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    return c


def test_shell_fp64_matches_restatement(S):
    import scft_oracle as O

    c = tiny_plate_case()
    s = dataclasses.replace(O.System.from_case(c), shell_lambda=LAM, shell_width=WIDTH)
    assert np.abs(s.tables["shellU"]).max() > 0.05 * abs(LAM)
    st = O.State.from_fields(s.g, c.fields)
    trace = O.run(s, st, 4)
    with S.Context(S.params_from_case(c, shell_lambda=LAM, shell_width=WIDTH)) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        rows = [ctx.calc_H()[0]]
        for _ in range(4):
            ctx.update_1s(1)
            rows.append(ctx.calc_H()[0])
        ra, rb, _ = ctx.density(0)
    rows = np.array(rows)
    assert np.abs(rows[:, 0] - trace[:, 1]).max() <= 1e-9 * np.abs(trace[:, 1]).max()
    assert np.abs(rows[:, 2] - trace[:, 3]).max() <= 1e-10 * np.abs(trace[:, 3]).max()
    assert rel(ra, st.out["rhoda"]) < 1e-10
    assert rel(rb, st.out["rhodb"]) < 1e-10


def test_shell_changes_the_solution(S):
    """Lambda < 0 attracts A: more A in the shell than without it."""
    import scft_oracle as O

    c = tiny_plate_case()
    s = dataclasses.replace(O.System.from_case(c), shell_lambda=LAM, shell_width=WIDTH)
    U = s.tables["shellU"]
    with S.Context([S.params_from_case(c), S.params_from_case(c, shell_lambda=LAM, shell_width=WIDTH)]) as ctx:
        for k in range(2):
            ctx.set_fields(k, c.fields)
        ctx.calc_poly_density()
        ra0 = ctx.density(0)[0].real
        ra1 = ctx.density(1)[0].real
    shell = U < 0.5 * U.min()
    assert (ra1[shell] - ra0[shell]).mean() > 0


def test_shell_mixed_matches_fp64(S):
    from scft.workloads import plate_params, seeded_fields

    out = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        p = plate_params(10.0, N=32, grid=(32, 32, 32), box_rg=(4.0, 4.0, 4.0), precision=prec, shell=True,
                         thickness_rg=0.4, radius_rg=1.0, xi_rg=0.2)
        f = seeded_fields(p, 3)
        with S.Context(p) as ctx:
            ctx.set_fields(0, f)
            ctx.calc_poly_density()
            ctx.update_1s(5)
            out[prec] = (ctx.calc_H()[0], ctx.density(0))
    (h64, d64), (h32, d32) = out[S.PREC_FP64], out[S.PREC_MIXED]
    assert abs(h32[0] - h64[0]) <= 2e-5 * abs(h64[0])
    assert rel(d32[0], d64[0]) < 2e-5
    assert rel(d32[1], d64[1]) < 2e-5


def small_shell_plate(S, theta_deg, prec=0, centers=((0.5, 0.5, 0.5),)):
    from scft.workloads import plate_params

    return plate_params(theta_deg, N=16, grid=(24, 24, 24), box_rg=(4.0, 4.0, 4.0), precision=prec, centers=centers,
                        thickness_rg=0.4, radius_rg=1.0, xi_rg=0.2, lam_pl=0.002, lam_mi=0.001, shell=True)


def H_and_grad(S, p, fields):
    with S.Context(p) as ctx:
        ctx.set_fields(0, fields)
        ctx.calc_poly_density()
        return ctx.calc_H()[0, 0], ctx.grad_geom()[0]


def test_shell_rotation_derivative(S):
    from scft.workloads import seeded_fields

    th, h = 10.0, 1e-3
    p0 = small_shell_plate(S, th)
    f = seeded_fields(p0, 7)
    f["wpl"] = 1j * 0.3 * np.cos(2 * np.pi * np.arange(24) / 24)[None, None, :] * np.ones((24, 24, 24))
    H0, g0 = H_and_grad(S, p0, f)
    Hp, _ = H_and_grad(S, small_shell_plate(S, th + math.degrees(h)), f)
    Hm, _ = H_and_grad(S, small_shell_plate(S, th - math.degrees(h)), f)
    fd = (Hp - Hm) / (2 * h)
    assert abs(g0[0, 0] - fd) <= 1e-5 * max(abs(fd), 1e-3 * abs(H0)), (g0[0, 0], fd)


def test_shell_mixed_gradient_matches_fp64(S):
    from scft.workloads import seeded_fields

    f = seeded_fields(small_shell_plate(S, 20.0), 9)
    g = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        with S.Context(small_shell_plate(S, 20.0, prec)) as ctx:
            ctx.set_fields(0, f)
            ctx.calc_poly_density()
            ctx.update_1s(3)
            g[prec] = ctx.grad_geom()[0]
    assert np.abs(g[S.PREC_MIXED][0] - g[S.PREC_FP64][0]).max() <= 1e-4 * np.abs(g[S.PREC_FP64][0]).max()


def test_shell_separation_derivative(S):
    from scft.workloads import seeded_fields

    def two(d):
        return small_shell_plate(S, 0.0, centers=((0.5, 0.5 - d / 2, 0.5), (0.5, 0.5 + d / 2, 0.5)))

    d, h = 0.3, 1e-4
    p0 = two(d)
    f = seeded_fields(p0, 8)
    H0, g0 = H_and_grad(S, p0, f)
    Hp, _ = H_and_grad(S, two(d + h), f)
    Hm, _ = H_and_grad(S, two(d - h), f)
    fd = (Hp - Hm) / (2 * h)
    an = p0.L[1] * (g0[1, 2] - g0[0, 2]) / 2
    assert abs(an - fd) <= 1e-5 * max(abs(fd), 1e-3 * abs(H0)), (an, fd)


def test_shell_needs_a_plate_and_a_width(S):
    for kw in (dict(n_exp_nr=0, shell_lambda=-0.1, shell_width=0.1), dict(n_exp_nr=1, shell_lambda=-0.1)):
        with pytest.raises(S.ScftError):
            S.Context(S.make_params(**kw))
