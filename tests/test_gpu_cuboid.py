"""The cuboid plate (SCFT_PLATE_CUBOID, an extension with no counterpart in
the reference): the plate of the single-plate configuration as written, a
slab of thickness L along the normal u and a 2R x 2R square in the plane,
1/8 erfc((|u.r| - L/2)/xi) erfc((|e1.r| - R)/xi) erfc((|e2.r| - R)/xi).

There is no reference output for it, so
* its profile is checked against the numpy restatement (cuboid_plate, pinned
  by its closed forms on the CPU) on both branches of the in-plane frame;
* the FP64 method with cuboid plates (with and without the shell potential)
  against the restatement extended the same way, at the plain method's bars
  (densities 1e-10, H 1e-9 relative), and the mixed form against the FP64
  method at its FP32 floor (2e-5);
* dH/dtheta and dH/dc (scft_grad_geom) of both forms against
  Richardson-extrapolated central differences of the FP64 H at fixed fields
  (1e-5 relative; 1e-4 for the mixed form), for bare, shelled, tilted and
  grafted cuboids, and across converged states (envelope theorem, 1e-4).
"""
import dataclasses
import math
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    scft.load()
    return scft


def rotz(v, deg):
    t = math.radians(deg)
    return (math.cos(t) * v[0] - math.sin(t) * v[1], math.sin(t) * v[0] + math.cos(t) * v[1], v[2])


def cuboid(S, theta_deg, prec=0, centers=((0.5, 0.5, 0.5),), shell=False, axis=None, grafted=False):
    """24^3, N = 16 cuboid plate(s) rotated by theta about z; axis replaces
    the unrotated normal (1, 0, 0)."""
    from scft.workloads import plate_params

    p = plate_params(theta_deg, N=16, grid=(24, 24, 24), box_rg=(4.0, 4.0, 4.0), precision=prec, centers=centers,
                     thickness_rg=0.4, radius_rg=0.9, xi_rg=0.2, lam_pl=0.002, lam_mi=0.001, shell=shell,
                     shape=S.PLATE_CUBOID)
    if axis is not None:
        u = rotz(axis, theta_deg)
        for j in range(2):
            for d in range(3):
                p.orient[j][d] = u[d]
    if grafted:
        p.sigma = 0.5 / ((16 - 1) / 6.0)
        p.Ng = 4
        p.chi_bc = p.chi_ab
    return p


def fields(p, seed):
    from scft.workloads import seeded_fields

    f = seeded_fields(p, seed)
    x = np.arange(24) / 24
    f["wpl"] = 1j * 0.3 * np.cos(2 * np.pi * x)[None, None, :] * np.ones((24, 24, 24))
    if p.Ng:
        f["wbcm"] = (0.2 * np.sin(2 * np.pi * x)[None, :, None] * np.ones((24, 24, 24))).astype(np.complex128)
    return f


def H_and_grad(S, p, f, iters=0):
    with S.Context(p) as ctx:
        ctx.set_fields(0, f)
        ctx.calc_poly_density()
        if iters:
            ctx.update_1s(iters)
        return ctx.calc_H()[0, 0], ctx.grad_geom()[0]


@pytest.mark.parametrize("axis", [(1.0, 0.0, 0.0), (0.35, 0.2, 0.9), (0.1, 0.05, 1.0)])
@pytest.mark.parametrize("theta", [0.0, 10.0, 37.0])
def test_cuboid_profile_matches_restatement(S, axis, theta):
    import scft_oracle as O

    centers = ((0.47, 0.52, 0.5), (0.2, 0.25, 0.7))
    p = cuboid(S, theta, centers=centers, axis=axis)
    with S.Context(p) as ctx:
        got = ctx.plate_density(0)
    u = np.asarray(rotz(axis, theta))
    u = u / np.linalg.norm(u)
    g = O.Grid(tuple(p.Nx), tuple(p.L))
    want = sum(O.cuboid_plate(g, p.L_nr, p.R_nr, p.xi_nr, c, u).real for c in centers)
    assert want.max() > 0.5
    assert np.abs(got - want).max() <= 1e-12


def tiny_plate_case():
    import json

    from ref_case import Case

    z = np.load(os.path.join(GOLDEN, "tiny_plate.npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    c.fields = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    return c


@pytest.mark.parametrize("shell", [False, True])
def test_cuboid_fp64_matches_restatement(S, shell):
    import scft_oracle as O

    c = tiny_plate_case()
    extra = dict(shell_lambda=-0.3, shell_width=0.4) if shell else {}
    s = dataclasses.replace(O.System.from_case(c), plate_shape=1, **extra)
    disc = O.System.from_case(c)
    assert rel(s.tables["rho_exp_nr"], disc.tables["rho_exp_nr"]) > 1e-3  # a different plate
    st = O.State.from_fields(s.g, c.fields)
    trace = O.run(s, st, 4)
    with S.Context(S.params_from_case(c, plate_shape=S.PLATE_CUBOID, **extra)) as ctx:
        assert np.abs(ctx.plate_density(0) - s.tables["rho_exp_nr"].real).max() <= 1e-12
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


def test_cuboid_mixed_matches_fp64(S):
    from scft.workloads import plate_params, seeded_fields

    out = {}
    for prec in (S.PREC_FP64, S.PREC_MIXED):
        p = plate_params(10.0, N=32, grid=(32, 32, 32), box_rg=(4.0, 4.0, 4.0), precision=prec, shell=True,
                         thickness_rg=0.4, radius_rg=0.9, xi_rg=0.2, shape=S.PLATE_CUBOID)
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


def check(an, fd, H0, tol):
    assert abs(an - fd) <= tol * max(abs(fd), 1e-3 * abs(H0)), (an, fd)


def central(Hf, x, h):
    """Richardson-extrapolated central difference of the FP64 H at fixed
    fields (steps h and h/2: the O(h^2) term cancels)."""
    d1 = (Hf(x + h) - Hf(x - h)) / (2 * h)
    d2 = (Hf(x + h / 2) - Hf(x - h / 2)) / h
    return (4 * d2 - d1) / 3


@pytest.mark.parametrize("kind", ["bare", "shell", "tilted", "grafted"])
def test_cuboid_rotation_derivative_at_fixed_fields(S, kind):
    """Both forms' dH/dtheta against the FP64 method's central difference
    (the mixed form's own H carries FP32 noise that a difference over 2e-4
    rad would amplify).  tilted: the axis has |u_z| >= 0.9, the second branch
    of the in-plane frame, whose rotation about z is not rigid."""
    kw = dict(shell=kind == "shell", grafted=kind == "grafted", axis=(0.3, 0.1, 0.95) if kind == "tilted" else None)
    # a small step: the profile's |u.r| kinks (at the plate's mid-planes) move
    # across grid points as the plate turns, which a wide difference feels
    th, h = 12.0, 2e-4
    f = fields(cuboid(S, th, **kw), 31)
    fd = central(lambda t: H_and_grad(S, cuboid(S, math.degrees(t), 0, **kw), f)[0], math.radians(th), h)
    for prec, tol in ((0, 1e-5), (1, 1e-4)):
        H0, g0 = H_and_grad(S, cuboid(S, th, prec, **kw), f)
        check(g0[0, 0], fd, H0, tol)


@pytest.mark.parametrize("kind", ["bare", "shell", "grafted"])
def test_cuboid_separation_derivative_at_fixed_fields(S, kind):
    kw = dict(shell=kind == "shell", grafted=kind == "grafted")

    def two(d, prec=0):
        return cuboid(S, 25.0, prec, centers=((0.5, 0.5 - d / 2, 0.5), (0.5, 0.5 + d / 2, 0.5)), **kw)

    d, h = 0.45, 2e-4
    f = fields(two(d), 32)
    fd = central(lambda x: H_and_grad(S, two(x), f)[0], d, h)
    for prec, tol in ((0, 1e-5), (1, 1e-4)):
        H0, g0 = H_and_grad(S, two(d, prec), f)
        an = two(d).L[1] * (g0[1, 2] - g0[0, 2]) / 2
        check(an, fd, H0, tol)


def test_cuboid_total_derivative_across_converged_states(S):
    """Envelope theorem for the cuboid with the shell: dH*/dtheta at the
    converged state against the central difference of converged H."""
    from scft.workloads import seeded_fields

    th, h = 20.0, 2e-3
    f0 = seeded_fields(cuboid(S, th, shell=True), 11)

    def converged(theta):
        with S.Context(cuboid(S, theta, shell=True)) as ctx:
            ctx.set_fields(0, f0)
            ctx.calc_poly_density()
            last = None
            for _ in range(60):
                ctx.update_1s(100)
                H = ctx.calc_H()[0, 0]
                if last is not None and abs(H - last) < 1e-11 * abs(H):
                    break
                last = H
            return H, ctx.grad_geom()[0, 0, 0]

    H0, g0 = converged(th)
    Hp, _ = converged(th + math.degrees(h))
    Hm, _ = converged(th - math.degrees(h))
    fd = (Hp - Hm) / (2 * h)
    assert abs(g0 - fd) <= 1e-4 * max(abs(fd), 1e-4 * abs(H0)), (g0, fd)
