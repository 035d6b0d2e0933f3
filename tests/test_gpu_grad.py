"""Geometric derivatives dH/dtheta and dH/d(separation) (scft_grad_geom).

1. At fixed fields they are the exact partial derivatives of H: checked
   against central differences with h = 1e-3 (relative bar 1e-5).
2. At a converged saddle point they are the total derivatives of the
   converged H (delta H / delta w = 0): checked against central differences
   of independently converged states (relative bar 1e-4).
3. A torch.autograd.Function built on the C ABI gives the same gradient.
"""
import math

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def S():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft

    return scft


def small_plate(S, theta_deg, N=16, grid=(24, 24, 24), prec=0, centers=((0.5, 0.5, 0.5),)):
    from scft.workloads import plate_params

    return plate_params(theta_deg, N=N, grid=grid, box_rg=(4.0, 4.0, 4.0), precision=prec, centers=centers,
                        thickness_rg=0.4, radius_rg=1.0, xi_rg=0.2, lam_pl=0.002, lam_mi=0.001)


def H_at(S, p, fields, iters=0):
    with S.Context(p) as ctx:
        ctx.set_fields(0, fields)
        ctx.calc_poly_density()
        if iters:
            ctx.update_1s(iters)
        h = ctx.calc_H()[0, 0]
        g = ctx.grad_geom()[0]
        f = ctx.get_fields(0)
    return h, g, f


def test_rotation_derivative_at_fixed_fields(S):
    from scft.workloads import seeded_fields

    th, h = 10.0, 1e-3
    p0 = small_plate(S, th)
    f = seeded_fields(p0, 7)
    f["wpl"] = 1j * 0.3 * np.cos(2 * np.pi * np.arange(24) / 24)[None, None, :] * np.ones((24, 24, 24))
    H0, g0, _ = H_at(S, p0, f)
    Hp, _, _ = H_at(S, small_plate(S, th + math.degrees(h)), f)
    Hm, _, _ = H_at(S, small_plate(S, th - math.degrees(h)), f)
    fd = (Hp - Hm) / (2 * h)
    assert abs(g0[0, 0] - fd) <= 1e-5 * max(abs(fd), 1e-3 * abs(H0))


def test_separation_derivative_at_fixed_fields(S):
    from scft.workloads import seeded_fields

    def two(d):
        return small_plate(S, 0.0, centers=((0.5, 0.5 - d / 2, 0.5), (0.5, 0.5 + d / 2, 0.5)))

    d, h = 0.3, 1e-4
    p0 = two(d)
    f = seeded_fields(p0, 8)
    f["wpl"] = 1j * 0.2 * np.sin(2 * np.pi * np.arange(24) / 24)[None, :, None] * np.ones((24, 24, 24))
    H0, g0, _ = H_at(S, p0, f)
    Hp, _, _ = H_at(S, two(d + h), f)
    Hm, _, _ = H_at(S, two(d - h), f)
    fd = (Hp - Hm) / (2 * h)  # per unit of d in fractions of L_y
    Ly = p0.L[1]
    an = Ly * (g0[1, 2] - g0[0, 2]) / 2
    assert abs(an - fd) <= 1e-5 * max(abs(fd), 1e-3 * abs(H0))


def test_mixed_form_gives_the_same_gradient(S):
    from scft.workloads import seeded_fields

    p64 = small_plate(S, 20.0)
    p32 = small_plate(S, 20.0, prec=S.PREC_MIXED)
    f = seeded_fields(p64, 9)
    _, g64, _ = H_at(S, p64, f, iters=3)
    _, g32, _ = H_at(S, p32, f, iters=3)
    assert np.abs(g32[0] - g64[0]).max() <= 1e-4 * np.abs(g64[0]).max()


def test_total_derivative_across_converged_states(S):
    """Envelope theorem: dH*/dtheta from the gradient at the converged state
    equals the central difference of converged H at theta +- h."""
    from scft.workloads import seeded_fields

    th, h = 20.0, 2e-3
    f0 = seeded_fields(small_plate(S, th), 11)

    def converged(theta):
        p = small_plate(S, theta)
        with S.Context(p) as ctx:
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


def test_autograd_function_wrapper(S):
    """H(theta) at fixed fields as a torch.autograd.Function whose backward
    calls scft_grad_geom."""
    import torch

    from scft.workloads import seeded_fields

    f = seeded_fields(small_plate(S, 0.0), 12)
    f["wpl"] = 1j * 0.3 * np.cos(2 * np.pi * np.arange(24) / 24)[None, None, :] * np.ones((24, 24, 24))

    class PlateH(torch.autograd.Function):
        @staticmethod
        def forward(ctx_, theta):
            H, g, _ = H_at(S, small_plate(S, math.degrees(float(theta))), f)
            ctx_.save_for_backward(torch.tensor(g[0, 0], dtype=torch.float64))
            return torch.tensor(H, dtype=torch.float64)

        @staticmethod
        def backward(ctx_, grad_out):
            (g,) = ctx_.saved_tensors
            return grad_out * g

    theta = torch.tensor(math.radians(15.0), dtype=torch.float64, requires_grad=True)
    H = PlateH.apply(theta)
    H.backward()
    h = 1e-3
    fd = (PlateH.apply(torch.tensor(theta.item() + h)) - PlateH.apply(torch.tensor(theta.item() - h))) / (2 * h)
    assert abs(theta.grad.item() - fd.item()) <= 1e-5 * max(abs(fd.item()), 1e-3 * abs(H.item()))


def grafted(S, theta_deg, prec=0, centers=((0.5, 0.5, 0.5),)):
    """small_plate with grafted chains of Ng = 4 at sigma = 0.5 / Rg^2 (graft
    species A-like: chi_AC = 0, chi_BC = chi_AB)."""
    p = small_plate(S, theta_deg, prec=prec, centers=centers)
    p.sigma = 0.5 / ((16 - 1) / 6.0)
    p.Ng = 4
    p.chi_bc = p.chi_ab
    return p


def grafted_fields(p, seed):
    from scft.workloads import seeded_fields

    f = seeded_fields(p, seed)
    x = np.arange(24) / 24
    f["wpl"] = 1j * 0.3 * np.cos(2 * np.pi * x)[None, None, :] * np.ones((24, 24, 24))
    f["wbcm"] = (0.2 * np.sin(2 * np.pi * x)[None, :, None] * np.ones((24, 24, 24))).astype(np.complex128)
    return f


@pytest.mark.parametrize("prec", [0, 1])
def test_grafted_plate_derivatives_at_fixed_fields(S, prec):
    """Grafted plates: the graft map g ~ |grad rho_p(1.05 L, 1.05 R)| moves with
    the plate, so dH/dg gains -n_exp_nr ng_per_np Re int dg/dg_k log q_g
    (code/grafted_nanoparticle.cpp:82-112, code/initialize.cpp:160-200).
    Rotation and separation of two grafted plates against central
    differences of H at fixed fields."""
    th, h = 12.0, 1e-3
    f = grafted_fields(grafted(S, th), 21)
    H0, g0, _ = H_at(S, grafted(S, th, prec), f)
    Hp, _, _ = H_at(S, grafted(S, th + math.degrees(h), prec), f)
    Hm, _, _ = H_at(S, grafted(S, th - math.degrees(h), prec), f)
    fd = (Hp - Hm) / (2 * h)
    tol = 1e-5 if prec == 0 else 1e-4
    assert abs(g0[0, 0] - fd) <= tol * max(abs(fd), 1e-3 * abs(H0)), (g0[0, 0], fd)

    def two(d):
        return grafted(S, 0.0, prec, centers=((0.5, 0.5 - d / 2, 0.5), (0.5, 0.5 + d / 2, 0.5)))

    d, hd = 0.45, 1e-4
    H0, g0, _ = H_at(S, two(d), f)
    Hp, _, _ = H_at(S, two(d + hd), f)
    Hm, _, _ = H_at(S, two(d - hd), f)
    fd = (Hp - Hm) / (2 * hd)
    an = two(d).L[1] * (g0[1, 2] - g0[0, 2]) / 2
    assert abs(an - fd) <= tol * max(abs(fd), 1e-3 * abs(H0)), (an, fd)


def test_grafted_gradient_mixed_matches_fp64(S):
    f = grafted_fields(grafted(S, 25.0), 22)
    _, g64, _ = H_at(S, grafted(S, 25.0), f, iters=3)
    _, g32, _ = H_at(S, grafted(S, 25.0, S.PREC_MIXED), f, iters=3)
    assert np.abs(g32[0] - g64[0]).max() <= 1e-4 * np.abs(g64[0]).max()
