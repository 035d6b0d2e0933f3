"""Pins the cuboid plate restatement (oracle/scft_oracle.py cuboid_plate, a
project extension with no reference counterpart: SCFT_PLATE_CUBOID) by its
closed forms, so that the GPU cuboid can be checked against it.

* With the axis along x or z the cuboid is the outer product of three 1D
  profiles 1/2 erfc((|x| - h)/xi) (the two branches of the in-plane frame).
* Its frame is orthonormal and right-handed for any axis.
* A quarter turn about the axis maps it onto itself.
* With the reference's disc profile (explicit_nanorod, pinned to the
  reference's fixtures) it shares the slab factor along u.
"""
import numpy as np
import pytest
from scipy.special import erfc

import scft_oracle as O

L_NR, R_NR, XI = 0.6, 1.1, 0.2


def grid():
    return O.Grid((24, 24, 24), (4.0, 4.0, 4.0))


def profile_1d(g, d, half, center=0.5):
    x = g.dx[d] * np.arange(g.Nx[d]) - center * g.L[d]
    x = np.where(x >= 0.5 * g.L[d], x - g.L[d], np.where(x < -0.5 * g.L[d], x + g.L[d], x))
    return 0.5 * erfc((np.abs(x) - half) / XI)


@pytest.mark.parametrize("axis", ["x", "z"])
def test_axis_aligned_cuboid_is_an_outer_product(axis):
    g = grid()
    u = (1.0, 0.0, 0.0) if axis == "x" else (0.0, 0.0, 1.0)
    c = O.cuboid_plate(g, L_NR, R_NR, XI, (0.5, 0.5, 0.5), u)
    halves = (0.5 * L_NR, R_NR, R_NR) if axis == "x" else (R_NR, R_NR, 0.5 * L_NR)
    fx, fy, fz = (profile_1d(g, d, halves[d]) for d in range(3))
    want = fz[:, None, None] * fy[None, :, None] * fx[None, None, :]
    assert np.abs(c.imag).max() == 0.0
    np.testing.assert_allclose(c.real, want, rtol=1e-14, atol=1e-16)


def test_frame_is_orthonormal_and_right_handed():
    rng = np.random.default_rng(3)
    for u in list(rng.standard_normal((50, 3))) + [np.array([0.1, 0.2, 1.0]), np.array([1.0, 0.0, 0.0])]:
        u = u / np.linalg.norm(u)
        e1, e2 = O.cuboid_frame(u)
        E = np.stack([u, e1, e2])
        np.testing.assert_allclose(E @ E.T, np.eye(3), atol=1e-14)
        assert np.linalg.det(E) == pytest.approx(1.0, abs=1e-14)


def test_quarter_turn_about_the_axis_is_a_symmetry():
    g = grid()
    c = O.cuboid_plate(g, L_NR, R_NR, XI, (0.5, 0.5, 0.5), (1.0, 0.0, 0.0))
    # axis along x: swapping y and z turns the square by a quarter about x
    np.testing.assert_allclose(c, np.transpose(c, (1, 0, 2)), rtol=0, atol=1e-15)


def test_shares_the_slab_factor_with_the_disc():
    """Far inside the square / disc in the plane the two profiles reduce to
    the slab factor along u."""
    g = grid()
    u = (np.cos(0.3), np.sin(0.3), 0.0)
    big = 50.0
    cub = O.cuboid_plate(g, L_NR, big, XI, (0.5, 0.5, 0.5), u)
    disc = O.explicit_nanorod(g, L_NR, big, XI, (0.5, 0.5, 0.5), u)
    np.testing.assert_allclose(cub.real, disc.real, rtol=1e-14, atol=1e-300)
