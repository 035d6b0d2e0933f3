"""Workload definitions: the benchmark configurations in the reference's b-units.

Conversions (code/initialize.cpp:53-55): N = Nda + Ndb beads, bond length
b = 1, Rg^2 = (N-1)/6.  chiN is per chain, so chi = chiN/N per segment;
C = rho0 Rg^3 / N, so rho0 = C N / Rg^3; lengths quoted in Rg are multiplied
by Rg.  A plate is the reference's explicit particle (code/initialize.cpp:
578-612) with axis u = plate normal, thickness L_nr along u and radius R_nr.

Initial fields are seeded synthetic inputs (there is no dataset): w+ = 0 and
w_AB^- = 0.5*chi*cos(2*pi*x/Lx) + N(0, 0.01^2) per segment, from
numpy.random.default_rng(seed).
"""
from __future__ import annotations

import math

import numpy as np

from . import PLATE_CUBOID, PLATE_REFERENCE, PREC_FP64, PREC_MIXED, make_params

SWEEP_ANGLES = (0, 1, 2, 3, 4, 5, 6, 7, 8, 9, 10, 20, 30, 45, 90)


def rg(N: int) -> float:
    return math.sqrt((N - 1) / 6.0)


def plate_params(theta_deg: float, N: int = 100, fA: float = 0.5, chiN: float = 20.0, C: float = 50.0,
                 grid=(64, 64, 64), box_rg=(6.4, 6.4, 6.4), precision=PREC_FP64, lam_pl=0.002, lam_mi=0.0005,
                 centers=((0.5, 0.5, 0.5),), thickness_rg=0.2, radius_rg=0.8, xi_rg=0.1, sigma=0.0, Ng=0,
                 shell=False, shape=PLATE_REFERENCE):
    """Config 1 geometry: plate(s) rotated by theta about z, normal along x at 0.
    shell=True adds the A-attractive shell Lambda = -1/N in a 0.1 Rg shell;
    shape=PLATE_CUBOID makes each plate a cuboid (thickness along the normal,
    a 2 radius_rg x 2 radius_rg square in the plane) instead of the
    reference's disc."""
    R = rg(N)
    Nda = int(round(fA * N))
    th = math.radians(theta_deg)
    u = (math.cos(th), math.sin(th), 0.0)
    cs = list(centers) + [(0.5, 0.5, 0.5)] * (2 - len(centers))
    return make_params(Nda=Nda, Ndb=N - Nda, a_smear=0.2, rho0=C * N / R ** 3, chi_ab=chiN / N, kappa=50.0,
                       Nx=grid, L=tuple(b * R for b in box_rg), lam_pl=lam_pl, lam_mi=lam_mi,
                       n_exp_nr=len(centers), L_nr=thickness_rg * R, R_nr=radius_rg * R, xi_nr=xi_rg * R,
                       center=cs, orient=(u, u), precision=precision, sigma=sigma, Ng=Ng,
                       shell_lambda=(-1.0 / N if shell else 0.0), shell_width=(0.1 * R if shell else 0.0),
                       plate_shape=shape)


def seeded_fields(p, seed: int, periods: int = 1) -> dict:
    """w_AB^- = 0.5 chi cos(2 pi periods x / L_x) + N(0, 0.01^2) per segment."""
    nx, ny, nz = p.Nx[0], p.Nx[1], p.Nx[2]
    rng = np.random.default_rng(seed)
    x = np.arange(nx) * p.L[0] / nx
    wabm = 0.5 * p.chi_ab * np.cos(2 * np.pi * periods * x / p.L[0])[None, None, :] + \
        0.01 * rng.standard_normal((nz, ny, nx))
    return {"wabm": wabm.astype(np.complex128)}


def sweep15(precision=PREC_MIXED, grid=(64, 64, 64), N=100):
    """The 15-angle sweep at 64^3, N=100 (one instance per angle)."""
    return [plate_params(t, N=N, grid=grid, precision=precision) for t in SWEEP_ANGLES]


def sweep15_mixed_sizes(precision=PREC_MIXED):
    """Config 2: the 15 angles on a mix of 48^3, 64^3 and 96x64x64 grids with
    N in {64, 100}; the assignment is fixed by seed 2."""
    rng = np.random.default_rng(2)
    grids = [(48, 48, 48), (64, 64, 64), (96, 64, 64)]
    out = []
    for t in SWEEP_ANGLES:
        g = grids[int(rng.integers(3))]
        N = (64, 100)[int(rng.integers(2))]
        box = tuple(6.4 * n / 64 for n in g)
        out.append(plate_params(t, N=N, grid=g, box_rg=box, precision=precision))
    return out


SEPARATIONS = tuple(round(0.14 + 0.04 * k, 2) for k in range(9))


def separation9(precision=PREC_MIXED):
    """Config 3: two parallel plates (theta = 0, normal along x) at centre
    separations d = 0.14 .. 0.46 of the long box side, N = 100, chiN = 20, on
    a 64 x 64 x 128 grid (box 6.4 x 6.4 x 12.8 Rg) with the separation along
    the long axis z, perpendicular to the plate normal as in the reference's
    particle-separation sweep (there along L_y; the disc is symmetric about
    its normal, so the two set-ups are the same up to a rotation)."""
    return [plate_params(0.0, grid=(64, 64, 128), box_rg=(6.4, 6.4, 12.8), precision=precision,
                         centers=((0.5, 0.5, 0.5 - d / 2), (0.5, 0.5, 0.5 + d / 2))) for d in SEPARATIONS]


def large_grafted8(precision=PREC_MIXED):
    """Config 4: 128 x 128 x 256 grid, box 12.8 x 12.8 x 25.6 Rg, N = 200,
    f_A = 0.4, chiN = 30, two plates rotated by 20 degrees at d = 0.25 L_z,
    each grafted with chains of Ng = 20 at sigma = 0.5 / Rg^2 (graft species
    A-like: chi_AC = 0, chi_BC = chi_AB); 8 instances that differ in the seed
    of their initial fields (seeded_fields with 1000 + k and 3 lamellar
    periods across L_x in the bench).  Step sizes 0.0005 / 0.0002: both the
    FP64 method and the mixed form diverge at 0.0015 / 0.0004 here (graft
    propagator q_g <= 0 after ~10 iterations)."""
    N = 200
    out = []
    for _ in range(8):
        p = plate_params(20.0, N=N, fA=0.4, chiN=30.0, grid=(128, 128, 256), box_rg=(12.8, 12.8, 25.6),
                         precision=precision, lam_pl=0.0005, lam_mi=0.0002,
                         centers=((0.5, 0.5, 0.375), (0.5, 0.5, 0.625)), sigma=0.5 / rg(N) ** 2, Ng=20)
        p.chi_bc = p.chi_ab
        out.append(p)
    return out


WORKLOADS = {
    "plate64_N100": lambda prec: [plate_params(10.0, precision=prec)],
    "plate64_N100_shell": lambda prec: [plate_params(10.0, precision=prec, shell=True)],
    # config 1 as written: a 1.6 x 1.6 x 0.2 Rg cuboid with a 0.1 Rg interface,
    # rotated by 10 degrees, with the A-attractive shell
    "plate64_N100_cuboid_shell": lambda prec: [plate_params(10.0, precision=prec, shell=True, shape=PLATE_CUBOID)],
    "sweep15_64_N100_shell": lambda prec: [plate_params(t, precision=prec, shell=True) for t in SWEEP_ANGLES],
    "sweep15_64_N100": lambda prec: sweep15(precision=prec),
    "sweep15_mixed_sizes": lambda prec: sweep15_mixed_sizes(precision=prec),
    "sep9_64x64x128_N100": lambda prec: separation9(precision=prec),
    "graft8_128x128x256_N200": lambda prec: large_grafted8(precision=prec),
    # a small case of the 128 x 128 plane family (profiling captures)
    "sweep4_128x128x64_N50": lambda prec: [plate_params(t, N=50, grid=(128, 128, 64), box_rg=(12.8, 12.8, 6.4),
                                                        precision=prec) for t in (0, 10, 20, 30)],
}

# per-workload defaults of the bench: relaxation iterations, how many
# instances the FP64 comparison runs (the FP64 method needs ~16 GB per
# instance of the large grafted workload) and the lamellar periods of the
# seeded fields (one period across a 12.8 Rg box at chiN = 30, N = 200 makes q
# span ~e^15 across the box, far from any saddle point)
BENCH_DEFAULTS = {
    "graft8_128x128x256_N200": {"relax": 30, "plain_max": 2, "periods": 3},
}
