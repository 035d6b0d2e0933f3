"""Parity of the CUDA path (libscft via its C ABI) with the reference.

Sources of truth, in order: the golden fixtures written by the reference
itself (tests/golden/, make_golden.py) and the numpy restatement
(oracle/scft_oracle.py), which tests/test_oracle.py pins to those fixtures.

Tolerances (plain FP64 method): densities 1e-10 relative, H 1e-9 relative,
the bar set for this path; FFTs 1e-13 relative to numpy.
"""
import json
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

TINY = ["tiny_plate", "tiny_graft", "tiny_negab_oddN", "tiny_single_block"]
RHO_TOL = 1e-10
H_TOL = 1e-9


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def scft():
    import torch

    if not torch.cuda.is_available():
        pytest.fail("gpu tests need a CUDA device")
    import scft as S

    S.load()
    return S


def load_golden(name):
    from ref_case import Case

    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    c.fields = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    return c, z


@pytest.mark.parametrize("shape", [(8, 8, 8), (6, 10, 12), (16, 24, 48), (4, 9, 96), (64, 64, 64), (3, 32, 8),
                                   (4, 128, 128)])
def test_fft3d_matches_numpy(scft, shape):
    nz, ny, nx = shape
    p = scft.make_params(Nx=(nx, ny, nz), L=(1.0, 1.0, 1.0))
    rng = np.random.default_rng(nx * ny + nz)
    a = rng.standard_normal((2,) + shape) + 1j * rng.standard_normal((2,) + shape)
    with scft.Context(p) as ctx:
        f = ctx.fft3d(0, a, -1)
        b = ctx.fft3d(0, a, +1)
    M = nx * ny * nz
    ref_f = np.fft.fftn(a, axes=(1, 2, 3)) / M  # forward scaled by 1/M
    ref_b = np.fft.ifftn(a, axes=(1, 2, 3)) * M  # backward unscaled
    assert rel(f, ref_f) < 1e-13
    assert rel(b, ref_b) < 1e-13


@pytest.mark.parametrize("name", TINY)
def test_setup_tables_match_reference(scft, name):
    c, z = load_golden(name)
    sc = json.loads(str(z["scalars_json"]))
    with scft.Context(scft.params_from_case(c)) as ctx:
        info = ctx.info(0)
    assert abs(info["nD"] - sc["nD"]) <= 1e-12 * sc["nD"]
    assert abs(info["np_frac"] - sc["np_frac"]) <= 1e-12 * max(sc["np_frac"], 1e-300) + 1e-300
    assert abs(info["phiG"] - sc["phiG"]) <= 1e-12 * max(sc["phiG"], 1e-300) + 1e-300


@pytest.mark.parametrize("name", TINY)
def test_diblock_density_matches_reference(scft, name):
    """diblock_discrete + integrate_diblock_discrete on the reference's own
    smeared fields (code/diblock_discrete.cpp:4-95)."""
    c, z = load_golden(name)
    sc = json.loads(str(z["scalars_json"]))
    with scft.Context(scft.params_from_case(c)) as ctx:
        ra, rb, Q = ctx.diblock_density(0, z["smwa0"], z["smwb0"])
    assert abs(Q - complex(sc["Qd_re"], sc["Qd_im"])) <= RHO_TOL * abs(complex(sc["Qd_re"], sc["Qd_im"]))
    assert rel(ra, z["rhoda0"]) < RHO_TOL
    assert rel(rb, z["rhodb0"]) < RHO_TOL


@pytest.mark.parametrize("name", TINY)
def test_update_1s_trace_matches_reference(scft, name):
    """H and Q after every update_1s, final fields and densities."""
    c, z = load_golden(name)
    tr = z["trace"]
    iters = int(tr[-1, 0])
    with scft.Context(scft.params_from_case(c)) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        ra0, rb0, _ = ctx.density(0)
        rows = [ctx.calc_H()[0]]
        for _ in range(iters):
            ctx.update_1s(1)
            rows.append(ctx.calc_H()[0])
        f = ctx.get_fields(0)
        ra, rb, _ = ctx.density(0)
        sa, sb, _ = ctx.smeared(0)
    rows = np.array(rows)
    assert rel(ra0, z["rhoda0"]) < RHO_TOL
    assert rel(rb0, z["rhodb0"]) < RHO_TOL
    assert np.abs(rows[:, 0] - tr[:, 1]).max() <= H_TOL * np.abs(tr[:, 1]).max()
    assert np.abs(rows[:, 2] - tr[:, 3]).max() <= RHO_TOL * np.abs(tr[:, 3]).max()
    for k in ("wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm"):
        if np.abs(z[k]).max() > 0:
            assert rel(f[k], z[k]) < RHO_TOL, k
    assert rel(ra, z["rhoda"]) < RHO_TOL
    assert rel(rb, z["rhodb"]) < RHO_TOL
    assert rel(sa, z["smwa"]) < RHO_TOL
    assert rel(sb, z["smwb"]) < RHO_TOL


def test_batched_uneven_instances_match_reference(scft):
    """All tiny cases (different N, Na, chemistry, plates) in one context."""
    cases = [load_golden(n) for n in TINY if n != "tiny_graft"]
    params = [scft.params_from_case(c) for c, _ in cases]
    with scft.Context(params) as ctx:
        for k, (c, _) in enumerate(cases):
            ctx.set_fields(k, c.fields)
        ctx.calc_poly_density()
        H0 = ctx.calc_H()
        ctx.update_1s(4)
        H4 = ctx.calc_H()
        dens = [ctx.density(k) for k in range(len(cases))]
    import scft_oracle as O

    for k, (c, z) in enumerate(cases):
        tr = z["trace"]
        assert abs(H0[k, 0] - tr[0, 1]) <= H_TOL * abs(tr[0, 1])
        assert abs(H4[k, 0] - tr[4, 1]) <= H_TOL * abs(tr[4, 1])
        s = O.System.from_case(c)
        st = O.State.from_fields(s.g, c.fields)
        O.run(s, st, 4)
        assert rel(dens[k][0], st.out["rhoda"]) < RHO_TOL
        assert rel(dens[k][1], st.out["rhodb"]) < RHO_TOL


def test_homopolymer_matches_reference(scft):
    """scft_homopolymer_density against the reference's own
    homopolymer_discrete + integrate_homopoly_discrete (run by the oracle
    harness on the smeared w_A of tiny_plate; tests/golden/tiny_homopolymer.npz)."""
    c, _ = load_golden("tiny_plate")
    z = np.load(os.path.join(GOLDEN, "tiny_homopolymer.npz"))
    with scft.Context(scft.params_from_case(c)) as ctx:
        r, Q = ctx.homopolymer_density(0, z["W"], int(z["Nh"]), float(z["nK"]))
    Qr = complex(z["Q"])
    assert abs(Q - Qr) <= RHO_TOL * abs(Qr)
    assert rel(r, z["rho"]) < RHO_TOL


def test_homopolymer_matches_restatement(scft):
    """homopolymer_discrete + integrate_homopoly_discrete (dead in the shipped
    inputs, code/read_input.cpp:40-45) against the restatement."""
    import scft_oracle as O

    c, z = load_golden("tiny_plate")
    s = O.System.from_case(c)
    rng = np.random.default_rng(5)
    W = 0.2 * rng.standard_normal(s.g.shape) + 0j
    Qr, q = O.homopolymer_discrete(s, W, 7)
    rr = O.integrate_homopoly_discrete(s, q, Qr, 3.5, W, 7)
    with scft.Context(scft.params_from_case(c)) as ctx:
        r, Q = ctx.homopolymer_density(0, W, 7, 3.5)
    assert abs(Q - Qr) <= RHO_TOL * abs(Qr)
    assert rel(r, rr) < RHO_TOL


def test_config0_full_size_trace(scft):
    """Config 0 (32^3, N=32, 200 x update_1s): H every iteration against the
    reference's own trace, and digests of the final densities and fields."""
    import sys

    sys.path.insert(0, GOLDEN)
    from make_golden import config0_case, digest

    z = np.load(os.path.join(GOLDEN, "config0_32cubed_N32.npz"))
    c = config0_case()
    tr = z["trace"]
    with scft.Context(scft.params_from_case(c)) as ctx:
        ctx.set_fields(0, c.fields)
        ctx.calc_poly_density()
        rows = [ctx.calc_H()[0]]
        for _ in range(200):
            ctx.update_1s(1)
            rows.append(ctx.calc_H()[0])
        f = ctx.get_fields(0)
        ra, rb, _ = ctx.density(0)
    rows = np.array(rows)
    assert np.abs(rows[:, 0] - tr[:, 1]).max() <= H_TOL * np.abs(tr[:, 1]).max()
    for k, a in (("rhoda", ra), ("rhodb", rb), ("wpl", f["wpl"]), ("wabm", f["wabm"])):
        assert rel(digest(a), z["digest_" + k]) < RHO_TOL, k


def test_large_plane_in_global_memory_matches_restatement(scft):
    """A 128 x 128 FP64 plane (256 KB) does not fit in shared memory: the plane
    kernels then work on it in place in global memory.  Propagators and
    densities against the restatement (code/diblock_discrete.cpp:4-95)."""
    import scft_oracle as O

    Nx, L = (128, 128, 4), (8.0, 8.0, 1.0)
    s = O.System(Nda=4, Ndb=5, a_smear=0.2, rho0=5.0, chi_ab=0.5, chi_bc=0.0, chi_ac=0.0, kappa=50.0, Nx=Nx, L=L,
                 lam_pl=0.005, lam_mi=0.005)
    rng = np.random.default_rng(17)
    WA = 0.3 * rng.standard_normal(s.g.shape) + 0j
    WB = 0.3 * rng.standard_normal(s.g.shape) + 0j
    Qr, q, qd = O.diblock_discrete(s, WA, WB)
    ra_r, rb_r = O.integrate_diblock_discrete(s, q, qd, Qr, s.nD, WA, WB)
    with scft.Context(scft.make_params(Nda=4, Ndb=5, Nx=Nx, L=L)) as ctx:
        ra, rb, Q = ctx.diblock_density(0, WA, WB)
    assert abs(Q - Qr) <= RHO_TOL * abs(Qr)
    assert rel(ra, ra_r) < RHO_TOL
    assert rel(rb, rb_r) < RHO_TOL
