"""Pins the oracle: the numpy restatement (oracle/scft_oracle.py) and the FFT
shim used to compile the reference (oracle/fftw_shim/) against known answers
and against the golden fixtures produced by the reference itself."""
import ctypes
import json
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, ROOT

import scft_oracle as O
from ref_case import Case
import sys as _sys
_sys.path.insert(0, GOLDEN)

SHIM = os.path.join(ROOT, "oracle", "_ref", "libfftw_shim.so")
TINY = ["tiny_plate", "tiny_graft", "tiny_negab_oddN", "tiny_single_block"]


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    c.fields = {k[3:]: z[k] for k in z.files if k.startswith("in_")}
    return c, z


def rel(a, b):
    return float(np.abs(a - b).max() / max(np.abs(b).max(), 1e-300))


@pytest.fixture(scope="module")
def shim():
    if not os.path.exists(SHIM):
        subprocess.run(["make", "-C", os.path.join(ROOT, "oracle"), "shim"], check=True,
                       capture_output=True)
    lib = ctypes.CDLL(SHIM)
    lib.fftw_plan_dft.restype = ctypes.c_void_p
    lib.fftw_plan_dft.argtypes = [ctypes.c_int, ctypes.POINTER(ctypes.c_int), ctypes.c_void_p,
                                  ctypes.c_void_p, ctypes.c_int, ctypes.c_uint]
    lib.fftw_execute.argtypes = [ctypes.c_void_p]
    lib.fftw_destroy_plan.argtypes = [ctypes.c_void_p]
    return lib


def direct_dft(a, sign):
    """Known answer: the defining O(n^2) sum along each axis."""
    out = a.astype(np.complex128)
    for ax in range(a.ndim):
        n = a.shape[ax]
        j = np.arange(n)
        W = np.exp(sign * 2j * np.pi * (np.outer(j, j) % n) / n)
        out = np.moveaxis(np.tensordot(W, np.moveaxis(out, ax, 0), axes=(1, 0)), 0, ax)
    return out


@pytest.mark.parametrize("shape", [(8, 8, 8), (12, 10, 6), (6, 16, 9), (7, 11, 5), (3, 48, 2)])
@pytest.mark.parametrize("sign", [-1, 1])
def test_shim_fft_known_answer(shim, shape, sign):
    rng = np.random.default_rng(sum(shape))
    a = rng.standard_normal(shape) + 1j * rng.standard_normal(shape)
    out = np.zeros_like(a)
    n = (ctypes.c_int * 3)(*shape)
    p = shim.fftw_plan_dft(3, n, a.ctypes.data, out.ctypes.data, sign, 0)
    shim.fftw_execute(p)
    shim.fftw_destroy_plan(p)
    assert rel(out, direct_dft(a, sign)) < 1e-14


def test_shim_fft_in_place_and_zeroed_malloc(shim):
    shim.fftw_malloc.restype = ctypes.c_void_p
    shim.fftw_malloc.argtypes = [ctypes.c_size_t]
    shim.fftw_free.argtypes = [ctypes.c_void_p]
    p = shim.fftw_malloc(4096)
    assert all(b == 0 for b in ctypes.string_at(p, 4096))
    shim.fftw_free(p)
    rng = np.random.default_rng(3)
    a = rng.standard_normal((4, 6, 10)) + 0j
    ref = np.fft.fftn(a)
    n = (ctypes.c_int * 3)(4, 6, 10)
    pl = shim.fftw_plan_dft(3, n, a.ctypes.data, a.ctypes.data, -1, 0)
    shim.fftw_execute(pl)
    assert rel(a, ref) < 1e-14


def test_oracle_fft_conventions():
    g = O.Grid((6, 4, 10), (3.0, 2.0, 5.0))
    rng = np.random.default_rng(0)
    a = rng.standard_normal(g.shape) + 1j * rng.standard_normal(g.shape)
    # forward scaled by 1/M, backward unscaled (code/fft_wrappers.cpp:4-64)
    assert rel(O.fft_fwd(g, a), direct_dft(a, -1) / g.M) < 1e-14
    assert rel(O.fft_bck(g, O.fft_fwd(g, a)), a) < 1e-14


@pytest.mark.parametrize("name", TINY)
def test_restatement_matches_reference_fixture(name):
    c, z = load_golden(name)
    s = O.System.from_case(c)
    st = O.State.from_fields(s.g, c.fields)
    iters = int(z["trace"][-1, 0])
    rows = O.run(s, st, iters)
    tr = z["trace"]
    # H and Q per iteration: the bar is 1e-9 relative (H), found ~1e-15
    assert np.abs(rows[:, 1] - tr[:, 1]).max() <= 1e-12 * np.abs(tr[:, 1]).max()
    assert np.abs(rows[:, 3] - tr[:, 3]).max() <= 1e-12 * np.abs(tr[:, 3]).max()
    if c.sigma > 0:
        assert np.abs(rows[:, 5] - tr[:, 5]).max() <= 1e-12 * np.abs(tr[:, 5]).max()
    for k in ("hhat", "poly_bond_fft", "gaa", "gab", "gbb", "rho_exp_nr", "expl_grafts"):
        if np.abs(z[k]).max() > 0:
            assert rel(s.tables[k], z[k]) < 1e-12, k
    for k in ("wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm"):
        if np.abs(z[k]).max() > 0:
            assert rel(getattr(st, k), z[k]) < 1e-12, k
    for k in ("rhoda", "rhodb", "smwa", "smwb"):
        assert rel(st.out[k], z[k]) < 1e-12, k
    sc = json.loads(str(z["scalars_json"]))
    assert abs(s.nD - sc["nD"]) <= 1e-13 * sc["nD"]


@pytest.mark.parametrize("name", TINY)
def test_restatement_propagators_match_reference(name):
    c, z = load_golden(name)
    s = O.System.from_case(c)
    st = O.State.from_fields(s.g, c.fields)
    O.calc_poly_density(s, st, keep_hist=True)
    assert rel(st.out["qd"], z["qd0"]) < 1e-12
    assert rel(st.out["qddag"], z["qddag0"]) < 1e-12
    assert rel(st.out["rhoda"], z["rhoda0"]) < 1e-12


def test_restatement_homopolymer_matches_reference():
    """homopolymer_discrete + integrate_homopoly_discrete (code/
    homopolymer_discrete.cpp:3-55, code/calc_poly_density.cpp:193-212), dead
    in the shipped inputs, run by the oracle harness on the smeared w_A of the
    tiny_plate case (tests/golden/tiny_homopolymer.npz)."""
    c, _ = load_golden("tiny_plate")
    z = np.load(os.path.join(GOLDEN, "tiny_homopolymer.npz"))
    s = O.System.from_case(c)
    Nh, nK = int(z["Nh"]), float(z["nK"])
    Q, q = O.homopolymer_discrete(s, z["W"], Nh)
    rho = O.integrate_homopoly_discrete(s, q, Q, nK, z["W"], Nh)
    assert abs(Q - complex(z["Q"])) <= 1e-13 * abs(complex(z["Q"]))
    assert rel(rho, z["rho"]) < 1e-12


def test_segment_count_invariant():
    """code/simulate.cpp:61-72: integral(rho_A + rho_B) = nD * N."""
    c, _ = load_golden("tiny_plate")
    s = O.System.from_case(c)
    st = O.State.from_fields(s.g, c.fields)
    o = O.calc_poly_density(s, st)
    tot = O.integ_trapPBC(s.g, o["rhoda"] + o["rhodb"]).real
    assert abs(tot - s.nD * s.N) < 1e-10 * s.nD * s.N


def test_restatement_config0_trace():
    """Config 0 (32^3, N=32, 200 x update_1s): full-size H trace and digests."""
    z = np.load(os.path.join(GOLDEN, "config0_32cubed_N32.npz"))
    d = json.loads(str(z["case_json"]))
    c = Case(**{k: (tuple(map(tuple, v)) if k in ("centers", "orients", "ic") else
                    (tuple(v) if isinstance(v, list) else v)) for k, v in d.items()})
    from make_golden import config0_case, digest
    c.fields = config0_case().fields
    s = O.System.from_case(c)
    st = O.State.from_fields(s.g, c.fields)
    rows = O.run(s, st, 200)
    tr = z["trace"]
    assert np.abs(rows[:, 1] - tr[:, 1]).max() <= 1e-10 * np.abs(tr[:, 1]).max()
    for k in ("rhoda", "rhodb", "wpl", "wabm"):
        src = st.out[k] if k.startswith("rho") else getattr(st, k)
        assert rel(digest(src), z["digest_" + k]) < 1e-10, k


def test_shell_extension_profile():
    """The shell potential (an extension of the restatement, no reference
    counterpart): zero with Lambda = 0, of Lambda's sign, largest just outside
    the plate, and without effect on the reference path when off."""
    import dataclasses

    c, _ = load_golden("tiny_plate")
    s0 = O.System.from_case(c)
    assert np.abs(s0.tables["shellU"]).max() == 0.0
    s = dataclasses.replace(s0, shell_lambda=-0.3, shell_width=0.4)
    U = s.tables["shellU"]
    assert U.max() <= 1e-15 and U.min() < -0.05
    core = s.tables["rho_exp_nr"].real
    assert U[core > 0.9].mean() > U.min() / 4  # weak inside the core


@pytest.mark.parametrize("name", ["driver_euler", "driver_euler_negab"])
def test_restatement_euler_matches_reference_driver(name):
    """update_Euler (code/Euler_update.cpp) in the restatement against the
    reference's own simulate() run: itermax + 1 = 13 explicit steps (the loop
    runs iter = 0..itermax, code/simulate.cpp:85) from the same .res fields;
    final fields and unsmeared densities (*_c.p0.bin) from its output."""
    import struct

    _sys.path.insert(0, GOLDEN)
    from make_golden import driver_cases

    c = driver_cases()[name]
    s = O.System.from_case(c)
    assert s.update_scheme == 0
    st = O.State.from_fields(s.g, c.fields)
    O.run(s, st, 13)

    def read_bin(f):
        with open(os.path.join(GOLDEN, name, f + ".p0.bin.ref"), "rb") as fh:
            fh.read(4 + 12 + 24)
            _, ml = struct.unpack("2i", fh.read(8))
            return np.frombuffer(fh.read(16 * ml), dtype=np.complex128)

    got = {"wpl": st.wpl, "wabp": st.wabp, "wabm": st.wabm, "rhoda_c": st.out["rhoda"], "rhodb_c": st.out["rhodb"]}
    for k, v in got.items():
        ref = read_bin(k)
        assert np.abs(v.ravel() - ref).max() <= 1e-10 * np.abs(ref).max(), k
