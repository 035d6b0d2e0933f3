"""Failure detection on the host (no GPU): the driver's input checks, and the
compiled reference's own exits on the inputs the GPU failure tests use.

The reference stops the process on bad input (code/read_input.cpp:12-19,
40-45, 184-189, code/io_utils.cpp:138-177), on H = NaN (exit 1,
code/calc_h.cpp:38-61) and on a grafted propagator q_g[Ng-1] <= 0 at 5 or
more points (exit 4, code/grafted_nanoparticle.cpp:82-107).  The library
returns SCFT_ERR_NAN / SCFT_ERR_QNONPOS instead (tests/test_gpu_failures.py);
the driver scft_run prints the reason and exits 1, before any GPU work for
input errors, which is what these tests run.
"""
import math
import os
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG

DRIVER = os.path.join(PKG, "build", "scft_run")


def small_case(**kw):
    from ref_case import Case

    base = dict(Nx=(8, 10, 6), L=(4.0, 5.0, 3.5), a_smear=0.2, rho0=5.0, kappa=50.0, lam_pl=0.005, lam_mi=0.005,
                L_nr=0.6, R_nr=1.2, xi_nr=0.3, Nda=3, Ndb=5, chi_ab=0.5, n_exp_nr=1,
                centers=((0.4, 0.55, 0.5), (0.5, 0.5, 0.5)), orients=((0.9, 0.3, 0.1), (1.0, 0.0, 0.0)),
                itermax=3, print_freq=1)
    base.update(kw)
    return Case(**base)


def run_driver(d):
    if not os.path.exists(DRIVER):
        pytest.skip("driver not built")
    return subprocess.run([DRIVER, "--quiet", d], capture_output=True, text=True, timeout=120)


def test_driver_rejects_truncated_bcp_input(tmp_path):
    from ref_case import write_case

    c = small_case()
    write_case(str(tmp_path), c)
    p = tmp_path / "bcp.input"
    p.write_text("\n".join(p.read_text().splitlines()[:20]) + "\n")
    r = run_driver(str(tmp_path))
    assert r.returncode == 1
    assert "truncated or malformed" in r.stderr


def test_driver_rejects_plate_centre_outside_the_box(tmp_path):
    from ref_case import write_case

    write_case(str(tmp_path), small_case(centers=((1.4, 0.5, 0.5), (0.5, 0.5, 0.5))))
    r = run_driver(str(tmp_path))
    assert r.returncode == 1
    # the reference's own message (code/read_input.cpp)
    assert "Nanorod center isn't valid" in r.stderr


def test_driver_rejects_homopolymer_blend(tmp_path):
    from ref_case import write_case

    write_case(str(tmp_path), small_case(phiH=0.2, Nah=4))
    r = run_driver(str(tmp_path))
    assert r.returncode == 1
    assert "No homopolymer allowed" in r.stderr


def test_driver_rejects_short_resume_file_before_gpu_work(tmp_path):
    from ref_case import write_case

    c = small_case()
    c.fields = {"wabm": np.zeros(c.shape, np.complex128)}
    write_case(str(tmp_path), c)
    res = tmp_path / "wabm.res"
    lines = res.read_text().splitlines()
    res.write_text("\n".join(lines[: len(lines) // 2]) + "\n")
    r = run_driver(str(tmp_path))
    assert r.returncode == 1
    assert "fewer than Nx*Ny*Nz lines" in r.stderr
    # no context was made: the run stopped before scft_create
    assert "scft_create" not in r.stderr


def qnonpos_case():
    """tiny_graft with a uniform real wpl = pi / Ng: w_G = i wpl + ... turns
    q_g[Ng-1] = e^{-i pi} |q_g| negative at every grid point (the reference's
    phase convention keeps wpl imaginary; a real wpl is a valid but
    unphysical input)."""
    from test_gpu_parity import load_golden

    c, _ = load_golden("tiny_graft")
    c.fields = dict(c.fields)
    c.fields["wpl"] = np.full(c.shape, math.pi / c.Ng, np.complex128)
    return c


def nan_case():
    from test_gpu_parity import load_golden

    c, _ = load_golden("tiny_plate")
    c.fields = dict(c.fields)
    w = np.array(c.fields["wabm"])
    w[2, 3, 4] = np.nan
    c.fields["wabm"] = w
    return c


def test_reference_exits_4_when_graft_propagator_is_not_positive(tmp_path):
    from ref_case import REF_BIN, write_case

    if not os.path.exists(REF_BIN):
        pytest.skip("oracle binary not built")
    write_case(str(tmp_path), qnonpos_case())
    r = subprocess.run([REF_BIN, "dump", "0"], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert r.returncode == 4, r.stdout[-500:]


def test_reference_exits_1_on_nan_hamiltonian(tmp_path):
    from ref_case import REF_BIN, write_case

    if not os.path.exists(REF_BIN):
        pytest.skip("oracle binary not built")
    write_case(str(tmp_path), nan_case())
    r = subprocess.run([REF_BIN, "dump", "0"], cwd=str(tmp_path), capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "Hcur is NaN" in r.stdout
