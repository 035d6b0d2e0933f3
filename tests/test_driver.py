"""scft_run, the drop-in for the reference executable: bcp.input + w*.res in,
data.dat + *.p0.bin out, compared with what the reference's own simulate()
wrote for the same directory (tests/golden/driver_*, make_golden.py).

data.dat carries H with six decimals (code/simulate.cpp:132-135), so H and
-log Q are compared to 2e-6 absolute and the err column to 2e-3 relative; the
binary outputs hold full doubles and are compared to 1e-10 relative.
"""
import os
import shutil
import struct
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, PKG

DRIVER = os.path.join(PKG, "build", "scft_run")
CASES = ["driver_res", "driver_cos", "driver_euler", "driver_euler_negab"]


def read_bin(path):
    with open(path, "rb") as f:
        dim = struct.unpack("i", f.read(4))[0]
        nx = struct.unpack("3i", f.read(12))
        L = struct.unpack("3d", f.read(24))
        nprocs, ml = struct.unpack("2i", f.read(8))
        a = np.frombuffer(f.read(16 * ml), dtype=np.complex128)
    return dim, nx, L, nprocs, a


def read_dat(path):
    return np.loadtxt(path, ndmin=2)


def stage(tmp, name):
    src = os.path.join(GOLDEN, name)
    dst = os.path.join(tmp, name)
    os.makedirs(dst)
    for f in os.listdir(src):
        if not f.endswith(".ref"):
            shutil.copy(os.path.join(src, f), dst)
    return dst


def compare_run(run, name, h_abs=2e-6, bin_rel=1e-10):
    ref = read_dat(os.path.join(GOLDEN, name, "data.dat.ref"))
    got = read_dat(os.path.join(run, "data.dat"))
    assert got.shape == ref.shape
    assert (got[:, 0] == ref[:, 0]).all()
    for col in (1, 3):  # Re H, Re -log Qd
        assert np.abs(got[:, col] - ref[:, col]).max() <= h_abs * max(1.0, np.abs(ref[:, col]).max()), col
    assert np.allclose(got[:, 5:9], ref[:, 5:9])
    assert np.allclose(got[:, 9], ref[:, 9], rtol=2e-3, atol=1e-12)
    for f in ("wpl.p0.bin", "wabm.p0.bin", "rhoda.p0.bin", "rhodb.p0.bin", "rhoda_c.p0.bin"):
        d1, n1, L1, p1, a = read_bin(os.path.join(run, f))
        d0, n0, L0, p0, b = read_bin(os.path.join(GOLDEN, name, f + ".ref"))
        assert (d1, n1, L1, p1) == (d0, n0, L0, p0), f
        assert np.abs(a - b).max() <= bin_rel * np.abs(b).max(), f


@pytest.mark.gpu
@pytest.mark.parametrize("name", CASES)
def test_driver_matches_reference_run(tmp_path, name):
    run = stage(str(tmp_path), name)
    r = subprocess.run([DRIVER, "--quiet", run], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    compare_run(run, name)


@pytest.mark.gpu
def test_driver_batch_of_directories(tmp_path):
    """Runs with both update schemes in one batch."""
    runs = [stage(str(tmp_path), n) for n in CASES]
    r = subprocess.run([DRIVER, "--quiet"] + runs, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    for run, name in zip(runs, CASES):
        compare_run(run, name)


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["driver_res", "driver_euler"])
def test_driver_mixed_precision(tmp_path, name):
    run = stage(str(tmp_path), name)
    r = subprocess.run([DRIVER, "--quiet", "--mixed", run], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    ref = read_dat(os.path.join(GOLDEN, name, "data.dat.ref"))
    got = read_dat(os.path.join(run, "data.dat"))
    assert np.abs(got[:, 1] - ref[:, 1]).max() <= 2e-5 * np.abs(ref[:, 1]).max()


@pytest.mark.gpu
@pytest.mark.parametrize("name", ["driver_cl", "driver_cl_negab", "driver_cl_euler"])
def test_driver_complex_langevin_matches_reference(tmp_path, name):
    """do_CL = 1: the noise is the reference's own random stream (the fixture
    was written with idum = -12345), so fields, densities and the running
    averages match the reference run (code/1s_update.cpp:54-368,
    code/Euler_update.cpp:49-172, code/array_utils.cpp:13-45)."""
    run = stage(str(tmp_path), name)
    r = subprocess.run([DRIVER, "--quiet", "--seed", "12345", run], capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    compare_run(run, name)
    for f in ("avg_rhoda.p0.bin", "avg_rhodb.p0.bin"):
        _, _, _, _, a = read_bin(os.path.join(run, f))
        _, _, _, _, b = read_bin(os.path.join(GOLDEN, name, f + ".ref"))
        assert np.abs(a - b).max() <= 1e-10 * np.abs(b).max(), f


@pytest.mark.gpu
def test_complex_langevin_seed_changes_the_noise(tmp_path):
    runs = []
    for seed in ("12345", "777"):
        run = stage(str(tmp_path / seed), "driver_cl")
        r = subprocess.run([DRIVER, "--quiet", "--seed", seed, run], capture_output=True, text=True, timeout=600)
        assert r.returncode == 0, r.stderr
        runs.append(read_bin(os.path.join(run, "wpl.p0.bin"))[4])
    assert np.abs(runs[0] - runs[1]).max() > 1e-3 * np.abs(runs[0]).max()


def _driver_or_skip():
    if not os.path.exists(DRIVER):
        from scft.build import build

        build()
    return DRIVER


@pytest.mark.parametrize("edit,message", [
    (lambda s: s.replace("0.0 0  phiAH, Nah", "0.1 10  phiAH, Nah"), "homopolymer"),
    (lambda s: s.replace("0  do_fld_np", "1  do_fld_np"), "field-based"),
    (lambda s: s.replace("0  do_film", "1  do_film"), "films"),
])
def test_driver_rejects_inputs_like_the_reference(tmp_path, edit, message):
    """Input errors are reported before any GPU work (code/read_input.cpp:40-45,
    184-189), so this runs on the CPU."""
    drv = _driver_or_skip()
    run = stage(str(tmp_path), "driver_res")
    p = os.path.join(run, "bcp.input")
    s = open(p).read()
    s2 = edit(s)
    assert s2 != s
    open(p, "w").write(s2)
    r = subprocess.run([drv, "--quiet", run], capture_output=True, text=True, timeout=60)
    assert r.returncode == 1
    assert message in r.stderr
