"""Generates the committed golden fixtures in tests/golden/ by running the
reference SCFT code itself (compiled by oracle/Makefile into
oracle/_ref/scft_ref, Dim=3, FFT via the oracle shim).

    make -C oracle && python tests/golden/make_golden.py
    python tests/golden/make_golden.py --homopolymer | --separation
    python tests/golden/make_golden.py --large [name ...]   (configs 1, 3, 4;
                                                             about 20 min and
                                                             35 GB of host RAM)

Each fixture <name>.npz holds
  case_json      the bcp.input parameters (json text)
  in_<field>     the seeded initial fields written as w*.res
  trace          rows [iter, Re H, Im H, Re Qd, Im Qd, Re Qga, Im Qga] after
                 0..iters update_1s() calls, at full precision
  scalars_json   nD, phiD, Vf, np_frac, ... after initialisation
  <array>        reference outputs (see ARRAYS), or, for the large
                 config-0 case, per-array digests (see digest()).
"""
from __future__ import annotations

import json
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

from ref_case import Case, run_reference  # noqa: E402

ARRAYS = ["hhat", "poly_bond_fft", "gaa", "gab", "gbb", "rho_exp_nr", "expl_grafts", "smwa0", "smwb0",
          "rhoda0", "rhodb0", "wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm", "smwa", "smwb",
          "rhoda", "rhodb"]
DIGEST_IDX_SEED = 7


def seeded_fields(c: Case, seed: int, amp: float, noise: float, extra: bool) -> dict:
    """Lamellar w_AB^- along x plus small seeded noise; imaginary w+ and w_AB^+
    (the reference's mean-field phase convention, code/initialize.cpp:459-481)."""
    rng = np.random.default_rng(seed)
    x = np.arange(c.Nx[0]) * c.L[0] / c.Nx[0]
    f = {}
    f["wabm"] = (amp * np.cos(2 * np.pi * x / c.L[0])[None, None, :]
                 + noise * rng.standard_normal(c.shape)).astype(np.complex128)
    f["wpl"] = 1j * noise * rng.standard_normal(c.shape)
    f["wabp"] = 1j * noise * rng.standard_normal(c.shape)
    if extra:
        f["wbcm"] = (5 * noise * rng.standard_normal(c.shape)).astype(np.complex128)
        f["wbcp"] = 1j * noise * rng.standard_normal(c.shape)
        f["wacm"] = (5 * noise * rng.standard_normal(c.shape)).astype(np.complex128)
        f["wacp"] = 1j * 2 * noise * rng.standard_normal(c.shape)
    return f


def tiny_cases() -> dict:
    base = dict(Nx=(8, 10, 6), L=(4.0, 5.0, 3.5), a_smear=0.2, rho0=5.0, kappa=50.0, lam_pl=0.005,
                lam_mi=0.005, L_nr=0.6, R_nr=1.2, xi_nr=0.3)
    cases = {}
    c = Case(Nda=3, Ndb=5, chi_ab=0.5, n_exp_nr=1, centers=((0.4, 0.55, 0.5), (0.5, 0.5, 0.5)),
             orients=((0.9, 0.3, 0.1), (1.0, 0.0, 0.0)), **base)
    c.fields = seeded_fields(c, 1, 0.3, 0.01, False)
    cases["tiny_plate"] = (c, 6, True)
    c = Case(Nda=3, Ndb=5, chi_ab=0.5, chi_bc=-0.2, chi_ac=0.4, sigma=0.3, Ng=4, n_exp_nr=2,
             centers=((0.3, 0.5, 0.5), (0.7, 0.5, 0.5)), orients=((0.9, 0.3, 0.1), (0.2, 1.0, 0.0)),
             **base)
    c.fields = seeded_fields(c, 2, 0.3, 0.01, True)
    cases["tiny_graft"] = (c, 6, True)
    c = Case(Nda=3, Ndb=4, chi_ab=-0.3, n_exp_nr=0, **base)
    c.fields = seeded_fields(c, 3, 0.3, 0.01, False)
    cases["tiny_negab_oddN"] = (c, 6, True)
    c = Case(Nda=5, Ndb=0, chi_ab=0.5, n_exp_nr=1, centers=((0.5, 0.5, 0.5), (0.5, 0.5, 0.5)),
             orients=((1.0, 0.0, 0.0), (1.0, 0.0, 0.0)), **base)
    c.fields = seeded_fields(c, 4, 0.3, 0.01, False)
    cases["tiny_single_block"] = (c, 4, True)
    return cases


def config0_case() -> Case:
    """Config 0: AB diblock, N=32, f=0.5, chiN=20, C=50, 32^3 grid, box 4.0 Rg.
    b-units with Rg^2=(N-1)/6 (code/initialize.cpp:55): chi=chiN/N,
    rho0=C*N/Rg^3, w_AB^- = 0.5*chi*cos(2*pi*x/L) + N(0, 0.01^2) per segment."""
    N = 32
    Rg = np.sqrt((N - 1) / 6.0)
    Lb = 4.0 * Rg
    c = Case(Nda=16, Ndb=16, a_smear=0.2, rho0=50.0 * N / Rg ** 3, chi_ab=20.0 / N, kappa=50.0,
             Nx=(32, 32, 32), L=(Lb, Lb, Lb), lam_pl=0.005, lam_mi=0.005, n_exp_nr=0)
    rng = np.random.default_rng(20240)
    x = np.arange(32) * Lb / 32
    c.fields = {"wabm": (0.5 * c.chi_ab * np.cos(2 * np.pi * x / Lb)[None, None, :]
                         + 0.01 * rng.standard_normal(c.shape)).astype(np.complex128),
                "wpl": np.zeros(c.shape, np.complex128),
                "wabp": np.zeros(c.shape, np.complex128)}
    return c


def digest(a: np.ndarray, samples: int = 64) -> np.ndarray:
    """Size-independent summary: sum, sum of |.|^2, and `samples` sampled points."""
    a = a.ravel()
    idx = np.random.default_rng(DIGEST_IDX_SEED).choice(a.size, samples, replace=False)
    return np.concatenate([[a.sum(), (np.abs(a) ** 2).sum()], a[idx]])


# Benchmark configurations 1, 3 and 4 at full size, plain FP64 method: the
# reference runs `iters` update_1s() from the seeded fields of the bench
# workloads (scft/workloads.py); the fixtures hold the H/Q trace and digests
# (LARGE_SAMPLES points each) of the initial and final densities, fields and
# smeared fields, plus a digest of the seeded input so that a test can check
# that it regenerated the same fields.
LARGE_SAMPLES = 512
LARGE_ARRAYS = ["rhoda0", "rhodb0", "smwa0", "smwb0", "rhoda", "rhodb", "wpl", "wabp", "wabm", "smwa", "smwb"]


def large_cases() -> dict:
    """name -> (workload name, instance index, seed, lamellar periods, iters)."""
    return {
        "config1_plate64_N100": ("plate64_N100", 0, 1001, 1, 3),
        "config3_sep030_64x64x128_N100": ("sep9_64x64x128_N100", 4, 1004, 1, 3),
        "config4_graft_128x128x256_N200": ("graft8_128x128x256_N200", 0, 1000, 3, 1),
        # config 2's two non-64^3 grids (instances 5 and 9 of the mixed-size sweep)
        "config2_96x64x64_N100": ("sweep15_mixed_sizes", 5, 1005, 1, 3),
        "config2_48cubed_N100": ("sweep15_mixed_sizes", 9, 1009, 1, 3),
    }


def large_case(name: str):
    """(params, Case) of one large fixture, FP64 method, seeded fields included."""
    sys.path.insert(0, os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300"))
    import scft
    from scft.workloads import WORKLOADS, seeded_fields as ws
    from ref_case import case_from_params

    wl, k, seed, periods, iters = large_cases()[name]
    p = WORKLOADS[wl](scft.PREC_FP64)[k]
    return p, case_from_params(p, ws(p, seed, periods=periods)), iters


def make_large_fixtures(tmp, names=None):
    for name in (names or large_cases()):
        p, c, iters = large_case(name)
        out = run_reference(os.path.join(tmp, name), c, iters, hist=False, timeout=6 * 3600)
        z = {"case_json": case_json(c), "trace": out["trace"], "scalars_json": json.dumps(out["scalars"]),
             "digest_idx_seed": DIGEST_IDX_SEED, "samples": LARGE_SAMPLES,
             "digest_in_wabm": digest(c.fields["wabm"], LARGE_SAMPLES)}
        arrays = LARGE_ARRAYS + (["rhog_exp0", "rhog_exp"] if c.sigma > 0 and c.n_exp_nr > 0 else [])
        for k in arrays:
            z["digest_" + k] = digest(out[k], LARGE_SAMPLES)
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **z)
        print(name, "H0", out["trace"][0, 1], "H_end", out["trace"][-1, 1], flush=True)
        import shutil

        shutil.rmtree(os.path.join(tmp, name), ignore_errors=True)


def case_json(c: Case) -> str:
    d = {k: getattr(c, k) for k in c.__dataclass_fields__ if k != "fields"}
    return json.dumps(d)


def driver_cases() -> dict:
    """Runs of the reference's own driver (simulate(), data.dat and *.p0.bin)."""
    base = dict(Nx=(8, 10, 6), L=(4.0, 5.0, 3.5), a_smear=0.2, rho0=5.0, kappa=50.0, lam_pl=0.005,
                lam_mi=0.005, L_nr=0.6, R_nr=1.2, xi_nr=0.3, Nda=3, Ndb=5, chi_ab=0.5, n_exp_nr=1,
                centers=((0.4, 0.55, 0.5), (0.5, 0.5, 0.5)), orients=((0.9, 0.3, 0.1), (1.0, 0.0, 0.0)),
                itermax=12, print_freq=3)
    cases = {}
    c = Case(**base)
    c.fields = seeded_fields(c, 1, 0.3, 0.01, False)
    cases["driver_res"] = c
    c = Case(ic=((-2, 1.0, 0, 1.0), (-4, 1.0, 1, 1.0)), **base)
    c.fields = {}
    cases["driver_cos"] = c
    # explicit Euler update (update_scheme 0, code/Euler_update.cpp), both chi signs
    c = Case(update_scheme=0, **base)
    c.fields = seeded_fields(c, 2, 0.3, 0.01, False)
    cases["driver_euler"] = c
    c = Case(update_scheme=0, **dict(base, chi_ab=-0.5))
    c.fields = seeded_fields(c, 3, 0.3, 0.01, False)
    cases["driver_euler_negab"] = c
    # complex Langevin (do_CL = 1, the harness seeds ran2 with idum = -12345),
    # averages sampled every 2 iterations from iteration 4
    cl = dict(do_CL=1, sample_freq=2, sample_wait=4)
    c = Case(**cl, **base)
    c.fields = seeded_fields(c, 4, 0.3, 0.01, False)
    cases["driver_cl"] = c
    c = Case(**cl, **dict(base, chi_ab=-0.5))
    c.fields = seeded_fields(c, 5, 0.3, 0.01, False)
    cases["driver_cl_negab"] = c
    c = Case(update_scheme=0, **cl, **base)
    c.fields = seeded_fields(c, 6, 0.3, 0.01, False)
    cases["driver_cl_euler"] = c
    return cases


DRIVER_OUTPUTS = ["data.dat", "wpl.p0.bin", "wabp.p0.bin", "wabm.p0.bin", "rhoda.p0.bin", "rhodb.p0.bin",
                  "rhoda_c.p0.bin", "rhodb_c.p0.bin"]


CL_OUTPUTS = ["avg_rhoda.p0.bin", "avg_rhodb.p0.bin"]


def make_driver_fixtures(tmp):
    import shutil
    import subprocess

    from ref_case import REF_BIN, write_case

    for name, c in driver_cases().items():
        run = os.path.join(tmp, name)
        write_case(run, c)
        r = subprocess.run([REF_BIN, "simulate", "0"], cwd=run, capture_output=True, text=True, timeout=600)
        if r.returncode != 0:
            raise RuntimeError(r.stderr)
        out = os.path.join(HERE, name)
        os.makedirs(out, exist_ok=True)
        extra = CL_OUTPUTS if c.do_CL else []
        for f in ["bcp.input"] + [n + ".res" for n in c.fields] + DRIVER_OUTPUTS + extra:
            shutil.copy(os.path.join(run, f), os.path.join(out, f if f == "bcp.input" or f.endswith(".res")
                                                           else f + ".ref"))
        print(name, open(os.path.join(run, "data.dat")).read().splitlines()[-1])


# A separation sweep converged by the reference itself: two coplanar discs
# (normal along x, centres 0.5 -+ d/2 of L_z) on a 16 x 16 x 32 grid, N = 16,
# chiN = 20, C = 50, from one seeded field, SEP_ITERS update_1s() each (H
# then changes by ~1e-11 per iteration).  It checks the geometric derivative
# dH/dd against differences of H between separations the reference converged
# independently: central differences at 0.44 with h = 0.002, 0.001, 0.0005
# of L_z (H(d) carries a ripple of period 1/32 of L_z in the plate centre
# from the grid, so the difference needs a small h or Richardson
# extrapolation), and H at 0.36 .. 0.52.
SEP_D = (0.36, 0.40, 0.44, 0.48, 0.52)
SEP_FD = (0.438, 0.442, 0.439, 0.441, 0.4395, 0.4405)
SEP_ITERS = 4500


def separation_params(d, precision=0):
    sys.path.insert(0, os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300"))
    from scft.workloads import plate_params

    return plate_params(0.0, N=16, grid=(16, 16, 32), box_rg=(3.2, 3.2, 6.4), precision=precision,
                        centers=((0.5, 0.5, 0.5 - d / 2), (0.5, 0.5, 0.5 + d / 2)), thickness_rg=0.4,
                        radius_rg=1.0, xi_rg=0.2, lam_pl=0.004, lam_mi=0.001)


def separation_fields(p):
    sys.path.insert(0, os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300"))
    from scft.workloads import seeded_fields

    return seeded_fields(p, 1234)


def make_separation_fixture(tmp):
    from concurrent.futures import ThreadPoolExecutor

    from ref_case import case_from_params

    ds = list(SEP_D) + list(SEP_FD)

    def one(d):
        p = separation_params(d)
        c = case_from_params(p, separation_fields(p))
        out = run_reference(os.path.join(tmp, f"sep{d:.3f}"), c, SEP_ITERS, hist=False, timeout=6 * 3600)
        return out["trace"]

    with ThreadPoolExecutor(max_workers=min(8, len(ds))) as ex:
        traces = list(ex.map(one, ds))
    z = {"d": np.array(ds), "iters": SEP_ITERS,
         "H": np.array([t[-1, 1] for t in traces]), "Qd": np.array([t[-1, 3] for t in traces]),
         "dH_last": np.array([t[-1, 1] - t[-2, 1] for t in traces]),
         "trace_tail": np.array([t[-50:, :4] for t in traces])}
    np.savez_compressed(os.path.join(HERE, "separation_sweep_16x16x32_N16.npz"), **z)
    for d, t in zip(ds, traces):
        print(f"d={d}: H={t[-1, 1]!r} last change {t[-1, 1] - t[-2, 1]:.3e}")


def make_homopolymer_fixture(tmp, Nh=7, nK=3.5):
    """The reference's homopolymer_discrete + integrate_homopoly_discrete
    (dead in its shipped inputs) on the smeared w_A of the tiny_plate case,
    run through the oracle harness's homopoly mode."""
    import subprocess

    from ref_case import REF_BIN, load_f64, write_case

    c, _, _ = tiny_cases()["tiny_plate"]
    run = os.path.join(tmp, "homopoly")
    write_case(run, c)
    r = subprocess.run([REF_BIN, "homopoly", str(Nh), repr(nK)], cwd=run, capture_output=True, text=True,
                       timeout=600)
    if r.returncode != 0:
        raise RuntimeError(r.stderr)
    sc = {}
    for line in open(os.path.join(run, "homo.txt")):
        k, v = line.split()
        sc[k] = float(v)
    z = {"case_json": case_json(c), "Nh": Nh, "nK": nK, "W": load_f64(run, "homo_W", c),
         "rho": load_f64(run, "homo_rho", c), "Q": complex(sc["Q_re"], sc["Q_im"])}
    for k, v in c.fields.items():
        z["in_" + k] = v
    np.savez_compressed(os.path.join(HERE, "tiny_homopolymer.npz"), **z)
    print("tiny_homopolymer Q", z["Q"])


def main():
    tmp = tempfile.mkdtemp(prefix="golden_")
    if "--homopolymer" in sys.argv:
        make_homopolymer_fixture(tmp)
        return
    if "--separation" in sys.argv:
        make_separation_fixture(tmp)
        return
    if "--large" in sys.argv:
        names = [a for a in sys.argv[1:] if not a.startswith("--")]
        make_large_fixtures(tmp, names or None)
        return
    make_driver_fixtures(tmp)
    if "--driver-only" in sys.argv:
        return
    for name, (c, iters, hist) in tiny_cases().items():
        out = run_reference(os.path.join(tmp, name), c, iters, hist=hist)
        z = {"case_json": case_json(c), "trace": out["trace"], "scalars_json": json.dumps(out["scalars"])}
        for k, v in c.fields.items():
            z["in_" + k] = v
        for k in ARRAYS:
            z[k] = out[k]
        if c.sigma > 0 and c.n_exp_nr > 0:
            z["rhog_exp0"] = out["rhog_exp0"]
            z["rhog_exp"] = out["rhog_exp"]
            z["gc"] = out["gc"]
        if hist:
            z["qd0"], z["qddag0"] = out["qd0"], out["qddag0"]
        np.savez_compressed(os.path.join(HERE, name + ".npz"), **z)
        print(name, "H0", out["trace"][0, 1], "H_end", out["trace"][-1, 1])
    c = config0_case()
    out = run_reference(os.path.join(tmp, "config0"), c, 200, hist=False, timeout=3600)
    z = {"case_json": case_json(c), "trace": out["trace"], "scalars_json": json.dumps(out["scalars"]),
         "digest_idx_seed": DIGEST_IDX_SEED}
    for k in ["rhoda0", "rhodb0", "rhoda", "rhodb", "wpl", "wabp", "wabm", "smwa", "smwb"]:
        z["digest_" + k] = digest(out[k])
    np.savez_compressed(os.path.join(HERE, "config0_32cubed_N32.npz"), **z)
    print("config0 H0", out["trace"][0, 1], "H200", out["trace"][-1, 1])


if __name__ == "__main__":
    main()
