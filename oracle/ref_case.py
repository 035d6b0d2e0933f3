"""Input-file writer and runner for the compiled reference.  TEST INFRASTRUCTURE.

Writes a run directory in the reference's own formats and runs the oracle
binary oracle/_ref/scft_ref (reference sources + ref_harness.cpp) in it:

* ``bcp.input``: the positional layout read by code/read_input.cpp:30-236
  (one value group per line, blank + header line between sections, exactly
  as in angle-rotation/angle-10.00/bcp.input:1-52).
* ``w*.res``: resume fields read by code/io_utils.cpp:138-240: one line per
  grid point in stack order (x fastest, code/array_utils.cpp:80-87) holding
  Dim coordinates, then the real and imaginary parts.

Only tests/, the golden-fixture script and bench.py's CPU baseline use this.
"""
from __future__ import annotations

import os
import subprocess
from dataclasses import dataclass, field

import numpy as np

ORACLE_DIR = os.path.dirname(os.path.abspath(__file__))
REF_BIN = os.path.join(ORACLE_DIR, "_ref", "scft_ref")

FIELD_NAMES = ("wpl", "wabp", "wabm", "wbcp", "wbcm", "wacp", "wacm")


@dataclass
class Case:
    """All bcp.input parameters, in the reference's b-units."""

    Nda: int = 4
    Ndb: int = 4
    phiH: float = 0.0
    Nah: int = 0
    a_smear: float = 0.2
    rho0: float = 5.0
    chi_ab: float = 0.5
    chi_bc: float = 0.0
    chi_ac: float = 0.0
    kappa: float = 50.0
    ic: tuple = ((0, 1.0, 0, 1.0), (-4, 1.0, 1, 1.0))
    Nx: tuple = (8, 8, 8)
    L: tuple = (4.0, 4.0, 4.0)
    lam_pl: float = 0.005
    lam_mi: float = 0.005
    itermax: int = 1000
    print_freq: int = 1
    sample_freq: int = 50
    sample_wait: int = 0
    error_tol: float = 1e-10
    update_scheme: int = 1
    do_CL: int = 0
    n_exp_nr: int = 0
    np_type: int = 2
    np_chem: int = 0
    sigma: float = 0.0
    Ng: int = 0
    Nu: int = 12
    L_nr: float = 1.0
    R_nr: float = 1.0
    xi_nr: float = 0.2
    centers: tuple = ((0.5, 0.5, 0.5), (0.5, 0.5, 0.5))
    orients: tuple = ((1.0, 0.0, 0.0), (1.0, 0.0, 0.0))
    fields: dict = field(default_factory=dict)  # name -> complex array (Nz,Ny,Nx)

    @property
    def M(self) -> int:
        return int(np.prod(self.Nx))

    @property
    def shape(self) -> tuple:
        """numpy shape of a grid array: x is the fastest (last) axis."""
        return (self.Nx[2], self.Nx[1], self.Nx[0])


def case_from_params(p, fields=None) -> Case:
    """Case from a library parameter record (any object with the scft_params
    field names: Nda, Ndb, a_smear, rho0, chi_*, kappa, Nx, L, lam_*, n_exp_nr,
    np_chem, sigma, Ng, L_nr, R_nr, xi_nr, center, orient)."""
    c = Case(Nda=p.Nda, Ndb=p.Ndb, a_smear=p.a_smear, rho0=p.rho0, chi_ab=p.chi_ab, chi_bc=p.chi_bc,
             chi_ac=p.chi_ac, kappa=p.kappa, Nx=tuple(p.Nx), L=tuple(p.L), lam_pl=p.lam_pl, lam_mi=p.lam_mi,
             n_exp_nr=p.n_exp_nr, np_chem=p.np_chem, sigma=p.sigma, Ng=p.Ng, L_nr=p.L_nr, R_nr=p.R_nr,
             xi_nr=p.xi_nr, centers=tuple(tuple(p.center[j]) for j in range(2)),
             orients=tuple(tuple(p.orient[j]) for j in range(2)))
    c.fields = dict(fields or {})
    return c


def _g(v: float) -> str:
    return repr(float(v))


def bcp_input_text(c: Case) -> str:
    """Renders code/read_input.cpp's positional bcp.input layout."""
    ln = []
    ln.append("# Main parameters")
    ln.append(f"{c.Nda} {c.Ndb}  Na, Nb length of each diblock's block")
    ln.append(f"{_g(c.phiH)} {c.Nah}  phiAH, Nah")
    ln.append(f"{_g(c.a_smear)}  a, smearing length")
    ln.append(f"{_g(c.rho0)}  rho0, bulk density")
    ln.append("")
    ln.append("# Interaction parameters")
    ln.append(f"{_g(c.chi_ab)}  chiAB")
    ln.append(f"{_g(c.chi_bc)}  chiBC")
    ln.append(f"{_g(c.chi_ac)}  chiAC")
    ln.append(f"{_g(c.kappa)}  kappa")
    ln.append("")
    ln.append("# Init field cond flags")
    for f, pre, d, per in c.ic:
        ln.append(f"{int(f)} {_g(pre)} {int(d)} {_g(per)}  flag, prefactor, direction, periods")
    ln.append("")
    ln.append("# Simulation parameters")
    ln.append(" ".join(str(int(n)) for n in c.Nx) + "  Nx")
    ln.append(" ".join(_g(v) for v in c.L) + "  L")
    ln.append(f"{_g(c.lam_pl)} lam_pl")
    ln.append(f"{_g(c.lam_mi)} lam_mi")
    ln.append(f"{c.itermax} itermax")
    ln.append(f"{c.print_freq} print_freq")
    ln.append(f"{c.sample_freq} {c.sample_wait}  sample_freq, sample_wait")
    ln.append(f"{c.error_tol:.6e}  error_tol")
    ln.append(f"{c.update_scheme}  Update scheme")
    ln.append(f"{c.do_CL}  do_CL")
    ln.append("")
    ln.append("# Film parameters")
    ln.append("0  do_film")
    ln.append("2.0 0.5  wall thickness, interfacial width")
    ln.append("0.5 0.5  top wall lambda_A, lambda_B")
    ln.append("0.5 0.5  bottom wall lambda_A, lambda_B")
    ln.append("")
    ln.append("# Channel wall parameters")
    ln.append("0 0 2  do_channel")
    ln.append("2.5 1.0 0.2  wall_width channel_width xi")
    ln.append("")
    ln.append("# Nanoparticle parameters")
    ln.append(f"{c.n_exp_nr}  n_exp_nr")
    ln.append("0  do_fld_np")
    ln.append(f"{c.np_type}  np_type")
    ln.append(f"{c.np_chem}  np_chem")
    ln.append(f"{_g(c.sigma)}  sigma")
    ln.append(f"{c.Ng}  Ng")
    ln.append(f"{c.Nu}  Nu")
    ln.append("0.0  np_frac")
    ln.append(f"{_g(c.L_nr)} {_g(c.R_nr)} {_g(c.xi_nr)}  L_nr, R_nr, xi_nr")
    for j in range(2):
        ln.append(" ".join(_g(v) for v in c.centers[j]) + f"  center {j + 1}")
        ln.append(" ".join(_g(v) for v in c.orients[j]) + f"  orientation {j + 1}")
    return "\n".join(ln) + "\n"


def write_res(path: str, c: Case, w: np.ndarray) -> None:
    """code/io_utils.cpp:138-177 format (Dim=3): 'x y z re im' per point."""
    w = np.asarray(w, dtype=np.complex128).reshape(c.shape)
    nz, ny, nx = c.shape
    dx = [c.L[i] / c.Nx[i] for i in range(3)]
    iz, iy, ix = np.meshgrid(np.arange(nz), np.arange(ny), np.arange(nx), indexing="ij")
    cols = np.stack(
        [ix.ravel() * dx[0], iy.ravel() * dx[1], iz.ravel() * dx[2], w.real.ravel(), w.imag.ravel()],
        axis=1,
    )
    np.savetxt(path, cols, fmt="%.17g")


def write_case(dirpath: str, c: Case) -> None:
    os.makedirs(dirpath, exist_ok=True)
    with open(os.path.join(dirpath, "bcp.input"), "w") as f:
        f.write(bcp_input_text(c))
    for name in FIELD_NAMES:
        p = os.path.join(dirpath, name + ".res")
        if name in c.fields:
            write_res(p, c, c.fields[name])
        elif os.path.exists(p):
            os.remove(p)


def load_f64(dirpath: str, name: str, c: Case, steps: int | None = None) -> np.ndarray:
    a = np.fromfile(os.path.join(dirpath, name + ".f64"), dtype=np.complex128)
    if steps is None:
        return a.reshape(c.shape)
    return a.reshape((steps,) + c.shape)


def load_scalars(dirpath: str) -> dict:
    out = {}
    with open(os.path.join(dirpath, "scalars.txt")) as f:
        for line in f:
            k, v = line.split()
            out[k] = float(v)
    return out


def load_trace(dirpath: str) -> np.ndarray:
    """Rows: iter, Re H, Im H, Re Qd, Im Qd, Re Qga, Im Qga."""
    return np.loadtxt(os.path.join(dirpath, "trace.txt"), ndmin=2)


def run_reference(dirpath: str, c: Case, iters: int, hist: bool = False, timeout: float = 600) -> dict:
    """Runs the compiled reference in `dirpath` and returns its dumps."""
    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(f"oracle binary missing: {REF_BIN} (run make -C oracle)")
    write_case(dirpath, c)
    args = [REF_BIN, "dump", str(iters)] + (["hist"] if hist else [])
    r = subprocess.run(args, cwd=dirpath, capture_output=True, text=True, timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference failed ({r.returncode}):\n{r.stdout[-2000:]}\n{r.stderr[-2000:]}")
    out = {"scalars": load_scalars(dirpath), "trace": load_trace(dirpath), "stdout": r.stdout}
    names = ["hhat", "poly_bond_fft", "gaa", "gab", "gbb", "rho_exp_nr", "exp_nrH", "expl_grafts",
             "smwa0", "smwb0", "smwg0", "rhoda0", "rhodb0", "smwa", "smwb", "rhoda", "rhodb"]
    names += list(FIELD_NAMES)
    if c.sigma > 0:
        names.append("gc")
    if c.sigma > 0 and c.n_exp_nr > 0:
        names += ["rhog_exp0", "rhog_exp"]
    for n in names:
        out[n] = load_f64(dirpath, n, c)
    if hist:
        N = c.Nda + c.Ndb
        out["qd0"] = load_f64(dirpath, "qd0", c, N)
        out["qddag0"] = load_f64(dirpath, "qddag0", c, N)
        if c.sigma > 0 and c.n_exp_nr > 0:
            out["qg0"] = load_f64(dirpath, "qg0", c, c.Ng)
            out["qgdag0"] = load_f64(dirpath, "qgdag0", c, c.Ng)
    return out


def time_reference(dirpath: str, c: Case, iters: int, timeout: float = 3600, with_h: bool = False):
    """Seconds per update_1s() iteration of the compiled reference (and, with
    with_h, Re H after the `iters` updates)."""
    write_case(dirpath, c)
    r = subprocess.run([REF_BIN, "time", str(iters)], cwd=dirpath, capture_output=True, text=True,
                       timeout=timeout)
    if r.returncode != 0:
        raise RuntimeError(f"reference timing failed: {r.stderr[-2000:]}")
    secs = H = None
    for line in r.stdout.splitlines():
        if line.startswith("seconds_per_iter"):
            secs = float(line.split()[1])
        elif line.startswith("H "):
            H = float(line.split()[1])
    if secs is None:
        raise RuntimeError("no timing line in reference output")
    return (secs, H) if with_h else secs
