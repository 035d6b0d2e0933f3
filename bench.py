"""Benchmark of the SCFT hot path: SCFT iterations/s (update_1s steps summed
over all instances and ranks) at 64^3, N=100.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                    [--form mixed|plain] [--workload NAME]

A step is one update_1s iteration (k-space field update, smearing, both
propagator sweeps, densities) of every instance of the batch.  `value` is
timed with CUDA events on the library's own stream with the fields resident in
HBM; `e2e` is the same metric through the C ABI with host buffers: each step
is one scft_iterate_fields call on pinned host buffers, which copies every
instance's fields (w+ and the pairs of nonzero chi) from host memory, builds their densities, reads H
of those fields back, runs the field update and writes the updated fields
back into the same host buffers (the next step's input).  The working set of one step (propagator history,
fields, tables: >1 GB for the 15-instance batch) is larger than L2, so no
explicit L2 flush is done.

--impl reference times the reference's own code (compiled from its sources by
oracle/Makefile into oracle/_ref/scft_ref, FFTW API from the project's shim)
on the host cores, one process per instance.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from concurrent.futures import ThreadPoolExecutor

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "aligned-nanoplate-separation-and-rotation_gb300")
sys.path.insert(0, PKG)

METRIC = "SCFT iters/s @64^3,N=100"
# dram__bytes_read.sum + dram__bytes_write.sum of one launch of the dominant
# kernel, from an ncu capture of the same workload (the paired plane-pass step;
# profiles/mixed_kernels_sweep15_64_N100_ncu.txt).  Only valid for that workload.
NCU_TRAFFIC = {("sweep15_64_N100", "k_mix_plane64"): 125.904896e6 + 15.698944e6,
               # captured on sweep4_128x128x64_N50 (2,097,152 points of a paired step),
               # scaled by points to the 33,554,432 of one launch of this workload
               ("graft8_128x128x256_N200", "k_mix_plane128"): (67.17568e6 + 0.783104e6) * 16}
UNIT = "iters/s"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


# ---------------------------------------------------------------------------
# clocks sampled during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device_index=0):
        self.proc = None
        self.path = None
        self.dev = device_index

    def start(self):
        if not shutil.which("nvidia-smi"):
            return
        fd, self.path = tempfile.mkstemp(suffix=".csv")
        os.close(fd)
        self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.QUERY}",
                                      "--format=csv,noheader,nounits", "-lms", "50"],
                                     stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        # wait for the first sample so that the timed region is covered
        t0 = time.time()
        while time.time() - t0 < 3.0 and os.path.getsize(self.path) == 0:
            time.sleep(0.02)

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for n, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.remove(self.path)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(smax), "reasons": sorted(reasons),
                "samples": len(sm)}


# ---------------------------------------------------------------------------
# the compiled reference on the host cores
# ---------------------------------------------------------------------------
def time_reference(params, fields, iters, max_procs):
    """Runs `iters` update_1s of each instance in its own process (up to
    max_procs at once); returns (aggregate iters/s, processes, per-instance
    s/iter, per-instance Re H after the updates)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    from ref_case import REF_BIN, case_from_params, time_reference as tref

    if not os.path.exists(REF_BIN):
        raise FileNotFoundError(REF_BIN)
    tmp = tempfile.mkdtemp(prefix="scft_ref_")
    cases = [case_from_params(p, f) for p, f in zip(params, fields)]
    procs = max(1, min(max_procs, len(cases)))
    with ThreadPoolExecutor(max_workers=procs) as ex:
        res = list(ex.map(lambda kc: tref(os.path.join(tmp, f"inst{kc[0]}"), kc[1], iters, with_h=True),
                          list(enumerate(cases))))
    shutil.rmtree(tmp, ignore_errors=True)
    secs = [r[0] for r in res]
    waves = -(-len(cases) // procs)
    # instances run `procs` at a time; the batch takes `waves` rounds
    wall_per_iter = max(secs) * waves
    return len(cases) / wall_per_iter, procs, secs, [r[1] for r in res]


def mapped_repo_libraries() -> list:
    """Shared objects under the repository mapped into this process."""
    try:
        with open("/proc/self/maps") as f:
            paths = {ln.split()[-1] for ln in f if ln.rstrip().endswith(".so") or ".so." in ln}
    except OSError:
        return []
    return sorted(p for p in paths if p.startswith(ROOT))


def reference_arm(args, rank, params, fields, config):
    """--impl reference: the reference's own update_1s (oracle/_ref/scft_ref,
    compiled from its sources) on the host cores, one process per instance.
    Runs before anything loads libscft.so, so that this process maps none of
    the repository's libraries."""
    if rank != 0:
        return
    n_inst = len(params)
    cores = os.cpu_count() or 1
    iters = max(1, min(args.steps, 2))
    try:
        v, procs, secs, _ = time_reference(params, fields, iters, cores)
    except Exception as e:  # noqa: BLE001
        print(json.dumps({"impl": "reference", "unavailable": f"reference binary failed: {e}"}))
        return
    sample = (f"{n_inst} instances x {iters} update_1s each ({statistics.mean(secs):.2f} s per update per "
              f"process), one process per instance ({procs} at a time); reference code/ with Dim=3, FFTs by "
              f"the oracle shim; from the seeded fields (no relaxation)")
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": iters,
            "warmup": 0, "ms_per_step": 1e3 * n_inst / v, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "c128", "data": "synthetic seeded fields", "config": config,
            "impl": "reference",
            "steps_note": f"{iters} timed update_1s per instance (the GPU arm times --steps {args.steps})",
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": procs, "kind": "reference", "sample": sample},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "repo_libraries_mapped": mapped_repo_libraries()}
    print(json.dumps(line))


# ---------------------------------------------------------------------------
class Ranks:
    """One process per GPU, launched by torchrun (RANK, WORLD_SIZE, MASTER_*
    from the environment).  Instances are independent SCFT solves, so ranks
    exchange nothing but the barrier around the timed region and the maximum
    of their timings; with one rank both are no-ops."""

    def __init__(self, world: int, backend: str, device: str):
        self.world = world
        self.device = device
        self.dist = None
        if world > 1:
            import torch.distributed as dist

            dist.init_process_group(backend)
            self.dist = dist

    def barrier(self):
        if self.dist is not None:
            self.dist.barrier()

    def allmax(self, x: float) -> float:
        if self.dist is None:
            return x
        import torch

        t = torch.tensor([x], dtype=torch.float64, device=self.device)
        self.dist.all_reduce(t, op=self.dist.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.dist is not None:
            self.dist.destroy_process_group()
            self.dist = None


def job_rate(units_per_rank: float, world: int, seconds_max: float) -> float:
    """Whole-job rate: the units every rank processed (the same batch on each
    rank, weak scaling) over the slowest rank's time."""
    return units_per_rank * world / seconds_max


def fields_uploaded(p, form):
    """Fields scft_iterate_fields copies from the host for one instance: all
    7 in the FP64 method and with grafted chains or complex Langevin (it runs
    set_fields), w+ and the pairs of nonzero chi in the mixed form's graph."""
    if form != "mixed" or p.Ng > 0 or p.do_cl:
        return 7
    return fields_updated(p, form)


def fields_updated(p, form):
    """Fields scft_iterate_fields writes back for one instance: w+ and the
    pairs of nonzero chi in the mixed form (a pair whose chi is 0 is never
    updated), all 7 in the FP64 method."""
    if form != "mixed":
        return 7
    return 1 + 2 * sum(1 for chi in (p.chi_ab, p.chi_bc, p.chi_ac) if chi != 0.0)


def converge_to_stop_rule(ctx, n, V, tol, itmax, print_freq=25):
    """Iterates every instance of ctx until each has met the reference's stop
    rule (code/simulate.cpp:97-155: every print_freq iterations
    err = |H - H_previous| / V / print_freq, counted when below 10 tol; stop
    after iteration 25 once err < tol with more than 10 such counts), or
    until itmax.  Returns (iterations at which each instance met the rule or
    None, the last err of each instance, total iterations run)."""
    import numpy as np

    Ho = np.zeros(n)
    close = np.zeros(n, int)
    done = [None] * n
    err = np.full(n, np.inf)
    it = 0
    while it < itmax and any(d is None for d in done):
        ctx.update_1s(print_freq)
        it += print_freq
        H = ctx.calc_H()[:, 0]
        err = np.abs(H - Ho) / np.asarray(V) / print_freq
        Ho = H.copy()
        close += err < 10 * tol
        for k in range(n):
            if done[k] is None and it > 25 and err[k] < tol and close[k] > 10:
                done[k] = it
        if it % 1000 == 0:
            print(f"  iteration {it}: max err {err.max():.3e}, stopped {sum(d is not None for d in done)}/{n}",
                  file=sys.stderr, flush=True)
    return done, err, it


def converge_study(args):
    """Converged accuracy of the mixed form at 64^3, N=100: angles 0, 10, 45
    and 90 degrees, plus 10 -+ 0.5 degrees for central differences.

    1. Mixed form from the seeded start (seed 1000, the same field for every
       angle): the iteration at which each instance meets the reference's
       stop rule (error_tol --tol), then on to --tol-tight (or --itmax), so
       that the converged H is precise enough for a central difference.  Then
       10 - 0.5, 10 and 10 + 0.5 degrees start again from the converged 10
       degree fields (continuation, so that all three lie in the same basin:
       from the seeded start, nearby angles can settle into different
       lamellar states) and relax alike; the derivative is read there.
    2. FP64 method from the mixed form's converged fields to the stop rule
       (it starts next to its own saddle point).
    3. |dH| between the two converged states (absolute, per volume as the
       stop rule measures, relative); dH/dtheta at 10 degrees from each
       form's adjoint against central differences of each form's converged H.
    --converge-plate picks the plate: the reference's disc, or the cuboid with
    the A-attractive shell of the single-plate configuration as written.
    """
    import math

    import numpy as np
    import torch

    import scft
    from scft.workloads import plate_params, seeded_fields

    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    # the reference's disc, or the single-plate configuration as written (a
    # 1.6 x 1.6 x 0.2 Rg cuboid with the A-attractive shell)
    plate_kw = {"disc": {}, "cuboid_shell": {"shell": True, "shape": scft.PLATE_CUBOID}}[args.converge_plate]
    hdeg = 0.5
    thetas = [0.0, 10.0, 45.0, 90.0, 10.0 - hdeg, 10.0 + hdeg]
    n = 4
    t0 = time.time()

    def converge(prec, ths, start, tol, itmax):
        ps = [plate_params(t, precision=prec, **plate_kw) for t in ths]
        with scft.Context(ps) as ctx:
            for k in range(len(ps)):
                ctx.set_fields(k, start[k])
            ctx.calc_poly_density()
            V = [ctx.info(k)["V"] for k in range(len(ps))]
            ts = time.time()
            done, err, its = converge_to_stop_rule(ctx, len(ps), V, args.tol, itmax)
            # then on to the tighter tolerance
            while its < itmax and float(np.max(err)) > tol:
                d2, err, more = converge_to_stop_rule(ctx, len(ps), V, tol, min(2000, itmax - its))
                its += more
            r = {"H": ctx.calc_H()[:, 0].copy(), "g": ctx.grad_geom(), "done": done, "err": list(err), "its": its,
                 "V": V, "seconds": time.time() - ts, "fields": [ctx.get_fields(k) for k in range(len(ps))]}
        print(f"{len(ths)} instances: stop rule met at {done}; {its} iterations, last err {list(err)}, "
              f"{r['seconds']:.1f} s", file=sys.stderr, flush=True)
        return r

    f0 = seeded_fields(plate_params(0.0, **plate_kw), 1000)
    a = converge(scft.PREC_MIXED, thetas[:n], [f0] * n, args.tol_tight, args.itmax)
    # 10 - h, 10, 10 + h from the converged 10 degree fields, relaxed alike
    b = converge(scft.PREC_MIXED, [thetas[4], 10.0, thetas[5]], [a["fields"][1]] * 3, args.tol_tight, args.itmax)
    m = {"H": np.concatenate([a["H"], b["H"]]), "g": np.concatenate([a["g"], b["g"]]),
         "done": a["done"] + b["done"], "err": a["err"] + b["err"], "its": [a["its"], b["its"]],
         "seconds": a["seconds"] + b["seconds"]}
    d = converge(scft.PREC_FP64, thetas[:n] + [thetas[4], 10.0, thetas[5]], a["fields"] + b["fields"], args.tol,
                 args.itmax_fp64)
    dH = np.abs(m["H"][:n] - d["H"][:n])
    k10 = n + 1  # the 10 degree instance relaxed beside its neighbours
    two_h = math.radians(2 * hdeg)
    fd_m = (m["H"][n + 2] - m["H"][n]) / two_h
    fd_d = (d["H"][n + 2] - d["H"][n]) / two_h
    g_m, g_d = float(m["g"][k10, 0, 0]), float(d["g"][k10, 0, 0])
    line = {"study": "converged accuracy, mixed vs FP64", "plate": args.converge_plate, "grid": [64, 64, 64],
            "N": 100, "angles": thetas[:n],
            "stop_rule": {"error_tol": args.tol, "print_freq": 25, "reference": "code/simulate.cpp:97-155"},
            "mixed": {"from": "seeded start (seed 1000); 10 - 0.5, 10, 10 + 0.5 degrees again from the converged "
                              "10 degree fields",
                      "iterations_to_stop_rule": m["done"],
                      "iterations": m["its"], "then_to_error": args.tol_tight,
                      "last_err": [float(x) for x in m["err"]], "seconds": m["seconds"]},
            "fp64": {"from": "the mixed form's converged fields", "iterations_to_stop_rule": d["done"],
                     "iterations": d["its"], "last_err": [float(x) for x in d["err"]], "seconds": d["seconds"]},
            "H": {"angles": thetas[:n] + [thetas[4], 10.0, thetas[5]], "mixed": [float(x) for x in m["H"]],
                  "fp64": [float(x) for x in d["H"]]},
            "dH_abs": [float(x) for x in dH], "dH_per_volume": [float(x / v) for x, v in zip(dH, d["V"][:n])],
            "dH_rel": [float(x / abs(h)) for x, h in zip(dH, d["H"][:n])],
            "dHdtheta_10deg": {"mixed_adjoint": g_m, "fp64_adjoint": g_d,
                               "mixed_converged_central_difference": fd_m,
                               "fp64_converged_central_difference": fd_d, "h_deg": hdeg,
                               "mixed_adjoint_vs_fp64_fd_rel": abs(g_m - fd_d) / abs(fd_d),
                               "mixed_adjoint_vs_mixed_fd_rel": abs(g_m - fd_m) / abs(fd_m),
                               "mixed_vs_fp64_adjoint_rel": abs(g_m - g_d) / abs(g_d)},
            "seconds_total": time.time() - t0}
    print(json.dumps(line))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=100)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--form", choices=["mixed", "plain"], default=None)
    ap.add_argument("--workload", default="sweep15_64_N100")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--iterations-only", action="store_true",
                    help="warm-up + timed iterations only (for ncu launch lists)")
    ap.add_argument("--no-plain", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-autotune", action="store_true", help="keep the default launch schedule")
    ap.add_argument("--persistent", choices=["auto", "on", "off"], default="auto",
                    help="persistent sweep of 64^3 groups: autotuned (auto) or fixed")
    ap.add_argument("--plane-form", choices=["auto", "0", "1"], default="auto",
                    help="64-point plane pass: block-barrier (0) or warp-local (1) form, or autotuned")
    ap.add_argument("--sweep-groups", type=int, default=0, help="fixed number of sweep groups (0: autotune)")
    ap.add_argument("--sweep-phases", type=int, default=1, help="sequential phases with --sweep-groups")
    ap.add_argument("--plain-max", type=int, default=None,
                    help="instances in the FP64 comparison (default: all, fewer for the large workload)")
    ap.add_argument("--relax", type=int, default=None,
                    help="untimed mixed-form iterations from the seeded fields before anything is measured, so "
                         "that timing and the FP64 comparison start near the saddle point (0: seeded fields; "
                         "default 500, fewer for the large workload)")
    ap.add_argument("--converge", action="store_true",
                    help="convergence study instead of the timing: angles 0, 10, 45, 90 (and 10 +- 0.5 for the "
                         "FP64 finite difference) at 64^3, N=100, both forms from the same seeded start to the "
                         "reference's stop rule; prints one JSON line")
    ap.add_argument("--converge-plate", choices=["disc", "cuboid_shell"], default="disc",
                    help="plate of the --converge study")
    ap.add_argument("--tol", type=float, default=1e-8, help="error_tol of the stop rule (--converge)")
    ap.add_argument("--tol-tight", type=float, default=1e-11,
                    help="error the mixed form continues to after the stop rule (--converge)")
    ap.add_argument("--itmax", type=int, default=60000, help="iteration cap of the mixed form (--converge)")
    ap.add_argument("--itmax-fp64", type=int, default=3000, help="iteration cap of the FP64 method (--converge)")
    args = ap.parse_args()
    if args.converge:
        converge_study(args)
        return

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    # parameter records and constants only: nothing here loads libscft.so
    import scft
    from scft.workloads import BENCH_DEFAULTS, WORKLOADS, seeded_fields

    wd = BENCH_DEFAULTS.get(args.workload, {})
    if args.relax is None:
        args.relax = wd.get("relax", 500)
    if args.plain_max is None:
        args.plain_max = wd.get("plain_max", 0)

    form = args.form or "mixed"
    prec = scft.PREC_MIXED if form == "mixed" else scft.PREC_FP64
    params = WORKLOADS[args.workload](prec)
    fields = [seeded_fields(p, 1000 + k, periods=wd.get("periods", 1)) for k, p in enumerate(params)]
    n_inst = len(params)
    grids = sorted({"x".join(str(v) for v in p.Nx) for p in params})
    chains = sorted({p.Nda + p.Ndb for p in params})
    config = {"workload": f"{args.workload}: {n_inst} plate instance(s), grid(s) {', '.join(grids)}, "
                          f"N in {chains}, chiN=20, C=50, 1S update", "form": form, "instances_per_rank": n_inst,
              "grid": list(params[0].Nx), "N": params[0].Nda + params[0].Ndb,
              "relax_iterations": args.relax,
              "l2": "working set per step larger than L2 (no flush)"}

    if args.impl == "reference":
        reference_arm(args, rank, params, fields, config)
        return

    if form == "mixed" and not scft.mixed_available():
        raise SystemExit("libscft.so was built without the mixed form")

    import torch

    torch.cuda.set_device(local)
    ranks = Ranks(world, "nccl", "cuda")
    barrier, allmax = ranks.barrier, ranks.allmax

    if args.relax > 0 and scft.mixed_available():
        # near-saddle start: relax the seeded fields with the mixed form
        with scft.Context(WORKLOADS[args.workload](scft.PREC_MIXED)) as cr:
            for k in range(n_inst):
                cr.set_fields(k, fields[k])
            cr.calc_poly_density()
            cr.update_1s(args.relax)
            fields = [cr.get_fields(k) for k in range(n_inst)]
    ctx = scft.Context(params)
    for k in range(n_inst):
        ctx.set_fields(k, fields[k])
    ctx.calc_poly_density()
    schedule = None
    if form == "mixed":
        if args.sweep_groups > 0 or args.no_autotune or args.persistent != "auto" or args.plane_form != "auto":
            if args.sweep_groups > 0:
                ctx.set_sweep_groups(args.sweep_groups, args.sweep_phases)
            if args.persistent != "auto":
                ctx.set_persistent(args.persistent == "on")
            if args.plane_form != "auto":
                ctx.set_plane_form(int(args.plane_form))
            schedule = dict(ctx.schedule(), tuned=False)
        else:
            schedule = dict(ctx.autotune(3), tuned=True)
    if form == "mixed":
        plans = {}
        for k, p in enumerate(params):
            for d in range(3):
                plans.setdefault(str(p.Nx[d]), ctx.fft_plan(k, d))
        schedule["fft_plans"] = plans
    config["schedule"] = schedule
    stream = torch.cuda.ExternalStream(ctx.stream())
    ctx.update_1s(max(3, args.warmup))
    torch.cuda.synchronize()

    # ---- device-resident timed region
    clocks = ClockSampler(local)
    barrier()
    torch.cuda.synchronize()
    clocks.start()
    l0 = ctx.launch_count()
    e0 = torch.cuda.Event(enable_timing=True)
    e1 = torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    ctx.update_1s(args.steps)
    e1.record(stream)
    e1.synchronize()
    torch.cuda.synchronize()
    barrier()
    ck = clocks.stop()
    launches = ctx.launch_count() - l0
    ms = allmax(e0.elapsed_time(e1))
    H = ctx.calc_H()
    value = job_rate(n_inst * args.steps, world, ms / 1e3)
    if args.iterations_only:
        ctx.close()
        if rank == 0:
            print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "iterations_only": True}))
        ranks.close()
        return

    # ---- end to end through the C ABI with pinned host buffers
    import numpy as np

    M = [p.Nx[0] * p.Nx[1] * p.Nx[2] for p in params]
    host_in = []
    for k in range(n_inst):
        t = torch.zeros(7 * 2 * M[k], dtype=torch.float64, pin_memory=True)
        f = ctx.get_fields(k)
        arr = np.stack([f[n] for n in scft.FIELD_NAMES]).view(np.float64).ravel()
        t.numpy()[:] = arr
        host_in.append(t)
    host_out = torch.zeros(5 * n_inst, dtype=torch.float64, pin_memory=True)
    e2e_steps = max(1, min(args.steps, 10))
    ptrs = [t.data_ptr() for t in host_in]
    # one call per step (scft_iterate_fields, in place): upload of every
    # instance's fields from the host, their density build, H of those
    # fields read back, one update, the updated fields written back to the
    # same host buffers -- the host-held iteration continues the relaxed
    # state step by step; one untimed call first (it captures the call's
    # graph for these host buffers)
    ctx.iterate_fields_raw(ptrs, ptrs, host_out.data_ptr())
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ctx.iterate_fields_raw(ptrs, ptrs, host_out.data_ptr())
    torch.cuda.synchronize()
    t_e2e = allmax(time.perf_counter() - t0)
    # up: the fields the call reads; down: the updated fields it writes
    # back, H (5 doubles per instance) and, in the mixed form, the realness
    # check's maxima (128 doubles per instance)
    up = int(sum(fields_uploaded(p, form) * 16 * m for p, m in zip(params, M)))
    down = int(sum(fields_updated(p, form) * 16 * m for p, m in zip(params, M)))
    e2e = {"value": job_rate(n_inst * e2e_steps, world, t_e2e), "unit": UNIT,
           "call": "scft_iterate_fields",
           "h2d_bytes_per_step": up,
           "d2h_bytes_per_step": down + int(5 * 8 * n_inst + (128 * 8 * n_inst if form == "mixed" else 0))}

    # ---- the plain FP64 method on the same batch, same iteration count:
    # its rate (the metric's comparison) and the mixed form's H error
    plain = None
    if form == "mixed" and not args.no_plain:
        pp = WORKLOADS[args.workload](scft.PREC_FP64)
        n_cmp = min(n_inst, args.plain_max) if args.plain_max > 0 else n_inst
        psteps = min(args.steps, 20)  # the FP64 method is ~30x slower
        pp = pp[:n_cmp]
        # the mixed form over the same iterations as the FP64 run, for the errors
        with scft.Context(WORKLOADS[args.workload](scft.PREC_MIXED)[:n_cmp]) as cm:
            for k in range(n_cmp):
                cm.set_fields(k, fields[k])
            cm.calc_poly_density()
            cm.update_1s(max(3, args.warmup) + psteps)
            Hc = cm.calc_H()
            rho_mixed = [cm.density(k) for k in range(n_cmp)]
            try:
                g_mixed = cm.grad_geom()
            except scft.ScftError:  # grafted plates: no derivative
                g_mixed = None
        with scft.Context(pp) as c64:
            for k in range(n_cmp):
                c64.set_fields(k, fields[k])
            c64.calc_poly_density()
            c64.update_1s(max(3, args.warmup))
            s64 = torch.cuda.ExternalStream(c64.stream())
            f0 = torch.cuda.Event(enable_timing=True)
            f1 = torch.cuda.Event(enable_timing=True)
            barrier()
            f0.record(s64)
            c64.update_1s(psteps)
            f1.record(s64)
            f1.synchronize()
            ms64 = allmax(f0.elapsed_time(f1))
            H64 = c64.calc_H()
            try:
                g64 = c64.grad_geom()
            except scft.ScftError:
                g64 = None
            # the FP64 plane pass in isolation: HBM and FP64-FMA fractions
            prof64 = c64.profile_step(5)
            drho = []
            for k in range(n_cmp):
                a64, b64, _ = c64.density(k)
                a32, b32, _ = rho_mixed[k]
                drho.append(max(np.abs(a32 - a64).max() / np.abs(a64).max(),
                                np.abs(b32 - b64).max() / np.abs(b64).max()))
        dH = np.abs(Hc[:, 0] - H64[:, 0]) / np.abs(H64[:, 0])
        # dH/dtheta and dH/dc of the plate: max error over the instance's components
        # relative to its largest component
        dg = ([float(np.abs(a[0] - b[0]).max() / max(np.abs(b[0]).max(), 1e-300)) for a, b in zip(g_mixed, g64)]
              if g_mixed is not None and g64 is not None else [None] * n_cmp)
        import math

        hbm_peak, hbm_kind = peaks()
        f64_peak = scft.fp64_fma_rate(5)
        # conventional FFT count 5 E log2 E per 2-D transform of an E-point
        # plane, two transforms (inverse, forward) per plane and propagator
        flops = sum((1 if p.Nda in (0, p.Nda + p.Ndb) else 2) * p.Nx[2] * 2 * 5 * p.Nx[0] * p.Nx[1] *
                    math.log2(p.Nx[0] * p.Nx[1]) for p in pp)
        ach_b = prof64["bytes_plane"] / (prof64["ms_plane"] / 1e3) / 1e9
        ach_f = flops / (prof64["ms_plane"] / 1e3) / 1e9
        plain_roof = {"kernel": "k_prop_plane_f64", "ms_per_launch": prof64["ms_plane"],
                      "hbm": {"achieved": ach_b, "peak": hbm_peak, "unit": "GB/s", "frac": ach_b / hbm_peak,
                              "peak_kind": hbm_kind, "algorithmic_bytes_per_launch": prof64["bytes_plane"]},
                      "fp64": {"achieved": ach_f, "peak": f64_peak, "unit": "GFLOP/s", "frac": ach_f / f64_peak,
                               "peak_kind": "measured by scft_fp64_fma_rate (FMA chains over every SM)",
                               "flops_per_launch": flops}}
        plain = {"value": n_cmp * psteps * world / (ms64 / 1e3), "unit": UNIT, "ms_per_step": ms64 / psteps,
                 "roofline": plain_roof,
                 "instances": n_cmp, "steps": psteps,
                 "mixed_over_plain": (n_inst * args.steps * world / (ms / 1e3)) / (n_cmp * psteps * world /
                                                                                    (ms64 / 1e3)),
                 "dH_rel_max": float(dH.max()), "dH_rel_median": float(np.median(dH)),
                 "dH_abs_max": float(np.abs(Hc[:, 0] - H64[:, 0]).max()),
                 "dH_per_volume_max": float(max(abs(a - b) / (p.L[0] * p.L[1] * p.L[2])
                                                for a, b, p in zip(Hc[:, 0], H64[:, 0], pp))),
                 "dH_bar_reading": "relative |dH| / |H| <= 1e-6 (dH_rel_max); absolute and per volume also given",
                 "drho_rel_max": float(max(drho)),
                 "dgrad_rel_max": float(max(dg)) if dg[0] is not None else None,
                 "per_instance": [{"grid": list(p.Nx), "N": p.Nda + p.Ndb, "dH_rel": float(d), "drho_rel": float(r),
                                   "dgrad_rel": gg} for p, d, r, gg in zip(params, dH, drho, dg)],
                 "note": f"same batch, both forms from the fields after {args.relax} mixed-form iterations from "
                         f"the seeded start, then max(3, warmup) + {psteps} iterations each (the mixed form in a "
                         f"separate context); drho = max |rho32 - rho64| / max |rho64| over rho_A, rho_B"}

    # ---- dominant kernel, isolated (after the timed regions)
    hbm, peak_kind = peaks()
    sched = ctx.schedule() if form == "mixed" else {}
    sweep_roof = None
    if form == "mixed":
        sw = ctx.profile_sweep(5)
        a_sw = sw["bytes_sweep"] / (sw["ms_sweep"] / 1e3) / 1e9
        sweep_roof = {"ms_per_sweep": sw["ms_sweep"], "algorithmic_bytes_per_sweep": sw["bytes_sweep"],
                      "achieved": a_sw, "frac": a_sw / hbm,
                      "note": "whole FP32 sweep of the batch alone (no field work), current schedule"}
    prof = ctx.profile_step(20)
    nz0 = params[0].Nx[2]
    xy64 = all(p.Nx[0] == 64 and p.Nx[1] == 64 and p.Nx[2] == nz0 for p in params)
    xy128 = (not xy64 and nz0 in (64, 128, 256) and
             all(p.Nx[0] == 128 and p.Nx[1] == 128 and p.Nx[2] == nz0 for p in params))
    p64name = "k_mix_plane64w" if sched.get("plane_form") else "k_mix_plane64"

    def class_kernels(p):
        """The plane and z kernels the sweep runs for one instance."""
        X = tuple(p.Nx)
        if xy64:
            return p64name, {64: "k_mix_col64", 128: "k_mix_col128"}.get(nz0, "k_col_fft<float>")
        if xy128:
            return "k_mix_plane128", {64: "k_mix_col64", 128: "k_mix_col128", 256: "k_mix_col256"}[nz0]
        return {(64, 64, 64): (p64name, "k_mix_col64"), (96, 64, 64): ("k_mix_plane96", "k_mix_col64"),
                (48, 48, 48): ("k_mix_plane48", "k_mix_col48")}.get(X, ("k_mix_prop_plane", "k_col_fft<float>"))

    kinds = sorted(set(class_kernels(p) for p in params))
    pname = " + ".join(sorted(set(k[0] for k in kinds)))
    zname = " + ".join(sorted(set(k[1] for k in kinds)))
    kernel_names = {"mixed": (pname, zname),
                    "plain": ("k_prop_plane_f64", "k_col_fft<double> (bond kernel)")}
    dom = "plane" if prof["ms_plane"] >= prof["ms_col"] else "col"
    ms_k = prof["ms_" + dom]
    by = prof["bytes_" + dom]
    achieved = by / (ms_k / 1e3) / 1e9
    per_step = {"kernel": kernel_names[form][0 if dom == "plane" else 1], "ms_per_launch": ms_k,
                "algorithmic_bytes_per_launch": by, "achieved": achieved, "frac": achieved / hbm,
                "other_kernel": kernel_names[form][1 if dom == "plane" else 0],
                "other_kernel_ms_per_launch": prof["ms_col" if dom == "plane" else "ms_plane"]}
    if sched.get("persistent"):
        # the sweep is one launch of k_mix_sweep64 (per group): that launch is the dominant kernel
        roofline = {"bound": "hbm", "achieved": sweep_roof["achieved"], "peak": hbm, "unit": "GB/s",
                    "frac": sweep_roof["frac"], "traffic": NCU_TRAFFIC.get((args.workload, "sweep64")),
                    "kernel": "k_mix_sweep64", "peak_kind": peak_kind,
                    "ms_per_launch": sweep_roof["ms_per_sweep"] / max(1, sched.get("groups", 1)),
                    "algorithmic_bytes_per_launch": sweep_roof["algorithmic_bytes_per_sweep"] /
                    max(1, sched.get("groups", 1)),
                    "per_step_kernels_alone": per_step}
    else:
        roofline = {"bound": "hbm", "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm,
                    "traffic": NCU_TRAFFIC.get((args.workload, per_step["kernel"])),
                    "kernel": per_step["kernel"], "peak_kind": peak_kind, "ms_per_launch": ms_k,
                    "algorithmic_bytes_per_launch": by,
                    "other_kernel_ms_per_launch": per_step["other_kernel_ms_per_launch"]}
    if sweep_roof is not None:
        roofline["sweep"] = sweep_roof
    # the whole iteration against a per-iteration byte count of
    # B = M s [5 (N - 1) + 30]: five propagator-sized streams per step
    # (read and write of the working array in each of the two passes, one
    # history access) plus about 30 array passes of field work, s = 8 B
    # (FP32 propagators) or 16 B (FP64)
    s_b = 8.0 if form == "mixed" else 16.0
    b_it = sum(p.Nx[0] * p.Nx[1] * p.Nx[2] * s_b * (5 * (p.Nda + p.Ndb - 1) + 30) for p in params)
    a_it = b_it / (ms / args.steps / 1e3) / 1e9
    roofline["iteration"] = {"bytes_per_iteration": b_it, "ms_per_iteration": ms / args.steps, "achieved": a_it,
                             "frac": a_it / hbm,
                             "note": "B = M s [5(N-1) + 30] per instance and iteration (s = 8 B FP32, 16 B FP64), "
                                     "the timed iterations with field work and launch gaps"}
    ctx.close()

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        try:
            cores = os.cpu_count() or 1
            nb = min(n_inst, cores)
            v, procs, secs, h_ref = time_reference(params[:nb], fields[:nb], 1, cores)
            cpu = {"value": v, "unit": UNIT, "cores": procs, "kind": "reference",
                   "sample": f"{nb} instances x 1 update_1s, one process each; reference code/ (Dim=3, "
                             f"oracle FFT shim); {statistics.mean(secs):.2f} s/iter per process"}
            # the same update on the GPU's FP64 method from the same fields: H against the reference's
            with scft.Context(WORKLOADS[args.workload](scft.PREC_FP64)[:nb]) as c64:
                for k in range(nb):
                    c64.set_fields(k, fields[k])
                c64.calc_poly_density()
                c64.update_1s(1)
                h_gpu = c64.calc_H()[:, 0]
            cpu["H_fp64_gpu_vs_reference_rel_max"] = float(max(abs(a - b) / abs(b) for a, b in zip(h_gpu, h_ref)))
        except Exception as e:  # noqa: BLE001
            cpu = {"value": None, "unit": UNIT, "cores": 0, "kind": "reference", "sample": f"failed: {e}"}

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None,
                "dtype": "f32 propagators / f64 fields" if form == "mixed" else "c128 (complex f64)",
                "data": "synthetic seeded fields", "config": config, "e2e": e2e, "roofline": roofline,
                "cpu_baseline": cpu, "clocks": ck, "gpu_launches": launches,
                "plain_fp64": plain, "H_first_instance": float(H[0, 0])}
        print(json.dumps(line))
    ranks.close()


if __name__ == "__main__":
    main()
