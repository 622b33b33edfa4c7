"""Benchmark of the explicit impact step: element-steps/s on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--workload shell|quad|small|surrogate]
                    [--impl ours|reference]

Default workload: the large thin shell -- a cylinder R = 1 m, L = 4 m, t = 4 mm,
720 x 140 x 1 cells x 6 Kuhn tets = 604,800 tet10 elements, 1,213,920 nodes, aluminium
J2 (E 68.9 GPa, nu 0.33, rho 2700, sigma_y0 276 MPa, H 0.689 GPa), 5 m/s onto the
tangent plane, dt = 0.5 CFL, seeded synthetic mesh.  One "step" is one full solver
step (element internal force + J2 update, force assembly, contact, central-difference
update) over the whole mesh; the working set (~0.3 GB per step) exceeds L2, so no
flush is needed between steps.

Timing: after --preroll untimed steps (the impact under way, contact established) and
W warm-up steps, a window of K steps is timed with CUDA events on the solver's stream
and repeated back to back until at least --min-timed-s of device time is covered (the
clock sampler needs a region of that length); `value` is the median window.  At 5 m/s
the shell stays elastic (peak von Mises stress about 0.4 of yield), so the same mesh at
--plastic-speed (40 m/s, where a few per cent of the Gauss points yield) is timed the
same way and reported as `j2_active`.

Our arm prints one JSON line with value (device-resident), e2e (through the C ABI with
host buffers and the copies inside the timed region), the roofline of the dominant
kernel, the CPU baseline (the reference algorithm on one core and on all cores), the
accuracy against the FP64 run of the same formulation at both speeds, and sampled
clocks.  The reference arm (--impl reference) times the reference's CPU algorithm --
the oracle's restatement of it, bitwise identical to the compiled reference on the
golden fixtures, since the reference's compiled code cannot travel -- with all host
threads on whole-mesh steps (a sample of the elements when W + K steps would not fit
its time budget).

Under torchrun (N > 1) every rank runs its own replica (the step does not shard
across GPUs without a halo exchange; replicas only) and rank 0 reports the aggregate.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("element-steps/s on 1 GB300 vs plain GPU & host CPU; sweep runs/hr at "
          "≤2% peak-disp err")
UNIT = "element-steps/s"
MAT = dict(E=68.9e9, nu=0.33, rho=2700.0, sigma_y0=276e6, H=0.689e9)


def workload(name: str):
    from cppimpact_gb300 import meshgen as mg
    if name == "shell":
        m = mg.shell()
        setup = mg.impact_setup(m, 5.0, 0.0)
        desc = "shell R1 L4 t0.004 720x140x1 tet10 J2 5 m/s"
    elif name == "shell_half":
        m = mg.shell(n_theta=360)
        setup = mg.impact_setup(m, 5.0, 0.0)
        desc = "shell R1 L4 t0.004 360x140x1 tet10 J2 5 m/s (profiling size)"
    elif name == "quad":
        m = mg.cube(18, 2)
        setup = mg.impact_setup(m, 20.0, 1e-3)
        desc = "cube 18^3x6 tet10 J2 20 m/s"
    else:
        m = mg.cube(10, 1)
        setup = mg.impact_setup(m, 10.0, 1e-3)
        desc = "cube 10^3x6 tet4 J2 10 m/s"
    return m, setup, desc


# DRAM bytes (read + write) per step of the step kernel, from ncu captures: the task
# kernel on the full shell (profiles/k_flow_qp10_shell.md: one launch of 20 steps,
# divided by 20) and the fused kernel on the half shell (profiles/
# k_step_qp10_shell_half.md, scaled x2 for the full shell: elements and nodes double).
MEASURED_TRAFFIC = {("shell", 2): 6.97644e9 / 20, ("shell", 3): 2 * 117.996e6,
                    ("shell_half", 3): 117.996e6}


def algorithmic_bytes(npe: int, E: int, N: int):
    """Per step: 4 npe + 56 nq per element + 112 per node (X0 fp32, u/v fp64 r/w, m fp32).
    The element kernel alone: connectivity + stress state r/w + X0, u, v reads."""
    nq = 1 if npe == 4 else 4
    step = E * (4 * npe + 56 * nq) + 112 * N
    elem_kernel = E * (4 * npe + 56 * nq) + 60 * N
    return step, elem_kernel


class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled every 200 ms during a region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            p = [x.strip() for x in ln.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                mx.append(float(p[2]))
            except ValueError:
                continue
            for nm, val in zip(names, p[5:9]):
                if val.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": [], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx),
                "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup(n_gpus: int):
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if world > 1:
        import torch.distributed as dist
        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group("gloo", rank=rank, world_size=world)
    return rank, world


def barrier(world):
    if world > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, world: int) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def _ref_setup(m, setup):
    """Reference-law parameters (5-point K_e, row-sum mass, wall along the impact
    normal, include/dynamics_kernels.h:8-169) and one step's increment dt v0."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as op
    rp = op.ref_params(MAT["E"], MAT["nu"], MAT["rho"], setup["wall_offset"],
                       setup["wall_stiffness"], 1)
    dof = np.tile(np.asarray(setup["vel"], dtype=np.float64) * setup["dt"], m.num_nodes)
    return op, rp, dof


def cpu_baseline(m, setup, threads: int | None = None):
    """The reference's CPU algorithm (restated in oracle/ref_port.cpp: 5-point K_e, dense
    gemv, scatter, stress/strain output, row-sum mass assembled once, wall, gravity) over
    whole-mesh steps: all host threads (element loop split in contiguous ranges) and one
    thread (the reference itself is single-threaded)."""
    op, rp, dof = _ref_setup(m, setup)
    cores = os.cpu_count() or 1
    threads = threads or cores
    E = m.num_elements
    t_all = op.ref_time_steps(m.xloc, m.conn, rp, dof, 2, nthreads=threads, warmup=1)
    t_one = op.ref_time_steps(m.xloc, m.conn, rp, dof, 1, nthreads=1)
    return {"value": 2 * E / t_all, "unit": UNIT, "cores": cores, "cores_used": threads,
            "kind": "port",
            "sample": f"whole mesh ({E} elements), 2 steps after 1 warm-up step, reference "
                      f"force law (5-point K_e, gemv, stress/strain output), {t_all:.1f} s",
            "single_core": {"value": E / t_one, "cores_used": 1,
                            "sample": f"whole mesh, 1 step, {t_one:.1f} s"}}


def fp64_accuracy(m, setup, gpu, nsteps):
    """Error of the GPU run against the FP64 run of the same formulation (oracle/
    solver64.cpp, all host threads) on the full mesh after nsteps steps from the same
    start: relative L2 of the displacement, of the velocity change and of the plastic
    strain, the fraction of Gauss points that yielded, and whether the contact-node sets
    agree."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as op
    par = op.params(MAT["E"], MAT["nu"], MAT["rho"], MAT["sigma_y0"], MAT["H"], mode=op.J2,
                    lumping=op.LUMP_HRZ, wall_normal=setup["wall_normal"],
                    wall_offset=setup["wall_offset"], wall_stiffness=setup["wall_stiffness"])
    t0 = time.perf_counter()
    o = op.Solver(m.xloc, m.conn, par, nthreads=0)
    o.initialize(setup["vel"], setup["dt"])
    o.step(nsteps)
    ref = o.get()
    t = time.perf_counter() - t0

    def rel(a, b):
        return float(np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300))

    v0 = np.asarray(setup["vel"], dtype=np.float64)
    ever, ever_ref = (gpu["contact"] & 2) > 0, (ref["contact"] & 2) > 0
    return {"vs": "FP64 run of the same formulation (oracle, CPU)", "steps": nsteps,
            "disp_rel_l2": rel(gpu["x"] - m.xloc, ref["x"] - m.xloc),
            "dv_rel_l2": rel(gpu["v"] - v0, ref["v"] - v0),
            "epbar_rel_l2": rel(gpu["epbar"], ref["epbar"]) if ref["epbar"].max() > 0 else None,
            "epbar_max": float(ref["epbar"].max()),
            "yielded_qp_frac": float((ref["epbar"] > 0).mean()),
            "contact_nodes": int(ever_ref.sum()),
            "contact_sets_equal": bool(np.array_equal(ever, ever_ref)),
            "contact_nodes_differing": int((ever != ever_ref).sum()),
            "fp64_seconds": round(t, 1)}


def make_solver(m, setup, args):
    from cppimpact_gb300 import api
    s = api.Solver(m.xloc, m.conn, **MAT, mode=api.MODE_J2, lumping=api.LUMP_HRZ,
                   step_kernel=args.step_kernel, chunk_elements=args.chunk_elements,
                   chunk_nodes=args.chunk_nodes, block_threads=args.block_threads,
                   elem_lanes=args.elem_lanes,
                   wall_normal=setup["wall_normal"], wall_offset=setup["wall_offset"],
                   wall_stiffness=setup["wall_stiffness"],
                   device=int(os.environ.get("LOCAL_RANK", "0")))
    s.initialize(setup["vel"])
    s.start(setup["dt"])
    return s


def timed_window(s, args, world, min_ms):
    """Device time of K steps (CUDA events on the solver's stream, one ci_step call:
    K step launches and the end-of-call completion), repeated back to back with a
    barrier around each repetition until at least min_ms of device time is covered (so
    the sampled clocks see the region); max over ranks, median over repetitions."""
    first = s.time_steps(args.steps)
    reps = [first]
    n = max(3, int(np.ceil(min_ms / max(max_over_ranks(first, world), 1e-6))))
    for _ in range(n - 1):
        barrier(world)
        reps.append(s.time_steps(args.steps))
        barrier(world)
    med = max_over_ranks(statistics.median(reps), world)
    return med, reps


def yield_fraction(s):
    ep = s.state(("epbar",))["epbar"]
    return float((ep > 0).mean()), float(ep.max())


def run_ours(args, rank, world):
    m, setup, desc = workload(args.workload)
    N, E, npe = m.num_nodes, m.num_elements, m.npe
    s = make_solver(m, setup, args)
    # untimed: into the impact (contact established), then the warm-up steps
    s.step(args.preroll)
    s.step(max(args.warmup, 3))
    start_step = s.steps_done()
    yf0, _ = yield_fraction(s)
    barrier(world)
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        ms, reps = timed_window(s, args, world, 1e3 * args.min_timed_s)
    barrier(world)
    end_step = s.steps_done()
    yf1, ep1 = yield_fraction(s)
    ms_step = ms / args.steps
    value = world * E * args.steps / (ms / 1e3)
    # per-kernel device durations (separate pass, per-launch events)
    k_elem_ms, k_node_ms = s.time_kernels(min(args.steps, 200))
    step_bytes, elem_bytes = algorithmic_bytes(npe, E, N)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        pass
    peak = peaks.get("hbm_gbs", 6800.0)
    peak_src = "measured" if "hbm_gbs" in peaks else "fallback"
    sk = s.step_kernel()  # the kernel the solver runs (0 = automatic resolved)
    fused = sk != 1
    kbytes = step_bytes if fused else elem_bytes
    achieved = kbytes / (k_elem_ms * 1e-3) / 1e9
    kname = {0: "k_step (fused element force + J2 + assembly + node update)",
             1: "k_elem (element force + J2 + colour assembly)",
             2: "k_flow_qp10 (persistent task kernel: node and element tasks of every step)"}
    kname[3] = kname[0]
    roofline = {"bound": "hbm", "kernel": kname[sk],
                "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": peak_src,
                "traffic": (args.traffic if args.traffic is not None
                            else MEASURED_TRAFFIC.get((args.workload, sk))),
                "kernel_ms": round(k_elem_ms, 4),
                "other_kernel_ms_per_step": round(k_node_ms, 4),
                "bytes_formula": "E(4 npe + 56 nq) + 112 N" if fused else "E(4 npe + 56 nq) + 60 N"}
    step_roof = {"achieved": round(step_bytes / (ms_step * 1e-3) / 1e9, 1),
                 "frac": round(step_bytes / (ms_step * 1e-3) / 1e9 / peak, 4),
                 "bytes_per_elem_step": round(step_bytes / E, 1)}
    # end to end through the C ABI with host buffers: per call, upload the state,
    # advance S steps, read the state back (an export interval of the reference driver);
    # the state lives in pinned host buffers between calls
    S = args.e2e_interval
    try:
        import torch
        xh = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
        vh = torch.empty((N, 3), dtype=torch.float64, pin_memory=True).numpy()
    except (ImportError, RuntimeError):
        xh, vh = np.empty((N, 3)), np.empty((N, 3))
    s.get_xv(xh, vh)
    calls = max(1, int(np.ceil(args.min_timed_s / (S * ms_step * 1e-3))))
    barrier(world)
    t0 = time.perf_counter()
    for _ in range(calls):
        s.set_state(xh, vh)
        s.step(S)
        s.get_xv(xh, vh)
    t1 = time.perf_counter()
    barrier(world)
    e2e_s = max_over_ranks(t1 - t0, world)
    e2e = {"value": world * E * S * calls / e2e_s, "unit": UNIT,
           "h2d_bytes_per_step": 48 * N / S, "d2h_bytes_per_step": 48 * N / S,
           "steps_per_call": S, "calls": calls,
           "api": "per call: ci_set_state(x, v) + ci_step(S) + ci_get_state(x, v), pinned host buffers"}
    en = s.energy()
    # fused path: one step kernel per step + the end-of-call completion per window; task
    # kernel: one launch per window
    launches = (1 if sk == 2 else s.launches_per_step() * args.steps + 1) * len(reps)
    s.close()
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "state_dtype": "f64",
        "data": "synthetic (seeded mesh, seed 20261203)",
        "config": {"workload": desc, "elements": E, "nodes": N, "nodes_per_element": npe,
                   "dt": setup["dt"], "l2": "working set > L2 (no flush)",
                   "parallelism": f"replicas x{world}" if world > 1 else "single GPU"},
        "timing": {"repeats": len(reps), "statistic": "median over repeats of K-step windows",
                   "ms_per_step_min": min(reps) / args.steps,
                   "ms_per_step_max": max(reps) / args.steps,
                   "window_steps": [start_step, end_step],
                   "preroll_steps": args.preroll,
                   "yielded_qp_frac": [yf0, yf1], "epbar_max_end": ep1},
        "roofline": roofline, "step_roofline": step_roof, "e2e": e2e,
        "gpu_launches": launches,
        "clocks": clk.summary(),
        "energy_balance_rel": abs(en["balance"]) / max(en["kinetic0"], 1e-300),
    }
    if args.plastic_speed > 0 and args.workload in ("shell", "shell_half"):
        line["j2_active"] = run_plastic_window(args, world, m, peak, step_bytes)
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(m, setup)
    if rank == 0 and args.fp64_check_steps > 0:
        line["accuracy"] = accuracy_leg(args, m, setup, args.fp64_check_steps)
        if args.plastic_speed > 0 and args.fp64_check_plastic_steps > 0 and \
                args.workload in ("shell", "shell_half"):
            from cppimpact_gb300 import meshgen as mg
            ps = mg.impact_setup(m, args.plastic_speed, 0.0)
            line["accuracy_j2_active"] = accuracy_leg(args, m, ps, args.fp64_check_plastic_steps)
    if rank == 0 and args.sweep:
        line["sweep"] = run_sweep(args)
    if rank == 0 and args.sweep and args.surrogate and args.workload == "shell":
        line["surrogate"] = surrogate_summary()
    return line


def run_plastic_window(args, world, m, peak, step_bytes):
    """The same mesh hitting the plane at --plastic-speed, where the J2 return branch is
    taken (at the shell's own 5 m/s the peak von Mises stress stays near 0.4 of yield):
    timed like the headline after --plastic-preroll steps, with the yielded fraction of
    Gauss points at the start and end of the window."""
    from cppimpact_gb300 import meshgen as mg
    setup = mg.impact_setup(m, args.plastic_speed, 0.0)
    s = make_solver(m, setup, args)
    s.step(args.plastic_preroll)
    s.step(max(args.warmup, 3))
    start_step = s.steps_done()
    yf0, _ = yield_fraction(s)
    ms, reps = timed_window(s, args, world, 500.0)
    yf1, ep1 = yield_fraction(s)
    end_step = s.steps_done()
    k_ms, _ = s.time_kernels(min(args.steps, 200))
    s.close()
    ms_step = ms / args.steps
    return {"workload": f"{m.num_elements} tet10 shell, J2, {args.plastic_speed:g} m/s onto the "
                        "tangent plane",
            "value": world * m.num_elements * args.steps / (ms / 1e3), "unit": UNIT,
            "ms_per_step": ms_step, "repeats": len(reps), "window_steps": [start_step, end_step],
            "yielded_qp_frac": [yf0, yf1], "epbar_max_end": ep1,
            "kernel_ms": round(k_ms, 4),
            "roofline_frac": round(step_bytes / (k_ms * 1e-3) / 1e9 / peak, 4)}


def accuracy_leg(args, m, setup, nsteps):
    g = make_solver(m, setup, args)
    g.step(nsteps)
    st = g.state(("x", "v", "epbar", "contact"))
    g.close()
    out = fp64_accuracy(m, setup, st, nsteps)
    out["speed"] = float(np.linalg.norm(setup["vel"]))
    return out


def surrogate_summary():
    """The learned-surrogate sweep of `--workload surrogate` in brief: runs per hour of
    the surrogate with audit and fallback against the plain and the batched GPU solver
    on the same 512 held-out parameter sets, its errors against the solver, and its
    one-off cost."""
    from cppimpact_gb300 import surrogate as sg
    cfg = sg.Config()
    r = sg.study(cfg)
    rph, err = r["runs_per_hour"], r["errors"]["final_peak_disp"]
    return {"workload": f"cube {cfg.n_cube}^3x6 tet4, {cfg.n_train} training runs, "
                        f"{cfg.n_test} held-out parameter sets, {cfg.steps} steps",
            "runs_per_hour": rph["surrogate"], "vs_plain_gpu": r["speedup_vs_plain_gpu"],
            "vs_batched_gpu": rph["surrogate"] / rph["batched_solver"],
            "plain_gpu_runs_per_hour": rph["plain_gpu_solver"],
            "batched_gpu_runs_per_hour": rph["batched_solver"],
            "peak_disp_err": {"p95": err["p95"], "max": err["max"],
                              "within_2pct": 1.0 - err["frac_over_2pct"]},
            "reruns": r["audit"]["rerun"], "audit": r["audit"], "fit_s": r["fit"]["wall_s"],
            "one_off_s": r["one_off_s"], "amortised": r["amortised"],
            "break_even_queries": rph["break_even_queries"],
            "idw_peak_disp_err": {"p95": r["errors"]["idw_peak_disp"]["p95"],
                                  "within_2pct": 1.0 - r["errors"]["idw_peak_disp"]["frac_over_2pct"]},
            "gemm_tflops": r["gemm"]["square"]["tflops"]}


def cpu_sweep_baseline(inst, nsteps, seconds_budget: float = 6.0, sample: int = 4):
    """The reference's CPU algorithm (the oracle's restatement: RefCompat elastic law,
    z-axis wall, so tilt 0) on the sweep's tet4 instances, one thread: a bounded number
    of steps per instance, extrapolated to its full step count; runs/hour on one core
    and on all host cores (independent processes)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle_py as op
    tet4 = [d for d in inst if d["conn"].shape[1] == 4][:sample]
    if not tet4:
        return None
    run_s = []
    for d in tet4:
        # the same cube and speed with the wall untilted (normal +z, 1 mm below)
        rp = op.ref_params(d["E"], d["nu"], d["rho"], float(d["xloc"][:, 2].min()) - 1e-3,
                           d["wall_stiffness"], 1)
        full = nsteps(d)
        k = 8
        while True:
            t0 = time.perf_counter()
            op.ref_solve(d["xloc"], d["conn"], rp, d["vel"], d["dt"], (k - 1) * d["dt"] + 0.5 * d["dt"],
                         nthreads=1)
            t = time.perf_counter() - t0
            if t > seconds_budget / sample / 4 or k >= full:
                break
            k = min(full, k * 4)
        run_s.append(t * full / k)
    per_run = float(np.mean(run_s))
    cores = os.cpu_count() or 1
    return {"per_core": 3600.0 / per_run, "cores": cores, "all_cores": cores * 3600.0 / per_run,
            "sample": f"{len(tet4)} tet4 instances, tilt 0, RefCompat law, bounded steps "
                      f"extrapolated to each instance's full step count, 1 thread"}


def run_sweep(args, count=256, sample=16):
    """The batched sweep: runs/hour of the batch (one launch per step per element type)
    and of the plain solver running instances one at a time (device time of a sample,
    extrapolated to the whole sweep)."""
    from cppimpact_gb300 import api, sweep
    t0 = time.perf_counter()
    inst = sweep.make_instances(count)
    t_gen = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = api.Batch(inst, autotune_steps=args.autotune)
    t_create = time.perf_counter() - t0
    tuning = {f"tet{npe}": b.tuning(npe) for npe in (4, 10)
              if any(d["conn"].shape[1] == npe for d in inst)}
    b.run()  # warm-up run
    ms = b.run()
    def nsteps(d):
        n, t = 0, 0.0
        while t <= d["t_end"]:
            n += 1
            t += d["dt"]
        return n
    el_steps = sum(d["conn"].shape[0] * nsteps(d) for d in inst)
    # the plain solver (default tile shape): same instances one at a time (sampled);
    # its end states check the tuned batch (which may differ by FP32 rounding only)
    single_ms, rel = [], []
    for i, d in enumerate(inst[:sample]):
        s = api.Solver(d["xloc"], d["conn"], E=d["E"], nu=d["nu"], rho=d["rho"],
                       sigma_y0=d["sigma_y0"], H=d["H"], wall_normal=d["wall_normal"],
                       wall_offset=d["wall_offset"], wall_stiffness=d["wall_stiffness"])
        s.initialize(d["vel"])
        s.start(d["dt"])
        single_ms.append(s.time_steps(nsteps(d)))
        up = s.state(fields=("x",))["x"] - d["xloc"]
        ub = b.state(i)["x"] - d["xloc"]
        rel.append(float(np.linalg.norm(ub - up) / max(np.linalg.norm(up), 1e-300)))
        s.close()
    b.close()
    frac = sum(d["conn"].shape[0] for d in inst[:sample]) / sum(d["conn"].shape[0] for d in inst)
    plain_ms = sum(single_ms) / max(frac, 1e-12)
    cpu = None if args.no_cpu_baseline else cpu_sweep_baseline(inst, nsteps)
    return {"instances": count, "t_end_s": 2e-3, "batch_device_ms": ms,
            "cpu_reference_runs_per_hour": cpu,
            "runs_per_hour": count / (ms / 1e3) * 3600.0,
            "plain_gpu_runs_per_hour": count / (plain_ms / 1e3) * 3600.0,
            "speedup_vs_plain_gpu": plain_ms / ms,
            "element_steps_per_s": el_steps / (ms / 1e3),
            "plain_sample": sample,
            "setup_s": {"meshes": round(t_gen, 2), "plans_and_autotune": round(t_create, 2)},
            "autotune_steps": args.autotune, "tuning": tuning,
            "end_disp_rel_l2_vs_plain_max": max(rel),
            "note": "with the same tile shape each instance is bitwise its unbatched run "
                    "(tests/test_gpu_batch.py); the tuned shape differs from the plain "
                    "solver's default only by FP32 rounding (end_disp_rel_l2_vs_plain_max)"}


def run_surrogate(args, rank, world):
    """The learned-surrogate sweep (4096 training runs of the 12^3 x 6 tet4 cube, POD rank
    64, MLP 4-256-256-5120, 512 held-out parameter sets with audit and fallback): runs per
    hour against the plain GPU solver, errors against the solver, and the tensor-core
    roofline of the largest BF16 GEMM."""
    from cppimpact_gb300 import surrogate as sg
    if rank != 0:
        return None
    cfg = sg.Config()
    with ClockSampler(0) as clk:
        r = sg.study(cfg)
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except OSError:
        peaks = {}
    peak = peaks.get("bf16_tflops", 1900.0)
    g = r["gemm"]["square"]
    rph = r["runs_per_hour"]
    return {
        "metric": "surrogate sweep runs/hr vs plain GPU solver at <=2% peak-disp err",
        "value": rph["surrogate"], "unit": "runs/h", "n_gpus": 1, "steps": cfg.steps,
        "warmup": 0, "ms_per_step": None, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "bf16 GEMM / f32 solver", "data": "synthetic (seeded parameters)",
        "config": {"workload": f"surrogate: cube {cfg.n_cube}^3x6 tet4, {cfg.n_train} training runs, "
                               f"{cfg.n_test} held-out, snapshots every {cfg.every} of {cfg.steps} steps, "
                               f"POD rank {cfg.rank}, MLP 4-{cfg.hidden}-{cfg.hidden}-{cfg.rank * cfg.snaps}"},
        "speedup_vs_plain_gpu": r["speedup_vs_plain_gpu"],
        "roofline": {"bound": "tensor", "kernel": f"k_gemm_tma (A B^T, {g['shape'][0]}^3 BF16)",
                     "achieved": round(g["tflops"], 1), "peak": peak, "unit": "TFLOP/s",
                     "frac": round(g["tflops"] / peak, 4),
                     "peak_source": "measured" if "bf16_tflops" in peaks else "fallback",
                     "traffic": None,
                     "pod_projection": {"bound": "hbm", "achieved_gbs": round(r["gemm"]["pod"]["hbm_gbs"], 1),
                                        "peak_gbs": peaks.get("hbm_gbs", 6800.0),
                                        "tflops": round(r["gemm"]["pod"]["tflops"], 1)}},
        "surrogate": r, "clocks": clk.summary(),
    }


def run_reference(args, rank, world):
    """The reference's CPU algorithm (oracle/ref_port.cpp, bitwise identical to the
    compiled reference on the golden fixtures) with all host threads on the same
    workload: each step one reference update over a sample of the mesh's elements --
    the whole mesh when W + K such steps fit the time budget (about two minutes),
    else the first elements in mesh order."""
    m, setup, desc = workload(args.workload)
    if rank != 0:
        return None
    op, rp, dof = _ref_setup(m, setup)
    cores = os.cpu_count() or 1
    E = m.num_elements
    # probe the per-element rate on a slice, then size the sample
    ne_probe = min(E, 16384)
    t = op.ref_time_steps(m.xloc, m.conn[:ne_probe], rp, dof, 1, nthreads=cores)
    rate = ne_probe / max(t, 1e-9)
    ne = int(min(E, max(1024, rate * args.reference_budget_s / (args.steps + args.warmup))))
    conn = m.conn[:ne]
    used = np.unique(conn)
    remap = np.full(m.num_nodes, -1, np.int32)
    remap[used] = np.arange(used.size, dtype=np.int32)
    x, c = m.xloc[used], remap[conn]
    t = op.ref_time_steps(x, c, rp, dof[:3 * used.size], args.steps, nthreads=cores,
                          warmup=args.warmup)
    value = ne * args.steps / t
    sample = (f"{'whole mesh' if ne == E else f'first {ne} of {E} elements'} per step (one "
              f"reference update: 5-point K_e, gemv, scatter, stress/strain output, wall; mass "
              f"assembled once), {args.steps} steps after {args.warmup} warm-up")
    return {
        "metric": METRIC, "value": value, "unit": UNIT, "impl": "reference", "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t / args.steps,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (seeded mesh, seed 20261203)",
        "config": {"workload": desc, "elements": E, "nodes": m.num_nodes,
                   "nodes_per_element": m.npe, "dt": setup["dt"]},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "cores_used": cores,
                         "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20,
                    help="K: steps per timed window (repeated until --min-timed-s)")
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--workload", default="shell",
                    choices=["shell", "shell_half", "quad", "small", "surrogate"])
    ap.add_argument("--step-kernel", type=int, default=0,
                    help="0 automatic, 1 element + node kernels, 2 persistent task kernel "
                         "(tet10), 3 fused")
    ap.add_argument("--chunk-elements", type=int, default=0)
    ap.add_argument("--chunk-nodes", type=int, default=0)
    ap.add_argument("--block-threads", type=int, default=0)
    ap.add_argument("--elem-lanes", type=int, default=0)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--preroll", type=int, default=2000,
                    help="untimed steps before the warm-up: the timed windows lie inside the "
                         "impact (contact established)")
    ap.add_argument("--min-timed-s", type=float, default=1.0,
                    help="repeat the K-step window until this much device time is covered")
    ap.add_argument("--plastic-speed", type=float, default=40.0,
                    help="shell: also time and check the same mesh at this impact speed, where "
                         "it yields (0: off)")
    ap.add_argument("--plastic-preroll", type=int, default=1000)
    ap.add_argument("--e2e-interval", type=int, default=100)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--reference-budget-s", type=float, default=120.0,
                    help="--impl reference: wall-time budget of its warm-up + timed steps")
    ap.add_argument("--fp64-check-steps", type=int, default=2000,
                    help="steps of the GPU-vs-FP64 accuracy check on the full mesh (0: off)")
    ap.add_argument("--fp64-check-plastic-steps", type=int, default=1000,
                    help="steps of the same check at --plastic-speed (0: off)")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--sweep", type=int, default=1, help="also run the 256-instance batched sweep")
    ap.add_argument("--surrogate", type=int, default=1,
                    help="shell workload with --sweep: also run the surrogate sweep and report it "
                         "in brief")
    ap.add_argument("--autotune", type=int, default=128,
                    help="sweep: trial steps per candidate tile shape (0 = default shape)")
    ap.add_argument("--traffic", type=float, default=None,
                    help="dram bytes per element-kernel launch from an ncu capture")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)
    rank, world = dist_setup(args.gpus)
    if args.workload == "surrogate":
        line = ({"impl": "reference", "unavailable": "the reference has no surrogate; the "
                 "comparison is the plain GPU solver inside our line"}
                if args.impl == "reference" else run_surrogate(args, rank, world))
    elif args.impl == "reference":
        line = run_reference(args, rank, world)
    else:
        line = run_ours(args, rank, world)
    if rank == 0 and line is not None:
        print(json.dumps(line))
    if world > 1:
        import torch.distributed as dist
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
