#!/usr/bin/env python3
"""Benchmark of the residual-and-update loop (one JSON line on rank 0).

Workload (the 1-GPU configuration of the headline metric): isentropic vortex
on the periodic box [-5,5]^2, 1024x512 quads with interior nodes jittered by a
seeded uniform +-0.2h, each quad split along a seeded random diagonal ->
1,048,576 triangles; LSQ face-neighbour gradients (p=0), no limiter,
2nd-order upwind reconstruction, Roe flux, 3-stage SSP-RK with a CFL-0.8
time step.  A "step" is one RK step (3 residual evaluations + updates) over
all cells; the metric is cell-stage updates/s = ncells * 3 * steps / time.

  value     device-resident steps, CUDA events on the library's stream
  e2e       the same steps through the C-ABI with the state in pinned host
            memory: every step uploads U, runs the step, downloads U and the
            residual norms (all inside the timed region)
  roofline  dominant kernel: algorithmic bytes per launch / mean launch time
  cpu_baseline  the CPU oracle (a restatement of the Fortran reference) on
            the host cores, on a bounded sample of the same workload
  time_to_drop  wall time to a 1e-10 residual drop: the 261,120-cell
            NACA0012 O-grid (plain FP64 solver against the batched precision
            ladder) and an 8-case held-out airfoil sweep (plain FP64 against
            batched and learned+batched); rank 0 only

--impl reference times the reference's CPU algorithm (the oracle port: the
Fortran reference cannot be built without a Fortran compiler and MPI) on all
host threads and prints the same JSON line with "impl": "reference".
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "cell-stage updates/s"
NX, NY = 1024, 512


def workload(precision: int, grad_method: int = 3):
    import math

    from fvs2d_gb300 import Options, meshgen
    mesh = meshgen.periodic_square(NX, NY, jitter=0.2, seed=1, jitter_seed=2)
    opt = Options(vortex=True, vortex_x=0.0, vortex_y=0.0, vortex_kappa=5.0,
                  vortex_inf=(1.0, 0.5 * math.sqrt(1.4), 0.0, 1.0), grad_method=grad_method, lsq_stencil="fn",
                  lsq_pow=0.0, limiter=0, reconst=2, rk_nstages=3, rk_order=3, ssprk=True, cfl=0.8, dt_from_cfl=True,
                  precision=precision)
    return mesh, opt


def config_dict(ncells, nstages, precision_name, extra=None):
    d = {"workload": f"isentropic vortex, periodic [-5,5]^2, {NX}x{NY} quads jittered +-0.2h, seeded diagonals -> "
                     f"{ncells} triangles; LSQ-fn p=0, no limiter, 2nd-order upwind, Roe, SSP-RK3, CFL 0.8",
         "ncells": ncells, "stages_per_step": nstages, "precision": precision_name,
         "l2_policy": "inputs larger than L2 (device working set > 300 MB vs 129 MB L2)",
         "parallelism": "replicas (one independent mesh per GPU)"}
    if extra:
        d.update(extra)
    return d


def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


class NvmlClocks:
    """SM clock and clock-event reasons read through NVML every few
    milliseconds on a background thread during the timed region (read only;
    nothing is set).  Raises OSError where NVML is not available."""

    # clock-event reason bits of nvml.h
    REASONS = {0x4: "sw_power_cap", 0x8: "hw_slowdown", 0x20: "sw_thermal_slowdown", 0x40: "hw_thermal_slowdown"}

    def __init__(self, index: int, period_s: float = 0.005):
        import ctypes as C
        import threading
        lib = C.CDLL("libnvidia-ml.so.1")
        if lib.nvmlInit_v2() != 0:
            raise OSError("nvmlInit failed")
        self.lib, self.C = lib, C
        self.h = C.c_void_p()
        if lib.nvmlDeviceGetHandleByIndex_v2(C.c_uint(index), C.byref(self.h)) != 0:
            raise OSError("no NVML device")
        self.get_reasons = getattr(lib, "nvmlDeviceGetCurrentClocksEventReasons", None) or \
            lib.nvmlDeviceGetCurrentClocksThrottleReasons
        mx = C.c_uint(0)
        lib.nvmlDeviceGetMaxClockInfo(self.h, C.c_int(1), C.byref(mx))  # NVML_CLOCK_SM
        self.max_mhz = float(mx.value)
        self.sm, self.reasons = [], set()
        self.period = period_s
        self.running = True
        self.t = threading.Thread(target=self._loop, daemon=True)
        self.t.start()

    def _loop(self):
        C = self.C
        clk, rs = C.c_uint(0), C.c_ulonglong(0)
        while self.running:
            if self.lib.nvmlDeviceGetClockInfo(self.h, C.c_int(1), C.byref(clk)) == 0:
                self.sm.append(float(clk.value))
            if self.get_reasons(self.h, C.byref(rs)) == 0:
                for bit, name in self.REASONS.items():
                    if rs.value & bit:
                        self.reasons.add(name)
            time.sleep(self.period)

    def stop(self) -> dict:
        # the loop samples once on entry, so a short region still has a sample
        self.running = False
        self.t.join(2.0)
        self.lib.nvmlShutdown()
        return {"sm_mhz": statistics.median(self.sm) if self.sm else None, "sm_max_mhz": self.max_mhz,
                "reasons": sorted(self.reasons), "samples": len(self.sm), "source": "NVML, every 5 ms"}


def clock_sampler(index: int):
    """NVML sampling where the library loads, else nvidia-smi."""
    try:
        return NvmlClocks(index)
    except (OSError, AttributeError):
        return Clocks(index)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index: int):
        self.path = tempfile.mktemp(suffix=".csv")
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.f = open(self.path, "w")
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except Exception:
            self.p = None

    def stop(self) -> dict:
        if self.p is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.p.terminate()
        try:
            self.p.wait(5)
        except Exception:
            self.p.kill()
        self.f.close()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            t = [x.strip() for x in line.split(",")]
            if len(t) < 9:
                continue
            try:
                sm.append(float(t[1]))
                mx.append(float(t[2]))
            except ValueError:
                continue
            for n, v in zip(names, t[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            p = json.load(f)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def traffic_from_profile(kernel: str):
    """dram bytes per launch of a kernel from the committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        t = line.split()
        if len(t) >= 3 and not line.startswith("#") and t[0] == kernel:
            try:
                return float(t[2])
            except ValueError:
                return None
    return None


def pipe_note(kernel: str):
    """The compute pipe that binds a kernel, from the committed ncu summary
    (the fifth column of profiles/ncu_traffic.txt, when present)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        t = line.split(None, 4)
        if len(t) >= 5 and not line.startswith("#") and t[0] == kernel:
            return t[4].strip()
    return None


def fp64_pipe_frac(kernel: str):
    """sm__pipe_fp64_cycles_active of a kernel as a fraction of peak, from the
    committed ncu summary (the fourth column of profiles/ncu_traffic.txt)."""
    path = os.path.join(ROOT, "profiles", "ncu_traffic.txt")
    if not os.path.exists(path):
        return None
    for line in open(path):
        t = line.split()
        if len(t) >= 4 and not line.startswith("#") and t[0] == kernel:
            try:
                return round(float(t[3]) / 100.0, 4)
            except ValueError:
                return None
    return None


def algorithmic_bytes(kernel: str, ncells: int, nedges: int, tsize: int) -> float:
    """Compulsory bytes of one launch (every array read or written once) on
    the bench's unsteady workload, where no kernel reads or writes the
    wave-speed records (only a steady scheme's first stage needs them).

    gradient (LSQ-fn, tri): per cell own primitives 4T, stencil ptr 4 +
      3 ids 12 + 3 coefficients 6T (the LSQ weights are folded into them;
      the strict build reads 3T more), gradient out 8T.
    flux: per edge ids 8 + normal 2T + area T + two offsets 4T, flux*area out
      4T; per cell primitives, gradient and limiter 13T.
    update: per cell gather list 16 + vol 8 + U 32 read + U0 32 + U 32 write
      + primitives out 4T; per edge flux slot 4T read once.  Mixed (T = 4):
      gather list 16 + 1/vol 4 + primitives out 16, and the state as the
      mixed update moves it in an SSP-RK3 step: U read at every stage, the
      FP32 increment written at stages 1-2 and read at 2-3, U written at
      stage 3, i.e. (48 + 64 + 80) / 3 = 64 B per stage."""
    T = tsize
    if kernel == "gradient":
        return ncells * (4 * T + 16 + 6 * T + 8 * T)
    if kernel == "flux":
        return nedges * (8 + 7 * T + 4 * T) + ncells * 13 * T
    if kernel == "update":
        if T == 4:
            return ncells * (16 + 4 + 64 + 4 * T) + nedges * 4 * T
        return ncells * (16 + 8 + 32 + 32 + 32 + 4 * T) + nedges * 4 * T
    return 0.0


def step_bytes(prec: int) -> int:
    """Compulsory bytes of an ideally fused LSQ-fn stage per cell (every array
    read or written once): FP64 state U, U0 read and U written 96 B; cell
    geometry (3 neighbour ids, centroid, volume); LSQ-fn coefficients (3 x 2);
    face geometry for 1.5 faces (2 cell ids, normal and length, face centre).
    FP64 geometry: 96 + 36 + 48 + 72 = 252 B; FP32 geometry (mixed
    precision): 96 + 24 + 24 + 42 = 186 B."""
    from fvs2d_gb300 import PREC_MIXED
    return 186 if prec == PREC_MIXED else 252


def run_ours(args) -> dict:
    import numpy as np

    ws, rank, local = dist_env()
    if ws > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    import torch
    import torch.distributed as tdist

    from fvs2d_gb300 import PREC_FP64, PREC_FP64_DF, PREC_FP64_STRICT, PREC_MIXED, Solver, _build
    _build.build()
    if ws > 1:
        tdist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    prec = {"fp64": PREC_FP64, "fp64_strict": PREC_FP64_STRICT, "mixed": PREC_MIXED,
            "fp64_df": PREC_FP64_DF}[args.precision]
    mesh, opt = workload(prec)
    s = Solver(mesh, opt)
    s.initialize_solution()
    nc = s.ncells
    nst = s.sizes.nstages
    nedges = s.sizes.nedges
    u_init = s.cvar

    def barrier():
        torch.cuda.synchronize()
        if ws > 1:
            tdist.barrier()

    # warm-up (also derives dt and captures the step graph)
    s.steps_device(args.warmup)
    barrier()
    clk = clock_sampler(int(os.environ.get("CUDA_VISIBLE_DEVICES", "0").split(",")[0]) if ws > 1 else 0)
    ms = s.steps_device(args.steps)
    barrier()
    clocks = clk.stop()
    t = ms / 1e3
    t = max_over_ranks(t, "cuda")
    value = whole_job_value(ws, nc * nst * args.steps, t)

    # per-kernel timing of one step (CUDA events on the library stream)
    prof = {}
    for _ in range(3):
        for name, m in s.profile_step():
            prof.setdefault(name, []).append(m)
    per_launch = {k: statistics.mean(v) for k, v in prof.items()}
    counts = {k: len(v) // 3 for k, v in prof.items()}
    total = {k: per_launch[k] * counts[k] for k in per_launch}
    dom = max(total, key=total.get)
    tsize = 4 if prec == PREC_MIXED else 8
    alg = algorithmic_bytes(dom, nc, nedges, tsize)
    peak, peak_src = measured_peaks()
    achieved = alg / (per_launch[dom] / 1e3) / 1e9
    traffic = traffic_from_profile(f"{dom}:{args.precision}")
    roofline = {"bound": "hbm", "kernel": dom, "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "peak_source": f"{peak_src} (MEASURED_PEAKS.json hbm_gbs)",
                "traffic": traffic, "alg_bytes_per_launch": alg, "mean_launch_ms": round(per_launch[dom], 4),
                "kernel_share": {k: round(v / sum(total.values()), 4) for k, v in total.items()},
                "step_bytes_model": f"{step_bytes(prec)} B per cell-stage (ideal fused LSQ-fn stage, "
                                    f"{'FP32' if prec == PREC_MIXED else 'FP64'} geometry, FP64 state)",
                "compute_bound": pipe_note(f"{dom}:{args.precision}"),
                "fp64_pipe_frac": fp64_pipe_frac(f"{dom}:{args.precision}"),
                "step_frac_of_hbm": round(value / ws * step_bytes(prec) / (peak * 1e9), 4)}

    # end to end through the C-ABI with pinned host buffers
    host_u = torch.empty((nc, 4), dtype=torch.float64, pin_memory=True)
    host_u.numpy()[:] = u_init
    norms = np.empty((1, 4))
    e2e_steps = max(3, min(args.steps, 20))
    s.set_state_ptr(host_u.data_ptr())
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        s.set_state_ptr(host_u.data_ptr())
        norms = s.time_integration(0.0, 1)
        s.get_state_ptr(host_u.data_ptr())
    barrier()
    te = time.perf_counter() - t0
    e2e = {"value": ws * nc * nst * e2e_steps / te, "unit": METRIC, "h2d_bytes_per_step": nc * 32,
           "d2h_bytes_per_step": nc * 32 + norms.nbytes, "steps": e2e_steps,
           "path": "fvs_set_state + fvs_time_integration(1 step) + fvs_get_state, pinned host memory"}

    launches = s.launches_per_step() * args.steps
    out = {"metric": METRIC, "value": value, "unit": METRIC, "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
           "ms_per_step": t * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
           "dtype": {PREC_MIXED: "f32 flux/gradient/increment, f64 state",
                     PREC_FP64_DF: "df64 (FP32 pairs) arithmetic, f64 state"}.get(prec, "f64"),
           "data": "synthetic (seeded mesh generator, analytic vortex initial state)",
           "config": config_dict(nc, nst, args.precision), "e2e": e2e, "roofline": roofline, "clocks": clocks,
           "gpu_launches": launches}

    if rank == 0 and args.variants:
        var = {}
        for name, pr, gm in (("mixed_lsq", PREC_MIXED, 3), ("fp64_df_lsq", PREC_FP64_DF, 3),
                             ("fp64_strict_lsq", PREC_FP64_STRICT, 3), ("fp64_ggcb", PREC_FP64, 1),
                             ("fp64_ggnb", PREC_FP64, 2), ("mixed_ggnb", PREC_MIXED, 2), ("fp64_df_ggnb", PREC_FP64_DF, 2)):
            m2, o2 = workload(pr, gm)
            with Solver(m2, o2) as s2:
                s2.initialize_solution()
                s2.steps_device(3)
                vms = s2.steps_device(10)
                var[name] = {"value": s2.ncells * s2.sizes.nstages * 10 / (vms / 1e3), "ms_per_step": vms / 10}
        out["variants"] = var
    if rank == 0 and not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(mesh, opt, budget_s=args.cpu_budget)
    s.close()
    if rank == 0 and args.time_to_drop:
        out["time_to_drop"] = time_to_drop()
    if ws > 1:
        tdist.destroy_process_group()
    return out if rank == 0 else None


def time_to_drop() -> dict:
    """The second half of the headline metric, wall time to a 1e-10 drop of
    every RMS(dU) component, each with its own clock record:
      airfoil  the 261,120-cell NACA0012 O-grid (M 0.8, 1.25 deg, steady
               SSP-RK(4,2), local dt at CFL 1.25): the plain FP64 solver
               against the batched precision ladder (mixed, then defect
               correction, then an FP64 check)
      sweep    8 held-out airfoil cases of the reduced sweep distribution
               (W 64-192, R 32-96, Mach 0.3-0.85, AoA -2..4 deg): plain FP64,
               one solver per case, against the batched ladder from the free
               stream and from the learned warm start (an MLP trained on the
               GPU on 16 other cases' converged solutions)"""
    from fvs2d_gb300 import sweep_bench
    out = {}
    clk = clock_sampler(0)
    out["airfoil"] = sweep_bench.run_airfoil()
    out["airfoil"]["clocks"] = clk.stop()
    clk = clock_sampler(0)
    out["sweep"] = sweep_bench.run(n_train=16, n_test=8, race=False)
    out["sweep"]["clocks"] = clk.stop()
    return out


def max_over_ranks(seconds: float, device: str) -> float:
    """The slowest rank's time (every rank gets it); the time itself when no
    process group is initialised or it has one rank."""
    import torch
    import torch.distributed as tdist
    if not (tdist.is_available() and tdist.is_initialized()) or tdist.get_world_size() == 1:
        return seconds
    tt = torch.tensor([seconds], dtype=torch.float64, device=device)
    tdist.all_reduce(tt, op=tdist.ReduceOp.MAX)
    return float(tt.item())


def whole_job_value(world_size: int, units_per_rank: float, seconds: float) -> float:
    """Whole-job throughput of independent replicas: every rank processes the
    same number of units, the job takes the slowest rank's time."""
    return world_size * units_per_rank / seconds


def host_threads() -> int:
    try:
        return len(os.sched_getaffinity(0))
    except Exception:
        return os.cpu_count() or 1


def oracle_build(orc) -> str:
    return ("built -O3 -ffast-math like the reference's -Ofast" if orc.timed
            else "built -O2 -ffp-contract=off (the -O3 -ffast-math build was unavailable)")


def cpu_baseline(mesh, opt, budget_s: float = 12.0, nthreads: int | None = None) -> dict:
    """The oracle on the host cores: a bounded number of full-mesh steps."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    nthreads = nthreads or host_threads()
    orc = Oracle(mesh, opt, nthreads=nthreads, timed=True)
    orc.initialize_solution()
    t0 = time.perf_counter()
    orc.time_integration(0.0, 1)
    t1 = time.perf_counter() - t0
    k = int(max(1, min(50, budget_s / max(t1, 1e-6))))
    t0 = time.perf_counter()
    orc.time_integration(0.0, k)
    t = time.perf_counter() - t0
    nst = orc.sizes.nstages
    return {"value": orc.ncells * nst * k / t, "unit": METRIC, "cores": nthreads, "kind": "port",
            "sample": f"{k} full SSP-RK3 steps of the {orc.ncells}-cell mesh (after 1 untimed step), "
                      f"race-free OpenMP oracle with {nthreads} threads, {oracle_build(orc)}",
            "seconds": round(t, 3)}


def run_reference(args) -> dict | None:
    ws, rank, local = dist_env()
    if rank != 0:
        return None
    from fvs2d_gb300 import PREC_FP64
    mesh, opt = workload(PREC_FP64)
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    from oracle_lib import Oracle
    nth = host_threads()
    orc = Oracle(mesh, opt, nthreads=nth, timed=True)
    orc.initialize_solution()
    for _ in range(max(1, min(args.warmup, 1))):
        orc.time_integration(0.0, 1)
    # each timed step is one full RK step of the whole mesh; bound the count
    # so the run ends within a few minutes
    t0 = time.perf_counter()
    orc.time_integration(0.0, 1)
    t1 = time.perf_counter() - t0
    k = int(max(1, min(args.steps, 60.0 / max(t1, 1e-6))))
    t0 = time.perf_counter()
    orc.time_integration(0.0, k)
    t = time.perf_counter() - t0
    nc, nst = orc.ncells, orc.sizes.nstages
    v = nc * nst * k / t
    sample = (f"{k} full SSP-RK3 steps of the {nc}-cell mesh on {nth} host threads (race-free OpenMP restatement "
              f"of the Fortran reference, {oracle_build(orc)}; the reference itself needs a Fortran compiler and MPI)")
    return {"metric": METRIC, "value": v, "unit": METRIC, "n_gpus": ws, "steps": k, "warmup": args.warmup,
            "ms_per_step": t * 1e3 / k, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic (seeded mesh generator, analytic vortex initial state)",
            "config": config_dict(nc, nst, "fp64"), "impl": "reference",
            "cpu_baseline": {"value": v, "unit": METRIC, "cores": nth, "kind": "port", "sample": sample},
            "e2e": {"value": v, "unit": METRIC, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=50)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64", choices=["fp64", "fp64_strict", "mixed", "fp64_df"])
    ap.add_argument("--no-variants", dest="variants", action="store_false")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=12.0)
    ap.add_argument("--no-time-to-drop", dest="time_to_drop", action="store_false",
                    help="skip the time-to-1e-10-drop measurements (NACA0012 O-grid and an 8-case sweep, "
                         "about 90 s)")
    ap.add_argument("--workload", default="vortex", choices=["vortex", "sweep", "sweep-256", "airfoil",
                                                             "airfoil-limited", "vortex-period"],
                    help="vortex: the 1,048,576-cell throughput case (default); sweep: time to a 1e-10 drop on an "
                         "airfoil sweep, plain FP64 vs batched ladder vs learned warm start; airfoil: time to a "
                         "1e-10 drop on the 261,120-cell NACA0012 O-grid, plain FP64 vs the ladder; airfoil-limited: "
                         "the same O-grid with the configured second-order Venkatakrishnan scheme, FP64, CFL 1.25 "
                         "and 0.8, up to 50,000 steps; sweep-256: 256 held-out full-size cases, batched ladder "
                         "from the free stream and from the learned start (network trained on 256 other cases, "
                         "learning curve), plain FP64 on a 32-case subset; vortex-period: "
                         "errors of the arithmetic modes after one vortex period at 1,048,576 cells")
    ap.add_argument("--n-train", type=int, default=96)
    ap.add_argument("--n-test", type=int, default=24)
    ap.add_argument("--full-size", action="store_true",
                    help="sweep meshes from the full distribution (64-512 wall x 32-256 radial nodes) instead of "
                         "64-192 x 32-96")
    args = ap.parse_args()
    if args.workload in ("sweep", "sweep-256", "airfoil", "airfoil-limited", "vortex-period"):
        from fvs2d_gb300 import _build, accuracy, sweep_bench
        _build.build()
        clk = clock_sampler(int(os.environ.get("LOCAL_RANK", "0")))
        if args.workload == "vortex-period":
            out = accuracy.run()
        elif args.workload == "sweep":
            sizes = dict(wall=(64, 512), radial=(32, 256), race=False) if args.full_size else {}
            out = sweep_bench.run(args.n_train, args.n_test, **sizes)
        elif args.workload == "sweep-256":
            out = sweep_bench.run_scaled()
        elif args.workload == "airfoil-limited":
            out = sweep_bench.run_airfoil_limited()
        else:
            out = sweep_bench.run_airfoil()
        out["clocks"] = clk.stop()
        print(json.dumps(out), flush=True)
        return
    if args.warmup < 3 and args.impl == "ours":
        args.warmup = 3
    out = run_reference(args) if args.impl == "reference" else run_ours(args)
    if out is not None:
        print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
