"""Time-to-residual-drop on an airfoil sweep: plain FP64 vs batched +
mixed/FP64 ladder + learned warm start (the second half of the headline
metric).  Runs entirely on the GPU through the C-ABI; prints one JSON object.

  train   n_train cases (seed 5) solved by the batched ladder; their
          converged cells train the warm-start MLP on the GPU
  test    n_test held-out cases (seed 6), each solved three ways to the same
          absolute target, 1e-10 x the first-step RMS(dU_rho) of a
          free-stream start:
            plain    one FP64 Solver per case, one after the other
            batched  one batch, mixed until 1e-5 x target level, then the
                     defect-correction iteration (FP64 residual once per chunk,
                     FP32 linearised stages) to the target, confirmed by FP64
                     steps
            learned  the same ladder started from the network's prediction
            raced    every case started twice in one batch, from the
                     prediction and from the free stream; the first twin to
                     reach the target ends the pair
          errors: max |U - U_plain| / max|U_plain| of the final states, and
          the surrogate's error before any solver step
"""
from __future__ import annotations

import json
import sys
import time

import numpy as np

from . import PREC_FP64, PREC_MIXED, sweep
from .warmstart import WarmStart, build_dataset, features, reference_levels, solve_ladder, solve_ladder_raced


def run(n_train=96, n_test=24, wall=(64, 192), radial=(32, 96), max_steps=400000, epochs=30, seed_train=5,
        seed_test=6, drop=1e-10, switch=1e-5, race=True):
    out = {"distribution": {"wall": wall, "radial": radial, "mach": [0.3, 0.85], "aoa_deg": [-2, 4],
                            "n_train": n_train, "n_test": n_test, "seeds": [seed_train, seed_test]},
           "scheme": "steady SSP-RK(4,2), local dt CFL 1.25, first-order Roe (the reference's second-order "
                     "limited scheme stalls on these meshes), slip wall + free stream"}
    # ---- training data: converged solutions of the training sweep
    train = sweep.draw_cases(n_train, seed_train, wall, radial)
    tm = [c.mesh() for c in train]
    t0 = time.perf_counter()
    lv = reference_levels(train, tm)
    states, n1, n2, t_solve, _ph = solve_ladder(tm, [sweep.case_options(c, PREC_MIXED) for c in train], lv, switch, drop,
                                              max_steps)
    X, Y = build_dataset(train, states)
    t1 = time.perf_counter()
    ws = WarmStart(width=256, depth=4, seed=1)
    losses = ws.fit(X, Y, epochs=epochs, batch=4096, lr=1e-3, seed=2)
    t_train = time.perf_counter() - t1
    out["training"] = {"cells_train": int(sum(m.ncells for m in tm)), "samples": int(X.shape[0]),
                       "solve_seconds": round(t_solve, 2), "train_seconds": round(t_train, 2),
                       "loss_first_last": [float(losses[0]), float(losses[-1])],
                       "data_seconds": round(t1 - t0, 2)}
    # ---- held-out sweep
    test = sweep.draw_cases(n_test, seed_test, wall, radial)
    meshes = [c.mesh() for c in test]
    levels = reference_levels(test, meshes)
    plain_states = []
    steps_p, t_plain, firsts = sweep.run_plain(test, PREC_FP64, max_steps, drop, ref_levels=levels, check_every=500,
                                               states=plain_states, meshes=meshes)
    st_b, b1, b2, t_batch, ph_b = solve_ladder(meshes, [sweep.case_options(c, PREC_MIXED) for c in test], levels, switch, drop,
                                            max_steps)
    starts = [ws.predict_state(c, m) for c, m in zip(test, meshes)]
    st_l, l1, l2, t_learn, ph_l = solve_ladder(meshes, [sweep.case_options(c, PREC_MIXED) for c in test], levels, switch,
                                            drop, max_steps, starts=starts)
    if race:
        st_r, r1, r2, t_race, ph_r, winner = solve_ladder_raced(
            meshes, [sweep.case_options(c, PREC_MIXED) for c in test], levels, starts, switch=switch, drop=drop,
            max_steps=max_steps)

    def err(a, b):
        return float(max(np.abs(x - y).max() / np.abs(y).max() for x, y in zip(a, b)))

    def per_case(a, b):
        return [float(np.abs(x - y).max() / np.abs(y).max()) for x, y in zip(a, b)]

    sur_inf = float(max(np.abs(s - p).max() / np.abs(p).max() for s, p in zip(starts, plain_states)))
    sur_l2 = float(np.sqrt(np.mean([((s - p) ** 2).mean() / (p ** 2).mean() for s, p in zip(starts, plain_states)])))
    fs = [sweep.free_stream_state(c, m.ncells) for c, m in zip(test, meshes)]
    fs_inf = float(max(np.abs(s - p).max() / np.abs(p).max() for s, p in zip(fs, plain_states)))
    out["test"] = {
        "cells_test": int(sum(m.ncells for m in meshes)),
        "plain_fp64": {"seconds": round(t_plain, 3), "steps_total": int(steps_p.sum())},
        "batched_ladder": {"seconds": round(t_batch, 3), "steps_mixed": int(b1.max()), "steps_after_switch": int(b2.max()),
                           "linf_vs_plain": err(st_b, plain_states),
                           "phase_seconds": {k: round(v, 3) for k, v in ph_b.items()}},
        "learned_batched_ladder": {"seconds": round(t_learn, 3), "steps_mixed": int(l1.max()), "steps_after_switch": int(l2.max()),
                                   "linf_vs_plain": err(st_l, plain_states),
                                   "phase_seconds": {k: round(v, 3) for k, v in ph_l.items()}},
        "speedup_batched_vs_plain": round(t_plain / t_batch, 2),
        "speedup_learned_vs_plain": round(t_plain / t_learn, 2),
        "steps_total": {"plain": int(steps_p.sum()), "batched": int((b1 + b2).sum()), "learned": int((l1 + l2).sum())},
        "surrogate_error": {"linf_rel": sur_inf, "l2_rel": sur_l2, "free_stream_linf_rel": fs_inf},
        "cases": [[c.nw, c.nr, round(c.mach, 4), round(c.aoa, 3)] for c in test],
        "steps_per_case_plain": steps_p.tolist(),
        "steps_per_case_learned": (l1 + l2).tolist(),
        "steps_per_case_batched": (b1 + b2).tolist(),
        "linf_per_case_batched": per_case(st_b, plain_states),
        "linf_per_case_learned": per_case(st_l, plain_states),
    }
    if race:
        out["test"]["learned_raced_ladder"] = {
            "seconds": round(t_race, 3), "steps_mixed": int(r1.max()), "steps_after_switch": int(r2.max()),
            "linf_vs_plain": err(st_r, plain_states), "phase_seconds": {k: round(v, 3) for k, v in ph_r.items()},
            "learned_start_won": [int(w == 0) for w in winner]}
        out["test"]["speedup_learned_raced_vs_plain"] = round(t_plain / t_race, 2)
    return out


def run_scaled(n_train=256, n_test=256, n_plain=16, curve=(32, 64, 128, 256), wall=(64, 512), radial=(32, 256),
               max_steps=400000, epochs=30, seed_train=5, seed_test=6, drop=1e-10, switch=1e-5):
    """The sweep at the stated scale: n_test held-out cases of the full
    distribution (W 64-512, R 32-256: ~21M cells for 256 cases) solved by the
    batched ladder from the free stream and from the learned start, the
    network trained on the converged solutions of n_train other cases, with
    a learning curve (surrogate error on the held-out cases for networks
    trained on the first m training solutions).  The plain FP64 path (one
    Solver per case, ~40 min for 256 cases) runs on the first n_plain
    held-out cases, and both batched forms are timed on that subset too."""
    out = {"distribution": {"wall": wall, "radial": radial, "mach": [0.3, 0.85], "aoa_deg": [-2, 4],
                            "n_train": n_train, "n_test": n_test, "n_plain_subset": n_plain,
                            "seeds": [seed_train, seed_test]},
           "scheme": "steady SSP-RK(4,2), local dt CFL 1.25, first-order Roe, slip wall + free stream",
           "target": f"RMS(dU_k) <= {drop:g} x first-step RMS(dU_k) of a free-stream start, k = 1..4"}
    opts = lambda cs: [sweep.case_options(c, PREC_MIXED) for c in cs]  # noqa: E731
    t_start = time.perf_counter()

    def progress(phase, **kw):
        # one line per finished phase on stderr (the result is one JSON line on stdout)
        print(json.dumps({"phase": phase, "elapsed_s": round(time.perf_counter() - t_start, 1), **kw}),
              file=sys.stderr, flush=True)

    # ---- training solutions
    train = sweep.draw_cases(n_train, seed_train, wall, radial)
    tm = [c.mesh() for c in train]
    feats_tr = [features(c, m) for c, m in zip(train, tm)]
    progress("training meshes and features")
    lv_tr = reference_levels(train, tm)
    st_tr, t1, t2, t_tr, _ = solve_ladder(tm, opts(train), lv_tr, switch, drop, max_steps)
    out["training_solve"] = {"cells": int(sum(m.ncells for m in tm)), "seconds": round(t_tr, 2),
                             "steps_total": int((t1 + t2).sum())}
    progress("training solve", **out["training_solve"])
    # ---- held-out sweep from the free stream
    test = sweep.draw_cases(n_test, seed_test, wall, radial)
    meshes = [c.mesh() for c in test]
    feats_te = [features(c, m) for c, m in zip(test, meshes)]
    levels = reference_levels(test, meshes)
    st_b, b1, b2, t_b, ph_b = solve_ladder(meshes, opts(test), levels, switch, drop, max_steps)
    progress("held-out batched ladder", seconds=round(t_b, 2), steps_total=int((b1 + b2).sum()))
    fs = [sweep.free_stream_state(c, m.ncells) for c, m in zip(test, meshes)]

    def rel_err(a, b):
        e_inf = [float(np.abs(x - y).max() / np.abs(y).max()) for x, y in zip(a, b)]
        e_l2 = [float(np.sqrt(((x - y) ** 2).mean() / (y ** 2).mean())) for x, y in zip(a, b)]
        return e_inf, e_l2

    fs_inf, fs_l2 = rel_err(fs, st_b)
    # ---- learning curve
    rows, ws = [], None
    for m in curve:
        if m > n_train:
            continue
        X, Y = build_dataset(train[:m], st_tr[:m], feats=feats_tr[:m])
        t0 = time.perf_counter()
        ws = WarmStart(width=256, depth=4, seed=1)
        losses = ws.fit(X, Y, epochs=epochs, batch=4096, lr=1e-3, seed=2)
        t_fit = time.perf_counter() - t0
        starts = [ws.predict_state(c, mm, f) for c, mm, f in zip(test, meshes, feats_te)]
        e_inf, e_l2 = rel_err(starts, st_b)
        rows.append({"train_solutions": m, "samples": int(X.shape[0]), "train_seconds": round(t_fit, 2),
                     "loss_first_last": [float(losses[0]), float(losses[-1])],
                     "surrogate_l2_median": float(np.median(e_l2)), "surrogate_linf_median": float(np.median(e_inf))})
        progress("learning curve", **rows[-1])
    out["learning_curve"] = {"rows": rows, "free_stream_l2_median": float(np.median(fs_l2)),
                             "free_stream_linf_median": float(np.median(fs_inf))}
    # ---- held-out sweep from the learned start (largest network)
    starts = [ws.predict_state(c, mm, f) for c, mm, f in zip(test, meshes, feats_te)]
    st_l, l1, l2, t_l, ph_l = solve_ladder(meshes, opts(test), levels, switch, drop, max_steps, starts=starts)
    progress("held-out learned batched ladder", seconds=round(t_l, 2), steps_total=int((l1 + l2).sum()))
    l_inf, _ = rel_err(st_l, st_b)
    steps_b, steps_l = b1 + b2, l1 + l2
    out["all_cases"] = {
        "cells": int(sum(m.ncells for m in meshes)),
        "batched_ladder": {"seconds": round(t_b, 2), "steps_total": int(steps_b.sum()),
                           "phase_seconds": {k: round(v, 2) for k, v in ph_b.items()}},
        "learned_batched_ladder": {"seconds": round(t_l, 2), "steps_total": int(steps_l.sum()),
                                   "phase_seconds": {k: round(v, 2) for k, v in ph_l.items()}},
        "learned_vs_free_stream": {"wall_time_ratio": round(t_l / t_b, 3),
                                   "steps_ratio": round(float(steps_l.sum() / steps_b.sum()), 4),
                                   "cases_with_fewer_steps": int((steps_l < steps_b).sum()),
                                   "median_case_steps_ratio": float(np.median(steps_l / steps_b))},
        "linf_learned_vs_free_stream": {"max": float(max(l_inf)), "cases_le_1e-6": int(sum(e <= 1e-6 for e in l_inf))},
    }
    # ---- plain FP64 on the subset, both batched forms on the same subset
    sub = slice(0, min(n_plain, n_test))
    plain_states = []
    steps_p, t_p, _ = sweep.run_plain(test[sub], PREC_FP64, max_steps, drop, ref_levels=levels[sub], check_every=500,
                                      states=plain_states, meshes=meshes[sub])
    sb, s1, s2, t_sb, _ = solve_ladder(meshes[sub], opts(test[sub]), levels[sub], switch, drop, max_steps)
    sl, u1, u2, t_sl, _ = solve_ladder(meshes[sub], opts(test[sub]), levels[sub], switch, drop, max_steps,
                                       starts=starts[sub])
    progress("plain subset", seconds=round(t_p, 2), batched=round(t_sb, 2), learned=round(t_sl, 2))
    b_inf, _ = rel_err(sb, plain_states)
    lp_inf, _ = rel_err(sl, plain_states)
    out["plain_subset"] = {
        "cases": len(plain_states), "cells": int(sum(m.ncells for m in meshes[sub])),
        "plain_fp64": {"seconds": round(t_p, 2), "steps_total": int(steps_p.sum())},
        "batched_ladder": {"seconds": round(t_sb, 2), "steps_total": int((s1 + s2).sum())},
        "learned_batched_ladder": {"seconds": round(t_sl, 2), "steps_total": int((u1 + u2).sum())},
        "speedup_batched": round(t_p / t_sb, 2), "speedup_learned": round(t_p / t_sl, 2),
        "linf_vs_plain_batched": {"max": float(max(b_inf)), "cases_le_1e-6": int(sum(e <= 1e-6 for e in b_inf))},
        "linf_vs_plain_learned": {"max": float(max(lp_inf)), "cases_le_1e-6": int(sum(e <= 1e-6 for e in lp_inf))},
    }
    return out


def run_airfoil(nw=512, nr=256, mach=0.8, aoa=1.25, drop=1e-10, switch=1e-5, max_steps=400000):
    """Steady transonic NACA0012 O-grid (512 x 256 nodes, 261,120 cells,
    M 0.8, 1.25 deg) to a 1e-10 drop of every RMS(dU) component: the plain
    FP64 solver against a batch of one on the precision ladder with the
    defect-correction phase.  First-order reconstruction: the reference's
    second-order Venkatakrishnan scheme stalls on this mesh."""
    from .solver import Solver
    case = sweep.Case(nw, nr, mach, aoa)
    mesh = case.mesh()
    levels = reference_levels([case], [mesh])
    out = {"workload": f"NACA0012 O-grid {nw}x{nr} nodes, {mesh.ncells} cells, M {mach}, AoA {aoa} deg, steady "
                       "SSP-RK(4,2), local dt CFL 1.25, first-order Roe, slip wall + free stream",
           "target": f"RMS(dU_k) <= {drop:g} x first-step RMS(dU_k) of the free-stream start, k = 1..4"}
    t0 = time.perf_counter()
    with Solver(mesh, sweep.case_options(case, PREC_FP64)) as s:
        s.initialize_solution()
        n_plain, _ = sweep._run_absolute(s, max_steps, drop, levels[0], 1000)
        u_plain = s.cvar
    t_plain = time.perf_counter() - t0
    st, n1, n2, t_lad, ph = solve_ladder([mesh], [sweep.case_options(case, PREC_MIXED)], levels, switch, drop, max_steps,
                                         chunk=500)
    out["plain_fp64"] = {"seconds": round(t_plain, 3), "steps": int(n_plain)}
    out["ladder_dc"] = {"seconds": round(t_lad, 3), "steps_mixed": int(n1[0]), "steps_after_switch": int(n2[0]),
                        "phase_seconds": {k: round(v, 3) for k, v in ph.items()},
                        "linf_vs_plain": float(np.abs(st[0] - u_plain).max() / np.abs(u_plain).max())}
    out["speedup"] = round(t_plain / t_lad, 2)
    return out


def run_airfoil_limited(nw=512, nr=256, mach=0.8, aoa=1.25, cfls=(1.25, 0.8), max_steps=50000, drop=1e-10,
                        chunk=1000):
    """The NACA0012 O-grid as configured: LSQ face-neighbour gradients with
    the Venkatakrishnan limiter (K = 5, src/gradient_limiter.f90:113-117),
    second-order reconstruction, steady SSP-RK(4,2) with local time steps,
    on the FP64 drop-in path.  For each CFL: steps until every RMS(dU)
    component falls to `drop` x its first-step value, the step cap, or the
    first non-finite norm; the smallest RMS(dU_rho) ratio reached by 1k,
    10k and all steps; and the wall time."""
    from .options import Options
    from .solver import FvsError, Solver
    from .meshgen import naca0012_ogrid
    mesh = naca0012_ogrid(nw, nr)
    out = {"workload": f"NACA0012 O-grid {nw}x{nr} nodes, {mesh.ncells} cells, M {mach}, AoA {aoa} deg, steady "
                       "SSP-RK(4,2), local dt, LSQ-fn + Venkatakrishnan K=5, second-order upwind, Roe, FP64",
           "target": f"RMS(dU_k) <= {drop:g} x first-step RMS(dU_k), k = 1..4", "runs": []}
    for cfl in cfls:
        opt = Options(mach_inf=mach, aoa_inf_deg=aoa, steady=True, cfl=cfl, rk_nstages=4, rk_order=2, ssprk=True,
                      grad_method=3, lsq_stencil="fn", limiter=1, reconst=2, dt=0.01, precision=PREC_FP64)
        r = {"cfl": cfl}
        t0 = time.perf_counter()
        with Solver(mesh, opt) as s:
            s.initialize_solution()
            logs, done, status = [], 0, "step cap"
            while done < max_steps:
                n = min(chunk, max_steps - done)
                try:
                    log = s.time_integration(0.0, n)
                except FvsError as e:
                    status = f"non-finite: {e}"
                    break
                logs.append(log)
                done += n
                first = logs[0][0]
                hit = np.nonzero(np.all(log <= drop * first[None, :], axis=1))[0]
                if hit.size:
                    done += int(hit[0]) + 1 - n
                    status = "target reached"
                    break
        r["seconds"] = round(time.perf_counter() - t0, 2)
        r["status"] = status
        r["steps"] = int(done)
        if logs:
            rel = np.concatenate(logs)[:, 0] / logs[0][0][0]
            r["min_rho_ratio"] = {str(k): float(rel[:k].min()) for k in (1000, 10000, len(rel)) if k <= len(rel)}
            r["last_rho_ratio"] = float(rel[-1])
        out["runs"].append(r)
    return out


def profile_batch(ncases=16, steps=400, chunk=200, fused=False):
    """A fixed amount of batched work for kernel profiling: the 16-case reduced
    sweep (261,780 cells), persistent launches of 256 threads, tiles of 1024
    and 2 blocks per SM, `steps` mixed persistent steps (fused: the fused
    first-order stage, k_persistent_cell; else separate flux and update
    phases, k_persistent), then `steps` defect-correction steps, in chunks of
    `chunk`: one cooperative launch each, steps / chunk launches per phase.
    Returns the per-phase seconds."""
    from .batch import Batch
    cases = sweep.draw_cases(ncases, 6, (64, 192), (32, 96))
    meshes = [c.mesh() for c in cases]
    never = np.zeros((ncases, 4))
    out = {"cells": int(sum(m.ncells for m in meshes)), "steps": steps, "chunk": chunk}
    with Batch(meshes, [sweep.case_options(c, PREC_MIXED) for c in cases]) as b:
        b.initialize_solution()
        b.set_mode(False, fused=fused, fixed=True)
        b.set_launch(256, 1024, 2)
        b.steps(1)
        out["launch"] = {k: v for k, v in b.info().items() if k in ("block", "tile", "blocks_per_sm", "graph", "fused")}
        b.initialize_solution()
        t0 = time.perf_counter()
        b.run_to_level(steps, never, chunk)
        t1 = time.perf_counter()
        b.run_to_level(steps, never, chunk, dc=True)
        t2 = time.perf_counter()
    out["mixed_seconds"] = round(t1 - t0, 4)
    out["dc_seconds"] = round(t2 - t1, 4)
    return out


def airfoil_shapes(nw=512, nr=256, mach=0.8, aoa=1.25, steps=200):
    """Per-step device times of the config-3 O-grid (first order, mixed
    precision): the single-mesh Solver, and a batch of one in a set of launch
    shapes (persistent or graph of tile launches, separate phases or the fused
    first-order stage, block / tile / blocks per SM), each after 20 warm-up
    steps; then the autotuned shape, and the defect-correction iteration with
    its on-line shape trials over 2,000 steps.  FP64 Solver for reference."""
    from .batch import Batch
    from .solver import FvsError, Solver
    case = sweep.Case(nw, nr, mach, aoa)
    mesh = case.mesh()
    out = {"cells": mesh.ncells, "steps": steps}
    for name, prec in (("solver_mixed", PREC_MIXED), ("solver_fp64", PREC_FP64)):
        with Solver(mesh, sweep.case_options(case, prec)) as s:
            s.initialize_solution()
            s.steps_device(100)
            out[name + "_us_per_step"] = round(1000.0 * s.steps_device(1000) / 1000, 2)
    with Batch([mesh], [sweep.case_options(case, PREC_MIXED)]) as b:
        b.initialize_solution()
        out["autotune_us_per_step"] = round(1000.0 * b.autotune(3), 2)
        out["autotuned"] = b.info()
        b.steps(20)
        _, ms = b.steps(steps)
        out["batch_autotuned_us_per_step"] = round(1000.0 * ms / steps, 2)
        shapes = []
        for tiled in (False, True):
            for fused in (False, True):
                b.set_mode(tiled=tiled, fused=fused, fixed=True)
                for blk, tile, bps in ((256, 256, 1), (256, 256, 4), (256, 1024, 2), (128, 128, 4), (128, 512, 8),
                                       (256, 4096, 4)):
                    r = {"tiled": tiled, "fused": fused, "block": blk, "tile": tile, "blocks_per_sm": bps}
                    try:
                        b.set_launch(blk, tile, bps)
                        b.steps(20)
                        _, ms = b.steps(steps)
                        r["us_per_step"] = round(1000.0 * ms / steps, 2)
                    except FvsError as e:
                        r["refused"] = str(e)[:80]
                    shapes.append(r)
        out["shapes"] = shapes
        b.set_mode(tiled=True, fused=False, fixed=False)
        b.set_launch(256, 256, 1)
        never = np.zeros((1, 4))
        _, _, _, ms = b.run_to_level(2000, never, 500, dc=True)
        out["dc_us_per_step"] = round(1000.0 * ms / 2000, 2)
    return out


def main(argv=None):
    import argparse
    ap = argparse.ArgumentParser()
    ap.add_argument("--n-train", type=int, default=96)
    ap.add_argument("--n-test", type=int, default=24)
    ap.add_argument("--epochs", type=int, default=30)
    ap.add_argument("--profile-batch", action="store_true",
                    help="a fixed 16-case batched run (400 mixed + 400 defect-correction steps) for ncu")
    ap.add_argument("--fused", action="store_true", help="--profile-batch with the fused first-order stage")
    ap.add_argument("--airfoil-shapes", action="store_true",
                    help="per-step times of the config-3 O-grid: Solver and a batch of one in its launch shapes")
    a = ap.parse_args(argv)
    if a.airfoil_shapes:
        print(json.dumps(airfoil_shapes()), flush=True)
        return
    if a.profile_batch:
        print(json.dumps(profile_batch(fused=a.fused)), flush=True)
        return
    print(json.dumps(run(a.n_train, a.n_test, epochs=a.epochs)), flush=True)


if __name__ == "__main__":
    main()
