"""Benchmark: cell-updates/s of the split MUSCL-Hancock + HLLE update.

Workload (one GPU): 3-D perfect gas (gamma 1.4) on a uniform 256^3 FP64 grid,
periodic, Strang splitting (6 sweeps of dt/2 per step), CFL 0.8, seeded
piecewise-constant octants with Gaussian density bumps.  One "step" is one
Strang step: the device-side stable-dt pass, the dt selection and six fused
sweeps, all captured in CUDA graphs.  A cell-update is one cell advanced by
one directional sweep (6 * 256^3 per step).

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--precision fp64_exact] [--n 256]

Under torchrun every rank runs an independent replica of the workload on its
own GPU (the update has no data-path exchange on a single-level periodic
grid); `value` is the sum of the replicas' cell-updates over the slowest
rank's time.
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
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "cell-updates/s"
UNIT = "cell-updates/s"
# the solver's device-resident control block (fvs::Control): uploaded when a
# run starts, read back every 30 steps and when it ends
CONTROL_BYTES = 176


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--precision", default="fp64_fast",
                    choices=["fp64_exact", "fp64_fast", "fp64_df", "mixed"])
    ap.add_argument("--no-variants", action="store_true",
                    help="skip timing the other precision flavours")
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--cpu-sample-n", type=int, default=None,
                    help="edge of the cube the CPU reference arm times per step (default: "
                         "--n, the GPU arm's workload)")
    ap.add_argument("--no-reports", action="store_true",
                    help="skip the secondary workloads (learned start value, 2-D Godunov, "
                         "2-D cut cells)")
    ap.add_argument("--report", choices=["sod", "learned", "godunov", "amr", "cutcell",
                                         "hllem", "sweep_variants", "cutcell_sweeps"],
                    help="run only this secondary workload and print its JSON report")
    ap.add_argument("--mlp-samples", type=int, default=10_000_000)
    ap.add_argument("--mlp-epochs", type=int, default=24)
    ap.add_argument("--godunov-n", type=int, default=2048)
    ap.add_argument("--godunov-steps", type=int, default=200)
    ap.add_argument("--godunov-tols", default="1e-7,1e-12",
                    help="Newton tolerances of the 2-D Godunov report")
    ap.add_argument("--amr-n0", type=int, default=1024)
    ap.add_argument("--amr-steps", type=int, default=50)
    ap.add_argument("--amr-flavours", default="fp64_exact,fp64_fast,mixed")
    ap.add_argument("--cutcell-n", type=int, default=1024)
    ap.add_argument("--hllem-n", type=int, default=192)
    ap.add_argument("--hllem-steps", type=int, default=10)
    ap.add_argument("--cutcell-steps", type=int, default=400)
    ap.add_argument("--launch", action="append", default=[], metavar="DIR:SEG:VARIANT",
                    help="with --profile-steps: force a direction's segment length and launch "
                         "variant (fvs_solver_set_launch), e.g. 1:32:25 for the TMA-staged y "
                         "sweep; with --report amr: LEVEL:DIR:BLOCK:GRID:THREADS_PER_ROW "
                         "(fvs_amr_set_launch)")
    ap.add_argument("--profile-steps", type=int, default=0,
                    help="profiling aid: run this many Strang steps of the --n workload in "
                         "--precision with the default launch shapes (no autotuner, no "
                         "timing) and exit; the first sweep launches are then the x, y, z "
                         "sweeps of step 1 (with --report cutcell: the cut-cell workload)")
    return ap.parse_args()


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


class ClockSampler:
    """Samples nvidia-smi clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines: list[str] = []
        self._t = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (FileNotFoundError, OSError):
            self.proc = None
            return
        self._t = threading.Thread(target=self._read, daemon=True)
        self._t.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self._t:
            self._t.join(timeout=2)
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def load_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        d["source"] = "measured"
        return d
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "source": "fallback"}


def profile_value(name: str, key: str):
    """A 'key: value' figure recorded in a profiles/ summary, or None."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.strip().startswith(key + ":"):
            try:
                return float(ln.split(":", 1)[1])
            except ValueError:
                return None
    return None


def profile_traffic(name: str, cells: int):
    """DRAM bytes per sweep launch from an ncu capture of a smaller case:
    profiles/<name> records 'traffic_bytes_per_cell_update: <B>' (mean of the
    x, y, z launches), scaled here to `cells` cells per launch."""
    p = ROOT / "profiles" / name
    if not p.exists():
        return None
    for ln in p.read_text().splitlines():
        if ln.strip().startswith("traffic_bytes_per_cell_update:"):
            try:
                return float(ln.split(":", 1)[1]) * cells
            except ValueError:
                return None
    return None


def cpu_reference_rate(n: int, steps: int, threads: int) -> dict:
    """The oracle (scalar C++17 restatement of the reference's CPU update)
    advancing the same workload on an n^3 cube: cell-updates/s."""
    from oracle import oracle as orc
    from finitevolumesolver_gb300 import workloads
    cons = workloads.octants_3d(n)
    g = orc.Grid(3, [n] * 3, [0, 0, 0], [1.0 / n] * 3)
    m = orc.method()
    t0 = time.perf_counter()
    cons, dts, _ = g.run(m, cons, 0.8, 1e9, max_steps=steps, nthreads=threads)
    el = time.perf_counter() - t0
    return {"value": 6 * n ** 3 * steps / el, "seconds": el}


def report_sod(args, torch, fvs, workloads):
    """1-D Sod shock tube, 1024 cells, transmissive, MUSCL-Hancock/VanLeer +
    HLLE, CFL 0.8, to t = 0.2: every flavour against the oracle, cell by cell."""
    from oracle import build as obuild
    obuild.build()
    from oracle import oracle as orc
    n = 1024
    cons = workloads.sod_1d(n)
    g = orc.Grid(1, [n], [1], [1.0 / n])
    ref, ref_dts, _ = g.run(orc.method(), cons, 0.8, 0.2)
    out = {"workload": "1D Sod shock tube, 1024 cells on [0, 1], transmissive, MUSCL-Hancock/"
                       "VanLeer + HLLE, CFL 0.8, t = 0.2", "oracle_steps": len(ref_dts),
           "flavours": {}}
    for prec in ("fp64_exact", "fp64_fast", "fp64_df", "mixed"):
        s = fvs.Solver([n], [1.0 / n], "transmissive", method=fvs.make_method(precision=prec))
        s.upload(cons)
        t0 = time.perf_counter()
        st, dts = s.run(cfl=0.8, t_end=0.2, log_len=4096)
        el = time.perf_counter() - t0
        res = s.download()
        # |a - b| / (|b| + max |b| of the component): relative per cell, with
        # the component's scale as the floor for values crossing zero (momentum)
        scale = np.abs(ref).reshape(ref.shape[0], -1).max(axis=1)
        scale = scale.reshape((-1,) + (1,) * (ref.ndim - 1))
        rel = np.abs(res - ref) / (np.abs(ref) + scale)
        out["flavours"][prec] = {
            "steps": st.steps, "time": st.time, "wall_s": el,
            "same_dt_sequence": bool(len(dts) == len(ref_dts) and np.array_equal(dts, ref_dts)),
            "max_rel_diff_vs_oracle": float(rel.max()),
            "l1_density_vs_oracle": float(np.abs(res[0] - ref[0]).mean()),
            "bit_identical": bool(np.array_equal(res, ref))}
        s.close()
    return out


def report_mlp(args, torch, fvs, workloads):
    """Learned Newton start value: 10^7 Riemann problems (rho, p log-uniform
    on [1e-3, 1e1], u uniform on [-3c, 3c], vacuum-generating pairs redrawn),
    labels from the exact solver at tolerance 1e-12, Adam (lr 1e-3, batch
    8192) on the tensor cores; Newton iterations per problem on 10^6
    held-out problems for the mean, PVRS/TR and learned start values."""
    n = args.mlp_samples
    arr = workloads.riemann_samples(n, seed=2025)
    dev = [torch.from_numpy(a).cuda() for a in arr]
    del arr
    ps = torch.empty(n, dtype=torch.float64, device="cuda")
    st = torch.empty(n, dtype=torch.int32, device="cuda")
    m = fvs.make_method("godunov", guess="pvrs_tr", tolerance=1e-12, max_iterations=200)
    fvs.exact_riemann_star(m, *dev, ps, None, None, st)
    feat = torch.empty(n, 5, dtype=torch.float32, device="cuda")
    lab = torch.empty(n, dtype=torch.float32, device="cuda")
    fvs.riemann_features(1.4, *dev, feat, pstar=ps, labels=lab)
    torch.cuda.synchronize()
    ok = st == 1
    feat, lab = feat[ok].contiguous(), lab[ok].contiguous()
    del dev, ps, st
    ntrain = int(lab.numel())
    net = fvs.LearnedGuess(seed=11)
    net.set_normalization(feat)
    batch = 8192
    steps_per_epoch = (ntrain + batch - 1) // batch
    net.train(feat, lab, steps=20, batch=batch, lr=1e-3, seed=1)  # warm-up, graph capture
    losses = []
    t0 = time.perf_counter()
    for e in range(args.mlp_epochs):
        losses.append(net.train(feat, lab, steps=steps_per_epoch, batch=batch, lr=1e-3,
                                seed=100 + e))
    train_s = time.perf_counter() - t0
    steps = steps_per_epoch * args.mlp_epochs
    flop_per_step = 2 * batch * (5 * 64 + 3 * 64 * 64 + 64 * 5)
    # held-out problems
    nt = 1_000_000
    test = [torch.from_numpy(a).cuda() for a in workloads.riemann_samples(nt, seed=77)]
    tf = torch.empty(nt, 5, dtype=torch.float32, device="cuda")
    fvs.riemann_features(1.4, *test, tf)
    y = torch.empty(nt, dtype=torch.float32, device="cuda")
    net.predict(tf, y)
    torch.cuda.synchronize()
    t1 = time.perf_counter()
    for _ in range(5):
        net.predict(tf, y)
    torch.cuda.synchronize()
    infer_s = (time.perf_counter() - t1) / 5
    heldout = {}
    for tol in (1e-12, 1e-7):
        iters = {}
        for guess in ("mean", "pvrs_tr", "mlp"):
            mm = fvs.make_method("godunov", guess=guess, tolerance=tol, max_iterations=200,
                                 mlp_params=net.params_device_ptr() if guess == "mlp" else None)
            p2 = torch.empty(nt, dtype=torch.float64, device="cuda")
            it = torch.empty(nt, dtype=torch.int32, device="cuda")
            s2 = torch.empty_like(it)
            fvs.exact_riemann_star(mm, *test, p2, None, it, s2)
            torch.cuda.synchronize()
            iters[guess] = {"newton_iterations_per_problem": float(it.double().mean()),
                            "fallback_rate": float((s2 == 2).double().mean()),
                            "not_converged_rate": float((s2 == 0).double().mean())}
        heldout[f"newton_tol_{tol:g}_heldout"] = iters
    # the network's relative error in p* on the held-out problems (RMS of the
    # error in y = log(p*/max(pL, pR))), the accuracy the solver's gate assumes
    ps_ref = torch.empty(nt, dtype=torch.float64, device="cuda")
    st_ref = torch.empty(nt, dtype=torch.int32, device="cuda")
    fvs.exact_riemann_star(fvs.make_method("godunov", guess="pvrs_tr", tolerance=1e-12,
                                           max_iterations=200), *test, ps_ref, None, None, st_ref)
    yl = torch.empty(nt, dtype=torch.float32, device="cuda")
    fvs.riemann_features(1.4, *test, tf, pstar=ps_ref, labels=yl)
    torch.cuda.synchronize()
    okr = st_ref == 1
    rms_y = float(torch.sqrt(((y - yl)[okr].double() ** 2).mean()))
    return {
        "workload": f"{n} sampled Riemann problems ({ntrain} with a converged label), "
                    "5-64-64-1 GELU network, BF16 tcgen05 GEMMs, FP32 accumulation",
        "training": {"epochs": args.mlp_epochs, "steps": steps, "batch": batch,
                     "seconds": train_s, "samples_per_s": steps * batch / train_s,
                     "ms_per_step": 1e3 * train_s / steps,
                     "loss_first_epoch": losses[0], "loss_last_epoch": losses[-1],
                     "tensor_tflops": flop_per_step * steps / train_s / 1e12,
                     "note": "tiny GEMMs (K = 16 / 64, N = 64): latency-bound, "
                             "not tensor-throughput-bound"},
        "inference": {"problems": nt, "problems_per_s": nt / infer_s,
                      "rms_error_log_pstar": rms_y},
        **heldout,
    }, net


def report_godunov(args, torch, fvs, workloads, net, peaks=None):
    """2-D first-order Godunov with the exact Riemann solver on an n^2
    four-quadrant problem drawn from the sampled distribution, Strang
    splitting, autotuned launch shapes, for the three Newton start values at
    each Newton tolerance (the reference's 1e-7 and a tight 1e-12)."""
    n = args.godunov_n
    cons = workloads.quadrants_2d(n, seed=3)
    by_tol = {}
    for tol in (float(t) for t in args.godunov_tols.split(",")):
        out = {}
        finals = {}
        for guess in ("mean", "pvrs_tr", "mlp"):
            if guess == "mlp" and net is None:
                continue
            m = fvs.make_method("godunov", guess=guess, tolerance=tol,
                                mlp_params=net.params_device_ptr() if guess == "mlp" else None)
            s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive", method=m)
            stream = torch.cuda.ExternalStream(s.stream_handle())
            s.upload(cons)
            s.autotune()
            s.run(cfl=0.8, t_end=1e9, max_steps=3)
            s.upload(cons)
            s.set_cycle(0)
            s.set_time(0.0)
            s.newton_stats(reset=True)
            torch.cuda.synchronize()
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            st, _ = s.run(cfl=0.8, t_end=1e9, max_steps=args.godunov_steps)
            b.record(stream)
            torch.cuda.synchronize()
            ms = a.elapsed_time(b)
            it, fail, fb = s.newton_stats(fallbacks=True)
            faces = st.steps * 4 * (n + 1) * n
            rate = 4 * n * n * st.steps / (ms / 1e3)
            out[guess] = {"steps": st.steps, "ms_per_step": ms / max(st.steps, 1),
                          "cell_updates_per_s": rate, "autotuned": s.tuning(),
                          "hbm_frac_algorithmic": (rate * 64 / 1e9 / peaks["hbm_gbs"]
                                                   if peaks else None),
                          "newton_iterations_per_interface": it / faces,
                          "fallback_rate": fb / faces, "not_converged": fail}
            finals[guess] = s.download()
            s.close()
        if "mean" in finals:
            for g in finals:
                out[g]["max_abs_diff_vs_mean_start"] = float(
                    np.abs(finals[g] - finals["mean"]).max())
        if "pvrs_tr" in out and "mlp" in out:
            out["mlp_speedup_vs_pvrs_tr"] = (out["pvrs_tr"]["ms_per_step"] /
                                             out["mlp"]["ms_per_step"])
        by_tol[f"{tol:g}"] = out
    return {"workload": f"2D perfect gas {n}^2 four quadrants, Godunov + exact Riemann solver, "
                        "Strang, CFL 0.8, transmissive", "by_tolerance": by_tol}


def report_sweep_variants(args, torch, fvs, workloads, peaks):
    """Single sweeps of the --n^3 octants workload in --precision, timed with
    CUDA events on the solver's stream, for every launch variant and segment
    length the autotuner tries (mixed: x lanes-along-x 0/4/5 or marching
    10/14/15; y/z marching 0/4/5 or TMA-staged 20/24/25); the best segment
    length per variant, 80 B per cell-update."""
    n = args.n
    cons = workloads.octants_3d(n)
    s = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic",
                   method=fvs.make_method(precision=args.precision))
    s.upload(cons)
    stream = torch.cuda.ExternalStream(s.stream_handle())
    dt = 0.4 * s.ComputeStableDt(-1)
    mixed = args.precision == "mixed"
    out = {"workload": f"single sweeps of the 3D {n}^3 octants state, {args.precision}",
           "sweeps": {}}
    for d in range(3):
        if mixed:
            variants = [0, 4, 5, 10, 14, 15] if d == 0 else [0, 4, 5, 20, 24, 25]
        else:
            variants = [0]
        for v in variants:
            best = None
            segs = [16] if (mixed and d == 0 and v < 10) else [8, 16, 32, 64, 128, 256]
            for seg in segs:
                try:
                    s.set_launch(d, seg, v)
                except fvs.FvsError:
                    break  # a variant this grid does not have (odd nx: no TMA)
                ts = []
                for rep in range(6):
                    a = torch.cuda.Event(enable_timing=True)
                    b = torch.cuda.Event(enable_timing=True)
                    a.record(stream)
                    s.sweep(d, dt)
                    b.record(stream)
                    torch.cuda.synchronize()
                    if rep >= 2:
                        ts.append(a.elapsed_time(b))
                ms = float(np.mean(ts))
                if best is None or ms < best[0]:
                    best = (ms, seg)
            if best is not None:
                gbs = 80 * n ** 3 / (best[0] / 1e3) / 1e9
                out["sweeps"][f"dir{d}_variant{v}"] = {
                    "ms": best[0], "segment_cells": best[1], "GB_per_s": gbs,
                    "hbm_frac": gbs / peaks["hbm_gbs"]}
    s.close()
    return out


def report_cutcell_sweeps(args, torch, fvs, workloads):
    """Single x and y sweeps of the --cutcell-n^2 shock-over-circles state in
    --precision, timed with CUDA events on the solver's stream (the cut-cell
    sweep's band kernel runs on its side stream inside the timed region),
    with the autotuned launch shapes, and one Strang step averaged over 50;
    the same grid without a body for comparison."""
    n = args.cutcell_n
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    out = {"workload": f"2D {n}^2 Mach 2 shock, {args.precision}", "grids": {}}
    for body in (False, True):
        s = fvs.Solver([n, n], [1.0 / n] * 2, "transmissive",
                       method=fvs.make_method(precision=args.precision))
        if body:
            s.set_embedded_circles(circles)
        s.upload(cons)
        s.autotune()
        stream = torch.cuda.ExternalStream(s.stream_handle())
        dt = 0.2 * s.ComputeStableDt(-1)
        us = []
        for d in (0, 1):
            ts = []
            for rep in range(8):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                s.sweep(d, dt)
                b.record(stream)
                torch.cuda.synchronize()
                if rep >= 2:
                    ts.append(a.elapsed_time(b))
            us.append(float(np.mean(ts)) * 1e3)
        s.upload(cons)
        s.run(cfl=0.5, t_end=1e9, max_steps=3)
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        s.run(cfl=0.5, t_end=1e9, max_steps=50)
        b.record(stream)
        torch.cuda.synchronize()
        out["grids"]["cut_cells" if body else "no_body"] = {
            "sweep_us": {"x": us[0], "y": us[1]}, "step_us": a.elapsed_time(b) * 1e3 / 50,
            "autotuned": s.tuning()}
        s.close()
    return out


def report_amr(args, torch, fvs, workloads, peaks):
    """Batched AMR patch set: 2-D blast (p 10 inside r < 0.1 about a seeded
    centre), 3 levels, ratio 2, 4096 patches with extents from {8, 16, 32,
    64}, level 0 covering n0^2, MUSCL-Hancock/VanLeer + HLLE, subcycled
    coarse steps (one CUDA graph each), for the three precision flavours."""
    h, cons = workloads.amr_blast_2d(args.amr_n0, 3, seed=7, target=4096)
    cells = h.cells()
    upd_per_step = int(4 * sum(int(cells[l]) << l for l in range(h.nlevels)))
    if args.profile_steps > 0:
        # profiling aid: the first flavour, launch shapes from --launch
        # (LEVEL:DIR:BLOCK:GRID:THREADS_PER_ROW) or the defaults, no autotuner
        a = fvs.AmrSolver(h, fvs.make_method(precision=args.amr_flavours.split(",")[0]))
        for spec in args.launch:
            lv, d, block, grid, tpr = (int(v) for v in spec.split(":"))
            a.set_launch(lv, d, block, grid, tpr)
        a.upload(cons)
        st, _ = a.run(cfl=0.8, t_end=1e9, max_steps=args.profile_steps)
        a.close()
        return {"profile_steps": st.steps}
    out = {"workload": f"2D blast on {h.npatches} patches, 3 levels (level 0 {args.amr_n0}^2), "
                       "ratio 2, extents from {8,16,32,64}, MUSCL-Hancock/VanLeer + HLLE, "
                       "subcycled Strang coarse steps, CFL 0.8, transmissive",
           "patches_per_level": np.bincount(h.levels, minlength=3).tolist(),
           "cells_per_level": cells.tolist(), "cell_updates_per_coarse_step": upd_per_step,
           "coarse_steps": args.amr_steps, "flavours": {}}
    finals = {}
    for prec in args.amr_flavours.split(","):
        a = fvs.AmrSolver(h, fvs.make_method(precision=prec))
        stream = torch.cuda.ExternalStream(a.stream_handle())
        a.upload(cons)
        cfg = a.autotune()
        a.run(cfl=0.8, t_end=1e9, max_steps=2)
        a.upload(cons)
        torch.cuda.synchronize()
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        st, _ = a.run(cfl=0.8, t_end=1e9, max_steps=args.amr_steps)
        e1.record(stream)
        torch.cuda.synchronize()
        ms = e0.elapsed_time(e1)
        finals[prec] = a.download()
        rate = upd_per_step * st.steps / (ms / 1e3)
        out["flavours"][prec] = {
            "ms_per_coarse_step": ms / max(st.steps, 1), "cell_updates_per_s": rate,
            "restarts": st.restarts,
            "hbm_frac_algorithmic": rate * 64 / 1e9 / peaks["hbm_gbs"],
            "launch_block_grid_threads_per_row": cfg.tolist()}
        a.close()
    if "fp64_exact" in finals:
        parts_ref = h.split(finals["fp64_exact"])
        base = out["flavours"]["fp64_exact"]["cell_updates_per_s"]
        for prec, f in finals.items():
            parts = h.split(f)
            l1 = float(np.mean(np.concatenate([np.abs(p[0] - q[0]).ravel()
                                               for p, q in zip(parts, parts_ref)])))
            out["flavours"][prec]["l1_density_vs_fp64_exact"] = l1
            out["flavours"][prec]["speedup_vs_fp64_exact"] = \
                out["flavours"][prec]["cell_updates_per_s"] / base
    # CPU: the oracle's restatement, one coarse step of the same hierarchy
    from oracle import build as obuild
    obuild.build()
    from oracle import oracle as orc
    threads = orc.max_threads()
    t0 = time.perf_counter()
    orc.amr_run(h, cons, 0.8, 1e9, max_steps=1, nthreads=threads)
    cpu_s = time.perf_counter() - t0
    out["cpu_baseline"] = {"value": upd_per_step / cpu_s, "unit": "cell-updates/s",
                           "cores": threads, "kind": "port",
                           "sample": "1 coarse step of the same hierarchy"}
    return out


def report_cutcell(args, torch, fvs, workloads, peaks=None):
    """2-D KBN h-box cut cells: Mach 2 shock over 8 seeded circles on n^2,
    Strang MUSCL-Hancock/VanLeer + HLLE, in the exact FP64, fast FP64 and
    mixed flavours; L1 density error against exact FP64 (which is the
    oracle's arithmetic bit for bit) and the drift of the volume-weighted
    mass and energy totals."""
    n = args.cutcell_n
    circles, cons = workloads.shock_circles_2d(n, seed=5)
    out = {"workload": f"2D {n}^2 Mach 2 shock over 8 circles, KBN h-box MUSCL/VanLeer + HLLE, "
                       "Strang, CFL 0.5, transmissive", "flavours": {}}
    finals = {}
    for prec in ("fp64_exact", "fp64_fast", "mixed"):
        s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive",
                       method=fvs.make_method(precision=prec))
        s.set_embedded_circles(circles)
        stream = torch.cuda.ExternalStream(s.stream_handle())
        s.upload(cons)
        s.autotune()
        s.run(cfl=0.5, t_end=1e9, max_steps=3)
        s.upload(cons)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        st, _ = s.run(cfl=0.5, t_end=1e9, max_steps=args.cutcell_steps)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        finals[prec] = s.download()
        if prec == "fp64_exact":
            geo = s.cutcell_geometry()
            G = geo["ghost"]
            alpha = geo["alpha"][G:-G, G:-G]
            out["cut_cells"] = int(geo["cut"][G:-G, G:-G].sum())
        rate = 4 * n * n * st.steps / (ms / 1e3)
        seg, occ = s.tuning()
        out["flavours"][prec] = {
            "steps": st.steps, "restarts": st.restarts, "ms_per_step": ms / max(st.steps, 1),
            "cell_updates_per_s": rate,
            "autotuned": {"segment_cells": seg, "variant": occ}}
        if peaks:
            # 64 B state + 64 B geometry (alpha, beta, shielded weights, x_B, normal)
            out["flavours"][prec]["hbm_frac_algorithmic"] = rate * 128 / 1e9 / peaks["hbm_gbs"]
        s.close()
        # drift: the same flow in a closed box (reflective walls on the domain
        # boundary), where nothing enters or leaves, so the volume-weighted
        # mass and energy totals may change only by round-off.  Bodies that
        # cross a wall are left out: behind a reflective wall the reference
        # reflects the states but keeps the bodies' real geometry
        # (cutcell::ReflectiveBoundary), which exchanges mass with the ghost
        # layers where a body straddles the wall.
        inside = circles[(circles[:, 0] - circles[:, 2] > 0) & (circles[:, 0] + circles[:, 2] < 1) &
                         (circles[:, 1] - circles[:, 2] > 0) & (circles[:, 1] + circles[:, 2] < 1)]
        s = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "reflective",
                       method=fvs.make_method(precision=prec))
        s.set_embedded_circles(inside)
        s.upload(cons)
        st, _ = s.run(cfl=0.5, t_end=1e9, max_steps=args.cutcell_steps)
        closed = s.download()
        geo = s.cutcell_geometry()
        G = geo["ghost"]
        w = geo["alpha"][G:-G, G:-G][None, None]
        t0 = (cons * w).reshape(4, -1).sum(axis=1)
        t1 = (closed * w).reshape(4, -1).sum(axis=1)
        scale = (np.abs(cons) * w).reshape(4, -1).sum(axis=1)
        out["flavours"][prec]["closed_box_drift_rel"] = {
            "steps": st.steps, "circles": int(len(inside)),
            "mass": float(abs(t1[0] - t0[0]) / scale[0]),
            "energy": float(abs(t1[3] - t0[3]) / scale[3])}
        s.close()
    ref = finals["fp64_exact"]
    w = alpha[None, None]
    for prec, f in finals.items():
        tot_ref = (ref * w).reshape(4, -1).sum(axis=1)
        tot = (f * w).reshape(4, -1).sum(axis=1)
        out["flavours"][prec]["l1_density_vs_fp64_exact"] = float(
            (np.abs(f[0] - ref[0]) * alpha).sum() / alpha.sum())
        # transmissive run: mass and energy totals against the exact flavour's
        # (the flow leaves through the open boundary, so this is no drift;
        # closed_box_drift_rel is)
        out["flavours"][prec]["mass_energy_diff_vs_fp64_exact_rel"] = [
            float(abs(tot[k] - tot_ref[k]) / abs(tot_ref[k])) for k in (0, 3)]
        out["flavours"][prec]["speedup_vs_fp64_exact"] = (
            out["flavours"][prec]["cell_updates_per_s"] /
            out["flavours"]["fp64_exact"]["cell_updates_per_s"])
    return out


def report_hllem(args, torch, fvs, workloads, peaks=None):
    """HLLEM (Larrouturou) without reconstruction and with MUSCL-Hancock of the
    conservative variables, and the perfect gas's characteristic and primitive
    MUSCL-Hancock reconstructions with HLLEM (van Leer), exact FP64 (the only
    flavour of this family), on the 3-D octants workload at --hllem-n; the
    oracle's restatement timed on one Strang step of the same grid."""
    n = args.hllem_n
    cons = workloads.octants_3d(n)
    out = {"workload": f"3D perfect gas {n}^3 periodic, Strang, CFL 0.8, seeded octants + "
                       "Gaussian bumps, exact FP64", "methods": {}}
    from oracle import build as obuild
    obuild.build()
    from oracle import oracle as orc
    threads = orc.max_threads()
    kinds = {"hllem": orc.HLLEM, "muscl_hllem": orc.MUSCL_HLLEM, "muscl_char": orc.MUSCL_CHAR,
             "muscl_prim": orc.MUSCL_PRIM}
    for name, kind in kinds.items():
        s = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic",
                       method=fvs.make_method(flux_method=name, precision="fp64_exact"))
        stream = torch.cuda.ExternalStream(s.stream_handle())
        s.upload(cons)
        s.autotune()
        s.run(cfl=0.8, t_end=1e9, max_steps=3)
        s.upload(cons)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        st, dts = s.run(cfl=0.8, t_end=1e9, max_steps=args.hllem_steps, log_len=1)
        b.record(stream)
        torch.cuda.synchronize()
        ms = a.elapsed_time(b)
        rate = 6 * n ** 3 * st.steps / (ms / 1e3)
        rec = {"steps": st.steps, "restarts": st.restarts, "ms_per_step": ms / max(st.steps, 1),
               "cell_updates_per_s": rate}
        if peaks:
            rec["hbm_frac_algorithmic"] = rate * 80 / 1e9 / peaks["hbm_gbs"]
        # CPU: the oracle's restatement, one Strang step with the GPU's first dt
        g = orc.Grid(3, [n] * 3, [0, 0, 0], [1.0 / n] * 3)
        t0 = time.perf_counter()
        g.step(orc.method(kind=kind), cons, float(dts[0]), 0, nthreads=threads)
        cpu_s = time.perf_counter() - t0
        rec["cpu_baseline"] = {"value": 6 * n ** 3 / cpu_s, "unit": "cell-updates/s",
                               "cores": threads, "kind": "port",
                               "sample": "1 Strang step of the same grid"}
        out["methods"][name] = rec
        s.close()
    return out


def headline_config(n: int) -> dict:
    """The headline workload, the same dict in both arms."""
    return {"workload": f"3D perfect gas {n}^3 periodic, Strang MUSCL-Hancock/VanLeer + HLLE, "
                        "CFL 0.8, seeded octants + Gaussian bumps",
            "n": n, "sweeps_per_step": 6,
            "l2": f"inputs larger than L2 (state {5 * 8 * n ** 3 / 1e6:.0f} MB per copy)"}


def run_reference(args):
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import build as obuild
    obuild.build()
    from oracle import oracle as orc
    threads = orc.max_threads()
    n = args.cpu_sample_n or args.n
    # warm-up then timed steps, one oracle Strang step per bench step
    if args.warmup > 0:
        cpu_reference_rate(n, args.warmup, threads)
    r = cpu_reference_rate(n, args.steps, threads)
    line = {
        "impl": "reference", "metric": METRIC, "value": r["value"], "unit": UNIT,
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": 1e3 * r["seconds"] / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": headline_config(n),
        "parallelism": f"{threads} OpenMP threads (host cores)",
        "precision": "fp64_exact (the reference's operation order, no FMA)",
        "cpu_baseline": {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
                         "sample": f"{args.steps} Strang steps of the {n}^3 workload, "
                                   "from its initial state"},
        "e2e": {"value": r["value"], "unit": UNIT, "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    import torch
    import finitevolumesolver_gb300 as fvs
    from finitevolumesolver_gb300 import build, partition, workloads

    rank, world, local = dist_env()
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    build.build()
    if args.report == "cutcell" and args.profile_steps > 0:
        # profiling aid: the cut-cell workload in --precision, launch shapes from
        # --launch, default shapes elsewhere
        n = args.cutcell_n
        circles, cons = workloads.shock_circles_2d(n, seed=5)
        solver = fvs.Solver([n, n], [1.0 / n, 1.0 / n], "transmissive",
                            method=fvs.make_method(precision=args.precision))
        solver.set_embedded_circles(circles)
        for spec in args.launch:
            d, seg, var = (int(v) for v in spec.split(":"))
            solver.set_launch(d, seg, var)
        solver.upload(cons)
        st, _ = solver.run(cfl=0.5, t_end=1e9, max_steps=args.profile_steps)
        solver.close()
        if rank == 0:
            print(json.dumps({"profile_steps": st.steps, "cutcell_n": n,
                              "precision": args.precision}), flush=True)
        return
    if args.report:
        peaks = load_peaks()
        if args.report == "sod":
            rep = report_sod(args, torch, fvs, workloads)
        elif args.report == "learned":
            rep, _ = report_mlp(args, torch, fvs, workloads)
        elif args.report == "godunov":
            _, net = report_mlp(args, torch, fvs, workloads)
            rep = report_godunov(args, torch, fvs, workloads, net, peaks)
        elif args.report == "amr":
            rep = report_amr(args, torch, fvs, workloads, peaks)
        elif args.report == "sweep_variants":
            rep = report_sweep_variants(args, torch, fvs, workloads, peaks)
        elif args.report == "cutcell_sweeps":
            rep = report_cutcell_sweeps(args, torch, fvs, workloads)
        elif args.report == "hllem":
            rep = report_hllem(args, torch, fvs, workloads, peaks)
        else:
            rep = report_cutcell(args, torch, fvs, workloads, peaks)
        if rank == 0:
            print(json.dumps({"report": args.report, **rep}), flush=True)
        return
    n = args.n
    cells = n ** 3
    cons = workloads.octants_3d(n)
    if args.profile_steps > 0:
        solver = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic",
                            method=fvs.make_method(precision=args.precision))
        for spec in args.launch:
            d, seg, var = (int(v) for v in spec.split(":"))
            solver.set_launch(d, seg, var)
        solver.upload(cons)
        st, _ = solver.run(cfl=0.8, t_end=1e9, max_steps=args.profile_steps)
        solver.close()
        if rank == 0:
            print(json.dumps({"profile_steps": st.steps, "n": n, "precision": args.precision}),
                  flush=True)
        return
    peaks = load_peaks()
    algo_bytes = 16 * (3 + 2) * cells  # state read once + written once, FP64

    def barrier():
        if world > 1:
            torch.distributed.barrier()

    def measure(precision: str, with_clocks: bool):
        method = fvs.make_method(precision=precision)
        solver = fvs.Solver([n] * 3, [1.0 / n] * 3, "periodic", method=method)
        stream = torch.cuda.ExternalStream(solver.stream_handle())
        solver.upload(cons)
        segs = solver.autotune()
        segs = {"segment_cells": segs, "occupancy_variant": solver.tuning()[1]}
        if args.warmup:
            solver.run(cfl=0.8, t_end=1e9, max_steps=args.warmup)
        clocks = ClockSampler(torch.cuda.current_device()) if with_clocks else None
        if clocks:
            clocks.start()
        barrier()
        torch.cuda.synchronize()
        ev0 = torch.cuda.Event(enable_timing=True)
        ev1 = torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        st, _ = solver.run(cfl=0.8, t_end=1e9, max_steps=args.steps)
        ev1.record(stream)
        torch.cuda.synchronize()
        barrier()
        clk = clocks.stop() if clocks else None
        ms = ev0.elapsed_time(ev1)
        ms = partition.slowest(ms)  # max over ranks (identity on one rank)
        assert st.steps == args.steps, "run stopped early"
        final = solver.download()
        # dominant kernel: the fused sweep; time single launches per direction
        sweep_ms = []
        dt = 0.4 * solver.ComputeStableDt(-1)
        for rep in range(2):
            for d in range(3):
                a = torch.cuda.Event(enable_timing=True)
                b = torch.cuda.Event(enable_timing=True)
                a.record(stream)
                solver.sweep(d, dt)
                b.record(stream)
                torch.cuda.synchronize()
                if rep == 1:
                    sweep_ms.append(a.elapsed_time(b))
        sweep_s = statistics.mean(sweep_ms) / 1e3
        achieved = algo_bytes / sweep_s / 1e9
        res = {"ms": ms, "value": 6 * cells * args.steps * world / (ms / 1e3), "segs": segs,
               "final": final, "clocks": clk, "sweep_s": sweep_s, "achieved": achieved,
               "solver": solver}
        return res

    main = measure(args.precision, with_clocks=True)
    solver = main["solver"]

    # End to end through the public API with a host-resident state: every
    # step uploads the state from pinned host memory, advances it one Strang
    # step (stable dt, dt selection, six sweeps) and writes it back into the
    # same pinned buffer, the next step's input (fvs_solver_step_host: the
    # write-back overlaps the step's last sweep, slab by slab).  A second
    # figure keeps the state on the device between one upload and one
    # download.  Both legs get the same W untimed warm-up steps as the device
    # leg (the first host-resident step creates the copy streams and events).
    L = fvs.lib()
    state_bytes = cons.nbytes
    pinned = torch.from_numpy(cons).pin_memory()
    for _ in range(args.warmup):
        solver.step_host(pinned, cfl=0.8, t_end=1e9)
    torch.cuda.synchronize()
    e2e_restarts = 0
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st_h = solver.step_host(pinned, cfl=0.8, t_end=1e9)
        assert st_h.steps == 1
        e2e_restarts += st_h.restarts
    e2e_s = time.perf_counter() - t0
    e2e_value = 6 * cells * args.steps * world / e2e_s
    pinned.copy_(torch.from_numpy(cons))
    out_host = torch.empty_like(pinned).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    L.fvs_solver_upload(solver._h, pinned.data_ptr())
    solver.run(cfl=0.8, t_end=1e9, max_steps=args.steps)
    L.fvs_solver_download(solver._h, out_host.data_ptr())
    e2e_amortised = 6 * cells * args.steps * world / (time.perf_counter() - t0)
    solver.close()
    main.pop("solver")

    variants = {}
    if not args.no_variants:
        for prec in ("fp64_exact", "fp64_fast", "fp64_df", "mixed"):
            if prec == args.precision:
                continue
            r = measure(prec, with_clocks=False)
            r["solver"].close()
            r.pop("solver")
            variants[prec] = r
    ref_final = None
    if args.precision == "fp64_exact":
        ref_final = main["final"]
    elif "fp64_exact" in variants:
        ref_final = variants["fp64_exact"]["final"]

    def accuracy(final):
        if ref_final is None:
            return None
        l1 = float(np.abs(final[0] - ref_final[0]).mean())
        tot0 = cons.reshape(5, -1).sum(1)
        tot = final.reshape(5, -1).sum(1)
        scale = np.abs(cons).reshape(5, -1).sum(1)
        return {"l1_density_vs_fp64_exact": l1,
                "max_conservation_drift_rel": float(np.max(np.abs(tot - tot0) / scale))}

    cpu = None
    if rank == 0:
        from oracle import build as obuild
        obuild.build()
        from oracle import oracle as orc
        threads = orc.max_threads()
        r = cpu_reference_rate(n, 1, threads)
        cpu = {"value": r["value"], "unit": UNIT, "cores": threads, "kind": "port",
               "sample": f"1 Strang step of the {n}^3 workload ({6 * cells} cell-updates)"}

    reports = None
    if rank == 0 and not args.no_reports:
        reports = {}
        try:
            reports["sod_1d"] = report_sod(args, torch, fvs, workloads)
        except Exception as e:
            reports["sod_1d"] = {"error": repr(e)}
        try:
            reports["learned_start_value"], net = report_mlp(args, torch, fvs, workloads)
        except Exception as e:  # report the failure, keep the headline
            reports["learned_start_value"] = {"error": repr(e)}
            net = None
        for key, fn in (("godunov_2d", lambda: report_godunov(args, torch, fvs, workloads, net,
                                                              peaks)),
                        ("amr_2d", lambda: report_amr(args, torch, fvs, workloads, peaks)),
                        ("cutcell_2d", lambda: report_cutcell(args, torch, fvs, workloads,
                                                              peaks)),
                        ("hllem_3d", lambda: report_hllem(args, torch, fvs, workloads, peaks))):
            try:
                reports[key] = fn()
            except Exception as e:
                reports[key] = {"error": repr(e)}

    if rank == 0:
        traffic = profile_traffic(f"sweep_{args.precision}_160.md", cells)
        line = {
            "metric": METRIC, "value": main["value"], "unit": UNIT, "n_gpus": world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": main["ms"] / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic",
            "config": headline_config(n),
            "parallelism": "replicas" if world > 1 else "single GPU",
            "precision": args.precision, "autotuned": main["segs"],
            "roofline": {"bound": "hbm", "achieved": main["achieved"], "peak": peaks["hbm_gbs"],
                         "unit": "GB/s", "frac": main["achieved"] / peaks["hbm_gbs"],
                         "traffic": traffic,
                         "kernel": "SweepMarchKernel (fused flux + update + CFL)",
                         "algorithmic_bytes_per_launch": algo_bytes,
                         "launch_ms": main["sweep_s"] * 1e3, "peak_source": peaks["source"],
                         "fp64_pipe_active_frac": profile_value(
                             f"sweep_{args.precision}_160.md", "fp64_pipe_active_frac"),
                         "note": "the FP64 flavours are bound by the FP64 pipe (2 FP64 "
                                 "operations per SM and clock on GB300), not by HBM"},
            "cpu_baseline": cpu,
            "e2e": {"value": e2e_value, "unit": UNIT,
                    "h2d_bytes_per_step": state_bytes + CONTROL_BYTES,
                    "d2h_bytes_per_step": state_bytes + CONTROL_BYTES,
                    "mode": "host-resident state: every step uploads the state from pinned "
                            "host memory, advances it one Strang step and writes it back "
                            "(fvs_solver_step_host: the last sweep runs in 8 slabs and each "
                            "slab's copy overlaps the rest of the sweep)",
                    "restarts": e2e_restarts,
                    "amortised": {"value": e2e_amortised, "unit": UNIT,
                                  "h2d_bytes_per_step": (state_bytes + CONTROL_BYTES) /
                                  args.steps,
                                  "d2h_bytes_per_step": (state_bytes + CONTROL_BYTES * (
                                      args.steps // 30 + 1)) / args.steps,
                                  "mode": "one upload, K device-resident steps, one download"}},
            "gpu_launches": 9 * args.steps,
            "clocks": main["clocks"],
            "accuracy": accuracy(main["final"]),
            "variants": {k: {"value": v["value"], "ms_per_step": v["ms"] / args.steps,
                             "sweep_launch_ms": v["sweep_s"] * 1e3,
                             "autotuned": v["segs"],
                             "hbm_frac": v["achieved"] / peaks["hbm_gbs"],
                             "accuracy": accuracy(v["final"])}
                         for k, v in variants.items()},
            "reports": reports,
        }
        print(json.dumps(line), flush=True)
    if world > 1:
        torch.distributed.destroy_process_group()


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
