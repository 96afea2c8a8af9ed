"""Benchmark of the lattice-Boltzmann step on one GB300 (N GPUs: replicas).

Workload (default): the D3Q19 channel -- periodic in x and z, bounce-back
(NoSlip) walls at y = 0 and y = Ny, Guo body force 1e-6 along x, tau = 0.6,
rho = 1 + seeded uniform noise of amplitude 1e-4, u = 0 -- on a 512^3 grid
(2 x 20.4 GB of FP64 populations, far larger than the 129 MB L2, so no L2
flush is needed between steps).  One step = one advance() of the whole grid.

Prints one JSON line (rank 0):
  value     MLUPS with the populations resident in HBM (device-timed, CUDA
            events on the step kernel's stream)
  e2e       MLUPS through the C ABI with host buffers: every step uploads the
            populations from pinned host memory, advances, downloads them
  roofline  achieved HBM bandwidth of the step kernel (algorithmic bytes
            2*Q*8 per cell update) against the measured copy peak
  cpu_baseline  the reference's CPU step on the host cores, bounded sample of
            the same workload: its own src/LBM code (built by
            oracle/build_ref.sh from the checkout or the copy staged in
            baseline/_ref, kind "reference"), else the restatement ("port")

--impl reference: the same reference CPU step on the host cores with all
threads, on the same workload and metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

LATTICE_Q = {"D2Q9": 9, "D3Q15": 15, "D3Q19": 19, "D3Q27": 27}
ELEM = {"f64": 8, "f64_fast": 8, "f32": 4, "f16s": 2, "bf16s": 2, "f64x": 8, "f16c": 2, "f16w": 2}
DTYPE = {"f64": "f64", "f64_fast": "f64", "f32": "f32", "f16s": "f16 storage / f32 arithmetic",
         "bf16s": "bf16 storage / f32 arithmetic", "f16c": "custom 1-4-11 16-bit storage / f32 arithmetic",
         "f16w": "custom 1-3-12 16-bit storage of (f - w) / p, p the power of two nearest to w / f32 arithmetic",
         "f64x": "int64 fixed point (f/w in units of 2^-56), FP64-accurate"}
METRIC = "MLUPS"


def peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            p = json.load(fh)
        return float(p["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def ncu_traffic(workload: str):
    """Per-launch DRAM bytes of the step kernel from a committed ncu summary."""
    path = os.path.join(ROOT, "profiles", "traffic.json")
    try:
        with open(path) as fh:
            return json.load(fh).get(workload)
    except Exception:
        return None


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.25)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 8:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[4:8]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def channel_desc(m, n, precision, tau=0.6, F=1e-6):
    faces = ["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic", "Periodic"]
    return m.make_desc("D3Q19", n, 1.0 / tau, faces=faces, force=(F, 0.0, 0.0), precision=precision)


def channel_fields(n, seed=20261203):
    N = n[0] * n[1] * n[2]
    rng = np.random.default_rng(seed)
    return 1.0 + rng.uniform(-1e-4, 1e-4, N), np.zeros(3 * N)


def cpu_kind():
    """'reference' when the reference's own LBM sources are built on this host
    (oracle/_ref, from the checkout or the copy staged in baseline/_ref),
    else 'port' (the restatement, bit-identical to it)."""
    from oracle import oracle as O
    if not O.ref_available():
        try:
            O.build_ref()
        except Exception:
            pass
    return "reference" if O.ref_available() else "port"


def cpu_reference(n, steps, warmup, threads, kind="port"):
    """The reference CPU path on `threads` host threads: MLUPS.  kind
    'reference' runs the reference's own pullCollideFusedMF (its OpenMP
    MFIter loops over 8-cell tiles) and ghost fill; 'port' the restatement."""
    from oracle import oracle as O
    O.build()
    cfg = O.Config("D3Q19", n, omega=1.0 / 0.6, faces=["Periodic", "Periodic", "NoSlip", "NoSlip", "Periodic",
                                                       "Periodic"], force=(1e-6, 0.0, 0.0))
    sim = O.OracleSim(cfg, "ref" if kind == "reference" else "port")
    rho, u = channel_fields(n)
    sim.init_fields(rho, u)
    if warmup:
        sim.step(warmup, threads)
    t0 = time.perf_counter()
    sim.step(steps, threads)
    dt = time.perf_counter() - t0
    cells = n[0] * n[1] * n[2]
    return cells * steps / dt / 1e6, dt


def tgv3d_fields(n, u0):
    """3-D Taylor-Green vortex on a periodic n^3 box (project-defined, no
    reference counterpart): x = 2 pi (i + 1/2) / n,
    u = u0 (sin x cos y cos z, -cos x sin y cos z, 0),
    rho = 1 + 3 u0^2 / 16 (cos 2x + cos 2y)(cos 2z + 2) (the incompressible
    pressure over cs^2)."""
    t = 2.0 * np.pi * (np.arange(n) + 0.5) / n
    s, c = np.sin(t), np.cos(t)
    c2 = np.cos(2 * t)
    z, y, x = np.meshgrid(np.arange(n), np.arange(n), np.arange(n), indexing="ij", sparse=True)
    u = np.empty((3, n, n, n))
    u[0] = u0 * s[x] * c[y] * c[z]
    u[1] = -u0 * c[x] * s[y] * c[z]
    u[2] = 0.0
    rho = 1.0 + 3.0 * u0 * u0 / 16.0 * (c2[x] + c2[y]) * (c2[z] + 2.0)
    return rho.reshape(-1), u.reshape(-1)


def run_tgv3d(args):
    """Precision study: D3Q27 TGV at n^3, tau 0.52, u0 0.05; the shifted FP16,
    BF16, custom 1-4-11 (f16c) and weight-scaled 1-3-12 (f16w) storage
    against the FP64-accurate reference path, velocity L2 and kinetic-energy
    errors and FP64 mass / momentum sums every `every` steps."""
    import muphfasa_gb300 as m
    m.set_device(0)
    n, u0, tau = args.n, 0.05, 0.52
    every, total = args.every, args.tgv_steps
    rho, u = tgv3d_fields(n, u0)
    N = n ** 3
    names = [args.tgv_ref, "f16s", "bf16s", "f16c", "f16w"]
    sims = {}
    for p in names:
        s = m.Simulation(m.make_desc("D3Q27", (n, n, n), 1.0 / tau, precision=p))
        s.initialize(rho.copy(), u.copy())
        sims[p] = s
    del rho, u
    mass0 = {p: sims[p].reduce()[0] for p in names}
    ms = {p: 0.0 for p in names}
    table = []
    for step in range(every, total + 1, every):
        vel = {}
        row = {"step": step}
        for p in names:
            ms[p] += sims[p].advance_timed(every)
            r, v = sims[p].update_macroscopic()
            vel[p] = v
            sums = sims[p].reduce()
            row[p] = {"mass_drift": float((sums[0] - mass0[p]) / mass0[p]),
                      "momentum": [float(x) for x in sums[1:4]]}
        ref = vel[names[0]]
        ke_ref = 0.5 * float(np.dot(ref, ref)) / N
        nref = float(np.linalg.norm(ref))
        row[names[0]]["ke"] = ke_ref
        for p in names[1:]:
            d = vel[p] - ref
            ke = 0.5 * float(np.dot(vel[p], vel[p])) / N
            row[p].update({"u_l2_rel": float(np.linalg.norm(d)) / nref, "ke_rel": abs(ke - ke_ref) / ke_ref})
        del vel
        table.append(row)
        print(json.dumps({"progress": row}), file=sys.stderr, flush=True)
    mlups = {p: N * total / (ms[p] / 1e3) / 1e6 for p in names}
    bytes_cell = {"f64x": 432, "f64": 432, "f64_fast": 432, "f32": 216, "f16s": 108, "bf16s": 108, "f16c": 108, "f16w": 108}
    peak, kind = peaks()
    last = table[-1]
    line = {"metric": "velocity L2 error vs FP64-accurate reference (and MLUPS)",
            "value": last["f16s"]["u_l2_rel"], "unit": "relative", "n_gpus": 1, "steps": total, "warmup": 0,
            "higher_is_better": False, "scaling": "weak", "vs_baseline": None, "dtype": "f16 / bf16 / custom 1-4-11 / 1-3-12 storage, f32 collide",
            "data": "synthetic",
            "config": {"workload": f"tgv3d_d3q27_{n}^3", "lattice": "D3Q27", "grid": [n] * 3, "tau": tau, "u0": u0,
                       "reference_precision": names[0], "every": every,
                       "init": "u = u0 (sin x cos y cos z, -cos x sin y cos z, 0), "
                               "rho = 1 + 3 u0^2/16 (cos 2x + cos 2y)(cos 2z + 2)"},
            "mlups": {p: round(v, 1) for p, v in mlups.items()},
            "roofline_frac": {p: round(mlups[p] * 1e6 * bytes_cell[p] / 1e9 / peak, 4) for p in names},
            "table": table}
    print(json.dumps(line), flush=True)
    for s in sims.values():
        s.close()
    return 0


def run_ceiling(args):
    """The step's memory pattern without its arithmetic (mph_pull_copy_timed):
    pull-stencil copies of the D3Q19 / D3Q27 populations on an n^3 periodic
    grid for 8-, 4- and 2-byte elements; for 2 bytes the 16-bit step kernel's
    pattern (16-bit loads for x-shifted populations) and the word-and-shuffle
    pattern.  GB/s = 2 Q elem bytes x cells / time, against the measured copy
    peak."""
    import muphfasa_gb300 as m
    m.set_device(0)
    n = args.n
    peak, kind = peaks()
    rows = []
    for q in (19, 27):
        for elem, mode, name in ((8, 0, "8-byte, one cell per thread"), (4, 0, "4-byte, one cell per thread"),
                                 (2, 0, "2-byte, one cell per thread"),
                                 (2, 1, "2-byte pairs, 16-bit loads for x-shifted populations"),
                                 (2, 2, "2-byte pairs, aligned 32-bit words + warp shuffles")):
            best = min(m.pull_copy_ms(elem, mode, q, (n, n, n), reps=args.steps) for _ in range(3))
            gbs = 2 * q * elem * n ** 3 / (best / 1e3) / 1e9
            rows.append({"q": q, "elem_bytes": elem, "mode": mode, "pattern": name, "ms": round(best, 4),
                         "gbs": round(gbs, 1), "frac": round(gbs / peak, 4),
                         "glups": round(n ** 3 / (best / 1e3) / 1e9, 2)})
            print(json.dumps({"progress": rows[-1]}), file=sys.stderr, flush=True)
    # arithmetic pipes (mph_pipe_rate): operations per second and per SM per clock
    sm = ClockSampler(0)
    with sm:
        rates = {name: m.pipe_rate(op) for op, name in enumerate(("DFMA", "FFMA", "IMAD32", "UMULHI64+ADD",
                                                                  "I2F.F64.S64+DADD"))}
    clk = sm.summary()
    mhz = clk.get("sm_mhz") or 2070.0
    pipes = {k: {"gops": round(v / 1e9, 1), "per_sm_per_clk": round(v / 152 / (mhz * 1e6), 2)} for k, v in rates.items()}
    line = {"metric": "pull-stencil copy bandwidth (the step's memory pattern, no arithmetic)", "value": None,
            "unit": "GB/s", "n_gpus": 1, "steps": args.steps, "higher_is_better": True, "data": "synthetic",
            "config": {"workload": f"pull_copy_{n}^3", "best_of": 3, "peak": peak, "peak_kind": kind},
            "rows": rows, "pipes": pipes, "pipes_clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def tgv2d_fields(N, u0):
    """2-D Taylor-Green vortex of the benchmark's CPU-runnable configuration:
    u = u0 (sin kx cos ky, -cos kx sin ky), k = 2 pi / N, cell centres
    x = i + 1/2, rho = 1 - 3 u0^2 / 4 (cos 2kx + cos 2ky)."""
    k = 2.0 * math.pi / N
    x = np.arange(N) + 0.5
    X, Y = np.meshgrid(x, x, indexing="xy")
    ux = u0 * np.sin(k * X) * np.cos(k * Y)
    uy = -u0 * np.cos(k * X) * np.sin(k * Y)
    rho = 1.0 - 0.75 * u0 * u0 * (np.cos(2 * k * X) + np.cos(2 * k * Y))
    return rho.ravel(), np.concatenate([ux.ravel(), uy.ravel()])


def surrogate_measure(n, steps, warmup):
    """Training iterations of the warm-start U-Net (batch 8, n^2 cells):
    (seconds, last loss, parameters, clock summary)."""
    import muphfasa_gb300 as m
    from muphfasa_gb300 import surrogate as sg
    from muphfasa_gb300.surrogate import Trainer, UNet
    sync = lambda: m.check(sg._lib().mph_nn_sync(None))
    B = 8
    rng = np.random.default_rng(5)
    X = rng.standard_normal((B, n, n, 8)).astype(np.float32)
    Y = rng.standard_normal((B, n, n, 3)).astype(np.float32)
    M = (rng.random((B, n, n)) < 0.9).astype(np.float32)
    net = UNet(seed=1)
    tr = Trainer(net, B, n, n)
    for _ in range(warmup):
        tr.train_step(X, Y, M, 1e-4)
    sync()
    sm = ClockSampler(0)
    with sm:
        t0 = time.perf_counter()
        for _ in range(steps):
            loss = tr.train_step(X, Y, M, 1e-4)
        sync()
        dt = time.perf_counter() - t0
    return dt, float(loss), net.n_params(), sm.summary()


def run_surrogate(args):
    """Training throughput of the warm-start U-Net: Adam iterations (forward,
    masked loss, backward, gradient clipping, update) on seeded synthetic
    fields of the warm-start shape (batch 8, ws_n^2 cells, 8 input and 3
    output channels), timed end to end including the host-side input upload
    and loss download of every iteration."""
    import muphfasa_gb300 as m
    m.set_device(0)
    n = args.ws_n
    dt, loss, nparams, clk = surrogate_measure(n, args.steps, args.warmup)
    B = 8
    line = {"metric": "surrogate training iterations per second", "value": round(args.steps / dt, 2),
            "unit": "iterations/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(1e3 * dt / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "bf16 operands / f32 accumulate", "data": "synthetic",
            "config": {"workload": f"unet_train_{n}^2_batch{B}", "params": nparams,
                       "gemm": "tcgen05 BF16 (TMA-fed where operands are K-contiguous; mma.sync below 128 rows)"},
            "loss": round(loss, 6), "clocks": clk}
    print(json.dumps(line), flush=True)
    return 0


def run_tgv2d(args):
    """The CPU-runnable configuration: 2-D Taylor-Green vortex, D2Q9, periodic
    256^2, tau 0.8, u0 0.05, 5000 steps.  MLUPS per precision with the
    32-step CUDA-graph runs of small domains and with plain launches (one per
    step), the amplitude decay against exp(-2 nu k^2 t), and the reference's
    CPU step on the host cores on the same case."""
    import muphfasa_gb300 as m
    m.set_device(0)
    N, tau, u0, steps = args.n, 0.8, 0.05, args.tgv_steps
    nu = (tau - 0.5) / 3.0
    k = 2.0 * math.pi / N
    rho, u = tgv2d_fields(N, u0)
    rows = {}
    for p in ("f64", "f64x", "f32"):
        row = {}
        for mode, env in (("graph", None), ("plain", "0")):
            if env is None:
                os.environ.pop("MPH_GRAPH_STEPS", None)
            else:
                os.environ["MPH_GRAPH_STEPS"] = env
            s = m.Simulation(m.make_desc("D2Q9", (N, N), 1.0 / tau, precision=p))
            s.initialize(rho.copy(), u.copy())
            s.advance(args.warmup)
            with ClockSampler(0) as clk:
                ms = s.advance_timed(steps)
            _, us = s.update_macroscopic()
            amp = float(np.abs(us).max() / u0)
            row[mode] = {"mlups": round(N * N * steps / (ms / 1e3) / 1e6, 1), "ms_per_step": round(ms / steps, 5),
                         "decay_rel_err": abs(amp / math.exp(-2 * nu * k * k * (steps + args.warmup)) - 1.0),
                         "clocks": clk.summary()}
            s.close()
        row["graph_gain"] = round(row["graph"]["mlups"] / row["plain"]["mlups"], 3)
        rows[p] = row
    os.environ.pop("MPH_GRAPH_STEPS", None)
    from oracle import oracle as O
    kind = cpu_kind()
    o = O.OracleSim(O.Config("D2Q9", (N, N), omega=1.0 / tau), "ref" if kind == "reference" else "port")
    o.init_fields(rho, u)
    threads = os.cpu_count() or 1
    t0 = time.perf_counter()
    o.step(min(steps, 1000), threads)
    dt = time.perf_counter() - t0
    cpu = {"value": round(N * N * min(steps, 1000) / dt / 1e6, 3), "unit": "MLUPS", "cores": threads, "kind": kind,
           "sample": f"{N}^2, {min(steps, 1000)} steps, FP64, {threads} threads ({dt:.2f} s)"}
    line = {"metric": METRIC, "value": rows["f64"]["graph"]["mlups"], "unit": "MLUPS", "n_gpus": 1, "steps": steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
            "data": "synthetic", "config": {"workload": f"tgv2d_d2q9_{N}^2", "tau": tau, "u0": u0,
                                            "l2": "fits in L2 (the configuration's own size)"},
            "precisions": rows, "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)
    return 0


def warmstart_curves(ws, cases, fields, rest, max_steps, consistent):
    """Steps to 1e-8 against the relative error e of the initial field
    (converged fields + smooth noise), with the plain feq + f_neq start and with
    the consistent start (ws.consistent_start, `consistent` = (steps, rounds))."""
    amps = [0.3, 0.1, 3e-2, 1e-2, 1e-3, 1e-4, 1e-5, 1e-6, 0.0]
    rest = np.asarray(rest, float)
    out, secs = {}, 0.0
    for name, cons in (("feq_fneq", None), ("consistent", consistent)):
        rng = np.random.default_rng(0)
        run, inits, keys = [], [], []
        for c, (rho, u) in zip(cases, fields):
            for e in amps:
                run.append(c)
                inits.append(ws.perturbed_fields(c, rho, u, e, rng))
                keys.append(e)
        t0 = time.perf_counter()
        st, _, _, _ = ws.solve(run, inits, max_steps=max_steps, consistent=cons)
        secs += time.perf_counter() - t0
        rows = []
        for e in amps:
            se = np.array([x for x, k in zip(st, keys) if k == e], float)
            ok = (se > 0) & (rest > 0)
            rows.append({"rel_error": e, "steps_median": float(np.median(se[se > 0])) if np.any(se > 0) else None,
                         "gain_median": float(np.median(rest[ok] / se[ok])) if ok.any() else None})
        out[name] = rows
    out["consistent_start"] = {"steps": consistent[0], "rounds": consistent[1]}
    out["rest_steps_median"] = float(np.median(rest[rest > 0])) if np.any(rest > 0) else None
    out["cases"] = len(cases)
    return out, secs


def run_warmstart_curve(args, m, ws, log):
    """--ws-train 0: only the steps-vs-error curves, on the converged fields of
    the first --ws-curve held-out cases (no data generation, no training)."""
    n = args.ws_n
    test_cases = ws.draw_cases(args.ws_test, seed=202, sizes=(n,))
    sp, ref, secs_plain, _ = ws.solve(test_cases, None, max_steps=args.ws_max_steps)
    conv = [i for i in range(len(test_cases)) if sp[i] > 0][: args.ws_curve]
    curves, secs = warmstart_curves(ws, [test_cases[i] for i in conv], [ref[i] for i in conv], [sp[i] for i in conv],
                                    args.ws_max_steps, tuple(int(v) for v in args.ws_consistent.split(",")))
    line = {"metric": "steps to residual 1e-8 against the initial field's error", "value": None, "unit": "steps",
            "n_gpus": 1, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "solver int64 fixed point (FP64-accurate)", "data": "synthetic",
            "config": {"workload": f"warmstart_curve_d2q9_{n}^2", "test_cases": len(test_cases),
                       "Re": list(ws.RE), "U": list(ws.U)},
            "error_vs_steps": curves, "seconds": {"solve_from_rest": round(secs_plain, 1), "curves": round(secs, 1)}}
    print(json.dumps(line), flush=True)
    return 0


def run_warmstart(args):
    """Learned warm start: the plain solver (FP64-accurate fixed point, batch
    of all cases, converged cases leaving the batch) generates steady fields
    of seeded cavity / channel cases to the residual 1e-8; the U-Net is
    trained on them with the library's BF16 tensor-core kernels; held-out
    cases are solved to 1e-8 from rest and from the surrogate's prediction
    (feq + f_neq), in a batch and on single handles; and the steps to 1e-8
    are measured against the relative error of an initial field (converged
    held-out fields plus smooth noise), which says what surrogate error a
    given gain needs."""
    import muphfasa_gb300 as m
    from muphfasa_gb300 import warmstart as ws
    m.set_device(0)
    n = args.ws_n
    log = lambda *a: print(json.dumps({"progress": a}), file=sys.stderr, flush=True)
    if args.ws_train == 0:
        return run_warmstart_curve(args, m, ws, log)
    # draw ws_draw cases (at least ws_train) and keep the first ws_train that
    # reach the residual 1e-8: high-Re cases near tau = 1/2 diverge or stall
    train_cases = ws.draw_cases(max(args.ws_draw, args.ws_train), seed=101, sizes=(n,))
    test_cases = ws.draw_cases(args.ws_test, seed=202, sizes=(n,))
    st, fields, gen_secs, last = ws.solve(train_cases, max_steps=args.ws_gen_steps, tol=1e-8, check_every=2000,
                                          log=lambda *a: log("gen", *a) if a[0] % 20000 == 0 else None)
    keep = [i for i in range(len(train_cases)) if st[i] > 0][: args.ws_train]
    X, Y, M = ws.dataset([train_cases[i] for i in keep], [fields[i] for i in keep])
    log("generated", len(keep), X.shape[0], len(train_cases), round(gen_secs, 1))
    t1 = time.perf_counter()
    X, Y, M = ws.mirror_channels(X, Y, M)
    ntrain = X.shape[0]
    net, hist = ws.train(X, Y, M, epochs=args.ws_epochs, batch=8, lr=args.ws_lr,
                         log=lambda e, l: log("epoch", e, l) if e % 10 == 0 else None)
    train_secs = time.perf_counter() - t1
    sub_idx = keep[:64]  # error on (up to) 64 training fields, the held-out metric
    p_tr, _ = ws.predict(net, [train_cases[i] for i in sub_idx])
    train_err = [ws.field_error(train_cases[i], p, fields[i]) for i, p in zip(sub_idx, p_tr)]
    del X, Y, M
    preds, pred_secs = ws.predict(net, test_cases)
    sp, ref, secs_plain, rp = ws.solve(test_cases, None, max_steps=args.ws_max_steps)
    log("plain", int(np.sum(sp > 0)), round(secs_plain, 1))
    sw, _, secs_warm, rw = ws.solve(test_cases, preds, max_steps=args.ws_max_steps)
    log("warm", int(np.sum(sw > 0)), round(secs_warm, 1))
    both = (sp > 0) & (sw > 0)
    err_all = np.array([ws.field_error(c, p, r) if ok else np.nan for c, p, r, ok in zip(test_cases, preds, ref, sp > 0)])
    errs = err_all[~np.isnan(err_all)]
    by_kind = {k: float(np.nanmedian(err_all[[c["kind"] == k for c in test_cases]])) for k in ("cavity", "channel")}
    good = both & (err_all < 0.2)
    # steps to 1e-8 against the initial field's relative error (converged held-out fields + smooth noise)
    conv = [i for i in range(len(test_cases)) if sp[i] > 0][: args.ws_curve]
    curves, curve_secs = warmstart_curves(ws, [test_cases[i] for i in conv], [ref[i] for i in conv],
                                          [sp[i] for i in conv], args.ws_max_steps,
                                          tuple(int(v) for v in args.ws_consistent.split(",")))
    # single-case wall time (one FP64-accurate handle per case): rest vs predict + warm start
    single = []
    for c in [c for c, ok in zip(test_cases, both) if ok][: args.ws_single]:
        row = {}
        for mode in ("plain", "warm"):
            tt = time.perf_counter()
            s = m.Simulation(ws.case_desc(c, "f64x"))
            s.set_obstacles(ws.case_mask(c))
            if mode == "plain":
                s.initialize()
            else:
                (pr,), _ = ws.predict(net, [c], batch=1)
                s.initialize_neq(*pr)
            steps, r = 0, np.inf
            while steps < args.ws_max_steps and not r < 1e-8:
                s.advance(900)
                s.residual()
                s.advance(100)
                r, _ = s.residual()
                steps += 1000
            row[mode] = {"steps": steps, "seconds": round(time.perf_counter() - tt, 3)}
            s.close()
        single.append(row)
    ratio = sp[both] / sw[both]
    wall_single = [r["plain"]["seconds"] / r["warm"]["seconds"] for r in single]
    line = {"metric": "steps and wall time to residual 1e-8, warm start vs start from rest",
            "value": round(float(np.median(ratio)), 3) if ratio.size else None, "unit": "x (median over cases)",
            "n_gpus": 1, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "surrogate bf16 / f32 accumulate; solver int64 fixed point (FP64-accurate)", "data": "synthetic",
            "config": {"workload": f"warmstart_d2q9_{n}^2", "train_cases": len(train_cases),
                       "train_diverged": int(np.sum(st == -2)), "train_not_converged": int(np.sum(st == -1)),
                       "kept_at_1e-8": len(keep), "trained_on": int(ntrain), "test_cases": len(test_cases),
                       "epochs": args.ws_epochs, "gen_max_steps": args.ws_gen_steps, "params": net.n_params(),
                       "Re": list(ws.RE), "U": list(ws.U)},
            "steps_plain_median": float(np.median(sp[sp > 0])) if np.any(sp > 0) else None,
            "steps_warm_median": float(np.median(sw[sw > 0])) if np.any(sw > 0) else None,
            "steps_ratio_total": float(sp[both].sum() / sw[both].sum()) if np.any(both) else None,
            "converged": {"plain": int(np.sum(sp > 0)), "warm": int(np.sum(sw > 0)), "both": int(np.sum(both)),
                          "diverged_plain": int(np.sum(sp == -2))},
            "surrogate_u_error_train": float(np.median(train_err)) if train_err else None,
            "surrogate_u_error": {"median": float(np.median(errs)) if errs.size else None,
                                  "p10": float(np.percentile(errs, 10)) if errs.size else None,
                                  "p90": float(np.percentile(errs, 90)) if errs.size else None, "by_kind": by_kind},
            "steps_ratio_when_error_below_0.2": {"cases": int(good.sum()),
                                                 "median": float(np.median(sp[good] / sw[good])) if good.any() else None},
            "error_vs_steps": curves,
            "seconds": {"generate": round(gen_secs, 1), "train": round(train_secs, 1),
                        "predict_all": round(pred_secs, 3), "batch_plain": round(secs_plain, 1),
                        "batch_warm": round(secs_warm, 1), "curve": round(curve_secs, 1)},
            "batch_wall_ratio": round(secs_plain / secs_warm, 3) if secs_warm > 0 else None,
            "single_case_wall": {"cases": single,
                                 "median_ratio": float(np.median(wall_single)) if wall_single else None},
            "train_loss": [round(h, 6) for h in hist[:: max(1, len(hist) // 20)]] + [round(hist[-1], 6)]}
    print(json.dumps(line), flush=True)
    return 0


def cpu_model():
    """Host CPU name and core count (for the baseline record)."""
    name = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for ln in out.splitlines():
            if ln.startswith("Model name:"):
                name = ln.split(":", 1)[1].strip()
                break
    except Exception:
        pass
    return {"model": name, "nproc": os.cpu_count()}


def run_reference(args):
    from muphfasa_gb300 import replicas
    rank, world, _ = replicas.rank_info()
    if rank != 0:
        return 0
    threads = os.cpu_count() or 1
    n = (256, 256, 256)
    kind = cpu_kind()
    value, dt = cpu_reference(n, args.steps, args.warmup, threads, kind)
    what = ("the reference's own pullCollideFusedMF (src/LBM, OpenMP MFIter loops over 8-cell tiles) and ghost fill"
            if kind == "reference" else "the restated reference CPU path, OpenMP over cells")
    extra = {}
    if kind == "reference":  # the restatement beside it, 5 steps
        vp, _ = cpu_reference(n, 5, 1, threads, "port")
        extra = {"port": {"value": round(vp, 3), "unit": "MLUPS", "sample": f"{n[0]}^3, 5 steps, {threads} threads"}}
    line = {
        "impl": "reference", "metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(1e3 * dt / args.steps, 3),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": f"channel_d3q19_{args.n}^3", "lattice": "D3Q19", "grid": [args.n] * 3, "tau": 0.6,
                   "force": 1e-6, "sample_grid": list(n), "parallelism": "replicas"},
        "cpu_baseline": {"value": round(value, 3), "unit": "MLUPS", "cores": threads, "kind": kind,
                         "sample": f"{n[0]}^3 domain of the workload, {args.steps} steps after {args.warmup} warm-up, "
                                   f"{what}, {threads} threads",
                         "host": cpu_model(), **extra},
        "e2e": {"value": round(value, 3), "unit": "MLUPS", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)
    return 0


def batch_measure(m, domains, steps, warmup, prec, device=0):
    """512 independent lid-driven cavities, D2Q9, side log-uniform in [64, 512],
    Re log-uniform in [100, 5000] (tau = 0.5 + 3 u_lid N / Re): one batched
    kernel per step (CUDA graph) against one launch per domain.  Returns the
    record (MLUPS, roofline, looped MLUPS) and the clock summary."""
    descs = m.cavity_batch_descs(domains, precision=prec)
    batch = m.Batch(descs)
    for i in range(len(descs)):
        batch.initialize(i)
    batch.advance(warmup)
    total, kcells, nchunks, persistent = batch.info()
    with ClockSampler(device) as clk:
        ms = batch.advance_timed(steps)
    steps_loop = max(2, steps // 4)
    ms_loop = batch.advance_looped_timed(steps_loop)
    batch.close()
    q, es = 9, ELEM[prec]
    value = total * steps / (ms / 1e3) / 1e6
    looped = total * steps_loop / (ms_loop / 1e3) / 1e6
    achieved = 2 * q * es * total / (ms / steps / 1e3) / 1e9
    peak, kind = peaks()
    rec = {"metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "steps": steps, "warmup": warmup,
           "ms_per_step": round(ms / steps, 4), "dtype": DTYPE[prec],
           "config": {"workload": f"batch{domains}_cavities_d2q9", "domains": domains, "total_cells": total,
                      "side": [64, 512], "Re": [100, 5000], "lid": 0.1, "precision": prec,
                      "cells_per_thread": kcells, "chunks": nchunks, "persistent_grid": persistent,
                      "graph": "2-step CUDA graph", "l2": "inputs larger than L2 (no flush needed)"},
           "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                        "frac": round(achieved / peak, 4), "traffic": None, "peak_kind": kind,
                        "bytes_per_cell_update": 2 * q * es},
           "looped_single_domain": {"value": round(looped, 3), "unit": "MLUPS", "steps": steps_loop,
                                    "launches_per_step": domains},
           # chunk kernel + wall-cell kernel per step (every cavity has walls)
           "gpu_launches": 2 * steps}
    return rec, clk.summary()


def run_batch(args):
    import muphfasa_gb300 as m
    m.set_device(0)
    prec = args.precision  # every storage precision of the batch kernels
    rec, clocks = batch_measure(m, args.domains, args.steps, args.warmup, prec)
    line = {k: rec[k] for k in ("metric", "value", "unit")}
    line.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "ms_per_step": rec["ms_per_step"],
                 "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": rec["dtype"],
                 "data": "synthetic", "config": rec["config"], "roofline": rec["roofline"],
                 "looped_single_domain": rec["looped_single_domain"], "clocks": clocks,
                 "gpu_launches": rec["gpu_launches"]})
    print(json.dumps(line), flush=True)
    return 0


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=512, help="cells per side of the channel")
    ap.add_argument("--precision", default="f64x", choices=list(ELEM))
    ap.add_argument("--e2e-steps", type=int, default=5)
    ap.add_argument("--e2e-sweep", default="", help="comma-separated slab counts of the step_host pipeline to time")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--secondary-steps", type=int, default=40,
                    help="steps of the 512-cavity batch record added to the channel line (0: skip)")
    ap.add_argument("--domains", type=int, default=512, help="domains of the batch512 workload")
    ap.add_argument("--workload", default="channel", choices=["channel", "batch512", "tgv3d", "warmstart", "tgv2d", "ceiling",
                                                  "surrogate"],
                    help="channel: the D3Q19 channel (headline); batch512: 512 uneven D2Q9 cavities; "
                         "tgv3d: the D3Q27 precision study (use --n 384)")
    ap.add_argument("--tgv-steps", type=int, default=10000, help="tgv3d: total steps")
    ap.add_argument("--every", type=int, default=1000, help="tgv3d: steps between error samples")
    ap.add_argument("--ws-n", type=int, default=128, help="warmstart: cells per side")
    ap.add_argument("--ws-train", type=int, default=2000, help="warmstart: training cases")
    ap.add_argument("--ws-test", type=int, default=200, help="warmstart: held-out cases")
    ap.add_argument("--ws-draw", type=int, default=0,
                    help="warmstart: training cases drawn (default --ws-train); the first --ws-train that converge are kept")
    ap.add_argument("--ws-epochs", type=int, default=200)
    ap.add_argument("--ws-lr", type=float, default=2e-3)
    ap.add_argument("--ws-gen-steps", type=int, default=400000,
                    help="warmstart: step limit of the data generation (fields kept when converged to 1e-8)")
    ap.add_argument("--ws-max-steps", type=int, default=400000)
    ap.add_argument("--ws-curve", type=int, default=24, help="warmstart: held-out cases of the error-vs-steps curve")
    ap.add_argument("--ws-single", type=int, default=6, help="warmstart: cases timed on single handles")
    ap.add_argument("--ws-consistent", default="50,4",
                    help="warmstart: steps,rounds of the consistent start in the error-vs-steps curves")
    ap.add_argument("--tgv-ref", default="f64x", choices=["f64x", "f64", "f64_fast"],
                    help="tgv3d: reference precision (FP64 or the FP64-accurate fixed point)")
    args = ap.parse_args()
    if args.impl == "reference":
        return run_reference(args)
    if args.workload == "tgv3d":
        return run_tgv3d(args)
    if args.workload == "tgv2d":
        return run_tgv2d(args)
    if args.workload == "ceiling":
        return run_ceiling(args)
    if args.workload == "warmstart":
        return run_warmstart(args)
    if args.workload == "surrogate":
        return run_surrogate(args)
    if args.workload == "batch512":
        return run_batch(args)

    import muphfasa_gb300 as m
    from muphfasa_gb300 import replicas
    rank, world, local = replicas.rank_info()
    dist = replicas.init("nccl" if world > 1 else None)
    import torch
    if torch.cuda.is_available():
        torch.cuda.set_device(local)
    m.set_device(local)

    n = (args.n, args.n, args.n)
    q = 19
    cells = n[0] * n[1] * n[2]
    workload = f"channel_d3q19_{args.n}^3_{args.precision}"
    sim = m.Simulation(channel_desc(m, n, args.precision))
    rho, u = channel_fields(n, seed=20261203 + rank)
    sim.initialize(rho, u)
    del rho, u
    sim.advance(args.warmup)

    dev = torch.device("cuda", local) if torch.cuda.is_available() else "cpu"
    replicas.barrier(dist, dev)
    with ClockSampler(local) as clk:
        ms = sim.advance_timed(args.steps)  # CUDA events on the step kernels' stream
    ms_max = replicas.max_over_ranks(dist, ms, dev)
    total_cells = replicas.sum_over_ranks(dist, cells, dev)
    value = total_cells * args.steps / (ms_max / 1e3) / 1e6
    kernel_ms = ms / args.steps  # one step kernel per step
    alg_bytes = 2 * q * ELEM[args.precision] * cells  # per launch
    achieved = alg_bytes / (kernel_ms / 1e3) / 1e9
    peak, peak_kind = peaks()
    traffic = ncu_traffic(workload)

    # End to end through the C ABI with host buffers (pinned), every step:
    # upload f, one advance, download f.
    e2e = None
    if args.e2e_steps <= 0:
        e2e = {"value": None, "unit": "MLUPS", "skipped": "--e2e-steps 0"}
    try:
        if args.e2e_steps <= 0:
            raise StopIteration
        pinned = m.PinnedArray(q * cells)  # cudaHostAlloc'ed, not a pageable buffer
        f_host = pinned.array
        sim.f(out=f_host)
        sim.step_host(f_host, f_host, 1)  # warm-up of the path
        replicas.barrier(dist, dev)
        t0 = time.perf_counter()
        for _ in range(args.e2e_steps):
            sim.step_host(f_host, f_host, 1)
        dt = time.perf_counter() - t0
        dt = replicas.max_over_ranks(dist, dt, dev)
        e2e = {"value": round(total_cells * args.e2e_steps / dt / 1e6, 3), "unit": "MLUPS",
               "h2d_bytes_per_step": q * cells * 8, "d2h_bytes_per_step": q * cells * 8,
               "steps": args.e2e_steps, "host_buffers": "pinned (cudaHostAlloc)", "api": "mph_step_host"}
        if args.e2e_sweep and rank == 0:
            # Slab count of the host-copy pipeline (0: one block copy each
            # way), three interleaved rounds: the host link is shared.
            sweep = {}
            for _ in range(3):
                for S in args.e2e_sweep.split(","):
                    os.environ["MPH_STEP_HOST_SLABS"] = S
                    sim.step_host(f_host, f_host, 1)
                    t0 = time.perf_counter()
                    for _ in range(args.e2e_steps):
                        sim.step_host(f_host, f_host, 1)
                    sweep.setdefault(S, []).append(round(cells * args.e2e_steps / (time.perf_counter() - t0) / 1e6, 1))
            os.environ.pop("MPH_STEP_HOST_SLABS", None)
            e2e["slab_sweep_mlups"] = sweep
        del f_host
        pinned.close()
    except StopIteration:
        pass
    except Exception as ex:  # report, do not hide
        e2e = {"value": None, "unit": "MLUPS", "error": str(ex)[:200]}

    # Secondary record: the 512-cavity batch (FP32, 40 steps), timed in the
    # same run so its roofline fraction travels with the headline line.
    secondary = None
    if rank == 0 and args.secondary_steps > 0:
        try:
            rec, bclk = batch_measure(m, 512, args.secondary_steps, 4, "f32", device=local)
            rec["clocks"] = bclk
            secondary = {"batch512": rec}
        except Exception as ex:  # report, do not hide
            secondary = {"batch512": {"error": str(ex)[:200]}}
        # the warm-start surrogate's training throughput (128^2, batch 8)
        try:
            its = 50
            dt, _, nparams, sclk = surrogate_measure(128, its, 3)
            secondary["surrogate_train"] = {"metric": "U-Net training iterations per second (128^2, batch 8)",
                                            "value": round(its / dt, 2), "unit": "iterations/s",
                                            "ms_per_step": round(1e3 * dt / its, 3), "steps": its, "params": nparams,
                                            "clocks": sclk}
        except Exception as ex:
            secondary["surrogate_train"] = {"error": str(ex)[:200]}

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        sn = (256, 256, 256)
        kind = cpu_kind()
        v, dt = cpu_reference(sn, 20 if kind == "port" else 10, 1, threads, kind)
        v1, dt1 = cpu_reference((128, 128, 128), 4, 1, 1, kind)
        vp, dtp = cpu_reference(sn, 10, 1, threads, "port")
        cpu = {"value": round(v, 3), "unit": "MLUPS", "cores": threads, "kind": kind,
               "sample": f"{sn[0]}^3 domain of the workload, {20 if kind == 'port' else 10} steps after 1 warm-up, "
                         f"FP64, OpenMP {threads} threads ({dt:.2f} s)"
                         + ("; the reference's own src/LBM code" if kind == "reference" else ""),
               "single_thread": {"value": round(v1, 3), "sample": f"128^3, 4 steps, 1 thread ({dt1:.2f} s)"},
               "port": {"value": round(vp, 3), "sample": f"the restatement, {sn[0]}^3, 10 steps, {threads} threads "
                                                          f"({dtp:.2f} s)"},
               "host": cpu_model()}

    if rank == 0:
        line = {
            "metric": METRIC, "value": round(value, 3), "unit": "MLUPS", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 4), "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": DTYPE[args.precision], "data": "synthetic",
            "config": {"workload": workload, "lattice": "D3Q19", "grid": list(n), "tau": 0.6, "force": 1e-6,
                       "walls": "NoSlip at y=0 and y=Ny; periodic x, z", "precision": args.precision,
                       "init": "rho = 1 + U(-1e-4, 1e-4) seeded, u = 0",
                       "l2": "inputs larger than L2 (no flush needed)", "parallelism": f"replicas x{world}"},
            "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                         "frac": round(achieved / peak, 4), "traffic": traffic,
                         "peak_kind": peak_kind, "bytes_per_cell_update": 2 * q * ELEM[args.precision]},
            "e2e": e2e,
            "cpu_baseline": cpu,
            "clocks": clk.summary(),
            "gpu_launches": args.steps * sim.launches_per_step(),
            "secondary": secondary,
        }
        print(json.dumps(line), flush=True)
    sim.close()
    if dist is not None:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
