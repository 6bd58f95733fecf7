#!/usr/bin/env python3
"""Throughput benchmark of the superMC initial-condition path on GB300.

Workload: MC-KLN Pb+Pb at 2.76 TeV, A=B=208,
Woods-Saxon R=6.62 fm, a=0.546 fm, sigma_NN=64 mb, b^2 uniform on
[0,400] fm^2, 261x261 grid at dx=0.1 fm, saturation exponent 0.288;
eccentricities eps_2..eps_5.  One step = one batch of events generated
from Philox streams (sampling, pairing, thickness, per-cell KLN dN/dy,
eccentricities) -- the event loop of MakeDensity::generateEccTable.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]

Prints one JSON line (rank 0).  The GPU arm runs the batched path through
the C ABI; `value` keeps outputs in HBM, `e2e` copies every step's results
to pinned host memory inside the timed region.  The reference arm times the
reference algorithm's CPU restatement (the oracle port) on all host cores.
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

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)

EVENTS_PER_STEP = 10000
WORKLOAD = {
    "which_mc_model": 1, "sub_model": 7, "lambda": 0.288,
    "aproj": 208, "atarg": 208, "proj_r": 6.62, "proj_a": 0.546, "targ_r": 6.62, "targ_a": 0.546,
    "sigininn_override": 64.0, "ecm": 2760.0,
    "shape_of_nucleons": 4, "gauss_nucl_width": 0.5, "collision_criterion": 1, "shape_of_entropy": 2,
    "quark_width": 0.3, "alpha": 0.118, "bmin": 0.0, "bmax": 20.0, "npmin": 2, "npmax": 500,
    "maxx": 13.0, "maxy": 13.0, "dx": 0.1, "dy": 0.1, "finalfactor": 40.0, "tmax": 71, "tmax_subdivision": 3,
    "ecc_from_order": 2, "ecc_to_order": 5, "cc_fluctuation_model": 0,
}
WORKLOAD_NAME = "MC-KLN Pb+Pb 208+208, R=6.62 a=0.546, sigma_NN=64 mb, b^2~U[0,400], 261x261 dx=0.1, eps_2..eps_5"
METRIC = "events/s Pb+Pb 261^2 grid: batched split-prec vs plain GPU at matched epsilon_n error"


def peaks():
    try:
        with open(os.path.join(HERE, "MEASURED_PEAKS.json")) as f:
            m = json.load(f)
        return m["hbm_gbs"], m["bf16_tflops"], "measured"
    except Exception:
        return 6800.0, 1900.0, "fallback"


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi sampling of SM clocks and throttle reasons during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ------------------------------------------------------------------ oracle side
def oracle_params_for(vals: dict, kln_table=None):
    """smco_params of the workload (uses the library's constants formulae)."""
    import ctypes
    from oracle.oracle import Oracle, Params, _ptr
    from supermc_gb300.params import derive
    d = derive(vals)
    orc = Oracle()
    p = Params(nx=d.nx, ny=d.ny, xmax=vals["maxx"], ymax=vals["maxy"], dx=vals["dx"], dy=vals["dy"],
               width=d.width, quark_width=vals["quark_width"], dsq=d.dsq, sigin=d.sigin,
               sigma_gg=orc.lib.smco_sigeff(d.sigin, d.width), alpha=vals["alpha"],
               which_mc_model=int(vals["which_mc_model"]), sub_model=int(vals["sub_model"]),
               shape_of_nucleons=int(vals["shape_of_nucleons"]), shape_of_entropy=int(vals["shape_of_entropy"]),
               collision_criterion=int(vals["collision_criterion"]), final_factor=vals["finalfactor"],
               npmin=int(vals["npmin"]), npmax=int(vals["npmax"]))
    keep = None
    if kln_table is not None:
        import numpy as np
        keep = np.ascontiguousarray(kln_table, dtype=np.float64)
        p.kln_table = _ptr(keep)
        p.kln_tmax = keep.shape[0]
        p.kln_dT = 10.0 / d.sigin / int(vals["tmax_subdivision"])
    nuc = orc.nucleus(int(vals["aproj"]), 0, vals["proj_r"], vals["proj_a"], 0.0)
    return orc, p, nuc, keep


def _oracle_worker(args):
    """Runs the oracle's op-9 loop for one slice (process-pool worker)."""
    import ctypes
    import numpy as np
    vals, table, nev, seed = args
    orc, p, nuc, keep = oracle_params_for(vals, table)
    from oracle.oracle import _ptr
    out = np.zeros((nev, 49))
    t0 = time.perf_counter()
    rc = orc.lib.smco_run_ecc_table(ctypes.byref(p), ctypes.byref(nuc), ctypes.byref(nuc), vals["bmin"],
                                    vals["bmax"], nev, int(vals["ecc_from_order"]), int(vals["ecc_to_order"]),
                                    seed, 0, 0, _ptr(out))
    dt = time.perf_counter() - t0
    if rc < 0:
        raise RuntimeError(f"oracle loop failed: {rc}")
    return nev, dt


def oracle_kln_table(vals: dict, procs: int):
    """The MC-KLN dN/dy table by the oracle's FP64 quadrature, on CPU."""
    from oracle.oracle import kln_table
    from supermc_gb300.params import derive
    d = derive(vals)
    sub = int(vals["tmax_subdivision"])
    tmax = sub * (int(vals["tmax"]) - 1) + 1
    dT = 10.0 / d.sigin / sub
    rule = (int(vals["kln_npt"]), int(vals["kln_nkt"]), int(vals["kln_nphi"]))
    return kln_table(vals["ecm"], vals["lambda"], dT, tmax, rule, procs)


def run_reference(args, vals) -> dict:
    """Reference arm: the oracle port on all host cores."""
    import multiprocessing as mp
    from oracle.oracle import build_oracle
    build_oracle()
    procs = max(1, os.cpu_count() or 1)
    t_tab = time.perf_counter()
    table = oracle_kln_table(vals, procs) if int(vals["which_mc_model"]) == 1 else None
    t_tab = time.perf_counter() - t_tab
    per_proc = max(1, args.ref_events // procs)
    ctx = mp.get_context("spawn")
    rates = []
    with ctx.Pool(procs) as pool:
        for step in range(args.warmup + args.steps):
            t0 = time.perf_counter()
            res = pool.map(_oracle_worker, [(vals, table, per_proc, 1000 * step + k + 1) for k in range(procs)])
            dt = time.perf_counter() - t0
            if step >= args.warmup:
                rates.append(sum(r[0] for r in res) / dt)
    value = statistics.median(rates)
    ms = per_proc * procs / value * 1e3
    return {"metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (Monte-Carlo events, drand48 streams)",
            "config": {"workload": WORKLOAD_NAME, "events_per_step": per_proc * procs,
                       "parallelism": f"{procs} host processes"},
            "impl": "reference",
            "cpu_baseline": {"value": value, "unit": "events/s", "cores": procs, "kind": "port",
                             "sample": f"{per_proc} events per process x {procs} processes per step; "
                                       f"dN/dy table built once by the FP64 quadrature ({t_tab:.0f} s, untimed)",
                             "note": "the oracle's C restatement of the reference's op-9 loop (the reference's "
                                     "own binary is not built on this aarch64 host); on x86 the port takes "
                                     "about 1.4x the reference binary's time per event"},
            "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def cpu_baseline(vals, table, target_s: float = 12.0) -> dict:
    """The oracle port on one host core, bounded sample of the workload."""
    n = 64
    nev, dt = _oracle_worker((vals, table, n, 99))
    n2 = max(n, int(n * target_s / max(dt, 1e-3)))
    n2 = min(n2, 4000)
    nev, dt = _oracle_worker((vals, table, n2, 7))
    return {"value": nev / dt, "unit": "events/s", "cores": 1, "kind": "port",
            "note": "the oracle's C restatement of the reference's op-9 loop; on x86 it takes about 1.4x the "
                    "reference binary's time per event",
            "sample": f"{nev} events of the workload on one core ({dt:.1f} s), oracle op-9 loop with the "
                      "same dN/dy table"}


def eps_error(eng, vals, table, n: int = 256) -> float:
    """max |eps_n(GPU) - eps_n(FP64 oracle)|, n = 2..5, on generated events of
    the workload re-run through the oracle (with its own FP64 dN/dy table)
    from the GPU's own nucleon positions."""
    import numpy as np
    orc, p, nuc, keep = oracle_params_for(vals, table)
    ev = orc.event(p)
    g = eng.generate(10 ** 9, n, want=("ecc", "b", "positions"))
    A = eng.A
    worst = 0.0
    for k in range(n):
        ev.inject(g["positions"][k, :A], g["positions"][k, A:])
        ev.pair()
        if ev.thickness() or ev.density():
            continue
        ref = ev.eccentricities(2, 5, g["b"][k])
        for order in range(2, 6):
            for c in range(4):
                col = 5 * (order - 1) + c
                worst = max(worst, abs(ref[col] - g["ecc"][k, col]))
    return worst


# ------------------------------------------------------------------ mixed batch
MIXED_BASE = {
    "which_mc_model": 5, "sub_model": 1, "shape_of_nucleons": 4, "gauss_nucl_width": 0.5,
    "collision_criterion": 1, "shape_of_entropy": 2, "quark_width": 0.3, "alpha": 0.118, "bmin": 0.0,
    "bmax": 20.0, "npmin": 2, "npmax": 600, "maxx": 13.0, "maxy": 13.0, "dx": 0.1, "dy": 0.1,
    "finalfactor": 40.0, "ecc_from_order": 2, "ecc_to_order": 5, "cc_fluctuation_model": 0,
}
MIXED_SYSTEMS = [   # (share, parameters): p+Pb, d+Au, Cu+Cu, deformed U+U, Au+Au
    (1, {"aproj": 1, "atarg": 208, "ecm": 5020.0}),
    (2, {"aproj": 2, "atarg": 197, "ecm": 200.0}),
    (2, {"aproj": 63, "atarg": 63, "ecm": 200.0, "proj_r": 4.2, "proj_a": 0.596, "targ_r": 4.2, "targ_a": 0.596}),
    (2, {"aproj": 238, "atarg": 238, "ecm": 200.0, "proj_deformed": 1, "targ_deformed": 1, "proj_r": 6.81,
         "proj_a": 0.55, "targ_r": 6.81, "targ_a": 0.55}),
    (3, {"aproj": 197, "atarg": 197, "ecm": 200.0, "proj_r": 6.38, "proj_a": 0.535, "targ_r": 6.38,
         "targ_a": 0.535, "proj_d_min": 0.4, "targ_d_min": 0.4, "sigininn_override": 42.0}),
]


def mixed_batch(dev, stream, n: int) -> dict:
    """events/s of one mixed-system batch of n events (shares 1:2:2:2:3), as
    one CUDA graph (smc_generate_mixed_graph: captured by a first call, then
    replayed), events in HBM; the eager batch beside it."""
    import numpy as np
    import torch
    from supermc_gb300.engine import Engine
    eng = Engine(dict(MIXED_BASE, **MIXED_SYSTEMS[-1][1]), seed=2)
    eng.set_stream(stream.cuda_stream)
    tuning = eng.autotune(4096)   # on the Au+Au system, before timing
    shares = np.array([s for s, _ in MIXED_SYSTEMS], dtype=float)
    counts = np.floor(n * shares / shares.sum()).astype(int)
    counts[-1] += n - counts.sum()
    sel = np.random.default_rng(5).permutation(np.repeat(np.arange(len(counts)), counts)).astype(np.int32)
    systems = [p for _, p in MIXED_SYSTEMS]
    bufs = {"ecc": torch.empty((n, 49), dtype=torch.float64, device=dev),
            "npart": torch.empty((n, 2), dtype=torch.int32, device=dev)}
    def timed(first, graph):
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.generate_mixed(systems, sel, first_event=first, device_bufs=bufs, graph=graph)
        b.record(stream)
        torch.cuda.synchronize()
        return n / (a.elapsed_time(b) / 1e3)
    eng.generate_mixed(systems, sel, first_event=0, device_bufs=bufs, graph=True)   # eager + capture
    torch.cuda.synchronize()
    rates = [timed(n * (k + 1), True) for k in range(3)]
    eager = timed(n * 5, False)
    eng.close()
    return {"value": statistics.median(rates), "unit": "events/s", "events": n,
            "counts": counts.tolist(),
            "systems": "p+Pb 5.02 TeV, d+Au, Cu+Cu, deformed U+U, Au+Au (200 GeV) in shares 1:2:2:2:3, "
                       "MC-Glauber 261x261",
            "launch": "one CUDA graph per batch (smc_generate_mixed_graph), median of 3 replays",
            "eager_value": eager,
            "splat": "tensor cores" if tuning["tensor_cores"] else "CUDA cores", "chunk": tuning["chunk"]}


# differentiable Pb+Pb Glauber (radii by inverse CDF, so that positions move
# with R and a): 4096 events at seed 7, w = 0.5 fm, alpha = 0.118
DIFF_PARAMS = {
    "which_mc_model": 5, "sub_model": 1, "aproj": 208, "atarg": 208, "proj_r": 6.62, "proj_a": 0.546,
    "targ_r": 6.62, "targ_a": 0.546, "sigininn_override": 64.0, "ecm": 2760.0, "shape_of_nucleons": 4,
    "gauss_nucl_width": 0.5, "collision_criterion": 1, "shape_of_entropy": 2, "quark_width": 0.3, "alpha": 0.118,
    "bmin": 0.0, "bmax": 20.0, "npmin": 2, "npmax": 500, "maxx": 13.0, "maxy": 13.0, "dx": 0.1, "dy": 0.1,
    "finalfactor": 40.0, "ecc_from_order": 2, "ecc_to_order": 3, "cc_fluctuation_model": 0, "ws_inverse_cdf": 1,
}


def differentiable_batch(stream, n: int = 4096) -> dict:
    """Forward (smc_generate) and backward (smc_adjoint: forward recomputed,
    then the adjoint kernel) of <|eps_2|> over n events; rates in events/s."""
    import numpy as np
    import torch
    from supermc_gb300.engine import Engine
    eng = Engine(dict(DIFF_PARAMS), seed=7)
    eng.set_stream(stream.cuda_stream)
    tuning = eng.autotune(n)
    g = np.zeros((n, 2))
    g[:, 0] = 1.0 / n
    eng.generate(0, n, want=("ecc",))
    eng.adjoint(0, n, g_eps=g)
    torch.cuda.synchronize()

    def timed(fn):   # CUDA events on the engine's stream around one call, median of 3
        out = []
        for _ in range(3):
            a = torch.cuda.Event(enable_timing=True)
            b = torch.cuda.Event(enable_timing=True)
            a.record(stream)
            r = fn()
            b.record(stream)
            torch.cuda.synchronize()
            out.append(a.elapsed_time(b) / 1e3)
        return statistics.median(out), r
    t_fwd, _ = timed(lambda: eng.generate(0, n, want=("ecc",)))
    eng.reset_stats()
    eng.set_timing(True)
    t_fb, (grad, _) = timed(lambda: eng.adjoint(0, n, g_eps=g))
    st = eng.stats()
    eng.close()
    return {"forward": n / t_fwd, "forward_backward": n / t_fb, "unit": "events/s", "events": n,
            "timing": "CUDA events on the engine's stream around one call (host copies of the results "
                      "included), median of 3",
            "adjoint_kernel_ms": st["post_ms"] / 3, "grad_mean_eps2": {"w": grad[0], "alpha": grad[1],
                                                                      "R": grad[2], "a": grad[3]},
            "workload": "Pb+Pb 2.76 TeV, sigma_NN=64 mb, radii by inverse CDF, w=0.5 fm, alpha=0.118, 261x261",
            "splat": "tensor cores" if tuning["tensor_cores"] else "CUDA cores", "chunk": tuning["chunk"]}


AVG_BASE = {
    "which_mc_model": 5, "sub_model": 1, "shape_of_nucleons": 4, "gauss_nucl_width": 0.5, "collision_criterion": 1,
    "shape_of_entropy": 2, "quark_width": 0.3, "alpha": 0.118, "bmin": 0.0, "bmax": 20.0, "npmin": 2,
    "npmax": 500, "maxx": 12.5, "maxy": 12.5, "dx": 0.05, "dy": 0.05, "finalfactor": 40.0, "ecc_from_order": 2,
    "ecc_to_order": 2, "cc_fluctuation_model": 0,
}
AVG_SYSTEMS = {
    "Pb+Pb": ({"aproj": 208, "atarg": 208, "proj_r": 6.62, "proj_a": 0.546, "targ_r": 6.62, "targ_a": 0.546,
               "sigininn_override": 64.0, "ecm": 2760.0}, [2, 20, 40, 60, 80, 100, 150, 200, 250, 300, 417]),
    "O+O": ({"aproj": 16, "atarg": 16, "proj_r": 2.608, "proj_a": 0.513, "targ_r": 2.608, "targ_a": 0.513,
             "sigininn_override": 68.0, "ecm": 7000.0}, [2, 4, 6, 8, 10, 12, 14, 16, 20, 25, 33]),
}


def binned_average(stream, n: int) -> dict:
    """Npart-binned averages on the 501x501 grid (recentred, rotated to the
    second-order plane by bilinear resampling): events/s per system and the
    HBM roofline of the binned resampling kernel."""
    import torch
    from supermc_gb300.engine import Engine
    hbm_peak, _, peak_kind = peaks()
    out = {}
    for name, (sysp, edges) in AVG_SYSTEMS.items():
        eng = Engine(dict(AVG_BASE, **sysp), seed=3)
        eng.set_stream(stream.cuda_stream)
        tuning = eng.autotune(4096)
        eng.average_binned(0, min(n, 4096), edges, order=2, method=1)
        torch.cuda.synchronize()
        eng.reset_stats()
        eng.set_timing(True)
        t0 = time.perf_counter()
        _, counts = eng.average_binned(4096, n, edges, order=2, method=1)
        dt = time.perf_counter() - t0
        st = eng.stats()
        cells = eng.nx * eng.ny
        bytes_ev = 4.0 * cells   # one FP32 density read per event (bin sums stay on chip per chunk)
        achieved = bytes_ev * n / (st["post_ms"] / 1e3) / 1e9 if st["post_ms"] > 0 else None
        out[name] = {"value": n / dt, "unit": "events/s", "events": n, "counts": counts.tolist(),
                     "splat": "tensor cores" if tuning["tensor_cores"] else "CUDA cores", "chunk": tuning["chunk"],
                     "sample_ms": st["sample_ms"], "splat_ms": st["grid_ms"], "binned_ms": st["post_ms"],
                     "binned_roofline": {"bound": "hbm", "achieved": achieved, "peak": hbm_peak, "unit": "GB/s",
                                         "frac": achieved / hbm_peak if achieved else None,
                                         "work": "4*Nx*Ny bytes per event (its density, read once)",
                                         "peak_kind": peak_kind}}
        eng.close()
    return out


def grid_output_leg(eng, n: int) -> dict:
    """Operation 1 (MakeDensity::generate_profile_ebe, src/MakeDensity.cpp:
    574-694): every event's density grid and eccentricities copied to pinned
    host memory inside the call (smc_generate with host outputs)."""
    import ctypes
    import torch
    from supermc_gb300 import _lib
    hb = {"ecc": torch.empty((n, 49), dtype=torch.float64, pin_memory=True),
          "rho": torch.empty((n, eng.nx, eng.ny), dtype=torch.float32, pin_memory=True)}
    hnp = {k: v.numpy() for k, v in hb.items()}

    def step(first):
        o = eng._outputs(hnp, False)
        _lib.check(eng.lib.smc_generate(eng.h, first, n, ctypes.byref(o)), "smc_generate")
    step(10 ** 9)
    times = []
    for k in range(3):
        t0 = time.perf_counter()
        step(10 ** 9 + (k + 1) * n)
        times.append(time.perf_counter() - t0)
    dt = statistics.median(times)
    bytes_ev = 4 * eng.nx * eng.ny
    return {"value": n / dt, "unit": "events/s", "events": n, "density_bytes_per_event": bytes_ev,
            "density_GB_per_s": bytes_ev * n / dt / 1e9,
            "note": "smc_generate with pinned host outputs (FP32 density + eps line per event), "
                    "wall clock per call, median of 3"}


# ------------------------------------------------------------------ GPU arm
def run_gpu(args, vals) -> dict | None:
    import numpy as np
    import torch
    import torch.distributed as dist
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    from supermc_gb300.engine import Engine
    n = args.events
    t0 = time.perf_counter()
    eng = Engine({k: v for k, v in vals.items()}, seed=args.seed)
    t_init = time.perf_counter() - t0
    stream = torch.cuda.current_stream()
    eng.set_stream(stream.cuda_stream)
    dev = torch.device("cuda", local)
    # launch configuration (splat path, events per launch) tuned on this
    # workload before timing, like the context's construction
    tuning = eng.autotune(n) if args.autotune else None
    if not args.autotune and args.grid_path != "auto":
        eng.set_grid_path(args.grid_path == "tc")
        tuning = {"tensor_cores": args.grid_path == "tc", "chunk": 4096, "events_per_s": None}
    bufs = {"ecc": torch.empty((n, 49), dtype=torch.float64, device=dev),
            "npart": torch.empty((n, 2), dtype=torch.int32, device=dev),
            "ncoll": torch.empty((n,), dtype=torch.int32, device=dev),
            "b": torch.empty((n,), dtype=torch.float64, device=dev)}
    flush = torch.empty(int(256e6) // 4, dtype=torch.float32, device=dev)   # > L2 (129 MB)

    from supermc_gb300.distributed import step_events

    def first_event(step):   # disjoint event-id blocks per rank (no collective on the data path)
        return step_events(step, rank, world, n)

    # ---- device-resident value: the batch as one CUDA graph (captured by the
    # first warm-up step, replayed with new event ids)
    gen = eng.generate_graph_into if args.graph else eng.generate_into
    for s in range(args.warmup):
        gen(first_event(s), n, bufs)
    torch.cuda.synchronize()
    eng.reset_stats()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(args.steps)]
    clocks = ClockSampler(local)
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    clocks.start()
    for s in range(args.steps):
        flush.fill_(float(s))            # evict L2 between timed steps (outside the events)
        starts[s].record(stream)
        gen(first_event(args.warmup + s), n, bufs)
        ends[s].record(stream)
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    clk = clocks.stop()
    step_ms = [a.elapsed_time(b) for a, b in zip(starts, ends)]
    launches = eng.stats()["launches"]
    # per-kernel durations of the same batch, launched eagerly with CUDA
    # events around every kernel (a graph replay records none)
    eng.reset_stats()
    eng.set_timing(True)
    flush.fill_(0.5)
    eng.generate_into(first_event(args.warmup + args.steps), n, bufs)
    torch.cuda.synchronize()
    st = eng.stats()
    eng.set_timing(False)
    tot_ms = sum(step_ms)
    if world > 1:
        t = torch.tensor([tot_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        tot_ms = t.item()
    value = n * args.steps * world / (tot_ms / 1e3)

    # ---- end to end: same call with host (pinned) output buffers
    hb = {k: torch.empty(v.shape, dtype=v.dtype, pin_memory=True) for k, v in bufs.items()}
    hnp = {k: v.numpy() for k, v in hb.items()}
    from supermc_gb300 import _lib
    import ctypes

    def host_step(first):
        o = eng._outputs(hnp, False)
        _lib.check(eng.lib.smc_generate(eng.h, first, n, ctypes.byref(o)), "smc_generate")

    host_step(first_event(10 ** 6))
    torch.cuda.synchronize()
    if world > 1:
        dist.barrier()
    t0 = time.perf_counter()
    e_starts = torch.cuda.Event(enable_timing=True)
    e_ends = torch.cuda.Event(enable_timing=True)
    e_starts.record(stream)
    for s in range(args.steps):
        host_step(first_event(10 ** 6 + 1 + s))
    e_ends.record(stream)
    torch.cuda.synchronize()
    e2e_ms = e_starts.elapsed_time(e_ends)
    if world > 1:
        t = torch.tensor([e2e_ms], device=dev)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        e2e_ms = t.item()
    e2e = n * args.steps * world / (e2e_ms / 1e3)
    d2h = sum(v.numel() * v.element_size() for v in bufs.values())

    if rank != 0:
        if world > 1:
            dist.barrier()
            dist.destroy_process_group()
        return None

    # ---- the batched path with each splat (eager launches)
    paths = {}
    for tc in (True, False):
        eng.set_grid_path(tc)
        eng.generate_into(10 ** 8, n, bufs)
        torch.cuda.synchronize()
        a = torch.cuda.Event(enable_timing=True)
        b = torch.cuda.Event(enable_timing=True)
        a.record(stream)
        eng.generate_into(10 ** 8 + n, n, bufs)
        b.record(stream)
        torch.cuda.synchronize()
        paths[tc] = n / (a.elapsed_time(b) / 1e3)
    eng.set_grid_path(tuning["tensor_cores"] if tuning else True)

    # ---- mixed-system batch (p+Pb, d+Au, Cu+Cu, deformed U+U, Au+Au in the
    # proportions 1:2:2:2:3, MC-Glauber), one smc_generate_mixed call
    mixed = mixed_batch(dev, stream, args.mixed_events)
    diff = differentiable_batch(stream) if args.side_workloads else None
    grids = grid_output_leg(eng, args.grid_events) if args.side_workloads else None
    binned = binned_average(stream, args.binned_events) if args.side_workloads else None

    # ---- plain per-event path, same workload (sample)
    m = args.plain_events
    pb = {k: v[:m] for k, v in bufs.items()}
    eng.generate_into(10 ** 7, 16, pb, plain=True)
    torch.cuda.synchronize()
    a = torch.cuda.Event(enable_timing=True)
    b = torch.cuda.Event(enable_timing=True)
    a.record(stream)
    eng.generate_into(10 ** 7 + 100, m, pb, plain=True)
    b.record(stream)
    torch.cuda.synchronize()
    plain = m / (a.elapsed_time(b) / 1e3)

    # ---- roofline of the dominant kernel (the thickness/density splat)
    hbm_peak, tf_peak, peak_kind = peaks()
    from supermc_gb300.params import derive
    npart = bufs["npart"].cpu().numpy()
    nsrc = float(npart.sum(axis=1).mean())     # MC-KLN: T_A, T_B sources are the participants
    flops_per_event = 2.0 * eng.nx * eng.ny * nsrc
    grid_launch_ms = st["grid_ms"] / max(1, st["grid_launches"])
    events_per_launch = n / max(1, st["grid_launches"])
    achieved = flops_per_event * events_per_launch / (grid_launch_ms / 1e3) / 1e12
    tc_used = tuning["tensor_cores"] if tuning else True
    roof = {"bound": "tensor", "achieved": achieved, "peak": tf_peak, "unit": "TFLOP/s",
            "frac": achieved / tf_peak, "traffic": None,
            "kernel": ("k_grid_tc (tcgen05 split-TF32 thickness contraction, KLN lookup, eps_n)" if tc_used else
                       "k_grid (CUDA-core thickness splat, KLN lookup, eps_n)"),
            "work": "2*Nx*Ny*N_src FLOP per event (dense separable contraction), N_src = Npart",
            "peak_kind": f"bf16 dense, {peak_kind}",
            "sample_kernel_ms_per_launch": st["sample_ms"] / max(1, st["sample_launches"]),
            "grid_kernel_ms_per_launch": grid_launch_ms}
    # the work a splat must do: each thickness source adds to the cells within
    # its cut (r <= 5w: pi (5w)^2 / (dx dy) cells), one multiply-add each
    d = derive(vals)
    disk_cells = math.pi * (5 * d.width) ** 2 / (vals["dx"] * vals["dy"])
    useful = nsrc * disk_cells
    roof["useful"] = {"fma_per_event": useful, "tflops": 2 * useful * events_per_launch / (grid_launch_ms / 1e3) / 1e12,
                      "work": "N_src x cells within r <= 5w, one FMA each (the splat's own work; the dense count "
                              "above also spans the cells outside the cut)"}
    try:
        with open(os.path.join(HERE, "profiles", "traffic.json")) as f:
            tr = json.load(f)
        key = "k_grid_tc_bytes_per_event" if tc_used else "k_grid_cc_bytes_per_event"
        if key in tr:
            roof["traffic"] = tr[key] * events_per_launch
        ikey = "k_grid_tc_warp_inst_per_event" if tc_used else "k_grid_cc_warp_inst_per_event"
        if ikey in tr:
            # instruction issue: 4 schedulers per SM, one warp instruction each per clock
            sms = torch.cuda.get_device_properties(dev).multi_processor_count
            mhz = clk.get("sm_mhz") or 2070.0
            peak_inst = sms * 4 * mhz * 1e6
            inst = tr[ikey] * events_per_launch / (grid_launch_ms / 1e3)
            roof["issue"] = {"bound": "issue", "achieved": inst / 1e9, "peak": peak_inst / 1e9,
                             "unit": "G warp instructions/s", "frac": inst / peak_inst,
                             "warp_inst_per_event": tr[ikey],
                             "source": "instructions per event from one ncu capture (profiles/)"}
    except Exception:
        pass

    t_tab = time.perf_counter()
    otab = (oracle_kln_table(vals, max(1, os.cpu_count() or 1)) if int(vals["which_mc_model"]) == 1
            else None)
    t_tab = time.perf_counter() - t_tab
    base = cpu_baseline(vals, otab, args.cpu_seconds) if args.cpu_seconds > 0 else None
    err = eps_error(eng, vals, otab)
    line = {"metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": tot_ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None,
            "dtype": "f32 splat, dN/dy lookup and moments (double-float moment sums); f64 pairing, "
                     "centre-of-mass shift, dN/dy table and the table cells FP32 leaves undecided",
            "data": "synthetic (Monte-Carlo events from Philox streams)",
            "config": {"workload": WORKLOAD_NAME, "events_per_step": n, "grid": [eng.nx, eng.ny],
                       "parallelism": f"event data parallel, {world} GPU(s)",
                       "l2": "256 MB buffer written between timed steps",
                       "launch": ("one CUDA graph per step (smc_generate_graph)" if args.graph else
                                  "eager launches (smc_generate)"),
                       "tuning": tuning},
            "e2e": {"value": e2e, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": d2h,
                    "note": "smc_generate with pinned host output buffers; per-step input is the event range"},
            "gpu_launches": int(launches),
            "clocks": clk, "roofline": roof, "cpu_baseline": base,
            "plain_gpu": {"value": plain, "unit": "events/s", "events": m,
                          "batched_over_plain": value / plain},
            "mixed_batch": mixed,
            "differentiable": diff,
            "grid_output_op1": grids,
            "binned_average_501": binned,
            "batched_by_splat_path": {"tensor_cores": paths[True], "cuda_cores": paths[False], "unit": "events/s",
                                      "events": n, "note": "eager smc_generate with each splat (smc_set_grid_path)"},
            "eps_abs_err_vs_fp64_oracle": err,
            "eps_check": "256 generated events, oracle with its own FP64 dN/dy table "
                         f"(built on {os.cpu_count()} host cores in {t_tab:.0f} s)",
            "init_s": t_init}
    print(json.dumps(line), flush=True)
    if world > 1:
        dist.barrier()
        dist.destroy_process_group()
    return line


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--events", type=int, default=EVENTS_PER_STEP)
    ap.add_argument("--plain-events", type=int, default=200)
    ap.add_argument("--mixed-events", type=int, default=100000)
    ap.add_argument("--binned-events", type=int, default=1000000, help="per system (Pb+Pb and O+O)")
    ap.add_argument("--grid-events", type=int, default=4096, help="operation-1 leg: events per call")
    ap.add_argument("--side-workloads", type=int, default=1, help="differentiable and 501^2 binned workloads")
    ap.add_argument("--graph", type=int, default=1, help="time the batch as a CUDA graph (smc_generate_graph)")
    ap.add_argument("--autotune", type=int, default=1, help="tune the launch configuration before timing")
    ap.add_argument("--grid-path", default="auto", choices=["auto", "tc", "cc"],
                    help="with --autotune 0: the splat (tensor-core or CUDA-core)")
    ap.add_argument("--ref-events", type=int, default=EVENTS_PER_STEP,
                    help="reference arm: events per step (all cores)")
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--seed", type=int, default=1)
    args = ap.parse_args()
    from supermc_gb300.params import read_parameters
    vals = read_parameters(None, [f"{k}={v}" for k, v in WORKLOAD.items()])
    if args.impl == "reference":
        if int(os.environ.get("RANK", "0")) != 0:
            return
        print(json.dumps(run_reference(args, vals)), flush=True)
        return
    if args.warmup < 3:
        args.warmup = 3
    run_gpu(args, vals)


if __name__ == "__main__":
    main()
