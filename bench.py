#!/usr/bin/env python3
"""Benchmark of the synthesis hot path on the full-optical workload.

One step = one complete synthesis (reference-wavelength lines, hydrogen lines, 300,000 metal
lines, continuum-only and full radiative transfer) of a 56-layer atmosphere on a 700,001-point
grid (3000-10000 A at 0.01 A), mixed precision, inputs resident in HBM.  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the FP64 CPU restatement of the reference (the oracle, all host cores)
on a bounded sample of the same workload.
"""
import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))

METRIC = "spectra/s & line-layer-lambda evals/s, mixed vs plain FP64 at 1e-4 flux err"
FLOP_PER_EVAL = 24  # FP32 flop per Voigt evaluation (Harris branch, FMA = 2)
# bounded sample of the workload for the CPU baseline: 20 windows of 70 A spread evenly over
# 3000-10000 A (20% of the grid)
CPU_SAMPLE = [(3140.0 + 350.0 * k, 3210.0 + 350.0 * k) for k in range(20)]


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="korg", choices=["korg", "reference"])
    ap.add_argument("--lines", type=int, default=300_000)
    ap.add_argument("--wl", type=float, nargs=2, default=[3000.0, 10000.0],
                    help="wavelength range in A (the full workload is 3000-10000)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    return ap.parse_args()


def workload(n_lines, wl=(3000, 10000)):
    from korg_gb300 import synthetic
    return synthetic.config1(n_lines=n_lines, wl=tuple(wl))


def cpu_sample(n_lines, threads, _cache={}):
    """Time the oracle on the CPU sample; returns (spectra/s extrapolated, seconds, evals, info).

    The sample is the full workload (all lines, the same continuum and atmosphere) evaluated on
    20% of the grid points: 20 windows of 70 A spread evenly over 3000-10000 A."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from korg_gb300 import synthetic
    from korg_gb300.data import stark_profiles
    from korg_gb300.wavelengths import Wavelengths
    oracle.build()
    key = n_lines
    if key not in _cache:
        inp = synthetic.prepare(workload(n_lines))
        full_points = len(inp.wls)
        inp.wls = Wavelengths(CPU_SAMPLE)
        _cache[key] = (inp, full_points)
    inp, full_points = _cache[key]
    frac = len(inp.wls) / full_points
    t0 = time.perf_counter()
    _, _, _, _, ev = oracle.synthesize(inp, inp.linelist, inp.linelist5, stark_profiles(), inp.wls.all_wls,
                                       nthreads=threads)
    dt = time.perf_counter() - t0
    return frac / dt, dt, ev, (f"the full workload ({len(inp.linelist)} lines, H lines) evaluated on 20 windows "
                               f"of 70 A spread over 3000-10000 A ({len(inp.wls)} of {full_points} points, "
                               f"fraction {frac:.4f}); spectra/s = fraction / seconds")


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, index):
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--id={index}", f"--query-gpu={q}", "--format=csv,noheader,nounits",
                                       "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None

    def stop(self):
        if self.p is None:
            return None
        self.p.terminate()
        self.p.wait()
        self.f.seek(0)
        rows = [r.split(",") for r in self.f.read().strip().splitlines() if r.strip()]
        os.unlink(self.f.name)
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in rows:
            try:
                sm.append(float(r[1]))
                mx = max(mx, float(r[2]))
                for k, n in enumerate(names):
                    if r[5 + k].strip() == "Active":
                        reasons.add(n)
            except (ValueError, IndexError):
                continue
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": mx, "reasons": sorted(reasons), "samples": len(sm)}


def traffic_from_profiles():
    """DRAM bytes per launch of the tile kernel from the committed ncu summary, if present."""
    path = os.path.join(ROOT, "profiles", "ncu_line_tile_kernel_cfg1.md")
    if not os.path.exists(path):
        return None
    for line in open(path):
        if line.startswith("traffic_bytes_per_launch:"):
            try:
                return float(line.split(":")[1])
            except ValueError:
                return None
    return None


def run_reference(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    for _ in range(min(args.warmup, 1)):
        cpu_sample(args.lines, threads)
    secs, vals = [], []
    info, ev = "", 0
    for _ in range(args.steps):
        v, dt, ev, info = cpu_sample(args.lines, threads)
        secs.append(dt)
        vals.append(v)
    dt = statistics.mean(secs)
    value = statistics.mean(vals)
    out = {"impl": "reference", "metric": METRIC, "value": value, "unit": "spectra/s", "n_gpus": 0,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": dt * 1e3, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
           "config": {"workload": "full optical synthesis: 56 layers, 300k atomic lines + H lines, 3000-10000 A "
                                  "@ 0.01 A (700,001 points), Teff 5800 logg 4.4", "sample": info},
           "cpu_baseline": {"value": value, "unit": "spectra/s", "cores": threads, "kind": "port", "sample": info,
                            "evals_per_s": ev / dt},
           "e2e": {"value": value, "unit": "spectra/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(out), flush=True)


def dev_inputs(inp, torch, dev):
    """Upload prepared inputs into torch device tensors; returns structs + keep-alive list."""
    from korg_gb300 import _lib
    keep = []

    def d(a, dt=None):
        import numpy as np
        dt = dt or torch.float64
        t = torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(dev)
        keep.append(t)
        ptr = t.data_ptr()
        return C.cast(ptr, C.POINTER(C.c_double)) if dt == torch.float64 else C.cast(ptr, C.POINTER(C.c_int32))

    def lines(ll):
        return _lib.Lines(len(ll), d(ll.wl), d(ll.log_gf), d(ll.E_lower), d(ll.gamma_rad), d(ll.gamma_stark),
                          d(ll.vdW1), d(ll.vdW2), d(ll.mass), d(ll.is_mol, torch.int32), d(ll.species_idx, torch.int32))

    L = len(inp.T)
    lay = _lib.Layers(L, inp.n_div_U.shape[0], d(inp.T), d(inp.ne), d(inp.n_eff_vdW), d(inp.xi), d(inp.n_div_U))
    s = _lib.SynthInputs(lay, d(inp.tau_ref), d(inp.alpha_ref_cntm), d(inp.nH_I), d(inp.nHe_I), d(inp.UH_I),
                         inp.ref_wl, _lib.Cntm(len(inp.cntm_knots), d(inp.cntm_knots), d(inp.cntm_vals)),
                         int(inp.hydrogen_lines), int(inp.use_MHD), inp.hydrogen_window, inp.cutoff_threshold)
    l1, l5 = lines(inp.linelist), lines(inp.linelist5)
    w = torch.as_tensor(inp.wls.all_wls).to(dev)
    keep.append(w)
    return s, l1, l5, w, keep


def host_bytes(inp):
    n, n5, L = len(inp.linelist), len(inp.linelist5), len(inp.T)
    per_line = 8 * 8 + 2 * 4
    return (8 * len(inp.wls) + per_line * (n + n5) + 8 * L * (9 + inp.n_div_U.shape[0]) +
            8 * len(inp.cntm_knots) * (1 + L))


def run_korg(args):
    import numpy as np
    import torch
    import build as korg_build
    from korg_gb300 import _lib
    from korg_gb300.synthesize import synthesize_prepared
    from korg_gb300 import synthetic

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    dist = world > 1
    if dist:
        import torch.distributed as tdist
        tdist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    korg_build.build()

    t0 = time.perf_counter()
    work = workload(args.lines, args.wl)
    inp = synthetic.prepare(work)
    host_prep_s = time.perf_counter() - t0

    ctx = _lib.Context(local)
    ctx.ensure_stark()
    ctx.check(ctx.lib.korg_set_timing(ctx.h, 1))
    s, l1, l5, w, keep = dev_inputs(inp, torch, dev)
    nwl, L = len(inp.wls), len(inp.T)
    flux = torch.empty(nwl, dtype=torch.float64, device=dev)
    cntm = torch.empty_like(flux)
    flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=dev)
    stream = torch.cuda.current_stream(dev)

    def step(prec):
        rc = ctx.lib.korg_synthesize_dev(ctx.h, C.byref(s), C.byref(l1), C.byref(l5), w.data_ptr(), nwl, prec,
                                         flux.data_ptr(), cntm.data_ptr(), None, stream.cuda_stream)
        ctx.check(rc)

    for _ in range(args.warmup):
        step(_lib.KORG_MIXED)
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    torch.cuda.synchronize()
    clk = Clocks(local)
    times, tiles, stats = [], [], None
    for _ in range(args.steps):
        flush.zero_()  # L2 flush between steps, outside the timed events
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step(_lib.KORG_MIXED)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
        stats = ctx.stats()
        tiles.append(stats.ms_line_tile)
    torch.cuda.synchronize()
    if dist:
        tdist.barrier()
    clocks = clk.stop()
    ms = statistics.mean(times)
    if dist:
        t = torch.tensor([ms], device=dev)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
    flux32 = flux.cpu().numpy().copy()
    cntm32 = cntm.cpu().numpy().copy()
    evals = stats.line_evals
    stage = {"ref_lines": stats.ms_ref_lines, "hydrogen": stats.ms_hydrogen, "line_prep": stats.ms_line_prep,
             "line_tile": stats.ms_line_tile, "rt_both_passes": stats.ms_rt}

    # plain FP64 form of the same synthesis
    fp64 = None
    if not args.no_fp64:
        step(_lib.KORG_FP64)
        torch.cuda.synchronize()
        t64 = []
        for _ in range(2):
            flush.zero_()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            step(_lib.KORG_FP64)
            e1.record(stream)
            e1.synchronize()
            t64.append(e0.elapsed_time(e1))
        st64 = ctx.stats()
        f64 = flux.cpu().numpy()
        c64 = cntm.cpu().numpy()
        err = float(np.max(np.abs(flux32 / f64 - 1)))
        rms = float(np.sqrt(np.mean((flux32 / cntm32 - f64 / c64) ** 2)))
        fp64 = {"spectra_per_s": 1000.0 / statistics.mean(t64), "ms_per_step": statistics.mean(t64),
                "evals_per_s": st64.line_evals / (statistics.mean(t64) * 1e-3),
                "stages_ms": {"line_prep": st64.ms_line_prep, "line_tile": st64.ms_line_tile,
                              "hydrogen": st64.ms_hydrogen, "rt_both_passes": st64.ms_rt},
                "mixed_speedup": statistics.mean(t64) / ms,
                "mixed_max_rel_flux_err": err, "mixed_rectified_rms": rms}

    # end to end through the public host-pointer call: host inputs, H2D + compute + D2H
    ctx.check(ctx.lib.korg_set_timing(ctx.h, 0))
    synthesize_prepared(inp, precision="mixed", ctx=ctx)
    e2e_t = []
    for _ in range(max(2, args.steps)):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        res = synthesize_prepared(inp, precision="mixed", ctx=ctx)
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = statistics.mean(e2e_t)
    assert np.array_equal(res.flux, flux32)

    # roofline of the dominant kernel: the FP32 line-profile tile kernel
    peak = C.c_double(0)
    ctx.check(ctx.lib.korg_probe_flops(ctx.h, 0, C.byref(peak)))
    peak64 = C.c_double(0)
    ctx.check(ctx.lib.korg_probe_flops(ctx.h, 1, C.byref(peak64)))
    tile_ms = statistics.mean(tiles)
    achieved = evals * FLOP_PER_EVAL / (tile_ms * 1e-3) / 1e12
    rt_flop = 2 * L * nwl * 35
    rt_achieved = rt_flop / (stats.ms_rt * 1e-3) / 1e12

    cpu = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, ev_cpu, info = cpu_sample(args.lines, threads)
        cpu = {"value": v, "unit": "spectra/s", "cores": threads, "kind": "port", "sample": info,
               "evals_per_s": ev_cpu / dt, "seconds": dt}

    launches_per_step = 1 + 4 + (3 if inp.hydrogen_lines else 0) + 4 + 1
    out = {
        "metric": METRIC,
        "value": world * 1000.0 / ms,
        "unit": "spectra/s",
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": ms,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32 profiles + f64 tau/flux (mixed)",
        "data": "synthetic (seeded line list and stand-in atmosphere)",
        "config": {"workload": "full optical synthesis: 56 layers (Teff 5800, logg 4.4, [M/H] 0), "
                               f"{args.lines} atomic lines + hydrogen lines, {args.wl[0]:.0f}-{args.wl[1]:.0f} A "
                               f"@ 0.01 A ({nwl} points)",
                   "precision": "mixed",
                   "l2": f"flushed (256 MiB write) between steps; alpha {8 * L * nwl / 1e6:.0f} MB",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU",
                   "host_prep_s": host_prep_s},
        "evals_per_step": evals,
        "evals_per_s": world * evals / (ms * 1e-3),
        "stages_ms": stage,
        "fp64": fp64,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value, "traffic": traffic_from_profiles(),
                     "kernel": "line_tile_kernel<mixed> (metal lines)",
                     "algorithmic": f"{FLOP_PER_EVAL} FP32 flop x {evals} line-layer-lambda evals per launch",
                     "peak_source": "measured in-process (korg_probe_flops: FP32 FMA chains); "
                                    "MEASURED_PEAKS.json has no FP32 figure",
                     "rt_fp64": {"achieved": rt_achieved, "peak": peak64.value, "unit": "TFLOP/s",
                                 "frac": rt_achieved / peak64.value,
                                 "algorithmic": "35 FP64 flop x 2 passes x L x nwl"}},
        "cpu_baseline": cpu,
        "e2e": {"value": world / e2e_s, "unit": "spectra/s", "h2d_bytes_per_step": host_bytes(inp),
                "d2h_bytes_per_step": 16 * nwl},
        "gpu_launches": launches_per_step * args.steps,
        "clocks": clocks,
    }
    if rank == 0:
        print(json.dumps(out), flush=True)
    ctx.close()
    if dist:
        tdist.destroy_process_group()


if __name__ == "__main__":
    a = parse()
    if a.impl == "reference":
        run_reference(a)
    else:
        run_korg(a)
