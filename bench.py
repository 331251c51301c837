#!/usr/bin/env python3
"""Benchmark of the synthesis hot path on the full-optical workload.

One step = one complete synthesis (reference-wavelength lines, hydrogen lines, 300,000 metal
lines, continuum-only and full radiative transfer) of a 56-layer atmosphere on a 700,001-point
grid (3000-10000 A at 0.01 A), mixed precision, inputs resident in HBM.  Prints one JSON line.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]

--impl reference times the FP64 CPU restatement of the reference (the oracle, all host cores)
on a bounded sample of the same workload.

    python bench.py --workload adjoint

times the reverse mode on the adjoint configuration (72 layers, Teff 4500 K, logg 2.5,
[M/H] -0.5, 50k atomic + 20k CO/OH/CN lines, 15000-17000 A at 0.005 A): one step = forward
synthesis + rectified-flux loss + korg_synthesize_vjp_dev, against the forward alone.

    python bench.py --workload variants

times the large cool-star stress case: 80 layers, Teff 3500 K, logg 1.0, 1,000,000 lines (40%
atomic, 60% TiO/CO/OH/CN), 3000-10000 A at 0.01 A, as one batch of 16 abundance variants.

    python bench.py --workload batch [--spectra 256]

times the batched form instead: 256 atmospheres (Teff 3500-7000 K, logg 1-5, [M/H] -2.5..0.5),
each with its own random 20k-200k-line subset of a 500k-line atomic + molecular list, on the
400,001-point 15000-17000 A grid; one step = the whole batch through korg_synthesize_batch_dev
(CUDA-graph replay, autotuned tile shape).

    python bench.py --workload chemistry [--spectra 16]

times Korg's chemical equilibrium of every layer of up to 16 stars (Teff 3500-7000 K) in one
batched device call (--spectra 1: the 5777 K star alone).

    python bench.py --workload postprocess

times the post-processing of 64 synthesised spectra on that grid: rotational broadening
(apply_rotation) then the Gaussian LSF (R = 22,500) onto a 0.2 A observed grid.
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
import warnings

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))

METRIC = "spectra/s & line-layer-lambda evals/s, mixed vs plain FP64 at 1e-4 flux err"
FLOP_PER_EVAL = 24  # FP32 flop per Voigt evaluation (Harris branch, FMA = 2)
# bounded sample of the workload for the CPU baseline and the oracle comparison: the same range
# on a 0.05 A grid, whose wavelengths are exactly every 5th point of the 0.01 A grid (20% of the
# points, spread over the whole range, so line density and hydrogen windows are sampled evenly)
CPU_SAMPLE_STEP = 0.05

def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=None, help="timed steps (20; 3 for --workload batch)")
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="korg", choices=["korg", "reference"])
    ap.add_argument("--lines", type=int, default=300_000)
    ap.add_argument("--wl", type=float, nargs=2, default=[3000.0, 10000.0],
                    help="wavelength range in A (the full workload is 3000-10000)")
    ap.add_argument("--no-fp64", action="store_true", help="skip the plain FP64 comparison run")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample (and the oracle comparisons)")
    ap.add_argument("--no-configs", action="store_true",
                    help="skip the oracle comparison of the adjoint, batch and cool-star configurations")
    ap.add_argument("--no-adjoint", action="store_true", help="skip the reverse-mode measurement")
    ap.add_argument("--no-chemistry", action="store_true", help="skip the chemical-equilibrium measurement")
    ap.add_argument("--no-batch", action="store_true", help="skip the 16-spectrum batched-engine measurement")
    ap.add_argument("--workload", default="synth",
                    choices=["synth", "batch", "adjoint", "variants", "postprocess", "chemistry"])
    ap.add_argument("--tile", default=None, help="force the line tile shape: tw,stage,split (e.g. 64,32,1)")
    ap.add_argument("--spectra", type=int, default=256, help="batch workload: number of spectra")
    ap.add_argument("--adj-scale", type=float, default=1.0, help="adjoint workload: fraction of its 70k lines")
    return ap.parse_args()


def workload(n_lines, wl=(3000, 10000)):
    from korg_gb300 import synthetic
    return synthetic.config1(n_lines=n_lines, wl=tuple(wl))


def strided(inp, step_A):
    """Copy of prepared inputs on the same range(s) with a coarser step; its wavelengths are a
    subset of the original grid's (checked), every stride-th point."""
    import copy
    import numpy as np
    from korg_gb300.wavelengths import Wavelengths
    s = copy.copy(inp)
    a, b = inp.wls.eachwindow()[0]
    s.wls = Wavelengths((round(a * 1e8, 6), round(b * 1e8, 6), step_A))
    stride = (len(inp.wls) - 1) // (len(s.wls) - 1)
    assert len(inp.wls.ranges) == 1 and np.array_equal(s.wls.all_wls, inp.wls.all_wls[::stride])
    return s, stride


def oracle_flux(inp, threads):
    """The FP64 oracle's synthesis of prepared inputs: (flux, cntm, evals, seconds)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle
    from korg_gb300.data import stark_profiles
    oracle.build()
    t0 = time.perf_counter()
    flux, cntm, _, _, ev = oracle.synthesize(inp, inp.linelist, inp.linelist5, stark_profiles(), inp.wls.all_wls,
                                             nthreads=threads)
    return flux, cntm, ev, time.perf_counter() - t0


def cpu_continuum(inp):
    """Replace the continuum of prepared inputs by the FP64 CPU restatement of Korg's continuum
    absorption (the values the device computes for continuum="gpu", to rounding), so that a
    CPU-only process prepares the GPU arm's workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import numpy as np
    import continuum_oracle
    from korg_gb300.continuum import layer_inputs
    d = layer_inputs(inp.T, inp.ne, inp.number_densities)
    nu = 2.99792458e10 / inp.cntm_knots
    nu_ref = 2.99792458e10 / np.array([inp.ref_wl])
    for l in range(len(inp.T)):
        dl = {k: v[l] for k, v in d.items()}
        inp.cntm_vals[l] = continuum_oracle.total_continuum_absorption(nu, inp.T[l], dl["ne"], dl)
        inp.alpha_ref_cntm[l] = continuum_oracle.total_continuum_absorption(nu_ref, inp.T[l], dl["ne"], dl)[0]
    return inp


def _oracle_postprocess(a):
    """One spectrum of the FP64 post-processing restatement (spawn-pool worker): rotation of the
    grid's first `frac` of points, or the Gaussian LSF of the whole spectrum onto the observed
    grid.  Returns the seconds it took."""
    kind, seed, frac = a
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))
    import numpy as np
    import postprocess_oracle as po
    from korg_gb300.wavelengths import Wavelengths
    g = Wavelengths((15000, 17000, 0.005))
    f = 1 - 0.5 * np.random.default_rng(seed).random(len(g)) ** 8
    t1 = time.perf_counter()
    if kind == "rotation":
        sub = Wavelengths((15000, 15000 + 2000 * frac, 0.005))
        po.apply_rotation(f[:len(sub)], sub.all_wls, sub.ranges, 10.0, 0.6)
    else:
        for w in Wavelengths((15100, 16900, 0.2)).all_wls:
            lb, ub, phi = po.lsf_bounds_and_kernel(g.all_wls, w, 22_500.0, 4)
            float(np.sum(f[lb:ub + 1] * phi))
    return time.perf_counter() - t1


def _oracle_chem_layer(a):
    """One layer of the FP64 chemical-equilibrium restatement (spawn-pool worker)."""
    T, nt, ne, ab = a
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))
    import numpy as np
    import statmech_oracle
    from korg_gb300 import data
    from korg_gb300.statmech import default_equilibrium_tables
    out_ne, nd = statmech_oracle.chemical_equilibrium(T, nt, ne, ab, data.ionization_energies(),
                                                      data.default_partition_funcs(),
                                                      data.default_log_equilibrium_constants(),
                                                      electron_number_density_warn_threshold=np.inf)
    return out_ne, np.array([out_ne] + [nd[s] for s in default_equilibrium_tables().species[1:]])


def oracle_chemistry(T, n_tot, ne_model, ab, threads=None):
    """Chemical equilibrium of every layer with the FP64 CPU restatement, in a spawn pool: the
    same (T, n_tot, ne, abundances) -> (ne, {Species: n}) interface as the device solve."""
    import multiprocessing as mp
    import numpy as np
    from korg_gb300.statmech import default_equilibrium_tables
    T = np.atleast_1d(T)
    args = [(float(T[l]), float(np.broadcast_to(n_tot, T.shape)[l]), float(np.broadcast_to(ne_model, T.shape)[l]),
             np.asarray(ab)) for l in range(len(T))]
    with mp.get_context("spawn").Pool(min(len(args), threads or os.cpu_count() or 1)) as pool:
        res = pool.map(_oracle_chem_layer, args, chunksize=1)
    dens = np.stack([r[1] for r in res])
    species = default_equilibrium_tables().species
    return dens[:, 0].copy(), {sp: dens[:, k].copy() for k, sp in enumerate(species) if sp is not None}


CHEM_STARS = [(3500.0, 1.0, -2.5), (3500.0, 4.5, 0.0), (3800.0, 2.0, -1.0), (4000.0, 4.8, 0.5),
              (4200.0, 1.5, 0.0), (4500.0, 2.5, -0.5), (4800.0, 4.5, -2.0), (5000.0, 3.0, 0.3),
              (5300.0, 4.0, -1.5), (5600.0, 4.4, 0.0), (5777.0, 4.44, 0.0), (6000.0, 4.2, -0.7),
              (6300.0, 3.5, 0.2), (6600.0, 4.0, -2.5), (6800.0, 2.5, 0.0), (7000.0, 4.3, 0.5)]


def chemistry_measure(ctx, torch, dev, threads, n_stars=16, steps=3, warmup=1, cpu=True):
    """Chemical equilibrium (korg_chemical_equilibrium_dev) of every layer of n_stars 56-layer
    stars (the first n of CHEM_STARS, the 5777 K star alone for n_stars=1) in one batched call,
    device-timed, against the FP64 CPU restatement on every 8th layer."""
    import warnings
    import numpy as np
    from korg_gb300 import _lib, standin
    from korg_gb300.statmech import solve_layers
    atms = []
    for Teff, logg, m_H in ([CHEM_STARS[10]] if n_stars == 1 else CHEM_STARS[:n_stars]):
        atm, A_X = standin.synthetic_atmosphere(Teff, logg, m_H)
        ab = 10.0 ** (A_X - 12)
        atms.append((atm, ab / ab.sum()))
    T = np.concatenate([a.T for a, _ in atms])
    nt = np.concatenate([a.n_tot for a, _ in atms])
    ne = np.concatenate([a.ne for a, _ in atms])
    abund = np.stack([ab for _, ab in atms])
    atm_idx = np.concatenate([np.full(len(a.T), k, np.int32) for k, (a, _) in enumerate(atms)])
    L = len(T)
    tab = ctx.ensure_equilibrium()
    nspec = _lib.KORG_CHEM_MOL0 + len(tab.molecules)
    d = lambda a, dt=torch.float64: torch.as_tensor(np.ascontiguousarray(a)).to(dt).to(dev)
    tT, tnt, tne, tab_, tatm = d(T), d(nt), d(ne), d(abund), d(atm_idx, torch.int32)
    dens = torch.empty((L, nspec), dtype=torch.float64, device=dev)
    status = torch.empty(L, dtype=torch.int32, device=dev)
    info = torch.empty((L, 5), dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev)
    dp = lambda t: C.cast(t.data_ptr(), _lib._dp)

    def run(lo, hi, atm_ptr):
        y = _lib.ChemLayers(hi - lo, dp(tT[lo:hi]), dp(tnt[lo:hi]), dp(tne[lo:hi]), dp(tab_),
                            C.cast(atm_ptr, _lib._ip) if atm_ptr else None)
        ctx.check(ctx.lib.korg_chemical_equilibrium_dev(ctx.h, C.byref(y), len(atms), dens[lo:hi].data_ptr(),
                                                        status[lo:hi].data_ptr(), info[lo:hi].data_ptr(),
                                                        stream.cuda_stream))

    def timed(fn, reps=steps):
        for _ in range(warmup):
            fn()
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            fn()
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts)

    ms_all = timed(lambda: run(0, L, tatm.data_ptr()))
    st, inf, got = status.cpu().numpy(), info.cpu().numpy(), dens.cpu().numpy()
    # reverse mode at the solution: every density carries a cotangent
    gbar = torch.randn((L, nspec), dtype=torch.float64, device=dev, generator=torch.Generator(dev).manual_seed(5))
    dT, dnt = torch.empty(L, dtype=torch.float64, device=dev), torch.empty(L, dtype=torch.float64, device=dev)
    dab = torch.empty((L, 92), dtype=torch.float64, device=dev)
    vstatus = torch.empty(L, dtype=torch.int32, device=dev)
    yv = _lib.ChemLayers(L, dp(tT), dp(tnt), dp(tne), dp(tab_), C.cast(tatm.data_ptr(), _lib._ip))

    def vjp():
        ctx.check(ctx.lib.korg_chemical_equilibrium_vjp_dev(ctx.h, C.byref(yv), len(atms), dp(dens), dp(gbar), dp(dT),
                                                            dp(dnt), dp(dab), vstatus.data_ptr(), stream.cuda_stream))
    ms_vjp = timed(vjp)
    vjp_ok = int((vstatus == 0).sum().item())
    if n_stars == 1:
        return {"layers": L, "ms": ms_all, "layers_per_s": L / (ms_all * 1e-3), "status_ok": int((st == 0).sum()),
                "newton_iterations": float(inf[:, 0].sum()), "vjp_ms": ms_vjp, "vjp_status_ok": vjp_ok}
    k10 = 10 * 56  # the 5777 K star, the headline's atmosphere: what one synthesize pays
    ms_one = timed(lambda: run(k10, k10 + 56, 0), reps=5)
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        t1 = time.perf_counter()
        solve_layers(T, nt, ne, abund, atm=atm_idx, ctx=ctx)
        e2e_s = time.perf_counter() - t1
    if not cpu:
        return {"layers": L, "ms": ms_all, "layers_per_s": L / (ms_all * 1e-3), "one_atmosphere_ms": ms_one,
                "e2e_layers_per_s": L / e2e_s, "status_ok": int((st == 0).sum()), "newton_iterations": float(inf[:, 0].sum()),
                "fp64_fallback_steps": float(inf[:, 4].sum()), "vjp_ms": ms_vjp, "vjp_status_ok": vjp_ok}
    # FP64 CPU restatement on every 8th layer (spawn pool, all host cores)
    sample = np.arange(0, L, 8)
    t1 = time.perf_counter()
    import multiprocessing as mp
    with mp.get_context("spawn").Pool(min(len(sample), threads)) as pool:
        res = pool.map(_oracle_chem_layer, [(float(T[l]), float(nt[l]), float(ne[l]), abund[atm_idx[l]])
                                            for l in sample], chunksize=1)
    cpu_s = time.perf_counter() - t1
    worst = 0.0
    for (o_ne, o_vec), l in zip(res, sample):
        keep = o_vec > 1e-30 * nt[l]
        worst = max(worst, float(np.max(np.abs(got[l][keep] / o_vec[keep] - 1))))
    iters = float(inf[:, 0].sum())
    return {"workload": f"{len(atms)} stars x 56 layers (Teff 3500-7000 K, logg 1-5, [M/H] -2.5..0.5; grey "
                        f"atmospheres), {len(tab.molecules)} molecules, one batched call",
            "layers": L, "ms": ms_all, "layers_per_s": L / (ms_all * 1e-3),
            "one_atmosphere_ms": ms_one, "one_atmosphere": "the 5777 K, log g 4.44 star (56 layers)",
            "e2e_layers_per_s": L / e2e_s, "e2e": "host-pointer korg_chemical_equilibrium (H2D, solve, D2H)",
            "vjp_ms": ms_vjp, "vjp_layers_per_s": L / (ms_vjp * 1e-3), "vjp_status_ok": vjp_ok,
            "status_ok": int((st == 0).sum()), "newton_iterations": iters,
            "us_per_newton_iteration_per_layer": ms_all * 1e3 / iters * min(L, 152),
            "fp64_fallback_steps": float(inf[:, 4].sum()), "max_solves_per_layer": float(inf[:, 1].max()),
            "max_rel_density_err_vs_oracle": worst,
            "oracle_compare": f"every 8th layer ({len(sample)}), species above 1e-30 n_tot",
            "cpu_baseline": {"value": len(sample) / cpu_s, "unit": "layers/s", "cores": threads, "kind": "port",
                             "sample": f"{len(sample)} layers (every 8th) with the FP64 numpy restatement of "
                                       "statmech.jl, one layer per process"}}


def cpu_sample(inp_or_lines, threads, _cache={}):
    """Time the oracle on the CPU sample; returns (spectra/s, seconds, evals, info, flux, cntm).

    The sample is the full workload (all lines, the same continuum and atmosphere) on the same
    3000-10000 A range at 0.05 A: every 5th point of the 0.01 A grid, 20% of the points.  Given a
    line count, the workload is prepared here on the CPU (continuum from the CPU restatement)."""
    from korg_gb300 import synthetic
    key = inp_or_lines if isinstance(inp_or_lines, int) else id(inp_or_lines)
    if key not in _cache:
        inp = (cpu_continuum(synthetic.prepare(workload(inp_or_lines), chemistry=oracle_chemistry))
               if isinstance(inp_or_lines, int) else inp_or_lines)
        _cache[key] = (strided(inp, CPU_SAMPLE_STEP)[0], len(inp.wls))
    inp, full_points = _cache[key]
    frac = len(inp.wls) / full_points
    flux, cntm, ev, dt = oracle_flux(inp, threads)
    return frac / dt, dt, ev, (f"the full workload ({len(inp.linelist)} lines, H lines) on the same range at "
                               f"{CPU_SAMPLE_STEP} A, i.e. every 5th point of the grid ({len(inp.wls)} of "
                               f"{full_points} points, fraction {frac:.4f}); spectra/s = fraction / seconds"), flux, cntm


def flux_errors(flux, cntm, ref_flux, ref_cntm):
    """max relative flux error and rectified-flux RMS / max error of (flux, cntm) against a reference."""
    import numpy as np
    r, rr = flux / cntm, ref_flux / ref_cntm
    return {"max_rel_flux_err": float(np.max(np.abs(flux / ref_flux - 1))),
            "rectified_rms": float(np.sqrt(np.mean((r - rr) ** 2))),
            "max_rectified_err": float(np.max(np.abs(r - rr)))}


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


def replica_rate(ms, world, device, tdist=None):
    """Whole-job rate of `world` independent replicas (one spectrum per step each): the slowest
    rank's mean step time (max over ranks) and world spectra per that time."""
    if tdist is not None and world > 1:
        import torch
        t = torch.tensor([float(ms)], dtype=torch.float64, device=device)
        tdist.all_reduce(t, op=tdist.ReduceOp.MAX)
        ms = float(t.item())
    return ms, world * 1000.0 / ms


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
        v, dt, ev, info, _, _ = cpu_sample(args.lines, threads)
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
    from korg_gb300.api import synthesize_prepared
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

    ctx = _lib.Context(local)
    t0 = time.perf_counter()
    work = workload(args.lines, args.wl)
    with warnings.catch_warnings():  # the grey atmosphere's n_e is not Korg's: the n_e warning is expected
        warnings.simplefilter("ignore")
        inp = synthetic.prepare(work, continuum="gpu", chemistry="gpu", ctx=ctx)
    host_prep_s = time.perf_counter() - t0
    ctx.ensure_stark()
    ctx.check(ctx.lib.korg_set_timing(ctx.h, 1))
    if args.tile:
        tw, st, sp = (int(v) for v in args.tile.split(","))
        for prec in (_lib.KORG_MIXED, _lib.KORG_FP64):
            ctx.check(ctx.lib.korg_set_tile_config(ctx.h, len(inp.T), prec, tw, st, sp))
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
    ms, value = replica_rate(statistics.mean(times), world, dev, tdist if dist else None)
    flux32 = flux.cpu().numpy().copy()
    cntm32 = cntm.cpu().numpy().copy()
    evals = stats.line_evals
    stage = {"ref_lines": stats.ms_ref_lines, "hydrogen": stats.ms_hydrogen, "line_prep": stats.ms_line_prep,
             "line_tile": stats.ms_line_tile, "rt_both_passes": stats.ms_rt}

    # plain FP64 form of the same synthesis
    fp64, f64, c64 = None, None, None
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
        f64 = flux.cpu().numpy().copy()
        c64 = cntm.cpu().numpy().copy()
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

    cpu, parity = None, {}
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, ev_cpu, info, oflux, ocntm = cpu_sample(inp, threads)
        cpu = {"value": v, "unit": "spectra/s", "cores": threads, "kind": "port", "sample": info,
               "evals_per_s": ev_cpu / dt, "seconds": dt}
        # the headline's flux against the FP64 oracle at the sample's points (every 5th point)
        m = flux_errors(flux32[::5], cntm32[::5], oflux, ocntm)
        h = {"points": len(oflux), "mixed_max_rel_flux_err_vs_oracle": m["max_rel_flux_err"],
             "mixed_rectified_rms_vs_oracle": m["rectified_rms"],
             "mixed_max_rectified_err_vs_oracle": m["max_rectified_err"]}
        if f64 is not None:
            h["fp64_max_rel_flux_err_vs_oracle"] = flux_errors(f64[::5], c64[::5], oflux, ocntm)["max_rel_flux_err"]
            h["fp64_cntm_max_rel_err_vs_oracle"] = float(np.max(np.abs(c64[::5] / ocntm - 1)))
        parity["cfg1_full_optical"] = h
        _progress("headline CPU sample and oracle comparison done")
        if not args.no_configs:
            parity.update(configs_vs_oracle(ctx, threads))
    adj = adjoint_measure(ctx, torch, dev, steps=5) if rank == 0 and not args.no_adjoint else None
    chem = (chemistry_measure(ctx, torch, dev, os.cpu_count() or 1)
            if rank == 0 and not args.no_chemistry else None)
    batch = batch_measure(torch, dev) if rank == 0 and not args.no_batch else None

    # alpha init, reference-wavelength lines (5), hydrogen (3), metal lines (5), transfer
    launches_per_step = 1 + 5 + (3 if inp.hydrogen_lines else 0) + 5 + 1
    out = {
        "metric": METRIC,
        "value": value,
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
                   "chemistry": "device (korg_chemical_equilibrium: Korg's chemical equilibrium, 306 molecules)",
                   "continuum": "device (korg_continuum_absorption: Korg's continuum terms except metal bound-free)",
                   "l2": f"flushed (256 MiB write) between steps; alpha {8 * L * nwl / 1e6:.0f} MB",
                   "parallelism": f"replicas x{world}" if world > 1 else "1 GPU", "tile": args.tile or "default",
                   "host_prep_s": host_prep_s},
        "evals_per_step": evals,
        "evals_per_s": world * evals / (ms * 1e-3),
        "stages_ms": stage,
        "fp64": fp64,
        **{k: v for k, v in parity.get("cfg1_full_optical", {}).items() if k.endswith("_vs_oracle")},
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
        "parity_vs_oracle": parity,
        "adjoint": adj,
        "chemical_equilibrium": chem,
        "batch": batch,
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


def _batch_atmosphere(w):
    sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))
    from korg_gb300 import standin
    return standin.synthetic_atmosphere(w.Teff, w.logg, w.m_H, w.L)


def _fixed_chemistry(ne, nd, T, n_tot, A_X):
    return ne, nd


def _no_continuum(wls_cm, T, ne, n_HI, n_HII):
    """Placeholder continuum for the pool workers: the batch's continuum is evaluated afterwards on
    the device for every atmosphere (korg_continuum_absorption)."""
    import numpy as np
    return np.zeros(len(wls_cm))


def _prep_batch_one(a):
    sys.path.insert(0, os.path.join(ROOT, "korg.jl_gb300"))
    import functools
    from korg_gb300.api import prepare_synthesis
    w, (atm, A_X), ne, nd = a
    return prepare_synthesis(atm, w.linelist, A_X, w.wavelengths, vmic=w.vmic, hydrogen_lines=w.hydrogen_lines,
                             chemical_equilibrium=functools.partial(_fixed_chemistry, ne, nd),
                             continuum_opacity=_no_continuum)


def batch_inputs(n_spectra):
    """Host precompute of the batch workload: the atmospheres in a spawn pool, the chemical
    equilibrium of every layer of every atmosphere in one batched device call
    (korg_chemical_equilibrium), the rest of each spectrum's precompute in the pool, then Korg's
    continuum absorption of every atmosphere on the device (korg_continuum_absorption)."""
    import multiprocessing as mp
    import numpy as np
    from korg_gb300 import _lib, continuum, synthetic
    from korg_gb300.statmech import default_equilibrium_tables, solve_layers
    works = synthetic.config3(n_spectra=n_spectra)
    t0 = time.perf_counter()
    with mp.get_context("spawn").Pool(min(len(works), os.cpu_count() or 1)) as pool:
        atms = pool.map(_batch_atmosphere, works, chunksize=1)
    t1 = time.perf_counter()
    ctx = _lib.Context(0)
    abund = np.stack([10.0 ** (A_X - 12) / np.sum(10.0 ** (A_X - 12)) for _, A_X in atms])
    idx = np.concatenate([np.full(len(a.T), k, np.int32) for k, (a, _) in enumerate(atms)])
    ctx.ensure_equilibrium()
    t2 = time.perf_counter()
    dens, status, info = solve_layers(np.concatenate([a.T for a, _ in atms]), np.concatenate([a.n_tot for a, _ in atms]),
                                      np.concatenate([a.ne for a, _ in atms]), abund, atm=idx, ctx=ctx)
    t3 = time.perf_counter()
    species = default_equilibrium_tables().species
    chem = []
    for k in range(len(atms)):
        rows = dens[idx == k]
        chem.append((rows[:, 0].copy(), {sp: rows[:, j].copy() for j, sp in enumerate(species) if sp is not None}))
    with mp.get_context("spawn").Pool(min(len(works), os.cpu_count() or 1)) as pool:
        inps = pool.map(_prep_batch_one, [(w, a, c[0], c[1]) for w, a, c in zip(works, atms, chem)], chunksize=1)
    t4 = time.perf_counter()
    ctx.ensure_continuum()
    for inp in inps:
        d = continuum.layer_inputs(inp.T, inp.ne, inp.number_densities)
        inp.cntm_vals = continuum.absorption_from_inputs(inp.cntm_knots, d, ctx)
        inp.alpha_ref_cntm = continuum.absorption_from_inputs(np.array([inp.ref_wl]), d, ctx)[:, 0].copy()
    t5 = time.perf_counter()
    ctx.close()
    return inps, {"atmospheres_s": t1 - t0, "chemistry_s": t3 - t2, "chemistry_layers": len(idx),
                  "chemistry_newton_iterations": float(info[:, 0].sum()), "rest_s": t4 - t3,
                  "continuum_s": t5 - t4,
                  "chemistry": "korg_chemical_equilibrium, every layer of every atmosphere in one call (host pointers)",
                  "continuum": "korg_continuum_absorption per atmosphere (host pointers)"}


def cpu_sample_batch(inps, threads):
    """Oracle on the first spectra of the batch (their line counts spread over the batch's
    20k-200k), each over 10 windows of 20 A spread evenly over the grid (10% of it)."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import copy
    import oracle
    from korg_gb300.data import stark_profiles
    from korg_gb300.wavelengths import Wavelengths
    oracle.build()
    win = Wavelengths([(15090.0 + 200.0 * k, 15110.0 + 200.0 * k, 0.005) for k in range(10)])
    frac = len(win) / len(inps[0].wls)
    dt, ev = 0.0, 0
    for inp in inps:
        s = copy.copy(inp)
        s.wls = win
        t0 = time.perf_counter()
        ev += oracle.synthesize(s, s.linelist, s.linelist5, stark_profiles(), s.wls.all_wls, nthreads=threads)[4]
        dt += time.perf_counter() - t0
    return len(inps) * frac / dt, dt, ev, (f"spectra 0-{len(inps) - 1} of the batch "
                                           f"({', '.join(str(len(i.linelist)) for i in inps)} lines) on 10 windows "
                                           f"of 20 A ({len(win)} of {len(inps[0].wls)} points, fraction {frac:.4f}); "
                                           "spectra/s = spectra x fraction / seconds")


def batch_gradient(b, stream, t_forward_ms, steps=1):
    """Forward + rectified-flux loss + gradient of every spectrum of a batch, reusing the batched
    forward's opacity (korg_synthesize_batch_vjp_dev), against the batched forward alone."""
    import numpy as np
    import torch
    f, c = b.run(stream)
    torch.cuda.synchronize()
    noise = torch.as_tensor(np.random.default_rng(5).normal(0, 0.01, (b.n, b.nwl)), device=b.dev)
    obs = (f / c) * (1 + noise)
    times = []
    for _ in range(steps + 1):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        f, c = b.run(stream)
        rr = f / c - obs
        dF, dC = 2 * rr / c, -2 * rr * f / c ** 2
        b.vjp(dF, dC, reuse_forward=True, stream=stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    t = statistics.mean(times[1:])
    return {"forward_and_gradient_ms": t, "forward_ms": t_forward_ms,
            "gradient_over_forward": (t - t_forward_ms) / t_forward_ms,
            "note": "batched forward (graph replay), loss, then korg_synthesize_batch_vjp_dev reusing the forward's "
                    "opacity for every spectrum; gradient w.r.t. T, ne, n_eff_vdW, xi, n/U, log gf, continuum, "
                    "H-line inputs (hydrogen lines with their exact derivatives)"}


def batch_measure(torch, dev, n=16, steps=3):
    """The batched engine on n spectra of the batch workload (its distributions: Teff 3500-7000 K,
    20k-200k-line subsets, 15000-17000 A at 0.005 A): forward throughput (graph replay), the
    speed-up over the plain FP64 form and the mixed form's error on 2 of them, and forward + loss +
    gradient of the whole batch (korg_synthesize_batch_vjp_dev)."""
    import numpy as np
    from korg_gb300.batch import BatchSynthesis
    t0 = time.perf_counter()
    inps, _ = batch_inputs(n)
    host_s = time.perf_counter() - t0
    stream = torch.cuda.current_stream(dev)

    def timed(bs, reps):
        ts = []
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            bs.run(stream)
            e1.record(stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts)

    b = BatchSynthesis(inps, precision="mixed", use_graph=True, autotune=False, max_scratch_bytes=160 << 30)
    for _ in range(3):
        b.run(stream)
        torch.cuda.synchronize()
    ms = timed(b, steps)
    fm, cm = b.results()
    sub = inps[:2]
    b64 = BatchSynthesis(sub, precision="fp64", use_graph=False, autotune=False, max_scratch_bytes=160 << 30)
    b64.run(stream)
    torch.cuda.synchronize()
    ms64 = timed(b64, 1)
    f64, c64 = b64.results()
    b64.ctx.close()
    grad = batch_gradient(b, stream, ms)
    b.ctx.close()
    mixed, plain = 1000.0 * n / ms, 1000.0 * len(sub) / ms64
    return {"workload": f"{n} spectra of the batch workload (56 layers, Teff 3500-7000 K, logg 1-5, [M/H] "
                        f"-2.5..0.5, {sum(len(i.linelist) for i in inps)} lines in all, 15000-17000 A @ 0.005 A), "
                        "device chemistry and continuum",
            "spectra_per_s": mixed, "ms_per_batch": ms, "plain_fp64_spectra_per_s": plain,
            "plain_fp64": f"the same engine in plain FP64 on {len(sub)} of the spectra",
            "batched_speedup_vs_plain_fp64": mixed / plain,
            "mixed_max_rel_flux_err_vs_fp64": float(np.max(np.abs(fm[:len(sub)] / f64 - 1))),
            "mixed_rectified_rms_vs_fp64": float(np.sqrt(np.mean((fm[:len(sub)] / cm[:len(sub)] - f64 / c64) ** 2))),
            "gradient": {k: v for k, v in grad.items() if k != "note"}, "host_prep_s": host_s}


def _progress(msg, t0=time.perf_counter()):
    print(f"[bench {time.perf_counter() - t0:8.1f} s] {msg}", file=sys.stderr, flush=True)


def run_batch(args):
    import numpy as np
    t0 = time.perf_counter()
    _progress(f"host precompute of {args.spectra} spectra")
    inps, prep_parts = batch_inputs(args.spectra)
    host_prep_s = time.perf_counter() - t0
    _progress(f"host precompute done ({host_prep_s:.1f} s, {sum(len(i.linelist) for i in inps)} lines)")
    import torch
    import build as korg_build
    from korg_gb300 import _lib
    from korg_gb300.batch import BatchSynthesis
    korg_build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nwl, L, n = len(inps[0].wls), len(inps[0].T), len(inps)
    # one chunk: every spectrum's alpha and line scratch resident at once
    b = BatchSynthesis(inps, precision="mixed", use_graph=True, autotune=True, max_scratch_bytes=160 << 30)
    stream = torch.cuda.current_stream(dev)
    _progress("inputs resident on the device")
    for w in range(max(args.warmup, 3)):  # eager + autotune, capture, replay
        b.run(stream)
        torch.cuda.synchronize()
        _progress(f"warm-up {w} done")
    clk = Clocks(0)
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    torch.cuda.synchronize()
    clocks = clk.stop()
    ms = statistics.mean(times)
    _progress(f"timed steps done: {ms:.1f} ms per batch")
    flux_mixed, cntm_mixed = b.results()
    stats = b.ctx.stats()
    evals = stats.line_evals
    cfg = b.tile_config()
    # end to end: one pinned host->device copy of every input, the batch, flux back to the host
    out_host = torch.empty((n, nwl), dtype=torch.float64, pin_memory=True)
    e2e_t = []
    for _ in range(max(2, min(args.steps, 5))):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        b.upload()
        f, _ = b.run(stream)
        out_host.copy_(f, non_blocking=True)
        torch.cuda.synchronize()
        e2e_t.append(time.perf_counter() - t1)
    e2e_s = statistics.mean(e2e_t)
    assert np.array_equal(out_host.numpy(), flux_mixed)
    # stage times of one eager run (timing events are not part of the graph)
    b.ctx.check(b.ctx.lib.korg_set_batch_options(b.ctx.h, 0, 1, 160 << 30))
    b.ctx.check(b.ctx.lib.korg_set_timing(b.ctx.h, 1))
    b.run(stream)
    st = b.ctx.stats()
    b.ctx.check(b.ctx.lib.korg_set_timing(b.ctx.h, 0))
    peak = C.c_double(0)
    b.ctx.check(b.ctx.lib.korg_probe_flops(b.ctx.h, 0, C.byref(peak)))
    achieved = evals * FLOP_PER_EVAL / (st.ms_line_tile * 1e-3) / 1e12
    _progress("e2e and stage timing done")
    # plain FP64 and mixed on the first 8 spectra: speed-up and error of the mixed form
    sub = inps[:8]
    res = {}
    for prec in ("mixed", "fp64"):
        bs = BatchSynthesis(sub, precision=prec, use_graph=False, autotune=False, max_scratch_bytes=160 << 30)
        bs.run(stream)
        torch.cuda.synchronize()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        bs.run(stream)
        e1.record(stream)
        e1.synchronize()
        res[prec] = (e0.elapsed_time(e1), *bs.results())
        bs.ctx.close()
    fm, cm = res["mixed"][1], res["mixed"][2]
    f64, c64 = res["fp64"][1], res["fp64"][2]
    fp64 = {"spectra": len(sub), "spectra_per_s": 1000.0 * len(sub) / res["fp64"][0],
            "mixed_spectra_per_s": 1000.0 * len(sub) / res["mixed"][0],
            "mixed_speedup": res["fp64"][0] / res["mixed"][0],
            "mixed_max_rel_flux_err": float(np.max(np.abs(fm / f64 - 1))),
            "mixed_max_rectified_err": float(np.max(np.abs(fm / cm - f64 / c64))),
            "mixed_rectified_rms": float(np.sqrt(np.mean((fm / cm - f64 / c64) ** 2)))}
    _progress("FP64 comparison done")
    grad = None
    if not args.no_adjoint:
        b.ctx.check(b.ctx.lib.korg_set_batch_options(b.ctx.h, 1, 1, 160 << 30))
        grad = batch_gradient(b, stream, ms)
        _progress(f"batch gradient done: {grad['forward_and_gradient_ms']:.0f} ms")
    cpu = None
    if not args.no_cpu:
        threads = os.cpu_count() or 1
        v, dt, ev_cpu, info = cpu_sample_batch(inps[:4], threads)
        _progress("CPU sample done")
        cpu = {"value": v, "unit": "spectra/s", "cores": threads, "kind": "port", "sample": info,
               "evals_per_s": ev_cpu / dt, "seconds": dt}
    nchunk = 1
    out = {
        "metric": METRIC, "value": 1000.0 * n / ms, "unit": "spectra/s", "n_gpus": 1, "steps": args.steps,
        "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 profiles + f64 tau/flux (mixed)",
        "data": "synthetic (seeded line list and stand-in atmospheres)",
        "config": {"workload": f"batch of {n} spectra: 56 layers, Teff 3500-7000 K, logg 1-5, [M/H] -2.5..0.5, "
                               f"seeded random 20k-200k-line subsets of a 500k-line atomic + molecular list, "
                               f"15000-17000 A @ 0.005 A ({nwl} points); one step = the whole batch",
                   "precision": "mixed", "lines_per_spectrum": [len(i.linelist) for i in inps][:8] + ["..."],
                   "l2": f"batch alpha {8 * L * nwl * n / 1e9:.1f} GB >> L2", "graph": True, "tile": cfg,
                   "host_prep_s": host_prep_s, "host_prep_parts": prep_parts,
                   "chemistry": "device (korg_chemical_equilibrium, all atmospheres in one call)",
                   "continuum": "device (korg_continuum_absorption: Korg's terms but metal bound-free)"},
        "evals_per_step": evals, "evals_per_s": evals / (ms * 1e-3),
        "stages_ms": {"total_eager": st.ms_total, "line_tile_queue": st.ms_line_tile, "rt_all": st.ms_rt},
        "fp64": fp64,
        "gradient": grad,
        "roofline": {"bound": "fp32", "achieved": achieved, "peak": peak.value, "unit": "TFLOP/s",
                     "frac": achieved / peak.value, "traffic": None,
                     "kernel": "line_tile_queue_kernel<mixed> (one persistent launch over the batch)",
                     "algorithmic": f"{FLOP_PER_EVAL} FP32 flop x {evals} line-layer-lambda evals per launch",
                     "peak_source": "measured in-process (korg_probe_flops: FP32 FMA chains)"},
        "cpu_baseline": cpu,
        "e2e": {"value": n / e2e_s, "unit": "spectra/s", "h2d_bytes_per_step": b.h2d_bytes,
                "d2h_bytes_per_step": 8 * nwl * n},
        "gpu_launches": args.steps * (n * 14 + nchunk),
        "clocks": clocks,
    }
    print(json.dumps(out), flush=True)
    b.ctx.close()


def run_postprocess(args):
    """Post-processing of a stack of synthesised spectra, as a Fit loop does per evaluation:
    rotational broadening on the synthesis grid, then the Gaussian LSF onto the observed grid."""
    import numpy as np
    import torch
    import build as korg_build
    from korg_gb300 import _lib
    from korg_gb300.wavelengths import Wavelengths
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    korg_build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    nspec, vsini, eps, R = 64, 10.0, 0.6, 22_500.0
    g = Wavelengths((15000, 17000, 0.005))
    obs = Wavelengths((15100, 16900, 0.2)).all_wls
    nwl, nout = len(g), len(obs)
    rng = np.random.default_rng(0)
    host = torch.as_tensor(1 - 0.5 * rng.random((nspec, nwl)) ** 8).pin_memory()
    ctx = _lib.Context(0)
    w, o = torch.as_tensor(g.all_wls, device=dev), torch.as_tensor(obs, device=dev)
    tR = torch.tensor([R], dtype=torch.float64, device=dev)
    rg = (_lib.WlRange * len(g.ranges))(*[_lib.WlRange(n, a, b) for a, b, n in g.ranges])
    flux = host.to(dev)
    rot = torch.empty_like(flux)
    out = torch.empty((nspec, nout), dtype=torch.float64, device=dev)
    out_host = torch.empty((nspec, nout), dtype=torch.float64).pin_memory()
    stream = torch.cuda.current_stream(dev)

    def step():
        ctx.check(ctx.lib.korg_apply_rotation_dev(ctx.h, w.data_ptr(), nwl, rg, len(g.ranges), vsini, eps,
                                                  flux.data_ptr(), nspec, rot.data_ptr(), stream.cuda_stream))
        ctx.check(ctx.lib.korg_apply_lsf_dev(ctx.h, w.data_ptr(), nwl, o.data_ptr(), nout, tR.data_ptr(), 1, 4.0,
                                             rot.data_ptr(), nspec, out.data_ptr(), stream.cuda_stream))

    for _ in range(max(args.warmup, 3)):
        step()
    torch.cuda.synchronize()
    clk = Clocks(0)
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        step()
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clocks = clk.stop()
    ms = statistics.mean(times)
    # end to end: host stack in, observed-grid spectra out
    e2e = []
    for _ in range(max(2, args.steps)):
        torch.cuda.synchronize()
        t1 = time.perf_counter()
        flux.copy_(host, non_blocking=True)
        step()
        out_host.copy_(out, non_blocking=True)
        torch.cuda.synchronize()
        e2e.append(time.perf_counter() - t1)
    e2e_s = statistics.mean(e2e)
    # CPU: the FP64 restatement, one spectrum per host core (spawn pool): the Gaussian LSF of the
    # whole spectrum, and the rotation of a quarter of its grid (a uniform grid and one vsini: the
    # rotation's cost per point is the same everywhere), timed wall-clock per phase
    import multiprocessing as mp
    threads = os.cpu_count() or 1
    with mp.get_context("spawn").Pool(threads) as pool:
        pool.map(_oracle_postprocess, [("lsf", 0, 1.0)] * threads, chunksize=1)  # workers up and imported
        t1 = time.perf_counter()
        pool.map(_oracle_postprocess, [("rotation", k, 0.25) for k in range(threads)], chunksize=1)
        t_rot = (time.perf_counter() - t1) / 0.25
        t1 = time.perf_counter()
        pool.map(_oracle_postprocess, [("lsf", k, 1.0) for k in range(threads)], chunksize=1)
        t_lsf = time.perf_counter() - t1
    cpu_value = threads / (t_rot + t_lsf)
    out_json = {"metric": METRIC, "value": nspec * 1000.0 / ms, "unit": "spectra/s (post-processing)", "n_gpus": 1,
                "steps": args.steps, "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded spectra)",
                "config": {"workload": f"{nspec} spectra on 15000-17000 A @ 0.005 A ({nwl} points): rotation "
                                       f"(vsini {vsini} km/s, eps {eps}) then Gaussian LSF R={R:.0f} onto "
                                       f"15100-16900 A @ 0.2 A ({nout} points)",
                           "l2": f"stack {8 * nspec * nwl / 1e6:.0f} MB > L2"},
                "e2e": {"value": nspec / e2e_s, "unit": "spectra/s (post-processing)",
                        "h2d_bytes_per_step": 8 * nspec * nwl, "d2h_bytes_per_step": 8 * nspec * nout},
                "gpu_launches": 2,
                "cpu_baseline": {"value": cpu_value, "unit": "spectra/s (post-processing)", "cores": threads,
                                 "kind": "port", "sample": f"{threads} spectra, one per core (numpy restatement): "
                                                           "the LSF of each whole spectrum and the rotation of a "
                                                           "quarter of its grid, scaled by 4"},
                "clocks": clocks}
    print(json.dumps(out_json), flush=True)
    ctx.close()


def run_variants(args):
    import numpy as np
    import torch
    import build as korg_build
    from korg_gb300 import synthetic
    from korg_gb300.batch import BatchSynthesis
    korg_build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    t0 = time.perf_counter()
    _progress("preparing the 1M-line cool giant")
    with warnings.catch_warnings():
        warnings.simplefilter("ignore")
        base = synthetic.prepare(synthetic.config4(), continuum="gpu", chemistry="gpu")
    inps = synthetic.abundance_variants(base, 16)
    host_prep_s = time.perf_counter() - t0
    nwl, L = len(base.wls), len(base.T)
    b = BatchSynthesis(inps, precision="mixed", use_graph=True, autotune=True, max_scratch_bytes=160 << 30)
    stream = torch.cuda.current_stream(dev)
    for w in range(max(args.warmup, 3)):
        b.run(stream)
        torch.cuda.synchronize()
        _progress(f"warm-up {w} done")
    clk = Clocks(0)
    times = []
    for _ in range(args.steps):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        b.run(stream)
        e1.record(stream)
        e1.synchronize()
        times.append(e0.elapsed_time(e1))
    clocks = clk.stop()
    ms = statistics.mean(times)
    evals = b.ctx.stats().line_evals
    fm, cm = b.results()
    _progress(f"timed: {ms:.1f} ms per batch of 16")
    # plain FP64 of the first variant
    one = BatchSynthesis(inps[:1], precision="fp64", use_graph=False, max_scratch_bytes=160 << 30)
    one.run(stream)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    one.run(stream)
    e1.record(stream)
    e1.synchronize()
    t64 = e0.elapsed_time(e1)
    f64, c64 = one.results()
    one.ctx.close()
    grad = None if args.no_adjoint else batch_gradient(b, stream, ms)
    out = {"metric": METRIC, "value": 16 * 1000.0 / ms, "unit": "spectra/s", "n_gpus": 1, "steps": args.steps,
           "warmup": max(args.warmup, 3), "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32 profiles + f64 tau/flux (mixed)",
           "data": "synthetic (seeded line list and stand-in atmosphere)",
           "config": {"workload": f"16 abundance variants (n/U rows scaled by 10^U(-0.3, 0.3) dex per species) of an "
                                  f"80-layer Teff 3500 logg 1.0 atmosphere, {len(base.linelist)} lines (40% atomic, "
                                  f"60% TiO/CO/OH/CN), 3000-10000 A @ 0.01 A ({nwl} points); one step = the batch",
                      "tile": b.tile_config(), "host_prep_s": host_prep_s},
           "evals_per_step": evals, "evals_per_s": evals / (ms * 1e-3),
           "fp64": {"spectra_per_s": 1000.0 / t64, "mixed_speedup": (t64 / 1.0) / (ms / 16),
                    "mixed_max_rel_flux_err": float(np.max(np.abs(fm[0] / f64[0] - 1))),
                    "mixed_rectified_rms": float(np.sqrt(np.mean((fm[0] / cm[0] - f64[0] / c64[0]) ** 2)))},
           "gradient": grad, "clocks": clocks}
    print(json.dumps(out), flush=True)


class AdjointCase:
    """The adjoint configuration (72 layers, Teff 4500 K, logg 2.5, [M/H] -0.5, 50k atomic + 20k
    CO/OH/CN lines, 15000-17000 A at 0.005 A) resident on the device: forward synthesis, and
    forward + rectified-flux loss + korg_synthesize_vjp_dev against a seeded observation (the
    same star with log gf perturbed by N(0, 0.1) dex)."""

    def __init__(self, ctx, torch, dev, scale=1.0):
        import copy
        import numpy as np
        from korg_gb300 import _lib, synthetic
        from korg_gb300.api import synthesize_prepared
        self.torch, self.ctx, self.lib = torch, ctx, _lib
        with warnings.catch_warnings():
            warnings.simplefilter("ignore")
            inp = synthetic.prepare(synthetic.config2(n_atomic=int(50_000 * scale), n_mol=int(20_000 * scale)),
                                    continuum="gpu", chemistry="gpu", ctx=ctx)
        self.inp = inp
        self.nwl, L = len(inp.wls), len(inp.T)
        ctx.ensure_stark()
        o = copy.copy(inp)
        o.linelist = copy.copy(inp.linelist)
        o.linelist.log_gf = inp.linelist.log_gf + np.random.default_rng(1).normal(0, 0.1, len(inp.linelist))
        r = synthesize_prepared(o, precision="fp64", ctx=ctx)
        self.obs = torch.as_tensor(r.flux / r.cntm, device=dev)
        self.s, self.l1, self.l5, self.w, self.keep = dev_inputs(inp, torch, dev)
        self.flux = torch.empty(self.nwl, dtype=torch.float64, device=dev)
        self.cntm = torch.empty_like(self.flux)
        shapes = {"T": L, "ne": L, "n_eff_vdW": L, "xi": L, "n_div_U": inp.n_div_U.size, "nH_I": L, "nHe_I": L,
                  "UH_I": L, "log_gf": len(inp.linelist), "cntm_vals": inp.cntm_vals.size, "alpha_ref_cntm": L}
        self.gt = {k: torch.empty(n, dtype=torch.float64, device=dev) for k, n in shapes.items()}
        self.grads = _lib.SynthGrads(*[C.cast(self.gt[k].data_ptr(), _lib._dp) for k in shapes])
        self.stream = torch.cuda.current_stream(dev)

    def forward(self, prec):
        c = self.ctx
        c.check(c.lib.korg_synthesize_dev(c.h, C.byref(self.s), C.byref(self.l1), C.byref(self.l5), self.w.data_ptr(),
                                          self.nwl, prec, self.flux.data_ptr(), self.cntm.data_ptr(), None,
                                          self.stream.cuda_stream))

    def step(self, prec, flags=None):
        """loss and its gradient w.r.t. every hot-path input"""
        flags = self.lib.KORG_VJP_HYDROGEN if flags is None else flags
        self.forward(prec)
        flux, cntm, c = self.flux, self.cntm, self.ctx
        rr = flux / cntm - self.obs
        dF = 2 * rr / cntm
        dC = -2 * rr * flux / cntm ** 2
        c.check(c.lib.korg_synthesize_vjp_dev(c.h, C.byref(self.s), C.byref(self.l1), C.byref(self.l5),
                                              self.w.data_ptr(), self.nwl, prec, dF.data_ptr(), dC.data_ptr(),
                                              C.byref(self.grads), flags, self.stream.cuda_stream))
        return self.torch.sum(rr * rr)

    def timed(self, fn, reps):
        fn()
        self.torch.cuda.synchronize()
        ts = []
        for _ in range(reps):
            e0, e1 = self.torch.cuda.Event(enable_timing=True), self.torch.cuda.Event(enable_timing=True)
            e0.record(self.stream)
            fn()
            e1.record(self.stream)
            e1.synchronize()
            ts.append(e0.elapsed_time(e1))
        return statistics.mean(ts)

    def grads_host(self):
        return {k: v.cpu().numpy().copy() for k, v in self.gt.items()}

    def vjp_stages(self, prec):
        c = self.ctx
        c.check(c.lib.korg_set_timing(c.h, 1))
        self.step(prec)
        self.torch.cuda.synchronize()
        st = c.stats()
        c.check(c.lib.korg_set_timing(c.h, 0))
        return {"alpha_recompute": st.ms_vjp_alpha, "rt_adjoint": st.ms_vjp_rt, "hydrogen": st.ms_vjp_hydrogen,
                "lines": st.ms_vjp_lines}


def adjoint_measure(ctx, torch, dev, steps=5):
    """Cost of the gradient on the adjoint configuration (mixed precision), for the default line:
    forward alone, forward + loss + gradient, and the same reusing the forward's opacity."""
    a = AdjointCase(ctx, torch, dev)
    mixed = a.lib.KORG_MIXED
    t_fwd = a.timed(lambda: a.forward(mixed), steps)
    t_step = a.timed(lambda: a.step(mixed), steps)
    reuse = a.lib.KORG_VJP_HYDROGEN | a.lib.KORG_VJP_REUSE_FORWARD
    t_reuse = a.timed(lambda: a.step(mixed, reuse), steps)
    stages = a.vjp_stages(mixed)
    _progress(f"adjoint: forward {t_fwd:.1f} ms, forward + gradient {t_step:.1f} ms")
    return {"workload": f"72 layers, Teff 4500 logg 2.5 [M/H] -0.5, {len(a.inp.linelist)} lines (50k atomic + 20k "
                        f"CO/OH/CN), 15000-17000 A @ 0.005 A ({a.nwl} points), mixed precision; loss = sum of squared "
                        "rectified-flux residuals; gradient w.r.t. T, ne, n_eff_vdW, xi, n/U, log gf, continuum "
                        "knots, alpha_ref continuum, H-line inputs",
            "steps": steps, "forward_ms": t_fwd, "forward_and_gradient_ms": t_step,
            "gradient_over_forward": (t_step - t_fwd) / t_fwd, "vjp_stages_ms": stages,
            "reuse_forward": {"step_ms": t_reuse, "gradient_over_forward": (t_reuse - t_fwd) / t_fwd}}


def configs_vs_oracle(ctx, threads):
    """The plain FP64 and mixed GPU syntheses of the other configurations over their whole grids,
    compared with the FP64 oracle on a strided subset of the same grid (every 20th point of the
    0.005 A infrared grids, every 50th of the 0.01 A optical one)."""
    from korg_gb300 import synthetic
    from korg_gb300.api import synthesize_prepared
    gpu = dict(continuum="gpu", chemistry="gpu", ctx=ctx)
    warnings.simplefilter("ignore")  # the grey atmospheres' n_e differ from Korg's: expected
    cases = [("cfg2_adjoint_forward", lambda: synthetic.prepare(synthetic.config2(), **gpu), 0.1),
             ("cfg3_batch_spectrum0", lambda: synthetic.prepare(synthetic.config3(n_spectra=1)[0], **gpu), 0.1),
             ("cfg4_cool_star_variant0",
              lambda: synthetic.abundance_variants(synthetic.prepare(synthetic.config4(), **gpu), 1)[0], 0.5)]
    out = {}
    ctx.ensure_stark()
    for name, make, step in cases:
        inp = make()
        res = {}
        ctx.check(ctx.lib.korg_set_timing(ctx.h, 1))
        for prec in ("fp64", "mixed"):
            r = synthesize_prepared(inp, precision=prec, ctx=ctx)
            res[prec] = (r.flux, r.cntm, ctx.stats().ms_total)
        ctx.check(ctx.lib.korg_set_timing(ctx.h, 0))
        sub, stride = strided(inp, step)
        of, oc, ev, dt = oracle_flux(sub, threads)
        e64 = flux_errors(res["fp64"][0][::stride], res["fp64"][1][::stride], of, oc)
        e32 = flux_errors(res["mixed"][0][::stride], res["mixed"][1][::stride], of, oc)
        out[name] = {"lines": len(inp.linelist), "layers": len(inp.T), "points": len(inp.wls),
                     "compared_points": len(of), "fp64_max_rel_flux_err_vs_oracle": e64["max_rel_flux_err"],
                     "mixed_max_rel_flux_err_vs_oracle": e32["max_rel_flux_err"],
                     "mixed_rectified_rms_vs_oracle": e32["rectified_rms"],
                     "mixed_max_rectified_err_vs_oracle": e32["max_rectified_err"],
                     "gpu_fp64_ms": res["fp64"][2], "gpu_mixed_ms": res["mixed"][2], "oracle_s": dt}
        _progress(f"{name}: fp64 vs oracle {e64['max_rel_flux_err']:.2e}, mixed {e32['max_rel_flux_err']:.2e}")
    return out


def run_adjoint(args):
    import numpy as np
    import torch
    import build as korg_build
    from korg_gb300 import _lib
    korg_build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    _progress("preparing the adjoint configuration")
    ctx = _lib.Context(0)
    a = AdjointCase(ctx, torch, dev, args.adj_scale)
    inp, nwl = a.inp, a.nwl
    _progress("inputs resident")
    res = {}
    for name, prec in (("mixed", _lib.KORG_MIXED), ("fp64", _lib.KORG_FP64)):
        reps = args.steps if name == "mixed" else 1
        t_fwd = a.timed(lambda: a.forward(prec), reps)
        clk = Clocks(0) if name == "mixed" else None
        t_step = a.timed(lambda: a.step(prec), reps)
        clocks = clk.stop() if clk else None
        res[name] = (t_fwd, t_step, a.grads_host(), clocks)
        _progress(f"{name}: forward {t_fwd:.1f} ms, forward + gradient {t_step:.1f} ms")
    # stage times of one mixed step, and the step with the forward's opacity reused
    reuse = _lib.KORG_VJP_HYDROGEN | _lib.KORG_VJP_REUSE_FORWARD
    t_reuse = a.timed(lambda: a.step(_lib.KORG_MIXED, reuse), args.steps)
    g_reuse = a.grads_host()
    vjp_stages = a.vjp_stages(_lib.KORG_MIXED)
    stats = ctx.stats()
    g32, g64 = res["mixed"][2], res["fp64"][2]
    reuse_same = all(np.allclose(g_reuse[k], g32[k], rtol=1e-6, atol=0) for k in g32)
    agree = {k: float(np.max(np.abs(g32[k] - g64[k])) / max(np.max(np.abs(g64[k])), 1e-300))
             for k in ("T", "ne", "n_eff_vdW", "xi", "n_div_U", "log_gf", "nH_I", "UH_I")}
    t_fwd, t_step = res["mixed"][0], res["mixed"][1]
    out = {"metric": METRIC, "value": 1000.0 / t_step, "unit": "gradient steps/s (forward + loss + VJP)",
           "n_gpus": 1, "steps": args.steps, "warmup": 1, "ms_per_step": t_step, "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f32 profiles + f64 tau/flux (mixed)",
           "data": "synthetic (seeded line list and stand-in atmosphere)",
           "config": {"workload": f"adjoint: 72 layers, Teff 4500 logg 2.5 [M/H] -0.5, {len(inp.linelist)} lines "
                                  f"({round(50 * args.adj_scale, 1):g}k atomic + {round(20 * args.adj_scale, 1):g}k "
                                  f"CO/OH/CN), 15000-17000 A @ 0.005 A ({nwl} points); loss = "
                                  "sum of squared rectified-flux residuals; gradient w.r.t. T, ne, n_eff_vdW, xi, "
                                  "n/U, log gf, continuum, H-line inputs"},
           "forward_ms": t_fwd, "gradient_over_forward": (t_step - t_fwd) / t_fwd, "vjp_stages_ms": vjp_stages,
           "reuse_forward": {"step_ms": t_reuse, "gradient_over_forward": (t_reuse - t_fwd) / t_fwd,
                             "same_gradient": bool(reuse_same)},
           "fp64": {"forward_ms": res["fp64"][0], "step_ms": res["fp64"][1],
                    "gradient_over_forward": (res["fp64"][1] - res["fp64"][0]) / res["fp64"][0],
                    "mixed_step_speedup": res["fp64"][1] / t_step},
           "mixed_vs_fp64_gradient_max_rel": agree, "line_evals": stats.line_evals,
           "clocks": res["mixed"][3]}
    print(json.dumps(out), flush=True)
    ctx.close()


def run_chemistry(args):
    """Chemical equilibrium of every layer of a set of stars (--spectra stars, up to 16; 1: the
    5777 K star alone), one batched korg_chemical_equilibrium_dev call per step."""
    import torch
    import build as korg_build
    from korg_gb300 import _lib
    korg_build.build()
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    ctx = _lib.Context(0)
    n = max(1, min(args.spectra, len(CHEM_STARS)))
    clk = Clocks(0)
    r = chemistry_measure(ctx, torch, dev, os.cpu_count() or 1, n_stars=n, steps=args.steps,
                          warmup=max(args.warmup, 1), cpu=not args.no_cpu and n > 1)
    clocks = clk.stop()
    out = {"metric": "chemical-equilibrium layers/s", "value": r["layers_per_s"], "unit": "layers/s", "n_gpus": 1,
           "steps": args.steps, "warmup": max(args.warmup, 1), "ms_per_step": r["ms"], "higher_is_better": True,
           "scaling": "weak", "vs_baseline": None, "dtype": "f64 (FP32 factors + FP64 refinement)", "data": "synthetic",
           "config": {"workload": f"{n} star(s) x 56 layers, 306 molecules, one batched call per step"},
           "chemical_equilibrium": r, "gpu_launches": args.steps, "clocks": clocks}
    print(json.dumps(out), flush=True)
    ctx.close()


if __name__ == "__main__":
    a = parse()
    if a.steps is None:
        a.steps = 3 if a.workload == "batch" else 20
    if a.impl == "reference":
        run_reference(a)
    elif a.workload == "chemistry":
        run_chemistry(a)
    elif a.workload == "batch":
        run_batch(a)
    elif a.workload == "postprocess":
        run_postprocess(a)
    elif a.workload == "adjoint":
        run_adjoint(a)
    elif a.workload == "variants":
        run_variants(a)
    else:
        run_korg(a)
