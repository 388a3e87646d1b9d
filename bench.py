#!/usr/bin/env python3
"""MB-pol molecular-dynamics throughput on one GB300.

Workload (default): 4096 waters in a 4.967 nm cubic box (jittered 16^3
lattice, seeded; mbpol_openmm_plugin_gb300.systems.workload("box4096")),
the full MB-pol model (1B, 2B, 3B, electrostatics with PME at a 0.9 nm
real-space cutoff and Ewald tolerance 1e-5, induced dipoles converged to
1e-8 D, dispersion), NVE velocity Verlet at 0.2 fs.  A "step" is one MD step:
one full force/energy evaluation plus the integration.

  value  ns/day with everything resident in HBM (mbpol_md_run; CUDA events
         on the library's stream around the K timed steps)
  e2e    ns/day through the public API with host buffers: every step copies
         positions host->device (mbpol_set_positions), evaluates, and copies
         forces and energies device->host (mbpol_compute); the integration is
         done on the host, as OpenMM drives the reference plugin.

Inputs (positions, velocities) are ~0.4 MB; the per-step working set is a few
hundred MB of pair/trimer buffers and PME grids, larger than L2 only in part,
so config["l2"] states that no flush is done between steps.

--impl reference times the reference's algorithm on the host cores: the
oracle's C port (the reference's own CPU code cannot be built on the GPU
host) over a bounded sample of the same workload, extrapolated to one step.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

DT_PS = 0.0002  # 0.2 fs


def ns_per_day(seconds_per_step):
    return DT_PS * 1e-3 * 86400.0 / seconds_per_step


class ClockSampler:
    """nvidia-smi SM clock / throttle reasons sampled during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown," \
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, gpu=0):
        self.gpu = gpu
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.gpu), "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 6:
                continue
            try:
                sm.append(float(parts[0]))
                mx.append(float(parts[1]))
            except ValueError:
                continue
            for nm, v in zip(names, parts[2:6]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def build_workload(name, seed, guess, model="reference"):
    """model "reference": the reference's trimer rule and PME permanent field
    (parity); "physical": every trimer with a nonzero switch and the
    consistent PME field, for which forces are -dE/dx."""
    import mbpol_openmm_plugin_gb300 as mb
    from mbpol_openmm_plugin_gb300 import systems
    ws = systems.workload(name, seed)
    alpha, grid = mb.pme_parameters(ws.box, 0.9, 1e-5)
    phys = 1 if model == "physical" else 0
    sysm = mb.create_mbpol_system(ws, ewald_alpha=alpha, pme_grid=grid, ewald_tol=1e-5, target_epsilon=1e-8,
                                  guess=guess, trimer_rule=phys, pme_fixed_field=phys)
    return ws, sysm, alpha, grid


def maxwell_boltzmann(masses, T, seed):
    rng = np.random.default_rng(seed + 7)
    kT = 0.00831446261815324 * T
    v = np.zeros((len(masses), 3))
    for i, m in enumerate(masses):
        if m > 0:
            v[i] = rng.normal(0.0, np.sqrt(kT / m), 3)
    return v


# Algorithmic work per unit (reference operation counts, one flop per add or
# multiply, counted in poly-2b-v6x.cpp / poly-3b-v2x.cpp plus the variables,
# switch and chain rule around them): these stay fixed whatever the kernels do.
ALGO_FLOP_PER_UNIT = {"poly2b": 31200, "poly3b": 112600}
# DRAM bytes (dram__bytes_read.sum + dram__bytes_write.sum) of one launch of
# each polynomial kernel on box4096, measured with ncu --set full
# (profiles/poly_tc5_kernel_box4096.md, profiles/poly_df_kernel_box4096.md),
# and the units that launch processed; the traffic of a launch is scaled by
# its unit count.
NCU_TRAFFIC = {"poly3b": (60.182e6 + 354.333e6, 182343), "poly2b": (16.451e6, 65434)}


GUESS_MODE = {"plain": 1, "learned": 2, "extrapolation": 3}
GUESS_WEIGHTS = os.path.join(ROOT, "mbpol_openmm_plugin_gb300", "data", "dipole_guess_%s.npy")


def guess_params_source(args):
    path = GUESS_WEIGHTS % args.workload
    if not os.path.exists(path) and args.workload.startswith("box"):
        path = GUESS_WEIGHTS % "box4096"
    return "committed (%s)" % os.path.relpath(path, ROOT) if os.path.exists(path) else \
        "trained in this run on 200 NVT frames"


def guess_params(args):
    """The learned guess's parameter block: the committed one for the
    workload (trained by mbpol_openmm_plugin_gb300.train_guess on 2000 NVT
    frames of the same box), else one trained here on a short trajectory.
    A bulk box without its own block uses the 4096-water box's network (its
    inputs are per-molecule and local, plus the permanent field)."""
    path = GUESS_WEIGHTS % args.workload
    if not os.path.exists(path) and args.workload.startswith("box"):
        path = GUESS_WEIGHTS % "box4096"
    if os.path.exists(path):
        return np.load(path), guess_params_source(args)
    out = os.path.join("/tmp", "dipole_guess_%s_%d.npy" % (args.workload, os.getpid()))
    from mbpol_openmm_plugin_gb300 import train_guess
    train_guess.main(["--workload", args.workload, "--frames", "200", "--steps", "5000", "--out", out])
    return np.load(out), "trained in this run on 200 NVT frames"


CORRECTION_WEIGHTS = os.path.join(ROOT, "mbpol_openmm_plugin_gb300", "data", "dipole_correction_%s.npy")


def correction_params(args):
    """The correction network's parameter block for the learned arm (trained
    by mbpol_openmm_plugin_gb300.train_guess --network correction on NVT
    frames of the same box), or None."""
    path = CORRECTION_WEIGHTS % args.workload
    if not os.path.exists(path) and args.workload.startswith("box"):
        path = CORRECTION_WEIGHTS % "box4096"
    return np.load(path) if os.path.exists(path) and not args.no_correction else None


def md_context(args, guess, params=None, corr=None):
    """A context of the workload at the trajectory start every arm shares:
    the seeded box with Maxwell-Boltzmann velocities, `args.equilibrate`
    untimed MD steps (the history-based guesses reach their steady state
    after 12 solves), then the warm-up steps (first force evaluation, buffer
    growth).  Two contexts built alike reach the same state to ~1e-5 nm after
    200 steps (the forces are summed with FP64 atomics in no fixed order;
    e2e reports the difference)."""
    import mbpol_openmm_plugin_gb300 as mb
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    ws, sysm, alpha, grid = build_workload(args.workload, args.seed, GUESS_MODE[guess], args.model)
    ctx = mb.Context(sysm)
    ctx.setPositions(ws.positions)
    ctx._build()
    if params is not None:
        ctx.setDipoleGuessParameters(params)
    if corr is not None:
        ctx.selectDipoleGuessNetwork(ctx.CorrectionNetwork)
        ctx.setDipoleGuessParameters(corr)
        ctx.selectDipoleGuessNetwork(ctx.ColdStartNetwork)
    h = ctx._h
    box = np.ascontiguousarray(ws.box, np.float64)
    pos = np.ascontiguousarray(ws.positions, np.float64)
    masses = np.array(sysm.masses)
    vel = maxwell_boltzmann(masses, 300.0, args.seed)
    _capi.check(lib.mbpol_set_positions(h, _capi.ptr(pos), _capi.ptr(box)))
    _capi.check(lib.mbpol_set_masses(h, _capi.ptr(np.ascontiguousarray(masses))))
    _capi.check(lib.mbpol_set_velocities(h, _capi.ptr(np.ascontiguousarray(vel))))
    # the autotuner measures its 12 candidate launch shapes (3 steps each)
    # during the untimed equilibration steps
    _capi.check(lib.mbpol_set_autotune(h, 3 if getattr(args, "autotune", True) and args.equilibrate >= 36 else 0))
    ms, iters, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    _capi.check(lib.mbpol_md_run(h, args.equilibrate + args.warmup, DT_PS, 0.0, 0.0, args.seed, ctypes.byref(ms),
                                 _capi.ptr(en), ctypes.byref(iters)))
    return {"ctx": ctx, "h": h, "ws": ws, "sysm": sysm, "alpha": alpha, "grid": grid, "box": box,
            "masses": masses, "n": pos.shape[0]}


def launch_shape(lib, h):
    """The polynomial kernels' launch shape in use (mbpol_get_launch_shape)."""
    a, b, t = ctypes.c_int(), ctypes.c_int(), ctypes.c_int()
    lib.mbpol_get_launch_shape(h, ctypes.byref(a), ctypes.byref(b), ctypes.byref(t))
    return {"tensor_kernel_free_sms": a.value, "walk_free_blocks": b.value, "autotuned": bool(t.value)}


def md_steps(lib, h, nsteps, seed):
    """nsteps device-resident MD steps; (seconds per step from CUDA events on
    the library's stream, solver iterations per step, energies)."""
    from mbpol_openmm_plugin_gb300 import _capi
    ms, iters, en = ctypes.c_double(), ctypes.c_long(), np.zeros(6)
    _capi.check(lib.mbpol_md_run(h, nsteps, DT_PS, 0.0, 0.0, seed, ctypes.byref(ms), _capi.ptr(en),
                                 ctypes.byref(iters)))
    return ms.value / 1e3 / nsteps, iters.value / nsteps, en


def state(lib, h, n):
    from mbpol_openmm_plugin_gb300 import _capi
    pos, vel, f = np.zeros((n, 3)), np.zeros((n, 3)), np.zeros((n, 3))
    _capi.check(lib.mbpol_get_state(h, _capi.ptr(pos), _capi.ptr(vel), _capi.ptr(f)))
    return pos, vel, f


def arm(args, guess, params=None, corr=None):
    """One guess arm: K timed steps, then the metric's iteration average over
    `args.avg_steps` further steps of the same trajectory."""
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    c = md_context(args, guess, params, corr)
    step_s, it, _ = md_steps(lib, c["h"], args.steps, args.seed)
    out = {"ns_per_day": ns_per_day(step_s), "ms_per_step": step_s * 1e3, "solver_iterations_per_step": it,
           "launch_shape": launch_shape(lib, c["h"])}
    if args.avg_steps > 0:
        sl, itl, _ = md_steps(lib, c["h"], args.avg_steps, args.seed)
        out["long_run"] = {"steps": args.avg_steps, "ms_per_step": sl * 1e3, "ns_per_day": ns_per_day(sl),
                           "solver_iterations_per_step": itl}
    del c
    return out


def e2e_steps(lib, c, nsteps):
    """The same steps through the public API with host buffers, as OpenMM
    drives the reference plugin: every step copies the positions host->device
    (mbpol_set_positions), evaluates (mbpol_compute: energies and forces
    copied device->host) and integrates on the host (velocity Verlet)."""
    from mbpol_openmm_plugin_gb300 import _capi
    h, n, box = c["h"], c["n"], c["box"]
    hpos, hvel, forces = state(lib, h, n)
    masses = c["masses"]
    invm = np.where(masses > 0, 1.0 / np.where(masses > 0, masses, 1.0), 0.0)[:, None]
    e5 = np.zeros(5)
    t0 = time.perf_counter()
    for _ in range(nsteps):
        hvel += 0.5 * DT_PS * forces * invm
        hpos += DT_PS * hvel * (invm > 0)
        _capi.check(lib.mbpol_set_positions(h, _capi.ptr(hpos), _capi.ptr(box)))
        forces[:] = 0.0
        _capi.check(lib.mbpol_compute(h, _capi.ALL_TERMS, _capi.ptr(e5), _capi.ptr(forces)))
        hvel += 0.5 * DT_PS * forces * invm
    return (time.perf_counter() - t0) / nsteps, hpos


METRIC = "ns/day @4096 H2O PME, learned-guess vs plain GPU at <=1e-4 rel RMS force err"


def run_ours(args):
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    params, params_src = guess_params(args)
    corr = correction_params(args)
    # comparison arms first (each from the same trajectory start); the
    # learned arm without its correction network shows what the network adds
    others = {}
    for g in ("plain", "extrapolation", "learned"):
        if g != args.guess and not args.no_comparison:
            others[g] = arm(args, g, params if g == "learned" else None, corr if g == "learned" else None)
    if args.guess == "learned" and corr is not None and not args.no_comparison:
        others["learned_predictor_only"] = arm(args, "learned", params, None)
    # headline arm: context A times K device-resident steps (value), context
    # B, built and advanced alike, times the same K steps end to end (e2e)
    gp = params if args.guess == "learned" else None
    gc = corr if args.guess == "learned" else None
    ca = md_context(args, args.guess, gp, gc)
    cb = md_context(args, args.guess, gp, gc)
    h = ca["h"]
    # both contexts run the shape the autotuner chose for the first
    shape = launch_shape(lib, h)
    _capi.check(lib.mbpol_set_launch_shape(cb["h"], shape["tensor_kernel_free_sms"], shape["walk_free_blocks"]))
    pa, va, _ = state(lib, h, ca["n"])
    pb, vb, _ = state(lib, cb["h"], cb["n"])
    same_start = float(max(np.abs(pa - pb).max(), np.abs(va - vb).max()))
    sampler = ClockSampler()
    sampler.start()
    l0 = lib.mbpol_launch_count()
    step_s, solver_it, en = md_steps(lib, h, args.steps, args.seed)
    launches = int(lib.mbpol_launch_count() - l0)
    clocks = sampler.stop()
    e2e_s, pos_e2e = e2e_steps(lib, cb, args.steps)
    pos_dev, _, _ = state(lib, h, ca["n"])
    # atoms only: the host loop does not move the M sites, which the library
    # places from their waters at every evaluation
    atoms = ca["masses"] > 0
    same_end = float(np.abs(pos_dev[atoms] - pos_e2e[atoms]).max())
    counts_timed = ca["ctx"].getCounts()
    # per-kernel CUDA-event timers on K further steps (the events add
    # launches, so the timed steps above run without them); unit counts from
    # those same steps
    lib.mbpol_profile_enable(1)
    md_steps(lib, h, args.steps, args.seed)
    kern = {}
    for kid, kname in enumerate(_capi.KERNELS):
        t, nl = ctypes.c_double(), ctypes.c_long()
        lib.mbpol_profile_read(kid, ctypes.byref(t), ctypes.byref(nl))
        kern[kname] = {"total_ms": t.value, "launches": nl.value}
    lib.mbpol_profile_enable(0)
    counts = ca["ctx"].getCounts()
    long_run = None
    if args.avg_steps > 0:
        sl, itl, _ = md_steps(lib, h, args.avg_steps, args.seed)
        long_run = {"steps": args.avg_steps, "ms_per_step": sl * 1e3, "ns_per_day": ns_per_day(sl),
                    "solver_iterations_per_step": itl}
    drift = nve_drift(lib, h, args.drift_steps, ca["n"] // 4) if args.drift_steps > 0 else None
    ws, alpha, grid, n = ca["ws"], ca["alpha"], ca["grid"], ca["n"]
    value = ns_per_day(step_s)
    head = {"ns_per_day": value, "ms_per_step": step_s * 1e3, "solver_iterations_per_step": solver_it}
    if long_run:
        head["long_run"] = long_run
    arms = dict(others, **{args.guess: head})
    arms_ms = {g: round(a["ms_per_step"], 3) for g, a in arms.items()}
    if "plain" in arms:
        pl, hd = arms["plain"], arms[args.guess]
        arms_ms["%s_vs_plain" % args.guess] = round(pl["ms_per_step"] / hd["ms_per_step"], 3)
        if "long_run" in pl and "long_run" in hd:
            arms_ms["%s_vs_plain_long_run" % args.guess] = round(
                pl["long_run"]["ms_per_step"] / hd["long_run"]["ms_per_step"], 3)
    roof, secondary = rooflines(kern, counts, grid, n, clocks)
    out = {
        "metric": METRIC, "value": value, "unit": "ns/day", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": step_s * 1e3, "arms_ms_per_step": arms_ms, "higher_is_better": True, "scaling": "replicas",
        "vs_baseline": None,
        "dtype": "fp16 tensor-core pieces + fp32 sums (3B), double-float fp32 (2B), fp32 bulk, fp64 accumulation",
        "data": "synthetic (seeded lattice box)",
        "config": workload_config(args, ws, alpha, grid, params_src),
        "e2e": {"value": ns_per_day(e2e_s), "unit": "ns/day", "h2d_bytes_per_step": int(n * 24),
                "d2h_bytes_per_step": int(n * 24 + 5 * 8),
                "steps": "the same %d steps as value, from the same state (max |dx| at start %.1e nm, "
                         "of the atoms at the end %.1e nm)"
                         % (args.steps, same_start, same_end)},
        "gpu_launches": launches,
        "launch_shape": shape,
        "solver_iterations_per_step": solver_it,
        "guess_comparison": arms,
        "correction_network": "committed (%s)" % os.path.relpath(CORRECTION_WEIGHTS % "box4096", ROOT)
        if gc is not None else None,
        "counts": {"pairs_2b": int(counts[0]), "trimers": int(counts[1]), "elec_site_pairs": int(counts[2]),
                   "pme_grid_points": int(grid[0] * grid[1] * grid[2]) if grid else 0,
                   "trimers_in_timed_steps": int(counts_timed[1])},
        "kernels_ms_per_step": {k: v["total_ms"] / args.steps for k, v in kern.items()},
        "clocks": clocks,
        "roofline": roof,
        "roofline_memory_kernels": secondary,
        "energies_kJ_mol": {"1b": en[0], "2b": en[1], "3b": en[2], "elec": en[3], "disp": en[4], "kinetic": en[5]},
    }
    if drift is not None:
        out["nve_drift"] = drift
    del ca, cb
    if not args.no_accuracy:
        out["accuracy"] = accuracy_check()
    if not args.no_cpu_baseline:
        out["cpu_baseline"] = cpu_baseline(args, sample=True)
    return out


def profile_window(args):
    """The --guess arm's MD steps bracketed by cudaProfilerStart/Stop, so that
    a profiler started with --profile-from-start off sees only those steps'
    kernels (after the trajectory start and warm-up of md_context)."""
    from mbpol_openmm_plugin_gb300 import _capi
    lib = _capi.load()
    params, _ = guess_params(args)
    corr = correction_params(args) if args.guess == "learned" else None
    c = md_context(args, args.guess, params if args.guess == "learned" else None, corr)
    rt = None
    for name in ("libcudart.so.13", "libcudart.so"):
        try:
            rt = ctypes.CDLL(name)
            break
        except OSError:
            continue
    if rt is None:
        raise RuntimeError("the CUDA runtime library was not found")
    rt.cudaProfilerStart()
    l0 = lib.mbpol_launch_count()
    step_s, it, _ = md_steps(lib, c["h"], args.profile_window, args.seed)
    launches = int(lib.mbpol_launch_count() - l0)
    rt.cudaProfilerStop()
    return {"profile_window_steps": args.profile_window, "guess": args.guess, "ms_per_step": step_s * 1e3,
            "solver_iterations_per_step": it, "gpu_launches": launches, "counts": [int(v) for v in c["ctx"].getCounts()],
            "note": "timed under a profiler if one is attached: not a bench value"}


def workload_config(args, ws, alpha, grid, params_src):
    """The workload as both arms (ours and --impl reference) report it."""
    return {"workload": args.workload, "waters": int(ws.num_waters), "box_nm": float(ws.box[0]), "pme_alpha": alpha,
            "pme_grid": grid, "cutoff_nm": 0.9, "ewald_tol": 1e-5, "target_epsilon_D": 1e-8, "dt_fs": 0.2,
            "guess": args.guess, "guess_parameters": params_src, "seed": args.seed, "model": args.model,
            "equilibration_steps": args.equilibrate,
            "l2": "no flush: inputs larger than L2 (per step, the pair and trimer variable/gradient planes and "
                  "the PME grids exceed the 129 MB L2)"}


def tc_flop_per_trimer():
    """Executed tensor-core work of the three-body kernel (tcgen05) per
    trimer: blocks of S in the stream x 4 MMAs of M = 128 trimers, N = 64
    rows, K = 16 (2 flop per multiply-add), per 128-trimer tile."""
    try:
        import re
        src = open(os.path.join(ROOT, "mbpol_openmm_plugin_gb300", "_build", "poly_tc_tables.cpp")).read()
        nblk = int(re.search(r"poly3b_frag, \d+, \d+, (\d+),", src).group(1))
    except (OSError, AttributeError):
        nblk = 239
    return nblk * 4 * 2 * 128 * 64 * 16 / 128.0


def rooflines(kern, counts, grid, n, clocks):
    """The top kernel of the step's launch list, the three-body tensor
    kernel, against the measured tensor-core rate (executed tcgen05 work),
    with the FP32 view of the reference's operation count beside it; the
    two-body walk (nested) against the FP32 pipe.  The memory-bound
    electrostatics passes against the measured HBM copy rate (algorithmic
    bytes as in the reference's operation counts: pair index 4 B + cached
    pair coefficients 8 B per polarisable site pair within the cutoff, 36 B
    per polarisable site; PME pass: 125 grid updates of 4 B per site, 8 B per
    grid point for the FFT input and output, 16 B for the convolution).  The
    electrostatics timers run concurrently with the polynomial kernels, so
    their fractions are lower bounds."""
    sm_mhz = clocks.get("sm_mhz") or 2070.0
    fp32_peak = 152 * 128 * 2 * sm_mhz * 1e6 / 1e12
    per = {}
    for name, cidx in (("poly3b", 1), ("poly2b", 0)):
        if kern[name]["launches"]:
            per[name] = (kern[name]["total_ms"] / kern[name]["launches"], int(counts[cidx]))

    def poly_roof(name):
        ms, units = per[name]
        algo = ALGO_FLOP_PER_UNIT[name]
        fp32_view = {"achieved": units * algo / (ms * 1e-3) / 1e12, "peak": fp32_peak, "unit": "TFLOP/s",
                     "frac": units * algo / (ms * 1e-3) / 1e12 / fp32_peak,
                     "work": "%d units x %d algorithmic flop (reference operation count)" % (units, algo),
                     "peak_kind": "nominal FP32 rate at the median sampled SM clock (152 SM x 128 lanes x 2); "
                                  "MEASURED_PEAKS.json has no FP32 figure"}
        common = {"kernel": name, "traffic": NCU_TRAFFIC[name][0] * units / NCU_TRAFFIC[name][1],
                  "traffic_note": "DRAM bytes per launch from one ncu capture of this kernel (profiles/), scaled by "
                                  "units", "launch_ms": ms, "per_kernel_ms": {k: v[0] for k, v in per.items()}}
        if name == "poly3b":
            # the three-body kernel runs on the tensor cores: executed tcgen05
            # work against the measured dense fp16/bf16 rate
            tc = units * tc_flop_per_trimer() / (ms * 1e-3) / 1e12
            bf16 = measured_peak("bf16_tflops", 1905.0)
            r = {"bound": "tensor", "achieved": tc, "peak": bf16[0], "unit": "TFLOP/s", "frac": tc / bf16[0],
                 "work": "executed tcgen05.mma (M128 N64 K16) flop: %.0f per trimer x %d trimers" % (
                     tc_flop_per_trimer(), units),
                 "peak_kind": bf16[1] + " (dense bf16; fp16 runs at the same rate)",
                 "fp32_algorithmic_view": fp32_view}
        else:
            # the two-body double-float walk runs on the FP32 pipe
            r = dict(fp32_view, bound="fp32")
        r.update(common)
        return r

    roof = None
    secondary = {}
    if per:
        # the top kernel of the step's ncu launch list (the three-body tensor
        # kernel on box4096); inside the step the walk's event time can be the
        # longer of the two, because the solver iterations share its SMs
        dom = "poly3b" if "poly3b" in per else "poly2b"
        roof = poly_roof(dom)
        if dom == "poly3b" and "poly2b" in per:
            roof["two_body_walk"] = poly_roof("poly2b")
    hbm = measured_hbm_gbs()
    nsites = 3 * (n // 4)
    if kern["elec_direct_field"]["launches"] and counts[2] > 0:
        t = kern["elec_direct_field"]["total_ms"] / kern["elec_direct_field"]["launches"] * 1e-3
        b = 12 * int(counts[2]) + 36 * nsites
        secondary["induced_direct_field"] = {
            "bound": "hbm", "achieved": b / t / 1e9, "peak": hbm[0], "unit": "GB/s", "frac": b / t / 1e9 / hbm[0],
            "traffic": None, "work": "%d polarisable site pairs x 12 B + %d sites x 36 B" % (int(counts[2]), nsites),
            "launch_ms": t * 1e3, "peak_kind": hbm[1]}
    if grid and kern["elec_pme_dipoles"]["launches"]:
        t = kern["elec_pme_dipoles"]["total_ms"] / kern["elec_pme_dipoles"]["launches"] * 1e-3
        G = grid[0] * grid[1] * grid[2]
        b = nsites * 125 * 4 + 24 * G
        secondary["pme_dipole_pass"] = {
            "bound": "hbm", "achieved": b / t / 1e9, "peak": hbm[0], "unit": "GB/s", "frac": b / t / 1e9 / hbm[0],
            "traffic": None, "work": "%d sites x 125 x 4 B + %d grid points x 24 B (spread, cuFFT, gather)" % (nsites, G),
            "launch_ms": t * 1e3, "peak_kind": hbm[1]}
    return roof, secondary


def accuracy_check():
    """The metric's acceptance bar (total forces <= 1e-4 relative RMS, energy
    <= 1e-6 relative) on the FP64 reference outputs committed under
    tests/golden: the reference's 256-water PME box
    (python/tests/pdb_files/water256.pdb) and one frame of this benchmark's
    4096-water box at two frames: the seeded lattice
    (tests/golden/box4096_seed0.npz) and the same box after 3000 NVE MD
    steps (tests/golden/box4096_md3000.npz), at the timed settings (PME,
    1e-8 D, the reference's alpha*E start).  The lattice frame's total
    (2711 kJ/mol) cancels terms of up to 1.1e5 kJ/mol, so its energy error is
    judged against the sum of the terms' magnitudes; the MD frame's total
    (-72,836 kJ/mol) carries the bar itself (`passes_vs_total`)."""
    import mbpol_openmm_plugin_gb300 as mb
    from mbpol_openmm_plugin_gb300 import systems
    out = {}
    for key, fname in (("water256_pme", "pdb_water256_pme.npz"), ("box4096_seed0", "box4096_seed0.npz"),
                       ("box4096_md3000", "box4096_md3000.npz")):
        d = np.load(os.path.join(ROOT, "tests", "golden", fname))
        ws = systems.WaterSystem(d["positions"], d["box"], 0, key)
        s = mb.create_mbpol_system(ws, target_epsilon=1e-8, ewald_alpha=float(d["alpha"]),
                                   pme_grid=[int(v) for v in d["grid"]])
        ctx = mb.Context(s)
        ctx.setPositions(d["positions"])
        st = ctx.getState()
        e, eref = st.getPotentialEnergy(), float(d["etotal"])
        f, fref = np.asarray(st.getForces()), np.asarray(d["ftotal"])
        ferr = float(np.sqrt(np.sum((f - fref) ** 2) / np.sum(fref ** 2)))
        scale = float(sum(abs(float(d[k])) for k in ("e1", "e2", "e3", "edisp", "eelec")))
        out[key] = {"energy_rel": abs(e - eref) / abs(eref), "energy_rel_to_term_scale": abs(e - eref) / scale,
                    "force_rel_rms": ferr,
                    "passes": bool(abs(e - eref) <= 1e-6 * max(abs(eref), scale) and ferr <= 1e-4),
                    "passes_vs_total": bool(abs(e - eref) <= 1e-6 * abs(eref) and ferr <= 1e-4)}
        del ctx
    out["source"] = "FP64 reference outputs (compiled reference energies; oracle-port forces where the " \
                    "reference's PME forces are not finite)"
    return out


def measured_peak(key, fallback):
    """(value, source) of MEASURED_PEAKS.json, else the fallback figure of
    one earlier GB300 measurement."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)[key]), "measured (MEASURED_PEAKS.json %s)" % key
    except (OSError, KeyError, ValueError):
        return fallback, "fallback (one earlier GB300 measurement)"


def measured_hbm_gbs():
    return measured_peak("hbm_gbs", 6800.0)


def nve_drift(lib, h, nsteps, nwaters, block=10):
    """Total energy (potential + kinetic) every `block` NVE steps after the
    timed region; linear drift per ns and the fluctuation about the fit."""
    from mbpol_openmm_plugin_gb300 import _capi
    ms = ctypes.c_double()
    iters = ctypes.c_long()
    en = np.zeros(6)
    E = []
    for _ in range(max(nsteps // block, 2)):
        _capi.check(lib.mbpol_md_run(h, block, DT_PS, 0.0, 0.0, 0, ctypes.byref(ms), _capi.ptr(en),
                                     ctypes.byref(iters)))
        E.append(float(en.sum()))
    t = np.arange(1, len(E) + 1) * block * DT_PS * 1e-3  # ns
    fit = np.polyfit(t, E, 1)
    return {"steps": block * len(E), "kJ_mol_per_ns": float(fit[0]), "kJ_mol_per_ns_per_water": float(fit[0]) / nwaters,
            "fluctuation_kJ_mol": float(np.std(np.asarray(E) - np.polyval(fit, t))),
            "total_energy_first_last": [E[0], E[-1]]}


def run_clusters(args):
    """Batched independent clusters: one context evaluates all clusters of
    systems.batched_clusters (4096 clusters of 2-64 waters) per call, every
    kernel launched once over all of them.  A step is one evaluation of the
    whole batch through mbpol_compute (host buffers)."""
    import mbpol_openmm_plugin_gb300 as mb
    from mbpol_openmm_plugin_gb300 import _capi, systems
    lib = _capi.load()
    ws = systems.batched_clusters(seed=args.seed)
    ncl = int(ws.cluster_of_water.max()) + 1
    sysm = mb.create_mbpol_system(ws, target_epsilon=1e-8, guess=GUESS_MODE[args.guess] if args.guess != "learned" else 0)
    ctx = mb.Context(sysm)
    ctx.setPositions(ws.positions)
    ctx.setClusters(np.repeat(ws.cluster_of_water, 4))
    h = ctx._h
    n = ws.positions.shape[0]
    pos = np.ascontiguousarray(ws.positions, np.float64)
    e5 = np.zeros(5)
    forces = np.zeros((n, 3))
    # untimed: warm-up, then the autotuner's 12 candidate launch shapes (one
    # evaluation each)
    _capi.check(lib.mbpol_set_autotune(h, 1 if args.autotune else 0))
    for _ in range(args.warmup + (12 if args.autotune else 0)):
        _capi.check(lib.mbpol_set_positions(h, _capi.ptr(pos), None))
        _capi.check(lib.mbpol_compute(h, _capi.ALL_TERMS, _capi.ptr(e5), _capi.ptr(forces)))
    shape = launch_shape(lib, h)
    ts = []
    for _ in range(args.steps):
        forces[:] = 0.0
        t0 = time.perf_counter()
        _capi.check(lib.mbpol_set_positions(h, _capi.ptr(pos), None))
        _capi.check(lib.mbpol_compute(h, _capi.ALL_TERMS, _capi.ptr(e5), _capi.ptr(forces)))
        ts.append(time.perf_counter() - t0)
    # per-kernel event timers on further evaluations (they add launches)
    lib.mbpol_profile_enable(1)
    for _ in range(args.steps):
        _capi.check(lib.mbpol_set_positions(h, _capi.ptr(pos), None))
        _capi.check(lib.mbpol_compute(h, _capi.ALL_TERMS, _capi.ptr(e5), _capi.ptr(forces)))
    kern = {}
    for kid, kname in enumerate(_capi.KERNELS):
        t = ctypes.c_double()
        nl = ctypes.c_long()
        lib.mbpol_profile_read(kid, ctypes.byref(t), ctypes.byref(nl))
        kern[kname] = t.value / args.steps
    lib.mbpol_profile_enable(0)
    E, its = ctx.getClusterResults()
    c = ctx.getCounts()
    step_s = float(np.mean(ts))
    return {"metric": "batched cluster evaluations/s (4096 clusters of 2-64 waters)", "value": ncl / step_s,
            "unit": "clusters/s", "n_gpus": 1, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_s * 1e3, "higher_is_better": True, "scaling": "replicas", "vs_baseline": None,
            "dtype": "fp32+double-float polynomials, fp64 accumulation", "data": "synthetic (seeded clusters)",
            "config": {"workload": "clusters", "clusters": ncl, "waters": int(ws.num_waters),
                       "target_epsilon_D": 1e-8, "guess": "alpha*E (reference)" if args.guess == "learned" else args.guess,
                       "seed": args.seed, "launch_shape": shape},
            "e2e": {"value": ncl / step_s, "unit": "clusters/s", "h2d_bytes_per_step": int(n * 24),
                    "d2h_bytes_per_step": int(n * 24 + 40)},
            "solver_iterations": {"mean": float(its.mean()), "max": int(its.max())},
            "kernels_ms_per_step": kern,
            "counts": {"pairs_2b": int(c[0]), "trimers": int(c[1])}}


def cpu_baseline(args, sample=True):
    """The oracle's C port on the host (single thread, as the reference's
    Reference platform), on a bounded sample of the workload."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    try:
        import oracle
        its = None
        fx = os.path.join(ROOT, "tests", "golden", "%s_seed%d.npz" % (args.workload, args.seed))
        if os.path.exists(fx):
            # the reference's own iteration count on this frame (alpha*E start)
            its = int(np.load(fx)["iterations"])
        return oracle.time_reference_step(args.workload, args.seed, budget_s=args.cpu_budget, solver_iterations=its)
    except Exception as ex:  # the port not built / not available
        return {"value": None, "unit": "ns/day", "cores": 1, "kind": "port", "sample": "unavailable: %s" % ex}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="box4096")
    ap.add_argument("--guess", default="learned", choices=["plain", "extrapolation", "learned"])
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-comparison", action="store_true", help="time the --guess arm only")
    ap.add_argument("--profile-window", type=int, default=0,
                    help="profiling run: the --guess arm's context after equilibration and warm-up, then this many "
                         "MD steps between cudaProfilerStart and cudaProfilerStop (for ncu --profile-from-start off)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false",
                    help="fixed default launch shapes instead of the autotuner's choice")
    ap.add_argument("--no-correction", action="store_true",
                    help="learned arm without its correction network (the history predictor alone)")
    ap.add_argument("--drift-steps", type=int, default=0, help="NVE steps after the timed region for the drift")
    ap.add_argument("--avg-steps", type=int, default=1000,
                    help="MD steps after the timed ones over which iterations/step are averaged (0: none)")
    ap.add_argument("--no-accuracy", action="store_true", help="skip the reference-fixture accuracy check")
    ap.add_argument("--equilibrate", type=int, default=200,
                    help="untimed MD steps before the warm-up (trajectory start, every arm)")
    ap.add_argument("--model", default="reference", choices=["reference", "physical"],
                    help="physical: complete trimers and the consistent PME field (energy-conserving)")
    args = ap.parse_args()
    rank = int(os.environ.get("RANK", "0"))
    if args.impl == "reference":
        if rank != 0:
            return
        cb = cpu_baseline(args)
        from mbpol_openmm_plugin_gb300 import systems
        from mbpol_openmm_plugin_gb300.plugin import pme_parameters
        ws = systems.workload(args.workload, args.seed)
        alpha, grid = pme_parameters(ws.box, 0.9, 1e-5)
        out = {"impl": "reference", "metric": METRIC,
               "value": cb.get("value"), "unit": "ns/day", "n_gpus": args.gpus, "steps": args.steps,
               "warmup": args.warmup, "higher_is_better": True,
               "config": workload_config(args, ws, alpha, grid, guess_params_source(args)),
               "cpu_baseline": cb,
               "e2e": {"value": cb.get("value"), "unit": "ns/day", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        if cb.get("value") is None:
            out = {"impl": "reference", "unavailable": cb.get("sample")}
        print(json.dumps(out))
        return
    # one process per GPU; this path does not shard (a single periodic box):
    # extra ranks run independent replicas
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.gpus > 1:
        os.environ.setdefault("CUDA_VISIBLE_DEVICES", str(local))
    if args.profile_window > 0:
        out = profile_window(args)
    else:
        out = run_clusters(args) if args.workload == "clusters" else run_ours(args)
    if rank == 0:
        print(json.dumps(out))


if __name__ == "__main__":
    main()
