"""Benchmark of the GB300 RPMD engine: bead-steps/s, mixed form vs plain FP64.

One "step" is one RPMD velocity-Verlet step (Caracal's `verlet`,
src/verlet.f90:65) of every bead of every trajectory of the workload.

  value      bead-steps/s of the mixed form, state resident in HBM, the K timed
             steps in one persistent launch (CUDA events on the engine stream)
  plain_fp64 the same for the plain FP64 form
  e2e        bead-steps/s through the C-ABI with host buffers: each step copies
             q, p, dV/dq in from pinned memory, steps once, copies them out
  roofline   the step kernel against the measured FP64 (or FP32) pipe peak
  cpu_baseline  the oracle (the C++ restatement of Caracal's step) on the host
             cores, OpenMP over trajectories, bounded sample

`--impl reference` times the CPU restatement (Caracal's Fortran cannot be
built on this image) on all host cores with the same metric.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

# Algorithmic operations of one BKMP2 evaluation (one bead, reactant-like
# geometry, no compact-geometry terms), counted by instantiating the oracle's
# restatement of src/egrad_h3.f on an op-counting scalar; a CPU test checks
# this table against the oracle.
ALGO_PES_OPS = {
    "h3": {"add": 491, "mul": 738, "div": 82, "sqrt": 5, "exp": 11, "pow": 6},
    "ch4h": {"add": 3839, "mul": 7125, "div": 1812, "sqrt": 135, "exp": 54, "acos": 18, "tanh": 21,
             "cosh": 21},
    "ch4oh": {"add": 4063, "mul": 7423, "div": 1850, "sqrt": 140, "exp": 72, "pow": 3, "acos": 22,
              "tanh": 25, "cosh": 25},
    # synthetic C20H42 QMDFF (ff_eg + ff_nonb), thermal geometry (reference
    # geometry + N(0, 0.05 bohr) per coordinate, seed 0); asin counted with acos
    "qmdff": {"add": 92211, "mul": 117587, "div": 20592, "sqrt": 4525, "exp": 1415, "pow": 122,
              "sin": 633, "cos": 753, "acos": 291, "erf": 171},
    # GeH4 + OH: the CH4 + OH code with its own constants (the same counts at
    # workloads.geh4oh_geometry)
    "geh4oh": {"add": 4063, "mul": 7423, "div": 1850, "sqrt": 140, "exp": 72, "pow": 3, "acos": 22,
               "tanh": 25, "cosh": 25},
    # OH + H2 (Schatz-Elgersma), the reactant approach of workloads.oh3_geometry
    "oh3": {"add": 218, "mul": 199, "div": 43, "sqrt": 7, "exp": 14, "tanh": 6, "cosh": 6},
    # flexible SPC water, 64 molecules, periodic box 23.47 bohr, Coulomb
    # cutoff 6 A, thermal geometry (grid geometry + N(0, 0.05 bohr), seed 0)
    "water": {"add": 194295, "mul": 201198, "div": 9259, "sqrt": 18336, "exp": 128},
}
CALIB_OPS = {"fma": 0, "div": 1, "sqrt": 2, "exp": 3, "log": 4, "pow": 5, "sin": 6, "cos": 7,
             "acos": 8, "erf": 9, "tanh": 10, "cosh": 11}


TRANSCENDENTALS = ("exp", "log", "pow", "sin", "cos", "acos", "erf", "tanh", "cosh")


def algo_flops_per_bead_step(pes, natoms, nbeads, thermostat, w, transrot=True, recross=False):
    """Algorithmic FP work of one bead-step, (FP64 part, PES part, Gaussian
    pairs drawn) in flops and pairs.

    Counting: add, mul, div and sqrt are 1 flop each (as counted in the
    reference formulas by the oracle's op-counting instantiation);
    transcendentals are weighted by their measured cost on the pipe that runs
    them (w[k] = 2 x FMA rate / op rate, i.e. the FMA-pipe flops the op
    occupies).  PES: the table above.  Per-bead FP64 work outside the PES:
    Caracal's propagator as four length-P real FFTs per coordinate
    (2.5 P log2 P flops each) plus the 2x2 mode update (6 flops), two half
    kicks (4 flops per coordinate), transrot (30 flops per coordinate), PILE
    (per half step two FFT pairs), and for recrossing children the centroid
    and xi (3 flops per coordinate).  The Gaussian deviates (Box-Muller: a
    log, a sqrt, a sine and a cosine per pair) run in FP32 in both forms and
    are returned as a pair count, weighted on the FP32 pipe by the caller.
    """
    ops = ALGO_PES_OPS[pes]
    pes_f = sum(ops.get(k, 0) for k in ("add", "mul", "div", "sqrt"))
    pes_f += sum(ops.get(k, 0) * w[k] for k in TRANSCENDENTALS)
    nc = 3 * natoms
    lg = math.log2(nbeads) if nbeads > 1 else 0.0
    f64 = nc * (4 * 2.5 * lg + 6) + nc * 4
    if transrot:
        f64 += nc * 30
    pairs = 0.0
    if thermostat == "andersen":
        pairs = (nc / 2) / 70.0      # a full resample every ANDERSEN_STEP steps (70)
    if thermostat == "pile":
        f64 += 2 * nc * (2 * 2 * 2.5 * lg + 4)
        pairs = 2 * (nc / 2)
    if recross:
        f64 += nc * 3
    return f64, pes_f, pairs


def roofline(wl, mixed, ms, K, cal):
    """Roofline of one step-kernel launch against the measured pipe peaks.

    Plain form: everything on the FP64 pipe.  Mixed form: the PES on the FP32
    pipe, the rest on FP64; the two are combined into FP64-equivalent flops
    (FP32 flops x peak64/peak32), so frac is the fraction of the pipe-time
    lower bound that the launch reaches.
    """
    w64, w32 = cal["fp64"]["w"], cal["fp32"]["w"]
    n = len(wl.mass)
    rec = wl.extra.get("recross") is not None
    f64, pes64, pairs = algo_flops_per_bead_step(wl.pes, n, wl.nbeads, wl.thermostat, w64, wl.transrot, rec)
    _, pes32, _ = algo_flops_per_bead_step(wl.pes, n, wl.nbeads, wl.thermostat, w32, wl.transrot, rec)
    p64, p32 = cal["fp64"]["peak_tflops"], cal["fp32"]["peak_tflops"]
    draws32 = pairs * (w32["log"] + 1 + w32["sin"] + w32["cos"])   # FP32 Box-Muller, both forms
    units = wl.ntraj * wl.nbeads * K
    step = "step graph" if wl.pes in ("qmdff", "water") else "rpmd_run_kernel"
    if mixed:
        eq = f64 + (pes32 + draws32) * p64 / p32
        kern, bound = f"{step}<{wl.pes}, mixed>", "fp64+fp32 (FP64-equivalent)"
    else:
        eq = f64 + pes64 + draws32 * p64 / p32
        kern, bound = f"{step}<{wl.pes}, fp64>", "fp64"
    ach = eq * units / (ms * 1e-3) / 1e12
    return {"kernel": kern, "bound": bound, "achieved": ach, "peak": p64, "unit": "TFLOP/s",
            "frac": ach / p64, "traffic": None,
            "peak_source": "measured in this run (FP64/FP32 FMA microbenchmarks, cr_calibrate_op); "
                           "MEASURED_PEAKS.json holds only HBM and bf16 peaks",
            "algo_flops_per_bead_step": {"fp64": f64, "pes_fp64": pes64, "pes_fp32": pes32,
                                         "gaussian_fp32": draws32, "fp64_equivalent": eq}}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index=0):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
            time.sleep(0.3)
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for ln in self.proc.stdout:
            self.lines.append(ln.strip())

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.15)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=2)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx = float(parts[2])
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower() == "active":
                    reasons.add(n)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": mx, "reasons": ["unsampled"], "samples": 0}
        return {"sm_mhz": float(np.median(sm)), "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return json.load(fh)
    except Exception:
        return {}


def calibrate(L):
    """FP64 and FP32 FMA peaks and per-op costs (in FMAs) on this device."""
    out = {}
    for fp64, tag in ((1, "fp64"), (0, "fp32")):
        rates = {}
        for name, op in CALIB_OPS.items():
            r = np.zeros(1)
            iters = 20000 if name == "fma" else 400
            L.check(L.lib().cr_calibrate_op(fp64, op, iters, L.dptr(r)), "calibrate")
            rates[name] = float(r[0])
        fma = rates["fma"]
        out[tag] = {"fma_per_s": fma, "peak_tflops": 2 * fma / 1e12,
                    "w": {k: 2.0 * fma / v for k, v in rates.items() if k != "fma"}}
    # FP64 tensor-core MMA (m8n8k4) multiply-adds per second, for the bead
    # transform as a dense contraction against DFMA code
    r = np.zeros(1)
    L.check(L.lib().cr_calibrate_op(1, 12, 2000, L.dptr(r)), "calibrate dmma")
    out["fp64"]["dmma_fma_per_s"] = float(r[0])
    return out


def workload(name):
    from caracal_gb300 import workloads as W
    if name == "h3":
        return W.h3_config(ntraj=64, nbeads=16, thermostat="pile")
    if name == "h3_large":
        return W.h3_config(ntraj=4096, nbeads=16, thermostat="pile")
    if name in ("ch4h", "ch4h_small"):
        wl = W.ch4h_config(ntraj=4096 if name == "ch4h" else 256)
        wl.extra["recross"] = W.ch4h_recross_definition(wl.q0)
        return wl
    if name == "qmdff":
        return W.qmdff_config(ntraj=1024, nbeads=64)
    if name == "qmdff_small":
        return W.qmdff_config(ntraj=512, nbeads=64)
    if name == "water":
        return W.water_config(nwater=64, ntraj=64, nbeads=32)
    if name == "oh3":
        return W.oh3_config(ntraj=4096, nbeads=32)
    if name == "geh4oh":
        return W.geh4oh_md_config(ntraj=2048, nbeads=32)
    if name == "qmdff_npt":
        # C20H42 in a periodic 40 A box under 1 atm, Berendsen barostat
        wl = W.qmdff_config(ntraj=1024, nbeads=64)
        wl.name = "qmdff_npt_c20h42_box40A_P64_T1024"
        wl.extra.update(box_ang=[40.0] * 3, coul_cut_ang=50.0, vdw_cut_ang=10.0, npt_atm=1.0)
        return wl
    raise SystemExit(f"unknown workload {name}")


def make_pes(wl):
    """The engine's PES argument: a surface name, or the device QMDFF."""
    if wl.pes == "qmdff":
        from caracal_gb300.engine import QMDFFForceField
        if "gpu_ff" not in wl.extra:
            wl.extra["gpu_ff"] = QMDFFForceField(wl.extra["ff"])
            if "box_ang" in wl.extra:
                wl.extra["gpu_ff"].set_periodic(wl.extra["box_ang"], wl.extra["coul_cut_ang"], wl.extra["vdw_cut_ang"])
        return wl.extra["gpu_ff"]
    if wl.pes == "water":
        from caracal_gb300.engine import WaterBox
        if "gpu_ff" not in wl.extra:
            x = wl.extra
            wl.extra["gpu_ff"] = WaterBox(x["nwater"], box=x["box"], coul_cut=x["coul_cut"], zahn=x["zahn"])
        return wl.extra["gpu_ff"]
    return wl.pes


def make_engine(wl, precision, traj0=0, max_steps=0):
    """Engine for the workload: MD trajectories (positions + Andersen momenta +
    forces) or, for a recrossing workload, children from one parent geometry."""
    from caracal_gb300 import RPMDEngine
    eng = RPMDEngine(make_pes(wl), wl.mass, wl.nbeads, wl.ntraj, wl.dt_au, beta=wl.beta,
                     thermostat=wl.thermostat, andersen_step=wl.andersen_step,
                     pile_tau0_au=wl.pile_tau0_au, transrot=wl.transrot, precision=precision,
                     seed=wl.seed, traj0=traj0)
    if "npt_atm" in wl.extra:
        eng.set_npt(wl.extra["npt_atm"])
    rd = wl.extra.get("recross")
    if rd is not None:
        eng.set_recross(max_steps=max(1, max_steps), **rd)
        eng.init_children(np.repeat(wl.q0[None], wl.nbeads, axis=0))
    else:
        eng.init_positions(wl.q0, wl.sigma_bohr)
        eng.init_momenta()
        eng.compute_forces()
    return eng


class OracleRunner:
    """The oracle (C++ restatement of Caracal's step) advancing the workload on
    the host cores, OpenMP over trajectories.  MD workloads keep their state
    between calls; recrossing workloads restart the children each call."""

    def __init__(self, wl):
        from oracle import oracle as orc
        self.orc, self.wl = orc, wl
        if wl.pes == "qmdff":
            from caracal_gb300 import qmdff as Q
            orc.set_qmdff(wl.extra["ff"], Q.ElementTables.caracal())
            if "box_ang" in wl.extra:
                orc.set_qmdff_periodic(wl.extra["box_ang"], wl.extra["coul_cut_ang"], wl.extra["vdw_cut_ang"])
        self.npt = wl.extra.get("npt_atm")
        if wl.pes == "water":
            from caracal_gb300 import water as Wt
            x = wl.extra
            box, cut, za, zp = Wt.periodic_setup(x["box"], x["coul_cut"], x["zahn"])
            orc.set_water(x["nwater"], box, cut, x["zahn"], za, zp)
        self.cfg = orc.Config(wl.pes, wl.mass, wl.nbeads, wl.dt_au, wl.beta,
                              thermostat=wl.thermostat, andersen_step=wl.andersen_step,
                              pile_tau0=wl.pile_tau0_au, transrot=wl.transrot, seed=wl.seed)
        rd = wl.extra.get("recross")
        if rd is not None:
            self.xd = orc.make_xidef([a - 1 for a in rd["reac1"]], [a - 1 for a in rd["reac2"]],
                                     (rd["bond_form"][0] - 1, rd["bond_form"][1] - 1),
                                     (rd["bond_break"][0] - 1, rd["bond_break"][1] - 1),
                                     rd["form_ref"], rd["break_ref"], rd["r_inf"], rd["xi_ideal"])
            self.qpar = np.repeat(wl.q0[None], wl.nbeads, axis=0)
        else:
            self.xd = None
            self.q = orc.init_positions(self.cfg, wl.ntraj, wl.q0, wl.sigma_bohr)
            self.p = orc.init_momenta(self.cfg, wl.ntraj)
            self.f, _ = orc.init_forces(self.cfg, self.q)
            if self.npt is not None:
                self.box = np.tile(np.asarray(wl.extra["box_ang"]) / 0.52917721092, (wl.ntraj, 1))
        self.istep = 0

    def advance(self, nsteps, cores):
        if self.xd is not None:
            self.orc.recross_children(self.cfg, self.xd, self.wl.ntraj, self.qpar, nsteps, nthreads=cores)
        elif self.npt is not None:
            self.q, self.p, self.f, _, _, self.box, _ = self.orc.run_npt(
                self.cfg, self.q, self.p, self.f, nsteps, self.box, self.npt, istep0=self.istep, nthreads=cores)
        else:
            self.q, self.p, self.f, _, _ = self.orc.run(self.cfg, self.q, self.p, self.f, nsteps,
                                                         istep0=self.istep, nthreads=cores)
        self.istep += nsteps


def cpu_baseline(wl, target_s=12.0, nthreads=0):
    """The oracle on the host cores, a bounded sample of the workload."""
    run = OracleRunner(wl)
    cores = nthreads or os.cpu_count()
    n = 5
    t0 = time.perf_counter()
    run.advance(n, cores)
    dt = time.perf_counter() - t0
    steps = max(5, min(int(n * target_s / max(dt, 1e-6)), wl.nsteps))
    t0 = time.perf_counter()
    run.advance(steps, cores)
    el = time.perf_counter() - t0
    return {"value": wl.ntraj * wl.nbeads * steps / el, "unit": "bead-steps/s", "cores": cores,
            "kind": "port",
            "sample": f"{wl.ntraj} trajectories x {wl.nbeads} beads x {steps} steps of the workload "
                      f"(C++ restatement of Caracal's step, -O2, OpenMP over trajectories)"}


def dist_setup():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return rank, ws, dist
    return 0, 1, None


def run_reference(args):
    rank, ws, dist = dist_setup()
    wl = workload(args.workload)
    if rank != 0:
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    # W warm-up samples, then K timed samples; each sample = a bounded number of
    # steps of the whole workload on all host threads
    run = OracleRunner(wl)
    T = wl.ntraj
    cores = os.cpu_count()
    per = max(1, min(args.ref_steps_per_sample, wl.nsteps))
    for _ in range(args.warmup):
        run.advance(per, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        run.advance(per, cores)
    el = time.perf_counter() - t0
    v = T * wl.nbeads * per * args.steps / el
    line = {"impl": "reference", "metric": "bead-steps/s", "value": v, "unit": "bead-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el * 1e3 / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": wl.name, "ntraj": T, "nbeads": wl.nbeads, "pes": wl.pes,
                       "thermostat": wl.thermostat, "ref_steps_per_sample": per},
            "cpu_baseline": {"value": v, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{per} steps of {T}x{wl.nbeads} beads per timed sample; "
                                       "Caracal's Fortran is not buildable here, so its C++ "
                                       "restatement (oracle/) is timed"},
            "e2e": {"value": v, "unit": "bead-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_ours(args):
    import torch
    from caracal_gb300 import _lib as L

    rank, ws, dist = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    wl = workload(args.workload)
    K, W = args.steps, args.warmup
    cap = W + K * 52 + args.e2e_steps + 16  # every step the engines take in this process
    shape = [int(v) for v in args.launch.split(",")] if args.launch else None
    if args.profile:
        # only the engine launches (for ncu): W warm-up steps and K timed steps per form
        for prec in ("fp64", "mixed"):
            eng = make_engine(wl, prec, traj0=rank * wl.ntraj, max_steps=cap)
            if shape:
                eng.set_launch(*shape)
            eng.run(W)
            eng.run(K)
            print(json.dumps({"profile": wl.name, "precision": prec, "steps": K,
                              "kernel_ms": eng.last_kernel_ms(), "launch": eng.launch_info()}))
            eng.close()
        return
    cal = calibrate(L)
    eng_mx = make_engine(wl, "mixed", traj0=rank * wl.ntraj, max_steps=cap)
    eng_64 = make_engine(wl, "fp64", traj0=rank * wl.ntraj, max_steps=cap)
    # the launch-shape autotuner (threads per block and per bead) of the
    # persistent kernel, before any timing; it puts the state back
    tuned = {}
    if wl.pes not in ("qmdff", "water"):
        for name, eng in (("mixed", eng_mx), ("fp64", eng_64)):
            if shape:
                eng.set_launch(*shape)
                tuned[name] = {"threads_per_block": shape[0], "threads_per_bead": shape[1], "given": True}
                continue
            b, tpb, ms = eng.autotune(min(max(K, 10), 50))
            tuned[name] = {"threads_per_block": b, "threads_per_bead": tpb, "trial_ms_per_step": ms}
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")

    def timed_run(eng):
        eng.run(W)                       # warm-up launch (W steps)
        flush.zero_()                    # L2 (129 MB) flushed before the timed launch
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        eng.run(K)                       # K steps: one persistent launch (analytic PES) or K graph replays (QMDFF)
        torch.cuda.synchronize()
        ms = eng.last_kernel_ms()
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    # the plain FP64 arm: at least 200 timed steps (one launch, a few hundred
    # ms), so its rate -- the denominator of mixed/plain -- is stable
    K64 = max(K, 200)

    def timed_plain():
        eng_64.run(W)
        flush.zero_()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        eng_64.run(K64)
        torch.cuda.synchronize()
        ms = eng_64.last_kernel_ms()
        if dist:
            t = torch.tensor([ms], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            ms = float(t.item())
        return ms

    with ClockSampler(dev) as clk:
        ms_mx = timed_run(eng_mx)
        ms_64 = timed_plain()
        # keep the sampler alive over at least a few samples
        if ms_mx < 500:
            extra = max(1, int(500 / max(ms_mx, 1e-3)))
            for _ in range(min(extra, 50)):
                eng_mx.run(K)
    clocks = clk.summary()
    bead_steps = wl.ntraj * wl.nbeads * K
    value = ws * bead_steps / (ms_mx * 1e-3)
    plain = ws * wl.ntraj * wl.nbeads * K64 / (ms_64 * 1e-3)

    # force error of the mixed form against FP64 at the same positions (and,
    # under NpT, in the same boxes)
    q, p, f, e, st = eng_64.get_state()
    if "npt_atm" in wl.extra:
        # after a Berendsen step the stored forces belong to the coordinates
        # before the scaling (as Caracal's derivs do): recompute both forms
        eng_64.set_state(q, p)
        q, p, f, e, st = eng_64.get_state()
        eng_mx.set_npt(wl.extra["npt_atm"], eng_64.npt_state()[0])
    eng_mx.set_state(q, p)          # recomputes forces in the mixed form
    _, _, f_mx, e_mx, _ = eng_mx.get_state()
    ferr = float(np.max(np.abs(f_mx - f)) / np.max(np.abs(f)))
    eerr = float(np.max(np.abs(e_mx - e)) / np.max(np.abs(e)))

    # end to end through the C-ABI with pinned host buffers, every step
    import ctypes as C
    shape = (wl.ntraj, wl.nbeads, len(wl.mass), 3)
    nbytes = int(np.prod(shape)) * 8
    bufs = []
    for _ in range(3):
        ptr = C.c_void_p()
        L.check(L.lib().cr_host_alloc(C.byref(ptr), nbytes), "host_alloc")
        bufs.append((ptr, np.ctypeslib.as_array((C.c_double * (nbytes // 8)).from_address(ptr.value))
                     .reshape(shape)))
    (pq, hq), (pp, hp), (pf, hf) = bufs
    q, p, f, e, st = eng_mx.get_state()
    hq[...] = q
    hp[...] = p
    hf[...] = f
    he = np.zeros(wl.ntraj)
    K_e2e = min(K, args.e2e_steps)
    for _ in range(min(W, 3)):
        eng_mx.step_host(hq, hp, hf, he)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K_e2e):
        eng_mx.step_host(hq, hp, hf, he)
    el = time.perf_counter() - t0
    if dist:
        t = torch.tensor([el], device="cuda")
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        el = float(t.item())
    e2e = ws * wl.ntraj * wl.nbeads * K_e2e / el
    for ptr, _ in bufs:
        L.lib().cr_host_free(ptr)

    # the same with the caller's own (pageable) numpy arrays, as Caracal's
    # module arrays are: staged by the CUDA runtime, then page-locked in place
    # by cr_host_register (PinnedHost), which is how a Fortran caller would use it
    from caracal_gb300.engine import PinnedHost
    aq, ap, af, ae = q.copy(), p.copy(), f.copy(), np.zeros(wl.ntraj)

    def e2e_loop():
        for _ in range(min(W, 3)):
            eng_mx.step_host(aq, ap, af, ae)
        if dist:
            dist.barrier()
        t0 = time.perf_counter()
        for _ in range(K_e2e):
            eng_mx.step_host(aq, ap, af, ae)
        el = time.perf_counter() - t0
        if dist:
            t = torch.tensor([el], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            el = float(t.item())
        return ws * wl.ntraj * wl.nbeads * K_e2e / el

    e2e_pageable = e2e_loop()
    with PinnedHost(aq, ap, af):
        e2e_registered = e2e_loop()

    # rooflines of the step kernel (headline: the mixed form, whose launch `value` times)
    roof = roofline(wl, True, ms_mx, K, cal)
    roof_plain = roofline(wl, False, ms_64, K64, cal)
    kappa = None
    if wl.extra.get("recross") is not None:
        from caracal_gb300.replicas import allreduce_kappa
        num, den, _ = eng_64.kappa(cap)
        num, den = allreduce_kappa(num, den, dist)      # the replicas' children together
        kappa = {"steps": len(num), "kappa_last": float(num[-1] / den) if den else None,
                 "children": ws * wl.ntraj}
    info = eng_mx.launch_info()
    if tuned:
        info["threads_per_bead"] = eng_mx.launch()[2]
        info["autotuned"] = tuned
    line = {
        "metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": ms_mx / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32 (mixed form)", "data": "synthetic",
        "config": {"workload": wl.name, "pes": wl.pes, "ntraj": wl.ntraj, "nbeads": wl.nbeads,
                   "natoms": len(wl.mass), "thermostat": wl.thermostat, "kelvin": wl.kelvin,
                   "dt_fs": wl.dt_fs, "parallelism": f"replicas x{ws}",
                   "l2": "flushed (256 MB write) before the timed launch"
                         + ("; K steps in one launch" if wl.pes not in ("qmdff", "water") else
                            f"; state (3 x {nbytes / 1e6:.1f} MB) streamed every step (graph path)")},
        "plain_fp64": {"value": plain, "unit": "bead-steps/s", "ms_per_step": ms_64 / K64, "steps": K64},
        "mixed_over_plain": value / plain,
        "force_error_vs_fp64": ferr, "energy_error_vs_fp64": eerr,
        "e2e": {"value": e2e, "unit": "bead-steps/s", "steps": K_e2e,
                "h2d_bytes_per_step": 3 * nbytes, "d2h_bytes_per_step": 3 * nbytes + 8 * wl.ntraj},
        "e2e_caller_arrays": {"pageable": e2e_pageable, "registered": e2e_registered, "unit": "bead-steps/s",
                              "note": "the same loop on the caller's numpy arrays: pageable, then page-locked "
                                      "in place by cr_host_register"},
        "gpu_launches": info["launches"],
        "launch": info,
        "roofline": roof,
        "roofline_plain_fp64": roof_plain,
        "recross": kappa,
        "calibration": {"fp64_peak_tflops": cal["fp64"]["peak_tflops"],
                        "fp64_dmma_over_dfma": cal["fp64"]["dmma_fma_per_s"] / cal["fp64"]["fma_per_s"],
                        "fp32_peak_tflops": cal["fp32"]["peak_tflops"],
                        "fp64_op_cost_flops": cal["fp64"]["w"], "fp32_op_cost_flops": cal["fp32"]["w"]},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(wl, target_s=args.cpu_seconds)
    if wl.pes == "qmdff":
        gff = wl.extra["gpu_ff"]
        line["autotune"] = {"qmdff_egrad_kernel": {"fp64": gff.tuning("fp64"), "mixed": gff.tuning("mixed"),
                                                   "variants": "min blocks/SM 2,3,4 (fp64); 4,5,6 (mixed)"}}
    mp = measured_peaks()
    if mp:
        line["measured_peaks_file"] = {k: mp.get(k) for k in ("hbm_gbs", "bf16_tflops", "gpu_name")}
    if rank == 0:
        print(json.dumps(line))
    eng_mx.close()
    eng_64.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def class_list(name):
    from caracal_gb300 import workloads as W
    return W.mixed_classes(scale=1 if name == "classes" else 16)


def reference_classes(args):
    """`--impl reference` for the mixed-class workload: each class advanced by
    the oracle on all host threads for a bounded sample; the rate is the total
    bead-steps over the summed time (the classes run one after another)."""
    rank, ws, dist = dist_setup()
    classes = class_list(args.workload)
    if rank != 0:
        if dist:
            dist.barrier()
            dist.destroy_process_group()
        return
    cores = os.cpu_count()
    per = max(1, min(args.ref_steps_per_sample // 4, 1000))
    runs = [OracleRunner(wl) for wl in classes]
    for _ in range(args.warmup):
        for r in runs:
            r.advance(per, cores)
    el = 0.0
    for _ in range(args.steps):
        for r in runs:
            t0 = time.perf_counter()
            r.advance(per, cores)
            el += time.perf_counter() - t0
    units = sum(wl.ntraj * wl.nbeads for wl in classes) * per * args.steps
    v = units / el
    line = {"impl": "reference", "metric": "bead-steps/s", "value": v, "unit": "bead-steps/s",
            "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": el * 1e3 / (args.steps * per), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": args.workload, "classes": [wl.name for wl in classes],
                       "ref_steps_per_sample": per},
            "cpu_baseline": {"value": v, "unit": "bead-steps/s", "cores": cores, "kind": "port",
                             "sample": f"{per} steps of every class per timed sample; Caracal's Fortran "
                                       "is not buildable here, so its C++ restatement (oracle/) is timed"},
            "e2e": {"value": v, "unit": "bead-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_classes(args):
    """Trajectory classes of uneven atom and bead counts (H3, CH4H, CH4OH,
    QMDFF) stepped together by one graph launch per chunk (cr_batch), against
    the same engines run one after another (separate launches)."""
    import torch
    from caracal_gb300 import _lib as L
    from caracal_gb300 import RPMDBatch

    rank, ws, dist = dist_setup()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    classes = class_list(args.workload)
    K, W = args.steps, args.warmup
    cal = calibrate(L)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device="cuda")
    engs = {prec: [make_engine(wl, prec, traj0=rank * wl.ntraj) for wl in classes] for prec in ("mixed", "fp64")}

    def maxr(x):
        if dist:
            t = torch.tensor([x], device="cuda")
            dist.all_reduce(t, op=dist.ReduceOp.MAX)
            return float(t.item())
        return x

    def timed_batch(prec, sampler=None):
        b = RPMDBatch(engs[prec], chunk_steps=args.chunk)
        b.run(W)
        flush.zero_()
        torch.cuda.synchronize()
        if dist:
            dist.barrier()
        if sampler:
            with sampler:
                b.run(K)
        else:
            b.run(K)
        torch.cuda.synchronize()
        info = b.info()
        info["timeline"] = b.timeline()
        b.close()
        return maxr(info["ms"]), info

    def timed_separate(prec):
        per = []
        for e in engs[prec]:
            e.run(W)
        for e in engs[prec]:
            flush.zero_()
            torch.cuda.synchronize()
            e.run(K)
            per.append(maxr(e.last_kernel_ms()))
        return sum(per), per

    clk = ClockSampler(dev)
    ms_mx, info_mx = timed_batch("mixed", clk)
    clocks = clk.summary()
    ms_64, info_64 = timed_batch("fp64")
    sep_mx, per_mx = timed_separate("mixed")
    sep_64, per_64 = timed_separate("fp64")
    units = [wl.ntraj * wl.nbeads * K for wl in classes]
    total = sum(units)
    value = ws * total / (ms_mx * 1e-3)

    per_class = []
    for i, wl in enumerate(classes):
        q, p, f, e, st = engs["fp64"][i].get_state()
        em = engs["mixed"][i]
        em.set_state(q, p)
        _, _, f_mx, _, _ = em.get_state()
        ferr = float(np.max(np.abs(f_mx - f)) / np.max(np.abs(f)))
        per_class.append({"workload": wl.name, "pes": wl.pes, "natoms": len(wl.mass), "nbeads": wl.nbeads,
                          "ntraj": wl.ntraj, "thermostat": wl.thermostat,
                          "separate_mixed": ws * units[i] / (per_mx[i] * 1e-3),
                          "separate_fp64": ws * units[i] / (per_64[i] * 1e-3),
                          "force_error_vs_fp64": ferr})

    # end to end through the C-ABI each class's caller would use: every step
    # one cr_engine_step_host per class on its page-locked q, p, f (the
    # copies in and out of each class overlap with its own trajectory
    # groups' steps)
    import ctypes as C
    pinned, hostbufs = [], []
    for wl, eng in zip(classes, engs["mixed"]):
        shape = (wl.ntraj, wl.nbeads, len(wl.mass), 3)
        nb = int(np.prod(shape)) * 8
        arrs = []
        for _ in range(3):
            ptr = C.c_void_p()
            L.check(L.lib().cr_host_alloc(C.byref(ptr), nb), "host_alloc")
            pinned.append(ptr)
            arrs.append(np.ctypeslib.as_array((C.c_double * (nb // 8)).from_address(ptr.value)).reshape(shape))
        q, p, f, e, st = eng.get_state()
        arrs[0][...], arrs[1][...], arrs[2][...] = q, p, f
        hostbufs.append(arrs + [np.zeros(wl.ntraj)])
    K_e2e = min(K, max(1, args.e2e_steps // 10))
    for eng, (hq, hp, hf, he) in zip(engs["mixed"], hostbufs):
        eng.step_host(hq, hp, hf, he)
    if dist:
        dist.barrier()
    t0 = time.perf_counter()
    for _ in range(K_e2e):
        for eng, (hq, hp, hf, he) in zip(engs["mixed"], hostbufs):
            eng.step_host(hq, hp, hf, he)
    el = maxr(time.perf_counter() - t0)
    for ptr in pinned:
        L.lib().cr_host_free(ptr)
    nbytes = sum(wl.ntraj * wl.nbeads * len(wl.mass) * 3 * 8 for wl in classes)
    e2e = ws * sum(wl.ntraj * wl.nbeads for wl in classes) * K_e2e / el
    # concurrency of the classes inside one graph launch: the sum of the
    # branches' busy intervals over the span they cover (> 1: overlap)
    tl = info_mx["timeline"]
    span = max(e for _, e in tl) - min(b for b, _ in tl)
    busy = sum(e - b for b, e in tl)

    # roofline: the classes' algorithmic flops over the batched launch time
    p64, p32 = cal["fp64"]["peak_tflops"], cal["fp32"]["peak_tflops"]
    eq_mx = eq_64 = 0.0
    for wl, u in zip(classes, units):
        f64, pes64, pairs = algo_flops_per_bead_step(wl.pes, len(wl.mass), wl.nbeads, wl.thermostat,
                                                     cal["fp64"]["w"], wl.transrot)
        _, pes32, _ = algo_flops_per_bead_step(wl.pes, len(wl.mass), wl.nbeads, wl.thermostat,
                                               cal["fp32"]["w"], wl.transrot)
        w32 = cal["fp32"]["w"]
        draws = pairs * (w32["log"] + 1 + w32["sin"] + w32["cos"]) * p64 / p32
        eq_mx += (f64 + pes32 * p64 / p32 + draws) * u
        eq_64 += (f64 + pes64 + draws) * u
    ach = eq_mx / (ms_mx * 1e-3) / 1e12
    ach64 = eq_64 / (ms_64 * 1e-3) / 1e12
    line = {
        "metric": "bead-steps/s", "value": value, "unit": "bead-steps/s", "n_gpus": ws, "steps": K,
        "warmup": W, "ms_per_step": ms_mx / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64+f32 (mixed form)", "data": "synthetic",
        "config": {"workload": args.workload, "classes": [c["workload"] for c in per_class],
                   "chunk_steps": args.chunk, "parallelism": f"replicas x{ws}",
                   "l2": "flushed (256 MB write) before each timed run"},
        "plain_fp64": {"value": ws * total / (ms_64 * 1e-3), "unit": "bead-steps/s", "ms_per_step": ms_64 / K},
        "separate_launches": {"mixed": ws * total / (sep_mx * 1e-3), "fp64": ws * total / (sep_64 * 1e-3),
                              "unit": "bead-steps/s"},
        "batched_over_separate": {"mixed": sep_mx / ms_mx, "fp64": sep_64 / ms_64},
        "mixed_over_plain": ms_64 / ms_mx,
        "per_class": per_class,
        "e2e": {"value": e2e, "unit": "bead-steps/s", "steps": K_e2e, "h2d_bytes_per_step": 3 * nbytes,
                "d2h_bytes_per_step": 3 * nbytes + sum(8 * wl.ntraj for wl in classes),
                "path": "cr_engine_step_host per class, page-locked q, p, f"},
        "graph_timeline_ms": {"per_class": [{"workload": wl.name, "begin": b0, "end": b1}
                                            for wl, (b0, b1) in zip(classes, tl)],
                              "busy_over_span": busy / span if span > 0 else None,
                              "note": "one chunk's graph launch: each class branch's first and last node"},
        "gpu_launches": info_mx["launches"],
        "launch": {"graph_kernels_per_chunk": info_mx["graph_nodes"], "chunk_steps": args.chunk},
        "roofline": {"kernel": "cr_batch graph<mixed>", "bound": "fp64+fp32 (FP64-equivalent)",
                     "achieved": ach, "peak": p64, "unit": "TFLOP/s", "frac": ach / p64, "traffic": None,
                     "peak_source": "measured in this run (FP64/FP32 FMA microbenchmarks, cr_calibrate_op)"},
        "roofline_plain_fp64": {"achieved": ach64, "peak": p64, "unit": "TFLOP/s", "frac": ach64 / p64},
        "clocks": clocks,
    }
    if rank == 0 and not args.no_cpu_baseline:
        cb = [cpu_baseline(wl, target_s=args.cpu_seconds / 4) for wl in classes]
        rate = total / sum(u / c["value"] for u, c in zip(units, cb))
        line["cpu_baseline"] = {"value": rate, "unit": "bead-steps/s", "cores": cb[0]["cores"], "kind": "port",
                                "sample": "; ".join(c["sample"] for c in cb)}
    if rank == 0:
        print(json.dumps(line))
    for prec in engs:
        for e in engs[prec]:
            e.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def run_adjoint(args):
    """Derivative workloads on the synthetic C20H42 QMDFF:
    (1) force matching over 8192 bead geometries sampled from thermal RPMD
        trajectories (128 x 64 beads after 100 steps): loss and dL/dtheta over
        the bond, angle, torsion and charge parameters, plus the EVB coupling
        and first-force-field gradient of the dE-EVB pair;
    (2) the adjoint of a 200-step NVE trajectory (P=16, 64 trajectories,
        checkpoints every 20 steps).
    Timed on the device clock around the C-ABI calls (host arrays in and out)."""
    import torch
    from caracal_gb300 import qmdff as Q
    from caracal_gb300.engine import EVBPair, QMDFFForceField
    from caracal_gb300.fit import QMDFFParams, TrajectoryAdjoint, trajectory_engine
    from caracal_gb300 import workloads as Wk

    rank, ws, dist = dist_setup()
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    K, W = args.steps, args.warmup
    wl = Wk.qmdff_config(ntraj=128, nbeads=64)
    eng = make_engine(wl, "fp64", traj0=rank * wl.ntraj)
    eng.run(100)
    q, _, _, _, _ = eng.get_state()
    eng.close()
    x = q.reshape(-1, len(wl.mass), 3)
    ff = wl.extra["ff"]
    params = QMDFFParams(ff)
    gff = wl.extra["gpu_ff"]
    _, g_ref = gff.egrad(x)
    theta = params.theta() * np.random.default_rng(7).uniform(0.9, 1.1, params.size)
    f1 = QMDFFForceField(params.with_theta(theta))
    ff2 = QMDFFForceField(Q.alkane_evb_partner(ff))
    pair = EVBPair(f1, ff2, "1g", a=0.01, b=50.0)

    def fm_step():
        _, g = f1.egrad(x)
        G = x.shape[0]
        v = (2.0 / G) * (g - g_ref)
        raw = f1.param_vjp(x, v)
        return float(np.sum((g - g_ref) ** 2) / G), params.chain(raw, theta)

    def evb_step():
        _, g = pair.egrad(x)
        return pair.param_vjp(x, (2.0 / x.shape[0]) * (g - g_ref))

    def timed(fn, n):
        for _ in range(W):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(n):
            out = fn()
        torch.cuda.synchronize()
        return (time.perf_counter() - t0) / n, out

    t_fm, (loss, grad) = timed(fm_step, K)
    t_evb, _ = timed(evb_step, K)

    # trajectory adjoint
    mass = wl.mass
    P, T, nst, every = 16, 64, 200, 20
    rng = np.random.default_rng(11)
    shape = (T, P, len(mass), 3)
    q0 = ff.xyz[None, None] + rng.normal(0.0, 0.02, shape)
    p0 = rng.normal(0.0, 1.0, shape) * np.sqrt(mass[None, None, :, None] * P / wl.beta)
    e_t, g_t = trajectory_engine(params, theta, mass, P, T, wl.dt_au, wl.beta, q0, p0)
    adj = TrajectoryAdjoint(e_t, nst, every)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    adj.forward()
    t1 = time.perf_counter()
    qk, _, _, _, _ = e_t.get_state()
    raw, _, _ = adj.backward(qk - q0, np.zeros(shape))
    t2 = time.perf_counter()
    adj.close()
    e_t.close()
    g_t.close()
    line = {
        "metric": "geometries/s (force-matching loss + parameter gradient)", "value": x.shape[0] / t_fm,
        "unit": "geometries/s", "n_gpus": ws, "steps": K, "warmup": W, "ms_per_step": t_fm * 1e3,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "adjoint_c20h42", "geometries": int(x.shape[0]), "params": int(params.size),
                   "trajectory": {"nbeads": P, "ntraj": T, "steps": nst, "checkpoint_every": every}},
        "force_matching": {"loss": loss, "grad_norm": float(np.linalg.norm(grad)), "s_per_eval": t_fm},
        "evb_force_matching": {"geometries_per_s": x.shape[0] / t_evb, "basis": "1g"},
        "trajectory_adjoint": {"forward_s": t1 - t0, "backward_s": t2 - t1,
                               "bead_steps_per_s_backward": P * T * nst / (t2 - t1),
                               "backward_over_forward": (t2 - t1) / (t1 - t0)},
        "e2e": {"value": x.shape[0] / t_fm, "unit": "geometries/s", "h2d_bytes_per_step": int(2 * x.nbytes),
                "d2h_bytes_per_step": int(x.nbytes + 8 * params.size)},
    }
    if rank == 0:
        print(json.dumps(line))
    for o in (pair, f1, ff2, gff):
        o.close()
    if dist:
        dist.barrier()
        dist.destroy_process_group()


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=1000)
    ap.add_argument("--warmup", type=int, default=10)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="ch4h",
                    help="ch4h (CH4+H recrossing children, 4096 x 32 beads: the default), "
                         "ch4h_small, h3 (H+H2, 64 x 16), h3_large (4096 x 16), "
                         "qmdff (C20H42 QMDFF, 1024 x 64, Andersen 300 K), qmdff_small (512 x 64), "
                         "water (flexible SPC, 64 molecules, periodic, 64 x 32), oh3 (OH + H2, 4096 x 32), "
                         "geh4oh (GeH4 + OH, 2048 x 32, Andersen 300 K), "
                         "qmdff_npt (C20H42 in a 40 A box, 1 atm, Berendsen, 1024 x 64), "
                         "classes (H3 4096x8, CH4H 2048x32, CH4OH 512x64, QMDFF 128x128 in one batch), "
                         "classes_small (the same with 1/16 of the trajectories), "
                         "adjoint (force matching over 8192 C20H42 geometries and a 200-step trajectory adjoint)")
    ap.add_argument("--e2e-steps", type=int, default=200)
    ap.add_argument("--cpu-seconds", type=float, default=12.0)
    ap.add_argument("--ref-steps-per-sample", type=int, default=20)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--profile", action="store_true",
                    help="run only the engine launches (small ncu captures)")
    ap.add_argument("--chunk", type=int, default=50, help="steps per batch graph (classes workloads)")
    ap.add_argument("--launch", default="",
                    help="threads_per_block,threads_per_bead of the persistent kernel instead of the autotuner "
                         "(analytic workloads; used by the profiling commands)")
    args = ap.parse_args()
    if args.warmup < 3:
        args.warmup = 3
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        # N replicas need N ranks: start them with torch.distributed.run (one
        # process per GPU, rendezvous on 127.0.0.1)
        cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={args.gpus}",
               "--master-addr", "127.0.0.1", "--master-port", os.environ.get("MASTER_PORT", "29531"),
               os.path.abspath(__file__)] + sys.argv[1:]
        raise SystemExit(subprocess.call(cmd))
    if args.gpus != int(os.environ.get("WORLD_SIZE", "1")):
        raise SystemExit(f"--gpus {args.gpus} but WORLD_SIZE={os.environ.get('WORLD_SIZE', '1')}")
    if args.workload == "adjoint":
        if args.impl == "reference":
            print(json.dumps({"impl": "reference", "unavailable": "Caracal has no parameter gradients of "
                              "QMDFF losses (its EVB fit uses finite differences only)"}))
        else:
            run_adjoint(args)
        return
    if args.workload in ("classes", "classes_small"):
        if args.impl == "reference":
            reference_classes(args)
        else:
            run_classes(args)
        return
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
