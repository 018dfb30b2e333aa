#!/usr/bin/env python
"""Throughput of the GB300 particle path: particle-steps/s of the full
timestep (push + deposit + migrate + field update) on the dipole
magnetosphere workload:

  32^3 unit cells, 256 particles per cell (8,388,608): a neutral low-density
  plasma (plasma frequency 0.03, Debye length 0.16 cells) of electrons
  (q = -1e-3/128, q/m = -1) and ions (q = +1e-3/128, q/m = 0.01), 128 of
  each per cell, drifting Maxwellian v = (0.02, 0, 0) + N(0, 0.005); a static
  dipole B at the grid centre, moment set so |B| = 0.5 at 4 cells (B_z = 4,
  the 2 innermost cells masked: planetRadius = 2); electrons injected at the
  -x face, outflow at +x, periodic in y and z; dt = 0.05, c = 1.
  FP32 push/deposit with cell-relative positions (headline) and the FP64 GPU
  path on the same inputs.

  python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

Prints one JSON line. Under torchrun (N > 1) every rank runs an independent
replica (the path runs on one GPU; no collective on the data path) and rank 0
prints the whole-job value. `--impl reference` times the reference's CPU
algorithm (the CPU oracle: a restatement of the reference's timestep with its
data organisation) on the host cores, rank 0 only.
"""
import argparse
import ctypes as C
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "particle-steps/sec (push+deposit+migrate), FP32 vs FP64 GPU at stated error"
UNIT = "particle-steps/s"
CELLS = 32
PPC_SPECIES = 128
DT = 0.05
DRIFT = (0.02, 0.0, 0.0)
VTH = 0.005
CHARGE = 1e-3 / PPC_SPECIES  # macro-particle charge: plasma frequency sqrt(128 * CHARGE) = 0.03
WORKLOAD = ("dipole magnetosphere: 32^3 cells x 256 particles/cell (8,388,608; e-/ion 128+128), dipole |B|=0.5 at "
            "r=4 cells, core r<2 masked, drift vx=0.02 sigma=0.005, inject -x / outflow +x, dt=0.05")


def make_workload(seed):
    from allscale_ipic3d_gb300 import abi
    n = CELLS
    props = abi.Props.make(size=(n, n, n), cell_width=(1.0, 1.0, 1.0), dt=DT, speed_of_light=1.0, planet_radius=2.0,
                           object_center=(0.0, 0.0, 0.0), origin=(-n / 2,) * 3, external_b=(0.0, 0.0, 4.0))
    rng = np.random.default_rng(seed)
    nc = n ** 3
    per = 2 * PPC_SPECIES
    N = nc * per
    cell = np.repeat(np.arange(nc), per)
    cz, cy, cx = cell % n, (cell // n) % n, cell // (n * n)
    parts = np.zeros(N, abi.PARTICLE_DTYPE)
    parts["position"] = np.array(props.origin) + np.stack([cx, cy, cz], 1) + rng.random((N, 3))
    parts["velocity"] = np.array(DRIFT) + rng.normal(0.0, VTH, (N, 3))
    ion = (np.arange(N) % per) >= PPC_SPECIES
    parts["q"] = np.where(ion, 1.0, -1.0) * CHARGE
    parts["qom"] = np.where(ion, 0.01, -1.0)
    counts = np.full(nc, per, np.uint64)
    return props, parts, counts


# trial steps of the push-shape autotuner on a fresh process (one full pass
# over its candidate shapes); the reference arm runs as many untimed steps
AUTOTUNE_STEPS = 21


def headline_config(steps_before_timing):
    """The `config` object of both arms' JSON lines (identical by design)."""
    return {"workload": WORKLOAD, "cells": CELLS ** 3, "particles": CELLS ** 3 * 2 * PPC_SPECIES,
            "steps_before_timing": int(steps_before_timing),
            "l2": "inputs larger than L2: particle state 201 MB (FP32) / 403 MB (FP64) > 129 MB"}


def make_config(precision, graph=True):
    from allscale_ipic3d_gb300 import abi
    flags = abi.F_DIPOLE_IN_GATHER | abi.F_REFRESH_NODE_B | abi.F_INJECT_LOW_X
    if graph:
        flags |= abi.F_USE_GRAPH
    return abi.Config.make(precision=precision, mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG,
                           projector=abi.PROJECT_CIC, bc_low=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC],
                           bc_high=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC], flags=flags,
                           inject_per_cell=PPC_SPECIES * DRIFT[0] * DT, inject_q=-CHARGE,
                           inject_qom=-1.0, inject_drift=DRIFT, inject_vth=(VTH, VTH, VTH), seed=12345)


# ---- clocks --------------------------------------------------------------------
class ClockSampler:
    """nvidia-smi samples while the timed region runs."""

    def __init__(self, device=0, interval_ms=20):
        self.device, self.interval, self.rows, self.proc = device, interval_ms, [], None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + q,
                                          "--format=csv,noheader,nounits", "-lms", str(self.interval)],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
            time.sleep(0.15)
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            time.sleep(0.1)
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if len(r) > 4 + i and r[4 + i] == "Active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.rows)}


# ---- helpers ---------------------------------------------------------------------
def stream_events(sim):
    import torch
    st = torch.cuda.ExternalStream(sim.stream)
    return st, torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            return float(json.load(f)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    return 6800.0, "fallback 6.8 TB/s"


# DRAM bytes (read + write) per push launch on the headline workload, from
# one ncu capture of each kernel (k_push32_pipe with the push shape 256, 32,
# 2; k_push<double>); a citation of that capture, not a measurement of this
# run. FP32: one launch for both species; FP64: one launch per species.
PUSH_TRAFFIC = {"fp32": (436869120, "ncu capture of k_push32_pipe<3, 2, 15> on this workload (cited, not of this run)"),
                "fp64": (369767168, "ncu capture of k_push<double> on this workload (cited, not of this run)")}


def combine_ranks(ms, psteps, dist, device):
    """Whole-job figures over the ranks of a replica run: the slowest rank's
    time and the particle-steps of all ranks (every rank advances its own
    universe; nothing is exchanged on the data path)."""
    if dist is None:
        return ms, psteps
    import torch
    t = torch.tensor([ms, psteps], device=device, dtype=torch.float64)
    tmax = t.clone()
    dist.all_reduce(tmax, op=dist.ReduceOp.MAX)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    return float(tmax[0]), float(t[1])


def autotune(sim, limit=100):
    """The push-shape autotuner's trial steps (FP32 contexts): ordinary steps
    of the simulation, run before the warm-up and outside any timing, until
    the shape is chosen. Returns the steps run."""
    n = 0
    while n < limit:
        sim.step(1)
        n += 1
        if not sim.push_shape()["tuning"]:
            break
    return n


def run_timed(sim, warmup, steps, sampler=None, pre_steps=None):
    """The autotuner's trial steps (or `pre_steps` untimed steps, to keep
    another precision at the same step count), W untimed steps, then K steps
    bracketed by CUDA events on the library's stream (synchronised on both
    sides). Returns (ms, particle-steps, launches, particles, steps before
    the warm-up)."""
    import torch
    if pre_steps is None:
        pre_steps = autotune(sim)
    else:
        sim.step(pre_steps)
    sim.step(warmup)
    sim.synchronize()
    n0 = sim.particle_count()
    l0 = sim.stats()["kernel_launches"]
    st, e0, e1 = stream_events(sim)
    torch.cuda.synchronize()
    ctx = sampler if sampler is not None else _Null()
    with ctx:
        e0.record(st)
        sim.step(steps)
        e1.record(st)
        e1.synchronize()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    n1 = sim.particle_count()
    launches = sim.stats()["kernel_launches"] - l0
    return ms, 0.5 * (n0 + n1) * steps, launches, n0, pre_steps


class _Null:
    def __enter__(self):
        return self

    def __exit__(self, *a):
        pass


def push_roofline(sim, precision, nsteps, props, pops, headline=True):
    """Live CUDA-event times of the push phase over `nsteps` eager steps; the
    push kernel's algorithmic bytes per launch over its average launch
    duration. The FP32 push is one launch per step for all `pops` species
    populations; the FP64 push one launch per population (`pops` launches of
    equal size). Algorithmic bytes per population: the particles' state read
    and written once (12 x 4 B FP32, 12 x 8 B FP64), the per-cell field
    coefficients read once (FP32: 48 floats per cell) or the node E, B read
    once (FP64: 48 B per node), and the 4 FP64 node moments written once
    (32 B per node). The cited ncu DRAM traffic is the headline workload's:
    other workloads report traffic null."""
    sim.profile(True)
    sim.step(nsteps)
    prof = sim.profile_read(reset=True)
    sim.profile(False)
    push = prof["push"]
    per_launch_pops = pops if precision == "fp32" else 1
    launches_per_step = 1 if precision == "fp32" else pops
    ms_per = push["ms"] / max(push["launches"], 1) / launches_per_step
    parts = push["particles"] / max(push["launches"], 1) / launches_per_step
    elem = 4 if precision == "fp32" else 8
    nodes = (props.size[0] + 1) * (props.size[1] + 1) * (props.size[2] + 1)
    if precision == "fp32":
        bytes_per = parts * 12 * elem + per_launch_pops * (props.ncells * 48 * 4 + nodes * 32)
    else:
        bytes_per = parts * 12 * elem + nodes * (48 + 32)
    peak, src = measured_peak()
    achieved = bytes_per / (ms_per * 1e-3) / 1e9
    phases = {k: round(v["ms"] / max(v["launches"], 1), 5) for k, v in prof.items() if v["launches"]}
    return {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "traffic": PUSH_TRAFFIC[precision][0] if headline else None,
            "traffic_source": PUSH_TRAFFIC[precision][1] if headline else None,
            "kernel": ("ipg::k_push32_pipe<3, 2, 15>" if headline else "ipg::k_push32_pipe") if elem == 4
            else "ipg::k_push<double>",
            "bytes_per_launch": bytes_per, "ms_per_launch": ms_per, "launches_per_step": launches_per_step,
            "peak_source": src + ", burst copy", "phase_ms_per_step": phases}


def cpu_port_run(props, parts, counts, warmup, steps, budget_s, cfg=None):
    """The CPU oracle on the host cores: warmup steps, then up to `steps`
    steps or until budget_s seconds (config `cfg`, default the headline's)."""
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from common import OracleSim
    lib = oracle.load()
    threads = os.cpu_count() or 1
    lib.oracle_set_threads(threads)
    sim = OracleSim(props, cfg if cfg is not None else make_config(0, graph=False))
    sim.upload_particles(parts, counts)
    for _ in range(warmup):
        sim.step(1)
    n0 = lib.oracle_particle_count(sim.s)
    t0 = time.perf_counter()
    done = 0
    while done < steps:
        sim.step(1)
        done += 1
        if time.perf_counter() - t0 > budget_s:
            break
    dt = time.perf_counter() - t0
    n1 = lib.oracle_particle_count(sim.s)
    sim.close()
    return 0.5 * (n0 + n1) * done / dt, threads, done, dt


# ---- end to end ----------------------------------------------------------------------
def run_e2e(props, parts, counts, steps, dist=None):
    """The headline metric through the public API with host buffers, as the
    drop-in simulateSteps(1, universe) runs it every step: the reference's
    AoS particles (pinned host memory) up to the device, one step, every
    particle and the per-cell counts back into pinned host memory. Particle-
    steps per second of the whole round trip, every copy inside the timed
    region. Step k's download is asynchronous and completes before step
    k + 1's download starts, so its device-to-host copies run while step
    k + 1's particles go up (the link is full duplex); the timed region ends
    when the last download has landed. `sequential` is the same loop with
    the synchronous download (no overlap)."""
    import torch
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi
    host_in = torch.empty(parts.nbytes, dtype=torch.uint8, pin_memory=True).numpy().view(abi.PARTICLE_DTYPE)
    host_in[:] = parts
    cap = int(len(parts) * 1.05) + 4096  # room for the injected particles of a step
    host_out = torch.empty(cap * parts.itemsize, dtype=torch.uint8, pin_memory=True).numpy().view(abi.PARTICLE_DTYPE)
    out_counts = torch.zeros(len(counts), dtype=torch.int64, pin_memory=True).numpy().view(np.uint64)
    sim = g.Simulation(props, make_config(abi.FP32))
    sim.upload_particles(host_in, counts)
    autotune(sim)  # the shape the timed headline used (cached: no trials here)
    sim.upload_particles(host_in, counts)
    sim.step(1)
    sim.download_particles(out=(host_out, out_counts), ids=False)
    result = {"unit": UNIT, "steps": steps, "h2d_bytes_per_step": int(parts.nbytes + counts.nbytes)}
    for mode in ("sequential", "overlapped"):
        phase = {"upload": 0.0, "step": 0.0, "download": 0.0}
        d2h = 0
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for _ in range(steps):
            ta = time.perf_counter()
            sim.upload_particles(host_in, counts)
            tb = time.perf_counter()
            sim.step(1)
            sim.synchronize()
            tc = time.perf_counter()
            if mode == "overlapped":
                sim.download_wait()  # the previous step's particles
                n = sim.download_particles_async((host_out, out_counts))
            else:
                n = len(sim.download_particles(out=(host_out, out_counts), ids=False)[0])
            td = time.perf_counter()
            d2h += n * parts.itemsize + out_counts.nbytes
            phase["upload"] += tb - ta
            phase["step"] += tc - tb
            phase["download"] += td - tc
        sim.download_wait()
        secs = time.perf_counter() - t0
        ms, psteps = combine_ranks(1e3 * secs, float(len(parts) * steps), dist, "cuda")
        result[mode] = {"value": psteps / (ms * 1e-3), "ms_per_step": ms / steps,
                        "ms_per_phase": {k: round(1e3 * v / steps, 3) for k, v in phase.items()}}
        result["d2h_bytes_per_step"] = int(d2h // max(steps, 1))
    sim.close()
    result["value"] = result["overlapped"]["value"]
    result["host_link_gbs"] = {k: round(v, 1) for k, v in host_link_rates(parts.nbytes).items()}
    result["note"] = ("per step: upload of every particle (AoS, pinned host memory, chunked copies with the scatter "
                      "kernel behind them), one step, download of every particle and the per-cell counts (device "
                      "pack kernel, chunked copies behind it); `value` is the overlapped loop (a step's download "
                      "copies run during the next step's upload)")
    return result


def host_link_rates(nbytes):
    """Pinned host<->device copy rates (GB/s) over `nbytes`, CUDA events on
    one stream: H2D alone, D2H alone, and both directions at once on two
    streams (the link is full duplex)."""
    import torch
    h = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    h2 = torch.empty(nbytes, dtype=torch.uint8, pin_memory=True)
    d = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    d2 = torch.empty(nbytes, dtype=torch.uint8, device="cuda")
    s1, s2 = torch.cuda.Stream(), torch.cuda.Stream()
    out = {}
    for name in ("h2d", "d2h", "both"):
        best = None
        for _ in range(3):
            torch.cuda.synchronize()
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(s1)
            s2.wait_event(e0)
            if name in ("h2d", "both"):
                with torch.cuda.stream(s1):
                    d.copy_(h, non_blocking=True)
            if name in ("d2h", "both"):
                with torch.cuda.stream(s2 if name == "both" else s1):
                    h2.copy_(d2, non_blocking=True)
            s1.wait_stream(s2)
            e1.record(s1)
            e1.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = (2 if name == "both" else 1) * nbytes / (best * 1e-3) / 1e9
    return out


# ---- error statements ---------------------------------------------------------------
NO_ID = 0xFFFFFFFF  # particles made by the injection carry no id


def array_error(a, b):
    """Error of `a` against `b`: max |a - b| over max |b| (relative to the
    field's peak), and the max and median of |a - b| / |b| over the entries
    with |b| above 1e-6 of the peak."""
    a, b = np.asarray(a, np.float64), np.asarray(b, np.float64)
    d = np.abs(a - b)
    peak = float(np.abs(b).max()) if b.size else 0.0
    sel = np.abs(b) > 1e-6 * peak if peak > 0 else np.zeros(b.shape, bool)
    rel = d[sel] / np.abs(b[sel])
    return {"max_rel_to_peak": float(d.max() / peak) if peak > 0 else float(d.max(initial=0.0)),
            "max_rel": float(rel.max()) if rel.size else 0.0, "median_rel": float(np.median(rel)) if rel.size else 0.0,
            "peak": peak}


def particle_error(a, b, props):
    """Particle states of two runs matched by id (injected particles, which
    carry no id, are counted apart): position error in cell widths,
    velocity error relative to |v|."""
    (pa, ca, ia), (pb, cb, ib) = a, b
    ka, kb = ia != NO_ID, ib != NO_ID
    common, xa, xb = np.intersect1d(ia[ka], ib[kb], assume_unique=True, return_indices=True)
    ra, rb = pa[ka][xa], pb[kb][xb]
    w = np.array(props.cell_width, np.float64)
    dx = np.abs(ra["position"] - rb["position"]) / w
    vb = np.linalg.norm(rb["velocity"], axis=1)
    dv = np.linalg.norm(ra["velocity"] - rb["velocity"], axis=1) / np.where(vb > 0, vb, 1.0)
    return {"matched": int(len(common)), "only_first": int(ka.sum() - len(common)),
            "only_second": int(kb.sum() - len(common)),
            "injected": [int((~ka).sum()), int((~kb).sum())],
            "position_cells": {"max": float(dx.max(initial=0.0)), "median": float(np.median(dx)) if dx.size else 0.0},
            "velocity_rel": {"max": float(dv.max(initial=0.0)), "median": float(np.median(dv)) if dv.size else 0.0},
            "cell_counts": {"cells_differing": int((ca != cb).sum()),
                            "sum_abs_difference": int(np.abs(ca.astype(np.int64) - cb.astype(np.int64)).sum())}}


def conserved_error(a, b):
    """Relative error of every conserved quantity of `a` against `b`."""
    tot = lambda c: c["kinetic_energy"] + c["e_energy"] + c["b_energy"]
    out = {}
    for k in ("kinetic_energy", "e_energy", "b_energy", "total_momentum", "total_charge"):
        out[k] = abs(a[k] - b[k]) / abs(b[k]) if b[k] != 0 else abs(a[k] - b[k])
    out["total_energy"] = abs(tot(a) - tot(b)) / abs(tot(b))
    out["particles"] = [int(a["particles"]), int(b["particles"])]
    return out


def state_of(sim):
    """(particles with ids, fields, conserved) of a GPU or oracle run."""
    parts = sim.download_particles()
    f, bc, J, rho = sim.download_fields()
    return parts, (f, bc, J, rho), sim.conserved()


def state_error(a, b, props):
    """Every output of run `a` against run `b` (same steps from the same
    particles): E (node), Bc (cell centres), J and rho (nodes), the particle
    states matched by id, the per-cell counts and the conserved quantities."""
    (pa, (fa, ba, ja, ra), ca), (pb, (fb, bb, jb, rb), cb) = a, b
    return {"E": array_error(fa[..., 0:3], fb[..., 0:3]), "Bc": array_error(ba, bb), "J": array_error(ja, jb),
            "rho": array_error(ra, rb), "particles": particle_error(pa, pb, props),
            "conserved": conserved_error(ca, cb)}


def headline_errors(props, parts, counts, steps, cpu_steps):
    """The headline workload's error statement: FP32 GPU against FP64 GPU
    after `steps` steps, and FP64 GPU against the CPU oracle (the reference's
    double-precision algorithm) after `cpu_steps` steps, every output, from
    the same particles (ids tracked)."""
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi
    sys.path.insert(0, os.path.join(ROOT, "tests"))
    import oracle
    from common import OracleSim
    ids = np.arange(len(parts), dtype=np.uint32)
    out = {}
    sims = {}
    for name, prec in (("fp32", abi.FP32), ("fp64", abi.FP64)):
        cfg = make_config(prec, graph=True)
        cfg.flags |= abi.F_TRACK_IDS
        sim = g.Simulation(props, cfg)
        sim.upload_particles(parts, counts, ids)
        sims[name] = sim
    sims["fp64"].step(cpu_steps)
    s64_cpu = state_of(sims["fp64"])
    lib = oracle.load()
    lib.oracle_set_threads(os.cpu_count() or 1)
    cfg = make_config(abi.FP64, graph=False)
    cfg.flags |= abi.F_TRACK_IDS
    orc = OracleSim(props, cfg)
    orc.upload_particles(parts, counts, ids)
    orc.step(cpu_steps)
    orc.project()  # the oracle's J after its last move (the GPU deposits during the move)
    out["fp64_gpu_vs_cpu_oracle"] = dict(steps=cpu_steps, **state_error(s64_cpu, state_of(orc), props))
    orc.close()
    sims["fp64"].step(steps - cpu_steps)
    sims["fp32"].step(steps)
    out["fp32_vs_fp64_gpu"] = dict(steps=steps, **state_error(state_of(sims["fp32"]), state_of(sims["fp64"]), props))
    for s in sims.values():
        s.close()
    return out


# ---- batched ensemble -----------------------------------------------------------
ENS_SIZES = (8, 12, 16, 20, 24)
ENS_PPC = (16, 32, 64, 128, 256)
ENS_WORKLOAD = ("batched ensemble: 256 independent periodic universes, n^3 cells with n in {8,12,16,20,24} and "
                "ppc in {16,32,64,128,256} drawn uniformly (seed 12345+i), uniform B (|B| in [0.02,0.2], random "
                "direction) and E (|E| <= 0.02), Maxwellian sigma in [0.005,0.02], one species (q=-1/ppc, q/m=-1), "
                "dt=0.1, field-gather Boris mover + CIC deposit of J/rho + migration, fields static")


def universe_params(i):
    """(n, ppc, |B|, |E|, sigma) of universe i."""
    rng = np.random.default_rng(12345 + i)
    n = int(rng.choice(ENS_SIZES))
    ppc = int(rng.choice(ENS_PPC))
    d = rng.normal(size=3)
    B = rng.uniform(0.02, 0.2)
    e = rng.normal(size=3)
    E = rng.uniform(0.0, 0.02)
    return n, ppc, B, E, rng.uniform(0.005, 0.02)


def universe_props(i):
    from allscale_ipic3d_gb300 import abi
    rng = np.random.default_rng(12345 + i)
    n = int(rng.choice(ENS_SIZES))
    return abi.Props.make(size=(n, n, n), cell_width=(1.0, 1.0, 1.0), dt=0.1, speed_of_light=1.0)


def make_universe(i):
    """Universe i of the ensemble: props, particles grouped by cell, counts,
    field grids."""
    from allscale_ipic3d_gb300 import abi
    rng = np.random.default_rng(12345 + i)
    n = int(rng.choice(ENS_SIZES))
    ppc = int(rng.choice(ENS_PPC))
    d = rng.normal(size=3)
    B = d / np.linalg.norm(d) * rng.uniform(0.02, 0.2)
    e = rng.normal(size=3)
    E = e / np.linalg.norm(e) * rng.uniform(0.0, 0.02)
    sigma = rng.uniform(0.005, 0.02)
    props = universe_props(i)
    nc = n ** 3
    N = nc * ppc
    cell = np.repeat(np.arange(nc), ppc)
    parts = np.zeros(N, abi.PARTICLE_DTYPE)
    parts["position"] = np.stack([cell // (n * n), (cell // n) % n, cell % n], 1) + rng.random((N, 3))
    parts["velocity"] = rng.normal(0.0, sigma, (N, 3))
    parts["q"] = -1.0 / ppc
    parts["qom"] = -1.0
    f = np.zeros(abi.field_shape(props))
    f[..., 0:3] = E
    f[..., 3:6] = B
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., :] = B
    return props, parts, np.full(nc, ppc, np.uint64), f, bc


def ensemble_config(precision):
    from allscale_ipic3d_gb300 import abi
    return abi.Config.make(precision=precision, mover=abi.MOVER_FIELD, solver=abi.SOLVER_STATIC,
                           projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC, flags=abi.F_USE_GRAPH)


def timed_batch(batch, warmup, steps, sampler=None, pre_steps=None):
    """As run_timed, for a batch: the autotuner's trial steps (or
    `pre_steps`), W warm-up steps, K timed steps."""
    import torch
    if pre_steps is None:
        pre_steps = autotune(batch)
    elif pre_steps:
        batch.step(pre_steps)
    batch.step(warmup)
    batch.synchronize()
    st = torch.cuda.ExternalStream(batch.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    n0 = batch.stats()["particles"]
    l0 = batch.stats()["kernel_launches"]
    torch.cuda.synchronize()
    with (sampler if sampler is not None else _Null()):
        e0.record(st)
        batch.step(steps)
        e1.record(st)
        e1.synchronize()
    torch.cuda.synchronize()
    s = batch.stats()
    return e0.elapsed_time(e1), 0.5 * (n0 + s["particles"]) * steps, s["kernel_launches"] - l0, pre_steps


def timed_plain(batch, count, steps):
    """The plain (one universe at a time) form on the batch's universes: each
    universe's own graph, back to back on the batch's stream."""
    import torch
    st = torch.cuda.ExternalStream(batch.stream)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    us = [batch.universe(i) for i in range(count)]
    for u in us:  # untimed: each universe's autotuning and graph capture
        autotune(u)
        u.step(1)
    n0 = sum(u.particle_count() for u in us)
    torch.cuda.synchronize()
    e0.record(st)
    for u in us:
        u.step(steps)
    e1.record(st)
    e1.synchronize()
    torch.cuda.synchronize()
    n1 = sum(u.particle_count() for u in us)
    return e0.elapsed_time(e1), 0.5 * (n0 + n1) * steps


def run_ensemble(count, warmup, steps, local):
    """The batched ensemble in FP32 and FP64 (one launch per kernel per step
    for all universes), the plain FP64 form (one universe at a time), and the
    FP32 error against FP64 per universe."""
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi
    t_setup = time.perf_counter()
    props = [universe_props(i) for i in range(count)]
    b32 = g.Batch(props, ensemble_config(abi.FP32))
    b64 = g.Batch(props, ensemble_config(abi.FP64))
    total = 0
    for i in range(count):
        _, parts, counts, f, bc = make_universe(i)
        total += len(parts)
        for b in (b32, b64):
            b.universe(i).upload_fields(f, bc, None)
            b.universe(i).upload_particles(parts, counts)
    cells = int(sum(p.ncells for p in props))
    setup_s = time.perf_counter() - t_setup

    def ke_rel():
        rel, lost = [], 0
        for i in range(count):
            c32, c64 = b32.universe(i).conserved(), b64.universe(i).conserved()
            rel.append(abs(c32["kinetic_energy"] - c64["kinetic_energy"]) / abs(c64["kinetic_energy"]))
            lost += abs(int(c32["particles"]) - int(c64["particles"]))
        return np.array(rel), lost

    sampler = ClockSampler(local)
    ms32, ps32, launches32, pre = timed_batch(b32, warmup, steps, sampler)
    ms64, ps64, _, _ = timed_batch(b64, warmup, steps, pre_steps=pre)
    rel, lost = ke_rel()
    st32, st64 = b32.stats(), b64.stats()
    b32.close()
    b64.close()
    # the FP32 error against FP64 over the configuration's 100 steps from a
    # fresh start, every 20 steps (the FP32 batch's first steps are its push
    # autotuner's trials: ordinary steps of the simulation)
    b32 = g.Batch(props, ensemble_config(abi.FP32))
    b64 = g.Batch(props, ensemble_config(abi.FP64))
    for i in range(count):
        _, parts, counts, f, bc = make_universe(i)
        for b in (b32, b64):
            b.universe(i).upload_fields(f, bc, None)
            b.universe(i).upload_particles(parts, counts)
    curve = []
    for k in range(5):
        b32.step(20)
        b64.step(20)
        r, lost_k = ke_rel()
        curve.append({"step": 20 * (k + 1), "max": float(r.max()), "median": float(np.median(r)),
                      "particle_count_differences": lost_k})
    worst = [dict(zip(("universe", "n", "ppc", "B", "E", "sigma", "ke_rel"),
                      (int(i),) + tuple(universe_params(int(i))) + (float(rel[i]),)))
             for i in np.argsort(rel)[::-1][:4]]
    msp64, psp64 = timed_plain(b64, count, steps)
    msp32, psp32 = timed_plain(b32, count, steps)
    v32, v64 = ps32 / (ms32 * 1e-3), ps64 / (ms64 * 1e-3)
    vp64, vp32 = psp64 / (msp64 * 1e-3), psp32 / (msp32 * 1e-3)
    shape32 = b32.push_shape()
    b32.close()
    b64.close()
    return {"workload": ENS_WORKLOAD, "universes": count, "cells": cells, "particles": total,
            "steps": steps, "warmup": warmup, "setup_s": round(setup_s, 1),
            "fp32_batched": {"value": v32, "ms_per_step": ms32 / steps, "gpu_launches": int(launches32),
                             "push_shape": shape32, "autotune_steps": pre},
            "fp64_batched": {"value": v64, "ms_per_step": ms64 / steps},
            "fp64_plain": {"value": vp64, "ms_per_step": msp64 / steps},
            "fp32_plain": {"value": vp32, "ms_per_step": msp32 / steps},
            "fp32_batched_over_fp64_plain": v32 / vp64, "fp32_batched_over_fp64_batched": v32 / v64,
            "kinetic_energy_rel_fp32_vs_fp64": {"after_steps": pre + warmup + steps, "max": float(rel.max()),
                                                "median": float(np.median(rel)), "worst": worst,
                                                "particle_count_differences": lost,
                                                "first_100_steps": curve},
            "stats_fp32": st32, "stats_fp64": st64,
            "clocks": sampler.summary(), "unit": UNIT}


# ---- the other configurations (optional rows: --only c1|c3|c5) ---------------------
def seeded_plasma(rng, n, per_cell, species, origin=(0.0, 0.0, 0.0), drift=(0.0, 0.0, 0.0)):
    """Particles grouped by cell: per_cell[c] particles uniform in cell c of an
    n^3 unit-cell grid; species = [(q, qom, sigma, fraction)], Maxwellian."""
    from allscale_ipic3d_gb300 import abi
    nc = n ** 3
    N = int(per_cell.sum())
    cell = np.repeat(np.arange(nc), per_cell)
    parts = np.zeros(N, abi.PARTICLE_DTYPE)
    parts["position"] = np.array(origin) + np.stack([cell // (n * n), (cell // n) % n, cell % n], 1) + \
        rng.random((N, 3))
    frac = np.cumsum([sp[3] for sp in species])
    which = np.searchsorted(frac, rng.random(N) * frac[-1], side="right")
    sig = np.array([sp[2] for sp in species])[which]
    parts["velocity"] = np.array(drift) + rng.normal(0.0, 1.0, (N, 3)) * sig[:, None]
    parts["q"] = np.array([sp[0] for sp in species])[which]
    parts["qom"] = np.array([sp[1] for sp in species])[which]
    return parts, per_cell.astype(np.uint64)


def config_c1():
    """8^3 periodic unit cells, one species (q=-1, m=1), 64 ppc, sigma 0.01,
    B=(0,0,0.1), E=(0,0.01,0): E x B drift, dt=0.1, 100 steps, FP64."""
    from allscale_ipic3d_gb300 import abi
    rng = np.random.default_rng(12345)
    n = 8
    props = abi.Props.make(size=(n, n, n), dt=0.1)
    parts, counts = seeded_plasma(rng, n, np.full(n ** 3, 64), [(-1.0 / 64, -1.0, 0.01, 1.0)])
    f = np.zeros(abi.field_shape(props))
    f[..., 1] = 0.01
    f[..., 5] = 0.1
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., 2] = 0.1
    kw = dict(mover=abi.MOVER_FIELD, solver=abi.SOLVER_STATIC, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_USE_GRAPH)
    return ("C1 E x B drift: 8^3 periodic cells x 64 ppc (32,768), B=(0,0,0.1), E=(0,0.01,0), sigma 0.01, dt 0.1",
            props, parts, counts, (f, bc), kw, 100)


def config_c3():
    """64^3 cells, 134,217,728 particles: half uniform, half in a Gaussian blob
    (sigma 6 cells) centred at (40, 36, 32) cells; electrons (q/m -1,
    sigma 0.02) and ions (q/m 0.01, sigma 0.002); B=(0.05,0,0.1),
    self-consistent E (leapfrog), dt=0.05, 50 steps."""
    from allscale_ipic3d_gb300 import abi
    rng = np.random.default_rng(12345)
    n = 64
    N = 134217728
    uni = np.full(n ** 3, (N // 2) // n ** 3, np.int64)
    blob = rng.normal((40.0, 36.0, 32.0), 6.0, (N // 2, 3)).astype(np.int64) % n
    blob_cells = np.bincount((blob[:, 0] * n + blob[:, 1]) * n + blob[:, 2], minlength=n ** 3)
    del blob
    per = uni + blob_cells
    q = 1e-3 / 256  # macro-particle charge: plasma frequency ~0.03 in the uniform part
    parts, counts = seeded_plasma(rng, n, per, [(-q, -1.0, 0.02, 0.5), (q, 0.01, 0.002, 0.5)])
    props = abi.Props.make(size=(n, n, n), dt=0.05)
    f = np.zeros(abi.field_shape(props))
    f[..., 3] = 0.05
    f[..., 5] = 0.1
    bc = np.zeros(abi.bcfield_shape(props))
    bc[..., 0] = 0.05
    bc[..., 2] = 0.1
    kw = dict(mover=abi.MOVER_FIELD, solver=abi.SOLVER_LEAPFROG, projector=abi.PROJECT_CIC, bc=abi.BC_PERIODIC,
              flags=abi.F_USE_GRAPH | abi.F_REFRESH_NODE_B)
    return ("C3 uneven load: 64^3 periodic cells, 134,217,728 particles (half uniform, half a Gaussian blob "
            "sigma 6 cells at (40,36,32)), e-/ion (q/m -1 / 0.01, sigma 0.02 / 0.002), B=(0.05,0,0.1), "
            "self-consistent E (leapfrog), dt 0.05; per-cell counts %d..%d" % (per.min(), per.max()),
            props, parts, counts, (f, bc), kw, 50)


def config_c5():
    """128^3 cells x 128 ppc (268,435,456), electrons and ions (mass ratio
    100, sigma 0.02 / 0.002), static dipole (|B| = 0.5 at 4 cells, core r < 2
    masked) and a solar wind vx = 0.02 injected at -x, dt=0.05, 50 steps."""
    from allscale_ipic3d_gb300 import abi
    rng = np.random.default_rng(12345)
    n = 128
    q = 1e-3 / 64
    parts, counts = seeded_plasma(rng, n, np.full(n ** 3, 128), [(-q, -1.0, 0.02, 0.5), (q, 0.01, 0.002, 0.5)],
                                  origin=(-n / 2,) * 3, drift=DRIFT)
    props = abi.Props.make(size=(n, n, n), dt=DT, planet_radius=2.0, origin=(-n / 2,) * 3,
                           external_b=(0.0, 0.0, 4.0))
    kw = dict(mover=abi.MOVER_DIPOLE, solver=abi.SOLVER_STATIC, projector=abi.PROJECT_CIC,
              bc_low=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC],
              bc_high=[abi.BC_OPEN, abi.BC_PERIODIC, abi.BC_PERIODIC],
              flags=abi.F_USE_GRAPH | abi.F_INJECT_LOW_X, inject_per_cell=64 * DRIFT[0] * DT, inject_q=-q,
              inject_qom=-1.0, inject_drift=DRIFT, inject_vth=(0.02, 0.02, 0.02), seed=12345)
    return ("C5 large dipole: 128^3 cells x 128 ppc (268,435,456), e-/ion mass ratio 100 (sigma 0.02 / 0.002), "
            "static dipole |B|=0.5 at r=4 cells (core r<2 masked), solar wind vx=0.02 injected at -x, "
            "outflow +x, dt 0.05", props, parts, counts, None, kw, 50)


UDIST_N = 33554432


def config_udist():
    """The reference's own benchmark mode `:U:N` (benchmark.h:13-25, 81-92):
    32^3 cells of width 10, dt 0.15, N = 33,554,432 electrons (q -1, q/m -25)
    from the reference's initCells(uniform) (cell.h:638-697): its per-cell
    random streams, made on the device (ipic3d_gpu_init_uniform), positions
    uniform in the cell, velocities U(-0.2, 0.2); the reference's default
    policies (dipole mover with no external field, static fields, no
    projection, reflecting walls). The reference times 5 steps after 2
    warm-up steps; here 20. No host particles: `parts` is None."""
    from allscale_ipic3d_gb300 import abi
    n, w = 32, 10.0
    props = abi.Props.make(size=(n, n, n), cell_width=(w, w, w), dt=0.15)
    kw = dict(mover=abi.MOVER_DIPOLE, solver=abi.SOLVER_STATIC, projector=abi.PROJECT_NONE, bc=abi.BC_REFLECT,
              flags=abi.F_USE_GRAPH)
    return ("the reference's :U:N benchmark mode: 32^3 cells of width 10, N = 33,554,432 electrons from the "
            "reference's initCells(uniform) streams (made on the device), velocities U(-0.2,0.2), dipole mover "
            "without external field, static fields, no projection, reflecting walls, dt 0.15", props, None, None,
            None, kw, 20)


def run_config(name, warmup, local, steps=None, cpu=True):
    """FP32 and FP64 on the same inputs: particle-steps/s, the FP32 push's
    live roofline, the FP32 energy error against FP64 after the run, and a
    bounded CPU-oracle sample (C5, :U:N). `steps` overrides the
    configuration's timed steps."""
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi
    t0 = time.perf_counter()
    desc, props, parts, counts, fields, kw, nsteps = {"c1": config_c1, "c3": config_c3, "c5": config_c5,
                                                      "udist": config_udist}[name]()
    steps = nsteps if steps is None else steps
    res = {"workload": desc, "cells": props.ncells, "particles": int(len(parts)) if parts is not None else UDIST_N,
           "steps": steps, "warmup": warmup}
    species = [(-1.0, -25.0)] if parts is None else \
        sorted({(float(a), float(b)) for a, b in zip(parts["q"][:1000], parts["qom"][:1000])})
    cons = {}
    pre = None
    for pname, prec in (("fp32", abi.FP32), ("fp64", abi.FP64)):
        sim = g.Simulation(props, abi.Config.make(precision=prec, **kw))
        if fields is not None:
            sim.upload_fields(fields[0], fields[1], None)
        if parts is None:  # the reference's :U:N universe, made on the device
            t_init = time.perf_counter()
            sim.init_uniform(UDIST_N)
            res.setdefault("init_ms", {})[pname] = round(1e3 * (time.perf_counter() - t_init), 2)
        else:
            # register the species with a few particles, so that the large
            # upload takes the device path (one copy, classification on the GPU)
            first = np.unique(parts[["q", "qom"]][:100000], return_index=True)[1]
            c0 = np.zeros(props.ncells, np.uint64)
            c0[0] = len(first)
            sim.upload_particles(parts[first], c0)
            sim.upload_particles(parts, counts)
        sampler = ClockSampler(local)
        ms, ps, launches, n0, pre = run_timed(sim, warmup, steps, sampler if pname == "fp32" else None, pre)
        res[pname] = {"value": ps / (ms * 1e-3), "ms_per_step": ms / steps, "gpu_launches": int(launches),
                      "stats": sim.stats()}
        if pname == "fp32":
            res["clocks"] = sampler.summary()
            res["push_shape"] = sim.push_shape()
            res["autotune_steps"] = pre
        cons[pname] = sim.conserved()
        res[pname]["roofline"] = push_roofline(sim, pname, 5, props, len(species), headline=False)
        sim.close()
    tot = lambda c: c["kinetic_energy"] + c["e_energy"] + c["b_energy"]
    res["error_fp32_vs_fp64"] = {"steps": pre + warmup + steps + 5,
                                 "total_energy_rel": abs(tot(cons["fp32"]) - tot(cons["fp64"])) / abs(tot(cons["fp64"])),
                                 "kinetic_energy_rel": abs(cons["fp32"]["kinetic_energy"] -
                                                           cons["fp64"]["kinetic_energy"]) /
                                 abs(cons["fp64"]["kinetic_energy"]),
                                 "particles_fp32": cons["fp32"]["particles"],
                                 "particles_fp64": cons["fp64"]["particles"]}
    res["fp32_over_fp64"] = res["fp32"]["value"] / res["fp64"]["value"]
    res["value"] = res["fp32"]["value"]
    res["roofline"] = res["fp32"]["roofline"]
    res["configured_steps"] = nsteps
    if name == "c5" and cpu:  # the oracle port on a bounded sample: the full universe, a few steps
        cfg = abi.Config.make(precision=abi.FP64, **dict(kw, flags=kw["flags"] & ~abi.F_USE_GRAPH))
        v, cores, done, secs = cpu_port_run(props, parts, counts, 1, 3, 30.0, cfg)
        res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "the full universe (268,435,456 particles), %d timed steps (%.1f s) after "
                                         "1 warm-up step, all host threads" % (done, secs)}
    if name == "udist" and cpu:  # the reference's own CPU algorithm (the oracle port) on the same universe
        cfg = abi.Config.make(precision=abi.FP64, **{k: v for k, v in kw.items() if k != "flags"})
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        parts = np.zeros(UDIST_N, abi.PARTICLE_DTYPE)
        counts = np.zeros(props.ncells, np.uint64)
        t_init = time.perf_counter()
        oracle.load().oracle_init_uniform_bench(C.byref(props), UDIST_N, abi.vptr(parts), abi.vptr(counts))
        res.setdefault("init_ms", {})["cpu_port"] = round(1e3 * (time.perf_counter() - t_init), 2)
        v, cores, done, secs = cpu_port_run(props, parts, counts, 2, 5, 60.0, cfg)
        res["cpu_baseline"] = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
                               "sample": "the full universe, %d timed steps (%.1f s) after 2 warm-up steps, all host "
                                         "threads (the reference's benchmark.h protocol)" % (done, secs)}
    res["species"] = species
    res["setup_and_run_s"] = round(time.perf_counter() - t0, 1)
    return res


# ---- the standalone tracer (optional row: --only tracer) --------------------------
TRACER_T, TRACER_S, TRACER_R = 150, 10, 64
TRACER_N = 16 * 1000 * 1000


def run_tracer(warmup, steps, local, n=TRACER_N, e2e_steps=2, cpu_budget=15.0, cpu=True):
    """pic_tracer's default run (pic_tracer.cxx:153-158): N = 16M protons
    traced for T + 1 = 151 steps through the dipole on a 64^3 grid, a frame
    every S = 10 steps. Its metric is the one pic_tracer prints: (T + 1) N /
    seconds (pic_tracer.cxx:290). Particles are seeded synthetic draws of its
    distributions (uniform in the middle 3/4 of the box, normal speeds of
    width v_mod). One step = one trace of all N particles into the histogram
    (repetitions accumulate, as pic_tracer's M repetitions do); inputs (1 GB)
    exceed L2."""
    import torch
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi, tracer
    props = tracer.tracer_props(TRACER_R)
    steps1, frames = TRACER_T + 1, TRACER_T // TRACER_S + 1
    cells = props.ncells
    rng = np.random.default_rng(2024)
    low, hig = tracer.particle_box(props)
    parts = np.zeros(n, abi.PARTICLE_DTYPE)
    parts["position"] = rng.uniform(low, hig, (n, 3))
    parts["velocity"] = rng.standard_normal((n, 3)) * tracer.speed_scale(props)
    parts["q"] = tracer.ELEMENTARY_CHARGE
    parts["qom"] = tracer.ELEMENTARY_CHARGE / tracer.PROTON_MASS
    host = torch.from_numpy(parts.view(np.uint8)).pin_memory()
    dev = host.cuda()
    d_counts = torch.zeros(frames * cells, dtype=torch.int32, device="cuda")
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)

    def once():
        g.trace_device(props, dev.data_ptr(), n, steps1, TRACER_S, frames, d_counts.data_ptr(), st.cuda_stream)

    for _ in range(warmup):
        once()
    torch.cuda.synchronize()
    sampler = ClockSampler(local)
    with sampler:
        e0.record(st)
        for _ in range(steps):
            once()
        e1.record(st)
        torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    res = {"workload": "pic_tracer default run: N = 16,000,000 protons (10 MeV normal speeds), T = 150 (151 traced "
                       "steps), a frame every S = 10 steps, R = 64 (64^3 cells), dt 0.01, Earth dipole 3.07e-5 T"
                       if n == TRACER_N else "pic_tracer run with N = %d, T = 150, S = 10, R = 64" % n,
           "particles": n, "traced_steps": steps1, "frames": frames, "steps": steps, "warmup": warmup,
           "value": steps1 * n * steps / (ms * 1e-3), "unit": "particles/s", "ms_per_step": ms / steps,
           "gpu_launches": steps, "dtype": "f64", "clocks": sampler.summary(),
           "l2": "inputs larger than L2 (1 GB of particles)"}
    # end to end through ipic3d_gpu_trace: pinned host particles and histogram
    lib = g.library()
    h_counts = torch.zeros(frames * cells, dtype=torch.int32).pin_memory()
    rc = lib.ipic3d_gpu_trace(C.byref(props), host.data_ptr(), n, steps1, TRACER_S, frames, h_counts.data_ptr())
    assert rc == 0, rc
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        rc = lib.ipic3d_gpu_trace(C.byref(props), host.data_ptr(), n, steps1, TRACER_S, frames, h_counts.data_ptr())
        assert rc == 0, rc
    secs = time.perf_counter() - t0
    res["e2e"] = {"value": steps1 * n * e2e_steps / secs, "unit": "particles/s",
                  "h2d_bytes_per_step": n * 64 + frames * cells * 4, "d2h_bytes_per_step": frames * cells * 4}
    # every repetition adds the same histogram: the timed device runs did the work
    reps_dev, reps_host = warmup + steps, 1 + e2e_steps
    a = d_counts.cpu().numpy().astype(np.int64)
    b = h_counts.numpy().astype(np.int64)
    assert (a * reps_host == b * reps_dev).all(), "device and host-entry histograms disagree"
    res["frame_totals"] = (b.reshape(frames, cells).sum(axis=1) // reps_host).tolist()
    if cpu:  # the oracle's restatement of traceParticle on the host cores
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import oracle
        olib = oracle.load()
        threads = os.cpu_count() or 1
        olib.oracle_set_threads(threads)
        m = min(n, 20000)
        cnt = np.zeros(frames * cells, np.uint32)
        t0 = time.perf_counter()
        olib.oracle_trace(C.byref(props), abi.vptr(parts[:m]), m, steps1, TRACER_S, frames, abi.vptr(cnt))
        probe = time.perf_counter() - t0
        m2 = int(min(n, max(m, m * cpu_budget / max(probe, 1e-3))))
        cnt[:] = 0
        t0 = time.perf_counter()
        olib.oracle_trace(C.byref(props), abi.vptr(parts[:m2]), m2, steps1, TRACER_S, frames, abi.vptr(cnt))
        secs = time.perf_counter() - t0
        res["cpu_baseline"] = {"value": steps1 * m2 / secs, "unit": "particles/s", "cores": threads, "kind": "port",
                               "sample": "the first %d particles of the same set, all %d steps (%.1f s)" %
                                         (m2, steps1, secs)}
    return res


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--e2e-steps", type=int, default=10)
    ap.add_argument("--cpu-budget", type=float, default=20.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--only", default="all", choices=["all", "fp32", "fp64", "e2e", "ensemble", "c1", "c3", "c5", "udist", "tracer"],
                    help="fp32 / fp64: only that precision's timed run and its push roofline (profiling runs); "
                         "ensemble: only the batched ensemble; c1/c3/c5: that configuration alone")
    ap.add_argument("--tracer-particles", type=int, default=TRACER_N)
    ap.add_argument("--universes", type=int, default=256, help="universes of the batched ensemble")
    ap.add_argument("--ensemble-steps", type=int, default=100)
    ap.add_argument("--no-ensemble", action="store_true")
    ap.add_argument("--no-tracer", action="store_true", help="skip the standalone tracer's row in the full run")
    ap.add_argument("--no-error", action="store_true", help="skip the headline's error statement")
    ap.add_argument("--error-steps", type=int, default=100, help="steps of the FP32 vs FP64 GPU error statement")
    ap.add_argument("--error-cpu-steps", type=int, default=10, help="steps of the FP64 GPU vs CPU oracle statement")
    ap.add_argument("--no-configs", action="store_true", help="skip the C5 and :U:N rows in the full run")
    ap.add_argument("--c5-steps", type=int, default=20, help="timed steps of the C5 row in the full run")
    ap.add_argument("--push-shape", default=None,
                    help="ITEM,ITEM_CELLS,BLOCKS_PER_SM: fix the FP32 push shape of the headline run instead of "
                         "autotuning it (profiling runs, where a profiler's timing would steer the autotuner)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))

    if args.impl == "reference":
        if rank != 0:
            return 0
        props, parts, counts = make_workload(12345)
        # the same simulated interval as the GPU arm: its autotuner's trial
        # steps and its warm-up run untimed first
        pre = AUTOTUNE_STEPS + args.warmup
        value, cores, done, secs = cpu_port_run(props, parts, counts, pre, args.steps, 120.0)
        out = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": done, "warmup": args.warmup,
               "ms_per_step": 1e3 * secs / max(done, 1), "higher_is_better": True, "scaling": "weak",
               "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
               "config": headline_config(pre),
               "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": "the full workload, %d timed steps (%.1f s) after %d untimed steps (the GPU "
                                          "arm's autotuner trials and warm-up)" % (done, secs, pre)},
               "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
        print(json.dumps(out))
        return 0

    import torch
    torch.cuda.set_device(local)
    dist = None
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=torch.device("cuda", local))
    import allscale_ipic3d_gb300 as g
    from allscale_ipic3d_gb300 import abi

    if args.only in ("c1", "c3", "c5", "udist"):
        res = run_config(args.only, args.warmup, local)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "unit": UNIT, args.only: res}))
        return 0

    if args.only == "tracer":
        res = run_tracer(3, min(args.steps, 5), local, n=args.tracer_particles,
                         cpu=not args.no_cpu_baseline)
        if rank == 0:
            print(json.dumps({"metric": "particles/s (pic_tracer throughput: traced steps x particles / s)",
                              "tracer": res}))
        return 0

    if args.only == "ensemble":
        ens = run_ensemble(args.universes, args.warmup, args.ensemble_steps, local)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "ensemble": ens}))
        return 0

    props, parts, counts = make_workload(12345 + rank)
    ncells = props.ncells

    if args.only == "e2e":  # the end-to-end round trip alone
        res = run_e2e(props, parts, counts, args.e2e_steps, dist)
        if rank == 0:
            print(json.dumps({"metric": METRIC, "e2e": res}))
        return 0

    if args.only == "fp64":  # the FP64 GPU path alone (profiling runs of its push)
        sim64 = g.Simulation(props, make_config(abi.FP64))
        sim64.upload_particles(parts, counts)
        ms64, psteps64, launches64, n0, _ = run_timed(sim64, args.warmup, args.steps, pre_steps=0)
        roof64 = push_roofline(sim64, "fp64", 2, props, 2)
        out = {"metric": METRIC, "value": psteps64 / (ms64 * 1e-3), "unit": UNIT, "n_gpus": world,
               "steps": args.steps, "ms_per_step": ms64 / args.steps, "roofline": roof64, "stats": sim64.stats(),
               "gpu_launches": int(launches64), "dtype": "f64"}
        if rank == 0:
            print(json.dumps(out))
        sim64.close()
        return 0

    # ---- FP32 headline ----
    sim32 = g.Simulation(props, make_config(abi.FP32))
    sim32.upload_particles(parts, counts)
    if args.push_shape:
        item, item_cells, bps = (int(v) for v in args.push_shape.split(","))
        sim32.set_push_shape(item=item, item_cells=item_cells, blocks_per_sm=bps)
    if dist:
        dist.barrier()
    sampler = ClockSampler(local)
    ms32, psteps32, launches32, n0, tune_steps = run_timed(sim32, args.warmup, args.steps, sampler)
    shape32 = sim32.push_shape()
    if dist:
        dist.barrier()
    ms32, psteps32 = combine_ranks(ms32, psteps32, dist, "cuda")
    value32 = psteps32 / (ms32 * 1e-3)
    stats32 = sim32.stats()

    if args.only == "fp32":
        roof = push_roofline(sim32, "fp32", 20, props, 2)
        out = {"metric": METRIC, "value": value32, "unit": UNIT, "n_gpus": world, "steps": args.steps,
               "ms_per_step": ms32 / args.steps, "roofline": roof, "stats": stats32, "gpu_launches": int(launches32),
               "push_shape": shape32, "autotune_steps": tune_steps}
        if rank == 0:
            print(json.dumps(out))
        return 0

    # ---- FP64 GPU path, same inputs and steps ----
    sim64 = g.Simulation(props, make_config(abi.FP64))
    sim64.upload_particles(parts, counts)
    ms64, psteps64, _, _, _ = run_timed(sim64, args.warmup, args.steps, pre_steps=tune_steps)
    # error of the FP32 path against the FP64 GPU path: both ran the same
    # autotune + warm-up + timed steps from the same particles
    c32, c64 = sim32.conserved(), sim64.conserved()
    tot = lambda c: c["kinetic_energy"] + c["e_energy"] + c["b_energy"]
    err = {"steps": tune_steps + args.warmup + args.steps,
           "total_energy_rel": abs(tot(c32) - tot(c64)) / abs(tot(c64)),
           "kinetic_energy_rel": abs(c32["kinetic_energy"] - c64["kinetic_energy"]) / abs(c64["kinetic_energy"]),
           "particles_fp32": c32["particles"], "particles_fp64": c64["particles"]}
    value64 = psteps64 / (ms64 * 1e-3)
    stats64 = sim64.stats()
    # ---- live roofline of the push kernels (eager steps, CUDA events) ----
    roof = push_roofline(sim32, "fp32", 20, props, 2)
    roof64 = push_roofline(sim64, "fp64", 10, props, 2)
    sim64.close()

    # ---- end to end through the public API, host buffers ----
    e2e_res = run_e2e(props, parts, counts, args.e2e_steps, dist)

    tracer_row = None
    if not args.no_tracer and world == 1:  # pic_tracer's default run (its own metric), beside the headline
        try:
            tracer_row = run_tracer(3, 5, local, cpu_budget=8.0,
                                    cpu=rank == 0 and world == 1 and not args.no_cpu_baseline)
        except Exception as e:  # the headline line is printed regardless
            tracer_row = {"error": "%s: %s" % (type(e).__name__, e)}
        torch.cuda.empty_cache()

    ens = None
    if not args.no_ensemble:
        ens = run_ensemble(args.universes, args.warmup, args.ensemble_steps, local)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        pre = tune_steps + args.warmup
        v, cores, done, secs = cpu_port_run(props, parts, counts, pre, 50, args.cpu_budget)
        cpu = {"value": v, "unit": UNIT, "cores": cores, "kind": "port",
               "sample": "the full workload (8,388,608 particles), %d timed steps (%.1f s) after %d untimed steps "
                         "(the autotuner's trials and the warm-up), all host threads" % (done, secs, pre)}

    # ---- error of every output at the headline size, against both oracles ----
    errors = None
    if rank == 0 and not args.no_error:
        errors = headline_errors(props, parts, counts, args.error_steps, args.error_cpu_steps)

    # ---- the largest single-GPU configuration and the reference's own mode ----
    configs = {}
    if rank == 0 and world == 1 and not args.no_configs:
        for name, steps in (("c5", args.c5_steps), ("udist", 20)):
            try:
                configs[name] = run_config(name, args.warmup, local, steps=steps, cpu=not args.no_cpu_baseline)
            except Exception as e:  # the headline line is printed regardless
                configs[name] = {"error": "%s: %s" % (type(e).__name__, e)}
            torch.cuda.empty_cache()

    out = {
        "metric": METRIC, "value": value32, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms32 / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": headline_config(tune_steps + args.warmup),
        "setup": {"precision": "fp32 push/deposit (cell-relative), fp64 node moments/fields/reductions",
                  "particles_at_timing": int(n0), "graph": True,
                  "parallelism": "replicas" if world > 1 else "single", "push_shape": shape32,
                  "autotune_steps": tune_steps},
        "roofline": roof,
        "fp64": {"value": value64, "ms_per_step": ms64 / args.steps, "roofline": roof64, "stats": stats64},
        "fp32_over_fp64": value32 / value64,
        "error_fp32_vs_fp64": err,
        "error": errors,
        "stats": stats32,
        "cpu_baseline": cpu,
        "ensemble": ens,
        "tracer": tracer_row,
        "c5": configs.get("c5"),
        "udist": configs.get("udist"),
        "e2e": e2e_res,
        "clocks": sampler.summary(),
        "gpu_launches": int(launches32),
    }
    if rank == 0:
        print(json.dumps(out))
    sim32.close()
    if dist:
        dist.destroy_process_group()
    return 0


if __name__ == "__main__":
    sys.exit(main())
