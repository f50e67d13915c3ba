#!/usr/bin/env python3
"""Benchmarks of the GB300 FDTD engine.

Headline (one bench step = one whole simulation): 3-D Yee grid 256^3, FP64, 1000 time
steps; x-directed Gaussian plane wave (pulse 1/e half-width 14.1 cells = 28 steps) injected
through a TF/SF box [32,223]^3 that sits 16 cells inside a 16-cell CPML (m=3, kappa 15);
centred 48^3 dielectric cube eps_r = 6; snapshots of Ex..Hz every 250 steps; 8 seeded
point probes recording all six components every step.  Synthetic inputs of the stated
shapes (the reference ships no dataset).

value : Gcell-updates/s with the material already resident on the GPU (fields reset on
        the device, snapshots staged to pinned host memory as part of the workload).
e2e   : the same through the public API from host buffers: each step uploads the three
        material arrays from pinned memory and reads back every snapshot and the probe
        series.
roofline: FP64 bound.  The dominant update kernel's FP64 pipe instructions per launch over
        its mean CUDA-event time, against the FP64 FMA issue rate of a measured cuBLAS
        DGEMM; beside it the HBM fraction of the whole step (compulsory bytes per step from
        lx_params_step_bytes over ms_per_step) and of the dominant kernel alone.
configs: the other configurations, each with its own HBM roofline (compulsory bytes per
        cell update x cell updates / wall time): the 512^2 planar CPML run (FP64), the
        photonic-crystal precision study (FP64/FP32/FP16 storage, errors vs FP64), the
        256-lens batch (FP32) and a shortened Poisson serving stream (p50/p99).
cpu_baseline / --impl reference: the oracle (CPU restatement of the reference's loops,
        OpenMP like the reference, built -O3 like it) on the host cores, one process x all
        threads, on bounded samples of each configuration, with and without snapshot writes.
"""
from __future__ import annotations

import argparse
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "Gcell-updates/s & HBM GB/s vs peak, FP32 vs FP64 at stated err; p50/p99 latency"
UNIT = "Gcell-updates/s"
N = 256
STEPS = 1000
SNAP_EVERY = 250
CPML = 16
BOX = (32, 223)
CUBE = (104, 152)


def workload_params(precision: int = 0, n: int = N):
    """The 256^3 workload; n < 256 gives the same layout scaled down (profiling cases)."""
    from luxum_gb300 import params

    box = (CPML + 16, n - 1 - (CPML + 16))
    return params(isPlanar=0, Nx=n, Ny=n, Nz=n, dx=1e-3, dy=1e-3, dz=1e-3, S=0.5, num_timesteps=STEPS,
                  usePW=1, kx_pw=1.0, ky_pw=0.0, kz_pw=0.0, Ex_pw=0.0, Ey_pw=0.0, Ez_pw=1.0, off_pw=24.0,
                  x1_pw=box[0], x2_pw=box[1], y1_pw=box[0], y2_pw=box[1], z1_pw=box[0], z2_pw=box[1],
                  usePML=1, d_pml=CPML * 1e-3, sigma=0.65, sigma_m=3.0, kappa=15.0, a_max=0.0, a_m=1.0,
                  precision=precision, n_threads=os.cpu_count() or 1, monitor_every=1)


def planar_params(precision: int, n: int):
    """The 512^2 planar layout at n^2: CPML 20 cells, TF/SF box 10 cells inside it, Ey
    polarisation at normal incidence from the left."""
    from luxum_gb300 import params

    lo, hi = 30, n - 31
    return params(isPlanar=1, Nx=n, Ny=1, Nz=n, dx=1e-3, dy=1e-3, dz=1e-3, S=0.5, num_timesteps=STEPS,
                  usePW=1, kx_pw=1.0, ky_pw=0.0, kz_pw=0.0, Ex_pw=0.0, Ey_pw=1.0, Ez_pw=0.0, off_pw=26.0,
                  x1_pw=lo, x2_pw=hi, y1_pw=0, y2_pw=0, z1_pw=lo, z2_pw=hi, usePML=1, d_pml=20e-3, sigma=0.65,
                  sigma_m=3.0, kappa=5.0, a_max=0.05, a_m=1.0, precision=precision, n_threads=1, monitor_every=1)


def profile_case(n: int, steps: int, precision: int, planar: bool = False, io: bool = False) -> None:
    """Small case for ncu captures: the workload at n^3 (n=192: 0.6 GB resident at FP64,
    above the 129 MB L2), `steps` time steps after 60 untimed ones (wave inside the box).
    planar: the 512^2 layout at n^2 with its centred eps_r 10.89 square (n=4096: 0.47 GB at
    FP32 with the second state buffer).  io (3-D): the 8 probes every step and Ex..Hz
    snapshots every 2 steps, as the drop-in workload records them (probe and gather kernels)."""
    import __graft_entry__

    __graft_entry__.build()
    from luxum_gb300 import Sim

    if planar:
        sim = Sim(planar_params(precision, n))
        a, b = n * 224 // 512, n * 288 // 512
        sim.set_eps_box((a, 0, a), (b, 1, b), 10.89)
        sim.step(60)
        kt = sim.time_kernels(steps)  # CUDA events around each launch (meaningless under ncu)
        ms = kt["h_update"] + kt["e_update"]
        print(json.dumps({"profile_case": n, "planar": 1, "steps": 60 + steps, "precision": precision,
                          "update_ms_per_step": ms, "gcell_per_s": n * n / ms * 1e-6, "max_e2": sim.max_e2(),
                          "two_sweep": os.environ.get("LUXUM_TWO_SWEEP") == "1"}))
        sim.close()
        return
    sim = Sim(workload_params(precision, n))
    a, b = n * 104 // 256, n * 152 // 256
    sim.set_eps_box((a, a, a), (b, b, b), 6.0)
    if io:
        sim.set_probes(np.clip(probe_points() * n // N, 1, n - 2), 60 + steps)
        sim.set_snapshots(2, 0x3F, lambda t, c, arr: None)
    sim.step(60)
    sim.step(steps)
    sim.sync()
    print(json.dumps({"profile_case": n, "steps": 60 + steps, "precision": precision, "max_e2": sim.max_e2()}))
    sim.close()


def probe_points():
    rng = np.random.default_rng(2026)
    return rng.integers(BOX[0], BOX[1] + 1, size=(8, 3)).astype(np.int32)


def material(shape):
    """F of the reference's material files: Cb = dt/(eps0*(1+F*1e6)) gives eps_r = 6 in the cube."""
    F = np.zeros(shape)
    a, b = CUBE
    F[a:b, a:b, a:b] = (6.0 - 1.0) / 1e6
    return F


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) == 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in self.rows for i in range(4) if r[3 + i].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(self.rows), "reasons": reasons}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def fp64_peak_tflops(torch) -> float:
    """cuBLAS DGEMM 8192^3 (best of 3): the measured FP64 roof of this GPU."""
    a = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    b = torch.randn(8192, 8192, dtype=torch.float64, device="cuda")
    torch.matmul(a, b)
    torch.cuda.synchronize()
    best = 1e9
    for _ in range(3):
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        torch.matmul(a, b)
        e1.record()
        e1.synchronize()
        best = min(best, e0.elapsed_time(e1))
    del a, b
    return 2 * 8192 ** 3 / (best * 1e-3) / 1e12


def kernel_model(sim, p):
    """Algorithmic bytes and FP64 pipe instructions per launch of the H and E kernels.

    Bytes: every array a kernel must touch, once: H kernel reads E (3) and H (3) and writes
    H (3); E kernel reads H (3), E (3), Cb (3) and writes E (3); each stored psi entry is
    read and written once.  FP64 instructions per component: 2 differences, 1 subtraction
    and 1 FMA (4); per psi term: psi = b*psi + c*d (a multiply and an FMA) and d/kappa + psi
    (an FMA), 3; with the max monitor every step the E kernel also forms
    |E|^2 = Ex^2 + Ey^2 + Ez^2 per cell (a multiply and two FMAs, 3).  Flops count an FMA as 2.
    """
    info = sim.info()
    el = info["field_bytes"]
    cel = 8 if p.precision == 0 else 4
    cells = info["cells"]
    psi_h, psi_e = info["psi_h_entries"], info["psi_e_entries"]
    mon = p.monitor_every == 1
    h_bytes = cells * 9 * el + psi_h * 2 * cel
    e_bytes = cells * 9 * el + cells * 3 * cel + psi_e * 2 * cel
    h_ops = cells * 12 + psi_h * 3
    e_ops = cells * 12 + psi_e * 3 + (cells * 3 if mon else 0)
    h_flops = cells * 15 + psi_h * 5
    e_flops = cells * 15 + psi_e * 5 + (cells * 5 if mon else 0)
    return {"h_update": (h_bytes, h_ops, h_flops), "e_update": (e_bytes, e_ops, e_flops)}


def hbm_roof(bytes_per_step: float, steps: float, seconds: float, peak: float, peak_kind: str, **extra):
    """HBM roofline of a run: compulsory bytes per time step x time steps / wall time."""
    achieved = bytes_per_step * steps / seconds / 1e9
    d = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
         "peak_source": peak_kind, "bytes_per_step": bytes_per_step}
    d.update(extra)
    return d


# ------------------------------------------------------------------ CPU baseline (the oracle port)

def cpu_info(threads: int) -> dict:
    """One process (the reference's MPI is absent here, so one rank) x `threads` OpenMP threads."""
    model = None
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        for line in out.splitlines():
            if line.startswith("Model name:"):
                model = line.split(":", 1)[1].strip()
                break
    except (OSError, subprocess.SubprocessError):
        pass
    return {"ranks": 1, "threads": threads, "cores": threads, "cpu_model": model, "host_cpus": os.cpu_count(),
            "build": "gcc -O3 -fopenmp -ffp-contract=off (the reference builds with -O3, src/solvers/CMakeLists.txt:22)"}


def _dropin_oracle(threads: int):
    from oracle.oracle import OracleSim

    p = workload_params(0)
    o = OracleSim(p, threads=threads)
    for c in range(3):
        o.set_material(c, material(o.shape(c)), 1e6)
    o.step(1)  # first touch of the arrays
    return o


def run_cpu_sample(steps: int, threads: int):
    """`steps` time steps of the 256^3 workload on the oracle; (Gcell-updates/s, seconds)."""
    o = _dropin_oracle(threads)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    return N ** 3 * steps / dt / 1e9, dt


def _write_cost(o, comps, tmpdir: str) -> float:
    """Seconds to write one snapshot of `comps` (their contiguous doubles, one file each)."""
    t0 = time.perf_counter()
    for c in comps:
        o.append_raw(c, os.path.join(tmpdir, f"snap{c}.raw"))
    dt = time.perf_counter() - t0
    for c in comps:
        os.remove(os.path.join(tmpdir, f"snap{c}.raw"))
    return dt


def cpu_dropin(steps: int, threads: int) -> dict:
    """The 256^3 drop-in on the oracle: `steps` time steps timed without writes, one Ex..Hz
    snapshot write timed on its own, the 1000-step run (4 snapshots) extrapolated from both."""
    import tempfile

    o = _dropin_oracle(threads)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    with tempfile.TemporaryDirectory() as d:
        snap = _write_cost(o, range(6), d)
    o.close()
    run_s = dt * STEPS / steps
    return {"value": N ** 3 * steps / dt / 1e9, "unit": UNIT,
            "value_with_snapshots": N ** 3 * STEPS / (run_s + 4 * snap) / 1e9,
            "sample": f"{steps} time steps of the 1000-step 256^3 run ({N ** 3 * steps:.3g} cell-updates, {dt:.1f} s); "
                      f"one Ex..Hz snapshot write ({6 * 8 * N ** 3 / 1e9:.2f} GB, {snap:.2f} s) timed separately; "
                      "value_with_snapshots extrapolates to 1000 steps with 4 snapshots"}


def cpu_planar_full(threads: int) -> dict:
    """The 512^2 planar CPML configuration on the oracle, all 2000 steps, without and with the
    driver's Ey writes every 10 steps (two_dim_pml.cc:184)."""
    import tempfile

    from oracle.oracle import OracleSim

    out = {}
    for writes in (False, True):
        o = OracleSim(planar_params(0, 512), threads=threads)
        o.set_eps_box((224, 0, 224), (288, 1, 288), 10.89)
        with tempfile.TemporaryDirectory() as d:
            path = os.path.join(d, "Ey.raw")
            t0 = time.perf_counter()
            if writes:
                for t in range(2000):
                    o.step(1)
                    if t % 10 == 0:
                        o.append_raw(1, path)
            else:
                o.step(2000)
            dt = time.perf_counter() - t0
        o.close()
        out["value_with_snapshots" if writes else "value"] = 512 * 512 * 2000 / dt / 1e9
        out["seconds_with_snapshots" if writes else "seconds"] = dt
    out.update(unit=UNIT, sample="the full 2000-step run, without and with the 200 Ey writes")
    return out


def cpu_phc_window(steps: int, threads: int) -> dict:
    """A window of the photonic-crystal run on the oracle (FP64, both DFT planes), extrapolated."""
    from oracle.oracle import OracleSim

    c = PHC
    g_params = phc_params(0)
    o = OracleSim(g_params, threads=threads)
    for lo, hi, eps in phc_rods():
        o.set_eps_box(lo, hi, eps)
    o.add_dft_plane(0, 40, PHC_OMEGA, every=5)
    o.add_dft_plane(0, 470, PHC_OMEGA, every=5)
    o.step(1)
    t0 = time.perf_counter()
    o.step(steps)
    dt = time.perf_counter() - t0
    o.close()
    cells = c["nx"] * c["ny"] * c["nz"]
    v = cells * steps / dt / 1e9
    return {"value": v, "unit": UNIT, "sample": f"{steps}-step window of the 4000-step run ({dt:.1f} s); the full "
                                                f"run extrapolates to {cells * c['steps'] / v / 1e9 / 60:.0f} min"}


def cpu_lens_subset(n_sims: int, steps: int, threads: int) -> dict:
    """The first `n_sims` lens simulations of the batch workload, `steps` steps each, one after
    the other on the oracle (the reference runs one simulation per invocation)."""
    from oracle.oracle import OracleSim

    work = 0
    dt = 0.0
    for p, F in lens_specs(n_sims, 4, 0, steps):
        o = OracleSim(p, threads=threads)
        o.set_material(1, F, 1.0)
        o.step(1)
        t0 = time.perf_counter()
        o.step(steps)
        dt += time.perf_counter() - t0
        work += p.Nx * p.Nz * steps
        o.close()
    v = work / dt / 1e9
    return {"value": v, "unit": UNIT, "sample": f"{n_sims} of the 256 simulations, {steps} of their 3000 steps each "
                                                f"({work:.3g} cell-updates, {dt:.1f} s)"}


def lens_specs(n_sims: int, seed: int, precision: int, steps: int):
    """The batch workload: planar lens simulations of uneven size (seeded), as (params, F).

    Side N ~ U{128..1024}; half elliptic lenses (semi-axes 10-40 % of N, eps_r ~ U(1.5, 2.25)),
    half distorted lenses (same ellipse with a sinusoidal boundary perturbation of up to
    5 cells); Ey plane wave at normal incidence from the left through a TF/SF box 16 cells
    inside a 16-cell CPML (textbook CPML sign, kappa 5, a_max 0.05).  The lens enters as the
    material array F of Cb = dt/(eps0*(1+F)), i.e. F = eps_r - 1 on Ey (scale 1).
    """
    from luxum_gb300 import params

    rng = np.random.default_rng(seed)
    out = []
    for q in range(n_sims):
        n = int(rng.integers(128, 1025))
        box = (32, n - 33)
        p = params(isPlanar=1, Nx=n, Ny=1, Nz=n, dx=1e-3, dy=0.0, dz=1e-3, S=0.5, num_timesteps=steps, usePW=1,
                   kx_pw=1.0, Ey_pw=1.0, off_pw=24.0, x1_pw=box[0], x2_pw=box[1], z1_pw=box[0], z2_pw=box[1],
                   usePML=1, d_pml=0.016, sigma=0.65, sigma_m=3.0, kappa=5.0, a_max=0.05, a_m=1.0,
                   cpml_mode=1, precision=precision)
        a, b = rng.uniform(0.1, 0.4, 2) * n
        eps = rng.uniform(1.5, 2.25)
        x = np.arange(n)[:, None] - n / 2
        z = np.arange(n)[None, :] - n / 2
        r2 = (x / a) ** 2 + (z / b) ** 2
        if q % 2:
            th = np.arctan2(z / b, x / a)
            amp = rng.uniform(1.0, 5.0) / min(a, b)
            m = int(rng.integers(3, 9))
            inside = np.sqrt(r2) <= 1.0 + amp * np.sin(m * th + rng.uniform(0, 2 * np.pi))
        else:
            inside = r2 <= 1.0
        out.append((p, np.where(inside, eps - 1.0, 0.0).reshape(n, 1, n)))
    return out


def lens_sims(n_sims: int, seed: int, precision: int, steps: int):
    """Handles of lens_specs' simulations, with their lens maps on the device."""
    from luxum_gb300 import Sim

    sims = []
    for p, F in lens_specs(n_sims, seed, precision, steps):
        s = Sim(p)
        s.set_material(1, F, 1.0)
        sims.append(s)
    return sims


def box_sims(n_sims: int, seed: int, precision: int, steps: int, side=(64, 192)):
    """3-D batch workload: cubes of side U{64..192} (seeded), the serving requests' 3-D form:
    textbook CPML of min(16, side/8) cells, an Ez plane wave along x through a TF/SF box as
    deep again, and 1-4 dielectric boxes with eps_r ~ U(1, 12).  `side`: another side range
    (cubes under 64^3 share the batched 3-D launches; larger ones are launched one by one)."""
    from luxum_gb300 import Sim

    rng = np.random.default_rng(seed)
    sims = []
    for q in range(n_sims):
        n = int(rng.integers(side[0], side[1] + 1))
        m = serve_margin(n)
        p = serve_params({"side": n, "planar": False})
        p.precision = precision
        p.num_timesteps = steps
        s = Sim(p)
        for _ in range(int(rng.integers(1, 5))):
            c0 = rng.integers(2 * m + 2, n - 2 * m - 8, 3)
            w = rng.integers(4, max(5, n // 6), 3)
            lo = np.maximum(c0 - w // 2, 2 * m + 2)
            hi = np.minimum(c0 + w // 2, n - 2 * m - 8)
            s.set_eps_box(tuple(int(v) for v in lo), tuple(int(v) for v in hi), float(rng.uniform(1.0, 12.0)))
        sims.append(s)
    return sims


def run_batch(n_sims: int, steps: int, three: bool, runs: int, solo_sample: int, solo_steps: int, peak: float,
              peak_kind: str, side=(64, 192), march_fixed: int = 0) -> dict:
    """Uneven simulations stepped as one batch: planar lenses, or 3-D cubes (three)."""
    import torch

    from luxum_gb300 import Batch, step_bytes

    sims = box_sims(n_sims, 6, 1, steps, side) if three else lens_sims(n_sims, 4, 1, steps)
    cells = sum(s.p.Nx * s.p.Ny * s.p.Nz for s in sims)
    bytes_step = sum(step_bytes(s.p) for s in sims)
    batch = Batch(chunk=100)
    for s in sims:
        batch.add(s)
    t_tune = time.perf_counter()
    if march_fixed:  # a given tile shape (profiling runs: no tuning launches before the steps)
        batch.set_march(march_fixed, march_fixed)
        march = (march_fixed, march_fixed)
    else:
        march = batch.autotune(20)  # tile shape timed on twins of the members, outside the timed region
    t_tune = time.perf_counter() - t_tune

    def run():
        for s in sims:
            s.reset()
        batch.step(steps)

    run()  # warm-up: graph capture, first touch
    torch.cuda.synchronize()
    with ClockSampler(0) as clk:
        t0 = time.perf_counter()
        for _ in range(runs):
            run()
        torch.cuda.synchronize()
        dt = time.perf_counter() - t0
    value = cells * steps * runs / dt / 1e9
    # the same simulations one by one (unbatched), on a sample
    sample = sims[:solo_sample]
    scells = sum(s.p.Nx * s.p.Ny * s.p.Nz for s in sample)
    for s in sample:
        s.reset()
        s.step(100)
        s.sync()
    t0 = time.perf_counter()
    for s in sample:
        s.reset()
        s.step(solo_steps)
        s.sync()
    solo = scells * solo_steps / (time.perf_counter() - t0) / 1e9
    desc = (f"batch of {len(sims)} 3-D simulations, cubes of side U{{{side[0]}..{side[1]}}} seed 6, CPML min(16, side/8), TF/SF "
            f"plane wave, 1-4 eps boxes, FP32, {steps} steps, graph chunks of 100" if three else
            f"batch of {len(sims)} planar lens simulations, sides U{{128..1024}} seed 4, "
            f"CPML 16, TF/SF normal incidence, FP32, {steps} steps, graph chunks of 100")
    table = batch.tune_table()
    batch.close()
    for s in sims:
        s.close()
    return {"config": {"workload": desc, "cells": cells, "cell_updates_per_run": cells * steps,
                       "l2": f"no flush: resident state {bytes_step / 2 ** 30:.1f} GiB of traffic per step >> 129 MB L2"},
            "metric": "Gcell-updates/s (batched)", "value": value, "unit": UNIT, "runs": runs,
            "s_per_run": dt / runs, "dtype": "f32",
            "roofline": hbm_roof(bytes_step, steps * runs, dt, peak, peak_kind, bytes_per_cell_update=bytes_step / cells),
            "unbatched_sample": {"sims": len(sample), "value": solo, "steps": solo_steps,
                                 "note": "same simulations stepped one handle at a time with lx_sim_step"},
            "batched_over_unbatched": value / solo, "autotuned_march": {"planar_rows": march[0], "planes_3d": march[1],
                                                                       "table": table, "seconds": t_tune},
            "clocks": clk.summary()}


def bench_batch(args):
    """--config batch: 256 uneven planar simulations stepped as one batch (batch3d: 3-D cubes)."""
    import __graft_entry__

    __graft_entry__.build()
    peak, kind = measured_peaks()
    print(json.dumps(run_batch(args.batch_sims, args.batch_steps, args.config == "batch3d", args.steps,
                               args.solo_sample, args.solo_steps, peak, kind,
                               (args.batch_side_lo, args.batch_side_hi), args.batch_march)), flush=True)


def serve_requests(n: int, seed: int, rate: float):
    """Request stream: Poisson arrivals; 80 % planar (side log-uniform 256..2048), 20 % 3-D
    (side log-uniform 64..256); 1-8 random dielectric boxes with eps_r ~ U(1, 12)."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, n))
    reqs = []
    for q in range(n):
        planar = rng.random() < 0.8
        lo, hi = (256, 2048) if planar else (64, 256)
        side = int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))
        m = serve_margin(side)
        lo_b, hi_b = 2 * m + 2, side - 2 * m - 8  # scatterers between the TF/SF face and the monitor plane
        boxes = []
        for _ in range(int(rng.integers(1, 9))):
            c0 = rng.integers(lo_b, hi_b, 3)
            w = rng.integers(4, max(5, side // 6), 3)
            a = np.maximum(c0 - w // 2, lo_b)
            b = np.minimum(c0 + w // 2, hi_b)
            boxes.append(((int(a[0]), 0 if planar else int(a[1]), int(a[2])),
                          (int(b[0]), 1 if planar else int(b[1]), int(b[2])), float(rng.uniform(1.0, 12.0))))
        reqs.append({"id": q, "arrival": float(t[q]), "planar": planar, "side": side, "boxes": boxes})
    return reqs


SERVE_STEPS = 2000


def serve_margin(side: int) -> int:
    """CPML depth (cells); the TF/SF box starts the same depth further in."""
    return min(16, side // 8)
SERVE_OMEGA = 2 * np.pi * np.linspace(0.5e9, 10e9, 64)  # monitor frequencies (rad/s)


def serve_params(req):
    from luxum_gb300 import params

    n = req["side"]
    m = serve_margin(n)
    box = (2 * m, n - 1 - 2 * m)
    kw = dict(dx=1e-3, dy=1e-3, dz=1e-3, S=0.5, num_timesteps=SERVE_STEPS, usePW=1, kx_pw=1.0, off_pw=56.0 - 2 * m,
              x1_pw=box[0], x2_pw=box[1], y1_pw=box[0], y2_pw=box[1], z1_pw=box[0], z2_pw=box[1], usePML=1,
              d_pml=m * 1e-3, sigma=0.65, sigma_m=3.0, kappa=5.0, a_max=0.05, a_m=1.0, cpml_mode=1, precision=1)
    if req["planar"]:
        return params(isPlanar=1, Nx=n, Ny=1, Nz=n, Ey_pw=1.0, y1_pw=0, y2_pw=0, **{k: v for k, v in kw.items()
                                                                                 if k not in ("y1_pw", "y2_pw")})
    return params(isPlanar=0, Nx=n, Ny=n, Nz=n, Ez_pw=1.0, **kw)


SERVE_TABLE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "luxum_gb300", "serve_tile_shapes.json")


def load_serve_table():
    """The committed tile-shape table of the serving stream's request classes (empty if absent)."""
    if not os.path.exists(SERVE_TABLE):
        return []
    with open(SERVE_TABLE) as f:
        return json.load(f)["table"]


def bench_serve_tune(args):
    """--config serve-tune: writes the serving stream's tile-shape table (serve_table) to
    SERVE_TABLE.  Run in a process of its own: tuning in the serving process slowed the stream
    that followed (47 against 55 Gcell/s on 1000 requests), whether or not its table was used."""
    import __graft_entry__

    __graft_entry__.build()
    reqs = serve_requests(args.serve_requests, 5, args.serve_rate)
    table, seconds = serve_table(reqs)
    with open(SERVE_TABLE, "w") as f:
        json.dump({"table": table, "tuned_on": "twins of the first 64 requests of the seeded serving stream "
                   "(lx_batch_autotune, 10 steps per timing)", "seconds": round(seconds, 3)}, f, indent=1)
        f.write("\n")
    print(json.dumps({"table": table, "seconds": seconds, "path": SERVE_TABLE}), flush=True)


def serve_table(reqs, n: int = 64, steps: int = 10):
    """Tile shapes per request class for the server: lx_batch_autotune on twins of the stream's
    first n requests (a fixed sample), before the stream starts.  Returns (table, seconds)."""
    from luxum_gb300 import Batch, Sim

    t0 = time.perf_counter()
    sims = []
    b = Batch(chunk=0)
    for r in reqs[:n]:
        s = Sim(serve_params(r))
        for lo, hi, eps in r["boxes"]:
            s.set_eps_box(lo, hi, eps)
        b.add(s)
        sims.append(s)
    b.autotune(steps)
    table = b.tune_table()
    b.close()
    for s in sims:
        s.close()
    return table, time.perf_counter() - t0


def run_serve(n_requests: int, rate: float, budget_gb: float, chunk: int, peak: float, peak_kind: str,
              tune_steps: int | None = None) -> dict:
    """A Poisson request stream through the native server (lx_server_*): continuous batching
    under an HBM budget, latency taken by the server's own clock."""
    import torch

    from luxum_gb300 import LX_PREC_FP32, Server, step_bytes

    reqs = serve_requests(n_requests, 5, rate)
    table = load_serve_table()
    srv = Server(precision=LX_PREC_FP32, chunk=chunk, budget_bytes=budget_gb * 1e9, tune_steps=tune_steps,
                 tune_table=table)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    ids = []
    with ClockSampler(0) as clk:
        for r in reqs:  # submit each request at its arrival time
            d = r["arrival"] - (time.perf_counter() - t0)
            if d > 0:
                time.sleep(d)
            plane = r["side"] - 1 - 2 * serve_margin(r["side"]) - 4
            ids.append(srv.submit(serve_params(r), SERVE_STEPS, r["boxes"], (0, plane, SERVE_OMEGA, 10)))
        lat, work, failed, traffic = [], 0, 0, 0.0
        for rid, r in zip(ids, reqs):
            if srv.wait(rid) != "done":
                failed += 1
                continue
            flux = srv.flux(rid)
            assert np.all(np.isfinite(flux))
            t = srv.times(rid)
            lat.append(t[2] - t[0])
            work += r["side"] ** (2 if r["planar"] else 3) * SERVE_STEPS
            traffic += step_bytes(serve_params(r)) * SERVE_STEPS
            srv.release(rid)
        wall = time.perf_counter() - t0
    st = srv.stats()
    table = srv.tune_table()
    srv.close()
    lat = np.array(lat)
    offered = sum(r["side"] ** (2 if r["planar"] else 3) for r in reqs) * SERVE_STEPS / reqs[-1]["arrival"] / 1e9
    return {"config": {"workload": f"{len(reqs)} requests, Poisson {rate}/s (seed 5), 80% planar 256-2048, "
                                   f"20% 3-D 64-256, 1-8 eps boxes, {SERVE_STEPS} steps FP32, FP64 DFT 64 freqs at one "
                                   f"plane (sampled every 10 steps), budget {budget_gb} GB, chunk {chunk}; native "
                                   "server (lx_server_*)"},
            "metric": "p50/p99 latency and aggregate Gcell-updates/s", "p50_s": float(np.percentile(lat, 50)),
            "p99_s": float(np.percentile(lat, 99)), "mean_s": float(lat.mean()), "value": work / wall / 1e9,
            "unit": UNIT, "offered_gcells": offered, "wall_s": wall, "completed": int(lat.size), "failed": failed,
            "roofline": hbm_roof(traffic, 1, wall, peak, peak_kind, bytes_per_cell_update=traffic / max(work, 1),
                                 note="compulsory bytes of every completed request over the stream's wall time"),
            "sustained": bool(work / wall / 1e9 >= 0.95 * offered),
            "peak_running": st["peak_running"], "peak_budget_gb": st["peak_bytes_running"] / 1e9,
            "chunks": st["chunks"], "gpu_busy_s": st["busy_seconds"],
            "worker_seconds": {k: st[k + "_seconds"] for k in ("enqueue", "prepare", "wait", "join", "retire", "tune")},
            "tuned_march": {"table": table, "source": SERVE_TABLE, "seconds_online": st["tune_seconds"],
                            "note": "tile shape per request class, from lx_batch_autotune on twins of the stream's "
                                    "first 64 requests (bench.py --config serve-tune, its own process), given to the "
                                    "server at creation; classes tuned online while serving (tune_steps) add to it"},
            "dtype": "f32", "clocks": clk.summary()}


def serve_in_child(n_requests: int, rate: float, budget_gb: float, chunk: int) -> dict:
    """The serving stream in a process of its own, as a server runs in deployment.  Run after the
    other workloads in this process, the stream's handle creation slowed threefold and its rate
    fell 10-15 % (the cause is not identified; the twins of a batch tuner are enough to show it)."""
    import subprocess

    cmd = [sys.executable, os.path.abspath(__file__), "--config", "serve", "--serve-requests", str(n_requests),
           "--serve-rate", str(rate), "--serve-budget-gb", str(budget_gb), "--serve-chunk", str(chunk)]
    out = subprocess.run(cmd, capture_output=True, text=True, timeout=1800)
    lines = [l for l in out.stdout.splitlines() if l.startswith("{")]
    if out.returncode != 0 or not lines:
        raise RuntimeError(f"serving child failed ({out.returncode}): {out.stderr[-2000:]}")
    d = json.loads(lines[-1])
    d["process"] = "its own (a child of the bench process)"
    return d


def bench_serve(args):
    """--config serve: the full request stream (1000 requests by default)."""
    import __graft_entry__

    __graft_entry__.build()
    peak, kind = measured_peaks()
    print(json.dumps(run_serve(args.serve_requests, args.serve_rate, args.serve_budget_gb, args.serve_chunk, peak,
                               kind, args.serve_tune_steps)), flush=True)


PHC = dict(nx=512, ny=512, nz=128, steps=4000, cpml=20, period=40, rod=16, eps=12.0)
PHC_OMEGA = 2 * np.pi * np.linspace(2.0e9, 3.6e9, 64)


def phc_params(precision: int):
    """Photonic-crystal waveguide: CPML 20; Gaussian-pulsed sine on Ez at the defect entrance
    (omega 1.76e10 rad/s = 2.8 GHz, width 159 steps, centred at step 480)."""
    from luxum_gb300 import params

    c = PHC
    p = params(isPlanar=0, Nx=c["nx"], Ny=c["ny"], Nz=c["nz"], dx=1e-3, dy=1e-3, dz=1e-3, S=0.5,
               num_timesteps=c["steps"], usePML=1, d_pml=c["cpml"] * 1e-3, sigma=0.65, sigma_m=3.0, kappa=5.0,
               a_max=0.05, a_m=1.0, cpml_mode=1, usePS=1, source_kind=1, amp_source=1.0,
               omega_source=2 * np.pi * 2.8e9, src_t0=480.0, src_tw=159.0, precision=precision)
    p.Nx_source, p.Ny_source, p.Nz_source = c["cpml"] + 4, phc_defect(), c["nz"] // 2
    return p


def phc_defect() -> int:
    centres = [20 + PHC["period"] * m for m in range(13)]
    return min(centres, key=lambda y: abs(y - PHC["ny"] // 2))


def phc_rods():
    """Square eps_r 12 rods (16x16 cells, period 40, full height), the row nearest mid-y
    removed: (lo, hi, eps_r) boxes."""
    c = PHC
    centres = [20 + c["period"] * m for m in range(13)]
    h = c["rod"] // 2
    return [((xc - h, yc - h, 0), (xc + h, yc + h, c["nz"]), c["eps"])
            for xc in centres for yc in centres if yc != phc_defect()]


def phc_sim(precision: int):
    """The waveguide with FP64 DFT planes (64 frequencies, 2.0-3.6 GHz) across the guide at
    x = 40 (input) and x = 470 (output)."""
    from luxum_gb300 import Sim

    s = Sim(phc_params(precision))
    for lo, hi, eps in phc_rods():
        s.set_eps_box(lo, hi, eps)
    planes = (s.add_dft_plane(0, 40, PHC_OMEGA, every=5), s.add_dft_plane(0, 470, PHC_OMEGA, every=5))
    return s, planes


def run_phc(peak: float, peak_kind: str) -> dict:
    """The waveguide run in FP64, FP32 and FP16 storage; errors against FP64."""
    import torch

    from luxum_gb300 import step_bytes

    c = PHC
    cells = c["nx"] * c["ny"] * c["nz"]
    out = {}
    ref = None
    for prec, name in ((0, "fp64"), (1, "fp32"), (2, "fp16_storage")):
        s, (pin, pout) = phc_sim(prec)
        s.step(1)  # first touch
        s.reset()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        s.step(c["steps"])
        s.sync()
        dt = time.perf_counter() - t0
        fin, fout = s.dft_flux(pin), s.dft_flux(pout)
        T = fout / np.where(np.abs(fin) > 0, fin, np.nan)
        fields = [s.field(k) for k in range(6)]
        sb = step_bytes(s.p)
        entry = {"value": cells * c["steps"] / dt / 1e9, "unit": UNIT, "seconds": dt,
                 "roofline": hbm_roof(sb, c["steps"], dt, peak, peak_kind, bytes_per_cell_update=sb / cells)}
        if ref is None:
            ref = (fields, T, fin, fout)
            entry["transmission"] = {"f_ghz": (PHC_OMEGA[::8] / 2 / np.pi / 1e9).round(3).tolist(),
                                     "T": np.round(T[::8], 4).tolist()}
        else:
            errs = {}
            for grp, comps in (("E", (0, 1, 2)), ("H", (3, 4, 5))):
                num = sum(float(np.linalg.norm(fields[k] - ref[0][k])) ** 2 for k in comps)
                den = sum(float(np.linalg.norm(ref[0][k])) ** 2 for k in comps)
                errs[grp] = (num / den) ** 0.5
            entry["field_rel_l2_vs_fp64"] = errs
            entry["T_max_abs_err_vs_fp64"] = float(np.nanmax(np.abs(T - ref[1])))
            entry["T_rel_l2_vs_fp64"] = float(np.sqrt(np.nansum((T - ref[1]) ** 2) / np.nansum(ref[1] ** 2)))
            # the band where the input plane carries at least 1 % of its peak power (outside it
            # T is a ratio of two small numbers)
            band = np.abs(ref[2]) >= 0.01 * np.abs(ref[2]).max()
            entry["T_max_abs_err_in_band"] = float(np.max(np.abs(T - ref[1])[band]))
            entry["band_ghz"] = [float(PHC_OMEGA[band].min() / 2 / np.pi / 1e9), float(PHC_OMEGA[band].max() / 2 / np.pi / 1e9)]
            entry["flux_out_rel_l2_vs_fp64"] = float(np.linalg.norm(fout - ref[3]) / np.linalg.norm(ref[3]))
            entry["speedup_vs_fp64"] = out["fp64"]["seconds"] / dt
        out[name] = entry
        del fields
        s.close()
    return {"config": {"workload": "3-D photonic-crystal waveguide 512x512x128, eps_r 12 rods 16x16 cells period 40 "
                                   "with a one-row line defect, CPML 20, pulsed Ez point source, 4000 steps; FP64 DFT "
                                   "transmission (64 frequencies 2.0-3.6 GHz, planes x=40 and x=470)",
                       "l2": "no flush: resident state >= 1.5 GB >> 129 MB L2"},
            "metric": "Gcell-updates/s and error vs FP64 per precision", "results": out}


def bench_phc(args):
    """--config phc: the waveguide run in FP64, FP32 and FP16 storage; errors against FP64."""
    import __graft_entry__

    __graft_entry__.build()
    peak, kind = measured_peaks()
    print(json.dumps(run_phc(peak, kind)), flush=True)


def run_planar(runs: int, peak: float, peak_kind: str) -> dict:
    """The 512^2 planar CPML configuration (FP64, 2000 steps, Ey snapshots every 10 steps as
    two_dim_pml.cc:184 writes them, max|E|^2 every step), `runs` runs after one untimed."""
    import torch

    from luxum_gb300 import Sim, step_bytes

    p = planar_params(0, 512)
    p.num_timesteps = 2000
    s = Sim(p)
    s.set_eps_box((224, 0, 224), (288, 1, 288), 10.89)
    stream = torch.cuda.current_stream()
    s.set_stream(stream.cuda_stream)
    s.set_snapshots(10, 1 << 1, lambda t, comp, arr: None)

    def one():
        s.reset()
        s.step(2000)
        s.sync()

    one()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(runs):
        one()
    e1.record(stream)
    torch.cuda.synchronize()
    sec = e0.elapsed_time(e1) * 1e-3
    kt = s.time_kernels(200)
    sb = step_bytes(p)
    s.close()
    return {"config": {"workload": "2-D 512x512 (x-z plane, Ey), FP64, 2000 steps, TF/SF box [30,481]^2 normal "
                                   "incidence, eps_r 10.89 square [224,288)^2, CPML 20 (m=3, kappa 5, a_max 0.05), "
                                   "Ey snapshot every 10 steps staged to pinned host memory, max|E|^2 every step",
                       "l2": "state 9 MB: L2-resident, so the HBM fraction is not a bound here"},
            "value": 512 * 512 * 2000 * runs / sec / 1e9, "unit": UNIT, "runs": runs, "s_per_run": sec / runs,
            "dtype": "f64", "kernel_ms": kt,
            "roofline": hbm_roof(sb, 2000 * runs, sec, peak, peak_kind, bytes_per_cell_update=sb / 512 ** 2)}


def dist_setup(n_gpus: int, backend: str | None = None):
    """Rank, world size, local rank and the process group module (None for one process).
    Under torchrun every rank runs an independent replica of the workload: the single
    simulation does not shard, and no collective runs on the data path."""
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    pg = None
    if world > 1:
        import torch.distributed as dist

        os.environ.setdefault("MASTER_ADDR", "127.0.0.1")
        dist.init_process_group(backend or ("nccl" if n_gpus > 1 else "gloo"))
        pg = dist
    return rank, world, local, pg


def rank_max(pg, x: float) -> float:
    """Maximum of a host number over ranks (the job's time is its slowest rank's)."""
    if not pg:
        return x
    import torch

    dev = "cuda" if pg.get_backend() == "nccl" else "cpu"
    t = torch.tensor([x], dtype=torch.float64, device=dev)
    pg.all_reduce(t, op=pg.ReduceOp.MAX)
    return float(t.item())


def job_rate(units_per_rank: float, world: int, ms_max: float) -> float:
    """Whole-job throughput in G units/s: every rank's units over the slowest rank's time."""
    return units_per_rank * world / (ms_max * 1e-3) / 1e9


def bench_reference(args):
    """--impl reference: the reference's CPU path (the oracle port) on all host threads."""
    rank, world, local, pg = dist_setup(args.gpus)
    if rank != 0:
        return
    threads = os.cpu_count() or 1
    sample = args.cpu_sample_steps
    for _ in range(args.warmup):
        run_cpu_sample(max(1, sample // 4), threads)
    vals = []
    t_all = 0.0
    for _ in range(args.steps):
        v, dt = run_cpu_sample(sample, threads)
        vals.append(v)
        t_all += dt
    value = float(np.mean(vals))
    cpu = cpu_info(threads)
    cpu.update(value=value, unit=UNIT, kind="port",
               sample=f"{sample} time steps of the 256^3 workload per bench step ({N ** 3 * sample:.3g} "
                      "cell-updates), no snapshot writes; the reference needs blitz++, yaml-cpp 0.3, MPI and HDF5 "
                      "and is not buildable here, so its loops run as the oracle restatement (same loop nests, "
                      "OpenMP, FP64)")
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * t_all / args.steps,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": config_dict(f"each step: {sample} time steps of the 1000-step run"),
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "cpu_baseline": cpu}
    print(json.dumps(line), flush=True)


def config_dict(extra: str = ""):
    d = {"workload": f"3D Yee {N}^3 FP64, {STEPS} steps, CPML {CPML} (m=3, kappa 15), TF/SF x-wave box "
                     f"[{BOX[0]},{BOX[1]}]^3, eps_r 6 cube [{CUBE[0]},{CUBE[1]})^3, Ex..Hz snapshots every "
                     f"{SNAP_EVERY} steps, 8 probes x 6 components every step, max|E|^2 every step",
         "grid": [N, N, N], "time_steps_per_bench_step": STEPS, "cell_updates_per_bench_step": N ** 3 * STEPS,
         "l2": "no flush: resident state 5.4 GB >> 129 MB L2", "parallelism": "replicas (one independent sim per GPU)"}
    if extra:
        d["sample"] = extra
    return d


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--cpu-sample-steps", type=int, default=40)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-precision", action="store_true", help="skip the FP32 / FP16-storage lines")
    ap.add_argument("--no-suite", action="store_true", help="skip the other configurations (planar, phc, batch, serve)")
    ap.add_argument("--suite-serve-requests", type=int, default=200, help="requests of the serving stream in the suite")
    ap.add_argument("--cpu-phc-steps", type=int, default=20)
    ap.add_argument("--cpu-lens-steps", type=int, default=200)
    ap.add_argument("--profile", type=int, default=0, metavar="N",
                    help="run the N^3 profiling case instead of the benchmark (for ncu)")
    ap.add_argument("--profile-steps", type=int, default=4)
    ap.add_argument("--precision", type=int, default=0, help="profiling case precision: 0 fp64, 1 fp32, 2 fp16")
    ap.add_argument("--planar", action="store_true", help="profiling case: the planar layout at N^2")
    ap.add_argument("--profile-io", action="store_true", help="profiling case (3-D): probes and snapshots too")
    ap.add_argument("--batch-side-lo", type=int, default=64, help="batch3d: smallest cube side")
    ap.add_argument("--batch-side-hi", type=int, default=192, help="batch3d: largest cube side")
    ap.add_argument("--config", default="drop-in", choices=["drop-in", "batch", "batch3d", "serve", "serve-tune", "phc"],
                    help="drop-in: the headline 256^3 FP64 workload; batch: 256 uneven planar simulations")
    ap.add_argument("--batch-sims", type=int, default=256)
    ap.add_argument("--batch-steps", type=int, default=3000)
    ap.add_argument("--batch-march", type=int, default=0, choices=[0, 1, 2, 4, 8],
                    help="tile shape of the batched kernels (0: autotune before the timed steps)")
    ap.add_argument("--solo-sample", type=int, default=16)
    ap.add_argument("--solo-steps", type=int, default=300)
    ap.add_argument("--serve-requests", type=int, default=1000)
    ap.add_argument("--serve-rate", type=float, default=50.0)
    ap.add_argument("--serve-budget-gb", type=float, default=150.0)
    ap.add_argument("--serve-chunk", type=int, default=100)
    ap.add_argument("--serve-tune-steps", type=int, default=None,
                    help="steps per march when the server tunes a new request class (0: default tile shapes)")
    args = ap.parse_args()
    if args.config in ("batch", "batch3d"):
        if args.config == "batch3d" and args.batch_sims == 256:
            args.batch_sims, args.batch_steps = 48, 1000
        return bench_batch(args)
    if args.config == "serve-tune":
        return bench_serve_tune(args)
    if args.config == "serve":
        return bench_serve(args)
    if args.config == "phc":
        return bench_phc(args)
    if args.profile:
        return profile_case(args.profile, args.profile_steps, args.precision, args.planar, args.profile_io)
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        return bench_reference(args)

    rank, world, local, pg = dist_setup(args.gpus)
    import torch

    torch.cuda.set_device(local)
    import __graft_entry__

    if rank == 0 or not os.path.exists(os.path.join(ROOT, "luxum_gb300", "libluxum.so")):
        __graft_entry__.build()
    if pg:
        pg.barrier()
    from luxum_gb300 import Sim, step_bytes

    p = workload_params(0)
    sim = Sim(p)
    stream = torch.cuda.current_stream()
    sim.set_stream(stream.cuda_stream)
    F = [material(sim.shape(c)) for c in range(3)]
    for c in range(3):
        sim.set_material(c, F[c], 1e6)
    ijk = probe_points()
    sim.set_probes(ijk, STEPS)
    snap_bytes = [0]

    def sink(t, comp, arr):
        snap_bytes[0] += arr.nbytes

    sim.set_snapshots(SNAP_EVERY, 0x3F, sink)

    def one_run():
        sim.reset()
        sim.step(STEPS)

    for _ in range(args.warmup):
        one_run()
    sim.sync()

    def barrier():
        if pg:
            pg.barrier()
        torch.cuda.synchronize()

    # ---- device-resident timed region
    k0 = sim.counters()[0]
    with ClockSampler(local) as clk:
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        for _ in range(args.steps):
            one_run()
        sim.sync()
        e1.record(stream)
        barrier()
    ms = rank_max(pg, e0.elapsed_time(e1))
    launches = sim.counters()[0] - k0
    cell_updates = N ** 3 * STEPS * args.steps * world
    value = job_rate(N ** 3 * STEPS * args.steps, world, ms)

    # ---- end to end through the public API with pinned host buffers
    Fp = []
    for c in range(3):
        buf = torch.empty(F[c].shape, dtype=torch.float64, pin_memory=True)
        buf.numpy()[...] = F[c]
        Fp.append(buf)
    probe_host = np.empty((STEPS, 8, 6))
    barrier()
    _, h2d0, d2h0 = sim.counters()
    e2 = torch.cuda.Event(enable_timing=True)
    e3 = torch.cuda.Event(enable_timing=True)
    t_host = time.perf_counter()
    e2.record(stream)
    for _ in range(args.steps):
        sim.reset()
        for c in range(3):
            sim.set_material(c, Fp[c].numpy(), 1e6)
        sim.step(STEPS)
        probe_host[...] = sim.probes()
        sim.sync()
    e3.record(stream)
    barrier()
    t_host = time.perf_counter() - t_host
    ms_e2e = max(e2.elapsed_time(e3), 1e3 * t_host)
    _, h2d1, d2h1 = sim.counters()
    ms_e2e = rank_max(pg, ms_e2e)
    e2e = {"value": job_rate(N ** 3 * STEPS * args.steps, world, ms_e2e), "unit": UNIT,
           "h2d_bytes_per_step": (h2d1 - h2d0) // args.steps, "d2h_bytes_per_step": (d2h1 - d2h0) // args.steps}

    # ---- roofline: FP64 pipe of the dominant update kernel (instrumented pass, events around
    # each launch), then the HBM fractions of the whole step and of that kernel
    sim.reset()
    sim.step(120)  # wave inside the box, psi active
    kt = sim.time_kernels(40)
    model = kernel_model(sim, p)
    dom = max(("h_update", "e_update"), key=lambda k: kt[k])
    bytes_alg, ops_alg, flops_alg = model[dom]
    peak_bw, peak_kind = measured_peaks()
    fp64_peak = fp64_peak_tflops(torch)  # FLOP/s of a DGEMM: FMA instructions at half this rate
    ops_rate = ops_alg / (kt[dom] * 1e-3) / 1e12
    step_b = step_bytes(p)
    roofline = {"bound": "fp64", "achieved": ops_rate, "peak": fp64_peak / 2, "unit": "T FP64 instructions/s",
                "frac": ops_rate / (fp64_peak / 2), "traffic": None, "kernel": dom,
                "peak_source": "measured cuBLAS DGEMM 8192^3 (FP64 FMA issue rate = its FLOP/s / 2)",
                "ops_per_launch": ops_alg, "ms_per_launch": kt[dom],
                "flops": {"achieved_tflops": flops_alg / (kt[dom] * 1e-3) / 1e12, "peak_tflops": fp64_peak,
                          "frac": flops_alg / (kt[dom] * 1e-3) / 1e12 / fp64_peak, "flops_per_launch": flops_alg},
                "hbm_step": hbm_roof(step_b, STEPS * args.steps, ms * 1e-3, peak_bw, peak_kind,
                                     bytes_per_cell_update=step_b / N ** 3,
                                     note="compulsory bytes per step (lx_params_step_bytes) over ms_per_step"),
                "hbm_kernel": {"achieved": bytes_alg / (kt[dom] * 1e-3) / 1e9, "peak": peak_bw, "unit": "GB/s",
                               "frac": bytes_alg / (kt[dom] * 1e-3) / 1e9 / peak_bw, "bytes_per_launch": bytes_alg,
                               "note": "the dominant kernel's own compulsory bytes over its launch time"},
                "kernel_ms": kt}
    traffic_file = os.path.join(ROOT, "profiles", "traffic.json")
    if os.path.exists(traffic_file):
        try:
            with open(traffic_file) as f:
                tr = json.load(f).get(dom)
            if tr:
                roofline["traffic"] = tr["bytes_per_launch"]
                roofline["traffic_unit"] = "bytes per launch (DRAM read + write)"
                roofline["traffic_source"] = tr["source"]
        except (OSError, ValueError):
            pass

    # ---- reduced-precision forms of the same workload: throughput and error vs this FP64 run
    precision = {}
    if not args.no_precision:
        sim.reset()
        sim.step(STEPS)
        sim.sync()
        ref = [sim.field(c) for c in range(6)]
        for prec, name in ((1, "fp32"), (2, "fp16_storage")):
            q = Sim(workload_params(prec))
            q.set_stream(stream.cuda_stream)
            for c in range(3):
                q.set_material(c, F[c], 1e6)
            q.set_probes(ijk, STEPS)
            q.set_snapshots(SNAP_EVERY, 0x3F, sink)
            q.reset()
            q.step(STEPS)
            q.sync()
            barrier()
            f0, f1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            f0.record(stream)
            for _ in range(args.steps):
                q.reset()
                q.step(STEPS)
            q.sync()
            f1.record(stream)
            barrier()
            qms = rank_max(pg, f0.elapsed_time(f1))
            errs = {}
            for grp, comps in (("E", (0, 1, 2)), ("H", (3, 4, 5))):
                num = sum(float(np.linalg.norm(q.field(c) - ref[c])) ** 2 for c in comps)
                den = sum(float(np.linalg.norm(ref[c])) ** 2 for c in comps)
                errs[grp] = (num / den) ** 0.5 if den else None
            kq = q.time_kernels(40)
            qb = step_bytes(q.p)
            precision[name] = {"value": cell_updates / (qms * 1e-3) / 1e9, "unit": UNIT,
                               "ms_per_step": qms / args.steps, "speedup_vs_fp64": ms / qms,
                               "rel_l2_vs_fp64_after_1000_steps": errs, "kernel_ms": kq,
                               "roofline": hbm_roof(qb, STEPS * args.steps, qms * 1e-3, peak_bw, peak_kind,
                                                    bytes_per_cell_update=qb / N ** 3)}
            q.close()
        del ref

    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic", "config": config_dict(),
            "e2e": e2e, "roofline": roofline, "clocks": clk.summary(), "gpu_launches": launches,
            "max_e2_final": sim.max_e2(), "precision_forms": precision}
    sim.close()
    if rank == 0 and world == 1 and not args.no_suite:
        line["configs"] = {
            "planar_512_fp64": run_planar(5, peak_bw, peak_kind),
            "phc_precision_study": run_phc(peak_bw, peak_kind),
            "lens_batch_fp32": run_batch(256, 3000, False, 1, args.solo_sample, args.solo_steps, peak_bw, peak_kind),
            "serving_stream": serve_in_child(args.suite_serve_requests, args.serve_rate, args.serve_budget_gb,
                                             args.serve_chunk)}
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        threads = os.cpu_count() or 1
        cpu = cpu_info(threads)
        drop = cpu_dropin(args.cpu_sample_steps, threads)
        cpu.update(value=drop["value"], unit=UNIT, kind="port", sample=drop["sample"],
                   value_with_snapshots=drop["value_with_snapshots"])
        if not args.no_suite:
            cpu["configs"] = {"planar_512_fp64": cpu_planar_full(threads),
                              "phc_precision_study": cpu_phc_window(args.cpu_phc_steps, threads),
                              "lens_batch_fp32": cpu_lens_subset(16, args.cpu_lens_steps, threads)}
        line["cpu_baseline"] = cpu
    if rank == 0:
        print(json.dumps(line), flush=True)
    if pg:
        pg.barrier()
        pg.destroy_process_group()


if __name__ == "__main__":
    main()
