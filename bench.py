#!/usr/bin/env python3
"""Spin-trials/s of the Metropolis anneal on one GB300.

Workload (the headline configuration): a 256x256x1 film, dx = dy = 1 nm,
dz = 0.8 nm, Ms = 1.6e6 A/m, Aex = 16 pJ/m, Dind = 6 mJ/m^2, Ku1 = 2 MJ/m^3
along z, Bext = 0.3 T along z, 20 periodic images in x and y, open in z, demag
on, random unit-vector start from seed 256, anneal 1400 K -> 40 K by x0.90 per
stage with 10000 Metropolis sweeps per stage.  One bench step is one
temperature stage (10000 sweeps) of a batch of R = 64 replicas of that film
(seeds 256..319), all replicas advanced by every kernel launch (the replica
count of the batched path is free; throughput peaks around 64, whose working
set of ~200 MB is larger than L2).  The lattice states are resident in HBM
between steps; an L2 flush (a 512 MB write) separates the timed steps.  FP32
bulk arithmetic ("f32").  One lattice in FP32 and the plain FP64 path are timed
on the same film as well, and the FP64 CPU oracle on the host cores.

    python bench.py [--steps K] [--warmup W] [--gpus N] [--impl ours|reference]

N > 1 runs one independent replica per GPU (seeds 256 + rank); rank 0 prints
one JSON line.
"""
import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
PKG = os.path.join(ROOT, "micromagnetic-gpu-monte-carlo_gb300")
for p in (PKG, os.path.join(ROOT, "oracle")):
    if p not in sys.path:
        sys.path.insert(0, p)

import numpy as np  # noqa: E402

METRIC = "spin-trials/s, 256^2x1 demag on"
UNIT = "spin-trials/s"
WORKLOAD = dict(nx=256, ny=256, nz=1, dx=1e-9, dy=1e-9, dz=0.8e-9, ms=1.6e6, Aex=16e-12, Dind=6e-3, Ku1=2e6,
                anisUx=0.0, anisUy=0.0, anisUz=1.0, Bextx=0.0, Bexty=0.0, Bextz=0.3, pbc_x=20, pbc_y=20, pbc_z=0,
                cal_demag_flag=1, randomseed=256, use_random_init=1, Temperature_start=1400.0,
                Temperature_end=40.0, Temperature_step=0.9, Temperature_use_exp=1, circle_per_stage=10000,
                rand_block_size=40)
SWEEPS_PER_STAGE = 10000
CACHE_DIR = os.environ.get("MMC_BENCH_CACHE", "/tmp/mmc_bench_tensor_cache")


def stage_temperature(k):
    t = np.float32(1400.0)
    for _ in range(k):
        t = np.float32(t * np.float32(0.9))
    return float(t)


def ncu_traffic(kernel, shape, R):
    """(DRAM bytes per launch of R replicas, note on the capture) of `kernel`
    from the committed ncu summary: lines "dram_bytes_per_launch <kernel>
    <shape> [r<replicas>]: N" (no r token: 32 replicas).  Preference: a
    capture with R replicas at `shape`, then with R replicas at another shape
    (the autotuner's pick varies between runs), then a capture with another
    replica count scaled by the replicas (a launch's traffic is one pass over
    its replicas' data); else (None, None)."""
    p = os.path.join(ROOT, "profiles", "batched_256x256_kernels.md")
    if not os.path.exists(p):
        return None, None
    want = ",".join(str(v) for v in shape)
    best = None  # (rank, value, note)
    with open(p) as f:
        for line in f:
            parts = line.strip().split()
            if len(parts) not in (4, 5) or parts[0] != "dram_bytes_per_launch" or parts[1] != kernel:
                continue
            sh = parts[2].rstrip(":")
            r = int(parts[3].rstrip(":")[1:]) if len(parts) == 5 else 32
            try:
                val = float(parts[-1])
            except ValueError:
                continue
            rank = (0 if r == R else 2) + (0 if sh == want else 1)
            note = f"{r} replicas, shape {sh}" + ("" if r == R else f", scaled to {R} replicas")
            if best is None or rank < best[0]:
                best = (rank, val * R / r, note)
    return (best[1], best[2]) if best else (None, None)


def measured_peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi samples (200 ms) while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


def l2_flush(torch, dev, buf=[]):
    if not buf:
        buf.append(torch.empty(512 * 1024 * 1024 // 4, dtype=torch.float32, device=dev))
    buf[0].fill_(1.0)
    torch.cuda.synchronize(dev)


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist
        if not dist.is_initialized():
            dist.init_process_group("gloo")
        return dist, rank, local, world
    return None, rank, local, world


def workload_config(R, S, seeds):
    return {"workload": f"anneal stage of {R} replicas of the 256x256x1 film, demag, PBC 20 images (x,y), "
                        f"{S} sweeps/stage", "replicas_per_gpu": R, "seeds": f"{seeds[0]}..{seeds[-1]}",
            "sweeps_per_step": S, "cells_per_replica": 65536, "precision": "fp32 bulk, fp64 tensor and energy",
            "l2": "512 MB flush between timed steps"}


def replica_seeds(rank, R):
    """Seeds of rank `rank`'s replicas: 256.. on rank 0, disjoint across ranks."""
    return [256 + rank * R + r for r in range(R)]


def reduce_max(dist, v):
    if dist is None:
        return v
    import torch
    t = torch.tensor([v], dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t[0])


def barrier(dist):
    if dist is not None:
        dist.barrier()


def cpu_sample(O, k6, seconds=12.0, threads=0):
    """FP64 oracle sweeps of the same lattice on the host cores."""
    cfg = O.config(precision=64, **WORKLOAD)
    m = O.init_random(cfg, 256)
    n = m.shape[1]
    t0 = time.perf_counter()
    O.sweeps(cfg, k6, stage_temperature(0), 0, 0, 1, m, demag_mode=1, nthreads=threads)
    one = time.perf_counter() - t0
    ns = max(1, int(seconds / max(one, 1e-3)))
    t0 = time.perf_counter()
    O.sweeps(cfg, k6, stage_temperature(0), 0, 1, ns, m, demag_mode=1, nthreads=threads)
    dt = time.perf_counter() - t0
    return ns * n / dt, ns


def pt_farm(M, local, sweeps):
    """The batched parallel-tempering workload: 64 FP32 replicas (seeds 1..64)
    in 4 ladders of 16 temperatures geometric over 40-1400 K, swaps every 10
    sweeps; each ladder draws its square side from {64, 96, 128, 192, 256}, its
    B_z from U[0.1, 0.5] T and its DMI from U[3e-3, 6e-3] J/m^2 (a ladder
    shares one Hamiltonian so its swaps are valid); ladders of one side form
    one batch, all batches advance together as a farm, each with its autotuned
    launch shape."""
    rng = np.random.default_rng(64)
    sides = rng.choice([64, 96, 128, 192, 256], size=4)
    bz = rng.uniform(0.1, 0.5, size=4)
    dind = rng.uniform(3e-3, 6e-3, size=4)
    T = np.geomspace(40.0, 1400.0, 16)
    base = {k: v for k, v in WORKLOAD.items() if k not in ("nx", "ny", "Bextz", "Dind", "randomseed")}
    batches, seed, t0 = [], 1, time.perf_counter()
    for side in sorted(set(int(v) for v in sides)):
        ls = [i for i in range(4) if int(sides[i]) == side]
        cfgs = [M.Config.defaults(precision=32, nx=side, ny=side, randomseed=seed + k, Bextz=float(bz[ls[k // 16]]),
                                  Dind=float(dind[ls[k // 16]]), **base) for k in range(16 * len(ls))]
        b = M.Batch(cfgs, device=local)
        b.build_demag(CACHE_DIR)
        b.set_ladders(np.arange(16 * len(ls), dtype=np.int32).reshape(len(ls), 16), np.tile(T, (len(ls), 1)), 10,
                      1000 + seed)
        b.autotune(4)
        batches.append(b)
        seed += 16 * len(ls)
    setup = time.perf_counter() - t0
    with M.Farm(batches) as farm:
        farm.run_sweeps(0, 0, 200)
        farm.run_sweeps(1, 0, sweeps)
        ms = farm.last_run_ms()
    cells = sum(b.R * b.n for b in batches)
    att = acc = 0
    for b in batches:
        _, cnt = b.ladder_state()
        att += int(cnt[0])
        acc += int(cnt[1])
        b.close()
    return {"value": cells * sweeps / (ms / 1e3), "unit": UNIT, "replicas": 64, "ladders": 4,
            "sides": [int(v) for v in sides], "batches": len(batches), "swap_interval": 10, "sweeps": sweeps,
            "wall_ms": ms, "swap_acceptance": acc / max(att, 1), "setup_s": setup,
            "timing": "host wall clock of one farm call (all batches, their graphs and swap passes)"}


SLAB = dict(nx=512, ny=512, nz=8, dx=2e-9, dy=2e-9, dz=1e-9, ms=1.1e6, Aex=15e-12, Dind=3e-3, Ku1=0.8e6,
            anisUx=0.0, anisUy=0.0, anisUz=1.0, Bextx=0.0, Bexty=0.0, Bextz=0.2, pbc_x=10, pbc_y=10, pbc_z=0,
            cal_demag_flag=1, randomseed=7, use_random_init=1)


def launches_per_step(S, shape, R, graph_sweeps=32):
    """Kernel launches of one timed step of S sweeps with a launch shape: per
    sweep the row kernel and the column pass (row path), or the x, column and
    inverse x passes and the Metropolis launches (one tile or strip launch for
    both colours, or one per colour), once per replica part inside the
    32-sweep graphs and on one stream for the sweeps left over; one counter
    advance per graph and after the left-over sweeps."""
    per = 2 if shape[5] > 0 else 4 if shape[6] in (1, 4) else 5
    parts = 1 if shape[5] > 0 else min(shape[9], R)
    graphs, rem = divmod(S, graph_sweeps)
    return graphs * graph_sweeps * per * parts + rem * per + graphs + (1 if rem else 0)


def slab_line(M, local, sweeps):
    """The 3-D slab in FP32: 512x512x8 cells, PBC 10 images in x and y, open
    in z (padded to 15 layers), seed 7, one lattice on the pass kernels.  The
    tensor uses the far-field form beyond 32 cells (tensor_far_radius = 32),
    which is exact to about 1e-12 per term there and makes the setup seconds
    instead of the ~10 minutes of exact 64-term sums over 441 images."""
    t0 = time.perf_counter()
    lat = M.Lattice(M.Config.defaults(precision=32, tensor_far_radius=32, **SLAB), device=local)
    lat.build_demag(CACHE_DIR)
    setup = time.perf_counter() - t0
    T = [800.0 * 0.9 ** k for k in range(3)]
    lat.run_sweeps(T[0], 0, 0, 20)
    lat.run_sweeps(T[1], 1, 0, sweeps)
    ms = lat.last_run_ms()
    prof = lat.profile_sweeps(T[2], 2, 0, 20)
    n = SLAB["nx"] * SLAB["ny"] * SLAB["nz"]
    lat.close()
    return {"value": n * sweeps / (ms / 1e3), "unit": UNIT, "cells": n, "sweeps": sweeps,
            "us_per_sweep": 1e3 * ms / sweeps, "demag_us_per_sweep": 1e3 * prof[0] / 20,
            "metropolis_us_per_sweep": 1e3 * prof[1] / 20, "tensor_setup_s": setup,
            "tensor": "exact 64-term sums within 32 cells, far-field expansion beyond"}


def relax_line(M, local):
    """Gradient and relaxation on the 256x256x1 film in FP64: a short anneal
    (34 stages of 100 sweeps, seed 11), then projected steepest descent to a
    max torque |m x H|/Ms < 1e-6."""
    lat = M.Lattice(M.Config.defaults(precision=64, **dict(WORKLOAD, randomseed=11)), device=local)
    lat.build_demag(CACHE_DIR)
    for k in range(34):
        lat.run_sweeps(stage_temperature(k), k, 0, 100)
    e0 = lat.energy().e_total
    lat.grad()
    t0 = time.perf_counter()
    for _ in range(10):
        lat.grad()
    grad_ms = (time.perf_counter() - t0) / 10 * 1e3
    t0 = time.perf_counter()
    it, tq = lat.relax(1e-6, 200000)
    dt = time.perf_counter() - t0
    e1 = lat.energy().e_total
    lat.close()
    return {"precision": "fp64", "iterations": it, "max_torque": tq, "seconds": dt, "ms_per_iteration":
            1e3 * dt / max(it, 1), "energy_before_J": e0, "energy_after_J": e1, "grad_ms_with_copy_to_host": grad_ms}


def run_reference(args):
    """The reference's CPU path on the host cores.  The reference cannot be
    built (its Metropolis, energy and tensor-image kernel bodies are not
    published), so this arm runs the project's FP64 C++ restatement of the same
    sweep (the oracle) on every host core."""
    dist, rank, local, world = dist_setup()
    if rank != 0:
        return
    import oracle_ctypes as O  # the product library is not loaded on this arm
    cores = os.cpu_count() or 1
    # The sweep cost does not depend on the tensor values, so the sample uses the
    # 256x256 tensor with 2 images (20 images take ~40 core-minutes to build on
    # the CPU).
    tcfg = O.config(precision=64, **dict(WORKLOAD, pbc_x=2, pbc_y=2))
    k6 = O.tensor(tcfg)
    vals = []
    n_sw = 0
    for i in range(args.warmup + args.steps):
        v, ns = cpu_sample(O, k6, seconds=args.ref_seconds, threads=cores)
        if i >= args.warmup:
            vals.append(v)
            n_sw += ns
    value = statistics.mean(vals)
    sample = f"{n_sw} FP64 sweeps of the 256x256x1 lattice with FFT demag over {args.steps} steps"
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": dict(workload_config(args.batch, args.sweeps, replica_seeds(0, args.batch)),
                       precision="fp64 (the oracle port of the sweep)",
                       sample="the sweeps of one replica on all host cores; trials/s per trial does not depend "
                              "on the replica count"),
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": cores, "kind": "port", "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "reference not buildable (kernel bodies unpublished); FP64 C++ port of the sweep on all host cores",
    }
    print(json.dumps(line), flush=True)


def run_ours(args):
    dist, rank, local, world = dist_setup()
    import torch
    import mmc_ctypes as M
    import oracle_ctypes as O  # CPU-baseline leg only

    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    os.makedirs(CACHE_DIR, exist_ok=True)
    R = args.batch
    S = args.sweeps
    seeds = replica_seeds(rank, R)
    cfgs = [M.Config.defaults(precision=32, **dict(WORKLOAD, randomseed=sd)) for sd in seeds]
    t0 = time.perf_counter()
    batch = M.Batch(cfgs, device=local)
    batch.build_demag(CACHE_DIR)
    setup_s = time.perf_counter() - t0
    # launch shape: the fastest of all shapes on this device (bit-identical
    # results), or the one given (to profile the shape a plain run chose)
    batch.set_temperatures(np.full(R, stage_temperature(0)))
    t0 = time.perf_counter()
    if args.launch_shape:
        batch.set_launch_shape([int(v) for v in args.launch_shape.split(",")])
        tune_ms, tune_n = None, 0
    else:
        tune_ms, tune_n = batch.autotune(96)
    tune_s = time.perf_counter() - t0
    n = 65536

    def run_stage(k):
        batch.set_temperatures(np.full(R, stage_temperature(k)))
        batch.run_sweeps(k, 0, S)
        return batch.last_run_ms() / 1e3

    for k in range(args.warmup):
        run_stage(k)
    barrier(dist)
    torch.cuda.synchronize(dev)
    times = []
    with ClockSampler(local) as clk:
        torch.cuda.nvtx.range_push("timed")  # lets an ncu launch list cover exactly these steps
        for j in range(args.steps):
            l2_flush(torch, dev)
            times.append(run_stage(args.warmup + j))
        torch.cuda.nvtx.range_pop()
    torch.cuda.synchronize(dev)
    barrier(dist)
    total = reduce_max(dist, sum(times))
    value = world * args.steps * S * R * n / total

    # end to end through the public API: every step uploads all replicas from
    # pinned host memory, runs the stage and reads all replicas back
    pin = torch.empty((R, 3, n), dtype=torch.float64).pin_memory()
    pin_out = torch.empty((R, 3, n), dtype=torch.float64).pin_memory()
    host = pin.numpy()
    for r in range(R):
        host[r] = batch.get_m(r)
    L = M.lib()
    e2e_t = 0.0
    for j in range(args.steps):
        k = args.warmup + args.steps + j
        l2_flush(torch, dev)
        t0 = time.perf_counter()
        for r in range(R):
            M.check(L.mmc_batch_set_m(batch.h, r, M.dptr(host[r, 0]), M.dptr(host[r, 1]), M.dptr(host[r, 2])))
        batch.set_temperatures(np.full(R, stage_temperature(k)))
        batch.run_sweeps(k, 0, S)
        out = pin_out.numpy()
        for r in range(R):
            M.check(L.mmc_batch_get_m(batch.h, r, M.dptr(out[r, 0]), M.dptr(out[r, 1]), M.dptr(out[r, 2])))
        e2e_t += time.perf_counter() - t0
    e2e_t = reduce_max(dist, e2e_t)
    e2e = world * args.steps * S * R * n / e2e_t

    # per-kernel attribution (CUDA events on the batch's stream), same workload
    prof_sweeps = 200
    prof = batch.profile_sweeps(args.warmup, 0, prof_sweeps) / prof_sweeps  # ms per batch sweep
    s_ = 4
    hxp, nh = 130, 129 * 256
    shape = batch.launch_shape()
    if shape[5] > 0:  # film row kernel + column pass
        kbytes = {
            # m in and out, spectrum rows in and out (halo re-reads not counted)
            "k_rows": R * (2 * 3 * s_ * n + 2 * 3 * 2 * s_ * nh),
            "k_col_pass": R * 2 * (3 * 2 * s_ * nh) + 6 * 2 * s_ * nh,
        }
        fam = dict(zip(["k_rows", "k_col_pass"], prof[:2]))
    else:
        # tile / strip: both colours in one launch, else one launch per colour
        mc = {1: "k_mc_tile", 2: "k_mc_quad", 3: "k_mc_band", 4: "k_mc_strip", 5: "k_mc_pipe"}.get(shape[6],
                                                                                                  "k_mc_checker")
        # the film column pass held in registers (three components or one per thread)
        col = {2: "k_col_reg", 3: "k_col_reg3"}.get(shape[8], "k_col_pass")
        kbytes = {
            "k_x_forward": R * (3 * s_ * n + 3 * 2 * s_ * nh),
            col: R * 2 * (3 * 2 * s_ * nh) + 6 * 2 * s_ * nh,
            "k_x_inverse": R * (3 * 2 * s_ * nh + 3 * s_ * n),
            mc: R * n * 9 * s_,  # both colours: 36 B per trial
        }
        fam = dict(zip(["k_x_forward", col, "k_x_inverse", mc], prof[:4]))
    dom = max(fam, key=fam.get)
    # demag convolutions/s: the three pass kernels' time per batched sweep on
    # one stream (the pass-kernel path), R convolutions per sweep; bytes per
    # convolution in the model of the hot-path table: m in and h out
    # (6 s N) and the half spectra of K^ . M^ (6 x 2 s N_h)
    demag_line = None
    if shape[5] == 0:
        conv_ms = fam["k_x_forward"] + fam[col] + fam["k_x_inverse"]
        conv_bytes = 6 * s_ * n + 6 * 2 * s_ * nh
        conv_rate = R / (conv_ms * 1e-3)
        demag_line = {"value": conv_rate, "unit": "demag convolutions/s", "replicas": R,
                      "ms_per_batch": conv_ms, "bytes_per_convolution": conv_bytes,
                      "achieved_gbs": conv_rate * conv_bytes / 1e9,
                      "timing": "x forward + column + x inverse passes, CUDA events, one stream"}
    launches = 2 if dom in ("k_mc_checker", "k_mc_quad", "k_mc_band", "k_mc_pipe") else 1
    per_launch_ms = fam[dom] / launches
    bytes_launch = kbytes[dom] / launches
    peak, peak_kind = measured_peaks()
    if demag_line is not None:
        demag_line["frac"] = demag_line["achieved_gbs"] / peak
    traffic, tshape = ncu_traffic(dom, shape, R)
    achieved = bytes_launch / (per_launch_ms * 1e-3) / 1e9
    roofline = {"bound": "hbm", "kernel": dom, "achieved": achieved, "peak": peak, "unit": "GB/s",
                "frac": achieved / peak, "peak_source": peak_kind, "traffic": traffic, "traffic_capture": tshape,
                "algorithmic_bytes_per_launch": bytes_launch, "avg_ms_per_launch": per_launch_ms,
                "kernel_ms_per_batch_sweep": fam, "launch_shape": shape,
                "timing": "per-kernel CUDA events on the batch's stream over 200 sweeps launched on ONE stream "
                          "(mmc_batch_profile_sweeps): serialised launches, an upper bound on each kernel's time "
                          "in the timed run, whose graphs overlap the kernels of the replica parts on "
                          f"{shape[9]} streams",
                "bytes_model": "per replica: x passes 3*4*N real + 3*8*N_h complex; column pass (k_col_pass or "
                               "k_col_reg) 2*3*8*N_h "
                               "(+ 6*8*N_h shared tensor once); Metropolis 36 B per trial (both colours); row "
                               "kernel m in/out 2*3*4*N + spectrum rows in/out 2*3*8*N_h; N=65536, N_h=33024"}
    batch.close()

    # one lattice, FP32 (the film engine) and the plain FP64 path
    single = M.Lattice(M.Config.defaults(precision=32, **WORKLOAD), device=local)
    single.build_demag(CACHE_DIR)
    single.run_sweeps(stage_temperature(0), 0, 0, 1000)
    single.run_sweeps(stage_temperature(1), 1, 0, 4000)
    single_v = 4000 * n / (single.last_run_ms() / 1e3)
    single_engine = single.engine()
    phases = None
    if single_engine[0] == M.ENGINE_FUSED:
        # device timestamps of the film engine's phases (CTA 0), sweeps 2..14 of a 16-sweep launch
        st = single.profile_fused(stage_temperature(1), 1, 4000, 16).astype(np.float64)[2:15, :, 0]
        d = np.diff(st, axis=1).mean(axis=0) / 1e3
        names = ["copies", "demag_field_rows", "metropolis", "spectrum_rows", "barrier_1", "column_copies",
                 "column_phase", "barrier_2"]
        phases = {k: round(float(v), 3) for k, v in zip(names, d)}
        phases["sweep"] = round(float((st[1:, 0] - st[:-1, 0]).mean() / 1e3), 3)
    fp64_line = None
    if not args.no_fp64:
        lat64 = M.Lattice(M.Config.defaults(precision=64, sweep_engine=M.ENGINE_KERNELS, **WORKLOAD), device=local)
        lat64.build_demag(CACHE_DIR)
        lat64.run_sweeps(stage_temperature(0), 0, 0, 200)
        lat64.run_sweeps(stage_temperature(1), 1, 0, 1000)
        fp64 = 1000 * n / (lat64.last_run_ms() / 1e3)
        lat64.close()
        fp64_line = {"value": fp64, "unit": UNIT, "engine": "kernels", "lattices": 1,
                     "batched_fp32_over_fp64": value / world / fp64, "single_fp32_over_fp64": single_v / fp64}
        # the same batch in FP64: splits "batched FP32 over plain FP64" into its
        # batching part (FP64 batched / FP64 plain) and its precision part
        # (FP32 batched / FP64 batched)
        b64 = M.Batch([M.Config.defaults(precision=64, **dict(WORKLOAD, randomseed=sd)) for sd in seeds],
                      device=local)
        b64.build_demag(CACHE_DIR)
        b64.set_temperatures(np.full(R, stage_temperature(0)))
        b64.autotune(16)
        b64.run_sweeps(0, 0, 100)
        b64.set_temperatures(np.full(R, stage_temperature(1)))
        b64.run_sweeps(1, 0, 1000)
        fp64b = R * 1000 * n / (b64.last_run_ms() / 1e3)
        fp64_line["batched_fp64"] = {"value": fp64b, "unit": UNIT, "replicas": R,
                                     "launch_shape": list(b64.launch_shape())}
        fp64_line["batching_part"] = fp64b / fp64
        fp64_line["precision_part"] = value / world / fp64b
        b64.close()

    farm_line = None if args.no_farm else pt_farm(M, local, 2000)
    slab = None if args.no_slab else slab_line(M, local, 200)
    relax = None if args.no_relax else relax_line(M, local)

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1e3 * total / args.steps, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": workload_config(R, S, seeds),
        "e2e": {"value": e2e, "unit": UNIT, "h2d_bytes_per_step": R * 3 * n * 8, "d2h_bytes_per_step": R * 3 * n * 8},
        "roofline": roofline,
        "clocks": clk.summary(),
        "gpu_launches": args.steps * launches_per_step(S, shape, R),
        "demag_convolutions": demag_line,
        # the whole batched sweep of one rank against the same peak: every
        # kernel's algorithmic bytes (roofline.bytes_model) over the timed
        # region's time per sweep
        "sweep_roofline": {"algorithmic_bytes_per_sweep": sum(kbytes.values()),
                           "us_per_sweep": 1e6 * total / (args.steps * S),
                           "achieved_gbs": sum(kbytes.values()) / (total / (args.steps * S)) / 1e9,
                           "frac": sum(kbytes.values()) / (total / (args.steps * S)) / 1e9 / peak},
        "single_lattice_fp32": {"value": single_v, "unit": UNIT, "engine": single_engine,
                                "film_engine_phase_us": phases},
        "fp64_plain": fp64_line,
        "pt_farm_fp32": farm_line,
        "slab_512x512x8_fp32": slab,
        "relax": relax,
        "setup_s": setup_s,
        "autotune": {"candidates": tune_n, "best_ms_per_batch_sweep": tune_ms, "seconds": tune_s,
                     "launch_shape": list(shape)},
    }
    if rank == 0 and not args.no_cpu:
        k6 = single.tensor()
        v1, ns1 = cpu_sample(O, k6, seconds=args.cpu_seconds, threads=1)
        cores = os.cpu_count() or 1
        vN, nsN = cpu_sample(O, k6, seconds=args.cpu_seconds, threads=cores)
        line["cpu_baseline"] = {"value": vN, "unit": UNIT, "cores": cores, "kind": "port",
                                "sample": f"{nsN} FP64 sweeps of one 256x256x1 lattice (FFT demag), same tensor",
                                "single_thread": v1}
    single.close()
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--sweeps", type=int, default=SWEEPS_PER_STAGE)
    ap.add_argument("--batch", type=int, default=64, help="replicas of the 256x256x1 lattice per GPU")
    ap.add_argument("--cpu-seconds", type=float, default=8.0)
    ap.add_argument("--ref-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-fp64", action="store_true")
    ap.add_argument("--no-farm", action="store_true", help="skip the parallel-tempering farm line")
    ap.add_argument("--no-relax", action="store_true", help="skip the gradient / relaxation line")
    ap.add_argument("--no-slab", action="store_true", help="skip the 3-D slab line")
    ap.add_argument("--launch-shape", default="",
                    help="ten comma-separated values of a launch shape to use instead of autotuning")
    args = ap.parse_args()
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
