#!/usr/bin/env python
"""Benchmark: MD atom-steps/s of compressed se_e2_a on GB300.

Default workload (the ragged-batch configuration the target is quoted on):
512 independent water frames with 8..512 molecules each (24..1536 atoms,
398,850 atoms in all), each in its own cubic box at 1.0 g/cm^3, built by the
seeded water generator; compressed se_e2_a in FP32 (rcut 6, rcut_smth 0.5,
sel [46, 92], embedding [25, 50, 100] tabulated at stride 0.01 / 0.1,
extrapolate 5, axis 16, fitting [240, 240, 240]), seeded random weights,
davg/dstd from 16 seeded 192-atom frames.  One "step" = energy + force +
virial of all 512 frames with every neighbour list rebuilt.

  value   chosen form: all frames packed in one batch, the fused kernels
          captured in one CUDA graph, inputs resident in HBM
  e2e     the same step through the public API (se_a.CapturedStep): host
          coordinates copied in and every frame's energy / force / virial
          copied out, every step
  plain   the plain single-frame drop-in (uncompressed embedding as
          matmuls, operator form, eager), frame by frame over the batch
The 12,288-atom single frame (4096 H2O, 49.68 A box) is reported under
"water12k" with its own value, e2e, roofline and operator-kernel numbers.
Errors are stated against the FP64 CPU composite of the reference's op
sequence on the same frames.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
                  [--workload ragged512|water12k|md786k|train8x192]

With --gpus N > 1 outside a torch.distributed launch, the script re-launches
itself under torch.distributed.run with N ranks (one GPU each); every rank
takes its own 512 ragged frames (weak scaling, no collective in the step).
"""

from __future__ import annotations

import argparse
import copy
import json
import os
import re
import statistics
import subprocess
import sys
import tempfile
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

METRIC = "MD atom-steps/s on 1 GB300, chosen vs plain form at stated force error vs FP64"
WORKLOAD_RAGGED = ("512 ragged water frames, 8-512 molecules each (24-1536 atoms, 398850 atoms), "
                   "1.0 g/cm3 cubic PBC boxes, compressed se_e2_a FP32, every nlist rebuilt every "
                   "step, energy+force+virial of all frames in one packed graph-captured step")
WORKLOAD_12K = ("4096 H2O (12288 atoms), 49.68 A PBC box, compressed se_e2_a FP32, "
                "nlist rebuilt every step, energy+force+virial")
N_SIDE, BOX, SEED = 16, 49.68, 20261203
N_FRAMES, MOL_LO, MOL_HI = 512, 8, 512
CPU_SAMPLE_FRAMES = 64


def _dist():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def _pkg():
    from __graft_entry__ import load_package

    return load_package()


def _frame():
    import importlib

    _pkg()
    water = importlib.import_module("dpmd_public_gb300.water")
    return water.water_frame(N_SIDE, BOX, SEED)


def _ragged_frames(rank: int = 0, world: int = 1):
    """The frames of one rank and their global indices.  One GPU: the 512
    ragged frames.  N GPUs (weak scaling): the job holds N x 512 frames of
    the same distribution, partitioned across the ranks by atoms."""
    import importlib

    _pkg()
    water = importlib.import_module("dpmd_public_gb300.water")
    if world == 1:
        return water.ragged_frames(N_FRAMES, seed=SEED, lo=MOL_LO, hi=MOL_HI), \
            list(range(N_FRAMES))
    R = importlib.import_module("dpmd_public_gb300.replicas")
    n = N_FRAMES * world
    counts = water.ragged_counts(n, SEED, MOL_LO, MOL_HI)
    ids = R.frames_of_rank(3 * counts, world, rank)
    return water.ragged_frames(n, seed=SEED, lo=MOL_LO, hi=MOL_HI, which=ids), ids


def _stat_frames():
    import importlib

    water = importlib.import_module("dpmd_public_gb300.water")
    return [water.water_frame(4, 12.42, 5000 + s) for s in range(16)]


def _by_size(frames, k):
    """k frame indices spread over the size order (smallest and largest
    included)."""
    order = np.argsort([len(f[1]) for f in frames], kind="stable")
    pick = np.unique(np.round(np.linspace(0, len(order) - 1, k)).astype(int))
    return [int(order[p]) for p in pick]


def _cpu_sample(frames, n: int = CPU_SAMPLE_FRAMES):
    """A CPU timing sample of n frames evenly spaced in size order (every
    eighth frame for n = 64 of 512), so that it keeps the batch's size
    distribution."""
    order = np.argsort([len(f[1]) for f in frames], kind="stable")
    step = max(1, len(frames) // n)
    return [int(i) for i in order[step // 2::step]]


def _np_model(m64, cfg):
    return (cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), m64.tables_np,
            m64.infos_np)


def _cpu_model():
    """The model of the GPU arms rebuilt on the host alone (oracle env
    matrix for the statistics), for the CPU-only reference arm."""
    import importlib

    import oracle as O

    _pkg()
    mdl = importlib.import_module("dpmd_public_gb300.model")
    cfg = mdl.SeAConfig()
    params = mdl.init_params(cfg, SEED)
    ems, ats, mind = [], [], np.inf
    for c, t, b in _stat_frames():
        em, emd, rij, nl = O.prod_env_mat_a_pbc(c, t, b, np.zeros((2, cfg.nnei * 4)),
                                                np.ones((2, cfg.nnei * 4)), cfg.rcut, cfg.rcut_smth,
                                                list(cfg.sel))
        ems.append(em)
        ats.append(t)
        r = np.linalg.norm(rij.reshape(-1, 3), axis=1)
        mind = min(mind, r[nl >= 0].min())
    davg, dstd = mdl.stats_from_env(ems, ats, cfg)
    tabs, infos = mdl.build_tables(params, davg, dstd, mind, cfg)
    return cfg, params, davg, dstd, tabs, infos


# ---------------------------------------------------------------- clocks --
class Clocks:
    """nvidia-smi samples of one GPU's clocks and throttle reasons, every
    200 ms, into a temporary CSV that the bench parses."""

    def __init__(self, index: int):
        self.proc = None
        fd, self.path = tempfile.mkstemp(prefix=f"clocks_{os.getpid()}_", suffix=".csv")
        os.close(fd)
        self.index = index

    def __enter__(self):
        try:
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.index),
                 "--query-gpu=index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
                 "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=self.fh, stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def __exit__(self, *a):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def _nrows(self):
        try:
            with open(self.path) as fh:
                return sum(1 for _ in fh)
        except OSError:
            return 0

    def load(self, step, first_sample_s: float = 3.0, after_s: float = 0.45):
        """Keep the GPU busy with ``step`` (untimed) until the sampler has
        written its first row (pre-roll) or, with ``after_s``, for that long
        after the timed region (post-roll), so that the samples bracket the
        timed steps under the same load."""
        import torch

        t0 = time.perf_counter()
        n0 = self._nrows()
        while self.proc is not None:
            for _ in range(20):
                step()
            torch.cuda.synchronize()
            el = time.perf_counter() - t0
            if after_s is None and (self._nrows() > n0 or el > first_sample_s):
                break
            if after_s is not None and el > after_s:
                break

    def summary(self):
        if self.proc is None or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        rows = []
        for line in open(self.path):
            parts = [p.strip() for p in line.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append((float(parts[1]), float(parts[2]), parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for _, _, r in rows for k, v in enumerate(r) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r[0] for r in rows), "sm_max_mhz": max(r[1] for r in rows),
                "reasons": reasons, "samples": len(rows)}


# ----------------------------------------------------------- CPU baseline --


# ----------------------------------------------------------- CPU baseline --
def cpu_time_frames(frames, idx, model_np, passes: int, warmup: int = 1, cell_list=True,
                    dtype=np.float32):
    """Seconds per pass of the reference's CPU op sequence (oracle
    composite: copy_coord, candidate build, format, env mat, tabulate, BLAS
    fitting, tabulate grad, force, virial) over frames[idx], frame by frame
    as the reference processes them."""
    import composite

    cfg, params, davg, dstd, tabs, infos = model_np
    for k in idx[:max(0, warmup)]:
        c, t, b = frames[k]
        composite.energy_force_virial(cfg, params, davg, dstd, c, t, b, tabs, infos, dtype,
                                      cell_list=cell_list)
    t0 = time.perf_counter()
    for _ in range(passes):
        for k in idx:
            c, t, b = frames[k]
            composite.energy_force_virial(cfg, params, davg, dstd, c, t, b, tabs, infos, dtype,
                                          cell_list=cell_list)
    return (time.perf_counter() - t0) / passes


def cpu_baseline_ragged(frames, model_np, passes: int = 2):
    """The reference's CPU path on a bounded sample of the ragged batch
    (64 of the 512 frames, spread over the size order), with its O(N)
    cell-list neighbour build; the O(N^2) build_nlist_cpu variant alongside."""
    import oracle as O

    idx = _cpu_sample(frames)
    nat = sum(len(frames[k][1]) for k in idx)
    s = cpu_time_frames(frames, idx, model_np, passes)
    s_bf = cpu_time_frames(frames, idx, model_np, 1, warmup=0, cell_list=False)
    return {"value": nat / s, "unit": "atom-steps/s", "cores": O.num_threads(), "kind": "port",
            "sample": f"{len(idx)} of the 512 frames (every 8th in size order, {nat} atoms), "
                      f"{passes} passes after 1 warm-up frame, FP32, oracle composite of the "
                      f"reference's CPU op sequence with the cell-list build_nlist",
            "omp_num_threads": os.environ.get("OMP_NUM_THREADS", "unset"),
            "cpu_model": _cpu_model_name(),
            "brute_force_nlist_value": nat / s_bf}


def cpu_baseline_12k(frame, model_np, steps: int = 2):
    import oracle as O

    s = cpu_time_frames([frame], [0], model_np, steps)
    return {"value": len(frame[1]) / s, "unit": "atom-steps/s", "cores": O.num_threads(),
            "kind": "port",
            "sample": f"full 12288-atom frame, {steps} steps after 1 warm-up, FP32, oracle "
                      f"composite of the reference's CPU op sequence with the cell-list build_nlist"}


def _cpu_model_name() -> str:
    try:
        with open("/proc/cpuinfo") as fh:
            for line in fh:
                k = line.split(":")[0].strip().lower()
                if k in ("model name", "cpu part", "hardware"):
                    return line.split(":", 1)[1].strip()
    except OSError:
        pass
    import platform

    return platform.machine()


def reference_arm(args):
    """The reference's CPU implementation of the path (oracle port of its
    op sequence, all host threads) on the same workload, metric and unit:
    each step a bounded sample (the 64-frame sample of the ragged batch, or
    the full 12,288-atom frame)."""
    ws, rank, _ = _dist()
    if rank != 0:
        return 0
    import oracle as O

    model_np = _cpu_model()
    if args.workload == "water12k":
        frames, idx, workload = [_frame()], [0], WORKLOAD_12K
        sample = "full 12288-atom frame per step"
    else:
        frames = _ragged_frames(0)[0]
        idx, workload = _cpu_sample(frames, 32), WORKLOAD_RAGGED
        sample = (f"{len(idx)} of the 512 frames per step (every 16th in size order), "
                  f"frame by frame")
    nat = sum(len(frames[k][1]) for k in idx)
    steps = max(1, min(args.steps, 200))
    cpu_time_frames(frames, idx, model_np, max(1, args.warmup), warmup=0)
    s = cpu_time_frames(frames, idx, model_np, steps, warmup=0)
    value = nat / s
    line = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": args.gpus,
            "steps": steps, "warmup": args.warmup, "ms_per_step": s * 1e3,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded water generator, random-init weights)", "impl": "reference",
            "config": {"workload": workload, "atoms_per_step": nat,
                       "form": "reference CPU op sequence (oracle port), cell-list build_nlist"},
            "cpu_baseline": {"value": value, "unit": "atom-steps/s", "cores": O.num_threads(),
                             "kind": "port", "sample": f"{sample}, {nat} atoms, FP32",
                             "cpu_model": _cpu_model_name()},
            "e2e": {"value": value, "unit": "atom-steps/s", "h2d_bytes_per_step": 0,
                    "d2h_bytes_per_step": 0}}
    print(json.dumps(line))
    return 0


# ------------------------------------------------------------------ main --
def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=20)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--no-cpu", action="store_true", help="skip the timed CPU baseline")
    ap.add_argument("--fit-mode", default=None,
                    choices=["fp32", "tf32x3", "bf16", "native-fp32", "native-bf16x9", "native-tf32",
                             "native-bf16", "tc-f16x3"],
                    help="fitting net: tc-f16x3 (tcgen05 kernel, scaled FP16 hi/lo split; default "
                         "on one GPU), torch GEMMs (fp32, split tf32x3, bf16) or the native call "
                         "with a cuBLAS compute type (native-*; native-bf16x9 is the default when "
                         "WORLD_SIZE > 1)")
    ap.add_argument("--workload", default="ragged512",
                    choices=["ragged512", "water12k", "md786k", "train8x192"],
                    help="ragged512: 512 ragged frames in one packed graph step (the default line, "
                         "with the 12,288-atom frame as an extra key); water12k: the 12,288-atom "
                         "frame alone; md786k: 786,432-atom NVE MD; train8x192: training step")
    ap.add_argument("--no-12k", action="store_true",
                    help="ragged512: leave out the extra 12,288-atom measurements")
    ap.add_argument("--md-steps", type=int, default=1000)
    ap.add_argument("--md-skin", type=float, default=2.0,
                    help="md786k: neighbour-list skin in A (0: rebuild every step)")
    ap.add_argument("--md-rebuild", type=int, default=10,
                    help="md786k: steps between neighbour-list rebuilds")
    ap.add_argument("--md-out-scale", type=float, default=0.01,
                    help="md786k: scale of the random fitting output layer (physical force range)")
    ap.add_argument("--profile", action="store_true",
                    help="profiling run: set up, then 2 fused steps between "
                         "cudaProfilerStart/Stop (for ncu --profile-from-start off)")
    ap.add_argument("--profile-frames", type=int, default=N_FRAMES,
                    help="--profile with ragged512: frames of the profiled batch (the first k "
                         "of the 512)")
    args = ap.parse_args()
    args.warmup = max(3, args.warmup)
    ws, rank, _ = _dist()
    if args.gpus > 1 and "WORLD_SIZE" not in os.environ:
        return _relaunch(args.gpus)
    if args.fit_mode is None:
        # the tensor-core fitting stages operands with TMA, which jobs on two
        # or more GPUs keep out of: replicas there take the cuBLAS BF16x9 fitting
        args.fit_mode = "tc-f16x3" if ws == 1 else "native-bf16x9"
    if args.impl == "reference":
        return reference_arm(args)
    if args.workload == "md786k":
        return md_workload(args)
    if args.workload == "train8x192":
        return train_workload(args)
    if args.workload == "water12k":
        return water12k_main(args)
    return ragged_main(args)


def _relaunch(n: int) -> int:
    """Run this script under torch.distributed.run with n ranks (one GPU
    each, rendezvous on 127.0.0.1)."""
    import socket

    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    cmd = [sys.executable, "-m", "torch.distributed.run", "--nnodes=1", f"--nproc-per-node={n}",
           "--master-addr", "127.0.0.1", "--master-port", str(port), os.path.abspath(__file__)]
    cmd += sys.argv[1:]
    return subprocess.call(cmd)


def _init_dist(ws, local):
    import torch

    if ws > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    return torch.device("cuda", local)


def _barrier(ws):
    import torch

    if ws > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()


def _max_over_ranks(x: float, ws: int, dev) -> float:
    import torch

    if ws == 1:
        return x
    t = torch.tensor([x], device=dev, dtype=torch.float64)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return float(t)


def time_captured(step, flush, steps: int, warmup: int, ws: int, clk=None):
    """Device time per step of a captured step (CUDA events on the launching
    stream, L2 flushed between steps outside the events); the clock sampler,
    when given, brackets the timed steps under the same load.  Returns
    (ms per step, wall seconds of the timed region)."""
    import torch

    for _ in range(warmup):
        step.replay()
    _barrier(ws)
    st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    if clk is not None:
        clk.load(step.replay, after_s=None)  # pre-roll until the first clock sample
        _barrier(ws)
    wall0 = time.perf_counter()
    for k in range(steps):
        flush()
        st[k].record()
        step.replay()
        en[k].record()
    _barrier(ws)
    wall = time.perf_counter() - wall0
    if clk is not None:
        clk.load(step.replay)  # post-roll under the same load
    return sum(s.elapsed_time(e) for s, e in zip(st, en)) / steps, wall


def time_e2e(step, host_coord, flush, steps: int, ws: int):
    """The public call with host buffers: pinned host coordinates copied in,
    the graph replayed, the packed energies / virials / forces copied out,
    all inside the events of each step."""
    import torch

    for _ in range(3):
        step(host_coord)
    _barrier(ws)
    st = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    en = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    for k in range(steps):
        flush()
        st[k].record()
        step.h2d(step.h_coord)
        step.replay()
        step.d2h()
        en[k].record()
    _barrier(ws)
    return sum(s.elapsed_time(e) for s, e in zip(st, en)) / steps


def ragged_main(args):
    """The default line: 512 ragged frames in one packed, graph-captured
    fused step."""
    import importlib

    import torch

    ws, rank, local = _dist()
    dev = _init_dist(ws, local)
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False
    se_a, cfg, m64, model, plain = _setup_models(dev, args.fit_mode)
    L = importlib.import_module("dpmd_public_gb300._lib")
    frames, frame_ids = _ragged_frames(rank, ws)
    if args.profile:
        frames = frames[:args.profile_frames]
    nat = sum(len(f[1]) for f in frames)
    batch = model.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    host_coord = np.concatenate([f[0] for f in frames]).astype(np.float32)
    step = se_a.CapturedStep(model, batch, coord=host_coord)
    step.replay()
    torch.cuda.synchronize()
    if batch.status() != 0:
        raise RuntimeError(f"neighbour build status {batch.status()}")
    if args.profile:
        torch.cuda.profiler.start()
        for _ in range(2):
            step.replay()
        torch.cuda.synchronize()
        torch.cuda.profiler.stop()
        print(json.dumps({"profile": "ok", "frames": len(frames), "atoms": nat,
                          "status": batch.status()}))
        return 0
    launches = graph_kernels(step.graph)
    flush = L2Flush(dev)
    with Clocks(local) as clk:
        step_ms, wall = time_captured(step, flush, args.steps, args.warmup, ws, clk)
    step_ms = _max_over_ranks(step_ms, ws, dev)
    value = ws * nat / (step_ms * 1e-3)
    if batch.status() != 0:
        raise RuntimeError("neighbour build reported a device status during the timed steps")
    E_dev = batch.energy.clone()
    V_dev = batch.vir.clone()
    F_dev = batch.force.clone()

    e2e_ms = _max_over_ranks(time_e2e(step, host_coord, flush, args.steps, ws), ws, dev)
    e2e = {"value": ws * nat / (e2e_ms * 1e-3), "unit": "atom-steps/s",
           "h2d_bytes_per_step": step.h_coord.numel() * step.h_coord.element_size(),
           "d2h_bytes_per_step": step.h_out.numel()}
    # the e2e outputs are the resident step's outputs (same coordinates)
    same = bool(torch.equal(step.h_force, F_dev.cpu()))

    reps = max(3, min(args.steps, 10))
    kt = kernel_times(model, batch, step.coord, flush, reps=reps)
    dom = max(kt, key=lambda k: kt[k]["ms"])
    peaks = _peaks()
    roof = roofline(dom, kt[dom], nat, cfg, peaks, args.fit_mode)
    roof_parts = {}
    for k in kt:
        rp = roofline(k, kt[k], nat, cfg, peaks, args.fit_mode)
        roof_parts[k] = {x: rp[x] for x in ("kernel", "bound", "achieved", "unit", "frac",
                                            "ms_per_launch", "launches", "traffic") if x in rp}

    # the plain single-frame drop-in, frame by frame over the same batch
    pb = [(plain.batch([f[1]], f[2][None]), torch.tensor(f[0], dtype=torch.float32, device=dev))
          for f in frames]
    for b_, c_ in pb[:8]:
        plain.step_ops(b_, c_, compressed=False)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b_, c_ in pb:
        plain.step_ops(b_, c_, compressed=False)
    torch.cuda.synchronize()
    plain_ms = (time.perf_counter() - t0) * 1e3
    # the same drop-in with the compressed tables (tabulate_fusion_se_a op)
    cb = [(model.batch([f[1]], f[2][None]), c_) for f, (_, c_) in zip(frames, pb)]
    for b_, c_ in cb[:8]:
        model.step_ops(b_, c_, compressed=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for b_, c_ in cb:
        model.step_ops(b_, c_, compressed=True)
    torch.cuda.synchronize()
    comp_ms = (time.perf_counter() - t0) * 1e3
    del pb, cb

    tos = type_one_side_false(se_a, cfg, frames, dev, args, flush)

    out = {"metric": METRIC, "value": value, "unit": "atom-steps/s", "n_gpus": ws,
           "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded water generator, random-init weights)",
           "config": {"workload": WORKLOAD_RAGGED, "frames": len(frames), "atoms": nat,
                      "form": "fused compressed, all frames packed in one CUDA graph, "
                              "deterministic (fixed-point) sums",
                      "fitting_gemm": args.fit_mode, "l2": L2Flush.DESC,
                      "parallelism": f"replicas x{ws} (N x 512 frames partitioned by atoms)",
                      "wall_s": wall},
           "e2e": e2e,
           "gpu_launches": None if launches is None else launches["ours"] * args.steps,
           "graph_kernels_per_step": launches,
           "plain_per_frame": {"value": ws * nat / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                               "form": "plain single-frame drop-in: uncompressed operator form "
                                       "(env op, embedding matmuls, autograd, force/virial ops), "
                                       "eager, one frame at a time"},
           "chosen_over_plain": plain_ms / step_ms,
           "compressed_per_frame": {"value": ws * nat / (comp_ms * 1e-3), "ms_per_step": comp_ms,
                                    "form": "compressed operator form (tabulate_fusion_se_a), "
                                            "eager, one frame at a time"},
           "chosen_over_compressed_per_frame": comp_ms / step_ms,
           "type_one_side_false": tos,
           "kernels_ms": {k: v["ms"] for k, v in kt.items()},
           "roofline": roof, "roofline_parts": roof_parts,
           "autotune": L.autotune_report(),
           "clocks": clk.summary(),
           "e2e_outputs_equal_resident": same}
    if rank == 0:
        import composite

        np_model = _np_model(m64, cfg)
        errs = []
        for k in _by_size(frames, 8):
            c, t, b = frames[k]
            a0 = int(batch.plan.atom_off[k])
            n = len(t)
            E64, F64, V64, _ = composite.energy_force_virial(*np_model[:4], c, t, b, np_model[4],
                                                             np_model[5], cell_list=True)
            Fn = F_dev[a0:a0 + n].cpu().numpy().astype(np.float64)
            errs.append({"frame": k, "atoms": n,
                         "force_max_abs_eV_per_A": float(np.abs(Fn - F64).max()),
                         "energy_per_atom_eV": abs(float(E_dev[k]) - E64) / n,
                         "virial_max_abs_eV": float(np.abs(V_dev[k].cpu().numpy() - V64).max())})
        out["errors_vs_fp64"] = {
            "force_max_abs_eV_per_A": max(e["force_max_abs_eV_per_A"] for e in errs),
            "energy_per_atom_eV": max(e["energy_per_atom_eV"] for e in errs),
            "virial_max_abs_eV": max(e["virial_max_abs_eV"] for e in errs),
            "frames": errs,
            "reference": "FP64 CPU composite (oracle) of the compressed model, 8 frames spread "
                         "over the size order (smallest and largest included)"}
        if not args.no_cpu:
            out["cpu_baseline"] = cpu_baseline_ragged(frames, np_model)
    if ws > 1:
        # the per-frame results of every rank, in the job's frame order
        R = importlib.import_module("dpmd_public_gb300.replicas")
        offs = batch.plan.atom_off
        Fh = F_dev.cpu().numpy()
        Eg, Vg, Fg = R.gather_frame_results(
            frame_ids, E_dev.cpu().numpy(), V_dev.cpu().numpy(),
            [Fh[int(offs[k]):int(offs[k]) + len(f[1])] for k, f in enumerate(frames)],
            N_FRAMES * ws)
        out["replicas"] = {"frames_gathered": len(Fg), "atoms_gathered": int(sum(len(f) for f in Fg)),
                           "partition": "N x 512 frames, balanced by atoms (replicas.py)",
                           "energy_sum_eV": float(np.sum(Eg))}
    if not args.no_12k:
        del step
        out["water12k"] = water12k_leg(args, se_a, cfg, m64, model, dev, ws, rank, local, flush,
                                       full=False)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def type_one_side_false(se_a, cfg, frames, dev, args, flush):
    """The reference's argcheck default type_one_side = False (one table per
    (neighbour type, centre type) pair: four tables) on the same ragged
    batch: step time and the force error of the largest frame vs FP64."""
    import dataclasses

    import torch

    import composite

    cfg2 = dataclasses.replace(cfg, type_one_side=False)
    m64 = se_a.build_model(cfg2, SEED, _stat_frames(), dev, torch.float64)
    m = se_a.SeAModel(cfg2, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), dev,
                      torch.float32, m64.tables_np, m64.infos_np, fit_mode=args.fit_mode)
    b = m.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    step = se_a.CapturedStep(m, b, coord=np.concatenate([f[0] for f in frames]).astype(np.float32))
    ms, _ = time_captured(step, flush, max(3, min(args.steps, 10)), 3, 1)
    k = _by_size(frames, 2)[-1]
    c, t, bx = frames[k]
    a0 = int(b.plan.atom_off[k])
    np_model = _np_model(m64, cfg2)
    E64, F64, V64, _ = composite.energy_force_virial(*np_model[:4], c, t, bx, np_model[4],
                                                     np_model[5], cell_list=True)
    err = float(np.abs(b.force[a0:a0 + len(t)].cpu().numpy().astype(np.float64) - F64).max())
    nat = sum(len(f[1]) for f in frames)
    return {"value": nat / (ms * 1e-3), "ms_per_step": ms, "tables": len(m64.tables_np),
            "force_max_abs_eV_per_A_largest_frame": err,
            "form": "as the headline (fused, one packed CUDA graph) with type_one_side = False"}


def water12k_main(args):
    import torch

    ws, rank, local = _dist()
    dev = _init_dist(ws, local)
    torch.backends.cuda.matmul.allow_tf32 = False
    torch.backends.cudnn.allow_tf32 = False
    se_a, cfg, m64, model, _ = _setup_models(dev, args.fit_mode)
    out = water12k_leg(args, se_a, cfg, m64, model, dev, ws, rank, local, L2Flush(dev), full=True)
    if rank == 0:
        print(json.dumps(out))
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def water12k_leg(args, se_a, cfg, m64, model, dev, ws, rank, local, flush, full: bool):
    """The 12,288-atom single frame: value, e2e, per-part times and roofline,
    the operator-contract kernels' HBM fractions, errors vs FP64; with
    ``full`` also the atomic-sum variant, the plain forms and the CPU
    baseline (a line of its own)."""
    import importlib

    import torch

    L = importlib.import_module("dpmd_public_gb300._lib")
    c, t, b = _frame()
    nat = len(t)
    batch = model.batch([t], b[None])
    step = se_a.CapturedStep(model, batch, coord=c.astype(np.float32))
    step.replay()
    torch.cuda.synchronize()
    if batch.status() != 0:
        raise RuntimeError(f"neighbour build status {batch.status()}")
    launches = graph_kernels(step.graph)
    with Clocks(local) as clk:
        step_ms, wall = time_captured(step, flush, args.steps, args.warmup, ws, clk)
    step_ms = _max_over_ranks(step_ms, ws, dev)
    E_g, F_g, V_g = batch.energy.clone(), batch.force.clone(), batch.vir.clone()
    host_coord = c.astype(np.float32)
    e2e_ms = _max_over_ranks(time_e2e(step, host_coord, flush, args.steps, ws), ws, dev)
    e2e = {"value": ws * nat / (e2e_ms * 1e-3), "unit": "atom-steps/s",
           "h2d_bytes_per_step": step.h_coord.numel() * 4, "d2h_bytes_per_step": step.h_out.numel()}
    reps = max(3, min(args.steps, 10))
    kt = kernel_times(model, batch, step.coord, flush, reps=reps)
    dom = max(kt, key=lambda k: kt[k]["ms"])
    peaks = _peaks()
    roof = roofline(dom, kt[dom], nat, cfg, peaks, args.fit_mode)
    roof_parts = {}
    for k in kt:
        rp = roofline(k, kt[k], nat, cfg, peaks, args.fit_mode)
        roof_parts[k] = {x: rp[x] for x in ("kernel", "bound", "achieved", "unit", "frac",
                                            "ms_per_launch", "launches", "traffic") if x in rp}
    opk = op_kernel_times(model, batch, step.coord, flush, peaks, reps=reps)
    out = {"metric": METRIC, "value": ws * nat / (step_ms * 1e-3), "unit": "atom-steps/s",
           "n_gpus": ws, "steps": args.steps, "warmup": args.warmup, "ms_per_step": step_ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded water generator, random-init weights)",
           "config": {"workload": WORKLOAD_12K, "atoms": nat,
                      "form": "fused compressed, CUDA graph, deterministic (fixed-point) sums",
                      "fitting_gemm": args.fit_mode, "l2": L2Flush.DESC,
                      "parallelism": f"replicas x{ws}", "wall_s": wall},
           "e2e": e2e,
           "gpu_launches": None if launches is None else launches["ours"] * args.steps,
           "graph_kernels_per_step": launches,
           "kernels_ms": {k: v["ms"] for k, v in kt.items()},
           "roofline": roof, "roofline_parts": roof_parts, "op_kernels": opk,
           "clocks": clk.summary()}
    Fp = None
    if full:
        # the same step with floating-point atomic sums
        s2 = se_a.CapturedStep(model, batch, coord=step.coord, deterministic=False)
        det_ms, _ = time_captured(s2, flush, reps, 3, 1)
        del s2
        out["atomic_sums"] = {"value": ws * nat / (det_ms * 1e-3), "ms_per_step": det_ms,
                              "form": "the fused step with floating-point atomic force / virial / "
                                      "energy sums instead of the default fixed-point (bitwise "
                                      "reproducible) sums, CUDA graph"}
        mp = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), dev,
                           torch.float32)
        for _ in range(2):
            mp.step_ops(batch, step.coord, compressed=False)
        torch.cuda.synchronize()
        p0 = time.perf_counter()
        n_plain = max(2, min(args.steps, 5))
        for _ in range(n_plain):
            Ep, Fp, Vp = mp.step_ops(batch, step.coord, compressed=False)
        torch.cuda.synchronize()
        plain_ms = (time.perf_counter() - p0) / n_plain * 1e3
        out["plain"] = {"value": ws * nat / (plain_ms * 1e-3), "ms_per_step": plain_ms,
                        "form": "uncompressed drop-in (env op + matmul embedding + autograd + "
                                "force/virial ops), eager"}
        out["plain_tc"] = plain_tc_times(se_a, cfg, m64, args.fit_mode, t, b, step.coord, flush, ws)
    if rank == 0:
        import composite

        np_model = _np_model(m64, cfg)
        E64, F64, V64, _ = composite.energy_force_virial(*np_model[:4], c, t, b, np_model[4],
                                                         np_model[5], cell_list=True)
        Fn = F_g.cpu().numpy().astype(np.float64)
        out["errors_vs_fp64"] = {
            "force_max_abs_eV_per_A": float(np.abs(Fn - F64).max()),
            "force_rms_eV_per_A": float(np.sqrt(((Fn - F64) ** 2).mean())),
            "energy_per_atom_eV": abs(float(E_g[0]) - E64) / nat,
            "virial_max_abs_eV": float(np.abs(V_g[0].cpu().numpy() - V64).max()),
            "reference": "FP64 CPU composite (oracle) of the compressed model"}
        if full:
            errs = out["errors_vs_fp64"]
            errs["plain_force_max_abs_eV_per_A"] = float(np.abs(Fp.detach().cpu().numpy() - F64).max())
            errs["plain_tc_force_max_abs_eV_per_A_vs_plain_fp64"] = out["plain_tc"].pop(
                "_force_err_fn")(composite, np_model, c, t, b)
            if not args.no_cpu:
                out["cpu_baseline"] = cpu_baseline_12k((c, t, b), np_model)
    if not full:
        for k in ("metric", "unit", "n_gpus", "steps", "warmup", "higher_is_better", "scaling",
                  "vs_baseline", "dtype", "data"):
            out.pop(k, None)
    return out


def _setup_models(dev, fit_mode):
    import importlib

    import torch

    from __graft_entry__ import load_package

    pkg = load_package()
    pkg.load_library()
    importlib.import_module("dpmd_public_gb300._lib").set_autotune(True)
    se_a = importlib.import_module("dpmd_public_gb300.se_a")
    mdl = importlib.import_module("dpmd_public_gb300.model")
    cfg = mdl.SeAConfig()
    m64 = se_a.build_model(cfg, SEED, _stat_frames(), dev, torch.float64)
    mk = lambda compressed: se_a.SeAModel(
        cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), dev, torch.float32,
        m64.tables_np if compressed else None, m64.infos_np if compressed else None,
        fit_mode=fit_mode)
    return se_a, cfg, m64, mk(True), mk(False)


def train_workload(args):
    """Training step: 8 seeded 192-atom water frames in one packed batch of
    the compressed FP32 model, EnergyStdLoss (pref_e 0.02, pref_f 1000,
    pref_v 0.02) through the force and virial (double backward: tabulate
    grad-grad, prod_force_grad, prod_virial_grad) and its gradient wrt every
    fitting parameter; the fitting GEMMs in FP32 and in BF16 (FP32
    accumulation), the loss and gradients compared."""
    import importlib

    import torch

    torch.backends.cuda.matmul.allow_tf32 = False
    dev = torch.device("cuda", 0)
    se_a, cfg, m64, model, plain = _setup_models(dev, "fp32")
    water = importlib.import_module("dpmd_public_gb300.water")
    frames = [water.water_frame(4, 12.42, SEED + k) for k in range(8)]
    nat = sum(len(f[1]) for f in frames)
    batch = model.batch([f[1] for f in frames], np.stack([f[2] for f in frames]))
    coord = torch.tensor(np.concatenate([f[0] for f in frames]), dtype=torch.float32, device=dev)
    E0, F0, V0 = se_a.Trainable(model).energy_force_virial(batch, coord)
    gen = torch.Generator(device=dev).manual_seed(1)
    E_ref = (E0 + 0.1 * torch.randn(E0.shape, generator=gen, device=dev)).detach()
    F_ref = (F0 + 0.05 * torch.randn(F0.shape, generator=gen, device=dev)).detach()
    V_ref = (V0 + 0.1 * torch.randn(V0.shape, generator=gen, device=dev)).detach()
    res = {}
    for gemm in ("fp32", "bf16"):
        tr = se_a.Trainable(model, gemm)

        def step():
            E, F, V = tr.energy_force_virial(batch, coord)
            L = se_a.energy_std_loss(E, F, V, E_ref, F_ref, V_ref, len(frames[0][1]))
            return L, torch.autograd.grad(L, tr.params)

        for _ in range(args.warmup):
            step()
        torch.cuda.synchronize()
        st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        st.record()
        for _ in range(args.steps):
            L, g = step()
        en.record()
        torch.cuda.synchronize()
        res[gemm] = (st.elapsed_time(en) / args.steps, float(L.detach()),
                     torch.cat([x.reshape(-1) for x in g]))
    ms32, l32, g32 = res["fp32"]
    ms16, l16, g16 = res["bf16"]
    out = {"metric": "training atom-steps/s (force-loss step, double backward)",
           "value": nat / (ms32 * 1e-3), "unit": "atom-steps/s", "n_gpus": 1, "steps": args.steps,
           "warmup": args.warmup, "ms_per_step": ms32, "higher_is_better": True, "scaling": "weak",
           "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded water frames, random-init "
                                                     "weights, perturbed labels)",
           "config": {"workload": "8 x 192-atom water frames (12.42 A boxes), compressed se_e2_a FP32, "
                                  "EnergyStdLoss pref_e 0.02 / pref_f 1000 / pref_v 0.02, gradients wrt "
                                  "the fitting parameters", "atoms": nat,
                      "form": "operator form with autograd (eager)"},
           "bf16_fitting_gemms": {
               "value": nat / (ms16 * 1e-3), "ms_per_step": ms16,
               "loss_rel_diff_vs_fp32": abs(l16 - l32) / abs(l32),
               "grad_rel_l2_diff_vs_fp32": float((g16 - g32).norm() / g32.norm()),
               "grad_cosine_vs_fp32": float((g16.double() @ g32.double())
                                            / (g16.double().norm() * g32.double().norm())),
               "grad_max_abs_diff_vs_fp32": float((g16 - g32).abs().max())}}
    print(json.dumps(out))
    return 0


def md_workload(args):
    """262,144 H2O (786,432 atoms) in a 198.7 A box (64-molecule cell
    replicated 16^3, jittered), 330 K Maxwell-Boltzmann, velocity-Verlet
    NVE, dt 0.5 fs, the whole step captured in a CUDA graph; a 2 A skin
    with the Verlet list rebuilt every 10 steps (--md-skin 0: rebuilt every
    step)."""
    import importlib

    import torch

    dev = torch.device("cuda", 0)
    se_a, cfg, m64, _, _ = _setup_models(dev, args.fit_mode)
    # random weights give a potential without a repulsive core and forces far
    # beyond a liquid's; the output layer is scaled so that the forces stay
    # in a physical range (max |F| recorded in the trace) and the run
    # measures the integrator, not an exploding potential
    params = copy.deepcopy(m64.params_np)
    for net in params["fit"]:
        net["final"]["w"] = net["final"]["w"] * args.md_out_scale
        net["final"]["b"] = net["final"]["b"] * args.md_out_scale
    model = se_a.SeAModel(cfg, params, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(), dev,
                          torch.float32, m64.tables_np, m64.infos_np, fit_mode=args.fit_mode)
    water = importlib.import_module("dpmd_public_gb300.water")
    md = importlib.import_module("dpmd_public_gb300.md")
    c, t, b = water.replicated_frame(4, 12.42, 16, SEED)
    v = md.maxwell_boltzmann(t, 330.0, SEED)
    batch = model.batch([t], b[None], skin=args.md_skin)
    nve = md.NVE(model, batch, c, v, t, dt=0.5, rebuild_every=args.md_rebuild)
    nve.capture()
    e0 = nve.total_energy()
    torch.cuda.synchronize()
    trace = [(0, e0, nve.temperature(), float(nve.F.abs().max()))]
    chunk = max(1, args.md_steps // 10)
    st, en = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    ms = 0.0
    done = 0
    while done < args.md_steps:
        n = min(chunk, args.md_steps - done)
        st.record()
        nve.run(n)
        en.record()
        torch.cuda.synchronize()
        ms += st.elapsed_time(en)
        done += n
        trace.append((done, nve.total_energy(), nve.temperature(), float(nve.F.abs().max())))
    assert batch.status() == 0
    nat = len(t)
    drift = (trace[-1][1] - trace[0][1]) / nat / (args.md_steps * 0.5e-3)  # eV/atom/ps
    out = {"metric": METRIC, "value": nat * args.md_steps / (ms * 1e-3), "unit": "atom-steps/s",
           "n_gpus": 1, "steps": args.md_steps, "warmup": 2, "ms_per_step": ms / args.md_steps,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic", "config": {
               "workload": "262144 H2O (786432 atoms), 198.7 A box, NVE velocity-Verlet dt 0.5 fs, "
                           "330 K, whole step in a CUDA graph, " + (
                               f"{args.md_skin:g} A skin, list rebuilt every {args.md_rebuild} steps"
                               if args.md_skin > 0 else "nlist rebuilt every step"),
               "atoms": nat, "fitting_gemm": args.fit_mode,
               "model": f"random weights, fitting output layer x {args.md_out_scale}"},
           "energy_drift_eV_per_atom_per_ps": drift,
           "autotune": sys.modules["dpmd_public_gb300._lib"].autotune_report(),
           "trace": [{"step": s_, "etot_eV": e_, "T_K": T_, "max_abs_F_eV_per_A": f_}
                     for s_, e_, T_, f_ in trace]}
    print(json.dumps(out))
    return 0


def _new_graph():
    """A CUDA graph that keeps its cudaGraph_t after capture (so that its
    nodes can be listed), where this torch version offers that."""
    import torch

    try:
        return torch.cuda.CUDAGraph(keep_graph=True)
    except TypeError:
        return torch.cuda.CUDAGraph()


def graph_kernels(graph):
    """Kernel nodes of a captured step graph, counted by owner: this
    library's kernels (namespace gbdp) and everything else (torch,
    cuBLAS).  Read through the driver API; None when unavailable."""
    import ctypes

    try:
        h = graph.raw_cuda_graph()
        cu = ctypes.CDLL("libcuda.so.1")
    except Exception:
        return None

    class Params(ctypes.Structure):  # CUDA_KERNEL_NODE_PARAMS_v2
        _fields_ = [("func", ctypes.c_void_p), ("grid", ctypes.c_uint * 3),
                    ("block", ctypes.c_uint * 3), ("smem", ctypes.c_uint),
                    ("kernelParams", ctypes.c_void_p), ("extra", ctypes.c_void_p),
                    ("kern", ctypes.c_void_p), ("ctx", ctypes.c_void_p)]

    g = ctypes.c_void_p(h)
    n = ctypes.c_size_t(0)
    if cu.cuGraphGetNodes(g, None, ctypes.byref(n)) != 0:
        return None
    nodes = (ctypes.c_void_p * max(1, n.value))()
    if cu.cuGraphGetNodes(g, nodes, ctypes.byref(n)) != 0:
        return None
    ours, other, names = 0, 0, {}
    for i in range(n.value):
        ty = ctypes.c_int(-1)
        cu.cuGraphNodeGetType(ctypes.c_void_p(nodes[i]), ctypes.byref(ty))
        if ty.value != 0:  # CU_GRAPH_NODE_TYPE_KERNEL
            continue
        p = Params()
        name = ctypes.c_char_p()
        if cu.cuGraphKernelNodeGetParams_v2(ctypes.c_void_p(nodes[i]), ctypes.byref(p)) == 0:
            if p.func:
                cu.cuFuncGetName(ctypes.byref(name), ctypes.c_void_p(p.func))
            elif p.kern:
                cu.cuKernelGetName(ctypes.byref(name), ctypes.c_void_p(p.kern))
        nm = (name.value or b"?").decode(errors="replace")
        if "gbdp" in nm:
            ours += 1
            m = re.search(r"(k_[a-z0-9_]+)", nm)
            short = m.group(1) if m else nm
            names[short] = names.get(short, 0) + 1
        else:
            other += 1
    return {"ours": ours, "other": other, "ours_by_kernel": names}


class L2Flush:
    """Empties L2 between timed launches: a 256 MB write (larger than the
    129 MB L2), then a 256 MB read, so that the lines left in L2 are clean
    and the timed kernel does not pay for writing the flush back."""

    DESC = "flushed between timed steps (256 MB write, then 256 MB read)"

    def __init__(self, dev):
        import torch

        n = 256 * 1024 * 1024 // 4
        self.w = torch.empty(n, dtype=torch.float32, device=dev)
        self.r = torch.zeros(n, dtype=torch.float32, device=dev)
        self.o = torch.zeros((), dtype=torch.float32, device=dev)

    def __call__(self):
        import torch

        self.w.zero_()
        torch.sum(self.r, dim=0, out=self.o)


def kernel_times(model, batch, coord, flush, reps: int = 5):
    """Average device time of each part of the fused step (CUDA events on
    the launching stream, L2 flushed before each part)."""
    import ctypes

    import torch

    se_a = sys.modules["dpmd_public_gb300.se_a"]
    L = sys.modules["dpmd_public_gb300._lib"]
    cfg = model.cfg
    M, A = cfg.neuron[-1], cfg.axis_neuron
    lib = model._lib
    P = lambda x: ctypes.c_void_p(x.data_ptr())
    S = lambda: ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    b = batch
    ops = sys.modules["dpmd_public_gb300.ops"]

    def env():
        ops.env_mat_packed(b.plan, coord, b.atype, model.davg, model.dstd, cfg.rcut_smth, list(cfg.sel),
                           check_status=False, out=b.env)

    def fwd():
        if model._tc_nets is not None:
            lib.gbdp_se_a_descriptor_fwd_split_f32(P(b.X), P(b.D), P(b.D_lo), P(b.D_rs), P(b.env.em),
                                                   P(b.atype), P(b.drow), model._tab_ptrs,
                                                   model._tab_infos, cfg.ntypes, model._sel_c,
                                                   int(cfg.type_one_side), b.nloc, M, A, S())
        else:
            lib.gbdp_se_a_descriptor_fwd_f32(P(b.X), P(b.D), P(b.env.em), P(b.atype), P(b.drow),
                                             model._tab_ptrs, model._tab_infos, cfg.ntypes,
                                             model._sel_c, int(cfg.type_one_side), b.nloc, M, A, S())

    def fit():
        if model._tc_nets is not None:
            model.fitting_tc(b)
        else:
            model.fitting_rows(b)

    def bwd():
        lib.gbdp_se_a_descriptor_bwd_f32(
            P(b.force), P(b.vir), P(b.X), P(b.dD), P(b.drow), P(b.env.em), P(b.env.nlist_ext), P(b.env.ext_coord),
            P(b.env.ext_map), P(b.atype), P(model.dstd_inv), P(b.atom_frame), P(b.frame_aoff), P(b.frame_eoff),
            model._tab_ptrs, model._tab_infos, cfg.ntypes, model._sel_c, int(cfg.type_one_side),
            ctypes.c_float(cfg.rcut_smth), ctypes.c_float(cfg.rcut), b.nloc, b.nframes, M, A,
            P(b.force_fx()), S())

    parts = {"env_nlist": env, "desc_fwd": fwd, "fitting_gemm": fit, "desc_bwd": bwd}
    res = {}
    for name, fn in parts.items():
        ts = []
        for _ in range(reps):
            flush()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            fn()
            e.record()
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e))
        res[name] = {"ms": statistics.median(ts)}
    return res


def plain_tc_times(se_a, cfg, m64, fit_mode, t, b, coord, flush, ws, reps: int = 10):
    """The uncompressed model with the embedding nets on the tensor cores
    (BF16 MMAs, FP32 accumulation): the whole step captured in a CUDA graph
    and timed with CUDA events (L2 flushed between steps), plus the two
    embedding kernels alone."""
    import torch

    m = se_a.SeAModel(cfg, m64.params_np, m64.davg.cpu().numpy(), m64.dstd.cpu().numpy(),
                      coord.device, torch.float32, fit_mode=fit_mode)
    bt = m.batch([t], b[None])
    side = torch.cuda.Stream()
    side.wait_stream(torch.cuda.current_stream())
    with torch.cuda.stream(side):
        for _ in range(2):
            m.step_plain_tc(bt, coord)
    torch.cuda.current_stream().wait_stream(side)
    torch.cuda.synchronize()
    g = torch.cuda.CUDAGraph()
    with torch.cuda.graph(g):
        E, F, V = m.step_plain_tc(bt, coord)
    g.replay()
    torch.cuda.synchronize()
    if int(bt.emb_status.item()) != 0:
        raise RuntimeError("tensor-core embedding reported a device status")

    def timed(fn):
        ts = []
        for _ in range(reps):
            flush()
            s0, s1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s0.record()
            fn()
            s1.record()
            torch.cuda.synchronize()
            ts.append(s0.elapsed_time(s1))
        return statistics.median(ts)

    step_ms = timed(g.replay)
    em = bt.env_full.em
    fwd_ms = timed(lambda: m.embed_tc_forward(bt, em))
    bwd_ms = timed(lambda: m.embed_tc_backward(bt, em))
    nat = len(t)
    F_dev = F

    def force_err(composite, np_model, c, t_, b_):
        E64, F64, V64, _ = composite.energy_force_virial(*np_model[:4], c, t_, b_, None, None)
        return float(np.abs(F_dev.cpu().numpy().astype(np.float64) - F64).max())

    # MMA work per neighbour row (algorithmic widths): forward 1x25x50 + 50x100;
    # backward recomputes the forward and adds the two transposed products
    n1, n2, n3 = cfg.neuron
    rows = nat * cfg.nnei
    f_fwd = 2 * (n1 * n2 + n2 * n3) * rows
    return {"value": ws * nat / (step_ms * 1e-3), "ms_per_step": step_ms,
            "form": "uncompressed, embedding + G^T R on tcgen05 BF16 (FP32 accumulation), "
                    f"fitting {fit_mode}, force/virial operators; CUDA graph",
            "embed_fwd_ms": fwd_ms, "embed_bwd_ms": bwd_ms,
            "embed_mma_tflops": {"fwd": f_fwd / (fwd_ms * 1e-3) / 1e12,
                                 "bwd": 2 * f_fwd / (bwd_ms * 1e-3) / 1e12},
            "_force_err_fn": force_err}


def op_kernel_times(model, batch, coord, flush, peaks, reps: int = 5):
    """The operator-contract kernels (the reference's op sequence on the
    GPU) on the same frame, one at a time: device time per call (CUDA
    events, L2 flushed before each call), algorithmic HBM bytes per call
    (each op's inputs read once and outputs written once) and the fraction
    of the measured HBM bandwidth.  The env matrix and force / virial
    scatters are HBM-bound; the tabulation calls are bound by table rows
    through L2, so their HBM fraction is listed for reference only."""
    import torch

    ops = sys.modules["dpmd_public_gb300.ops"]
    cfg = model.cfg
    b = batch
    n, nn, M = b.nloc, cfg.nnei, cfg.neuron[-1]
    dev = coord.device
    dt = model.dtype
    f = 4
    env = ops.EnvMatResult()
    env.em = torch.empty((n, nn, 4), dtype=dt, device=dev)
    env.em_deriv = torch.empty((n, nn, 4, 3), dtype=dt, device=dev)
    env.rij = torch.empty((n, nn, 3), dtype=dt, device=dev)
    env.nlist = torch.empty((n, nn), dtype=torch.int32, device=dev)
    env.nlist_ext = None
    env.ext_coord = torch.empty((b.plan.ext_total, 3), dtype=dt, device=dev)
    env.ext_type = torch.empty((b.plan.ext_total,), dtype=torch.int32, device=dev)
    env.ext_map = torch.empty((b.plan.ext_total,), dtype=torch.int32, device=dev)
    env.ext_nall = torch.empty((b.nframes,), dtype=torch.int32, device=dev)

    def env_op():
        ops.env_mat_packed(b.plan, coord, b.atype, model.davg, model.dstd, cfg.rcut_smth,
                           list(cfg.sel), check_status=False, out=env)

    env_op()
    torch.cuda.synchronize()
    nall = int(env.ext_nall[0])
    gen = torch.Generator(device=dev).manual_seed(3)
    net = torch.randn((1, n * nn * 4), generator=gen, device=dev, dtype=dt)
    natoms = torch.tensor([n, nall, 0, 0], dtype=torch.int32)
    ed, rij, nl = env.em_deriv.reshape(1, -1), env.rij.reshape(1, -1), env.nlist.reshape(1, -1)
    # one tabulation call per neighbour-type section over all atoms (table of
    # the O-centred net), inputs made contiguous beforehand
    sec = cfg.sec
    tab = []
    for tj in range(cfg.ntypes):
        k = tj if cfg.type_one_side else tj * cfg.ntypes
        rr = env.em[:, sec[tj]:sec[tj + 1], :].contiguous()
        tab.append((model.tables[k], model.table_info_t[k], rr[:, :, :1].reshape(-1, 1).contiguous(),
                    rr, torch.randn((n, 4, M), generator=gen, device=dev, dtype=dt)))
    parts = {
        # coord + type in, ghosts (~nall - nloc) written; em, em_deriv, rij, nlist out
        "prod_env_mat_a": (env_op, n * (16 + nn * (16 + 48 + 12 + 4)) + (nall - n) * 20),
        "prod_force_se_a": (lambda: ops.prod_force_se_a_impl(net, ed, nl, natoms, nn, 0),
                            n * nn * (16 + 48 + 4) + nall * 12),
        "prod_force_se_a_det": (lambda: ops.prod_force_se_a_impl(net, ed, nl, natoms, nn, 0, True),
                                n * nn * (16 + 48 + 4) + nall * 12),
        "prod_virial_se_a": (lambda: ops.prod_virial_se_a_impl(net, ed, rij, nl, natoms, nn, 0),
                             n * nn * (16 + 48 + 12 + 4) + nall * 36 + 36),
        # both outputs from one pass over the shared inputs
        "prod_force_virial_se_a": (
            lambda: ops.prod_force_virial_se_a_impl(net, ed, rij, nl, natoms, nn, 0),
            n * nn * (16 + 48 + 12 + 4) + nall * (12 + 36) + 36),
        "tabulate_fusion_se_a": (lambda: [ops.tabulate_forward(t_, i_, x_, e_, M)
                                          for t_, i_, x_, e_, _ in tab],
                                 sum(x_.numel() * f * 5 + n * 4 * M * f for _, _, x_, _, _ in tab)),
        "tabulate_fusion_se_a_grad": (lambda: [ops.tabulate_grad(t_, i_, x_, e_, d_)
                                               for t_, i_, x_, e_, d_ in tab],
                                      sum(x_.numel() * f * 10 + n * 4 * M * f
                                          for _, _, x_, _, _ in tab)),
    }
    res = {}
    for name, (fn, nbytes) in parts.items():
        # each op captured in its own graph, so that host work between its
        # launches (argument checks, output allocation) is not timed
        side = torch.cuda.Stream()
        side.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(side):
            fn()
        torch.cuda.current_stream().wait_stream(side)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            fn()
        g.replay()
        ts = []
        for _ in range(reps):
            flush()
            s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            s.record()
            g.replay()
            e.record()
            torch.cuda.synchronize()
            ts.append(s.elapsed_time(e))
        del g
        ms = statistics.median(ts)
        gbs = nbytes / (ms * 1e-3) / 1e9
        res[name] = {"ms": ms, "alg_bytes": nbytes, "achieved_gbs": gbs,
                     "frac_hbm": gbs / peaks["hbm_gbs"],
                     "bound": "L2 table rows" if name.startswith("tab") else "hbm"}
    return res


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return {"hbm_gbs": d["hbm_gbs"], "bf16_tflops": d["bf16_tflops"], "src": "measured"}
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "src": "fallback"}


# algorithmic HBM bytes per local atom of each part (FP32, nnei 138, M 100,
# A 16): inputs read once, outputs written once
def _alg_bytes(name, cfg, fit_mode="tc-f16x3"):
    nn, M, A = cfg.nnei, cfg.neuron[-1], cfg.axis_neuron
    f = 4
    if name == "env_nlist":
        # coord + type in; em, nlist (local + ext) out; ghosts ~0.9 x nloc x 16 B
        return 12 + 4 + nn * 4 * f + 2 * nn * 4 + 16
    if name == "desc_fwd":
        # em in; X, D out (D as FP16 hi and lo, 4 bytes an element with its
        # row scale, for the tensor-core fitting)
        return nn * 4 * f + 4 * M * f + M * A * f + 4 + (4 if fit_mode == "tc-f16x3" else 0)
    if name == "desc_bwd":
        # X, dE/dD, em, nlist_ext in; ~91 neighbour coords (L2) ; force out
        return 4 * M * f + M * A * f + nn * 4 * f + nn * 4 + 12
    if name == "fitting_gemm":
        return 2 * M * A * f  # D in, dE/dD out
    return 0


# algorithmic FLOPs per row of the fitting net (forward and backward GEMMs,
# FP32 products): D W1, H1 W2, H2 W3, H3 w_out; GZ3 W3^T, GZ2 W2^T, GZ1 W1^T
def _fit_flops(cfg):
    w = [cfg.dim_descrpt] + list(cfg.fitting)
    fwd = sum(w[i] * w[i + 1] for i in range(len(w) - 1)) + w[-1]
    bwd = sum(w[i] * w[i + 1] for i in range(len(w) - 1))
    return 2 * (fwd + bwd)


PART_KERNEL = {"env_nlist": "k_nlist_env (+ cell build and ghost fill)",
               "desc_fwd": "k_desc_fwd", "desc_bwd": "k_desc_bwd"}

# dram__bytes_read.sum + dram__bytes_write.sum per local atom, from one ncu
# capture of the 12,288-atom step (profiles/k_desc_fwd_bwd_12288.md,
# profiles/k_fit_tc_12288.md: the six fitting GEMM launches summed), scaled
# to a launch by the atoms it processes (the traffic of these kernels grows
# in proportion to the atoms)
NCU_TRAFFIC_ATOM = {"desc_bwd": 133.1e6 / 12288, "desc_fwd": 65.7e6 / 12288,
                    "fitting_gemm": 6 * 40.6e6 / 12288}
NCU_TRAFFIC_SRC = "ncu capture of the 12,288-atom step, scaled by atoms"


def roofline(name, t, nat, cfg, peaks, fit_mode):
    ms = t["ms"]
    if name == "fitting_gemm":
        tc = fit_mode == "tc-f16x3"
        nl = 6 if tc else 1
        flops = _fit_flops(cfg) * nat
        ach = flops / (ms * 1e-3) / 1e12
        peak = peaks["bf16_tflops"]
        out = {"kernel": "k_fit_tc + k_fit_pers" if tc else f"cuBLAS ({fit_mode}) + k_fit_*", "bound": "tensor",
               "achieved": ach, "peak": peak, "unit": "TFLOP/s", "frac": ach / peak,
               "traffic": NCU_TRAFFIC_ATOM[name] * nat / nl if tc else None,
               "traffic_src": NCU_TRAFFIC_SRC if tc else None,
               "peak_src": peaks["src"] + " (dense BF16, burst)",
               "alg_flops_per_launch": flops / nl, "launches": nl, "ms_per_launch": ms / nl}
        if tc:
            # FP32 products as 3 FP16 MMAs at the BF16 rate: 1/3 of peak
            out["ceiling_f16x3_tflops"] = peak / 3
            out["frac_of_f16x3_ceiling"] = ach / (peak / 3)
        return out
    alg = _alg_bytes(name, cfg, fit_mode) * nat
    ach = alg / (ms * 1e-3) / 1e9
    return {"kernel": PART_KERNEL.get(name, name), "bound": "hbm", "achieved": ach,
            "peak": peaks["hbm_gbs"], "unit": "GB/s", "frac": ach / peaks["hbm_gbs"],
            "traffic": (NCU_TRAFFIC_ATOM[name] * nat) if name in NCU_TRAFFIC_ATOM else None,
            "traffic_src": NCU_TRAFFIC_SRC if name in NCU_TRAFFIC_ATOM else None,
            "peak_src": peaks["src"],
            "alg_bytes_per_launch": alg, "launches": 1, "ms_per_launch": ms}


if __name__ == "__main__":
    sys.exit(main())
