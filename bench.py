#!/usr/bin/env python
"""Benchmark of the fused D3Q19 wall-wind step on GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--workload c2|c1|c3]

Workload (default c2, the headline case): 800 x 160 x 160 cells (H = 40,
domain 20H x 4H x 4H), an ellipsoid-packed stone wall 0.75H thick at x = 5H,
porosity 0.2, seed 1, ground at z = 0, inlet u = 0.05 (z/H)^(1/7), Re_H = 1e4,
Cs = 0.1, float32 populations, 2 % Gaussian initial noise.  A step is one
timestep of the whole lattice in the averaging phase of the run: the fused
step, plus the float64 mean-field accumulation on every 5th step, as the solve
runs it.  Each lattice is 1.56 GB (> 129 MB L2), so no L2 flush is needed
between steps.

One JSON line on rank 0:
  value     MLUPS (all nx*ny*nz cells, the reference's convention) with the
            state resident in HBM, K steps timed with CUDA events
  e2e       the same metric through the public WallSolver API from host
            buffers: mask and inlet upload, segment classification, init, K
            steps, force-series download, all inside the timed region
  roofline  the step kernel alone (CUDA events around K eager launches):
            152 B x fluid cells per launch / mean launch time vs the measured
            HBM copy bandwidth
  cpu_baseline  the CPU oracle (float32, OpenMP, all host cores) on a crop of
            the same workload, about 10 s of CPU time
--impl reference times that CPU implementation alone (the reference's own
Warp CPU path is unavailable: Warp cannot be installed here or on the GPU machine).
Under torchrun each rank runs its own replica (the path is not sharded).
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
PKG = os.path.join(ROOT, "jeju-stonewall-lbm_gb300")
for _p in (ROOT, PKG):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "D3Q19 MLUPS & %HBM roofline; wall solves/hr + p99 latency at Cd err<=1% vs FP64"
BYTES_PER_CELL = {"f32": 152, "f64": 304, "f16": 76, "bf16": 76}

WORKLOADS = {
    "c1": dict(H=16, n_total=2000, porosity=0.2, seed=0),
    "c2": dict(H=40, n_total=40000, porosity=0.2, seed=1),
    "c3": dict(H=64, n_total=20000, porosity=0.3, seed=0),
}


def bench_config(name, p, dtype):
    """The workload description both arms print (same dict, so the two lines can be matched)."""
    w = WORKLOADS[name]
    return dict(workload=f"{name}: {p.nx}x{p.ny}x{p.nz} H={p.H} ellipsoid wall porosity {w['porosity']} "
                         f"seed {w['seed']}", grid=[p.nx, p.ny, p.nz], H=p.H, porosity=w["porosity"], seed=w["seed"],
                dtype=dtype, phase="averaging (accumulate every 5th step)")


def workload(name):
    from stonewall.geometry import ellipsoid_wall
    from stonewall.params import baseline_params, flags_from_wall
    w = WORKLOADS[name]
    p = baseline_params(w["H"], w["n_total"])
    wall, frac = ellipsoid_wall(w["porosity"], p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=w["seed"])
    return p, flags_from_wall(wall, p.nx, p.ny, p.nz), frac


# ---------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi samples during the timed region (SM clock, throttle reasons)."""
    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index, self.proc, self.lines = index, None, []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except (OSError, FileNotFoundError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.thread.join(timeout=2)

    def rows(self):
        return len(self.lines)

    def summary(self):
        rows = []
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                rows.append(dict(sm=float(parts[1]), smax=float(parts[2]), reasons=parts[5:9]))
            except ValueError:
                continue
        if not rows:
            return None
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        active = sorted({n for r in rows for n, v in zip(names, r["reasons"]) if v.lower() == "active"})
        return {"sm_mhz": statistics.median(r["sm"] for r in rows), "sm_max_mhz": max(r["smax"] for r in rows),
                "reasons": active, "samples": len(rows)}


def measured_peak():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(path) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured"
    except (OSError, KeyError, ValueError):
        return 6800.0, "fallback"


def profiled_traffic(dtype, cells):
    """DRAM bytes per step launch from the committed ncu summary (bytes per cell x cells), or None."""
    path = os.path.join(ROOT, "profiles", f"step_{dtype}_dram_per_cell.txt")
    try:
        with open(path) as fh:
            for line in fh:
                if line.startswith("dram_bytes_per_cell:"):
                    return float(line.split(":")[1]) * cells
    except OSError:
        pass
    return None


def cpu_model():
    """The host CPU's model name (Linux /proc/cpuinfo; 'model name', or the Arm 'CPU part' line)."""
    try:
        with open("/proc/cpuinfo") as fh:
            text = fh.read()
    except OSError:
        return "unknown"
    arm_parts = {"0xd4f": "Arm Neoverse-V2", "0xd40": "Arm Neoverse-V1", "0xd0c": "Arm Neoverse-N1",
                 "0xd49": "Arm Neoverse-N2", "0xd8e": "Arm Neoverse-N3", "0xd84": "Arm Neoverse-V3"}
    for key in ("model name", "Model", "CPU part"):
        for line in text.splitlines():
            if line.startswith(key):
                v = line.split(":", 1)[1].strip()
                return arm_parts.get(v, f"CPU part {v}") if key == "CPU part" else v
    return "unknown"


# ---------------------------------------------------------------- CPU oracle timing
def cpu_sample(p, flag, target_s=10.0, max_steps=None):
    """Time the CPU oracle on an x-crop of the workload around the wall.  Returns dict."""
    from oracle import oracle as O
    threads = O.max_threads()
    x0, x1 = max(0, p.X0 - 20), min(p.nx, p.X0 + p.T + 50)
    crop = np.ascontiguousarray(flag[x0:x1])
    nxc = crop.shape[0]
    f = O.init(crop, p.uin, noise=0.02, seed=1)
    fb = np.zeros_like(f)
    O.step(f, crop, p.uin, np.float32(p.nu0), np.float32(p.Cs), nxc - 10, np.float32(0.05), f_out=fb)  # warm
    steps, t0 = 0, time.perf_counter()
    while True:
        O.step(f, crop, p.uin, np.float32(p.nu0), np.float32(p.Cs), nxc - 10, np.float32(0.05), f_out=fb)
        f, fb = fb, f
        steps += 1
        el = time.perf_counter() - t0
        if el >= target_s or (max_steps and steps >= max_steps):
            break
    cells = crop.size
    return dict(value=round(cells * steps / el / 1e6, 2), unit="MLUPS", cores=threads, kind="port",
                cpu=cpu_model(), host_cpus=os.cpu_count(),
                sample=f"{steps} float32 steps of an x-crop {nxc}x{p.ny}x{p.nz} ({cells/1e6:.2f} M cells) of the "
                       f"workload around the wall, {el:.1f} s, oracle/sw_oracle.cpp with {threads} OpenMP threads")


# ---------------------------------------------------------------- distributed helpers
def dist_env():
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return ws, rank, local


def barrier(ws):
    if ws > 1:
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x, ws, device="cpu"):
    """The largest of the ranks' values (the timing rule: the slowest replica sets the step time)."""
    if ws == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def run_reference(a):
    ws, rank, _ = dist_env()
    if rank != 0:
        return 0
    p, flag, frac = workload(a.workload)
    from oracle import oracle as O
    threads = O.max_threads()
    # size the per-step sample so the whole run stays within ~2 minutes
    probe = cpu_sample(p, flag, target_s=2.0)
    crop_cells = (min(p.nx, p.X0 + p.T + 50) - max(0, p.X0 - 20)) * p.ny * p.nz
    per_step = crop_cells / (probe["value"] * 1e6)
    budget = min(2.0, 120.0 / max(1, a.steps + a.warmup))
    planes = max(4, min(p.nx, int(budget / per_step * (crop_cells / (p.ny * p.nz)))))
    x0 = max(0, min(p.X0 - 20, p.nx - planes))
    crop = np.ascontiguousarray(flag[x0:x0 + planes])
    nxc = crop.shape[0]
    f = O.init(crop, p.uin, noise=0.02, seed=1)
    fb = np.zeros_like(f)
    args = (np.float32(p.nu0), np.float32(p.Cs), nxc - 10, np.float32(0.05))
    for _ in range(a.warmup):
        O.step(f, crop, p.uin, *args[:3], args[3], f_out=fb)
        f, fb = fb, f
    t0 = time.perf_counter()
    for _ in range(a.steps):
        O.step(f, crop, p.uin, *args[:3], args[3], f_out=fb)
        f, fb = fb, f
    el = time.perf_counter() - t0
    mlups = crop.size * a.steps / el / 1e6
    sample = (f"each step: one float32 timestep of an x-crop {nxc}x{p.ny}x{p.nz} ({crop.size/1e6:.2f} M cells) of "
              f"the workload; CPU oracle oracle/sw_oracle.cpp (restatement of lbm3d.py k_step; Warp's CPU device "
              f"is unavailable) with {threads} OpenMP threads")
    line = dict(metric=METRIC, value=round(mlups, 2), unit="MLUPS", n_gpus=a.gpus, steps=a.steps, warmup=a.warmup,
                ms_per_step=round(el / a.steps * 1e3, 3), higher_is_better=True, scaling="weak", vs_baseline=None,
                dtype="f32", data="synthetic", impl="reference",
                config=bench_config(a.workload, p, "f32"),
                sample_grid=[nxc, p.ny, p.nz],
                cpu_baseline=dict(value=round(mlups, 2), unit="MLUPS", cores=threads, kind="port", sample=sample,
                                  cpu=cpu_model(), host_cpus=os.cpu_count()),
                e2e=dict(value=round(mlups, 2), unit="MLUPS", h2d_bytes_per_step=0, d2h_bytes_per_step=0))
    print(json.dumps(line), flush=True)
    return 0


def run_ours(a):
    import torch
    ws, rank, local = dist_env()
    if ws > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl" if torch.cuda.is_available() else "gloo")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    from stonewall import _native
    from stonewall import kernels as K
    from stonewall.solver import WallSolver
    L = _native.lib()
    p, flag, frac = workload(a.workload)
    dtype = a.dtype
    cells = p.cells
    fluid_cells = int((flag == 0).sum())
    W, Ks = a.warmup, a.steps
    chunk = min(a.chunk, Ks)          # the timed steps replay CUDA graphs of `chunk` steps

    # --- resident run: averaging phase of the solve (step + accumulation every 5th step)
    n_total = p.n_total
    solver = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, n_total, n_spin=0, dtype=dtype, device=dev,
                        chunk=chunk)
    solver.init(noise=0.02, seed=1, noise_kind="gauss")
    solver.advance(W)
    if a.cfg is None:
        cfg, cfg_times = solver.autotune()                           # launch configuration, untimed
        cfg_acc = L.sw_get_step_config_accum(solver.dtype)
    else:
        _native.check(L.sw_set_step_config(solver.dtype, a.cfg), "sw_set_step_config")
        _native.check(L.sw_set_step_config_accum(solver.dtype, a.cfg), "sw_set_step_config_accum")
        cfg, cfg_acc, cfg_times = a.cfg, a.cfg, {}
    solver.advance(max(W, 2 * chunk))                                # warm-up, graph capture included
    torch.cuda.synchronize()
    barrier(ws)
    launches0 = solver.launches
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        torch.cuda.synchronize()
        e0.record()
        solver.advance(Ks, check=False)      # graph replays; the status word is read after e1
        e1.record()
        torch.cuda.synchronize()
        solver.check_status()
        gpu_launches = solver.launches - launches0
        clocks = clk.summary()
        if clocks is None or clocks["samples"] < 3:
            # the timed region was shorter than three sampling intervals: sample the same steps,
            # continued right after it, for about a second (untimed)
            t_end = time.perf_counter() + 1.0
            while (time.perf_counter() < t_end or clk.rows() < 3) and time.perf_counter() < t_end + 5.0:
                if solver.t + chunk > solver.n_total:
                    break
                solver.advance(chunk, check=False)
                torch.cuda.synchronize()
            clocks = clk.summary()
            if clocks is not None:
                clocks["sampled"] = ("the same steps continued for ~1 s right after the timed region, which is "
                                     "shorter than three 200 ms sampling intervals")
        else:
            clocks["sampled"] = "during the timed region"
    barrier(ws)
    ms = max_over_ranks(e0.elapsed_time(e1), ws, dev)
    value = ws * cells * Ks / (ms * 1e-3) / 1e6

    # --- roofline: the step kernel alone, eager launches on this stream
    g = solver.grid
    src, dst = solver.f[0], solver.f[1]
    for i in range(3):
        K.k_step(src, dst, solver.flags, solver.uin, g.nx, g.ny, g.nz, p.nu0, p.Cs, p.x_sponge, 0.05, None, 0)
        src, dst = dst, src
    torch.cuda.synchronize()
    stream = torch.cuda.current_stream()
    r0, r1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    r0.record(stream)
    for i in range(Ks):
        K.k_step(src, dst, solver.flags, solver.uin, g.nx, g.ny, g.nz, p.nu0, p.Cs, p.x_sponge, 0.05, None, 0,
                 stream=stream)
        src, dst = dst, src
    r1.record(stream)
    torch.cuda.synchronize()
    step_ms = r0.elapsed_time(r1) / Ks
    alg_bytes = BYTES_PER_CELL[dtype] * fluid_cells
    peak, peak_kind = measured_peak()
    achieved = alg_bytes / (step_ms * 1e-3) / 1e9
    traffic = profiled_traffic(dtype, cells)
    roofline = dict(bound="hbm", achieved=round(achieved, 1), peak=peak, unit="GB/s", frac=round(achieved / peak, 4),
                    traffic=traffic, peak_source=f"{peak_kind} (MEASURED_PEAKS.json hbm_gbs)" if peak_kind ==
                    "measured" else "fallback 6.8 TB/s",
                    kernel="k_step_pull" if cfg < 4 else ("k_step_pair" if cfg < 8 else "k_step_tma"),
                    step_ms=round(step_ms, 4), alg_bytes_per_launch=alg_bytes,
                    bytes_per_fluid_cell=BYTES_PER_CELL[dtype])
    del solver
    torch.cuda.empty_cache()

    # --- end to end through the public API, host buffers in and out
    flag_pin = torch.from_numpy(flag).pin_memory()
    uin_pin = torch.from_numpy(p.uin.copy()).pin_memory()
    solver = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, max(Ks, 2 * chunk), n_spin=0, dtype=dtype,
                        device=dev, chunk=chunk)
    solver.init(noise=0.02, seed=1, noise_kind="gauss")
    solver.advance(min(solver.n_total, 2 * chunk))                 # capture graphs outside the timed region
    force_host = torch.empty((Ks, g.nz, 2), dtype=torch.int64).pin_memory()
    torch.cuda.synchronize()
    barrier(ws)
    x0, x1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    x0.record()
    solver.reload(flag_pin, uin_pin)        # H2D of the mask and inlet, re-classification
    solver.init(noise=0.02, seed=1, noise_kind="gauss")
    solver.advance(Ks)                      # reads the status word at the end
    force_host.copy_(solver.force.data[:Ks], non_blocking=True)
    x1.record()
    torch.cuda.synchronize()
    barrier(ws)
    e2e_ms = max_over_ranks(x0.elapsed_time(x1), ws, dev)
    e2e = dict(value=round(ws * cells * Ks / (e2e_ms * 1e-3) / 1e6, 1), unit="MLUPS",
               h2d_bytes_per_step=round((flag.nbytes + p.uin.nbytes) / Ks, 1),
               d2h_bytes_per_step=g.nz * 2 * 8 + 4, ms_total=round(e2e_ms, 3))
    del solver
    torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and ws == 1 and not a.no_cpu:
        cpu = cpu_sample(p, flag, target_s=a.cpu_seconds)

    if rank == 0:
        line = dict(metric=METRIC, value=round(value, 1), unit="MLUPS", n_gpus=ws, steps=Ks, warmup=W,
                    ms_per_step=round(ms / Ks, 4), higher_is_better=True, scaling="weak", vs_baseline=None,
                    dtype=dtype, data="synthetic", config=bench_config(a.workload, p, dtype),
                    run=dict(cells=cells, fluid_cells=fluid_cells, fluid_mlups=round(value * fluid_cells / cells, 1),
                             solid_fraction_of_wall_box=round(frac, 4),
                             l2="no flush: each lattice is %.2f GB > 129 MB L2" % (cells * 76 / 1e9 *
                                                                                    BYTES_PER_CELL[dtype] / 152),
                             timed_steps=f"{Ks} steps as {Ks // chunk} replays of a {chunk}-step CUDA graph"
                                         + (f" + {Ks % chunk} eager launches" if Ks % chunk else ""),
                             parallelism=f"replicas x{ws}", step_config=cfg, step_config_accum=cfg_acc,
                             step_config_ms={str(k): round(v, 4) for k, v in cfg_times.items()}),
                    roofline=roofline, cpu_baseline=cpu, e2e=e2e, gpu_launches=gpu_launches,
                    clocks=clocks)
        print(json.dumps(line), flush=True)
    if ws > 1:
        torch.distributed.destroy_process_group()
    return 0


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=500)
    ap.add_argument("--warmup", type=int, default=20)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--dtype", default="f32", choices=sorted(BYTES_PER_CELL))
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--cpu-seconds", type=float, default=10.0)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--cfg", type=int, default=None,
                    help="use this step launch configuration instead of autotuning (for profiling commands)")
    a = ap.parse_args(argv)
    if a.warmup < 3:
        ap.error("--warmup must be at least 3")
    if a.impl == "reference":
        return run_reference(a)
    return run_ours(a)


if __name__ == "__main__":
    sys.exit(main())
