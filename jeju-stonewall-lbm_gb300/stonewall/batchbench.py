"""Many-wall batch run: aggregate throughput and per-wall accuracy against the plain form.

    python -m stonewall.batchbench [--walls 64] [--steps 10000] [--dtype f16] [--no-plain]
                                   [--H 40] [--porosity 0.2] [--seed 0] [--mode persistent --cfg 4]

Walls: for i in 0..walls-1, rng = default_rng(i) draws H from {16, 24, 32, 40}
and porosity from U[0, 0.5] (--H / --porosity fix them for every wall); each
wall is an ellipsoid-packed stone wall with seed seed + i in a 20H x 4H x 4H
domain (stonewall.params.baseline_params).  All walls
advance together in one persistent launch per step (stonewall.batch.Batch),
replayed from a captured CUDA graph, or as one graph of per-wall launches
per chunk (the autotuner picks the faster mode).  The plain form is the same walls solved
one after another by WallSolver in float32.  Prints one JSON line: aggregate
MLUPS, wall solves per hour for both forms and their ratio, and the per-wall
relative errors of mean and peak Cd and peak Cm of the batch against the plain
form.
"""
import argparse
import json
import time

import numpy as np
import torch

from .batch import Batch
from .geometry import ellipsoid_wall
from .metrics import device_stats
from .params import baseline_params, flags_from_wall
from .solver import WallSolver


def wall_specs(n, H=None, porosity=None, seed=0):
    out = []
    for i in range(n):
        rng = np.random.default_rng(i)
        h = int(rng.choice([16, 24, 32, 40]))
        por = float(rng.uniform(0.0, 0.5))
        out.append(dict(i=i, H=h if H is None else int(H), porosity=por if porosity is None else float(porosity),
                        seed=seed + i))
    return out


def make_solver(spec, n_total, dtype, device="cuda", noise_seed=None):
    p = baseline_params(spec["H"], n_total)
    wall, frac = ellipsoid_wall(spec["porosity"], p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=spec["seed"])
    flag = flags_from_wall(wall, p.nx, p.ny, p.nz)
    s = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, n_total, n_spin=p.n_spin, dtype=dtype, device=device)
    s.init(noise=0.02, seed=spec["seed"] if noise_seed is None else noise_seed, noise_kind="gauss")
    s.params = p
    return s


def wall_stats(s):
    return device_stats(s.force, s.params.UH, s.params.H, s.params.ny, s.n_spin)


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-12)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--walls", type=int, default=64)
    ap.add_argument("--steps", type=int, default=10000)
    ap.add_argument("--dtype", default="f16")
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--no-plain", action="store_true", help="skip the float32 one-wall-at-a-time reference")
    ap.add_argument("--mode", default="auto", choices=["auto", "persistent", "graph"],
                    help="batch mode (auto: the autotuner times both)")
    ap.add_argument("--H", type=int, default=None, help="wall height of every wall (default: drawn per wall)")
    ap.add_argument("--porosity", type=float, default=None, help="porosity of every wall (default: drawn)")
    ap.add_argument("--seed", type=int, default=0, help="mask seed of wall 0 (wall i: seed + i)")
    ap.add_argument("--cfg", type=int, default=None,
                    help="persistent kernel launch configuration (with --mode persistent; skips the autotuner)")
    a = ap.parse_args(argv)
    if a.cfg is not None and a.mode != "persistent":
        ap.error("--cfg selects a configuration of the persistent kernel: give --mode persistent")
    specs = wall_specs(a.walls, a.H, a.porosity, a.seed)
    t_build = time.time()
    batch = Batch(dtype=a.dtype, chunk=a.chunk, max_members=max(64, a.walls))
    members = [batch.add(make_solver(sp, a.steps, a.dtype)) for sp in specs]
    t_build = time.time() - t_build
    modes = ("persistent", "graph") if a.mode == "auto" else (a.mode,)
    if a.cfg is None:
        cfg, cfg_times = batch.autotune(modes=modes)
    else:
        batch.cfg, batch.mode, cfg_times = a.cfg, "persistent", {}
    cells = batch.cells()
    torch.cuda.synchronize()
    t0 = time.time()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    batch.run()
    e1.record()
    torch.cuda.synchronize()
    wall_s = time.time() - t0
    gpu_ms = e0.elapsed_time(e1)
    batch_stats = [wall_stats(m) for m in members]
    out = dict(walls=a.walls, steps=a.steps, dtype=a.dtype, cells=cells, batch_mode=batch.mode, batch_cfg=batch.cfg,
               batch_cfg_ms={str(k): round(v, 3) for k, v in cfg_times.items()},
               batch_seconds=round(wall_s, 3), batch_gpu_ms=round(gpu_ms, 1),
               batch_mlups=round(cells * a.steps / (gpu_ms * 1e-3) / 1e6, 1),
               batch_solves_per_hour=round(a.walls / wall_s * 3600, 1), setup_seconds=round(t_build, 1),
               hbm_gb=round(torch.cuda.max_memory_allocated() / 1e9, 2))
    del batch, members
    torch.cuda.empty_cache()
    if not a.no_plain:
        errs = []
        plain_s = 0.0
        for sp, bs in zip(specs, batch_stats):
            s = make_solver(sp, a.steps, "f32")
            s.autotune()
            torch.cuda.synchronize()
            t1 = time.time()
            s.advance(a.steps)
            torch.cuda.synchronize()
            plain_s += time.time() - t1
            ps = wall_stats(s)
            errs.append(dict(i=sp["i"], H=sp["H"], porosity=round(sp["porosity"], 3), Cd=rel(bs["Cd"], ps["Cd"]),
                             CdMax=rel(bs["CdMax"], ps["CdMax"]), CmMax=rel(bs["CmMax"], ps["CmMax"])))
            del s
            torch.cuda.empty_cache()
        out.update(plain_seconds=round(plain_s, 3), plain_solves_per_hour=round(a.walls / plain_s * 3600, 1),
                   solves_per_hour_ratio=round(plain_s / wall_s, 3),
                   cd_rel_err_max=max(e["Cd"] for e in errs), cd_peak_rel_err_max=max(e["CdMax"] for e in errs),
                   cm_peak_rel_err_max=max(e["CmMax"] for e in errs),
                   cd_rel_err_median=float(np.median([e["Cd"] for e in errs])),
                   per_wall=[{k: (round(v, 6) if isinstance(v, float) else v) for k, v in e.items()} for e in errs])
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    main()
