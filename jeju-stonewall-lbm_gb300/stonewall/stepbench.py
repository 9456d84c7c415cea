"""Step-kernel timings on one wall, CUDA events around back-to-back launches.

    python -m stonewall.stepbench [--H 40] [--porosity 0.2] [--seed 1] [--dtype f16]
                                  [--cfgs 3,10,15] [--reps 20] [--aa] [--ground-only]

The wall is the bench's headline case by default (H = 40: 800 x 160 x 160, the
ellipsoid-packed wall, porosity 0.2, seed 1).  For every launch configuration
of the two-lattice step (lbm3d.py:57-155) given, or every one the storage type
supports, it times plain steps and accumulating steps (the float64 mean-field
sums of lbm3d.py:367-369 fused in) with the force series on, each state
stepped from the other lattice so nothing drifts.  --aa also times the
in-place AA steps, odd and even apart.  --ground-only removes the stones (the
ground stays), which shows what the wall's segments cost.  One JSON line:
milliseconds per step.
"""
import argparse
import json

import numpy as np
import torch

from . import _native as N
from .fields import Accum, Flags, ForceSeries, Grid, Lattice, StatusWord
from .geometry import ellipsoid_wall
from .kernels import DeviceVector, k_init, k_step, k_step_aa
from .params import baseline_params, flags_from_wall


def _time(fn, reps, warm=3):
    for _ in range(warm):
        fn()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    for _ in range(reps):
        fn()
    e1.record()
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--H", type=int, default=40)
    ap.add_argument("--porosity", type=float, default=0.2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--dtype", default="f16", choices=["f32", "f64", "f16", "bf16"])
    ap.add_argument("--cfgs", default=None, help="comma-separated launch configurations (default: all supported)")
    ap.add_argument("--reps", type=int, default=20)
    ap.add_argument("--aa", action="store_true", help="also time the in-place AA steps")
    ap.add_argument("--ground-only", action="store_true", help="remove the stones, keep the ground")
    a = ap.parse_args(argv)

    p = baseline_params(a.H, 1000)
    wall, _ = ellipsoid_wall(a.porosity, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=a.seed)
    flag = flags_from_wall(wall, p.nx, p.ny, p.nz)
    if a.ground_only:
        flag[:, :, 1:] = 0
    g = Grid(p.nx, p.ny, p.nz)
    fl, uv = Flags(g, flag), DeviceVector(p.uin)
    code = N.dtype_code(a.dtype)
    L = N.lib()
    if a.cfgs:
        cfgs = [int(c) for c in a.cfgs.split(",")]
    else:
        cfgs = [c for c in range(L.sw_step_config_count()) if c < 4 or code in (N.SW_F16_SHIFT, N.SW_BF16_SHIFT)]
    f = [Lattice(g, a.dtype), Lattice(g, a.dtype).zero_()]
    k_init(f[0], fl, uv, 0.02, a.seed, "gauss")
    acc, force, status = Accum(g), ForceSeries(2, g.nz), StatusWord()
    out = dict(grid=[g.nx, g.ny, g.nz], dtype=a.dtype, ground_only=a.ground_only, tiles=fl.tile_counts(), ms={})
    for cfg in cfgs:
        for accum in (False, True):
            def go():
                k_step(f[0], f[1], fl, uv, g.nx, g.ny, g.nz, p.nu0, p.Cs, p.x_sponge, 0.05, force, 1,
                       acc=acc if accum else None, status=status, cfg=cfg)
                f[0], f[1] = f[1], f[0]
            out["ms"][f"{cfg}{'a' if accum else ''}"] = round(_time(go, 2 * a.reps), 4)
    if a.aa:
        ghost = torch.empty(L.sw_aa_ghost_elems(g.gp) * N.DTYPE_BYTES[code], dtype=torch.uint8, device="cuda")
        fa = Lattice(g, a.dtype)
        k_init(fa, fl, uv, 0.02, a.seed, "gauss")
        for accum in (False, True):
            ev = [torch.cuda.Event(enable_timing=True) for _ in range(2 * a.reps + 1)]
            steps = [lambda t=t: k_step_aa(fa, t % 2 == 0, fl, uv, p.nu0, p.Cs, p.x_sponge, 0.05, force, 1,
                                           ghost=ghost, acc=acc if accum else None, status=status)
                     for t in range(2)]
            for t in range(4):
                steps[t % 2]()
            torch.cuda.synchronize()
            ev[0].record()
            for t in range(2 * a.reps):
                steps[t % 2]()
                ev[t + 1].record()
            torch.cuda.synchronize()
            dt = [ev[t].elapsed_time(ev[t + 1]) for t in range(2 * a.reps)]
            tag = "a" if accum else ""
            out["ms"][f"aa_odd{tag}"] = round(float(np.mean(dt[0::2])), 4)
            out["ms"][f"aa_even{tag}"] = round(float(np.mean(dt[1::2])), 4)
    word = status.read()
    if word:
        raise SystemExit(f"status word {word:#x} after the timed steps")
    print(json.dumps(out))


if __name__ == "__main__":
    main()
