"""Storage-precision study: one wall solved with each storage type, compared with float64.

    python -m stonewall.study --H 64 --porosity 0.3 --seed 0 --steps 20000 --dtypes f64,f32,f16,bf16
    python -m stonewall.study --H 40 --porosity 0,0.2,0.4 --seed 0,1,2 --steps 40000 --dtypes f64,f32,f16

For every (porosity, seed) wall -- an ellipsoid-packed stone wall in a
20H x 4H x 4H domain (stonewall.params.baseline_params: Re_H = 1e4, Cs = 0.1,
inlet 0.05 (z/H)^(1/7), 2 % Gaussian initial noise) -- each storage type runs
the same fused step from the same initial state for the same number of steps
(spin-up as in baseline_params).  Per run: mean and peak Cd, force RMS (the
std of Cd), mean and peak overturning moment Cm, the recirculation area of the
mean field (export3d.py:169-184 on the every-2nd-cell mean field), MLUPS
(CUDA events around the solve); per storage type other than float64, the
relative error of each against the float64-storage run of the same kernel.

The flow behind the wall is turbulent, so two runs that differ in the last
bit of the initial state end with different (equally valid) histories, and
their statistics differ by the sampling error of the averaging window.
--floor f32 measures that floor: the same storage type again from an initial
state with a different noise seed (same mask), and its relative difference to
the first run.  Precision errors are only resolved above that floor.
Prints one JSON line.
"""
import argparse
import json
import time

import numpy as np
import torch

from .geometry import ellipsoid_wall
from .metrics import coefficients, device_recirculation_area, stats
from .params import baseline_params, flags_from_wall
from .solver import WallSolver

KEYS = ("Cd", "CdMax", "CdStd", "Cm", "CmMax", "recirc")


def solve(p, flag, dtype, seed, steps, noise_seed=None):
    s = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, steps, n_spin=p.n_spin, dtype=dtype)
    s.init(noise=0.02, seed=seed if noise_seed is None else noise_seed, noise_kind="gauss")
    s.autotune()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    s.run()
    e1.record()
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    co = coefficients(s.force_series(), p.UH, p.H, p.ny)
    st = stats(co["Cd"], co["Cm"], co["Cl"], p.n_spin)
    st["recirc"] = device_recirculation_area(s.acc, s.n_acc, s.flags, p.H, p.X0, p.UH)
    st["mlups"] = s.grid.cells * steps / (ms * 1e-3) / 1e6
    st["seconds"] = ms * 1e-3
    del s
    torch.cuda.empty_cache()
    return st, co["Cd"]


def rel(a, b):
    return abs(a - b) / max(abs(b), 1e-12)


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--H", type=int, default=64)
    ap.add_argument("--porosity", default="0.3", help="comma-separated")
    ap.add_argument("--seed", default="0", help="comma-separated, one per porosity")
    ap.add_argument("--steps", type=int, default=20000)
    ap.add_argument("--dtypes", default="f64,f32,f16,bf16", help="the first is the reference")
    ap.add_argument("--floor", default="", help="storage types to run again from another initial noise seed")
    a = ap.parse_args(argv)
    pors = [float(v) for v in a.porosity.split(",")]
    seeds = [int(v) for v in a.seed.split(",")]
    if len(seeds) == 1:
        seeds = seeds * len(pors)
    dtypes = a.dtypes.split(",")
    out = dict(H=a.H, steps=a.steps, reference=dtypes[0], walls=[])
    for por, seed in zip(pors, seeds):
        p = baseline_params(a.H, a.steps)
        wall, frac = ellipsoid_wall(por, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=seed)
        flag = flags_from_wall(wall, p.nx, p.ny, p.nz)
        w = dict(porosity=por, seed=seed, grid=[p.nx, p.ny, p.nz], n_spin=p.n_spin, solid_fraction=float(frac),
                 runs={})
        series = {}
        for dt in dtypes:
            t0 = time.time()
            st, cd = solve(p, flag, dt, seed, a.steps)
            series[dt] = cd
            w["runs"][dt] = {k: (round(v, 6) if isinstance(v, float) else v) for k, v in st.items()}
            print(f"# H={a.H} porosity={por} seed={seed} {dt}: {time.time() - t0:.1f}s {json.dumps(w['runs'][dt])}",
                  flush=True)
        ref = w["runs"][dtypes[0]]
        w["rel_err"] = {dt: {k: float(f"{rel(w['runs'][dt][k], ref[k]):.3e}") for k in KEYS}
                        for dt in dtypes[1:]}
        for dt in dtypes[1:]:
            d = series[dt][p.n_spin:] - series[dtypes[0]][p.n_spin:]
            w["rel_err"][dt]["Cd_series_rms"] = float(f"{np.sqrt((d ** 2).mean()) / abs(ref['Cd']):.3e}")
        w["floor"] = {}
        for dt in [v for v in a.floor.split(",") if v]:
            st, _ = solve(p, flag, dt, seed, a.steps, noise_seed=seed + 1000)
            base = w["runs"][dt] if dt in w["runs"] else solve(p, flag, dt, seed, a.steps)[0]
            w["floor"][dt] = {k: float(f"{rel(st[k], base[k]):.3e}") for k in KEYS}
            print(f"# floor {dt}: {json.dumps(w['floor'][dt])}", flush=True)
        out["walls"].append(w)
    print(json.dumps(out), flush=True)
    return out


if __name__ == "__main__":
    main()
