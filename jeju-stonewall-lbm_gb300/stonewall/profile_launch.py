"""Three launches of one step kernel on one wall, for profilers (ncu -k ... -s 1 -c 1).

    python -m stonewall.profile_launch [--H 40] [--dtype f16] [--cfg 8] [--batch]

The wall is by default the 800 x 160 x 160 headline case (H = 40, ellipsoid
wall, porosity 0.2, seed 1, 2 % Gaussian initial noise).  Without --batch the
single-lattice step runs in launch configuration --cfg (sw_step_cfg); with
--batch the persistent batched kernel (stonewall.batch.Batch, this wall
alone) runs in that configuration.  Each launch steps the same state into the
spare lattice without forces or sums, so all three do identical work.
"""
import argparse

import torch

from . import _native as N
from .batch import Batch
from .geometry import ellipsoid_wall
from .params import baseline_params, flags_from_wall
from .solver import WallSolver


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--H", type=int, default=40)
    ap.add_argument("--porosity", type=float, default=0.2)
    ap.add_argument("--seed", type=int, default=1)
    ap.add_argument("--dtype", default="f16")
    ap.add_argument("--cfg", type=int, default=0)
    ap.add_argument("--batch", action="store_true", help="the persistent batched kernel instead")
    a = ap.parse_args(argv)
    p = baseline_params(a.H, 1000)
    wall, _ = ellipsoid_wall(a.porosity, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=a.seed)
    flag = flags_from_wall(wall, p.nx, p.ny, p.nz)
    s = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, 1000, n_spin=0, dtype=a.dtype)
    s.init(noise=0.02, seed=a.seed, noise_kind="gauss")
    if a.batch:
        b = Batch(dtype=a.dtype, chunk=10, cfg=a.cfg)
        b.add(s)
        b._fill(1, tuning=True)
        for _ in range(3):
            b._launch(0)
    else:
        L, g = N.lib(), s.grid
        for _ in range(3):
            N.check(L.sw_step_cfg(g.gp, s.dtype, s.f[0].ptr, s.f[1].ptr, s.flags.ptr, s.flags.tiles_ptr, s.uin.ptr,
                                  s.nu0, s.cs, s.x_sponge, s.nu_sponge, None, 0, None, a.cfg, None), "sw_step_cfg")
    torch.cuda.synchronize()
    print(f"ok: {a.dtype} cfg {a.cfg} {'batch' if a.batch else 'single'} {p.nx}x{p.ny}x{p.nz}", flush=True)


if __name__ == "__main__":
    main()
