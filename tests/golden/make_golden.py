"""Generate the golden fixtures in tests/golden/ by running the reference itself.

    python tests/golden/make_golden.py --ref <reference checkout>   (or STONEWALL_REFERENCE=<path>)

Needs the reference sources (stonewall3d/lbm3d.py, stonewall3d/geometry.py); the
fixtures it writes are committed, so nothing else needs the sources.  lbm3d.py
imports NVIDIA Warp, which is not installed; _warp_standin.py is installed as
``warp`` and runs the reference's kernel bodies thread by thread in float32
(see that module for what it does and does not reproduce of Warp).

Fixtures:
  tables.npz        C, W, OPP, MIRZ exactly as lbm3d.py:20-28 builds them
  step_box.npz      16x6x9 grid, a stone block + a lone stone next to the top
                    and the periodic edge, ground, inlet, outlet, sponge:
                    k_init then 4 ping-pong k_step, k_macro and k_accum
  step_rand.npz     12x5x7 grid, random stones plus interior GROUND cells,
                    3 steps with a different viscosity / Cs / sponge
  step_edge.npz     9x1x3 grid: the span one cell wide (y wraps onto itself),
                    stones in the top and outlet planes, sponge over half the grid
  driver_small.npz  lbm3d.main() end to end on a 32x8x13 grid (H=4, 10 steps,
                    snapshots, a checkpoint, Q-criterion frames); the .npz the
                    reference writes, unchanged, plus its argv
  driver_small_ckpt.npz  the checkpoint that run writes at step 5 (the
                    reference removes it when the run completes; kept here
                    by copying it just before): f, force, uacc, snaps_*, state
  geometry.npz      geometry.build_wall masks (bit-packed) and porosities
  postprocess.npz   the reference's Cd / Cm statistics of the driver case and its
                    reverse-flow area of a seeded mean field
"""
import argparse
import json
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load_reference(ref):
    sys.path.insert(0, HERE)
    import _warp_standin
    sys.modules["warp"] = _warp_standin
    sys.path.insert(0, os.path.join(ref, "stonewall3d"))
    import lbm3d
    import geometry
    return lbm3d, geometry, _warp_standin


def run_steps(lbm3d, wp, flag, uin, nu0, cs, x_sponge, nu_sponge, n_steps, noise, seed):
    nx, ny, nz = flag.shape
    Q = 19
    f0 = wp.zeros((Q, nx, ny, nz), dtype=float)
    f1 = wp.zeros((Q, nx, ny, nz), dtype=float)
    flag_d = wp.array(flag, dtype=wp.uint8)
    uin_d = wp.array(uin, dtype=float)
    cx, cy, cz = (wp.array(np.ascontiguousarray(lbm3d.C[:, k]), dtype=wp.int32) for k in range(3))
    w_d = wp.array(lbm3d.W, dtype=float)
    opp_d = wp.array(lbm3d.OPP, dtype=wp.int32)
    mirz_d = wp.array(lbm3d.MIRZ, dtype=wp.int32)
    force = np.zeros((n_steps, nz, 2), np.float64)          # float64 target: see _warp_standin
    wp.launch(lbm3d.k_init, dim=(nx, ny, nz), inputs=[f0, flag_d, uin_d, cx, cy, cz, w_d, noise, seed])
    out = dict(flag=flag, uin=uin, f_init=f0.numpy(),
               params=np.array([nu0, cs, x_sponge, nu_sponge, noise, seed, n_steps], np.float64))
    for t in range(n_steps):
        wp.launch(lbm3d.k_step, dim=(nx, ny, nz),
                  inputs=[f0, f1, flag_d, uin_d, cx, cy, cz, w_d, opp_d, mirz_d,
                          nx, ny, nz, nu0, cs, x_sponge, nu_sponge, force, t])
        f0, f1 = f1, f0
        out[f"f_step{t + 1}"] = f0.numpy()
        out[f"f_other{t + 1}"] = f1.numpy()               # the stale lattice (solid cells never written)
        print(f"  step {t + 1}/{n_steps}", flush=True)
    out["force"] = force
    U = wp.zeros((4, nx, ny, nz), dtype=float)
    wp.launch(lbm3d.k_macro, dim=(nx, ny, nz), inputs=[f0, flag_d, cx, cy, cz, U])
    Uacc = wp.zeros((4, nx, ny, nz), dtype=float)
    wp.launch(lbm3d.k_accum, dim=(4, nx, ny, nz), inputs=[U, Uacc])
    wp.launch(lbm3d.k_accum, dim=(4, nx, ny, nz), inputs=[U, Uacc])
    out["macro"] = U.numpy()
    out["accum2"] = Uacc.numpy()
    return out


def inlet_profile(nz, H, U0):
    """Same formula as lbm3d.py:272-275 (used only to make realistic fixture inputs)."""
    zeta = np.arange(nz) - 0.5
    uin = (U0 * np.clip(zeta / (3.0 * H), 0, 1) ** (1 / 7)).astype(np.float32)
    uin[0] = 0.0
    return uin


def write_postprocess(out, driver_npz):
    """postprocess.npz: the reference's own Cd / Cm statistics (postprocess.py:46-83, on the driver
    case's .npz) and reverse-flow area (export3d.py:169-184, on a seeded mean field with a
    reverse-flow pocket behind a block of stones).  export3d.py imports scikit-image for its
    meshes, which is not installed: a stand-in marching_cubes returns a one-triangle mesh, which
    the area does not use."""
    import types
    import postprocess
    m, payload, _ = postprocess.case_payload(driver_npz)
    meas = types.ModuleType("skimage.measure")
    meas.marching_cubes = lambda vol, level: (np.zeros((3, 3)), np.array([[0, 1, 2]]), None, None)
    sk = types.ModuleType("skimage")
    sk.measure = meas
    sys.modules.setdefault("skimage", sk)
    sys.modules.setdefault("skimage.measure", meas)
    import export3d
    rng = np.random.default_rng(3)
    H, X0, nx, ny, nz, UH = 8, 40, 160, 32, 33, 0.05
    ux = rng.normal(0.03, 0.01, (3, nx // 2, ny // 2, (nz + 1) // 2)).astype(np.float16)
    ux[0, 22:36, 3:12, 1:6] = -0.01                               # the pocket
    wall = np.zeros((nx // 2, ny // 2, (nz + 1) // 2), bool)
    wall[20:23, :, 1:4] = True
    z = export3d.reverse_zone(dict(mean3d_ds2=ux, wall_ds2=wall), dict(H=H, X0=X0, UH=UH, ny=ny, nx=nx, nz=nz))
    np.savez_compressed(os.path.join(out, "postprocess.npz"), stats=np.array(json.dumps(payload["stats"])),
                        n_spin=np.array(m["n_spin"]), ux_ds2=ux, wall_ds2=wall,
                        params=np.array([H, X0, nx, ny, nz, UH]), area=np.array(z["area"]))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=os.environ.get("STONEWALL_REFERENCE"),
                    help="checkout of the reference repository (default: $STONEWALL_REFERENCE)")
    ap.add_argument("--out", default=HERE)
    ap.add_argument("--only", default="", help="comma-separated fixture names to (re)write (default: all)")
    a = ap.parse_args()
    if not a.ref:
        ap.error("give the reference checkout with --ref or STONEWALL_REFERENCE")
    lbm3d, geometry, wp = load_reference(a.ref)
    only = set(v for v in a.only.split(",") if v)

    def wanted(name):
        return not only or name in only

    if wanted("tables"):
        np.savez_compressed(os.path.join(a.out, "tables.npz"), C=lbm3d.C, W=lbm3d.W, OPP=lbm3d.OPP,
                        MIRZ=lbm3d.MIRZ, flags=np.array([lbm3d.FLUID, lbm3d.WALL, lbm3d.GROUND]))

    # case 1: a stone block, a lone stone beside the top and the periodic edge
    print("step_box", flush=True)
    nx, ny, nz = 16, 6, 9
    flag = np.zeros((nx, ny, nz), np.uint8)
    flag[6:8, 1:4, 1:5] = lbm3d.WALL
    flag[10, 5, nz - 2] = lbm3d.WALL
    flag[13, 0, 3] = lbm3d.WALL
    flag[:, :, 0] = lbm3d.GROUND
    uin = inlet_profile(nz, 3, 0.08)
    out = run_steps(lbm3d, wp, flag, uin, nu0=np.float32(0.002), cs=0.1, x_sponge=11, nu_sponge=0.05,
                    n_steps=4, noise=0.02, seed=3)
    if wanted("step_box"):
        np.savez_compressed(os.path.join(a.out, "step_box.npz"), **out)

    # case 2: random stones and interior GROUND cells (bounce-back without force)
    print("step_rand", flush=True)
    nx, ny, nz = 12, 5, 7
    rng = np.random.default_rng(11)
    flag = np.zeros((nx, ny, nz), np.uint8)
    sub = rng.random((8, ny, 5)) < 0.2
    flag[2:10, :, 1:6][sub] = lbm3d.WALL
    flag[4, 2, 5] = lbm3d.GROUND
    flag[9, 4, 2] = lbm3d.GROUND
    flag[:, :, 0] = lbm3d.GROUND
    flag[0, 1, 3] = lbm3d.WALL                                # a stone in the inlet plane
    flag[nx - 1, 3, 4] = lbm3d.WALL                           # and one in the outlet plane
    uin = inlet_profile(nz, 2, 0.06)
    out = run_steps(lbm3d, wp, flag, uin, nu0=0.01, cs=0.16, x_sponge=8, nu_sponge=0.05,
                    n_steps=3, noise=0.05, seed=5)
    if wanted("step_rand"):
        np.savez_compressed(os.path.join(a.out, "step_rand.npz"), **out)

    # case 2b: edges -- a one-cell-wide periodic span (y wraps onto itself), two fluid levels
    # under the free-slip top, a stone in the top plane and one in the outlet plane, the
    # reference's default Cs, the sponge covering half the domain
    print("step_edge", flush=True)
    nx, ny, nz = 9, 1, 3
    flag = np.zeros((nx, ny, nz), np.uint8)
    flag[:, :, 0] = lbm3d.GROUND
    flag[4, 0, 2] = lbm3d.WALL
    flag[nx - 1, 0, 1] = lbm3d.WALL
    uin = inlet_profile(nz, 1, 0.05)
    out = run_steps(lbm3d, wp, flag, uin, nu0=0.002, cs=0.16, x_sponge=4, nu_sponge=0.05,
                    n_steps=3, noise=0.04, seed=9)
    if wanted("step_edge"):
        np.savez_compressed(os.path.join(a.out, "step_edge.npz"), **out)

    # case 3: the reference driver end to end
    print("driver_small", flush=True)
    tmp = tempfile.mkdtemp()
    argv = ["lbm3d.py", "--case", "g", "--porosity", "0.2", "--H", "4", "--up", "2", "--down", "6",
            "--span", "2", "--height", "3", "--t-spinup", "0.1", "--t-avg", "0.1", "--snap-dt", "0.05",
            "--ckpt-every", "5", "--device", "cpu", "--out", tmp]
    old = sys.argv
    sys.argv = argv
    kept, rmtree = {}, shutil.rmtree

    def keep_then_remove(path, *args, **kw):        # the finished run removes its checkpoint: copy it first
        if os.path.basename(path) == "g.ckpt" and os.path.isdir(path):
            kept["g.ckpt"] = shutil.copytree(path, os.path.join(tempfile.mkdtemp(), "g.ckpt"))
        return rmtree(path, *args, **kw)
    lbm3d.shutil.rmtree = keep_then_remove
    try:
        lbm3d.main()
    finally:
        sys.argv = old
        lbm3d.shutil.rmtree = rmtree
    d = dict(np.load(os.path.join(tmp, "g.npz")))
    d["argv"] = np.array(json.dumps(argv[1:-2]))
    if wanted("driver_small"):
        np.savez_compressed(os.path.join(a.out, "driver_small.npz"), **d)
    if wanted("postprocess"):
        write_postprocess(a.out, os.path.join(tmp, "g.npz"))
    if wanted("driver_small_ckpt"):
        ck = kept["g.ckpt"]
        c = {k: np.load(os.path.join(ck, k + ".npy")) for k in ("f", "force", "uacc", "snaps_xz", "snaps_xy",
                                                                 "snaps_q")}
        with open(os.path.join(ck, "state.json")) as fh:
            c["state"] = np.array(fh.read())
        np.savez_compressed(os.path.join(a.out, "driver_small_ckpt.npz"), **c)
    shutil.rmtree(tmp)

    # geometry: the reference's mask producer
    print("geometry", flush=True)
    g = {}
    specs = [(0.0, 8, 7), (0.2, 8, 7), (0.4, 8, 7), (0.2, 16, 7), (0.4, 12, 3), (0.0, 12, 1)]
    for k, (por, H, seed) in enumerate(specs):
        nx, ny, nz = 20 * H, 4 * H, 8 * H + 1
        X0, T = 4 * H, max(2, int(round(0.3 * H)))
        m, phi = geometry.build_wall(por, H, nx, ny, nz, X0, T, seed=seed, verbose=False)
        g[f"mask{k}"] = np.packbits(m.ravel())
        g[f"spec{k}"] = np.array([por, H, seed, nx, ny, nz, X0, T, phi], np.float64)
    g["n"] = np.array(len(specs))
    if wanted("geometry"):
        np.savez_compressed(os.path.join(a.out, "geometry.npz"), **g)
    print("done", flush=True)


if __name__ == "__main__":
    main()
