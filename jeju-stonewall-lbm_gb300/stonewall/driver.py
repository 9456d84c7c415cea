"""Command-line driver with the flags and outputs of stonewall3d/lbm3d.py main() (lbm3d.py:241-428).

    python lbm3d.py --case p20 --porosity 0.2                  # H=40, GPU
    python lbm3d.py --case quick --porosity 0.2 --H 16 --t-spinup 2 --t-avg 2 --out quick

Writes <out>/<case>.npz with the reference's keys (Cd, Cl, Cm, fx_profile, the
mean-field cuts, mean3d_ds2, the wall cuts, meta) and resumable checkpoints in
<out>/<case>.ckpt/ (same files and signature rule as lbm3d.py:322-355).

Differences, all opt-in except the last:
  --dtype f32|f64|f16|bf16   storage of the populations (f32 = the reference)
  --geom course|ellipsoid    the reference's course-stacked wall, or ellipsoid packing
  --inlet clip3H|powerlaw-H  the reference's profile, or u = U0 (z/H)^(1/7) without clipping
  --noise-dist uniform|gauss
  --nz-extra                 cells added to height*H for nz (the reference adds 1)
  Snapshots are taken as lbm3d.py:363-377 takes them: every snap_every steps
  after the spin-up the macro field of the state, its y = y_mid and z = z_half
  planes (float16) and, every snap3d_every-th snapshot, a Q-criterion frame
  max-pooled over ds^3 blocks and log-quantised to uint8 -- all on the GPU
  (sw_slice_xz, sw_slice_xy, sw_qcoarse); they travel in the checkpoints.
"""
import argparse
import json
import os
import shutil
import sys
import time

import numpy as np


def parse(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--case", required=True, help="output name, e.g. solid / p20 / p40")
    ap.add_argument("--porosity", type=float, required=True, help="frontal open-area fraction of the wall")
    ap.add_argument("--H", type=int, default=40, help="wall height in cells (resolution)")
    ap.add_argument("--device", default="cuda", help="cuda / cuda:0 (no CPU path)")
    ap.add_argument("--seed", type=int, default=7, help="stone layout seed")
    ap.add_argument("--Re", type=float, default=15000, help="Reynolds number U_H*H/nu")
    ap.add_argument("--U0", type=float, default=0.08, help="free-stream speed (lattice units)")
    ap.add_argument("--Cs", type=float, default=0.16, help="Smagorinsky constant")
    ap.add_argument("--up", type=float, default=4, help="domain length upstream of the wall [H]")
    ap.add_argument("--down", type=float, default=16, help="domain length downstream of the wall [H]")
    ap.add_argument("--span", type=float, default=4, help="domain width along the wall (periodic) [H]")
    ap.add_argument("--height", type=float, default=8, help="domain height [H]")
    ap.add_argument("--thick", type=float, default=0.3, help="wall thickness [H]")
    ap.add_argument("--t-spinup", type=float, default=20, help="spin-up time before averaging [H/U_H]")
    ap.add_argument("--t-avg", type=float, default=30, help="averaging / recording time [H/U_H]")
    ap.add_argument("--snap-dt", type=float, default=0.25, help="animation snapshot interval [H/U_H]")
    ap.add_argument("--snap3d-every", type=int, default=2,
                    help="save a 3D Q-criterion frame every N-th snapshot (0 = off)")
    ap.add_argument("--snap3d-ds", type=int, default=0, help="3D frame downsampling (0 = auto, about 13 voxels per H)")
    ap.add_argument("--out", default="results", help="output directory")
    ap.add_argument("--ckpt-every", type=int, default=5000, help="checkpoint every N steps (0 = off)")
    ap.add_argument("--no-resume", action="store_true", help="ignore an existing checkpoint")
    ap.add_argument("--dtype", default="f32", help="population storage: f32, f64, f16, bf16")
    ap.add_argument("--geom", default="course", choices=["course", "ellipsoid"])
    ap.add_argument("--inlet", default="clip3H", choices=["clip3H", "powerlaw-H"])
    ap.add_argument("--noise-dist", default="uniform", choices=["uniform", "gauss"])
    ap.add_argument("--nz-extra", type=int, default=1, help="nz = height*H + nz_extra")
    ap.add_argument("--chunk", type=int, default=50, help="steps per replayed CUDA graph")
    return ap.parse_args(argv)


def derive(a):
    """Grid and physics from the flags (lbm3d.py:269-282, plus the opt-in variants)."""
    from .params import reference_params
    p = reference_params(H=a.H, Re=a.Re, U0=a.U0, Cs=a.Cs, up=a.up, down=a.down, span=a.span, height=a.height,
                         thick=a.thick, t_spinup=a.t_spinup, t_avg=a.t_avg, snap_dt=a.snap_dt)
    if a.nz_extra != 1 or a.inlet != "clip3H":
        nz = int(round(a.height * a.H)) + a.nz_extra
        zeta = np.arange(nz) - 0.5
        if a.inlet == "clip3H":
            uin = (a.U0 * np.clip(zeta / (3.0 * a.H), 0, 1) ** (1 / 7)).astype(np.float32)
        else:
            uin = (a.U0 * np.clip(zeta / a.H, 0, None) ** (1 / 7)).astype(np.float32)
            p.UH = float(a.U0)
            p.nu0 = p.UH * a.H / a.Re
            p.t_unit = a.H / p.UH
            p.n_spin, p.n_avg = int(a.t_spinup * p.t_unit), int(a.t_avg * p.t_unit)
            p.snap_every = max(1, int(round(a.snap_dt * p.t_unit)))
        uin[0] = 0.0
        p.nz, p.uin = nz, uin
    return p


def main(argv=None):
    a = parse(argv)
    import torch
    from .geometry import course_wall, ellipsoid_wall
    from .metrics import coefficients, fx_profile
    from .params import flags_from_wall
    from .solver import Diverged, WallSolver

    if not a.device.startswith("cuda") or not torch.cuda.is_available():
        raise SystemExit("this solver runs on a CUDA GPU only (no CPU path)")
    dev = torch.device(a.device)
    if dev.index is not None:
        torch.cuda.set_device(dev)
    p = derive(a)
    H, nx, ny, nz, X0, T = p.H, p.nx, p.ny, p.nz, p.X0, p.T
    print(f"[grid] {nx}x{ny}x{nz} = {nx*ny*nz/1e6:.1f} M cells | U_H={p.UH:.4f} nu={p.nu0:.2e} "
          f"tau0={3*p.nu0+0.5:.5f} Re={a.Re:.0f} steps={p.n_total} (H/U = {p.t_unit:.0f} steps) dtype={a.dtype}",
          flush=True)
    if a.geom == "course":
        wall, phi = course_wall(a.porosity, H, nx, ny, nz, X0, T, seed=a.seed, verbose=True)
    else:
        wall, phi = ellipsoid_wall(a.porosity, H, nx, ny, nz, X0, T, seed=a.seed, verbose=True)
    flag = flags_from_wall(wall, nx, ny, nz)
    solver = WallSolver(flag, p.uin, p.nu0, a.Cs, p.x_sponge, p.n_total, n_spin=p.n_spin, nu_sponge=p.nu_sponge,
                        dtype=a.dtype, device=a.device, chunk=a.chunk)
    ds3 = a.snap3d_ds if a.snap3d_ds > 0 else max(1, int(round(H / 13)))
    y_mid, z_half = ny // 2, int(round(0.5 * H)) + 1
    q_x0 = max(1, X0 - int(round(0.5 * H)))
    q_dims = (min(int(round(9.0 * H)), nx - 1 - q_x0) // ds3, ny // ds3, min(int(round(2.5 * H)), nz - 1) // ds3)
    q_scale, QMAX = (H / p.UH) ** 2, 400.0
    snaps_xz, snaps_xy, snaps_q = [], [], []
    os.makedirs(a.out, exist_ok=True)
    ckpt = os.path.join(a.out, f"{a.case}.ckpt")
    sig = dict(grid=[nx, ny, nz], H=H, porosity=a.porosity, seed=a.seed, Re=a.Re, U0=a.U0, Cs=a.Cs,
               n_spin=p.n_spin, n_total=p.n_total, snap_every=p.snap_every, snap3d=[a.snap3d_every, ds3])
    if a.dtype != "f32" or a.geom != "course" or a.inlet != "clip3H" or a.noise_dist != "uniform" or a.nz_extra != 1:
        sig.update(dtype=a.dtype, geom=a.geom, inlet=a.inlet, noise=a.noise_dist, nz_extra=a.nz_extra)
    if os.path.isdir(ckpt) and not a.no_resume:
        try:
            solver.load_checkpoint(ckpt, sig)
        except ValueError:
            raise SystemExit(f"[{a.case}] checkpoint {ckpt} was made with different settings; "
                             f"use the same options, or --no-resume to start over")
        snaps_xz = list(np.load(os.path.join(ckpt, "snaps_xz.npy")))
        snaps_xy = list(np.load(os.path.join(ckpt, "snaps_xy.npy")))
        snaps_q = list(np.load(os.path.join(ckpt, "snaps_q.npy")))
        print(f"[{a.case}] resumed from step {solver.t} ({solver.t/p.t_unit:.1f} H/U)", flush=True)
    else:
        solver.init(noise=0.02, seed=a.seed, noise_kind=a.noise_dist)
    # launch configuration for this grid and storage type (times each one on the spare lattice;
    # the state and the results do not change)
    cfg, _ = solver.autotune()
    print(f"[{a.case}] step launch configuration {cfg}", flush=True)

    t0 = time.time()
    t_start = solver.t
    every = a.ckpt_every if a.ckpt_every > 0 else p.n_total
    snap0 = p.n_spin + 1                       # the state after step n_spin is the first snapshot

    def next_snap(t):
        return snap0 if t < snap0 else snap0 + ((t - snap0) // p.snap_every + 1) * p.snap_every

    while solver.t < p.n_total:
        nxt = min(p.n_total, (solver.t // 1000 + 1) * 1000, next_snap(solver.t))
        if a.ckpt_every > 0:
            nxt = min(nxt, (solver.t // every + 1) * every)
        solver.advance(nxt - solver.t)
        t = solver.t
        k = t - snap0
        if k >= 0 and k % p.snap_every == 0:                       # lbm3d.py:363-377
            xz, xy = solver.snapshot(y_mid, z_half)
            snaps_xz.append(xz)
            snaps_xy.append(xy)
            if a.snap3d_every > 0 and (k // p.snap_every) % a.snap3d_every == 0:
                snaps_q.append(solver.q_frame(q_x0, ds3, q_dims, q_scale, QMAX, macro_ready=True))
        if a.ckpt_every > 0 and t % a.ckpt_every == 0 and t < p.n_total:
            solver.save_checkpoint(ckpt, sig, extra=dict(
                snaps_xz=np.array(snaps_xz), snaps_xy=np.array(snaps_xy),
                snaps_q=np.array(snaps_q, dtype=np.uint8).reshape(-1, *q_dims)), background=True)
            print(f"[{a.case}] checkpoint at step {t} taken (written in the background)", flush=True)
        if t % 1000 == 0 or t == p.n_total:
            torch.cuda.synchronize()
            el = time.time() - t0
            done = t - t_start
            mlups = done * nx * ny * nz / max(el, 1e-9) / 1e6
            chk = ""
            if t % 5000 == 0 or t == p.n_total:
                try:
                    solver.check_finite()
                except Diverged:
                    raise SystemExit(f"[{a.case}] diverged at step {t}")
                u = solver.macro()
                chk = f" rho[{u[0].min():.3f},{u[0].max():.3f}] |u|max/U_H={np.abs(u[1:]).max()/p.UH:.2f}"
            print(f"[{a.case}] step {t}/{p.n_total}  t={t/p.t_unit:.1f} H/U  {mlups:.0f} MLUPS  "
                  f"eta {el/max(done,1)*(p.n_total-t)/60:.1f} min{chk}", flush=True)

    solver.wait_checkpoint()
    fh = solver.force_series()
    co = coefficients(fh, p.UH, H, ny, p.zeta)
    mean = solver.mean_field()
    np.savez_compressed(
        os.path.join(a.out, f"{a.case}.npz"),
        Cd=co["Cd"].astype(np.float32), Cl=co["Cl"].astype(np.float32), Cm=co["Cm"].astype(np.float32),
        fx_profile=fx_profile(fh, p.UH, ny, p.n_spin).astype(np.float32),
        mean_xz_mid=mean[:, :, y_mid, :].astype(np.float32),
        mean_xz_spanavg=np.where(wall.any(1)[None], np.nan, mean.mean(2)).astype(np.float32),
        mean_xy_half=mean[:, :, :, z_half].astype(np.float32),
        mean3d_ds2=mean[1:, ::2, ::2, ::2].astype(np.float16),
        snaps_xz=np.array(snaps_xz), snaps_xy=np.array(snaps_xy),
        wall_xz=wall[:, y_mid, :], wall_xy=wall[:, :, z_half], wall_front=wall.any(0), wall_top=wall.any(2),
        wall_ds2=wall[::2, ::2, ::2],
        snaps_q=np.array(snaps_q, dtype=np.uint8).reshape(-1, *q_dims),
        meta=json.dumps(dict(case=a.case, porosity_target=a.porosity, porosity=float(phi), H=H, T=T, X0=X0,
                             q3d=dict(x0=q_x0, ds=ds3, dims=list(q_dims), qmax=QMAX,
                                      every=a.snap3d_every * p.snap_every),
                             nx=nx, ny=ny, nz=nz, UH=p.UH, U0=a.U0, Re=a.Re, nu=p.nu0, Cs=a.Cs,
                             n_spin=p.n_spin, n_avg=p.n_avg, steps_per_unit=p.t_unit, snap_every=p.snap_every,
                             y_mid=y_mid, z_half=z_half, seed=a.seed, device=a.device,
                             wall_seconds=time.time() - t0, dtype=a.dtype, geom=a.geom, inlet=a.inlet,
                             noise=a.noise_dist)))
    s = slice(p.n_spin, None)
    Cd, Cm = co["Cd"][s], co["Cm"][s]
    print(f"[{a.case}] done. porosity={phi:.3f}  Cd mean={Cd.mean():.3f} max={Cd.max():.3f}  "
          f"Cm mean={Cm.mean():.3f}", flush=True)
    if os.path.isdir(ckpt):
        shutil.rmtree(ckpt)
    return 0


if __name__ == "__main__":
    sys.exit(main())
