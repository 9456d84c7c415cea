"""Wall-load coefficients, their statistics and the recirculation area.

coefficients():  lbm3d.py:396-407 -- Fx, Fz and the overturning moment about
                 the wall base from the per-level force series, normalised by
                 q_ref = U_H^2 / 2 and the frontal area H * ny.
stats():         postprocess.py:65-82 -- mean / peak / std of Cd (std is the
                 force RMS about the mean), mean / peak Cm, mean Cl over
                 t >= n_spin.  Computed in float64.
device_stats():  the same two steps on the GPU from the device force series
                 (sw_coefficients, sw_coef_stats): 48 bytes come back instead
                 of the whole series.
recirculation_area(): export3d.py:169-184 -- cells of the every-2nd-cell mean
                 field with u_x < 0 in [X0, X0 + 10H) x [0, 2H) after the
                 same masking and one 3-point box blur, times 8 / (H^2 ny).
device_recirculation_area(): the same from the device float64 sums
                 (sw_recirc_count): the box, blur and count on the GPU, 8 bytes
                 back instead of the mean field.
"""
import numpy as np


def coefficients(force, UH, H, ny, zeta=None):
    """force: (n, nz, 2) float64 -> dict of Cd, Cl, Cm (float64 arrays of length n)."""
    f = np.asarray(force, dtype=np.float64)
    nz = f.shape[1]
    zeta = np.arange(nz) - 0.5 if zeta is None else zeta
    qref = 0.5 * UH ** 2
    A = H * ny
    Fx = f[:, :, 0].sum(1)
    Fz = f[:, :, 1].sum(1)
    M = (f[:, :, 0] * zeta[None, :]).sum(1)
    return dict(Cd=Fx / (qref * A), Cl=Fz / (qref * A), Cm=M / (qref * A * H), Fx=Fx, Fz=Fz, M=M)


def stats(Cd, Cm, Cl, n_spin):
    Cd, Cm, Cl = (np.asarray(a, dtype=np.float64)[n_spin:] for a in (Cd, Cm, Cl))
    if len(Cd) == 0:
        return dict(Cd=float("nan"), CdMax=float("nan"), CdStd=float("nan"), Cm=float("nan"),
                    CmMax=float("nan"), Cl=float("nan"))
    return dict(Cd=float(Cd.mean()), CdMax=float(Cd.max()), CdStd=float(Cd.std()),
                Cm=float(Cm.mean()), CmMax=float(Cm.max()), Cl=float(Cl.mean()))


STAT_KEYS = ("Cd", "CdMax", "CdStd", "Cm", "CmMax", "Cl")


def device_coefficients(force, UH, H, ny, stream=None):
    """coefficients() on the GPU from a stonewall.fields.ForceSeries: a float64 CUDA tensor (3, n) of
    Cd, Cl, Cm."""
    import torch
    from . import _native as N
    from .fields import _ptr, _stream
    coef = torch.empty((3, force.n_steps), dtype=torch.float64, device=force.data.device)
    N.check(N.lib().sw_coefficients(force.ptr, force.n_steps, force.nz, float(UH), float(H), int(ny), _ptr(coef),
                                    _stream(stream)), "sw_coefficients")
    return coef


def device_stats(force, UH, H, ny, n_spin, stream=None):
    """stats(coefficients(...)) computed on the GPU; the same dict, 6 floats downloaded."""
    import torch
    from . import _native as N
    from .fields import _ptr, _stream
    coef = device_coefficients(force, UH, H, ny, stream)
    out = torch.empty(6, dtype=torch.float64, device=coef.device)
    N.check(N.lib().sw_coef_stats(_ptr(coef), force.n_steps, int(n_spin), _ptr(out), _stream(stream)),
            "sw_coef_stats")
    return dict(zip(STAT_KEYS, (float(v) for v in out.cpu().tolist())))


def device_recirculation_area(accum, n_acc, flags, H, X0, UH, stream=None):
    """recirculation_area() of the time-mean field on the GPU, from the float64 sums in a
    stonewall.fields.Accum (n_acc accumulated states) and the Flags of the same grid: the
    every-2nd-cell box, blur and count run on the device and 8 bytes come back.  Equal to
    recirculation_area(mean_ux[::2, ::2, ::2], (flag != 0)[::2, ::2, ::2], H, X0, UH, ny)."""
    import torch
    from . import _native as N
    from .fields import _ptr, _stream
    g = accum.grid
    L = N.lib()
    nbytes = L.sw_recirc_scratch_bytes(g.gp, int(H), int(X0))
    if nbytes < 0:
        raise ValueError(f"no recirculation box for H={H}, X0={X0} on {g.nx}x{g.ny}x{g.nz}")
    scratch = torch.empty(nbytes // 4, dtype=torch.float32, device=accum.data.device)
    count = torch.empty(1, dtype=torch.int64, device=accum.data.device)
    N.check(L.sw_recirc_count(g.gp, accum.ptr, int(n_acc), flags.ptr, int(H), int(X0), float(UH), _ptr(scratch),
                              nbytes, _ptr(count), _stream(stream)), "sw_recirc_count")
    return float(int(count.item()) * 8) / (H ** 2 * g.ny)


def fx_profile(force, UH, ny, n_spin):
    """Time-mean drag per level, lbm3d.py:408."""
    f = np.asarray(force, dtype=np.float64)
    return f[n_spin:, :, 0].mean(0) / (0.5 * UH ** 2 * ny)


def box_blur(a, n=1):
    """Separable 3-point box blur with edge padding, n passes (export3d.py:23-35)."""
    a = a.astype(np.float32)
    for _ in range(n):
        for ax in range(3):
            pad = [(1, 1) if i == ax else (0, 0) for i in range(3)]
            p = np.pad(a, pad, mode="edge")
            lo = [slice(None)] * 3
            mid = [slice(None)] * 3
            hi = [slice(None)] * 3
            lo[ax], mid[ax], hi[ax] = slice(0, -2), slice(1, -1), slice(2, None)
            a = (p[tuple(lo)] + p[tuple(mid)] + p[tuple(hi)]) / 3.0
    return a


def recirculation_area(mean3d_ds2_ux, wall_ds2, H, X0, UH, ny):
    """Reverse-flow area per unit wall length, in H^2 (export3d.py:169-184)."""
    ux = np.asarray(mean3d_ds2_ux).astype(np.float32)
    i0, i1 = X0 // 2, min(ux.shape[0], (X0 + 10 * H) // 2)
    k1 = min(ux.shape[2], int(2 * H) // 2)
    sub = np.where(wall_ds2[i0:i1, :, :k1], 0.05, ux[i0:i1, :, :k1]) / UH
    sub[:, :, 0] = sub[:, :, 1]
    sub = np.pad(box_blur(sub, 1), 1, constant_values=1.0)
    if sub.min() >= 0:
        return 0.0
    return float((sub[1:-1, 1:-1, 1:-1] < 0).sum() * 8) / (H ** 2 * ny)
