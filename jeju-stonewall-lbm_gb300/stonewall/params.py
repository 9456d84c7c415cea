"""Run parameters of a wall solve: grid, inlet profile, viscosity, step counts.

reference_params() derives them exactly as lbm3d.py:269-282 does from its
command-line flags (20H x 4H x (8H+1) domain, clipped 1/7 power law over 3H,
Re and U0 given).  baseline_params() derives the workload family used for
measurement: 20H x 4H x 4H, wall 0.75H thick at x = 5H, inlet
u(z) = U_H (z/H)^(1/7) without clipping (U_H = 0.05), Re_H = 1e4, Cs = 0.1, and
a fixed total step count; the spin-up is the reference's 20 H/U_H when the run
is long enough, else its first 40 %.
"""
from dataclasses import dataclass, field

import numpy as np


@dataclass
class RunParams:
    H: int
    nx: int
    ny: int
    nz: int
    X0: int                  # wall front (cells)
    T: int                   # wall thickness (cells)
    uin: np.ndarray          # float32 [nz] inlet speed per level
    UH: float                # reference speed at the wall top
    nu0: float
    Re: float
    U0: float
    Cs: float
    n_spin: int
    n_avg: int
    x_sponge: int
    nu_sponge: float = 0.05
    snap_every: int = 1
    t_unit: float = 1.0      # steps per H / U_H
    extra: dict = field(default_factory=dict)

    @property
    def n_total(self):
        return self.n_spin + self.n_avg

    @property
    def zeta(self):
        """Height of cell centres above the ground (lbm3d.py:272)."""
        return np.arange(self.nz) - 0.5

    @property
    def cells(self):
        return self.nx * self.ny * self.nz


def reference_params(H=40, Re=15000.0, U0=0.08, Cs=0.16, up=4.0, down=16.0, span=4.0, height=8.0, thick=0.3,
                     t_spinup=20.0, t_avg=30.0, snap_dt=0.25):
    """lbm3d.py:269-282 (flag defaults of lbm3d.py:245-258)."""
    nx, ny, nz = int(round((up + down) * H)), int(round(span * H)), int(round(height * H)) + 1
    X0, T = int(round(up * H)), max(2, int(round(thick * H)))
    zeta = np.arange(nz) - 0.5
    delta = 3.0 * H
    uin = (U0 * np.clip(zeta / delta, 0, 1) ** (1 / 7)).astype(np.float32)
    uin[0] = 0.0
    UH = float(U0 * (H / delta) ** (1 / 7))
    nu0 = UH * H / Re
    t_unit = H / UH
    n_spin, n_avg = int(t_spinup * t_unit), int(t_avg * t_unit)
    snap_every = max(1, int(round(snap_dt * t_unit)))
    x_sponge = int(nx - 3 * H)
    return RunParams(H=H, nx=nx, ny=ny, nz=nz, X0=X0, T=T, uin=uin, UH=UH, nu0=nu0, Re=Re, U0=U0, Cs=Cs,
                     n_spin=n_spin, n_avg=n_avg, x_sponge=x_sponge, snap_every=snap_every, t_unit=t_unit)


def baseline_params(H, n_total, Re=1e4, UH=0.05, Cs=0.1, up=5.0, down=15.0, span=4.0, height=4.0, thick=0.75):
    """The measured workload family: 20H x 4H x 4H, power-law inlet u = U_H (z/H)^(1/7)."""
    nx, ny, nz = int(round((up + down) * H)), int(round(span * H)), int(round(height * H))
    X0, T = int(round(up * H)), max(2, int(round(thick * H)))
    zeta = np.arange(nz) - 0.5
    uin = (UH * np.clip(zeta / H, 0, None) ** (1 / 7)).astype(np.float32)
    uin[0] = 0.0
    nu0 = UH * H / Re
    t_unit = H / UH
    n_spin = int(20 * t_unit) if n_total >= 2 * int(20 * t_unit) else int(0.4 * n_total)
    return RunParams(H=H, nx=nx, ny=ny, nz=nz, X0=X0, T=T, uin=uin, UH=UH, nu0=nu0, Re=Re, U0=UH, Cs=Cs,
                     n_spin=n_spin, n_avg=n_total - n_spin, x_sponge=int(nx - 3 * H), t_unit=t_unit)


def flags_from_wall(wall, nx, ny, nz):
    """uint8 flags: stones WALL, ground plane GROUND (lbm3d.py:288-290)."""
    flag = np.zeros((nx, ny, nz), np.uint8)
    flag[wall] = 1
    flag[:, :, 0] = 2
    return flag
