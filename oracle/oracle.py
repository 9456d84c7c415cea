"""ctypes front-end of the CPU oracle (TEST INFRASTRUCTURE ONLY).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline legs use this
module, as the checker or as the timed CPU baseline.  Arrays use the
reference's layout (stonewall3d/lbm3d.py:293-303): f[19, nx, ny, nz],
flag[nx, ny, nz], u[4, nx, ny, nz], all C-contiguous, z fastest.
"""
import ctypes

import numpy as np

from . import build_oracle  # noqa: F401  (package-relative when imported as oracle.oracle)

_LIB = None


def lib():
    global _LIB
    if _LIB is None:
        path = build_oracle.build()
        L = ctypes.CDLL(path)
        P = ctypes.c_void_p
        i32, f32, f64 = ctypes.c_int, ctypes.c_float, ctypes.c_double
        L.sw_oracle_tables.argtypes = [P, P, P, P]
        L.sw_oracle_init_f32.argtypes = [P, P, P, i32, i32, i32, f32, i32, i32]
        L.sw_oracle_init_f64.argtypes = [P, P, P, i32, i32, i32, f64, i32, i32]
        L.sw_oracle_step_f32.argtypes = [P, P, P, P, i32, i32, i32, f32, f32, i32, f32, P]
        L.sw_oracle_step_f64.argtypes = [P, P, P, P, i32, i32, i32, f64, f64, i32, f64, P]
        L.sw_oracle_macro_f32.argtypes = [P, P, i32, i32, i32, P]
        L.sw_oracle_macro_f64.argtypes = [P, P, i32, i32, i32, P]
        L.sw_oracle_accum.argtypes = [P, P, ctypes.c_longlong]
        L.sw_oracle_max_threads.restype = i32
        L.sw_oracle_set_threads.argtypes = [i32]
        _LIB = L
    return _LIB


def _p(a):
    return a.ctypes.data_as(ctypes.c_void_p)


def _check(a, dtype, shape=None):
    assert a.dtype == dtype and a.flags.c_contiguous, (a.dtype, a.flags)
    if shape is not None:
        assert a.shape == tuple(shape), (a.shape, shape)


def set_threads(n):
    lib().sw_oracle_set_threads(int(n))


def max_threads():
    return lib().sw_oracle_max_threads()


def tables():
    c = np.zeros((19, 3), np.int32)
    w = np.zeros(19, np.float32)
    opp = np.zeros(19, np.int32)
    mirz = np.zeros(19, np.int32)
    lib().sw_oracle_tables(_p(c), _p(w), _p(opp), _p(mirz))
    return c, w, opp, mirz


def init(flag, uin, noise=0.02, seed=7, noise_kind=0, dtype=np.float32):
    """k_init (lbm3d.py:39-54); noise_kind 0 = uniform (reference), 1 = Gaussian."""
    nx, ny, nz = flag.shape
    _check(flag, np.uint8)
    uin = np.ascontiguousarray(uin, dtype=dtype)
    f = np.zeros((19, nx, ny, nz), dtype)
    fn = lib().sw_oracle_init_f32 if dtype == np.float32 else lib().sw_oracle_init_f64
    fn(_p(f), _p(flag), _p(uin), nx, ny, nz, noise, seed, noise_kind)
    return f


def step(f_in, flag, uin, nu0, cs, x_sponge, nu_sponge=0.05, f_out=None, force_row=None):
    """One k_step (lbm3d.py:57-155).  Returns (f_out, force_row[nz, 2] float64).

    Like the reference, cells that are not fluid are never written: pass the
    previous f_out to keep the ping-pong semantics of lbm3d.py:293-294,362.
    """
    dtype = f_in.dtype
    nx, ny, nz = flag.shape
    _check(f_in, dtype, (19, nx, ny, nz))
    _check(flag, np.uint8)
    uin = np.ascontiguousarray(uin, dtype=dtype)
    if f_out is None:
        f_out = np.zeros_like(f_in)
    _check(f_out, dtype, f_in.shape)
    if force_row is None:
        force_row = np.zeros((nz, 2), np.float64)
    fn = lib().sw_oracle_step_f32 if dtype == np.float32 else lib().sw_oracle_step_f64
    fn(_p(f_in), _p(f_out), _p(flag), _p(uin), nx, ny, nz, nu0, cs, int(x_sponge), nu_sponge, _p(force_row))
    return f_out, force_row


def macro(f, flag):
    """k_macro (lbm3d.py:158-182): u[0]=rho, u[1:4]=velocity; solids -> (1, 0, 0, 0)."""
    nx, ny, nz = flag.shape
    u = np.zeros((4, nx, ny, nz), f.dtype)
    fn = lib().sw_oracle_macro_f32 if f.dtype == np.float32 else lib().sw_oracle_macro_f64
    fn(_p(np.ascontiguousarray(f)), _p(flag), nx, ny, nz, _p(u))
    return u


def accum(u, acc):
    """k_accum (lbm3d.py:185-188), accumulated in float64."""
    _check(u, np.float32)
    _check(acc, np.float64, u.shape)
    lib().sw_oracle_accum(_p(u), _p(acc), u.size)
    return acc


def slice_xz(u, y0):
    """k_slice_xz (lbm3d.py:191-194)."""
    return np.ascontiguousarray(u[:, :, y0, :])


def slice_xy(u, z0):
    """k_slice_xy (lbm3d.py:197-200)."""
    return np.ascontiguousarray(u[:, :, :, z0])


def qcoarse(u, flag, x0, ds, dims):
    """k_qcoarse with q_at (lbm3d.py:203-238) in float32 numpy, the same expression order per cell:
    Q = -1/2 A_ij A_ji of the central-difference gradient, 0 next to non-fluid cells and outside
    1 <= x < nx-1, 1 <= z < nz-1 (y periodic), then max(0, block max) over ds^3 blocks from x0."""
    u = np.asarray(u, np.float32)
    nx, ny, nz = flag.shape
    half = np.float32(0.5)

    def sh(a, dx, dy, dz):
        return np.roll(a, -dy, axis=1)[1 + dx:nx - 1 + dx, :, 1 + dz:nz - 1 + dz]

    def grad(c, dx, dy, dz):
        return half * (sh(u[c], dx, dy, dz) - sh(u[c], -dx, -dy, -dz))

    a11, a12, a13 = grad(1, 1, 0, 0), grad(1, 0, 1, 0), grad(1, 0, 0, 1)
    a21, a22, a23 = grad(2, 1, 0, 0), grad(2, 0, 1, 0), grad(2, 0, 0, 1)
    a31, a32, a33 = grad(3, 1, 0, 0), grad(3, 0, 1, 0), grad(3, 0, 0, 1)
    q = -0.5 * (a11 * a11 + a22 * a22 + a33 * a33 + 2.0 * (a12 * a21 + a13 * a31 + a23 * a32))
    solid = flag != 0
    near = np.zeros(q.shape, bool)
    for d in ((0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1)):
        near |= sh(solid, *d)
    Q = np.zeros((nx, ny, nz), np.float32)
    Q[1:nx - 1, :, 1:nz - 1] = np.where(near, np.float32(0.0), q)
    di, dj, dk = dims
    blk = Q[x0:x0 + di * ds, :dj * ds, :dk * ds].reshape(di, ds, dj, ds, dk, ds)
    return np.maximum(np.float32(0.0), blk.max(axis=(1, 3, 5)))


def run(f0, flag, uin, nu0, cs, x_sponge, n_steps, nu_sponge=0.05):
    """n_steps of ping-pong stepping from f0 (lbm3d.py:358-362).  Returns (f, force[n, nz, 2])."""
    fa = f0.copy()
    fb = np.zeros_like(f0)
    force = np.zeros((n_steps, flag.shape[2], 2), np.float64)
    for t in range(n_steps):
        step(fa, flag, uin, nu0, cs, x_sponge, nu_sponge, f_out=fb, force_row=force[t])
        fa, fb = fb, fa
    return fa, force
