"""Helpers shared by the GPU tests: run the sm_103a path through the package API."""
import numpy as np


def make_mask(nx, ny, nz, seed, density=0.15, x_lo=None, x_hi=None, z_hi=None, extras=True):
    """A random stone mask with a ground plane, touching every boundary the step handles."""
    from stonewall.lattice import GROUND, WALL
    rng = np.random.default_rng(seed)
    flag = np.zeros((nx, ny, nz), np.uint8)
    x_lo = 2 if x_lo is None else x_lo
    x_hi = nx - 2 if x_hi is None else x_hi
    z_hi = nz - 1 if z_hi is None else z_hi
    sub = rng.random((x_hi - x_lo, ny, z_hi - 1)) < density
    flag[x_lo:x_hi, :, 1:z_hi][sub] = WALL
    if extras:
        flag[0, ny // 2, nz // 2] = WALL              # a stone in the inlet plane
        flag[nx - 1, 1, nz // 3] = WALL               # one in the outlet plane
        flag[nx // 2, 0, nz - 1] = WALL               # one in the top plane, on the periodic edge
        flag[nx // 3, ny - 1, 2] = GROUND             # interior ground cell: bounce-back, no force
    flag[:, :, 0] = GROUND
    return flag


def inlet(nz, H, U0=0.08):
    zeta = np.arange(nz) - 0.5
    u = (U0 * np.clip(zeta / (3.0 * H), 0, 1) ** (1 / 7)).astype(np.float32)
    u[0] = 0.0
    return u


def gpu_run(flag, uin, f_init, nu0, cs, x_sponge, nu_sponge, n, dtype="f32", ref_dtype=np.float32):
    """n ping-pong steps on the GPU from f_init (reference layout).  Returns (f, f_other, force)."""
    from stonewall.fields import Flags, ForceSeries, Grid, Lattice
    from stonewall.kernels import DeviceVector, k_step
    nx, ny, nz = flag.shape
    grid = Grid(nx, ny, nz)
    flags = Flags(grid, flag)
    uv = DeviceVector(uin)
    fa = Lattice(grid, dtype).assign(f_init)
    fb = Lattice(grid, dtype).zero_()
    force = ForceSeries(max(n, 1), nz)
    for t in range(n):
        k_step(fa, fb, flags, uv, nx, ny, nz, nu0, cs, x_sponge, nu_sponge, force, t)
        fa, fb = fb, fa
    return fa.numpy(ref_dtype), fb.numpy(ref_dtype), force.numpy()[:n]


def assert_fields_close(got, want, flag, rtol):
    """Fluid cells within rtol; non-fluid cells must be untouched (bit-equal)."""
    fluid = np.broadcast_to(flag == 0, want.shape)
    np.testing.assert_allclose(got[fluid], want[fluid], rtol=rtol, atol=0)
    np.testing.assert_array_equal(got[~fluid], want[~fluid])


def assert_force_close(got, want, rtol):
    scale = max(np.abs(want).max(), 1e-30)
    np.testing.assert_allclose(got, want, rtol=rtol, atol=rtol * scale)
