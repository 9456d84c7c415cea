"""sw_step_noalloc: the step for callers that cannot allocate device memory.

Such callers (a host that only receives device pointers from an allocator it
does not own, or a loop that must not call cudaMalloc / cudaFree because they
can synchronise the device) cannot supply the row-segment buffer that sw_step
takes; sw_step_noalloc keeps it in a fixed array inside the library.  These
tests call it through the C ABI and compare it with sw_step on the same
inputs, on consecutive calls with different grids (the array keeps the
previous call's contents, which must not leak into the next result).

The file is named to be collected last.
"""
import ctypes

import numpy as np
import pytest

RTOL = 1e-5


def _bind(L):
    from stonewall import _native as N
    fn = L.sw_step_noalloc
    P = ctypes.c_void_p
    fn.argtypes = [ctypes.POINTER(N.SwGeom), ctypes.c_int, P, P, P, P, ctypes.c_double, ctypes.c_double,
                   ctypes.c_int32, ctypes.c_double, P, ctypes.c_int64, P]
    fn.restype = ctypes.c_int
    return fn


def test_noalloc_rejects_oversize_grids(native_lib):
    """The size limit is checked on the host before anything is launched."""
    from stonewall import _native as N
    fn = _bind(native_lib)
    g = N.geom(2048, 512, 256)                         # 2^23 segments > SW_NOALLOC_MAX_SEGMENTS
    dummy = ctypes.c_void_p(256)
    rc = fn(ctypes.byref(g), N.SW_F32, dummy, ctypes.c_void_p(512), dummy, dummy, 0.0, 0.1, 0, 0.05, None, 0, None)
    assert rc == 7                                       # SW_ERR_TOO_LARGE
    assert b"scratch" in native_lib.sw_status_string(rc)


def _case(nx, ny, nz, seed):
    from gpu_helpers import inlet, make_mask
    from oracle import oracle
    flag = make_mask(nx, ny, nz, seed)
    uin = inlet(nz, max(2, nz // 4))
    f0 = oracle.init(flag, uin, noise=0.05, seed=seed)
    return flag, uin, f0


def _step_both(fn, flag, uin, f0, t, dtype="f32"):
    """One step through sw_step (with its own segment buffer) and one through sw_step_noalloc."""
    import torch
    from stonewall import _native as N
    from stonewall.fields import Flags, ForceSeries, Grid, Lattice
    from stonewall.kernels import DeviceVector, k_step
    nx, ny, nz = flag.shape
    grid = Grid(nx, ny, nz)
    flags = Flags(grid, flag)
    uv = DeviceVector(uin)
    src = Lattice(grid, dtype).assign(f0)
    want, got = Lattice(grid, dtype).zero_(), Lattice(grid, dtype).zero_()
    f_want, f_got = ForceSeries(t + 1, nz), ForceSeries(t + 1, nz)
    k_step(src, want, flags, uv, nx, ny, nz, 2e-3, 0.1, nx - nx // 5, 0.05, f_want, t)
    stream = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    rc = fn(ctypes.byref(grid.geom), src.dtype, src.ptr, got.ptr, flags.ptr, uv.ptr, 2e-3, 0.1, nx - nx // 5, 0.05,
            f_got.ptr, t, stream)
    assert rc == 0, native_status(rc)
    torch.cuda.synchronize()
    return want.numpy(), got.numpy(), f_want.numpy()[t], f_got.numpy()[t]


def native_status(rc):
    from stonewall import _native as N
    return N.lib().sw_status_string(rc).decode()


# a larger grid first, then smaller ones whose row has an odd number of 32-cell segments (the
# two-cells-per-thread kernels read segment pairs), then the first grid again: the array keeps
# the previous call's classes past the current grid, which must not reach the result
GRIDS = (((200, 24, 21), 4, 2), ((96, 16, 17), 1, 0), ((45, 7, 10), 2, 3), ((200, 24, 21), 4, 1))


@pytest.mark.gpu
@pytest.mark.parametrize("dtype,cfg", [("f32", None), ("f16", 4), ("f16", 8)])
def test_noalloc_matches_sw_step_on_consecutive_calls(dtype, cfg, cuda, native_lib):
    """The same results as sw_step, call after call: 32-bit storage in the installed configuration;
    16-bit storage through the two-cells-per-thread kernel (4) and the TMA-staged one (8)."""
    from stonewall import _native as N
    fn = _bind(native_lib)
    code = N.dtype_code(dtype)
    old = native_lib.sw_get_step_config(code)
    if cfg is not None:
        N.check(native_lib.sw_set_step_config(code, cfg), "sw_set_step_config")
    try:
        for shape, seed, t in GRIDS:
            flag, uin, f0 = _case(*shape, seed)
            want, got, fw, fg = _step_both(fn, flag, uin, f0, t, dtype)
            fluid = np.broadcast_to(flag == 0, want.shape)
            if dtype == "f32":
                np.testing.assert_allclose(got[fluid], want[fluid], rtol=RTOL, atol=0)
                np.testing.assert_allclose(fg, fw, rtol=RTOL, atol=RTOL * max(np.abs(fw).max(), 1e-30))
            else:                                  # the same kernel on the same inputs: the same bits
                np.testing.assert_array_equal(got[fluid], want[fluid])
                np.testing.assert_array_equal(fg, fw)
            np.testing.assert_array_equal(got[~fluid], want[~fluid])
        assert native_lib.sw_tma_timeouts() == 0
    finally:
        native_lib.sw_set_step_config(code, old)
