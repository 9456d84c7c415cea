"""Viewer payload on the GPU: velocity slices and Q-criterion frames (lbm3d.py:191-238).

The macro field is bit-exact against the oracle (k_macro), the slices are
copies of it, and the Q-criterion kernel evaluates the reference's float32
expression in its order without contraction, so all three are checked for
bit equality against the oracle's numpy restatement on a developed flow.
"""
import numpy as np
import pytest

from gpu_helpers import inlet, make_mask

pytestmark = pytest.mark.gpu


def test_slices_and_q_frame_match_oracle(cuda, oracle_mod):
    import torch
    from stonewall.fields import Flags, Grid, Lattice, Macro
    from stonewall.kernels import k_macro, k_qcoarse, k_slice_xy, k_slice_xz
    nx, ny, nz = 70, 14, 19
    flag = make_mask(nx, ny, nz, 11, density=0.2)
    uin = inlet(nz, 4)
    f0 = oracle_mod.init(flag, uin, noise=0.05, seed=11)
    f, _ = oracle_mod.run(f0, flag, uin, np.float32(2e-3), np.float32(0.1), nx - 12, 6, np.float32(0.05))
    want_u = oracle_mod.macro(f, flag)
    g = Grid(nx, ny, nz)
    fl = Flags(g, flag)
    u = Macro(g)
    k_macro(Lattice(g, "f32").assign(f), fl, u)
    np.testing.assert_array_equal(u.numpy(), want_u)
    xz = torch.empty((4, nx, nz), dtype=torch.float32, device="cuda")
    xy = torch.empty((4, nx, ny), dtype=torch.float32, device="cuda")
    k_slice_xz(u, ny // 2, xz)
    k_slice_xy(u, 5, xy)
    np.testing.assert_array_equal(xz.cpu().numpy(), oracle_mod.slice_xz(want_u, ny // 2))
    np.testing.assert_array_equal(xy.cpu().numpy(), oracle_mod.slice_xy(want_u, 5))
    for x0, ds in ((1, 1), (3, 2), (10, 3)):
        dims = ((nx - 1 - x0) // ds, ny // ds, (nz - 1) // ds)
        q = torch.empty(dims, dtype=torch.float32, device="cuda")
        k_qcoarse(u, fl, x0, ds, nx, ny, nz, q)
        want = oracle_mod.qcoarse(want_u, flag, x0, ds, dims)
        assert (want > 0).any()
        np.testing.assert_array_equal(q.cpu().numpy(), want)


def test_q_frame_rejects_out_of_range_crops(cuda):
    import ctypes
    from stonewall import _native as N
    g = N.geom(40, 8, 10)
    L = N.lib()
    P = ctypes.c_void_p(16)
    assert L.sw_qcoarse(ctypes.byref(g), P, P, 1, 2, 20, 4, 5, P, None) == N.SW_ERR_BAD_ARG   # x0 + di ds > nx
    assert L.sw_qcoarse(ctypes.byref(g), P, P, 1, 2, 10, 5, 5, P, None) == N.SW_ERR_BAD_ARG   # dj ds > ny
    assert L.sw_slice_xz(ctypes.byref(g), P, 8, P, None) == N.SW_ERR_BAD_ARG
