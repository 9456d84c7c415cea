"""The AA-pattern (one lattice, in place) step against the two-lattice step.

Both run the same cells through the same collision, pull sources, bounce-back
and momentum exchange; only where the populations sit in memory differs.  The
in-place kernels are compiled separately, and the compiler may fuse a
multiply-add there that it keeps apart in the two-lattice kernel, so values
are held to a few units in the last place of the storage format (after up to
42 steps), forces and sums to the matching relative bar, instead of bit
equality.  A race in the in-place update would move values by orders of
magnitude more.  The mask touches every boundary kind (inlet and outlet
stones, a stone on the periodic edge of the top plane, interior ground), nx is
not a multiple of 32, and the runs cross the spin-up boundary and go through
graph replay.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

DTYPES = ["f32", "f64", "f16", "bf16"]
W0 = np.array([1 / 3] + [1 / 18] * 6 + [1 / 36] * 12)
# relative precision of what is stored: f32 / f64 values, 16-bit deviations f - w
EPS = {"f32": 2.0 ** -24, "f64": 2.0 ** -53, "f16": 2.0 ** -11, "bf16": 2.0 ** -8}


def _pair(flag, uin, n_total, n_spin, dtype, chunk=8):
    from stonewall.solver import WallSolver
    out = []
    for pattern in ("ab", "aa"):
        s = WallSolver(flag, uin, 2e-3, 0.1, flag.shape[0] - 8, n_total, n_spin=n_spin, dtype=dtype, chunk=chunk,
                       pattern=pattern)
        out.append(s.init(noise=0.03, seed=4, noise_kind="gauss"))
    return out


def _ref_dtype(dtype):
    return np.float64 if dtype == "f64" else np.float32


def _close(got, want, dtype, what, ulps=64):
    """|got - want| <= ulps units of the stored format's last place at the field's scale."""
    scale = np.abs(want - W0.reshape((19,) + (1,) * (want.ndim - 1))).max() if dtype in ("f16", "bf16") \
        else np.abs(want).max()
    err = np.abs(got.astype(np.float64) - want.astype(np.float64)).max()
    assert err <= ulps * EPS[dtype] * scale, f"{what}: max |diff| {err:.3g} vs scale {scale:.3g}"


@pytest.mark.parametrize("dtype", DTYPES)
def test_aa_equals_two_lattice_step(dtype, cuda):
    from gpu_helpers import inlet, make_mask
    flag = make_mask(45, 10, 13, 5)
    uin = inlet(13, 3)
    ab, aa = _pair(flag, uin, 42, 7, dtype)
    assert aa.memory_bytes() < ab.memory_bytes()
    rd = _ref_dtype(dtype)
    for n in (2, 16, 24):                      # eager steps, then graph replay (chunk 8)
        ab.advance(n)
        aa.advance(n)
        assert aa.t == ab.t
        a, b = aa.state_numpy(rd), ab.state_numpy(rd)
        fluid = np.broadcast_to(flag == 0, a.shape)
        np.testing.assert_array_equal(a[~fluid], b[~fluid])          # non-fluid cells are never written
        _close(a[:, flag == 0], b[:, flag == 0], dtype, f"state after {aa.t} steps")
    # per dtype: force relative to its largest value; rho and u per accumulated state
    force_rel, rho_tol, u_tol = {"f64": (1e-10, 1e-12, 1e-12), "f32": (1e-5, 1e-5, 1e-6),
                                 "f16": (1e-3, 2e-4, 1e-4), "bf16": (8e-3, 1.6e-3, 8e-4)}[dtype]
    fa, fb = aa.force_series(), ab.force_series()
    np.testing.assert_allclose(fa, fb, rtol=0, atol=force_rel * np.abs(fb).max())
    assert aa.n_acc == ab.n_acc == len(range(7, 42, 5))
    sa, sb = aa.sums(), ab.sums()
    np.testing.assert_allclose(sa[0], sb[0], rtol=0, atol=aa.n_acc * rho_tol)
    np.testing.assert_allclose(sa[1:], sb[1:], rtol=0, atol=aa.n_acc * u_tol)
    ma, mb = aa.macro(), ab.macro()
    np.testing.assert_allclose(ma[0], mb[0], rtol=0, atol=rho_tol)
    np.testing.assert_allclose(ma[1:], mb[1:], rtol=0, atol=u_tol)


@pytest.mark.parametrize("dtype", ["f16", "bf16"])
def test_aa_open_inlet_pairs_equal_two_lattice_step(dtype, cuda):
    """Stones only mid-channel, nx = 200: the 16-bit odd step's first segment pairs (inlet column
    included) and its interior pairs take the two-cell path, not the per-cell one."""
    from gpu_helpers import inlet, make_mask
    flag = make_mask(200, 12, 13, 6, x_lo=90, x_hi=110, extras=False)
    uin = inlet(13, 3)
    ab, aa = _pair(flag, uin, 30, 10, dtype)
    for n in (2, 4, 24):                        # states are read after even steps
        ab.advance(n)
        aa.advance(n)
        a, b = aa.state_numpy(np.float32), ab.state_numpy(np.float32)
        fluid = np.broadcast_to(flag == 0, a.shape)
        np.testing.assert_array_equal(a[~fluid], b[~fluid])
        _close(a[:, flag == 0], b[:, flag == 0], dtype, f"state after {aa.t} steps")
    tol = {"f16": (2e-4, 1e-4), "bf16": (1.6e-3, 8e-4)}[dtype]
    sa, sb = aa.sums(), ab.sums()
    np.testing.assert_allclose(sa[0], sb[0], rtol=0, atol=aa.n_acc * tol[0])
    np.testing.assert_allclose(sa[1:], sb[1:], rtol=0, atol=aa.n_acc * tol[1])


@pytest.mark.parametrize("dtype", ["f16", "bf16"])
def test_aa_without_tma_staging_equals_two_lattice_step(dtype, cuda):
    """The 16-bit AA steps with plain loads (the form used when no tensor maps can be made)."""
    from gpu_helpers import inlet, make_mask
    from stonewall import _native as N
    L = N.lib()
    old = L.sw_debug_aa_tma(0)
    try:
        for flag in (make_mask(45, 10, 13, 5), make_mask(200, 12, 13, 6, x_lo=90, x_hi=110, extras=False)):
            ab, aa = _pair(flag, inlet(13, 3), 24, 6, dtype)
            for n in (2, 22):
                ab.advance(n)
                aa.advance(n)
                a, b = aa.state_numpy(np.float32), ab.state_numpy(np.float32)
                fluid = np.broadcast_to(flag == 0, a.shape)
                np.testing.assert_array_equal(a[~fluid], b[~fluid])
                _close(a[:, flag == 0], b[:, flag == 0], dtype, f"state after {aa.t} steps")
    finally:
        L.sw_debug_aa_tma(old)


def test_aa_f32_matches_oracle(cuda, oracle_mod):
    """Ten in-place steps against ten steps of the CPU restatement of the reference kernel."""
    from gpu_helpers import assert_fields_close, assert_force_close, inlet, make_mask
    from stonewall.solver import WallSolver
    nx, ny, nz = 96, 16, 17
    flag = make_mask(nx, ny, nz, 3)
    uin = inlet(nz, 4)
    f0 = oracle_mod.init(flag, uin, noise=0.05, seed=3)
    args = (np.float32(2e-3), np.float32(0.1), nx - nx // 5, np.float32(0.05))
    n = 10
    want, want_force = oracle_mod.run(f0, flag, uin, *args[:3], n, args[3])
    s = WallSolver(flag, uin, float(args[0]), float(args[1]), args[2], n, n_spin=n, nu_sponge=float(args[3]),
                   dtype="f32", pattern="aa", chunk=4)
    s.f[0].assign(f0)
    s.advance(n)
    assert_fields_close(s.state_numpy(), want, flag, 1e-5)       # the two-lattice step's bar
    assert_force_close(s.force_series(), want_force, 1e-5)


def test_aa_odd_state_is_not_exposed(cuda):
    from gpu_helpers import inlet, make_mask
    flag = make_mask(40, 8, 10, 6)
    ab, aa = _pair(flag, inlet(10, 3), 10, 0, "f32")
    aa.step()
    with pytest.raises(RuntimeError):
        aa.state_numpy()
    with pytest.raises(RuntimeError):
        aa.macro()
    aa.step()
    aa.state_numpy()


def test_aa_checkpoint_resumes_in_two_lattice_solver(tmp_path, cuda):
    """An AA checkpoint is an ordinary checkpoint: a two-lattice solver resumes it."""
    from gpu_helpers import inlet, make_mask
    flag = make_mask(40, 12, 14, 10)
    uin = inlet(14, 4)
    full, aa = _pair(flag, uin, 48, 10, "f32")
    full.advance(48)
    aa.advance(24)
    aa.save_checkpoint(str(tmp_path / "ck"), sig="x")
    from stonewall.solver import WallSolver
    rest = WallSolver(flag, uin, 2e-3, 0.1, flag.shape[0] - 8, 48, n_spin=10, dtype="f32", chunk=8)
    rest.load_checkpoint(str(tmp_path / "ck"), sig="x")
    rest.advance(24)
    _close(rest.state_numpy()[:, flag == 0], full.state_numpy()[:, flag == 0], "f32", "resumed state")
    fr, ff = rest.force_series(), full.force_series()
    np.testing.assert_allclose(fr, ff, rtol=0, atol=64 * EPS["f32"] * np.abs(ff).max())
    np.testing.assert_allclose(rest.sums(), full.sums(), rtol=0, atol=1e-5 * rest.n_acc)


def test_aa_abi_rejects_bad_arguments(cuda):
    import ctypes
    import torch
    from stonewall import _native as N
    from stonewall.fields import Flags, Grid, Lattice
    from stonewall.kernels import DeviceVector
    from gpu_helpers import inlet, make_mask
    flag = make_mask(40, 8, 10, 6)
    g = Grid(*flag.shape)
    fl = Flags(g, flag)
    f = Lattice(g, "f32")
    uv = DeviceVector(inlet(10, 3))
    ghost = torch.empty(N.lib().sw_aa_ghost_elems(g.gp) * 4, dtype=torch.uint8, device="cuda")
    L = N.lib()
    args = lambda odd, gh: (g.gp, f.dtype, f.ptr, odd, fl.ptr, fl.tiles_ptr, uv.ptr, 2e-3, 0.1, 32, 0.05,
                            None, 0, None, gh, None, None)
    assert L.sw_step_aa(*args(2, ghost.data_ptr())) == N.SW_ERR_BAD_ARG
    assert L.sw_step_aa(*args(-1, ghost.data_ptr())) == N.SW_ERR_BAD_ARG
    assert L.sw_step_aa(*args(1, None)) == N.SW_ERR_BAD_ARG
    assert L.sw_aa_ghost_elems(ctypes.byref(N.SwGeom(0, 1, 1, 32))) < 0
