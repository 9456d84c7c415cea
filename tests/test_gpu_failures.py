"""Failure detection on the device, tested without a device fault.

The reference finds divergence on the host, from the macro field every 5000
steps (lbm3d.py:386-391).  Here the step kernels set bits of a per-lattice
device status word: SW_STATUS_NONFINITE when a fluid cell pulls a non-finite
density, SW_STATUS_TIMEOUT when a block of the TMA-staged step gives up its
bounded wait for the copies of a stage.  The failures are made on the host:
  * a NaN written into one population of the host array before upload;
  * the TMA blocks' poll limit set to 0 (sw_debug_tma_poll_limit), so that every
    block gives up at its first stage at once; the block still lets the copies
    it issued land (that wait keeps its normal bound) before it leaves, and the
    context stays usable, which the test checks by stepping again.
The solver, the batch and the server turn the bits into Diverged /
DeviceWaitTimeout, and the server fails only the request concerned.
"""
import numpy as np
import pytest

from gpu_helpers import inlet, make_mask

pytestmark = pytest.mark.gpu


def _case(seed=1, shape=(64, 16, 17)):
    from oracle import oracle
    nx, ny, nz = shape
    flag = make_mask(nx, ny, nz, seed)
    uin = inlet(nz, max(2, nz // 4))
    return flag, uin, oracle.init(flag, uin, noise=0.05, seed=seed)


def _poison(f, flag, pop=3):
    """f with one population of one interior fluid cell set to NaN (host side)."""
    bad = f.copy()
    xs, ys, zs = np.nonzero(flag == 0)
    k = np.argmin(np.abs(xs - flag.shape[0] // 2) + np.abs(zs - flag.shape[2] // 2))
    bad[pop, xs[k], ys[k], zs[k]] = np.nan
    return bad


def _one_step(flag, uin, f0, dtype, cfg, n=1):
    from stonewall.fields import Flags, ForceSeries, Grid, Lattice, StatusWord
    from stonewall.kernels import DeviceVector, k_step
    nx, ny, nz = flag.shape
    g = Grid(nx, ny, nz)
    flags, uv = Flags(g, flag), DeviceVector(uin)
    fa, fb = Lattice(g, dtype).assign(f0), Lattice(g, dtype).zero_()
    force, status = ForceSeries(n, nz), StatusWord()
    for t in range(n):
        k_step(fa, fb, flags, uv, nx, ny, nz, 2e-3, 0.1, nx - 10, 0.05, force, t, status=status, cfg=cfg)
        fa, fb = fb, fa
    return status.read(), fa


@pytest.mark.parametrize("dtype,cfg", [("f32", 0), ("f32", 3), ("f64", 0), ("f16", 0), ("f16", 4), ("f16", 8),
                                       ("bf16", 5), ("bf16", 9)])
def test_nonfinite_density_sets_the_status_word(dtype, cfg, cuda):
    from stonewall import _native as N
    flag, uin, f0 = _case()
    clean, _ = _one_step(flag, uin, f0, dtype, cfg)
    assert clean == 0
    word, _ = _one_step(flag, uin, _poison(f0, flag), dtype, cfg)
    assert word & N.SW_STATUS_NONFINITE and not word & N.SW_STATUS_TIMEOUT
    assert N.lib().sw_status_error(word) == N.SW_ERR_NONFINITE


@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_nonfinite_density_in_the_aa_step(dtype, cuda):
    import torch
    from stonewall import _native as N
    from stonewall.fields import Flags, Grid, Lattice, StatusWord
    from stonewall.kernels import DeviceVector, k_step_aa
    flag, uin, f0 = _case(2, (45, 7, 10))
    g = Grid(*flag.shape)
    flags, uv = Flags(g, flag), DeviceVector(uin)
    ghost = torch.empty(N.lib().sw_aa_ghost_elems(g.gp) * 4, dtype=torch.uint8, device="cuda")
    for f_init, want in ((f0, 0), (_poison(f0, flag), N.SW_STATUS_NONFINITE)):
        f, status = Lattice(g, dtype).assign(f_init), StatusWord()
        for t in range(2):
            k_step_aa(f, t == 0, flags, uv, 2e-3, 0.1, 35, 0.05, None, t, ghost=ghost, status=status)
        assert status.read() == want


def test_aa_tma_timeout_is_reported_and_the_context_stays_usable(cuda):
    """Poll limit 0 on the TMA-staged 16-bit AA steps: both step kinds report SW_STATUS_TIMEOUT and the
    blocks' copies land before they leave; with the limit restored an AA pair of steps from a fresh
    state equals a clean run."""
    import torch
    from stonewall import _native as N
    from stonewall.fields import Flags, Grid, Lattice, StatusWord
    from stonewall.kernels import DeviceVector, k_step_aa
    L = N.lib()
    flag, uin, f0 = _case(3, (96, 16, 17))
    g = Grid(*flag.shape)
    flags, uv = Flags(g, flag), DeviceVector(uin)
    ghost = torch.empty(L.sw_aa_ghost_elems(g.gp) * 2, dtype=torch.uint8, device="cuda")

    def two_steps():
        f, status = Lattice(g, "f16").assign(f0), StatusWord()
        for t in range(2):
            k_step_aa(f, t == 0, flags, uv, 2e-3, 0.1, 86, 0.05, None, t, ghost=ghost, status=status)
        return status.read(), f.numpy(np.float64)

    word0, ref = two_steps()
    assert word0 == 0
    L.sw_tma_timeouts()                                  # clear the counter
    old = L.sw_debug_tma_poll_limit(0)
    try:
        word, _ = two_steps()
        blocks = L.sw_tma_timeouts()
    finally:
        L.sw_debug_tma_poll_limit(old)
    assert word & N.SW_STATUS_TIMEOUT and blocks > 0
    word2, again = two_steps()
    assert word2 == 0 and L.sw_tma_timeouts() == 0
    np.testing.assert_array_equal(again, ref)


def test_tma_timeout_is_reported_and_the_context_stays_usable(cuda):
    """Poll limit 0: every TMA-staged block gives up at its first stage.  The status word and the
    process-wide counter report it, the autotuner drops the configuration, and with the limit
    restored the same launch computes the step again (equal to the two-cells-per-thread kernel)."""
    from stonewall import _native as N
    L = N.lib()
    flag, uin, f0 = _case(3, (96, 16, 17))
    ref_word, ref = _one_step(flag, uin, f0, "f16", 4)
    assert ref_word == 0
    L.sw_tma_timeouts()                                  # clear the counter
    old = L.sw_debug_tma_poll_limit(0)
    try:
        word, _ = _one_step(flag, uin, f0, "f16", 8)
        blocks = L.sw_tma_timeouts()
        from stonewall.solver import WallSolver
        s = WallSolver(flag, uin, 2e-3, 0.1, 86, 10, dtype="f16").init(noise=0.02, seed=1)
        from stonewall.autotune import time_configs
        times = time_configs(s, repeats=1, warmup=1)
    finally:
        L.sw_debug_tma_poll_limit(old)
    assert word & N.SW_STATUS_TIMEOUT
    assert L.sw_status_error(word) == N.SW_ERR_TIMEOUT
    assert blocks > 0
    assert set(times) == set(range(8))                   # the TMA-staged configurations (8 and up) were left out
    word2, again = _one_step(flag, uin, f0, "f16", 8)
    assert word2 == 0 and L.sw_tma_timeouts() == 0
    np.testing.assert_array_equal(again.numpy(np.float64), ref.numpy(np.float64))


def test_wall_solver_raises_on_divergence_and_on_timeout(cuda):
    from stonewall import _native as N
    from stonewall.solver import DeviceWaitTimeout, Diverged, WallSolver
    flag, uin, f0 = _case(4, (64, 16, 17))
    s = WallSolver(flag, uin, 2e-3, 0.1, 54, 20, dtype="f32", chunk=5)
    s.state.assign(_poison(f0, flag))
    with pytest.raises(Diverged):
        s.advance(10)
    s.state.assign(f0)
    s.status.clear()
    s.advance(10)                                        # clean again
    t = WallSolver(flag, uin, 2e-3, 0.1, 54, 20, dtype="f16", chunk=5)
    t.state.assign(f0)
    L = N.lib()
    cfg_old = L.sw_get_step_config(N.SW_F16_SHIFT)
    N.check(L.sw_set_step_config(N.SW_F16_SHIFT, 8), "sw_set_step_config")
    old = L.sw_debug_tma_poll_limit(0)
    try:
        with pytest.raises(DeviceWaitTimeout):
            t.advance(5, use_graphs=False)
    finally:
        L.sw_debug_tma_poll_limit(old)
        L.sw_set_step_config(N.SW_F16_SHIFT, cfg_old)
        L.sw_tma_timeouts()


@pytest.mark.parametrize("mode", ["persistent", "graph"])
def test_batch_reports_only_the_failed_member(mode, cuda):
    from stonewall.batch import Batch
    from stonewall.solver import Diverged, WallSolver

    def member(shape, seed, poison):
        flag, uin, f0 = _case(seed, shape)
        s = WallSolver(flag, uin, 2e-3, 0.1, shape[0] - 10, 20, n_spin=5, dtype="f16")
        s.state.assign(_poison(f0, flag) if poison else f0)
        return s

    shapes = [((64, 16, 17), 1), ((45, 7, 10), 2), ((96, 12, 21), 3)]
    alone = []
    for shape, seed in shapes:
        b = Batch(dtype="f16", chunk=5, mode=mode)
        m = b.add(member(shape, seed, False))
        b.advance(20, check=True)
        alone.append(m.state.numpy(np.float64))
    mix = Batch(dtype="f16", chunk=5, mode=mode)
    ms = [mix.add(member(shape, seed, i == 1)) for i, (shape, seed) in enumerate(shapes)]
    mix.advance(20)
    bad = mix.failures()
    assert list(bad) == [ms[1]] and isinstance(bad[ms[1]], Diverged)
    with pytest.raises(Diverged):
        mix.check()
    for i in (0, 2):
        np.testing.assert_array_equal(ms[i].state.numpy(np.float64), alone[i])


def test_server_fails_only_the_diverged_request(monkeypatch, cuda):
    """A NaN planted on the host into one request's initial state: that request comes back failed
    (and does not count as completed), the others give the same statistics as solved alone."""
    from stonewall import serve
    from stonewall.serve import Request, Server, run_alone, solve_stats
    reqs = [Request(rid=i, t_arrive=0.0, H=8, porosity=0.2, U=0.05, steps=160, dtype=dt, seed=50 + i)
            for i, dt in enumerate(["f16", "f16", "f32", "f16"])]
    orig = serve.make_solver

    def planted(req, p, flag, device="cuda", pattern="ab"):
        s = orig(req, p, flag, device, pattern)
        if req.rid == 1:
            s.state.assign(_poison(s.state.numpy(), flag))
        return s
    monkeypatch.setattr(serve, "make_solver", planted)
    srv = Server(cap_bytes=1e12, chunk=16, check_every=3)
    out = srv.serve(reqs)
    monkeypatch.setattr(serve, "make_solver", orig)
    by = {r.rid: r for r in out}
    assert by[1].result["failed"] == "Diverged" and by[1].result["steps_done"] < 160
    assert srv.failed == 1 and not srv.resident and srv.used == 0
    summ = Server.summary(out, 10.0)
    assert summ["completed"] == 3 and summ["failed"] == 1
    for rid in (0, 2, 3):
        st = solve_stats(run_alone(by[rid]))
        assert st == by[rid].result["stats"], rid
