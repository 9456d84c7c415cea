"""The bounds-checked build: no step kernel computes an element offset outside its plane.

libstonewall_check.so is the same sources compiled with -DSW_CHECK: every computed
neighbour, target and cell offset of the step kernels (one and two cells per
thread, TMA-staged, in-place AA, persistent batch) is tested against its
population plane, and one that falls outside sets SW_STATUS_BOUNDS in the
lattice's status word instead of being used.  These tests run every kernel form
and launch configuration, plain and accumulating, on grids with padding, odd and
two-cell spans, stones in the inlet, outlet and top planes and interior ground,
and require the status word to stay clear.  (A planted out-of-bounds access is
not run on the GPU: the mask and grid cases are what can reach the edges.)
"""
import pytest

from gpu_helpers import inlet, make_mask

pytestmark = pytest.mark.gpu

SHAPES = [((45, 7, 10), 1), ((33, 2, 6), 2), ((96, 16, 17), 3), ((70, 13, 11), 4)]


@pytest.fixture(scope="module")
def checked_lib(native_lib):
    """Swap the package onto the bounds-checked library for this module's tests."""
    from stonewall import _native as N
    from stonewall import build
    path = build.build(check=True)
    saved = N._lib
    N._lib = N.load(path)
    yield N._lib
    N._lib = saved


def _case(shape, seed):
    from oracle import oracle
    nx, ny, nz = shape
    flag = make_mask(nx, ny, nz, seed)
    uin = inlet(nz, max(2, nz // 4))
    return flag, uin, oracle.init(flag, uin, noise=0.05, seed=seed)


@pytest.mark.parametrize("dtype", ["f32", "f64", "f16", "bf16"])
def test_every_step_configuration_stays_in_bounds(dtype, checked_lib, cuda):
    from stonewall import _native as N
    from stonewall.fields import Accum, Flags, ForceSeries, Grid, Lattice, StatusWord
    from stonewall.kernels import DeviceVector, k_step
    L = checked_lib
    for shape, seed in SHAPES:
        flag, uin, f0 = _case(shape, seed)
        nx, ny, nz = shape
        g = Grid(nx, ny, nz)
        flags, uv = Flags(g, flag), DeviceVector(uin)
        for cfg in range(L.sw_step_config_count()):
            if cfg >= 4 and dtype in ("f32", "f64"):
                continue
            for acc in (None, Accum(g)):
                a, b = Lattice(g, dtype).assign(f0), Lattice(g, dtype).zero_()
                status = StatusWord()
                force = ForceSeries(3, nz)
                for t in range(3):
                    try:
                        k_step(a, b, flags, uv, nx, ny, nz, 2e-3, 0.1, nx - nx // 5, 0.05, force, t, acc=acc,
                               status=status, cfg=cfg)
                    except N.StonewallError as e:
                        raise AssertionError(f"{dtype} {shape} cfg {cfg} acc {acc is not None}: {e}") from e
                    a, b = b, a
                word = status.read()
                assert word == 0, f"{dtype} {shape} cfg {cfg} acc {acc is not None}: status {word:#x}"
    assert L.sw_tma_timeouts() == 0
    assert N.lib() is L


@pytest.mark.parametrize("dtype", ["f32", "f16", "bf16"])
def test_aa_steps_stay_in_bounds(dtype, checked_lib, cuda):
    import torch
    from stonewall import _native as N
    from stonewall.fields import Accum, Flags, ForceSeries, Grid, Lattice, StatusWord
    from stonewall.kernels import DeviceVector, k_step_aa
    for shape, seed in SHAPES:
        flag, uin, f0 = _case(shape, seed)
        nx, ny, nz = shape
        g = Grid(nx, ny, nz)
        flags, uv = Flags(g, flag), DeviceVector(uin)
        ghost = torch.empty(N.lib().sw_aa_ghost_elems(g.gp) * 8, dtype=torch.uint8, device="cuda")
        for acc in (None, Accum(g)):
            f, status, force = Lattice(g, dtype).assign(f0), StatusWord(), ForceSeries(4, nz)
            for t in range(4):
                k_step_aa(f, t % 2 == 0, flags, uv, 2e-3, 0.1, nx - nx // 5, 0.05, force, t, ghost=ghost, acc=acc,
                          status=status)
            assert status.read() == 0, (dtype, shape)


@pytest.mark.parametrize("mode", ["persistent", "graph"])
@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_batches_stay_in_bounds(dtype, mode, checked_lib, cuda):
    from stonewall import _native as N
    from stonewall.batch import Batch, _valid
    from stonewall.solver import WallSolver
    code = N.dtype_code(dtype)
    cfgs = [c for c in range(8) if _valid(code, c)] if mode == "persistent" else [None]
    for cfg in cfgs:
        b = Batch(dtype=dtype, chunk=4, mode=mode, cfg=cfg)
        members = []
        for shape, seed in SHAPES:
            flag, uin, f0 = _case(shape, seed)
            s = WallSolver(flag, uin, 2e-3, 0.1, shape[0] - shape[0] // 5, 8, n_spin=3, dtype=dtype, chunk=4)
            s.state.assign(f0)
            members.append(b.add(s))
        b.advance(8)
        words = b.status_words().cpu().tolist()
        assert words == [0] * len(members), (dtype, mode, cfg, words)
