"""Batched stepping: many walls in one persistent launch per step, or one graph
of per-wall launches per chunk.

A wall's results must not depend on the batch it runs in (alone vs in the mix:
bit-identical), members with their own step counters and lengths advance
independently, the batched kernel computes the single-lattice step, and the
graph mode runs exactly the single-lattice launches.
"""
import numpy as np
import pytest

from gpu_helpers import inlet, make_mask

pytestmark = pytest.mark.gpu


def _member(shape, seed, n_total, n_spin, dtype, pattern="ab"):
    from stonewall.solver import WallSolver
    nx, ny, nz = shape
    flag = make_mask(nx, ny, nz, seed)
    s = WallSolver(flag, inlet(nz, max(2, nz // 4)), 2e-3, 0.1, nx - nx // 5, n_total, n_spin=n_spin, dtype=dtype,
                   pattern=pattern)
    return s.init(noise=0.03, seed=seed, noise_kind="gauss")


SHAPES = [((64, 16, 17), 1), ((96, 12, 21), 2), ((45, 7, 10), 3)]


def _snapshot(m):
    return m.state.numpy(np.float64), m.force.data.cpu().numpy().copy(), m.sums(), m.t, m.n_acc


@pytest.mark.parametrize("mode", ["persistent", "graph"])
@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_alone_equals_in_the_mix(dtype, mode, cuda):
    from stonewall.batch import Batch
    alone = []
    for shape, seed in SHAPES:
        b = Batch(dtype=dtype, chunk=8, mode=mode)
        m = b.add(_member(shape, seed, 40, 12, dtype))
        b.advance(40)
        alone.append(_snapshot(m))
    mix = Batch(dtype=dtype, chunk=8, mode=mode)
    ms = [mix.add(_member(shape, seed, 40, 12, dtype)) for shape, seed in SHAPES]
    mix.advance(40)
    for a, m in zip(alone, ms):
        b = _snapshot(m)
        np.testing.assert_array_equal(a[0], b[0])
        np.testing.assert_array_equal(a[1], b[1])
        np.testing.assert_array_equal(a[2], b[2])
        assert a[3:] == b[3:] == (40, len(range(12, 40, 5)))


def test_batch_matches_single_lattice_step(cuda):
    """The batched kernel computes the same step as the single-lattice kernel (fp32, 1e-5)."""
    from gpu_helpers import assert_fields_close, assert_force_close
    from stonewall.batch import Batch
    for shape, seed in SHAPES:
        ref = _member(shape, seed, 30, 5, "f32")
        ref.advance(30, use_graphs=False)
        b = Batch(dtype="f32", chunk=10)
        m = b.add(_member(shape, seed, 30, 5, "f32"))
        b.advance(30)
        flag = ref.flags.host
        assert_fields_close(m.state.numpy(), ref.state.numpy(), flag, 1e-5)
        assert_force_close(m.force_series(), ref.force_series(), 1e-5)
        np.testing.assert_allclose(m.sums(), ref.sums(), rtol=1e-5, atol=1e-7)
        assert m.n_acc == ref.n_acc


@pytest.mark.parametrize("mode", ["persistent", "graph"])
def test_members_with_their_own_clocks(mode, cuda):
    """Staggered members: one admitted late, one finishing mid-chunk; each equals its own solo run."""
    from stonewall.batch import Batch
    b = Batch(dtype="f16", chunk=8, mode=mode)
    m1 = b.add(_member(SHAPES[0][0], 1, 30, 4, "f16"))
    b.advance(11)                                  # m1 at t = 11
    m2 = b.add(_member(SHAPES[1][0], 2, 13, 4, "f16"))
    b.advance(16)                                  # m1 -> 27, m2 -> 13 (finished mid-chunk)
    assert (m1.t, m2.t) == (27, 13)
    b.advance(10)
    assert (m1.t, m2.t) == (30, 13) and not b.pending()
    for m, (shape, seed), n in ((m1, SHAPES[0], 30), (m2, SHAPES[1], 13)):
        solo = Batch(dtype="f16", chunk=8, mode=mode)
        r = solo.add(_member(shape, seed, n, 4, "f16"))
        solo.advance(n)
        a, c = _snapshot(m), _snapshot(r)
        for u, v in zip(a[:3], c[:3]):
            np.testing.assert_array_equal(u, v)
        assert a[3:] == c[3:]


@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_graph_mode_is_the_single_lattice_solve(dtype, cuda):
    """Graph mode launches the single-lattice kernels: bit-identical to WallSolver.advance."""
    from stonewall.batch import Batch
    refs = []
    for shape, seed in SHAPES:
        r = _member(shape, seed, 37, 6, dtype)
        r.advance(37)
        refs.append(_snapshot(r))
    b = Batch(dtype=dtype, chunk=10, mode="graph")
    ms = [b.add(_member(shape, seed, 37, 6, dtype)) for shape, seed in SHAPES]
    b.advance(37)
    assert b.launches == 3 * 37
    for a, m in zip(refs, ms):
        c = _snapshot(m)
        for u, v in zip(a[:3], c[:3]):
            np.testing.assert_array_equal(u, v)
        assert a[3:] == c[3:]


def test_autotune_keeps_the_states(cuda):
    from stonewall.batch import Batch
    b = Batch(dtype="f16", chunk=8)
    ms = [b.add(_member(shape, seed, 20, 4, "f16")) for shape, seed in SHAPES]
    before = [m.state.numpy(np.float64) for m in ms]
    best, times = b.autotune(repeats=2)
    assert "graph" in times and best in times
    assert b.mode == ("graph" if best == "graph" else "persistent")
    for m, x in zip(ms, before):
        np.testing.assert_array_equal(m.state.numpy(np.float64), x)
    b.advance(20)
    assert not b.pending()


@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_aa_members_in_graph_mode_equal_their_solo_runs(dtype, cuda):
    """In-place (AA) members beside two-lattice ones, odd chunk lengths (the odd/even parity carries
    across chunks): every member ends with the bits of its own solo run."""
    from stonewall.batch import Batch
    plan = [(SHAPES[0], "aa", 40), (SHAPES[1], "ab", 40), (SHAPES[2], "aa", 26)]
    b = Batch(dtype=dtype, chunk=7, mode="graph")
    ms = [b.add(_member(shape, seed, n, 9, dtype, pattern)) for (shape, seed), pattern, n in plan]
    assert b.autotune()[0] == "graph"              # installs the two-lattice member's configuration
    solo = []
    for (shape, seed), pattern, n in plan:
        r = _member(shape, seed, n, 9, dtype, pattern)
        r.advance(n, use_graphs=False)
        solo.append(_snapshot(r))
    b.advance(40)
    assert not b.pending()
    for want, m in zip(solo, ms):
        got = _snapshot(m)
        for u, v in zip(want[:3], got[:3]):
            np.testing.assert_array_equal(u, v)
        assert want[3:] == got[3:]


def test_aa_members_need_graph_mode(cuda):
    from stonewall.batch import Batch
    with pytest.raises(ValueError):
        Batch(dtype="f16", mode="persistent").add(_member(SHAPES[0][0], 1, 10, 2, "f16", "aa"))
