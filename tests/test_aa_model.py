"""The AA-pattern access plan (tests/aa_model.py) against the ping-pong pull, on the CPU.

Random stones, interior ground cells, stones in the inlet, outlet and top
planes, the periodic edge: after one odd and one even AA step the state must
equal two ping-pong steps exactly, and the odd step must write every slot at
most once and never into a slot another cell reads.
"""
import numpy as np
import pytest

from aa_model import aa_two_steps, pingpong_step


def _mask(shape, seed, density):
    rng = np.random.default_rng(seed)
    f = (rng.random(shape) < density).astype(np.uint8)
    f[:, :, 0] = 2
    f[0, 0, 1] = 1
    f[-1, -1, -1] = 1
    f[shape[0] // 2, 0, -1] = 1
    return f


@pytest.mark.parametrize("shape,seed,density", [((6, 4, 5), 0, 0.15), ((7, 3, 4), 1, 0.3), ((5, 5, 6), 2, 0.0),
                                                ((8, 2, 4), 3, 0.25), ((4, 1, 3), 4, 0.2), ((9, 5, 7), 5, 0.35),
                                                ((6, 6, 4), 6, 0.45), ((3, 2, 2), 7, 0.1)])
def test_aa_two_steps_equal_pingpong(shape, seed, density):
    flag = _mask(shape, seed, density)
    rng = np.random.default_rng(seed + 100)
    S = rng.random((19,) + shape)
    M = rng.standard_normal((19, 19))
    want = pingpong_step(pingpong_step(S, flag, M), flag, M)
    got, problems = aa_two_steps(S, flag, M)
    assert problems == []
    fluid = np.broadcast_to(flag == 0, want.shape)
    np.testing.assert_allclose(got[fluid], want[fluid], rtol=1e-12, atol=1e-12)


def test_aa_plan_on_generated_masks():
    """The same property on masks drawn by hypothesis (shapes down to one row, dense and empty
    stone fills, stones anywhere including the inlet, outlet and top planes)."""
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=40, deadline=None, derandomize=True)
    @hyp.given(nx=st.integers(3, 7), ny=st.integers(1, 4), nz=st.integers(2, 5), seed=st.integers(0, 10 ** 6),
               density=st.floats(0.0, 0.6))
    def check(nx, ny, nz, seed, density):
        rng = np.random.default_rng(seed)
        flag = (rng.random((nx, ny, nz)) < density).astype(np.uint8)
        flag[:, :, 0] = 2
        S = rng.random((19, nx, ny, nz))
        M = rng.standard_normal((19, 19))
        want = pingpong_step(pingpong_step(S, flag, M), flag, M)
        got, problems = aa_two_steps(S, flag, M)
        assert problems == []
        fluid = np.broadcast_to(flag == 0, want.shape)
        np.testing.assert_allclose(got[fluid], want[fluid], rtol=1e-12, atol=1e-12)

    check()


def _segment_checked(flag, x_lo, x_hi, y, z):
    """k_build_tiles' CHECK class of the cells x_lo..x_hi-1 of row (y, z): a cell is not fluid, or a
    fluid cell past the inlet has a pull source that is not fluid (lbm3d.py:77-95)."""
    from aa_model import pull_source
    nx = flag.shape[0]
    for x in range(x_lo, min(x_hi, nx)):
        if flag[x, y, z] != 0:
            return True
        if x > 0 and any(pull_source(flag, x, y, z, i)[2] for i in range(1, 19)):
            return True
    return False


@pytest.mark.parametrize("seed", range(6))
def test_inlet_cell_targets_of_open_first_pairs(seed):
    """The 16-bit odd step runs the first 64-cell pair of a row on the two-cell path when neither of
    its segments is checked; its inlet cell then writes its c_x = +1 populations to column 1 without
    a flag test.  Those targets are pull sources of the row's x = 1 cell, so they are fluid."""
    from aa_model import C, odd_targets
    rng = np.random.default_rng(seed)
    nx, ny, nz = 70, 24, 9
    flag = (rng.random((nx, ny, nz)) < 0.0005 * (1 + seed)).astype(np.uint8)
    for _ in range(6):                                   # stones in columns 0 and 1 next to open rows
        flag[int(rng.integers(0, 2)), int(rng.integers(0, ny)), int(rng.integers(1, nz))] = 1
    flag[:, :, 0] = 2
    open_rows = 0
    for y in range(ny):
        for z in range(1, nz - 1):
            if flag[0, y, z] != 0 or _segment_checked(flag, 0, 32, y, z) or _segment_checked(flag, 32, 64, y, z):
                continue
            open_rows += 1
            for k in range(19):
                if C[k][0] != 1:
                    continue
                t = (1, (y + C[k][1]) % ny, z + C[k][2])
                assert flag[t] == 0, (y, z, k, t)
                assert (k, t) in odd_targets(flag, (0, y, z), k)
    assert open_rows > 0
