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
