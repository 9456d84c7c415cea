"""Wall-load coefficients and their statistics on the GPU (sw_coefficients, sw_coef_stats) against
stonewall.metrics on the host, which is pinned to the reference's own postprocess.py output
(test_oracle_golden.py).  Reference: lbm3d.py:396-407 (Cd, Cl, Cm series), postprocess.py:65-82
(mean / peak / std of Cd, mean / peak Cm, mean Cl after the spin-up).  The device sums the levels
and the steps in another order than NumPy, so the bar is 1e-12 relative, not bit equality."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RTOL = 1e-12


def _series(n, nz, seed):
    """A fixed-point force series (n, nz, 2) with drag-like mean and fluctuations."""
    import torch
    from stonewall.fields import ForceSeries
    rng = np.random.default_rng(seed)
    f = np.empty((n, nz, 2))
    f[:, :, 0] = 0.02 + 0.01 * rng.standard_normal((n, nz)) + 0.005 * np.sin(np.arange(n))[:, None]
    f[:, :, 1] = 0.003 * rng.standard_normal((n, nz))
    fs = ForceSeries(n, nz)
    fs.data.copy_(torch.from_numpy(np.rint(f * 2.0 ** 40).astype(np.int64)))
    return fs


@pytest.mark.parametrize("n,nz,n_spin", [(1000, 160, 400), (40000, 193, 16000), (7, 33, 0), (5, 9, 4)])
def test_device_coefficients_and_stats_match_the_host(n, nz, n_spin, cuda):
    from stonewall.metrics import coefficients, device_coefficients, device_stats, stats
    fs = _series(n, nz, n + nz)
    UH, H, ny = 0.05, 40.0, 160
    host = coefficients(fs.numpy(), UH, H, ny)
    dev = device_coefficients(fs, UH, H, ny).cpu().numpy()
    for k, name in enumerate(("Cd", "Cl", "Cm")):
        np.testing.assert_allclose(dev[k], host[name], rtol=RTOL, atol=RTOL * np.abs(host[name]).max())
    want = stats(host["Cd"], host["Cm"], host["Cl"], n_spin)
    got = device_stats(fs, UH, H, ny, n_spin)
    for key, v in want.items():
        assert abs(got[key] - v) <= RTOL * max(abs(v), 1e-300) or got[key] == v, (key, got[key], v)


def test_empty_window_gives_nan(cuda):
    from stonewall.metrics import device_stats
    fs = _series(10, 8, 1)
    got = device_stats(fs, 0.05, 16.0, 64, 10)
    assert all(np.isnan(v) for v in got.values())


def test_solver_statistics_on_device_equal_the_host(cuda):
    """A real solve (320x64x64, 300 steps): the server's device statistics against the host path."""
    from stonewall.serve import Request, make_solver, prepare, solve_stats, solve_stats_host
    req = Request(rid=0, t_arrive=0.0, H=16, porosity=0.2, U=0.05, steps=300, dtype="f16", seed=3)
    p, flag = prepare(req)
    s = make_solver(req, p, flag)
    s.advance(300)
    got, want = solve_stats(s), solve_stats_host(s)
    for key, v in want.items():
        assert abs(got[key] - v) <= RTOL * abs(v), (key, got[key], v)
