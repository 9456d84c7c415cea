"""Wall-load coefficients and their statistics on the GPU (sw_coefficients, sw_coef_stats) against
stonewall.metrics on the host, which is pinned to the reference's own postprocess.py output
(test_oracle_golden.py).  Reference: lbm3d.py:396-407 (Cd, Cl, Cm series), postprocess.py:65-82
(mean / peak / std of Cd, mean / peak Cm, mean Cl after the spin-up).  The device sums the levels
and the steps in another order than NumPy, so the bar is 1e-12 relative, not bit equality.
The recirculation area (sw_recirc_count, export3d.py:169-184) is float32 element-wise work in
the host's order, so there the bar is equality."""
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


def _acc_with_mean(grid, mean_ref, n_acc):
    """An Accum whose sums are n_acc * mean_ref ((4, nx, ny, nz) float64, reference layout)."""
    import torch
    from stonewall.fields import Accum
    a = Accum(grid)
    dev = a.data.view(4, grid.nz, grid.ny, grid.pitch)
    dev[:, :, :, :grid.nx] = torch.from_numpy(mean_ref * n_acc).permute(0, 3, 2, 1).to(dev.device)
    return a


@pytest.mark.parametrize("shape,H,X0,seed", [((160, 32, 33), 8, 40, 0), ((97, 13, 9), 4, 21, 1),
                                             ((61, 20, 40), 6, 18, 2), ((50, 8, 64), 16, 7, 3)])
def test_device_recirculation_area_equals_the_host(shape, H, X0, seed, cuda):
    """Mean fields near zero (so the blur's rounding decides cells), stones and ground, odd sizes,
    a box clipped by the outlet (last case: X0 + 10 H past nx) and by the height (first: 2 H < nz)."""
    from gpu_helpers import make_mask
    from stonewall.fields import Flags, Grid
    from stonewall.metrics import device_recirculation_area, recirculation_area
    nx, ny, nz = shape
    rng = np.random.default_rng(seed)
    flag = make_mask(nx, ny, nz, seed)
    UH, n_acc = 0.05, 7
    mean = rng.standard_normal((4, nx, ny, nz)) * 0.01 + 0.002
    g = Grid(nx, ny, nz)
    acc, flags = _acc_with_mean(g, mean, n_acc), Flags(g, flag)
    sums = acc.numpy()
    want = recirculation_area((sums[1] / n_acc)[::2, ::2, ::2], (flag != 0)[::2, ::2, ::2], H, X0, UH, ny)
    got = device_recirculation_area(acc, n_acc, flags, H, X0, UH)
    assert want > 0
    assert got == want


def test_device_recirculation_area_of_a_solve(cuda):
    """A real solve (H = 16, 600 steps, sums after the spin-up): the device area equals the host's
    on the downloaded mean field, as study.py computes it."""
    from stonewall.metrics import device_recirculation_area, recirculation_area
    from stonewall.serve import Request, make_solver, prepare
    req = Request(rid=0, t_arrive=0.0, H=16, porosity=0.2, U=0.05, steps=600, dtype="f32", seed=5)
    p, flag = prepare(req)
    s = make_solver(req, p, flag)
    s.advance(600)
    assert s.n_acc > 0
    mean_ux = s.mean_field()[1]
    want = recirculation_area(mean_ux[::2, ::2, ::2], (flag != 0)[::2, ::2, ::2], p.H, p.X0, p.UH, p.ny)
    got = device_recirculation_area(s.acc, s.n_acc, s.flags, p.H, p.X0, p.UH)
    assert got == want
