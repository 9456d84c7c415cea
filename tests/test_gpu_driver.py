"""The driver-level contract: lbm3d.py's CLI end to end, graph replay, checkpoints.

driver_small.npz is what the reference's own main() wrote for a 32x8x13 grid
(H = 4, 10 steps, porosity 0.2, seed 7; make_golden.py).  Our driver, given
the same flags, must write the same file: identical geometry outputs and
metadata, coefficient series and mean fields within the float32 parity bar.
"""
import json
import os

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def _run_driver(tmp_path, argv):
    from stonewall.driver import main
    assert main(argv + ["--out", str(tmp_path)]) == 0
    return dict(np.load(os.path.join(tmp_path, "g.npz")))


def _reference_argv(d):
    argv = json.loads(str(d["argv"]))
    argv[argv.index("--device") + 1] = "cuda"
    return argv


def test_driver_matches_reference_main(tmp_path, cuda):
    d = golden("driver_small")
    got = _run_driver(tmp_path, _reference_argv(d))
    _assert_matches_reference(got, d)


def test_driver_resumes_a_reference_checkpoint(tmp_path, cuda):
    """The checkpoint the reference's main() wrote at step 5 (its float32 files, lbm3d.py:342-355)
    resumed by this driver: the finished outputs equal the reference's uninterrupted run."""
    d, c = golden("driver_small"), golden("driver_small_ckpt")
    ck = tmp_path / "g.ckpt"
    ck.mkdir()
    for k in ("f", "force", "uacc", "snaps_xz", "snaps_xy", "snaps_q"):
        np.save(ck / f"{k}.npy", c[k])
    (ck / "state.json").write_text(str(c["state"]))
    assert json.loads(str(c["state"]))["t"] == 5
    got = _run_driver(tmp_path, _reference_argv(d))
    assert not ck.exists()                                     # removed once the run completed
    _assert_matches_reference(got, d)


def _assert_matches_reference(got, d):
    for k in ("wall_xz", "wall_xy", "wall_front", "wall_top", "wall_ds2"):
        np.testing.assert_array_equal(got[k], d[k], err_msg=k)
    m_ref, m_got = json.loads(str(d["meta"])), json.loads(str(got["meta"]))
    for k in ("nx", "ny", "nz", "H", "T", "X0", "UH", "nu", "n_spin", "n_avg", "snap_every", "y_mid", "z_half",
              "porosity", "q3d"):
        assert m_got[k] == m_ref[k], k
    for k in ("Cd", "Cl", "Cm"):
        scale = np.abs(d[k]).max()
        np.testing.assert_allclose(got[k], d[k], rtol=1e-4, atol=1e-5 * scale, err_msg=k)
    np.testing.assert_allclose(got["fx_profile"], d["fx_profile"], rtol=1e-4,
                               atol=1e-5 * np.abs(d["fx_profile"]).max())
    for k in ("mean_xz_mid", "mean_xy_half"):
        np.testing.assert_allclose(got[k], d[k], rtol=1e-5, atol=1e-6, err_msg=k)
    a, b = got["mean_xz_spanavg"], d["mean_xz_spanavg"]
    np.testing.assert_array_equal(np.isnan(a), np.isnan(b))
    np.testing.assert_allclose(a[~np.isnan(a)], b[~np.isnan(b)], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(got["mean3d_ds2"].astype(np.float32), d["mean3d_ds2"].astype(np.float32),
                               rtol=2e-3, atol=1e-4)
    # snapshots: float16 planes of velocities that agree to 1e-5 round to the same or an adjacent
    # float16; Q frames are log-quantised to uint8, a level apart at most
    for k in ("snaps_xz", "snaps_xy"):
        assert got[k].shape == d[k].shape and got[k].dtype == np.float16, k
        np.testing.assert_allclose(got[k].astype(np.float32), d[k].astype(np.float32), rtol=1e-3, atol=1e-6,
                                   err_msg=k)
    assert got["snaps_q"].shape == d["snaps_q"].shape and got["snaps_q"].dtype == np.uint8
    assert d["snaps_q"].max() > 0
    assert np.abs(got["snaps_q"].astype(int) - d["snaps_q"].astype(int)).max() <= 1


def _solver(flag, uin, n_total, n_spin, chunk=8, dtype="f32"):
    from stonewall.solver import WallSolver
    s = WallSolver(flag, uin, 2e-3, 0.1, flag.shape[0] - 8, n_total, n_spin=n_spin, dtype=dtype, chunk=chunk)
    return s.init(noise=0.03, seed=4, noise_kind="gauss")


def test_graph_replay_equals_eager(cuda):
    from gpu_helpers import inlet, make_mask
    flag = make_mask(40, 12, 14, 9)
    uin = inlet(14, 4)
    a = _solver(flag, uin, 60, 13)
    a.advance(60, use_graphs=False)
    b = _solver(flag, uin, 60, 13)
    b.advance(60)
    assert b.launches >= 60
    np.testing.assert_array_equal(a.state.numpy(), b.state.numpy())
    np.testing.assert_array_equal(a.force.data.cpu().numpy(), b.force.data.cpu().numpy())
    np.testing.assert_array_equal(a.acc.numpy(), b.acc.numpy())
    assert a.n_acc == b.n_acc == len(range(13, 60, 5))


@pytest.mark.parametrize("background", [False, True])
@pytest.mark.parametrize("dtype", ["f32", "f16"])
def test_resume_is_bit_identical(tmp_path, cuda, dtype, background):
    """Checkpoint at step 25, resume in a new solver, finish: same forces, sums and state.  With
    background=True the writing overlaps 20 more steps of the solver that took it."""
    from gpu_helpers import inlet, make_mask
    flag = make_mask(40, 12, 14, 10)
    uin = inlet(14, 4)
    full = _solver(flag, uin, 50, 10, dtype=dtype)
    full.advance(50)
    part = _solver(flag, uin, 50, 10, dtype=dtype)
    part.advance(25)
    ck = str(tmp_path / "c.ckpt")
    part.save_checkpoint(ck, dict(a=1), background=background)
    if background:
        part.advance(20)                           # overwrites the state the checkpoint was taken from
        part.wait_checkpoint()
    res = _solver(flag, uin, 50, 10, dtype=dtype)
    info = res.load_checkpoint(ck, dict(a=1))
    assert info["t"] == 25
    res.advance(25)
    fluid = np.broadcast_to(flag == 0, (19,) + flag.shape)
    np.testing.assert_array_equal(res.state.numpy()[fluid], full.state.numpy()[fluid])
    np.testing.assert_array_equal(res.force.data.cpu().numpy(), full.force.data.cpu().numpy())
    np.testing.assert_array_equal(res.sums(), full.sums())
    with pytest.raises(ValueError):
        _solver(flag, uin, 50, 10, dtype=dtype).load_checkpoint(ck, dict(a=2))
