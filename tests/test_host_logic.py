"""Host-side logic that needs no GPU: accumulation schedules, request streams and footprints,
batch table layout, graph-batch argument checks."""
import ctypes

import numpy as np
import pytest


def test_acc_steps_counts_the_accumulating_steps():
    from stonewall.batch import acc_steps
    for t0 in range(0, 40, 3):
        for n in range(0, 25, 4):
            for n_spin in (0, 7, 30):
                for every in (1, 5):
                    want = sum(1 for t in range(t0, t0 + n) if t >= n_spin and (t - n_spin) % every == 0)
                    assert acc_steps(t0, n, n_spin, every) == want, (t0, n, n_spin, every)


def test_batch_entry_matches_the_c_layout():
    """sw_batch_entry in include/stonewall.h: 160 bytes, the fields at their C offsets (sw_capi.cu
    asserts the same sizes and offsets at compile time)."""
    from stonewall.batch import SwBatchEntry, SwBatchHeader
    assert ctypes.sizeof(SwBatchEntry) == 160
    assert ctypes.sizeof(SwBatchHeader) == 32
    assert SwBatchHeader.next_item.offset == 16 and SwBatchHeader.done_blocks.offset == 24
    off = {name: getattr(SwBatchEntry, name).offset for name, _ in SwBatchEntry._fields_}
    assert off["geom"] == 0 and off["item0"] == 16 and off["f"] == 32 and off["nu0"] == 88
    assert off["x_sponge"] == 112 and off["t0"] == 128 and off["steps_left"] == 136 and off["status"] == 144
    assert off["ghost"] == 152


def test_poisson_requests_are_seeded_and_in_range():
    from stonewall.serve import cells_of, footprint, poisson_requests
    a = poisson_requests(2.0, 60.0, seed=3)
    b = poisson_requests(2.0, 60.0, seed=3)
    assert [(r.t_arrive, r.H, r.steps, r.dtype) for r in a] == [(r.t_arrive, r.H, r.steps, r.dtype) for r in b]
    assert 60 < len(a) < 200                                   # about rate x duration
    t = np.array([r.t_arrive for r in a])
    assert (np.diff(t) > 0).all() and t[-1] < 60.0
    for r in a:
        assert 16 <= r.H <= 48 and 5000 <= r.steps <= 40000 and 0.03 <= r.U <= 0.06 and 0 <= r.porosity <= 0.5
        assert r.dtype in ("f32", "f16")
        cells = cells_of(r)
        per_cell = 2 * 19 * (4 if r.dtype == "f32" else 2) + 33
        assert footprint(r) >= per_cell * cells


def test_graph_batch_rejects_bad_arguments(native_lib):
    from stonewall import _native as N
    from stonewall.batch import SwBatchEntry, _bind
    L = _bind()
    tab = (SwBatchEntry * 2)()
    assert L.sw_batch_graph_run(None, ctypes.addressof(tab), 1, N.SW_F16_SHIFT, 10, None) == N.SW_ERR_BAD_ARG
    assert L.sw_batch_graph_create(None) == N.SW_ERR_BAD_ARG
    assert L.sw_batch_graph_destroy(None) == N.SW_OK
    assert L.sw_batch_graph_launches(None) == -1


def test_driver_derives_the_reference_grid_and_physics():
    """The CLI's grid, inlet speed, viscosity and step counts against what the reference's own
    main() recorded for the same flags (driver_small.npz meta, lbm3d.py:269-282)."""
    import json
    from conftest import golden
    from stonewall.driver import derive, parse
    d = golden("driver_small")
    meta, argv = json.loads(str(d["meta"])), json.loads(str(d["argv"]))
    p = derive(parse(argv))
    assert (p.nx, p.ny, p.nz, p.H, p.T, p.X0) == (meta["nx"], meta["ny"], meta["nz"], meta["H"], meta["T"], meta["X0"])
    assert (p.n_spin, p.n_avg, p.snap_every) == (meta["n_spin"], meta["n_avg"], meta["snap_every"])
    assert p.UH == pytest.approx(meta["UH"], rel=1e-12)
    assert p.nu0 == pytest.approx(meta["nu"], rel=1e-12)
    assert p.t_unit == pytest.approx(meta["steps_per_unit"], rel=1e-12)
    H = p.H
    ds3 = max(1, int(round(H / 13)))
    q_x0 = max(1, p.X0 - int(round(0.5 * H)))
    q_dims = [min(int(round(9.0 * H)), p.nx - 1 - q_x0) // ds3, p.ny // ds3, min(int(round(2.5 * H)), p.nz - 1) // ds3]
    assert meta["q3d"]["x0"] == q_x0 and meta["q3d"]["ds"] == ds3 and meta["q3d"]["dims"] == q_dims
    assert meta["y_mid"] == p.ny // 2 and meta["z_half"] == int(round(0.5 * H)) + 1


def test_server_admission_rules(monkeypatch):
    """First come first served under the byte cap, the resident-cells limit and the batch tables'
    capacity -- the admission logic alone, with stand-ins for the GPU solvers."""
    import concurrent.futures as cf
    from types import SimpleNamespace
    import stonewall.serve as S

    class FakeBatch:
        def __init__(self, cap):
            self.members, self.max_members = [], cap

        def add(self, s):
            self.members.append(s)

    def fake_solver(req, p, flag, device, pattern="ab"):
        return SimpleNamespace(grid=SimpleNamespace(cells=S.cells_of(req)), autotune=lambda: None, t=0,
                               n_total=req.steps)

    monkeypatch.setattr(S, "make_solver", fake_solver)
    reqs = S.poisson_requests(5.0, 4.0, seed=11, H_range=(16, 20), steps=(100, 200))
    done = cf.Future()
    done.set_result((None, None))
    srv = object.__new__(S.Server)
    srv.cap, srv.max_cells, srv.cells, srv.used, srv.device = 3.2 * max(S.footprint(r) for r in reqs), float("inf"), 0, 0.0, None
    srv.resident, srv._tuned, srv.pattern = {}, set(), "ab"
    srv.batches = {"f32": FakeBatch(2), "f16": FakeBatch(2)}
    queue = list(reqs)
    srv._admit(queue, {r.rid: done for r in reqs}, 0.0)
    admitted = [r for r in reqs if r.rid in srv.resident]
    assert admitted == reqs[:len(admitted)]                       # a prefix: first come first served
    assert srv.used <= srv.cap and all(len(b.members) <= 2 for b in srv.batches.values())
    nxt = queue[0]
    blocked_by_table = len(srv.batches[nxt.dtype].members) == 2
    blocked_by_cap = srv.used + S.footprint(nxt) > srv.cap
    assert blocked_by_table or blocked_by_cap                     # the head waits for a reason


@pytest.mark.parametrize("H,n,grid", [(16, 2000, (320, 64, 64)), (40, 40000, (800, 160, 160)),
                                      (64, 20000, (1280, 256, 256))])
def test_baseline_workload_parameters(H, n, grid):
    """The measured workloads: 20H x 4H x 4H, wall 0.75H thick at x = 5H, inlet 0.05 (z/H)^(1/7),
    Re_H = 1e4, Cs = 0.1; spin-up 20 H/U_H when the run is long enough, else the first 40 %."""
    from stonewall.params import baseline_params
    p = baseline_params(H, n)
    assert (p.nx, p.ny, p.nz) == grid
    assert (p.X0, p.T) == (5 * H, round(0.75 * H))
    assert p.UH == 0.05 and p.Cs == 0.1 and p.nu0 == pytest.approx(0.05 * H / 1e4)
    z = np.arange(p.nz) - 0.5
    want = (0.05 * np.clip(z / H, 0, None) ** (1 / 7)).astype(np.float32)
    want[0] = 0.0
    np.testing.assert_array_equal(p.uin, want)
    t_unit = H / 0.05
    assert p.n_spin == (int(20 * t_unit) if n >= 2 * int(20 * t_unit) else int(0.4 * n))
    assert p.n_spin + p.n_avg == n and p.x_sponge == p.nx - 3 * H
