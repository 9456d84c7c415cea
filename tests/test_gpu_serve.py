"""The solve server: admission under a memory cap, continuous batching, alone vs in the mix.

Small walls (H 8..12) and short budgets keep this to seconds; the cap is set so
that only a few solves fit at once and the others wait in the queue.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _requests():
    from stonewall.serve import poisson_requests
    return poisson_requests(rate=20.0, duration=0.6, seed=3, H_range=(8, 12), steps=(60, 200), f16_share=0.5)


def test_server_completes_everything_under_the_cap(cuda):
    from stonewall.serve import Server, footprint
    reqs = _requests()
    assert len(reqs) >= 6 and {r.dtype for r in reqs} == {"f32", "f16"}
    cap = 2.5 * max(footprint(r) for r in reqs)
    srv = Server(cap_bytes=cap, chunk=16)
    out = srv.serve(reqs)
    assert all(r.result is not None for r in out)
    assert srv.max_used <= cap
    assert srv.used == 0 and not srv.resident
    admits = sorted(out, key=lambda r: r.t_admit)
    assert [r.rid for r in admits] == [r.rid for r in sorted(out, key=lambda r: r.t_arrive)]   # first come first served
    summ = Server.summary(out, 10.0)
    assert summ["completed"] == len(reqs) and summ["p99_latency_s"] >= summ["p50_latency_s"]


@pytest.mark.parametrize("mode", ["graph", "persistent"])
def test_result_is_the_same_alone_and_in_the_mix(mode, cuda):
    from stonewall.serve import Server, run_alone, solve_stats
    reqs = _requests()
    srv = Server(cap_bytes=1e12, chunk=16, mode=mode)
    out = srv.serve(reqs)
    for r in out[:4]:
        alone = run_alone(r, mode=mode)
        st = solve_stats(alone)
        for k, v in st.items():
            assert v == r.result["stats"][k] or (np.isnan(v) and np.isnan(r.result["stats"][k])), (r.rid, k)


def test_server_solves_in_place(cuda):
    """pattern "aa": every request on one lattice (smaller footprint), odd chunks carry the AA
    parity; each result equals the same request solved alone in place."""
    from stonewall.serve import Server, footprint, run_alone, solve_stats
    reqs = _requests()
    assert all(footprint(r, "aa") < footprint(r) for r in reqs)
    srv = Server(cap_bytes=1e12, chunk=15, pattern="aa")
    out = srv.serve(reqs)
    assert all(r.result is not None and "failed" not in r.result for r in out)
    for r in out[:3]:
        st = solve_stats(run_alone(r, pattern="aa"))
        for k, v in st.items():
            assert v == r.result["stats"][k] or (np.isnan(v) and np.isnan(r.result["stats"][k])), (r.rid, k)
    with pytest.raises(ValueError):
        Server(pattern="aa", mode="persistent")


def test_plain_form_serves_the_same_stream(cuda):
    """The comparison form: one float32 solve at a time, first come first served."""
    from stonewall.serve import PlainServer, Server
    reqs = _requests()
    out = PlainServer(chunk=16).serve(reqs)
    assert all(r.result is not None for r in out)
    done = sorted(out, key=lambda r: r.result["t_done"])
    assert [r.rid for r in done] == [r.rid for r in sorted(out, key=lambda r: r.t_arrive)]
    assert all(r.result["wait"] >= 0 for r in out)
    summ = Server.summary(out, 10.0)
    assert summ["completed"] == len(reqs)


def test_resident_cells_cap_limits_concurrency(cuda):
    from stonewall.serve import Server, cells_of
    reqs = _requests()
    cap_cells = 1.5 * max(cells_of(r) for r in reqs)
    srv = Server(cap_bytes=1e12, chunk=16, max_cells=cap_cells)
    seen = []
    orig = srv._admit

    def spy(queue, prepared, now):
        orig(queue, prepared, now)
        seen.append(srv.cells)
    srv._admit = spy
    out = srv.serve(reqs)
    assert all(r.result is not None for r in out)
    assert max(seen) <= cap_cells


@pytest.mark.parametrize("plain", [False, True])
def test_command_line_end_to_end(plain, cuda):
    from stonewall.serve import main
    argv = ["--minutes", "0.01", "--rate", "300", "--h-lo", "8", "--h-hi", "10", "--steps-lo", "60",
            "--steps-hi", "120", "--chunk", "16", "--seed", "5"] + (["--plain"] if plain else ["--fp64-check", "1"])
    summ = main(argv)
    assert summ["completed"] == summ["requests"] > 0
    assert summ["p99_latency_s"] >= summ["p50_latency_s"] >= 0
    assert summ["form"].startswith("plain" if plain else "batched")
    if not plain:
        assert len(summ["fp64_check"]) == 1 and summ["fp64_check"][0]["Cd"] < 0.05
