"""Continuous-batching solve server: wall-design requests in, wall-load statistics out.

    python -m stonewall.serve [--minutes 30] [--rate 2] [--cap-gb 160] [--seed 0] ...

Requests arrive as a Poisson process (seeded).  Each asks for one wall: H
from U{H_lo..H_hi}, porosity U[0, 0.5], inlet speed U_H U[0.03, 0.06], a step
budget U[5000, 40000], a fresh seeded ellipsoid-packed stone mask, and a
storage type (fp32 or fp16-shifted, by a seeded coin).  The server:

  * builds masks on host threads while requests wait (CPU work off the loop);
  * admits queued requests first-come first-served while their device
    footprint (both lattices, flags, sums, force series) fits under the cap
    and the resident cells stay under --max-cells (beyond what saturates the
    GPU more residents only stretch every solve's time to result);
  * keeps every admitted solve resident and advances all of them together:
    one Batch per storage type advances all of its solves by `chunk` steps
    per loop iteration (graph mode by default: one CUDA graph of per-solve
    step chains on parallel branches; or the persistent batched kernel), so
    requests that arrive while others run join at the next chunk boundary;
  * retires finished solves (force series -> Cd, Cm statistics), frees their
    memory and admits more;
  * fails a solve whose steps reported a non-finite density or a device wait
    time-out (its status word, read at retirement and every few chunks for
    all residents): that request alone gets a failure result, is retired at
    once and counts as not completed; the others are unaffected.

Reported: p50 / p99 time-to-result (arrival to result), queueing and run
times, solves per hour over the run, GPU throughput.  A solve's result does
not depend on what it shared the GPU with (see stonewall.batch).

--plain serves the same stream the plain way for comparison: one request at a
time, first come first served, float32 storage whatever the request asked
for, one WallSolver per request (graph-replayed steps, no batching).
"""
import argparse
import concurrent.futures as cf
import json
import time
from dataclasses import dataclass, field

import numpy as np
import torch

from .batch import Batch
from .geometry import ellipsoid_wall
from .metrics import coefficients, device_recirculation_area, device_stats, recirculation_area, stats
from .params import baseline_params, flags_from_wall
from . import trace
from .solver import DeviceWaitTimeout, Diverged, WallSolver

DTYPE_BYTES = {"f32": 4, "f16": 2, "bf16": 2, "f64": 8}


@dataclass
class Request:
    rid: int
    t_arrive: float
    H: int
    porosity: float
    U: float
    steps: int
    dtype: str
    seed: int
    result: dict = field(default=None)


def poisson_requests(rate, duration, seed=0, H_range=(16, 48), porosity=(0.0, 0.5), U=(0.03, 0.06),
                     steps=(5000, 40000), f16_share=0.5):
    """Requests with exponential inter-arrival times (mean 1/rate) over [0, duration) seconds."""
    rng = np.random.default_rng(seed)
    out, t, rid = [], 0.0, 0
    while True:
        t += float(rng.exponential(1.0 / rate))
        if t >= duration:
            return out
        out.append(Request(rid=rid, t_arrive=t, H=int(rng.integers(H_range[0], H_range[1] + 1)),
                           porosity=float(rng.uniform(*porosity)), U=float(rng.uniform(*U)),
                           steps=int(rng.integers(steps[0], steps[1] + 1)),
                           dtype="f16" if rng.random() < f16_share else "f32", seed=1000 + rid))
        rid += 1


def footprint(req, pattern="ab"):
    """Device bytes a request holds while resident: two lattices (pattern "ab") or one and the
    outlet ghost (pattern "aa", in place), flags, segment classes, float64 sums, force series."""
    p = baseline_params(req.H, req.steps, UH=req.U)
    pitch = (p.nx + 31) // 32 * 32
    cells = pitch * p.ny * p.nz
    lattices = 2 * 19 * DTYPE_BYTES[req.dtype] * cells if pattern == "ab" else \
        19 * DTYPE_BYTES[req.dtype] * cells + 5 * p.ny * p.nz * DTYPE_BYTES[req.dtype]
    return lattices + 32 * cells + cells + cells // 32 + req.steps * p.nz * 16 + p.nz * 4


def cells_of(req):
    p = baseline_params(req.H, req.steps, UH=req.U)
    return p.nx * p.ny * p.nz


def prepare(req, mask_device=None):
    """A request's parameters and flag array (run on a worker thread).  mask_device: pack the stones
    on that GPU (the host packer's mask, on a stream of its own beside the solves)."""
    p = baseline_params(req.H, req.steps, UH=req.U)
    wall, frac = ellipsoid_wall(req.porosity, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=req.seed, device=mask_device)
    return p, flags_from_wall(wall, p.nx, p.ny, p.nz)


def make_solver(req, p, flag, device="cuda", pattern="ab"):
    s = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, req.steps, n_spin=p.n_spin, dtype=req.dtype,
                   device=device, pattern=pattern)
    s.init(noise=0.02, seed=req.seed, noise_kind="gauss")
    s.params = p
    return s


def failure_result(req, s, err, now):
    """The result of a request whose solve failed (diverged or timed out)."""
    return dict(failed=type(err).__name__, error=str(err), t_done=now, latency=now - req.t_arrive,
                wait=req.t_admit - req.t_arrive, run=now - req.t_admit, cells=s.grid.cells, steps_done=s.t)


def solve_stats(s):
    """The solve's Cd / Cm statistics and recirculation area, reduced on the GPU (56 bytes read back
    instead of the force series and the mean field)."""
    p = s.params
    st = device_stats(s.force, p.UH, p.H, p.ny, s.n_spin)
    st["recirc"] = device_recirculation_area(s.acc, s.n_acc, s.flags, p.H, p.X0, p.UH)
    return st


def solve_stats_host(s):
    """The same statistics from the downloaded force series and mean field (stonewall.metrics on the host)."""
    p = s.params
    co = coefficients(s.force_series(), p.UH, p.H, p.ny)
    st = stats(co["Cd"], co["Cm"], co["Cl"], s.n_spin)
    wall = s.flags.numpy() != 0
    st["recirc"] = recirculation_area(s.mean_field()[1][::2, ::2, ::2], wall[::2, ::2, ::2], p.H, p.X0, p.UH, p.ny)
    return st


class Server:
    def __init__(self, cap_bytes=160e9, chunk=50, max_members=256, device="cuda", workers=4, clock=time.monotonic,
                 mode="graph", max_cells=None, check_every=20, mask_device="cuda", pattern="ab"):
        """pattern "aa": every request is solved in place (one lattice: about half the memory of
        "ab"), which the graph batch mode runs."""
        if pattern not in ("ab", "aa") or (pattern == "aa" and mode != "graph"):
            raise ValueError("pattern is 'ab', or 'aa' with mode 'graph'")
        self.pattern = pattern
        self.cap = float(cap_bytes)
        self.max_cells = float(max_cells) if max_cells else float("inf")
        self.cells = 0
        # the persistent mode's table uploads are double-buffered by events, the graph mode's executable
        # graphs by the handle: neither needs the device idle between chunks
        self.persistent_sync = False
        self.chunk = int(chunk)
        self.device = torch.device(device)
        if mode == "graph":
            from .batch import GRAPH_MAX
            max_members = min(max_members, GRAPH_MAX)
        self.batches = {dt: Batch(dtype=dt, chunk=chunk, max_members=max_members, device=device, mode=mode)
                        for dt in ("f32", "f16")}
        self._tuned = set()
        self.pool = cf.ThreadPoolExecutor(max_workers=workers)
        self.clock = clock
        self.check_every = int(check_every)       # loop iterations between status checks of all residents
        self.mask_device = mask_device             # where the stone masks are packed (None: host)
        self.failed = 0
        self.resident = {}                         # rid -> (request, solver, bytes)
        self.used = 0.0
        self.log = []

    def _prepare(self, req):
        out = prepare(req, self.mask_device)
        req.t_prepared = self.clock() - self._t0              # arrival -> mask ready: the preparation lag
        return out

    def _admit(self, queue, prepared, now):
        while queue:
            req = queue[0]
            fut = prepared.get(req.rid)
            if fut is None or not fut.done():
                return                               # head still being prepared: keep FIFO order
            need = footprint(req, self.pattern)
            if need > self.cap:
                raise ValueError(f"request {req.rid} needs {need/1e9:.1f} GB, more than the cap")
            if self.used + need > self.cap:
                return
            if self.resident and self.cells + cells_of(req) > self.max_cells:
                return
            b = self.batches[req.dtype]
            if len(b.members) >= b.max_members:           # the batch's table (graph mode: 256 walls) is full
                return
            queue.pop(0)
            p, flag = fut.result()
            del prepared[req.rid]
            s = make_solver(req, p, flag, self.device, self.pattern)
            if req.dtype not in self._tuned:             # the storage type's step configurations, once
                s.autotune()
                self._tuned.add(req.dtype)
            self.batches[req.dtype].add(s)
            self.resident[req.rid] = (req, s, need)
            self.used += need
            self.cells += s.grid.cells
            req.t_admit = now

    def _release(self, rid):
        req, s, need = self.resident.pop(rid)
        self.batches[req.dtype].remove(s)
        self.used -= need
        self.cells -= s.grid.cells
        return req, s

    def _fail(self, rid, err):
        req, s = self._release(rid)
        req.result = failure_result(req, s, err, self.clock() - self._t0)
        self.failed += 1

    def _check_residents(self):
        """Read every resident's status word (one gather per batch) and fail the ones that report."""
        for b in self.batches.values():
            if not b.members:
                continue
            bad = b.failures()
            for rid, (req, s, need) in list(self.resident.items()):
                if s in bad:
                    self._fail(rid, bad[s])

    def _retire(self, now):
        done = [rid for rid, (req, s, need) in self.resident.items() if s.t >= s.n_total]
        for rid in done:
            req, s, need = self.resident[rid]
            st = solve_stats(s)                    # reduced on the GPU: waits for the solve's last chunk
            err = s.status_error()
            if err is not None:
                self._fail(rid, err)
                continue
            req, s = self._release(rid)
            now = self.clock() - self._t0
            req.result = dict(stats=st, t_done=now, latency=now - req.t_arrive, wait=req.t_admit - req.t_arrive,
                              run=now - req.t_admit, cells=s.grid.cells,
                              prep=getattr(req, "t_prepared", req.t_admit) - req.t_arrive)
            del s
        return len(done)

    def serve(self, requests, max_seconds=None, drain=True, log_every=30.0):
        """Replay the request stream in real time.  Returns the requests (with .result when done)."""
        reqs = sorted(requests, key=lambda r: r.t_arrive)
        queue, prepared = [], {}
        t0 = self._t0 = self.clock()
        i = 0
        last_log = 0.0
        self.max_used = 0.0
        it = 0
        while True:
            it += 1
            now = self.clock() - t0
            while i < len(reqs) and reqs[i].t_arrive <= now:
                queue.append(reqs[i])
                prepared[reqs[i].rid] = self.pool.submit(self._prepare, reqs[i])
                i += 1
            with trace.range("server admit"):
                self._admit(queue, prepared, now)
            active = [b for b in self.batches.values() if b.pending()]
            self.max_used = max(self.max_used, self.used)
            if active:
                for b in active:             # enqueued; the host goes on admitting and retiring meanwhile
                    b.advance(self.chunk)    # (step counts are host-side; a batch keeps <= 2 chunks queued)
                if self.persistent_sync:
                    torch.cuda.synchronize()
            else:
                if i >= len(reqs) and not queue:
                    break
                time.sleep(0.005)
            if self.check_every and it % self.check_every == 0 and self.resident:
                with trace.range("server status check"):
                    self._check_residents()
            now = self.clock() - t0
            with trace.range("server retire"):
                self._retire(now)
            if max_seconds is not None and now > max_seconds and not drain:
                break
            if max_seconds is not None and now > max_seconds and drain and i < len(reqs):
                reqs = reqs[:i]                          # stop accepting new arrivals, finish the rest
            if now - last_log > log_every:
                last_log = now
                self.log.append(dict(t=round(now, 1), resident=len(self.resident), queued=len(queue),
                                     used_gb=round(self.used / 1e9, 1),
                                     done=sum(1 for r in reqs[:i] if r.result is not None)))
        self.pool.shutdown(wait=False)
        self.unfinished = dict(queued=len(queue), resident=len(self.resident))
        return reqs

    @staticmethod
    def summary(reqs, elapsed):
        failed = [r for r in reqs if r.result is not None and "failed" in r.result]
        done = [r for r in reqs if r.result is not None and "failed" not in r.result]
        lat = np.array([r.result["latency"] for r in done]) if done else np.zeros(1)
        wait = np.array([r.result["wait"] for r in done]) if done else np.zeros(1)
        prep = np.array([r.result.get("prep", 0.0) for r in done]) if done else np.zeros(1)
        cell_steps = sum(r.result["cells"] * r.steps for r in done)
        return dict(requests=len(reqs), completed=len(done), elapsed_s=round(elapsed, 1),
                    solves_per_hour=round(len(done) / elapsed * 3600, 1) if elapsed > 0 else 0.0,
                    p50_latency_s=round(float(np.percentile(lat, 50)), 2),
                    p99_latency_s=round(float(np.percentile(lat, 99)), 2),
                    p50_wait_s=round(float(np.percentile(wait, 50)), 2),
                    p50_prep_s=round(float(np.percentile(prep, 50)), 3),
                    p99_prep_s=round(float(np.percentile(prep, 99)), 3),
                    mean_glups=round(cell_steps / elapsed / 1e9, 2) if elapsed > 0 else 0.0,
                    f16_share=round(np.mean([r.dtype == "f16" for r in done]), 3) if done else 0.0,
                    failed=len(failed))


class PlainServer:
    """The plain form: one request at a time, first come first served, float32, no batching."""

    def __init__(self, chunk=50, device="cuda", workers=4, clock=time.monotonic, mask_device="cuda"):
        self.chunk, self.device, self.clock = int(chunk), torch.device(device), clock
        self.mask_device = mask_device
        self.pool = cf.ThreadPoolExecutor(max_workers=workers)
        self.log, self.max_used = [], 0.0

    def serve(self, requests, max_seconds=None, drain=True, log_every=30.0):
        reqs = sorted(requests, key=lambda r: r.t_arrive)
        queue, prepared = [], {}
        t0 = self.clock()
        i, tuned = 0, False
        while True:
            now = self.clock() - t0
            while i < len(reqs) and reqs[i].t_arrive <= now:
                queue.append(reqs[i])
                prepared[reqs[i].rid] = self.pool.submit(prepare, reqs[i], self.mask_device)
                i += 1
            if max_seconds is not None and now > max_seconds and not drain:
                break
            if not queue:
                if i >= len(reqs):
                    break
                time.sleep(0.005)
                continue
            req = queue.pop(0)
            p, flag = prepared.pop(req.rid).result()
            req.t_admit = self.clock() - t0
            s = WallSolver(flag, p.uin, p.nu0, p.Cs, p.x_sponge, req.steps, n_spin=p.n_spin, dtype="f32",
                           device=self.device, chunk=self.chunk)
            s.init(noise=0.02, seed=req.seed, noise_kind="gauss")
            s.params = p
            if not tuned:
                s.autotune()
                tuned = True
            try:
                s.advance(req.steps)                     # reads the status word at the end
            except (Diverged, DeviceWaitTimeout) as err:
                req.result = failure_result(req, s, err, self.clock() - t0)
                del s
                continue
            st = solve_stats(s)
            now = self.clock() - t0
            req.result = dict(stats=st, t_done=now, latency=now - req.t_arrive, wait=req.t_admit - req.t_arrive,
                              run=now - req.t_admit, cells=s.grid.cells)
            self.max_used = max(self.max_used, s.memory_bytes())
            del s
            if max_seconds is not None and now > max_seconds and drain and i < len(reqs):
                reqs = reqs[:i]
        self.pool.shutdown(wait=False)
        self.unfinished = dict(queued=len(queue), resident=0)
        return reqs


def run_alone(req, device="cuda", mode="graph", pattern="ab"):
    """The same request solved by itself (its own batch), for alone-vs-mix checks and FP64 references."""
    p, flag = prepare(req)
    s = make_solver(req, p, flag, device, pattern)
    b = Batch(dtype=req.dtype, chunk=50, max_members=4, device=device, mode=mode)
    b.add(s)
    b.run()
    return s


def main(argv=None):
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--minutes", type=float, default=30.0, help="arrival window")
    ap.add_argument("--rate", type=float, default=2.0, help="mean arrivals per second")
    ap.add_argument("--cap-gb", type=float, default=160.0)
    ap.add_argument("--seed", type=int, default=0)
    ap.add_argument("--h-lo", type=int, default=16)
    ap.add_argument("--h-hi", type=int, default=48)
    ap.add_argument("--steps-lo", type=int, default=5000)
    ap.add_argument("--steps-hi", type=int, default=40000)
    ap.add_argument("--f16-share", type=float, default=0.5)
    ap.add_argument("--chunk", type=int, default=50)
    ap.add_argument("--mode", default="graph", choices=["graph", "persistent"], help="batch mode")
    ap.add_argument("--max-cells", type=float, default=1.2e8, help="resident cells admitted at most (0 = no limit)")
    ap.add_argument("--plain", action="store_true", help="serve the plain way (one float32 solve at a time)")
    ap.add_argument("--no-drain", action="store_true", help="stop at the end of the window (unfinished solves count as not done)")
    ap.add_argument("--fp64-check", type=int, default=0, help="re-run this many completed requests in float64")
    ap.add_argument("--host-masks", action="store_true", help="pack the stone masks on the host instead of the GPU")
    ap.add_argument("--pattern", default="ab", choices=["ab", "aa"],
                    help="aa: solve every request in place (one lattice, graph mode)")
    a = ap.parse_args(argv)
    reqs = poisson_requests(a.rate, a.minutes * 60.0, seed=a.seed, H_range=(a.h_lo, a.h_hi),
                            steps=(a.steps_lo, a.steps_hi), f16_share=a.f16_share)
    if a.plain:
        srv = PlainServer(chunk=a.chunk, mask_device=None if a.host_masks else "cuda")
    else:
        srv = Server(cap_bytes=a.cap_gb * 1e9, chunk=a.chunk, mode=a.mode, max_cells=a.max_cells or None,
                     mask_device=None if a.host_masks else "cuda", pattern=a.pattern)
    t0 = time.monotonic()
    out = srv.serve(reqs, max_seconds=a.minutes * 60.0, drain=not a.no_drain)
    elapsed = time.monotonic() - t0
    summ = Server.summary(out, elapsed)
    summ.update(form="plain (float32, one at a time)" if a.plain else f"batched ({a.mode}, pattern {a.pattern})",
                unfinished_at_end=srv.unfinished,
                max_resident_gb=round(srv.max_used / 1e9, 2), cap_gb=a.cap_gb, arrivals_per_s=a.rate,
                window_minutes=a.minutes, seed=a.seed, drained=not a.no_drain)
    if a.fp64_check:
        done = sorted([r for r in out if r.result is not None and "failed" not in r.result],
                      key=lambda r: r.H * r.steps)[:a.fp64_check]
        errs = []
        for r in done:
            ref = run_alone(Request(rid=r.rid, t_arrive=r.t_arrive, H=r.H, porosity=r.porosity, U=r.U, steps=r.steps,
                                    dtype="f64", seed=r.seed))
            rs = solve_stats(ref)
            errs.append(dict(rid=r.rid, dtype=r.dtype, H=r.H,
                             Cd=abs(r.result["stats"]["Cd"] - rs["Cd"]) / abs(rs["Cd"]),
                             CdMax=abs(r.result["stats"]["CdMax"] - rs["CdMax"]) / abs(rs["CdMax"])))
            del ref
            torch.cuda.empty_cache()
        summ["fp64_check"] = errs
    summ["log"] = srv.log[-10:]
    print(json.dumps(summ), flush=True)
    return summ


if __name__ == "__main__":
    main()
