"""Batch: many wall solves advanced together on one GPU.

Each member is a WallSolver (its own buffers, mask, inlet, force series and
sums); the batch describes all members in a table (sw_batch_entry,
include/stonewall.h).  Two modes advance the table:

  "persistent": the table lives in device memory and sw_batch_step walks
      every member's work in one launch of (SMs x resident blocks) per step.
      Runs of `chunk` steps are replayed from a CUDA graph captured once per
      chunk size: the kernel reads the table when it runs, so between replays
      the host only rewrites each member's step counter, remaining steps and
      current buffer (and, for serving, adds or drops members).
  "graph": sw_batch_graph_run captures, per chunk, one chain of
      single-lattice step launches per member on parallel graph branches and
      launches the graph; the executable graph is updated in place while the
      composition keeps its shape.

autotune() times both and keeps the faster.  All members share one storage
type.  Members on the in-place AA pattern (half the memory of a wall) run in
graph mode, as chains of alternating odd and even in-place steps.

A member's results do not depend on the others (cells are owned by one
thread, wall forces are integer sums), so a wall gives the same bits alone
and in any mix; tests/test_gpu_batch.py checks this.
"""
import ctypes

import torch

from . import _native as N
from . import trace
from .fields import StatusWord, _stream


class SwBatchEntry(ctypes.Structure):
    _fields_ = [("geom", N.SwGeom), ("item0", ctypes.c_int64), ("items", ctypes.c_int64),
                ("f", ctypes.c_void_p * 2), ("flag", ctypes.c_void_p), ("tiles", ctypes.c_void_p),
                ("uin", ctypes.c_void_p), ("force", ctypes.c_void_p), ("acc", ctypes.c_void_p),
                ("nu0", ctypes.c_double), ("cs", ctypes.c_double), ("nu_sponge", ctypes.c_double),
                ("x_sponge", ctypes.c_int32), ("n_spin", ctypes.c_int32), ("acc_every", ctypes.c_int32),
                ("cur0", ctypes.c_int32), ("t0", ctypes.c_int64), ("steps_left", ctypes.c_int64),
                ("status", ctypes.c_void_p), ("ghost", ctypes.c_void_p)]


class SwBatchHeader(ctypes.Structure):
    _fields_ = [("n", ctypes.c_int32), ("reserved", ctypes.c_int32), ("total_items", ctypes.c_int64),
                ("next_item", ctypes.c_uint64), ("done_blocks", ctypes.c_uint32), ("reserved2", ctypes.c_uint32)]


def _bind():
    L = N.lib()
    if not hasattr(L.sw_batch_prepare, "_sw_bound"):
        P = ctypes.c_void_p
        L.sw_batch_prepare.argtypes = [P, ctypes.c_int32, ctypes.c_int, ctypes.c_int, P]
        L.sw_batch_prepare.restype = ctypes.c_int
        L.sw_batch_step.argtypes = [P, P, ctypes.c_int, ctypes.c_int, ctypes.c_int32, P]
        L.sw_batch_step.restype = ctypes.c_int
        L.sw_batch_setup.argtypes = [ctypes.c_int, ctypes.c_int]
        L.sw_batch_setup.restype = ctypes.c_int
        L.sw_batch_graph_create.argtypes = [ctypes.POINTER(P)]
        L.sw_batch_graph_create.restype = ctypes.c_int
        L.sw_batch_graph_destroy.argtypes = [P]
        L.sw_batch_graph_destroy.restype = ctypes.c_int
        L.sw_batch_graph_run.argtypes = [P, P, ctypes.c_int32, ctypes.c_int, ctypes.c_int32, P]
        L.sw_batch_graph_run.restype = ctypes.c_int
        L.sw_batch_graph_launches.argtypes = [P]
        L.sw_batch_graph_launches.restype = ctypes.c_int64
        L.sw_batch_prepare._sw_bound = True
    return L


def acc_steps(t0, n, n_spin, every):
    """How many of the steps t0 .. t0+n-1 accumulate (t >= n_spin, (t - n_spin) % every == 0)."""
    lo = max(t0, n_spin)
    hi = t0 + n
    if hi <= lo:
        return 0
    first = lo + (-(lo - n_spin)) % every
    return 0 if first >= hi else (hi - 1 - first) // every + 1


GRAPH_MAX = 256          # SW_BATCH_MAX_ENTRIES: lattices per sw_batch_graph_run


class Batch:
    def __init__(self, dtype="f16", device="cuda", chunk=50, max_members=512, cfg=None, mode="persistent"):
        self.dtype = N.dtype_code(dtype)
        self.device = torch.device(device)
        self.chunk = int(chunk)
        self.max_members = int(max_members)
        self.members = []
        self.cfg = cfg if cfg is not None else (4 if self.dtype in (N.SW_F16_SHIFT, N.SW_BF16_SHIFT) else 3)
        esz = ctypes.sizeof(SwBatchEntry)
        self._table_dev = torch.zeros(self.max_members * esz, dtype=torch.uint8, device=self.device)
        self._hdr_dev = torch.zeros(ctypes.sizeof(SwBatchHeader), dtype=torch.uint8, device=self.device)
        # two pinned host copies, alternated so that one can be rewritten while the other uploads
        self._table_host = [(SwBatchEntry * self.max_members)() for _ in range(2)]
        self._hdr_host = [SwBatchHeader() for _ in range(2)]
        self._pinned = [torch.empty(self.max_members * esz + ctypes.sizeof(SwBatchHeader), dtype=torch.uint8)
                        .pin_memory() for _ in range(2)]
        self._upload_done = [None, None]
        self._slot = 0
        self._graphs = {}
        self.launches = 0
        if mode not in ("persistent", "graph"):
            raise ValueError("mode is 'persistent' or 'graph'")
        self.mode = mode
        self._handle = None
        self._scratch_status = StatusWord(device=self.device)   # tuning launches report here
        _bind()

    def __del__(self):
        h = getattr(self, "_handle", None)
        if h is not None:
            try:
                N.lib().sw_batch_graph_destroy(h)
            except Exception:
                pass

    def _graph_handle(self):
        if self._handle is None:
            h = ctypes.c_void_p()
            N.check(N.lib().sw_batch_graph_create(ctypes.byref(h)), "sw_batch_graph_create")
            self._handle = h
        return self._handle

    # ------------------------------------------------------------ membership
    def add(self, solver):
        """Add a WallSolver.  Members on the in-place AA pattern (half the memory) run in graph mode
        only: their chains alternate the odd and even in-place steps."""
        if solver.dtype != self.dtype:
            raise ValueError("all members of a batch share one storage type")
        if getattr(solver, "pattern", "ab") == "aa" and self.mode != "graph":
            raise ValueError("in-place (AA) members need graph mode")
        if len(self.members) >= self.max_members:
            raise RuntimeError("batch is full")
        self.members.append(solver)
        return solver

    def remove(self, solver):
        self.members = [m for m in self.members if m is not solver]

    def pending(self):
        return [m for m in self.members if m.t < m.n_total]

    # ------------------------------------------------------------ table
    def _fill(self, n_steps, tuning=False, upload=True):
        slot = self._slot
        self._slot ^= 1
        if self._upload_done[slot] is not None:
            self._upload_done[slot].synchronize()
        tab, hdr = self._table_host[slot], self._hdr_host[slot]
        live = [m for m in self.members if m.t < m.n_total]
        for i, m in enumerate(live):
            e = tab[i]
            e.geom = m.grid.geom
            aa = getattr(m, "pattern", "ab") == "aa"
            e.f[0] = m.f[0].data.data_ptr()
            e.f[1] = m.f[0 if aa else 1].data.data_ptr()
            e.ghost = m.ghost.data_ptr() if aa else None
            e.flag = m.flags.flag.data_ptr()
            e.tiles = m.flags.tiles.data_ptr()
            e.uin = m.uin.data.data_ptr()
            e.force = None if tuning else m.force.data.data_ptr()
            e.acc = None if tuning else m.acc.data.data_ptr()
            e.status = (self._scratch_status if tuning else m.status).data.data_ptr()
            e.nu0, e.cs, e.nu_sponge = m.nu0, m.cs, m.nu_sponge
            e.x_sponge, e.n_spin, e.acc_every = m.x_sponge, m.n_spin, m.acc_every
            e.cur0 = (0 if m.aa_odd_next else 1) if aa else m.cur
            e.t0 = m.t
            e.steps_left = min(n_steps, m.n_total - m.t)
        if not live or not upload:
            return slot, live
        N.check(N.lib().sw_batch_prepare(ctypes.byref(tab), len(live), self.dtype, self.cfg, ctypes.byref(hdr)),
                "sw_batch_prepare")
        esz = ctypes.sizeof(SwBatchEntry)
        buf = self._pinned[slot]
        nbytes = len(live) * esz
        ctypes.memmove(buf.data_ptr(), ctypes.addressof(tab), nbytes)
        ctypes.memmove(buf.data_ptr() + self.max_members * esz, ctypes.addressof(hdr), ctypes.sizeof(hdr))
        self._table_dev[:nbytes].copy_(buf[:nbytes], non_blocking=True)
        self._hdr_dev.copy_(buf[self.max_members * esz:], non_blocking=True)
        ev = torch.cuda.Event()
        ev.record()
        self._upload_done[slot] = ev
        return slot, live

    def _launch(self, k):
        N.check(N.lib().sw_batch_step(ctypes.c_void_p(self._hdr_dev.data_ptr()),
                                      ctypes.c_void_p(self._table_dev.data_ptr()), self.dtype, self.cfg, int(k),
                                      _stream(None)), "sw_batch_step")

    def _graph(self, n):
        key = (n, self.cfg)
        if key not in self._graphs:
            N.check(N.lib().sw_batch_setup(self.dtype, self.cfg), "sw_batch_setup")   # no device queries in capture
            g = torch.cuda.CUDAGraph()
            with N.CAPTURE_LOCK:
                torch.cuda.synchronize()
                with torch.cuda.graph(g, capture_error_mode="thread_local"):
                    for k in range(n):
                        self._launch(k)
            self._graphs[key] = g
        return self._graphs[key]

    def _graph_run(self, slot, n_live, c):
        if n_live > GRAPH_MAX:
            raise RuntimeError(f"graph mode takes at most {GRAPH_MAX} lattices")
        with N.CAPTURE_LOCK:                     # the call captures the chunk's graph
            N.check(N.lib().sw_batch_graph_run(self._graph_handle(), ctypes.addressof(self._table_host[slot]),
                                               n_live, self.dtype, int(c), _stream(None)), "sw_batch_graph_run")

    # ------------------------------------------------------------ failures
    def status_words(self, members=None):
        """The members' status words gathered on the device (one int32 each, in member order)."""
        ms = self.members if members is None else members
        if not ms:
            return torch.zeros(0, dtype=torch.int32, device=self.device)
        return torch.cat([m.status.data for m in ms])

    def failures(self, members=None):
        """{member: Diverged | DeviceWaitTimeout} for members whose steps reported a failure so far.
        One gather and one read of all status words (waits for the queued steps)."""
        from .solver import status_exception
        ms = list(self.members if members is None else members)
        words = self.status_words(ms).cpu().tolist()
        out = {}
        for m, w in zip(ms, words):
            err = status_exception(w, f"batch member at step {m.t}")
            if err is not None:
                out[m] = err
        return out

    def check(self):
        """Raise the first member failure, if any."""
        bad = self.failures()
        if bad:
            raise next(iter(bad.values()))
        return True

    # ------------------------------------------------------------ stepping
    def advance(self, n, use_graphs=True, check=False):
        """Advance every unfinished member by up to n steps (each stops at its own n_total).  With
        check, the members' status words are read at the end and a failure raises; without (the
        default, as the solve server advances), the steps stay queued and failures are read with
        failures() when the caller chooses."""
        n = int(n)
        while n > 0:
            c = min(self.chunk, n)
            graph_mode = self.mode == "graph"
            slot, live = self._fill(c, upload=not graph_mode)
            if not live:
                return self
            if graph_mode:
                with trace.range(f"batch graph chunk ({len(live)} walls, {c} steps)"):
                    self._graph_run(slot, len(live), c)
                self.launches += sum(min(c, m.n_total - m.t) for m in live)
            elif use_graphs and c == self.chunk:
                with trace.range(f"batch persistent chunk ({len(live)} walls, {c} steps)"):
                    self._graph(c).replay()
                self.launches += c
            else:
                for k in range(c):
                    self._launch(k)
                self.launches += c
            for m in live:
                s = min(c, m.n_total - m.t)
                m.n_acc += acc_steps(m.t, s, m.n_spin, m.acc_every)
                m.t += s
                if getattr(m, "pattern", "ab") == "aa":
                    m.aa_odd_next ^= bool(s & 1)
                else:
                    m.cur ^= (s & 1)
            n -= c
        if check:
            self.check()
        return self

    def run(self):
        """Advance until every member has finished; a member's failure raises."""
        while self.pending():
            self.advance(self.chunk * 20, check=True)
        return self

    def cells(self):
        return sum(m.grid.cells for m in self.members)

    def autotune(self, repeats=5, modes=("persistent", "graph")):
        """Time the persistent kernel in every configuration this storage type has, and the graph
        mode (with the single-lattice configurations tuned on the largest member), on the current
        members; keep the fastest.  Each timed step recomputes every member's next state into its
        spare buffer with forces and sums switched off, so the members' states are not changed.
        Returns (best, times): best is a configuration number or "graph"."""
        times = {}
        if any(getattr(m, "pattern", "ab") == "aa" for m in self.members):
            # in-place members: graph mode, and no trial steps (they would change those states); the
            # two-lattice members' configurations are still tuned on the largest of them
            ab = [m for m in self.pending() if getattr(m, "pattern", "ab") == "ab"]
            if ab:
                from . import autotune as single
                single.tune(max(ab, key=lambda m: m.grid.cells))
            self.mode = "graph"
            return "graph", times
        if "persistent" in modes:
            for cfg in range(N.lib().sw_step_config_count()):
                if not _valid(self.dtype, cfg):
                    continue
                self.cfg = cfg
                self._fill(1, tuning=True)
                self._launch(0)
                torch.cuda.synchronize()
                e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                e0.record()
                for _ in range(repeats):
                    self._launch(0)
                e1.record()
                torch.cuda.synchronize()
                times[cfg] = e0.elapsed_time(e1) / repeats
            self.cfg = min(times, key=times.get)
        live = self.pending()
        if "graph" in modes and 0 < len(live) <= GRAPH_MAX:
            from . import autotune as single
            single.tune(max(live, key=lambda m: m.grid.cells))
            slot, lv = self._fill(1, tuning=True, upload=False)
            self._graph_run(slot, len(lv), 1)                       # instantiate
            torch.cuda.synchronize()
            if hasattr(torch.cuda, "_sleep"):
                torch.cuda._sleep(50_000_000)                       # let the host run ahead of the device
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record()
            for _ in range(repeats):
                self._graph_run(slot, len(lv), 1)
            e1.record()
            torch.cuda.synchronize()
            times["graph"] = e0.elapsed_time(e1) / repeats
        best = min(times, key=times.get)
        self.mode = "graph" if best == "graph" else "persistent"
        return best, times


def _valid(dtype, cfg):
    """Configurations of the persistent batched kernel (the TMA-staged ones, 8 and up, are not)."""
    return cfg < 4 or (cfg < 8 and dtype in (N.SW_F16_SHIFT, N.SW_BF16_SHIFT))
