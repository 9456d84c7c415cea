"""WallSolver: one wall solve resident on the GPU, the public driver-level API.

It owns what lbm3d.py:292-313 allocates (two lattices, flags, inlet, force
series, the running mean) and replaces the time loop of lbm3d.py:358-370:
each step is one fused k_step, and after the spin-up every 5th state is
accumulated (k_macro + k_accum fused, sums in float64).  Runs of steps are
replayed as CUDA graphs of `chunk` steps; the per-step force rows of a graph
go to a ring buffer that is copied into the series after each replay, so one
captured graph serves every chunk with the same ping-pong parity and
accumulation phase.

Checkpoints use the reference's directory format (lbm3d.py:342-355):
f.npy (19, nx, ny, nz), force.npy (n_total, nz, 2), uacc.npy (4, nx, ny, nz),
snaps_*.npy and state.json {t, n_acc, sig}, written to <dir>.tmp and swapped
in once complete.  force and uacc are stored in float64 (the reference writes
float32), which makes a resumed run bit-identical to an uninterrupted one;
float32 files from the reference load as well.
"""
import json
import os
import shutil
import threading
import warnings

import numpy as np
import torch

from . import _native as N
from . import kernels as K
from . import trace
from .fields import Accum, Flags, ForceSeries, Grid, Lattice, Macro, StatusWord


class Diverged(RuntimeError):
    """The solve produced a non-finite state (lbm3d.py:386-391 exits with "diverged")."""
    status = N.SW_ERR_NONFINITE


class DeviceWaitTimeout(RuntimeError):
    """A bounded device wait of the TMA-staged step gave up: the step's results are not valid."""
    status = N.SW_ERR_TIMEOUT


class BiasedStorageWarning(UserWarning):
    """A storage type whose measured wall loads are biased against float64 storage."""


BF16_WARNING = ("bf16 shifted storage keeps 8 bits of f - w: on the 800x160x160 walls its mean Cd came out "
                "14-26 % above float64 storage; use f16 (or f32) for wall loads")


def status_exception(word, where):
    """The exception a non-zero status word stands for (None for 0)."""
    err = N.lib().sw_status_error(int(word) & 0xFFFFFFFF)
    if err == N.SW_ERR_TIMEOUT:
        return DeviceWaitTimeout(f"{where}: a TMA-staged step block timed out (status word {word:#x})")
    if err == N.SW_ERR_NONFINITE:
        return Diverged(f"{where}: non-finite density (status word {word:#x})")
    return None


class WallSolver:
    """pattern "ab": two lattices, each step pulls from one into the other (lbm3d.py:293-294, 362).
    pattern "aa": one lattice updated in place (half the memory), odd and even steps alternating;
    states, checkpoints and mean fields can be taken after an even number of steps."""

    def __init__(self, flag, uin, nu0, cs, x_sponge, n_total, n_spin=0, nu_sponge=0.05, dtype="f32",
                 device="cuda", acc_every=5, chunk=50, pattern="ab"):
        flag = np.asarray(flag, dtype=np.uint8)
        nx, ny, nz = flag.shape
        uin = np.asarray(uin, dtype=np.float32)
        if uin.shape != (nz,):
            raise ValueError(f"uin has shape {uin.shape}, expected ({nz},)")
        self.device = torch.device(device)
        self.grid = Grid(nx, ny, nz)
        self.flags = Flags(self.grid, flag, device=self.device)
        self.uin = K.DeviceVector(uin, device=self.device)
        self.nu0, self.cs, self.x_sponge, self.nu_sponge = float(nu0), float(cs), int(x_sponge), float(nu_sponge)
        self.n_total, self.n_spin, self.acc_every = int(n_total), int(n_spin), int(acc_every)
        if pattern not in ("ab", "aa"):
            raise ValueError("pattern is 'ab' (two lattices) or 'aa' (one lattice, in place)")
        if N.dtype_code(dtype) == N.SW_BF16_SHIFT:
            warnings.warn(BF16_WARNING, BiasedStorageWarning, stacklevel=2)
        self.pattern = pattern
        if pattern == "ab":
            self.f = [Lattice(self.grid, dtype, device=self.device),
                      Lattice(self.grid, dtype, device=self.device).zero_()]   # f1 = zeros, lbm3d.py:294
        else:
            self.f = [Lattice(self.grid, dtype, device=self.device)]
            nb = N.lib().sw_aa_ghost_elems(self.grid.gp) * N.DTYPE_BYTES[self.f[0].dtype]
            self.ghost = torch.empty(int(nb), dtype=torch.uint8, device=self.device)
            if chunk % 2:
                raise ValueError("the AA pattern replays graphs of an even number of steps")
        self.aa_odd_next = True      # AA: the next step is an odd one (the state is readable)
        self.cur = 0
        self.status = StatusWord(device=self.device)   # divergence and time-out bits of every step
        self.force = ForceSeries(self.n_total, nz, device=self.device)
        self.acc = Accum(self.grid, device=self.device)
        self.t = 0
        self.n_acc = 0
        self.chunk = int(chunk)
        self._graphs = {}
        self._ring = None
        self.launches = 0          # kernels of this library launched by advance()
        self._ckpt_host = None     # pinned host buffers of the checkpoint writer (reused)
        self._ckpt_stream = None
        self._ckpt_thread = None
        self._ckpt_error = None

    # ------------------------------------------------------------ state
    @property
    def state(self):
        """The lattice holding the current populations (the reference's f0 after the swap).
        AA pattern: the single lattice, which holds the state after an even number of steps."""
        return self.f[self.cur] if self.pattern == "ab" else self.f[0]

    def state_numpy(self, ref_dtype=np.float32):
        """Current populations in the reference layout (19, nx, ny, nz)."""
        self._readable()
        return self.state.numpy(ref_dtype)

    def _readable(self):
        if self.pattern == "aa" and not self.aa_odd_next:
            raise RuntimeError("AA pattern: the state can be read after an even number of steps only")

    @property
    def dtype(self):
        return self.f[0].dtype

    def memory_bytes(self):
        g = self.grid
        return (sum(f.nbytes for f in self.f) + self.flags.flag.numel() + self.flags.tiles.numel()
                + self.force.data.numel() * 8 + self.acc.data.numel() * 8
                + (self.ghost.numel() if self.pattern == "aa" else 0))

    def reload(self, flag, uin):
        """Start over with a new mask and inlet profile (torch tensors, pinned host memory copies
        asynchronously): resets the step counter, forces and sums; keeps buffers and graphs."""
        self.flags.load(flag)
        if tuple(uin.shape) != (self.grid.nz,):
            raise ValueError("uin has the wrong length")
        self.uin.data.copy_(uin, non_blocking=True)
        self.force.data.zero_()
        self.acc.data.zero_()
        self.status.clear()
        self.t, self.n_acc, self.cur = 0, 0, 0
        self.aa_odd_next = True
        return self

    def autotune(self, repeats=8):
        """Time the step's launch configurations on this grid and install the fastest for this
        storage type (stonewall.autotune); the state is not modified.  Returns (cfg, times)."""
        from . import autotune
        if self.pattern == "aa":
            return N.lib().sw_get_step_config(self.dtype), {}   # the in-place step has one configuration
        return autotune.tune(self, repeats=repeats)

    def init(self, noise=0.02, seed=7, noise_kind="uniform"):
        """k_init on the current lattice (lbm3d.py:340); clears the status word."""
        K.k_init(self.state, self.flags, self.uin, noise, seed, noise_kind)
        self.status.clear()
        return self

    # ------------------------------------------------------------ stepping
    def _step(self, force_rows, t_index, accumulate=False):
        g = self.grid
        if self.pattern == "aa":
            K.k_step_aa(self.f[0], self.aa_odd_next, self.flags, self.uin, self.nu0, self.cs, self.x_sponge,
                        self.nu_sponge, force_rows, t_index, ghost=self.ghost, acc=self.acc if accumulate else None,
                        status=self.status)
            self.aa_odd_next = not self.aa_odd_next
            return
        src, dst = self.f[self.cur], self.f[1 - self.cur]
        K.k_step(src, dst, self.flags, self.uin, g.nx, g.ny, g.nz, self.nu0, self.cs, self.x_sponge,
                 self.nu_sponge, force_rows, t_index, acc=self.acc if accumulate else None, status=self.status)
        self.cur ^= 1

    def _accumulate_now(self, t):
        return t >= self.n_spin and (t - self.n_spin) % self.acc_every == 0

    def step(self):
        """One eager step (lbm3d.py:359-370)."""
        if self.t >= self.n_total:
            raise RuntimeError("the run is complete")
        acc = self._accumulate_now(self.t)
        self._step(self.force, self.t, accumulate=acc)
        self.launches += 1
        self.n_acc += int(acc)
        self.t += 1

    def _graph_for(self, key):
        if key in self._graphs:
            return self._graphs[key]
        n, cur0, phase = key[:3]
        if self._ring is None or self._ring.n_steps != n:
            self._ring = ForceSeries(n, self.grid.nz, device=self.device)
        ring = self._ring
        saved = (self.cur, self.aa_odd_next)
        self.cur = cur0
        graph = torch.cuda.CUDAGraph()
        with N.CAPTURE_LOCK:                     # no other thread's GPU work inside the capture
            torch.cuda.synchronize()
            with torch.cuda.graph(graph, capture_error_mode="thread_local"):
                ring.data.zero_()
                for j in range(n):
                    self._step(ring, j, accumulate=phase is not None and (phase + j) % self.acc_every == 0)
        self.cur, self.aa_odd_next = saved
        n_acc = 0 if phase is None else sum(1 for j in range(n) if (phase + j) % self.acc_every == 0)
        self._graphs[key] = (graph, n_acc)
        return self._graphs[key]

    def advance(self, n, use_graphs=True, check=True):
        """Run n steps (graph-replayed in chunks where possible).  With check (the default) the status
        word is read once at the end -- one wait for the queued steps -- and a diverged state or a
        timed-out step raises Diverged / DeviceWaitTimeout; without, the steps stay queued."""
        n = min(int(n), self.n_total - self.t)
        c = self.chunk
        while n > 0:
            t = self.t
            same_side = t >= self.n_spin or t + c <= self.n_spin
            if use_graphs and n >= c and same_side and (self.pattern == "ab" or self.aa_odd_next):
                phase = (t - self.n_spin) % self.acc_every if t >= self.n_spin else None
                graph, n_acc = self._graph_for((c, self.cur, phase))
                with trace.range(f"solver chunk t={t}"):
                    graph.replay()
                self.force.data[t:t + c].copy_(self._ring.data)
                self.cur ^= (c & 1) if self.pattern == "ab" else 0
                self.t += c
                self.n_acc += n_acc
                self.launches += c
                n -= c
            else:
                self.step()
                n -= 1
        if check:
            self.check_status()
        return self

    def status_error(self):
        """The failure recorded in the status word so far (Diverged / DeviceWaitTimeout), or None.
        Reads the word: waits for the steps queued so far."""
        return status_exception(self.status.read(), f"step {self.t}")

    def check_status(self):
        """Raise the failure recorded in the status word, if any."""
        err = self.status_error()
        if err is not None:
            raise err
        return True

    def run(self, check_every=5000, log=None):
        """Advance to n_total with a finiteness check every check_every steps (lbm3d.py:386-391)."""
        while self.t < self.n_total:
            nxt = min(self.n_total, (self.t // check_every + 1) * check_every)
            self.advance(nxt - self.t)
            self.check_finite()
            if log:
                log(self)
        return self

    # ------------------------------------------------------------ outputs
    def macro(self):
        """rho, ux, uy, uz of the current state in the reference layout (k_macro, lbm3d.py:367)."""
        self._readable()
        u = Macro(self.grid, device=self.device)
        K.k_macro(self.state, self.flags, u)
        return u.numpy()

    def _macro_dev(self):
        """The macro field of the current state on the device (one buffer, reused)."""
        self._readable()
        if getattr(self, "_u", None) is None:
            self._u = Macro(self.grid, device=self.device)
        K.k_macro(self.state, self.flags, self._u)
        return self._u

    def snapshot(self, y_mid, z_half):
        """ux, uy, uz on the planes y = y_mid and z = z_half as float16 (3, nx, nz), (3, nx, ny):
        lbm3d.py:366-375 (k_macro, k_slice_xz, k_slice_xy, [1:].astype(float16))."""
        u = self._macro_dev()
        g = self.grid
        xz = torch.empty((4, g.nx, g.nz), dtype=torch.float32, device=self.device)
        xy = torch.empty((4, g.nx, g.ny), dtype=torch.float32, device=self.device)
        K.k_slice_xz(u, y_mid, xz)
        K.k_slice_xy(u, z_half, xy)
        return xz.cpu().numpy()[1:].astype(np.float16), xy.cpu().numpy()[1:].astype(np.float16)

    def q_frame(self, x0, ds, dims, q_scale, qmax=400.0, macro_ready=False):
        """Q-criterion frame of the current state: k_qcoarse then the reference's log quantisation
        to uint8 (lbm3d.py:315-318).  macro_ready: reuse the macro field of the last snapshot()."""
        u = self._u if macro_ready and getattr(self, "_u", None) is not None else self._macro_dev()
        q = torch.empty(tuple(dims), dtype=torch.float32, device=self.device)
        g = self.grid
        K.k_qcoarse(u, self.flags, x0, ds, g.nx, g.ny, g.nz, q)
        q = np.clip(q.cpu().numpy() * q_scale, 0, qmax)
        return np.round(255 * np.log1p(q) / np.log1p(qmax)).astype(np.uint8)

    def check_finite(self):
        if self.pattern == "aa" and not self.aa_odd_next:
            return True                 # checked at the next even boundary
        u = Macro(self.grid, device=self.device)
        K.k_macro(self.state, self.flags, u)
        if not bool(torch.isfinite(u.data).all()):
            raise Diverged(f"diverged at step {self.t}")
        return True

    def force_series(self):
        """(n_total, nz, 2) float64."""
        return self.force.numpy()

    def sums(self):
        """Running sums of (rho, u), reference layout, solids at n_acc * (1, 0, 0, 0) (lbm3d.py:303)."""
        return self.acc.numpy(solid=self.flags.host != 0, n_acc=self.n_acc)

    def mean_field(self):
        """Time-mean (rho, u) over the accumulated states, float64 (lbm3d.py:402)."""
        return self.sums() / max(self.n_acc, 1)

    # ------------------------------------------------------------ checkpoints
    def save_checkpoint(self, path, sig, extra=None, background=False):
        """Write the checkpoint directory (lbm3d.py:342-355).  The state, sums and force series are
        copied on the device right away, in stream order after the steps so far; with background=True
        the device-to-host transfer (a side stream, into reused pinned buffers) and the file writes
        (a writer thread) overlap the steps that follow.  One checkpoint is in flight at a time;
        wait_checkpoint() joins it and raises what it raised."""
        self.wait_checkpoint()
        self._readable()
        g = self.grid
        ref64 = self.dtype == 1
        main = torch.cuda.current_stream()
        from . import _native as N
        from .fields import _ptr, _stream
        f_dev = torch.empty((19, g.nx, g.ny, g.nz), dtype=torch.float64 if ref64 else torch.float32,
                            device=self.device)
        rd = N.SW_F64 if ref64 else N.SW_F32
        N.check(N.lib().sw_unpack_f(g.gp, self.dtype, rd, self.state.ptr, _ptr(f_dev), _stream(main)), "sw_unpack_f")
        acc_dev = torch.empty((4, g.nx, g.ny, g.nz), dtype=torch.float64, device=self.device)
        N.check(N.lib().sw_unpack_acc(g.gp, self.acc.ptr, _ptr(acc_dev), _stream(main)), "sw_unpack_acc")
        force_dev = self.force.data.clone()
        taken = torch.cuda.Event()
        taken.record(main)
        host = self._ckpt_host
        if host is None or host[0].shape != f_dev.shape or host[0].dtype != f_dev.dtype:
            host = tuple(torch.empty(t.shape, dtype=t.dtype, pin_memory=True) for t in (f_dev, acc_dev, force_dev))
            self._ckpt_host = host
        if self._ckpt_stream is None:
            self._ckpt_stream = torch.cuda.Stream(device=self.device)
        side = self._ckpt_stream
        side.wait_event(taken)
        with torch.cuda.stream(side):
            for h, d in zip(host, (f_dev, acc_dev, force_dev)):
                h.copy_(d, non_blocking=True)
                d.record_stream(side)
        copied = torch.cuda.Event()
        copied.record(side)
        solid, n_acc, state = self.flags.host != 0, self.n_acc, dict(t=self.t, n_acc=self.n_acc, sig=sig)
        extra = dict(extra or {})

        def write():
            copied.synchronize()
            f_h, acc_h, force_h = (h.numpy() for h in host)
            acc_h[0][solid] = float(n_acc)                          # what k_macro + k_accum give solids
            acc_h[1:, solid] = 0.0
            tmp = path + ".tmp"
            if os.path.isdir(tmp):
                shutil.rmtree(tmp)
            os.makedirs(tmp)
            np.save(os.path.join(tmp, "f.npy"), f_h)
            np.save(os.path.join(tmp, "force.npy"), force_h.astype(np.float64) / N.FORCE_SCALE)
            np.save(os.path.join(tmp, "uacc.npy"), acc_h)
            np.save(os.path.join(tmp, "snaps_xz.npy"),
                    extra.get("snaps_xz", np.zeros((0, 3, g.nx, g.nz), np.float16)))
            np.save(os.path.join(tmp, "snaps_xy.npy"),
                    extra.get("snaps_xy", np.zeros((0, 3, g.nx, g.ny), np.float16)))
            np.save(os.path.join(tmp, "snaps_q.npy"), extra.get("snaps_q", np.zeros((0, 1, 1, 1), np.uint8)))
            with open(os.path.join(tmp, "state.json"), "w") as fh:
                json.dump(state, fh)
            if os.path.isdir(path):
                shutil.rmtree(path)
            os.replace(tmp, path)

        if not background:
            write()
            return

        def run():
            try:
                write()
            except BaseException as e:      # handed to wait_checkpoint()
                self._ckpt_error = e

        self._ckpt_thread = threading.Thread(target=run, name="checkpoint-writer", daemon=True)
        self._ckpt_thread.start()

    def wait_checkpoint(self):
        """Join the checkpoint being written in the background, if any."""
        t = getattr(self, "_ckpt_thread", None)
        if t is not None:
            t.join()
            self._ckpt_thread = None
        err, self._ckpt_error = getattr(self, "_ckpt_error", None), None
        if err is not None:
            raise err

    def load_checkpoint(self, path, sig):
        self.wait_checkpoint()
        with open(os.path.join(path, "state.json")) as fh:
            info = json.load(fh)
        if info["sig"] != sig:
            raise ValueError(f"checkpoint {path} was made with different settings")
        self.t, self.n_acc = int(info["t"]), int(info["n_acc"])
        self.status.clear()
        self.cur = 0
        self.aa_odd_next = True
        self.f[0].assign(np.load(os.path.join(path, "f.npy")))
        if self.pattern == "ab":
            self.f[1].zero_()
        self.force.assign(np.load(os.path.join(path, "force.npy")))
        self.acc.assign(np.load(os.path.join(path, "uacc.npy")))
        self._graphs.clear()
        return info
