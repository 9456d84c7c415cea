"""Device-resident fields in the kernels' layout, with conversion to the reference's layout.

The reference allocates Warp arrays (lbm3d.py:292-313) shaped
f (19, nx, ny, nz), flag (nx, ny, nz), U / Uacc (4, nx, ny, nz) and
force (n_total, nz, 2), all z fastest.  These classes hold the same data in
the x-fastest padded layout of include/stonewall.h; ``numpy()`` and
``assign()`` speak the reference's layout, exactly like the Warp arrays'
``.numpy()`` / ``.assign()`` that lbm3d.py uses for checkpoints
(lbm3d.py:332-334, 345-347).  Device memory comes from PyTorch's allocator.
"""
import ctypes

import numpy as np
import torch

from . import _native as N
from .lattice import Q


def _stream(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return ctypes.c_void_p(s.cuda_stream)


def _ptr(t):
    return ctypes.c_void_p(t.data_ptr())


class Grid:
    """Extents of one lattice and its padded device geometry (sw_geom)."""

    def __init__(self, nx, ny, nz):
        self.geom = N.geom(nx, ny, nz)
        self.nx, self.ny, self.nz, self.pitch = int(nx), int(ny), int(nz), self.geom.pitch
        self.cells = self.nx * self.ny * self.nz
        self.cells_padded = self.nz * self.ny * self.pitch
        self.tiles = self.cells_padded // 32

    @property
    def gp(self):
        return ctypes.byref(self.geom)

    def __repr__(self):
        return f"Grid({self.nx}x{self.ny}x{self.nz}, pitch {self.pitch})"


class Lattice:
    """Populations f_i in device layout, stored as ``dtype`` (f32, f64, f16 / bf16 shifted)."""

    def __init__(self, grid, dtype="f32", device="cuda", data=None):
        self.grid = grid
        self.dtype = N.dtype_code(dtype)
        nbytes = Q * grid.cells_padded * N.DTYPE_BYTES[self.dtype]
        self.data = data if data is not None else torch.empty(nbytes, dtype=torch.uint8, device=device)
        assert self.data.numel() == nbytes and self.data.data_ptr() % 16 == 0

    @property
    def ptr(self):
        return _ptr(self.data)

    @property
    def nbytes(self):
        return self.data.numel()

    def zero_(self):
        self.data.zero_()
        return self

    def numpy(self, ref_dtype=np.float32, stream=None):
        """f in the reference layout (19, nx, ny, nz); shifted formats are returned as f = w + delta."""
        g = self.grid
        rd = N.SW_F64 if np.dtype(ref_dtype) == np.float64 else N.SW_F32
        tdt = torch.float64 if rd == N.SW_F64 else torch.float32
        out = torch.empty((Q, g.nx, g.ny, g.nz), dtype=tdt, device=self.data.device)
        N.check(N.lib().sw_unpack_f(g.gp, self.dtype, rd, self.ptr, _ptr(out), _stream(stream)), "sw_unpack_f")
        return out.cpu().numpy()

    def assign(self, f_ref, stream=None):
        """Load f from the reference layout (19, nx, ny, nz), float32 or float64 (numpy or torch)."""
        g = self.grid
        t = torch.as_tensor(np.ascontiguousarray(f_ref) if isinstance(f_ref, np.ndarray) else f_ref)
        if tuple(t.shape) != (Q, g.nx, g.ny, g.nz):
            raise ValueError(f"f has shape {tuple(t.shape)}, expected {(Q, g.nx, g.ny, g.nz)}")
        if t.dtype not in (torch.float32, torch.float64):
            t = t.to(torch.float32)
        t = t.to(self.data.device).contiguous()
        rd = N.SW_F64 if t.dtype == torch.float64 else N.SW_F32
        N.check(N.lib().sw_pack_f(g.gp, self.dtype, rd, _ptr(t), self.ptr, _stream(stream)), "sw_pack_f")
        torch.cuda.current_stream().synchronize() if stream is None else stream.synchronize()
        return self


class Flags:
    """Cell flags (0 fluid, 1 stone, 2 ground) plus the per-segment tile classes for the step."""

    def __init__(self, grid, flag_ref, device="cuda", stream=None):
        self.grid = grid
        f = np.ascontiguousarray(np.asarray(flag_ref).astype(np.uint8))
        if f.shape != (grid.nx, grid.ny, grid.nz):
            raise ValueError(f"flag has shape {f.shape}, expected {(grid.nx, grid.ny, grid.nz)}")
        self.host = f
        self.flag = torch.empty(grid.cells_padded, dtype=torch.uint8, device=device)
        self.tiles = torch.empty(grid.tiles, dtype=torch.uint8, device=device)
        self._ref = torch.empty((grid.nx, grid.ny, grid.nz), dtype=torch.uint8, device=device)
        self.load(torch.from_numpy(f), stream=stream)
        (stream or torch.cuda.current_stream()).synchronize()

    def load(self, flag_ref, stream=None):
        """Copy flags (reference layout, host or device tensor; pinned host memory copies
        asynchronously) into the device layout and reclassify the row segments."""
        g = self.grid
        if tuple(flag_ref.shape) != (g.nx, g.ny, g.nz) or flag_ref.dtype != torch.uint8:
            raise ValueError(f"flag must be uint8 {(g.nx, g.ny, g.nz)}")
        self._ref.copy_(flag_ref, non_blocking=True)
        s = _stream(stream)
        N.check(N.lib().sw_pack_flag(g.gp, _ptr(self._ref), _ptr(self.flag), s), "sw_pack_flag")
        N.check(N.lib().sw_build_tiles(g.gp, _ptr(self.flag), _ptr(self.tiles), s), "sw_build_tiles")

    @property
    def ptr(self):
        return _ptr(self.flag)

    @property
    def tiles_ptr(self):
        return _ptr(self.tiles)

    def numpy(self):
        return self.host.copy()

    def tile_counts(self):
        """How many row segments take the fast path, the checked path, the force path, or are skipped."""
        t = self.tiles.cpu().numpy()
        return dict(skipped=int((t & 1).sum()), checked=int(((t & 2) > 0).sum()),
                    force=int(((t & 4) > 0).sum()), fast=int((t == 0).sum()), total=int(t.size))


class Macro:
    """rho, ux, uy, uz per cell (float32), the reference's U (lbm3d.py:302)."""

    def __init__(self, grid, device="cuda"):
        self.grid = grid
        self.data = torch.zeros(4 * grid.cells_padded, dtype=torch.float32, device=device)

    @property
    def ptr(self):
        return _ptr(self.data)

    def numpy(self, stream=None):
        g = self.grid
        out = torch.empty((4, g.nx, g.ny, g.nz), dtype=torch.float32, device=self.data.device)
        N.check(N.lib().sw_unpack_u(g.gp, self.ptr, _ptr(out), _stream(stream)), "sw_unpack_u")
        return out.cpu().numpy()


class Accum:
    """Running sums of U in float64, the reference's Uacc (lbm3d.py:303)."""

    def __init__(self, grid, device="cuda"):
        self.grid = grid
        self.data = torch.zeros(4 * grid.cells_padded, dtype=torch.float64, device=device)

    @property
    def ptr(self):
        return _ptr(self.data)

    def numpy(self, stream=None, solid=None, n_acc=None):
        """Sums in the reference layout.  With ``solid`` (bool (nx, ny, nz)) and ``n_acc`` the
        non-fluid cells are set to n_acc * (1, 0, 0, 0), what k_macro + k_accum give them."""
        g = self.grid
        out = torch.empty((4, g.nx, g.ny, g.nz), dtype=torch.float64, device=self.data.device)
        N.check(N.lib().sw_unpack_acc(g.gp, self.ptr, _ptr(out), _stream(stream)), "sw_unpack_acc")
        a = out.cpu().numpy()
        if solid is not None:
            a[0][solid] = float(n_acc)
            a[1:, solid] = 0.0
        return a

    def assign(self, acc_ref):
        """Load sums from the reference layout (4, nx, ny, nz) (resume, lbm3d.py:334)."""
        g = self.grid
        a = np.asarray(acc_ref, dtype=np.float64)
        if a.shape != (4, g.nx, g.ny, g.nz):
            raise ValueError(f"acc has shape {a.shape}, expected {(4, g.nx, g.ny, g.nz)}")
        dev = np.zeros((4, g.nz, g.ny, g.pitch), np.float64)
        dev[:, :, :, :g.nx] = a.transpose(0, 3, 2, 1)
        self.data.copy_(torch.from_numpy(dev.ravel()))
        return self


class ForceSeries:
    """Per-step, per-level wall force, force[t][z][0..1] of lbm3d.py:301, in 2^-40 fixed point."""

    def __init__(self, n_steps, nz, device="cuda"):
        self.n_steps, self.nz = int(n_steps), int(nz)
        self.data = torch.zeros((self.n_steps, self.nz, 2), dtype=torch.int64, device=device)

    @property
    def ptr(self):
        return _ptr(self.data)

    def numpy(self):
        """(n_steps, nz, 2) float64."""
        return self.data.cpu().numpy().astype(np.float64) / N.FORCE_SCALE

    def assign(self, force_ref):
        f = np.asarray(force_ref, dtype=np.float64)
        if f.shape != (self.n_steps, self.nz, 2):
            raise ValueError(f"force has shape {f.shape}, expected {(self.n_steps, self.nz, 2)}")
        self.data.copy_(torch.from_numpy(np.rint(f * N.FORCE_SCALE).astype(np.int64)))
        return self


class StatusWord:
    """A lattice's device status word: the checked step kernels OR SW_STATUS_NONFINITE (a fluid
    cell pulled a non-finite density) and SW_STATUS_TIMEOUT (a TMA-staged block gave up waiting)
    into it.  This is the device side of the reference's divergence check (lbm3d.py:386-391),
    which looks at the macro field every 5000 steps; here every fluid cell of every step counts."""

    def __init__(self, device="cuda"):
        self.data = torch.zeros(1, dtype=torch.int32, device=device)

    @property
    def ptr(self):
        return _ptr(self.data)

    def clear(self):
        self.data.zero_()
        return self

    def read(self):
        """The word's bits (waits for the work queued so far on the current stream)."""
        return int(self.data.item()) & 0xFFFFFFFF

    def error(self, word=None):
        """SW_OK, SW_ERR_TIMEOUT or SW_ERR_NONFINITE for the word (read now if not given)."""
        return N.lib().sw_status_error(self.read() if word is None else int(word))
