"""The reference's kernel interface, backed by the sm_103a kernels of libstonewall.so.

stonewall3d/lbm3d.py drives its solver through
``wp.launch(k_<name>, dim=..., inputs=[...], device=dev)``.  This module keeps
those names and argument lists:

    launch(k_init,  dim, [f, flag, uin, cx, cy, cz, w, noise, seed])            lbm3d.py:340
    launch(k_step,  dim, [f_in, f_out, flag, uin, cx, cy, cz, w, opp, mirz,
                          nx, ny, nz, nu0, Cs, x_sponge, nu_sponge, force, t])  lbm3d.py:359-361
    launch(k_macro, dim, [f, flag, cx, cy, cz, U])                              lbm3d.py:367
    launch(k_accum, dim, [U, Uacc])                                             lbm3d.py:369

with the arrays being the device fields of stonewall.fields.  The D3Q19
tables in the input lists are checked against the compiled-in set and
otherwise ignored.  The direct forms (k_step(f_in, f_out, flag, uin, ...))
take the same arguments without the tables.  Errors raise (StonewallError
for a failing native call, ValueError / TypeError for bad arguments), as a
failing wp.launch raises.
"""
import numpy as np
import torch

from . import _native as N
from .fields import Accum, Flags, ForceSeries, Lattice, Macro, StatusWord, _ptr, _stream
from .lattice import check_tables


class DeviceVector:
    """A small float32 device array (the inlet profile uin, lbm3d.py:296)."""

    def __init__(self, values, device="cuda"):
        self.host = np.ascontiguousarray(np.asarray(values, dtype=np.float32))
        self.data = torch.from_numpy(self.host.copy()).to(device)

    @property
    def ptr(self):
        return _ptr(self.data)

    def numpy(self):
        return self.host.copy()


def _uin(uin):
    if isinstance(uin, DeviceVector):
        return uin
    raise TypeError("uin must be a stonewall.kernels.DeviceVector")


def _same_grid(*fields):
    g = fields[0].grid
    for f in fields[1:]:
        if (f.grid.nx, f.grid.ny, f.grid.nz) != (g.nx, g.ny, g.nz):
            raise ValueError("fields belong to different grids")
    return g


NOISE_KINDS = {"uniform": N.SW_NOISE_UNIFORM, "gauss": N.SW_NOISE_GAUSSIAN, "gaussian": N.SW_NOISE_GAUSSIAN}


def k_init(f: Lattice, flag: Flags, uin, noise=0.02, seed=7, noise_kind="uniform", stream=None):
    """lbm3d.py:39-54: rest-density equilibrium with a perturbed inlet velocity."""
    g = _same_grid(f, flag)
    kind = NOISE_KINDS[noise_kind] if isinstance(noise_kind, str) else int(noise_kind)
    N.check(N.lib().sw_init(g.gp, f.dtype, f.ptr, flag.ptr, _uin(uin).ptr, float(noise), int(seed), kind,
                            _stream(stream)), "sw_init")


def k_step(f_in: Lattice, f_out: Lattice, flag: Flags, uin, nx, ny, nz, nu0, cs, x_sponge, nu_sponge=0.05,
           force: ForceSeries = None, t=0, stream=None, acc: Accum = None, status: StatusWord = None, cfg=None):
    """lbm3d.py:57-155: one fused timestep f_in -> f_out; force[t] receives the wall force.

    With ``acc`` the new state's (rho, u) of every fluid cell is also added to
    the running sums (k_macro + k_accum of lbm3d.py:367-369 in the same pass).
    With ``status`` (a StatusWord) the step reports non-finite densities and
    TMA wait time-outs into it (sw_step_checked); ``cfg`` picks a launch
    configuration instead of the installed one.
    """
    g = _same_grid(f_in, f_out, flag)
    if (int(nx), int(ny), int(nz)) != (g.nx, g.ny, g.nz):
        raise ValueError(f"extents {(nx, ny, nz)} do not match the fields' grid {g}")
    if f_in.dtype != f_out.dtype:
        raise ValueError("f_in and f_out have different storage types")
    fptr = None
    if force is not None:
        if force.nz != g.nz or not (0 <= int(t) < force.n_steps):
            raise ValueError(f"step {t} outside the force series ({force.n_steps} x {force.nz})")
        fptr = force.ptr
    if status is not None or cfg is not None:
        if acc is not None:
            _same_grid(f_in, acc)
        N.check(N.lib().sw_step_checked(g.gp, f_in.dtype, f_in.ptr, f_out.ptr, flag.ptr, flag.tiles_ptr,
                                        _uin(uin).ptr, float(nu0), float(cs), int(x_sponge), float(nu_sponge),
                                        fptr, int(t), acc.ptr if acc is not None else None,
                                        -1 if cfg is None else int(cfg),
                                        status.ptr if status is not None else None, _stream(stream)),
                "sw_step_checked")
    elif acc is None:
        N.check(N.lib().sw_step(g.gp, f_in.dtype, f_in.ptr, f_out.ptr, flag.ptr, flag.tiles_ptr, _uin(uin).ptr,
                                float(nu0), float(cs), int(x_sponge), float(nu_sponge), fptr, int(t),
                                _stream(stream)), "sw_step")
    else:
        _same_grid(f_in, acc)
        N.check(N.lib().sw_step_accum(g.gp, f_in.dtype, f_in.ptr, f_out.ptr, flag.ptr, flag.tiles_ptr,
                                      _uin(uin).ptr, float(nu0), float(cs), int(x_sponge), float(nu_sponge), fptr,
                                      int(t), acc.ptr, _stream(stream)), "sw_step_accum")


def k_step_aa(f: Lattice, odd, flag: Flags, uin, nu0, cs, x_sponge, nu_sponge=0.05,
              force: ForceSeries = None, t=0, ghost=None, acc: Accum = None, stream=None,
              status: StatusWord = None):
    """One AA-pattern step on a single lattice, in place (see include/stonewall.h, sw_step_aa)."""
    g = _same_grid(f, flag)
    if ghost is None or ghost.numel() < N.lib().sw_aa_ghost_elems(g.gp) * N.DTYPE_BYTES[f.dtype]:
        raise ValueError("ghost buffer too small")
    fptr = None
    if force is not None:
        if force.nz != g.nz or not (0 <= int(t) < force.n_steps):
            raise ValueError(f"step {t} outside the force series ({force.n_steps} x {force.nz})")
        fptr = force.ptr
    N.check(N.lib().sw_step_aa(g.gp, f.dtype, f.ptr, int(bool(odd)), flag.ptr, flag.tiles_ptr,
                               _uin(uin).ptr, float(nu0), float(cs), int(x_sponge), float(nu_sponge), fptr, int(t),
                               acc.ptr if acc is not None else None, _ptr(ghost),
                               status.ptr if status is not None else None, _stream(stream)), "sw_step_aa")


def k_macro(f: Lattice, flag: Flags, u: Macro, stream=None):
    """lbm3d.py:158-182."""
    g = _same_grid(f, flag, u)
    N.check(N.lib().sw_macro(g.gp, f.dtype, f.ptr, flag.ptr, u.ptr, _stream(stream)), "sw_macro")


def k_accum(u: Macro, acc: Accum, stream=None):
    """lbm3d.py:185-188 (sums kept in float64)."""
    g = _same_grid(u, acc)
    N.check(N.lib().sw_accum(g.gp, u.ptr, acc.ptr, _stream(stream)), "sw_accum")


def k_macro_accum(f: Lattice, flag: Flags, acc: Accum, u: Macro = None, stream=None):
    """k_macro then k_accum (lbm3d.py:367-369) in one pass over f."""
    g = _same_grid(f, flag, acc)
    N.check(N.lib().sw_macro_accum(g.gp, f.dtype, f.ptr, flag.ptr, u.ptr if u is not None else None, acc.ptr,
                                   _stream(stream)), "sw_macro_accum")


def _out_f32(out, shape, what):
    if not (isinstance(out, torch.Tensor) and out.is_cuda and out.dtype == torch.float32 and out.is_contiguous()
            and tuple(out.shape) == tuple(shape)):
        raise ValueError(f"{what}: out must be a contiguous float32 CUDA tensor of shape {tuple(shape)}")
    return _ptr(out)


def k_slice_xz(u: Macro, y0, out, stream=None):
    """lbm3d.py:191-194: out[c, x, z] = u[c, x, y0, z] (out: float32 CUDA tensor (4, nx, nz))."""
    g = u.grid
    N.check(N.lib().sw_slice_xz(g.gp, u.ptr, int(y0), _out_f32(out, (4, g.nx, g.nz), "k_slice_xz"),
                                _stream(stream)), "sw_slice_xz")


def k_slice_xy(u: Macro, z0, out, stream=None):
    """lbm3d.py:197-200: out[c, x, y] = u[c, x, y, z0] (out: float32 CUDA tensor (4, nx, ny))."""
    g = u.grid
    N.check(N.lib().sw_slice_xy(g.gp, u.ptr, int(z0), _out_f32(out, (4, g.nx, g.ny), "k_slice_xy"),
                                _stream(stream)), "sw_slice_xy")


def k_qcoarse(u: Macro, flag: Flags, x0, ds, nx, ny, nz, out, stream=None):
    """lbm3d.py:225-238: Q-criterion max-pooled over ds^3 blocks from x = x0 (out: float32 CUDA tensor)."""
    g = _same_grid(u, flag)
    if (int(nx), int(ny), int(nz)) != (g.nx, g.ny, g.nz):
        raise ValueError("k_qcoarse: grid extents do not match the field")
    di, dj, dk = (int(v) for v in out.shape)
    N.check(N.lib().sw_qcoarse(g.gp, u.ptr, flag.ptr, int(x0), int(ds), di, dj, dk,
                               _out_f32(out, (di, dj, dk), "k_qcoarse"), _stream(stream)), "sw_qcoarse")


def launch(kernel, dim, inputs, device=None, stream=None):
    """wp.launch-compatible entry: the reference's input lists, tables included."""
    a = list(inputs)
    if kernel is k_init:
        f, flag, uin, cx, cy, cz, w, noise, seed = a
        _check_c(cx, cy, cz)
        _check_w(w)
        _check_dim(dim, f.grid)
        return k_init(f, flag, uin, noise, seed, stream=stream)
    if kernel is k_step:
        (f_in, f_out, flag, uin, cx, cy, cz, w, opp, mirz, nx, ny, nz, nu0, cs, x_sponge, nu_sponge, force,
         t) = a
        check_tables(*(_as_np(v) for v in (cx, cy, cz, w, opp, mirz)))
        _check_dim(dim, f_in.grid)
        return k_step(f_in, f_out, flag, uin, nx, ny, nz, nu0, cs, x_sponge, nu_sponge, force, t, stream=stream)
    if kernel is k_macro:
        f, flag, cx, cy, cz, u = a
        _check_c(cx, cy, cz)
        _check_dim(dim, f.grid)
        return k_macro(f, flag, u, stream=stream)
    if kernel is k_accum:
        u, acc = a
        return k_accum(u, acc, stream=stream)
    if kernel is k_slice_xz:
        u, y0, out = a
        return k_slice_xz(u, y0, out, stream=stream)
    if kernel is k_slice_xy:
        u, z0, out = a
        return k_slice_xy(u, z0, out, stream=stream)
    if kernel is k_qcoarse:
        u, flag, x0, ds, nx, ny, nz, out = a
        if tuple(int(d) for d in dim) != tuple(out.shape):
            raise ValueError("k_qcoarse: launch dim must be the output shape")
        return k_qcoarse(u, flag, x0, ds, nx, ny, nz, out, stream=stream)
    raise ValueError(f"unknown kernel {kernel!r}")


def _as_np(a):
    if isinstance(a, DeviceVector):
        return a.host
    if isinstance(a, torch.Tensor):
        return a.detach().cpu().numpy()
    return np.asarray(a)


def _check_c(cx, cy, cz):
    from .lattice import C
    for k, arr in enumerate((cx, cy, cz)):
        if not np.array_equal(_as_np(arr).astype(np.int32).ravel(), C[:, k]):
            raise ValueError("velocity table differs from the D3Q19 set compiled into the kernels")


def _check_w(w):
    from .lattice import W
    if not np.array_equal(_as_np(w).astype(np.float32).ravel(), W):
        raise ValueError("weight table differs from the D3Q19 set compiled into the kernels")


def _check_dim(dim, grid):
    if tuple(int(d) for d in dim) != (grid.nx, grid.ny, grid.nz):
        raise ValueError(f"launch dim {tuple(dim)} does not match the grid {grid}")


def synchronize_device(device=None):
    torch.cuda.synchronize()


def tables_host():
    """The reference's table arrays (cx, cy, cz, w, opp, mirz) for launch() input lists."""
    from .lattice import C, MIRZ, OPP, W
    return (np.ascontiguousarray(C[:, 0]), np.ascontiguousarray(C[:, 1]), np.ascontiguousarray(C[:, 2]), W, OPP,
            MIRZ)


__all__ = ["DeviceVector", "k_init", "k_step", "k_step_aa", "k_macro", "k_accum", "k_macro_accum", "k_slice_xz",
           "k_slice_xy", "k_qcoarse", "launch",
           "synchronize_device", "tables_host"]
