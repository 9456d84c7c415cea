"""Launch-configuration autotuner for the fused step.

The step is compiled in several launch configurations (block shape x register
budget, SW_STEP_CONFIGS in csrc/sw_step.cuh).  Which one hides memory latency
best depends on the storage type and the grid, so it is measured: each
configuration steps the solver's current state into its spare lattice a few
times (the state itself is not modified, and the spare lattice is overwritten
by the next real step anyway), timed with CUDA events, and the fastest is
installed for that storage type with sw_set_step_config.  Results are cached
per (device name, dtype, grid) for the life of the process.
"""
import torch

from . import _native as N
from .fields import _stream

_CACHE = {}


def config_count():
    return N.lib().sw_step_config_count()


def time_configs(solver, repeats=8, warmup=2, acc=None):
    """Mean step time in ms of every configuration on the solver's grid (with `acc`, an Accum
    that receives throw-away sums, the accumulating variant).  A configuration whose TMA-staged
    blocks gave up waiting for their copies (a time-out in its status word or in
    sw_tma_timeouts) computed an invalid step and is left out, so it can never win by skipping work."""
    from .fields import StatusWord
    L = N.lib()
    g = solver.grid
    src, dst = solver.f[solver.cur], solver.f[1 - solver.cur]
    stream = torch.cuda.current_stream()
    accp = acc.ptr if acc is not None else None
    status = StatusWord(device=solver.device)
    res = {}
    for cfg in range(config_count()):
        status.clear()
        L.sw_tma_timeouts()                           # read and clear the process-wide counter

        def launch():
            return L.sw_step_checked(g.gp, src.dtype, src.ptr, dst.ptr, solver.flags.ptr, solver.flags.tiles_ptr,
                                     solver.uin.ptr, solver.nu0, solver.cs, solver.x_sponge, solver.nu_sponge,
                                     None, 0, accp, cfg, status.ptr, _stream(stream))
        rc = launch()
        if rc == N.SW_ERR_UNSUPPORTED:
            continue                                  # not compiled for this storage type
        N.check(rc, "sw_step_checked")
        for _ in range(warmup - 1):
            N.check(launch(), "sw_step_checked")
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record()
        for _ in range(repeats):
            N.check(launch(), "sw_step_checked")
        e1.record()
        torch.cuda.synchronize()
        timed_out = bool(status.read() & N.SW_STATUS_TIMEOUT)
        if L.sw_tma_timeouts() != 0 or timed_out:      # (reading the counter also clears it)
            continue
        res[cfg] = e0.elapsed_time(e1) / repeats
    if not res:
        raise RuntimeError("no launch configuration completed a step without a device wait time-out")
    return res


def tune(solver, repeats=8, force=False, accumulating=True):
    """Pick and install the fastest configuration for the solver's storage type, for plain and for
    accumulating steps; returns (cfg, times) of the plain steps."""
    from .fields import Accum
    g = solver.grid
    key = (torch.cuda.get_device_name(solver.device), solver.dtype, g.nx, g.ny, g.nz)
    if key in _CACHE and not force:
        best, times, best_acc = _CACHE[key]
    else:
        times = time_configs(solver, repeats=repeats)
        best = min(times, key=times.get)
        best_acc = best
        if accumulating:
            scratch = Accum(g, device=solver.device)
            acc_times = time_configs(solver, repeats=max(2, repeats // 2), acc=scratch)
            best_acc = min(acc_times, key=acc_times.get)
            del scratch
        _CACHE[key] = (best, times, best_acc)
    N.check(N.lib().sw_set_step_config(solver.dtype, best), "sw_set_step_config")
    N.check(N.lib().sw_set_step_config_accum(solver.dtype, best_acc), "sw_set_step_config_accum")
    return best, times


def current(dtype):
    return N.lib().sw_get_step_config(N.dtype_code(dtype))


__all__ = ["tune", "time_configs", "config_count", "current"]
