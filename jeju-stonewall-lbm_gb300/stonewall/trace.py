"""NVTX ranges for timeline profilers (Nsight Systems, ncu's range filters).

trace.range("name") marks a host-side phase -- a solver's graph replay, a
batch chunk, the server's admission, retirement or status check -- on the
CUDA timeline.  Without a profiler attached the markers cost a function call.
"""
import contextlib

import torch


@contextlib.contextmanager
def range(name):  # noqa: A001  (the NVTX term)
    torch.cuda.nvtx.range_push(name)
    try:
        yield
    finally:
        torch.cuda.nvtx.range_pop()
