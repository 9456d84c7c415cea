"""D3Q19 lattice tables and cell flags.

The direction order, weights and the opposite / z-mirror maps are those of
stonewall3d/lbm3d.py:20-30: the order is part of the checkpoint format
(f.npy stores populations in this order), so it must stay identical.  The
CUDA kernels compile the same tables in (csrc/sw_common.cuh); tests compare
the two with the reference's own arrays.
"""
import numpy as np

Q = 19

# rest, the 6 axis directions (+-x, +-y, +-z), then the 12 edge directions in
# (+,+), (-,-), (+,-), (-,+) order for the xy, xz and yz planes
_AXES = [(1, 0, 0), (0, 1, 0), (0, 0, 1)]


def _velocities():
    c = [(0, 0, 0)]
    for a in _AXES:
        c.append(a)
        c.append(tuple(-v for v in a))
    for p, q in ((0, 1), (0, 2), (1, 2)):
        for sp, sq in ((1, 1), (-1, -1), (1, -1), (-1, 1)):
            v = [0, 0, 0]
            v[p], v[q] = sp, sq
            c.append(tuple(v))
    return np.array(c, dtype=np.int32)


C = _velocities()
W = np.array([1 / 3 if (v == 0).all() else (1 / 18 if np.abs(v).sum() == 1 else 1 / 36) for v in C],
             dtype=np.float32)
OPP = np.array([int(np.flatnonzero((C == -v).all(1))[0]) for v in C], dtype=np.int32)
MIRZ = np.array([int(np.flatnonzero((C == v * np.array([1, 1, -1])).all(1))[0]) for v in C], dtype=np.int32)

FLUID, WALL, GROUND = 0, 1, 2


def check_tables(cx, cy, cz, w, opp, mirz):
    """Raise ValueError unless the given arrays are this D3Q19 set (the kernels have it compiled in)."""
    got = [np.asarray(a).ravel() for a in (cx, cy, cz, w, opp, mirz)]
    want = [C[:, 0], C[:, 1], C[:, 2], W, OPP, MIRZ]
    for name, g, e in zip(("cx", "cy", "cz", "w", "opp", "mirz"), got, want):
        if g.shape != e.shape or not np.array_equal(g.astype(e.dtype), e):
            raise ValueError(f"lattice table {name} differs from the D3Q19 set compiled into the kernels")
