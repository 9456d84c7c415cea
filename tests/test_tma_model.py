"""CPU model of the TMA-staged step's addressing (csrc/sw_tma.cuh).

For every fast-path cell and population it rebuilds where the kernel reads the
pulled value -- the stage box of the population (origin x0 - 8, y0 - c_y, the
level z - c_z or, at the top, the mirrored population on level z), the warp's
row in it or the one-row wrap slot, the lane's word and half -- and checks that
this is the source the reference pull names (lbm3d.py:77-97: periodic y, the
outlet copying its own column, the top mirroring z).  Grids with odd sizes,
one-row-group widths and a last segment that ends mid-warp.
"""
import pytest

from aa_model import C, MIRZ

WY, BOX_X = 4, 80


def pull_source(nx, ny, nz, x, y, z, i):
    """(xs, ys, zs, j) of the reference pull for an all-fluid neighbourhood."""
    xs, ys, zs, j = x - C[i][0], (y - C[i][1]) % ny, z - C[i][2], i
    if xs >= nx:
        xs = x
    if zs >= nz:
        zs, j = z, MIRZ[i]
    return xs, ys, zs, j


def staged_source(nx, ny, nz, x, y, z, i):
    """What the kernel reads for cell x (lane l of pair segment bx, warp row y)."""
    bx, lane = x // 64, (x % 64) // 2
    x0 = 64 * bx + 2 * lane                          # the lane's first cell
    half = x - x0                                    # 0: cell x0, 1: cell x0 + 1
    y0 = (y // WY) * WY
    w = y - y0
    ex, ey, ez = C[i]
    top = z == nz - 1
    pop = MIRZ[i] if (ez == -1 and top) else i
    zl = z if (ez == -1 and top) else z - ez
    # the box row the warp reads: rows y0 - ey .. y0 - ey + 3 of the box; the wrap slot
    # holds row ny - 1 (c_y = +1, y = 0) or row 0 (c_y = -1, y = ny - 1)
    if ey == 1 and y == 0:
        row_y = ny - 1
    elif ey == -1 and y == ny - 1:
        row_y = 0
    else:
        row_y = y0 - ey + w
        assert 0 <= row_y < ny                       # inside the lattice: no zero fill used
    box_x0 = 64 * bx - 8
    lane_word = 4 + lane                             # elements 8 + 2 lane, 9 + 2 lane
    has_b, has_r = x0 + 1 < nx, x0 + 2 < nx
    if ex == 0:
        elem = 2 * lane_word + half
    elif ex == 1:                                    # (hi(word - 1), lo(word))
        elem = 2 * (lane_word - 1) + 1 if half == 0 else 2 * lane_word
    else:                                            # (has_b ? own.y : own.x, has_r ? lo(word + 1) : own.y)
        if half == 0:
            elem = 2 * lane_word + (1 if has_b else 0)
        else:
            elem = 2 * (lane_word + 1) if has_r else 2 * lane_word + 1
    xs = box_x0 + elem
    assert 0 <= elem < BOX_X
    return xs, row_y, zl, pop


@pytest.mark.parametrize("shape", [(64, 4, 3), (70, 9, 5), (129, 6, 4), (200, 13, 7), (33, 1, 3)])
def test_staged_reads_are_the_pull_sources(shape):
    nx, ny, nz = shape
    for x in range(1, nx):                           # x = 0 is the inlet (no pulls)
        for y in range(ny):
            for z in range(1, nz):                   # z = 0 is ground: never the fast path
                for i in range(19):
                    assert staged_source(nx, ny, nz, x, y, z, i) == pull_source(nx, ny, nz, x, y, z, i), \
                        (shape, x, y, z, i)


def test_staged_reads_on_generated_grids():
    hyp = pytest.importorskip("hypothesis")
    st = pytest.importorskip("hypothesis.strategies")

    @hyp.settings(max_examples=15, deadline=None, derandomize=True)
    @hyp.given(nx=st.integers(2, 140), ny=st.integers(1, 11), nz=st.integers(2, 5))
    def check(nx, ny, nz):
        for x in range(1, nx):
            for y in range(ny):
                for z in range(1, nz):
                    for i in range(19):
                        assert staged_source(nx, ny, nz, x, y, z, i) == pull_source(nx, ny, nz, x, y, z, i)

    check()
