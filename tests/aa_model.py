"""CPU model of the AA-pattern (in-place) step, used to check its memory access plan.

The ping-pong step pulls, for every fluid non-inlet cell x and direction i, the
population j at source s (pull_source below, the rules of lbm3d.py:77-95:
periodic y, outlet copies column x, top mirrors z, non-fluid sources bounce
back f_opp(i) from x itself).  The AA pattern keeps one lattice A and
alternates two kernels:

  odd  step: the state S (post-collision) sits in "swapped" slots,
             A[opp(k)][x] = S_k(x) (the kernels keep slot s in plane opp(s),
             so in memory that is the usual layout, plane k = S_k); a
             state in plain slots, A[k] = S_k, would race: cell x reads
             A[i] of x - c_i, which cell x - 2 c_i rewrites.  Cell x
             gathers what the pull would read
             (slot opp(j) at s, or slot i at x for a bounce-back), collides,
             and scatters each new S_k(x) to every slot the next even step
             will read it from (odd_targets).  The outlet copy (a cell at
             x = nx - 1 takes c_x = -1 populations from its own column) is the
             one rule without that symmetry: its slots are rewritten in the
             same step by other cells.  So the five c_x = -1 populations of
             the outlet plane are copied to a ghost buffer before the odd
             step, and the outlet copies read the ghost;
  even step: cell x reads A[i][x] for all i (everything arrived in place),
             collides, writes S_k(x) to A[opp(k)][x].

The checks in tests/test_aa_model.py run these plans on small grids with
every boundary kind and verify: no slot is written twice, every slot a cell
reads in the odd step is written (if at all) by that same cell, and two AA
steps give exactly what two ping-pong steps give.
"""
import numpy as np

C = np.array([(0, 0, 0), (1, 0, 0), (-1, 0, 0), (0, 1, 0), (0, -1, 0), (0, 0, 1), (0, 0, -1),
              (1, 1, 0), (-1, -1, 0), (1, -1, 0), (-1, 1, 0), (1, 0, 1), (-1, 0, -1), (1, 0, -1), (-1, 0, 1),
              (0, 1, 1), (0, -1, -1), (0, 1, -1), (0, -1, 1)])
OPP = [0, 2, 1, 4, 3, 6, 5, 8, 7, 10, 9, 12, 11, 14, 13, 16, 15, 18, 17]
MIRZ = [0, 1, 2, 3, 4, 6, 5, 7, 8, 9, 10, 13, 14, 11, 12, 17, 18, 15, 16]


def pull_source(flag, x, y, z, i, clamped=False):
    """((xs, ys, zs), j, bounced[, clamped]) for cell (x, y, z) and direction i."""
    nx, ny, nz = flag.shape
    xs, ys, zs, j = x - C[i][0], (y - C[i][1]) % ny, z - C[i][2], i
    cl = False
    if xs >= nx:
        xs, cl = x, True
    if zs >= nz:
        zs, j = z, MIRZ[i]
    b = zs < 0 or flag[xs, ys, zs] != 0
    return ((xs, ys, zs), j, b, cl) if clamped else ((xs, ys, zs), j, b)


def pulls(flag, x):
    return x[0] > 0 and flag[x] == 0


def odd_targets(flag, x, k):
    """Slots (population, cell) that must receive S_k(x) in the odd step.

    (a) the cell x + c_k when it is inside the domain and fluid (it pulls k from x);
    (b) at the outlet (x = nx - 1) for c_x = -1: the cell (nx - 1, y + c_y, z + c_z),
        which copies column nx - 1 instead of pulling from x = nx;
    (c) at the top (z = nz - 1) for c_z = +1: the cell (x + c_x, y + c_y, nz - 1),
        which mirrors z and takes population k into its slot MIRZ(k);
        with c_x = -1 at the outlet also (nx - 1, y + c_y, nz - 1);
    (d) x itself, slot opp(k), when the pull of opp(k) at x bounces back.
    Cells that do not pull (inlet x = 0) may receive harmless writes; solid
    cells never do.
    """
    nx, ny, nz = flag.shape
    cx, cy, cz = C[k]
    out = []
    X, Y, Z = x
    yk = (Y + cy) % ny
    if pull_source(flag, X, Y, Z, OPP[k])[2]:
        out.append((OPP[k], (X, Y, Z)))                                    # (d)
    tx, tz = X + cx, Z + cz
    if 0 <= tx < nx and 0 <= tz < nz and flag[tx, yk, tz] == 0:
        out.append((k, (tx, yk, tz)))                                      # (a)
    if X == nx - 1 and cx == -1 and 0 <= tz < nz and flag[X, yk, tz] == 0:
        out.append((k, (X, yk, tz)))                                       # (b)
    if Z == nz - 1 and cz == 1:
        if 0 <= tx < nx and flag[tx, yk, Z] == 0:
            out.append((MIRZ[k], (tx, yk, Z)))                             # (c)
        if X == nx - 1 and cx == -1 and flag[X, yk, Z] == 0:
            out.append((MIRZ[k], (X, yk, Z)))                              # (c) at the outlet
    return out


def collide_linear(g, M):
    return M @ g


def pingpong_step(S, flag, M):
    nx, ny, nz = flag.shape
    out = S.copy()
    for x in np.ndindex(nx, ny, nz):
        if flag[x] != 0:
            continue
        if x[0] == 0:
            out[:, x[0], x[1], x[2]] = M[0]                                 # any fixed inlet state
            continue
        g = np.empty(19)
        for i in range(19):
            s, j, b = pull_source(flag, *x, i)
            g[i] = S[OPP[i], x[0], x[1], x[2]] if b else S[j, s[0], s[1], s[2]]
        out[:, x[0], x[1], x[2]] = collide_linear(g, M)
    return out


def aa_two_steps(S, flag, M, check=True):
    """Run odd + even AA steps on S; returns (state after 2 steps, access log problems)."""
    nx, ny, nz = flag.shape
    A = np.empty_like(S)
    for k in range(19):
        A[OPP[k]] = S[k]                                                    # swapped slots
    problems = []
    # odd step: one pass; outlet copies read the ghost (the state before the step)
    writer = {}
    readers = {}
    ghost = A.copy()
    for x in np.ndindex(nx, ny, nz):
        if flag[x] != 0:
            continue
        if x[0] == 0:
            new = M[0].copy()
        else:
            g = np.empty(19)
            for i in range(19):
                s, j, b, cl = pull_source(flag, *x, i, clamped=True)
                slot = (i, x) if b else (OPP[j], tuple(s))
                if cl and not b:
                    g[i] = ghost[slot[0]][slot[1]]
                    continue
                readers.setdefault(slot, set()).add(x)
                g[i] = A[slot[0]][slot[1]] if slot not in writer else np.nan   # must not be written yet
                if slot in writer and writer[slot] != x:
                    problems.append(("read after another cell wrote", slot, writer[slot], x))
            new = collide_linear(g, M)
        for k in range(19):
            for (p, cell) in odd_targets(flag, x, k):
                key = (p, cell)
                if key in writer:
                    problems.append(("written twice", key, writer[key], x))
                writer[key] = x
                A[p][cell] = new[k]
    for key, w in writer.items():
        for r in readers.get(key, ()):
            if r != w:
                problems.append(("read by another cell", key, w, r))
    # even step: everything in place
    B = A.copy()
    for x in np.ndindex(nx, ny, nz):
        if flag[x] != 0:
            continue
        new = M[0].copy() if x[0] == 0 else collide_linear(np.array([A[i][x] for i in range(19)]), M)
        for k in range(19):
            B[OPP[k]][x] = new[k]
    S2 = np.empty_like(S)
    for k in range(19):
        S2[k] = B[OPP[k]]
    return S2, problems
