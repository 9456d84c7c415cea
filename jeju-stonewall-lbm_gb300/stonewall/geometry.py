"""Stone-wall voxel masks (host side, NumPy; produced once per solve, not timed).

Two producers:

course_wall(...)    the reference's dry-stone wall of stonewall3d/geometry.py:
                    superellipsoid stones laid course by course, each dropped on
                    the ones below, then shrunk in place by a common factor found
                    by bisection so the frontal (see-through) porosity hits the
                    target; porosity 0 adds a mortar core.  Same seed -> same
                    mask as the reference: the random draws happen in the same
                    order and every inside test uses the same arithmetic.
ellipsoid_wall(...) ellipsoids with semi-axes U[0.15H, 0.3H] and a uniformly
                    random orientation, placed at uniformly random centres in
                    the wall box and kept only while the box's solid fraction
                    stays at or below 1 - porosity (a candidate that would
                    overshoot by more than half of its own new volume is
                    rejected); porosity 0 fills the box.

Both return a bool mask (nx, ny, nz), y periodic, cell k centred at height
k - 0.5 above the ground; the caller adds the ground plane (flag[:, :, 0]).
"""
import numpy as np


# ---------------------------------------------------------------- reference wall (geometry.py)
def _half_height(dy, b, p):
    """Superellipse half-height at offset dy (zero outside |dy| < b), geometry.py:13-16."""
    r = 1.0 - np.clip(np.abs(dy) / b, 0, 1) ** p
    return np.where(np.abs(dy) < b, r ** (1.0 / p), 0.0)


def _draw_courses(H, Ly, rng):
    """Course heights, then per course stone lengths and shapes (geometry.py:19-41, same draw order)."""
    heights, z = [], 0.0
    while z < H * 0.97:
        h = rng.uniform(0.26, 0.38) * H
        heights.append(h)
        z += h
    courses = []
    for h in heights:
        lengths, total = [], 0.0
        while total < Ly:
            L = rng.uniform(0.45, 0.9) * H
            lengths.append(L)
            total += L
        lengths = np.array(lengths) * Ly / total
        y = rng.uniform(0, Ly)
        course = []
        for L in lengths:
            c = 0.5 * h * rng.uniform(0.85, 1.1)
            p = rng.uniform(2.2, 3.2)
            dx = rng.uniform(-0.08, 0.08)
            ax = rng.uniform(0.85, 1.0)
            course.append(dict(yc=(y + L / 2) % Ly, L=L, c=c, p=p, dx=dx, ax=ax))
            y += L
        courses.append(course)
    return courses


def _lay(courses, gap, H, Ly):
    """Drop the stones course by course onto the running top profile (geometry.py:44-65)."""
    ny = int(round(Ly))
    yc = np.arange(ny) + 0.5
    top = np.zeros(ny)
    stones = []
    for course in courses:
        new_top = top.copy()
        for st in course:
            b = 0.5 * st["L"] * (1.0 - gap)
            dy = (yc - st["yc"] + Ly / 2) % Ly - Ly / 2
            prof = _half_height(dy, b, st["p"]) * st["c"]
            inside = np.abs(dy) < b
            zc = np.max(top[inside] + prof[inside])
            new_top = np.where(inside, np.maximum(new_top, zc + prof), new_top)
            stones.append(dict(st, b=b, zc=zc))
        top = new_top
    stretch = H / top.mean()
    for st in stones:
        st["zc"] *= stretch
        st["c"] *= stretch
    return stones


def _voxelize(stones, nx, ny, nz, X0, T):
    """Cells whose centre lies inside a stone's superellipsoid (geometry.py:68-84)."""
    m = np.zeros((nx, ny, nz), bool)
    xmid = X0 + T / 2
    for st in stones:
        a, b, c, p = st["ax"] * T / 2, st["b"], st["c"], st["p"]
        xc = xmid + st["dx"] * T
        xi = np.arange(int(np.floor(xc - a)), int(np.ceil(xc + a)) + 1)
        ki = np.arange(max(1, int(np.floor(st["zc"] - c))), min(nz, int(np.ceil(st["zc"] + c)) + 2))
        yi = np.arange(int(np.floor(st["yc"] - b)) - 1, int(np.ceil(st["yc"] + b)) + 2)
        if len(xi) == 0 or len(ki) == 0:
            continue
        X, Y, K = np.meshgrid(xi + 0.5, yi + 0.5, ki - 0.5, indexing="ij")
        r = (np.abs(X - xc) / a) ** p + (np.abs(Y - st["yc"]) / b) ** p + (np.abs(K - st["zc"]) / c) ** p
        hit = r <= 1.0
        xs, ys, ks = np.meshgrid(xi, yi % ny, ki, indexing="ij")
        m[xs[hit], ys[hit], ks[hit]] = True
    return m


def _silhouette(stones, ny, nz):
    """Wall outline seen along x (geometry.py:87-97)."""
    yc = np.arange(ny) + 0.5
    kc = np.arange(nz) - 0.5
    m = np.zeros((ny, nz), bool)
    for st in stones:
        dy = (yc - st["yc"] + ny / 2) % ny - ny / 2
        half = _half_height(dy, st["b"], st["p"]) * st["c"]
        m |= np.abs(kc[None, :] - st["zc"]) < half[:, None]
    m[:, 0] = False
    return m


def frontal_porosity(front, H):
    """See-through fraction of the nominal face y in [0, Ly), height in [0, H) (geometry.py:100-102)."""
    return 1.0 - front[:, 1:int(round(H)) + 1].mean()


def _tag_anchors(stones, ny):
    """Mark top-line stones and ground stones (geometry.py:105-118)."""
    yc = np.arange(ny) + 0.5
    env = np.zeros(ny)
    tops = []
    for st in stones:
        dy = (yc - st["yc"] + ny / 2) % ny - ny / 2
        t = np.where(np.abs(dy) < st["b"], st["zc"] + _half_height(dy, st["b"], st["p"]) * st["c"], -np.inf)
        tops.append(t)
        env = np.maximum(env, t)
    for st, t in zip(stones, tops):
        st["top"] = bool(np.any(t >= env - 0.5))
        st["ground"] = bool(st["zc"] - st["c"] < 0.02 * st["c"] + 1e-6)
    return stones


def _shrunk(stones, s):
    """Scale y and z extents by s about each centre; top stones keep their top, ground stones
    keep touching the ground (geometry.py:121-132)."""
    out = []
    for st in stones:
        n = dict(st, b=st["b"] * s, c=st["c"] * s)
        if st["top"]:
            n["zc"] = st["zc"] + st["c"] * (1 - s)
        elif st["ground"]:
            n["zc"] = st["zc"] - st["c"] * (1 - s)
        out.append(n)
    return out


def course_wall(porosity, H, nx, ny, nz, X0, T, seed=7, verbose=False):
    """The reference's wall (geometry.py:135-161).  Returns (mask, frontal porosity)."""
    rng = np.random.default_rng(seed)
    base = _tag_anchors(_lay(_draw_courses(H, ny, rng), 0.0, H, ny), ny)
    if porosity <= 0.0:
        m = _voxelize(base, nx, ny, nz, X0, T)
        xa, xb = X0 + int(round(0.15 * T)), X0 + int(round(0.85 * T))
        col = m.any(axis=0)
        for j in range(ny):
            ks = np.nonzero(col[j])[0]
            if len(ks):
                m[xa:max(xb, xa + 1), j, 1:ks.max() + 1] = True
        s = 1.0
    else:
        lo, hi = 0.4, 1.2
        for _ in range(24):
            s = 0.5 * (lo + hi)
            phi = frontal_porosity(_silhouette(_shrunk(base, s), ny, nz), H)
            lo, hi = (s, hi) if phi > porosity else (lo, s)
        m = _voxelize(_shrunk(base, s), nx, ny, nz, X0, T)
    phi = frontal_porosity(m.any(axis=0), H)
    if verbose:
        print(f"[wall] stones={len(base)} scale={s:.3f} frontal porosity={phi:.3f}", flush=True)
    return m, phi


# ---------------------------------------------------------------- ellipsoid packing
def _random_rotation(rng):
    """Uniform random rotation matrix (normalised Gaussian quaternion)."""
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    w, x, y, z = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def ellipsoid_wall(porosity, H, nx, ny, nz, X0, T, seed=0, height=None, max_tries=200000, verbose=False):
    """Rejection-packed ellipsoid stones in the box x in [X0, X0+T), all y (periodic), z in [1, height].

    Returns (mask, solid fraction of the box).  The fill stops once the box's
    solid fraction reaches 1 - porosity (to within half a stone).
    """
    height = int(round(H)) if height is None else int(height)
    z_hi = min(nz, 1 + height)
    m = np.zeros((nx, ny, nz), bool)
    box = (slice(X0, X0 + T), slice(0, ny), slice(1, z_hi))
    box_cells = T * ny * (z_hi - 1)
    target = (1.0 - porosity) * box_cells
    if porosity <= 0.0:
        m[box] = True
        return m, 1.0
    rng = np.random.default_rng(seed)
    solid = 0
    tries = 0
    while solid < target - 0.5 and tries < max_tries:
        tries += 1
        centre = np.array([rng.uniform(X0, X0 + T), rng.uniform(0, ny), rng.uniform(0.5, z_hi - 0.5)])
        semi = rng.uniform(0.15 * H, 0.3 * H, size=3)
        R = _random_rotation(rng)
        ext = semi.max()
        lo = np.floor(centre - ext).astype(int)
        hi = np.ceil(centre + ext).astype(int) + 1
        xi = np.arange(max(lo[0], X0), min(hi[0], X0 + T))
        ki = np.arange(max(lo[2], 1), min(hi[2], z_hi))
        yi = np.arange(lo[1], hi[1])
        if len(xi) == 0 or len(ki) == 0:
            continue
        X, Y, K = np.meshgrid(xi + 0.5, yi + 0.5, ki - 0.5, indexing="ij")
        d = np.stack([X - centre[0], Y - centre[1], K - centre[2]], -1) @ R   # body frame
        inside = ((d / semi) ** 2).sum(-1) <= 1.0
        xs, ys, ks = np.meshgrid(xi, yi % ny, ki, indexing="ij")
        xs, ys, ks = xs[inside], ys[inside], ks[inside]
        new = ~m[xs, ys, ks]
        n_new = int(np.unique(np.stack([xs[new], ys[new], ks[new]]), axis=1).shape[1]) if new.any() else 0
        if n_new == 0 or solid + n_new > target + 0.5 * n_new:
            continue
        m[xs, ys, ks] = True
        solid += n_new
    frac = float(m[box].sum()) / box_cells
    if verbose:
        print(f"[wall] ellipsoids: solid fraction {frac:.3f} (target {1 - porosity:.3f}) after {tries} tries",
              flush=True)
    return m, frac
