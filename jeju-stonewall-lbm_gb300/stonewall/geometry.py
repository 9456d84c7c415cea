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

With device="cuda" the per-cell work runs on the GPU (csrc/sw_geometry.cu):
the ellipsoid packer's accept/reject loop over candidates drawn here in the
same order, and the course wall's rasteriser; the masks are the host
generators' bit for bit (the random draws and the bisection stay here, the
packer's inside test is the same FMA-free float64 expression on both sides,
and the few rasteriser cells too close to a stone surface for two pow
implementations to agree are decided here).
"""
import ctypes

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


def _stone_box(st, nz, X0, T):
    """A stone's superellipsoid parameters and cell ranges (geometry.py:72-78)."""
    a, b, c, p = st["ax"] * T / 2, st["b"], st["c"], st["p"]
    xc = X0 + T / 2 + st["dx"] * T
    xr = (int(np.floor(xc - a)), int(np.ceil(xc + a)) + 1)
    kr = (max(1, int(np.floor(st["zc"] - c))), min(nz, int(np.ceil(st["zc"] + c)) + 2))
    yr = (int(np.floor(st["yc"] - b)) - 1, int(np.ceil(st["yc"] + b)) + 2)
    return xc, a, b, c, p, xr, yr, kr


def _superellipsoid_r(X, Y, K, xc, yc, zc, a, b, c, p):
    return (np.abs(X - xc) / a) ** p + (np.abs(Y - yc) / b) ** p + (np.abs(K - zc) / c) ** p


def _voxelize(stones, nx, ny, nz, X0, T, device=None):
    """Cells whose centre lies inside a stone's superellipsoid (geometry.py:68-84)."""
    if device is not None:
        return _voxelize_device(stones, nx, ny, nz, X0, T, device)
    m = np.zeros((nx, ny, nz), bool)
    for st in stones:
        xc, a, b, c, p, xr, yr, kr = _stone_box(st, nz, X0, T)
        xi, yi, ki = np.arange(*xr), np.arange(*yr), np.arange(*kr)
        if len(xi) == 0 or len(ki) == 0:
            continue
        X, Y, K = np.meshgrid(xi + 0.5, yi + 0.5, ki - 0.5, indexing="ij")
        hit = _superellipsoid_r(X, Y, K, xc, st["yc"], st["zc"], a, b, c, p) <= 1.0
        xs, ys, ks = np.meshgrid(xi, yi % ny, ki, indexing="ij")
        m[xs[hit], ys[hit], ks[hit]] = True
    return m


STONE_DTYPE = np.dtype([("xc", "f8"), ("yc", "f8"), ("zc", "f8"), ("a", "f8"), ("b", "f8"), ("c", "f8"),
                        ("p", "f8"), ("x0", "i4"), ("x1", "i4"), ("y0", "i4"), ("y1", "i4"), ("k0", "i4"),
                        ("k1", "i4")])                                  # sw_stone


def _voxelize_device(stones, nx, ny, nz, X0, T, device, cap=4096):
    """_voxelize on the GPU (sw_voxelize_stones); the cells it leaves undecided are decided here."""
    import torch
    from . import _native as N
    from .fields import _ptr
    recs = np.zeros(len(stones), STONE_DTYPE)
    for i, st in enumerate(stones):
        xc, a, b, c, p, xr, yr, kr = _stone_box(st, nz, X0, T)
        if xr[1] > xr[0] and kr[1] > kr[0] and (xr[0] < 0 or xr[1] > nx):
            raise ValueError(f"stone {i} reaches past the x extent of the grid")
        recs[i] = (xc, st["yc"], st["zc"], a, b, c, p, xr[0], xr[1], yr[0], yr[1], kr[0], kr[1])
    dev = torch.device(device)
    stream = torch.cuda.Stream(device=dev)                  # beside the solves' stream
    with N.CAPTURE_LOCK, torch.cuda.stream(stream):
        st_dev = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
        mask = torch.zeros(nx * ny * nz, dtype=torch.uint8, device=dev)
        amb = torch.zeros(1 + 4 * cap, dtype=torch.int32, device=dev)
        N.check(N.lib().sw_voxelize_stones(_ptr(st_dev), len(recs), nx, ny, nz, _ptr(mask), _ptr(amb), cap,
                                           ctypes.c_void_p(stream.cuda_stream)), "sw_voxelize_stones")
        m = mask.cpu().numpy().astype(bool).reshape(nx, ny, nz)
        amb_h = amb.cpu().numpy()
    n_amb = int(amb_h[0])
    if n_amb > cap:
        raise RuntimeError(f"{n_amb} cells next to stone surfaces exceed the list of {cap}")
    for s_i, x, yy, k in amb_h[1:1 + 4 * n_amb].reshape(-1, 4):
        r = recs[s_i]
        v = _superellipsoid_r(np.array([x + 0.5]), np.array([yy + 0.5]), np.array([k - 0.5]), r["xc"], r["yc"],
                              r["zc"], r["a"], r["b"], r["c"], r["p"])
        if v[0] <= 1.0:
            m[x, yy % ny, k] = True
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


def course_wall(porosity, H, nx, ny, nz, X0, T, seed=7, verbose=False, device=None):
    """The reference's wall (geometry.py:135-161).  Returns (mask, frontal porosity).  device: rasterise
    the stones on that GPU (the same mask)."""
    rng = np.random.default_rng(seed)
    base = _tag_anchors(_lay(_draw_courses(H, ny, rng), 0.0, H, ny), ny)
    if porosity <= 0.0:
        m = _voxelize(base, nx, ny, nz, X0, T, device)
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
        m = _voxelize(_shrunk(base, s), nx, ny, nz, X0, T, device)
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


def _draw_candidate(rng, H, ny, X0, T, z_hi):
    """One candidate stone of the packer, in the generator's draw order: centre, semi-axes,
    rotation, and the cell ranges of its bounding cube clipped to the wall box."""
    centre = np.array([rng.uniform(X0, X0 + T), rng.uniform(0, ny), rng.uniform(0.5, z_hi - 0.5)])
    semi = rng.uniform(0.15 * H, 0.3 * H, size=3)
    R = _random_rotation(rng)
    ext = semi.max()
    lo = np.floor(centre - ext).astype(int)
    hi = np.ceil(centre + ext).astype(int) + 1
    xr = (max(lo[0], X0), min(hi[0], X0 + T))
    kr = (max(lo[2], 1), min(hi[2], z_hi))
    return centre, semi, R, xr, (int(lo[1]), int(hi[1])), kr


def _ellipsoid_inside(X, Y, K, centre, semi, R):
    """Cell centres inside the rotated ellipsoid: body-frame coordinates d_j = sum_i a_i R[i, j] and
    sum_j (d_j / semi_j)^2 <= 1, each sum taken left to right (no matrix product, so the same float64
    operations run on any machine and in the GPU packer)."""
    dx, dy, dz = X - centre[0], Y - centre[1], K - centre[2]
    t0 = ((dx * R[0, 0] + dy * R[1, 0]) + dz * R[2, 0]) / semi[0]
    t1 = ((dx * R[0, 1] + dy * R[1, 1]) + dz * R[2, 1]) / semi[1]
    t2 = ((dx * R[0, 2] + dy * R[1, 2]) + dz * R[2, 2]) / semi[2]
    return ((t0 * t0 + t1 * t1) + t2 * t2) <= 1.0


ELLIPSOID_DTYPE = np.dtype([("centre", "f8", 3), ("semi", "f8", 3), ("rot", "f8", 9), ("x0", "i4"), ("x1", "i4"),
                            ("y0", "i4"), ("y1", "i4"), ("k0", "i4"), ("k1", "i4")])     # sw_ellipsoid


def ellipsoid_wall(porosity, H, nx, ny, nz, X0, T, seed=0, height=None, max_tries=200000, verbose=False,
                   device=None):
    """Rejection-packed ellipsoid stones in the box x in [X0, X0+T), all y (periodic), z in [1, height].

    Returns (mask, solid fraction of the box).  The fill stops once the box's
    solid fraction reaches 1 - porosity (to within half a stone).  device: run the
    accept/reject loop on that GPU (the same mask).
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
    if device is not None:
        tries = _pack_device(m, rng, H, ny, X0, T, z_hi, target, max_tries, device)
    else:
        solid = 0
        tries = 0
        while solid < target - 0.5 and tries < max_tries:
            tries += 1
            centre, semi, R, xr, yr, kr = _draw_candidate(rng, H, ny, X0, T, z_hi)
            xi, yi, ki = np.arange(*xr), np.arange(*yr), np.arange(*kr)
            if len(xi) == 0 or len(ki) == 0:
                continue
            X, Y, K = np.meshgrid(xi + 0.5, yi + 0.5, ki - 0.5, indexing="ij")
            inside = _ellipsoid_inside(X, Y, K, centre, semi, R)
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


def _pack_device(m, rng, H, ny, X0, T, z_hi, target, max_tries, device, first_batch=256, batch=1024):
    """The packer's loop on the GPU (sw_pack_ellipsoids), candidates drawn here in batches; fills m's
    wall box and returns the number of tries, as the host loop would."""
    import torch
    from . import _native as N
    from .fields import _ptr
    dev = torch.device(device)
    nbytes = int(N.lib().sw_pack_box_bytes(T, ny, z_hi))
    if nbytes < 0:
        raise ValueError("bad wall box")
    stream = torch.cuda.Stream(device=dev)                  # beside the solves' stream
    with N.CAPTURE_LOCK, torch.cuda.stream(stream):
        bits = torch.zeros(nbytes // 4, dtype=torch.int32, device=dev)
        state = torch.zeros(2, dtype=torch.int64, device=dev)
    tries = 0
    solid = 0
    n = min(first_batch, max_tries)
    while solid < target - 0.5 and tries < max_tries:
        n = min(n, max_tries - tries)
        recs = np.zeros(n, ELLIPSOID_DTYPE)                  # drawn on the host, outside the lock
        for i in range(n):
            centre, semi, R, xr, yr, kr = _draw_candidate(rng, H, ny, X0, T, z_hi)
            if yr[1] - yr[0] > ny:
                raise ValueError("a stone wider than the span: its cells would wrap onto themselves")
            recs[i] = (centre, semi, R.ravel(), xr[0], xr[1], yr[0], yr[1], kr[0], kr[1])
        with N.CAPTURE_LOCK, torch.cuda.stream(stream):
            cand = torch.from_numpy(recs.view(np.uint8).copy()).to(dev)
            N.check(N.lib().sw_pack_ellipsoids(_ptr(cand), n, X0, T, ny, z_hi, float(target), _ptr(bits),
                                               _ptr(state), ctypes.c_void_p(stream.cuda_stream)),
                    "sw_pack_ellipsoids")
            solid, used = (int(v) for v in state.cpu().tolist())
        tries += used
        n = batch
    with N.CAPTURE_LOCK, torch.cuda.stream(stream):
        words = bits.cpu().numpy().view(np.uint32)
    flat = np.unpackbits(words.view(np.uint8), bitorder="little")[:T * ny * (z_hi - 1)].astype(bool)
    m[X0:X0 + T, :, 1:z_hi] = flat.reshape(T, ny, z_hi - 1)
    return tries
