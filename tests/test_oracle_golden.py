"""Pin the CPU oracle against the reference's own kernels (tests/golden, made by make_golden.py).

The fixtures come from lbm3d.py's k_init / k_step / k_macro / k_accum bodies
run in float32; the oracle evaluates the same expressions in the same order,
so every field must match bit for bit, the never-written solid cells of the
stale lattice included.
"""
import numpy as np
import pytest

from conftest import golden


@pytest.mark.parametrize("case", ["step_box", "step_rand", "step_edge"])
def test_oracle_matches_reference_kernels(case, oracle_mod):
    d = golden(case)
    flag, uin = d["flag"], d["uin"]
    nu0, cs, x_sponge, nu_sponge, noise, seed, n = d["params"]
    f0 = oracle_mod.init(flag, uin, noise=np.float32(noise), seed=int(seed))
    np.testing.assert_array_equal(f0, d["f_init"])
    fa, fb = f0.copy(), np.zeros_like(f0)              # f1 starts as zeros (lbm3d.py:294)
    for t in range(int(n)):
        row = np.zeros((flag.shape[2], 2))
        oracle_mod.step(fa, flag, uin, np.float32(nu0), np.float32(cs), int(x_sponge), np.float32(nu_sponge),
                        f_out=fb, force_row=row)
        fa, fb = fb, fa
        np.testing.assert_array_equal(fa, d[f"f_step{t + 1}"])
        np.testing.assert_array_equal(fb, d[f"f_other{t + 1}"])
        np.testing.assert_allclose(row, d["force"][t], rtol=1e-12, atol=1e-15)
    u = oracle_mod.macro(fa, flag)
    np.testing.assert_array_equal(u, d["macro"])
    acc = np.zeros(u.shape, np.float64)
    oracle_mod.accum(u, acc)
    oracle_mod.accum(u, acc)
    np.testing.assert_array_equal(acc.astype(np.float32), d["accum2"])


def test_oracle_tables_match_reference(oracle_mod):
    d = golden("tables")
    c, w, opp, mirz = oracle_mod.tables()
    np.testing.assert_array_equal(c, d["C"])
    np.testing.assert_array_equal(w, d["W"])
    np.testing.assert_array_equal(opp, d["OPP"])
    np.testing.assert_array_equal(mirz, d["MIRZ"])


def test_oracle_f64_close_to_f32(oracle_mod):
    """The float64 restatement follows the float32 one to float32 rounding."""
    d = golden("step_box")
    flag, uin = d["flag"], d["uin"]
    nu0, cs, x_sponge, nu_sponge, noise, seed, n = d["params"]
    f32, _ = oracle_mod.run(d["f_init"], flag, uin, np.float32(nu0), np.float32(cs), int(x_sponge), 3,
                            np.float32(nu_sponge))
    f64, _ = oracle_mod.run(d["f_init"].astype(np.float64), flag, uin, float(np.float32(nu0)),
                            float(np.float32(cs)), int(x_sponge), 3, float(np.float32(nu_sponge)))
    fluid = np.broadcast_to(flag == 0, f32.shape)
    np.testing.assert_allclose(f32[fluid], f64[fluid], rtol=2e-6)


def test_oracle_thread_count_invariance(oracle_mod):
    """Forces and fields do not depend on the number of OpenMP threads."""
    d = golden("step_rand")
    flag, uin = d["flag"], d["uin"]
    nu0, cs, x_sponge, nu_sponge, noise, seed, n = d["params"]
    outs = []
    nmax = oracle_mod.max_threads()
    for nt in (1, max(2, nmax)):
        oracle_mod.set_threads(nt)
        outs.append(oracle_mod.run(d["f_init"], flag, uin, np.float32(nu0), np.float32(cs), int(x_sponge), 3,
                                   np.float32(nu_sponge)))
    oracle_mod.set_threads(nmax)
    np.testing.assert_array_equal(outs[0][0], outs[1][0])
    np.testing.assert_array_equal(outs[0][1], outs[1][1])


def test_oracle_qcoarse_equals_the_per_cell_loop():
    """The vectorised k_qcoarse restatement against a per-cell loop over q_at (lbm3d.py:203-238)."""
    from oracle import oracle as O
    rng = np.random.default_rng(5)
    nx, ny, nz = 12, 5, 7
    u = rng.normal(0, 0.05, (4, nx, ny, nz)).astype(np.float32)
    flag = (rng.random((nx, ny, nz)) < 0.1).astype(np.uint8)
    h = np.float32(0.5)

    def q_at(x, y, z):
        yp, ym = (y + 1) % ny, (y - 1 + ny) % ny
        if (flag[x, y, z] or flag[x + 1, y, z] or flag[x - 1, y, z] or flag[x, yp, z] or flag[x, ym, z]
                or flag[x, y, z + 1] or flag[x, y, z - 1]):
            return np.float32(0.0)
        g = [[h * (u[c, x + 1, y, z] - u[c, x - 1, y, z]), h * (u[c, x, yp, z] - u[c, x, ym, z]),
              h * (u[c, x, y, z + 1] - u[c, x, y, z - 1])] for c in (1, 2, 3)]
        return np.float32(-0.5) * (g[0][0] * g[0][0] + g[1][1] * g[1][1] + g[2][2] * g[2][2]
                                   + np.float32(2.0) * (g[0][1] * g[1][0] + g[0][2] * g[2][0] + g[1][2] * g[2][1]))

    for x0, ds in ((1, 1), (2, 2)):
        dims = ((nx - 1 - x0) // ds, ny // ds, (nz - 1) // ds)
        want = np.zeros(dims, np.float32)
        for i, j, k in np.ndindex(*dims):
            best = np.float32(0.0)
            for a, b, c in np.ndindex(ds, ds, ds):
                x, y, z = x0 + i * ds + a, j * ds + b, k * ds + c
                if 1 <= x < nx - 1 and 1 <= z < nz - 1:
                    best = max(best, q_at(x, y, z))
            want[i, j, k] = best
        np.testing.assert_array_equal(O.qcoarse(u, flag, x0, ds, dims), want)


def test_reference_checkpoint_continues_to_the_reference_result():
    """The reference's step-5 checkpoint of the driver case, advanced 5 steps by the oracle from the
    reference's own mask and parameters, gives the reference run's Cd / Cm for steps 5-9."""
    import json
    from oracle import oracle as O
    from stonewall.driver import derive, parse
    from stonewall.geometry import course_wall
    from stonewall.metrics import coefficients
    from stonewall.params import flags_from_wall
    d, c = golden("driver_small"), golden("driver_small_ckpt")
    p = derive(parse(json.loads(str(d["argv"]))))
    wall, _ = course_wall(0.2, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=7)
    flag = flags_from_wall(wall, p.nx, p.ny, p.nz)
    t0 = json.loads(str(c["state"]))["t"]
    f, force = O.run(c["f"], flag, p.uin, np.float32(p.nu0), np.float32(0.16), p.x_sponge, p.n_total - t0,
                     np.float32(p.nu_sponge))
    full = np.concatenate([c["force"][:t0].astype(np.float64), force])
    co = coefficients(full, p.UH, p.H, p.ny, p.zeta)
    for k in ("Cd", "Cm"):
        np.testing.assert_allclose(co[k], d[k], rtol=1e-5, atol=1e-6 * np.abs(d[k]).max(), err_msg=k)


def test_course_wall_reproduces_the_reference_masks():
    """stonewall.geometry.course_wall restates geometry.build_wall (geometry.py:135-161): the same
    seed gives the same mask and frontal porosity as the reference's own generator."""
    from stonewall.geometry import course_wall
    g = golden("geometry")
    for k in range(int(g["n"])):
        por, H, seed, nx, ny, nz, X0, T, phi = g[f"spec{k}"]
        shape = (int(nx), int(ny), int(nz))
        want = np.unpackbits(g[f"mask{k}"])[:int(np.prod(shape))].reshape(shape).astype(bool)
        got, got_phi = course_wall(float(por), int(H), *shape, int(X0), int(T), seed=int(seed))
        np.testing.assert_array_equal(got, want, err_msg=f"mask {k}")
        assert got_phi == pytest.approx(phi, abs=1e-12), k


def test_ellipsoid_wall_properties():
    """The BASELINE wall generator: seeded, confined to the wall box above the ground, and filled
    to the target solid fraction within half a stone."""
    from stonewall.geometry import ellipsoid_wall
    from stonewall.params import baseline_params
    for H, por, seed in ((16, 0.2, 0), (24, 0.45, 3), (16, 0.0, 1)):
        p = baseline_params(H, 1000)
        a, fa = ellipsoid_wall(por, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=seed)
        b, fb = ellipsoid_wall(por, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=seed)
        np.testing.assert_array_equal(a, b)
        assert fa == fb
        outside = a.copy()
        outside[p.X0:p.X0 + p.T, :, 1:1 + H] = False
        assert not outside.any()                                   # stones only in the wall box
        assert abs(fa - (1 - por)) < 0.02


def test_statistics_and_reverse_flow_area_match_the_reference():
    """stonewall.metrics against the reference's own postprocess.py statistics (on the driver
    case's Cd / Cm / Cl series) and export3d.py reverse-flow area (on a seeded mean field)."""
    import json
    from stonewall.metrics import recirculation_area, stats
    g, d = golden("postprocess"), golden("driver_small")
    want = json.loads(str(g["stats"]))
    got = stats(d["Cd"], d["Cm"], d["Cl"], int(g["n_spin"]))
    for k, v in want.items():
        assert got[k] == pytest.approx(v, rel=1e-6, abs=1e-6), k       # the reference sums in float32
    H, X0, nx, ny, nz, UH = g["params"]
    area = recirculation_area(g["ux_ds2"][0], g["wall_ds2"], int(H), int(X0), float(UH), int(ny))
    assert area > 0 and area == float(g["area"])
