"""Stone-wall masks on the GPU (csrc/sw_geometry.cu) against the host generators, bit for bit.

course_wall with device="cuda" rasterises the stones on the GPU (geometry.py:68-84); it must give
the six masks of the reference's own generator (tests/golden/geometry.npz, made by the reference's
geometry.build_wall).  ellipsoid_wall with device="cuda" runs the packer's accept/reject loop on
the GPU over candidates drawn on the host; it must give the host packer's mask for the wall
heights, porosities and seeds of the measured workloads and the serving range (H 16..48).
"""
import time

import numpy as np
import pytest

from conftest import golden

pytestmark = pytest.mark.gpu


def test_course_wall_on_the_gpu_reproduces_the_reference_masks(cuda):
    from stonewall.geometry import course_wall
    g = golden("geometry")
    for k in range(int(g["n"])):
        por, H, seed, nx, ny, nz, X0, T, phi = g[f"spec{k}"]
        shape = (int(nx), int(ny), int(nz))
        want = np.unpackbits(g[f"mask{k}"])[:int(np.prod(shape))].reshape(shape).astype(bool)
        got, got_phi = course_wall(float(por), int(H), *shape, int(X0), int(T), seed=int(seed), device="cuda")
        np.testing.assert_array_equal(got, want, err_msg=f"mask {k}")
        assert got_phi == pytest.approx(phi, abs=1e-12), k


CASES = [(H, por, seed) for H in (16, 24, 32, 40, 48) for por, seed in ((0.1, 11), (0.3, 12), (0.5, 13))]
CASES += [(40, 0.2, 1), (40, 0.0, 0), (40, 0.4, 2), (64, 0.3, 0)]                 # the c2 walls and c3


@pytest.mark.parametrize("H,porosity,seed", CASES)
def test_ellipsoid_wall_on_the_gpu_equals_the_host_packer(H, porosity, seed, cuda):
    from stonewall.geometry import ellipsoid_wall
    from stonewall.params import baseline_params
    p = baseline_params(H, 1000)
    t0 = time.perf_counter()
    want, fw = ellipsoid_wall(porosity, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=seed)
    t1 = time.perf_counter()
    got, fg = ellipsoid_wall(porosity, p.H, p.nx, p.ny, p.nz, p.X0, p.T, seed=seed, device="cuda")
    t2 = time.perf_counter()
    print(f"H={H} porosity={porosity}: host {t1 - t0:.3f} s, device {t2 - t1:.3f} s")
    np.testing.assert_array_equal(got, want)
    assert fg == fw


def test_packer_rejects_oversize_boxes(native_lib):
    from stonewall import _native as N
    L = native_lib
    assert L.sw_pack_box_bytes(48, 256, 65) == (48 * 256 * 64 + 31) // 32 * 4
    assert L.sw_pack_box_bytes(0, 256, 65) == -1
    import ctypes
    buf = np.zeros(16, np.int64)
    p = ctypes.c_void_p(buf.ctypes.data)
    assert L.sw_pack_ellipsoids(p, 1, 0, 120, 480, 121, 1.0, p, p, None) == N.SW_ERR_TOO_LARGE  # H = 120
