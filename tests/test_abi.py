"""The C ABI library builds, loads and exports every function include/stonewall.h declares.

CPU only: no call here launches device work.
"""
import ctypes
import os
import re

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "stonewall.h")


def declared_functions():
    text = open(HEADER).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(sw_[a-z0-9_]+)\s*\(", text)))


def test_header_declares_the_kernel_entry_points():
    names = declared_functions()
    for must in ("sw_init", "sw_step", "sw_macro", "sw_accum", "sw_macro_accum", "sw_pack_f", "sw_unpack_f",
                 "sw_build_tiles", "sw_geom_make"):
        assert must in names


def test_library_exports_every_declared_symbol(native_lib):
    missing = [n for n in declared_functions() if not hasattr(native_lib, n)]
    assert not missing, missing


def test_host_only_entry_points(native_lib):
    from stonewall import _native as N
    assert b"sm_103a" in native_lib.sw_version()
    g = N.geom(45, 7, 10)
    assert (g.nx, g.ny, g.nz, g.pitch) == (45, 7, 10, 64)
    assert native_lib.sw_cells_padded(ctypes.byref(g)) == 10 * 7 * 64
    assert native_lib.sw_lattice_elems(ctypes.byref(g)) == 19 * 10 * 7 * 64
    assert native_lib.sw_tile_count(ctypes.byref(g)) == 10 * 7 * 2
    assert [native_lib.sw_dtype_size(d) for d in range(5)] == [4, 8, 2, 2, 0]
    bad = N.SwGeom()
    assert native_lib.sw_geom_make(0, 4, 4, ctypes.byref(bad)) == N.SW_ERR_BAD_ARG
    assert native_lib.sw_geom_make(1 << 16, 1 << 16, 1 << 10, ctypes.byref(bad)) == N.SW_ERR_BAD_ARG
    for s in range(7):
        assert native_lib.sw_status_string(s)


def test_entry_points_reject_bad_arguments_before_launching(native_lib):
    """Argument checks run on the host: null pointers, bad dtype, aliasing, misalignment."""
    from stonewall import _native as N
    g = N.geom(32, 4, 4)
    gp = ctypes.byref(g)
    buf = np.zeros(64, np.uint8)
    p = ctypes.c_void_p(buf.ctypes.data)
    L = native_lib
    assert L.sw_step(gp, 0, None, p, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None) == N.SW_ERR_BAD_ARG
    assert L.sw_step(gp, 9, p, ctypes.c_void_p(buf.ctypes.data + 32), p, p, p, 0.0, 0.0, 0, 0.0, None, 0,
                     None) == N.SW_ERR_BAD_ARG
    assert L.sw_step(gp, 0, p, p, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None) == N.SW_ERR_BAD_ARG  # in place
    assert L.sw_step(gp, 0, p, ctypes.c_void_p(buf.ctypes.data + 4), p, p, p, 0.0, 0.0, 0, 0.0, None, 0,
                     None) == N.SW_ERR_BAD_ARG                                                    # misaligned
    assert L.sw_init(gp, 0, p, p, p, 0.02, 1, 7, None) == N.SW_ERR_BAD_ARG                       # noise kind
    assert L.sw_pack_f(gp, 0, 2, p, p, None) == N.SW_ERR_BAD_ARG                                  # ref dtype
    assert L.sw_force_to_f64(None, None, -1, None) == N.SW_ERR_BAD_ARG
    q = ctypes.c_void_p(buf.ctypes.data + 32)
    assert L.sw_step_checked(gp, 0, p, q, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None, -2, None,
                             None) == N.SW_ERR_BAD_ARG                                           # cfg < -1
    assert L.sw_step_checked(gp, 0, p, q, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None, 8, None,
                             None) == N.SW_ERR_UNSUPPORTED                                       # TMA: 16-bit only
    assert L.sw_step_checked(gp, 0, p, q, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None, -1,
                             ctypes.c_void_p(buf.ctypes.data + 2), None) == N.SW_ERR_BAD_ARG     # status misaligned
    assert L.sw_step_cfg(gp, 0, p, q, p, p, p, 0.0, 0.0, 0, 0.0, None, 0, None, -1, None) == N.SW_ERR_BAD_ARG
    assert L.sw_coefficients(p, 4, 0, 0.05, 40.0, 160, p, None) == N.SW_ERR_BAD_ARG               # nz
    assert L.sw_coefficients(p, 4, 8, 0.0, 40.0, 160, p, None) == N.SW_ERR_BAD_ARG                # U_H
    assert L.sw_coefficients(ctypes.c_void_p(buf.ctypes.data + 8), 4, 8, 0.05, 40.0, 160, p,
                             None) == N.SW_ERR_BAD_ARG                                             # misaligned rows
    assert L.sw_coef_stats(p, 4, -1, p, None) == N.SW_ERR_BAD_ARG
    assert L.sw_coef_stats(p, 4, 0, None, None) == N.SW_ERR_BAD_ARG
    # recirculation box on 32x4x4, H = 2, X0 = 4: i in [2, 12), j < 2, k < 2 -> two float buffers
    assert L.sw_recirc_scratch_bytes(gp, 2, 4) == 2 * 10 * 2 * 2 * 4
    assert L.sw_recirc_scratch_bytes(gp, 1, 4) == N.SW_ERR_BAD_ARG                              # one level
    assert L.sw_recirc_scratch_bytes(gp, 2, 40) == N.SW_ERR_BAD_ARG                             # past the outlet
    assert L.sw_recirc_scratch_bytes(gp, 0, 4) == N.SW_ERR_BAD_ARG
    p8 = ctypes.c_void_p(buf.ctypes.data + 8)
    assert L.sw_recirc_count(gp, p, 1, p, 2, 4, 0.05, p, 100, p8, None) == N.SW_ERR_BAD_ARG      # scratch small
    assert L.sw_recirc_count(gp, p, 1, p, 2, 4, 0.0, p, 320, p8, None) == N.SW_ERR_BAD_ARG       # U_H
    assert L.sw_recirc_count(gp, p, -1, p, 2, 4, 0.05, p, 320, p8, None) == N.SW_ERR_BAD_ARG     # n_acc
    assert L.sw_recirc_count(gp, p, 1, p, 2, 4, 0.05, p, 320, ctypes.c_void_p(buf.ctypes.data + 4),
                             None) == N.SW_ERR_BAD_ARG                                           # count misaligned
    assert L.sw_recirc_count(gp, None, 1, p, 2, 4, 0.05, p, 320, p8, None) == N.SW_ERR_BAD_ARG


def test_status_words_map_to_errors(native_lib):
    """sw_status_error: the time-out bit wins (the timed-out cells were not written), then divergence."""
    from stonewall import _native as N
    L = native_lib
    assert L.sw_status_error(0) == N.SW_OK
    assert L.sw_status_error(N.SW_STATUS_NONFINITE) == N.SW_ERR_NONFINITE
    assert L.sw_status_error(N.SW_STATUS_TIMEOUT) == N.SW_ERR_TIMEOUT
    assert L.sw_status_error(N.SW_STATUS_TIMEOUT | N.SW_STATUS_NONFINITE) == N.SW_ERR_TIMEOUT
    assert L.sw_status_error(0x80) == N.SW_OK                                # bits nobody sets
    from stonewall.solver import DeviceWaitTimeout, Diverged, status_exception
    assert status_exception(0, "x") is None
    assert isinstance(status_exception(1, "x"), Diverged)
    assert isinstance(status_exception(3, "x"), DeviceWaitTimeout)


def test_tma_poll_limit_hook_reads_and_restores(native_lib):
    L = native_lib
    old = L.sw_debug_tma_poll_limit(-1)                 # read only
    assert old == 1 << 14
    assert L.sw_debug_tma_poll_limit(0) == old
    assert L.sw_debug_tma_poll_limit(-1) == 0
    assert L.sw_debug_tma_poll_limit(old) == 0
    assert L.sw_debug_tma_poll_limit(-1) == old


def test_native_unavailable_is_loud(monkeypatch, tmp_path):
    """With the library missing the package raises; there is no CPU fallback."""
    from stonewall import _native as N
    monkeypatch.setattr(N, "_lib", None)
    monkeypatch.setattr(N, "LIB_PATH", str(tmp_path / "missing.so"))
    with pytest.raises(N.NativeUnavailable):
        N.lib()


def test_recirculation_box_matches_the_host_slices(native_lib):
    """sw_recirc_scratch_bytes sizes the box that recirculation_area (export3d.py:177-179) slices
    out of the every-2nd-cell field: i in [X0 // 2, min(ceil(nx / 2), (X0 + 10 H) // 2)), every j,
    k < min(ceil(nz / 2), 2 H // 2); empty or one-level boxes are refused."""
    from stonewall import _native as N
    rng = np.random.default_rng(11)
    for _ in range(300):
        nx, ny, nz = (int(v) for v in rng.integers(2, 400, 3))
        H, X0 = int(rng.integers(1, 60)), int(rng.integers(0, 500))
        g = N.geom(nx, ny, nz)
        shape = [len(range(n)[::2]) for n in (nx, ny, nz)]          # the every-2nd-cell field
        i0, i1 = X0 // 2, min(shape[0], (X0 + 10 * H) // 2)
        k1 = min(shape[2], int(2 * H) // 2)
        sub = (len(range(shape[0])[i0:i1]), shape[1], len(range(shape[2])[:k1]))   # ux[i0:i1, :, :k1]
        got = native_lib.sw_recirc_scratch_bytes(ctypes.byref(g), H, X0)
        if np.prod(sub) == 0 or sub[2] < 2:
            assert got == N.SW_ERR_BAD_ARG, (nx, ny, nz, H, X0)
        else:
            assert got == 2 * int(np.prod(sub)) * 4, (nx, ny, nz, H, X0)


def test_aa_tma_hook_reads_and_restores(native_lib):
    L = native_lib
    assert L.sw_debug_aa_tma(-1) == 1                   # read only: staged by default
    assert L.sw_debug_aa_tma(0) == 1
    assert L.sw_debug_aa_tma(-1) == 0
    assert L.sw_debug_aa_tma(5) == 0                    # any non-zero value switches it on
    assert L.sw_debug_aa_tma(-1) == 1
