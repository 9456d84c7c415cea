"""The boundary is a C ABI: a plain C program, built with gcc against include/stonewall.h and
linked to libstonewall.so, calls the host-side entry points (CPU only, no device work)."""
import os
import shutil
import subprocess

import pytest

from conftest import ROOT


def test_plain_c_caller(native_lib, tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    libdir = os.path.join(ROOT, "jeju-stonewall-lbm_gb300", "stonewall")
    exe = str(tmp_path / "host_calls")
    src = os.path.join(ROOT, "tests", "c_abi", "host_calls.c")
    subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"), src, "-o", exe,
                    "-L", libdir, "-lstonewall", f"-Wl,-rpath,{libdir}"], check=True)
    r = subprocess.run([exe], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert "c abi ok" in r.stdout
