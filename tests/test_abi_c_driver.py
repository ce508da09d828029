"""The C ABI driven from a plain C11 program (tests/c_abi/abi_driver.c) that
includes only include/radiantium.h and links the library: the boundary a native
host binding uses, with no Python in between.  On CPU the program is compiled
with every warning as an error and runs the calls that need no device; on a GPU
it renders with the path integrator and the light tracer, traces rays, reads
the counters and checks the error paths."""
import os
import subprocess

import pytest

from radiantium_gb300 import native as N

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c_abi", "abi_driver.c")


def _compile(tmp_path):
    if not os.path.exists(N.LIB_PATH):
        from radiantium_gb300 import build
        build.build()
    lib_dir = os.path.dirname(N.LIB_PATH)
    exe = str(tmp_path / "abi_driver")
    cmd = ["gcc", "-std=c11", "-O1", "-Wall", "-Wextra", "-Werror", "-I", os.path.join(ROOT, "include"), SRC,
           "-o", exe, "-L", lib_dir, "-lradiantium_gb300", f"-Wl,-rpath,{lib_dir}", "-lm"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_driver_without_gpu(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe, "--no-gpu"], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi ok" in r.stdout


@pytest.mark.gpu
def test_c_driver_on_gpu(tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "abi ok" in r.stdout
