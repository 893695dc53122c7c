"""A C89 VSIPL application (tests/c/vsip_app.c) built against the public
header and linked with the GPU library alone: it compiles and links on any
host; on a GPU it runs the fftm and single-FFT calls on user data and checks
them against direct DFTs."""
import os
import subprocess

import pytest

import jvsip_gb300 as J

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def build_app(tmp_path):
    J.lib()
    exe = tmp_path / "vsip_app"
    libdir = os.path.dirname(J.LIB_PATH)
    subprocess.check_call(["gcc", "-std=c89", "-pedantic", "-Wall", "-Werror", "-O1",
                           "-I", os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "c", "vsip_app.c"),
                           "-o", str(exe), "-L", libdir, "-Wl,-rpath," + libdir, "-ljvsip_fftm_gb300", "-lm"])
    return exe


def test_c_app_compiles_and_links(tmp_path):
    exe = build_app(tmp_path)
    assert exe.exists()


@pytest.mark.gpu
def test_c_app_runs_on_the_gpu(tmp_path):
    exe = build_app(tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("OK")
