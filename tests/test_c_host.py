"""The drop-in boundary from C: tests/c/host_example.c (a host written like the
reference's harness) compiles against include/tay.h and links libtay_gb300.so; on a GPU
it runs one-group, two-group and batched states and checks what it reads back."""
import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "c", "host_example.c")
LIBDIR = os.path.join(ROOT, "tay_gb300")


def _compile(tmp_path):
    cc = shutil.which("gcc") or shutil.which("cc")
    if not cc:
        pytest.skip("no C compiler")
    exe = os.path.join(str(tmp_path), "host_example")
    subprocess.run([cc, "-std=gnu11", "-O1", "-Wall", "-Werror", "-Wno-unused-result", "-I", os.path.join(ROOT, "include"),
                    SRC, "-o", exe, "-L", LIBDIR, "-ltay_gb300", "-Wl,-rpath," + LIBDIR, "-lm"], check=True)
    return exe


def test_c_host_compiles_and_links(built, tmp_path):
    assert os.path.exists(_compile(tmp_path))


@pytest.mark.gpu
def test_c_host_runs(gpu, tmp_path):
    exe = _compile(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok")
