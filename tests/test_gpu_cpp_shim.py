"""The C++ drop-in header compiles against a reference-style caller and runs on the GPU."""
import os
import subprocess

import pytest

from conftest import PKG, ROOT


def test_shim_compiles_without_gpu(lvg, tmp_path):
    """Compile-only check of include/louvain_gb300.hxx (no GPU needed)."""
    exe = tmp_path / "shim_test.o"
    subprocess.run(["g++", "-std=c++17", "-O2", "-c", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_test.cpp"), "-o", str(exe)], check=True)


@pytest.mark.gpu
def test_shim_program_runs(cuda, tmp_path):
    exe = tmp_path / "shim_test"
    libdir = os.path.join(PKG, "lib")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "shim_test.cpp"), "-L", libdir, "-llouvain_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "bad 0" in r.stdout
