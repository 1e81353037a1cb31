"""The C ABI used from plain C (tests/abi/hvp_from_c.c): no Python, no PyTorch in
the program.  On the CPU the program must compile against include/tatva_gb300.h and
link against libtatva_gb300.so; on a GPU it must run and pass its own checks (a
constant-strain field has zero interior rows of K v; FP32 agrees with FP64)."""

import os
import shutil
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")


def _build(tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    exe = str(tmp_path / "hvp_from_c")
    libdir = os.path.join(ROOT, "tatva_gb300")
    cmd = ["gcc", "-std=c11", "-O2", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
           "-I", os.path.join(CUDA, "include"), os.path.join(ROOT, "tests", "abi", "hvp_from_c.c"),
           "-o", exe, "-L", libdir, "-ltatva_gb300", "-L", os.path.join(CUDA, "lib64"),
           "-lcudart", "-lm", f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{os.path.join(CUDA, 'lib64')}"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_c_program_compiles_and_links(tmp_path):
    _build(tmp_path)


@pytest.mark.gpu
def test_c_program_runs_on_gpu(tmp_path, cuda):
    exe = _build(tmp_path)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
    assert r.stdout.strip().endswith("ok"), r.stdout
