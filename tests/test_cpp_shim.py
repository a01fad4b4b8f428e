"""The header-only C++ shim (include/tval3/tval3.hpp) compiles the way a
reference caller is written and links against the C-ABI library; on a GPU it
reconstructs and maps argument errors to tval3_gpu_exception."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "tests" / "cpp" / "shim_example.cpp"


SRC2D = ROOT / "tests" / "cpp" / "shim2d_example.cpp"


def _compile(lib, tmp_path, src=SRC):
    from tval3_gb300.capi import LIB_PATH
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    exe = tmp_path / src.stem
    cmd = [gxx, "-std=c++17", "-Wall", "-Wextra", "-Werror", f"-I{ROOT / 'include'}", str(src),
           f"-L{LIB_PATH.parent}", "-ltval3_gb300", f"-Wl,-rpath,{LIB_PATH.parent}", "-o", str(exe)]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    return exe


def test_shim_compiles_and_links(lib, tmp_path):
    assert _compile(lib, tmp_path).exists()


def test_shim_2d_compiles_and_links(lib, tmp_path):
    """A caller written against the 2D reference's untemplated containers
    (2d/container_host.h, 2d/tval3_gpu.h) compiles unchanged."""
    assert _compile(lib, tmp_path, SRC2D).exists()


def test_shim_c_header_is_plain_c(tmp_path):
    gcc = shutil.which("gcc")
    if not gcc:
        pytest.skip("gcc not available")
    src = tmp_path / "c_only.c"
    src.write_text('#include "tval3/tval3_c.h"\nint main(void) { tval3_options o; tval3_options_default(&o); '
                   'return o.maxit == 1025 ? 0 : 1; }\n')
    r = subprocess.run([gcc, "-std=c99", "-Wall", "-Werror", "-c", f"-I{ROOT / 'include'}", str(src), "-o",
                        str(tmp_path / "c_only.o")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr


@pytest.mark.gpu
def test_shim_runs_on_gpu(cuda, tmp_path):
    exe = _compile(None, tmp_path)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "iters 20" in r.stdout or "iters" in r.stdout
    assert "geometry f64 iters" in r.stdout
    assert "rejected: Argument error: b.len must be equal to A.dim_y!" in r.stdout


@pytest.mark.gpu
def test_shim_2d_runs_on_gpu(cuda, tmp_path):
    """The 2D caller reconstructs through the CSC, dense and CSR forms of the
    same matrix (CSC and CSR bit-identical), and gets the reference's
    exceptions for a bad assignment and a bad b."""
    exe = _compile(None, tmp_path, SRC2D)
    r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "sparse iters" in r.stdout and "dense iters" in r.stdout
    assert "csr iters" in r.stdout and "same 1" in r.stdout
    assert "assignment rejected" in r.stdout
    assert "rejected: Argument error:" in r.stdout
