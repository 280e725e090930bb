"""The C++ host interface (include/frehg_gb300.hpp) compiled with g++: a syntax check here, and on
the GPU the test program tests/cpp/test_cpp_api.cpp linked against the library and run (the
linear-solver seam on a manufactured Laplacian in FP64 and mixed precision, the seam's error
behaviour, the ReSolver interface on the closed box)."""
import os
import subprocess

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
SRC = os.path.join(ROOT, "tests", "cpp", "test_cpp_api.cpp")
INC = os.path.join(ROOT, "include")


def test_cpp_header_compiles():
    subprocess.run(["g++", "-std=c++17", "-Wall", "-Wextra", "-Werror", "-fsyntax-only",
                    "-I", INC, SRC], check=True)


@pytest.mark.gpu
def test_cpp_program_runs(gpu_lib):
    libdir = os.path.dirname(gpu_lib._name)
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_cpp_api")
    subprocess.run(["g++", "-std=c++17", "-O2", "-I", INC, SRC, "-L", libdir, "-lfrehg_gb300",
                    f"-Wl,-rpath,{libdir}", "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=300)
    print(r.stdout)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout


def test_decomp3d_on_the_cpu():
    """the Decomp3D of the C++ mirror (header only): numbering, STAR stencil, pack / unpack"""
    src = os.path.join(ROOT, "tests", "cpp", "test_decomp3d.cpp")
    out_dir = os.path.join(ROOT, "tests", "cpp", "_build")
    os.makedirs(out_dir, exist_ok=True)
    exe = os.path.join(out_dir, "test_decomp3d")
    subprocess.run(["g++", "-std=c++17", "-O1", "-Wall", "-Wextra", "-Werror", "-I", INC, src,
                    "-o", exe], check=True)
    r = subprocess.run([exe], capture_output=True, text=True, timeout=60)
    assert r.returncode == 0, r.stdout + r.stderr
    assert "ALL OK" in r.stdout
