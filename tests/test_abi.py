"""The C-ABI library: exports every symbol include/frehg_gb300.h declares, struct layouts agree
with the ctypes mirror, and the package fails loudly without its CUDA library (no CPU path)."""
import ctypes as C
import os
import re
import subprocess
import tempfile

import pytest

from frehg_gb300 import abi

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "frehg_gb300.h")


def declared_functions():
    txt = open(HEADER).read()
    return sorted(set(re.findall(r"^[a-z_ 0-9\*]*?\b(frehg_[a-z0-9_]+)\(", txt, re.M)))


def test_header_and_mirror_agree():
    assert set(declared_functions()) == set(abi.SIGNATURES)


def test_library_exports_every_symbol(gpu_lib):
    lib = C.CDLL(abi.LIB_PATH)
    missing = [f for f in declared_functions() if not hasattr(lib, f)]
    assert not missing, missing


def test_build_arch_is_sm103(gpu_lib):
    assert gpu_lib.frehg_build_arch() == 103


def test_struct_layout_matches_c():
    src = r'''
#include <stddef.h>
#include <stdio.h>
#include "frehg_gb300.h"
int main(void) {
  printf("%zu %zu %zu %zu %zu %zu %zu\n", sizeof(frehg_soil_params), sizeof(frehg_re_params),
         sizeof(frehg_solver_config), sizeof(frehg_re_counters),
         offsetof(frehg_re_params, bc_type), offsetof(frehg_re_params, scheme),
         offsetof(frehg_solver_config, rtol));
  return 0;
}
'''
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "p.c")
        exe = os.path.join(d, "p")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe], check=True)
        got = [int(v) for v in subprocess.run([exe], capture_output=True, text=True,
                                              check=True).stdout.split()]
    want = [C.sizeof(abi.SoilParams), C.sizeof(abi.ReParams), C.sizeof(abi.SolverConfig),
            C.sizeof(abi.ReCounters), abi.ReParams.bc_type.offset, abi.ReParams.scheme.offset,
            abi.SolverConfig.rtol.offset]
    assert got == want


def test_defaults_match_reference(gpu_lib):
    p = abi.ReParams()
    gpu_lib.frehg_re_params_default(C.byref(p))
    mine = abi.ReParams()
    for f, _ in abi.ReParams._fields_:
        if f in ("soil", "bc_type"):
            continue
        assert getattr(p, f) == getattr(mine, f), f
    assert list(p.bc_type) == [0, 0, 0, 0, 0, 1]


def test_missing_library_fails_loudly(tmp_path):
    with pytest.raises(RuntimeError):
        abi.load_library(str(tmp_path / "nope.so"))
