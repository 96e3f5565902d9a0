"""CPU checks of the C ABI: the sm_103a library builds, loads, exports every
symbol declared in include/*.h, and the ctypes structures match the C
layout.  No kernel is launched."""
import ctypes
import os
import re
import subprocess
import tempfile

import pytest

from taichi_elements_gb300 import _lib, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER_DIR = os.path.join(ROOT, "include")


def declared_symbols():
    syms = set()
    for fn in os.listdir(HEADER_DIR):
        if not fn.endswith(".h"):
            continue
        text = open(os.path.join(HEADER_DIR, fn)).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*int\s+(mpm_\w+)\s*\(", text, flags=re.M):
            syms.add(m.group(1))
    return syms


@pytest.fixture(scope="module")
def lib():
    path = build.build_library()
    return ctypes.CDLL(str(path))


def test_library_exports_every_declared_symbol(lib):
    syms = declared_symbols()
    assert len(syms) >= 10
    for s in sorted(syms):
        assert hasattr(lib, s), s
    # the Python binding types every declared entry point
    assert syms <= set(_lib.SIGNATURES)


def test_abi_version(lib):
    lib.mpm_abi_version.restype = ctypes.c_int
    assert lib.mpm_abi_version() == _lib.ABI_VERSION


def _c_layout():
    src = r"""
#include <stdio.h>
#include <stddef.h>
#include "mpm_gb300.h"
#define P(T, f) printf(#T "." #f " %zu\n", offsetof(T, f))
int main(void) {
  printf("MpmParams %zu\nMpmCollider %zu\nMpmViews %zu\n", sizeof(MpmParams), sizeof(MpmCollider), sizeof(MpmViews));
  P(MpmParams, win_lo); P(MpmParams, chunk); P(MpmParams, plasticity); P(MpmParams, dx); P(MpmParams, gravity); P(MpmParams, stress_k);
  P(MpmParams, sand_k); P(MpmParams, colliders); P(MpmCollider, normal); P(MpmCollider, friction);
  P(MpmViews, grid_vel);
  return 0;
}
"""
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "l.c")
        exe = os.path.join(d, "l")
        open(c, "w").write(src)
        subprocess.run(["gcc", "-I", HEADER_DIR, "-o", exe, c], check=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout
    return dict(line.rsplit(" ", 1) for line in out.strip().splitlines())


def test_ctypes_struct_layout_matches_c():
    lay = _c_layout()
    assert int(lay["MpmParams"]) == ctypes.sizeof(_lib.MpmParams)
    assert int(lay["MpmCollider"]) == ctypes.sizeof(_lib.MpmCollider)
    assert int(lay["MpmViews"]) == ctypes.sizeof(_lib.MpmViews)
    for key, (cls, field) in {
            "MpmParams.win_lo": (_lib.MpmParams, "win_lo"), "MpmParams.chunk": (_lib.MpmParams, "chunk"),
            "MpmParams.plasticity": (_lib.MpmParams, "plasticity"),
            "MpmParams.dx": (_lib.MpmParams, "dx"), "MpmParams.gravity": (_lib.MpmParams, "gravity"),
            "MpmParams.stress_k": (_lib.MpmParams, "stress_k"), "MpmParams.sand_k": (_lib.MpmParams, "sand_k"),
            "MpmParams.colliders": (_lib.MpmParams, "colliders"),
            "MpmCollider.normal": (_lib.MpmCollider, "normal"),
            "MpmCollider.friction": (_lib.MpmCollider, "friction"),
            "MpmViews.grid_vel": (_lib.MpmViews, "grid_vel")}.items():
        assert int(lay[key]) == getattr(cls, field).offset, key


def test_argument_validation_without_gpu(lib):
    """Entry points reject bad parameters before touching the device."""
    L = _lib.load(build_if_missing=False)
    p = _lib.MpmParams()
    size = ctypes.c_size_t(0)
    assert L.mpm_workspace_bytes(ctypes.byref(p), 1024, ctypes.byref(size)) == -1  # version 0
    p.version = _lib.ABI_VERSION
    p.win_nb[0] = p.win_nb[1] = p.win_nb[2] = 8
    p.chunk = 512
    assert L.mpm_workspace_bytes(ctypes.byref(p), 1024, ctypes.byref(size)) == 0
    assert size.value > 8 * 8 * 8 * 64 * 32
    p.chunk = 100  # not a multiple of 32
    assert L.mpm_workspace_bytes(ctypes.byref(p), 1024, ctypes.byref(size)) == -1
    p.chunk = 512
    p.win_lo[0] = 3  # window origin must be block aligned
    assert L.mpm_workspace_bytes(ctypes.byref(p), 1024, ctypes.byref(size)) == -1
    assert L.mpm_gather_rows(None, 10, 5, 0, 3, None, None) == -1
    assert L.mpm_constitutive_eval(ctypes.byref(p), 4, None, None, None, None, None, 1e-4, None) == -1
    assert L.mpm_constitutive_eval(ctypes.byref(p), -1, None, None, None, None, None, 1e-4, None) == -1


def test_solver_refuses_without_cuda():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a CUDA device is present")
    from taichi_elements_gb300.mpm_solver import MPMSolver
    with pytest.raises(RuntimeError):
        MPMSolver((16, 16, 16))


def test_unsupported_flags_raise():
    from taichi_elements_gb300.mpm_solver import MPMSolver
    with pytest.raises(NotImplementedError):
        MPMSolver((16, 16))

