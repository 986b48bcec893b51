"""The C-ABI library builds, loads and exports every symbol the header declares
(no CUDA calls: runs without a GPU)."""
import ctypes
import os
import re

from obvhs_gb300 import _native as N
from obvhs_gb300 import build as B

HEADER = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "include", "obvhs_gb300.h")


def declared():
    src = open(HEADER).read()
    return sorted(set(re.findall(r"^OBVHS_API [^(]*?\b(obvhs_\w+)\(", src, flags=re.M)))


def test_header_declares_the_binding():
    assert declared() == sorted(N.SIGNATURES)


def test_library_exports_every_symbol():
    lib = ctypes.CDLL(B.build())
    for name in declared():
        assert hasattr(lib, name), name


def test_library_targets_sm_103a_only():
    assert B.ARCH == ["-gencode", "arch=compute_103a,code=sm_103a"]


def _kernel_bodies(src):
    """(name, first statement) of every __global__ definition in `src`."""
    out = []
    for m in re.finditer(r"__global__", src):
        k, depth = m.end(), 0
        while True:
            ch = src[k]
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
            elif depth == 0 and ch in "{;":
                break
            k += 1
        if src[k] == "{":
            name = re.findall(r"(\w+)\s*\(", src[m.end():k])
            first = src[k + 1:].lstrip().split(";", 1)[0]
            out.append((name[-1] if name else "?", first))
    return out


def test_every_kernel_waits_for_its_predecessor_first():
    """Kernels go out as programmatic dependent launches: each must wait for
    the previous kernel before its first memory access, and all launches go
    through launch_k (no <<<>>>), so none bypasses that rule."""
    csrc = os.path.join(os.path.dirname(B.__file__), "csrc")
    n = 0
    for f in sorted(os.listdir(csrc)):
        if not f.endswith((".cu", ".cuh", ".h")):
            continue
        src = open(os.path.join(csrc, f)).read()
        assert not re.search(r"<<<[^;]*>>>\s*\(", src), f
        for name, first in _kernel_bodies(src):
            assert first == "grid_dep_wait()", (f, name, first)
            n += 1
    assert n >= 70
