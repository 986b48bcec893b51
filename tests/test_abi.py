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
