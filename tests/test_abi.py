"""The C ABI library loads and exports every function include/realflare_gb300.h declares;
the Python layer refuses to run without a GPU instead of falling back."""
from __future__ import annotations

import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    names = []
    for f in os.listdir(os.path.join(ROOT, 'include')):
        if f.endswith('.h'):
            text = open(os.path.join(ROOT, 'include', f)).read()
            text = re.sub(r'/\*.*?\*/', '', text, flags=re.S)
            names += re.findall(r'^[A-Za-z_][\w \*]*?\b(rf_\w+)\s*\(', text, flags=re.M)
    return sorted(set(names))


def test_library_exports_every_declared_symbol():
    from realflare_gb300 import build

    if not os.path.exists(build.LIB):
        build.build()
    lib = ctypes.CDLL(build.LIB)
    names = declared_functions()
    assert len(names) >= 20
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    from realflare_gb300._abi import SIGNATURES

    assert set(SIGNATURES) <= set(names)
    lib.rf_version.restype = ctypes.c_char_p
    assert b'sm_103a' in lib.rf_version()


def test_no_cpu_fallback_without_gpu():
    torch = pytest.importorskip('torch')
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from realflare_gb300.data import RealflareError
    from realflare_gb300.tasks import RaytracingTask

    with pytest.raises(RealflareError):
        RaytracingTask()


def test_host_only_calls_without_a_gpu():
    """Calls that issue no CUDA work answer without a device: the texture cache reset reports
    the missing device instead of touching it."""
    torch = pytest.importorskip('torch')
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from realflare_gb300 import build
    from realflare_gb300._abi import RF_ERR_CUDA

    if not os.path.exists(build.LIB):
        build.build()
    lib = ctypes.CDLL(build.LIB)
    assert lib.rf_ghost_textures_forget() == RF_ERR_CUDA
