"""The C-ABI library builds, loads and exports every symbol include/saigegpu.h declares (no GPU needed)."""
import ctypes
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def header_symbols():
    src = open(os.path.join(ROOT, "include", "saigegpu.h")).read()
    return sorted(set(re.findall(r"\b(sg_[A-Za-z0-9_]+)\s*\(", src)))


def test_library_exports_every_header_symbol():
    from saigegpu import build, _lib
    build.build_lib()
    lib = ctypes.CDLL(build.LIB)
    syms = header_symbols()
    assert len(syms) > 40
    missing = [s for s in syms if not hasattr(lib, s)]
    assert not missing, missing
    # the ctypes table covers the header too
    assert not [s for s in syms if s not in _lib.SIGNATURES], [s for s in syms if s not in _lib.SIGNATURES]


def test_context_without_gpu_fails_cleanly():
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from saigegpu import Context, SaigeGpuError
    with pytest.raises(SaigeGpuError):
        Context(0)


def test_null_context_calls_return_invalid():
    from saigegpu import load
    lib = load()
    assert lib.sg_engine_run(None, 1, None) == 1
    assert lib.sg_grm_build(None, 0) == 1
