"""CPU checks of the C ABI: the shared library builds, loads and exports every symbol
include/jues_gpu.h declares; no compute call is made without a GPU."""
import os
import re

import pytest

from conftest import ROOT


def declared_symbols():
    with open(os.path.join(ROOT, "include", "jues_gpu.h")) as f:
        src = f.read()
    return sorted(set(re.findall(r"JUES_API\s+[\w\s\*]+?\b(jues_\w+)\s*\(", src)))


def test_header_declares_the_reference_entry_points():
    syms = declared_symbols()
    for s in ("jues_tei_transform", "jues_get_eri", "jues_rmp2", "jues_rccd", "jues_rccsd",
              "jues_ctx_create", "jues_last_error"):
        assert s in syms


def test_library_exports_every_declared_symbol():
    from juesgpu import _lib
    lib = _lib.load()
    for s in declared_symbols():
        assert hasattr(lib, s), s
        assert s in _lib.SIGNATURES, f"{s} has no ctypes signature"


def test_context_without_gpu_fails_loudly():
    import juesgpu
    from juesgpu import _lib
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a GPU is present")
    except ImportError:
        pass
    with pytest.raises(juesgpu.JuESError) as ei:
        _lib.Context(0)
    assert ei.value.code == _lib.ENODEV


def test_missing_library_is_an_error(tmp_path):
    from juesgpu import _lib
    with pytest.raises(_lib.JuESError):
        _lib.load(str(tmp_path / "libjuesgpu.so"))


def test_block_shapes_follow_get_eri_conventions():
    from juesgpu.IntegralTransformation import block_shape
    from juesgpu.synthetic import make_system
    w = make_system(9, 3, 27).wfn()
    assert block_shape(w, "OOVV") == (3, 3, 6, 6)
    assert block_shape(w, "OVVO") == (3, 6, 6, 3)
    assert block_shape(w, "OOVV", "chem") == (3, 3, 6, 6)
    assert block_shape(w, "OVOV", "chem") == (3, 6, 3, 6)
    assert block_shape(w, "OOVV", fcn=1) == (2, 2, 6, 6)
    with pytest.raises(ValueError):
        block_shape(w, "OOVX")
