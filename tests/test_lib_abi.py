"""The C-ABI library loads and exports every entry point include/cody_gpu.h declares (no GPU needed)."""
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _declared():
    src = open(os.path.join(ROOT, "include", "cody_gpu.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(cgpu_[a-z0-9_]+)\s*\(", src)))


@pytest.fixture(scope="module")
def lib():
    from codyfortran_gb300 import build, engine
    build.build()
    return engine.load_library()


def test_every_declared_symbol_is_exported(lib):
    names = _declared()
    assert len(names) >= 25
    for n in names:
        assert hasattr(lib, n), n


def test_python_binding_covers_header():
    from codyfortran_gb300 import engine
    assert set(_declared()) == set(engine.EXPORTED)


def test_create_without_gpu_fails_loudly(lib):
    """On a machine without a GPU the context refuses to start (no CPU fallback)."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    from codyfortran_gb300 import engine, spec as S
    with pytest.raises(engine.CodyError):
        engine.Engine(S.cfg_helium_small())


def test_null_context_is_an_argument_error(lib):
    import ctypes as C
    assert lib.cgpu_synchronize(None) == 1
    assert lib.cgpu_ctx_destroy(None) == 0
    sz = (C.c_int * 6)()
    assert lib.cgpu_sizes(None, sz) == 1
