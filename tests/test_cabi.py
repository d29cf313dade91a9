"""C ABI checks that need no GPU: the library builds/loads, exports every
function declared in include/gomelt.h, and rejects invalid arguments before
launching anything."""

import ctypes as C
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared():
    with open(os.path.join(ROOT, "include", "gomelt.h")) as f:
        text = f.read()
    return sorted(set(re.findall(r"^(?:int|long long|const char\*)\s+(gm_\w+)\(", text, flags=re.M)))


@pytest.fixture(scope="module")
def lib():
    import build_lib

    build_lib.build()
    import _native

    return _native.lib()


def test_all_declared_symbols_exported(lib):
    names = declared()
    assert len(names) >= 15
    for n in names:
        assert hasattr(lib, n), n


def test_version(lib):
    assert b"sm_103a" in lib.gm_version()


def test_argument_validation_without_gpu(lib):
    import _native as N

    a = N.gm_level_args()
    p = N.gm_props()
    assert lib.gm_level_step(C.byref(a), C.byref(p), None) == N.GM_ERR_ARG  # null T
    a.T_in = a.T_out = 16  # aliasing in/out
    a.dt = 8
    a.nx = a.ny = a.nz = 4
    assert lib.gm_level_step(C.byref(a), C.byref(p), None) == N.GM_ERR_ARG
    assert lib.gm_interp(None, None) == N.GM_ERR_ARG
    g = N.gm_interp_args()
    g.nterms = 4
    assert lib.gm_interp(C.byref(g), None) == N.GM_ERR_ARG
    assert lib.gm_couple_partials_size(None) == -1
    cg = N.gm_couple_args()
    assert lib.gm_couple(C.byref(cg), C.byref(p), None) == N.GM_ERR_ARG
    assert lib.gm_clamp_min(7, None, 0, 0.0, None) == N.GM_ERR_ARG
    assert lib.gm_clamp_min(N.GM_F32, 16, -1, 0.0, None) == N.GM_ERR_ARG
