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
    # two Level-3 steps a launch: the first step's arguments are checked as gm_level_step's, then
    # the second step's dt, the phase buffers and the ring arrays, before any launch
    b = N.gm_level2_args()
    assert lib.gm_level_step2(C.byref(b), C.byref(p), None) == N.GM_ERR_ARG  # null T
    b.level.T_in, b.level.T_out, b.level.dt = 16, 32, 8
    b.level.nx = b.level.ny = b.level.nz = 4
    b.level.ne_planes = 3
    assert lib.gm_level_step2(C.byref(b), C.byref(p), None) == N.GM_ERR_ARG  # no dt2, phases, ring
    assert lib.gm_level_step2(None, C.byref(p), None) == N.GM_ERR_ARG
    s2 = N.gm_level_shape(1, 30, 4, 2, 6)  # kernel 1 is the one-step kernel's shape
    assert lib.gm_level_step2_shape(C.byref(b), C.byref(p), C.byref(s2), None) == N.GM_ERR_ARG
    assert lib.gm_level_autotune2(C.byref(b), C.byref(p), 0, None, None) == N.GM_ERR_ARG


def test_launch_shape_and_batch_validation_without_gpu(lib):
    """Invalid launch shapes, batch sizes, coupling methods and source-table
    types are refused on the host before any launch (the fake device
    addresses below are never dereferenced)."""
    import _native as N

    a = N.gm_level_args()
    a.dtype = N.GM_F32
    a.T_in, a.T_out, a.dt = 16, 32, 8
    a.nx = a.ny = a.nz = 4
    a.ne_planes = 3
    p = N.gm_props()
    assert lib.gm_level_step_shape(C.byref(a), C.byref(p), None, None) == N.GM_ERR_ARG
    bad_shapes = [
        (2, 32, 1, 2, 4),   # no such kernel
        (0, 24, 1, 2, 4),   # element tiles are 32 x 8 or 16 x 16
        (1, 30, 2, 3, 4),   # separable: 1, 2 or 4 rows a thread
        (1, 30, 9, 2, 4),   # at most 8 warps a CTA
        (1, 30, 0, 2, 4),
        (1, 30, 2, 2, 33),  # at most 32 planes a chunk
        (1, 30, 2, 2, 0),
    ]
    for s in bad_shapes:
        shape = N.gm_level_shape(*s)
        assert lib.gm_level_step_shape(C.byref(a), C.byref(p), C.byref(shape), None) == N.GM_ERR_ARG, s
    out = N.gm_tune_result()
    assert lib.gm_level_autotune(C.byref(a), C.byref(p), 0, C.byref(out), None) == N.GM_ERR_ARG
    assert lib.gm_level_batched_desc_size(0, N.GM_F32) == -1
    info = N.gm_batch_info()
    assert lib.gm_level_batched_prepare(None, 1, C.byref(p), 64, 1 << 20, C.byref(info), None) == N.GM_ERR_ARG
    assert lib.gm_level_batched_prepare(C.byref(a), 0, C.byref(p), 64, 1 << 20, C.byref(info), None) == N.GM_ERR_ARG
    # source tables: no rows, unknown type
    nodes = (C.c_int * 3)(4, 4, 4)
    org = (C.c_double * 3)(0.0, 0.0, 0.0)
    h = (C.c_double * 3)(0.01, 0.01, 0.01)
    assert lib.gm_fine_source_tables(N.GM_F32, nodes, org, h, 64, 0, C.byref(p), 128, None) == N.GM_ERR_ARG
    assert lib.gm_fine_source_tables(7, nodes, org, h, 64, 1, C.byref(p), 128, None) == N.GM_ERR_ARG

    # coupling: a geometry of 2 coarse elements per axis with fake tables
    g = N.gm_couple_args()
    g.dtype = N.GM_F32
    fake = C.cast(256, C.POINTER(C.c_int))
    for d in range(3):
        ax = g.geom.ax[d]
        ax.nfe, ax.cw, ax.node0, ax.cb_lo, ax.ncb, ax.flo, ax.fhi, ax.rmax, ax.H = 8, 512, fake, 0, 2, fake, fake, 4, 0.02
        g.fine_nodes[d] = 9
        g.fine_h[d] = 0.005
        g.out_lo[d] = 0
        g.out_n[d] = 3
    g.T, g.Tp, g.out, g.partials, g.partials_cap = 1024, 2048, 4096, 8192, 1 << 20
    g.method = 3  # no such method
    assert lib.gm_couple(C.byref(g), C.byref(p), None) == N.GM_ERR_ARG
    g.method = 0
    g.base = g.out  # base onto the output it is read from
    assert lib.gm_couple(C.byref(g), C.byref(p), None) == N.GM_ERR_ARG
    g.base = None
    g.out_n[0] = 2  # output box smaller than the coupling box
    assert lib.gm_couple(C.byref(g), C.byref(p), None) == N.GM_ERR_ARG
    g.out_n[0] = 3
    g.method = 2  # the separable contraction needs constant k and rho*c
    p.k_bulk_a1 = 0.01
    assert lib.gm_couple(C.byref(g), C.byref(p), None) == N.GM_ERR_ARG
    g.dTa = 16384  # dTa without dTb
    p.k_bulk_a1 = 0.0
    assert lib.gm_couple(C.byref(g), C.byref(p), None) == N.GM_ERR_ARG
