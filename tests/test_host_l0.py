"""The host side of the bit-packed Level-0 phase store without a GPU:
engine.l0_pack / l0_unpack (used to load a saved Level 0 and to read it back)
follow the layout include/gomelt.h states for the device kernels -- node
(x, y, z) is bit x % 32 of word (z * ny + y) * ceil(nx / 32) + x / 32 -- and
the word count agrees with the library's gm_l0_words."""

import ctypes as C

import numpy as np
import pytest
import torch

SIZES = [(1, 1, 1), (31, 2, 3), (32, 3, 2), (33, 4, 5), (64, 1, 1), (97, 5, 3), (161, 7, 4)]


def _reference_words(s1, nodes):
    """Pack by the stated layout, one node at a time."""
    nx, ny, nz = nodes
    wpr = (nx + 31) // 32
    w = np.zeros(wpr * ny * nz, dtype=np.uint32)
    v = np.asarray(s1).reshape(nz, ny, nx)
    for z in range(nz):
        for y in range(ny):
            for x in range(nx):
                if v[z, y, x] > 0.499:
                    w[(z * ny + y) * wpr + x // 32] |= np.uint32(1) << np.uint32(x % 32)
    return w.view(np.int32)


@pytest.mark.parametrize("nodes", SIZES)
def test_pack_layout_and_round_trip(nodes):
    import engine as E

    rng = np.random.default_rng(sum(nodes))
    n = nodes[0] * nodes[1] * nodes[2]
    # S1 as the reference stores it (floats); the store keeps S1 > 0.499
    s1 = rng.choice([0.0, 0.2, 0.499, 0.4991, 0.5, 1.0], size=n)
    words = E.l0_pack(torch.as_tensor(s1), nodes)
    assert words.dtype == torch.int32 and words.numel() == E.l0_words(nodes)
    assert np.array_equal(words.numpy(), _reference_words(s1, nodes))
    back = E.l0_unpack(words, nodes)
    assert back.dtype == torch.uint8 and back.numel() == n
    assert np.array_equal(back.numpy(), (s1 > 0.499).astype(np.uint8))


def test_padding_bits_stay_clear():
    import engine as E

    nodes = (33, 2, 2)
    words = E.l0_pack(torch.ones(33 * 2 * 2, dtype=torch.float64), nodes).numpy().view(np.uint32)
    assert np.all(words[0::2] == 0xFFFFFFFF) and np.all(words[1::2] == 1)


@pytest.fixture(scope="module")
def lib():
    import build_lib

    build_lib.build()
    import _native

    return _native.lib()


@pytest.mark.parametrize("nodes", SIZES + [(1601, 1601, 201)])
def test_word_count_matches_library(lib, nodes):
    import engine as E

    assert lib.gm_l0_words(*(C.c_longlong(v) for v in nodes)) == E.l0_words(nodes)


def test_word_count_rejects_empty_grid(lib):
    assert lib.gm_l0_words(C.c_longlong(0), C.c_longlong(4), C.c_longlong(4)) == -1
