"""Brick orders of the host store (the converter's -bricklayout,
CmdLineConverter/main.cpp:175-178): scanline, Morton, Hilbert and seeded
random orders are permutations of any brick grid; the Morton order
interleaves x, y, z bits; the Hilbert curve of a 2^b cube starts at the
origin, visits every cell once and steps to a face neighbour each time."""
import ctypes as C

import numpy as np
import pytest

from imagevis3d_gb300 import _lib as L


def order(nb, kind, seed=7):
    n = nb[0] * nb[1] * nb[2]
    out = (C.c_int32 * n)()
    L.call("gbvr_brick_order", (C.c_int32 * 3)(*nb), kind, seed, out, n)
    return np.array(out[:], np.int64)


def coords(i, nb):
    return i % nb[0], (i // nb[0]) % nb[1], i // (nb[0] * nb[1])


@pytest.mark.parametrize("nb", [(1, 1, 1), (2, 2, 2), (3, 5, 2), (9, 9, 9), (17, 17, 9), (6, 1, 4)])
@pytest.mark.parametrize("kind", [0, 1, 2, 3])
def test_every_order_is_a_permutation(nb, kind):
    p = order(nb, kind)
    n = nb[0] * nb[1] * nb[2]
    assert sorted(p.tolist()) == list(range(n))
    if kind == 0:
        assert p.tolist() == list(range(n))


def test_morton_interleaves_the_bits():
    nb = (4, 4, 4)
    p = order(nb, 1)
    for k, i in enumerate(p):
        x, y, z = coords(int(i), nb)
        key = 0
        for b in range(2):
            key |= ((x >> b) & 1) << (3 * b) | ((y >> b) & 1) << (3 * b + 1) | ((z >> b) & 1) << (3 * b + 2)
        assert key == k


@pytest.mark.parametrize("bits", [1, 2, 3, 4])
def test_hilbert_curve_steps_to_face_neighbours(bits):
    lib = L.lib()
    side = 1 << bits
    pos = {}
    for z in range(side):
        for y in range(side):
            for x in range(side):
                pos[int(lib.gbvr_hilbert3(x, y, z, bits))] = (x, y, z)
    assert sorted(pos) == list(range(side ** 3))
    assert pos[0] == (0, 0, 0)
    for h in range(1, side ** 3):
        a, b = np.array(pos[h - 1]), np.array(pos[h])
        assert np.abs(a - b).sum() == 1, h


def test_hilbert_order_of_a_grid_follows_the_enclosing_cube():
    """A 5 x 3 x 6 grid in Hilbert order: the bricks sorted by their positions
    on the 8^3 cube's curve."""
    lib = L.lib()
    nb = (5, 3, 6)
    p = order(nb, 2)
    keys = [int(lib.gbvr_hilbert3(*coords(int(i), nb), 3)) for i in p]
    assert keys == sorted(keys)


def test_random_order_is_seeded():
    nb = (7, 5, 3)
    a, b, c = order(nb, 3, 1), order(nb, 3, 1), order(nb, 3, 2)
    assert np.array_equal(a, b) and not np.array_equal(a, c)


def test_unknown_order_is_rejected():
    with pytest.raises(Exception):
        order((2, 2, 2), 4)
