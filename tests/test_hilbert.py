"""The Hilbert processing order's index (Skilling's transpose form, the steps
of hilbert3 in computer_graphics_lab_00_gb300/csrc/sph_grid.cu), checked on
the CPU: on a 2^b cube it is a bijection onto 0 .. 8^b - 1, and cells with
consecutive indices share a face — the locality the order is for."""
from __future__ import annotations

import itertools

import pytest


def spread3(v: int) -> int:
    out = 0
    for bit in range(10):
        out |= ((v >> bit) & 1) << (3 * bit)
    return out


def hilbert3(x0: int, x1: int, x2: int, bits: int) -> int:
    x = [x0, x1, x2]
    top = 1 << (bits - 1)
    q = top
    while q > 1:
        low = q - 1
        for i in range(3):
            if x[i] & q:
                x[0] ^= low
            else:
                swap = (x[0] ^ x[i]) & low
                x[0] ^= swap
                x[i] ^= swap
        q >>= 1
    x[1] ^= x[0]
    x[2] ^= x[1]
    flip = 0
    q = top
    while q > 1:
        if x[2] & q:
            flip ^= q - 1
        q >>= 1
    return (spread3(x[0] ^ flip) << 2) | (spread3(x[1] ^ flip) << 1) | spread3(x[2] ^ flip)


@pytest.mark.parametrize("bits", [1, 2, 3, 4])
def test_hilbert_index_is_a_face_adjacent_bijection(bits):
    side = 1 << bits
    cell_of = {}
    for c in itertools.product(range(side), repeat=3):
        cell_of[hilbert3(*c, bits)] = c
    assert sorted(cell_of) == list(range(side ** 3))
    for k in range(side ** 3 - 1):
        a, b = cell_of[k], cell_of[k + 1]
        assert sum(abs(u - v) for u, v in zip(a, b)) == 1, (k, a, b)
