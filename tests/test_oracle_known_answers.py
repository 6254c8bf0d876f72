"""Pin the oracle to the reference's own known-answer unit tests.

tst/unit/test_logical_location.cpp:123-189 (Morton numbers built by hand),
:196-294 (ownership arrays determined by drawing the tree) and :296-423 (index-range
masks per topological element).
"""
import numpy as np

import oracle_lib as O

# TopologicalElement values (src/basic_types.hpp:156-165)
CC, F1, F2, F3, E1, E2, E3, NN = 0, 3, 4, 5, 6, 7, 8, 9


def _leaves():
    """RefineLocation sequence of test_logical_location.cpp:125-131."""
    leaves = {(0, 0, 0, 0)}

    def refine(loc):
        if loc in leaves:
            leaves.remove(loc)
            lev, a, b, c = loc
            for i in (0, 1):
                for j in (0, 1):
                    for k in (0, 1):
                        leaves.add((lev + 1, 2 * a + i, 2 * b + j, 2 * c + k))

    refine((0, 0, 0, 0))
    refine((1, 0, 0, 0))
    refine((1, 1, 1, 1))
    refine((2, 3, 3, 3))
    return sorted(leaves)


def _hand_morton(level, l1, l2, l3):
    bits = 0
    for i in range(level):
        place = 1 << (level - 1 - i)
        if l3 // place == 1:
            bits |= 1 << (62 - (3 * i + 0))
        l3 %= place
        if l2 // place == 1:
            bits |= 1 << (62 - (3 * i + 1))
        l2 %= place
        if l1 // place == 1:
            bits |= 1 << (62 - (3 * i + 2))
        l1 %= place
    return bits


def test_morton_by_hand():
    last = 0
    ordered = sorted(_leaves(), key=lambda l: (int(O.morton(*l)[0]), int(O.morton(*l)[1]), l[0]))
    for leaf in ordered:
        m = O.morton(*leaf)
        assert int(m[0]) == _hand_morton(*leaf)
        assert int(m[1]) == 0 and int(m[2]) == 0
        assert int(m[0]) > last or int(m[0]) == 0
        last = int(m[0])


def _own(main):
    return O.ownership(main, _leaves())


def _bits(pred):
    out = 0
    for a in (-1, 0, 1):
        for b in (-1, 0, 1):
            for c in (-1, 0, 1):
                if pred(a, b, c):
                    out |= O.bit(a, b, c)
    return out


def test_ownership_block_2_2_3_3():
    assert _own((2, 2, 3, 3)) == _bits(lambda a, b, c: a != 1)


def test_ownership_block_2_1_1_1():
    assert _own((2, 1, 1, 1)) == _bits(lambda a, b, c: (a, b, c) != (1, 1, 1))


def test_ownership_block_2_0_0_0_uniform_pattern():
    assert _own((2, 0, 0, 0)) == _bits(lambda a, b, c: a <= 0 and b <= 0 and c <= 0)


def test_ownership_finest_corner_owns_everything():
    assert _own((3, 7, 7, 7)) == _bits(lambda a, b, c: True)


def _active(mask, N=3):
    """SpatiallyMaskedIndexer::IsActive over the index cube [0, N]^3."""
    out = np.zeros((N + 1, N + 1, N + 1), bool)
    for k in range(N + 1):
        for j in range(N + 1):
            for i in range(N + 1):
                ii = (i == N) - (i == 0)
                jj = (j == N) - (j == 0)
                kk = (k == N) - (k == 0)
                out[k, j, i] = bool(mask & O.bit(ii, jj, kk))
    return out


HAND = _bits(lambda a, b, c: (a <= 0 and b <= 0 and c <= 0) or (a, b, c) == (-1, 1, 1))
K, J, I = np.meshgrid(np.arange(4), np.arange(4), np.arange(4), indexing="ij")
N = 3


def test_mask_f1_all_active():
    assert _active(O.range_mask(F1, HAND, -1, 0, 0)).all()


def test_mask_f2_excludes_upper_j():
    a = _active(O.range_mask(F2, HAND, -1, 0, 0))
    assert np.array_equal(a, J != N)


def test_mask_f3_excludes_upper_k():
    a = _active(O.range_mask(F3, HAND, -1, 0, 0))
    assert np.array_equal(a, K != N)


def test_mask_e3_excludes_upper_j():
    a = _active(O.range_mask(E3, HAND, -1, 0, 0))
    assert np.array_equal(a, J != N)


def test_mask_e2_excludes_upper_k():
    a = _active(O.range_mask(E2, HAND, -1, 0, 0))
    assert np.array_equal(a, K != N)


def test_mask_e1_excludes_upper_j_or_k():
    a = _active(O.range_mask(E1, HAND, -1, 0, 0))
    assert np.array_equal(a, (K != N) & (J != N))


def test_mask_nn():
    a = _active(O.range_mask(NN, HAND, -1, 0, 0))
    expect = ((K != N) & (J != N)) | ((I == 0) & (J == N) & (K == N))
    assert np.array_equal(a, expect)
