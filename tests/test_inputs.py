"""Seeded input generators (include/bale_inputs.h): determinism, ranges and
the structural invariants the kernels and the reference rely on."""
from __future__ import annotations

import numpy as np
import pytest


def test_splitmix64_reference_value(bale):
    # SplitMix64 started at 0: the first output is the published 0xE220A8397B1DCDAF.
    assert bale.splitmix64(0, 0) == 0xE220A8397B1DCDAF


def test_uniform_is_seeded_ranged_and_thread_independent(bale):
    a = bale.gen_uniform(100_003, 1_000_000, 1)
    b = bale.gen_uniform(100_003, 1_000_000, 1)
    np.testing.assert_array_equal(a, b)
    assert a.min() >= 0 and a.max() < 1_000_000
    assert not np.array_equal(a, bale.gen_uniform(100_003, 1_000_000, 2))
    bale.set_host_threads(1)
    try:
        c = bale.gen_uniform(100_003, 1_000_000, 1)
    finally:
        bale.set_host_threads(0)
    np.testing.assert_array_equal(a, c)
    p = bale.gen_uniform(1000, 77, 3, packed=True)
    np.testing.assert_array_equal(p >> 16, bale.gen_uniform(1000, 77, 3))
    assert not (p & 0xFFFF).any()


def test_uniform_rejects_bad_arguments(bale):
    with pytest.raises(bale.BaleError):
        bale.gen_uniform(10, 0, 1)


def test_keyed_perm_is_a_bijection(bale):
    for rng in (1, 2, 7, 1000, 4099):
        img = np.array([bale.keyed_perm(r, rng, 5) for r in range(rng)])
        assert sorted(img.tolist()) == list(range(rng))


def test_zipf_is_skewed_over_a_permutation(bale):
    rng = 1 << 20
    z = bale.gen_zipf(400_000, rng, 1.1, 4, 5)
    assert z.min() >= 0 and z.max() < rng
    vals, cnt = np.unique(z, return_counts=True)
    top = vals[np.argmax(cnt)]
    assert top == bale.keyed_perm(0, rng, 5)  # rank 0 is the most frequent
    # P(rank 0) for Zipf(1.1) over 2^20 ranks is about 1/zeta-ish ~ 0.09
    assert 0.05 < cnt.max() / z.size < 0.15
    np.testing.assert_array_equal(z, bale.gen_zipf(400_000, rng, 1.1, 4, 5))


def test_rmat_is_strict_lower_tidy_deduplicated_and_degree_ordered(bale, oracle):
    L = bale.gen_rmat(12, 16, 0.57, 0.19, 0.19, 6)
    assert L.numrows == 1 << 12
    assert oracle.is_strict_lower_tidy(L.offset, L.nonzero)
    deg = np.diff(L.offset)
    # symmetric degree = row length + column count
    sym = deg + np.bincount(L.nonzero, minlength=L.numrows)
    assert (np.diff(sym) <= 0).all(), "labels must be in descending degree order"
    assert L.nnz <= 16 << 12
    L2 = bale.gen_rmat(12, 16, 0.57, 0.19, 0.19, 6)
    np.testing.assert_array_equal(L.nonzero, L2.nonzero)


def test_erdos_renyi_density(bale, oracle):
    n = 1 << 14
    L = bale.gen_erdos_renyi(n, 32.0 / n, 7)
    assert oracle.is_strict_lower_tidy(L.offset, L.nonzero)
    avg = 2.0 * L.nnz / n
    assert 30.0 < avg < 34.0


def test_kronecker_shapes(bale):
    L = bale.gen_kronecker(1, [3, 4, 5, 9])
    assert L.numrows == 4 * 5 * 6 * 10
    assert bale.kronecker_triangles(1, [3, 4, 5, 9]) == 9107
    assert bale.kronecker_triangles(2, [3, 4, 5, 9, 2]) == 155
    assert bale.kronecker_triangles(0, [3, 4]) == 0
