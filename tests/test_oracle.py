"""The CPU oracle (oracle/bale_oracle.c) pinned against the reference.

* against the golden vectors recorded from the reference's own compiled
  sources (tests/golden/make_golden.py);
* against the reference's built-in self-checks (known answers);
* directly against oracle/_ref on fresh seeded inputs when that library is
  present (it is only built where the reference tree exists).
"""
from __future__ import annotations

import numpy as np
import pytest

from oracle.pyoracle import REF_LIB, Reference


def _cases(d, suffix):
    return sorted({k.split("/")[0] for k in d.files if k.endswith(suffix)})


def test_histo_matches_reference_golden(oracle, golden):
    d = golden("histo")
    for name in _cases(d, "/index"):
        index = d[f"{name}/index"]
        pck = (index << 16).astype(np.int64)
        c = d[f"{name}/counts0"].copy()
        oracle.histo_agi(index, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_agi"], err_msg=name)
        oracle.histo_exstack(pck, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_exstack"], err_msg=name)
        oracle.histo_exstack(pck, c)
        np.testing.assert_array_equal(c, d[f"{name}/after_exstack2"], err_msg=name)


def test_ig_matches_reference_golden(oracle, golden):
    d = golden("ig")
    for name in _cases(d, "/index"):
        index, table = d[f"{name}/index"], d[f"{name}/table"]
        np.testing.assert_array_equal(oracle.ig_agi(index, table), d[f"{name}/tgt"], err_msg=name)
        pck = (index << 16).astype(np.int64)
        np.testing.assert_array_equal(oracle.ig_exstack(pck, table), d[f"{name}/tgt"], err_msg=name)
        assert d[f"{name}/exstack_variants_agree"].all()


def test_triangles_match_reference_golden(oracle, golden):
    d = golden("triangles")
    for g in d["graphs"]:
        off, col = d[f"{g}/offset"], d[f"{g}/nonzero"]
        assert oracle.is_strict_lower_tidy(off, col), g
        cnt, pulled = oracle.triangle_agi(off, col)
        ref_cnt, ref_sr = d[f"{g}/triangle_agi"]
        assert cnt == ref_cnt, g
        assert pulled == ref_sr, g  # the AGI "shared refs" tally is pinned too
        pc, pushed = oracle.triangle_exstack_push(off, col)
        assert pc == d[f"{g}/triangle_exstack_push"][0], g
        assert pushed == d[f"{g}/triangle_exstack_push"][1], g
        for k in ("triangle_exstack2_push", "triangle_agi_iter"):
            assert d[f"{g}/{k}"][0] == cnt, (g, k)
        closed = int(d[f"{g}/closed_form"][0])
        if closed >= 0:
            assert cnt == closed, g


def test_histo_self_check_known_answer(oracle, bale):
    """apps/histo_src/histo.upc:208-227: after every model has added each
    update once, subtracting num_models per update leaves all counters 0."""
    index = bale.gen_uniform(50_000, 3_000, 99)
    counts = np.zeros(3_000, np.int64)
    num_models = 3
    for _ in range(num_models):
        oracle.histo_agi(index, counts)
    np.subtract.at(counts, index, num_models)
    assert not counts.any()


def test_ig_self_check_known_answer(oracle, bale):
    """apps/ig_src/ig.upc:96-114, :158-161: table[i] = -(i+1) makes every
    gathered value -(index+1)."""
    index = bale.gen_uniform(40_000, 5_000, 98)
    tgt = oracle.ig_agi(index, bale.gen_negative_table(5_000))
    np.testing.assert_array_equal(tgt, -(index + 1))


@pytest.mark.parametrize("mode,specs", [(0, [3, 4, 5, 9]), (1, [3, 4, 5, 9]), (2, [3, 4, 5, 9, 2]),
                                        (1, [1, 4, 9, 16]), (2, [2, 3, 4, 5])])
def test_kronecker_closed_forms(oracle, bale, mode, specs):
    """apps/triangle_src/triangle.upc:278-295 closed forms."""
    L = bale.gen_kronecker(mode, specs)
    cnt, _ = oracle.triangle_agi(L.offset, L.nonzero)
    assert cnt == bale.kronecker_triangles(mode, specs)
    assert oracle.triangle_exstack_push(L.offset, L.nonzero)[0] == cnt


def test_work_model_matches_pulls(oracle, golden):
    """triangle.upc:325-361: pulls = sum deg*colcount; the AGI tally adds two
    offset reads per (i,j) after the first of each row."""
    d = golden("triangles")
    for g in d["graphs"]:
        off, col = d[f"{g}/offset"], d[f"{g}/nonzero"]
        pulls, pushes = oracle.triangle_work(off, col)
        deg = np.diff(off)
        assert pushes == int((deg * (deg - 1) // 2).sum())
        _, pulled = oracle.triangle_agi(off, col)
        first_skipped = int((deg > 0).sum())
        # pulled = sum over (i,j) not first of (2 + deg(j))
        rowid = np.repeat(np.arange(deg.size), deg)
        not_first = np.ones(col.size, bool)
        not_first[off[:-1][deg > 0]] = False
        assert pulled == int((2 + deg[col[not_first]]).sum())
        assert pulls == int(deg[col].sum())
        assert first_skipped == int((deg > 0).sum()) and rowid.size == col.size


def test_multithreaded_oracle_equals_serial(oracle, bale):
    index = bale.gen_uniform(200_000, 10_000, 5)
    a, b = np.zeros(10_000, np.int64), np.zeros(10_000, np.int64)
    oracle.histo_agi(index, a)
    oracle.histo_agi_mt(index, b, 4)
    np.testing.assert_array_equal(a, b)
    table = bale.gen_values(10_000, 6)
    t = np.empty(index.size, np.int64)
    oracle.ig_agi_mt(t, index, table, 4)
    np.testing.assert_array_equal(t, oracle.ig_agi(index, table))
    L = bale.gen_rmat(11, 16, 0.57, 0.19, 0.19, 7)
    assert oracle.triangle_agi_mt(L.offset, L.nonzero, 4) == oracle.triangle_agi(L.offset, L.nonzero)[0]


@pytest.mark.skipif(not REF_LIB.exists(), reason="reference library not built here")
def test_oracle_equals_reference_on_fresh_inputs(oracle, bale):
    ref = Reference()
    import ctypes as C

    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))  # noqa: E731
    for seed in (101, 202):
        index = bale.gen_uniform(30_000, 7_777, seed)
        c1, c2 = np.zeros(7_777, np.int64), np.zeros(7_777, np.int64)
        ref.lib.histo_agi(P(index), index.size, P(c1))
        oracle.histo_agi(index, c2)
        np.testing.assert_array_equal(c1, c2)
        table = bale.gen_values(7_777, seed + 1)
        t1 = np.zeros(index.size, np.int64)
        ref.lib.ig_agi(P(t1), P(index), index.size, P(table))
        np.testing.assert_array_equal(t1, oracle.ig_agi(index, table))
    for scale, seed in ((11, 3), (12, 4)):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed)
        r = ref.triangles(L.offset, L.nonzero)
        assert oracle.triangle_agi(L.offset, L.nonzero) == r["triangle_agi"]
        assert oracle.triangle_exstack_push(L.offset, L.nonzero) == r["triangle_exstack_push"]
    off, col = ref.erdos_renyi_lower(5000, 20.0 / 5000, 777)
    assert oracle.triangle_agi(off, col) == ref.triangles(off, col)["triangle_agi"]


def test_spmat_transpose_and_permute_match_reference_golden(oracle, golden):
    d = golden("spmat")
    for t in d["mats"]:
        off, col, nc = d[f"{t}/offset"], d[f"{t}/nonzero"], int(d[f"{t}/numcols"][0])
        to, tc = oracle.transpose(off, col, nc)
        np.testing.assert_array_equal(to, d[f"{t}/t_offset"], err_msg=str(t))
        np.testing.assert_array_equal(tc, d[f"{t}/t_nonzero"], err_msg=str(t))
        po, pc = oracle.permute(off, col, d[f"{t}/rperminv"], d[f"{t}/cperminv"])
        np.testing.assert_array_equal(po, d[f"{t}/p_offset"], err_msg=str(t))
        np.testing.assert_array_equal(pc, d[f"{t}/p_nonzero"], err_msg=str(t))


def test_rand_perm_matches_reference_golden(oracle, golden):
    d = golden("spmat")
    for p in d["perms"]:
        _, n, seed = str(p).split("_")
        np.testing.assert_array_equal(oracle.rand_perm(int(n), int(seed)), d[p], err_msg=str(p))


def test_rand_perm_exstack_matches_reference_golden(oracle, golden):
    d = golden("spmat")
    for p in d["xperms"]:
        _, n, seed, b = str(p).split("_")
        np.testing.assert_array_equal(oracle.rand_perm_exstack(int(n), int(seed), int(b)), d[p], err_msg=str(p))
    # rand_permp is the exstack form with buffers of 1024, not rand_permp_agi
    np.testing.assert_array_equal(d["permp_100000_31"], d["xperm_100000_31_1024"])
    assert not np.array_equal(d["permp_100000_31"], d["perm_100000_31"])


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_spmat_restatements_match_reference_on_fresh_inputs(oracle, bale):
    ref = Reference()
    for seed in (3, 4):
        L = bale.gen_rmat(10, 8, 0.57, 0.19, 0.19, seed)
        n = L.numrows
        to, tc = oracle.transpose(L.offset, L.nonzero, n)
        ro, rc = ref.transpose(L.offset, L.nonzero, n)
        np.testing.assert_array_equal(to, ro)
        np.testing.assert_array_equal(tc, rc)
        rinv = np.argsort(bale.gen_values(n, seed)).astype(np.int64)
        cinv = np.argsort(bale.gen_values(n, seed + 9)).astype(np.int64)
        po, pc = oracle.permute(L.offset, L.nonzero, rinv, cinv)
        qo, qc = ref.permute(L.offset, L.nonzero, n, rinv, cinv)
        np.testing.assert_array_equal(po, qo)
        np.testing.assert_array_equal(pc, qc)
        np.testing.assert_array_equal(oracle.rand_perm(5000 + seed, seed), ref.rand_perm(5000 + seed, seed))
        for b in (1, 3, 1000, 5003, 10_000):
            np.testing.assert_array_equal(oracle.rand_perm_exstack(5000 + seed, seed, b),
                                          ref.rand_perm_exstack(5000 + seed, seed, b), err_msg=str(b))


def _small_matrices(r: int, c: int, descending: bool):
    """Every r x c 0/1 matrix as a CSR, each row's columns ascending or descending."""
    for mask in range(1 << (r * c)):
        rows = [[j for j in range(c) if mask >> (i * c + j) & 1] for i in range(r)]
        if descending:
            rows = [row[::-1] for row in rows]
        off = np.zeros(r + 1, np.int64)
        off[1:] = np.cumsum([len(x) for x in rows])
        yield off, np.array([j for x in rows for j in x], np.int64)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_spmat_restatements_match_reference_on_every_small_matrix(oracle):
    import itertools

    ref = Reference()
    for r, c in [(3, 3), (2, 4), (4, 2), (1, 5), (5, 1)]:
        for desc in (False, True):
            for off, col in _small_matrices(r, c, desc):
                to, tc = oracle.transpose(off, col, c)
                ro, rc = ref.transpose(off, col, c)
                assert np.array_equal(to, ro) and np.array_equal(tc, rc), (r, c, desc, off, col)
    for r, c in [(3, 3), (2, 4), (4, 2)]:
        mats = list(_small_matrices(r, c, False))[::37] + list(_small_matrices(r, c, True))[-1:]
        for rp in itertools.permutations(range(r)):
            for cp in itertools.permutations(range(c)):
                rinv, cinv = np.array(rp, np.int64), np.array(cp, np.int64)
                for off, col in mats:
                    po, pc = oracle.permute(off, col, rinv, cinv)
                    qo, qc = ref.permute(off, col, c, rinv, cinv)
                    assert np.array_equal(po, qo) and np.array_equal(pc, qc), (rp, cp, off, col)


def _tiny_graphs(nmax: int = 5):
    """Every strictly lower, ascending CSR on 1..nmax vertices."""
    for n in range(1, nmax + 1):
        pairs = [(i, j) for i in range(n) for j in range(i)]
        for mask in range(1 << len(pairs)):
            rows = [[] for _ in range(n)]
            for b, (i, j) in enumerate(pairs):
                if mask >> b & 1:
                    rows[i].append(j)
            off = np.zeros(n + 1, np.int64)
            off[1:] = np.cumsum([len(r) for r in rows])
            yield off, np.array([j for r in rows for j in r], np.int64)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_triangle_restatements_match_every_reference_variant_on_every_tiny_graph(oracle):
    ref = Reference()
    for off, col in _tiny_graphs():
        r = ref.triangles(off, col)
        cnt, pulls = oracle.triangle_agi(off, col)
        pcnt, pushes = oracle.triangle_exstack_push(off, col)
        assert {v[0] for v in r.values()} == {cnt} == {pcnt}, (off, col, r)
        assert r["triangle_agi"][1] == pulls, (off, col)
        assert r["triangle_exstack_push"][1] == pushes, (off, col)


def _libc():
    import ctypes

    libc = ctypes.CDLL(None)
    libc.srand48.argtypes = [ctypes.c_long]
    libc.srand48.restype = None
    libc.lrand48.restype = ctypes.c_long
    return libc


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
@pytest.mark.parametrize("mode", [0, 1, 2])
def test_kronecker_generator_builds_the_reference_graph(bale, mode):
    """bale_gen_kronecker against the triangle app's own -K construction,
    nonzero for nonzero: the closed-form counts hold for exactly that graph."""
    ref = Reference()
    for specs in ([3, 4], [1, 2, 3], [3, 4, 5, 9], [2, 3, 4, 5, 2], [1, 4, 9, 16], [5, 1, 7]):
        L = bale.gen_kronecker(mode, specs)
        ro, rc = ref.kronecker_lower(mode, specs)
        np.testing.assert_array_equal(L.offset, ro, err_msg=f"{mode} {specs}")
        np.testing.assert_array_equal(L.nonzero, rc, err_msg=f"{mode} {specs}")


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_reference_alg_1_counts_equal_alg_0(oracle, bale):
    """The drop-ins compute alg 0 from L for either alg; the reference's alg 1
    (L and U*L with U = L^T, triangle_agi.upc:100-136) must count the same,
    in every variant, on every tiny graph and on R-MAT graphs."""
    import ctypes as C

    ref = Reference()
    graphs = list(_tiny_graphs())
    for scale, seed in ((9, 3), (10, 4)):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed)
        graphs.append((L.offset, L.nonzero))
    for off, col in graphs:
        n = off.size - 1
        uo, uc = oracle.transpose(off, col, n)
        want = oracle.triangle_agi(off, col)[0]
        Lm, Um = ref._mat(off, col), ref._mat(uo, uc)  # square: U = L^T has n rows too
        for name, extra in (("triangle_agi", ()), ("triangle_exstack_push", (1024,)),
                            ("triangle_exstack2_push", (1024,)), ("triangle_agi_iter", ())):
            cnt, sr = C.c_int64(0), C.c_int64(0)
            assert getattr(ref.lib, name)(C.byref(cnt), C.byref(sr), C.byref(Lm), C.byref(Um), 1, *extra) >= 0
            assert cnt.value == want, (name, off, col)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_rand_perm_seed_zero_continues_the_c_library_stream(oracle):
    """Seed 0 does not reseed (spmat_agi.upc:61, spmat_exstack.upc:92): the
    permutation depends on the drand48 state the caller left, and every call
    leaves the stream just past its last draw.  Sequences of calls from the
    same starting state, read out with a final lrand48(), must agree."""
    libc, ref = _libc(), Reference()

    def run(impl, call):
        if call[0] == "agi":
            return impl.rand_perm(call[1], call[2])
        return impl.rand_perm_exstack(call[1], call[2], call[3])

    sequences = [
        [("agi", 10, 0), ("agi", 1, 0), ("x", 7, 0, 3), ("x", 100, 0, 1024), ("x", 33, 0, 1)],
        [("agi", 5, 9), ("agi", 12, 0), ("x", 40, 4, 2), ("x", 40, 0, 2), ("agi", 3, 0)],
        [("x", 1000, 0, 7), ("agi", 1000, 0), ("x", 64, 0, 64), ("x", 65, 0, 64)],
    ]
    for start in (0, 5, 123456):
        for calls in sequences:
            libc.srand48(start)
            ours = [run(oracle, c) for c in calls]
            ours_next = libc.lrand48()
            libc.srand48(start)
            theirs = [run(ref, c) for c in calls]
            theirs_next = libc.lrand48()
            for c, a, b in zip(calls, ours, theirs):
                np.testing.assert_array_equal(a, b, err_msg=f"start {start} {c}")
            assert ours_next == theirs_next, (start, calls)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_rand_perm_restatements_match_reference_for_small_n(oracle):
    ref = Reference()
    for n in range(1, 130):
        for seed in (1, 77, 2 ** 32 + 5):
            np.testing.assert_array_equal(oracle.rand_perm(n, seed), ref.rand_perm(n, seed), err_msg=f"{n} {seed}")
            for b in sorted({1, 2, 3, 7, n, 1024}):
                np.testing.assert_array_equal(oracle.rand_perm_exstack(n, seed, b), ref.rand_perm_exstack(n, seed, b),
                                              err_msg=f"{n} {seed} {b}")


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_histo_and_ig_restatements_match_every_reference_variant_on_tiny_inputs(oracle):
    """Every index array of length 1..4 over tables of 1..3 entries, through
    the reference's agi, exstack and exstack2 variants (buffers of 1 and
    1024) and the oracle."""
    import ctypes as C
    import itertools

    ref = Reference()
    P = lambda a: a.ctypes.data_as(C.POINTER(C.c_int64))  # noqa: E731
    for t in (1, 2, 3):
        table = -(np.arange(t, dtype=np.int64) + 1) * 1000003
        for length in (1, 2, 3, 4):
            for idx in itertools.product(range(t), repeat=length):
                index = np.array(idx, np.int64)
                pck = index << 16
                want = np.zeros(t, np.int64)
                oracle.histo_agi(index, want)
                got = np.zeros(t, np.int64)
                assert ref.lib.histo_agi(P(index), length, P(got)) >= 0
                np.testing.assert_array_equal(got, want)
                for fn in ("histo_exstack", "histo_exstack2"):
                    for b in (1, 1024):
                        got = np.zeros(t, np.int64)
                        assert getattr(ref.lib, fn)(P(pck), length, P(got), b) >= 0
                        np.testing.assert_array_equal(got, want, err_msg=f"{fn} {b} {idx}")
                gather = oracle.ig_agi(index, table)
                tgt = np.zeros(length, np.int64)
                assert ref.lib.ig_agi(P(tgt), P(index), length, P(table)) >= 0
                np.testing.assert_array_equal(tgt, gather)
                for fn in ("ig_exstack", "ig_exstack2"):
                    for b in (1, 1024):
                        tgt = np.zeros(length, np.int64)
                        assert getattr(ref.lib, fn)(P(tgt), P(pck), length, P(table), b) >= 0
                        np.testing.assert_array_equal(tgt, gather, err_msg=f"{fn} {b} {idx}")


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_file_restatements_match_reference_on_small_matrices(oracle, tmp_path, monkeypatch):
    """MatrixMarket files the reference writes, and the same entries shuffled,
    read by both readers; binary datasets written by both writers."""
    import shutil
    from pathlib import Path

    ref = Reference()
    rng = np.random.default_rng(5)
    monkeypatch.chdir(tmp_path)  # short relative names: the reference's file names are 64-byte buffers
    for r, c in [(3, 3), (2, 4), (4, 2)]:
        for k, (off, col) in enumerate(_small_matrices(r, c, False)):
            ref.write_mm(off, col, c, "a.mm")
            lines = Path("a.mm").read_text().splitlines()
            body = lines[2:]
            Path("s.mm").write_text("\n".join(lines[:2] + [body[i] for i in rng.permutation(len(body))]) + "\n")
            # the integer field: a value after each entry, read and dropped
            Path("i.mm").write_text("\n".join(["%%MatrixMarket matrix coordinate integer", lines[1]] +
                                              [f"{e} {int(v)}" for e, v in zip(body, rng.integers(-9, 99, len(body)))])
                                    + "\n")
            # repeated entries are kept, in file order within each row
            dup = body + [body[i] for i in rng.integers(0, len(body), len(body) // 2)] if body else []
            dup = [dup[i] for i in rng.permutation(len(dup))]
            Path("d.mm").write_text("\n".join(["%%MatrixMarket matrix coordinate pattern", f"{r} {c} {len(dup)}"]
                                              + dup) + "\n")
            for path in ("a.mm", "s.mm", "i.mm", "d.mm"):
                oo, oc, onc = oracle.read_mm(path)
                ro, rc, rnc = ref.read_mm(path)
                assert onc == rnc == c and np.array_equal(oo, ro) and np.array_equal(oc, rc), (r, c, k, path)
            oracle.write_dataset(off, col, c, "o")
            ref.write_dataset(off, col, c, "r")
            for name in ("metadata", "rowcnt_0", "nonzero_0"):
                assert Path("o", name).read_bytes() == Path("r", name).read_bytes(), (r, c, k, name)
            shutil.rmtree("o")
            shutil.rmtree("r")


def test_matrix_market_reader_matches_reference_golden(oracle, golden):
    from pathlib import Path

    gdir = Path(__file__).resolve().parent / "golden"
    d = golden("spmat")
    for f in d["mm_files"]:
        off, col, nc = oracle.read_mm(gdir / str(f))
        np.testing.assert_array_equal(off, d[f"mm/{f}/offset"], err_msg=str(f))
        np.testing.assert_array_equal(col, d[f"mm/{f}/nonzero"], err_msg=str(f))
        assert nc == int(d[f"mm/{f}/numcols"][0])


@pytest.mark.parametrize("n,rng,seed", [(0, 5, 1), (1, 1, 2), (12_345, 1_000_000, 1), ((1 << 20) + 7, 1 << 26, 3),
                                        (70_000, (1 << 40) + 3, 9)])
def test_oracle_generators_equal_the_library_generators(oracle, bale, n, rng, seed):
    """The reference arm of the benchmark builds its inputs with the oracle's
    SplitMix64 generators so that it never loads the GPU library; they must
    give exactly the library's buffers, for any thread count."""
    want_u = bale.gen_uniform(n, rng, seed)
    want_v = bale.gen_values(n, seed)
    for threads in (1, 3, 0):
        np.testing.assert_array_equal(oracle.gen_uniform(n, rng, seed, threads), want_u)
        np.testing.assert_array_equal(oracle.gen_values(n, seed, threads), want_v)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_alg1_restatement_matches_reference_with_any_upper_u(oracle, bale):
    """The restatement of triangle_agi's alg 1 (triangle_agi.upc:100-136) gives
    the reference's count and shared-reference tally for U = L^T and for
    upper matrices U that are not L^T (another graph's transpose, L^T with
    entries dropped): alg 1 sums |U_i and U_j| over L's nonzeros whatever U
    is.  U's column array carries one zero past its end, as the reference
    reads the first column of an empty last row."""
    import ctypes as C

    ref = Reference()
    rng = np.random.default_rng(5)
    cases = []
    for off, col in list(_tiny_graphs())[::37]:
        cases.append((off, col, off, col))
    for scale, seed in ((8, 3), (9, 4)):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed)
        cases.append((L.offset, L.nonzero, L.offset, L.nonzero))
        L2 = bale.gen_rmat(scale, 8, 0.57, 0.19, 0.19, seed + 10)
        cases.append((L.offset, L.nonzero, L2.offset, L2.nonzero))  # U from another graph
        keep = rng.random(L.nnz) < 0.7
        rows = np.repeat(np.arange(L.numrows), np.diff(L.offset))
        off3 = np.zeros(L.numrows + 1, np.int64)
        np.add.at(off3, rows[keep] + 1, 1)
        cases.append((L.offset, L.nonzero, np.cumsum(off3), np.ascontiguousarray(L.nonzero[keep])))
    for loff, lcol, moff, mcol in cases:
        n = loff.size - 1
        uo, uc = oracle.transpose(moff, mcol, n)
        ucp = np.concatenate([uc, np.zeros(1, np.int64)])
        Lm = ref._mat(loff, lcol)
        Um = ref._mat(uo, ucp)
        Um.nnz = Um.lnnz = uc.size
        cnt, sr = C.c_int64(0), C.c_int64(0)
        assert ref.lib.triangle_agi(C.byref(cnt), C.byref(sr), C.byref(Lm), C.byref(Um), 1) >= 0
        got = oracle.triangle_agi_alg1(loff, lcol, uo, uc)
        assert got == (cnt.value, sr.value)


@pytest.mark.skipif(not REF_LIB.exists(), reason="oracle/_ref is built only where the reference tree exists")
def test_rand_permp_exstack2_is_the_exstack_form(oracle, golden):
    """The reference's rand_permp_exstack2 returns rand_permp_exstack (spmat/
    spmat_exstack2.upc:60-73): its golden outputs equal the exstack
    restatement's, and the reference's two functions agree on fresh cases."""
    d = golden("spmat")
    for p in d["x2perms"]:
        _, n, seed, b = str(p).split("_")
        np.testing.assert_array_equal(oracle.rand_perm_exstack(int(n), int(seed), int(b)), d[p], err_msg=str(p))
    ref = Reference()
    for n, seed, b in ((77, 3, 5), (2048, 11, 1024)):
        np.testing.assert_array_equal(ref.rand_perm_exstack2(n, seed, b), ref.rand_perm_exstack(n, seed, b))


def test_buffered_exstack_restatements_match_reference_golden(oracle, golden):
    """The one-PE exstack model (buffers, exchange, FIFO pops) gives the
    reference's results for every buffer size, including one package."""
    d = golden("histo")
    for name in _cases(d, "/index"):
        index = d[f"{name}/index"]
        pck = (index << 16).astype(np.int64)
        for buf in (1, 7, 1024):
            c = d[f"{name}/after_agi"].copy()
            oracle.histo_exstack_buffered(pck, c, buf)
            np.testing.assert_array_equal(c, d[f"{name}/after_exstack"], err_msg=f"{name} buf {buf}")
    d = golden("ig")
    for name in _cases(d, "/index"):
        index, table = d[f"{name}/index"], d[f"{name}/table"]
        pck = (index << 16).astype(np.int64)
        for buf in (1, 7, 1024):
            np.testing.assert_array_equal(oracle.ig_exstack_buffered(pck, table, buf), d[f"{name}/tgt"],
                                          err_msg=f"{name} buf {buf}")
    d = golden("triangles")
    for g in d["graphs"]:
        off, col = d[f"{g}/offset"], d[f"{g}/nonzero"]
        for buf in (1, 5, 1024):
            assert oracle.triangle_exstack_push_buffered(off, col, buf) == tuple(
                int(x) for x in d[f"{g}/triangle_exstack_push"]), (g, buf)


def test_sampled_row_loops_add_up(oracle, bale):
    """Row samples of the AGI and buffered exstack loops partition the count."""
    L = bale.gen_rmat(12, 16, 0.57, 0.19, 0.19, 9)
    whole = oracle.triangle_agi(L.offset, L.nonzero)[0]
    assert sum(oracle.triangle_agi_sampled(L.offset, L.nonzero, r, 5) for r in range(5)) == whole
    assert sum(oracle.triangle_exstack_push_buffered(L.offset, L.nonzero, 64, r, 5)[0] for r in range(5)) == whole
    for bad in ((0, 0), (0, -1)):
        with pytest.raises(ValueError):
            oracle.triangle_exstack_push_buffered(L.offset, L.nonzero, 64, *bad)
    with pytest.raises(ValueError):
        oracle.histo_exstack_buffered(np.zeros(3, np.int64), np.zeros(1, np.int64), 0)
