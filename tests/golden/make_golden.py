"""Regenerate the golden vectors in tests/golden/ from the reference itself.

    python tests/golden/make_golden.py

Compiles the reference's own unmodified histo / ig / triangles / spmat sources
against the single-PE shim (oracle/Makefile target ``ref``, reads the
reference tree, writes only oracle/_ref/) and records, for small seeded
inputs, what the reference returns:

* histo.npz      -- counts after histo_agi, then histo_exstack, then
                    histo_exstack2 add into the same array (the reference app
                    accumulates across models, apps/histo_src/histo.upc:161-213);
* ig.npz         -- tgt from ig_agi, and whether ig_exstack and ig_exstack2
                    returned the same vector;
* spmat.npz      -- transpose_matrix_agi and permute_matrix_agi of small
                    matrices (an R-MAT lower matrix, the reference's own
                    Erdos-Renyi graph, a rectangular matrix with empty rows),
                    rand_permp_agi(n, seed) and rand_permp_exstack(n, seed,
                    buf_cnt) permutations, one rand_permp, and the reference's
                    read_matrix_mm_to_dist of MatrixMarket files written by its
                    write_matrix_mm (*.mm, committed beside the vectors) and of
                    a hand-made integer file with rows out of order;
* ds_<tag>/      -- binary datasets (metadata, rowcnt_0, nonzero_0) that
                    write_sparse_matrix_agi writes for two of those matrices
                    (write_sparse_matrix_exstack writes the same bytes);
* triangles.npz  -- count and shared-refs/pushes of triangle_agi,
                    triangle_exstack_push, triangle_exstack2_push and the
                    alternate triangle_agi_iter on Kronecker graphs (closed-form
                    answers), the reference's own Erdos-Renyi graph, and R-MAT
                    graphs from this package's generator.

The inputs are stored next to the outputs, so the fixtures need neither the
reference nor the generators to be checked.
"""
from __future__ import annotations

import sys
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import bale_old_gb300 as bale  # noqa: E402  (inputs only)
from oracle.pyoracle import Reference, build_ref  # noqa: E402

OUT = Path(__file__).resolve().parent


def _p(a):
    import ctypes as C
    return a.ctypes.data_as(C.POINTER(C.c_int64))


def make_histo(ref: Reference) -> dict:
    cases = {}
    # (name, num updates, table size, generator)
    specs = [
        ("uniform", 20_000, 5_000, lambda n, t: bale.gen_uniform(n, t, 11), True),
        ("zipf_small_table", 20_000, 64, lambda n, t: bale.gen_zipf(n, t, 1.1, 21, 22), True),
        ("uniform_big_table", 10_000, 100_000, lambda n, t: bale.gen_uniform(n, t, 31), False),
        ("ragged_odd", 1_001, 997, lambda n, t: bale.gen_uniform(n, t, 41), True),
    ]
    for name, n, t, gen, nonzero_start in specs:
        index = np.ascontiguousarray(gen(n, t))
        pck = bale.pack_index(index)
        # a non-zero start checks that the drop-ins ADD into counts
        counts0 = bale.gen_uniform(t, 1000, 12) if nonzero_start else np.zeros(t, np.int64)
        c = counts0.copy()
        assert ref.lib.histo_agi(_p(index), n, _p(c)) >= 0
        after_agi = c.copy()
        assert ref.lib.histo_exstack(_p(pck), n, _p(c), 1024) >= 0
        after_exstack = c.copy()
        assert ref.lib.histo_exstack2(_p(pck), n, _p(c), 1024) >= 0
        after_exstack2 = c.copy()
        cases.update({f"{name}/index": index, f"{name}/counts0": counts0,
                      f"{name}/after_agi": after_agi, f"{name}/after_exstack": after_exstack,
                      f"{name}/after_exstack2": after_exstack2})
    return cases


def make_ig(ref: Reference) -> dict:
    cases = {}
    specs = [
        ("uniform", 20_000, 4_096, lambda n, t: bale.gen_uniform(n, t, 14), lambda t: bale.gen_values(t, 13)),
        ("negative_table", 10_000, 3_000, lambda n, t: bale.gen_uniform(n, t, 15), bale.gen_negative_table),
        ("zipf", 10_000, 10_000, lambda n, t: bale.gen_zipf(n, t, 1.1, 16, 17), lambda t: bale.gen_values(t, 18)),
        ("ragged_odd", 999, 1_001, lambda n, t: bale.gen_uniform(n, t, 19), lambda t: bale.gen_values(t, 20)),
    ]
    for name, n, t, gidx, gtab in specs:
        index = np.ascontiguousarray(gidx(n, t))
        pck = bale.pack_index(index)
        table = np.ascontiguousarray(gtab(t))
        outs = {}
        for fn, arg, extra in (("ig_agi", index, ()), ("ig_exstack", pck, (1024,)), ("ig_exstack2", pck, (1024,))):
            tgt = np.zeros(n, np.int64)
            assert getattr(ref.lib, fn)(_p(tgt), _p(arg), n, _p(table), *extra) >= 0
            outs[fn] = tgt
        # the three reference variants agree; store one vector and the agreement
        same = [bool(np.array_equal(outs["ig_agi"], outs[k])) for k in ("ig_exstack", "ig_exstack2")]
        cases.update({f"{name}/index": index, f"{name}/table": table, f"{name}/tgt": outs["ig_agi"],
                      f"{name}/exstack_variants_agree": np.array(same)})
    return cases


def make_triangles(ref: Reference) -> dict:
    cases = {}
    graphs = []
    for mode, specs in ((1, [3, 4, 5, 9]), (2, [3, 4, 5, 9, 2]), (0, [3, 4, 5, 9]), (1, [2, 2, 3])):
        L = bale.gen_kronecker(mode, specs)
        tag = "kron" + str(mode) + "_" + "_".join(map(str, specs))
        graphs.append((tag, L.offset, L.nonzero, bale.kronecker_triangles(mode, specs)))
    off, col = ref.erdos_renyi_lower(3000, 24.0 / 3000, 12345)
    graphs.append(("ref_erdos_renyi_3000", off, col, -1))
    for scale, seed in ((9, 6), (10, 1006)):
        L = bale.gen_rmat(scale, 16, 0.57, 0.19, 0.19, seed)
        graphs.append((f"rmat{scale}", L.offset, L.nonzero, -1))
    names = []
    for tag, off, col, closed in graphs:
        res = ref.triangles(off, col)
        names.append(tag)
        cases[f"{tag}/offset"] = off
        cases[f"{tag}/nonzero"] = col
        cases[f"{tag}/closed_form"] = np.array([closed], np.int64)
        for k, (cnt, sr) in res.items():
            cases[f"{tag}/{k}"] = np.array([cnt, sr], np.int64)
    cases["graphs"] = np.array(names)
    return cases


def make_spmat(ref: Reference) -> dict:
    """transpose_matrix_agi, permute_matrix_agi and rand_permp_agi at one PE."""
    cases = {}
    mats = []
    L = bale.gen_rmat(8, 16, 0.57, 0.19, 0.19, 7)
    mats.append(("rmat8_lower", L.offset, L.nonzero, L.numrows))
    off, col = ref.erdos_renyi_lower(500, 10.0 / 500, 4242)
    mats.append(("ref_erdos_renyi_500", off, col, 500))
    # a rectangular matrix with empty rows and ascending random columns
    rng = np.random.default_rng(17)
    rows, ncols = 300, 517
    lens = rng.integers(0, 12, rows)
    lens[rng.integers(0, rows, 40)] = 0
    cols = [np.sort(rng.choice(ncols, size=k, replace=False)) for k in lens]
    mats.append(("rect_300x517", np.concatenate([[0], np.cumsum(lens)]).astype(np.int64),
                 np.concatenate(cols).astype(np.int64), ncols))
    mats.append(("one_row", np.array([0, 0], np.int64), np.zeros(0, np.int64), 1))
    names = []
    for k, (tag, off, col, ncols) in enumerate(mats):
        n = off.size - 1
        t_off, t_col = ref.transpose(off, col, ncols)
        rinv = np.argsort(bale.gen_values(n, 60 + k)).astype(np.int64)
        cinv = np.argsort(bale.gen_values(ncols, 70 + k)).astype(np.int64)
        p_off, p_col = ref.permute(off, col, ncols, rinv, cinv)
        names.append(tag)
        cases.update({f"{tag}/offset": off, f"{tag}/nonzero": col, f"{tag}/numcols": np.array([ncols], np.int64),
                      f"{tag}/t_offset": t_off, f"{tag}/t_nonzero": t_col,
                      f"{tag}/rperminv": rinv, f"{tag}/cperminv": cinv,
                      f"{tag}/p_offset": p_off, f"{tag}/p_nonzero": p_col})
    cases["mats"] = np.array(names)
    perms = []
    for n, seed in ((1, 1), (2, 7), (10, 12345), (1000, 99), (100_000, 31)):
        perms.append(f"perm_{n}_{seed}")
        cases[f"perm_{n}_{seed}"] = ref.rand_perm(n, seed)
    cases["perms"] = np.array(perms)
    # rand_permp_exstack(n, seed, buf_cnt): rounds that fill the buffer
    # (buf_cnt < n), the rounds after (buf_cnt near n), and one round
    # (buf_cnt >= n); rand_permp is buf_cnt = 1024
    xperms = []
    for n, seed, b in ((1, 1, 1024), (5, 3, 1), (40, 9, 2), (1000, 99, 7), (1023, 5, 1024), (1024, 5, 1024),
                       (1025, 5, 1024), (3000, 2, 4096), (5000, 8, 64), (100_000, 31, 1024)):
        xperms.append(f"xperm_{n}_{seed}_{b}")
        cases[f"xperm_{n}_{seed}_{b}"] = ref.rand_perm_exstack(n, seed, b)
    cases["xperms"] = np.array(xperms)
    cases["permp_100000_31"] = ref.rand_permp(100_000, 31)
    # rand_permp_exstack2(n, seed, buf_cnt), as the randperm app's model 4 calls it
    x2perms = []
    for n, seed, b in ((1, 1, 1024), (40, 9, 2), (1000, 99, 7), (5000, 8, 64), (100_000, 31, 1024)):
        x2perms.append(f"x2perm_{n}_{seed}_{b}")
        cases[f"x2perm_{n}_{seed}_{b}"] = ref.rand_perm_exstack2(n, seed, b)
    cases["x2perms"] = np.array(x2perms)
    # MatrixMarket: files written by the reference's writer, and a hand-made
    # one with rows out of order, comment-free, integer field; read back by
    # the reference's reader
    mm = []
    for tag in ("rmat8_lower", "rect_300x517"):
        path = OUT / f"{tag}.mm"
        ref.write_mm(cases[f"{tag}/offset"], cases[f"{tag}/nonzero"], int(cases[f"{tag}/numcols"][0]), str(path))
        mm.append(path.name)
    path = OUT / "unordered_integer.mm"
    lines = ["%%MatrixMarket matrix coordinate integer", "5 7 9",
             "3 2 10", "1 7 -4", "3 1 5", "5 5 1", "1 1 2", "3 6 7", "2 4 0", "5 1 3", "1 3 9"]
    path.write_text("\n".join(lines) + "\n")
    mm.append(path.name)
    for name in mm:
        off, col, nc = ref.read_mm(str(OUT / name))
        cases.update({f"mm/{name}/offset": off, f"mm/{name}/nonzero": col,
                      f"mm/{name}/numcols": np.array([nc], np.int64)})
    cases["mm_files"] = np.array(mm)
    return cases


def make_datasets(ref: Reference, spmat: dict) -> list[str]:
    """Binary sparse matrix datasets: write_sparse_matrix_agi of two of the
    spmat matrices at one PE, copied to ds_<tag>/ (metadata, rowcnt_0,
    nonzero_0); write_sparse_matrix_exstack (buffers of 1024 and of 16
    packages) must write the same bytes."""
    import filecmp
    import os
    import shutil
    import tempfile

    made = []
    for tag in ("rmat8_lower", "rect_300x517"):
        off, col = spmat[f"{tag}/offset"], spmat[f"{tag}/nonzero"]
        nc = int(spmat[f"{tag}/numcols"][0])
        tmp = tempfile.mkdtemp(prefix="bds")
        cwd = os.getcwd()
        try:
            os.chdir(tmp)  # the reference builds file names in 64-byte buffers
            ref.write_dataset(off, col, nc, "agi")
            for b in (1024, 16):
                ref.write_dataset(off, col, nc, f"ex{b}", buf_cnt=b)
                for f in ("metadata", "rowcnt_0", "nonzero_0"):
                    assert filecmp.cmp(f"agi/{f}", f"ex{b}/{f}", shallow=False), (tag, b, f)
            dst = OUT / f"ds_{tag}"
            shutil.rmtree(dst, ignore_errors=True)
            shutil.copytree("agi", dst)
        finally:
            os.chdir(cwd)
            shutil.rmtree(tmp)
        made.append(f"ds_{tag}")
    return made


def main() -> int:
    if build_ref() is None:
        print("reference tree not found; cannot regenerate golden vectors", file=sys.stderr)
        return 1
    ref = Reference()
    np.savez_compressed(OUT / "histo.npz", **make_histo(ref))
    np.savez_compressed(OUT / "ig.npz", **make_ig(ref))
    np.savez_compressed(OUT / "triangles.npz", **make_triangles(ref))
    spmat = make_spmat(ref)
    np.savez_compressed(OUT / "spmat.npz", **spmat)
    for d in make_datasets(ref, spmat):
        print(d, sum(f.stat().st_size for f in (OUT / d).iterdir()), "bytes")
    for f in ("histo.npz", "ig.npz", "triangles.npz", "spmat.npz", "rmat8_lower.mm", "rect_300x517.mm",
              "unordered_integer.mm"):
        print(f, (OUT / f).stat().st_size, "bytes")
    return 0


if __name__ == "__main__":
    sys.exit(main())
