"""The serving loop: every request's result is exact, and is the same when the
request runs alone as when it runs inside a mixed, overlapping trace."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _world(bale, serve_mod, server, seed: int):
    """Resident objects: three tables, two counter arrays, two graphs."""
    tables = [bale.gen_values(t, seed + i) for i, t in enumerate((1 << 10, 1 << 16, (1 << 22) + 3))]
    tids = [server.add_table(t) for t in tables]
    cids = [server.add_counts(c) for c in (1000, 1 << 20)]
    graphs = [bale.gen_rmat(sc, 16, 0.57, 0.19, 0.19, seed + sc) for sc in (10, 14)]
    gids = [server.add_graph(L) for L in graphs]
    return tables, tids, cids, graphs, gids


def _trace(bale, serve_mod, world, nreq: int, seed: int, rate: float):
    tables, tids, cids, graphs, gids = world
    rng = np.random.default_rng(seed)
    arrivals = serve_mod.poisson_arrivals(nreq, rate, seed)
    reqs, expect = [], []
    for k in range(nreq):
        u = rng.random()
        n = int(np.exp(rng.uniform(np.log(1), np.log(1 << 20))))
        if u < 0.6:
            j = int(rng.integers(len(tids)))
            t = tables[j].size
            idx = bale.gen_uniform(n, t, 1000 * seed + k)
            out = np.full(n, 7, np.int64)
            reqs.append(serve_mod.ig(tids[j], idx, out, arrivals[k]))
            expect.append(("ig", tables[j][idx]))
        elif u < 0.9:
            j = int(rng.integers(len(cids)))
            c = (1000, 1 << 20)[j]
            idx = bale.gen_uniform(n, c, 2000 * seed + k)
            reqs.append(serve_mod.histo(cids[j], idx, arrivals[k]))
            expect.append(("histo", (j, idx)))
        else:
            j = int(rng.integers(len(gids)))
            out = np.zeros(1, np.int64)
            reqs.append(serve_mod.triangles(gids[j], out, arrivals[k]))
            expect.append(("tri", j))
    return reqs, expect


def _check(oracle, world, server, reqs, expect):
    tables, tids, cids, graphs, gids = world
    want_counts = {j: np.zeros((1000, 1 << 20)[j], np.int64) for j in range(2)}
    tri_want = [oracle.triangle_agi(L.offset, L.nonzero)[0] for L in graphs]
    for r, (kind, e) in zip(reqs, expect):
        if kind == "ig":
            np.testing.assert_array_equal(r.out, e)
        elif kind == "tri":
            assert int(r.out[0]) == tri_want[e]
        else:
            j, idx = e
            want_counts[j] += np.bincount(idx, minlength=want_counts[j].size)
    for j, c in enumerate(cids):
        np.testing.assert_array_equal(server.read_counts(c), want_counts[j])


def test_mixed_trace_is_exact(cuda, bale, oracle):
    from bale_old_gb300 import serve

    with serve.Server(arena_bytes=1 << 30, max_active=32) as s:
        world = _world(bale, serve, s, 3)
        reqs, expect = _trace(bale, serve, world, 150, seed=5, rate=20_000.0)
        lat, st = s.run(reqs)
        assert (lat > 0).all() and st["p99_s"] >= st["p50_s"] > 0
        assert st["ticks"] > 1 and st["bad"] == 0 and st["max_active"] > 1
        _check(oracle, world, s, reqs, expect)


class knobs:
    """Set tuning knobs for a block, restoring the previous values after."""

    def __init__(self, bale, **kv):
        self.bale, self.kv = bale, {k.replace("__", "."): v for k, v in kv.items()}

    def __enter__(self):
        self.old = {k: self.bale.tune_get(k) for k in self.kv}
        for k, v in self.kv.items():
            self.bale.tune_set(k, v)

    def __exit__(self, *exc):
        for k, v in self.old.items():
            self.bale.tune_set(k, v)


# thresholds low enough that most requests of the trace run as express
# kernels, on both the direct and the region-partitioned ig / histo paths
EXPRESS_RULES = dict(batch__standalone_min=1 << 14, batch__standalone_min_edges=1 << 10,
                     ig__part_min_table_bytes=1 << 20, ig__part_min_requests=1 << 16,
                     histo__part_min_table_bytes=1 << 20, histo__part_min_updates=1 << 16)


@pytest.mark.parametrize("express", [0, 1])
def test_express_requests_are_exact(cuda, bale, oracle, express):
    """Large requests on their own kernels beside the ticks: same results."""
    from bale_old_gb300 import serve

    with knobs(bale, serve__express=express, serve__express_streams=3, **EXPRESS_RULES):
        with serve.Server(arena_bytes=1 << 30, max_active=24) as s:
            world = _world(bale, serve, s, 11)
            reqs, expect = _trace(bale, serve, world, 120, seed=13, rate=10_000.0)
            lat, st = s.run(reqs)
            assert st["bad"] == 0 and (lat > 0).all()
            if express:
                assert st["express"] > 10 and st["ticks"] > 0
            else:
                assert st["express"] == 0
            _check(oracle, world, s, reqs, expect)


def test_result_is_the_same_alone_and_in_the_mix(cuda, bale, oracle):
    """Run a trace, then each request again on its own: identical results."""
    from bale_old_gb300 import serve

    with serve.Server(arena_bytes=1 << 30, max_active=16) as s:
        world = _world(bale, serve, s, 7)
        reqs, expect = _trace(bale, serve, world, 60, seed=9, rate=0.0)  # all arrive at once
        s.run(reqs)
        mixed = [None if r.out is None else r.out.copy() for r in reqs]
        for k, r in enumerate(reqs):
            if r.kind == serve.HISTO:
                continue
            r.out[:] = -1
            r.arrival = 0.0
            s.run([r])
            np.testing.assert_array_equal(r.out, mixed[k], err_msg=f"request {k} alone vs mixed")
        # histo: a request alone on fresh counters equals its share of the mix
        hk = [k for k, r in enumerate(reqs) if r.kind == serve.HISTO]
        if hk:
            r = reqs[hk[0]]
            fresh = s.add_counts((1000, 1 << 20)[cids_index(world, r.obj)])
            s.run([serve.histo(fresh, r.index)])
            np.testing.assert_array_equal(s.read_counts(fresh),
                                          np.bincount(r.index, minlength=(1000, 1 << 20)[cids_index(world, r.obj)]))


def cids_index(world, obj):
    return world[2].index(obj)


def test_tiny_arena_forces_admission_waits(cuda, bale, oracle):
    """A 2 MiB arena holds two 1 MiB ig requests at a time: the other ten wait
    for arena space (not for slots) and still complete exactly."""
    from bale_old_gb300 import serve

    with serve.Server(arena_bytes=2 << 20, max_active=16) as s:
        table = bale.gen_values(1 << 20, 3)
        t = s.add_table(table)
        n = 1 << 16  # index + values = 1 MiB
        reqs = [serve.ig(t, bale.gen_uniform(n, 1 << 20, 40 + k), np.zeros(n, np.int64), 0.0) for k in range(12)]
        lat, st = s.run(reqs)
        assert st["admission_waits"] > 0 and st["max_active"] <= 2
        for r in reqs:
            np.testing.assert_array_equal(r.out, table[r.index])


def test_registration_refused_when_free_hbm_is_short(cuda, bale):
    """Admission control is tested on the host: a reserve larger than the
    device makes every registration fail with BALE_EBUSY, nothing faults."""
    from bale_old_gb300 import serve

    with serve.Server(arena_bytes=1 << 20, max_active=4) as s:
        bale.tune_set("serve.reserve_bytes", 1 << 50)
        try:
            with pytest.raises(bale.BaleError, match="status 6"):
                s.add_table(np.arange(1000, dtype=np.int64))
        finally:
            bale.tune_set("serve.reserve_bytes", -1)
        assert s.add_table(np.arange(1000, dtype=np.int64)) >= 0


def test_malformed_graph_is_refused_at_registration(cuda, bale):
    """A graph whose rows are not ascending inside [0,i) is refused with
    BALE_EINPUT (status 2) when it is registered; a good one is accepted."""
    from bale_old_gb300 import serve

    m = 40
    off = np.zeros(m + 1, np.int64)
    off[1:] = np.cumsum(np.arange(m))
    col = np.concatenate([np.arange(i, dtype=np.int64) for i in range(m)])
    bad = col.copy()
    bad[off[30] + 3], bad[off[30] + 4] = bad[off[30] + 4], bad[off[30] + 3]
    with serve.Server(arena_bytes=1 << 20, max_active=4) as s:
        with pytest.raises(bale.BaleError, match="status 2"):
            s.add_graph(bale.SparseMatrix(off, bad))
        g = s.add_graph(bale.SparseMatrix(off, col))
        out = np.zeros(1, np.int64)
        s.run([serve.triangles(g, out)])
        assert int(out[0]) == m * (m - 1) * (m - 2) // 6


def test_invalid_requests_are_rejected(cuda, bale):
    from bale_old_gb300 import serve

    with serve.Server(arena_bytes=1 << 20, max_active=4) as s:
        t = s.add_table(np.arange(100, dtype=np.int64))
        c = s.add_counts(10)
        idx = np.arange(10, dtype=np.int64)
        with pytest.raises(bale.BaleError):
            s.run([serve.Request(serve.HISTO, t, idx, None, 0.0)])  # a table is not a counter array
        with pytest.raises(bale.BaleError):
            s.run([serve.ig(c + 5, idx, np.zeros(10, np.int64))])  # no such object
        lat, st = s.run([])
        assert lat.size == 0
