"""Autotuner for the size-class choices of libbale_gb300 (its tuning knobs).

    python -m bale_old_gb300.autotune [--out bale_old_gb300/tuning/gb300.tune] [--quick]

Every knob selects among kernel variants that compute identical results, so
tuning only moves time.  On the current GPU the tuner measures, with CUDA
events after warm-up:

* ig    -- direct vs region-partitioned gather across table sizes and
           request counts -> ig.part_min_table_bytes, ig.part_min_requests;
* histo -- plain L2 reductions vs the region partition across table sizes
           -> histo.part_min_table_bytes, histo.part_min_updates;
* tri   -- the intersection strategy per graph: wedge probes (bitmap and
           staged search at the far vertex) or the bitmap/search hybrid over
           rows i, timed on R-MAT, Erdos-Renyi and Kronecker graphs, with the
           rule keyed on the reference's work model (pulls and pushes,
           apps/triangle_src/triangle.upc:325-369) fitted to the times ->
           tri.wedge_pull_pct, tri.wedge_push_per_nnz;
* batch -- tile sizes per size class, the standalone thresholds and the
           number of side streams of the batched graph, by coordinate
           descent on the small and full uneven mixes (bale_old_gb300.mix).

The winners go to a plain "name value" file (loadable from C with
bale_tune_load) and every measurement to a JSON report next to it.  The
package applies bale_old_gb300/tuning/gb300.tune at import when it exists.
"""
from __future__ import annotations

import argparse
import json
import sys
import time
from pathlib import Path

HERE = Path(__file__).resolve().parent
DEFAULT_OUT = HERE / "tuning" / "gb300.tune"


def _time(fn, reps: int = 5, warmup: int = 2) -> float:
    """Average milliseconds of fn() on the current stream."""
    import torch

    for _ in range(warmup):
        fn()
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    for _ in range(reps):
        fn()
    b.record()
    b.synchronize()
    return a.elapsed_time(b) / reps


def _crossover(rows: list[dict], key: str, fast: str, slow: str) -> int | None:
    """Smallest value of `key` from which `fast` beats `slow` at every larger value."""
    vals = sorted({r[key] for r in rows})
    best = None
    for v in reversed(vals):
        sub = [r for r in rows if r[key] == v]
        if all(r[fast] < r[slow] for r in sub):
            best = v
        else:
            break
    return best


def tune_ig(quick: bool) -> tuple[dict, list]:
    import torch

    import bale_old_gb300 as bale

    dev = torch.device("cuda:0")
    rows = []
    tlogs = (22, 23, 24, 25, 26) if quick else (21, 22, 23, 24, 25, 26, 27)
    nlogs = (20, 24) if quick else (18, 20, 22, 24, 26)
    for tl in tlogs:
        table = torch.empty(1 << tl, dtype=torch.int64, device=dev)
        bale.gen_values_dev(table, 2)
        for nl in nlogs:
            index = torch.empty(1 << nl, dtype=torch.int64, device=dev)
            bale.gen_uniform_dev(index, 1 << tl, 3)
            tgt = torch.empty_like(index)
            r = {"table_bytes": 8 << tl, "requests": 1 << nl}
            for mode in (0, 1):
                bale.tune_set("ig.mode", mode)
                r[f"mode{mode}_ms"] = round(_time(lambda: bale.ig_dev(tgt, index, table)), 4)
            rows.append(r)
            del index, tgt
        del table
    bale.tune_set("ig.mode", -1)
    torch.cuda.empty_cache()
    big_n = [r for r in rows if r["requests"] == max(x["requests"] for x in rows)]
    tb = _crossover(big_n, "table_bytes", "mode1_ms", "mode0_ms")
    knobs = {}
    if tb is not None:
        knobs["ig.part_min_table_bytes"] = tb - 1
        at_tb = [r for r in rows if r["table_bytes"] >= tb]
        nmin = _crossover(at_tb, "requests", "mode1_ms", "mode0_ms")
        if nmin is not None:
            knobs["ig.part_min_requests"] = nmin
    return knobs, rows


def tune_histo(quick: bool) -> tuple[dict, list]:
    import torch

    import bale_old_gb300 as bale

    dev = torch.device("cuda:0")
    rows = []
    tlogs = (22, 23, 24, 25, 26) if quick else (21, 22, 23, 24, 25, 26, 27)
    nlogs = (24, 26) if quick else (22, 24, 26)
    index = torch.empty(1 << max(nlogs), dtype=torch.int64, device=dev)
    for tl in tlogs:
        counts = torch.zeros(1 << tl, dtype=torch.int64, device=dev)
        for nl in nlogs:
            idx = index[: 1 << nl]
            bale.gen_uniform_dev(idx, 1 << tl, 4)
            r = {"table_bytes": 8 << tl, "updates": 1 << nl}
            for mode in (2, 3):
                bale.tune_set("histo.mode", mode)
                r[f"mode{mode}_ms"] = round(_time(lambda: bale.histo_dev(counts, idx)), 4)
            rows.append(r)
        del counts
    bale.tune_set("histo.mode", -1)
    del index
    torch.cuda.empty_cache()
    knobs = {}
    big_n = [r for r in rows if r["updates"] == max(x["updates"] for x in rows)]
    tb = _crossover(big_n, "table_bytes", "mode3_ms", "mode2_ms")
    if tb is not None:
        knobs["histo.part_min_table_bytes"] = tb - 1
        at_tb = [r for r in rows if r["table_bytes"] >= tb]
        nmin = _crossover(at_tb, "updates", "mode3_ms", "mode2_ms")
        if nmin is not None:
            knobs["histo.part_min_updates"] = nmin
    return knobs, rows


def work_model(offset, nonzero) -> tuple[int, int]:
    """The reference's work model of alg 0 (apps/triangle_src/triangle.upc:
    325-369): pulls = sum over nonzeros (i,j) of d_j; pushes = sum over rows
    of C(d, 2)."""
    import numpy as np

    deg = np.diff(offset)
    pushes = int((deg * (deg - 1) // 2).sum())
    pulls = int(deg[nonzero].sum()) if nonzero.size else 0
    return pulls, pushes


def fit_tri_rule(rows: list[dict]) -> tuple[int, int]:
    """Thresholds (pull_pct, push_per_nnz) of the rule "wedges when pulls >=
    pull_pct % of the pushes or pushes >= push_per_nnz per nonzero" that
    minimise the summed time of the chosen path over the measured graphs;
    ties go to the larger thresholds.  rows: pulls, pushes, nnz, wedge_ms,
    hybrid_ms."""
    ratios = sorted({r["pulls"] * 100.0 / max(r["pushes"], 1) for r in rows})
    per_nnz = sorted({r["pushes"] / max(r["nnz"], 1) for r in rows})
    pct_cands = sorted({int(x) + 1 for x in ratios} | {int((a + b) / 2) for a, b in zip(ratios, ratios[1:])} | {150})
    ppn_cands = sorted({int(x) + 1 for x in per_nnz} | {int((a + b) / 2) for a, b in zip(per_nnz, per_nnz[1:])}
                       | {128, 1 << 30})

    def cost(pct, ppn):
        t = 0.0
        for r in rows:
            wedge = r["pushes"] == 0 or r["pulls"] * 100 >= pct * r["pushes"] or r["pushes"] >= ppn * r["nnz"]
            t += r["wedge_ms"] if wedge else r["hybrid_ms"]
        return t

    best = min(((cost(p, q), -p, -q) for p in pct_cands for q in ppn_cands))
    return -best[1], -best[2]


def tune_tri(quick: bool) -> tuple[dict, list]:
    import torch

    import bale_old_gb300 as bale

    dev = torch.device("cuda:0")
    graphs = [("rmat", s) for s in ((18, 20) if quick else (16, 18, 20, 21))]
    graphs += [("er", (lg, d)) for lg, d in (((19, 32), (20, 32), (18, 128)) if quick else
                                              ((19, 32), (20, 32), (21, 32), (18, 64), (18, 128), (20, 64)))]
    graphs += [("kron", (3, 4, 5, 9, 16, 25))]
    rows = []
    bale.tune_set("tri.choose_min_nnz", 1)  # the choice is what is being fitted
    for kind, g in graphs:
        if kind == "rmat":
            L = bale.gen_rmat(g, 16, 0.57, 0.19, 0.19, 6)
        elif kind == "er":
            L = bale.gen_erdos_renyi(1 << g[0], g[1] / (1 << g[0]), 7)
        else:
            L = bale.gen_kronecker(1, list(g))
        off, col = torch.from_numpy(L.offset).to(dev), torch.from_numpy(L.nonzero).to(dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        pulls, pushes = work_model(L.offset, L.nonzero)
        r = {"graph": f"{kind} {g}", "nnz": L.nnz, "pulls": pulls, "pushes": pushes}
        for mode, key in ((2, "wedge_ms"), (1, "hybrid_ms")):
            bale.tune_set("tri.mode", mode)
            r[key] = round(_time(lambda: bale.triangle_dev(off, col, cnt), reps=3), 4)
        rows.append(r)
        del off, col
    bale.tune_set("tri.mode", -1)
    bale.tune_set("tri.choose_min_nnz", -1)
    torch.cuda.empty_cache()
    pct, ppn = fit_tri_rule(rows)
    return {"tri.wedge_pull_pct": pct, "tri.wedge_push_per_nnz": ppn}, rows


def _batch_time(inst, reps: int) -> float:
    from .mix import as_batch

    with as_batch(inst) as b:
        return _time(b.run, reps=reps, warmup=1)


def tune_batch(quick: bool) -> tuple[dict, list]:
    import torch

    import bale_old_gb300 as bale

    from .mix import MIX_FULL, MIX_SMALL, build_mix

    dev = torch.device("cuda:0")
    rows, knobs = [], {}
    small = build_mix(dev, MIX_SMALL)
    tiles = (1 << 15, 1 << 16, 1 << 17, 1 << 18)
    plan = [("batch.histo_tile", tiles), ("batch.histo_l2_tile", tiles), ("batch.ig_tile", tiles),
            ("batch.tri_light_rows", (1 << 13, 1 << 15, 1 << 17)), ("batch.tri_heavy_rows", (1, 4))]
    for cls in ("small", "medium"):
        for base, cands in plan:
            name = f"{base}.{cls}"
            res = {}
            for v in cands:
                bale.tune_set(name, v)
                res[v] = _batch_time(small, 3)
            best = min(res, key=res.get)
            bale.tune_set(name, best)
            knobs[name] = best
            rows.append({"mix": "small", "knob": name, "ms": {str(k): round(v, 4) for k, v in res.items()},
                         "best": best})
    del small
    torch.cuda.empty_cache()
    if not quick:
        full = build_mix(dev, MIX_FULL)
        for name, cands in (("batch.standalone_min_edges", (1 << 14, 1 << 16, 1 << 18, 1 << 19, 1 << 20, 1 << 21)),
                            ("batch.standalone_min", (1 << 19, 1 << 20, 1 << 21, 1 << 22, 1 << 23)),
                            ("batch.streams", (4, 8, 16))):
            res = {}
            for v in cands:
                bale.tune_set(name, v)
                res[v] = _batch_time(full, 2)
            best = min(res, key=res.get)
            bale.tune_set(name, best)
            knobs[name] = best
            rows.append({"mix": "full", "knob": name, "ms": {str(k): round(v, 4) for k, v in res.items()},
                         "best": best})
        del full
        torch.cuda.empty_cache()
    return knobs, rows


def save(knobs: dict, report: dict, out: Path) -> None:
    out.parent.mkdir(parents=True, exist_ok=True)
    lines = [f"# written by python -m bale_old_gb300.autotune on {report.get('gpu', '?')}",
             "# name value  (bale_tune_set knobs; -1 restores the built-in rule)"]
    lines += [f"{k} {int(v)}" for k, v in sorted(knobs.items())]
    out.write_text("\n".join(lines) + "\n")
    out.with_name(out.stem + "_report.json").write_text(json.dumps(report, indent=1) + "\n")


def load(path: Path | str = DEFAULT_OUT) -> int:
    """Apply a tuning file; returns the number of knobs applied (0 if absent)."""
    from . import _lib

    p = Path(path)
    if not p.exists():
        return 0
    return max(0, int(_lib.bale_tune_load(str(p).encode())))


def main(argv=None) -> int:
    import torch

    import bale_old_gb300 as bale

    ap = argparse.ArgumentParser()
    ap.add_argument("--out", type=Path, default=DEFAULT_OUT)
    ap.add_argument("--quick", action="store_true", help="fewer sizes; skips the full-mix thresholds")
    ap.add_argument("--only", choices=["ig", "histo", "tri", "batch"], help="tune one part, keep the file's others")
    a = ap.parse_args(argv)
    if not torch.cuda.is_available():
        print("autotune needs a CUDA device", file=sys.stderr)
        return 1
    for name in bale.tune_knobs():  # measure from the built-in rules
        bale.tune_set(name, -1)
    t0 = time.time()
    report = {"gpu": torch.cuda.get_device_name(0)}
    knobs = {}
    if a.only and a.out.exists():  # keep the other parts' knobs and report
        for line in a.out.read_text().splitlines():
            f = line.split()
            if len(f) == 2 and not line.startswith("#"):
                knobs[f[0]] = int(f[1])
        rep = a.out.with_name(a.out.stem + "_report.json")
        if rep.exists():
            report.update({k: v for k, v in json.loads(rep.read_text()).items() if k not in ("gpu", "seconds")})
    for part, fn in (("ig", tune_ig), ("histo", tune_histo), ("tri", tune_tri), ("batch", tune_batch)):
        if a.only and part != a.only:
            continue
        k, rows = fn(a.quick)
        knobs.update(k)
        report[part] = {"chosen": k, "measurements": rows}
        print(part, k, flush=True)
    report["seconds"] = round(time.time() - t0, 1)
    save(knobs, report, a.out)
    print(f"wrote {a.out} ({len(knobs)} knobs) in {report['seconds']} s")
    return 0


if __name__ == "__main__":
    sys.exit(main())
