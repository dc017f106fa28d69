"""The tuning knob table of libbale_gb300 (bale_tune_set/get/load) and the
autotuner's file format, on the host: no GPU, no compute calls.  Every knob
selects among kernel variants with identical results, so these tests check
only that values land where they are named and that bad input is refused."""
from __future__ import annotations

from pathlib import Path

import pytest

from bale_old_gb300 import autotune


@pytest.fixture()
def knobs(bale):
    """The knob values at entry (the committed tuning file applied at import),
    put back afterwards so that later tests see the same state."""
    before = bale.tune_knobs()
    yield before
    for k, v in before.items():
        bale.tune_set(k, v)
    assert bale.tune_knobs() == before


def test_knob_names_are_unique_and_dotted(bale, knobs):
    names = list(knobs)
    assert len(names) == len(set(names)) > 0
    assert all("." in n and n == n.strip() for n in names)


def test_set_get_round_trip_and_automatic(bale, knobs):
    for name in knobs:
        bale.tune_set(name, 12345)
        assert bale.tune_get(name) == 12345
        bale.tune_set(name, -1)  # the built-in size rule
        assert bale.tune_get(name) == -1


def test_unknown_knob_is_refused(bale, knobs):
    with pytest.raises(bale.BaleError, match="unknown tuning knob"):
        bale.tune_set("ig.no_such_knob", 1)
    with pytest.raises(bale.BaleError, match="unknown tuning knob"):
        bale.tune_get("ig.no_such_knob")
    assert bale.tune_knobs() == knobs


def test_committed_tuning_file_names_only_library_knobs(bale, knobs):
    path = autotune.DEFAULT_OUT
    assert path.exists()
    seen = {}
    for line in path.read_text().splitlines():
        if not line or line.startswith("#"):
            continue
        name, value = line.split()
        seen[name] = int(value)
    assert seen and set(seen) <= set(knobs), set(seen) - set(knobs)
    # applied at import: the library holds the file's values
    assert all(knobs[k] == v for k, v in seen.items())


def test_save_then_load_applies_the_file(bale, knobs, tmp_path: Path):
    names = sorted(knobs)[:3]
    chosen = {n: 1000 + i for i, n in enumerate(names)}
    out = tmp_path / "t.tune"
    autotune.save(chosen, {"gpu": "test"}, out)
    assert (tmp_path / "t_report.json").exists()
    for n in names:
        bale.tune_set(n, -1)
    assert autotune.load(out) == len(names)
    assert {n: bale.tune_get(n) for n in names} == chosen


def test_load_skips_comments_unknown_and_malformed_lines(bale, knobs, tmp_path: Path):
    name = sorted(knobs)[0]
    f = tmp_path / "mixed.tune"
    f.write_text(f"# comment {name} 7\n"
                 "no.such.knob 5\n"
                 f"{name}\n"            # no value
                 "\n"
                 f"{name} 4242\n")
    assert autotune.load(f) == 1
    assert bale.tune_get(name) == 4242


def test_load_of_a_missing_file(bale, knobs, tmp_path: Path):
    assert autotune.load(tmp_path / "absent.tune") == 0
    from bale_old_gb300 import _lib

    assert _lib.bale_tune_load(str(tmp_path / "absent.tune").encode()) == -1
    assert "cannot open" in bale._last_error()
    assert bale.tune_knobs() == knobs


def test_tri_rule_fit_picks_the_faster_path():
    """The intersection-strategy fit: graphs with hubs (pulls well above the
    pushes) are faster by wedges, graphs without by the hybrid; the fitted
    thresholds send each measured graph to its faster path."""
    rows = [
        {"graph": "rmat", "nnz": 100, "pulls": 400, "pushes": 100, "wedge_ms": 1.0, "hybrid_ms": 3.0},
        {"graph": "rmat2", "nnz": 100, "pulls": 210, "pushes": 100, "wedge_ms": 1.0, "hybrid_ms": 2.0},
        {"graph": "er", "nnz": 100, "pulls": 100, "pushes": 100, "wedge_ms": 1.2, "hybrid_ms": 1.0},
        {"graph": "kron", "nnz": 10, "pulls": 30, "pushes": 3000, "wedge_ms": 0.5, "hybrid_ms": 0.7},
    ]
    pct, ppn = autotune.fit_tri_rule(rows)
    for r in rows:
        wedge = r["pulls"] * 100 >= pct * r["pushes"] or r["pushes"] >= ppn * r["nnz"]
        assert wedge == (r["wedge_ms"] < r["hybrid_ms"]), (r, pct, ppn)


def test_work_model_matches_the_oracle(oracle):
    """pulls and pushes as the autotuner computes them equal the oracle's
    restatement of the reference app's work model."""
    import numpy as np

    import bale_old_gb300 as bale

    L = bale.gen_rmat(10, 16, 0.57, 0.19, 0.19, 3)
    assert autotune.work_model(L.offset, L.nonzero) == oracle.triangle_work(L.offset, L.nonzero)
    assert autotune.work_model(np.zeros(1, np.int64), np.zeros(0, np.int64)) == (0, 0)
