"""The product (bale_old_gb300 and libbale_gb300.so) never imports, links or
loads the oracle or the reference build under oracle/: those are test
infrastructure, used by tests/, the smoke entry and the bench's CPU baseline
only.  Checked statically over the sources and at run time in a fresh
process."""
from __future__ import annotations

import re
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[1]
PKG = ROOT / "bale_old_gb300"


def test_product_sources_do_not_reference_the_oracle():
    pat = re.compile(r"(^|\s)(import|from)\s+oracle\b|libbale_oracle|libbale_ref|oracle/_ref|oracle/_build|"
                     r"pyoracle|bale_oracle\.h", re.M)
    files = [p for pat_ in ("*.py", "*.cu", "*.cuh", "*.c", "*.h") for p in PKG.rglob(pat_)]
    files += list((ROOT / "include").glob("*.h"))
    hits = [str(p.relative_to(ROOT)) for p in files if "_build" not in p.parts and pat.search(p.read_text())]
    assert not hits, hits


def test_build_recipe_links_only_the_package_sources():
    text = (PKG / "build.py").read_text()
    assert "oracle" not in text


def test_importing_and_using_the_package_loads_no_oracle_code():
    code = r"""
import sys
import bale_old_gb300 as bale
x = bale.gen_uniform(1000, 77, 5)
L = bale.gen_rmat(8, 4, 0.57, 0.19, 0.19, 3)
assert x.size == 1000 and L.nnz > 0
mods = [m for m in sys.modules if m == "oracle" or m.startswith("oracle.")]
maps = open("/proc/self/maps").read()
libs = sorted({line.split()[-1] for line in maps.splitlines() if line.split()[-1].endswith(".so")})
bad = [l for l in libs if "/oracle/" in l or "bale_oracle" in l or "bale_ref" in l]
ours = [l for l in libs if l.endswith("libbale_gb300.so")]
print("mods", mods, "bad", bad, "ours", len(ours))
assert not mods and not bad and len(ours) == 1
"""
    r = subprocess.run([sys.executable, "-c", code], cwd=ROOT, capture_output=True, text=True, timeout=300)
    assert r.returncode == 0, r.stdout + r.stderr
