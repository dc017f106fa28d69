"""The uneven instance mixes of the batched configuration.

MIX_FULL is the 512-instance mix: 256 histograms (tables log-uniform in
[1K, 16M] counters, updates log-uniform in [10K, 64M]), 192 gathers (tables
[1K, 64M], requests [10K, 128M]) and 64 R-MAT triangle counts (scales 10..20,
edge factor 16, quadrants (0.57, 0.19, 0.19, 0.05)).  MIX_SMALL keeps the
same shape with every size capped near 2^20, where per-launch costs dominate.
Instance k is seeded with seed + k; index arrays and tables are generated
directly on the device (bit-identical to the host generators), graphs on
the host.
"""
from __future__ import annotations

import numpy as np

MIX_FULL = {"histo_t": (1_000, 16 << 20), "histo_n": (10_000, 64 << 20), "ig_t": (1_000, 64 << 20),
            "ig_n": (10_000, 128 << 20), "scales": (10, 20)}
MIX_SMALL = {"histo_t": (1_000, 1 << 20), "histo_n": (10_000, 1 << 20), "ig_t": (1_000, 4 << 20),
             "ig_n": (10_000, 1 << 20), "scales": (8, 14)}


def build_mix(dev, spec=None, seed: int = 1000, counts=(256, 192, 64)):
    """Returns [(kind, out, a, b, items)]: kind "histo" (out counts, a index),
    "ig" (out tgt, a index, b table) or "tri" (out count, a offsets,
    b nonzeros); items = updates, requests or nonzeros."""
    import torch

    import bale_old_gb300 as bale

    spec = spec or MIX_FULL
    rng = np.random.default_rng(seed)
    logu = lambda lo, hi: int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))  # noqa: E731
    inst = []
    k = 0
    for _ in range(counts[0]):
        t, n = logu(*spec["histo_t"]), logu(*spec["histo_n"])
        idx = torch.empty(n, dtype=torch.int64, device=dev)
        bale.gen_uniform_dev(idx, t, seed + k)
        inst.append(("histo", torch.zeros(t, dtype=torch.int64, device=dev), idx, None, n))
        k += 1
    for _ in range(counts[1]):
        t, n = logu(*spec["ig_t"]), logu(*spec["ig_n"])
        idx = torch.empty(n, dtype=torch.int64, device=dev)
        tab = torch.empty(t, dtype=torch.int64, device=dev)
        bale.gen_uniform_dev(idx, t, seed + k)
        bale.gen_values_dev(tab, seed + k + 1_000_000)
        inst.append(("ig", torch.empty(n, dtype=torch.int64, device=dev), idx, tab, n))
        k += 1
    for _ in range(counts[2]):
        sc = int(rng.integers(spec["scales"][0], spec["scales"][1] + 1))
        L = bale.gen_rmat(sc, 16, 0.57, 0.19, 0.19, seed + k)
        inst.append(("tri", torch.zeros(1, dtype=torch.int64, device=dev), torch.from_numpy(L.offset).to(dev),
                     torch.from_numpy(L.nonzero).to(dev), L.nnz))
        k += 1
    torch.cuda.synchronize()
    return inst


def run_plain(inst) -> None:
    """Every instance through its own device entry point, back to back on one stream."""
    import bale_old_gb300 as bale

    for kind, out, a, b, _ in inst:
        if kind == "histo":
            bale.histo_dev(out, a)
        elif kind == "ig":
            bale.ig_dev(out, a, b)
        else:
            bale.triangle_dev(a, b, out)


def as_batch(inst):
    """A Batch over the mix's instances."""
    from . import batch as bb

    return bb.Batch([bb.histo(x[1], x[2]) if x[0] == "histo" else bb.ig(x[1], x[2], x[3]) if x[0] == "ig"
                     else bb.triangles(x[2], x[3], x[1]) for x in inst])
