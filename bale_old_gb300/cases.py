"""Single-configuration runs of each kernel, for profilers and quick timing.

    python -m bale_old_gb300.cases ig --table-log2 26 --requests-log2 25 [--mode 1]
    python -m bale_old_gb300.cases histo --counters 1000000 --updates 10000000 [--mode 2]
    python -m bale_old_gb300.cases triangles --scale 20 [--mode 1]
    python -m bale_old_gb300.cases randperm --elements-log2 26 [--buf-cnt 1024]
    python -m bale_old_gb300.cases graph --scale 20

Each builds its seeded input, moves it to cuda:0 and runs the device entry
point --reps times (default 2), then prints one line.  Knob values given on
the command line (--mode) pin the kernel variant.
"""
from __future__ import annotations

import argparse
import sys


def main(argv=None) -> int:
    import torch

    import bale_old_gb300 as bale

    ap = argparse.ArgumentParser()
    ap.add_argument("kernel", choices=["ig", "histo", "triangles", "randperm", "graph"])
    ap.add_argument("--table-log2", type=int, default=26)
    ap.add_argument("--requests-log2", type=int, default=25)
    ap.add_argument("--zipf", action="store_true")
    ap.add_argument("--counters", type=int, default=1_000_000)
    ap.add_argument("--updates", type=int, default=10_000_000)
    ap.add_argument("--scale", type=int, default=20)
    ap.add_argument("--elements-log2", type=int, default=26)
    ap.add_argument("--buf-cnt", type=int, default=0, help="randperm: 0 = rand_permp_agi, else rand_permp_exstack")
    ap.add_argument("--mode", type=int, default=-1)
    ap.add_argument("--reps", type=int, default=2)
    a = ap.parse_args(argv)
    dev = torch.device("cuda:0")
    if a.kernel == "ig":
        bale.tune_set("ig.mode", a.mode)
        t = 1 << a.table_log2
        table = torch.from_numpy(bale.gen_values(t, 2)).to(dev)
        idx = bale.gen_zipf(1 << a.requests_log2, t, 1.1, 4, 5) if a.zipf else bale.gen_uniform(1 << a.requests_log2, t, 3)
        index = torch.from_numpy(idx).to(dev)
        tgt = torch.empty_like(index)
        for _ in range(a.reps):
            bale.ig_dev(tgt, index, table)
    elif a.kernel == "histo":
        bale.tune_set("histo.mode", a.mode)
        index = torch.from_numpy(bale.gen_uniform(a.updates, a.counters, 1)).to(dev)
        counts = torch.zeros(a.counters, dtype=torch.int64, device=dev)
        for _ in range(a.reps):
            bale.histo_dev(counts, index)
    elif a.kernel == "randperm":
        n = 1 << a.elements_log2
        for _ in range(a.reps):
            if a.buf_cnt:
                bale.rand_perm_exstack_dev(n, 31, a.buf_cnt, device=dev)
            else:
                bale.rand_perm_dev(n, 31, device=dev)
    elif a.kernel == "graph":
        for _ in range(a.reps):
            bale.gen_rmat_dev(a.scale, 16, 0.57, 0.19, 0.19, 6, device=dev)
    else:
        bale.tune_set("tri.mode", a.mode)
        L = bale.gen_rmat(a.scale, 16, 0.57, 0.19, 0.19, 6)
        off = torch.from_numpy(L.offset).to(dev)
        col = torch.from_numpy(L.nonzero).to(dev)
        cnt = torch.zeros(1, dtype=torch.int64, device=dev)
        for _ in range(a.reps):
            bale.triangle_dev(off, col, cnt)
    torch.cuda.synchronize()
    print(f"{a.kernel}: {a.reps} runs done")
    return 0


if __name__ == "__main__":
    sys.exit(main())
