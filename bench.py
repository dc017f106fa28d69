"""Benchmark of the GB300 irregular-access core.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload ig|ig_zipf|histo|triangles|graph|spmat|
                                batch|batch_small|serve] [--only]

Prints one JSON line (rank 0).  A "step" is one pass of a workload's kernels
over its whole synthetic input (seeded SplitMix64 streams; R-MAT graph):

* ig        (headline): 2^26-entry int64 table of random values, 2^28
            uniform requests -> GUP/s (10^9 requests/s);
* ig_zipf   : same table, requests Zipf(1.1) over a keyed permutation;
* histo     : 10^7 uniform updates into 10^6 int64 counters -> GUP/s;
* triangles : R-MAT scale 22, edge factor 16, (0.57,0.19,0.19,0.05),
            symmetrised, degree-ordered strictly lower L -> edges/s (nnz(L)/s),
            with an Erdos-Renyi 2^20 sub-result (default and merge modes);
* graph     : the same R-MAT graph generated and built into the
            degree-ordered lower CSR on the device -> G input edges/s;
* spmat     : transpose and permutation of that matrix, random
            permutations of 2^26 (agi and exstack), MatrixMarket read and
            binary dataset write/read -> G nonzeros/s (transpose headline);
* batch     : the uneven 512-instance mix (256 histo, 192 ig, 64 R-MAT
            triangle instances) in one CUDA graph, against the same instances
            launched one by one -> G items/s (updates + requests + edges);
* batch_small: the same kinds with small instances (launch-bound mix);
* serve     : Poisson arrivals against resident tables, counters and graphs,
            rates swept to saturation -> G items/s with p50/p99 latency.

The headline workload fills the top-level keys; unless --only is given the
others are measured in the same run and reported under "workloads".

``value``: device time from CUDA events on the launching stream, inputs
resident in HBM, W warm-up steps then K timed steps.  The ig index/output
streams (2 GiB each) and the triangle CSR (513 MiB) exceed L2; for histo,
whose inputs fit in L2, and for triangles too, a 256 MiB buffer is
rewritten between timed steps (outside the events).
``e2e``: the same metric through the reference-facing C ABI (ig_agi,
histo_agi, triangle_agi) with pinned host buffers, copies inside the timed
region.  ``cpu_baseline``: the oracle restatement of the reference's AGI loop
on all host threads, on a bounded sample.  ``--impl reference`` times that
CPU implementation alone.

Under torchrun every rank runs its own copy on its own GPU (weak scaling,
replicas: no data-path collective); rank 0 reports the job total over the
max of the ranks' times.
"""
from __future__ import annotations

import argparse
import json
import os
import shutil
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

HBM_FALLBACK_GBS = 6800.0
IG_TABLE = 1 << 26
IG_REQUESTS = 1 << 28
HISTO_COUNTS = 1_000_000
HISTO_UPDATES = 10_000_000
TRI_SCALE = 22
FLUSH_BYTES = 256 << 20


# ---------------------------------------------------------------------------
# distributed plumbing (torchrun sets RANK/WORLD_SIZE/LOCAL_RANK)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as dist

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            dist.init_process_group(backend=backend)
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def max(self, x: float) -> float:
        """Max of x over ranks (the job's time is its slowest rank's)."""
        if not self.pg:
            return x
        import torch

        dev = "cuda" if self.pg.get_backend() == "nccl" else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.pg.all_reduce(t, op=self.pg.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def job_rate(units_per_rank: int, seconds_max: float, world: int) -> float:
    """Whole-job throughput: every rank processed units_per_rank in at most
    seconds_max (the max over ranks)."""
    return world * units_per_rank / seconds_max


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def committed_traffic() -> dict:
    """Per-step DRAM bytes from the committed ncu summaries (profiles/)."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


# ---------------------------------------------------------------------------
# clocks sampled while a timed region runs
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
    NAMES = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.path = None

    def __enter__(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}",
                 "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        except (OSError, ValueError):
            self.proc = None
        return self

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()
            self.fh.close()

    def summary(self) -> dict:
        if not self.path or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, smax, reasons = [], None, set()
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(self.NAMES, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# timing helpers
# ---------------------------------------------------------------------------
def time_device(fn, steps: int, warmup: int, between=None) -> float:
    """Average CUDA-event time (ms) of fn() per step on the current stream."""
    import torch

    stream = torch.cuda.current_stream()
    for _ in range(warmup):
        if between:
            between()
        fn()
    torch.cuda.synchronize()
    total = 0.0
    for _ in range(steps):
        if between:
            between()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        total += a.elapsed_time(b)
    return total / steps


def time_host(fn, steps: int, warmup: int) -> float:
    """Average wall seconds of a synchronous call."""
    for _ in range(warmup):
        fn()
    t0 = time.perf_counter()
    for _ in range(steps):
        fn()
    return (time.perf_counter() - t0) / steps


def time_host_calls(fn, steps: int, warmup: int) -> tuple[float, dict]:
    """Average wall seconds of a synchronous call, and the spread of the
    single calls (median, min, max, in ms)."""
    for _ in range(warmup):
        fn()
    each = []
    for _ in range(steps):
        t0 = time.perf_counter()
        fn()
        each.append(time.perf_counter() - t0)
    srt = sorted(each)
    spread = {"calls": len(each), "median_ms": round(srt[len(srt) // 2] * 1e3, 3), "min_ms": round(srt[0] * 1e3, 3),
              "max_ms": round(srt[-1] * 1e3, 3)}
    return sum(each) / len(each), spread


# ---------------------------------------------------------------------------
# workloads: each returns a dict with value/roofline/e2e/... for one rank
# ---------------------------------------------------------------------------
def ig_inputs(bale, zipf: bool):
    table = bale.gen_values(IG_TABLE, 2)
    index = bale.gen_zipf(IG_REQUESTS, IG_TABLE, 1.1, 4, 5) if zipf else bale.gen_uniform(IG_REQUESTS, IG_TABLE, 3)
    return index, table


def run_ig(ctx, zipf: bool) -> dict:
    import torch

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    index_h, table_h = ig_inputs(bale, zipf)
    n = index_h.size
    index = torch.from_numpy(index_h).to(dev)
    table = torch.from_numpy(table_h).to(dev)
    tgt = torch.empty_like(index)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    fn = lambda: bale.ig_dev(tgt, index, table, bad=bad)  # noqa: E731
    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        ms = time_device(fn, args.steps, args.warmup)
    ms_max = ctx["dist"].max(ms)
    torch.cuda.synchronize()
    s = slice(0, 1 << 22)
    ok = bool(np.array_equal(tgt[s].cpu().numpy(), table_h[index_h[s]])) and int(bad.item()) == 0
    part = table_h.size * 8 > (96 << 20) and n >= (1 << 20)
    # tables beyond L2: the skew test, then partition + gather + unpermute
    # and the direct gather, of which one side returns at once on the device
    kernels = 5 if part else 1
    algo = 48 * n  # 8 B index + 32 B table sector + 8 B output per request
    wl = "ig_zipf" if zipf else "ig"
    out = {
        "metric": "GUP/s index gather (10^9 requests/s)",
        "value": round(job_rate(n, ms_max / 1e3, ctx["dist"].world) / 1e9, 4), "unit": "GUP/s",
        "ms_per_step": round(ms_max, 4), "parity_sample_ok": ok,
        "roofline": roofline(ctx, wl, algo, ms / 1e3,
                             "ig: skew test, then region-partitioned gather (partition + gather + unpermute) "
                             "or, for a skewed stream, the direct gather" if part else "ig_gather_kernel"),
        "clocks": clocks.summary(),
        "gpu_launches": kernels * args.steps,
        "config": {"workload": f"ig {'Zipf(1.1) over a keyed permutation' if zipf else 'uniform'}: "
                               "2^26-entry int64 table, 2^28 int64 requests",
                   "table_entries": IG_TABLE, "requests": n,
                   "l2": "index and output streams (2 GiB each) exceed L2; no flush"},
    }
    del index, table, tgt
    if not zipf:
        pin_idx = torch.from_numpy(index_h).pin_memory()
        pin_tab = torch.from_numpy(table_h).pin_memory()
        pin_tgt = torch.empty(n, dtype=torch.int64).pin_memory()
        torch.cuda.empty_cache()
        call = lambda: bale.ig_agi(pin_tgt.numpy(), pin_idx.numpy(), pin_tab.numpy())  # noqa: E731
        ctx["dist"].barrier()
        e2e_s, e2e_spread = time_host_calls(call, args.steps, min(args.warmup, 3))
        e2e_s = ctx["dist"].max(e2e_s)
        out["e2e"] = {"value": round(job_rate(n, e2e_s, ctx["dist"].world) / 1e9, 4), "unit": "GUP/s",
                      "ms_per_step": round(e2e_s * 1e3, 3), "h2d_bytes_per_step": 8 * n + 8 * IG_TABLE,
                      "d2h_bytes_per_step": 8 * n, "path": "ig_agi C ABI, pinned host buffers",
                      "parity_sample_ok": bool(np.array_equal(pin_tgt.numpy()[s], table_h[index_h[s]])),
                      "per_call": e2e_spread,
                      "copy_bound": "the host link measured 211 GB/s H2D, 193 GB/s D2H, 343 GB/s both ways at once "
                                    "(one or eight copy streams alike, and a kernel reading mapped host memory): "
                                    "4.83 GB per call needs >= 14.1 ms"}
        if ctx["cpu"]:
            sample = np.ascontiguousarray(index_h[: 1 << 25])

            def cpu_leg():
                out["cpu_baseline"] = cpu_ig(sample, table_h, ctx["budget"])
                out["cpu_baseline"]["one_pe"] = one_pe_legs("ig", 2.0, index=sample[: 1 << 23], table=table_h)

            ctx["later"].append(cpu_leg)
    return out


def run_histo(ctx) -> dict:
    import torch

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    index_h = bale.gen_uniform(HISTO_UPDATES, HISTO_COUNTS, 1)
    want = np.bincount(index_h, minlength=HISTO_COUNTS)
    index = torch.from_numpy(index_h).to(dev)
    counts = torch.zeros(HISTO_COUNTS, dtype=torch.int64, device=dev)
    bad = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    fn = lambda: bale.histo_dev(counts, index, bad=bad)  # noqa: E731
    between = lambda: flush.fill_(1)  # noqa: E731
    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        ms = time_device(fn, args.steps, args.warmup, between)
    ms_max = ctx["dist"].max(ms)
    torch.cuda.synchronize()
    reps = args.steps + args.warmup
    ok = bool(np.array_equal(counts.cpu().numpy(), reps * want)) and int(bad.item()) == 0
    n = HISTO_UPDATES
    algo = 72 * n  # 8 B index + 32 B sector read + 32 B write-back per update
    # the bound that binds here: the L2 reduction rate into the same 10^6
    # counters, measured live (the update without its index stream)
    probe = torch.zeros(HISTO_COUNTS, dtype=torch.int64, device=dev)
    red_ms = time_device(lambda: bale.l2_red_rate(probe, n), args.steps, args.warmup, between)
    red_peak = n / (red_ms / 1e3) / 1e9
    del probe
    achieved = n / (ms / 1e3) / 1e9
    dram = ctx["traffic"].get("histo", {}).get("dram_bytes_per_step")
    out = {"metric": "GUP/s histogram (10^9 updates/s)",
           "value": round(job_rate(n, ms_max / 1e3, ctx["dist"].world) / 1e9, 4), "unit": "GUP/s",
           "ms_per_step": round(ms_max, 4), "parity_ok": ok,
           # the 8 MB table is L2-resident, so the bound is the L2's rate of
           # 64-bit reductions, not HBM: one red.global.add.u64 per update
           "roofline": {"bound": "l2", "kernel": "histo_global_kernel (plain L2 reductions)",
                        "achieved": round(achieved, 2), "peak": round(red_peak, 2), "unit": "G reductions/s",
                        "frac": round(achieved / red_peak, 4),
                        "peak_source": "measured live in this run: bale_l2_red_rate issues the same "
                                       "red.global.add.u64 at hashed positions of the same 10^6 counters with no "
                                       "index stream (10^7 reductions), CUDA events",
                        "ncu_l2_throughput_pct": 70.6, "ncu_source": "profiles/histo_plain_l2_1e6_counters.md",
                        "traffic": dram, "dram_gbs": round(dram / (ms / 1e3) / 1e9, 1) if dram else None,
                        "hbm_model": {"algorithmic_bytes_per_step": algo,
                                      "achieved_gbs": round(algo / (ms / 1e3) / 1e9, 1),
                                      "note": "72 B/update (index + sector read + write-back) applies to tables "
                                              "beyond L2; it reads above HBM peak here"}},
           "clocks": clocks.summary(), "gpu_launches": args.steps,
           "config": {"workload": "histo: 10^7 uniform updates into 10^6 int64 counters",
                      "updates": n, "counters": HISTO_COUNTS,
                      "l2": "inputs fit in L2: a 256 MiB buffer is rewritten between steps"}}
    del index, counts, flush
    pin_idx = torch.from_numpy(index_h).pin_memory()
    pin_cnt = torch.zeros(HISTO_COUNTS, dtype=torch.int64).pin_memory()
    call = lambda: bale.histo_agi(pin_idx.numpy(), pin_cnt.numpy())  # noqa: E731
    ctx["dist"].barrier()
    e2e_s, e2e_spread = time_host_calls(call, args.steps, min(args.warmup, 3))
    e2e_s = ctx["dist"].max(e2e_s)
    calls = args.steps + min(args.warmup, 3)
    out["e2e"] = {"value": round(job_rate(n, e2e_s, ctx["dist"].world) / 1e9, 4), "unit": "GUP/s",
                  "ms_per_step": round(e2e_s * 1e3, 3), "h2d_bytes_per_step": 8 * n + 8 * HISTO_COUNTS,
                  "d2h_bytes_per_step": 8 * HISTO_COUNTS, "path": "histo_agi C ABI, pinned host buffers",
                  "parity_ok": bool(np.array_equal(pin_cnt.numpy(), calls * want)), "per_call": e2e_spread}
    if ctx["cpu"]:
        def cpu_leg():
            out["cpu_baseline"] = cpu_histo(index_h, ctx["budget"])
            out["cpu_baseline"]["one_pe"] = one_pe_legs("histo", 2.0, index=index_h)

        ctx["later"].append(cpu_leg)
    return out


def run_triangles(ctx) -> dict:
    import torch

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    t0 = time.perf_counter()
    L = bale.gen_rmat(TRI_SCALE, 16, 0.57, 0.19, 0.19, 6)
    gen_s = time.perf_counter() - t0
    n, nnz = L.numrows, L.nnz
    off = torch.from_numpy(L.offset).to(dev)
    col = torch.from_numpy(L.nonzero).to(dev)
    cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.int32, device=dev)
    fn = lambda: bale.triangle_dev(off, col, cnt)  # noqa: E731
    between = lambda: flush.fill_(1)  # noqa: E731
    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        ms = time_device(fn, args.steps, args.warmup, between)
    ms_max = ctx["dist"].max(ms)
    torch.cuda.synchronize()
    per_step = int(cnt.item()) // (args.steps + args.warmup)
    deg = np.diff(L.offset)
    pulls = int(deg[L.nonzero].sum())
    rowid = np.repeat(np.arange(n, dtype=np.int64), deg)
    pos = np.arange(nnz, dtype=np.int64) - L.offset[rowid]
    live = (pos > 0) & (deg[L.nonzero] > 0)
    pushes = int(pos[live].sum())
    records = int(live.sum())
    del rowid, pos, live
    # the dominant kernels alone: counting from a prepared graph (the wedge
    # probe kernel and the dense-pair kernel); their algorithmic bytes are the
    # push model's -- every probed prefix element read once as a u32 (the
    # dense pairs counted as the pushes they replace), the 8-byte prefix
    # records, and rows j read twice (set and clear) as u32
    wedge_bytes = 4 * pushes + 8 * records + 8 * nnz
    with bale.TrianglePrepared(off, col) as g:
        cnt2 = torch.zeros(1, dtype=torch.int64, device=dev)
        count_ms = time_device(lambda: g.count(cnt2), args.steps, args.warmup, between)
    count_ms = ctx["dist"].max(count_ms)
    out = {"metric": "edges/s triangle counting (nnz(L) per second)",
           "value": round(job_rate(nnz, ms_max / 1e3, ctx["dist"].world) / 1e9, 4), "unit": "Gedges/s",
           "ms_per_step": round(ms_max, 4), "triangles": per_step,
           # the count kernel is bound by instruction issue (ncu: issue active
           # ~69%, most probes served from L2), so its DRAM traffic (ncu,
           # per launch) over the live kernel time is a fraction of HBM, and
           # the push-model bytes (L2 + DRAM) are reported beside it
           "roofline": tri_roofline(ctx, wedge_bytes, count_ms / 1e3, ms_max),
           "roofline_pull_model": {"algorithmic_bytes_per_step": 8 * (n + 1) + 8 * nnz + 8 * pulls,
                                   "achieved_gbs": round((8 * (n + 1) + 8 * nnz + 8 * pulls) / ms_max * 1e-6, 1),
                                   "note": "the AGI loop's pull model (8 B per row-j element scanned); the "
                                           "wedge kernels probe 4x fewer elements, so this reads above 1"},
           "count_kernel_ms": round(count_ms, 4),
           # per call: the path choice, the wedge scan, row bitmaps, hub scan, 3
           # offset kernels, fill, probes, dense pairs, and the 4 hybrid kernels
           # that return at once when the wedges are chosen
           "clocks": clocks.summary(), "gpu_launches": 14 * args.steps,
           "config": {"workload": "triangles: R-MAT scale 22, edge factor 16, (0.57,0.19,0.19,0.05), "
                                  "symmetrised, deduplicated, degree-ordered strictly lower L",
                      "n": n, "nnz": nnz, "pulls": pulls, "pushes": pushes, "generate_s": round(gen_s, 2),
                      "l2": "the 513 MiB CSR exceeds L2; a 256 MiB buffer is also rewritten between steps"}}
    # the Erdos-Renyi variant (n = 2^20, average degree 32): the default path
    # (which picks the hybrid for a graph without hubs) and, for comparison,
    # the merge kernel (tri.mode 0)
    E = bale.gen_erdos_renyi(1 << 20, 32.0 / (1 << 20), 7)
    e_off, e_col = torch.from_numpy(E.offset).to(dev), torch.from_numpy(E.nonzero).to(dev)
    e_cnt = torch.zeros(1, dtype=torch.int64, device=dev)
    er = {}
    for mode, name in ((-1, "default"), (0, "merge")):
        bale.tune_set("tri.mode", mode)
        try:
            e_ms = ctx["dist"].max(time_device(lambda: bale.triangle_dev(e_off, e_col, e_cnt), args.steps,
                                               args.warmup, between))
        finally:
            bale.tune_set("tri.mode", -1)
        er[name] = {"value": round(job_rate(E.nnz, e_ms / 1e3, ctx["dist"].world) / 1e9, 4), "unit": "Gedges/s",
                    "ms_per_step": round(e_ms, 4)}
    e_cnt.zero_()
    bale.triangle_dev(e_off, e_col, e_cnt)
    torch.cuda.synchronize()
    out["erdos_renyi"] = {**er, "triangles": int(e_cnt.item()), "n": E.numrows, "nnz": E.nnz,
                          "how": "gen_erdos_renyi(2^20, 32/2^20, seed 7), lower triangle"}
    if ctx["cpu"]:  # the count against the oracle's AGI loop
        er_count = int(e_cnt.item())
        ctx["later"].append(lambda: out["erdos_renyi"].__setitem__(
            "parity_ok", _oracle().triangle_agi_mt(E.offset, E.nonzero) == er_count))
    del off, col, flush, e_off, e_col
    torch.cuda.empty_cache()
    res = {}

    def call():
        res["r"] = bale.triangle_agi(L)

    ctx["dist"].barrier()
    e2e_s, e2e_spread = time_host_calls(call, args.steps, min(args.warmup, 3))
    e2e_s = ctx["dist"].max(e2e_s)
    out["e2e"] = {"value": round(job_rate(nnz, e2e_s, ctx["dist"].world) / 1e9, 4), "unit": "Gedges/s",
                  "ms_per_step": round(e2e_s * 1e3, 3), "h2d_bytes_per_step": 8 * (n + 1) + 8 * nnz,
                  "d2h_bytes_per_step": 32, "path": "triangle_agi C ABI (numpy host buffers)",
                  "triangles": res["r"][0], "per_call": e2e_spread}
    if ctx["cpu"]:
        def cpu_leg():
            out["cpu_baseline"] = cpu_triangles(L, ctx["budget"])
            out["parity_ok"] = out["cpu_baseline"].get("triangles") == per_step == res["r"][0]
            out["cpu_baseline"]["one_pe"] = one_pe_legs("triangles", 0, offset=L.offset, nonzero=L.nonzero,
                                                         row_step=256)

        ctx["later"].append(cpu_leg)
    return out


def run_graph(ctx) -> dict:
    """Building the triangle input on the device: R-MAT scale 22 generated
    and turned into the degree-ordered strictly lower CSR (bale_gen_rmat_dev),
    against the same build on the host cores (bale_gen_rmat)."""
    import torch

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    S, ef = TRI_SCALE, 16
    m = ef << S
    holder = {}

    def fn():
        holder["g"] = bale.gen_rmat_dev(S, ef, 0.57, 0.19, 0.19, 6, device=dev)

    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        ms = time_device(fn, args.steps, args.warmup)
    ms_max = ctx["dist"].max(ms)
    off, col = holder.pop("g")
    nnz = col.numel()
    offs_h, col_h = off.cpu().numpy(), col.cpu().numpy()
    maxdeg = int((np.diff(offs_h) + np.bincount(col_h, minlength=1 << S)).max())
    p_edges, p_vert, p_lower = (2 * S + 1 + 7) // 8, (S + maxdeg.bit_length() + 7) // 8, (2 * S + 7) // 8
    # the dominant work: three LSD radix sorts, each reading its 8-byte keys
    # once for the digit counts of all passes, then every 8-bit pass reading
    # and writing each key once
    algo = 16 * (p_edges * m + p_vert * (1 << S) + p_lower * nnz) + 8 * (m + (1 << S) + nnz)
    # edge keys, per sort the digit counts + starts + one kernel per pass,
    # dedup (flag, 3 scan kernels, compact), max, vertex keys, labels, lower keys, CSR
    launches = 1 + (2 + p_edges) + 1 + 3 + 1 + 1 + 1 + (2 + p_vert) + 1 + 1 + (2 + p_lower) + 2
    out = {"metric": "G input edges/s building the degree-ordered lower CSR (R-MAT scale 22) on the device",
           "value": round(job_rate(m, ms_max / 1e3, ctx["dist"].world) / 1e9, 4), "unit": "G edges/s",
           "ms_per_step": round(ms_max, 3), "nnz": nnz,
           "roofline": roofline(ctx, "graph", algo, ms / 1e3,
                                "the build's radix sorts (one digit count per sort, one look-back scatter "
                                "per 8-bit pass) and graph steps",
                                note="algorithmic bytes: 16 B per key per 8-bit pass plus 8 B per key per sort "
                                     "over the m edge keys (45 bits), the 2^22 vertex keys and the nnz lower keys "
                                     "(44 bits); the generation, dedup and CSR steps are not counted"),
           "clocks": clocks.summary(), "gpu_launches": launches * args.steps,
           "config": {"workload": "R-MAT scale 22, edge factor 16, (0.57,0.19,0.19,0.05): 67,108,864 generated "
                                  "edges -> symmetrised, deduplicated, degree-ordered strictly lower CSR",
                      "edges": m, "nnz": nnz}}
    if ctx["cpu"]:
        t0 = time.perf_counter()
        L = bale.gen_rmat(S, ef, 0.57, 0.19, 0.19, 6)
        secs = time.perf_counter() - t0
        out["cpu_baseline"] = {"value": round(m / secs / 1e9, 5), "unit": "G edges/s",
                               "cores": _oracle().num_cpus(), "kind": "port",
                               "sample": "1 x the same build on the host (bale_gen_rmat: parallel radix sort, "
                                         "counting-sort relabel, per-row sort)", "seconds": round(secs, 2)}
        out["parity_ok"] = bool(np.array_equal(offs_h, L.offset) and np.array_equal(col_h, L.nonzero))
    del off, col
    torch.cuda.empty_cache()
    return out


def run_spmat(ctx) -> dict:
    """spmat's transpose, permutation and random permutations on the device
    (the R-MAT scale-22 lower matrix, 2^26-entry permutations), the
    MatrixMarket reader (scale-20 file) and the binary dataset writer and
    reader (scale 22), against the oracle's one-thread restatements of the
    reference at one PE."""
    import torch

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    S = TRI_SCALE
    off, col = bale.gen_rmat_dev(S, 16, 0.57, 0.19, 0.19, 6, device=dev)
    n, nnz = off.numel() - 1, col.numel()
    rinv = bale.rand_perm_dev(n, 11, device=dev)
    cinv = bale.rand_perm_dev(n, 12, device=dev)
    np_ = 1 << 26
    holder = {}
    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        t_ms = time_device(lambda: holder.__setitem__("t", bale.transpose_dev(off, col, n)), args.steps, args.warmup)
        p_ms = time_device(lambda: holder.__setitem__("p", bale.permute_dev(off, col, n, rinv, cinv)),
                           args.steps, args.warmup)
        r_ms = time_device(lambda: holder.__setitem__("r", bale.rand_perm_dev(np_, 31, device=dev)),
                           args.steps, args.warmup)
        x_ms = time_device(lambda: holder.__setitem__("x", bale.rand_perm_exstack_dev(np_, 31, 1024, device=dev)),
                           args.steps, args.warmup)
    t_ms, p_ms, r_ms, x_ms = (ctx["dist"].max(x) for x in (t_ms, p_ms, r_ms, x_ms))
    # MatrixMarket: the scale-20 lower matrix written with the reference's
    # format, read back (file read, upload, parse, sort) on the device
    import tempfile
    L20 = bale.gen_rmat(20, 16, 0.57, 0.19, 0.19, 6)
    mm_dir = tempfile.mkdtemp(prefix="bale_mm_")
    mm_path = f"{mm_dir}/rmat20.mm"
    bale.write_matrix_mm(L20, mm_path)
    mm_bytes = os.path.getsize(mm_path)
    mm_s = time_host(lambda: bale.read_matrix_mm_dev(mm_path, device=dev), args.steps, min(args.warmup, 2))
    mm_ok = True
    # binary dataset of the scale-22 lower matrix: written from and read back
    # into device memory (files in the page cache)
    ds_dir = f"{mm_dir}/ds22"
    ds_steps = min(args.steps, 3)
    dw_s = time_host(lambda: bale.write_sparse_matrix_dev(ds_dir, off, col, n), ds_steps, 1)
    dr_s = time_host(lambda: holder.__setitem__("d", bale.read_sparse_matrix_dev(ds_dir, device=dev)), ds_steps, 1)
    ds_bytes = sum(os.path.getsize(f"{ds_dir}/{f}") for f in os.listdir(ds_dir))
    ds_ok = bool(torch.equal(holder["d"][0], off) and torch.equal(holder["d"][1], col))
    w = ctx["dist"].world
    out = {"metric": "G nonzeros/s transposing the R-MAT scale-22 lower matrix on the device",
           "value": round(job_rate(nnz, t_ms / 1e3, w) / 1e9, 4), "unit": "G nonzeros/s",
           "ms_per_step": round(t_ms, 3),
           "permute": {"value": round(job_rate(nnz, p_ms / 1e3, w) / 1e9, 4), "unit": "G nonzeros/s",
                       "ms_per_step": round(p_ms, 3)},
           "rand_perm": {"value": round(job_rate(np_, r_ms / 1e3, w) / 1e9, 4), "unit": "G elements/s",
                         "ms_per_step": round(r_ms, 3), "n": np_, "how": "rand_permp_agi"},
           "rand_permp": {"value": round(job_rate(np_, x_ms / 1e3, w) / 1e9, 4), "unit": "G elements/s",
                          "ms_per_step": round(x_ms, 3), "n": np_,
                          "how": "rand_permp = rand_permp_exstack with buffers of 1024"},
           "read_matrix_mm": {"value": round(L20.nnz / mm_s / 1e9, 4), "unit": "G nonzeros/s",
                              "ms_per_step": round(mm_s * 1e3, 3), "file_bytes": mm_bytes, "nnz": L20.nnz,
                              "how": "bale_read_matrix_mm_dev on R-MAT scale 20 (file in the page cache)"},
           "dataset": {"write_G_nonzeros_s": round(nnz / dw_s / 1e9, 4), "read_G_nonzeros_s": round(nnz / dr_s / 1e9, 4),
                       "write_ms": round(dw_s * 1e3, 2), "read_ms": round(dr_s * 1e3, 2), "bytes": ds_bytes,
                       "write_GB_s": round(ds_bytes / dw_s / 1e9, 3), "read_GB_s": round(ds_bytes / dr_s / 1e9, 3),
                       "how": "bale_write_sparse_matrix_dev / bale_read_sparse_matrix_dev of the scale-22 lower "
                              "matrix, one writer (files in the page cache)"},
           # transpose: the sort dominates -- 8 B per key for its digit counts, 16 B per key per 8-bit pass
           "roofline": roofline(ctx, "spmat", (16 * ((2 * S + 7) // 8) + 8) * nnz, t_ms / 1e3,
                                "transpose: radix sort of (column, row) keys",
                                note="algorithmic bytes: 16 B per key per 8-bit pass (44-bit keys) plus 8 B per "
                                     "key for the digit counts; the check, key and CSR kernels are not counted"),
           # a transpose step: the CSR check, the key pass, the sort's digit counts and starts, ceil(44/8) = 6
           # look-back scatter passes, then the CSR offsets and columns
           "clocks": clocks.summary(), "gpu_launches": (2 + 2 + 6 + 2) * args.steps,
           "config": {"workload": "transpose_matrix / permute_matrix of the R-MAT scale-22 degree-ordered lower "
                                  "matrix (n = 2^22, 64,155,075 nonzeros); rand_permp_agi and rand_permp of 2^26 "
                                  "elements",
                      "nnz": nnz}}
    if ctx["cpu"]:
        orc = _oracle()
        offh, colh = off.cpu().numpy(), col.cpu().numpy()
        t0 = time.perf_counter()
        to, tc = orc.transpose(offh, colh, n)
        t_cpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        orc.permute(offh, colh, rinv.cpu().numpy(), cinv.cpu().numpy())
        p_cpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        rp = orc.rand_perm(1 << 22, 31)
        r_cpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        xp = orc.rand_perm_exstack(1 << 22, 31, 1024)
        x_cpu = time.perf_counter() - t0
        t0 = time.perf_counter()
        mo, mc, _ = orc.read_mm(mm_path)
        m_cpu = time.perf_counter() - t0
        do, dc, _ = bale.read_matrix_mm_dev(mm_path, device=dev)
        mm_ok = bool(np.array_equal(do.cpu().numpy(), mo) and np.array_equal(dc.cpu().numpy(), mc))
        out["read_matrix_mm"]["cpu_G_nonzeros_s"] = round(L20.nnz / m_cpu / 1e9, 5)
        t0 = time.perf_counter()
        orc.write_dataset(offh, colh, n, f"{mm_dir}/ds22_cpu")
        out["dataset"]["cpu_write_G_nonzeros_s"] = round(nnz / (time.perf_counter() - t0) / 1e9, 4)
        out["dataset"]["cpu_write_how"] = "write_sparse_matrix_agi at one PE (oracle restatement) from host arrays"
        shutil.rmtree(f"{mm_dir}/ds22_cpu", ignore_errors=True)
        out["cpu_baseline"] = {"value": round(nnz / t_cpu / 1e9, 5), "unit": "G nonzeros/s", "cores": 1,
                               "kind": "port",
                               "sample": "transpose_matrix_agi at one PE (oracle restatement) of the same matrix",
                               "permute_G_nonzeros_s": round(nnz / p_cpu / 1e9, 5),
                               "rand_perm_G_elements_s": round((1 << 22) / r_cpu / 1e9, 5),
                               "rand_permp_G_elements_s": round((1 << 22) / x_cpu / 1e9, 5),
                               "rand_perm_sample": "2^22 elements (dart throwing over lrand48)"}
        gt = holder["t"]
        out["parity_ok"] = mm_ok and ds_ok and bool(np.array_equal(gt[0].cpu().numpy(), to) and np.array_equal(gt[1].cpu().numpy(), tc)
                                and np.array_equal(bale.rand_perm_dev(1 << 22, 31, device=dev).cpu().numpy(), rp)
                                and np.array_equal(bale.rand_perm_exstack_dev(1 << 22, 31, 1024,
                                                                              device=dev).cpu().numpy(), xp))
    holder.clear()
    shutil.rmtree(mm_dir, ignore_errors=True)
    del off, col, rinv, cinv
    torch.cuda.empty_cache()
    return out


def run_batch(ctx, small: bool = False) -> dict:
    import torch

    from bale_old_gb300 import batch as bb
    from bale_old_gb300.mix import MIX_FULL, MIX_SMALL, as_batch, build_mix, run_plain

    bale, dev, args = ctx["bale"], ctx["dev"], ctx["args"]
    t0 = time.perf_counter()
    spec = MIX_SMALL if small else MIX_FULL
    inst = build_mix(dev, spec)
    gen_s = time.perf_counter() - t0
    items = sum(x[4] for x in inst)
    kinds = {"histo": 0, "ig": 0, "tri": 0}
    for x in inst:
        kinds[x[0]] += x[4]
    # plain per-instance launches
    with ClockSampler(ctx["gpu"]) as clocks:
        ctx["dist"].barrier()
        plain_ms = time_device(lambda: run_plain(inst), args.steps, args.warmup)
    plain_out = [x[1].clone() for x in inst]
    for x in inst:
        if x[0] != "ig":
            x[1].zero_()
    # batched: one graph launch per step
    b = as_batch(inst)
    ctx["dist"].barrier()
    batch_ms = time_device(b.run, args.steps, args.warmup)
    torch.cuda.synchronize()
    same_as_plain = all(torch.equal(o, x[1]) for o, x in zip(plain_out, inst)) and not b.bad().any()
    del plain_out
    # every instance against the oracle: counts = replays x the histogram,
    # tgt = table[index], count = replays x the AGI count
    oracle_ok, oracle_s = check_mix_with_oracle(inst, args.steps + args.warmup)
    ok = same_as_plain and oracle_ok
    stats = b.stats()
    side = b.plan()
    b.close()
    plain_ms, batch_ms = ctx["dist"].max(plain_ms), ctx["dist"].max(batch_ms)
    w = ctx["dist"].world
    # per-instance launches, synchronised after each one (a drop-in caller's pattern)
    def plain_sync():
        for x in inst:
            run_plain([x])
            torch.cuda.synchronize()
    sync_s = ctx["dist"].max(time_host(plain_sync, max(1, args.steps // 3), 1))
    bound = batch_bound(inst, side, args)
    name = "small-instance 512 mix" if small else "uneven 512-instance mix"
    return {"metric": f"G items/s on the {name} (updates + requests + edges), batched",
            "value": round(job_rate(items, batch_ms / 1e3, w) / 1e9, 4), "unit": "G items/s",
            "ms_per_step": round(batch_ms, 3),
            "plain": {"value": round(job_rate(items, plain_ms / 1e3, w) / 1e9, 4), "unit": "G items/s",
                      "ms_per_step": round(plain_ms, 3),
                      "how": "each instance's device entry point, back to back on one stream"},
            "plain_sync": {"value": round(job_rate(items, sync_s, w) / 1e9, 4), "unit": "G items/s",
                           "ms_per_step": round(sync_s * 1e3, 3),
                           "how": "each instance's device entry point, synchronised after each instance"},
            "batched_vs_plain": round(plain_ms / batch_ms, 3), "batched_vs_plain_sync": round(sync_s * 1e3 / batch_ms, 3),
            "batched_bound_ms": bound["bound_ms"], "ratio_ceiling": round(plain_ms / bound["bound_ms"], 3),
            "bound": bound,
            "parity_ok": bool(ok), "parity": {"oracle_ok": bool(oracle_ok), "same_as_plain": bool(same_as_plain),
                                              "how": "every instance against the oracle's AGI loops on the host "
                                                     "(histo_agi_mt, ig_agi_mt, triangle_agi_mt)",
                                              "check_s": round(oracle_s, 1)},
            "batch_stats": stats, "clocks": clocks.summary(),
            "gpu_launches": args.steps,
            "config": {"workload": f"batched {name}: 256 histo + 192 ig + 64 R-MAT triangle instances, "
                                   f"log-uniform sizes {spec}",
                       "items_per_step": items, "items_by_kind": kinds, "generate_s": round(gen_s, 1),
                       "l2": "the mix's working set (~60 GB) exceeds L2; no flush"}}


def batch_bound(inst, side, args) -> dict:
    """The mix's time if every instance ran at the best rate its kernel
    reaches on this GPU, with no launch gaps or idle SMs: each instance is
    timed alone (CUDA events around its own entry point), the best items/s of
    each class (histo and ig split by whether the table fits in L2) is that
    class's rate, and the bound is the sum over instances of items / rate.
    Beside it: the work queue alone (the small instances as one batch), the
    standalone instances alone (one batch of them, on their side streams),
    and how much of the shorter of the two the full batch hides."""
    import torch

    from bale_old_gb300 import batch as bb
    from bale_old_gb300.mix import run_plain

    l2 = 96 << 20
    stream = torch.cuda.current_stream()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in inst]
    run_plain(inst)  # warm
    torch.cuda.synchronize()
    for x, (a, b) in zip(inst, ev):
        a.record(stream)
        run_plain([x])
        b.record(stream)
    torch.cuda.synchronize()
    alone = [a.elapsed_time(b) for a, b in ev]

    def cls(x):
        if x[0] == "tri":
            return "tri"
        table_bytes = 8 * (x[3].numel() if x[0] == "ig" else x[1].numel())
        return f"{x[0]}_{'l2' if table_bytes <= l2 else 'hbm'}"

    best = {}
    for x, t in zip(inst, alone):
        c = cls(x)
        best[c] = max(best.get(c, 0.0), x[4] / t)  # items per ms
    bound_ms = sum(x[4] / best[cls(x)] for x in inst)
    small = [x for x, s in zip(inst, side) if s < 0]
    big = [x for x, s in zip(inst, side) if s >= 0]

    def batch_time(sub):
        if not sub:
            return 0.0
        for x in sub:
            if x[0] != "ig":
                x[1].zero_()
        with bb.Batch([bb.histo(x[1], x[2]) if x[0] == "histo" else bb.ig(x[1], x[2], x[3]) if x[0] == "ig"
                       else bb.triangles(x[2], x[3], x[1]) for x in sub]) as sb:
            return time_device(sb.run, args.steps, args.warmup)

    queue_ms, standalone_ms = batch_time(small), batch_time(big)
    return {"bound_ms": round(bound_ms, 3),
            "best_rates_G_items_s": {c: round(r / 1e6, 2) for c, r in sorted(best.items())},
            "alone_sum_ms": round(sum(alone), 3),
            "standalone_alone_sum_ms": round(sum(t for t, s in zip(alone, side) if s >= 0), 3),
            "queue_instances": len(small), "standalone_instances": len(big),
            "queue_only_batch_ms": round(queue_ms, 3), "standalone_only_batch_ms": round(standalone_ms, 3),
            "how": "bound = sum over instances of items / (best items/s of its class, each instance timed alone "
                   "with CUDA events); queue_only / standalone_only: the two halves of the plan as batches of "
                   "their own"}


def check_mix_with_oracle(inst, reps: int) -> tuple[bool, float]:
    """Each instance of a mix after `reps` batched replays, against the
    oracle's multi-threaded AGI restatements on the host: histo counts equal
    reps x the oracle's histogram, ig outputs equal the oracle's gather,
    triangle counts equal reps x the oracle's count.  Returns (all equal,
    seconds spent)."""
    orc = _oracle()
    t0 = time.perf_counter()
    ok = True
    for kind, out, a, b, _ in inst:
        if kind == "histo":
            want = np.zeros(out.numel(), np.int64)
            orc.histo_agi_mt(a.cpu().numpy(), want)
            ok &= bool(np.array_equal(out.cpu().numpy(), reps * want))
        elif kind == "ig":
            idx = a.cpu().numpy()
            want = np.empty(idx.size, np.int64)
            orc.ig_agi_mt(want, idx, b.cpu().numpy())
            ok &= bool(np.array_equal(out.cpu().numpy(), want))
        else:
            want = orc.triangle_agi_mt(a.cpu().numpy(), b.cpu().numpy())
            ok &= int(out.item()) == reps * want
        if not ok:
            break
    return ok, time.perf_counter() - t0


def run_serve(ctx) -> dict:
    """Serving: Poisson arrivals of 60% ig / 30% histo / 10% triangle requests
    (sizes log-uniform as in the batched mix; graphs R-MAT scales 12-20)
    against resident tables, counters and graphs; rates swept from light load
    to saturation; p50/p99 latency and throughput per rate."""
    import torch

    from bale_old_gb300 import serve as sv

    bale, args = ctx["bale"], ctx["args"]
    rng = np.random.default_rng(4242)
    logu = lambda lo, hi: int(round(np.exp(rng.uniform(np.log(lo), np.log(hi)))))  # noqa: E731
    nreq = 200
    t0 = time.perf_counter()
    s = sv.Server(arena_bytes=48 << 30, max_active=64)
    # resident objects
    tables = [logu(1_000, 64 << 20) for _ in range(8)]
    tids = [s.add_table(bale.gen_values(t, 50 + i)) for i, t in enumerate(tables)]
    counters = [logu(1_000, 16 << 20) for _ in range(8)]
    cids = [s.add_counts(c) for c in counters]
    graphs = [bale.gen_rmat(sc, 16, 0.57, 0.19, 0.19, 70 + sc) for sc in (12, 14, 16, 18, 19, 20)]
    gids = [s.add_graph(L) for L in graphs]
    # requests: each ig/histo request reads a prefix of its object's pinned index pool
    kinds, objs, sizes = [], [], []
    for _ in range(nreq):
        u = rng.random()
        if u < 0.6:
            kinds.append("ig"); objs.append(int(rng.integers(8))); sizes.append(logu(10_000, 128 << 20))
        elif u < 0.9:
            kinds.append("histo"); objs.append(int(rng.integers(8))); sizes.append(logu(10_000, 64 << 20))
        else:
            kinds.append("tri"); objs.append(int(rng.integers(len(graphs)))); sizes.append(0)
    pools = {}
    for kind, o, n in zip(kinds, objs, sizes):
        if kind != "tri":
            key = (kind, o)
            pools[key] = max(pools.get(key, 0), n)
    pinned = {}
    for (kind, o), n in pools.items():
        rngmax = tables[o] if kind == "ig" else counters[o]
        pinned[(kind, o)] = torch.from_numpy(bale.gen_uniform(n, rngmax, 90 + o + (0 if kind == "ig" else 100))).pin_memory()
    out_total = sum(n for k, n in zip(kinds, sizes) if k == "ig")
    out_pool = torch.empty(out_total, dtype=torch.int64).pin_memory()
    tri_out = np.zeros((nreq, 1), np.int64)
    items = sum(sizes) + sum(graphs[o].nnz for k, o in zip(kinds, objs) if k == "tri")
    h2d = 8 * sum(sizes)  # index arrays of the ig and histo requests
    d2h = 8 * sum(n for k, n in zip(kinds, sizes) if k == "ig") + 8 * kinds.count("tri")
    gen_s = time.perf_counter() - t0

    def trace(arrivals):
        reqs, off = [], 0
        for k, (kind, o, n) in enumerate(zip(kinds, objs, sizes)):
            if kind == "ig":
                reqs.append(sv.ig(tids[o], pinned[(kind, o)].numpy()[:n], out_pool.numpy()[off:off + n], arrivals[k]))
                off += n
            elif kind == "histo":
                reqs.append(sv.histo(cids[o], pinned[(kind, o)].numpy()[:n], arrivals[k]))
            else:
                reqs.append(sv.triangles(gids[o], tri_out[k], arrivals[k]))
        return reqs

    # capacity: everything arrives at once
    s.run(trace(np.zeros(nreq)))  # warm-up
    _, cap = s.run(trace(np.zeros(nreq)))
    cap_rate = nreq / cap["makespan_s"]
    # each offered rate on three Poisson traces (arrival seeds): the median
    # and the spread (min, max) of p50 / p99 / throughput
    rates = []
    for frac in (0.25, 0.5, 0.75, 1.0, 1.5):
        runs = [s.run(trace(sv.poisson_arrivals(nreq, frac * cap_rate, seed)))[1] for seed in (17, 18, 19)]

        def med(key, scale=1.0):
            v = sorted(r[key] * scale for r in runs)
            return {"median": round(v[1], 3), "min": round(v[0], 3), "max": round(v[2], 3)}

        rates.append({"offered_requests_per_s": round(frac * cap_rate, 2), "load": frac, "traces": len(runs),
                      "p50_ms": med("p50_s", 1e3), "p99_ms": med("p99_s", 1e3), "mean_ms": med("mean_s", 1e3),
                      "G_items_per_s": med("items_per_s", 1e-9),
                      "ticks": [r["ticks"] for r in runs], "max_active": [r["max_active"] for r in runs],
                      "admission_waits": [r["admission_waits"] for r in runs],
                      "express_requests": runs[0]["express"]})
    # exactness of the last run: triangle counts and a sample of ig values
    ok = True
    tri_want = {}
    for k, (kind, o) in enumerate(zip(kinds, objs)):
        if kind == "tri":
            if o not in tri_want:
                L = graphs[o]
                c = torch.zeros(1, dtype=torch.int64, device=ctx["dev"])
                bale.triangle_dev(torch.from_numpy(L.offset).to(ctx["dev"]), torch.from_numpy(L.nonzero).to(ctx["dev"]), c)
                tri_want[o] = int(c.item())
            ok &= int(tri_out[k][0]) == tri_want[o]
    k0 = kinds.index("ig")
    t = bale.gen_values(tables[objs[k0]], 50 + objs[k0])
    ok &= bool(np.array_equal(out_pool.numpy()[: min(sizes[k0], 1 << 20)],
                              t[pinned[("ig", objs[k0])].numpy()[: min(sizes[k0], 1 << 20)]]))
    s.close()
    return {"metric": "served G items/s at saturation (updates + requests + edges), p50/p99 per offered rate",
            "value": round(cap["items_per_s"] / 1e9, 4), "unit": "G items/s",
            "ms_per_step": round(cap["makespan_s"] * 1e3, 3), "parity_ok": bool(ok),
            "capacity_requests_per_s": round(cap_rate, 2),
            "saturation": {"p50_ms": round(cap["p50_s"] * 1e3, 3), "p99_ms": round(cap["p99_s"] * 1e3, 3),
                           "ticks": cap["ticks"], "max_active": cap["max_active"],
                           "gpu_busy_s": round(cap["gpu_busy_s"], 4), "loop_iters": cap["loop_iters"],
                           "tasks": cap["tasks"], "express_requests": cap["express"]},
            "rates": rates, "gpu_launches": cap["ticks"],
            "config": {"workload": "serving: Poisson arrivals, 60% ig / 30% histo / 10% triangles, 200 requests, "
                                   "8 resident tables (1K-64M entries), 8 counter arrays (1K-16M), "
                                   "6 resident R-MAT graphs (scales 12-20); request sizes log-uniform "
                                   "(ig 10K-128M, histo 10K-64M); pinned host index and output buffers",
                       "items_per_trace": items, "h2d_bytes_per_trace": h2d, "d2h_bytes_per_trace": d2h,
                       "setup_s": round(gen_s, 1)}}


def tri_roofline(ctx, push_bytes: int, count_s: float, step_ms: float) -> dict:
    """The wedge count kernel's roofline: bound by instruction issue; DRAM
    bytes per launch from the committed ncu capture over the live kernel
    time, against the measured HBM peak; the push-model bytes beside it."""
    tr = ctx["traffic"].get("triangles", {})
    dram = tr.get("dram_bytes_per_step")
    achieved = dram / count_s / 1e9 if dram else None
    return {"bound": "issue", "kernel": "wedge_count_kernel (one warp per row j: bitmap / staged search over the "
                                        "incoming prefixes) + wedge_dense_kernel (bitmap AND of the dense pairs)",
            "achieved": round(achieved, 1) if achieved else None, "peak": ctx["peak"], "peak_source": ctx["peak_src"],
            "unit": "GB/s", "frac": round(achieved / ctx["peak"], 4) if achieved else None, "traffic": dram,
            "what": "DRAM bytes of one count (both kernels, ncu) over their live time: their share of HBM",
            "issue_active_ncu": tr.get("issue_active"), "ncu_source": tr.get("summary"),
            "count_kernel_ms": round(count_s * 1e3, 4),
            "push_model": {"bytes_per_launch": push_bytes, "achieved_gbs": round(push_bytes / count_s / 1e9, 1),
                           "note": "4 B per probed prefix element (exstack pushes, "
                                   "apps/triangle_src/triangle.upc:344-349; the dense pairs as the pushes they "
                                   "replace), 8 B per prefix record, 8 B per nonzero for row j: L2 and DRAM bytes "
                                   "together"},
            "note": f"the step also runs the prepare kernels (validate, transpose, row bitmaps): "
                    f"{round(step_ms - count_s * 1e3, 3)} ms of the {round(step_ms, 3)} ms step"}


def roofline(ctx, wl: str, algo_bytes: int, seconds: float, kernel: str, note: str | None = None) -> dict:
    peak = ctx["peak"]
    achieved = algo_bytes / seconds / 1e9
    tr = ctx["traffic"].get(wl, {}).get("dram_bytes_per_step")
    r = {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": peak,
         "peak_source": ctx["peak_src"], "unit": "GB/s", "frac": round(achieved / peak, 4), "traffic": tr,
         "algorithmic_bytes_per_step": algo_bytes}
    if note:
        r["note"] = note
    return r


# ---------------------------------------------------------------------------
# CPU baseline: the oracle restatement of the reference's AGI loops
# ---------------------------------------------------------------------------
def _oracle():
    from oracle.pyoracle import Oracle

    return Oracle()


def cpu_ig(index_h, table_h, budget_s: float) -> dict:
    orc = _oracle()
    cores = orc.num_cpus()
    sample = np.ascontiguousarray(index_h[: 1 << 25])
    tgt = np.empty(sample.size, np.int64)
    reps, t0 = 0, time.perf_counter()
    while True:
        orc.ig_agi_mt(tgt, sample, table_h, cores)
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    secs = time.perf_counter() - t0
    return {"value": round(reps * sample.size / secs / 1e9, 5), "unit": "GUP/s", "cores": cores, "kind": "port",
            "sample": f"{reps} x the first 2^25 requests against the full 2^26 table "
                      "(ig_agi loop, apps/ig_src/ig_agi.upc:61-64, one pthread per core)"}


def cpu_histo(index_h, budget_s: float) -> dict:
    orc = _oracle()
    cores = orc.num_cpus()
    counts = np.zeros(HISTO_COUNTS, np.int64)
    reps, t0 = 0, time.perf_counter()
    while True:
        orc.histo_agi_mt(index_h, counts, cores)
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            break
    secs = time.perf_counter() - t0
    return {"value": round(reps * index_h.size / secs / 1e9, 5), "unit": "GUP/s", "cores": cores, "kind": "port",
            "sample": f"{reps} x all 10^7 updates (histo_agi loop, apps/histo_src/histo_agi.upc:61-66, "
                      "relaxed atomic adds, one pthread per core)"}


def _reps(fn, budget_s: float) -> tuple[int, float]:
    reps, t0 = 0, time.perf_counter()
    while True:
        fn()
        reps += 1
        if time.perf_counter() - t0 >= budget_s:
            return reps, time.perf_counter() - t0


def one_pe_legs(kind: str, budget_s: float, **a) -> dict:
    """The AGI loop and the exstack variant (its buffers of 1024 packages,
    exchange and pops modelled at one PE) on one host thread: the reference's
    single-PE runs, restated, on a bounded sample."""
    orc = _oracle()
    if kind == "ig":
        idx, table = a["index"], a["table"]
        pck = (idx << 16).astype(np.int64)
        ra, sa = _reps(lambda: orc.ig_agi(idx, table), budget_s)
        rx, sx = _reps(lambda: orc.ig_exstack_buffered(pck, table, 1024), budget_s)
        n, unit = idx.size, "GUP/s"
        sample = f"the first {idx.size} requests against the full table (ig_agi, ig_exstack)"
    elif kind == "histo":
        idx = a["index"]
        pck = (idx << 16).astype(np.int64)
        counts = np.zeros(HISTO_COUNTS, np.int64)
        ra, sa = _reps(lambda: orc.histo_agi(idx, counts), budget_s)
        rx, sx = _reps(lambda: orc.histo_exstack_buffered(pck, counts, 1024), budget_s)
        n, unit = idx.size, "GUP/s"
        sample = "all 10^7 updates (histo_agi, histo_exstack)"
    else:
        off, col, step = a["offset"], a["nonzero"], a["row_step"]
        rows = np.arange(0, off.size - 1, step)
        n, unit = int((off[rows + 1] - off[rows]).sum()), "G edges/s"
        t0 = time.perf_counter()
        ca = orc.triangle_agi_sampled(off, col, 0, step)
        ra, sa = 1, time.perf_counter() - t0
        t0 = time.perf_counter()
        cx, _ = orc.triangle_exstack_push_buffered(off, col, 1024, 0, step)
        rx, sx = 1, time.perf_counter() - t0
        sample = f"rows 0, {step}, {2 * step}, ... ({n} nonzeros; triangle_agi alg 0, triangle_exstack_push)"
        if ca != cx:
            return {"error": f"sampled counts differ: {ca} against {cx}"}
    return {"cores": 1, "kind": "port", "unit": unit, "sample": sample,
            "agi": round(ra * n / sa / 1e9, 6), "exstack": round(rx * n / sx / 1e9, 6)}


def cpu_triangles(L, budget_s: float) -> dict:
    orc = _oracle()
    cores = orc.num_cpus()
    t0 = time.perf_counter()
    cnt = orc.triangle_agi_mt(L.offset, L.nonzero, cores)
    secs = time.perf_counter() - t0
    return {"value": round(L.nnz / secs / 1e9, 5), "unit": "Gedges/s", "cores": cores, "kind": "port",
            "sample": "1 x the full scale-22 graph (triangle_agi alg 0 loop, "
                      "apps/triangle_src/triangle_agi.upc:69-99, rows shared dynamically by pthreads)",
            "seconds": round(secs, 2), "triangles": cnt}


# ---------------------------------------------------------------------------
def run_gb300(args, dist: Dist) -> dict | None:
    import torch

    import bale_old_gb300 as bale

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    peaks = measured_peaks()
    ctx = {"bale": bale, "dev": dev, "args": args, "dist": dist, "gpu": dist.local,
           "peak": float(peaks.get("hbm_gbs") or HBM_FALLBACK_GBS),
           "peak_src": "measured (MEASURED_PEAKS.json hbm_gbs)" if peaks.get("hbm_gbs") else "fallback",
           "traffic": committed_traffic(), "cpu": dist.rank == 0 and not args.no_cpu_baseline,
           "budget": args.cpu_budget, "later": []}
    runners = {"ig": lambda: run_ig(ctx, False), "ig_zipf": lambda: run_ig(ctx, True),
               "histo": lambda: run_histo(ctx), "triangles": lambda: run_triangles(ctx),
               "batch": lambda: run_batch(ctx), "batch_small": lambda: run_batch(ctx, small=True),
               "serve": lambda: run_serve(ctx), "graph": lambda: run_graph(ctx), "spmat": lambda: run_spmat(ctx)}
    head = runners[args.workload]()
    bale.release_buffers()
    torch.cuda.empty_cache()
    others = {}
    if not args.only:
        # each workload starts with the library's cached buffers released
        for wl in ("ig_zipf", "histo", "triangles", "serve", "graph", "spmat", "batch", "batch_small", "ig"):
            if wl != args.workload:
                others[wl] = runners[wl]()
                bale.release_buffers()
                torch.cuda.empty_cache()
    # The ig, histo and triangle CPU legs (all host threads, 10-30 s each)
    # run after every GPU measurement: run before it, they left the serving
    # loop measuring about half the capacity it measures in a process with
    # no CPU legs, with the SM clock at its maximum throughout.
    for leg in ctx["later"]:
        leg()
    if not args.only:
        head["workloads"] = others
        # last key of the line: one short entry per workload, so that a
        # reader keeping only the line's tail still sees every result
        head["summary"] = {args.workload: summarize(head), **{wl: summarize(r) for wl, r in others.items()}}
    return head


def summarize(r: dict) -> dict:
    """value, roofline fraction, parity and the main ratio of one workload."""
    out = {"value": r.get("value"), "unit": r.get("unit")}
    rf = r.get("roofline") or {}
    if rf.get("frac") is not None:
        out["frac"] = rf["frac"]
        out["bound"] = rf.get("bound")
    par = [r[k] for k in ("parity_ok", "parity_sample_ok") if k in r]
    if par:
        out["parity"] = all(par)
    if "e2e" in r:
        out["e2e"] = r["e2e"].get("value")
    if "cpu_baseline" in r:
        out["cpu"] = r["cpu_baseline"].get("value")
    for k in ("batched_vs_plain", "batched_bound_ms", "triangles"):
        if k in r:
            out[k] = r[k]
    if "saturation" in r:
        out["p50_ms"], out["p99_ms"] = r["saturation"]["p50_ms"], r["saturation"]["p99_ms"]
    if "rates" in r:
        out["p50_ms_by_load"] = {str(x["load"]): x["p50_ms"]["median"] for x in r["rates"]}
    if "erdos_renyi" in r:
        er = r["erdos_renyi"]
        out["er"] = {"value": er["default"]["value"], "parity": er.get("parity_ok")}
    return out


def run_reference(args, dist: Dist) -> dict | None:
    """The CPU implementation of the path: the oracle restatement of the
    reference's AGI loops on all host threads, over the whole workload per
    step (all 2^28 requests; all 10^7 updates).  Inputs come from the
    oracle's own SplitMix64 generators (equal to the GPU library's, pinned by
    tests/test_oracle.py), so this process never loads the GPU library."""
    if dist.rank != 0:
        return None
    orc = _oracle()
    cores = orc.num_cpus()
    wl = args.workload
    if wl == "ig":
        table_h = orc.gen_values(IG_TABLE, 2)
        index_h = orc.gen_uniform(IG_REQUESTS, IG_TABLE, 3)
        tgt = np.empty(index_h.size, np.int64)
        secs = time_host(lambda: orc.ig_agi_mt(tgt, index_h, table_h, cores), args.steps, args.warmup)
        ok = bool(np.array_equal(tgt[: 1 << 20], table_h[index_h[: 1 << 20]]))
        v, unit, metric = IG_REQUESTS / secs / 1e9, "GUP/s", "GUP/s index gather (10^9 requests/s)"
        desc = "all 2^28 uniform requests per step against the full 2^26-entry table"
        work = {"workload": "ig uniform: 2^26-entry int64 table, 2^28 int64 requests", "table_entries": IG_TABLE,
                "requests": IG_REQUESTS}
    elif wl == "histo":
        index_h = orc.gen_uniform(HISTO_UPDATES, HISTO_COUNTS, 1)
        counts = np.zeros(HISTO_COUNTS, np.int64)
        secs = time_host(lambda: orc.histo_agi_mt(index_h, counts, cores), args.steps, args.warmup)
        ok = int(counts.sum()) == (args.steps + args.warmup) * HISTO_UPDATES
        v, unit, metric = HISTO_UPDATES / secs / 1e9, "GUP/s", "GUP/s histogram (10^9 updates/s)"
        desc = "all 10^7 updates per step into the 10^6 counters"
        work = {"workload": "histo: 10^7 uniform updates into 10^6 int64 counters", "updates": HISTO_UPDATES,
                "counters": HISTO_COUNTS}
    else:
        return {"impl": "reference", "unavailable": f"the CPU reference arm builds its inputs without the GPU library for the ig and "
                               f"histo workloads only; {wl} needs the library's generators"}
    return {"metric": metric, "value": round(v, 5), "unit": unit, "impl": "reference",
            "ms_per_step": round(secs * 1e3, 3), "parity_sample_ok": ok,
            "cpu_baseline": {"value": round(v, 5), "unit": unit, "cores": cores, "kind": "port", "sample": desc},
            "e2e": {"value": round(v, 5), "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config": {**work, "note": "oracle restatement of the reference's AGI loop (apps/ig_src/ig_agi.upc:61-64, "
                                       "apps/histo_src/histo_agi.upc:61-66), one pthread per core; the reference's "
                                       "own build runs one PE, single-threaded, and exists only where its source "
                                       "tree does"}}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ig", choices=["ig", "ig_zipf", "histo", "triangles", "graph", "spmat", "batch", "batch_small", "serve"])
    ap.add_argument("--only", action="store_true", help="measure the selected workload only")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--cpu-budget", type=float, default=8.0, help="seconds of CPU baseline per workload")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    dist = Dist()
    try:
        res = run_reference(args, dist) if args.impl == "reference" else run_gb300(args, dist)
        if dist.rank == 0 and res is not None and "unavailable" in res:
            print(json.dumps({"impl": res["impl"], "unavailable": res["unavailable"]}), flush=True)
        elif dist.rank == 0 and res is not None:
            line = {"metric": res.pop("metric"), "value": res.pop("value"), "unit": res.pop("unit"),
                    "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
                    "ms_per_step": res.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded SplitMix64 / R-MAT)"}
            line.update(res)
            print(json.dumps(line), flush=True)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
