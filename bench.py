"""Benchmark of the GB300 irregular-access core.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--workload ig|ig_zipf|histo|triangles]

One JSON line on stdout (rank 0).  A "step" is one pass of the workload's
kernel over its whole synthetic input:

* ig        (default, the headline): 2^26-entry int64 table of seeded random
            values, 2^28 uniform requests -> GUP/s (10^9 requests/s);
* ig_zipf   : same, requests Zipf(1.1) over a keyed permutation of the table;
* histo     : 10^7 uniform updates into 10^6 int64 counters -> GUP/s;
* triangles : R-MAT scale 22, edge factor 16, (0.57,0.19,0.19,0.05), degree
            ordered strictly lower L -> edges/s (nnz(L) per second).

``value`` is device-timed with inputs resident in HBM (CUDA events on the
launching stream, W warm-up steps, K timed steps; the index streams are
larger than L2 so no flush is needed, except histo whose 80 MB stream is
followed by a 256 MiB L2 flush write each step, outside the kernel's own
events).  ``e2e`` is the same metric through the reference-facing C ABI
(ig_agi / histo_agi / triangle_agi) with pinned host buffers, copies
included.  ``--impl reference`` times the CPU implementation of the path
(the oracle restatement of the reference's AGI loop, all host threads) on a
bounded sample of the same workload.

Under torchrun every rank runs its own copy of the workload on its own GPU
(weak scaling); rank 0 reports the job total over the max of the ranks' times.
"""
from __future__ import annotations

import argparse
import json
import os
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


# ---------------------------------------------------------------------------
# distributed plumbing (torchrun sets RANK/WORLD_SIZE/LOCAL_RANK)
# ---------------------------------------------------------------------------
class Dist:
    def __init__(self, want_gpus: int):
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


def measured_peaks() -> dict:
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


def committed_traffic() -> dict:
    """Per-launch DRAM bytes from the committed ncu summaries (profiles/)."""
    p = ROOT / "profiles" / "traffic.json"
    if p.exists():
        try:
            return json.loads(p.read_text())
        except ValueError:
            pass
    return {}


# ---------------------------------------------------------------------------
# clocks sampled while the timed region runs
# ---------------------------------------------------------------------------
class ClockSampler:
    QUERY = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
             "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

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
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits",
                 "-lms", "100"], stdout=self.fh, stderr=subprocess.DEVNULL)
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
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = float(f[2])
            except ValueError:
                continue
            for name, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(name)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": smax,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
IG_TABLE = 1 << 26
IG_REQUESTS = 1 << 28
HISTO_COUNTS = 1_000_000
HISTO_UPDATES = 10_000_000
TRI_SCALE = 22


def gen_ig_inputs(bale, zipf: bool):
    table = bale.gen_values(IG_TABLE, 2)
    if zipf:
        index = bale.gen_zipf(IG_REQUESTS, IG_TABLE, 1.1, 4, 5)
    else:
        index = bale.gen_uniform(IG_REQUESTS, IG_TABLE, 3)
    return index, table


def time_device(fn, steps: int, warmup: int, stream, between=None):
    """Average CUDA-event time of fn() per step (ms), on `stream`."""
    import torch

    for _ in range(warmup):
        if between:
            between()
        fn()
    torch.cuda.synchronize()
    per = []
    total = 0.0
    for _ in range(steps):
        if between:
            between()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        b.synchronize()
        per.append(a.elapsed_time(b))
        total += per[-1]
    return total / steps, per


def run_gb300(args, dist: Dist) -> dict | None:
    import torch

    import bale_old_gb300 as bale

    dev = torch.device("cuda", dist.local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    peaks = measured_peaks()
    hbm = float(peaks.get("hbm_gbs") or HBM_FALLBACK_GBS)
    peak_note = "measured" if peaks.get("hbm_gbs") else "fallback"
    traffic = committed_traffic()
    wl = args.workload
    flush = None
    result: dict = {}

    if wl in ("ig", "ig_zipf"):
        index_h, table_h = gen_ig_inputs(bale, wl == "ig_zipf")
        n = index_h.size
        index = torch.from_numpy(index_h).to(dev)
        table = torch.from_numpy(table_h).to(dev)
        tgt = torch.empty_like(index)
        bad = torch.zeros(1, dtype=torch.int64, device=dev)
        fn = lambda: bale.ig_dev(tgt, index, table, bad=bad)  # noqa: E731
        units, unit_name = n, "GUP/s"
        algo_bytes = 48 * n  # 8 B index + 32 B table sector + 8 B output
        kernel = "ig_gather_kernel"
        config = {"workload": f"ig {'zipf(1.1) over a keyed permutation' if wl == 'ig_zipf' else 'uniform'}: "
                              f"2^26-entry int64 table, 2^28 int64 requests",
                  "table_entries": IG_TABLE, "requests": n,
                  "l2": "index and output streams (2 GiB each) exceed L2; no flush"}
        metric = "GUP/s index gather (10^9 requests/s)"

        def check():
            torch.cuda.synchronize()
            s = slice(0, 1 << 20)
            want = table_h[index_h[s]]
            return bool(np.array_equal(tgt[s].cpu().numpy(), want)) and int(bad.item()) == 0

        pin_idx = torch.from_numpy(index_h).pin_memory()
        pin_tab = torch.from_numpy(table_h).pin_memory()
        pin_tgt = torch.empty(n, dtype=torch.int64).pin_memory()

        def e2e_call():
            t = bale.ig_agi(pin_tgt.numpy(), pin_idx.numpy(), pin_tab.numpy())
            return t

        h2d, d2h = 8 * n + 8 * IG_TABLE, 8 * n
        e2e_check = lambda: bool(np.array_equal(pin_tgt.numpy()[: 1 << 20], table_h[index_h[: 1 << 20]]))  # noqa: E731
    else:
        raise SystemExit(f"unknown workload {wl}")

    # device-timed region (inputs resident)
    dist.barrier()
    with ClockSampler(dist.local) as clocks:
        ms, per = time_device(fn, args.steps, args.warmup, stream, between=flush)
    ok = check()
    ms_max = dist.max(ms)
    value = dist.world * units / (ms_max / 1e3) / 1e9
    kernel_s = ms / 1e3
    achieved = algo_bytes / kernel_s / 1e9
    tr = traffic.get(wl, {}).get("dram_bytes_per_launch")
    result.update({
        "metric": metric, "value": round(value, 4), "unit": unit_name,
        "ms_per_step": round(ms_max, 4), "parity_sample_ok": ok,
        "roofline": {"bound": "hbm", "kernel": kernel, "achieved": round(achieved, 1), "peak": hbm,
                     "peak_source": peak_note, "unit": "GB/s", "frac": round(achieved / hbm, 4),
                     "traffic": tr, "algorithmic_bytes_per_launch": algo_bytes},
        "clocks": clocks.summary(), "config": config,
        "gpu_launches": args.steps,
    })

    # e2e through the C ABI (host pinned buffers, copies inside)
    for _ in range(max(1, args.warmup)):
        e2e_call()
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        e2e_call()
    e2e_s = dist.max((time.perf_counter() - t0) / args.steps)
    result["e2e"] = {"value": round(dist.world * units / e2e_s / 1e9, 4), "unit": unit_name,
                     "ms_per_step": round(e2e_s * 1e3, 3), "h2d_bytes_per_step": h2d,
                     "d2h_bytes_per_step": d2h, "path": "ig_agi C ABI, pinned host buffers",
                     "parity_sample_ok": e2e_check()}

    if dist.rank == 0 and not args.no_cpu_baseline:
        result["cpu_baseline"] = cpu_baseline(wl, index_h, table_h)
    return result


def cpu_baseline(wl: str, index_h, table_h, budget_s: float = 10.0) -> dict:
    """The oracle restatement of ig_agi on all host threads, on a bounded
    sample: the first 2^25 requests of the same workload, repeated for about
    budget_s seconds."""
    from oracle.pyoracle import Oracle

    orc = Oracle()
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
    return {"value": round(reps * sample.size / secs / 1e9, 5), "unit": "GUP/s", "cores": cores,
            "kind": "port", "sample": f"{reps} x first 2^25 requests of the {wl} workload against "
                                       "the full 2^26 table (oracle ig_agi loop, pthreads)"}


def run_reference(args, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    import bale_old_gb300 as bale
    from oracle.pyoracle import Oracle

    orc = Oracle()
    cores = orc.num_cpus()
    wl = args.workload
    if wl not in ("ig", "ig_zipf"):
        raise SystemExit(f"unknown workload {wl}")
    index_h, table_h = gen_ig_inputs(bale, wl == "ig_zipf")
    sample = np.ascontiguousarray(index_h[: 1 << 26])
    tgt = np.empty(sample.size, np.int64)
    for _ in range(args.warmup):
        orc.ig_agi_mt(tgt, sample, table_h, cores)
    t0 = time.perf_counter()
    for _ in range(args.steps):
        orc.ig_agi_mt(tgt, sample, table_h, cores)
    secs = (time.perf_counter() - t0) / args.steps
    v = sample.size / secs / 1e9
    return {"metric": "GUP/s index gather (10^9 requests/s)", "value": round(v, 5), "unit": "GUP/s",
            "impl": "reference", "ms_per_step": round(secs * 1e3, 3),
            "cpu_baseline": {"value": round(v, 5), "unit": "GUP/s", "cores": cores, "kind": "port",
                             "sample": "first 2^26 of the 2^28 requests per step, full 2^26 table"},
            "e2e": {"value": round(v, 5), "unit": "GUP/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "config": {"workload": f"{wl}: 2^26-entry int64 table, 2^28 requests (2^26-request sample per step)"}}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="ig", choices=["ig", "ig_zipf", "histo", "triangles"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    args = ap.parse_args(argv)
    args.warmup = max(args.warmup, 3)
    dist = Dist(args.gpus)
    try:
        res = run_reference(args, dist) if args.impl == "reference" else run_gb300(args, dist)
        if dist.rank == 0 and res is not None:
            line = {"metric": res.pop("metric"), "value": res.pop("value"), "unit": res.pop("unit"),
                    "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
                    "ms_per_step": res.pop("ms_per_step"), "higher_is_better": True, "scaling": "weak",
                    "vs_baseline": None, "dtype": "int64", "data": "synthetic (seeded SplitMix64)"}
            line.update(res)
            print(json.dumps(line), flush=True)
    finally:
        dist.close()
    return 0


if __name__ == "__main__":
    sys.exit(main())
