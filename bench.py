"""Benchmark of the batched seed-extension path on one GB300.

Workload (the batched-extension configuration): a 5 Mbp variation graph with a
variant every ~100 bp (70% SNPs, 30% indels of 1-20 bp), 50k reads log-normal
with mean 10 kbp clipped to 1-50 kbp at U[5%,15%] error, one exact 15-mer seed
per read taken from the true path, and both extensions of each seed
(GraphAligner::getTwoDirectionalTrace) -> ~100k extensions, bandwidth 10,
default X-drop, unlimited tangle effort.  Seeded synthetic data stands in for
real reads (no public dataset is named for this path).

A step is one pass of getReverseTraceFromSeed (fill + traceback) over the whole
batch.  `value` is aligned read bp per second with the batch resident in HBM
(device time of the fill and traceback kernels, CUDA events on their stream);
`e2e` is the same through the host-buffer C-ABI call ga_extend_batch with the
requests in pinned memory and the results copied back, timed around the call.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "read bp aligned/s"
UNIT = "read bp/s"
WORKLOAD = "batched seed extension: 5 Mbp VG (variant/100 bp), 50k reads lognormal mean 10 kbp [1,50] kbp, err U[5,15]%, exact 15-mer seed, both directions, bandwidth 10"
INT32_OPS_PER_STEP = 40          # 20 u64 ops (two 32-bit halves each) per Myers column step
PEAKS = os.path.join(ROOT, "MEASURED_PEAKS.json")


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--reads", type=int, default=50_000)
    ap.add_argument("--cpu-sample-bp", type=float, default=200e6)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--plain-sample", type=int, default=300, help="extensions timed one launch each (0: skip)")
    ap.add_argument("--workload", default="extend", choices=["extend", "reads-vg", "reads-dbg", "pipeline", "serve"],
                    help="extend: the batched-extension line; the others print read-level lines")
    ap.add_argument("--reads-n", type=int, default=0, help="reads of a read-level workload (0: its default)")
    ap.add_argument("--rates", default="10,20,40,60", help="serve: Poisson arrival rates, reads/s")
    ap.add_argument("--plain-reads", type=int, default=40, help="serve: reads timed one ga_align_reads call each")
    ap.add_argument("--serve-seconds", type=float, default=8.0, help="serve: seconds of Poisson arrivals per rate")
    ap.add_argument("--serve-min-reads", type=int, default=500, help="serve: reads per rate at least")
    ap.add_argument("--cpu-reads", type=int, default=40, help="read-level: reads of the CPU baseline sample")
    ap.add_argument("--multiseed", action="store_true", help="read-level: --multiseed-DP 1 (one multiseed DP per read)")
    ap.add_argument("--no-autotune", dest="autotune", action="store_false", help="extend: keep the default launch shape")
    ap.add_argument("--truncate", type=int, default=0, help="extend: cut every extension to this many bases (small profiling cases)")
    ap.add_argument("--arena-gb", type=float, default=0, help="DP-table arena size (default: from the batch or the reads)")
    return ap.parse_args()


def combine_ranks(units: float, seconds: float, world: int, device=None):
    """Whole-job figures of a replicated run: the units all ranks processed and the slowest
    rank's time (all_reduce SUM / MAX over the default process group); the inputs
    themselves when world == 1."""
    if world <= 1:
        return float(units), float(seconds)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(units)], dtype=torch.float64, device=device)
    s = torch.tensor([float(seconds)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.SUM)
    dist.all_reduce(s, op=dist.ReduceOp.MAX)
    return float(t.item()), float(s.item())


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def make_workload(n_reads: int, rank: int, truncate: int = 0, native: bool = True):
    """The batch's graph and extensions.  native=False builds the graph with the Python
    restatement of the builder (tests/gfa_restatement.py, array for array the native
    builder's graph), so that a process timing the CPU implementation never loads the
    product's library."""
    from graphaligner_gb300 import datagen as dg
    from graphaligner_gb300.extend import pack_batch
    vg = dg.batch_vg(0)
    if native:
        from graphaligner_gb300 import graph as gg
        g = gg.build_from_gfa(vg.to_gfa())
    else:
        sys.path.insert(0, os.path.join(ROOT, "tests"))
        import gfa_restatement
        g = gfa_restatement.build_from_gfa(vg.to_gfa())
    ext = dg.batch_extension_workload(n_reads, graph_seed=0, read_seed=1 + rank)
    seqs = [x[:truncate] for x in ext.seqs] if truncate else ext.seqs
    batch = pack_batch(g, seqs, ext.bignode, ext.offset)
    return g, batch


def workload_config(g, batch, params, world: int) -> dict:
    return {"workload": WORKLOAD, "extensions": int(batch.num), "read_bp": int(batch.seq_len.astype(np.int64).sum()),
            "graph_nodes": int(g.num_nodes), "bandwidth": int(params.bandwidth), "xdrop": int(params.xdrop),
            "l2": "inputs larger than L2 (sequences + DP-table arena written every step)",
            "parallelism": f"replicas{world}"}


def trace_checksums(res, idx) -> np.ndarray:
    """Per extension at idx, a 64-bit checksum of its packed trace items (each item mixed with
    its position, so reordered or shifted items change it); 0 for an empty trace."""
    idx = np.asarray(idx, dtype=np.int64)
    out = np.zeros(len(idx), dtype=np.uint64)
    for a in range(0, len(idx), 4096):
        sel = idx[a:a + 4096]
        lens = res.trace_len[sel].astype(np.int64)
        offs = res.trace_offset[sel].astype(np.int64)
        total = int(lens.sum())
        if total == 0:
            continue
        seg = np.cumsum(lens) - lens
        within = np.arange(total, dtype=np.int64) - np.repeat(seg, lens)
        items = res.trace_items[np.repeat(offs, lens) + within]
        mixed = (items ^ (within.astype(np.uint64) * np.uint64(0x9E3779B97F4A7C15))) * np.uint64(0xBF58476D1CE4E5B9)
        nz = lens > 0
        part = np.zeros(len(sel), dtype=np.uint64)
        part[nz] = np.add.reduceat(mixed, seg[nz])
        out[a:a + 4096] = part
    return out


def result_key(res, idx) -> np.ndarray:
    """(status, score, items, item checksum) per extension at idx: equal keys mean equal results."""
    idx = np.asarray(idx, dtype=np.int64)
    return np.stack([res.status[idx].astype(np.int64), res.score[idx].astype(np.int64),
                     res.trace_len[idx].astype(np.int64), trace_checksums(res, idx).view(np.int64)])


def aligned_bp(res) -> int:
    """Read bp covered by the successful extensions: seqPos of the alignment end + 1
    (the first trace item in DP order)."""
    total = 0
    ok = np.nonzero(res.status == 0)[0]
    first = res.trace_items[res.trace_offset[ok].astype(np.int64)]
    total = int(((first >> np.uint64(39)).astype(np.int64)).sum())
    return total


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""

    FIELDS = "clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 7:
                continue
            try:
                sm.append(float(f[0]))
                mx = max(mx, float(f[1]))
            except ValueError:
                continue
            for name, v in zip(names, f[3:7]):
                if v.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx or None,
                "reasons": sorted(reasons), "samples": len(sm)}


def cpu_baseline(g, batch, params, sample_bp: float, threads: int):
    """The oracle port of getReverseTraceFromSeed on the host cores over a bounded
    sample (every k-th extension until sample_bp read bp), all threads."""
    import oracle
    from graphaligner_gb300.extend import pack_batch
    oracle.build(reference=False)
    lens = batch.seq_len.astype(np.int64)
    step = max(1, int(lens.sum() / sample_bp))
    idx = np.arange(0, batch.num, step)
    seqs = [bytes(batch.seq[int(batch.seq_offset[i]):int(batch.seq_offset[i]) + int(lens[i])]) for i in idx]
    sub = batch.subset(idx)
    t = time.perf_counter()
    res = oracle.extend(g, params, sub, threads=threads)
    dt = time.perf_counter() - t
    bp = aligned_bp(res)
    return {"value": bp / dt, "unit": UNIT, "cores": threads, "kind": "port", "seconds": dt,
            "sample": f"{len(idx)} of {batch.num} extensions (every {step}th, {int(lens[idx].sum())} read bp), oracle restatement in C++, {threads} threads, {dt:.1f} s"}, res, idx


def repo_libraries_loaded() -> list:
    """The shared libraries under this repository that this process has mapped (/proc/self/maps)."""
    found = set()
    try:
        for line in open("/proc/self/maps"):
            path = line.split()[-1] if len(line.split()) >= 6 else ""
            if path.endswith(".so") and os.path.realpath(path).startswith(os.path.realpath(ROOT) + os.sep):
                found.add(os.path.relpath(os.path.realpath(path), os.path.realpath(ROOT)))
    except OSError:
        pass
    return sorted(found)


def run_reference(args, rank, world):
    """The reference arm: the CPU implementation of the path on this machine's host cores.  It
    builds its graph with the Python restatement and times the oracle, so the product's
    library is never loaded in this process."""
    if rank != 0:
        return
    from graphaligner_gb300.extend import ExtendParams
    g, batch = make_workload(args.reads, 0, args.truncate, native=False)
    params = ExtendParams(bandwidth=10)
    threads = os.cpu_count() or 1
    vals, secs = [], []
    for i in range(args.warmup + args.steps):
        cb, _, _ = cpu_baseline(g, batch, params, args.cpu_sample_bp, threads)
        if i >= args.warmup:
            vals.append(cb["value"])
            secs.append(cb["seconds"])
    v = statistics.median(vals)
    line = {"metric": METRIC, "value": v, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": statistics.median(secs) * 1e3, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "u64", "data": "synthetic (seeded generator; graph, reads and seeds as the workload describes)",
            "impl": "reference", "config": workload_config(g, batch, params, world),
            "cpu_baseline": {"value": v, "unit": UNIT, "cores": threads, "kind": "port", "sample": cb["sample"]},
            "e2e": {"value": v, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "repo_libraries_loaded": repo_libraries_loaded(),
            "note": "the reference's own C++ source is not present where this runs; the oracle restatement (bit-exact with it on the golden vectors) is timed; a step is the bounded sample of the batch named in cpu_baseline.sample"}
    print(json.dumps(line), flush=True)


READ_WORKLOADS = {
    "reads-vg": "read-level -x vg: 50 kbp VG (bubble/200 bp, 70% SNP, 30% indel 1-20 bp), 200 reads U[5,15] kbp at 10% error",
    "reads-dbg": "read-level -x dbg: k=63 dBG of a 10 Mbp genome + 200 copies of a 5 kbp repeat (1-3% div.) + 400 tandem arrays (period 2-50), 20 kbp reads at 12% error",
    "pipeline": "read-level -x vg: 50 Mbp VG (variant/100 bp, 70% SNP, 30% indel 1-50 bp), reads log-normal N50 ~20 kbp [0.5,100] kbp at U[5,15]% error",
    "serve": "serving -x dbg: the reads-dbg graph resident, reads log-normal N50 ~20 kbp [0.5,100] kbp at U[5,15]% error, Poisson arrivals",
}


def make_read_workload(name: str, n_reads: int):
    """(graph, names, seqs, preset name, arena bytes) of a read-level workload."""
    from graphaligner_gb300 import datagen as dg
    from graphaligner_gb300 import graph as gg
    if name == "reads-vg":
        vg = dg.small_vg(0)
        reads = dg.small_vg_reads(vg, n_reads or 200, 1)
        # the same graph as the reference built it (its numbering, component and chain order)
        golden = os.path.join(ROOT, "tests", "golden", "vg50k_graph.gag.gz")
        if os.path.exists(golden):
            import gzip
            import tempfile
            with tempfile.NamedTemporaryFile(suffix=".gag") as f:
                f.write(gzip.open(golden).read())
                f.flush()
                return gg.load_gag(f.name), reads, "vg"
        return gg.build_from_gfa(vg.to_gfa()), reads, "vg"
    if name in ("reads-dbg", "serve"):
        genome = dg.stress_dbg_genome(0)
        g = gg.build_from_gfa(dg.compact_dbg(genome, 63))
        if name == "reads-dbg":
            reads = dg.dbg_reads(genome, n_reads or 2000, 20_000, 0.12, 1)
        else:
            reads = dg.sample_genome_reads(genome, n_reads or 4000, 2, dg.lognormal_length(15_600, 0.7, 500, 100_000),
                                           dg.uniform_error(0.05, 0.15))
        return g, reads, "dbg"
    if name == "pipeline":
        vg = dg.make_variation_graph(50_000_000, 100, 0.7, 50, 0)
        reads = dg.sample_reads(vg, n_reads or 50_000, 1, dg.lognormal_length(15_600, 0.7, 500, 100_000), dg.uniform_error(0.05, 0.15))
        return gg.build_from_gfa(vg.to_gfa()), reads, "vg"
    raise ValueError(name)


def run_reads(args):
    """Read-level lines: seeding + seed loops + extensions + selection + GAF through ga_align_reads
    (or the ga_server_* loop for 'serve'), host buffers in, GAF text out."""
    import torch
    torch.cuda.set_device(0)
    from graphaligner_gb300 import build
    from graphaligner_gb300.align import Aligner, preset
    from graphaligner_gb300.extend import DeviceGraph, Extender
    build()
    t0 = time.perf_counter()
    g, reads, preset_name = make_read_workload(args.workload, args.reads_n)
    gen_s = time.perf_counter() - t0
    names = [r.name for r in reads]
    seqs = [r.seq for r in reads]
    read_bp = int(sum(len(s) for s in seqs))
    arena = int(args.arena_gb * (1 << 30)) if args.arena_gb else int(min(96 << 30, max(4 << 30, read_bp * 24)))
    t0 = time.perf_counter()
    dgraph = DeviceGraph(g)
    ext = Extender(dgraph, arena_bytes=arena)
    aligner = Aligner(ext, g, preset(preset_name, multiseed=args.multiseed))
    index_s = time.perf_counter() - t0
    line = {"metric": METRIC, "unit": UNIT, "n_gpus": 1, "higher_is_better": True, "dtype": "u64",
            "data": "synthetic (seeded generator)", "config": {"workload": READ_WORKLOADS[args.workload], "reads": len(seqs),
            "read_bp": read_bp, "graph_nodes": g.num_nodes, "preset": preset_name, "multiseed_dp": bool(args.multiseed)},
            "workload_gen_s": gen_s, "graph_upload_and_index_s": index_s}
    if args.workload == "serve":
        with ClockSampler(0) as clocks:
            line.update(run_serving(args, aligner, names, seqs))
        line["clocks"] = clocks.summary()
    else:
        # warm-up on a slice, then timed passes over all reads
        aligner.align(names[:64], seqs[:64])
        with ClockSampler(0) as clocks:
            times = []
            for _ in range(max(1, args.steps)):
                t = time.perf_counter()
                gaf = aligner.align(names, seqs)
                times.append(time.perf_counter() - t)
        st = aligner.stats()
        wall = statistics.median(times)
        line.update({"value": st["bp_aligned"] / wall, "steps": len(times), "warmup": 1, "ms_per_step": wall * 1e3,
                     "gcups": st["cell_steps"] * 64 / (st["extend_ms"] / 1e3) / 1e9 if st["extend_ms"] else None,
                     "stats": st, "gaf_bytes": len(gaf), "clocks": clocks.summary(),
                     "e2e": {"value": st["bp_aligned"] / wall, "unit": UNIT, "h2d_bytes_per_step": read_bp, "d2h_bytes_per_step": len(gaf)}})
        if args.workload == "reads-vg":
            import gzip
            golden = os.path.join(ROOT, "tests", "golden", "vg50k_ms_b10.gaf.gz" if args.multiseed else "vg50k_b10.gaf.gz")
            if os.path.exists(golden):
                line["gaf_identical_to_reference"] = gzip.open(golden, "rt").read() == gaf
        line["index"] = {k: v for k, v in aligner.index().items()}
        if not args.no_cpu_baseline:
            line["cpu_baseline"], line["cpu_sample_gaf_identical"], host_index = read_cpu_baseline(g, names, seqs, preset_name, gaf,
                                                                                                  args.cpu_reads, args.multiseed)
            line["index"]["identical_to_host_build"] = index_checksums(aligner) == host_index.pop("checksums")
            line["index"].update(host_index)
    print(json.dumps(line), flush=True)


def index_checksums(aligner):
    """sum of v[i] * (2i + 1) mod 2^64 over each array of the GPU-built index, with maxCount
    and the sizes (the harness's indexdump prints the same for the host build)."""
    info, keys, start, pos = aligner.index(arrays=True)

    def s(v):
        return int(np.sum(v * (2 * np.arange(len(v), dtype=np.uint64) + 1), dtype=np.uint64))
    return [info["max_count"], info["num_keys"], info["num_positions"], s(keys), s(start), s(pos)]


def read_cpu_baseline(g, names, seqs, preset_name, gaf, n_sample, multiseed=False):
    """The same read-level flow on the host cores in the reference's worker shape
    (Aligner.cpp:777-785): one read per thread, each through its seeding and whole seed loop,
    every core busy (tests/harness/pipeline.cpp, the package's host code with the oracle's
    extensions), on an evenly spaced sample of at least four reads per core.  Its GAF lines must
    equal the GPU's lines for those reads."""
    import subprocess
    import tempfile
    from graphaligner_gb300 import graph as gg
    exe = os.path.join(ROOT, "tests", "_build", "pipeline")
    srcs = [os.path.join(ROOT, "tests", "harness", "pipeline.cpp"),
            os.path.join(ROOT, "graphaligner_gb300", "csrc", "readalign.cpp"),
            os.path.join(ROOT, "graphaligner_gb300", "csrc", "seeding.cpp"),
            os.path.join(ROOT, "oracle", "ga_oracle.cpp")]
    os.makedirs(os.path.dirname(exe), exist_ok=True)
    subprocess.run(["g++", "-std=c++17", "-O2", "-o", exe, *srcs, "-lpthread"], check=True)
    cores = os.cpu_count() or 1
    mode = "gafreadsdbg" if preset_name == "dbg" else "gafreads"
    if multiseed:
        # the multiseed DPs and backward extensions of the sample on every core
        mode = "gafmsdbg" if preset_name == "dbg" else "gafms"
    bw = "5" if preset_name == "dbg" else "10"
    n_sample = min(len(seqs), max(n_sample, 4 * cores))
    with tempfile.TemporaryDirectory() as td:
        gag = os.path.join(td, "g.gag")
        gg.save_gag(g, gag)
        # the host index build on all cores, the start-up work the GPU build replaces
        k, w, discard = (19, 30, 0.0002) if preset_name == "dbg" else (15, 20, 0.001)
        fa = os.path.join(td, "r.fa")
        open(fa, "w").write(">x\nA\n")
        f = subprocess.run([exe, gag, fa, "indexdump", str(k), str(w), str(discard), "-"], check=True, capture_output=True, text=True).stdout.split()
        f = dict(zip(f[0::2], (int(v) for v in f[1::2])))
        host_index = {"host_build_ms": f["ms"], "host_build_threads": f["threads"],
                      "checksums": [f["maxCount"], f["keys"], f["positions"], f["sumKeys"], f["sumStart"], f["sumPos"]]}
        # an evenly spaced sample, grown fourfold until its seed loops take 2.5 s or more
        while True:
            idx = list(range(0, len(seqs), max(1, len(seqs) // n_sample)))[:n_sample]
            with open(fa, "w") as fh:
                for i in idx:
                    fh.write(f">{names[i]}\n{seqs[i].decode()}\n")
            out = subprocess.run([exe, gag, fa, mode, bw, "-", str(cores)], check=True, capture_output=True, text=True)
            bp, dt = 0, 1e-9
            for ln in out.stderr.splitlines():
                if ln.startswith("rounds "):
                    fl = ln.split()
                    bp = int(fl[5])
                    dt = float(fl[9])      # seeding + seed loops + GAF, after the index build
            if dt >= 2.5 or n_sample >= len(seqs):
                break
            n_sample = min(len(seqs), n_sample * 4)
    want = {names[i] for i in idx}
    gpu_lines = [ln for ln in gaf.splitlines(keepends=True) if ln.split("\t", 1)[0] in want]
    cpu_lines = out.stdout.splitlines(keepends=True)
    return ({"value": bp / dt, "unit": UNIT, "cores": cores, "kind": "port",
             "sample": f"{len(idx)} of {len(seqs)} reads (evenly spaced), " + (
                 f"the multiseed DPs and then the backward extensions, reads across {cores} threads; the package's host read-level code with the oracle restatement's multiseed DP and extensions"
                 if multiseed else
                 f"one read per thread through its whole seed loop on {cores} threads (the reference's worker shape); the package's host read-level code with the oracle restatement's extensions")
             + f", {dt:.1f} s after the index build"},
            sorted(gpu_lines) == sorted(cpu_lines), host_index)


def run_serving(args, aligner, names, seqs):
    """Poisson arrivals at each rate of --rates (reads/s); p50/p99 submit->GAF latency and
    throughput, and the plain per-read form (one ga_align_reads call per read) on a sample."""
    from graphaligner_gb300.serve import Server
    rng = np.random.default_rng(2)
    out = {"sweep": []}
    rates = [float(x) for x in args.rates.split(",")]
    pos = 0
    for rate in rates:
        # about --serve-seconds of arrivals per rate, reads taken in order from the workload
        n = int(max(args.serve_min_reads, rate * args.serve_seconds))
        idx = [(pos + k) % len(seqs) for k in range(n)]
        pos += n
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(idx)))
        got = {}
        with Server(aligner) as srv:
            t0 = time.perf_counter()
            for k, i in enumerate(idx):
                delay = arrivals[k] - (time.perf_counter() - t0)
                if delay > 0:
                    time.sleep(delay)
                srv.submit(names[i], seqs[i])
                for r in srv.poll():
                    got[r.ticket] = r
            while len(got) < len(idx):
                for r in srv.poll(wait_ms=200):
                    got[r.ticket] = r
            span = time.perf_counter() - t0
            st = srv.stats()
        lat = np.array([r.latency_ms for r in got.values()])
        bp = sum(r.bp_aligned for r in got.values())
        out["sweep"].append({"offered_reads_per_s": rate, "reads": len(idx), "achieved_reads_per_s": len(idx) / span,
                             "read_bp_aligned_per_s": bp / span, "p50_ms": float(np.percentile(lat, 50)),
                             "p99_ms": float(np.percentile(lat, 99)), "max_ms": float(lat.max()),
                             "queue_p99_ms": float(np.percentile([r.queue_ms for r in got.values()], 99)),
                             "rounds": st["rounds"], "mixed_rounds": st["mixed_rounds"], "max_in_flight": st["max_in_flight"],
                             "failed": int(sum(1 for r in got.values() if r.status != 0))})
    # plain form: each read alone through ga_align_reads, back to back
    sample = list(range(0, len(seqs), max(1, len(seqs) // args.plain_reads)))[:args.plain_reads]
    lat = []
    bp = 0
    t0 = time.perf_counter()
    for i in sample:
        t = time.perf_counter()
        aligner.align([names[i]], [seqs[i]])
        lat.append((time.perf_counter() - t) * 1e3)
        bp += aligner.stats()["bp_aligned"]
    span = time.perf_counter() - t0
    out["plain_per_read"] = {"reads": len(sample), "reads_per_s": len(sample) / span, "read_bp_aligned_per_s": bp / span,
                             "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
    best = max(out["sweep"], key=lambda x: x["read_bp_aligned_per_s"])
    out["value"] = best["read_bp_aligned_per_s"]
    return out


def main():
    args = parse()
    rank, world, local = dist_env()
    if args.impl == "reference":
        run_reference(args, rank, world)
        return
    if args.workload != "extend":
        run_reads(args)
        return
    import torch
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    from graphaligner_gb300 import build
    from graphaligner_gb300._lib import lib, check
    from graphaligner_gb300 import _abi
    from graphaligner_gb300._abi import ptr
    from graphaligner_gb300.extend import DeviceGraph, Extender, ExtendParams, alloc_results, results_desc
    build()
    L = lib()

    # ---- workload (host) ----
    t0 = time.perf_counter()
    g, batch = make_workload(args.reads, rank, args.truncate)
    gen_s = time.perf_counter() - t0
    params = ExtendParams(bandwidth=10)

    # pinned host buffers of the end-to-end measurement, allocated before anything else
    # makes large host allocations (the copies' speed depends on how these pages lie)
    def pinned(nbytes):
        p = ctypes.c_void_p()
        check(L.ga_host_alloc(ctypes.c_uint64(nbytes), ctypes.byref(p)))
        return p
    host_bufs = []
    def pinned_like(a):
        p = pinned(a.nbytes)
        host_bufs.append(p)
        arr = np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)), shape=(a.nbytes,)).view(a.dtype)
        arr[:] = a
        return arr
    def pinned_zeros(count, dtype):
        nbytes = int(count) * np.dtype(dtype).itemsize
        p = pinned(nbytes)
        host_bufs.append(p)
        ctypes.memset(p, 0, nbytes)
        return np.ctypeslib.as_array(ctypes.cast(p, ctypes.POINTER(ctypes.c_uint8)), shape=(nbytes,)).view(dtype)
    from graphaligner_gb300.extend import PackedBatch, BatchResult
    hb = PackedBatch(pinned_like(batch.seq), pinned_like(batch.seq_offset), pinned_like(batch.seq_len),
                     pinned_like(batch.start_node), pinned_like(batch.start_offset), pinned_like(batch.trace_offset),
                     pinned_like(batch.trace_capacity))
    hr = BatchResult(pinned_zeros(batch.num, np.int32), pinned_zeros(batch.num, np.int32), pinned_zeros(batch.num, np.uint32),
                     pinned_zeros(max(batch.total_items, 1), np.uint64), hb.trace_offset, pinned_zeros(batch.num, np.uint64))
    h2d = int(hb.seq.nbytes + batch.num * (8 + 4 + 4 + 4 + 8 + 4 + 4))
    d2h = int(batch.num * (4 + 4 + 4 + 8) + batch.total_items * 8)

    dgraph = DeviceGraph(g, device=local)
    arena = int(min(64 << 30, max(4 << 30, int(batch.seq_len.astype(np.int64).sum()) * 24)))
    if args.arena_gb:
        arena = int(args.arena_gb * (1 << 30))
    ext = Extender(dgraph, arena_bytes=arena)
    # launch shape for this workload class, tuned before the timed region on an independent batch
    # of the same class and size (other read seed)
    if args.autotune:
        _, tune_batch = make_workload(args.reads, rank + 100, args.truncate)
        tuning = ext.autotune(params, tune_batch, sample_every=1)
        tuning["tuned_on"] = f"an independent batch of {tune_batch.num} extensions (read seed {rank + 101})"
        del tune_batch
    else:
        tuning = {"chosen": ext.launch_shape().as_dict()}

    # ---- device-resident batch ----
    dev = torch.device("cuda", local)
    def to_dev(a, dt):
        return torch.from_numpy(np.ascontiguousarray(a).view(dt)).to(dev)
    d_seq = to_dev(batch.seq, np.uint8)
    d_soff = to_dev(batch.seq_offset, np.int64)
    d_slen = to_dev(batch.seq_len, np.int32)
    d_sn = to_dev(batch.start_node, np.int32)
    d_so = to_dev(batch.start_offset, np.int32)
    d_toff = to_dev(batch.trace_offset, np.int64)
    d_tcap = to_dev(batch.trace_capacity, np.int32)
    n = batch.num
    d_status = torch.empty(n, dtype=torch.int32, device=dev)
    d_score = torch.empty(n, dtype=torch.int32, device=dev)
    d_tlen = torch.empty(n, dtype=torch.int32, device=dev)
    d_items = torch.empty(max(batch.total_items, 1), dtype=torch.int64, device=dev)
    d_steps = torch.empty(n, dtype=torch.int64, device=dev)
    u8, u32, u64, i32 = ctypes.c_uint8, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_int32
    def P(t, c):
        return ctypes.cast(ctypes.c_void_p(t.data_ptr()), ctypes.POINTER(c))
    dbatch = _abi.BatchDesc(n, P(d_seq, u8), P(d_soff, u64), P(d_slen, u32), P(d_sn, u32), P(d_so, u32), P(d_toff, u64), P(d_tcap, u32))
    dres = _abi.Results(P(d_status, i32), P(d_score, i32), P(d_tlen, u32), P(d_items, u64), P(d_steps, u64))
    cparams = params.c()
    stream = torch.cuda.current_stream(dev)

    def device_step():
        check(L.ga_extend_batch_device(ext.handle, ctypes.byref(cparams), ctypes.byref(dbatch), ctypes.byref(dres),
                                       ctypes.c_void_p(stream.cuda_stream)))
        ms = ctypes.c_float()
        check(L.ga_extender_last_kernel_ms(ext.handle, ctypes.byref(ms)))
        launches = ctypes.c_uint32()
        check(L.ga_extender_last_launches(ext.handle, ctypes.byref(launches)))
        return ms.value, launches.value

    for _ in range(args.warmup):
        device_step()
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    kernel_ms, launches = [], 0
    with ClockSampler(local) as clocks:
        torch.cuda.synchronize()
        wall0 = time.perf_counter()
        for _ in range(args.steps):
            k, nl = device_step()
            kernel_ms.append(k)
            launches += nl
        torch.cuda.synchronize()
        wall = time.perf_counter() - wall0
    kernel_s = sum(kernel_ms) / 1e3
    # DP-table bytes of the timed batch (later calls below overwrite the extender's figure)
    arena_bytes = ctypes.c_uint64()
    check(L.ga_extender_last_arena_bytes(ext.handle, ctypes.byref(arena_bytes)))

    # results of the last step
    res = alloc_results(batch)
    res.status[:] = d_status.cpu().numpy()
    res.score[:] = d_score.cpu().numpy()
    res.trace_len[:] = d_tlen.cpu().numpy().view(np.uint32)
    res.cell_steps[:] = d_steps.cpu().numpy().view(np.uint64)
    res.trace_items[:] = d_items.cpu().numpy().view(np.uint64)
    bp = aligned_bp(res)
    steps_total = int(res.cell_steps.sum())
    statuses = {int(s): int(c) for s, c in zip(*np.unique(res.status, return_counts=True))}

    job_bp, kernel_s = combine_ranks(bp * args.steps, kernel_s, world, dev)
    value = job_bp / kernel_s
    ms_per_step = kernel_s * 1e3 / args.steps
    job_steps, _ = combine_ranks(steps_total * args.steps, kernel_s, world, dev)
    gcups = job_steps * 64 / kernel_s / 1e9

    # ---- end to end through the host-buffer C ABI, pinned host memory ----
    ext.run(params, hb, hr)   # warm the staging buffers
    e2e_times, e2e_parts = [], []
    for _ in range(max(1, min(args.steps, 3))):
        torch.cuda.synchronize()
        t = time.perf_counter()
        ext.run(params, hb, hr)
        e2e_times.append(time.perf_counter() - t)
        # where the step's time went: copies in, kernels, copies out (CUDA events of the call)
        h2d_ms, d2h_ms, k_ms = ctypes.c_float(), ctypes.c_float(), ctypes.c_float()
        check(L.ga_extender_last_copy_ms(ext.handle, ctypes.byref(h2d_ms), ctypes.byref(d2h_ms)))
        check(L.ga_extender_last_kernel_ms(ext.handle, ctypes.byref(k_ms)))
        e2e_parts.append((h2d_ms.value, k_ms.value, d2h_ms.value))
    # every extension's status, score and trace (checksum of its packed items) against the device run
    e2e_same = bool(np.array_equal(result_key(hr, np.arange(n)), result_key(res, np.arange(n))))
    job_bp_e2e, e2e_s = combine_ranks(bp, statistics.median(e2e_times), world, dev)
    e2e_value = job_bp_e2e / e2e_s

    # ---- the plain form: one launch per extension, waited for, on a sample ----
    plain = None
    if rank == 0 and args.plain_sample > 0:
        pidx = np.unique(np.linspace(0, n - 1, min(n, args.plain_sample)).astype(np.int64))
        def Pi(t, c, i):
            return ctypes.cast(ctypes.c_void_p(t.data_ptr() + i * t.element_size()), ctypes.POINTER(c))
        plain_ms = 0.0
        torch.cuda.synchronize()
        t = time.perf_counter()
        for i in pidx:
            i = int(i)
            b1 = _abi.BatchDesc(1, P(d_seq, u8), Pi(d_soff, u64, i), Pi(d_slen, u32, i), Pi(d_sn, u32, i), Pi(d_so, u32, i),
                                Pi(d_toff, u64, i), Pi(d_tcap, u32, i))
            r1 = _abi.Results(Pi(d_status, i32, i), Pi(d_score, i32, i), Pi(d_tlen, u32, i), P(d_items, u64), Pi(d_steps, u64, i))
            check(L.ga_extend_batch_device(ext.handle, ctypes.byref(cparams), ctypes.byref(b1), ctypes.byref(r1),
                                           ctypes.c_void_p(stream.cuda_stream)))
            ms = ctypes.c_float()
            check(L.ga_extender_last_kernel_ms(ext.handle, ctypes.byref(ms)))
            plain_ms += ms.value
        torch.cuda.synchronize()
        plain_wall = time.perf_counter() - t
        pres = alloc_results(batch)
        pres.status[:] = d_status.cpu().numpy()
        pres.score[:] = d_score.cpu().numpy()
        pres.trace_len[:] = d_tlen.cpu().numpy().view(np.uint32)
        pres.trace_items[:] = d_items.cpu().numpy().view(np.uint64)
        same = bool(np.array_equal(result_key(pres, pidx), result_key(res, pidx)))
        del pres
        first = res.trace_items[res.trace_offset[pidx].astype(np.int64)]
        pbp = int(np.where(res.status[pidx] == 0, (first >> np.uint64(39)).astype(np.int64), 0).sum())
        plain = {"value": pbp / plain_wall, "unit": UNIT, "kernel_only_value": pbp / (plain_ms / 1e3),
                 "sample": f"{len(pidx)} of {n} extensions, evenly spaced, {pbp} aligned bp",
                 "batched_over_plain": value / (pbp / plain_wall), "same_results": same,
                 "form": "ga_extend_batch_device with one extension per call (one fill+traceback launch, waited for), batch resident in HBM"}

    # ---- CPU baseline last (host threads, no process pool: the GPU timings above are not
    # disturbed by its large host allocations); its sample must agree with the GPU ----
    cpu = None
    cpu_agree = None
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        cpu, cpu_res, cpu_idx = cpu_baseline(g, batch, params, args.cpu_sample_bp, os.cpu_count() or 1)
        cpu_agree = bool(np.array_equal(result_key(cpu_res, np.arange(len(cpu_idx))), result_key(res, cpu_idx)))

    # ---- roofline ----
    peaks = json.load(open(PEAKS)) if os.path.exists(PEAKS) else {}
    hbm_peak = peaks.get("hbm_gbs", 6800.0)
    step_s = statistics.median(kernel_ms) / 1e3
    # the bound: the Myers column steps of the fill at 40 INT32 ops each (20 u64 ops,
    # GraphAlignerBitvectorCommon.h:242-262) against the INT32 issue rate measured on this GPU
    int_peak = ctypes.c_double()
    check(L.ga_measure_int32_peak(local, ctypes.byref(int_peak)))
    alu_achieved = steps_total * INT32_OPS_PER_STEP / step_s
    # beside it, HBM: algorithmic bytes per step are the reads, the DP tables (written by the fill,
    # read by the traceback) and the trace items written; DRAM traffic per read bp comes from an
    # ncu capture of both kernels on a smaller case of the same batch, scaled by read bp
    read_bp_total = int(batch.seq_len.astype(np.int64).sum())
    alg_bytes = int(batch.seq.nbytes + 2 * arena_bytes.value + int(res.trace_len.astype(np.int64).sum()) * 8)
    achieved_gbs = alg_bytes / step_s / 1e9
    traffic = None
    tpath = os.path.join(ROOT, "profiles", "extension_kernels_traffic.json")
    if os.path.exists(tpath):
        t = json.load(open(tpath))
        traffic = t.get("bytes_per_read_bp", 0) * read_bp_total

    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u64",
        "data": "synthetic (seeded generator; graph, reads and seeds as the workload describes)",
        "config": workload_config(g, batch, params, world),
        "gcups": gcups,
        "launch_shape": tuning,
        "gpu_launches": launches,
        "statuses": statuses,
        "kernel_ms": statistics.median(kernel_ms), "wall_s_timed_region": wall,
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                "seconds_per_step": statistics.median(e2e_times), "same_results": e2e_same,
                "ms_h2d_kernel_d2h": [[round(v, 1) for v in part] for part in e2e_parts]},
        "roofline": {"bound": "int32", "achieved": alu_achieved / 1e12, "peak": int_peak.value / 1e12, "unit": "Tint32op/s",
                     "frac": alu_achieved / int_peak.value, "traffic": traffic,
                     "kernel": "fill_kernel + trace_kernel (one step: both launches)",
                     "ops_per_column_step": INT32_OPS_PER_STEP, "column_steps": steps_total,
                     "peak_source": "ga_measure_int32_peak (independent xor+add chains, this GPU)",
                     "hbm": {"achieved": achieved_gbs, "peak": hbm_peak, "unit": "GB/s", "frac": achieved_gbs / hbm_peak,
                             "algorithmic_bytes": alg_bytes, "traffic_bytes": traffic,
                             "peak_source": "MEASURED_PEAKS.json hbm_gbs" if "hbm_gbs" in peaks else "fallback 6.8 TB/s"}},
        "cpu_baseline": cpu, "cpu_sample_agrees": cpu_agree,
        "plain_per_extension": plain,
        "clocks": clocks.summary(),
        "workload_gen_s": gen_s,
    }
    if rank == 0:
        print(json.dumps(line), flush=True)
    ext.close()
    dgraph.close()
    for p in host_bufs:
        L.ga_host_free(p)
    if world > 1:
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
