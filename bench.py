#!/usr/bin/env python3
"""Benchmark of the GB300 FM-index read-mapping path.

Metric: reads/s of 100 bp reads mapped with at most one error (BWSearch1:
four vector searches + the 1-error helper on both strands, every hit located
with the sampled suffix array and the karyotype), bit-exact to the reference.

Workload (default ``c2``): a seeded 100 Mbp synthetic genome (GC 41 %, plus
5 % of its length as copies of 300 bp elements at 85-95 % identity) and 2 M
reads of 100 bp per GPU with per-base 0.5 % substitutions, 0.02 % insertions
and 0.02 % deletions, capped at one edit per read, from either strand.  The
index is built by this repository's builder at the reference's default
ratios (O table every 64 rows, SA sample every 16 rows).  No public dataset
is used.

One step = one mapping call over the whole read batch.  ``value`` is measured
with the reads already resident in HBM (CUDA events on the library's stream,
L2 flushed with a 256 MiB write before every step); ``e2e`` goes through the
C ABI call ``bwt_gpu_search_batch`` with pinned host reads and host result
arrays, host<->device copies inside the timed region.

Secondary legs in the same JSON line (not the headline): the serving form
(p50/p99 latency under Poisson load), CAL generation, the alignment-list
entry points, and the k-error block search of bwt_map_inexact_read_2
(``block_search``: its kernels' device time, the bwt_gpu_block_search call with
host buffers, a sector census, and bwt_map_inexact_array_list_2).

After the timed steps the oracle (the C restatement in oracle/, pinned
bit-exact to the reference's search code) maps the whole batch on the host
cores, or an evenly spread sample of at least 50 000 reads where the whole
batch would take longer than ~30 s; its time is ``cpu_baseline`` and its
output is compared record for record with the timed steps' outputs of the
plain form, the batched form and the e2e call (``parity``).  The batched
form's autotuner runs first on a held-out batch of the same workload (another
seed), not on the timed reads.

Workloads: ``c2`` (default, above), ``c1`` (4 Mbp i.i.d. genome, 200k x 100
bp error-free reads, plain exact search on both strands + locate), ``c3``
(4M reads of 36-250 bp), ``c4`` (3.1 Gbp genome, 20M x 150 bp reads).

``--impl reference`` times the reference algorithm on the host cores (the C
restatement in oracle/, OpenMP over all cores) on a bounded sample of the
same workload.

Multi-GPU: reads are independent, so each rank maps its own read batch
against its own copy of the index (weak scaling, no collective on the data
path); rank 0 prints the line.
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT / "hpg-libs_gb300"))
sys.path.insert(0, str(ROOT))

METRIC = "reads/s, 100bp ≤1 err bit-exact; batched+served vs plain, 1 GB300; p50/p99 ms"

WORKLOADS = {
    "c2": dict(desc="100 Mbp genome (GC 41%, 5% 300 bp repeat copies at 85-95% identity); 2M x 100 bp reads "
                    "per GPU, 0.5%/0.02%/0.02% subst/ins/del per base capped at one edit; BWSearch1 + locate",
               genome="repeats", genome_bp=100_000_000, reads=2_000_000, read_len=100, edits="per_base_capped"),
    "c2_profile": dict(desc="profiling size of c2: the same 100 Mbp genome and index, 200k x 100 bp reads",
                       genome="repeats", genome_bp=100_000_000, reads=200_000, read_len=100,
                       edits="per_base_capped"),
    "c3": dict(desc="100 Mbp genome (as c2); 4M reads of 36-250 bp per GPU (uniform), 30% exact, 50% one "
                    "substitution, 20% one 1-bp indel; BWSearch1 + locate",
               genome="repeats", genome_bp=100_000_000, reads=4_000_000, read_len=(36, 250),
               edits="mix_30_50_20"),
    "c4": dict(desc="3.1 Gbp human-like genome (GC 41%; 10% 300 bp and 17% 6 kbp element copies at 80-98% "
                    "identity, 18% perfect tandem runs of 1-6 bp units, 20-149 bp long); 20M x 150 bp reads per "
                    "GPU at 1% per-base substitution (uncapped, <=1 edit searched); BWSearch1 + locate; index "
                    "built with the GPU builder",
               genome="large", genome_bp=3_100_000_000, reads=20_000_000, read_len=150, edits="subst_1pct"),
    "c1": dict(desc="4 Mbp i.i.d. genome; 200k x 100 bp error-free reads from either strand; plain exact "
                    "search (BWExactSearchBackward on both strands) + locate",
               genome="iid", genome_bp=4_000_000, reads=200_000, read_len=100, edits="none", mode="exact"),
    "small": dict(desc="2 Mbp genome (repeats); 100k x 100 bp reads; BWSearch1 + locate (smoke-size)",
                  genome="repeats", genome_bp=2_000_000, reads=100_000, read_len=100, edits="per_base_capped"),
}

MAX_RESULTS = 1024
SA_RATIO = 16
TUNE_SEED_OFFSET = 1000  # the autotuner's read batch: same workload, another seed (held out from the timed reads)


def wl_mode(wl: dict) -> int:
    from hpgbwt import lib
    return lib.MODE_EXACT if wl.get("mode") == "exact" else lib.MODE_SEARCH1


def bench_config(wl: dict, n_reads: int, world: int, total_bases: int) -> dict:
    """The workload description both arms print (same keys, so the lines compare)."""
    return {"workload": wl["desc"], "genome_bp": wl["genome_bp"], "reads_per_gpu": n_reads,
            "read_len": wl["read_len"], "search": wl.get("mode", "search1"), "max_results": MAX_RESULTS,
            "sa_ratio": SA_RATIO, "o_ratio": 64,
            "l2": f"flushed (256 MiB write) before every step; reads {total_bases / 1e6:.0f} MB > L2",
            "parallelism": f"replica x{world} (reads sharded)"}
SERVE_MAX_BATCH = 1 << 21  # reads per served batch at most
SERVE_LOCATE_LIMIT = 10_000  # serving against the 3.1 Gbp genome: rows per (read, strand) list located at most


def log(*a):
    print(*a, file=sys.stderr, flush=True)


class Dist:
    """Ranks of a torchrun launch: one replica per GPU, reads sharded by rank
    (each rank draws its own seeded batch), no collective on the data path --
    only the timing barrier and max/sum of scalars.  NCCL on GPUs; gloo where
    no GPU is visible (the CPU tests of this logic)."""

    def __init__(self, gpus: int, backend: str | None = None):
        self.world = int(os.environ.get("WORLD_SIZE", "1"))
        self.rank = int(os.environ.get("RANK", "0"))
        self.local = int(os.environ.get("LOCAL_RANK", "0"))
        self.pg = None
        self.device = "cpu"
        if self.world > 1:
            import torch
            import torch.distributed as dist
            backend = backend or ("nccl" if torch.cuda.is_available() else "gloo")
            if backend == "nccl":
                torch.cuda.set_device(self.local)
                self.device = f"cuda:{self.local}"
                dist.init_process_group("nccl", device_id=torch.device("cuda", self.local))
            else:
                dist.init_process_group("gloo")
            self.pg = dist

    def barrier(self):
        if self.pg:
            self.pg.barrier()

    def _reduce(self, v: float, op) -> float:
        import torch
        t = torch.tensor([v], dtype=torch.float64, device=self.device)
        self.pg.all_reduce(t, op=op)
        return float(t.item())

    def max(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.MAX) if self.pg else v

    def sum(self, v: float) -> float:
        return self._reduce(v, self.pg.ReduceOp.SUM) if self.pg else v

    def close(self):
        if self.pg:
            self.pg.destroy_process_group()


def read_seed(rank: int) -> int:
    """Each rank's read batch: the same generator, its own seed (weak scaling)."""
    return 2 + rank


def prepare(wl: dict, rank: int, dist):
    """Genome + index (shared by ranks, cached per call) and this rank's reads."""
    t0 = time.time()
    index_dir, genome, t_gen = genome_and_index(wl, rank, dist)
    reads = make_reads(wl, genome, read_seed(rank))
    log(f"[bench] rank {rank}: genome ({t_gen:.1f}s) + index + reads ready in {time.time() - t0:.1f}s")
    return index_dir, reads, genome


def genome_and_index(wl: dict, rank: int, dist):
    """The workload's genome and the directory of its index (built by rank 0 once
    per cache directory; the 3.1 Gbp genome on rank 0's GPU)."""
    from hpgbwt import lib, synth
    key = f"{wl['genome']}_{wl['genome_bp']}_r{SA_RATIO}"
    base = Path(os.environ.get("HPG_BENCH_CACHE", tempfile.gettempdir())) / "hpgbwt_bench" / key
    t0 = time.time()
    large = wl["genome"] == "large"
    if large:
        genome = synth.genome_large(wl["genome_bp"], 1)
    else:
        genome = synth.genome(wl["genome"], wl["genome_bp"], 1)
    t_gen = time.time() - t0
    if rank == 0 and not (base / "index" / "Si.vec").exists():
        base.mkdir(parents=True, exist_ok=True)
        synth.write_fasta(str(base / "genome.fa"), genome)
        t1 = time.time()
        # the 3.1 Gbp genome is indexed on this rank's GPU (the host builder takes tens of minutes)
        lib.build_index(str(base / "genome.fa"), str(base / "index"), SA_RATIO, device=dist.local if large else -1)
        log(f"[bench] index of {wl['genome_bp'] // 1_000_000} Mbp built in {time.time() - t1:.1f}s "
            f"({'GPU' if large else 'host'} suffix arrays)")
    dist.barrier()
    return str(base / "index"), genome, t_gen


def make_reads(wl: dict, genome, seed: int):
    """A read batch of the workload's shape drawn with `seed`."""
    from hpgbwt import synth
    if wl["edits"] == "subst_1pct":
        return synth.reads_large(genome, wl["reads"], seed, wl["read_len"], 0.01)
    if isinstance(wl["read_len"], tuple):
        lo, hi = wl["read_len"]
        return synth.reads_fast_var(genome, wl["reads"], seed, lo, hi, wl["edits"])
    return synth.reads_fast(genome, wl["reads"], seed, wl["read_len"], wl["edits"])


class ClockSampler:
    """nvidia-smi samples during the timed region."""

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.rows: list[list[str]] = []

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
             "clocks_event_reasons.sw_power_cap")
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thr = threading.Thread(target=self._read, daemon=True)
            self.thr.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([x.strip() for x in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm = []
        mx = None
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            try:
                sm.append(float(r[0]))
                mx = float(r[1])
                for nm, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(nm)
            except (ValueError, IndexError):
                continue
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm), "sm_min_mhz": min(sm) if sm else None}


def measured_peaks() -> tuple[float, str]:
    p = ROOT / "MEASURED_PEAKS.json"
    try:
        return float(json.loads(p.read_text())["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def profiled_traffic(workload: str, kernel: str, tuning: dict) -> tuple[float | None, str | None]:
    """DRAM bytes (read + write) of one search step of `kernel` on this exact
    workload, from the committed one-pass ncu capture of the full-size step
    (profiles/<kernel>_<workload>_traffic.txt: a line "dram_bytes_per_step: B"
    and a line "tuning: k=v ..."), and where it came from; (None, reason) where
    no capture of this workload at this tuning exists."""
    p = ROOT / "profiles" / f"{kernel}_{workload}_traffic.txt"
    if not p.exists():
        return None, None
    val, want = None, {}
    for line in p.read_text().splitlines():
        if line.startswith("dram_bytes_per_step:"):
            try:
                val = float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None, None
        elif line.startswith("tuning:"):
            want = dict(kv.split("=") for kv in line.split(":", 1)[1].split())
    if any(str(tuning.get(k)) != v for k, v in want.items()):
        return None, f"{p.name} was captured at {want}, not at this run's tuning"
    return val, f"ncu capture of this workload's full step at this tuning, {p.name}"


def compare_results(got, want) -> dict:
    """Field-by-field comparison of two flat results of the same reads."""
    out = {"equal": True}
    for name in ("rs_count", "rs_truncated", "hits", "locs"):
        a, b = getattr(got, name), getattr(want, name)
        if len(a) != len(b) or not np.array_equal(a, b):
            out["equal"] = False
            if len(a) != len(b):
                out[name] = f"{len(a)} against {len(b)} records"
            else:
                i = int(np.nonzero(a != b)[0][0])
                out[name] = f"first difference at record {i}"
    return out


def oracle_leg(index_dir: str, reads, mode: int, gpu: dict, seconds: float = 12.0) -> tuple[dict, dict]:
    """The oracle (the C restatement in oracle/, OpenMP over all host cores) on
    the whole batch when that takes under ~30 s, else on an evenly spread sample
    of at least 50 000 reads; its time is the CPU baseline and its output the
    parity check of every GPU result in `gpu` (name -> lib.Result of the whole
    batch, from the timed steps)."""
    from oracle.pyoracle import PortOracle
    ora = PortOracle(index_dir)
    threads = os.cpu_count() or 1
    n_total = len(reads)
    # rate from a probe grown until it runs long enough for the thread start-up not to count
    m = 2000
    while True:
        probe = reads.subset(np.arange(min(m, n_total)))
        t = time.perf_counter()
        ora.search(probe, mode=mode, max_results=MAX_RESULTS, threads=threads)
        dt = max(time.perf_counter() - t, 1e-6)
        rate = len(probe) / dt
        if dt >= 0.5 or len(probe) >= n_total:
            break
        m *= 4
    if rate * 30.0 >= n_total:
        idx = np.arange(n_total)
        what = f"the whole {n_total}-read batch"
    else:
        k = int(min(n_total, max(50_000, rate * seconds)))
        idx = np.unique(np.linspace(0, n_total - 1, k).astype(np.int64))
        what = f"{len(idx)} reads spread evenly over the {n_total}-read batch"
    sample = reads if len(idx) == n_total else reads.subset(idx)
    t = time.perf_counter()
    want = ora.search(sample, mode=mode, max_results=MAX_RESULTS, threads=threads)
    dt = time.perf_counter() - t
    parity = {"reads_checked": int(len(idx)), "of_reads": int(n_total), "sample": what,
              "oracle": "oracle/fm_oracle.c (pinned bit-exact to the reference's own search code)",
              "hits": int(len(want.hits)), "located_rows": int(len(want.locs))}
    eq = True
    for name, res in gpu.items():
        sub = res if len(idx) == n_total else res.subset(idx)
        c = compare_results(sub, want)
        parity[name] = c
        eq = eq and c["equal"]
    parity["equal"] = eq
    base = {"value": round(len(idx) / dt, 1), "unit": "reads/s", "cores": threads, "kind": "port",
            "sample": f"{what}, same index, OpenMP over {threads} host threads ({dt:.1f}s)"}
    if mode == 1:
        # the k-error block search of bwt_map_inexact_read_2 on a smaller sample (~3 s)
        nb = int(min(n_total, max(2000, rate * 3.0)))
        t = time.perf_counter()
        ora.block_search(reads.subset(np.arange(nb)), max_results=MAX_RESULTS, threads=threads)
        dtb = time.perf_counter() - t
        base["block_search"] = {"value": round(nb / dtb, 1), "unit": "reads/s",
                                "sample": f"first {nb} reads, {threads} host threads ({dtb:.1f}s)"}
    ora.close()
    return base, parity


def fetch_result(gi, rs, n: int):
    """Host copy of a device-resident result (bwt_gpu_search_device's output)."""
    from hpgbwt import lib
    hits = np.empty(int(rs.n_hits), dtype=lib.HIT_DTYPE)
    locs = np.empty(int(rs.n_locs), dtype=lib.LOC_DTYPE)
    cnt = np.empty(2 * n, dtype=np.uint32)
    trn = np.empty(2 * n, dtype=np.uint8)
    gi.copy_result(rs, hits.ctypes.data, locs.ctypes.data, cnt.ctypes.data, trn.ctypes.data)
    return lib.Result(hits, locs, cnt, trn)


def _pct(v: list[float], q: float) -> float:
    if not v:
        return float("nan")
    s = sorted(v)
    return s[min(len(s) - 1, max(0, int(round(q / 100.0 * (len(s) - 1)))))]


def serve_run(gi, seq_ptr: int, off_ptr: int, pool_n: int, draw_size, load: float | None, seconds: float,
              rng: np.random.Generator, sat: float | None = None, burst: int = 192, max_batch: int = 1 << 20,
              srv=None) -> dict:
    """One serving measurement through bwt_gpu_server_*: with load None a burst
    of requests submitted at once (saturated throughput); else Poisson arrivals
    offering `load` x `sat` reads/s for `seconds`.  Requests are slices of a
    pinned read pool; latency is submit (scheduled arrival, when the submitter
    lags) to results readable in host memory.  A server passed in is kept open
    (a long-running server, its result buffers already grown); else one is
    made for this run."""
    import ctypes
    import queue
    from hpgbwt import lib
    L = gi.lib
    own = srv is None
    if own:
        srv = lib.Server(gi, max_batch_reads=max_batch, max_results=MAX_RESULTS)
    st0 = srv.stats()
    pend: queue.Queue = queue.Queue()
    lat: list[float] = []
    done_reads = [0]
    t_done = [0.0]

    def waiter():
        rs = lib.ResultSetC()
        lt = ctypes.c_double()
        while True:
            item = pend.get()
            if item is None:
                return
            tk, n, lag = item
            if L.bwt_gpu_server_wait(srv.handle, tk, ctypes.byref(rs), ctypes.byref(lt), -1) != 0:
                raise RuntimeError(L.bwt_gpu_last_error().decode())
            lat.append(lt.value + lag)
            done_reads[0] += n
            t_done[0] = time.perf_counter()
            L.bwt_gpu_server_release(srv.handle, tk)

    def submit(n: int) -> int:
        start = int(rng.integers(0, pool_n - n + 1))
        t = ctypes.c_uint64()
        if L.bwt_gpu_server_submit(srv.handle, seq_ptr, off_ptr + 8 * start, n, ctypes.byref(t)) != 0:
            raise RuntimeError(L.bwt_gpu_last_error().decode())
        return t.value

    th = threading.Thread(target=waiter, daemon=True)
    th.start()
    import torch
    clk = ClockSampler(torch.cuda.current_device()) if load is not None else None
    if clk:
        clk.__enter__()
    t0 = time.perf_counter()
    offered = None
    n_req = 0
    if load is None:
        for _ in range(burst):
            n = draw_size()
            pend.put((submit(n), n, 0.0))
            n_req += 1
    else:
        mean_n = float(np.mean([draw_size() for _ in range(4096)]))
        rate = load * sat / mean_n  # requests per second
        offered = load * sat
        t_next = t0
        while t_next - t0 < seconds:
            t_next += rng.exponential(1.0 / rate)
            while True:
                now = time.perf_counter()
                if now >= t_next:
                    break
                time.sleep(min(t_next - now, 0.0005))
            n = draw_size()
            tk = submit(n)
            pend.put((tk, n, max(0.0, time.perf_counter() - t_next) * 1e3))
            n_req += 1
    pend.put(None)
    th.join()
    if clk:
        clk.__exit__(None, None, None)
    st = srv.stats()
    if own:
        srv.close()
    span = t_done[0] - t0
    nb = st["batches"] - st0["batches"]
    out = {"requests": n_req, "reads": done_reads[0], "achieved_reads_per_s": round(done_reads[0] / span, 1),
           "p50_ms": round(_pct(lat, 50), 3), "p99_ms": round(_pct(lat, 99), 3), "max_ms": round(max(lat), 3),
           "mean_ms": round(float(np.mean(lat)), 3), "batches": int(nb),
           "mean_batch_reads": round((st["reads"] - st0["reads"]) / max(1, nb), 1),
           "mean_batch_requests": round((st["requests"] - st0["requests"]) / max(1, nb), 2),
           "max_batch_requests": int(st["max_batch_requests"]), "pool_regrowths": int(st["regrowths"] - st0["regrowths"]),
           "plan_hbm_bytes": int(st["plan_bytes"]), "hbm_budget_bytes": int(st["hbm_budget"])}
    if offered is not None:
        out = {"offered_load": load, "offered_reads_per_s": round(offered, 1), **out, "clocks": clk.summary()}
    return out


def serve_cases(gi, cases, log, locate_limit: int, rng: np.random.Generator, max_batch: int) -> dict:
    """Each case (name, ReadSet pool, request-size draw) on one server, as a
    long-running service: a warm-up burst (it captures the plans the case needs
    and grows the result buffers), the saturated rate of a burst of about 48M
    reads, then Poisson arrivals at 10-90 % of that rate for 2 s each."""
    import torch
    from hpgbwt import lib
    res = {"locate_limit": locate_limit, "max_batch_reads": max_batch}
    gi.set_locate_limit(locate_limit)
    for name, pool, draw in cases:
        sq = torch.from_numpy(pool.seq).pin_memory()
        of = torch.from_numpy(pool.offsets.view(np.int64)).pin_memory()
        mean_n = float(np.mean([draw() for _ in range(4096)]))
        burst = max(192, int(48e6 / mean_n))
        args = (gi, sq.data_ptr(), of.data_ptr(), len(pool), draw)
        srv = lib.Server(gi, max_batch_reads=max_batch, max_results=MAX_RESULTS)
        serve_run(*args, None, 0, rng, burst=burst, srv=srv)
        sat = serve_run(*args, None, 0, rng, burst=burst, srv=srv)
        sweep = {}
        for load in (0.1, 0.3, 0.5, 0.7, 0.9):  # offered load as a fraction of the saturated rate
            sweep[f"{int(load * 100)}pct"] = serve_run(*args, load, 2.0, rng, sat=sat["achieved_reads_per_s"],
                                                       srv=srv)
        srv.close()
        loaded = sweep["70pct"]
        res[name] = {"saturated_reads_per_s": sat["achieved_reads_per_s"], "saturated_burst_requests": burst,
                     "saturated_mean_batch_reads": sat["mean_batch_reads"], "at_70pct_load": loaded,
                     "load_sweep": {k: {"p50_ms": v["p50_ms"], "p99_ms": v["p99_ms"],
                                        "achieved_reads_per_s": v["achieved_reads_per_s"],
                                        "sm_mhz": v["clocks"].get("sm_mhz"), "sm_min_mhz": v["clocks"].get("sm_min_mhz"),
                                        "clock_reasons": v["clocks"].get("reasons")} for k, v in sweep.items()}}
        log(f"[bench] serving {name} sweep: " + ", ".join(f"{k} p50 {v['p50_ms']} p99 {v['p99_ms']}"
                                                         for k, v in sweep.items()))
        log(f"[bench] serving {name}: saturated {sat['achieved_reads_per_s'] / 1e6:.1f} M reads/s; at 70% "
            f"p50 {loaded['p50_ms']} ms p99 {loaded['p99_ms']} ms, {loaded['mean_batch_requests']} req/batch")
    gi.set_locate_limit(0)
    return res


def log_uniform_sizes(rng: np.random.Generator, lo: int = 1024, hi: int = 262144):
    return lambda: int(np.exp(rng.uniform(np.log(lo), np.log(hi))))


def serving(gi, reads, genome, log, read_label: str = "100bp", locate_limit: int = 0) -> dict:
    """The serving form: 64k-read requests of the batch read model, and requests
    of log-uniform 1k-256k reads of 50-300 bp.  A nonzero locate_limit leaves
    lists covering more rows unlocated (against a 3.1 Gbp genome with perfect
    tandem runs, a 50 bp read inside a homopolymer run covers millions of rows)."""
    from hpgbwt import synth
    rng = np.random.default_rng(7)
    t = time.time()
    mix = synth.reads_fast_var(genome, 600_000, 11, 50, 300, "subst_capped")
    log(f"[bench] serving read pools ready ({time.time() - t:.1f}s)")
    cases = [(f"requests_64k_{read_label}", reads, lambda: 65536),
             ("requests_1k_256k_50_300bp", mix, log_uniform_sizes(rng))]
    return serve_cases(gi, cases, log, locate_limit, rng, SERVE_MAX_BATCH)


def served_parity(gi, index_dir: str, pool, rng: np.random.Generator, locate_limit: int, n_req: int = 16,
                  max_reads: int = 300_000) -> dict:
    """n_req requests of log-uniform 1k-64k reads (at most max_reads in all)
    submitted together to one server, each result compared record for record
    with the oracle's search of the same reads."""
    from hpgbwt import lib
    from oracle.pyoracle import PortOracle
    draw = log_uniform_sizes(rng, 1024, 65536)
    sizes = []
    while len(sizes) < n_req and sum(sizes) < max_reads:
        sizes.append(min(draw(), max_reads - sum(sizes)))
    subs = []
    for k in sizes:
        a = int(rng.integers(0, len(pool) - k + 1))
        subs.append(pool.subset(np.arange(a, a + k)))
    gi.set_locate_limit(locate_limit)
    srv = lib.Server(gi, max_batch_reads=SERVE_MAX_BATCH, max_results=MAX_RESULTS)
    tickets = [srv.submit(r.seq, r.offsets) for r in subs]
    got = [srv.wait(t)[0] for t in tickets]
    st = srv.stats()
    srv.close()
    gi.set_locate_limit(0)
    ora = PortOracle(index_dir)
    threads = os.cpu_count() or 1
    out = {"requests": len(subs), "reads": int(sum(sizes)), "batches": int(st["batches"]),
           "max_batch_requests": int(st["max_batch_requests"]), "locate_limit": locate_limit,
           "oracle": "oracle/fm_oracle.c (pinned bit-exact to the reference's own search code)",
           "hits": 0, "located_rows": 0, "equal": True}
    for i, (r, g) in enumerate(zip(subs, got)):
        want = ora.search(r, mode=lib.MODE_SEARCH1, max_results=MAX_RESULTS, threads=threads,
                          locate_limit=locate_limit)
        out["hits"] += int(len(want.hits))
        out["located_rows"] += int(len(want.locs))
        c = compare_results(g, want)
        if not c["equal"]:
            out["equal"] = False
            out.setdefault("differences", {})[f"request {i}"] = c
    ora.close()
    return out


def serving_large(dist, log) -> dict:
    """The serving form against the 3.1 Gbp index: the genome of the c4
    workload, indexed on this GPU; requests of log-uniform 1k-256k reads of
    uniform 50-300 bp at 0.5 % per-base substitution (uncapped), <=1 error
    searched, Poisson arrivals at 10-90 % of the saturated rate; then a burst of
    requests checked against the oracle."""
    from hpgbwt import lib, synth
    t0 = time.time()
    wl = WORKLOADS["c4"]
    index_dir, genome, t_gen = genome_and_index(wl, dist.rank, dist)
    t_index = time.time() - t0
    gi = lib.GpuIndex(index_dir, device=dist.local)
    t = time.time()
    pool = synth.reads_fast_var(genome, 600_000, 11, 50, 300, "none", subst_rate=0.005)
    log(f"[bench] 3.1 Gbp serving: genome {t_gen:.1f}s, genome + index {t_index:.1f}s, read pool "
        f"{time.time() - t:.1f}s")
    # the batched search autotuned on a held-out pool of the same request read model
    # (under the serving locate limit: without it, reads inside long tandem runs
    # cover more rows than any batch can locate)
    import torch
    t = time.time()
    gi.set_locate_limit(SERVE_LOCATE_LIMIT)
    tune = synth.reads_fast_var(genome, 600_000, 12, 50, 300, "none", subst_rate=0.005)
    t_seq = torch.from_numpy(tune.seq).to(f"cuda:{dist.local}")
    t_off = torch.from_numpy(tune.offsets.view(np.int64)).to(f"cuda:{dist.local}")
    table = gi.autotune(t_seq.data_ptr(), t_off.data_ptr(), len(tune), int(tune.offsets[-1]),
                        int(np.diff(tune.offsets).max()), MAX_RESULTS)
    del t_seq, t_off, tune
    best = min(table, key=lambda r: r["search_us"])
    log(f"[bench] 3.1 Gbp serving: autotune {len(table)} settings in {time.time() - t:.1f}s, best {best}")
    rng = np.random.default_rng(7)
    res = serve_cases(gi, [("requests_1k_256k_50_300bp", pool, log_uniform_sizes(rng))], log,
                      SERVE_LOCATE_LIMIT, rng, SERVE_MAX_BATCH)
    res["parity"] = served_parity(gi, index_dir, pool, rng, SERVE_LOCATE_LIMIT)
    log(f"[bench] 3.1 Gbp serving parity against the oracle: {res['parity']}")
    res["workload"] = ("3.1 Gbp genome of the c4 workload, index built on this GPU; requests of log-uniform "
                       "1k-256k reads of uniform 50-300 bp at 0.5% per-base substitution (uncapped), <=1 error "
                       "searched; Poisson arrivals at 10-90% of the saturated rate")
    res["genome_and_index_s"] = round(t_index, 1)
    res["tuning"] = dict(gi.get_tuning(), wave_group=gi.wave_group(), block_load_mode=gi.load_mode(),
                         start_table=gi.start_table(), direction_split=gi.direction_split(),
                         tuned_on="held-out pool of 600k request reads (seed 12)")
    gi.close()
    return res


def cal_generation(gi, reads, log, n: int) -> dict:
    """bwt_generate_cals_batch (seeds on the GPU, CALs on the host threads) over the
    first n reads of the batch: seed size 16, filter_seed_mappings 300,
    min_cal_size 20, max_intron_size 500000; the best of three calls."""
    rs = [bytes(reads.seq[int(reads.offsets[i]):int(reads.offsets[i + 1])]) for i in range(min(n, len(reads)))]
    best, counts = None, []
    for _ in range(3):
        counts = gi.generate_cals(rs, 1)
        best = gi.last_cal_seconds if best is None else min(best, gi.last_cal_seconds)
    out = {"reads": len(rs), "seconds": round(best, 4), "reads_per_s": round(len(rs) / best, 1),
           "cals_per_read": round(sum(counts) / max(1, len(rs)), 3), "host_threads": os.cpu_count(),
           "params": {"seed_size": 16, "filter_seed_mappings": 300, "min_cal_size": 20, "max_intron_size": 500000}}
    log(f"[bench] CAL generation: {out['reads_per_s'] / 1e6:.2f} M reads/s over {len(rs)} reads, "
        f"{out['cals_per_read']} CALs per read")
    return out


def alignment_lists(gi, reads, log, n: int) -> dict:
    """bwt_map_inexact_batch, the reference's alignment-list entry point, over the
    first n reads of the batch with filter_read_mappings 200: BWSearch1, the row
    filter, the located rows, the 10 bp merge and the list order on the device
    (device_seconds), the alignment_t records and their strings allocated on the
    host threads; the best of three calls.  A fastq batch's indices are C ints, so
    n stops where the bases (with one terminator a read) reach 2^31 bytes."""
    n = min(n, len(reads))
    fit = np.asarray(reads.offsets[1:], dtype=np.int64) + np.arange(1, len(reads) + 1) < 2 ** 31 - 1
    n = min(n, int(np.count_nonzero(fit)))
    seq = reads.seq[:int(reads.offsets[n])]
    offs = reads.offsets[:n + 1]
    best, dev, count = None, None, 0
    for _ in range(3):
        count = gi.map_inexact_batch_arrays(seq, offs, 200)
        if best is None or gi.last_map_seconds < best:
            best, dev = gi.last_map_seconds, gi.last_map_device_seconds
    out = {"reads": n, "seconds": round(best, 4), "reads_per_s": round(n / best, 1),
           "device_seconds": round(dev, 4), "host_seconds": round(best - dev, 4),
           "alignments_per_read": round(count / max(1, n), 3), "filter_read_mappings": 200}
    log(f"[bench] bwt_map_inexact_batch: {out['reads_per_s'] / 1e6:.2f} M reads/s over {n} reads "
        f"(device pass {dev * 1e3:.1f} ms, host records {(best - dev) * 1e3:.1f} ms), "
        f"{out['alignments_per_read']} alignments per read")
    return out


def block_search_leg(gi, reads, log, n_lists: int) -> dict:
    """The k-error block search of bwt_map_inexact_read_2 (bwt_gpu_block_search: host reads
    in, results, located rows and anchors out) over the whole batch, 1024-result lists; the
    best of three calls, with the search kernels' device time.  Then
    bwt_map_inexact_array_list_2 (alignment records built on the host) over the first
    n_lists reads, filter_read_mappings 200."""
    from hpgbwt import lib
    n = len(reads)
    seq = np.ascontiguousarray(reads.seq)
    offs = np.ascontiguousarray(reads.offsets)
    anchors = np.zeros(4 * n + 1, dtype=lib.ANCHOR_DTYPE)
    n_anch = np.zeros(2 * n + 1, dtype=np.uint8)
    best, kms, hits, locs = None, None, 0, 0
    for _ in range(3):
        rs = lib.ResultSetC()
        t = time.perf_counter()
        rc = gi.lib.bwt_gpu_block_search(gi.handle, seq.ctypes.data, offs.ctypes.data, n, MAX_RESULTS,
                                         lib.ctypes.byref(rs), anchors.ctypes.data, n_anch.ctypes.data)
        dt = time.perf_counter() - t
        if rc != 0:
            raise RuntimeError(gi.lib.bwt_gpu_last_error().decode())
        hits, locs = int(rs.n_hits), int(rs.n_locs)
        gi.lib.bwt_gpu_result_free(lib.ctypes.byref(rs))
        best = dt if best is None else min(best, dt)
        k = gi.block_search_ms()
        kms = k if kms is None else min(kms, k)
    # one more call with the sector census on (not timed): occupancy-block sectors the kernel reads
    gi.set_census(True)
    rs = lib.ResultSetC()
    if gi.lib.bwt_gpu_block_search(gi.handle, seq.ctypes.data, offs.ctypes.data, n, MAX_RESULTS,
                                   lib.ctypes.byref(rs), None, None) != 0:
        raise RuntimeError(gi.lib.bwt_gpu_last_error().decode())
    gi.lib.bwt_gpu_result_free(lib.ctypes.byref(rs))
    sectors = gi.census()
    gi.set_census(False)
    out = {"reads": n, "seconds": round(best, 4), "reads_per_s": round(n / best, 1),
           "kernel_ms": round(kms, 3), "kernel_reads_per_s": round(n / (kms * 1e-3), 1),
           "sectors_per_read": round(sectors / max(1, n), 2),
           "gather_gsectors_per_s": round(sectors / (kms * 1e-3) / 1e9, 1),
           "hits_per_read": round(hits / max(1, n), 3), "located_rows_per_read": round(locs / max(1, n), 3),
           "max_results": MAX_RESULTS}
    log(f"[bench] block search: kernel {out['kernel_reads_per_s'] / 1e6:.1f} M reads/s ({kms:.2f} ms), "
        f"call {out['reads_per_s'] / 1e6:.2f} M reads/s, {out['hits_per_read']} hits per read")
    if n_lists > 0:
        rs_ = [bytes(reads.seq[int(reads.offsets[i]):int(reads.offsets[i + 1])]) for i in range(min(n_lists, n))]
        bl, count = None, 0
        for _ in range(3):
            count = gi.map_block_array_list(rs_, 200)
            bl = gi.last_map_seconds if bl is None else min(bl, gi.last_map_seconds)
        out["array_list_2"] = {"reads": len(rs_), "seconds": round(bl, 4), "reads_per_s": round(len(rs_) / bl, 1),
                               "alignments_per_read": round(count / max(1, len(rs_)), 3),
                               "filter_read_mappings": 200}
        log(f"[bench] bwt_map_inexact_array_list_2: {len(rs_) / bl / 1e6:.2f} M reads/s over {len(rs_)} reads, "
            f"{count / max(1, len(rs_)):.3f} alignments per read")
    return out


def run_gb300(args, wl: dict, dist: Dist) -> dict | None:
    import torch
    from hpgbwt import lib
    dev = dist.local
    torch.cuda.set_device(dev)
    index_dir, reads, genome = prepare(wl, dist.rank, dist)
    mode = wl_mode(wl)
    gi = lib.GpuIndex(index_dir, device=dev)
    n = len(reads)
    total = int(reads.offsets[-1])
    max_len = int(np.diff(reads.offsets).max())
    d_seq = torch.from_numpy(reads.seq).to(f"cuda:{dev}")
    d_off = torch.from_numpy(reads.offsets.view(np.int64)).to(f"cuda:{dev}")
    torch.cuda.synchronize()
    stream = torch.cuda.ExternalStream(gi.stream(), device=f"cuda:{dev}")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{dev}")

    def make_step(form):
        def step():
            return gi.search_device(d_seq.data_ptr(), d_off.data_ptr(), n, total, max_len, mode, form, MAX_RESULTS)
        return step

    def timed(form):
        """census run, W warm-up steps, K timed steps (L2 flushed before each);
        the last timed step's output is copied to the host for the parity check."""
        step = make_step(form)
        gi.set_census(True)
        rs = step()
        sectors = gi.census()
        gi.set_census(False)
        for _ in range(args.warmup):
            step()
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
              for _ in range(args.steps)]
        stage_sum = [0.0, 0.0, 0.0, 0.0, 0.0]
        dist.barrier()
        torch.cuda.synchronize()
        l0 = lib.launch_count()
        last = None
        with ClockSampler(dev) as clk:
            for i in range(args.steps):
                flush.fill_(i & 0xFF)
                torch.cuda.synchronize()
                ev[i][0].record(stream)
                last = step()
                ev[i][1].record(stream)
                ev[i][1].synchronize()
                stage_sum = [a + b for a, b in zip(stage_sum, gi.stage_ms())]
        launches = lib.launch_count() - l0
        torch.cuda.synchronize()
        dist.barrier()
        ms = dist.max(sum(a.elapsed_time(b) for a, b in ev))
        out = fetch_result(gi, last, n)
        return {"ms": ms, "sectors": sectors, "stages": [x / args.steps for x in stage_sum], "launches": launches,
                "clocks": clk.summary(), "n_hits": int(rs.n_hits), "n_locs": int(rs.n_locs), "result": out}

    total_reads = dist.sum(float(n))
    # autotune the batched form (untimed) on a held-out batch of the same workload
    table = []
    if args.tuning:
        vals = [int(x) for x in args.tuning.split(",")]
        st, ch, mb, lm = vals[:4]
        if st == -2:  # warp-cooperative form, `ch` reads per warp group
            gi.set_tuning(0, 4, 1, mb)
            gi.set_wave_group(ch)
        else:
            gi.set_tuning(0, st, ch, mb)
        gi.set_load_mode(lm)
        if len(vals) > 4:
            gi.set_start_table(vals[4])
        if len(vals) > 5:
            gi.set_direction_split(vals[5])
        if len(vals) > 6:
            gi.set_idle_batch(vals[6])
    elif not args.no_autotune:
        t0 = time.time()
        tune = make_reads(wl, genome, read_seed(dist.rank) + TUNE_SEED_OFFSET)
        t_seq = torch.from_numpy(tune.seq).to(f"cuda:{dev}")
        t_off = torch.from_numpy(tune.offsets.view(np.int64)).to(f"cuda:{dev}")
        table = gi.autotune(t_seq.data_ptr(), t_off.data_ptr(), len(tune), int(tune.offsets[-1]),
                            int(np.diff(tune.offsets).max()), MAX_RESULTS)
        del t_seq, t_off, tune
        torch.cuda.synchronize()
        log(f"[bench] autotune on a held-out batch (seed {read_seed(dist.rank) + TUNE_SEED_OFFSET}): "
            f"{len(table)} settings in {time.time() - t0:.1f}s, best {min(table, key=lambda r: r['search_us'])}")
        for r in sorted(table, key=lambda r: r["search_us"])[:8]:
            log(f"[bench]   {r}")
    res = {}
    for name, form in (("plain", lib.FORM_PLAIN), ("batched", lib.FORM_BATCHED)):
        res[name] = timed(form)
        res[name]["value"] = total_reads * args.steps / (res[name]["ms"] / 1e3)
        log(f"[bench] {name}: {res[name]['value'] / 1e6:.1f} M reads/s, stages {res[name]['stages']}")
    head = res["batched"]
    form = lib.FORM_BATCHED
    value = head["value"]
    ms_max = head["ms"]
    launches = head["launches"]
    clk_summary = head["clocks"]
    # algorithmic sectors: the census of the plain form, which walks every step
    # of the reference's searches (a start table in the batched form stands one
    # lookup for its first steps, so its own census counts fewer sectors)
    sectors = res["plain"]["sectors"]
    gathered = head["sectors"]
    stage_sum = [x * args.steps for x in head["stages"]]
    n_hits, n_locs = head["n_hits"], head["n_locs"]

    # e2e: host buffers through the C ABI (pinned reads in, host records out)
    pin_seq = torch.from_numpy(reads.seq).pin_memory()
    pin_off = torch.from_numpy(reads.offsets.view(np.int64)).pin_memory()
    rsc = lib.ResultSetC()
    e2e_t = []
    e2e_result = None
    for i in range(args.warmup + args.steps):
        t = time.perf_counter()
        rc = gi.lib.bwt_gpu_search_batch(gi.handle, mode, form, pin_seq.data_ptr(), pin_off.data_ptr(),
                                         n, MAX_RESULTS, lib.ctypes.byref(rsc))
        dt = time.perf_counter() - t
        if rc != 0:
            raise RuntimeError(gi.lib.bwt_gpu_last_error().decode())
        if i >= args.warmup:
            e2e_t.append(dt)
        e_hits, e_locs = int(rsc.n_hits), int(rsc.n_locs)
        if i == args.warmup + args.steps - 1:
            e2e_result = lib.result_from_c(rsc, n)
        gi.lib.bwt_gpu_result_free(lib.ctypes.byref(rsc))
    log(f"[bench] e2e calls (ms): {[round(x * 1e3, 2) for x in e2e_t]}")
    rl = wl["read_len"]
    search1 = mode == lib.MODE_SEARCH1
    serve = serving(gi, reads, genome, log, f"{rl[0]}_{rl[1]}bp" if isinstance(rl, tuple) else f"{rl}bp",
                    SERVE_LOCATE_LIMIT if wl["genome"] == "large" else 0) if search1 and not args.no_serving else None
    cals = cal_generation(gi, reads, log, args.cal_reads) if search1 and args.cal_reads > 0 else None
    alns = alignment_lists(gi, reads, log, len(reads)) if search1 and args.cal_reads > 0 else None
    block = block_search_leg(gi, reads, log, args.cal_reads) if search1 and not args.no_block else None
    e2e_s = dist.max(sum(e2e_t))
    e2e_value = total_reads * args.steps / e2e_s
    h2d = total + 8 * (n + 1)
    d2h = 32 * e_hits + 32 * e_locs + 2 * n * 4 + 2 * n

    # rooflines of the dominant kernel (the search kernel of the headline form)
    per_step = [x / args.steps for x in stage_sum]
    search_ms = per_step[1]
    peak, peak_kind = measured_peaks()
    algo_bytes = 32.0 * sectors + total + 16.0 * n_hits
    achieved = algo_bytes / (search_ms * 1e-3) / 1e9
    kernel = "wave_search_kernel" if gi.wave_group() else "batched_search_kernel"
    traffic, traffic_src = profiled_traffic(args.workload, kernel,
                                            {"group": gi.wave_group(), "start_table": gi.start_table(),
                                             "load_mode": gi.load_mode(), "direction_split": gi.direction_split()})
    roofline = {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                "frac": round(achieved / peak, 4), "traffic": traffic,
                "basis": "algorithmic bytes (census index sectors of the reference's steps x 32 B + read bytes + "
                         "16 B per hit) over the search stage's CUDA-event time, against the measured HBM copy "
                         "bandwidth; the index is mostly served from L2, so this is not DRAM throughput "
                         "(dram_frac is)",
                "kernel": kernel, "peak_kind": peak_kind,
                "algorithmic_bytes_per_read": round(algo_bytes / n, 1),
                "traffic_source": traffic_src,
                "dram_gbs": round(traffic / (search_ms * 1e-3) / 1e9, 1) if traffic else None,
                "dram_frac": round(traffic / (search_ms * 1e-3) / 1e9 / peak, 4) if traffic else None}
    gather = None
    if dist.rank == 0:
        rate = sectors / (search_ms * 1e-3)
        grate = gathered / (search_ms * 1e-3)
        gather = {"sectors_per_s": round(rate, 1), "sectors_per_read": round(sectors / n, 2),
                  "gathered_sectors_per_s": round(grate, 1), "gathered_sectors_per_read": round(gathered / n, 2)}
        if wl["genome"] == "large":
            # a uniform random probe over 3.1 GB is no ceiling for the search's skewed,
            # L2-heavy access mix (every walk starts in the same few blocks)
            gather.update({"ceiling_sectors_per_s": None, "frac": None, "frac_gathered": None,
                           "note": "no gather ceiling matches this index's access mix; see the HBM view"})
        else:
            ib = gi.index_bytes()
            best = 0.0
            for blocks in (152 * 8, 152 * 16):
                best = max(best, lib.gather_ceiling(dev, ib, blocks, 1024))
            gather.update({"ceiling_sectors_per_s": round(best, 1), "buffer_bytes": ib,
                           "frac": round(rate / best, 4), "frac_gathered": round(grate / best, 4),
                           "basis": "frac: census sectors of the reference's steps (what the plain form "
                                    "gathers); frac_gathered: sectors the batched form itself gathered (its start "
                                    "table stands one lookup for a chain's first steps)"})
    out = None
    if dist.rank == 0:
        base, parity = (None, None)
        if not args.no_cpu_baseline:
            gpu_res = {"batched": head["result"], "plain": res["plain"]["result"], "e2e": e2e_result}
            base, parity = oracle_leg(index_dir, reads, mode, gpu_res)
            log(f"[bench] parity against the oracle: {parity}")
        out = {
            "metric": METRIC, "value": round(value, 1), "unit": "reads/s", "n_gpus": dist.world,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(ms_max / args.steps, 3),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "u32",
            "data": "synthetic (seeded genome and reads; no public dataset)",
            "config": bench_config(wl, n, dist.world, total),
            "e2e": {"value": round(e2e_value, 1), "unit": "reads/s", "h2d_bytes_per_step": h2d,
                    "d2h_bytes_per_step": d2h, "api": "bwt_gpu_search_batch"},
            "gpu_launches": int(launches),
            "parity": parity,
            "gather_roofline": gather,
            "roofline": roofline,
            "cpu_baseline": base,
            "clocks": clk_summary,
            "stages_ms": {"encode": round(per_step[0], 3), "search": round(per_step[1], 3),
                          "of_which_drain": round(per_step[4], 3), "finalize": round(per_step[2], 3),
                          "locate": round(per_step[3], 3)},
            "hits_per_step": n_hits, "located_rows_per_step": n_locs,
            "forms": {k: {"reads_per_s": round(v["value"], 1), "ms_per_step": round(v["ms"] / args.steps, 3),
                          "stages_ms": [round(x, 3) for x in v["stages"]], "sectors_per_read": round(v["sectors"] / n, 2)}
                      for k, v in res.items()},
            "batched_over_plain": round(res["batched"]["value"] / res["plain"]["value"], 3),
            "serving": serve,
            "cal_generation": cals,
            "alignment_lists": alns,
            "block_search": block,
            "tuning": dict(gi.get_tuning(), block_load_mode=gi.load_mode(), start_table=gi.start_table(),
                           direction_split=gi.direction_split(), idle_batch=gi.idle_batch()),
            "autotune": ({"settings": len(table), "tuned_on": "held-out batch of the same workload (seed "
                          f"{read_seed(dist.rank) + TUNE_SEED_OFFSET})",
                          "best_search_ms": min(r["search_us"] for r in table) / 1e3,
                          "worst_search_ms": max(r["search_us"] for r in table) / 1e3} if table else None),
        }
    gi.close()
    if out is not None and dist.world == 1 and wl["genome"] != "large" and not (args.no_serving or args.no_large):
        out["serving_3g"] = serving_large(dist, log)
    return out


def run_reference(args, wl: dict, dist: Dist) -> dict | None:
    if dist.rank != 0:
        return None
    index_dir, reads, _ = prepare(wl, 0, dist)
    mode = wl_mode(wl)
    from oracle.pyoracle import PortOracle
    ora = PortOracle(index_dir)
    threads = os.cpu_count() or 1
    probe = reads.subset(np.arange(min(2000, len(reads))))
    t = time.perf_counter()
    ora.search(probe, mode=mode, max_results=MAX_RESULTS, threads=threads)
    rate = len(probe) / max(time.perf_counter() - t, 1e-6)
    per_step = int(min(len(reads), max(len(probe), rate * 20.0 / max(1, args.steps))))
    sample = reads.subset(np.arange(per_step))
    for _ in range(min(args.warmup, 1)):
        ora.search(probe, mode=mode, max_results=MAX_RESULTS, threads=threads)
    t = time.perf_counter()
    for _ in range(args.steps):
        ora.search(sample, mode=mode, max_results=MAX_RESULTS, threads=threads)
    dt = time.perf_counter() - t
    value = per_step * args.steps / dt
    desc = (f"{per_step} reads per step (bounded sample of the {len(reads)}-read batch), OpenMP over {threads} "
            f"host threads; the C restatement oracle/fm_oracle.c, pinned bit-exact to the reference's own "
            f"search code (the compiled reference itself is built only where its source tree is)")
    return {"metric": METRIC, "value": round(value, 1), "unit": "reads/s", "impl": "reference",
            "n_gpus": dist.world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": round(dt * 1e3 / args.steps, 3), "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "u32", "data": "synthetic (seeded genome and reads; no public dataset)",
            "config": bench_config(wl, len(reads), dist.world, int(reads.offsets[-1])),
            "cpu_baseline": {"value": round(value, 1), "unit": "reads/s", "cores": threads, "kind": "port",
                             "sample": desc},
            "e2e": {"value": round(value, 1), "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="c2", choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-autotune", action="store_true", help="keep the library's default batched tuning")
    ap.add_argument("--no-serving", action="store_true", help="skip the serving-form latency measurement")
    ap.add_argument("--no-block", action="store_true", help="skip the k-error block search leg")
    ap.add_argument("--no-large", action="store_true",
                    help="skip serving against the 3.1 Gbp index (built on the GPU) after the workload's legs")
    ap.add_argument("--cal-reads", type=int, default=200_000,
                    help="reads of the batch taken through bwt_generate_cals_batch and bwt_map_inexact_batch "
                         "(0: skip)")
    ap.add_argument("--tuning", default="", help="fix the batched tuning: stack,chains_per_claim,register_bound,"
                                                 "block_load_mode[,start_table[,direction_split[,idle_batch]]] (stack 0 = split, -1 = lockstep, "
                                                 "-2 = warp-cooperative with chains_per_claim reads per warp group)")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    wl = WORKLOADS[args.workload]
    if args.impl == "reference":
        rank = int(os.environ.get("RANK", "0"))
        if rank != 0:
            return 0
        from hpgbwt import build as hbuild
        hbuild.build_lib()
        hbuild.build_oracle()
        out = run_reference(args, wl, _Rank0())
    else:
        from hpgbwt import build as hbuild
        hbuild.build_lib()
        hbuild.build_oracle()
        dist = Dist(args.gpus)
        try:
            out = run_gb300(args, wl, dist)
        finally:
            dist.close()
    if out is not None:
        print(json.dumps(out), flush=True)
    return 0


class _Rank0:
    """Rank 0 of a reference-arm run: no process group, nothing to wait for."""
    rank = 0
    local = 0
    world = int(os.environ.get("WORLD_SIZE", "1"))

    def barrier(self):
        pass


if __name__ == "__main__":
    sys.exit(main())
