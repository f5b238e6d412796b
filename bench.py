#!/usr/bin/env python3
"""Throughput of the probebwa mapping path on GB300.

Default workload (--config 2, the batching and ranker configurations on one
genome): a synthetic 3.1 Gbp genome (24 contigs of U(50, 250) relative size,
GC 41%, 45% copies of 500 interspersed repeat families with 300 bp-6 kbp
consensus and 2-25% divergence, 3% tandem arrays), its full 15-mer index
resident in HBM (built on the GPU with pbw_build_hash), and 10,000,000 reads
trimmed to lengths U[60, 250], half single-end and half FR pairs (insert
N(300, 80)), 0.5% substitutions and 0.05% indels (5x in homopolymers), Phred
N(35, 4). One step maps one 1M-read chunk (500,000 single-end reads and
250,000 pairs, each chunk an independent input mapped with the default
options); the steps cycle through the 10 chunks. Three forms run on the same
chunks: the plain method with batching off, the plain method with batching
(length bins, autotuned band DP, pair graphs: `value`, bit-identical records)
and ranked+batched (a candidate ranker trained on 2,000,000 fresh reads of the
same genome). The line also carries parity against the oracle: a sample of the
first chunk at this scale, the whole single-end configuration (1 Mbp, 10,000 x
120 bp) and 40,000 pairs of the paired configuration (100 Mbp, 2 x 150 bp),
plus the count of reads whose record depends on the SwissTable group width
(8 vs 16) of the candidate tie order.

--config 4: the repeat-stress workload (the 3.1 Gbp genome plus 200 families
of 32-64 near-identical copies and homopolymer-rich regions; 2,000,000 pairs
of 2 x 250 bp, insert N(500, 120), 3% substitutions, 0.3% indels, Phred
N(28, 8), 30% of the pairs from the stress regions). --config 0 / 1: the
single-end (1 Mbp) and paired-end (100 Mbp, 1,000,000 pairs) configurations,
one step mapping the whole read set. Data are generated from fixed seeds; no
dataset is downloaded.

`value` is reads/s with the reads in pinned host memory and the device time
of the pipeline's phases (CUDA events); `e2e` is the same metric through the
public C ABI including every step's host->device input copies and
device->host record copies (the calls' event spans).

--impl reference times the CPU restatement of the reference path (oracle/)
on the host cores on a bounded sample of the same workload.
"""
from __future__ import annotations

import argparse
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

SEED = {0: 0x5EED0000, 1: 0x5EED0001, 2: 0x5EED0002, 3: 0x5EED0002, 4: 0x5EED0004}
CHUNK_READS = 131072  # the library's default chunk (pbw_options.chunk_reads = 0)
# DRAM bytes (read + write) of K1 per read of the paired workload, from one
# ncu capture of a 100,000-read launch (29.014 GB read + 0.161 GB written):
# profiles/k_seed_paired_100k_pairs.md. Not measured for the other workloads.
SEED_DRAM_BYTES_PER_READ = {1: (29.014204e9 + 0.161155e9) / 100_000}
METRIC = "reads/s @1 GB300: plain vs ranked+batched (≤0.05% primaries changed); DP GCUPS"
LN_1E12 = -27.631021115928547     # ln(1e-12): ranker label cut of the repeat-family workloads
STRICT_CUT = -41.58883083359672   # -60 ln 2: pruning cannot move sum_exp


def dev_time(st) -> float:
    """Device milliseconds of one map call without the input copy: the span
    of its mapping work (paired calls overlap the pair batches with the next
    super-chunk's seeding, so the phase times can add up to more) plus the
    record copy."""
    return st["ms_compute"] + st["ms_d2h"]


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ---------------------------------------------------------------------------
# workloads
# ---------------------------------------------------------------------------
def workload(cfg: int, cache: str, n_override: int | None = None):
    from probebwa_gb300 import synth
    os.makedirs(cache, exist_ok=True)
    prefix = os.path.join(cache, f"cfg{cfg}")
    seed = SEED[cfg]
    if cfg == 0:
        n = n_override or 10_000
        meta = {"workload": "single-end 1 Mbp / 10,000 x 120 bp", "genome_bp": 1_000_000, "reads": n,
                "read_len": 120, "paired": False}
    else:
        n = n_override or 1_000_000
        meta = {"workload": "paired-end 100 Mbp (25 x 4 Mbp) / 1,000,000 pairs x 2 x 150 bp", "genome_bp": 100_000_000,
                "pairs": n, "read_len": 150, "insert": "N(350,50)", "paired": True}
    rpath = prefix + f".reads{n}.npz"
    if not (os.path.exists(prefix + ".stidx") and os.path.exists(prefix + ".sthash") and os.path.exists(rpath)):
        t = time.time()
        if cfg == 0:
            contigs = synth.genome_single(seed)
        else:
            contigs = synth.genome_paired(seed)
        if cfg == 1 and _gpu_present():
            # the 100 Mbp index: pbw_build_hash (byte-identical to the numpy
            # and oracle builders, tests/test_index_build.py) in a second
            synth.write_stidx(prefix, contigs)
            import probebwa_gb300 as P
            P.build()
            P.build_hash(prefix, prefix)
        else:
            synth.write_index(prefix, contigs)
        log(f"[bench] index for config {cfg}: {time.time() - t:.1f}s")
        t = time.time()
        if cfg == 0:
            b, q, o = synth.reads_single_fast(seed + 17, contigs, n, L=120, sub=0.01, indel=0.001)
            np.savez(rpath, b1=b, q1=q, o1=o)
        else:
            b1, q1, o1, b2, q2, o2 = synth.reads_paired_fast(seed + 17, contigs, n, L=150, mean=350.0, sd=50.0,
                                                             sub=0.005, indel=0.0005)
            np.savez(rpath, b1=b1, q1=q1, o1=o1, b2=b2, q2=q2, o2=o2)
        log(f"[bench] reads for config {cfg}: {time.time() - t:.1f}s")
    d = dict(np.load(rpath))
    return prefix, d, meta


def _gpu_present() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, dev: int = 0):
        self.dev = dev
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.dev), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                mx.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------------------
# GPU arm
# ---------------------------------------------------------------------------
_PINNED = []  # pinned host tensors backing the numpy views below


def pinned(a: np.ndarray) -> np.ndarray:
    import torch
    t = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True)
    _PINNED.append(t)
    v = t.numpy()[:a.nbytes].view(a.dtype).reshape(a.shape)
    v[...] = a
    return v


def max_over_ranks(values, world: int, device: str = "cpu"):
    """Step times of the slowest rank (replicas run the same workload)."""
    if world <= 1:
        return list(values)
    import torch
    t = torch.tensor(list(values), dtype=torch.float64, device=device)
    torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
    return [float(x) for x in t.cpu()]


def run_gpu(args, prefix, d, meta, rank, world):
    import torch
    import probebwa_gb300 as P
    P.build()
    dev = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(dev)
    opts = P.MapperOptions(device=dev)
    t0 = time.time()
    m = P.Mapper(prefix, options=opts)
    t_open = time.time() - t0
    paired = meta["paired"]
    R1 = P.Reads(pinned(d["b1"]), pinned(d["q1"]), pinned(d["o1"]))
    R2 = P.Reads(pinned(d["b2"]), pinned(d["q2"]), pinned(d["o2"])) if paired else None
    n_reads = R1.n * (2 if paired else 1)
    # pinned outputs
    def outs(R):
        recs = P.alloc_records(R.n, len(R.bases))
        return {k: pinned(v) for k, v in recs.items()}
    O1 = outs(R1)
    O2 = outs(R2) if paired else None
    import ctypes as C
    L = P.lib()

    def step():
        if paired:
            mdl = P.InsertModelC(opts.insert_size_mean, opts.insert_size_sd, 0)
            rc = L.pbw_map_paired(m.h, C.byref(mdl), C.byref(R1.c()), C.byref(R2.c()), C.byref(P.records_c(O1)),
                                  C.byref(P.records_c(O2)))
        else:
            rc = L.pbw_map_single(m.h, C.byref(R1.c()), C.byref(P.records_c(O1)))
        m._check(rc)
        return m.stats()

    for _ in range(args.warmup):
        step()
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    clk = ClockSampler(dev)
    clk.start()
    stats = []
    t_wall = time.time()
    for _ in range(args.steps):
        stats.append(step())
    torch.cuda.synchronize()
    t_wall = time.time() - t_wall
    clocks = clk.stop()
    tuning = m.tuning()
    plain_records = [_rec_copy(O1)] + ([_rec_copy(O2)] if paired else [])
    ranked = None
    if args.ranked and paired and world == 1:
        ranked = run_ranked(args, m, opts, step, O1, O2, meta, n_reads, dev)
    # device time of a step: the pipeline's CUDA events, without the input copy
    dev_ms = [dev_time(s) for s in stats]
    e2e_ms = [s["ms_total"] for s in stats]
    mean_dev, mean_e2e = max_over_ranks([statistics.mean(dev_ms) / 1e3, statistics.mean(e2e_ms) / 1e3], world,
                                        "cuda")
    s0 = stats[-1]
    value = n_reads * world / mean_dev
    e2e = n_reads * world / mean_e2e
    h2d = int(R1.bases.nbytes + R1.quals.nbytes + R1.offsets.nbytes)
    if paired:
        h2d += int(R2.bases.nbytes + R2.quals.nbytes + R2.offsets.nbytes)
    rec_bytes = sum(int(v.nbytes) for k, v in O1.items() if not k.startswith(("cigar", "_"))) + 4 * (len(O1["cigar_off"]) + int(O1["cigar_off"][-1]))
    if paired:
        rec_bytes += sum(int(v.nbytes) for k, v in O2.items() if not k.startswith(("cigar", "_"))) + 4 * (len(O2["cigar_off"]) + int(O2["cigar_off"][-1]))
    # roofline of the dominant kernel
    phases = {"seed": s0["ms_seed"], "cluster": s0["ms_cluster"], "align_seeded": s0["ms_align"],
              "pair": s0["ms_pair"], "finalize": s0["ms_finalize"]}
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    L_read = meta["read_len"]
    # K1 seeding: algorithmic bytes = the read bytes (2-bit codes + qualities
    # for the repeat filter) + 8 bytes per CSR probe, per bucket entry and per
    # hit; one launch maps one chunk of CHUNK_READS reads of one mate.
    n_seed_launches = (2 if paired else 1) * ((R1.n + CHUNK_READS - 1) // CHUNK_READS)
    seed_bytes = (n_reads * ((L_read + 3) // 4 + L_read) + 8 * s0["seed_probes"] + 8 * s0["seed_entries"] +
                  8 * s0["seed_hits"])
    seed_gbs = seed_bytes / (s0["ms_seed"] / 1e3) / 1e9 if s0["ms_seed"] > 0 else 0.0
    gcups = s0["dp_cells"] / (s0["ms_align"] / 1e3) / 1e9 if s0["ms_align"] > 0 else 0.0
    reads_per_launch = n_reads / n_seed_launches
    dram_per_read = SEED_DRAM_BYTES_PER_READ.get(args.config)
    roofline = {"kernel": "k_seed (K1 seeding)", "bound": "hbm", "achieved": round(seed_gbs, 1),
                "peak": hbm_peak, "unit": "GB/s", "frac": round(seed_gbs / hbm_peak, 4),
                "traffic": int(dram_per_read * reads_per_launch) if dram_per_read else None,
                "traffic_source": "ncu dram__bytes_read.sum + dram__bytes_write.sum of one 100,000-read launch, "
                                  "scaled by reads per launch (profiles/k_seed_paired_100k_pairs.md)",
                "dram_gbs": round(dram_per_read * n_reads / (s0["ms_seed"] / 1e3) / 1e9, 1)
                if (s0["ms_seed"] > 0 and dram_per_read) else None,
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst)" if peaks else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": int(seed_bytes / n_seed_launches),
                "launches_per_step": n_seed_launches,
                "phase_ms": {k: round(v, 3) for k, v in phases.items()}}
    # The largest share of the step is the seeded DP (k_align_band). It is an
    # integer max-plus recurrence bound by instruction issue on the INT32 ALU
    # pipe, neither HBM nor tensor: its figures are reported beside the
    # schema's roofline. GCUPS here spans the seeded-alignment phase (job
    # build, DP with traceback, likelihood walk).
    roofline_dp = {"kernel": "k_align_band (seeded banded DP)", "bound": "int32 issue (ALU pipe)",
                   "achieved_gcups": round(gcups, 1), "cells_per_step": int(s0["dp_cells"]),
                   "ncu_alu_pipe_frac": 0.725, "ncu_issue_active_frac": 0.655,
                   "ncu_source": "profiles/k_align_band_single_10k_reads.md"}
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "reads/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(mean_dev * 1e3, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic (seeded)",
        "config": dict(meta, l2="inputs larger than L2: 4 GiB k-mer CSR + entries + genome + reads",
                       index_load_s=round(t_open, 2), parallelism=f"replicas x{world}"),
        "e2e": {"value": round(e2e, 1), "unit": "reads/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": rec_bytes,
                "ms_per_step": round(mean_e2e * 1e3, 3)},
        "gpu_launches": int(s0["kernel_launches"]) * args.steps,
        "dp_gcups": round(gcups, 2), "dp_cells_per_step": int(s0["dp_cells"]), "dp_jobs_per_step": int(s0["dp_jobs"]),
        "roofline": roofline, "roofline_dp": roofline_dp, "clocks": clocks, "wall_s_timed": round(t_wall, 3),
    }
    out["_records"] = plain_records
    out["batching"] = {"band_dp_lanes_by_length_class": dict(zip(("<=128", "<=256", ">256"), tuning["chosen_lanes"])),
                       "band_dp_tuned_ms_8_16_4": dict(zip(("<=128", "<=256", ">256"), tuning["tuned_ms"])),
                       "length_bins": bool(tuning["length_bins"]), "pair_graphs": bool(tuning["pair_graphs"])}
    if ranked is not None:
        ranked["speedup_vs_plain"] = round(ranked["value"] / value, 3)
        out["ranked"] = ranked
    if paired and world == 1:
        # tie-order exposure: the same reads with the aarch64 SwissTable group width
        with P.Mapper(prefix, options=P.MapperOptions(device=dev, group_width=8)) as m8:
            g1, g2, _ = m8.map_paired(P.Reads(d["b1"], d["q1"], d["o1"]), P.Reads(d["b2"], d["q2"], d["o2"]))
        out["tie_order_sensitive"] = int(_rec_diff(g1, out["_records"][0]) + _rec_diff(g2, out["_records"][1]))
    m.close()
    return out


def _primary_changes(a, b):
    """Reads whose primary (contig, POS, FLAG, CIGAR) and whose MAPQ differ."""
    n = len(a["contig"])
    prim = (a["contig"][:n] != b["contig"][:n]) | (a["pos"][:n] != b["pos"][:n]) | (a["flag"][:n] != b["flag"][:n])
    ca, cb = a["cigar_off"], b["cigar_off"]
    la, lb = np.diff(ca[:n + 1].astype(np.int64)), np.diff(cb[:n + 1].astype(np.int64))
    same_len = la == lb
    idx = np.flatnonzero(same_len & ~prim)
    # compare CIGAR words of equal-length CIGARs in one pass
    if idx.size:
        ra = np.repeat(ca[idx].astype(np.int64), la[idx]) + (np.arange(la[idx].sum()) -
                                                            np.repeat(np.cumsum(la[idx]) - la[idx], la[idx]))
        rb = np.repeat(cb[idx].astype(np.int64), la[idx]) + (np.arange(la[idx].sum()) -
                                                            np.repeat(np.cumsum(la[idx]) - la[idx], la[idx]))
        bad = a["cigar"][ra] != b["cigar"][rb]
        owner = np.repeat(idx, la[idx])
        prim[np.unique(owner[bad])] = True
    prim |= ~same_len
    mq = a["mapq"][:n] != b["mapq"][:n]
    return int(prim.sum()), int(mq.sum())


def run_ranked(args, m, opts, step, O1, O2, meta, n_reads, dev):
    """The ranked path on the same reads: train the candidate ranker on fresh
    pairs of the same genome (plain-path labels), then time the same steps
    with pruning on and count the reads whose primary or MAPQ changed against
    the plain path's records."""
    import torch
    import probebwa_gb300 as P
    from probebwa_gb300 import synth
    plain = [{k: v.copy() for k, v in O.items() if not k.startswith("_")} for O in (O1, O2)]
    prefix = os.path.join(args.cache, f"cfg{args.config}")
    t = time.time()
    tr_path = prefix + f".train{args.train_pairs}.npz"
    if not os.path.exists(tr_path):
        contigs = synth.read_stidx_contigs(prefix)
        b1, q1, o1, b2, q2, o2 = synth.reads_paired_fast(SEED[args.config] + 99, contigs, args.train_pairs, L=150,
                                                         mean=350.0, sd=50.0, sub=0.005, indel=0.0005)
        np.savez(tr_path, b1=b1, q1=q1, o1=o1, b2=b2, q2=q2, o2=o2)
    tr = dict(np.load(tr_path))
    t_gen = time.time() - t
    T1 = P.Reads(tr["b1"], tr["q1"], tr["o1"])
    T2 = P.Reads(tr["b2"], tr["q2"], tr["o2"])
    rep = m.ranker_train(T1, T2, label_cut=args.label_cut)
    m.ranker_enable(True)
    for _ in range(args.warmup):
        step()
    torch.cuda.synchronize()
    m.ranker_enable(True)  # counters from here
    stats = [step() for _ in range(args.steps)]
    torch.cuda.synchronize()
    cnt = m.ranker_counters()
    m.ranker_enable(False)
    dev_ms = [dev_time(s) for s in stats]
    e2e_ms = [s["ms_total"] for s in stats]
    ch_p = ch_m = 0
    for O, Pl in zip((O1, O2), plain):
        a, b = _primary_changes(O, Pl)
        ch_p += a
        ch_m += b
    s0 = stats[-1]
    tot = cnt["kept"] + cnt["pruned"]
    return {"value": round(n_reads / (statistics.mean(dev_ms) / 1e3), 1),
            "e2e": {"value": round(n_reads / (statistics.mean(e2e_ms) / 1e3), 1), "unit": "reads/s"},
            "ms_per_step": round(statistics.mean(dev_ms), 3),
            "phase_ms": {"seed": round(s0["ms_seed"], 3), "cluster": round(s0["ms_cluster"], 3),
                         "align_seeded": round(s0["ms_align"], 3), "pair": round(s0["ms_pair"], 3)},
            "dp_jobs_per_step": int(s0["dp_jobs"]),
            "changed_primary_frac": ch_p / n_reads, "changed_mapq_frac": ch_m / n_reads,
            "changed_primaries": ch_p, "changed_mapqs": ch_m,
            "candidates_pruned_frac": round(cnt["pruned"] / tot, 4) if tot else 0.0,
            "reads_kept_whole": cnt["reads_whole"],
            "train": {"pairs": args.train_pairs, "label_cut": args.label_cut, "samples": rep["samples"], "positives": rep["positives"],
                      "loss_first": round(rep["loss_first"], 5), "loss_last": round(rep["loss_last"], 5),
                      "train_recall": round(rep["train_recall"], 6), "train_prune": round(rep["train_prune"], 4),
                      "ms_collect": round(rep["ms_collect"], 1), "ms_train": round(rep["ms_train"], 1),
                      "s_generate": round(t_gen, 1), "reads": "fresh pairs of the same genome (seed + 99)"}}


# ---------------------------------------------------------------------------
# CPU (reference path restatement)
# ---------------------------------------------------------------------------
def cpu_time(prefix, d, meta, n_sample: int, threads: int, records=False):
    from oracle import pyoracle as O
    O.build()
    m = O.Mapper(prefix, threads=threads)
    paired = meta["paired"]
    o1 = d["o1"]
    k = min(n_sample, len(o1) - 1)
    R1 = O.Reads(d["b1"][:int(o1[k])], d["q1"][:int(o1[k])], o1[:k + 1])
    if paired:
        o2 = d["o2"]
        R2 = O.Reads(d["b2"][:int(o2[k])], d["q2"][:int(o2[k])], o2[:k + 1])
        t, r1, r2 = m.time_map_paired(R1, R2)
        recs = [r1, r2]
        reads = 2 * k
    else:
        t, r1 = m.time_map_single(R1)
        recs = [r1]
        reads = k
    m.close()
    return (reads, t, recs) if records else (reads, t)


def cpu_baseline(prefix, d, meta, gpu_records=None):
    """The oracle on the first reads (pairs) of the workload on every host
    thread: its reads/s, and its records against the GPU's for the same reads
    (the GPU mapped them as the first reads of the whole set, which the batch
    schedule makes equivalent)."""
    threads = os.cpu_count() or 1
    n = 40_000 if meta["paired"] else 10_000
    reads, t, recs = cpu_time(prefix, d, meta, n, threads, records=True)
    cb = {"value": round(reads / t, 1), "unit": "reads/s", "cores": threads, "kind": "port",
          "sample": f"first {reads} reads ({'pairs' if meta['paired'] else 'reads'} incl. the serial warm-up) "
                    f"of the same workload, oracle/ C++ restatement, {threads} threads"}
    if gpu_records is None:
        return cb
    par = [record_parity(g, e, len(e["contig"])) for g, e in zip(gpu_records, recs)]
    parity = {"compared": sum(p["compared"] for p in par), "mismatched": sum(p["mismatched"] for p in par),
              "by_read_set": par, "sample": cb["sample"]}
    return cb, parity


def run_reference(args, prefix, d, meta):
    threads = os.cpu_count() or 1
    n = 50_000 if meta["paired"] else 10_000
    for _ in range(args.warmup):
        cpu_time(prefix, d, meta, min(n, 2000), threads)
    times, reads = [], 0
    for _ in range(args.steps):
        reads, t = cpu_time(prefix, d, meta, n, threads)
        times.append(t)
    v = reads / statistics.mean(times)
    cb = {"value": round(v, 1), "unit": "reads/s", "cores": threads, "kind": "port",
          "sample": f"first {reads} reads of the workload per step (oracle/ C++ restatement of the reference CPU path)"}
    return {"impl": "reference", "metric": METRIC, "value": round(v, 1), "unit": "reads/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(times) * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded)", "config": meta, "cpu_baseline": cb,
            "e2e": {"value": round(v, 1), "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


# ---------------------------------------------------------------------------
# stages around the mapping path: index build, SAM output, the command line
# ---------------------------------------------------------------------------
def _stage_line(stage, meta, value, unit, extra):
    out = {"stage": stage, "metric": f"{stage} throughput", "value": round(value, 3), "unit": unit, "n_gpus": 1,
           "higher_is_better": True, "data": "synthetic (seeded)", "config": meta}
    out.update(extra)
    return out


def _sha(path):
    import hashlib
    h = hashlib.sha256()
    with open(path, "rb") as f:
        for b in iter(lambda: f.read(1 << 24), b""):
            h.update(b)
    return h.hexdigest()


def run_stage_index(args, prefix, meta):
    """build-hash of the workload's genome: pbw_build_hash (GPU) against the
    oracle's builder (one host thread); the two .sthash files must be equal."""
    import probebwa_gb300 as P
    from oracle import pyoracle as O
    P.build()
    O.build()
    out = os.path.join(args.cache, "stage_index_gpu")
    for _ in range(max(1, args.warmup)):
        P.build_hash(prefix, out)
    times = []
    for _ in range(args.steps):
        t = time.time()
        P.build_hash(prefix, out)
        times.append(time.time() - t)
    ref = os.path.join(args.cache, "stage_index_cpu")
    t = time.time()
    O.build_hash(prefix, ref)
    t_cpu = time.time() - t
    same = _sha(out + ".sthash") == _sha(ref + ".sthash")
    bp = meta["genome_bp"]
    v = bp / statistics.mean(times)
    return _stage_line("index", meta, v / 1e6, "Mbp/s", {
        "wall_s": [round(x, 3) for x in times], "sthash_bytes": os.path.getsize(out + ".sthash"),
        "parity": "sthash byte-identical to the oracle's" if same else "MISMATCH",
        "timed": "whole pbw_build_hash call: .stidx read + upload, device build, table download, .sthash write",
        "cpu_baseline": {"value": round(bp / t_cpu / 1e6, 3), "unit": "Mbp/s", "cores": 1, "kind": "port",
                         "sample": "whole genome, oracle/ HashTableBuilder restatement"}})


def _map_records(P, m, d, meta, opts):
    import ctypes as C
    R1 = P.Reads(d["b1"], d["q1"], d["o1"])
    R2 = P.Reads(d["b2"], d["q2"], d["o2"]) if meta["paired"] else None
    R1.ids = [f"p{i}" for i in range(R1.n)]
    O1 = P.alloc_records(R1.n, len(R1.bases))
    if R2 is not None:
        R2.ids = R1.ids
        O2 = P.alloc_records(R2.n, len(R2.bases))
        mdl = P.InsertModelC(opts.insert_size_mean, opts.insert_size_sd, 0)
        m._check(P.lib().pbw_map_paired(m.h, C.byref(mdl), C.byref(R1.c()), C.byref(R2.c()),
                                        C.byref(P.records_c(O1)), C.byref(P.records_c(O2))))
        return [(R1, O1), (R2, O2)]
    m._check(P.lib().pbw_map_single(m.h, C.byref(R1.c()), C.byref(P.records_c(O1))))
    return [(R1, O1)]


def run_stage_sam(args, prefix, d, meta):
    """SAM text of every record of one map call: pbw_sam_format (device
    formatting, inputs up and text down inside the timing) against the
    oracle's SAM writer on a sample."""
    import ctypes as C
    import probebwa_gb300 as P
    from oracle import pyoracle as O
    P.build()
    O.build()
    opts = P.MapperOptions()
    m = P.Mapper(prefix, options=opts)
    sources = _map_records(P, m, d, meta, opts)
    arr, keep = m._sam_sources(sources)
    so = P.SamOptionsC(b"probebwa map", None, 0)
    n = C.c_uint64(0)
    L = P.lib()
    m._check(L.pbw_sam_format(m.h, C.byref(so), len(sources), arr, None, 0, None, 0, C.byref(n)))
    buf = pinned(np.zeros(n.value, np.uint8))
    n_rec = sum(len(o["contig"]) for _, o in sources)

    def once():
        m._check(L.pbw_sam_format(m.h, C.byref(so), len(sources), arr, None, 0, None, 0, C.byref(n)))
        m._check(L.pbw_sam_format(m.h, C.byref(so), len(sources), arr, None, 0, _ptr_np(buf), buf.size, C.byref(n)))

    for _ in range(max(1, args.warmup)):
        once()
    times = []
    for _ in range(args.steps):
        t = time.time()
        once()
        times.append(time.time() - t)
    v = n_rec / statistics.mean(times)
    # oracle on a sample of the records
    k = min(100_000, len(sources[0][1]["contig"]))
    om = O.Mapper(prefix)
    sub = []
    for R, rec in sources:
        o = R.offsets[:k + 1]
        Rs = O.Reads(R.bases[:int(o[-1])], R.quals[:int(o[-1])], o, R.ids[:k])
        rs = {key: (val[:k] if key not in ("cigar_off", "cigar") else val) for key, val in rec.items()
              if not key.startswith("_")}
        rs["cigar_off"] = rec["cigar_off"][:k + 1]
        sub.append((Rs, rs))
    path = os.path.join(args.cache, "stage_sam_cpu.sam")
    t = time.time()
    text = om.sam_text(path, sub)
    t_cpu = time.time() - t
    gpu_sample = m.sam_text(sources, np.arange(k * len(sources), dtype=np.uint64))
    om.close()
    m.close()
    return _stage_line("sam", meta, v, "records/s", {
        "sam_bytes": int(n.value), "gb_per_s": round(n.value / statistics.mean(times) / 1e9, 3),
        "wall_s": [round(x, 4) for x in times],
        "parity": ("first %d records byte-identical to the oracle's SAM" % (k * len(sources)))
        if gpu_sample == text else "MISMATCH",
        "timed": "pbw_sam_format sizing + formatting calls: records, reads and IDs up, text down",
        "cpu_baseline": {"value": round(k * len(sources) / t_cpu, 1), "unit": "records/s", "cores": 1, "kind": "port",
                         "sample": f"first {k * len(sources)} records, oracle/ format_sam_records restatement"}})


def _ptr_np(a):
    return a.ctypes.data


def _write_fastq(path, b, q, o, tag):
    """Fixed-length reads as FASTQ with fixed-width IDs (Phred+33)."""
    n = len(o) - 1
    L = int(o[1] - o[0]) if n else 0
    if n and not np.all(np.diff(o) == L):
        raise ValueError("fixed-length reads expected")
    ids = np.char.encode(np.char.add(f"@{tag}", np.char.zfill(np.arange(n).astype(str), 8)))
    w = len(ids[0]) if n else 0
    rec = np.empty((n, w + 1 + L + 3 + L + 1), np.uint8)
    rec[:, :w] = np.frombuffer(b"".join(ids.tolist()), np.uint8).reshape(n, w)
    rec[:, w] = 10
    rec[:, w + 1:w + 1 + L] = b[:n * L].reshape(n, L)
    rec[:, w + 1 + L:w + 4 + L] = np.frombuffer(b"\n+\n", np.uint8)
    rec[:, w + 4 + L:w + 4 + 2 * L] = q[:n * L].reshape(n, L) + 33
    rec[:, -1] = 10
    with open(path, "wb") as f:
        f.write(rec.tobytes())


def run_stage_cli(args, prefix, d, meta):
    """`probebwa map` end to end (process start, index load, FASTQ parse,
    mapping, SAM written to a file) against the oracle's command line on a
    sample of the same reads."""
    import probebwa_gb300 as P
    from oracle import pyoracle as O
    from probebwa_gb300 import native_build
    P.build()
    O.build()
    paired = meta["paired"]
    files = [os.path.join(args.cache, f"stage_cli_r{m}.fq") for m in ((1, 2) if paired else (1,))]
    for mate, fp in zip((1, 2), files):
        if not os.path.exists(fp):
            _write_fastq(fp, d[f"b{mate}"], d[f"q{mate}"], d[f"o{mate}"], "r")
    n_reads = (len(d["o1"]) - 1) * len(files)
    out = os.path.join(args.cache, "stage_cli_gpu.sam")
    cmd = ["probebwa", "map", "-g", prefix, "-h", prefix, "-o", out, "-M", *files]
    for _ in range(max(1, min(args.warmup, 1))):
        subprocess.run(cmd, executable=native_build.CLI, check=True)
    times = []
    for _ in range(args.steps):
        t = time.time()
        subprocess.run(cmd, executable=native_build.CLI, check=True)
        times.append(time.time() - t)
    # the oracle's command line on the first k reads (pairs) of the same files
    k = 20_000 if paired else 10_000
    rec_len = os.path.getsize(files[0]) // (len(d["o1"]) - 1)
    small = []
    for fp in files:
        sp = fp.replace(".fq", f".first{k}.fq")
        if not os.path.exists(sp):
            with open(fp, "rb") as f, open(sp, "wb") as g:
                g.write(f.read(rec_len * k))
        small.append(sp)
    ref_out = os.path.join(args.cache, "stage_cli_cpu.sam")
    threads = os.cpu_count() or 1
    rcmd = ["probebwa", "map", "-g", prefix, "-h", prefix, "-t", str(threads), "-o", ref_out, "-M", *small]
    t = time.time()
    subprocess.run(rcmd, executable=O.CLI_PATH, check=True)
    t_cpu = time.time() - t
    gcmd = ["probebwa", "map", "-g", prefix, "-h", prefix, "-t", str(threads), "-o", ref_out + ".gpu", "-M", *small]
    subprocess.run(gcmd, executable=native_build.CLI, check=True)
    same = ([x for x in open(ref_out, "rb").read().split(b"\n") if not x.startswith(b"@PG")] ==
            [x for x in open(ref_out + ".gpu", "rb").read().split(b"\n") if not x.startswith(b"@PG")])
    v = n_reads / statistics.mean(times)
    return _stage_line("cli", meta, v, "reads/s", {
        "wall_s": [round(x, 2) for x in times], "sam_bytes": os.path.getsize(out),
        "parity": (f"SAM of the first {k * len(files)} reads identical to the oracle CLI's (the @PG line, which "
                   "echoes each argv, excluded)") if same else "MISMATCH",
        "timed": "wall time of the whole command, index load included",
        "cpu_baseline": {"value": round(k * len(files) / t_cpu, 1), "unit": "reads/s", "cores": threads,
                         "kind": "port", "sample": f"oracle command line on the first {k * len(files)} reads "
                                                   f"({'pairs' if paired else 'reads'}), index load included"}})


def batch_workload(args):
    """Mixed-length workload of the batching configuration, scaled to one
    box's minutes: a 300 Mbp genome (12 contigs of U(50, 250) relative size,
    GC 41%, 45% copies of 500 interspersed repeat families with 300 bp-6 kbp
    consensus and 2-25% divergence, 3% tandem arrays); 1,000,000 single-end
    reads and 500,000 pairs (insert N(300, 80)) trimmed to lengths U[60, 250],
    0.5% substitutions and 0.05% indels; fresh reads of the same kind (200,000
    single-end, 100,000 pairs) to train the ranker. The index is built with
    pbw_build_hash."""
    import probebwa_gb300 as P
    from probebwa_gb300 import synth
    seed = 0x5EED0002
    os.makedirs(args.cache, exist_ok=True)
    prefix = os.path.join(args.cache, "batch")
    rp = prefix + ".reads.npz"
    if not (os.path.exists(prefix + ".sthash") and os.path.exists(rp)):
        t = time.time()
        contigs = synth.genome_families(seed)
        synth.write_stidx(prefix, contigs)
        P.build_hash(prefix, prefix)
        log(f"[bench] batch genome + index: {time.time() - t:.1f}s")
        t = time.time()
        d = {}
        for tag, n_se, n_pe, s0 in (("ev", 1_000_000, 500_000, 11), ("tr", 200_000, 100_000, 23)):
            b, q, o = synth.reads_single_fast(seed + s0, contigs, n_se, L=250, sub=0.005, indel=0.0005)
            d[f"{tag}_s_b"], d[f"{tag}_s_q"], d[f"{tag}_s_o"] = synth.trim_lengths(seed + s0 + 1, b, q, o)
            b1, q1, o1, b2, q2, o2 = synth.reads_paired_fast(seed + s0 + 2, contigs, n_pe, L=250, mean=300.0, sd=80.0,
                                                             sub=0.005, indel=0.0005)
            d[f"{tag}_1_b"], d[f"{tag}_1_q"], d[f"{tag}_1_o"] = synth.trim_lengths(seed + s0 + 3, b1, q1, o1)
            d[f"{tag}_2_b"], d[f"{tag}_2_q"], d[f"{tag}_2_o"] = synth.trim_lengths(seed + s0 + 4, b2, q2, o2)
        np.savez(rp, **d)
        log(f"[bench] batch reads: {time.time() - t:.1f}s")
    d = dict(np.load(rp))
    return prefix, d


def run_stage_batch(args):
    """Plain, batched (length bins + tuned band DP + pair graphs) and
    ranked+batched mapping of the mixed-length workload, device time per
    pass; changed primaries and MAPQs of the ranked records against the plain
    ones on the same reads."""
    import probebwa_gb300 as P
    P.build()
    prefix, d = batch_workload(args)
    R = lambda tag, k: P.Reads(d[f"{tag}_{k}_b"], d[f"{tag}_{k}_q"], d[f"{tag}_{k}_o"])
    se, p1, p2 = R("ev", "s"), R("ev", "1"), R("ev", "2")
    n_reads = se.n + p1.n + p2.n

    def dev_ms(st):
        return dev_time(st)

    def timed(m, fn):
        for _ in range(max(1, args.warmup)):
            fn()
        ts, out = [], None
        for _ in range(args.steps):
            out = fn()
            ts.append(dev_ms(m.stats()))
        return statistics.mean(ts), out

    res = {}
    with P.Mapper(prefix) as ms, P.Mapper(prefix) as mp:
        modes = {"plain": dict(length_bins=0, autotune=0, band_lanes=8, pair_graphs=0),
                 "batched": dict(length_bins=1, autotune=1, band_lanes=0, pair_graphs=1)}
        recs = {}
        for name, kw in modes.items():
            ms.set_tuning(**kw)
            mp.set_tuning(**kw)
            t_se, o_se = timed(ms, lambda: ms.map_single(se))
            t_pe, o_pe = timed(mp, lambda: mp.map_paired(p1, p2))
            recs[name] = (o_se, o_pe[0], o_pe[1])
            res[name] = {"ms_single": round(t_se, 2), "ms_pairs": round(t_pe, 2),
                         "reads_per_s": round(n_reads / ((t_se + t_pe) / 1e3), 1)}
        res["batched"]["tuning_single"] = ms.tuning()
        res["batched"]["tuning_pairs"] = mp.tuning()
        rep_s = ms.ranker_train(R("tr", "s"), label_cut=args.label_cut)
        rep_p = mp.ranker_train(R("tr", "1"), R("tr", "2"), label_cut=args.label_cut)
        ms.ranker_enable(True)
        mp.ranker_enable(True)
        t_se, o_se = timed(ms, lambda: ms.map_single(se))
        t_pe, o_pe = timed(mp, lambda: mp.map_paired(p1, p2))
        cs, cp = ms.ranker_counters(), mp.ranker_counters()
    ch_p = ch_m = 0
    for a, b in zip((o_se, o_pe[0], o_pe[1]), recs["plain"]):
        x, y = _primary_changes(a, b)
        ch_p += x
        ch_m += y
    same_batched = sum(sum(_primary_changes(a, b)) for a, b in zip(recs["batched"], recs["plain"]))
    res["ranked_batched"] = {"ms_single": round(t_se, 2), "ms_pairs": round(t_pe, 2),
                             "reads_per_s": round(n_reads / ((t_se + t_pe) / 1e3), 1),
                             "changed_primary_frac": ch_p / n_reads, "changed_mapq_frac": ch_m / n_reads,
                             "candidates_pruned_frac_single": round(cs["pruned"] / max(1, cs["kept"] + cs["pruned"]), 4),
                             "candidates_pruned_frac_pairs": round(cp["pruned"] / max(1, cp["kept"] + cp["pruned"]), 4),
                             "train_single": {k: rep_s[k] for k in ("samples", "positives", "train_recall", "train_prune")},
                             "train_pairs": {k: rep_p[k] for k in ("samples", "positives", "train_recall", "train_prune")}}
    res["batched"]["records_differing_from_plain"] = int(same_batched)
    v = res["ranked_batched"]["reads_per_s"]
    meta = {"workload": "mixed-length 60-250 bp: 300 Mbp genome (45% repeat families, 3% tandem), "
                        "1,000,000 single-end reads + 500,000 pairs", "reads": n_reads}
    return _stage_line("batch", meta, v, "reads/s", dict(res, speedup_vs_plain=round(v / res["plain"]["reads_per_s"], 3)))


# ---------------------------------------------------------------------------
# parity: records of the GPU path against the oracle's, field by field
# ---------------------------------------------------------------------------
PARITY_EXACT = ("contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen", "as_score", "nm")


def _cigar_rows(r, n):
    """Per record the CIGAR words as bytes (for a row-by-row comparison)."""
    co = r["cigar_off"].astype(np.int64)
    cg = r["cigar"]
    return [cg[co[i]:co[i + 1]].tobytes() for i in range(n)]


def record_parity(got: dict, exp: dict, n: int | None = None, posterior_ulps: int = 4) -> dict:
    """Reads whose records differ: bit-exact on every integer field, the
    CIGAR and the log-likelihood bits; the posterior within a few ulps (its
    last step is pow(10, -phred / 10) of a continuous phred). Returns the
    count compared, the count mismatched and the mismatches per field."""
    n = len(exp["contig"]) if n is None else n
    bad = np.zeros(n, bool)
    fields = {}
    for k in PARITY_EXACT:
        d = got[k][:n] != exp[k][:n]
        if d.any():
            fields[k] = int(d.sum())
        bad |= d
    d = got["log_lk"][:n].view(np.uint64) != exp["log_lk"][:n].view(np.uint64)
    if d.any():
        fields["log_lk"] = int(d.sum())
    bad |= d
    ep = exp["posterior"][:n]
    d = np.abs(got["posterior"][:n] - ep) > posterior_ulps * np.spacing(np.maximum(np.abs(ep), 1e-300))
    if d.any():
        fields["posterior"] = int(d.sum())
    bad |= d
    gc, ec = _cigar_rows(got, n), _cigar_rows(exp, n)
    d = np.array([a != b for a, b in zip(gc, ec)], bool) if n else np.zeros(0, bool)
    if d.any():
        fields["cigar"] = int(d.sum())
    bad |= d
    return {"compared": int(n), "mismatched": int(bad.sum()), "fields": fields}


def _slice_reads(b, q, o, k):
    o = o[:k + 1]
    return b[:int(o[-1])], q[:int(o[-1])], o


def _rec_copy(recs, n=None):
    n = len(recs["contig"]) if n is None else n
    out = {k: np.array(v[:n]) for k, v in recs.items() if not k.startswith("_") and k not in ("cigar_off", "cigar")}
    co = recs["cigar_off"][:n + 1]
    out["cigar_off"] = np.array(co)
    out["cigar"] = np.array(recs["cigar"][:int(co[-1])])
    return out


def _rec_diff(a, b):
    """Reads whose record differs in any field (tie-order exposure, batching
    identity)."""
    return record_parity(a, b)["mismatched"]


# ---------------------------------------------------------------------------
# hg38-scale workloads (configurations 2, 3 and 4)
# ---------------------------------------------------------------------------
class HgWorkload:
    """Genome, index files and read chunks of the 3.1 Gbp configurations."""

    def __init__(self, args, cfg: int):
        import torch
        import probebwa_gb300 as P
        from probebwa_gb300 import synth_gpu as S
        P.build()
        self.cfg = 4 if cfg == 4 else 2
        seed = SEED[self.cfg]
        total = int(args.genome_bp)
        cache = os.path.join(args.cache, f"hg{self.cfg}_{total}")
        os.makedirs(cache, exist_ok=True)
        self.prefix = os.path.join(cache, "genome")
        t = time.time()
        names, lens, codes = S.genome_hg(SEED[2], total=total)
        self.regions = None
        if self.cfg == 4:
            codes, self.regions = S.add_stress(seed, codes, lens)
        self.names, self.lens, self.codes = names, lens, codes
        self.t_genome = time.time() - t
        # the index files are cached per box; a checksum of the generated
        # genome guards against a stale cache
        g = torch.as_tensor(codes).cuda()
        w = torch.arange(1, 8, device=g.device, dtype=torch.int64).repeat(len(codes) // 7 + 1)[:len(codes)]
        csum = int((g.to(torch.int64) * w).sum().item())
        meta_path = os.path.join(cache, "meta.json")
        meta = json.load(open(meta_path)) if os.path.exists(meta_path) else {}
        t = time.time()
        if meta.get("checksum") != csum or not os.path.exists(self.prefix + ".sthash"):
            S.write_stidx(self.prefix, names, lens, codes)
            P.build_hash(self.prefix, self.prefix)
            json.dump({"checksum": csum}, open(meta_path, "w"))
            self.index_built = True
        else:
            self.index_built = False
        self.t_index = time.time() - t
        t = time.time()
        self.chunks, self.train = [], None
        if self.cfg == 2:
            self.n_chunks = args.hg_chunks
            for c in range(self.n_chunks):
                se = S.reads(seed + 1000 + 2 * c, names, lens, codes, args.hg_se, 250, trim=(60, 250), g_dev=g)
                pe = S.reads(seed + 1001 + 2 * c, names, lens, codes, args.hg_pairs, 250, paired=True, mean=300.0,
                             sd=80.0, trim=(60, 250), g_dev=g)
                self.chunks.append({"se": se, "pe": pe})
            if args.train_reads:
                tr_se = S.reads(seed + 99, names, lens, codes, args.train_reads // 2, 250, trim=(60, 250), g_dev=g)
                tr_pe = S.reads(seed + 98, names, lens, codes, args.train_reads // 4, 250, paired=True, mean=300.0,
                                sd=80.0, trim=(60, 250), g_dev=g)
                self.train = {"se": tr_se, "pe": tr_pe}
            self.insert = (300.0, 80.0)
        else:
            self.n_chunks = args.hg_chunks
            kw = dict(paired=True, mean=500.0, sd=120.0, sub=0.03, indel=0.003, qmu=28.0, qsd=8.0,
                      regions=self.regions, region_frac=0.3, g_dev=g)
            for c in range(self.n_chunks):
                pe = S.reads(seed + 1001 + 2 * c, names, lens, codes, args.stress_pairs, 250, **kw)
                self.chunks.append({"se": None, "pe": pe})
            if args.train_reads:
                self.train = {"se": None, "pe": S.reads(seed + 98, names, lens, codes, args.train_reads // 2, 250,
                                                        **kw)}
            self.insert = (500.0, 120.0)
        del g
        torch.cuda.empty_cache()
        self.t_reads = time.time() - t
        self.reads_per_chunk = [(len(c["se"][2]) - 1 if c["se"] else 0) + 2 * (len(c["pe"][2]) - 1)
                                for c in self.chunks]

    def meta(self):
        if self.cfg == 2:
            w = ("batching + ranker: 3.1 Gbp hg38-scale genome (24 contigs, 45% from 500 repeat families, 3% tandem), "
                 f"{sum(self.reads_per_chunk):,} reads of 60-250 bp in {self.n_chunks} chunks of "
                 f"{self.reads_per_chunk[0]:,} (half single-end, half pairs, insert N(300,80))")
        else:
            w = ("repeat stress: 3.1 Gbp genome + 200 families x 32-64 near-identical copies + homopolymer-rich "
                 f"regions, {sum(self.reads_per_chunk) // 2:,} pairs 2x250 in {self.n_chunks} chunks, insert "
                 "N(500,120), 3% subs, 0.3% indels, Q N(28,8)")
        return {"workload": w, "genome_bp": int(np.sum(self.lens)), "contigs": len(self.lens),
                "reads": int(sum(self.reads_per_chunk)), "chunks": self.n_chunks,
                "reads_per_step": int(self.reads_per_chunk[0]), "paired": True,
                "seed": SEED[self.cfg], "generate_s": round(self.t_genome + self.t_reads, 1),
                "index_s": round(self.t_index, 1), "index_built_here": self.index_built}


def _hg_inputs(P, W):
    """Pinned host copies of every chunk's reads (the C ABI's inputs)."""
    out = []
    for c in W.chunks:
        d = {}
        if c["se"] is not None:
            d["se"] = P.Reads(*[pinned(x) for x in c["se"]])
        b1, q1, o1, b2, q2, o2 = c["pe"]
        d["p1"] = P.Reads(pinned(b1), pinned(q1), pinned(o1))
        d["p2"] = P.Reads(pinned(b2), pinned(q2), pinned(o2))
        out.append(d)
    return out


class HgRunner:
    """Maps the chunks through the C ABI with pinned host buffers; one handle
    for single-end reads and one for pairs (each has its own ranker)."""

    def __init__(self, P, W, inputs, group_width=16, concurrent=True):
        import ctypes as C
        self.P, self.W, self.C, self.L = P, W, C, P.lib()
        self.concurrent = concurrent
        self.inputs = inputs
        opts = P.MapperOptions(group_width=group_width)
        self.opts = opts
        t = time.time()
        self.ms = P.Mapper(W.prefix, options=opts) if W.cfg == 2 else None
        self.mp = P.Mapper(W.prefix, options=opts)
        self.t_open = time.time() - t
        n_se = max([len(d["se"].offsets) - 1 for d in inputs if "se" in d] + [0])
        b_se = max([len(d["se"].bases) for d in inputs if "se" in d] + [0])
        n_pe = max(len(d["p1"].offsets) - 1 for d in inputs)
        b_pe = max(max(len(d["p1"].bases), len(d["p2"].bases)) for d in inputs)
        pin = lambda r: {k: pinned(v) for k, v in r.items()}
        self.o_se = pin(P.alloc_records(n_se, b_se)) if n_se else None
        self.o_p1 = pin(P.alloc_records(n_pe, b_pe))
        self.o_p2 = pin(P.alloc_records(n_pe, b_pe))

    def handles(self):
        return [m for m in (self.ms, self.mp) if m is not None]

    def set_tuning(self, **kw):
        for m in self.handles():
            m.set_tuning(**kw)

    def _view(self, o, n):
        r = {k: v[:n] for k, v in o.items() if k not in ("cigar_off", "cigar") and not k.startswith("_")}
        r["cigar_off"] = o["cigar_off"][:n + 1]
        r["cigar"] = o["cigar"]
        return r

    def step(self, c):
        """Maps chunk c; returns (reads, device ms, end-to-end ms, stats list).

        The single-end and the paired call run on their own handles; with
        `concurrent` they are issued from two host threads at once, so the
        single-end work fills the SMs the paired call's serial pair batches
        leave idle. Device ms is then the union of the calls' device spans
        (compute span on the device clock, plus the record copy), end-to-end
        ms the host wall time of the step (input copies, mapping and record
        copies of both calls)."""
        P, C, L = self.P, self.C, self.L
        d = self.inputs[c]
        reads = 0
        calls = []
        if "se" in d:
            R = d["se"]
            o = self._view(self.o_se, R.n)
            calls.append((self.ms, lambda R=R, o=o: L.pbw_map_single(self.ms.h, C.byref(R.c()),
                                                                    C.byref(P.records_c(o)))))
            reads += R.n
        R1, R2 = d["p1"], d["p2"]
        o1, o2 = self._view(self.o_p1, R1.n), self._view(self.o_p2, R2.n)
        mdl = P.InsertModelC(self.opts.insert_size_mean, self.opts.insert_size_sd, 0)
        calls.append((self.mp, lambda: L.pbw_map_paired(self.mp.h, C.byref(mdl), C.byref(R1.c()), C.byref(R2.c()),
                                                        C.byref(P.records_c(o1)), C.byref(P.records_c(o2)))))
        reads += R1.n + R2.n
        rcs = [None] * len(calls)
        t = time.perf_counter()
        if self.concurrent and len(calls) > 1:
            import threading

            def run(i):
                rcs[i] = calls[i][1]()
            th = [threading.Thread(target=run, args=(i,)) for i in range(len(calls))]
            for x in th:
                x.start()
            for x in th:
                x.join()
        else:
            for i, (_, fn) in enumerate(calls):
                rcs[i] = fn()
        wall = (time.perf_counter() - t) * 1e3
        for (m, _), rc in zip(calls, rcs):
            m._check(rc)
        stats = [m.stats() for m, _ in calls]
        if self.concurrent and len(calls) > 1:
            dev = max(s["t_compute_end_ms"] + s["ms_d2h"] for s in stats) - min(s["t_compute_begin_ms"] for s in stats)
            e2e = wall
        else:
            dev = sum(dev_time(s) for s in stats)
            e2e = sum(s["ms_total"] for s in stats)
        return reads, dev, e2e, stats

    def records(self, c):
        """Copies of the records of the chunk mapped last (chunk c)."""
        d = self.inputs[c]
        out = {}
        if "se" in d:
            out["se"] = _rec_copy(self._view(self.o_se, d["se"].n))
        out["p1"] = _rec_copy(self._view(self.o_p1, d["p1"].n))
        out["p2"] = _rec_copy(self._view(self.o_p2, d["p2"].n))
        return out

    def close(self):
        for m in self.handles():
            m.close()


def _sum_stats(stats):
    keys = ("ms_seed", "ms_cluster", "ms_align", "ms_pair", "ms_finalize", "ms_d2h", "ms_total", "seed_probes",
            "seed_entries", "seed_hits", "dp_jobs", "dp_cells", "kernel_launches", "window_jobs", "window_cells")
    out = {k: 0 for k in keys}
    for s in stats:
        for k in keys:
            out[k] += s[k]
    return out


def _timed_steps(R, W, warmup, steps, start, keep=None, clock=False):
    """warmup + steps chunk maps from chunk `start` on; returns the timed
    steps' totals and (with keep) the records of every chunk mapped."""
    c = start
    for _ in range(warmup):
        R.step(c % W.n_chunks)
        if keep is not None and c % W.n_chunks not in keep:
            keep[c % W.n_chunks] = R.records(c % W.n_chunks)
        c += 1
    clk = ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) if clock else None
    if clk:
        clk.start()
    reads = dev = e2e = 0.0
    all_stats = []
    per_step = []
    for _ in range(steps):
        ci = c % W.n_chunks
        n, d, e, st = R.step(ci)
        if keep is not None and ci not in keep:
            keep[ci] = R.records(ci)
        reads += n
        dev += d
        e2e += e
        all_stats += st
        per_step.append(d)
        c += 1
    clocks = clk.stop() if clk else None
    return {"reads": reads, "dev_ms": dev, "e2e_ms": e2e, "stats": _sum_stats(all_stats), "clocks": clocks,
            "step_ms": per_step, "next": c}


def _changes(recs, base):
    """Reads whose primary (contig, POS, FLAG, CIGAR) or MAPQ changed."""
    cp = cm = n = 0
    for ci, r in recs.items():
        for k in r:
            a, b = _primary_changes(r[k], base[ci][k])
            cp += a
            cm += b
            n += len(r[k]["contig"])
    return cp, cm, n


def _h2d_d2h(inputs, R, c):
    d = inputs[c]
    h2d = sum(int(x.bases.nbytes + x.quals.nbytes + x.offsets.nbytes) for k, x in d.items())
    d2h = 0
    for k, x in d.items():
        o = R.records(c)[k]
        d2h += sum(int(v.nbytes) for kk, v in o.items() if kk not in ("cigar",)) + 4 * len(o["cigar"])
    return h2d, d2h


def hg_oracle_sample(W, n_se, n_pairs, threads):
    """The oracle on the first n_se single-end reads and n_pairs pairs of
    chunk 0 (mapped from the default insert model, as the GPU maps the
    chunk): records and the seconds each part took."""
    from oracle import pyoracle as O
    O.build()
    t = time.time()
    om = O.Mapper(W.prefix, threads=threads)
    t_open = time.time() - t
    c = W.chunks[0]
    out, secs, reads = {}, 0.0, 0
    if c["se"] is not None and n_se:
        b, q, o = _slice_reads(*c["se"], n_se)
        t, out["se"] = om.time_map_single(O.Reads(b, q, o))
        secs += t
        reads += n_se
    b1, q1, o1, b2, q2, o2 = c["pe"]
    R1 = O.Reads(*_slice_reads(b1, q1, o1, n_pairs))
    R2 = O.Reads(*_slice_reads(b2, q2, o2, n_pairs))
    t, out["p1"], out["p2"] = om.time_map_paired(R1, R2)
    secs += t
    reads += 2 * n_pairs
    om.close()
    return out, secs, reads, t_open


# DRAM traffic of K1 per read on the 3.1 Gbp workload (ncu dram__bytes_read.sum +
# dram__bytes_write.sum of a 131,072-read launch: 133.21 GB)
SEED_TRAFFIC_PER_READ_HG = 133.212596736e9 / 131072


def int32_peak():
    """Measured INT32 add and max throughput of this GPU (independent chains,
    CUDA events): G ops/s."""
    import ctypes as C
    import probebwa_gb300 as P
    L = P.lib()
    add, mx = C.c_double(0), C.c_double(0)
    rc = L.pbw_int32_peak(0, C.byref(add), C.byref(mx))
    return (add.value, mx.value) if rc == 0 else (None, None)


def run_hg(args, rank, world):
    import torch
    import probebwa_gb300 as P
    torch.cuda.set_device(int(os.environ.get("LOCAL_RANK", "0")))
    t_all = time.time()
    W = HgWorkload(args, args.config)
    log(f"[bench] hg workload ready: genome {W.t_genome:.1f}s index {W.t_index:.1f}s reads {W.t_reads:.1f}s")
    inputs = _hg_inputs(P, W)
    R = HgRunner(P, W, inputs, concurrent=bool(args.hg_concurrent))
    log(f"[bench] handles open: {R.t_open:.1f}s")
    plain = {}
    # 1. the plain method with batching (the drop-in path; `value`)
    main = _timed_steps(R, W, args.warmup, args.steps, 0, keep=plain, clock=True)
    tuning = {k: (m.tuning() if m else None) for k, m in (("single", R.ms), ("pairs", R.mp))}
    nxt = main["next"]
    # every chunk's plain records (for the other forms' comparisons)
    for ci in range(W.n_chunks):
        if ci not in plain:
            R.step(ci)
            plain[ci] = R.records(ci)
    h2d, d2h = _h2d_d2h(inputs, R, (nxt - 1) % W.n_chunks)
    steps_other = min(args.steps, args.other_steps) if args.other_steps else args.steps
    warm_other = max(3, min(args.warmup, 3))
    # 2. batching off
    R.set_tuning(length_bins=0, autotune=0, band_lanes=8, pair_graphs=0)
    recs_u = {}
    unb = _timed_steps(R, W, warm_other, steps_other, 0, keep=recs_u)
    R.set_tuning(length_bins=1, autotune=1, band_lanes=0, pair_graphs=1)
    differ_unbatched = sum(_rec_diff(recs_u[ci][k], plain[ci][k]) for ci in recs_u for k in recs_u[ci])
    # 3. ranked + batched: rankers trained on fresh reads of the same genome
    t = time.time()
    cut = args.label_cut
    train = {}
    if R.ms is not None and W.train["se"] is not None:
        train["single"] = R.ms.ranker_train(P.Reads(*W.train["se"]), label_cut=cut)
        R.ms.ranker_enable(True)
    b1, q1, o1, b2, q2, o2 = W.train["pe"]
    train["pairs"] = R.mp.ranker_train(P.Reads(b1, q1, o1), P.Reads(b2, q2, o2), label_cut=cut)
    R.mp.ranker_enable(True)
    t_train = time.time() - t
    for m in R.handles():
        m.ranker_enable(True)  # counters from here
    recs_r = {}
    rk = _timed_steps(R, W, warm_other, steps_other, 0, keep=recs_r)
    cnt = [m.ranker_counters() for m in R.handles()]
    for m in R.handles():
        m.ranker_enable(False)
    ch_p, ch_m, n_cmp = _changes(recs_r, plain)
    R.close()
    # 4. tie-order exposure: chunk 0 with the aarch64 SwissTable group width
    R8 = HgRunner(P, W, inputs[:1], group_width=8)
    R8.step(0)
    r8 = R8.records(0)
    R8.close()
    tie = sum(_rec_diff(r8[k], plain[0][k]) for k in r8)
    n_tie = sum(len(r8[k]["contig"]) for k in r8)
    # 5. parity against the oracle on a sample of chunk 0 (also the CPU baseline)
    threads = os.cpu_count() or 1
    orc, t_cpu, n_cpu, t_orc_open = hg_oracle_sample(W, args.parity_se if W.cfg == 2 else 0, args.parity_pairs,
                                                     threads)
    par = {}
    for k, r in orc.items():
        par[k] = record_parity(plain[0][k], r, len(r["contig"]))
    # rooflines
    s = main["stats"]
    value = main["reads"] / (main["dev_ms"] / 1e3)
    e2e = main["reads"] / (main["e2e_ms"] / 1e3)
    peaks = {}
    try:
        peaks = json.load(open(os.path.join(ROOT, "MEASURED_PEAKS.json")))
    except Exception:
        pass
    hbm_peak = float(peaks.get("hbm_gbs", 6800.0))
    bases = sum(int(inputs[ci % W.n_chunks][k].offsets[-1]) for ci in range(args.steps)
                for k in inputs[ci % W.n_chunks])
    n_launch_seed = sum(-(-(len(inputs[ci % W.n_chunks][k].offsets) - 1) // CHUNK_READS)
                        for ci in range(args.steps) for k in inputs[ci % W.n_chunks])
    bases_reads = sum(len(inputs[ci % W.n_chunks][k].offsets) - 1 for ci in range(args.steps)
                      for k in inputs[ci % W.n_chunks])
    seed_bytes = (bases + (bases + 3) // 4) + 8 * (s["seed_probes"] + s["seed_entries"] + s["seed_hits"])
    seed_gbs = seed_bytes / (s["ms_seed"] / 1e3) / 1e9 if s["ms_seed"] > 0 else 0.0
    reads_per_launch = bases_reads / max(n_launch_seed, 1)
    roofline = {"kernel": "k_seed (K1 seeding)", "bound": "hbm", "achieved": round(seed_gbs, 1), "peak": hbm_peak,
                "unit": "GB/s", "frac": round(seed_gbs / hbm_peak, 4),
                "traffic": int(SEED_TRAFFIC_PER_READ_HG * reads_per_launch),
                "traffic_note": "DRAM bytes per launch: 1.016 MB per read (ncu dram__bytes_read + dram__bytes_write "
                                "of a 131,072-read launch of this workload) x the reads of a launch",
                "peak_source": "MEASURED_PEAKS.json hbm_gbs (burst), of measured" if peaks else "fallback 6800 GB/s",
                "algorithmic_bytes_per_launch": int(seed_bytes / max(n_launch_seed, 1)),
                "launches_in_timed_region": int(n_launch_seed)}
    add_g, max_g = int32_peak()
    gcups = s["dp_cells"] / (s["ms_align"] / 1e3) / 1e9 if s["ms_align"] > 0 else 0.0
    int_peak = max(x for x in (add_g, max_g) if x) if (add_g or max_g) else None
    roofline_dp = {"kernel": "k_align_band (seeded banded DP, the seeded-alignment phase)", "bound": "int32 issue",
                   "achieved_gcups": round(gcups, 1), "int_ops_per_cell": 10,
                   "achieved_gops": round(gcups * 10, 1),
                   "peak_gops": round(int_peak, 1) if int_peak else None,
                   "frac": round(gcups * 10 / int_peak, 4) if int_peak else None,
                   "peak_source": ("pbw_int32_peak: independent add.s32 / max.s32 chains, CUDA events, the larger "
                                   f"of add {add_g:.0f} and max {max_g:.0f} G ops/s") if int_peak else None,
                   "cells_in_timed_region": int(s["dp_cells"])}
    phases = {k[3:]: round(s[k], 2) for k in ("ms_seed", "ms_cluster", "ms_align", "ms_pair", "ms_finalize",
                                                "ms_d2h")}
    tot_r = sum(c["kept"] + c["pruned"] for c in cnt)
    out = {
        "metric": METRIC, "value": round(value, 1), "unit": "reads/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(main["dev_ms"] / args.steps, 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64", "data": "synthetic (seeded)",
        "config": dict(W.meta(), l2="inputs larger than L2: 4 GiB k-mer CSR + ~10 GB positions + genome + reads",
                       parallelism=f"replicas x{world}", handles_open_s=round(R.t_open, 1),
                       step="one 1M-read chunk (single-end call + paired call on their own handles"
                            + (", issued at once from two host threads; value = the union of the calls' device "
                               "spans, e2e = host wall time of both calls" if R.concurrent else "")
                            + "), chunks cycled"),
        "e2e": {"value": round(e2e, 1), "unit": "reads/s", "h2d_bytes_per_step": int(h2d),
                "d2h_bytes_per_step": int(d2h), "ms_per_step": round(main["e2e_ms"] / args.steps, 3)},
        "gpu_launches": int(s["kernel_launches"]),
        "dp_gcups": round(gcups, 2), "dp_cells_per_step": int(s["dp_cells"] / args.steps),
        "phase_ms_per_step": {k: round(v / args.steps, 2) for k, v in phases.items()},
        "roofline": roofline, "roofline_dp": roofline_dp, "clocks": main["clocks"],
        "modes": {
            "plain_unbatched": {"value": round(unb["reads"] / (unb["dev_ms"] / 1e3), 1), "steps": steps_other,
                                "records_differing_from_batched": int(differ_unbatched)},
            "plain_batched": {"value": round(value, 1), "steps": args.steps},
            "ranked_batched": {"value": round(rk["reads"] / (rk["dev_ms"] / 1e3), 1), "steps": steps_other,
                               "e2e": round(rk["reads"] / (rk["e2e_ms"] / 1e3), 1),
                               "changed_primary_frac": ch_p / max(n_cmp, 1),
                               "changed_mapq_frac": ch_m / max(n_cmp, 1), "reads_compared": int(n_cmp),
                               "candidates_pruned_frac": round(sum(c["pruned"] for c in cnt) / tot_r, 4) if tot_r
                               else 0.0,
                               "label_cut": cut, "train_s": round(t_train, 1),
                               "train": {k: {kk: v[kk] for kk in ("samples", "positives", "train_recall",
                                                                  "train_prune")} for k, v in train.items()}},
        },
        "batching": {"tuning": tuning},
        "parity": {"oracle_sample": par, "compared": sum(v["compared"] for v in par.values()),
                   "mismatched": sum(v["mismatched"] for v in par.values()),
                   "sample": f"chunk 0: first {args.parity_se if W.cfg == 2 else 0} single-end reads and "
                             f"first {args.parity_pairs} pairs",
                   "tie_order_sensitive": int(tie), "tie_order_compared": int(n_tie),
                   "tie_order_note": "reads of chunk 0 whose record differs between SwissTable group widths 16 "
                                     "(x86_64, the default) and 8 (aarch64)"},
    }
    r_u = out["modes"]["plain_unbatched"]["value"]
    out["modes"]["speedup_ranked_batched_vs_plain_unbatched"] = round(out["modes"]["ranked_batched"]["value"] / r_u, 3)
    out["modes"]["speedup_ranked_batched_vs_plain_batched"] = round(out["modes"]["ranked_batched"]["value"] / value, 3)
    out["cpu_baseline"] = {"value": round(n_cpu / t_cpu, 1), "unit": "reads/s", "cores": threads, "kind": "port",
                           "sample": f"the oracle parity sample ({n_cpu} reads of chunk 0), oracle/ C++ "
                                     f"restatement on {threads} threads; oracle index load {t_orc_open:.1f}s "
                                     "not timed"}
    if args.small_parity and W.cfg == 2:
        out["parity"]["single_end_config"] = small_parity(args, 0)
        out["parity"]["paired_config"] = small_parity(args, 1)
    out["wall_s"] = round(time.time() - t_all, 1)
    return out


def run_stage_hgstep(args):
    """One step of the 3.1 Gbp workload (chunk 0: the single-end call, then
    the paired call) and the calls' stats; with --hg-chunks 1 --train-reads 0
    it generates only that chunk. The profiles of the 3.1 Gbp workload run
    this under ncu."""
    import probebwa_gb300 as P
    W = HgWorkload(args, args.config)
    inputs = _hg_inputs(P, W)
    R = HgRunner(P, W, inputs, concurrent=False)
    reads, dev, e2e, stats = R.step(0)
    R.close()
    return {"stage": "hgstep", "config": W.meta(), "reads": int(reads), "device_ms": round(dev, 2),
            "e2e_ms": round(e2e, 2), "calls": stats}


def small_parity(args, cfg):
    """The GPU path against the oracle on the whole single-end configuration
    (cfg 0, 10,000 reads) or on 40,000 pairs of the paired one (cfg 1)."""
    import probebwa_gb300 as P
    from oracle import pyoracle as O
    n = 10_000 if cfg == 0 else args.parity_cfg1_pairs
    prefix, d, meta = workload(cfg, args.cache, n)
    O.build()
    om = O.Mapper(prefix, threads=os.cpu_count() or 1)
    with P.Mapper(prefix) as m:
        if cfg == 0:
            R = P.Reads(d["b1"], d["q1"], d["o1"])
            got = {"se": m.map_single(R)}
            exp = {"se": om.map_single(O.Reads(R.bases, R.quals, R.offsets))}
        else:
            R1, R2 = P.Reads(d["b1"], d["q1"], d["o1"]), P.Reads(d["b2"], d["q2"], d["o2"])
            g1, g2, _ = m.map_paired(R1, R2)
            e1, e2, _ = om.map_paired(O.Reads(R1.bases, R1.quals, R1.offsets), O.Reads(R2.bases, R2.quals, R2.offsets))
            got, exp = {"p1": g1, "p2": g2}, {"p1": e1, "p2": e2}
    with P.Mapper(prefix, group_width=8) as m8:
        if cfg == 0:
            g8 = {"se": m8.map_single(R)}
        else:
            a, b, _ = m8.map_paired(R1, R2)
            g8 = {"p1": a, "p2": b}
    om.close()
    par = {k: record_parity(got[k], exp[k]) for k in got}
    return {"workload": meta["workload"] + (f" (first {n} pairs)" if cfg == 1 else ""),
            "compared": sum(v["compared"] for v in par.values()),
            "mismatched": sum(v["mismatched"] for v in par.values()), "by_read_set": par,
            "tie_order_sensitive": int(sum(_rec_diff(g8[k], got[k]) for k in got))}


def run_reference_hg(args):
    """The oracle (C++ restatement of the reference's CPU path) on a bounded
    sample of each step's chunk, all host threads."""
    W = HgWorkload(args, args.config)
    from oracle import pyoracle as O
    O.build()
    threads = os.cpu_count() or 1
    t = time.time()
    om = O.Mapper(W.prefix, threads=threads)
    t_open = time.time() - t
    n_se, n_pe = args.ref_se, args.ref_pairs

    def one(c):
        ch = W.chunks[c % W.n_chunks]
        secs, reads = 0.0, 0
        if ch["se"] is not None and n_se:
            tt, _ = om.time_map_single(O.Reads(*_slice_reads(*ch["se"], n_se)))
            secs += tt
            reads += n_se
        b1, q1, o1, b2, q2, o2 = ch["pe"]
        tt, _, _ = om.time_map_paired(O.Reads(*_slice_reads(b1, q1, o1, n_pe)), O.Reads(*_slice_reads(b2, q2, o2, n_pe)))
        return secs + tt, reads + 2 * n_pe

    for c in range(args.warmup):
        one(c)
    times, reads = [], 0
    for c in range(args.steps):
        tt, n = one(args.warmup + c)
        times.append(tt)
        reads += n
    om.close()
    v = reads / sum(times)
    sample = (f"per step the first {n_se if W.cfg == 2 else 0} single-end reads and {n_pe} pairs of that step's "
              f"1M-read chunk ({'half single-end, half pairs' if W.cfg == 2 else 'pairs'}), oracle/ C++ restatement "
              f"of the reference CPU path on {threads} threads; index load {t_open:.1f}s not timed")
    cb = {"value": round(v, 1), "unit": "reads/s", "cores": threads, "kind": "port", "sample": sample}
    return {"impl": "reference", "metric": METRIC, "value": round(v, 1), "unit": "reads/s", "n_gpus": 1,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": round(statistics.mean(times) * 1e3, 1),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "int32+f64",
            "data": "synthetic (seeded)", "config": W.meta(), "cpu_baseline": cb,
            "e2e": {"value": round(v, 1), "unit": "reads/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=2, choices=[0, 1, 2, 3, 4],
                    help="2 (default) and 3: the 3.1 Gbp batching + ranker workload; 4: repeat stress; "
                         "0 / 1: the single-end and paired configurations")
    ap.add_argument("--n", type=int, default=None, help="override read / pair count (configs 0 and 1)")
    ap.add_argument("--cache", default=os.environ.get("PBW_BENCH_CACHE", "/tmp/pbw_bench_cache"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ranked", type=int, default=1, help="also time the ranked path (configs 0 / 1, 1 GPU)")
    ap.add_argument("--train-pairs", type=int, default=250_000, help="fresh pairs the ranker is trained on (config 1)")
    ap.add_argument("--label-cut", type=float, default=None,
                    help="ranker training label: lk - lk_max >= cut (default: ln 1e-12 for the repeat-family "
                         "workloads, -60 ln 2, where pruning cannot move sum_exp, for the paired one)")
    # hg38-scale workloads
    ap.add_argument("--genome-bp", type=float, default=3.1e9)
    ap.add_argument("--hg-chunks", type=int, default=10)
    ap.add_argument("--hg-se", type=int, default=500_000, help="single-end reads per chunk (config 2)")
    ap.add_argument("--hg-pairs", type=int, default=250_000, help="pairs per chunk (config 2)")
    ap.add_argument("--stress-pairs", type=int, default=250_000, help="pairs per chunk (config 4)")
    ap.add_argument("--train-reads", type=int, default=2_000_000, help="fresh reads the rankers are trained on")
    ap.add_argument("--hg-concurrent", type=int, default=0,
                    help="issue a step's single-end and paired calls from two host threads (configs 2 and 3); "
                         "off by default: the persistent kernels of the two calls take turns on the SMs "
                         "(measured 681 K vs 704 K reads/s)")
    ap.add_argument("--other-steps", type=int, default=10, help="timed steps of the unbatched and ranked forms")
    ap.add_argument("--parity-se", type=int, default=50_000)
    ap.add_argument("--parity-pairs", type=int, default=25_000)
    ap.add_argument("--parity-cfg1-pairs", type=int, default=40_000)
    ap.add_argument("--small-parity", type=int, default=1, help="add configs 0 / 1 parity to the config 2 line")
    ap.add_argument("--ref-se", type=int, default=8_000)
    ap.add_argument("--ref-pairs", type=int, default=4_000)
    ap.add_argument("--stage", default="map", choices=["map", "index", "sam", "cli", "batch", "hgstep"],
                    help="map: the mapping path (default); index / sam / cli: build-hash, SAM output and the "
                         "command line, each against the oracle; hgstep: one step of configs 2-4 (the single-end "
                         "and the paired call of chunk 0, once each) and its stats, the case the profiles capture")
    args = ap.parse_args()
    hg = args.config in (2, 3, 4)
    if args.label_cut is None:
        args.label_cut = LN_1E12 if (args.stage == "batch" or hg) else STRICT_CUT
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        if hg:
            print(json.dumps(run_reference_hg(args)), flush=True)
            return
        prefix, d, meta = workload(args.config, args.cache, args.n)
        print(json.dumps(run_reference(args, prefix, d, meta)), flush=True)
        return
    if args.stage == "batch":
        if rank == 0:
            print(json.dumps(run_stage_batch(args)), flush=True)
        return
    if args.stage == "hgstep":
        if rank == 0:
            print(json.dumps(run_stage_hgstep(args)), flush=True)
        return
    if args.stage != "map":
        if rank != 0:
            return
        prefix, d, meta = workload(args.config, args.cache, args.n)
        fn = {"index": lambda: run_stage_index(args, prefix, meta), "sam": lambda: run_stage_sam(args, prefix, d, meta),
              "cli": lambda: run_stage_cli(args, prefix, d, meta)}[args.stage]
        print(json.dumps(fn()), flush=True)
        return
    if world > 1:
        import torch
        torch.distributed.init_process_group("nccl")
    if hg:
        out = run_hg(args, rank, world)
    else:
        prefix, d, meta = workload(args.config, args.cache, args.n)
        out = run_gpu(args, prefix, d, meta, rank, world)
        recs = out.pop("_records")
        if rank == 0 and not args.no_cpu_baseline:
            out["cpu_baseline"], out["parity"] = cpu_baseline(prefix, d, meta, recs)
            if "tie_order_sensitive" in out:
                out["parity"]["tie_order_sensitive"] = out.pop("tie_order_sensitive")
    if rank == 0:
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
