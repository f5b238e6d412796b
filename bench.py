#!/usr/bin/env python3
"""Throughput of the probebwa mapping path on GB300.

Workload (default): the paired-end configuration -- a synthetic 100 Mbp genome
(25 x 4 Mbp, GC 41%, 5% segmental duplications of 1-10 kbp in 2-8 copies at
95-99.5% identity, homopolymer runs of 6-15 bp at 1 per 2 kbp) and 1,000,000
read pairs of 2 x 150 bp (insert N(350, 50), FR, 0.5% substitutions and
0.05% indels enriched 5x in homopolymers, Phred N(35, 4) clipped to [2, 41]),
mapped with the reference's default options. --config 0 selects the
single-end configuration (1 Mbp genome with 20 planted 2 kbp repeat copies,
10,000 x 120 bp reads). Data are generated from fixed seeds; no dataset is
downloaded.

One step maps the whole read set once. `value` is reads/s with the reads
already in device memory (pbw_map_*_device-style timing from CUDA events on
the pipeline's stream); `e2e` is the same metric through the public C ABI with
pinned host buffers, host->device input copies and device->host record copies
inside the timed region.

--impl reference times the CPU restatement of the reference path (oracle/)
on the host cores instead.
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

SEED = {0: 0x5EED0000, 1: 0x5EED0001}
CHUNK_READS = 131072  # the library's default chunk (pbw_options.chunk_reads = 0)
# DRAM bytes (read + write) of K1 per read of the paired workload, from one
# ncu capture of a 100,000-read launch (29.014 GB read + 0.161 GB written):
# profiles/k_seed_paired_100k_pairs.md. Not measured for the single-end one.
SEED_DRAM_BYTES_PER_READ = {1: (29.014204e9 + 0.161155e9) / 100_000}
METRIC = "reads/s @1 GB300: plain vs ranked+batched (≤0.05% primaries changed); DP GCUPS"


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
    ranked = None
    if args.ranked and paired and world == 1:
        ranked = run_ranked(args, m, opts, step, O1, O2, meta, n_reads, dev)
    # device time of a step: the pipeline's CUDA events, without the input copy
    dev_ms = [s["ms_seed"] + s["ms_cluster"] + s["ms_align"] + s["ms_pair"] + s["ms_finalize"] + s["ms_d2h"]
              for s in stats]
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
    out["batching"] = {"band_dp_lanes_by_length_class": dict(zip(("<=128", "<=256", ">256"), tuning["chosen_lanes"])),
                       "band_dp_tuned_ms_8_16": dict(zip(("<=128", "<=256", ">256"), tuning["tuned_ms"])),
                       "length_bins": bool(tuning["length_bins"]), "pair_graphs": bool(tuning["pair_graphs"])}
    if ranked is not None:
        ranked["speedup_vs_plain"] = round(ranked["value"] / value, 3)
        out["ranked"] = ranked
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
    dev_ms = [s["ms_seed"] + s["ms_cluster"] + s["ms_align"] + s["ms_pair"] + s["ms_finalize"] + s["ms_d2h"]
              for s in stats]
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
def cpu_time(prefix, d, meta, n_sample: int, threads: int):
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
        t, _, _ = m.time_map_paired(R1, R2)
        reads = 2 * k
    else:
        t, _ = m.time_map_single(R1)
        reads = k
    m.close()
    return reads, t


def cpu_baseline(prefix, d, meta):
    threads = os.cpu_count() or 1
    n = 40_000 if meta["paired"] else 10_000
    reads, t = cpu_time(prefix, d, meta, n, threads)
    return {"value": round(reads / t, 1), "unit": "reads/s", "cores": threads, "kind": "port",
            "sample": f"first {reads} reads ({'pairs' if meta['paired'] else 'reads'} incl. the serial warm-up) "
                      f"of the same workload, oracle/ C++ restatement, {threads} threads"}


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
        return st["ms_seed"] + st["ms_cluster"] + st["ms_align"] + st["ms_pair"] + st["ms_finalize"] + st["ms_d2h"]

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


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--config", type=int, default=1, choices=[0, 1])
    ap.add_argument("--n", type=int, default=None, help="override read / pair count")
    ap.add_argument("--cache", default=os.environ.get("PBW_BENCH_CACHE", "/tmp/pbw_bench_cache"))
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--ranked", type=int, default=1, help="also time the ranked path (pairs, 1 GPU)")
    ap.add_argument("--train-pairs", type=int, default=250_000, help="fresh pairs the ranker is trained on")
    ap.add_argument("--label-cut", type=float, default=None,
                    help="ranker training label: lk - lk_max >= cut (default: -60 ln 2 for the paired "
                         "workload, where pruning then cannot move sum_exp; ln 1e-12 for --stage batch)")
    ap.add_argument("--stage", default="map", choices=["map", "index", "sam", "cli", "batch"],
                    help="map: the mapping path (default); index / sam / cli: build-hash, SAM output and the "
                         "command line, each against the oracle")
    args = ap.parse_args()
    if args.label_cut is None:
        args.label_cut = -27.631021115928547 if args.stage == "batch" else -41.58883083359672
    args.warmup = max(args.warmup, 3) if args.impl == "gb300" else args.warmup
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    if args.impl == "reference":
        if rank != 0:
            return
        prefix, d, meta = workload(args.config, args.cache, args.n)
        print(json.dumps(run_reference(args, prefix, d, meta)), flush=True)
        return
    if args.stage == "batch":
        if rank == 0:
            print(json.dumps(run_stage_batch(args)), flush=True)
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
    prefix, d, meta = workload(args.config, args.cache, args.n)
    out = run_gpu(args, prefix, d, meta, rank, world)
    if rank == 0:
        if not args.no_cpu_baseline:
            out["cpu_baseline"] = cpu_baseline(prefix, d, meta)
        print(json.dumps(out), flush=True)
    if world > 1:
        import torch
        torch.distributed.destroy_process_group()


if __name__ == "__main__":
    main()
