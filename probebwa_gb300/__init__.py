"""probebwa_gb300: the probebwa read-mapping hot path on a GB300 (sm_103a).

Python mirror of the reference's mapper / align / mapq interface over the C
ABI in include/probebwa_gpu.h (ctypes; plain pointers and sizes). The compute
path is the CUDA library probebwa_gb300/_lib/libprobebwa_gb300.so; importing a
mapping entry point without it raises instead of falling back to the CPU.

Reference interfaces mirrored (GUIBA-EX/probebwa):
  SingleEndMapper.map              src/mapper/single.rs:164-209
  PairedEndMapper.map_pairs_batch  src/mapper/paired.rs:127-146 (+ lib.rs:145-185 schedule)
  SmithWatermanAligner.align       src/align/smith_waterman.rs:113-255
  find_seed_hits                   src/mapper/seeds.rs:91-151
  cluster_hits                     src/mapper/candidates.rs:30-78
  MapperOptions                    src/types.rs:207-249
"""
from __future__ import annotations

import ctypes as C
import os
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_lib", "libprobebwa_gb300.so")

PBW_OK = 0
ERRORS = {-1: "invalid argument", -2: "I/O error", -3: "malformed index file", -4: "CUDA error",
          -5: "out of memory", -6: "input beyond a device limit", -7: "output capacity too small",
          -8: "device kernel error"}
MAX_READ_LEN = 1024


class PbwError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__(f"{ERRORS.get(code, 'error')} ({code}): {msg}")
        self.code = code


class OptionsC(C.Structure):
    _fields_ = [
        ("substitution_rate", C.c_double),
        ("insert_size_mean", C.c_double),
        ("insert_size_sd", C.c_double),
        ("max_indel_len", C.c_uint64),
        ("gap_open_phred", C.c_uint32),
        ("gap_extend_phred", C.c_uint32),
        ("sv_prior_phred", C.c_double),
        ("group_width", C.c_int32),
        ("device", C.c_int32),
        ("chunk_reads", C.c_uint64),
    ]


class ReadsC(C.Structure):
    _fields_ = [("n", C.c_uint64), ("bases", C.c_void_p), ("quals", C.c_void_p), ("offsets", C.c_void_p)]


class RecordsC(C.Structure):
    _fields_ = [("n", C.c_uint64)] + [(k, C.c_void_p) for k in (
        "contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen", "log_lk", "posterior", "as_score", "nm",
        "cigar_off", "cigar")] + [("cigar_cap", C.c_uint64)]


class SamOptionsC(C.Structure):
    _fields_ = [("command_line", C.c_char_p), ("read_group", C.c_char_p), ("coordinate_sorted", C.c_int32)]


class SamSourceC(C.Structure):
    _fields_ = [("reads", C.POINTER(ReadsC)), ("read_ids", C.POINTER(C.c_char_p)), ("recs", C.POINTER(RecordsC))]


class RankerOptionsC(C.Structure):
    _fields_ = [("epochs", C.c_uint32), ("batch", C.c_uint32), ("lr", C.c_double), ("recall", C.c_double),
                ("positive_weight", C.c_double), ("seed", C.c_uint64), ("label_cut", C.c_double)]


class RankerReportC(C.Structure):
    _fields_ = [("samples", C.c_uint64), ("positives", C.c_uint64), ("loss_first", C.c_double),
                ("loss_last", C.c_double), ("tau", C.c_double), ("train_recall", C.c_double),
                ("train_prune", C.c_double), ("ms_collect", C.c_double), ("ms_train", C.c_double)]


class TuningC(C.Structure):
    _fields_ = [("autotune", C.c_int32), ("band_lanes", C.c_int32), ("length_bins", C.c_int32),
                ("pair_graphs", C.c_int32), ("chosen_lanes", C.c_int32 * 3), ("tuned_ms", (C.c_float * 3) * 3),
                ("wait_polls", C.c_uint32), ("ovf_slice_hits", C.c_uint32), ("k2_threads", C.c_int32 * 2),
                ("k2_chosen", C.c_int32 * 2), ("k2_tuned_ms", (C.c_float * 3) * 2)]


class InsertModelC(C.Structure):
    _fields_ = [("mean", C.c_double), ("sd", C.c_double), ("n_observed", C.c_uint64)]


class StatsC(C.Structure):
    _fields_ = [(k, C.c_double) for k in ("ms_total", "ms_h2d", "ms_seed", "ms_cluster", "ms_align", "ms_finalize",
                                           "ms_pair", "ms_d2h")] + \
               [(k, C.c_uint64) for k in ("seed_probes", "seed_entries", "seed_hits", "dp_jobs", "dp_cells",
                                          "kernel_launches", "window_jobs", "window_cells")] + \
               [("ms_compute", C.c_double), ("t_compute_begin_ms", C.c_double), ("t_compute_end_ms", C.c_double)]


_lib = None

EXPORTS = ["pbw_default_options", "pbw_open", "pbw_close", "pbw_last_error", "pbw_num_contigs", "pbw_total_length",
           "pbw_contig_name", "pbw_contig_length", "pbw_map_single", "pbw_map_paired", "pbw_align_batch",
           "pbw_seed_batch", "pbw_cluster_batch", "pbw_last_stats", "pbw_map_single_device", "pbw_write_sam"]


def build(verbose: bool = False) -> str:
    from . import native_build as _b
    return _b.build(verbose=verbose)


def lib():
    """Load the native library (raises if it was not built)."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"probebwa_gb300 native library missing: {LIB_PATH} (run probebwa_gb300.build())")
        L = C.CDLL(LIB_PATH)
        vp, u64, i64, u32, dbl, cp = C.c_void_p, C.c_uint64, C.c_int64, C.c_uint32, C.c_double, C.c_char_p
        L.pbw_default_options.argtypes = [C.POINTER(OptionsC)]
        L.pbw_open.argtypes = [cp, cp, C.POINTER(OptionsC), C.POINTER(vp)]
        L.pbw_close.argtypes = [vp]
        L.pbw_last_error.argtypes = [vp]
        L.pbw_last_error.restype = cp
        L.pbw_num_contigs.argtypes = [vp]
        L.pbw_num_contigs.restype = u64
        L.pbw_total_length.argtypes = [vp]
        L.pbw_total_length.restype = u64
        L.pbw_contig_name.argtypes = [vp, u64]
        L.pbw_contig_name.restype = cp
        L.pbw_contig_length.argtypes = [vp, u64]
        L.pbw_contig_length.restype = u64
        L.pbw_map_single.argtypes = [vp, C.POINTER(ReadsC), C.POINTER(RecordsC)]
        L.pbw_map_single_device.argtypes = [vp, C.POINTER(ReadsC), C.POINTER(RecordsC)]
        if hasattr(L, "pbw_map_paired"):
            L.pbw_map_paired.argtypes = [vp, C.POINTER(InsertModelC), C.POINTER(ReadsC), C.POINTER(ReadsC),
                                         C.POINTER(RecordsC), C.POINTER(RecordsC)]
        L.pbw_align_batch.argtypes = [vp, u64, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, u64]
        L.pbw_mapq_batch.argtypes = [vp, C.POINTER(ReadsC), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.pbw_records_reserve.argtypes = [C.POINTER(ReadsC), vp, vp]
        L.pbw_reads_load.argtypes = [cp, C.c_int, C.c_uint8, cp, C.POINTER(vp)]
        L.pbw_reads_get.argtypes = [vp, C.POINTER(ReadsC)]
        L.pbw_reads_id.argtypes = [vp, u64]
        L.pbw_reads_id.restype = cp
        L.pbw_reads_free.argtypes = [vp]
        L.pbw_seed_batch.argtypes = [vp, C.POINTER(ReadsC), vp, vp, vp, u64, vp, vp, u64]
        L.pbw_cluster_batch.argtypes = [vp, C.POINTER(ReadsC), u32, vp, vp, vp, vp, vp, vp]
        L.pbw_last_stats.argtypes = [vp, C.POINTER(StatsC)]
        L.pbw_write_sam.argtypes = [vp, cp, cp, C.POINTER(ReadsC), C.POINTER(cp), C.POINTER(RecordsC)]
        L.pbw_sam_write.argtypes = [vp, C.POINTER(SamOptionsC), u32, C.POINTER(SamSourceC), vp, u64, cp]
        L.pbw_sam_format.argtypes = [vp, C.POINTER(SamOptionsC), u32, C.POINTER(SamSourceC), vp, u64, vp, u64, vp]
        L.pbw_sort_coordinate.argtypes = [vp, u32, C.POINTER(SamSourceC), vp, u64, vp]
        L.pbw_bam_write.argtypes = [vp, C.POINTER(SamOptionsC), u32, C.POINTER(SamSourceC), vp, u64, cp, C.c_int32]
        L.pbw_bam_write_text.argtypes = [C.c_char_p, u64, cp, C.c_int32]
        L.pbw_build_genome.argtypes = [cp, cp, cp, u32, C.POINTER(cp)]
        L.pbw_get_tuning.argtypes = [vp, C.POINTER(TuningC)]
        L.pbw_set_tuning.argtypes = [vp, C.POINTER(TuningC)]
        L.pbw_ranker_default_options.argtypes = [C.POINTER(RankerOptionsC)]
        L.pbw_ranker_train.argtypes = [vp, C.POINTER(ReadsC), C.POINTER(ReadsC), C.POINTER(RankerOptionsC),
                                       C.POINTER(RankerReportC)]
        L.pbw_ranker_enable.argtypes = [vp, C.c_int32]
        L.pbw_ranker_counters.argtypes = [vp, vp, vp, vp]
        L.pbw_ranker_export.argtypes = [vp, vp, u64, vp]
        L.pbw_ranker_import.argtypes = [vp, vp, u64]
        L.pbw_ranker_score.argtypes = [vp, vp, u64, vp]
        L.pbw_build_hash.argtypes = [cp, cp, u64, u64, u64, C.c_int32]
        L.pbw_int32_peak.argtypes = [C.c_int32, vp, vp]
        if hasattr(L, "pbw_align_noalloc"):
            L.pbw_align_noalloc.argtypes = [u64, vp, vp, vp, vp, vp, vp, vp, u32, u32, vp, vp, vp, vp, u32, vp]
        _lib = L
    return _lib


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


@dataclass
class MapperOptions:
    """MapperOptions (src/types.rs:207-249) plus device settings."""
    substitution_rate: float = 0.001
    insert_size_mean: float = 250.0
    insert_size_sd: float = 60.0
    max_indel_len: int = 30
    gap_open_phred: int = 40
    gap_extend_phred: int = 3
    sv_prior_phred: float = 55.0
    group_width: int = 16
    device: int = 0
    chunk_reads: int = 0

    def c(self) -> OptionsC:
        return OptionsC(self.substitution_rate, self.insert_size_mean, self.insert_size_sd, self.max_indel_len,
                        self.gap_open_phred, self.gap_extend_phred, self.sv_prior_phred, self.group_width,
                        self.device, self.chunk_reads)


class Reads:
    """Reads as SoA numpy arrays: bases (uint8), Phred scores (uint8), n+1 offsets."""

    def __init__(self, bases, quals, offsets, ids=None):
        self.bases = np.ascontiguousarray(bases, dtype=np.uint8)
        self.quals = np.ascontiguousarray(quals, dtype=np.uint8)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.ids = ids if ids is not None else [f"r{i}" for i in range(len(self.offsets) - 1)]

    @property
    def n(self) -> int:
        return len(self.offsets) - 1

    @staticmethod
    def from_lists(seqs, quals=None, ids=None) -> "Reads":
        seqs = [s.encode() if isinstance(s, str) else bytes(s) for s in seqs]
        if quals is None:
            quals = [bytes([40] * len(s)) for s in seqs]
        quals = [bytes(q) for q in quals]
        offs = np.zeros(len(seqs) + 1, dtype=np.uint64)
        if seqs:
            offs[1:] = np.cumsum([len(s) for s in seqs])
        b = np.frombuffer(b"".join(seqs) + b"\0", dtype=np.uint8)[:-1].copy()
        q = np.frombuffer(b"".join(quals) + b"\0", dtype=np.uint8)[:-1].copy()
        return Reads(b, q, offs, ids)

    def c(self) -> ReadsC:
        if self.bases.size == 0:
            self._keep = (np.zeros(1, np.uint8), np.zeros(1, np.uint8))
            return ReadsC(self.n, _ptr(self._keep[0]), _ptr(self._keep[1]), _ptr(self.offsets))
        return ReadsC(self.n, _ptr(self.bases), _ptr(self.quals), _ptr(self.offsets))

    def seq(self, i: int) -> bytes:
        return self.bases[int(self.offsets[i]):int(self.offsets[i + 1])].tobytes()


RECORD_FIELDS = (("contig", np.int32), ("pos", np.uint64), ("mapq", np.uint8), ("flag", np.uint16),
                 ("mate_contig", np.int32), ("mate_pos", np.uint64), ("tlen", np.int64), ("log_lk", np.float64),
                 ("posterior", np.float64), ("as_score", np.int32), ("nm", np.int32))


def alloc_records(n: int, total_len: int) -> dict:
    r = {k: np.zeros(max(n, 1), t)[:n] for k, t in RECORD_FIELDS}
    r["cigar_off"] = np.zeros(n + 1, np.uint32)
    r["cigar"] = np.zeros(2 * total_len + 2 * n + 16, np.uint32)
    return r


def records_c(r: dict) -> RecordsC:
    n = len(r["contig"])
    keep = [r[k] if r[k].size else np.zeros(1, r[k].dtype) for k, _ in RECORD_FIELDS]
    r["_keep"] = keep
    return RecordsC(n, *[_ptr(a) for a in keep], _ptr(r["cigar_off"]), _ptr(r["cigar"]), len(r["cigar"]))


def pack_mapq_items(items):
    """Flattens per-read MAPQ inputs (dicts with lks, repeat, rev, ref, cigar)
    into the concatenated arrays of the *_mapq_batch entry points."""
    n = len(items)
    lk_off = np.zeros(n + 1, np.uint64)
    win_off = np.zeros(n + 1, np.uint64)
    ref_off = np.zeros(n + 1, np.uint64)
    cig_off = np.zeros(n + 1, np.uint32)
    lk_off[1:] = np.cumsum([len(it["lks"]) for it in items])
    win_off[1:] = np.cumsum([len(it["repeat"]) for it in items])
    ref_off[1:] = np.cumsum([len(it["ref"]) for it in items])
    cig_off[1:] = np.cumsum([len(it["cigar"]) for it in items])
    lks = np.concatenate([np.asarray(it["lks"], np.float64) for it in items] + [np.zeros(1)])
    rep = np.concatenate([np.asarray(it["repeat"], np.float64) for it in items] + [np.zeros(1)])
    rev = np.array([1 if it["rev"] else 0 for it in items], np.uint8)
    refs = np.frombuffer(b"".join(bytes(it["ref"]) for it in items) + b"\0", np.uint8).copy()
    cig = np.concatenate([np.asarray(it["cigar"], np.uint32) for it in items] + [np.zeros(1, np.uint32)])
    out = {"mapq": np.zeros(n, np.uint8), "posterior": np.zeros(n, np.float64), "best": np.zeros(n, np.uint32),
           "sum_exp": np.zeros(n, np.float64)}
    return (lk_off, lks, win_off, rep, rev, ref_off, refs, cig_off, cig), out



OPS = "MIDXSH"


def cigar_strings(r: dict) -> list:
    co, cg = r["cigar_off"], r["cigar"]
    return ["".join(f"{int(w) >> 4}{OPS[int(w) & 15]}" for w in cg[co[i]:co[i + 1]])
            for i in range(len(r["contig"]))]


def _read_ids(L, h, n: int) -> list:
    """The n read IDs of a read set: one read of the block they are stored
    in back to back (NUL after each), or one call per ID when an ID holds a
    NUL of its own."""
    if n == 0:
        return []
    raw = C.cast(L.pbw_reads_id, C.CFUNCTYPE(C.c_void_p, C.c_void_p, C.c_uint64))
    a0, an = raw(h, 0), raw(h, n - 1)
    block = C.string_at(a0, an - a0 + len(C.string_at(an)))
    ids = block.decode("utf-8", "replace").split("\0")
    if len(ids) != n:
        ids = [L.pbw_reads_id(h, i).decode("utf-8", "replace") for i in range(n)]
    return ids


def load_reads(path: str, fasta: bool = False, quality_offset: int = 33, adapter: str | bytes | None = None) -> "Reads":
    """read_reads_files_with_preprocessing for one file (src/io/fastx.rs:19-48)
    through pbw_reads_load: bases, Phred scores and IDs as a Reads object."""
    L = lib()
    if isinstance(adapter, str):
        adapter = adapter.encode()
    h = C.c_void_p()
    rc = L.pbw_reads_load(path.encode(), 1 if fasta else 0, quality_offset, adapter, C.byref(h))
    if rc != 0:
        raise PbwError(rc, L.pbw_last_error(None).decode())
    try:
        v = ReadsC()
        L.pbw_reads_get(h, C.byref(v))
        n = int(v.n)
        offs = np.ctypeslib.as_array(C.cast(v.offsets, C.POINTER(C.c_uint64)), shape=(n + 1,)).copy()
        tot = int(offs[-1])
        if tot:
            bases = np.ctypeslib.as_array(C.cast(v.bases, C.POINTER(C.c_uint8)), shape=(tot,)).copy()
            quals = np.ctypeslib.as_array(C.cast(v.quals, C.POINTER(C.c_uint8)), shape=(tot,)).copy()
        else:
            bases = np.zeros(0, np.uint8)
            quals = np.zeros(0, np.uint8)
        ids = _read_ids(L, h, n)
    finally:
        L.pbw_reads_free(h)
    return Reads(bases, quals, offs, ids)


def bam_from_sam(sam: bytes, path: str, index: bool = False) -> None:
    """write_bam / write_bam_indexed (src/io/bam.rs:19-57) on SAM text through
    pbw_bam_write_text: the stream as BGZF BAM at path, the reference
    dictionary from its @SQ lines, and a BAI at path + '.bai' when index is
    set (an @HD SO:coordinate stream). Host code: no device is needed."""
    L = lib()
    sam = bytes(sam)
    rc = L.pbw_bam_write_text(sam, len(sam), path.encode(), 1 if index else 0)
    if rc != 0:
        raise PbwError(rc, L.pbw_last_error(None).decode())


def build_genome(out_prefix: str, fasta_paths, species: str = "species", assembly: str = "assembly") -> None:
    """build-genome (GenomeIndexBuilder, src/index/genome.rs:98-148) through
    pbw_build_genome: FASTA files -> out_prefix.stidx."""
    L = lib()
    arr = (C.c_char_p * max(len(fasta_paths), 1))(*[p.encode() for p in fasta_paths])
    rc = L.pbw_build_genome(out_prefix.encode(), species.encode(), assembly.encode(), len(fasta_paths), arr)
    if rc != 0:
        raise PbwError(rc, L.pbw_last_error(None).decode())


def build_hash(genome_prefix: str, out_prefix: str, k: int = 15, stride: int = 5, max_count: int = 300,
               device: int = 0) -> None:
    """build-hash (HashTableBuilder, src/index/hashtable.rs:248-322) on the
    GPU through pbw_build_hash: genome_prefix.stidx -> out_prefix.sthash."""
    L = lib()
    rc = L.pbw_build_hash(genome_prefix.encode(), out_prefix.encode(), k, stride, max_count, device)
    if rc != 0:
        raise PbwError(rc, L.pbw_last_error(None).decode())


class Mapper:
    """One device handle: index resident in HBM plus the mapping pipeline."""

    def __init__(self, genome_prefix: str, hash_prefix: str | None = None, options: MapperOptions | None = None,
                 **kw):
        self.options = options or MapperOptions(**kw)
        self._opt = self.options.c()
        h = C.c_void_p()
        rc = lib().pbw_open(genome_prefix.encode(), (hash_prefix or genome_prefix).encode(), C.byref(self._opt),
                            C.byref(h))
        if rc != PBW_OK:
            raise PbwError(rc, lib().pbw_last_error(None).decode())
        self.h = h

    def _check(self, rc):
        if rc != PBW_OK:
            raise PbwError(rc, lib().pbw_last_error(self.h).decode())

    def close(self):
        if getattr(self, "h", None):
            lib().pbw_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    @property
    def contigs(self):
        L = lib()
        return [(L.pbw_contig_name(self.h, i).decode(), L.pbw_contig_length(self.h, i))
                for i in range(L.pbw_num_contigs(self.h))]

    def map_single(self, reads: Reads) -> dict:
        recs = alloc_records(reads.n, len(reads.bases))
        self._check(lib().pbw_map_single(self.h, C.byref(reads.c()), C.byref(records_c(recs))))
        return recs

    def map_paired(self, r1: Reads, r2: Reads, mean=None, sd=None):
        m = InsertModelC(self.options.insert_size_mean if mean is None else mean,
                         self.options.insert_size_sd if sd is None else sd, 0)
        o1 = alloc_records(r1.n, len(r1.bases))
        o2 = alloc_records(r2.n, len(r2.bases))
        self._check(lib().pbw_map_paired(self.h, C.byref(m), C.byref(r1.c()), C.byref(r2.c()),
                                         C.byref(records_c(o1)), C.byref(records_c(o2))))
        return o1, o2, (m.mean, m.sd, m.n_observed)

    def stats(self) -> dict:
        s = StatsC()
        self._check(lib().pbw_last_stats(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in StatsC._fields_}

    def seed_batch(self, reads: Reads, hit_cap: int | None = None):
        """find_seed_hits per read: (hit_off, packed hits, read_pos, win_off, repeat_prob)."""
        n = reads.n
        # in-buffer reads hold at most 4096 hits each; over-capacity reads
        # share the 16 M-hit overflow pool of a chunk
        hit_cap = hit_cap or (4096 * max(n, 1) + (16 << 20) * (1 + n // 131072))
        hit_off = np.zeros(n + 1, np.uint64)
        hits = np.zeros(hit_cap, np.uint64)
        rpos = np.zeros(hit_cap, np.uint32)
        win_cap = max(len(reads.bases), 1)
        win_off = np.zeros(n + 1, np.uint64)
        rep = np.zeros(win_cap, np.float64)
        self._check(lib().pbw_seed_batch(self.h, C.byref(reads.c()), _ptr(hit_off), _ptr(hits), _ptr(rpos), hit_cap,
                                         _ptr(win_off), _ptr(rep), win_cap))
        return hit_off, hits[:hit_off[-1]], rpos[:hit_off[-1]], win_off, rep[:win_off[-1]]

    def cluster_batch(self, reads: Reads, max_per_read: int = 64):
        """cluster_hits per read: first max_per_read candidates and the full count."""
        n = reads.n
        nc = np.zeros(max(n, 1), np.uint32)
        tc = np.zeros(max(n, 1), np.uint32)
        cc = np.zeros(max(n, 1) * max_per_read, np.uint32)
        cp = np.zeros(max(n, 1) * max_per_read, np.uint64)
        cs = np.zeros(max(n, 1) * max_per_read, np.uint8)
        sc = np.zeros(max(n, 1) * max_per_read, np.float64)
        self._check(lib().pbw_cluster_batch(self.h, C.byref(reads.c()), max_per_read, _ptr(nc), _ptr(tc), _ptr(cc),
                                            _ptr(cp), _ptr(cs), _ptr(sc)))
        return nc[:n], tc[:n], cc.reshape(-1, max_per_read)[:n], cp.reshape(-1, max_per_read)[:n], \
            cs.reshape(-1, max_per_read)[:n], sc.reshape(-1, max_per_read)[:n]

    def align_batch(self, problems):
        """SmithWatermanAligner::align for a list of (read, qual, ref, hint, band)."""
        n = len(problems)
        reads = [bytes(p[0]) for p in problems]
        quals = [bytes(p[1]) for p in problems]
        refs = [bytes(p[2]) for p in problems]
        ro = np.zeros(n + 1, np.uint64)
        fo = np.zeros(n + 1, np.uint64)
        ro[1:] = np.cumsum([len(x) for x in reads])
        fo[1:] = np.cumsum([len(x) for x in refs])
        rb = np.frombuffer(b"".join(reads) + b"\0", np.uint8)[:-1].copy()
        qb = np.frombuffer(b"".join(quals) + b"\0", np.uint8)[:-1].copy()
        fb = np.frombuffer(b"".join(refs) + b"\0", np.uint8)[:-1].copy()
        rb = rb if rb.size else np.zeros(1, np.uint8)
        qb = qb if qb.size else np.zeros(1, np.uint8)
        fb = fb if fb.size else np.zeros(1, np.uint8)
        hint = np.array([p[3] for p in problems], np.int64)
        band = np.array([p[4] for p in problems], np.uint64)
        score = np.zeros(n, np.int32)
        off = np.zeros(n, np.uint64)
        cap = int(2 * ro[-1] + fo[-1] + 8 * n + 8)
        co = np.zeros(n + 1, np.uint32)
        cg = np.zeros(cap, np.uint32)
        self._check(lib().pbw_align_batch(self.h, n, _ptr(rb), _ptr(qb), _ptr(ro), _ptr(fb), _ptr(fo), _ptr(hint),
                                          _ptr(band), _ptr(score), _ptr(off), _ptr(co), _ptr(cg), cap))
        out = []
        for i in range(n):
            cig = "".join(f"{int(w) >> 4}{OPS[int(w) & 15]}" for w in cg[co[i]:co[i + 1]])
            out.append((int(score[i]), cig, int(off[i])))
        return out

    def write_sam(self, path: str, reads: Reads, recs: dict, command_line: str = "probebwa map"):
        ids = (C.c_char_p * max(reads.n, 1))(*[i.encode() for i in reads.ids])
        self._check(lib().pbw_write_sam(self.h, path.encode(), command_line.encode(), C.byref(reads.c()), ids,
                                        C.byref(records_c(recs))))

    def _sam_sources(self, sources):
        """sources: [(Reads, records dict)] -- one (single-end) or two (mates)."""
        keep = []
        arr = (SamSourceC * len(sources))()
        for k, (reads, recs) in enumerate(sources):
            rc_ = reads.c()
            ids = (C.c_char_p * max(reads.n, 1))(*[i.encode() for i in reads.ids])
            cr = records_c(recs)
            keep += [rc_, ids, cr]
            arr[k] = SamSourceC(C.pointer(rc_), ids, C.pointer(cr))
        return arr, keep

    def sam_text(self, sources, sel=None, command_line: str = "probebwa map", read_group: str | None = None,
                 coordinate_sorted: bool = False) -> bytes:
        """SAM stream of the selected records (format_sam_records_sorted,
        sam.rs:83-108), formatted on the device. Record r of source s is
        number r * len(sources) + s; sel=None takes all in number order."""
        arr, keep = self._sam_sources(sources)
        o = SamOptionsC(command_line.encode(), read_group.encode() if read_group is not None else None,
                        1 if coordinate_sorted else 0)
        sp, ns = (None, 0)
        if sel is not None:
            # an empty selection still passes a list: NULL means every record
            sel = np.ascontiguousarray(sel, dtype=np.uint64)
            keep.append(sel if sel.size else np.zeros(1, np.uint64))
            sp, ns = (_ptr(keep[-1]), int(sel.size))
        n = C.c_uint64(0)
        self._check(lib().pbw_sam_format(self.h, C.byref(o), len(sources), arr, sp, ns, None, 0, C.byref(n)))
        buf = C.create_string_buffer(max(n.value, 1))
        self._check(lib().pbw_sam_format(self.h, C.byref(o), len(sources), arr, sp, ns, buf, n.value, C.byref(n)))
        return buf.raw[:n.value]

    def write_bam(self, path: str, sources, sel=None, command_line: str = "probebwa map",
                  read_group: str | None = None, coordinate_sorted: bool = False, index: bool = False):
        """The SAM stream of sam_text as BGZF BAM (write_bam, src/io/bam.rs:19-57),
        with a BAI at path + '.bai' when index is set (coordinate-sorted records)."""
        arr, keep = self._sam_sources(sources)
        o = SamOptionsC(command_line.encode(), read_group.encode() if read_group is not None else None,
                        1 if coordinate_sorted else 0)
        sp, ns = (None, 0)
        if sel is not None:
            sel = np.ascontiguousarray(sel, dtype=np.uint64)
            keep.append(sel if sel.size else np.zeros(1, np.uint64))
            sp, ns = (_ptr(keep[-1]), int(sel.size))
        self._check(lib().pbw_bam_write(self.h, C.byref(o), len(sources), arr, sp, ns, path.encode(),
                                        1 if index else 0))

    def sort_coordinate(self, sources, sel=None) -> np.ndarray:
        """sort_for_coordinate_order (sam.rs:114-124) of the selected record
        numbers, on the device."""
        arr, keep = self._sam_sources(sources)
        if sel is None:
            sel = np.arange(len(sources[0][1]["contig"]) * len(sources), dtype=np.uint64)
        sel = np.ascontiguousarray(sel, dtype=np.uint64)
        out = np.zeros(max(sel.size, 1), np.uint64)
        self._check(lib().pbw_sort_coordinate(self.h, len(sources), arr, _ptr(sel) if sel.size else None,
                                              int(sel.size), _ptr(out)))
        return out[:sel.size]

    def tuning(self) -> dict:
        """Batching settings and the band-DP forms the tuner chose (pbw_get_tuning)."""
        t = TuningC()
        self._check(lib().pbw_get_tuning(self.h, C.byref(t)))
        return {"autotune": t.autotune, "band_lanes": t.band_lanes, "length_bins": t.length_bins,
                "pair_graphs": t.pair_graphs, "chosen_lanes": list(t.chosen_lanes),
                "tuned_ms": [list(r) for r in t.tuned_ms], "wait_polls": t.wait_polls,
                "ovf_slice_hits": t.ovf_slice_hits, "k2_threads": list(t.k2_threads),
                "k2_chosen": list(t.k2_chosen), "k2_tuned_ms": [list(r) for r in t.k2_tuned_ms]}

    def set_tuning(self, **kw):
        """pbw_set_tuning: autotune, band_lanes (0, 4, 8, 16), length_bins, pair_graphs, wait_polls,
        ovf_slice_hits, k2_threads (two of 0, 256, 512, 1024)."""
        t = TuningC()
        self._check(lib().pbw_get_tuning(self.h, C.byref(t)))
        for k, v in kw.items():
            if k == "k2_threads":
                for i, x in enumerate(v):
                    t.k2_threads[i] = int(x)
            else:
                setattr(t, k, int(v))
        self._check(lib().pbw_set_tuning(self.h, C.byref(t)))

    def ranker_train(self, r1: Reads, r2: Reads | None = None, **kw) -> dict:
        """Trains the candidate ranker on these reads (pairs when r2 is given)
        with labels from the plain path; returns the training report."""
        o = RankerOptionsC()
        lib().pbw_ranker_default_options(C.byref(o))
        for k, v in kw.items():
            setattr(o, k, v)
        rep = RankerReportC()
        c2 = C.byref(r2.c()) if r2 is not None else None
        self._check(lib().pbw_ranker_train(self.h, C.byref(r1.c()), c2, C.byref(o), C.byref(rep)))
        return {k: getattr(rep, k) for k, _ in RankerReportC._fields_}

    def ranker_enable(self, on: bool = True):
        self._check(lib().pbw_ranker_enable(self.h, 1 if on else 0))

    def ranker_counters(self) -> dict:
        v = [C.c_uint64(0) for _ in range(3)]
        self._check(lib().pbw_ranker_counters(self.h, *[C.byref(x) for x in v]))
        return {"kept": v[0].value, "pruned": v[1].value, "reads_whole": v[2].value}

    def ranker_export(self) -> np.ndarray:
        n = C.c_uint64(0)
        self._check(lib().pbw_ranker_export(self.h, None, 0, C.byref(n)))
        out = np.zeros(n.value, np.float32)
        self._check(lib().pbw_ranker_export(self.h, _ptr(out), n.value, C.byref(n)))
        return out

    def ranker_import(self, model: np.ndarray):
        model = np.ascontiguousarray(model, dtype=np.float32)
        self._check(lib().pbw_ranker_import(self.h, _ptr(model), model.size))

    def ranker_score(self, feat: np.ndarray) -> np.ndarray:
        feat = np.ascontiguousarray(feat, dtype=np.float32).reshape(-1, 12)
        out = np.zeros(max(len(feat), 1), np.float32)
        self._check(lib().pbw_ranker_score(self.h, _ptr(feat) if len(feat) else None, len(feat), _ptr(out)))
        return out[:len(feat)]

    def mapq_batch(self, reads: Reads, items) -> dict:
        """MapqCalculator::select_best + finalize_mapq (bayesian.rs:193-201,
        251-282) per read. items: one dict per read with lks (candidate
        log-likelihoods), repeat (per-window repeat probabilities), rev,
        ref (the winner's reference window) and cigar (packed u32)."""
        (lk_off, lks, win_off, rep, rev, ref_off, refs, cig_off, cig), out = pack_mapq_items(items)
        self._check(lib().pbw_mapq_batch(self.h, C.byref(reads.c()), _ptr(lk_off), _ptr(lks), _ptr(win_off),
                                         _ptr(rep), _ptr(rev), _ptr(ref_off), _ptr(refs), _ptr(cig_off), _ptr(cig),
                                         _ptr(out["mapq"]), _ptr(out["posterior"]), _ptr(out["best"]),
                                         _ptr(out["sum_exp"])))
        return out

    @staticmethod
    def records_reserve(reads: Reads) -> tuple:
        n = np.zeros(1, np.uint64)
        cap = np.zeros(1, np.uint64)
        rc = lib().pbw_records_reserve(C.byref(reads.c()), _ptr(n), _ptr(cap))
        if rc != 0:
            raise RuntimeError("pbw_records_reserve failed")
        return int(n[0]), int(cap[0])


# ---- reference-shaped API ----

class SingleEndMapper:
    """SingleEndMapper (src/mapper/single.rs:33-209) over one device handle."""

    def __init__(self, genome_prefix: str, hash_prefix: str | None = None, options: MapperOptions | None = None):
        self.mapper = Mapper(genome_prefix, hash_prefix, options)

    def map(self, reads: Reads) -> dict:
        return self.mapper.map_single(reads)


class PairedEndMapper:
    """PairedEndMapper (src/mapper/paired.rs:76-146) with the map_paired schedule of src/lib.rs:145-185."""

    def __init__(self, genome_prefix: str, hash_prefix: str | None = None, options: MapperOptions | None = None):
        self.mapper = Mapper(genome_prefix, hash_prefix, options)
        o = self.mapper.options
        self.insert_model = (o.insert_size_mean, o.insert_size_sd, 0)

    def map_pairs(self, r1: Reads, r2: Reads):
        m, s, _ = self.insert_model
        o1, o2, model = self.mapper.map_paired(r1, r2, m, s)
        self.insert_model = model
        return o1, o2
