"""ctypes binding of the CPU oracle (oracle/oracle.cpp).

TEST INFRASTRUCTURE ONLY: the checker for the GB300 mapper and the timed CPU
baseline. Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline /
reference legs may import this module. The product (probebwa_gb300/) never
does.
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")


CLI_PATH = os.path.join(HERE, "_build", "probebwa_oracle")


def build(quiet: bool = True) -> str:
    """Compile the oracle with its Makefile (make is incremental)."""
    out = subprocess.run(["make", "-C", HERE], capture_output=True, text=True)
    if out.returncode != 0:
        raise RuntimeError("oracle build failed:\n" + out.stdout + out.stderr)
    if not quiet:
        print(out.stdout)
    return LIB_PATH


class Options(C.Structure):
    _fields_ = [
        ("substitution_rate", C.c_double),
        ("insert_size_mean", C.c_double),
        ("insert_size_sd", C.c_double),
        ("max_indel_len", C.c_uint64),
        ("gap_open_phred", C.c_uint32),
        ("gap_extend_phred", C.c_uint32),
        ("sv_prior_phred", C.c_double),
        ("threads", C.c_int32),
        ("group_width", C.c_int32),
        ("dense_min_buckets", C.c_uint64),
    ]


class ReadsC(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("bases", C.c_void_p),
        ("quals", C.c_void_p),
        ("offsets", C.c_void_p),
    ]


class RecordsC(C.Structure):
    _fields_ = [
        ("n", C.c_uint64),
        ("contig", C.c_void_p),
        ("pos", C.c_void_p),
        ("mapq", C.c_void_p),
        ("flag", C.c_void_p),
        ("mate_contig", C.c_void_p),
        ("mate_pos", C.c_void_p),
        ("tlen", C.c_void_p),
        ("log_lk", C.c_void_p),
        ("posterior", C.c_void_p),
        ("as_score", C.c_void_p),
        ("nm", C.c_void_p),
        ("cigar_off", C.c_void_p),
        ("cigar", C.c_void_p),
        ("cigar_cap", C.c_uint64),
    ]


class InsertModelC(C.Structure):
    _fields_ = [("mean", C.c_double), ("sd", C.c_double), ("n_observed", C.c_uint64)]


_lib = None


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        vp, u64, i64, u32, i32, dbl, cp = C.c_void_p, C.c_uint64, C.c_int64, C.c_uint32, C.c_int32, C.c_double, C.c_char_p
        L.orc_last_error.restype = cp
        L.orc_default_options.argtypes = [C.POINTER(Options)]
        L.orc_build_genome.argtypes = [cp, cp, cp, C.c_int, C.POINTER(cp)]
        L.orc_build_genome_from_seqs.argtypes = [cp, cp, cp, C.c_int, C.POINTER(cp), C.POINTER(vp), C.POINTER(u64)]
        L.orc_build_hash.argtypes = [cp, cp, u64, u64, u64]
        L.orc_open.argtypes = [cp, cp, C.POINTER(Options)]
        L.orc_open.restype = vp
        L.orc_close.argtypes = [vp]
        L.orc_num_contigs.argtypes = [vp]
        L.orc_num_contigs.restype = u64
        L.orc_genome_total_length.argtypes = [vp]
        L.orc_genome_total_length.restype = u64
        L.orc_map_single.argtypes = [vp, C.POINTER(ReadsC), C.POINTER(RecordsC)]
        L.orc_map_paired.argtypes = [vp, C.POINTER(InsertModelC), C.POINTER(ReadsC), C.POINTER(ReadsC),
                                     C.POINTER(RecordsC), C.POINTER(RecordsC)]
        L.orc_time_map_single.argtypes = [vp, C.POINTER(ReadsC), C.POINTER(RecordsC)]
        L.orc_time_map_single.restype = dbl
        L.orc_time_map_paired.argtypes = L.orc_map_paired.argtypes
        L.orc_time_map_paired.restype = dbl
        L.orc_seed_read.argtypes = [vp, vp, vp, u64, vp, vp, vp, vp, u64, vp]
        L.orc_seed_read.restype = i64
        L.orc_cluster_read.argtypes = [vp, vp, vp, u64, vp, vp, vp, vp, u64]
        L.orc_cluster_read.restype = i64
        L.orc_align.argtypes = [vp, vp, u64, vp, u64, i64, u64, u32, u32, vp, vp, vp, u64, vp]
        L.orc_mapq_batch.argtypes = [vp, C.POINTER(ReadsC), vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp, vp]
        L.orc_write_sam.argtypes = [vp, cp, cp, C.POINTER(ReadsC), C.POINTER(cp), C.POINTER(RecordsC)]
        L.orc_sam_write.argtypes = [vp, cp, cp, C.c_int, u32, vp, vp, vp, vp, u64, cp]
        L.orc_sort_coordinate.argtypes = [vp, u32, vp, vp, u64, vp]
        L.orc_reads_parse.argtypes = [cp, C.c_int, C.c_uint8, cp]
        L.orc_reads_parse.restype = vp
        L.orc_reads_count.argtypes = [vp]
        L.orc_reads_count.restype = u64
        L.orc_reads_total_bases.argtypes = [vp]
        L.orc_reads_total_bases.restype = u64
        L.orc_reads_export.argtypes = [vp, vp, vp, vp]
        L.orc_reads_id.argtypes = [vp, u64]
        L.orc_reads_id.restype = cp
        L.orc_reads_free.argtypes = [vp]
        _lib = L
    return _lib


def _err():
    return lib().orc_last_error().decode()


def default_options(**kw) -> Options:
    o = Options()
    lib().orc_default_options(C.byref(o))
    for k, v in kw.items():
        setattr(o, k, v)
    return o


def _ptr(a: np.ndarray) -> int:
    return a.ctypes.data


class Reads:
    """Reads as SoA numpy arrays (bases uint8, quals uint8, offsets uint64)."""

    def __init__(self, bases: np.ndarray, quals: np.ndarray, offsets: np.ndarray, ids=None):
        self.bases = np.ascontiguousarray(bases, dtype=np.uint8)
        self.quals = np.ascontiguousarray(quals, dtype=np.uint8)
        self.offsets = np.ascontiguousarray(offsets, dtype=np.uint64)
        self.ids = ids

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
        offs[1:] = np.cumsum([len(s) for s in seqs])
        b = np.frombuffer(b"".join(seqs), dtype=np.uint8).copy() if seqs else np.zeros(0, np.uint8)
        q = np.frombuffer(b"".join(quals), dtype=np.uint8).copy() if quals else np.zeros(0, np.uint8)
        if ids is None:
            ids = [f"r{i}" for i in range(len(seqs))]
        return Reads(b, q, offs, ids)

    def c(self) -> ReadsC:
        # keep 1-byte arrays alive even when empty
        if self.bases.size == 0:
            self.bases = np.zeros(1, np.uint8)[:0]
            self.quals = np.zeros(1, np.uint8)[:0]
        return ReadsC(self.n, _ptr(self.bases), _ptr(self.quals), _ptr(self.offsets))

    def seq(self, i: int) -> bytes:
        return self.bases[int(self.offsets[i]):int(self.offsets[i + 1])].tobytes()

    def qual(self, i: int) -> bytes:
        return self.quals[int(self.offsets[i]):int(self.offsets[i + 1])].tobytes()


def alloc_records(n: int, total_len: int) -> dict:
    cap = 2 * total_len + 2 * n + 16
    return {
        "contig": np.zeros(n, np.int32),
        "pos": np.zeros(n, np.uint64),
        "mapq": np.zeros(n, np.uint8),
        "flag": np.zeros(n, np.uint16),
        "mate_contig": np.zeros(n, np.int32),
        "mate_pos": np.zeros(n, np.uint64),
        "tlen": np.zeros(n, np.int64),
        "log_lk": np.zeros(n, np.float64),
        "posterior": np.zeros(n, np.float64),
        "as_score": np.zeros(n, np.int32),
        "nm": np.zeros(n, np.int32),
        "cigar_off": np.zeros(n + 1, np.uint32),
        "cigar": np.zeros(cap, np.uint32),
    }


def records_c(r: dict) -> RecordsC:
    n = len(r["contig"])
    return RecordsC(n, *[_ptr(r[k]) for k in ("contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen",
                                               "log_lk", "posterior", "as_score", "nm", "cigar_off", "cigar")],
                    len(r["cigar"]))


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
    out = []
    co, cg = r["cigar_off"], r["cigar"]
    for i in range(len(r["contig"])):
        s = "".join(f"{int(w) >> 4}{OPS[int(w) & 15]}" for w in cg[co[i]:co[i + 1]])
        out.append(s)
    return out


def build_genome_from_seqs(prefix: str, contigs, species="test", assembly="t1"):
    names = [n.encode() for n, _ in contigs]
    seqs = [s.encode() if isinstance(s, str) else bytes(s) for _, s in contigs]
    bufs = [C.create_string_buffer(s, len(s) + 1) for s in seqs]
    n = len(contigs)
    arr_names = (C.c_char_p * n)(*names)
    arr_seqs = (C.c_void_p * n)(*[C.addressof(b) for b in bufs])
    arr_lens = (C.c_uint64 * n)(*[len(s) for s in seqs])
    rc = lib().orc_build_genome_from_seqs(prefix.encode(), species.encode(), assembly.encode(), n, arr_names,
                                          arr_seqs, arr_lens)
    if rc != 0:
        raise RuntimeError(_err())


def build_genome_from_fasta(prefix: str, fasta_paths, species="test", assembly="t1"):
    arr = (C.c_char_p * len(fasta_paths))(*[p.encode() for p in fasta_paths])
    rc = lib().orc_build_genome(prefix.encode(), species.encode(), assembly.encode(), len(fasta_paths), arr)
    if rc != 0:
        raise RuntimeError(_err())


def build_hash(genome_prefix: str, out_prefix: str, k=15, stride=5, max_count=300):
    rc = lib().orc_build_hash(genome_prefix.encode(), out_prefix.encode(), k, stride, max_count)
    if rc != 0:
        raise RuntimeError(_err())


def build_index(prefix: str, contigs, **kw):
    build_genome_from_seqs(prefix, contigs)
    build_hash(prefix, prefix, **kw)


class Mapper:
    def __init__(self, genome_prefix: str, hash_prefix: str | None = None, **opts):
        self.opts = default_options(**opts)
        h = lib().orc_open(genome_prefix.encode(), (hash_prefix or genome_prefix).encode(), C.byref(self.opts))
        if not h:
            raise RuntimeError(_err())
        self.h = h

    def close(self):
        if self.h:
            lib().orc_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def map_single(self, reads: Reads) -> dict:
        recs = alloc_records(reads.n, len(reads.bases))
        rc = lib().orc_map_single(self.h, C.byref(reads.c()), C.byref(records_c(recs)))
        if rc != 0:
            raise RuntimeError(_err())
        return recs

    def time_map_single(self, reads: Reads):
        recs = alloc_records(reads.n, len(reads.bases))
        t = lib().orc_time_map_single(self.h, C.byref(reads.c()), C.byref(records_c(recs)))
        return t, recs

    def map_paired(self, r1: Reads, r2: Reads, mean=None, sd=None):
        m = InsertModelC(self.opts.insert_size_mean if mean is None else mean,
                         self.opts.insert_size_sd if sd is None else sd, 0)
        o1 = alloc_records(r1.n, len(r1.bases))
        o2 = alloc_records(r2.n, len(r2.bases))
        rc = lib().orc_map_paired(self.h, C.byref(m), C.byref(r1.c()), C.byref(r2.c()), C.byref(records_c(o1)),
                                  C.byref(records_c(o2)))
        if rc != 0:
            raise RuntimeError(_err())
        return o1, o2, (m.mean, m.sd, m.n_observed)

    def time_map_paired(self, r1: Reads, r2: Reads):
        m = InsertModelC(self.opts.insert_size_mean, self.opts.insert_size_sd, 0)
        o1 = alloc_records(r1.n, len(r1.bases))
        o2 = alloc_records(r2.n, len(r2.bases))
        t = lib().orc_time_map_paired(self.h, C.byref(m), C.byref(r1.c()), C.byref(r2.c()), C.byref(records_c(o1)),
                                      C.byref(records_c(o2)))
        return t, o1, o2

    def seed_read(self, seq: bytes, qual: bytes, cap=1 << 16):
        L = len(seq)
        s = np.frombuffer(seq, np.uint8).copy() if L else np.zeros(1, np.uint8)
        q = np.frombuffer(qual, np.uint8).copy() if L else np.zeros(1, np.uint8)
        rp = np.zeros(cap, np.uint64)
        hc = np.zeros(cap, np.uint32)
        hp = np.zeros(cap, np.uint64)
        hs = np.zeros(cap, np.uint8)
        rep = np.zeros(max(L, 1), np.float64)
        n = lib().orc_seed_read(self.h, _ptr(s), _ptr(q), L, _ptr(rp), _ptr(hc), _ptr(hp), _ptr(hs), cap, _ptr(rep))
        if n < 0:
            raise RuntimeError(f"hit capacity exceeded ({-n})")
        nw = max(L - 14, 0)
        return rp[:n], hc[:n], hp[:n], hs[:n], rep[:nw]

    def cluster_read(self, seq: bytes, qual: bytes, cap=1 << 16):
        L = len(seq)
        s = np.frombuffer(seq, np.uint8).copy() if L else np.zeros(1, np.uint8)
        q = np.frombuffer(qual, np.uint8).copy() if L else np.zeros(1, np.uint8)
        cc = np.zeros(cap, np.uint32)
        cp = np.zeros(cap, np.uint64)
        cs = np.zeros(cap, np.uint8)
        sc = np.zeros(cap, np.float64)
        n = lib().orc_cluster_read(self.h, _ptr(s), _ptr(q), L, _ptr(cc), _ptr(cp), _ptr(cs), _ptr(sc), cap)
        if n < 0:
            raise RuntimeError(f"candidate capacity exceeded ({-n})")
        return cc[:n], cp[:n], cs[:n], sc[:n]

    def _sources(self, sources):
        keep = []
        rp = (C.c_void_p * len(sources))()
        ip = (C.c_void_p * len(sources))()
        sp = (C.c_void_p * len(sources))()
        for k, (reads, recs) in enumerate(sources):
            rc_ = reads.c()
            ids = (C.c_char_p * max(reads.n, 1))(*[i.encode() for i in reads.ids])
            cr = records_c(recs)
            keep += [rc_, ids, cr]
            rp[k] = C.addressof(rc_)
            ip[k] = C.addressof(ids)
            sp[k] = C.addressof(cr)
        return rp, ip, sp, keep

    def sam_text(self, path: str, sources, sel=None, command_line="probebwa map", read_group=None,
                 coordinate_sorted=False) -> bytes:
        """format_sam_records_sorted (sam.rs:83-108) over the records numbered
        r * len(sources) + s listed in sel (all, in number order, by default);
        written to path and returned."""
        rp, ip, sp, keep = self._sources(sources)
        if sel is None:
            sel = np.arange(len(sources[0][1]["contig"]) * len(sources), dtype=np.uint64)
        sel = np.ascontiguousarray(sel, dtype=np.uint64)
        selk = sel if sel.size else np.zeros(1, np.uint64)
        rc = lib().orc_sam_write(self.h, command_line.encode(), read_group.encode() if read_group is not None else None,
                                 1 if coordinate_sorted else 0, len(sources), rp, ip, sp, _ptr(selk), sel.size,
                                 path.encode())
        if rc != 0:
            raise RuntimeError(_err())
        with open(path, "rb") as f:
            return f.read()

    def sort_coordinate(self, sources, sel=None) -> np.ndarray:
        """sort_for_coordinate_order (sam.rs:114-124) of record numbers."""
        rp, ip, sp, keep = self._sources(sources)
        if sel is None:
            sel = np.arange(len(sources[0][1]["contig"]) * len(sources), dtype=np.uint64)
        sel = np.ascontiguousarray(sel, dtype=np.uint64)
        out = np.zeros(max(sel.size, 1), np.uint64)
        selk = sel if sel.size else np.zeros(1, np.uint64)
        lib().orc_sort_coordinate(self.h, len(sources), sp, _ptr(selk), sel.size, _ptr(out))
        return out[:sel.size]

    def write_sam(self, path: str, reads: Reads, recs: dict, command_line="probebwa map"):
        ids = (C.c_char_p * reads.n)(*[i.encode() for i in reads.ids])
        rc = lib().orc_write_sam(self.h, path.encode(), command_line.encode(), C.byref(reads.c()), ids,
                                 C.byref(records_c(recs)))
        if rc != 0:
            raise RuntimeError(_err())

    def mapq_batch(self, reads: Reads, items) -> dict:
        """select_best + finalize_mapq per read; items as pack_mapq_items."""
        (lk_off, lks, win_off, rep, rev, ref_off, refs, cig_off, cig), out = pack_mapq_items(items)
        rc = lib().orc_mapq_batch(self.h, C.byref(reads.c()), _ptr(lk_off), _ptr(lks), _ptr(win_off), _ptr(rep),
                                  _ptr(rev), _ptr(ref_off), _ptr(refs), _ptr(cig_off), _ptr(cig), _ptr(out["mapq"]),
                                  _ptr(out["posterior"]), _ptr(out["best"]), _ptr(out["sum_exp"]))
        if rc != 0:
            raise RuntimeError("orc_mapq_batch failed")
        return out


def align(read: bytes, qual: bytes, ref: bytes, hint: int, band: int, gop=40, gep=3):
    """SmithWatermanAligner::new(band, gop, gep).align(read, qual, ref, hint)."""
    r = np.frombuffer(read, np.uint8).copy() if read else np.zeros(1, np.uint8)
    q = np.frombuffer(qual, np.uint8).copy() if qual else np.zeros(1, np.uint8)
    f = np.frombuffer(ref, np.uint8).copy() if ref else np.zeros(1, np.uint8)
    score = np.zeros(1, np.int32)
    off = np.zeros(1, np.uint64)
    cap = 2 * len(read) + len(ref) + 8
    cg = np.zeros(cap, np.uint32)
    nops = np.zeros(1, np.uint64)
    rc = lib().orc_align(_ptr(r), _ptr(q), len(read), _ptr(f), len(ref), hint, band, gop, gep, _ptr(score),
                         _ptr(off), _ptr(cg), cap, _ptr(nops))
    if rc != 0:
        raise RuntimeError("cigar capacity")
    cig = "".join(f"{int(w) >> 4}{OPS[int(w) & 15]}" for w in cg[:int(nops[0])])
    return int(score[0]), cig, int(off[0])


def parse_reads(path: str, fasta=False, quality_offset=33, adapter=None) -> Reads:
    h = lib().orc_reads_parse(path.encode(), 1 if fasta else 0, quality_offset,
                              adapter.encode() if adapter else None)
    if not h:
        raise RuntimeError(_err())
    try:
        n = lib().orc_reads_count(h)
        tot = lib().orc_reads_total_bases(h)
        b = np.zeros(max(tot, 1), np.uint8)
        q = np.zeros(max(tot, 1), np.uint8)
        o = np.zeros(n + 1, np.uint64)
        lib().orc_reads_export(h, _ptr(b), _ptr(q), _ptr(o))
        ids = [lib().orc_reads_id(h, i).decode() for i in range(n)]
        return Reads(b[:tot], q[:tot], o, ids)
    finally:
        lib().orc_reads_free(h)
