"""Seeded synthetic genomes, reads and index files for the benchmark workloads.

No public dataset is used: genomes and reads are generated from fixed seeds
with the shapes and value distributions of the benchmark configurations
(GC 41%, planted repeat copies, segmental duplications, homopolymer runs,
substitution/indel errors, Phred qualities from a clipped normal).

write_index() writes .stidx / .sthash files in the reference's bincode layout
(src/index/genome.rs:72-94, src/index/hashtable.rs:60-87,248-322) with numpy:
forward 15-mers at positions i % 5 == 0, then reverse-complement 15-mers at
rc index i % 5 == 0 (stored at forward coordinate len-i-15), N-containing
windows skipped, the first 300 occurrences of each hash kept in scan order,
buckets in ascending hash order.
"""
from __future__ import annotations

import os
import struct

import numpy as np

ASCII = np.frombuffer(b"ACGTN", dtype=np.uint8)
GC41 = np.array([0.295, 0.205, 0.205, 0.295])  # A C G T


def rand_codes(rng: np.random.Generator, n: int, p=GC41) -> np.ndarray:
    return rng.choice(4, size=n, p=p).astype(np.uint8)


def mutate_subs(rng, codes: np.ndarray, rate: float) -> np.ndarray:
    out = codes.copy()
    m = rng.random(len(out)) < rate
    out[m] = (out[m] + rng.integers(1, 4, size=int(m.sum()))) % 4
    return out


# ---------------------------------------------------------------------------
# genomes
# ---------------------------------------------------------------------------
def genome_single(seed: int, length=1_000_000, n_copies=20, copy_len=2000):
    """1 contig, GC 41%, n_copies planted copies of one copy_len unit at U(97, 99.5)% identity."""
    rng = np.random.default_rng(seed)
    g = rand_codes(rng, length)
    unit = rand_codes(rng, copy_len)
    starts = np.sort(rng.choice(np.arange(0, length - copy_len, copy_len), size=n_copies, replace=False))
    for s in starts:
        ident = rng.uniform(0.97, 0.995)
        g[s:s + copy_len] = mutate_subs(rng, unit, 1.0 - ident)
    return [("chr1", g)]


def genome_paired(seed: int, n_contigs=25, contig_len=4_000_000, dup_frac=0.05, hp_rate=1 / 2000):
    """25 x 4 Mbp, GC 41%, 5% segmental duplications (1-10 kbp, 2-8 copies,
    95-99.5% identity), homopolymer runs of 6-15 bp at 1 per 2 kbp."""
    rng = np.random.default_rng(seed)
    contigs = [rand_codes(rng, contig_len) for _ in range(n_contigs)]
    total = n_contigs * contig_len
    target = int(dup_frac * total)
    placed = 0
    while placed < target:
        L = int(rng.integers(1000, 10_001))
        ncopy = int(rng.integers(2, 9))
        sc = int(rng.integers(n_contigs))
        ss = int(rng.integers(0, contig_len - L))
        unit = contigs[sc][ss:ss + L].copy()
        for _ in range(ncopy - 1):
            c = int(rng.integers(n_contigs))
            s = int(rng.integers(0, contig_len - L))
            contigs[c][s:s + L] = mutate_subs(rng, unit, 1.0 - rng.uniform(0.95, 0.995))
            placed += L
    for c in contigs:
        nh = rng.poisson(len(c) * hp_rate)
        pos = rng.integers(0, len(c) - 16, size=nh)
        lens = rng.integers(6, 16, size=nh)
        base = rng.integers(0, 4, size=nh)
        for p, l, b in zip(pos, lens, base):
            c[p:p + l] = b
    return [(f"chr{i + 1}", c) for i, c in enumerate(contigs)]


# ---------------------------------------------------------------------------
# reads
# ---------------------------------------------------------------------------
def genome_families(seed: int, total=300_000_000, n_contigs=12, family_frac=0.45, n_families=500,
                    cons_len=(300, 6000), divergence=(0.02, 0.25), tandem_frac=0.03):
    """Contig lengths U(50, 250) scaled to `total`, GC 41%; `family_frac` of the
    bases are copies of `n_families` interspersed repeat families (consensus
    300 bp-6 kbp, each copy diverged by U(2, 25)% substitutions), and
    `tandem_frac` are tandem arrays of short units (2-50 bp)."""
    rng = np.random.default_rng(seed)
    w = rng.uniform(50, 250, n_contigs)
    lens = np.maximum((w / w.sum() * total).astype(np.int64), 10_000)
    g = rand_codes(rng, int(lens.sum()))
    cons = [rand_codes(rng, int(rng.integers(cons_len[0], cons_len[1] + 1))) for _ in range(n_families)]
    # copies: families drawn in proportion, placed at random non-overlapping slots
    target = int(family_frac * len(g))
    placed = 0
    starts = np.sort(rng.choice(len(g) - cons_len[1] - 1, size=int(target / np.mean(cons_len) * 1.2), replace=False))
    last_end = 0
    for st in starts:
        if placed >= target:
            break
        if st < last_end:
            continue
        fam = cons[int(rng.integers(0, n_families))]
        cp = mutate_subs(rng, fam, rng.uniform(*divergence))
        g[st:st + len(cp)] = cp
        last_end = st + len(cp)
        placed += len(cp)
    # tandem arrays
    t_target = int(tandem_frac * len(g))
    t_placed = 0
    while t_placed < t_target:
        unit = rand_codes(rng, int(rng.integers(2, 51)))
        reps = int(rng.integers(10, 200))
        arr = np.tile(unit, reps)
        st = int(rng.integers(0, len(g) - len(arr)))
        g[st:st + len(arr)] = mutate_subs(rng, arr, 0.02)
        t_placed += len(arr)
    out, o = [], 0
    for i, L in enumerate(lens):
        out.append((f"chr{i + 1}", g[o:o + L].copy()))
        o += L
    return out


def trim_lengths(seed: int, bases: np.ndarray, quals: np.ndarray, offs: np.ndarray, lo=60, hi=250):
    """Each read cut to a length drawn from U[lo, hi] (its 3' end dropped), as
    after adapter trimming; reads shorter than the draw are kept whole."""
    rng = np.random.default_rng(seed)
    n = len(offs) - 1
    L = np.diff(offs).astype(np.int64)
    keep = np.minimum(rng.integers(lo, hi + 1, n), L)
    starts = offs[:-1].astype(np.int64)
    idx = np.repeat(starts, keep) + (np.arange(keep.sum()) - np.repeat(np.cumsum(keep) - keep, keep))
    no = np.zeros(n + 1, np.uint64)
    no[1:] = np.cumsum(keep)
    return bases[idx], quals[idx], no


def _quals(rng, n, mu=35.0, sd=4.0):
    return np.clip(np.rint(rng.normal(mu, sd, size=n)), 2, 41).astype(np.uint8)


def _errors(rng, frag: np.ndarray, sub_rate: float, indel_rate: float, hp_mask=None, hp_boost=5.0):
    """Substitutions (with lowered quality) and geometric(mean 1.5) indels."""
    L = len(frag)
    rate_s = np.full(L, sub_rate)
    rate_i = np.full(L, indel_rate)
    if hp_mask is not None:
        rate_s[hp_mask] *= hp_boost
        rate_i[hp_mask] *= hp_boost
    out = list(frag)
    subs = np.nonzero(rng.random(L) < rate_s)[0]
    lowered = set()
    for p in subs:
        out[p] = (out[p] + int(rng.integers(1, 4))) % 4
        lowered.add(int(p))
    indel_pos = np.nonzero(rng.random(L) < rate_i)[0]
    if len(indel_pos) == 0:
        return np.array(out, np.uint8), lowered
    res = []
    low2 = set()
    i = 0
    ip = set(int(x) for x in indel_pos)
    while i < L:
        if i in ip:
            ln = int(rng.geometric(2 / 3))
            if rng.random() < 0.5:  # insertion of random bases
                for _ in range(ln):
                    res.append(int(rng.integers(4)))
                res.append(out[i])
                if i in lowered:
                    low2.add(len(res) - 1)
                i += 1
            else:  # deletion skips reference
                i += ln
            continue
        res.append(out[i])
        if i in lowered:
            low2.add(len(res) - 1)
        i += 1
    return np.array(res, np.uint8), low2


def _make_read(rng, frag, sub, indel, qmu, qsd, L, hp_mask=None):
    seq, low = _errors(rng, frag, sub, indel, hp_mask)
    seq = seq[:L]
    q = _quals(rng, len(seq), qmu, qsd)
    for p in low:
        if p < len(q):
            q[p] = np.clip(np.rint(rng.normal(12, 4)), 2, 41)
    return seq, q


def _rc(codes):
    return (3 - codes[::-1]).astype(np.uint8)


def reads_single(seed: int, contigs, n=10_000, L=120, sub=0.01, indel=0.001, qmu=35.0, qsd=4.0):
    """n reads of length L, uniform start, both strands (50/50)."""
    rng = np.random.default_rng(seed)
    seqs, quals, truth = [], [], []
    lens = np.array([len(c) for _, c in contigs])
    cum = np.cumsum(lens)
    for i in range(n):
        g = int(rng.integers(0, cum[-1]))
        ci = int(np.searchsorted(cum, g, side="right"))
        c = contigs[ci][1]
        s = int(rng.integers(0, len(c) - L - 8))
        frag = c[s:s + L + 8]
        seq, q = _make_read(rng, frag, sub, indel, qmu, qsd, L)
        rev = bool(rng.random() < 0.5)
        if rev:
            seq, q = _rc(seq), q[::-1].copy()
        seqs.append(ASCII[seq].tobytes())
        quals.append(q.tobytes())
        truth.append((ci, s, rev))
    return seqs, quals, truth


def reads_paired(seed: int, contigs, n_pairs, L=150, mean=350.0, sd=50.0, sub=0.005, indel=0.0005, qmu=35.0,
                 qsd=4.0):
    """FR pairs: mate1 forward from the fragment start, mate2 the reverse complement of its end."""
    rng = np.random.default_rng(seed)
    s1, q1, s2, q2, truth = [], [], [], [], []
    lens = np.array([len(c) for _, c in contigs])
    cum = np.cumsum(lens)
    for i in range(n_pairs):
        g = int(rng.integers(0, cum[-1]))
        ci = int(np.searchsorted(cum, g, side="right"))
        c = contigs[ci][1]
        ins = int(max(L + 10, round(rng.normal(mean, sd))))
        s = int(rng.integers(0, len(c) - ins - 8))
        f1 = c[s:s + L + 8]
        e = s + ins
        f2 = _rc(c[max(e - L - 8, 0):e])
        hp1 = _hp_mask(f1)
        hp2 = _hp_mask(f2)
        a, qa = _make_read(rng, f1, sub, indel, qmu, qsd, L, hp1)
        b, qb = _make_read(rng, f2, sub, indel, qmu, qsd, L, hp2)
        if rng.random() < 0.5:
            a, qa, b, qb = b, qb, a, qa
        s1.append(ASCII[a].tobytes())
        q1.append(qa.tobytes())
        s2.append(ASCII[b].tobytes())
        q2.append(qb.tobytes())
        truth.append((ci, s, ins))
    return s1, q1, s2, q2, truth


def _hp_mask(codes, min_run=6):
    if len(codes) == 0:
        return np.zeros(0, bool)
    change = np.concatenate([[True], codes[1:] != codes[:-1]])
    idx = np.cumsum(change) - 1
    runlen = np.bincount(idx)[idx]
    return runlen >= min_run


# ---------------------------------------------------------------------------
# index files
# ---------------------------------------------------------------------------
def _mix32(h: np.ndarray) -> np.ndarray:
    h = h.astype(np.uint32)
    h ^= h >> np.uint32(16)
    h *= np.uint32(0x7FEB352D)
    h ^= h >> np.uint32(15)
    h *= np.uint32(0x846CA68B)
    h ^= h >> np.uint32(16)
    return h


def _kmer_codes_at(codes: np.ndarray, idx: np.ndarray, k=15):
    """Raw 30-bit codes of the k-windows starting at idx, and whether each is ACGT-only (codes 0-3, 4 = N)."""
    raw = np.zeros(len(idx), np.uint32)
    for t in range(k):
        raw = (raw << np.uint32(2)) | (codes[idx + t].astype(np.uint32) & np.uint32(3))
    isn = np.concatenate([[0], np.cumsum(codes > 3, dtype=np.int64)])
    ok = (isn[idx + k] - isn[idx]) == 0
    return raw, ok


def pack_contig(codes: np.ndarray):
    """Contig::from_ascii (src/index/genome.rs:17-45): 2-bit packing + N runs."""
    L = len(codes)
    bits = np.where(codes > 3, 0, codes).astype(np.uint8)
    pad = (-L) % 4
    b = np.concatenate([bits, np.zeros(pad, np.uint8)]).reshape(-1, 4)
    packed = (b[:, 0] | (b[:, 1] << 2) | (b[:, 2] << 4) | (b[:, 3] << 6)).astype(np.uint8)
    isn = codes > 3
    runs = []
    if isn.any():
        d = np.diff(np.concatenate([[0], isn.astype(np.int8), [0]]))
        st = np.nonzero(d == 1)[0]
        en = np.nonzero(d == -1)[0]
        runs = list(zip(st.tolist(), en.tolist()))
    return packed, runs


def read_stidx_contigs(prefix: str):
    """Contigs of a .stidx file as (name, codes) with codes A0 C1 G2 T3 N4
    (Contig::slice, src/index/genome.rs:48-68, for whole contigs)."""
    data = open(prefix + ".stidx", "rb").read()
    p = 0

    def u64():
        nonlocal p
        v = struct.unpack_from("<Q", data, p)[0]
        p += 8
        return v

    def string():
        nonlocal p
        n = u64()
        v = data[p:p + n].decode()
        p += n
        return v

    string()
    string()
    out = []
    for _ in range(u64()):
        name = string()
        npk = u64()
        packed = np.frombuffer(data, np.uint8, npk, p)
        p += npk
        nr = u64()
        runs = np.frombuffer(data, np.uint32, 2 * nr, p).reshape(-1, 2)
        p += 8 * nr
        length = u64()
        codes = np.stack([(packed >> (2 * k)) & 3 for k in range(4)], axis=1).reshape(-1)[:length].astype(np.uint8)
        for a, b in runs:
            codes[a:min(b, length)] = 4
        out.append((name, codes))
    return out


def write_stidx(prefix: str, contigs, species="synthetic", assembly="synthetic"):
    with open(prefix + ".stidx", "wb") as f:
        def s(x: str):
            b = x.encode()
            f.write(struct.pack("<Q", len(b)))
            f.write(b)
        s(species)
        s(assembly)
        f.write(struct.pack("<Q", len(contigs)))
        total = 0
        for name, codes in contigs:
            packed, runs = pack_contig(codes)
            s(name)
            f.write(struct.pack("<Q", len(packed)))
            f.write(packed.tobytes())
            f.write(struct.pack("<Q", len(runs)))
            if runs:
                f.write(np.array(runs, np.uint32).tobytes())
            f.write(struct.pack("<Q", len(codes)))
            total += len(codes)
        f.write(struct.pack("<Q", total))


def build_sthash(contigs, k=15, stride=5, max_count=300):
    """HashTableBuilder::build restated with numpy; returns (keys, offs, counts, positions)."""
    hs, ps = [], []
    for cid, (_, codes) in enumerate(contigs):
        L = len(codes)
        if L < k:
            continue
        idx = np.arange(0, L - k + 1, stride, dtype=np.int64)
        raw, ok = _kmer_codes_at(codes, idx, k)
        sel = idx[ok]
        hs.append(_mix32(raw[ok]))
        ps.append((np.uint64(cid) << np.uint64(40)) | sel.astype(np.uint64))
        rc = np.where(codes > 3, 4, 3 - codes)[::-1].astype(np.uint8)
        rraw, rok = _kmer_codes_at(rc, idx, k)
        sel = idx[rok]
        hs.append(_mix32(rraw[rok]))
        fpos = (L - sel - k).astype(np.uint64)
        ps.append((np.uint64(1) << np.uint64(63)) | (np.uint64(cid) << np.uint64(40)) | fpos)
    h = np.concatenate(hs) if hs else np.zeros(0, np.uint32)
    p = np.concatenate(ps) if ps else np.zeros(0, np.uint64)
    order = np.argsort(h, kind="stable")
    h = h[order]
    p = p[order]
    if len(h) == 0:
        return np.zeros(0, np.uint32), np.zeros(0, np.uint32), np.zeros(0, np.uint32), p
    start = np.empty(len(h), bool)
    start[0] = True
    np.not_equal(h[1:], h[:-1], out=start[1:])
    gs = np.flatnonzero(start)
    glen = np.diff(np.append(gs, len(h)))
    rank = np.arange(len(h)) - np.repeat(gs, glen)
    keep = rank < max_count
    if not keep.all():
        h = h[keep]
        p = p[keep]
        start = start[keep]
        gs = np.flatnonzero(start)
    keys = h[gs]
    counts = np.diff(np.append(gs, len(h))).astype(np.uint32)
    offs = gs.astype(np.uint32)
    return keys, offs, counts, p


def write_sthash(prefix: str, contigs, k=15, stride=5, max_count=300):
    keys, offs, counts, pos = build_sthash(contigs, k, stride, max_count)
    with open(prefix + ".sthash", "wb") as f:
        f.write(struct.pack("<Q", len(keys)))
        tab = np.stack([keys, offs, counts], axis=1).astype(np.uint32)
        f.write(tab.tobytes())
        f.write(struct.pack("<Q", len(pos)))
        f.write(pos.astype(np.uint64).tobytes())
        f.write(struct.pack("<QQQ", k, stride, int(counts.sum()) if len(counts) else 0))


def write_index(prefix: str, contigs, **kw):
    os.makedirs(os.path.dirname(os.path.abspath(prefix)), exist_ok=True)
    write_stidx(prefix, contigs)
    write_sthash(prefix, contigs, **kw)


def contigs_from_strings(contigs):
    lut = np.full(256, 4, np.uint8)
    for i, c in enumerate(b"ACGT"):
        lut[c] = i
        lut[c + 32] = i
    return [(n, lut[np.frombuffer(s.encode() if isinstance(s, str) else s, np.uint8)]) for n, s in contigs]


# ---------------------------------------------------------------------------
# vectorised read generation for the large workloads
# ---------------------------------------------------------------------------
def _concat(contigs):
    lens = np.array([len(c) for _, c in contigs], np.int64)
    starts = np.concatenate([[0], np.cumsum(lens)[:-1]])
    return np.concatenate([c for _, c in contigs]).astype(np.uint8), starts, lens


def _hp_mask_genome(g: np.ndarray, min_run=6) -> np.ndarray:
    ch = np.flatnonzero(g[1:] != g[:-1]) + 1
    starts = np.concatenate([[0], ch])
    lens = np.diff(np.append(starts, len(g)))
    return np.repeat(lens >= min_run, lens)


def _hp_mask_rows(f: np.ndarray, min_run=6) -> np.ndarray:
    """Per row: positions inside a run of >= min_run equal bases (within the row)."""
    n, W = f.shape
    eq = np.zeros((n, W + 1), np.int32)
    eq[:, 1:W] = (f[:, 1:] == f[:, :-1])
    c = np.cumsum(eq, axis=1)
    k = min_run - 1  # a run of min_run bases has min_run-1 equal neighbours
    full = np.zeros((n, W), bool)
    if W > k:
        win = (c[:, k:W] - c[:, 0:W - k]) == k  # window ending at column j (j >= k) is one run
        for t in range(k + 1):
            full[:, t:W - k + t] |= win
    return full


def _apply_errors_vec(rng, frags: np.ndarray, hp: np.ndarray, L: int, sub: float, indel: float, qmu: float,
                      qsd: float):
    """frags: (n, L + pad) base codes; hp: same-shape homopolymer mask (5x error rates).
    Returns lists of (codes, quals) of length L (indel reads handled one by one)."""
    n, W = frags.shape
    rate_s = np.where(hp, 5 * sub, sub)
    rate_i = np.where(hp, 5 * indel, indel)
    subm = rng.random((n, W)) < rate_s
    out = frags.copy()
    out[subm] = (out[subm] + rng.integers(1, 4, size=int(subm.sum()))).astype(np.uint8) % 4
    q = np.clip(np.rint(rng.normal(qmu, qsd, size=(n, W))), 2, 41).astype(np.uint8)
    low = np.clip(np.rint(rng.normal(12, 4, size=int(subm.sum()))), 2, 41).astype(np.uint8)
    q[subm] = low
    indm = rng.random((n, W)) < rate_i
    has = np.nonzero(indm[:, :L].any(axis=1))[0]
    seqs = out[:, :L].copy()
    quals = q[:, :L].copy()
    er, ec = np.nonzero(indm[has])
    bounds = np.searchsorted(er, np.arange(len(has) + 1))
    for hi, r in enumerate(has):
        ev = ec[bounds[hi]:bounds[hi + 1]]
        pieces, qp = [], []
        i = 0
        for e in ev:
            if e < i:
                continue
            pieces.append(out[r, i:e])
            qp.append(q[r, i:e])
            ln = int(rng.geometric(2 / 3))
            if rng.random() < 0.5:  # insertion before base e
                pieces.append(rng.integers(0, 4, size=ln).astype(np.uint8))
                qp.append(np.full(ln, q[r, e], np.uint8))
                i = e
            else:  # deletion of ln reference bases
                i = e + ln
            if sum(len(x) for x in pieces) >= L:
                break
        pieces.append(out[r, i:])
        qp.append(q[r, i:])
        sq = np.concatenate(pieces)[:L]
        qq = np.concatenate(qp)[:L]
        if len(sq) < L:
            sq = np.concatenate([sq, np.zeros(L - len(sq), np.uint8)])
            qq = np.concatenate([qq, np.full(L - len(qq), 30, np.uint8)])
        seqs[r] = sq
        quals[r] = qq
    return seqs, quals


def reads_paired_fast(seed: int, contigs, n_pairs: int, L=150, mean=350.0, sd=50.0, sub=0.005, indel=0.0005,
                      qmu=35.0, qsd=4.0, chunk=200_000):
    """Vectorised FR pairs (same model as reads_paired): returns SoA arrays
    (bases1, quals1, offs1, bases2, quals2, offs2) of fixed-length-L reads."""
    rng = np.random.default_rng(seed)
    g, starts, lens = _concat(contigs)
    pad = 8
    b1s, q1s, b2s, q2s = [], [], [], []
    done = 0
    while done < n_pairs:
        n = min(chunk, n_pairs - done)
        ci = rng.choice(len(lens), size=n, p=lens / lens.sum())
        ins = np.maximum(L + 10, np.rint(rng.normal(mean, sd, size=n))).astype(np.int64)
        s = (rng.random(n) * (lens[ci] - ins - pad - 1)).astype(np.int64)
        gs = starts[ci] + s
        ge = gs + ins
        idx1 = gs[:, None] + np.arange(L + pad)[None, :]
        idx2 = (ge - 1)[:, None] - np.arange(L + pad)[None, :]
        f1 = g[idx1]
        f2 = np.where(g[idx2] > 3, 4, 3 - g[idx2]).astype(np.uint8)
        a, qa = _apply_errors_vec(rng, f1, _hp_mask_rows(f1), L, sub, indel, qmu, qsd)
        b, qb = _apply_errors_vec(rng, f2, _hp_mask_rows(f2), L, sub, indel, qmu, qsd)
        swap = rng.random(n) < 0.5
        a2 = np.where(swap[:, None], b, a)
        b2 = np.where(swap[:, None], a, b)
        qa2 = np.where(swap[:, None], qb, qa)
        qb2 = np.where(swap[:, None], qa, qb)
        b1s.append(ASCII[a2].reshape(-1))
        q1s.append(qa2.reshape(-1))
        b2s.append(ASCII[b2].reshape(-1))
        q2s.append(qb2.reshape(-1))
        done += n
    offs = np.arange(n_pairs + 1, dtype=np.uint64) * np.uint64(L)
    return (np.concatenate(b1s), np.concatenate(q1s), offs, np.concatenate(b2s), np.concatenate(q2s), offs.copy())


def reads_single_fast(seed: int, contigs, n: int, L=120, sub=0.01, indel=0.001, qmu=35.0, qsd=4.0):
    """Vectorised single-end reads, both strands: (bases, quals, offsets)."""
    rng = np.random.default_rng(seed)
    g, starts, lens = _concat(contigs)
    pad = 8
    ci = rng.choice(len(lens), size=n, p=lens / lens.sum())
    s = (rng.random(n) * (lens[ci] - L - pad - 1)).astype(np.int64)
    idx = (starts[ci] + s)[:, None] + np.arange(L + pad)[None, :]
    f = g[idx]
    a, q = _apply_errors_vec(rng, f, np.zeros(f.shape, bool), L, sub, indel, qmu, qsd)
    rev = rng.random(n) < 0.5
    rc = np.where(a[:, ::-1] > 3, 4, 3 - a[:, ::-1]).astype(np.uint8)
    a = np.where(rev[:, None], rc, a)
    q = np.where(rev[:, None], q[:, ::-1], q)
    offs = np.arange(n + 1, dtype=np.uint64) * np.uint64(L)
    return ASCII[a].reshape(-1), q.reshape(-1).copy(), offs
