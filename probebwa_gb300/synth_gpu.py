"""Seeded synthetic genomes and reads at human-genome scale, generated with
torch on a CUDA device (or on the CPU for small cases).

The hg38-scale workloads (a 3.1 Gbp genome, 10-12 million reads) take
minutes with the numpy generators of synth.py; here every step is a tensor
operation:

* genome_hg(): 24 contigs of U(50, 250) relative size scaled to the total,
  GC 41%; 45% of the bases are copies of 500 interspersed repeat families
  (consensus 300 bp-6 kbp, each copy diverged by U(2, 25)% substitutions) and
  3% tandem arrays (units of 2-50 bp repeated 10-200 times, 2% divergence).
  The layout is a chain of [unique gap][insert] segments whose gap length is
  exponential with the mean that gives those fractions.
* add_stress(): the stress genome's extra content, laid over a genome: 200
  families of 32-64 near-identical copies (99-99.9% identity) and
  homopolymer-rich regions (runs of 8-20 bp, one per 500 bp).
* reads(): single-end reads or FR pairs (insert N(mean, sd)) of length L,
  both strands, substitutions (quality lowered to N(12, 4) at substituted
  bases) and geometric(mean 1.5) indels, both 5x more frequent inside
  homopolymers of 6 or more bases, Phred N(qmu, qsd) clipped to [2, 41];
  optionally trimmed to lengths U[lo, hi] (3' end dropped).

Results are numpy arrays in the layouts synth.py uses (base codes A0 C1 G2 T3
N4 for genomes; ASCII bases, raw Phred scores and u64 offsets for reads), so
write_stidx() output and the reads feed the same C ABI. A fixed seed gives the
same data on the same device type and torch version.
"""
from __future__ import annotations

import math
import struct

import numpy as np

GC41 = (0.295, 0.205, 0.205, 0.295)  # A C G T
ASCII = np.frombuffer(b"ACGTN", dtype=np.uint8)


def _torch():
    import torch
    return torch


def _dev(device):
    torch = _torch()
    if device is None:
        device = "cuda" if torch.cuda.is_available() else "cpu"
    return torch.device(device)


def _gen(device, seed: int):
    torch = _torch()
    g = torch.Generator(device=device)
    g.manual_seed(int(seed) & ((1 << 63) - 1))
    return g


def _rand_codes(n: int, gen, device, out=None):
    """n base codes with P(A)=P(T)=0.295, P(C)=P(G)=0.205 (uint8)."""
    torch = _torch()
    u = torch.rand(n, generator=gen, device=device)
    c = (u >= GC41[0]).to(torch.uint8) + (u >= GC41[0] + GC41[1]).to(torch.uint8) + \
        (u >= GC41[0] + GC41[1] + GC41[2]).to(torch.uint8)
    if out is not None:
        out.copy_(c)
        return out
    return c


def _mutate_(vals, rate, gen):
    """In place: each base (code < 4) replaced by one of the 3 others with
    probability rate (a scalar or a tensor of vals' shape)."""
    torch = _torch()
    m = torch.rand(vals.shape, generator=gen, device=vals.device) < rate
    m &= vals < 4
    shift = torch.randint(1, 4, vals.shape, generator=gen, device=vals.device, dtype=torch.uint8)
    vals.copy_(torch.where(m, (vals + shift) % 4, vals))
    return vals


def _segments(n, lens):
    """Concatenated ranges [0, lens[i]) for every i: (segment index, offset)."""
    torch = _torch()
    seg = torch.repeat_interleave(torch.arange(n, device=lens.device), lens)
    start = torch.cumsum(lens, 0) - lens
    off = torch.arange(int(lens.sum()), device=lens.device) - torch.repeat_interleave(start, lens)
    return seg, off


def genome_hg(seed: int, total: int = 3_100_000_000, n_contigs: int = 24, family_frac: float = 0.45,
              n_families: int = 500, cons_len=(300, 6000), divergence=(0.02, 0.25), tandem_frac: float = 0.03,
              device=None, chunk_bases: int = 1 << 28):
    """Returns (names, lengths, codes): codes is one uint8 numpy array of all
    contigs back to back (codes A0 C1 G2 T3)."""
    torch = _torch()
    dev = _dev(device)
    rng = np.random.default_rng(seed)
    gen = _gen(dev, seed + 1)
    w = rng.uniform(50, 250, n_contigs)
    lens = np.maximum((w / w.sum() * total).astype(np.int64), 10_000)
    total = int(lens.sum())
    g = torch.empty(total, dtype=torch.uint8, device=dev)
    for a in range(0, total, chunk_bases):
        b = min(total, a + chunk_bases)
        _rand_codes(b - a, gen, dev, out=g[a:b])
    cons_l = rng.integers(cons_len[0], cons_len[1] + 1, size=n_families)
    cons_off = np.concatenate([[0], np.cumsum(cons_l)])
    cons = _rand_codes(int(cons_off[-1]), gen, dev)
    # layout: [gap][insert] segments; inserts are family copies with
    # probability a, tandem arrays otherwise
    e_fam = float(np.mean(cons_len))
    e_tan = 26.0 * 105.0
    a = (family_frac * e_tan) / (family_frac * e_tan + tandem_frac * e_fam) if tandem_frac > 0 else 1.0
    d = (a * e_fam) / family_frac
    gap_mean = max(d - a * e_fam - (1 - a) * e_tan, 1.0)
    n_seg = int(total / d * 1.15) + 16
    is_fam = rng.random(n_seg) < a
    fam = rng.integers(0, n_families, size=n_seg)
    t_unit = rng.integers(2, 51, size=n_seg)
    t_reps = rng.integers(10, 200, size=n_seg)
    ins_len = np.where(is_fam, cons_l[fam], t_unit * t_reps).astype(np.int64)
    gap = rng.exponential(gap_mean, size=n_seg).astype(np.int64)
    ins_start = np.cumsum(gap + ins_len) - ins_len
    keep = ins_start + ins_len <= total
    ins_start, ins_len, is_fam, fam, t_unit = ins_start[keep], ins_len[keep], is_fam[keep], fam[keep], t_unit[keep]
    div = rng.uniform(divergence[0], divergence[1], size=len(ins_start))
    # family copies, in chunks of about chunk_bases bases
    for sel, kind in ((np.flatnonzero(is_fam), "fam"), (np.flatnonzero(~is_fam), "tan")):
        if kind == "tan":
            # one random unit per array, repeated
            u_off = np.concatenate([[0], np.cumsum(t_unit[sel])])
            units = _rand_codes(int(u_off[-1]), gen, dev)
        cum = np.cumsum(ins_len[sel])
        lo = 0
        while lo < len(sel):
            hi = int(np.searchsorted(cum, (cum[lo - 1] if lo else 0) + chunk_bases, side="right"))
            hi = max(hi, lo + 1)
            idx = sel[lo:hi]
            ln = torch.as_tensor(ins_len[idx], device=dev)
            seg, off = _segments(len(idx), ln)
            dst = torch.as_tensor(ins_start[idx], device=dev)[seg] + off
            if kind == "fam":
                src = torch.as_tensor(cons_off[fam[idx]], device=dev)[seg] + off
                vals = cons[src]
                rate = torch.as_tensor(div[idx], device=dev, dtype=torch.float32)[seg]
            else:
                ul = torch.as_tensor(t_unit[idx], device=dev)[seg]
                src = torch.as_tensor(u_off[lo:hi], device=dev)[seg] + off % ul
                vals = units[src]
                rate = 0.02
            _mutate_(vals, rate, gen)
            g[dst] = vals
            lo = hi
    names = [f"chr{i + 1}" for i in range(n_contigs)]
    return names, lens, g.cpu().numpy()


def add_stress(seed: int, codes: np.ndarray, lens, n_families: int = 200, copies=(32, 64),
               identity=(0.99, 0.999), fam_len=(300, 6000), hp_region_bp: int = 60_000_000, hp_every: int = 500,
               hp_len=(8, 20), device=None):
    """Lays near-identical repeat families and homopolymer-rich regions over
    a genome (in place on a copy). Returns (codes, regions): regions is a
    list of (start, end) intervals of the genome holding the stress content,
    from which a share of the stress workload's reads is drawn."""
    torch = _torch()
    dev = _dev(device)
    rng = np.random.default_rng(seed)
    gen = _gen(dev, seed + 1)
    g = torch.as_tensor(codes).to(dev, copy=True)
    total = len(codes)
    regions = []
    # near-identical families: copies placed in one band per family
    fl = rng.integers(fam_len[0], fam_len[1] + 1, size=n_families)
    nc = rng.integers(copies[0], copies[1] + 1, size=n_families)
    span = int((fl * nc).sum() * 1.5) + 64 * int(nc.sum())
    base = int(rng.integers(0, total - span - hp_region_bp - 1))
    pos = base
    for f in range(n_families):
        unit = _rand_codes(int(fl[f]), gen, dev)
        start_f = pos
        for _ in range(int(nc[f])):
            v = unit.clone()
            _mutate_(v, float(1.0 - rng.uniform(identity[0], identity[1])), gen)
            g[pos:pos + len(v)] = v
            pos += len(v) + int(rng.integers(20, int(fl[f]) // 2 + 21))
        regions.append((start_f, pos))
    # homopolymer-rich region after the families
    hp0 = pos + 1000
    n_hp = hp_region_bp // hp_every
    hp_pos = hp0 + np.sort(rng.choice(hp_region_bp - hp_len[1], size=n_hp, replace=False))
    hl = rng.integers(hp_len[0], hp_len[1] + 1, size=n_hp)
    hb = rng.integers(0, 4, size=n_hp)
    ln = torch.as_tensor(hl, device=dev)
    seg, off = _segments(n_hp, ln)
    dst = torch.as_tensor(hp_pos, device=dev)[seg] + off
    g[dst] = torch.as_tensor(hb.astype(np.uint8), device=dev)[seg]
    regions.append((hp0, hp0 + hp_region_bp))
    return g.cpu().numpy(), regions


def contigs_of(names, lens, codes):
    """(name, codes view) list over the back-to-back array."""
    out, o = [], 0
    for nm, L in zip(names, lens):
        out.append((nm, codes[o:o + int(L)]))
        o += int(L)
    return out


def write_stidx(prefix: str, names, lens, codes: np.ndarray, species="synthetic", assembly="synthetic", device=None):
    """GenomeIndex::save (src/index/genome.rs:72-94) for N-free contigs:
    bincode of {species, assembly, contigs: [{name, packed, n_runs, length}],
    total_length}; the 2-bit packing (base p at bits (p % 4) * 2 of byte p / 4,
    genome.rs:17-45) runs on the device."""
    torch = _torch()
    dev = _dev(device)
    with open(prefix + ".stidx", "wb") as f:
        def s(x: str):
            b = x.encode()
            f.write(struct.pack("<Q", len(b)))
            f.write(b)
        s(species)
        s(assembly)
        f.write(struct.pack("<Q", len(names)))
        o = 0
        for nm, L in zip(names, lens):
            L = int(L)
            s(nm)
            npk = (L + 3) // 4
            f.write(struct.pack("<Q", npk))
            step = 1 << 28
            for a in range(0, L, step):
                b = min(L, a + step)
                c = torch.as_tensor(codes[o + a:o + b]).to(dev)
                if (b - a) % 4:
                    c = torch.cat([c, torch.zeros(4 - (b - a) % 4, dtype=torch.uint8, device=dev)])
                if bool((c > 3).any()):
                    raise ValueError("write_stidx: N bases are not supported here (use synth.write_stidx)")
                c = c.view(-1, 4)
                pk = c[:, 0] | (c[:, 1] << 2) | (c[:, 2] << 4) | (c[:, 3] << 6)
                f.write(pk.cpu().numpy().tobytes())
            f.write(struct.pack("<Q", 0))
            f.write(struct.pack("<Q", L))
            o += L
        f.write(struct.pack("<Q", int(np.sum(lens))))


def _hp_mask(f, min_run=6):
    """Per row of codes f (n, W): positions inside a run of >= min_run equal bases."""
    torch = _torch()
    n, W = f.shape
    eq = torch.zeros((n, W), dtype=torch.int32, device=f.device)
    eq[:, 1:] = (f[:, 1:] == f[:, :-1]).to(torch.int32)
    c = torch.cumsum(eq, 1)
    k = min_run - 1
    full = torch.zeros((n, W), dtype=torch.bool, device=f.device)
    if W > k:
        win = (c[:, k:] - c[:, :W - k]) == k
        for t in range(k + 1):
            full[:, t:W - k + t] |= win
    return full


def _apply_errors(frag, L, sub, indel, qmu, qsd, gen):
    """frag (n, W) codes, W > L. Returns (codes (n, L), quals (n, L)) after
    substitutions and indels (rates x5 inside homopolymers)."""
    torch = _torch()
    dev = frag.device
    n, W = frag.shape
    hp = _hp_mask(frag)
    rs = torch.where(hp, 5 * sub, sub)
    ri = torch.where(hp, 5 * indel, indel)
    subm = (torch.rand((n, W), generator=gen, device=dev) < rs) & (frag < 4)
    shift = torch.randint(1, 4, (n, W), generator=gen, device=dev, dtype=torch.uint8)
    out = torch.where(subm, (frag + shift) % 4, frag)
    q = torch.clamp(torch.round(torch.randn((n, W), generator=gen, device=dev) * qsd + qmu), 2, 41)
    ql = torch.clamp(torch.round(torch.randn((n, W), generator=gen, device=dev) * 4.0 + 12.0), 2, 41)
    q = torch.where(subm, ql, q).to(torch.uint8)
    ev = torch.rand((n, W), generator=gen, device=dev) < ri
    if not bool(ev.any()):
        return out[:, :L], q[:, :L]
    is_ins = ev & (torch.rand((n, W), generator=gen, device=dev) < 0.5)
    is_del = ev & ~is_ins
    # geometric(p = 2/3) lengths, capped at 8
    u = torch.rand((n, W), generator=gen, device=dev).clamp_min(1e-12)
    ln = torch.clamp(torch.floor(torch.log(u) / math.log(1.0 / 3.0)).to(torch.int32) + 1, 1, 8)
    cover = torch.zeros((n, W), dtype=torch.bool, device=dev)
    for k in range(8):
        sh = is_del & (ln > k)
        cover[:, k:] |= sh[:, :W - k]
    emit = torch.where(cover, 0, 1 + torch.where(is_ins, ln, 0)).to(torch.int32)
    cum = torch.cumsum(emit, 1)
    cum = cum.to(torch.int64)
    o = torch.arange(L, device=dev, dtype=torch.int64).expand(n, L).contiguous()
    p = torch.searchsorted(cum, o, right=True).clamp_max(W - 1)
    start = torch.gather(cum, 1, p) - torch.gather(emit, 1, p)
    k = o - start
    n_ins = torch.gather(emit, 1, p) - 1
    inserted = k < n_ins
    rnd = torch.randint(0, 4, (n, L), generator=gen, device=dev, dtype=torch.uint8)
    base = torch.where(inserted, rnd, torch.gather(out, 1, p))
    qual = torch.gather(q, 1, p)
    return base, qual


def _rc(codes):
    torch = _torch()
    r = torch.flip(codes, [1])
    return torch.where(r > 3, r, 3 - r)


def _pick_starts(n, span, starts_t, lens_t, gen, regions=None, region_frac=0.0):
    """Genome offsets of n fragments of span[i] bases inside one contig each,
    contigs drawn in proportion to their length; a region_frac share drawn
    uniformly inside the given (start, end) regions instead."""
    torch = _torch()
    dev = lens_t.device
    cum = torch.cumsum(lens_t, 0)
    u = torch.rand(n, generator=gen, device=dev, dtype=torch.float64)
    ci = torch.searchsorted(cum, (u * float(cum[-1])).to(torch.int64), right=True).clamp_max(len(lens_t) - 1)
    room = (lens_t[ci] - span - 1).clamp_min(1)
    s = (torch.rand(n, generator=gen, device=dev, dtype=torch.float64) * room.to(torch.float64)).to(torch.int64)
    gs = starts_t[ci] + s
    if regions and region_frac > 0:
        rs = torch.as_tensor([a for a, _ in regions], device=dev, dtype=torch.int64)
        rl = torch.as_tensor([b - a for a, b in regions], device=dev, dtype=torch.int64)
        pick = torch.rand(n, generator=gen, device=dev) < region_frac
        rc = torch.searchsorted(torch.cumsum(rl, 0),
                                (torch.rand(n, generator=gen, device=dev, dtype=torch.float64) *
                                 float(rl.sum())).to(torch.int64), right=True).clamp_max(len(rl) - 1)
        off = (torch.rand(n, generator=gen, device=dev, dtype=torch.float64) *
               (rl[rc] - span).clamp_min(1).to(torch.float64)).to(torch.int64)
        gs = torch.where(pick, rs[rc] + off, gs)
    return gs


def _pack_reads(codes, quals, lens):
    """(n, L) codes/quals and per-read lengths -> ASCII bytes, quals, offsets (numpy)."""
    torch = _torch()
    n, L = codes.shape
    mask = torch.arange(L, device=codes.device).expand(n, L) < lens[:, None]
    asc = torch.as_tensor(ASCII.copy(), device=codes.device)[codes.long()]
    b = asc[mask].cpu().numpy()
    q = quals[mask].cpu().numpy()
    offs = np.zeros(n + 1, np.uint64)
    offs[1:] = np.cumsum(lens.cpu().numpy().astype(np.uint64))
    return b, q, offs


def reads(seed: int, names, lens, codes, n: int, L: int, paired: bool = False, mean: float = 300.0,
          sd: float = 80.0, sub: float = 0.005, indel: float = 0.0005, qmu: float = 35.0, qsd: float = 4.0,
          trim=None, regions=None, region_frac: float = 0.0, device=None, chunk: int = 1 << 20, g_dev=None):
    """n single-end reads, or n FR pairs, of length L (see the module text).
    trim=(lo, hi): each read cut to a length drawn from U[lo, hi] (reads
    shorter than the draw are kept whole). Returns (bases, quals, offsets) or,
    for pairs, (b1, q1, o1, b2, q2, o2) as numpy arrays. g_dev: the genome
    already on the device (uint8 tensor), to share it between calls."""
    torch = _torch()
    dev = _dev(device)
    gen = _gen(dev, seed)
    g = g_dev if g_dev is not None else torch.as_tensor(codes).to(dev)
    lens_t = torch.as_tensor(np.asarray(lens, np.int64), device=dev)
    starts_t = torch.cumsum(lens_t, 0) - lens_t
    pad = 16
    W = L + pad
    ar = torch.arange(W, device=dev)
    outs = [[], [], [], [], [], []]
    done = 0
    while done < n:
        m = min(chunk, n - done)
        if paired:
            ins = torch.clamp(torch.round(torch.randn(m, generator=gen, device=dev, dtype=torch.float64) * sd + mean),
                              min=L + 10).to(torch.int64)
            span = ins + pad
        else:
            span = torch.full((m,), W, dtype=torch.int64, device=dev)
        gs = _pick_starts(m, span, starts_t, lens_t, gen, regions, region_frac)
        f1 = g[(gs[:, None] + ar[None, :]).clamp_max(len(g) - 1)]
        a, qa = _apply_errors(f1, L, sub, indel, qmu, qsd, gen)
        if paired:
            ge = gs + ins
            f2 = _rc(g[(ge[:, None] - W + ar[None, :]).clamp(0, len(g) - 1)])
            b, qb = _apply_errors(f2, L, sub, indel, qmu, qsd, gen)
            swap = (torch.rand(m, generator=gen, device=dev) < 0.5)[:, None]
            a, b = torch.where(swap, b, a), torch.where(swap, a, b)
            qa, qb = torch.where(swap, qb, qa), torch.where(swap, qa, qb)
            mates = ((a, qa), (b, qb))
        else:
            rev = (torch.rand(m, generator=gen, device=dev) < 0.5)[:, None]
            a = torch.where(rev, _rc(a), a)
            qa = torch.where(rev, torch.flip(qa, [1]), qa)
            mates = ((a, qa),)
        for k, (c, q) in enumerate(mates):
            if trim:
                ln = torch.randint(trim[0], trim[1] + 1, (m,), generator=gen, device=dev).clamp_max(L)
            else:
                ln = torch.full((m,), L, device=dev, dtype=torch.int64)
            bb, qq, oo = _pack_reads(c, q, ln)
            outs[3 * k].append(bb)
            outs[3 * k + 1].append(qq)
            outs[3 * k + 2].append(oo)
        done += m

    def cat(bs, qs, os_):
        o = [os_[0]]
        for x in os_[1:]:
            o.append(x[1:] + o[-1][-1])
        return np.concatenate(bs), np.concatenate(qs), np.concatenate(o)

    r1 = cat(outs[0], outs[1], outs[2])
    if not paired:
        return r1
    return r1 + cat(outs[3], outs[4], outs[5])
