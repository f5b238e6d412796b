"""Stage-level parity of seeding (K1) and clustering (K2) through the C ABI.

pbw_seed_batch is find_seed_hits (src/mapper/seeds.rs:91-151): every hit in
emission order (read position, contig, position, strand) and the bits of
every repeat_prob entry. pbw_cluster_batch is cluster_hits
(src/mapper/candidates.rs:30-78): the ordered candidate list well past the 20
that the mapper aligns (the ranker's input is the list before take(20)) and
the full count. Both are compared read by read with the oracle's twins
(orc_seed_read, orc_cluster_read) on repeat-family genomes, a many-contig
genome whose (contig, strand) group order decides ties, and a genome whose
reads overflow the per-read hit buffer.
"""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def _repeat_genome(tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(301, length=300_000, n_copies=30, copy_len=2000)
    prefix = str(tmp_path / "rep")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(302, contigs, n=400, L=150, sub=0.01, indel=0.001)
    s2, q2, _ = synth.reads_single(303, contigs, n=200, L=60, sub=0.02, indel=0.002)
    return prefix, seqs + s2, quals + q2


def _multi_contig_genome(tmp_path):
    from probebwa_gb300 import synth
    rng = np.random.default_rng(305)
    unit = synth.rand_codes(rng, 2500)
    contigs = []
    for c in range(16):
        g = synth.rand_codes(rng, 15_000)
        for _ in range(2):
            s = int(rng.integers(0, 15_000 - 2500))
            g[s:s + 2500] = synth.mutate_subs(rng, unit, 0.003)
        contigs.append((f"c{c}", g))
    prefix = str(tmp_path / "multi")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(306, contigs, n=300, L=120, sub=0.01, indel=0.001)
    for i in range(150):
        s = int(rng.integers(0, 2500 - 120))
        frag = unit[s:s + 120]
        if i % 2:
            frag = 3 - frag[::-1]
        seqs.append(synth.ASCII[frag].tobytes())
        quals.append(bytes(rng.integers(15, 41, size=120).astype(np.uint8)))
    return prefix, seqs, quals


def _overflow_genome(tmp_path):
    """1,500 near-identical copies of a 1 kbp unit: reads from the unit with
    one private change per 15-mer window hit the copies through their
    one-mismatch neighbours and produce far more than 4096 hits."""
    from probebwa_gb300 import synth
    rng = np.random.default_rng(307)
    unit = synth.rand_codes(rng, 1000)
    parts = []
    for _ in range(1500):
        parts.append(synth.mutate_subs(rng, unit, 0.003))
        parts.append(synth.rand_codes(rng, int(rng.integers(3, 40))))
    g = np.concatenate(parts)
    prefix = str(tmp_path / "ovf")
    synth.write_index(prefix, [("rep", g)])
    seqs, quals = [], []
    for i in range(24):
        s = int(rng.integers(0, 1000 - 150))
        frag = unit[s:s + 150].copy()
        frag[::16] = (frag[::16] + 1) % 4
        if i % 2:
            frag = 3 - frag[::-1]
        seqs.append(synth.ASCII[frag].tobytes())
        quals.append(bytes(rng.integers(20, 41, size=150).astype(np.uint8)))
    s2, q2, _ = synth.reads_single(308, [("rep", g)], n=60, L=150)
    return prefix, seqs + s2, quals + q2


def _wide_group_genome(tmp_path, n_contigs=200, L=100, copies=1):
    """n_contigs contigs, each with copies of a 1 kbp unit forward and as
    many reverse-complemented: a read of L bases from the unit hits
    2 * n_contigs (contig, strand) groups. With 200 contigs that is ~310
    groups after the bucket cap (the block-wide group order of reads over
    256 groups) and ~5,100-5,400 hits, over the 4096-hit buffer of 100-base
    reads (list mode)."""
    from probebwa_gb300 import synth
    rng = np.random.default_rng(311)
    unit = synth.rand_codes(rng, 1000)
    contigs = []
    for c in range(n_contigs):
        g = synth.rand_codes(rng, 4000 * copies)
        for j in range(copies):
            o = 4000 * j
            g[o + 500:o + 1500] = synth.mutate_subs(rng, unit, 0.002)
            g[o + 2500:o + 3500] = 3 - synth.mutate_subs(rng, unit, 0.002)[::-1]
        contigs.append((f"w{c}", g))
    prefix = str(tmp_path / "wide")
    synth.write_index(prefix, contigs)
    seqs, quals = [], []
    for i in range(12):
        s = int(rng.integers(0, 1000 - L))
        frag = unit[s:s + L].copy()
        if i % 2:
            frag = 3 - frag[::-1]
        seqs.append(synth.ASCII[frag].tobytes())
        quals.append(bytes(rng.integers(20, 41, size=L).astype(np.uint8)))
    return prefix, seqs, quals


def _edge_reads(seqs, quals):
    """Reads the seeding loop treats specially: empty, shorter than k,
    exactly k, N runs and IUPAC letters inside windows, lower case."""
    base = seqs[0]
    extra = [b"", b"ACGT", base[:14], base[:15], base[:60].lower(), base[:40] + b"NNNNN" + base[45:100],
             base[:30] + b"RYKM" + base[34:90], b"N" * 50]
    return seqs + extra, quals + [bytes([30] * len(x)) for x in extra]


def _check_seeds(P, oracle, prefix, seqs, quals, chunk_reads=0):
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix, chunk_reads=chunk_reads) as m:
        hit_off, hits, rpos, win_off, rep = m.seed_batch(R)
    om = oracle.Mapper(prefix)
    n_hits = 0
    for i, (s, q) in enumerate(zip(seqs, quals)):
        e_rp, e_c, e_p, e_s, e_rep = om.seed_read(s, q, cap=1 << 20)
        a, b = int(hit_off[i]), int(hit_off[i + 1])
        g = hits[a:b]
        got = np.stack([rpos[a:b].astype(np.uint64), (g >> np.uint64(40)) & np.uint64((1 << 23) - 1),
                        g & np.uint64((1 << 40) - 1), g >> np.uint64(63)], axis=1)
        exp = np.stack([e_rp, e_c.astype(np.uint64), e_p, e_s.astype(np.uint64)], axis=1)
        assert got.shape == exp.shape, f"read {i}: {b - a} hits, oracle {len(e_rp)}"
        assert np.array_equal(got, exp), f"read {i}: first differing hit {np.nonzero((got != exp).any(1))[0][:3]}"
        wa, wb = int(win_off[i]), int(win_off[i + 1])
        assert np.array_equal(rep[wa:wb].view(np.uint64), e_rep.view(np.uint64)), f"read {i}: repeat_prob bits"
        n_hits += b - a
    om.close()
    return hit_off, n_hits


def _check_clusters(P, oracle, prefix, seqs, quals, group_width=16, max_per_read=64, chunk_reads=0):
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix, group_width=group_width, chunk_reads=chunk_reads) as m:
        nc, tc, cc, cp, cs, sc = m.cluster_batch(R, max_per_read=max_per_read)
    om = oracle.Mapper(prefix, group_width=group_width)
    past20 = 0
    for i, (s, q) in enumerate(zip(seqs, quals)):
        e_c, e_p, e_s, e_sc = om.cluster_read(s, q, cap=1 << 20)
        assert tc[i] == len(e_c), f"read {i}: {tc[i]} candidates, oracle {len(e_c)}"
        k = min(len(e_c), max_per_read)
        assert nc[i] == k
        got = (cc[i, :k].tolist(), cp[i, :k].tolist(), cs[i, :k].tolist(), sc[i, :k].tolist())
        exp = (e_c[:k].tolist(), e_p[:k].tolist(), e_s[:k].tolist(), e_sc[:k].tolist())
        assert got == exp, f"read {i} (group width {group_width}): ordered candidate list differs"
        past20 += max(0, k - 20)
    om.close()
    return tc, past20


def test_seed_hits_repeat_families(P, oracle, tmp_path):
    prefix, seqs, quals = _repeat_genome(tmp_path)
    seqs, quals = _edge_reads(seqs, quals)
    hit_off, n = _check_seeds(P, oracle, prefix, seqs, quals)
    assert n > 10 * len(seqs)


def test_seed_hits_chunked(P, oracle, tmp_path):
    """Chunk boundaries (chunk_reads = 97) change nothing."""
    prefix, seqs, quals = _repeat_genome(tmp_path)
    _check_seeds(P, oracle, prefix, seqs[:300], quals[:300], chunk_reads=97)


def test_seed_hits_over_capacity(P, oracle, tmp_path):
    prefix, seqs, quals = _overflow_genome(tmp_path)
    hit_off, n = _check_seeds(P, oracle, prefix, seqs, quals)
    per_read = np.diff(hit_off.astype(np.int64))
    assert (per_read > 4096).sum() >= 10, "the case must overflow the per-read buffer"


@pytest.mark.parametrize("group_width", [16, 8])
def test_candidates_many_contigs(P, oracle, tmp_path, group_width):
    prefix, seqs, quals = _multi_contig_genome(tmp_path)
    seqs, quals = _edge_reads(seqs, quals)
    tc, past20 = _check_clusters(P, oracle, prefix, seqs, quals, group_width=group_width)
    assert (tc > 20).sum() > 20 and past20 > 0, "the case must have candidates past take(20)"


def test_candidates_repeat_families(P, oracle, tmp_path):
    prefix, seqs, quals = _repeat_genome(tmp_path)
    _check_clusters(P, oracle, prefix, seqs, quals, max_per_read=40, chunk_reads=211)


def test_candidates_over_capacity(P, oracle, tmp_path):
    prefix, seqs, quals = _overflow_genome(tmp_path)
    tc, _ = _check_clusters(P, oracle, prefix, seqs, quals, max_per_read=256)
    assert tc.max() > 20


def test_overflow_pool_in_slices(P, oracle, tmp_path):
    """Over-capacity reads are seeded and clustered one pool slice at a time.
    With the slice lowered to 64 K hits the reads of this case need several
    slices; seeds, candidates and whole records must not change."""
    from gpu_helpers import compare_records
    prefix, seqs, quals = _overflow_genome(tmp_path)
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix) as m:
        m.set_tuning(ovf_slice_hits=1 << 16)
        hit_off, hits, rpos, win_off, rep = m.seed_batch(R)
        over = np.diff(hit_off.astype(np.int64))
        assert over[over > 4096].sum() > 3 * (1 << 16), "the case must span several slices"
        nc, tc, cc, cp, cs, sc = m.cluster_batch(R, max_per_read=64)
        got = m.map_single(R)
    om = oracle.Mapper(prefix)
    for i, (s, q) in enumerate(zip(seqs, quals)):
        e_rp, e_c, e_p, e_s, e_rep = om.seed_read(s, q, cap=1 << 20)
        a, b = int(hit_off[i]), int(hit_off[i + 1])
        assert np.array_equal(rpos[a:b].astype(np.uint64), e_rp), i
        assert np.array_equal(hits[a:b] & np.uint64((1 << 40) - 1), e_p), i
        e_c2, e_p2, e_s2, e_sc2 = om.cluster_read(s, q, cap=1 << 20)
        k = min(len(e_c2), 64)
        assert tc[i] == len(e_c2) and cp[i, :k].tolist() == e_p2[:k].tolist(), i
    exp = om.map_single(oracle.Reads(R.bases, R.quals, R.offsets, R.ids))
    compare_records(P, oracle, got, exp, "sliced overflow pool")


@pytest.mark.parametrize("group_width", [16, 8])
def test_candidates_over_256_groups(P, oracle, tmp_path, group_width):
    prefix, seqs, quals = _wide_group_genome(tmp_path)
    tc, _ = _check_clusters(P, oracle, prefix, seqs, quals, group_width=group_width, max_per_read=256)
    assert tc.min() > 256, "every read must have clusters in more than 256 groups"


@pytest.mark.parametrize("n_contigs,L,copies,group_width", [(22, 100, 1, 16), (28, 100, 1, 8), (28, 170, 4, 16),
                                                            (26, 170, 4, 8)])
def test_candidates_near_register_replay_limit(P, oracle, tmp_path, n_contigs, L, copies, group_width):
    """44 to 56 (contig, strand) groups per read, the top of the one-warp
    register replay of the group order (up to 56 groups: a 64-bucket table).
    100-base reads (~730-990 hits) take the shared-memory tiers, where the
    groups are collected before the bins; 170-base reads of the 4-copy
    genome (~6,200-7,000 hits) take the global-slab tier, whose group table
    then sits in shared memory."""
    prefix, seqs, quals = _wide_group_genome(tmp_path, n_contigs, L, copies)
    tc, _ = _check_clusters(P, oracle, prefix, seqs, quals, group_width=group_width, max_per_read=256)
    assert tc.min() >= 2 * n_contigs, "every read must have clusters in all of its groups"
    with P.Mapper(prefix) as m:
        per = np.diff(m.seed_batch(P.Reads.from_lists(seqs, quals))[0].astype(np.int64))
    lo, hi = (0, 4096) if L == 100 else (4096, 16384)
    assert ((per > lo) & (per <= hi)).all(), (per.min(), per.max())


def test_cluster_block_sizes_agree(P, tmp_path):
    """The K2 block size of the 4096-hit and slab tiers (tuned, or forced with
    k2_threads) changes no candidate and no record. 200-base reads of a genome
    with 250 copies of a 2 kbp unit fill both tiers."""
    from probebwa_gb300 import synth
    contigs = synth.genome_single(301, length=700_000, n_copies=250, copy_len=2000)
    prefix = str(tmp_path / "rep250")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(302, contigs, n=200, L=200, sub=0.01, indel=0.001)
    R = P.Reads.from_lists(seqs, quals)
    outs = []
    for k2 in ((1024, 1024), (512, 512), (256, 256), (0, 0)):
        with P.Mapper(prefix) as m:
            m.set_tuning(k2_threads=k2)
            c = m.cluster_batch(R, max_per_read=64)
            rec = m.map_single(R)
            t = m.tuning()
        outs.append((c, rec))
        if k2 == (0, 0):
            assert all(x in (256, 512, 1024) for x in t["k2_chosen"]), t
    with P.Mapper(prefix) as m:
        hit_off = m.seed_batch(R)[0]
    per = np.diff(hit_off.astype(np.int64))
    assert ((per > 2048) & (per <= 4096)).any() and ((per > 4096) & (per <= 16384)).any(), "both tiers must be used"
    c0, r0 = outs[0]
    for c, r in outs[1:]:
        for a, b in zip(c, c0):
            assert np.array_equal(a, b)
        for k in ("contig", "pos", "mapq", "flag", "as_score", "nm", "cigar_off"):
            assert np.array_equal(r[k], r0[k]), k
