"""Single-end mapping on the GPU through the C ABI, against the oracle and
the reference's own known answers."""
from __future__ import annotations

import numpy as np
import pytest

import kat_cases as K
from gpu_helpers import compare_records, to_oracle_reads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def _index(tmp_path, name, contigs_str):
    from probebwa_gb300 import synth
    prefix = str(tmp_path / name)
    synth.write_index(prefix, synth.contigs_from_strings(contigs_str))
    return prefix


def _parity(P, oracle, prefix, R, **opts):
    with P.Mapper(prefix, **opts) as m:
        got = m.map_single(R)
    om = oracle.Mapper(prefix, **{k: v for k, v in opts.items() if k in ("group_width", "max_indel_len")})
    exp = om.map_single(to_oracle_reads(oracle, R))
    om.close()
    return got, exp


def test_kat_forward_reverse(P, oracle, tmp_path):
    contigs, reads, expect = K.fwd_rev()
    prefix = _index(tmp_path, "g", contigs)
    R = P.Reads.from_lists([s for _, s in reads], ids=[i for i, _ in reads])
    with P.Mapper(prefix) as m:
        rec = m.map_single(R)
    cig = P.cigar_strings(rec)
    for i, e in enumerate(expect):
        assert rec["pos"][i] == e["pos"] and cig[i] == e["cigar"] and rec["mapq"][i] == e["mapq"]
        assert bool(rec["flag"][i] & 0x10) == e["rev"]


def test_kat_mismatch_deletion_unmapped(P, oracle, tmp_path):
    contigs, reads = K.mismatch_del_garbage()
    prefix = _index(tmp_path, "g", contigs)
    R = P.Reads.from_lists([s for _, s in reads], ids=[i for i, _ in reads])
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "mismatch/del/garbage")
    assert got["pos"][0] == 41 and got["mapq"][0] == 80
    assert got["pos"][2] == 0 and P.cigar_strings(got)[2] == "40S"


def test_kat_large_deletion_and_large_contig(P, oracle, tmp_path):
    contigs, reads = K.large_deletion()
    prefix = _index(tmp_path, "g1", contigs)
    R = P.Reads.from_lists([s for _, s in reads])
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "large deletion")
    assert got["pos"][0] == 101 and "25D" in P.cigar_strings(got)[0] or \
        sum(int(x[:-1]) for x in __import__("re").findall(r"\d+D", P.cigar_strings(got)[0])) == 25
    contigs, reads = K.large_contig()
    prefix = _index(tmp_path, "g2", contigs)
    R = P.Reads.from_lists([s for _, s in reads])
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "large contig")
    assert got["pos"][0] == 70_001 and got["mapq"][0] == 99


def test_kat_n_run_and_accuracy(P, oracle, tmp_path):
    contigs, reads = K.n_run()
    prefix = _index(tmp_path, "g1", contigs)
    R = P.Reads.from_lists([s for _, s in reads], ids=[i for i, _ in reads])
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "n-run")
    assert got["pos"][0] == 106 and got["pos"][1] == 151 and got["mapq"][1] == 80
    contigs, reads, truth = K.synthetic_accuracy()
    prefix = _index(tmp_path, "g2", contigs)
    R = P.Reads.from_lists([s for _, s in reads])
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "synthetic accuracy")
    ok = sum(1 for i, (p, rev) in enumerate(truth)
             if got["contig"][i] == 0 and bool(got["flag"][i] & 0x10) == rev and abs(int(got["pos"][i]) - p) <= 2)
    assert ok / len(truth) >= 0.95


@pytest.mark.parametrize("seed,L,sub,indel", [(1, 120, 0.01, 0.001), (2, 60, 0.02, 0.002), (3, 150, 0.005, 0.0005),
                                              (4, 250, 0.03, 0.003)])
def test_parity_synthetic_repeats(P, oracle, tmp_path, seed, L, sub, indel):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(100 + seed, length=200_000, n_copies=20, copy_len=2000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(200 + seed, contigs, n=1500, L=L, sub=sub, indel=indel)
    R = P.Reads.from_lists(seqs, quals)
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, f"synthetic seed={seed} L={L}")
    assert (got["pos"] > 0).mean() > 0.8


def test_parity_multi_contig_group_widths(P, oracle, tmp_path):
    """Many contigs make the (contig, strand) group order matter for ties."""
    from probebwa_gb300 import synth
    rng = np.random.default_rng(5)
    unit = synth.rand_codes(rng, 3000)
    contigs = []
    for c in range(12):
        g = synth.rand_codes(rng, 20_000)
        for _ in range(3):
            s = int(rng.integers(0, 20_000 - 3000))
            g[s:s + 3000] = synth.mutate_subs(rng, unit, 0.002)
        contigs.append((f"c{c}", g))
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(9, contigs, n=1500, L=100, sub=0.01, indel=0.001)
    # plus reads drawn straight from the repeat unit: exact ties across contigs
    for i in range(300):
        s = int(rng.integers(0, 3000 - 100))
        frag = unit[s:s + 100]
        if i % 2:
            frag = (3 - frag[::-1])
        seqs.append(synth.ASCII[frag].tobytes())
        quals.append(bytes([35] * 100))
    R = P.Reads.from_lists(seqs, quals)
    for gw in (16, 8):
        got, exp = _parity(P, oracle, prefix, R, group_width=gw)
        compare_records(P, oracle, got, exp, f"group_width={gw}")


def test_edge_case_reads(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(31, length=30_000, n_copies=3, copy_len=500)
    g = contigs[0][1]
    s = lambda a, b: synth.ASCII[g[a:b]].tobytes()
    seqs = [b"", b"ACGT", s(100, 114), s(100, 115), s(0, 80), s(30_000 - 90, 30_000),
            s(5000, 5100).lower(), s(6000, 6050) + b"NNNNN" + s(6055, 6100),
            s(7000, 7040) + b"RYKM" + s(7044, 7100), b"N" * 60, s(8000, 8000 + 1024),
            bytes(synth.ASCII[(3 - g[9000:9120])[::-1]]), s(20_000, 20_200)]
    quals = [bytes(np.random.default_rng(i).integers(2, 42, size=len(x)).astype(np.uint8)) for i, x in enumerate(seqs)]
    quals[3] = bytes([0] * len(seqs[3]))
    R = P.Reads.from_lists(seqs, quals)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    got, exp = _parity(P, oracle, prefix, R)
    compare_records(P, oracle, got, exp, "edge cases")


def test_chunking_is_invisible(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(41, length=100_000, n_copies=10, copy_len=1000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(42, contigs, n=1000, L=100)
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix, chunk_reads=97) as m:
        a = m.map_single(R)
    with P.Mapper(prefix) as m:
        b = m.map_single(R)
    compare_records(P, oracle, a, b, "chunked vs whole")


def test_sam_text_matches_oracle(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(51, length=40_000, n_copies=4, copy_len=500)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(52, contigs, n=300, L=90)
    seqs.append(b"")
    quals.append(b"")
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix) as m:
        got = m.map_single(R)
        m.write_sam(str(tmp_path / "gpu.sam"), R, got)
    om = oracle.Mapper(prefix)
    exp = om.map_single(to_oracle_reads(oracle, R))
    om.write_sam(str(tmp_path / "cpu.sam"), to_oracle_reads(oracle, R), exp)
    a = open(tmp_path / "gpu.sam", "rb").read()
    b = open(tmp_path / "cpu.sam", "rb").read()
    assert a == b


def test_reads_over_seed_hit_capacity(P, oracle, tmp_path):
    """Reads whose one-mismatch neighbours hit a high-copy repeat family
    produce far more than 4096 seed hits; they go through the overflow pool
    (list-mode seeding and global-scratch clustering) and must still match."""
    from probebwa_gb300 import synth
    rng = np.random.default_rng(77)
    unit = synth.rand_codes(rng, 1000)
    parts = []
    for _ in range(1500):
        parts.append(synth.mutate_subs(rng, unit, 0.003))
        parts.append(synth.rand_codes(rng, int(rng.integers(3, 40))))
    g = np.concatenate(parts)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, [("rep", g)])
    seqs, quals = [], []
    for i in range(40):
        s = int(rng.integers(0, 1000 - 150))
        frag = unit[s:s + 150].copy()
        frag[::16] = (frag[::16] + 1) % 4  # one private change in every 15-mer window
        if i % 2:
            frag = (3 - frag[::-1])
        seqs.append(synth.ASCII[frag].tobytes())
        quals.append(bytes(rng.integers(20, 41, size=150).astype(np.uint8)))
    seqs2, quals2, _ = synth.reads_single(78, [("rep", g)], n=200, L=150)
    R = P.Reads.from_lists(seqs + seqs2, quals + quals2)
    with P.Mapper(prefix) as m:
        got = m.map_single(R)
        st = m.stats()
    om = oracle.Mapper(prefix)
    exp = om.map_single(to_oracle_reads(oracle, R))
    compare_records(P, oracle, got, exp, "over-capacity reads")
    assert st["seed_hits"] > 4096 * 5
