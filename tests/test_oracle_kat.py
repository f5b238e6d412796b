"""Pins the CPU oracle against the reference's own known-answer tests.

Every assertion here restates one in the reference's test suite
(tests/mapping.rs, tests/integration.rs, tests/cli.rs and the unit tests in
src/index/hashtable.rs), run through the oracle instead of the Rust crate.
"""
from __future__ import annotations

import os
import re

import pytest

import kat_cases as K
import sthash_py as SH

# The reference checkout, when present, supplies the E. coli literals of its
# DP known-answer test at run time (they are not copied into this repository).
REF_INTEGRATION = os.path.join(os.environ.get("PBW_REFERENCE_DIR", os.path.join(os.sep, "root", "reference")),
                               "tests", "integration.rs")


def _index(oracle, tmp_path, contigs, name="ref", **kw):
    prefix = str(tmp_path / name)
    oracle.build_index(prefix, contigs, **kw)
    return prefix


def _map(oracle, prefix, reads, quals=None):
    R = oracle.Reads.from_lists([s for _, s in reads], quals, [i for i, _ in reads])
    m = oracle.Mapper(prefix)
    recs = m.map_single(R)
    cig = oracle.cigar_strings(recs)
    m.close()
    return recs, cig


def _cigar_totals(c):
    tot = {"M": 0, "I": 0, "D": 0}
    for n, op in re.findall(r"(\d+)([MIDSH])", c):
        if op in tot:
            tot[op] += int(n)
    return tot["M"], tot["D"], tot["I"]


def test_forward_and_reverse_strand(oracle, tmp_path):
    contigs, reads, expect = K.fwd_rev()
    prefix = _index(oracle, tmp_path, contigs)
    recs, cig = _map(oracle, prefix, reads)
    for i, e in enumerate(expect):
        assert recs["contig"][i] == 0
        assert recs["pos"][i] == e["pos"]
        assert bool(recs["flag"][i] & 0x10) == e["rev"]
        assert cig[i] == e["cigar"]
        assert recs["mapq"][i] == e["mapq"]


def test_mismatch_deletion_and_unmapped(oracle, tmp_path):
    contigs, reads = K.mismatch_del_garbage()
    prefix = _index(oracle, tmp_path, contigs)
    recs, cig = _map(oracle, prefix, reads)
    assert recs["pos"][0] == 41 and cig[0] == "40M" and recs["mapq"][0] == 80
    assert recs["pos"][1] == 41
    assert _cigar_totals(cig[1]) == (38, 2, 0)
    assert recs["mapq"][1] > 0
    assert recs["pos"][2] == 0 and recs["mapq"][2] == 0
    assert cig[2] == "40S" and recs["contig"][2] == -1


def test_large_deletion_is_found(oracle, tmp_path):
    contigs, reads = K.large_deletion()
    prefix = _index(oracle, tmp_path, contigs)
    recs, cig = _map(oracle, prefix, reads)
    assert recs["pos"][0] == 101
    assert _cigar_totals(cig[0])[1] == 25


def test_paired_end_proper_and_improper(oracle, tmp_path):
    contigs, fr, ff = K.paired_fr_ff()
    prefix = _index(oracle, tmp_path, contigs)
    m = oracle.Mapper(prefix)
    r1 = oracle.Reads.from_lists([fr[0]], ids=["pair1"])
    r2 = oracle.Reads.from_lists([fr[1]], ids=["pair1"])
    o1, o2, _ = m.map_paired(r1, r2)
    assert o1["flag"][0] & 0x40 and o2["flag"][0] & 0x80
    assert o1["flag"][0] & 0x2 and o2["flag"][0] & 0x2
    assert not (o1["flag"][0] & 0x10) and (o2["flag"][0] & 0x10)
    assert o1["tlen"][0] == 200 and o2["tlen"][0] == -200
    r1 = oracle.Reads.from_lists([ff[0]], ids=["ffpair"])
    r2 = oracle.Reads.from_lists([ff[1]], ids=["ffpair"])
    o1, o2, _ = m.map_paired(r1, r2)
    assert not (o1["flag"][0] & 0x2) and not (o2["flag"][0] & 0x2)


def test_large_contig_positions(oracle, tmp_path):
    contigs, reads = K.large_contig()
    prefix = _index(oracle, tmp_path, contigs)
    recs, _ = _map(oracle, prefix, reads)
    assert recs["contig"][0] == 0
    assert recs["pos"][0] == 70_001
    assert recs["mapq"][0] == 99


def test_mate_rescue(oracle, tmp_path):
    contigs, m1, m2 = K.mate_rescue()
    prefix = _index(oracle, tmp_path, contigs)
    recs, _ = _map(oracle, prefix, [("pair1", m2)])
    assert recs["pos"][0] == 0
    m = oracle.Mapper(prefix)
    o1, o2, _ = m.map_paired(oracle.Reads.from_lists([m1]), oracle.Reads.from_lists([m2]))
    assert o1["pos"][0] == 41
    assert o2["pos"][0] != 0 and o2["contig"][0] == 0
    assert o2["flag"][0] & 0x10
    assert abs(int(o2["pos"][0]) - 201) <= 5


def test_n_run_round_trip(oracle, tmp_path):
    contigs, reads = K.n_run()
    prefix = _index(oracle, tmp_path, contigs)
    R = oracle.Reads.from_lists([s for _, s in reads], ids=[i for i, _ in reads])
    m = oracle.Mapper(prefix)
    recs = m.map_single(R)
    assert recs["pos"][0] == 106
    # SEQ of the in-gap read starts with 15 N (aligned orientation)
    sam = tmp_path / "o.sam"
    m.write_sam(str(sam), R, recs)
    lines = [l.split("\t") for l in open(sam).read().splitlines() if not l.startswith("@")]
    seq0 = lines[0][9] if not (recs["flag"][0] & 0x10) else lines[0][9]
    assert seq0[:15] == "N" * 15
    assert recs["pos"][1] == 151 and recs["mapq"][1] == 80


def test_synthetic_scale_accuracy(oracle, tmp_path):
    contigs, reads, truth = K.synthetic_accuracy()
    prefix = _index(oracle, tmp_path, contigs)
    recs, _ = _map(oracle, prefix, reads)
    ok = 0
    for i, (p, rev) in enumerate(truth):
        if recs["contig"][i] == 0 and bool(recs["flag"][i] & 0x10) == rev and abs(int(recs["pos"][i]) - p) <= 2:
            ok += 1
    assert ok / len(truth) >= 0.95


def test_paired_disambiguates_repeat_copy(oracle, tmp_path):
    contigs, (r1, q1), (r2, q2), true_pos, decoy_pos = K.repeat_disambiguation()
    prefix = _index(oracle, tmp_path, contigs)
    m = oracle.Mapper(prefix)
    alone = m.map_single(oracle.Reads.from_lists([r2], [q2]))
    assert alone["pos"][0] == decoy_pos + 1
    o1, o2, _ = m.map_paired(oracle.Reads.from_lists([r1], [q1]), oracle.Reads.from_lists([r2], [q2]))
    assert o1["pos"][0] == 1
    assert o2["pos"][0] == true_pos + 1
    assert o2["flag"][0] & 0x10
    assert (o1["flag"][0] & 0x2) and (o2["flag"][0] & 0x2)
    assert o2["mapq"][0] > 0


def test_adapter_strip(oracle, tmp_path):
    contigs, read, adapter = K.adapter_strip()
    prefix = _index(oracle, tmp_path, contigs)
    fq = tmp_path / "r.fq"
    fq.write_text(f"@r1\n{read}\n+\n{'I' * len(read)}\n")
    R = oracle.parse_reads(str(fq), adapter=adapter)
    m = oracle.Mapper(prefix)
    recs = m.map_single(R)
    assert recs["pos"][0] == 41
    assert oracle.cigar_strings(recs)[0] == "40M"
    assert R.n == 1 and len(R.seq(0)) == 40


def test_fastq_empty_record_does_not_desync(oracle, tmp_path):
    p = tmp_path / "e.fq"
    p.write_text("@empty\n\n+\n\n@normal\nACGT\n+\nIIII\n")
    R = oracle.parse_reads(str(p))
    assert R.ids == ["empty", "normal"]
    assert R.seq(0) == b"" and R.seq(1) == b"ACGT"
    assert list(R.qual(1)) == [40, 40, 40, 40]


def test_fasta_multi_record(oracle, tmp_path):
    p = tmp_path / "m.fa"
    p.write_text(">r1\nACGT\n>r2\nTTTT\n>r3\nGGGG\n>r4\nCCCC\n")
    R = oracle.parse_reads(str(p), fasta=True)
    assert R.ids == ["r1", "r2", "r3", "r4"]
    g = tmp_path / "g.fa"
    g.write_text(">c1\nAAAA\n>c2\nCCCC\n>c3\nGGGG\n>c4\nTTTT\n")
    oracle.build_genome_from_fasta(str(tmp_path / "genome"), [str(g)])
    idx = SH.read_stidx(str(tmp_path / "genome.stidx"))
    assert [c["name"] for c in idx["contigs"]] == ["c1", "c2", "c3", "c4"]


def test_pack_unpack_position():
    # tests/integration.rs:43-64 restated on the packing formula the files use
    def pack(c, p, rev):
        return (int(rev) << 63) | ((c & ((1 << 23) - 1)) << 40) | (p & ((1 << 40) - 1))

    for c, p, rev in [(5, 1234, False), (5, 1234, True), (42, 200_000_000, False)]:
        assert SH.unpack(pack(c, p, rev)) == (c, p, rev)


def test_hash_kmer_contract():
    # tests/integration.rs:31-40
    assert SH.hash_kmer("ACGTACGTACGTACG") == SH.hash_kmer("ACGTACGTACGTACG")
    assert SH.hash_kmer("ACGTACGTACGTACG") != SH.hash_kmer("TTTTTTTTTTTTTTT")


def test_n_windows_are_not_indexed(oracle, tmp_path):
    # src/index/hashtable.rs:336-391 (stride 1)
    seq = "A" * 20 + "N" * 20 + "C" * 20
    prefix = _index(oracle, tmp_path, [("c1", seq)], stride=1)
    ht = SH.read_sthash(prefix + ".sthash")
    for p in ht["positions"]:
        c, pos, rev = SH.unpack(int(p))
        if not rev and 6 <= pos < 40:
            assert pos + 15 <= 20 or pos >= 40
    allA = SH.bucket(ht, "A" * 15)
    assert any(SH.unpack(p)[1] == 0 and not SH.unpack(p)[2] for p in allA)
    for p in allA:
        c, pos, rev = SH.unpack(p)
        if not rev:
            assert pos + 15 <= 20 or pos >= 40


def test_max_count_caps_repetitive_kmer(oracle, tmp_path):
    # src/index/hashtable.rs:411-437
    unit = "ACGTACGTACGTACG"
    prefix = _index(oracle, tmp_path, [("c1", unit * 50)], stride=1, max_count=5)
    ht = SH.read_sthash(prefix + ".sthash")
    assert len(SH.bucket(ht, unit)) == 5


def _integration_literal(name):
    src = open(REF_INTEGRATION).read()
    m = re.search(r"const %s: &\[u8\] = b\"([ACGTN]+)\";" % name, src)
    return m.group(1).encode()


@pytest.mark.skipif(not os.path.exists(REF_INTEGRATION), reason="reference sources not present")
def test_divergent_region_dp_kat(oracle):
    # tests/integration.rs:131-153, literals read from the reference at run time
    window = _integration_literal("WINDOW")
    read = _integration_literal("READ")
    score, cig, off = oracle.align(read, bytes([30] * len(read)), window, 513, len(window))
    assert off == 513
    assert "I" not in cig and "D" not in cig


def test_aligner_edge_cases(oracle):
    # smith_waterman.rs:166-168: empty inputs return a soft clip
    assert oracle.align(b"", b"", b"ACGT", 0, 30) == (0, "0S", 0)
    assert oracle.align(b"ACGT", b"\x1e" * 4, b"", 0, 30) == (0, "4S", 0)
    # exact match inside a padded window
    s, c, o = oracle.align(b"ACGTTGCAAC", b"\x1e" * 10, b"GGGGGACGTTGCAACGGGG", 5, 30)
    assert (c, o) == ("10M", 5) and s == 200
