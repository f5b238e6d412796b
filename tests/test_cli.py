"""The `probebwa` command line (probebwa_gb300/cli) and the device SAM
writer / coordinate sort behind it, against the oracle's restatement of
src/main.rs and src/io/sam.rs.

CPU tests pin the oracle's command line against the reference's own CLI tests
(tests/cli.rs) and check that both command lines reject the same bad
arguments with the same exit status. GPU tests compare the SAM bytes of the
two command lines, run with the same argv, and the device formatter and sort
against the oracle on records built to hit every formatting branch."""
from __future__ import annotations

import os
import subprocess

import numpy as np
import pytest

import kat_cases as K


def _fastq(path, recs, qual_char="I"):
    with open(path, "w") as f:
        for i, s in recs:
            f.write(f"@{i}\n{s}\n+\n{qual_char * len(s)}\n")
    return str(path)


def _run(exe, args, **kw):
    """Runs a command line with argv[0] = "probebwa" (the @PG CL: line echoes argv)."""
    return subprocess.run(["probebwa", *args], executable=exe, capture_output=True, timeout=600, **kw)


@pytest.fixture(scope="module")
def clis(oracle):
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import native_build
    return native_build.CLI, oracle.CLI_PATH


def _index(oracle, tmp_path, contigs, name="ref"):
    prefix = str(tmp_path / name)
    oracle.build_index(prefix, contigs)
    return prefix


# ---- the oracle's command line against tests/cli.rs ----

def test_oracle_cli_labelfilter(oracle, tmp_path, clis):
    """test_labelfilter_restricts_output_to_matching_read_ids (tests/cli.rs:81-110)."""
    g = K.Xorshift64(100).gen_seq(400)
    prefix = _index(oracle, tmp_path, [("chr1", g)])
    fq = _fastq(tmp_path / "reads.fq", [("keep_1", g[40:80]), ("drop_1", g[200:240])])
    r = _run(clis[1], ["map", "--genome", prefix, "--hash", prefix, "-M", fq, "--labelfilter", "keep_"])
    assert r.returncode == 0, r.stderr
    lines = r.stdout.decode().splitlines()
    assert any(ln.startswith("keep_1\t") for ln in lines)
    assert not any(ln.startswith("drop_1\t") for ln in lines)


def test_oracle_cli_adapter_strip(oracle, tmp_path, clis):
    """test_adapter_strip_trims_3prime_readthrough (tests/cli.rs:112-146)."""
    contigs, read, adapter = K.adapter_strip()
    prefix = _index(oracle, tmp_path, contigs)
    fq = _fastq(tmp_path / "reads.fq", [("r1", read)])
    r = _run(clis[1], ["map", "--genome", prefix, "--hash", prefix, "-M", fq, "--adapter-strip", adapter])
    assert r.returncode == 0, r.stderr
    line = next(ln for ln in r.stdout.decode().splitlines() if ln.startswith("r1\t"))
    f = line.split("\t")
    assert f[3] == "41" and f[5] == "40M" and len(f[9]) == 40


def test_oracle_cli_header_and_pairs(oracle, tmp_path, clis):
    """Header lines of format_sam_records (sam.rs:92-104) with a read group,
    and mates interleaved in pair order (lib.rs:171-181)."""
    g = K.Xorshift64(99).gen_seq(400)
    prefix = _index(oracle, tmp_path, [("chr1", g)])
    fq1 = _fastq(tmp_path / "r1.fq", [("p1/1", g[40:90]), ("p2/1", g[100:150])])
    fq2 = _fastq(tmp_path / "r2.fq", [("p1/2", K.revcomp(g[190:240])), ("p2/2", K.revcomp(g[250:300]))])
    args = ["map", "-g", prefix, "-h", prefix, "--readgroup", "ID:rg1,SM:s1", "-M", fq1, fq2]
    r = _run(clis[1], args)
    assert r.returncode == 0, r.stderr
    lines = r.stdout.decode().splitlines()
    assert lines[0] == "@HD\tVN:1.6\tSO:unsorted"
    assert lines[1] == "@SQ\tSN:chr1\tLN:400"
    assert lines[2] == "@PG\tID:probebwa\tPN:probebwa\tVN:0.1.0\tCL:probebwa " + " ".join(args)
    assert lines[3] == "@RG\tID:rg1\tSM:s1"
    names = [ln.split("\t")[0] for ln in lines[4:]]
    assert names == ["p1", "p1", "p2", "p2"]
    flags = [int(ln.split("\t")[1]) for ln in lines[4:]]
    assert [f & 0xC0 for f in flags] == [0x40, 0x80, 0x40, 0x80]
    assert all(ln.endswith("\tRG:Z:rg1") for ln in lines[4:])


# ---- argument handling: both command lines agree (no device needed) ----

BAD_ARGS = [
    ([], 2),
    (["align"], 2),
    (["map", "-g", "x"], 2),
    (["map", "--hash", "x"], 2),
    (["map", "-g", "x", "-h", "x", "--bogus"], 2),
    (["map", "-g", "x", "-g", "y", "-h", "x"], 2),
    (["map", "-g", "x", "-h", "x", "--phred64", "--phred64"], 2),
    (["map", "-g", "x", "-h", "x", "--phred64=true"], 2),
    (["map", "-g", "x", "-h", "x", "-s", "abc"], 2),
    (["map", "-g", "x", "-h", "x", "-s", "0x10"], 2),
    (["map", "-g", "x", "-h", "x", "--gapopen", "-1"], 2),
    (["map", "-g", "x", "-h", "x", "--gapopen", "4294967296"], 2),
    (["map", "-g", "x", "-h", "x", "-t", "1.5"], 2),
    (["map", "-g", "x", "-h", "x", "-M"], 2),
    (["map", "-g", "x", "-h"], 2),
    (["map", "-g", "x", "-h", "x", "--inputformat", "sam"], 1),
    (["map", "-g", "x", "-h", "x", "-f", "cram"], 1),
    (["map", "-g", "x", "-h", "x", "--outputformat=json"], 1),
    (["map", "-g", "x", "-h", "x", "--readgroup", "SM:s1"], 1),
    (["map", "-g", "x", "-h", "x", "--readgroup", "ID:a,SM"], 1),
    (["map", "-g", "x", "-h", "x", "--readgroup", ""], 1),
]


def test_cli_build_genome_like_oracle(clis, tmp_path):
    """`probebwa build-genome -s -a -G out files...` (main.rs:33-41) writes
    the .stidx the oracle's command line writes, byte for byte; a missing
    input file fails on both."""
    g = K.Xorshift64(55).gen_seq(3000)
    f1 = tmp_path / "a.fa"
    f1.write_text(f">c1 first\n{g[:1000]}\n{g[1000:1500].lower()}\n>c2\n{g[1500:2000]}NNNN{g[2000:2200]}\n")
    f2 = tmp_path / "b.fa"
    f2.write_text(f">c3\n{g[2200:]}\n")
    outs = []
    for exe, name in ((clis[0], "mine"), (clis[1], "ref")):
        r = _run(exe, ["build-genome", "-s", "homo", "-a", "t2", "-G", str(tmp_path / name), str(f1), str(f2)])
        assert r.returncode == 0, r.stderr
        outs.append((tmp_path / f"{name}.stidx").read_bytes())
    assert outs[0] == outs[1]
    for exe in clis:
        bad = _run(exe, ["build-genome", "-s", "x", "-a", "y", "-G", str(tmp_path / "z"), str(tmp_path / "absent.fa")])
        assert bad.returncode != 0


@pytest.mark.parametrize("args,code", BAD_ARGS)
def test_cli_rejects_bad_arguments_like_oracle(clis, args, code):
    mine = _run(clis[0], args)
    ref = _run(clis[1], args)
    assert ref.returncode == code, ref.stderr
    assert mine.returncode == code, mine.stderr
    assert mine.stdout == b""


def test_oracle_sort_coordinate_semantics(oracle, tmp_path):
    """sort_for_coordinate_order (sam.rs:114-124): contig index by name (a
    repeated name takes its last index), then position, unmapped last, ties
    in input order."""
    g = K.Xorshift64(5).gen_seq(300)
    prefix = str(tmp_path / "dup")
    oracle.build_genome_from_seqs(prefix, [("a", g[:100]), ("b", g[100:200]), ("a", g[200:300])])
    oracle.build_hash(prefix, prefix)
    m = oracle.Mapper(prefix)
    n = 7
    recs = oracle.alloc_records(n, 0)
    recs["contig"][:] = [0, 1, 2, 1, -1, 0, 1]
    recs["pos"][:] = [5, 9, 3, 9, 0, 0, 2]
    R = oracle.Reads.from_lists([b""] * n)
    order = m.sort_coordinate([(R, recs)]).tolist()
    # contig 0 and 2 share the name "a" -> both rank 2; "b" -> rank 1
    assert order == [6, 1, 3, 2, 0, 4, 5]


# ---- GPU: SAM bytes of the two command lines ----

def _genome(tmp_path, oracle):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(61, length=60_000, n_copies=6, copy_len=800)
    parts = [("chrA", contigs[0][1][:30_000]), ("chrB", contigs[0][1][30_000:])]
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, parts)
    return prefix, parts


def _write_reads(path, seqs, quals, ids, offset=33, fasta=False):
    with open(path, "wb") as f:
        for i, s, q in zip(ids, seqs, quals):
            if fasta:
                f.write(b">" + i.encode() + b"\n" + s + b"\n")
            else:
                f.write(b"@" + i.encode() + b"\n" + s + b"\n+\n" + bytes(min(c + offset, 126) for c in q) + b"\n")
    return str(path)


@pytest.mark.gpu
def test_cli_sam_matches_oracle_cli(oracle, tmp_path, clis):
    from probebwa_gb300 import synth
    prefix, parts = _genome(tmp_path, oracle)
    seqs, quals, _ = synth.reads_single(62, parts, n=400, L=100)
    ids = [f"{'keep' if i % 3 else 'skip'}_{i}" for i in range(len(seqs))]
    seqs[5] = seqs[5].lower()
    seqs.append(b"")
    quals.append(b"")
    ids.append("empty_read")
    fq = _write_reads(tmp_path / "s.fq", seqs, quals, ids)
    fq64 = _write_reads(tmp_path / "s64.fq", seqs, quals, ids, offset=64)
    fa = _write_reads(tmp_path / "s.fa", seqs, quals, ids, fasta=True)
    s1, q1, s2, q2, _ = synth.reads_paired(63, parts, 300, L=100, mean=300, sd=40)
    p1 = _write_reads(tmp_path / "p1.fq", s1, q1, [f"pair{i}/1" for i in range(len(s1))])
    p2 = _write_reads(tmp_path / "p2.fq", s2, q2, [f"pair{i}/2" for i in range(len(s2))])
    runs = [
        ["map", "-g", prefix, "-h", prefix, "-M", fq],
        ["map", "--genome", prefix, "--hash", prefix, "--labelfilter", "keep", "--readgroup", "ID:x,PL:illumina",
         "-M", fq],
        ["map", "-g", prefix, "-h", prefix, "--phred64", "-s", "0.01", "--gapopen", "35", "-M", fq64],
        ["map", "-g", prefix, "-h", prefix, "--inputformat", "fasta", "--adapter-strip", "ACGTACGTAC", "-M", fa],
        ["map", "-g", prefix, "-h", prefix, "-M", p1, p2],
        ["map", "-g", prefix, "-h", prefix, "--svprior", "40", "--labelfilter", "pair1", "-M", p1, "-M", p2],
        ["map", "-g", prefix, "-h", prefix, "-M", fq, fq, "-M", fq64, "--inputformat", "fastq"],
    ]
    for args in runs:
        mine = _run(clis[0], args)
        ref = _run(clis[1], args)
        assert ref.returncode == 0, (args, ref.stderr)
        assert mine.returncode == 0, (args, mine.stderr)
        assert mine.stdout == ref.stdout, f"SAM differs for {args}"
    # the errors that come after mapping
    for args in (["map", "-g", prefix, "-h", prefix, "--index", "-M", fq],
                 ["map", "-g", prefix, "-h", prefix, "-f", "bam", "--index", "-M", fq],
                 ["map", "-g", prefix, "-h", prefix, "-M", p1, fq]):
        assert _run(clis[0], args).returncode == _run(clis[1], args).returncode == 1


@pytest.mark.gpu
def test_cli_output_file_matches_stdout(oracle, tmp_path, clis):
    from probebwa_gb300 import synth
    prefix, parts = _genome(tmp_path, oracle)
    seqs, quals, _ = synth.reads_single(64, parts, n=100, L=80)
    fq = _write_reads(tmp_path / "s.fq", seqs, quals, [f"r{i}" for i in range(len(seqs))])
    mine_path = str(tmp_path / "mine.sam")
    ref_path = str(tmp_path / "ref.sam")
    args = ["map", "-g", prefix, "-h", prefix, "-M", fq]
    assert _run(clis[0], args + ["-o", mine_path]).returncode == 0
    assert _run(clis[1], args + ["-o", ref_path]).returncode == 0
    a = open(mine_path, "rb").read().split(b"\n")
    b = open(ref_path, "rb").read().split(b"\n")
    # the @PG CL: lines differ only by their own -o path
    assert [x for x in a if not x.startswith(b"@PG")] == [x for x in b if not x.startswith(b"@PG")]


# ---- GPU: the device SAM formatter and coordinate sort ----

def _random_records(O, rng, reads, n_contigs, span=5000):
    n = reads.n
    lens = np.diff(reads.offsets)
    recs = O.alloc_records(n, int(lens.sum()))
    mapped = rng.random(n) < 0.85
    recs["contig"][:] = np.where(mapped, rng.integers(0, n_contigs, n), -1)
    recs["pos"][:] = np.where(mapped, rng.integers(1, span, n), 0)
    recs["pos"][: n // 10] = recs["pos"][n // 10: 2 * (n // 10)]  # ties in position
    recs["contig"][: n // 10] = recs["contig"][n // 10: 2 * (n // 10)]
    recs["mapq"][:] = rng.integers(0, 256, n)
    flag = rng.integers(0, 4096, n)
    recs["flag"][:] = np.where(mapped, flag, flag & ~0x10)
    recs["flag"][rng.random(n) < 0.05] |= 0x10  # reverse flag on some unmapped records too
    recs["mate_contig"][:] = np.where(rng.random(n) < 0.5, rng.integers(-1, n_contigs, n), -1)
    recs["mate_pos"][:] = rng.integers(0, 1 << 40, n) * (rng.random(n) < 0.5)
    recs["tlen"][:] = rng.integers(-(1 << 40), 1 << 40, n) * (rng.random(n) < 0.5)
    co = 0
    for i in range(n):
        recs["cigar_off"][i] = co
        k = int(rng.integers(0, 6)) if mapped[i] else 0
        for _ in range(k):
            recs["cigar"][co] = (int(rng.integers(1, 100000)) << 4) | int(rng.choice([0, 1, 2, 4]))
            co += 1
    recs["cigar_off"][n] = co
    return recs


def _random_reads(P, rng, n):
    seqs, quals, ids = [], [], []
    for i in range(n):
        L = int(rng.integers(0, 200))
        s = bytearray(rng.choice(list(b"ACGTNacgtnRY"), L).astype(np.uint8).tobytes())
        q = bytearray(rng.integers(0, 60, L).astype(np.uint8).tobytes())
        if i % 7 == 0 and L > 4:
            q[1:3] = rng.integers(0x80, 0x100, 2).astype(np.uint8).tobytes()  # invalid UTF-8 in QUAL
        if i % 11 == 0 and L > 4:
            s[2:4] = "é".encode()  # valid two-byte UTF-8 in SEQ
            q[0:2] = "é".encode()
        if i % 13 == 0 and L > 5:
            q[L - 1] = 0xE2  # truncated three-byte sequence at the end
            s[L - 2:L] = b"\xe2\x82"
        seqs.append(bytes(s))
        quals.append(bytes(q))
        ids.append(("read_%d_" % i) + "x" * int(rng.integers(0, 40)))
    return P.Reads.from_lists(seqs, quals, ids)


@pytest.mark.gpu
def test_sam_formatter_matches_oracle(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    g = K.Xorshift64(7).gen_seq(6000)
    prefix = str(tmp_path / "dup")
    oracle.build_genome_from_seqs(prefix, [("a", g[:2000]), ("chr_b", g[2000:4000]), ("a", g[4000:])])
    oracle.build_hash(prefix, prefix)
    rng = np.random.default_rng(11)
    R1 = _random_reads(P, rng, 900)
    R2 = _random_reads(P, rng, 900)
    rec1 = _random_records(oracle, rng, R1, 3)
    rec2 = _random_records(oracle, rng, R2, 3)
    O1 = oracle.Reads(R1.bases, R1.quals, R1.offsets, R1.ids)
    O2 = oracle.Reads(R2.bases, R2.quals, R2.offsets, R2.ids)
    om = oracle.Mapper(prefix)
    with P.Mapper(prefix) as m:
        for sources, osrc in (([(R1, rec1)], [(O1, rec1)]), ([(R1, rec1), (R2, rec2)], [(O1, rec1), (O2, rec2)])):
            n = len(sources) * R1.n
            sels = [None, rng.permutation(n)[: n // 2], np.zeros(0, np.uint64)]
            for sel in sels:
                for rg in (None, "ID:grp,SM:x,LB:y"):
                    got = m.sam_text(sources, sel, command_line="probebwa map -x", read_group=rg,
                                     coordinate_sorted=sel is not None)
                    exp = om.sam_text(str(tmp_path / "o.sam"), osrc, sel, command_line="probebwa map -x",
                                      read_group=rg, coordinate_sorted=sel is not None)
                    assert got == exp
            order = m.sort_coordinate(sources)
            assert order.tolist() == om.sort_coordinate(osrc).tolist()
            part = rng.permutation(n)[: n // 3]
            assert m.sort_coordinate(sources, part).tolist() == om.sort_coordinate(osrc, part).tolist()
        with pytest.raises(P.PbwError):
            m.sam_text([(R1, rec1)], read_group="SM:x")
        with pytest.raises(P.PbwError):
            m.sam_text([(R1, rec1)], sel=[R1.n])


@pytest.mark.gpu
def test_coordinate_sort_large_is_stable(oracle, tmp_path):
    """Many equal keys over several radix passes and tiles: the device order
    equals the oracle's stable sort."""
    import probebwa_gb300 as P
    P.build()
    g = K.Xorshift64(8).gen_seq(3000)
    prefix = str(tmp_path / "g")
    oracle.build_genome_from_seqs(prefix, [(f"c{i}", g[i * 100:(i + 1) * 100]) for i in range(30)])
    oracle.build_hash(prefix, prefix)
    rng = np.random.default_rng(3)
    n = 300_000
    recs = oracle.alloc_records(n, 0)
    recs["contig"][:] = rng.integers(0, 30, n)
    recs["pos"][:] = rng.integers(0, 50, n) * 100_003  # 4 radix passes; position 0 = unmapped
    R = P.Reads.from_lists([b""] * n)
    O = oracle.Reads(R.bases, R.quals, R.offsets, R.ids)
    om = oracle.Mapper(prefix)
    with P.Mapper(prefix) as m:
        got = m.sort_coordinate([(R, recs)])
    exp = om.sort_coordinate([(O, recs)])
    assert np.array_equal(got, exp)
