"""Index building behind the C ABI against the oracle's builders:
pbw_build_genome (.stidx, host) and pbw_build_hash (.sthash, on the GPU)
must write the same bytes as the oracle's restatement of GenomeIndexBuilder
and HashTableBuilder (src/index/genome.rs, src/index/hashtable.rs)."""
from __future__ import annotations

import gzip
import subprocess

import numpy as np
import pytest

import kat_cases as K


def _fasta(path, records, crlf=False):
    nl = "\r\n" if crlf else "\n"
    with open(path, "w") as f:
        for name, seq in records:
            f.write(f">{name}{nl}")
            for i in range(0, len(seq), 60):
                f.write(seq[i:i + 60] + nl)
    return str(path)


def _genome_records(seed):
    rng = np.random.default_rng(seed)
    g = K.Xorshift64(seed).gen_seq(5000)
    recs = [
        ("chr1 description text", g[:1200]),
        ("lower", g[1200:1900].lower()),
        ("nruns", g[1900:2100] + "N" * 37 + g[2100:2300] + "NNRYKM" + g[2300:2400] + "n" * 5),
        ("short", "ACGTACG"),
        ("empty", ""),
        ("allN", "N" * 50),
        ("repeat", "ACGT" * 400),
        ("tail_n", g[2400:2731] + "N"),
    ]
    # a random soft-masked, IUPAC-sprinkled contig
    s = list(g[2731:4731])
    for i in rng.choice(len(s), 40, replace=False):
        s[i] = "acgtNRYSWKMBDHV"[int(rng.integers(0, 15))]
    recs.append(("mixed", "".join(s)))
    return recs


def test_build_genome_matches_oracle(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    recs = _genome_records(1)
    f1 = _fasta(tmp_path / "a.fa", recs[:4])
    f2 = _fasta(tmp_path / "b.fa", recs[4:], crlf=True)
    P.build_genome(str(tmp_path / "mine"), [f1, f2], "homo", "t2")
    oracle.build_genome_from_fasta(str(tmp_path / "ref"), [f1, f2], "homo", "t2")
    assert open(tmp_path / "mine.stidx", "rb").read() == open(tmp_path / "ref.stidx", "rb").read()
    # gzip input: the same index as the plain file
    gz = tmp_path / "a.fa.gz"
    gz.write_bytes(gzip.compress(open(f1, "rb").read()))
    P.build_genome(str(tmp_path / "gz"), [str(gz), f2], "homo", "t2")
    assert open(tmp_path / "gz.stidx", "rb").read() == open(tmp_path / "ref.stidx", "rb").read()


def test_build_genome_edge_files(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    cases = {
        "lead.fa": "junk before\n\n>x  y\nAC GT\n  >z\nGG\n>>w\n",
        "empty.fa": "",
        "noheader.fa": "ACGT\nACGT\n",
        "unicode.fa": ">a b\nAC GT\n　>c\nTT\n",
    }
    for name, text in cases.items():
        p = tmp_path / name
        p.write_text(text)
        P.build_genome(str(tmp_path / "m"), [str(p)])
        oracle.build_genome_from_fasta(str(tmp_path / "r"), [str(p)], "species", "assembly")
        assert open(tmp_path / "m.stidx", "rb").read() == open(tmp_path / "r.stidx", "rb").read(), name
    bad = tmp_path / "bad.fa"
    bad.write_bytes(b">a\nAC\xffGT\n")
    with pytest.raises(P.PbwError):
        P.build_genome(str(tmp_path / "m"), [str(bad)])
    with pytest.raises(RuntimeError):
        oracle.build_genome_from_fasta(str(tmp_path / "r"), [str(bad)])
    with pytest.raises(P.PbwError):
        P.build_genome(str(tmp_path / "m"), [str(tmp_path / "absent.fa")])


def test_cli_build_genome_matches_oracle_cli(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import native_build
    recs = _genome_records(2)
    f1 = _fasta(tmp_path / "a.fa", recs)
    outs = []
    for exe, tag in ((native_build.CLI, "mine"), (oracle.CLI_PATH, "ref")):
        r = subprocess.run(["probebwa", "build-genome", "-s", "sp", f1, "--assembly", "as1", "-G",
                            str(tmp_path / tag)], executable=exe, capture_output=True, timeout=120)
        assert r.returncode == 0, r.stderr
        outs.append(r.stdout.replace(tag.encode(), b"X"))
    assert outs[0] == outs[1]
    assert open(tmp_path / "mine.stidx", "rb").read() == open(tmp_path / "ref.stidx", "rb").read()
    for exe in (native_build.CLI, oracle.CLI_PATH):
        r = subprocess.run(["probebwa", "build-genome", "-s", "sp", f1], executable=exe, capture_output=True)
        assert r.returncode == 2


HASH_PARAMS = [(15, 5, 300), (15, 1, 300), (15, 3, 7), (11, 5, 300), (20, 4, 300), (32, 2, 5), (1, 1, 3),
               (15, 5, 1), (15, 7, 0)]


@pytest.mark.gpu
@pytest.mark.parametrize("k,stride,cap", HASH_PARAMS)
def test_build_hash_matches_oracle(oracle, tmp_path, k, stride, cap):
    import probebwa_gb300 as P
    P.build()
    recs = _genome_records(3)
    f = _fasta(tmp_path / "g.fa", recs)
    prefix = str(tmp_path / "g")
    oracle.build_genome_from_fasta(prefix, [f])
    P.build_hash(prefix, str(tmp_path / "mine"), k, stride, cap)
    oracle.build_hash(prefix, str(tmp_path / "ref"), k, stride, cap)
    assert open(tmp_path / "mine.sthash", "rb").read() == open(tmp_path / "ref.sthash", "rb").read()


@pytest.mark.gpu
def test_build_hash_large_genome_and_map(oracle, tmp_path):
    """A 4 Mbp genome with planted repeats (buckets over the 300 cap) builds the
    same table as the oracle, and mapping against the GPU-built table gives the
    oracle's records."""
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import synth
    contigs = synth.genome_single(71, length=2_000_000, n_copies=400, copy_len=1500)
    contigs.append(("second", synth.genome_single(72, length=2_000_000, n_copies=10, copy_len=500)[0][1]))
    prefix = str(tmp_path / "g")
    synth.write_stidx(prefix, contigs)
    P.build_hash(prefix, str(tmp_path / "mine"))
    oracle.build_hash(prefix, str(tmp_path / "ref"))
    a = open(tmp_path / "mine.sthash", "rb").read()
    assert a == open(tmp_path / "ref.sthash", "rb").read()
    seqs, quals, _ = synth.reads_single(73, contigs, n=500, L=120)
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix, str(tmp_path / "mine")) as m:
        got = m.map_single(R)
    om = oracle.Mapper(prefix, str(tmp_path / "ref"))
    exp = om.map_single(oracle.Reads(R.bases, R.quals, R.offsets, R.ids))
    from gpu_helpers import compare_records
    compare_records(P, oracle, got, exp, "GPU-built table")


@pytest.mark.gpu
def test_cli_build_hash_matches_oracle_cli(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import native_build
    f = _fasta(tmp_path / "g.fa", _genome_records(4))
    prefix = str(tmp_path / "g")
    oracle.build_genome_from_fasta(prefix, [f])
    for exe, tag in ((native_build.CLI, "mine"), (oracle.CLI_PATH, "ref")):
        r = subprocess.run(["probebwa", "build-hash", "--genome", prefix, "-H", str(tmp_path / tag)],
                           executable=exe, capture_output=True, timeout=120)
        assert r.returncode == 0, r.stderr
    assert open(tmp_path / "mine.sthash", "rb").read() == open(tmp_path / "ref.sthash", "rb").read()
