"""BAM output and its BAI (src/io/bam.rs, main.rs --outputformat bam /
--index) on the GPU build: the reference's own CLI tests (tests/cli.rs:46-80,
148-195) restated against the probebwa command line, and every BAM record
decoded and compared with the SAM stream it is encoded from."""
from __future__ import annotations

import gzip
import subprocess

import numpy as np
import pytest

import kat_cases as K
from bam_helpers import decode_bai, decode_bam, same_as_sam, voffsets

pytestmark = pytest.mark.gpu


def _run(exe, args):
    return subprocess.run(["probebwa", *args], executable=exe, capture_output=True, timeout=600)


@pytest.fixture(scope="module")
def cli():
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import native_build
    return native_build.CLI


def _fastq(path, recs):
    with open(path, "w") as f:
        for i, s in recs:
            f.write(f"@{i}\n{s}\n+\n{'I' * len(s)}\n")
    return str(path)


def test_cli_bam_is_bgzf_bam(oracle, tmp_path, cli):
    """test_bam_output_is_valid_bgzf_bam (tests/cli.rs:46-80)."""
    g = K.Xorshift64(99).gen_seq(400)
    prefix = str(tmp_path / "ref")
    oracle.build_index(prefix, [("chr1", g)])
    fq = _fastq(tmp_path / "reads.fq", [("r1", g[40:80])])
    bam = tmp_path / "out.bam"
    r = _run(cli, ["map", "--genome", prefix, "--hash", prefix, "-M", fq, "--outputformat", "bam", "--output",
                   str(bam)])
    assert r.returncode == 0, r.stderr
    data = bam.read_bytes()
    assert gzip.decompress(data)[:4] == b"BAM\x01"
    assert data[-28:] == bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")
    sam = _run(cli, ["map", "--genome", prefix, "--hash", prefix, "-M", fq])
    # the @PG line echoes the argv, which differs between the two runs
    t, _, recs = decode_bam(data)
    assert recs[0]["name"] == "r1" and recs[0]["pos"] == 40 and recs[0]["cigar"] == "40M"
    assert sam.returncode == 0
    assert _run(cli, ["map", "-g", prefix, "-h", prefix, "-M", fq, "-f", "bam"]).returncode == 1


def test_cli_bam_index(oracle, tmp_path, cli):
    """test_index_produces_a_valid_bai_alongside_the_bam (tests/cli.rs:148-195)."""
    g = K.Xorshift64(102).gen_seq(2000)
    prefix = str(tmp_path / "ref")
    oracle.build_index(prefix, [("chr1", g)])
    fq = _fastq(tmp_path / "reads.fq", [("late", g[1000:1040]), ("early", g[40:80])])
    bam = tmp_path / "out.bam"
    r = _run(cli, ["map", "--genome", prefix, "--hash", prefix, "-M", fq, "--outputformat", "bam", "--output",
                   str(bam), "--index"])
    assert r.returncode == 0, r.stderr
    bai = (tmp_path / "out.bam.bai").read_bytes()
    assert bai[:4] == b"BAI\x01"
    raw = gzip.decompress(bam.read_bytes())
    assert raw.find(b"early") < raw.find(b"late")
    text, _, recs = decode_bam(bam.read_bytes())
    assert "SO:coordinate" in text.splitlines()[0]


def test_bam_records_and_index_match_sam(tmp_path):
    import probebwa_gb300 as P
    P.build()
    from probebwa_gb300 import synth
    contigs = synth.genome_paired(111, n_contigs=3, contig_len=200_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    a1, b1, a2, b2, _ = synth.reads_paired(112, contigs, 1500, L=150, mean=350, sd=50)
    # raw Phred scores of 33-60: the range a SAM parser accepts as QUAL characters
    rng = np.random.default_rng(113)
    b1 = [bytes(rng.integers(33, 61, len(s)).astype(np.uint8)) for s in a1]
    b2 = [bytes(rng.integers(33, 61, len(s)).astype(np.uint8)) for s in a2]
    R1 = P.Reads.from_lists(a1, b1, [f"p{i}" for i in range(len(a1))])
    R2 = P.Reads.from_lists(a2, b2, [f"p{i}" for i in range(len(a2))])
    with P.Mapper(prefix) as m:
        o1, o2, _ = m.map_paired(R1, R2)
        src = [(R1, o1), (R2, o2)]
        path = str(tmp_path / "o.bam")
        m.write_bam(path, src, read_group="ID:g1,SM:x")
        same_as_sam(m.sam_text(src, read_group="ID:g1,SM:x"), open(path, "rb").read())
        order = m.sort_coordinate(src)
        m.write_bam(path, src, sel=order, coordinate_sorted=True, index=True)
        data = open(path, "rb").read()
        sorted_sam = m.sam_text(src, sel=order, coordinate_sorted=True)
        recs = same_as_sam(sorted_sam, data)
        # the same stream through the text entry point (write_bam on SAM text):
        # the same BAM and BAI bytes
        P.bam_from_sam(sorted_sam, str(tmp_path / "t.bam"), index=True)
        assert open(str(tmp_path / "t.bam"), "rb").read() == data
        assert open(str(tmp_path / "t.bam.bai"), "rb").read() == open(path + ".bai", "rb").read()
        # low scores are not QUAL characters: the encoder refuses them as a SAM parser does
        Rq = P.Reads.from_lists(a1[:5], [bytes([20] * len(s)) for s in a1[:5]])
        oq = m.map_single(Rq)
        with pytest.raises(P.PbwError):
            m.write_bam(str(tmp_path / "bad.bam"), [(Rq, oq)])
    index, no_coor = decode_bai(open(path + ".bai", "rb").read())
    v = voffsets(data)
    raw_hdr = gzip.decompress(data)
    assert no_coor == sum(1 for r in recs if r["ref"] < 0)
    for r in recs:
        if r["ref"] < 0:
            continue
        bins, lin = index[r["ref"]]
        vo = v(r["start"])
        assert any(b <= vo < e for b, e in bins[r["bin"]]), r["name"]
        assert lin[r["pos"] >> 14] <= vo
    assert raw_hdr[:4] == b"BAM\x01"
