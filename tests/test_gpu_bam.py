"""BAM output and its BAI (src/io/bam.rs, main.rs --outputformat bam /
--index) on the GPU build: the reference's own CLI tests (tests/cli.rs:46-80,
148-195) restated against the probebwa command line, and every BAM record
decoded and compared with the SAM stream it is encoded from."""
from __future__ import annotations

import gzip
import struct
import subprocess

import numpy as np
import pytest

import kat_cases as K

pytestmark = pytest.mark.gpu

OPS = "MIDNSHP=X"
SEQ = "=ACMGRSVTWYHKDBN"


def decode_bam(data: bytes):
    raw = gzip.decompress(data)
    assert raw[:4] == b"BAM\x01"
    p = 4
    (l_text,) = struct.unpack_from("<i", raw, p)
    p += 4
    text = raw[p:p + l_text].decode()
    p += l_text
    (n_ref,) = struct.unpack_from("<i", raw, p)
    p += 4
    refs = []
    for _ in range(n_ref):
        (ln,) = struct.unpack_from("<i", raw, p)
        p += 4
        name = raw[p:p + ln - 1].decode()
        p += ln
        (lr,) = struct.unpack_from("<i", raw, p)
        p += 4
        refs.append((name, lr))
    recs = []
    while p < len(raw):
        start = p
        (bs,) = struct.unpack_from("<i", raw, p)
        ref, pos, lrn, mapq, bin_, ncig, flag, lseq, nref, npos, tlen = struct.unpack_from("<iiBBHHHiiii", raw, p + 4)
        q = p + 36
        name = raw[q:q + lrn - 1].decode()
        q += lrn
        cig = struct.unpack_from(f"<{ncig}I", raw, q)
        q += 4 * ncig
        sq = raw[q:q + (lseq + 1) // 2]
        q += (lseq + 1) // 2
        seq = "".join(SEQ[(sq[i // 2] >> (4 if i % 2 == 0 else 0)) & 15] for i in range(lseq))
        qual = raw[q:q + lseq]
        q += lseq
        aux = raw[q:start + 4 + bs]
        recs.append(dict(start=start, name=name, flag=flag, ref=ref, pos=pos, mapq=mapq, bin=bin_,
                         cigar="".join(f"{c >> 4}{OPS[c & 15]}" for c in cig), nref=nref, npos=npos, tlen=tlen,
                         seq=seq, qual=bytes(qual), aux=aux))
        p = start + 4 + bs
    return text, refs, recs


def sam_lines(text: bytes):
    lines = text.decode("utf-8", "replace").split("\n")
    hdr = [x for x in lines if x.startswith("@")]
    return "\n".join(hdr) + "\n", [x.split("\t") for x in lines if x and not x.startswith("@")]


def _same_as_sam(sam: bytes, bam: bytes):
    hdr, rows = sam_lines(sam)
    text, refs, recs = decode_bam(bam)
    assert text == hdr
    names = [r[0] for r in refs]
    assert len(rows) == len(recs)
    for f, r in zip(rows, recs):
        assert r["name"] == f[0] and r["flag"] == int(f[1]) and r["mapq"] == int(f[4])
        assert (names[r["ref"]] if r["ref"] >= 0 else "*") == f[2]
        assert r["pos"] + 1 == int(f[3])
        assert (r["cigar"] or "*") == f[5]
        assert (names[r["nref"]] if r["nref"] >= 0 else "*") == f[6]
        assert r["npos"] + 1 == int(f[7]) and r["tlen"] == int(f[8])
        assert r["seq"] == f[9]
        assert bytes(c + 33 for c in r["qual"]) == f[10].encode()
        rg = [x for x in f[11:] if x.startswith("RG:Z:")]
        assert r["aux"] == (b"RGZ" + rg[0][5:].encode() + b"\0" if rg else b"")
    return recs


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


def _decode_bai(b: bytes):
    assert b[:4] == b"BAI\x01"
    p = 8
    (n_ref,) = struct.unpack_from("<i", b, 4)
    out = []
    for _ in range(n_ref):
        (nb,) = struct.unpack_from("<i", b, p)
        p += 4
        bins = {}
        for _ in range(nb):
            bn, nc = struct.unpack_from("<Ii", b, p)
            p += 8
            bins[bn] = [struct.unpack_from("<QQ", b, p + 16 * k) for k in range(nc)]
            p += 16 * nc
        (ni,) = struct.unpack_from("<i", b, p)
        p += 4
        lin = struct.unpack_from(f"<{ni}Q", b, p)
        p += 8 * ni
        out.append((bins, lin))
    (no_coor,) = struct.unpack_from("<Q", b, p)
    return out, no_coor


def _voffsets(data: bytes):
    """Uncompressed stream offset -> virtual offset, from the BGZF blocks."""
    blocks, c = [], 0
    while c < len(data):
        (bsize,) = struct.unpack_from("<H", data, c + 16)
        isize = struct.unpack_from("<I", data, c + bsize + 1 - 4)[0]
        blocks.append((c, isize))
        c += bsize + 1
    starts = np.cumsum([0] + [s for _, s in blocks])

    def v(u):
        b = int(np.searchsorted(starts, u, side="right") - 1)
        return (blocks[b][0] << 16) | int(u - starts[b])
    return v


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
        _same_as_sam(m.sam_text(src, read_group="ID:g1,SM:x"), open(path, "rb").read())
        order = m.sort_coordinate(src)
        m.write_bam(path, src, sel=order, coordinate_sorted=True, index=True)
        data = open(path, "rb").read()
        recs = _same_as_sam(m.sam_text(src, sel=order, coordinate_sorted=True), data)
        # low scores are not QUAL characters: the encoder refuses them as a SAM parser does
        Rq = P.Reads.from_lists(a1[:5], [bytes([20] * len(s)) for s in a1[:5]])
        oq = m.map_single(Rq)
        with pytest.raises(P.PbwError):
            m.write_bam(str(tmp_path / "bad.bam"), [(Rq, oq)])
    index, no_coor = _decode_bai(open(path + ".bai", "rb").read())
    v = _voffsets(data)
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
