"""BAM from SAM text (write_bam / write_bam_indexed, src/io/bam.rs:19-57) on
the host through pbw_bam_write_text: the oracle maps pairs and formats the
SAM stream, the library encodes it, and every BAM record, the reference
dictionary and the BAI are decoded and checked against that stream. No
device is used."""
from __future__ import annotations

import gzip

import numpy as np
import pytest

from bam_helpers import decode_bai, decode_bam, same_as_sam, voffsets


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


@pytest.fixture(scope="module")
def mapped(oracle, tmp_path_factory):
    from probebwa_gb300 import synth
    d = tmp_path_factory.mktemp("bamtext")
    contigs = synth.genome_paired(121, n_contigs=3, contig_len=60_000)
    prefix = str(d / "g")
    synth.write_index(prefix, contigs)
    a1, _, a2, _, _ = synth.reads_paired(122, contigs, 300, L=150, mean=350, sd=50)
    # raw Phred scores of 33-60: the range a SAM parser accepts as QUAL characters
    rng = np.random.default_rng(123)
    b1 = [bytes(rng.integers(33, 61, len(s)).astype(np.uint8)) for s in a1]
    b2 = [bytes(rng.integers(33, 61, len(s)).astype(np.uint8)) for s in a2]
    ids = [f"p{i}" for i in range(len(a1))]
    R1 = oracle.Reads.from_lists(a1, b1, ids)
    R2 = oracle.Reads.from_lists(a2, b2, ids)
    om = oracle.Mapper(prefix)
    o1, o2, _ = om.map_paired(R1, R2)
    return d, om, [(R1, o1), (R2, o2)], contigs


def test_records_match_sam(P, mapped):
    d, om, src, contigs = mapped
    sam = om.sam_text(str(d / "a.sam"), src, read_group="ID:g1,SM:x")
    path = str(d / "a.bam")
    P.bam_from_sam(sam, path)
    data = open(path, "rb").read()
    assert data[-28:] == bytes.fromhex("1f8b08040000000000ff0600424302001b0003000000000000000000")
    recs = same_as_sam(sam, data)
    assert len(recs) == 2 * len(src[0][1]["contig"])
    _, refs, _ = decode_bam(data)
    assert [n for n, _ in refs] == [n for n, _ in contigs] and [ln for _, ln in refs] == [len(c) for _, c in contigs]


def test_sorted_stream_and_index(P, mapped):
    d, om, src, _ = mapped
    order = om.sort_coordinate(src)
    sam = om.sam_text(str(d / "s.sam"), src, sel=order, coordinate_sorted=True)
    path = str(d / "s.bam")
    P.bam_from_sam(sam, path, index=True)
    data = open(path, "rb").read()
    recs = same_as_sam(sam, data)
    index, no_coor = decode_bai(open(path + ".bai", "rb").read())
    v = voffsets(data)
    assert no_coor == sum(1 for r in recs if r["ref"] < 0)
    keys = [(r["ref"] if r["ref"] >= 0 else 1 << 30, r["pos"]) for r in recs]
    assert keys == sorted(keys)
    for r in recs:
        if r["ref"] < 0:
            continue
        bins, lin = index[r["ref"]]
        vo = v(r["start"])
        assert any(b <= vo < e for b, e in bins[r["bin"]]), r["name"]
        assert lin[r["pos"] >> 14] <= vo
    assert gzip.decompress(data)[:4] == b"BAM\x01"


def test_refusals(P, mapped, oracle):
    d, om, src, _ = mapped
    sam = om.sam_text(str(d / "u.sam"), src)
    # an index needs a coordinate-sorted stream
    with pytest.raises(P.PbwError):
        P.bam_from_sam(sam, str(d / "u.bam"), index=True)
    # raw scores below '!' are not QUAL characters
    R = src[0][0]
    seqs = [R.bases[R.offsets[i]:R.offsets[i + 1]].tobytes() for i in range(5)]
    Rq = oracle.Reads.from_lists(seqs, [bytes([20] * len(s)) for s in seqs])
    oq = om.map_single(Rq)
    low = om.sam_text(str(d / "q.sam"), [(Rq, oq)])
    with pytest.raises(P.PbwError, match="record"):
        P.bam_from_sam(low, str(d / "q.bam"))
    # the dictionary comes from @SQ: a record on a contig it lacks, an @SQ without LN
    lines = sam.split(b"\n")
    sq = [x for x in lines if x.startswith(b"@SQ")]
    first_name = sq[0].split(b"\t")[1][3:]
    assert any(x.split(b"\t")[2] == first_name for x in lines if x and not x.startswith(b"@"))
    no_first = b"\n".join(x for x in lines if x != sq[0])
    with pytest.raises(P.PbwError, match="record"):
        P.bam_from_sam(no_first, str(d / "r.bam"))
    no_ln = sam.replace(sq[0], b"\t".join(f for f in sq[0].split(b"\t") if not f.startswith(b"LN:")))
    with pytest.raises(P.PbwError, match="SQ"):
        P.bam_from_sam(no_ln, str(d / "l.bam"))
