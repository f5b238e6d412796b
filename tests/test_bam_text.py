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
    # an index needs a coordinate-sorted stream, and records in that order
    with pytest.raises(P.PbwError, match="coordinate"):
        P.bam_from_sam(sam, str(d / "u.bam"), index=True)
    lines = sam.rstrip(b"\n").split(b"\n")
    hdr = [x.replace(b"SO:unsorted", b"SO:coordinate") for x in lines if x.startswith(b"@")]
    placed = [x for x in lines if not x.startswith(b"@") and x.split(b"\t")[2] != b"*"]
    assert len(placed) > 2
    order = sorted(range(len(placed)), key=lambda i: (placed[i].split(b"\t")[2], int(placed[i].split(b"\t")[3])))
    swapped = [placed[i] for i in order]
    swapped[0], swapped[-1] = swapped[-1], swapped[0]
    with pytest.raises(P.PbwError, match="out of coordinate order"):
        P.bam_from_sam(b"\n".join(hdr + swapped) + b"\n", str(d / "o.bam"), index=True)
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


HDR = b"@HD\tVN:1.6\tSO:unsorted\n@SQ\tSN:c1\tLN:1000\n"


@pytest.mark.parametrize("rec,why", [
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT", "fewer than 11 fields"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT\tIIII\tXX", "optional field"),
    (b"r1\t0\tc1\t99999999999999999999999\t60\t4M\t*\t0\t0\tACGT\tIIII", "number"),
    (b"r1\t0\tc1\t2147483648\t60\t4M\t*\t0\t0\tACGT\tIIII", "number"),
    (b"r1\t0\tc1\t10\t256\t4M\t*\t0\t0\tACGT\tIIII", "number"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t-2147483648\tACGT\tIIII", "number"),
    (b"r1\t0\tc1\t10\t60\t268435456M\t*\t0\t0\tACGT\tIIII", "CIGAR"),
    (b"r1\t0\tc1\t10\t60\t99999999999999999999M\t*\t0\t0\tACGT\tIIII", "CIGAR"),
    (b"r1\t0\tc1\t10\t60\t4Q\t*\t0\t0\tACGT\tIIII", "CIGAR"),
    (b"r1\t0\tc1\t10\t60\tM\t*\t0\t0\tACGT\tIIII", "CIGAR"),
    (b"r1\t0\tc1\t2147483000\t60\t100000M\t*\t0\t0\tACGT\tIIII", "2\\^31"),
    (b"r1\t0\tc2\t10\t60\t4M\t*\t0\t0\tACGT\tIIII", "missing from the header"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tAC!T\tIIII", "sequence base"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT\tIII", "differ in length"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT\tIIII\tNM:i:99999999999", "optional field"),
    (b"r1\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT\tIIII\tXA:f:1.5", "optional field type"),
    (b"\t0\tc1\t10\t60\t4M\t*\t0\t0\tACGT\tIIII", "read name"),
])
def test_malformed_records_are_errors(P, tmp_path, rec, why):
    """Caller text is parsed defensively: every malformed or out-of-range
    record is an error naming the record, never a crash or a silently
    truncated field."""
    with pytest.raises(P.PbwError, match=why):
        P.bam_from_sam(HDR + rec + b"\n", str(tmp_path / "m.bam"))


def test_well_formed_record_round_trip(P, tmp_path):
    rec = b"r1\t16\tc1\t10\t60\t2M1I1M\t=\t100\t-5\tACGT\t!I~5\tRG:Z:g1\tNM:i:-3\n"
    path = str(tmp_path / "ok.bam")
    P.bam_from_sam(HDR + rec, path)
    text, refs, recs = decode_bam(open(path, "rb").read())
    assert refs == [("c1", 1000)] and len(recs) == 1
    r = recs[0]
    assert (r["name"], r["flag"], r["ref"], r["pos"], r["mapq"], r["cigar"]) == ("r1", 16, 0, 9, 60, "2M1I1M")
    assert (r["nref"], r["npos"], r["tlen"], r["seq"]) == (0, 99, -5, "ACGT")
    assert r["qual"] == bytes([0, 40, 93, 20])
    assert r["aux"] == b"RGZg1\0" + b"NMi" + (-3).to_bytes(4, "little", signed=True)


def _big_sam(n, bad=None):
    """n records of 150 bases (about 9 MB for 25,000), the record numbered
    bad with an invalid base."""
    rng = np.random.default_rng(7)
    hdr = b"@HD\tVN:1.6\tSO:coordinate\n" + b"".join(b"@SQ\tSN:c%d\tLN:5000000\n" % i for i in range(3))
    seq = np.frombuffer(b"ACGT", np.uint8)[rng.integers(0, 4, (n, 150))]
    qual = (rng.integers(0, 41, (n, 150)) + 33).astype(np.uint8)
    lines = []
    for i in range(n):
        s = seq[i].tobytes() if i != bad else b"AC!" + seq[i].tobytes()[3:]
        c = i * 3 // n
        lines.append(b"r%d\t99\tc%d\t%d\t60\t150M\tc%d\t%d\t300\t" % (i, c, 1 + i * 100, c, 151 + i * 100)
                     + s + b"\t" + qual[i].tobytes() + b"\n")
    return hdr + b"".join(lines)


def test_large_stream_encoded_in_slices(P, tmp_path):
    """Streams over 4 MB are encoded in slices on several threads: the
    records, their order, the BAI and the number of a failing record are
    those of the whole stream."""
    sam = _big_sam(25_000)
    path = str(tmp_path / "big.bam")
    P.bam_from_sam(sam, path, index=True)
    data = open(path, "rb").read()
    recs = same_as_sam(sam, data)
    assert [r["name"] for r in recs] == [f"r{i}" for i in range(25_000)]
    index, no_coor = decode_bai(open(path + ".bai", "rb").read())
    v = voffsets(data)
    for r in recs[::97]:
        bins, lin = index[r["ref"]]
        vo = v(r["start"])
        assert any(b <= vo < e for b, e in bins[r["bin"]])
        assert lin[r["pos"] >> 14] <= vo
    for bad in (3, 17_321, 24_999):
        with pytest.raises(P.PbwError, match=f"record {bad}: invalid sequence base"):
            P.bam_from_sam(_big_sam(25_000, bad=bad), str(tmp_path / "bad.bam"))
