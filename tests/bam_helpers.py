"""BAM / BAI decoding for the tests: BGZF members gunzipped as one stream,
records unpacked field by field (SAM specification section 4.2), the BAI's
bins, chunks and linear index (section 5.2), and the virtual offsets of a
BGZF file's bytes."""
from __future__ import annotations

import gzip
import struct

import numpy as np

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


def same_as_sam(sam: bytes, bam: bytes):
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


def decode_bai(b: bytes):
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


def voffsets(data: bytes):
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
