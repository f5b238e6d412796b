"""pbw_reads_load (the FASTQ / FASTA reads loader behind the C ABI) against
the oracle's parser (src/io/fastx.rs) on the same files: bases, Phred scores,
offsets and IDs byte for byte. Host-only: no device is touched."""
import numpy as np
import pytest

FILES = {
    "plain.fq": (False, "@r1 desc\nACGTACGT\n+\nIIIIIIII\n@r2\nacgtnNNa\n+r2\n!!!!####\n"),
    "multiline.fq": (False, "@m1/1\nACGT\nTTGG\n+\nIIII\nJJJJ\n@m2/2\nGG\nCC\n+\n####\n"),
    "crlf.fq": (False, "@c1\r\nACGT\r\n+\r\nIIII\r\n@c2 x y\r\nTTTT\r\n+\r\nABCD\r\n"),
    "empty_seq.fq": (False, "@empty\n\n+\n\n@normal\nACGT\n+\nIIII\n"),
    "short_qual.fq": (False, "@s1\nACGTACGT\n+\nIII\n@s2\nAC\n+\nIIIIII\n"),
    "at_header.fq": (False, "@@doubled/2\nACGTA\n+\nIIIII\n@ \nAAAA\n+\nIIII\n"),
    "ws.fq": (False, "@w1\n  ACGT \t\n+  \n IIII\n@w2\tname\nGGGG\n+\nIII\nI\n"),
    "no_final_nl.fq": (False, "@n1\nACGT\n+\nIIII\n@n2\nTTTT\n+\nIIII"),
    "plain.fa": (True, ">r1 desc\nACGT\nACGT\n>r2\nttgg\n>r3/1\n\n>r4\nNNNN\n"),
    "leading_text.fa": (True, "junk line\n\n>a\nAC GT\n>>b\nGG\r\nCC\r\n"),
    "empty.fa": (True, ""),
    "header_only.fa": (True, ">x\n"),
    "empty.fq": (False, ""),
    "unicode_ws.fq": (False, "@u1\u00a0desc\nAC\u2003GT\u3000\n+\u0085\nIIII\n@\u2000u2 x\nGGCC\u00a0\n+\nIIII\n"),
    "unicode_qual.fq": (False, "@q1\nACGT\n+\nI\u00e9I\n@q2\nAC\n+\nII\n"),
    "unicode_ws.fa": (True, ">a\u205fb\nAC\u1680\n\u202f>b\nGG\n"),
}

ADAPTER = "AGATCGGAAGAGC"


def _adapter_file(tmp_path):
    recs = [
        ("full", "ACGTTGCAACGTTGCA" + ADAPTER),
        ("partial", "GGGGCCCCAAAATTTT" + ADAPTER[:7]),
        ("onemm", "TTTTGGGGCCCC" + "AGATCGTAAGAGC"),
        ("lower", "ACACACACAC" + ADAPTER.lower()[:9]),
        ("short5", "ACGTACGTAC" + ADAPTER[:5]),
        ("none", "ACGTACGTACGTACGT"),
        ("tiny", "AGATC"),
    ]
    text = "".join(f"@{n}\n{s}\n+\n{'I' * len(s)}\n" for n, s in recs)
    p = tmp_path / "adapt.fq"
    p.write_text(text)
    return p


def _same(a, b):
    assert a.ids == b.ids
    assert np.array_equal(a.offsets, b.offsets)
    tot = int(a.offsets[-1])
    assert np.array_equal(a.bases[:tot], b.bases[:tot])
    assert np.array_equal(a.quals[:tot], b.quals[:tot])


@pytest.mark.parametrize("name", sorted(FILES))
@pytest.mark.parametrize("qoff", [33, 64])
def test_loader_matches_oracle(oracle, tmp_path, name, qoff):
    import probebwa_gb300 as P
    P.build()
    fasta, text = FILES[name]
    p = tmp_path / name
    p.write_bytes(text.encode())
    got = P.load_reads(str(p), fasta=fasta, quality_offset=qoff)
    want = oracle.parse_reads(str(p), fasta=fasta, quality_offset=qoff)
    _same(got, want)


def test_loader_adapter_matches_oracle(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    p = _adapter_file(tmp_path)
    got = P.load_reads(str(p), adapter=ADAPTER)
    want = oracle.parse_reads(str(p), adapter=ADAPTER)
    _same(got, want)
    lens = np.diff(got.offsets).tolist()
    # full adapter, 7-base tail, one mismatch in 13, lower case cut; 5 bases and no adapter kept
    assert lens[:4] == [16, 16, 12, 10]
    assert lens[4] == 15 and lens[5] == 16
    assert lens[6] == 5  # shorter than the 6-base minimum overlap


def test_loader_random_fastq_matches_oracle(oracle, tmp_path):
    import probebwa_gb300 as P
    P.build()
    rng = np.random.default_rng(7)
    lines = []
    for i in range(400):
        n = int(rng.integers(0, 300))
        seq = "".join(rng.choice(list("ACGTNacgtn"), n))
        ql = n + int(rng.integers(-3, 3)) if n > 3 else n
        qual = "".join(chr(int(c)) for c in rng.integers(33, 75, max(ql, 0)))
        sfx = ["", "/1", "/2", " extra"][i % 4]
        if n > 80 and i % 3 == 0:
            seq = seq[:40] + "\n" + seq[40:]
            qual = qual[:50] + "\n" + qual[50:]
        lines.append(f"@read{i}{sfx}\n{seq}\n+\n{qual}\n")
    p = tmp_path / "rand.fq"
    p.write_text("".join(lines))
    for adapter in (None, ADAPTER):
        got = P.load_reads(str(p), adapter=adapter)
        want = oracle.parse_reads(str(p), adapter=adapter)
        _same(got, want)


def test_loader_missing_file_raises(tmp_path):
    import probebwa_gb300 as P
    P.build()
    with pytest.raises(P.PbwError):
        P.load_reads(str(tmp_path / "absent.fq"))


@pytest.mark.parametrize("fasta", [False, True])
def test_loader_rejects_non_utf8_like_oracle(oracle, tmp_path, fasta):
    import probebwa_gb300 as P
    P.build()
    p = tmp_path / "bad.txt"
    body = b">r1\nAC\xffGT\n" if fasta else b"@r1\nACGT\n+\nII\xc3I\n"
    p.write_bytes(body)
    with pytest.raises(RuntimeError):
        oracle.parse_reads(str(p), fasta=fasta)
    with pytest.raises(P.PbwError):
        P.load_reads(str(p), fasta=fasta)


def test_loader_reads_gzip_members(oracle, tmp_path):
    """A .gz path is gunzipped (all members, as MultiGzDecoder) before parsing;
    the oracle parses the same text uncompressed."""
    import gzip
    import probebwa_gb300 as P
    P.build()
    text = "".join(f"@g{i}/1\n{'ACGT' * (i % 7 + 1)}\n+\n{'I' * (4 * (i % 7 + 1))}\n" for i in range(300))
    half = len(text) // 2
    cut = text.index("@", half)
    plain = tmp_path / "g.fq"
    plain.write_text(text)
    gz = tmp_path / "g.fq.gz"
    gz.write_bytes(gzip.compress(text[:cut].encode()) + gzip.compress(text[cut:].encode()))
    _same(P.load_reads(str(gz)), oracle.parse_reads(str(plain)))
    corrupt = tmp_path / "c.fq.gz"
    corrupt.write_bytes(gzip.compress(text.encode())[:-20])
    with pytest.raises(P.PbwError):
        P.load_reads(str(corrupt))


# multi-byte forms that std::str::from_utf8 accepts or rejects, for the word
# boundaries of the validator's ASCII fast path
UTF8_FORMS = [
    (b"\xc3\xa9", True),          # U+00E9
    (b"\xe2\x80\x83", True),      # U+2003
    (b"\xf0\x9f\x98\x80", True),  # U+1F600
    (b"\x80", False),             # lone continuation byte
    (b"\xc0\xaf", False),         # overlong
    (b"\xed\xa0\x80", False),     # surrogate
    (b"\xe2\x80", False),         # truncated
    (b"\xf4\x90\x80\x80", False),  # above U+10FFFF
]


@pytest.mark.parametrize("form,ok", UTF8_FORMS)
def test_utf8_check_at_every_word_offset(oracle, tmp_path, form, ok):
    """The validator skips ASCII 8 bytes at a time: a multi-byte form at each
    offset of the first words (in the ID, after a padding of k bytes) is
    accepted or refused exactly as the oracle's (from_utf8) check does."""
    import probebwa_gb300 as P
    P.build()
    for k in range(17):
        body = b"@" + b"x" * k + form + b"\nACGT\n+\nIIII\n@r2\nGG\n+\nII\n"
        p = tmp_path / f"u{k}.fq"
        p.write_bytes(body)
        if ok:
            _same(P.load_reads(str(p)), oracle.parse_reads(str(p)))
        else:
            with pytest.raises(RuntimeError):
                oracle.parse_reads(str(p))
            with pytest.raises(P.PbwError):
                P.load_reads(str(p))


def test_loader_reads_from_a_pipe(oracle, tmp_path):
    """A regular file is mapped; a pipe (no size, no mapping) is read as a
    stream: the same reads either way."""
    import os
    import threading
    import probebwa_gb300 as P
    P.build()
    text = FILES["multiline.fq"][1] + FILES["plain.fq"][1]
    plain = tmp_path / "p.fq"
    plain.write_text(text)
    fifo = tmp_path / "pipe.fq"
    os.mkfifo(fifo)

    def writer():
        with open(fifo, "w") as f:
            f.write(text)
    t = threading.Thread(target=writer)
    t.start()
    got = P.load_reads(str(fifo))
    t.join(timeout=30)
    _same(got, oracle.parse_reads(str(plain)))
    _same(P.load_reads(str(plain)), oracle.parse_reads(str(plain)))
