"""MapqCalculator stage on the GPU (pbw_mapq_batch) against the oracle's
select_best + finalize_mapq on the same inputs."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

OPCODE = {"M": 0, "I": 1, "D": 2, "S": 4}


def _pack(cig: str) -> np.ndarray:
    out, num = [], ""
    for ch in cig:
        if ch.isdigit():
            num += ch
        else:
            out.append((int(num) << 4) | OPCODE[ch])
            num = ""
    return np.array(out, np.uint32)


def _revcomp(b: bytes) -> bytes:
    comp = {ord("A"): ord("T"), ord("T"): ord("A"), ord("C"): ord("G"), ord("G"): ord("C")}
    return bytes(comp.get(x, ord("N")) for x in reversed(b.upper()))


def _items(seed, oracle, n=500):
    rng = np.random.default_rng(seed)
    seqs, quals, items = [], [], []
    for i in range(n):
        L = int(rng.integers(8, 220))
        core = rng.choice(list(b"ACGT"), size=L).astype(np.uint8)
        if i % 7 == 0:
            core[rng.integers(0, L)] = ord("N")
        if i % 11 == 0:
            core[rng.integers(0, L)] = ord("R")
        read = core.tobytes()
        if i % 5 == 0:
            read = read.lower()
        q = rng.integers(2, 42, size=L).astype(np.uint8)
        if i % 9 == 0:
            q[: L // 3] = 5
        rev = bool(rng.integers(0, 2))
        query = _revcomp(read) if rev else read.upper()
        qq = q[::-1].tobytes() if rev else q.tobytes()
        # reference window around a mutated copy of the query
        ref = bytearray(rng.choice(list(b"ACGT"), size=10).astype(np.uint8).tobytes())
        body = bytearray(query.replace(b"R", b"A"))
        for _ in range(int(rng.integers(0, 6))):
            body[int(rng.integers(0, len(body)))] = int(rng.choice(list(b"ACGTN")))
        if len(body) > 20 and rng.random() < 0.3:
            p = int(rng.integers(5, len(body) - 5))
            body = body[:p] + body[p + int(rng.integers(1, 4)):]
        ref += body + bytearray(rng.choice(list(b"ACGT"), size=30).astype(np.uint8).tobytes())
        score, cig, off = oracle.align(query, qq, bytes(ref), 10, 30)
        packed = _pack(cig)
        span = sum(int(w) >> 4 for w in packed if (int(w) & 15) in (0, 2))
        window = bytes(ref[off:off + span])
        nc = int(rng.integers(1, 21))
        lks = list(rng.normal(-120, 40, size=nc))
        if nc > 2 and i % 4 == 0:
            lks[int(rng.integers(0, nc))] = max(lks)  # a tie for the last maximum
        nw = max(L - 14, 0)
        kind = rng.integers(0, 3, size=nw)
        rep = np.where(kind == 0, 0.0, np.where(kind == 1, 1.0, rng.random(nw)))
        seqs.append(read)
        quals.append(q.tobytes())
        items.append({"lks": lks, "repeat": rep, "rev": rev, "ref": window, "cigar": packed})
    return seqs, quals, items


def test_mapq_batch_matches_oracle(oracle, tmp_path):
    import probebwa_gb300 as P
    from probebwa_gb300 import synth
    P.build()
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, synth.genome_single(3, length=50_000, n_copies=3, copy_len=500))
    seqs, quals, items = _items(17, oracle)
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix) as m:
        got = m.mapq_batch(R, items)
    om = oracle.Mapper(prefix)
    exp = om.mapq_batch(oracle.Reads(R.bases, R.quals, R.offsets, R.ids), items)
    om.close()
    assert np.array_equal(got["best"], exp["best"])
    assert np.array_equal(got["mapq"], exp["mapq"]), np.nonzero(got["mapq"] != exp["mapq"])[0][:10]
    # sum_exp: a sum of exp() terms, each within an ulp of the host libm's;
    # posterior = 1 - 10^(-phred/10): its error is that of the pow() term,
    # so the tolerance is in ulps of max(posterior, 1 - posterior)
    tol = 4 * np.spacing(np.abs(exp["sum_exp"]))
    bad = np.nonzero(np.abs(got["sum_exp"] - exp["sum_exp"]) > tol)[0]
    assert len(bad) == 0, ("sum_exp", bad[:10])
    tol = 4 * np.spacing(np.maximum(np.abs(exp["posterior"]), np.abs(1.0 - exp["posterior"])))
    bad = np.nonzero(np.abs(got["posterior"] - exp["posterior"]) > tol)[0]
    assert len(bad) == 0, ("posterior", bad[:10], got["posterior"][bad[:3]], exp["posterior"][bad[:3]])
    assert (exp["mapq"] > 0).sum() > 50 and (exp["mapq"] == 0).sum() > 5
