"""K3 (banded affine DP + traceback) through pbw_align_batch against the
oracle's SmithWatermanAligner restatement on the same problems: score, CIGAR
and reference offset bit-exact."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def M(tmp_path_factory):
    import probebwa_gb300 as P
    from probebwa_gb300 import synth
    P.build()
    d = tmp_path_factory.mktemp("idx")
    prefix = str(d / "g")
    synth.write_index(prefix, synth.contigs_from_strings([("c", "ACGT" * 40)]))
    m = P.Mapper(prefix)
    yield m
    m.close()


def _b(a) -> bytes:
    return np.asarray(a, dtype=np.uint8).tobytes()


def _mutate(rng, s: bytes, sub: float, indel: float) -> bytes:
    out = bytearray()
    for c in s:
        r = rng.random()
        if r < indel / 2:
            continue
        if r < indel:
            out += _b(rng.choice(list(b"ACGT"), size=int(rng.integers(1, 4))))
        if rng.random() < sub:
            c = int(rng.choice([x for x in b"ACGT" if x != c]))
        out.append(c)
    return bytes(out)


def _problems(seed, n, kind):
    rng = np.random.default_rng(seed)
    probs = []
    for _ in range(n):
        if kind == "seeded":
            L = int(rng.integers(15, 200))
            ref = _b(rng.choice(list(b"ACGT"), size=L + 40))
            start = int(rng.integers(0, 21))
            read = _mutate(rng, ref[start:start + L], 0.03, 0.02)
            if rng.random() < 0.1:
                ref = ref[:int(rng.integers(1, len(ref)))]  # truncated by a contig end
            probs.append((read, bytes(rng.integers(2, 42, size=len(read)).astype(np.uint8)), ref, 10, 30))
        elif kind == "window":
            L = int(rng.integers(30, 160))
            rad = int(rng.integers(L, L + 300))
            ref = _b(rng.choice(list(b"ACGT"), size=L + 2 * rad))
            exp = int(rng.integers(0, rad + 1))
            read = _mutate(rng, ref[exp:exp + L], 0.05, 0.02)
            probs.append((read, bytes(rng.integers(2, 42, size=len(read)).astype(np.uint8)), ref, exp, len(ref)))
        elif kind == "wide":
            # windows of up to 40 column tiles: every warp of the window DP
            # takes several tiles and reuses its boundary buffer; half of
            # them banded, with hints that start or end the band off the window
            L = int(rng.integers(30, 320))
            n = int(rng.integers(500, 5000))
            ref = _b(rng.choice(list(b"ACGT"), size=n))
            exp = int(rng.integers(0, n - L))
            read = _mutate(rng, ref[exp:exp + L], 0.05, 0.03)
            if rng.random() < 0.5:
                probs.append((read, bytes(rng.integers(2, 42, size=len(read)).astype(np.uint8)), ref, exp, n))
            else:
                hint = int(rng.integers(-300, n + 300))
                band = int(rng.integers(32, 700))
                probs.append((read, bytes(rng.integers(2, 42, size=len(read)).astype(np.uint8)), ref, hint, band))
        else:  # arbitrary bands and hints, homopolymers and N
            L = int(rng.integers(1, 120))
            n = int(rng.integers(1, 220))
            alphabet = list(b"ACGTN") if rng.random() < 0.3 else list(b"AC")
            ref = _b(rng.choice(alphabet, size=n))
            read = _b(rng.choice(list(b"ACGTNR"), size=L))
            hint = int(rng.integers(-60, 200))
            band = int(rng.integers(0, 80))
            probs.append((read, bytes(rng.integers(0, 60, size=L).astype(np.uint8)), ref, hint, band))
    return probs


@pytest.mark.parametrize("kind,seed,n", [("seeded", 1, 3000), ("window", 2, 400), ("odd", 3, 3000), ("wide", 4, 120)])
def test_align_batch_matches_oracle(M, oracle, kind, seed, n):
    probs = _problems(seed, n, kind)
    got = M.align_batch(probs)
    bad = []
    for i, (r, q, f, h, b) in enumerate(probs):
        e = oracle.align(r, q, f, h, b)
        if got[i] != e:
            bad.append((i, got[i], e, h, b, len(r), len(f)))
    assert not bad, f"{len(bad)} mismatches, first: {bad[:3]}"


def test_align_empty_inputs(M, oracle):
    probs = [(b"", b"", b"ACGT", 0, 30), (b"ACGT", b"\x1e" * 4, b"", 0, 30), (b"A", b"\x1e", b"A", 0, 0)]
    got = M.align_batch(probs)
    for p, g in zip(probs, got):
        assert g == oracle.align(*p)


def test_window_wait_limit_gives_an_error(M, oracle):
    """The whole-window DP's warps wait for their left neighbour with a
    bounded spin. With the poll limit lowered to 1 the waits of multi-tile
    windows give up: the call returns PBW_ERR_DEVICE with its reason instead
    of hanging, and the handle maps correctly again once the limit is back."""
    import probebwa_gb300 as P
    probs = _problems(14, 40, "window")
    M.set_tuning(wait_polls=1)
    try:
        with pytest.raises(P.PbwError, match="wavefront wait"):
            M.align_batch(probs)
    finally:
        M.set_tuning(wait_polls=0)
    assert M.tuning()["wait_polls"] == 0
    got = M.align_batch(probs)
    assert got == [oracle.align(*p) for p in probs]
