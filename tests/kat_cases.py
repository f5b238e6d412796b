"""Known-answer scenarios restated from the reference's own tests.

Each builder regenerates the inputs of one reference test with the same
Xorshift64 generator (Marsaglia 13/7/17 shifts, bases ACGT[x % 4];
tests/mapping.rs:48-65) and returns the genome, the reads and the expected
values the reference test asserts. The same scenarios run against the CPU
oracle (test_oracle_kat.py) and the GPU path (test_gpu_kat.py).
"""
from __future__ import annotations

MASK64 = (1 << 64) - 1


class Xorshift64:
    """tests/mapping.rs:48-65."""

    def __init__(self, seed: int):
        self.s = seed & MASK64

    def next_u64(self) -> int:
        x = self.s
        x ^= (x << 13) & MASK64
        x ^= x >> 7
        x ^= (x << 17) & MASK64
        self.s = x
        return x

    def gen_seq(self, n: int) -> str:
        return "".join("ACGT"[self.next_u64() % 4] for _ in range(n))


def revcomp(s: str) -> str:
    """tests/mapping.rs:31-35."""
    m = {"A": "T", "T": "A", "C": "G", "G": "C"}
    return "".join(m.get(c, "N") for c in reversed(s))


def q40(seq: str) -> bytes:
    """FASTQ 'I' qualities (Phred+33 -> 40), tests/mapping.rs:21-29."""
    return bytes([40] * len(seq))


def fwd_rev():
    """test_forward_and_reverse_strand_mapping (tests/mapping.rs:67-103)."""
    g = Xorshift64(42).gen_seq(400)
    reads = [("fwd", g[40:80]), ("rev", revcomp(g[200:240]))]
    expect = [dict(pos=41, rev=False, cigar="40M", mapq=80), dict(pos=201, rev=True, cigar="40M", mapq=80)]
    return [("chr1", g)], reads, expect


def mismatch_del_garbage():
    """test_mismatch_deletion_and_unmapped (tests/mapping.rs:105-160)."""
    g = Xorshift64(7).gen_seq(400)
    base = g[40:80]
    mm = list(base)
    mm[10] = "C" if mm[10] == "A" else "A"
    reads = [("mismatch", "".join(mm)), ("del", base[0:20] + base[22:]), ("garbage", "T" * 40)]
    return [("chr1", g)], reads


def large_deletion():
    """test_large_deletion_is_found (tests/mapping.rs:171-193)."""
    g = Xorshift64(555).gen_seq(500)
    w = g[100:160]
    return [("chr1", g)], [("bigdel", w[:25] + w[50:])]


def paired_fr_ff():
    """test_paired_end_proper_and_improper (tests/mapping.rs:195-233)."""
    g = Xorshift64(99).gen_seq(400)
    fr = (g[40:80], revcomp(g[200:240]))
    ff = (g[40:80], g[200:240])
    return [("chr1", g)], fr, ff


def large_contig():
    """test_large_contig_positions (tests/mapping.rs:240-258)."""
    g = Xorshift64(2024).gen_seq(80_000)
    return [("chr1", g)], [("deep", g[70_000:70_050])]


def mate_rescue():
    """test_mate_rescue_recovers_unseedable_mate (tests/mapping.rs:267-302)."""
    g = Xorshift64(2468).gen_seq(400)
    m1 = g[40:80]
    m2 = list(revcomp(g[200:240]))
    for p in range(0, len(m2), 6):
        m2[p] = next(b for b in "ACGT" if b != m2[p])
    return [("chr1", g)], m1, "".join(m2)


def n_run():
    """test_n_run_round_trip (tests/mapping.rs:304-334)."""
    rng = Xorshift64(7)
    left = rng.gen_seq(100)
    right = rng.gen_seq(100)
    g = left + "N" * 20 + right
    return [("chrN", g)], [("in_gap", g[105:135]), ("right_unique", g[150:190])]


def synthetic_accuracy():
    """test_synthetic_scale_mapping_accuracy (tests/mapping.rs:342-394)."""
    rng = Xorshift64(12345)
    glen, rlen, n = 20_000, 60, 300
    g = rng.gen_seq(glen)
    reads, truth = [], []
    for i in range(n):
        start = rng.next_u64() % (glen - rlen)
        b = list(g[start:start + rlen])
        if rng.next_u64() % 10 < 3:
            p = rng.next_u64() % rlen
            b[p] = next(x for x in "ACGT" if x != b[p])
        s = "".join(b)
        rev = rng.next_u64() % 2 == 0
        if rev:
            s = revcomp(s)
        reads.append((f"r{i}", s))
        truth.append((start + 1, rev))
    return [("chr1", g)], reads, truth


def repeat_disambiguation():
    """test_paired_disambiguates_repeat_copy_via_anchor (tests/mapping.rs:421-507)."""
    rng = Xorshift64(2026)
    unique_a = rng.gen_seq(100)
    spacer = rng.gen_seq(110)
    unit = rng.gen_seq(100)
    filler = rng.gen_seq(10_000)
    diff = 20
    tc = list(unit)
    tc[diff] = {"A": "C", "C": "A", "G": "T"}.get(tc[diff], "G")
    true_copy = "".join(tc)
    g = unique_a + spacer + true_copy + filler + unit
    true_pos = len(unique_a) + len(spacer)
    decoy_pos = len(g) - len(unit)
    r1 = unique_a[0:40]
    q1 = bytes([35] * 40)
    r2 = revcomp(unit[0:40])
    q2 = [35] * 40
    q2[39 - diff] = 10
    return [("chr1", g)], (r1, q1), (r2, bytes(q2)), true_pos, decoy_pos


def adapter_strip():
    """test_adapter_strip_trims_3prime_readthrough (tests/cli.rs:112-146)."""
    g = Xorshift64(101).gen_seq(400)
    adapter = "AGATCGGAAGAGCACACGTC"
    return [("chr1", g)], g[40:80] + adapter, adapter
