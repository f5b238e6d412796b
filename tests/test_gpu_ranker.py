"""The learned candidate ranker (no counterpart in the reference) on the GPU:
its tensor-core inference against an FP32 restatement of the same BF16
network, its training on plain-path labels, and the records of ranked
mapping against the plain path on the same reads."""
from __future__ import annotations

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

RK_F, RK_H = 12, 64


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def bf16(x):
    """Round float32 to bfloat16 (nearest, ties to even), back as float32."""
    u = np.asarray(x, np.float32).view(np.uint32).astype(np.uint64)
    r = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return r.astype(np.uint32).view(np.float32)


def reference_logits(model, feat):
    norm, w = model[:2 * RK_F], model[2 * RK_F:-1]
    mean, inv = norm[:RK_F], norm[RK_F:]
    W1 = w[:RK_H * RK_F].reshape(RK_H, RK_F)
    o = RK_H * RK_F
    b1 = w[o:o + RK_H]
    o += RK_H
    W2 = w[o:o + RK_H * RK_H].reshape(RK_H, RK_H)
    o += RK_H * RK_H
    b2 = w[o:o + RK_H]
    o += RK_H
    w3 = w[o:o + RK_H]
    b3 = w[o + RK_H]
    x = bf16((feat.astype(np.float32) - mean) * inv)
    h1 = bf16(np.maximum(x.astype(np.float64) @ bf16(W1).T.astype(np.float64) + b1, 0))
    h2 = np.maximum(h1.astype(np.float64) @ bf16(W2).T.astype(np.float64) + b2, 0)
    return (h2 @ w3.astype(np.float64) + b3).astype(np.float32)


def _single_workload(tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(81, length=400_000, n_copies=40, copy_len=1500)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    return prefix, contigs


def _records_diff(a, b):
    """Reads whose primary (contig, POS, FLAG, CIGAR) or MAPQ differ."""
    n = len(a["contig"])
    diff = (a["contig"] != b["contig"]) | (a["pos"] != b["pos"]) | (a["flag"] != b["flag"]) | (a["mapq"] != b["mapq"])
    ca = [a["cigar"][a["cigar_off"][i]:a["cigar_off"][i + 1]].tobytes() for i in range(n)]
    cb = [b["cigar"][b["cigar_off"][i]:b["cigar_off"][i + 1]].tobytes() for i in range(n)]
    diff |= np.array([x != y for x, y in zip(ca, cb)])
    return np.flatnonzero(diff)


def test_ranker_inference_matches_fp32_restatement(P, tmp_path):
    from probebwa_gb300 import synth
    prefix, contigs = _single_workload(tmp_path)
    seqs, quals, _ = synth.reads_single(82, contigs, n=2000, L=120)
    R = P.Reads.from_lists(seqs, quals)
    with P.Mapper(prefix) as m:
        rep = m.ranker_train(R, epochs=2)
        assert rep["samples"] > 0 and 0 < rep["positives"] < rep["samples"]
        model = m.ranker_export()
        assert model.size == 2 * RK_F + 5057 + 1
        rng = np.random.default_rng(5)
        feat = np.abs(rng.normal(size=(1000, RK_F)).astype(np.float32)) * np.array(
            [3, 3, 3, 6, 6, 120, 35, 10, 1, 19, 20, 4], np.float32)
        feat[:, 8] = (feat[:, 8] > 0.5).astype(np.float32)
        got = m.ranker_score(feat)
    want = reference_logits(model, feat)
    # BF16 activations can round differently where the tensor core's FP32
    # sums differ in their last bits; the logits then differ by a small amount
    assert np.allclose(got, want, rtol=2e-2, atol=5e-2), np.max(np.abs(got - want))
    assert np.mean(np.abs(got - want) < 1e-3 * np.maximum(1, np.abs(want))) > 0.95


def test_ranker_single_end_against_plain(P, tmp_path):
    from probebwa_gb300 import synth
    prefix, contigs = _single_workload(tmp_path)
    s_tr, q_tr, _ = synth.reads_single(83, contigs, n=6000, L=120)
    s_ev, q_ev, _ = synth.reads_single(84, contigs, n=3000, L=120)
    Rtr = P.Reads.from_lists(s_tr, q_tr)
    Rev = P.Reads.from_lists(s_ev, q_ev)
    with P.Mapper(prefix) as m:
        plain = m.map_single(Rev)
        rep = m.ranker_train(Rtr)
        assert rep["train_recall"] >= 0.999
        m.ranker_enable(True)
        ranked = m.map_single(Rev)
        c = m.ranker_counters()
        m.ranker_enable(False)
        again = m.map_single(Rev)
    # ranker off is the plain path exactly
    assert _records_diff(plain, again).size == 0
    assert np.array_equal(plain["posterior"].view(np.uint64), again["posterior"].view(np.uint64))
    # this genome is 15% repeat copies, so many candidates are real: the
    # ranker prunes the rest
    assert c["kept"] > 0 and c["pruned"] > 0, c
    changed = _records_diff(plain, ranked)
    assert changed.size <= max(2, int(0.005 * Rev.n)), changed[:10]


def test_ranker_paired_against_plain(P, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_paired(91, n_contigs=3, contig_len=300_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    a1, b1, a2, b2, _ = synth.reads_paired(92, contigs, 3000, L=150, mean=350, sd=50)
    e1, f1, e2, f2, _ = synth.reads_paired(93, contigs, 1500, L=150, mean=350, sd=50)
    T1, T2 = P.Reads.from_lists(a1, b1), P.Reads.from_lists(a2, b2)
    E1, E2 = P.Reads.from_lists(e1, f1), P.Reads.from_lists(e2, f2)
    with P.Mapper(prefix) as m:
        p1, p2, _ = m.map_paired(E1, E2)
        m.ranker_train(T1, T2)
        model = m.ranker_export()
        m.ranker_enable(True)
        r1, r2, _ = m.map_paired(E1, E2)
        c = m.ranker_counters()
    assert c["kept"] > 0 and c["pruned"] > 0, c
    changed = np.union1d(_records_diff(p1, r1), _records_diff(p2, r2))
    assert changed.size <= max(3, int(0.01 * E1.n)), changed[:10]
    # a model moved to another handle prunes the same way
    with P.Mapper(prefix) as m2:
        m2.ranker_import(model)
        m2.ranker_enable(True)
        s1, s2, _ = m2.map_paired(E1, E2)
    assert _records_diff(r1, s1).size == 0 and _records_diff(r2, s2).size == 0


def test_ranker_paired_super_chunks(P, tmp_path):
    """Pairs in several super-chunks (chunk_reads = 2000): each super-chunk's
    seeding and seeded DP run beside the previous one's pair batches, with the
    mate feature taken from the insert model of two super-chunks before.
    Ranked records stay within 1% of the plain ones and a second call gives
    the same records."""
    from probebwa_gb300 import synth
    contigs = synth.genome_paired(95, n_contigs=3, contig_len=300_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    a1, b1, a2, b2, _ = synth.reads_paired(96, contigs, 3000, L=150, mean=350, sd=50)
    e1, f1, e2, f2, _ = synth.reads_paired(97, contigs, 4700, L=150, mean=350, sd=50)
    T1, T2 = P.Reads.from_lists(a1, b1), P.Reads.from_lists(a2, b2)
    E1, E2 = P.Reads.from_lists(e1, f1), P.Reads.from_lists(e2, f2)
    with P.Mapper(prefix, chunk_reads=2000) as m:
        p1, p2, pm = m.map_paired(E1, E2)
        m.ranker_train(T1, T2)
        m.ranker_enable(True)
        r1, r2, rm = m.map_paired(E1, E2)
        s1, s2, sm = m.map_paired(E1, E2)
    assert rm == sm
    assert _records_diff(r1, s1).size == 0 and _records_diff(r2, s2).size == 0
    changed = np.union1d(_records_diff(p1, r1), _records_diff(p2, r2))
    assert changed.size <= max(3, int(0.01 * E1.n)), changed[:10]
