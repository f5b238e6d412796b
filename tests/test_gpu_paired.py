"""Paired-end mapping on the GPU (joint posterior, mate rescue, 500-pair
serial warm-up + 2000-pair frozen-model batches) against the oracle and the
reference's own known answers."""
from __future__ import annotations

import numpy as np
import pytest

import kat_cases as K
from gpu_helpers import compare_records, to_oracle_reads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def _index(tmp_path, name, contigs_str):
    from probebwa_gb300 import synth
    prefix = str(tmp_path / name)
    synth.write_index(prefix, synth.contigs_from_strings(contigs_str))
    return prefix


def _pair_parity(P, oracle, prefix, R1, R2, label, **opts):
    with P.Mapper(prefix, **opts) as m:
        g1, g2, gmodel = m.map_paired(R1, R2)
    om = oracle.Mapper(prefix, **{k: v for k, v in opts.items() if k in ("group_width", "max_indel_len",
                                                                         "insert_size_mean", "insert_size_sd")})
    e1, e2, emodel = om.map_paired(to_oracle_reads(oracle, R1), to_oracle_reads(oracle, R2))
    om.close()
    compare_records(P, oracle, g1, e1, label + " mate1")
    compare_records(P, oracle, g2, e2, label + " mate2")
    assert gmodel[2] == emodel[2], (gmodel, emodel)
    assert abs(gmodel[0] - emodel[0]) <= 1e-9 * max(1.0, abs(emodel[0]))
    assert abs(gmodel[1] - emodel[1]) <= 1e-9 * max(1.0, abs(emodel[1]))
    return g1, g2


def test_kat_proper_and_improper(P, oracle, tmp_path):
    contigs, fr, ff = K.paired_fr_ff()
    prefix = _index(tmp_path, "g", contigs)
    g1, g2 = _pair_parity(P, oracle, prefix, P.Reads.from_lists([fr[0]]), P.Reads.from_lists([fr[1]]), "FR")
    assert g1["flag"][0] & 0x2 and g2["flag"][0] & 0x2 and g1["flag"][0] & 0x40 and g2["flag"][0] & 0x80
    assert g1["tlen"][0] == 200 and g2["tlen"][0] == -200
    g1, g2 = _pair_parity(P, oracle, prefix, P.Reads.from_lists([ff[0]]), P.Reads.from_lists([ff[1]]), "FF")
    assert not (g1["flag"][0] & 0x2) and not (g2["flag"][0] & 0x2)


def test_kat_mate_rescue(P, oracle, tmp_path):
    contigs, m1, m2 = K.mate_rescue()
    prefix = _index(tmp_path, "g", contigs)
    g1, g2 = _pair_parity(P, oracle, prefix, P.Reads.from_lists([m1]), P.Reads.from_lists([m2]), "rescue")
    assert g1["pos"][0] == 41 and g2["pos"][0] != 0 and g2["flag"][0] & 0x10
    assert abs(int(g2["pos"][0]) - 201) <= 5


def test_kat_repeat_disambiguation(P, oracle, tmp_path):
    contigs, (r1, q1), (r2, q2), true_pos, decoy = K.repeat_disambiguation()
    prefix = _index(tmp_path, "g", contigs)
    g1, g2 = _pair_parity(P, oracle, prefix, P.Reads.from_lists([r1], [q1]), P.Reads.from_lists([r2], [q2]),
                          "repeat")
    assert g1["pos"][0] == 1 and g2["pos"][0] == true_pos + 1
    assert g2["flag"][0] & 0x10 and g1["flag"][0] & 0x2 and g2["mapq"][0] > 0


def _paired_genome(seed, n_contigs=3, contig_len=300_000):
    from probebwa_gb300 import synth
    return synth.genome_paired(seed, n_contigs=n_contigs, contig_len=contig_len, dup_frac=0.05)


@pytest.mark.parametrize("seed,n_pairs,L,mean,sd,sub,indel", [
    (1, 3000, 150, 350.0, 50.0, 0.005, 0.0005),
    (2, 2600, 100, 300.0, 80.0, 0.02, 0.002),
    (3, 1200, 250, 500.0, 120.0, 0.03, 0.003),
])
def test_parity_synthetic_pairs(P, oracle, tmp_path, seed, n_pairs, L, mean, sd, sub, indel):
    from probebwa_gb300 import synth
    contigs = _paired_genome(10 + seed)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    s1, q1, s2, q2, _ = synth.reads_paired(20 + seed, contigs, n_pairs, L=L, mean=mean, sd=sd, sub=sub, indel=indel)
    # a few pairs whose second mate is unseedable (forces rescue) or garbage
    rng = np.random.default_rng(seed)
    for i in range(0, n_pairs, 97):
        b = bytearray(s2[i])
        for p in range(0, len(b), 6):
            b[p] = next(x for x in b"ACGT" if x != b[p])
        s2[i] = bytes(b)
    for i in range(5, n_pairs, 211):
        s1[i] = bytes(rng.choice(list(b"ACGT"), size=len(s1[i])).astype(np.uint8))
    R1 = P.Reads.from_lists(s1, q1)
    R2 = P.Reads.from_lists(s2, q2)
    g1, g2 = _pair_parity(P, oracle, prefix, R1, R2, f"pairs seed={seed}")
    assert (g1["flag"] & 0x2).astype(bool).mean() > 0.5


def test_super_chunks_are_invisible(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = _paired_genome(31, n_contigs=2, contig_len=200_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    s1, q1, s2, q2, _ = synth.reads_paired(32, contigs, 4700, L=120)
    R1 = P.Reads.from_lists(s1, q1)
    R2 = P.Reads.from_lists(s2, q2)
    _pair_parity(P, oracle, prefix, R1, R2, "chunk=2000", chunk_reads=2000)


def test_pinned_inputs_upload_per_super_chunk(P, tmp_path):
    """From pinned host memory the reads are copied up one super-chunk at a
    time while earlier super-chunks are mapped: the records are those of the
    same call from pageable memory (copied before mapping starts)."""
    torch = pytest.importorskip("torch")
    from probebwa_gb300 import synth
    contigs = _paired_genome(33, n_contigs=2, contig_len=200_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    s1, q1, s2, q2, _ = synth.reads_paired(34, contigs, 9000, L=150)
    R1 = P.Reads.from_lists(s1, q1)
    R2 = P.Reads.from_lists(s2, q2)
    keep = []

    def pinned(a):
        t = torch.empty(max(a.nbytes, 1), dtype=torch.uint8, pin_memory=True)
        keep.append(t)
        v = t.numpy()[:a.nbytes].view(a.dtype).reshape(a.shape)
        v[...] = a
        return v

    P1 = P.Reads(pinned(R1.bases), pinned(R1.quals), pinned(R1.offsets))
    P2 = P.Reads(pinned(R2.bases), pinned(R2.quals), pinned(R2.offsets))
    assert P1.bases.ctypes.data == keep[0].data_ptr()  # no copy back to pageable memory
    with P.Mapper(prefix, chunk_reads=2000) as m:
        a1, a2, am = m.map_paired(R1, R2)
        b1, b2, bm = m.map_paired(P1, P2)
        st = m.stats()
    assert am == bm
    for x, y in ((a1, b1), (a2, b2)):
        for k in ("contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen", "as_score", "nm", "cigar_off"):
            assert np.array_equal(x[k], y[k]), k
        n = int(x["cigar_off"][-1])
        assert np.array_equal(x["cigar"][:n], y["cigar"][:n])
        assert np.array_equal(x["log_lk"].view(np.uint64), y["log_lk"].view(np.uint64))
    assert st["ms_total"] > 0 and st["ms_h2d"] >= 0
