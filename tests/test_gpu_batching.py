"""Batching on the GPU (no counterpart in the reference): the 16-lane form
of the seeded band DP, the length-binned work queue, the autotuner's
choice and the per-batch CUDA graphs of the paired path must all give the
records of the plain, untuned path, which the oracle pins."""
from __future__ import annotations

import numpy as np
import pytest

from gpu_helpers import compare_records, to_oracle_reads

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def _same(a, b):
    for k in ("contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen", "as_score", "nm", "cigar_off"):
        assert np.array_equal(a[k], b[k]), k
    n = int(a["cigar_off"][-1])
    assert np.array_equal(a["cigar"][:n], b["cigar"][:n])
    assert np.array_equal(a["log_lk"].view(np.uint64), b["log_lk"].view(np.uint64))
    assert np.array_equal(a["posterior"].view(np.uint64), b["posterior"].view(np.uint64))


def _mixed_reads(P, contigs, seed, n_per=300):
    from probebwa_gb300 import synth
    seqs, quals = [], []
    for i, L in enumerate(range(60, 251, 19)):
        s, q, _ = synth.reads_single(seed + i, contigs, n=n_per, L=L)
        seqs += s
        quals += q
    rng = np.random.default_rng(seed)
    order = rng.permutation(len(seqs))
    return P.Reads.from_lists([seqs[i] for i in order], [quals[i] for i in order])


def test_band_dp_16_lanes_matches_oracle(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(101, length=300_000, n_copies=20, copy_len=1000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    R = _mixed_reads(P, contigs, 102, n_per=150)
    with P.Mapper(prefix) as m:
        m.set_tuning(band_lanes=16, autotune=0)
        got16 = m.map_single(R)
        m.set_tuning(band_lanes=8, autotune=0)
        got8 = m.map_single(R)
    om = oracle.Mapper(prefix)
    exp = om.map_single(to_oracle_reads(oracle, R))
    compare_records(P, oracle, got16, exp, "16 lanes")
    _same(got16, got8)


@pytest.mark.parametrize("band", [30, 20, 17, 10])
def test_band_dp_4_lanes_matches_oracle(P, oracle, tmp_path, band):
    """4 lanes of 16 columns (bands 16-31; the last band column 2*band + 1
    sits at lane position 13, 9 and 3 for bands 30, 20 and 17); band 10 has
    no 4-lane form and runs the 8-lane one."""
    from probebwa_gb300 import synth
    contigs = synth.genome_single(105 + band, length=300_000, n_copies=20, copy_len=1000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    R = _mixed_reads(P, contigs, 106 + band, n_per=120)
    with P.Mapper(prefix, options=P.MapperOptions(max_indel_len=band)) as m:
        m.set_tuning(band_lanes=4, autotune=0)
        got4 = m.map_single(R)
        m.set_tuning(band_lanes=8, autotune=0)
        got8 = m.map_single(R)
    om = oracle.Mapper(prefix, max_indel_len=band)
    exp = om.map_single(to_oracle_reads(oracle, R))
    om.close()
    compare_records(P, oracle, got4, exp, f"4 lanes, band {band}")
    _same(got4, got8)


def test_length_bins_and_autotune_keep_records(P, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(103, length=500_000, n_copies=30, copy_len=1500)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    R = _mixed_reads(P, contigs, 104)
    with P.Mapper(prefix, chunk_reads=997) as m:
        m.set_tuning(length_bins=0, autotune=0, band_lanes=8)
        base = m.map_single(R)
        m.set_tuning(length_bins=1, autotune=1, band_lanes=0)
        tuned = m.map_single(R)
        t = m.tuning()
        again = m.map_single(R)
    _same(base, tuned)
    _same(base, again)
    # reads of 60-250 bases: the <= 256 class (and the <= 128 one) got a form
    # (the default band, 30, has all three forms)
    assert t["chosen_lanes"][1] in (4, 8, 16) and min(t["tuned_ms"][1]) > 0, t


def test_pair_graphs_keep_records(P, oracle, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_paired(105, n_contigs=3, contig_len=300_000)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    a1, b1, a2, b2, _ = synth.reads_paired(106, contigs, 2600, L=150, mean=350, sd=50)
    R1, R2 = P.Reads.from_lists(a1, b1), P.Reads.from_lists(a2, b2)
    with P.Mapper(prefix, chunk_reads=2000) as m:
        m.set_tuning(pair_graphs=0)
        d1, d2, dm = m.map_paired(R1, R2)
        m.set_tuning(pair_graphs=1)
        g1, g2, gm = m.map_paired(R1, R2)
    _same(d1, g1)
    _same(d2, g2)
    assert dm == gm
    om = oracle.Mapper(prefix)
    e1, e2, em = om.map_paired(to_oracle_reads(oracle, R1), to_oracle_reads(oracle, R2))
    compare_records(P, oracle, g1, e1, "graphs mate 1")
    compare_records(P, oracle, g2, e2, "graphs mate 2")
