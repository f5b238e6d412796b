"""Two handles mapping at once from two host threads (a single-end call and a
paired call on the same GPU, as the benchmark issues them): the records are
those of the same calls made one after the other, and the calls' compute
spans on the device clock overlap."""
from __future__ import annotations

import threading

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def P():
    import probebwa_gb300 as P
    P.build()
    return P


def _records_equal(a, b, label):
    for k in ("contig", "pos", "mapq", "flag", "as_score", "nm", "cigar_off"):
        assert np.array_equal(a[k], b[k]), (label, k)
    n = int(a["cigar_off"][-1])
    assert np.array_equal(a["cigar"][:n], b["cigar"][:n]), label
    assert np.array_equal(a["log_lk"].view(np.uint64), b["log_lk"].view(np.uint64)), label


def test_single_and_paired_handles_at_once(P, tmp_path):
    from probebwa_gb300 import synth
    contigs = synth.genome_single(41, length=400_000, n_copies=20, copy_len=1500)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(42, contigs, n=6000, L=150, sub=0.01, indel=0.001)
    s1, q1, s2, q2, _ = synth.reads_paired(43, contigs, 4000, L=150)
    RS = P.Reads.from_lists(seqs, quals)
    R1, R2 = P.Reads.from_lists(s1, q1), P.Reads.from_lists(s2, q2)
    with P.Mapper(prefix, chunk_reads=2000) as ms, P.Mapper(prefix, chunk_reads=2000) as mp:
        seq_se = ms.map_single(RS)
        seq_p1, seq_p2, seq_model = mp.map_paired(R1, R2)
        out, err = {}, []

        def run_se():
            try:
                out["se"] = ms.map_single(RS)
                out["se_st"] = ms.stats()
            except Exception as e:  # surfaced in the main thread
                err.append(e)

        def run_pe():
            try:
                out["pe"] = mp.map_paired(R1, R2)
                out["pe_st"] = mp.stats()
            except Exception as e:
                err.append(e)

        for _ in range(2):
            th = [threading.Thread(target=run_se), threading.Thread(target=run_pe)]
            for t in th:
                t.start()
            for t in th:
                t.join()
            assert not err, err
            _records_equal(out["se"], seq_se, "single-end")
            p1, p2, model = out["pe"]
            _records_equal(p1, seq_p1, "mate 1")
            _records_equal(p2, seq_p2, "mate 2")
            assert model == seq_model
            for k in ("se_st", "pe_st"):
                st = out[k]
                assert st["t_compute_end_ms"] > st["t_compute_begin_ms"] >= 0.0
                assert abs((st["t_compute_end_ms"] - st["t_compute_begin_ms"]) - st["ms_compute"]) < 1e-3
