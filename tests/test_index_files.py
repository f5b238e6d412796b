"""The product's index writer (probebwa_gb300.synth) against the oracle's
restatement of GenomeIndex::save / HashTableBuilder::build: byte-identical
.stidx and .sthash files."""
import numpy as np

import kat_cases as K
from probebwa_gb300 import synth


def _cases():
    yield "kat_fwdrev", K.fwd_rev()[0]
    yield "nrun", K.n_run()[0]
    g = synth.genome_single(7, length=60_000, n_copies=5, copy_len=800)
    yield "repeats", [(n, bytes(synth.ASCII[c])) for n, c in g]
    yield "lower_and_iupac", [("c1", "acgtNNNNRYacgtacgtacgtacgtacgtACGTAAAAAAAAAAAAAAAAAAAAAAAAAAA" * 3),
                              ("c2", "ACG"), ("c3", "")]
    yield "tandem", [("c1", "ACGTACGTACGTACG" * 400)]


def test_index_files_match_oracle(oracle, tmp_path):
    for name, contigs in _cases():
        contigs = [(n, s.decode() if isinstance(s, bytes) else s) for n, s in contigs]
        a = str(tmp_path / f"{name}_oracle")
        oracle.build_index(a, contigs)
        b = str(tmp_path / f"{name}_product")
        synth.write_index(b, synth.contigs_from_strings(contigs))
        # species/assembly strings differ by design; compare from the contig list on
        sa = open(a + ".stidx", "rb").read()
        sb = open(b + ".stidx", "rb").read()
        import sthash_py as SH
        ia, ib = SH.read_stidx(a + ".stidx"), SH.read_stidx(b + ".stidx")
        assert [c["name"] for c in ia["contigs"]] == [c["name"] for c in ib["contigs"]]
        for ca, cb in zip(ia["contigs"], ib["contigs"]):
            assert ca["length"] == cb["length"]
            assert np.array_equal(ca["packed"], cb["packed"]), name
            assert np.array_equal(ca["n_runs"], cb["n_runs"]), name
        assert ia["total_length"] == ib["total_length"]
        assert open(a + ".sthash", "rb").read() == open(b + ".sthash", "rb").read(), name
        del sa, sb


def test_oracle_direct_address_load_maps_the_same(oracle, tmp_path):
    """Large .sthash tables load into the oracle as a direct-address array
    over the 32-bit hash (filled by every host thread) instead of the
    open-addressed map; forced here on a small genome, both loads must map
    every read identically."""
    import numpy as np
    from probebwa_gb300 import synth
    contigs = synth.genome_single(61, length=120_000, n_copies=6, copy_len=800)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, contigs)
    seqs, quals, _ = synth.reads_single(62, contigs, n=300, L=100, sub=0.01, indel=0.001)
    R = oracle.Reads.from_lists(seqs, quals)
    a = oracle.Mapper(prefix).map_single(R)
    b = oracle.Mapper(prefix, dense_min_buckets=0).map_single(R)
    for k in ("contig", "pos", "mapq", "flag", "as_score", "nm"):
        assert np.array_equal(a[k], b[k]), k
    assert np.array_equal(a["log_lk"].view(np.uint64), b["log_lk"].view(np.uint64))
    assert oracle.cigar_strings(a) == oracle.cigar_strings(b)


def test_hg_scale_generator_small_case(tmp_path):
    """The tensor generator of the hg38-scale workloads, run small on the
    CPU: base composition, repeat content, the device 2-bit packing of
    write_stidx against the numpy reader, and read shapes and ranges."""
    pytest = __import__("pytest")
    pytest.importorskip("torch")
    from probebwa_gb300 import synth_gpu as S
    names, lens, codes = S.genome_hg(5, total=3_000_000, n_contigs=4, device="cpu")
    assert len(codes) == int(np.sum(lens)) and codes.max() < 4
    frac = np.bincount(codes, minlength=4) / len(codes)
    assert abs(frac[0] - 0.295) < 0.01 and abs(frac[1] - 0.205) < 0.01
    prefix = str(tmp_path / "hg")
    S.write_stidx(prefix, names, lens, codes, device="cpu")
    back = synth.read_stidx_contigs(prefix)
    for (n1, c1), (n2, c2) in zip(back, S.contigs_of(names, lens, codes)):
        assert n1 == n2 and np.array_equal(c1, c2)
    b, q, o = S.reads(6, names, lens, codes, 500, 250, trim=(60, 250), device="cpu")
    ln = np.diff(o.astype(np.int64))
    assert len(ln) == 500 and ln.min() >= 60 and ln.max() <= 250 and len(b) == o[-1]
    assert q.min() >= 2 and q.max() <= 41 and set(np.unique(b).tolist()) <= set(b"ACGT")
    r = S.reads(7, names, lens, codes, 300, 150, paired=True, mean=350.0, sd=50.0, device="cpu")
    assert len(r) == 6 and np.array_equal(r[2], r[5]) and r[2][-1] == 300 * 150
    stressed, regions = S.add_stress(8, codes, lens, n_families=5, hp_region_bp=200_000, device="cpu")
    assert (stressed != codes).any() and len(regions) == 6
