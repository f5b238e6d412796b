"""The C ABI library loads and exports every entry point include/*.h declares."""
import glob
import os
import re

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    syms = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        src = open(h).read()
        src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
        for m in re.finditer(r"^[A-Za-z_][\w \*]*?\b(pbw_\w+)\s*\(", src, flags=re.M):
            syms.add(m.group(1))
    return syms


def test_library_exports_declared_symbols():
    import probebwa_gb300 as P
    P.build()
    L = P.lib()
    syms = declared_symbols()
    assert "pbw_open" in syms and "pbw_map_single" in syms
    missing = [s for s in sorted(syms) if not hasattr(L, s)]
    assert not missing, f"not exported: {missing}"


def test_records_reserve_sizes():
    """pbw_records_reserve needs no device: one record per read and a CIGAR
    capacity of 2 * bases + 2 * reads + 1."""
    import probebwa_gb300 as P
    P.build()
    R = P.Reads.from_lists([b"ACGT" * 10, b"", b"A" * 151], [b"I" * 40, b"", b"I" * 151])
    n, cap = P.Mapper.records_reserve(R)
    assert n == 3 and cap == 2 * 191 + 2 * 3 + 1
