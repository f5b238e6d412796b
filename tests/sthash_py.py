"""Numpy readers for the bincode .stidx / .sthash index files.

bincode 1.3.3 legacy encoding: fixint little-endian, u64 lengths
(src/index/genome.rs:72-77, src/index/hashtable.rs:60-70). Test helper used
to inspect index files written by either builder.
"""
from __future__ import annotations

import struct

import numpy as np


def read_sthash(path: str):
    data = open(path, "rb").read()
    p = 0
    (n,) = struct.unpack_from("<Q", data, p)
    p += 8
    tab = np.frombuffer(data, dtype=np.uint32, count=3 * n, offset=p).reshape(n, 3)
    p += 12 * n
    (npos,) = struct.unpack_from("<Q", data, p)
    p += 8
    pos = np.frombuffer(data, dtype=np.uint64, count=npos, offset=p)
    p += 8 * npos
    k, stride, total = struct.unpack_from("<QQQ", data, p)
    return {"keys": tab[:, 0].copy(), "off": tab[:, 1].copy(), "cnt": tab[:, 2].copy(), "positions": pos.copy(),
            "k": k, "stride": stride, "total": total}


def read_stidx(path: str):
    data = open(path, "rb").read()
    p = 0

    def u64():
        nonlocal p
        (v,) = struct.unpack_from("<Q", data, p)
        p += 8
        return v

    def string():
        nonlocal p
        n = u64()
        s = data[p:p + n].decode()
        p += n
        return s

    species = string()
    assembly = string()
    contigs = []
    for _ in range(u64()):
        name = string()
        npk = u64()
        packed = np.frombuffer(data, np.uint8, count=npk, offset=p).copy()
        p += npk
        nr = u64()
        runs = np.frombuffer(data, np.uint32, count=2 * nr, offset=p).reshape(nr, 2).copy()
        p += 8 * nr
        length = u64()
        contigs.append({"name": name, "packed": packed, "n_runs": runs, "length": length})
    total = u64()
    return {"species": species, "assembly": assembly, "contigs": contigs, "total_length": total}


def mix32(h: int) -> int:
    """src/index/hashtable.rs:117-124."""
    M = 0xFFFFFFFF
    h ^= h >> 16
    h = (h * 0x7FEB352D) & M
    h ^= h >> 15
    h = (h * 0x846CA68B) & M
    h ^= h >> 16
    return h


def hash_kmer(kmer: str) -> int:
    """src/index/hashtable.rs:107-113."""
    raw = 0
    for c in kmer[:15]:
        raw = ((raw << 2) | {"A": 0, "C": 1, "G": 2, "T": 3}.get(c.upper(), 0)) & 0xFFFFFFFF
    return mix32(raw)


def unpack(p: int):
    """src/index/hashtable.rs:166-171 -> (contig, pos, reverse)."""
    return (p >> 40) & ((1 << 23) - 1), p & ((1 << 40) - 1), bool((p >> 63) & 1)


def bucket(ht, kmer: str):
    h = hash_kmer(kmer)
    idx = np.nonzero(ht["keys"] == h)[0]
    if len(idx) == 0:
        return []
    i = idx[0]
    return [int(x) for x in ht["positions"][ht["off"][i]:ht["off"][i] + ht["cnt"][i]]]
