"""Shared helpers for the GPU parity tests (GPU path vs the CPU oracle)."""
from __future__ import annotations

import numpy as np

RECORD_KEYS_EXACT = ("contig", "pos", "mapq", "flag", "mate_contig", "mate_pos", "tlen", "as_score", "nm")


def cuda_available() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def to_oracle_reads(O, R):
    return O.Reads(R.bases, R.quals, R.offsets, R.ids)


def compare_records(P, O, got: dict, exp: dict, label: str = "", posterior_ulps: int = 4):
    """Bit-exact on every integer field, the CIGAR and the log-likelihood bits;
    posterior within a few ulps (its last step is pow(10, -phred/10) of a
    continuous phred)."""
    n = len(exp["contig"])
    bad = []
    for k in RECORD_KEYS_EXACT:
        d = np.nonzero(got[k][:n] != exp[k][:n])[0]
        if len(d):
            bad.append((k, d[:10].tolist(), got[k][d[:3]].tolist(), exp[k][d[:3]].tolist()))
    gl = got["log_lk"][:n].view(np.uint64)
    el = exp["log_lk"][:n].view(np.uint64)
    d = np.nonzero(gl != el)[0]
    if len(d):
        bad.append(("log_lk", d[:10].tolist(), got["log_lk"][d[:3]].tolist(), exp["log_lk"][d[:3]].tolist()))
    gp = got["posterior"][:n]
    ep = exp["posterior"][:n]
    tol = posterior_ulps * np.spacing(np.maximum(np.abs(ep), 1e-300))
    d = np.nonzero(np.abs(gp - ep) > tol)[0]
    if len(d):
        bad.append(("posterior", d[:10].tolist(), gp[d[:3]].tolist(), ep[d[:3]].tolist()))
    gc = P.cigar_strings(got)
    ec = O.cigar_strings(exp)
    d = [i for i in range(n) if gc[i] != ec[i]]
    if d:
        bad.append(("cigar", d[:10], [gc[i] for i in d[:3]], [ec[i] for i in d[:3]]))
    assert not bad, f"{label}: GPU/oracle mismatch: {bad}"
