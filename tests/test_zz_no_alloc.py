"""The allocation-free alignment entry point (pbw_align_noalloc) against the
regular one (pbw_align_batch) on the same problems.

pbw_align_noalloc serves callers that must not call cudaMalloc: a host
application whose own allocator has reserved the GPU's memory, or a loop
with a fixed device-memory budget. All its scratch sits in a static device
array. Its inputs and outputs here are device buffers that the test
allocates. Two calls in a row check that the reused scratch carries nothing
from one call into the next, and the device's free memory is read around the
second call to check that the call itself allocates nothing. Collected last
on purpose."""
from __future__ import annotations

import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _problems(seed, n):
    rng = np.random.default_rng(seed)
    out = []
    for k in range(n):
        L = int(rng.integers(20, 200))
        if k % 2 == 0:  # seeded window: band 30, hint 10
            ref = rng.choice(list(b"ACGT"), size=L + 40).astype(np.uint8)
            s = int(rng.integers(0, 21))
            read = ref[s:s + L].copy()
            hint, band = 10, 30
        else:  # whole-window alignment
            rad = int(rng.integers(L, L + 200))
            ref = rng.choice(list(b"ACGT"), size=min(L + 2 * rad, 2048)).astype(np.uint8)
            s = int(rng.integers(0, max(1, len(ref) - L)))
            read = ref[s:s + L].copy()
            hint, band = min(s, rad), len(ref)
        m = rng.random(len(read)) < 0.03
        read[m] = rng.choice(list(b"ACGT"), size=int(m.sum())).astype(np.uint8)
        if rng.random() < 0.3:
            p = int(rng.integers(1, len(read) - 1))
            read = np.concatenate([read[:p], read[p + int(rng.integers(1, 4)):]])
        qual = rng.integers(2, 42, size=len(read)).astype(np.uint8)
        out.append((read.tobytes(), qual.tobytes(), ref.tobytes(), hint, band))
    return out


def test_noalloc_matches_align_batch(tmp_path):
    torch = pytest.importorskip("torch")
    import probebwa_gb300 as P
    from probebwa_gb300 import synth
    P.build()
    probs = _problems(123, 600)
    prefix = str(tmp_path / "g")
    synth.write_index(prefix, synth.contigs_from_strings([("c", "ACGT" * 50)]))
    with P.Mapper(prefix) as m:
        expected = m.align_batch(probs)
    n = len(probs)
    ro = np.zeros(n + 1, np.uint64)
    fo = np.zeros(n + 1, np.uint64)
    ro[1:] = np.cumsum([len(p[0]) for p in probs])
    fo[1:] = np.cumsum([len(p[2]) for p in probs])
    dev = torch.device("cuda", 0)

    def d(a):
        return torch.from_numpy(np.array(a, copy=True)).to(dev)

    reads = d(np.frombuffer(b"".join(p[0] for p in probs), np.uint8))
    quals = d(np.frombuffer(b"".join(p[1] for p in probs), np.uint8))
    refs = d(np.frombuffer(b"".join(p[2] for p in probs), np.uint8))
    read_off = d(ro.view(np.int64))
    ref_off = d(fo.view(np.int64))
    hint = d(np.array([p[3] for p in probs], np.int64))
    band = d(np.array([p[4] for p in probs], np.uint64).view(np.int64))
    stride = 512
    stream = torch.cuda.current_stream(dev)
    L = P.lib()
    for call in range(2):
        score = torch.full((n,), -7, dtype=torch.int32, device=dev)
        offset = torch.zeros(n, dtype=torch.int64, device=dev)
        n_ops = torch.zeros(n, dtype=torch.int32, device=dev)
        cigar = torch.zeros(n * stride, dtype=torch.int32, device=dev)
        torch.cuda.synchronize(dev)
        free_before = torch.cuda.mem_get_info(dev)[0]
        rc = L.pbw_align_noalloc(n, reads.data_ptr(), quals.data_ptr(), read_off.data_ptr(), refs.data_ptr(),
                                 ref_off.data_ptr(), hint.data_ptr(), band.data_ptr(), 40, 3, score.data_ptr(),
                                 offset.data_ptr(), n_ops.data_ptr(), cigar.data_ptr(), stride,
                                 C.c_void_p(stream.cuda_stream))
        assert rc == 0, L.pbw_last_error(None).decode()
        if call == 1:  # the first call's module loading is behind us
            assert torch.cuda.mem_get_info(dev)[0] == free_before, "the call changed the device's free memory"
        sc = score.cpu().numpy()
        of = offset.cpu().numpy()
        no = n_ops.cpu().numpy()
        cg = cigar.cpu().numpy().view(np.uint32).reshape(n, stride)
        for i, (es, ec, eo) in enumerate(expected):
            cig = "".join(f"{int(w) >> 4}{'MIDXSH'[int(w) & 15]}" for w in cg[i, :no[i]])
            assert (int(sc[i]), cig, int(of[i])) == (es, ec, eo), (call, i)


def test_noalloc_rejects_oversized_inputs():
    torch = pytest.importorskip("torch")
    import probebwa_gb300 as P
    P.build()
    L = P.lib()
    dev = torch.device("cuda", 0)
    z = torch.zeros(16, dtype=torch.int64, device=dev)
    rc = L.pbw_align_noalloc(5000, z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(), z.data_ptr(),
                             z.data_ptr(), z.data_ptr(), 40, 3, z.data_ptr(), z.data_ptr(), z.data_ptr(),
                             z.data_ptr(), 8, None)
    assert rc == -6 and b"at most 4096" in L.pbw_last_error(None)


def _device_problems(torch, dev, probs):
    n = len(probs)
    ro = np.zeros(n + 1, np.uint64)
    fo = np.zeros(n + 1, np.uint64)
    ro[1:] = np.cumsum([len(p[0]) for p in probs])
    fo[1:] = np.cumsum([len(p[2]) for p in probs])

    def d(a):
        return torch.from_numpy(np.array(a, copy=True)).to(dev)

    return (d(np.frombuffer(b"".join(p[0] for p in probs), np.uint8)),
            d(np.frombuffer(b"".join(p[1] for p in probs), np.uint8)),
            d(ro.view(np.int64)), d(np.frombuffer(b"".join(p[2] for p in probs), np.uint8)),
            d(fo.view(np.int64)), d(np.array([p[3] for p in probs], np.int64)),
            d(np.array([p[4] for p in probs], np.uint64).view(np.int64)))


def test_noalloc_device_side_limits():
    """A 300-base read (limit 256) is caught on the device: PBW_ERR_LIMIT,
    while the problems within the limits are still aligned; a CIGAR longer
    than cigar_stride gives PBW_ERR_CAPACITY."""
    torch = pytest.importorskip("torch")
    import probebwa_gb300 as P
    P.build()
    L = P.lib()
    dev = torch.device("cuda", 0)
    probs = _problems(7, 40)
    rng = np.random.default_rng(8)
    ref = rng.choice(list(b"ACGT"), size=400).astype(np.uint8)
    long_read = ref[20:320].tobytes()
    probs[5] = (long_read, bytes([30] * 300), ref.tobytes(), 20, 400)
    args = _device_problems(torch, dev, probs)
    n = len(probs)
    stride = 512
    score = torch.full((n,), -7, dtype=torch.int32, device=dev)
    offset = torch.zeros(n, dtype=torch.int64, device=dev)
    n_ops = torch.zeros(n, dtype=torch.int32, device=dev)
    cigar = torch.zeros(n * stride, dtype=torch.int32, device=dev)
    outs = (score.data_ptr(), offset.data_ptr(), n_ops.data_ptr(), cigar.data_ptr())
    ptrs = [a.data_ptr() for a in args]
    rc = L.pbw_align_noalloc(n, *ptrs, 40, 3, *outs, stride, None)
    assert rc == -6, rc
    assert b"longer than 256" in L.pbw_last_error(None)
    assert int(n_ops[5].item()) == 0
    ok = [i for i in range(n) if i != 5]
    assert (score.cpu().numpy()[ok] != -7).all(), "problems within the limits are aligned"
    # the same problems without the long read, with room for 1 operation per CIGAR
    probs[5] = probs[4]
    args = _device_problems(torch, dev, probs)
    ptrs = [a.data_ptr() for a in args]
    rc = L.pbw_align_noalloc(n, *ptrs, 40, 3, *outs, 1, None)
    assert rc == -7 and b"cigar_stride" in L.pbw_last_error(None)
    # and a clean call afterwards: the error word does not leak into it
    rc = L.pbw_align_noalloc(n, *ptrs, 40, 3, *outs, stride, None)
    assert rc == 0, L.pbw_last_error(None).decode()
