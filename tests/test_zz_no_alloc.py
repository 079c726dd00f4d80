"""pq_suffix_sort_static: the suffix sort for callers that cannot allocate device memory.

Called through the C ABI with caller-owned device buffers (torch tensors here), twice in a row on
each input, and compared with the allocating entry point (pq_sort + pq_get_sa) on the same reads.
Suffix arrays are integer data: the comparison is exact.  Around the second call of each input
(the first one has loaded every kernel that input needs) the device's free memory must not move:
the entry point allocates nothing.  The inputs cover reads longer and shorter than the sort's
14-base key, and an output suffix array that does not start on a 16-byte boundary.  This file is
collected last so that a run stopping at the first failure has run every other test already.
"""
import ctypes as ct

import numpy as np
import pytest

import pasqual_gb300 as pq
from pasqual_gb300 import synth

pytestmark = pytest.mark.gpu

MAX_SUFFIXES = 1 << 20   # PQ_STATIC_SORT_MAX_SUFFIXES


def static_sort_fn(width):
    lib = pq.load_library(width)
    f = lib.pq_suffix_sort_static
    f.restype = ct.c_int
    f.argtypes = [ct.c_void_p, ct.c_uint64 if width == 64 else ct.c_uint32, ct.c_int, ct.c_int,
                  ct.c_void_p, ct.c_void_p]
    return f


def reference_sa(reads, t, width, direction):
    with pq.Pasqual(width) as P:
        P.set_reads(reads, t)
        P.sort(direction)
        return P.get_sa(direction)


def cases():
    """(reads, t, direction, output offset in entries)."""
    return [
        (synth.reads_for_coverage(synth.genome(30000, 0.41, 0.1, (0.01, 0.01), seed=3), 100, 25,
                                  0.005, seed=4), 63, 0, 0),
        (synth.reads_for_coverage(synth.genome(20000, 0.5, seed=5), 60, 30, 0.0, seed=6), 31, 1, 0),
        # reads no longer than the 14-base key: the sort ends after its radix passes
        (synth.reads_for_coverage(synth.genome(8000, 0.5, seed=7), 12, 20, 0.0, seed=8), 10, 0, 0),
        # suffix array one entry past a 16-byte boundary
        (synth.reads_for_coverage(synth.genome(15000, 0.45, 0.05, (0.01, 0.01), seed=9), 80, 20,
                                  0.003, seed=10), 47, 1, 1),
    ]


@pytest.mark.parametrize("width", [32, 64])
def test_static_sort_matches_allocating_sort_twice(width):
    import torch
    f = static_sort_fn(width)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    tdt = torch.int64 if width == 64 else torch.int32
    ndt = np.uint64 if width == 64 else np.uint32
    work = []
    for reads, t, direction, off in cases():
        reads = np.ascontiguousarray(reads[: MAX_SUFFIXES // reads.shape[1]])
        work.append((reads, direction, off, reference_sa(reads, t, width, direction)))
    for reads, direction, off, want in work:
        n = reads.size
        d_reads = torch.from_numpy(reads).to(dev)
        d_sa = torch.empty((n + off,), dtype=tdt, device=dev)
        ptr = d_sa.data_ptr() + off * d_sa.element_size()
        for call in range(2):
            d_sa.fill_(-1)
            torch.cuda.synchronize(dev)
            free_before = torch.cuda.mem_get_info(dev)[0]
            rc = f(d_reads.data_ptr(), reads.shape[0], reads.shape[1], direction, ptr,
                   stream.cuda_stream)
            assert rc == 0
            free_after = torch.cuda.mem_get_info(dev)[0]   # the call has synchronised its stream
            got = d_sa[off:].cpu().numpy().view(ndt)
            assert np.array_equal(got, want), "call %d" % call
            if call == 1:
                assert free_after == free_before, "device memory moved: %d bytes" % (free_before - free_after)


def test_static_sort_rejects_bad_codes():
    """A byte that is not a base code 1..4 is refused before sorting (it would corrupt the 2-bit
    packing), and the next valid call still sorts correctly."""
    import torch
    f = static_sort_fn(32)
    dev = torch.device("cuda", 0)
    reads = synth.reads_for_coverage(synth.genome(5000, 0.5, seed=11), 50, 10, 0.0, seed=12)
    want = reference_sa(reads, 31, 32, 0)
    bad = reads.copy()
    bad[7, 13] = 0
    d_sa = torch.empty((reads.size,), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    assert f(torch.from_numpy(bad).to(dev).data_ptr(), bad.shape[0], 50, 0, d_sa.data_ptr(), stream) == 1
    assert f(torch.from_numpy(reads).to(dev).data_ptr(), reads.shape[0], 50, 0, d_sa.data_ptr(), stream) == 0
    assert np.array_equal(d_sa.cpu().numpy().view(np.uint32), want)


def test_static_sort_rejects_oversize():
    f = static_sort_fn(32)
    # rejected before any device access: the pointers are never dereferenced
    assert f(None, MAX_SUFFIXES // 100 + 1, 100, 0, None, None) == 6   # PQ_ERR_CAPACITY
