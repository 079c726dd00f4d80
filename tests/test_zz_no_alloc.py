"""pq_suffix_sort_static: the suffix sort for callers that cannot allocate device memory.

Called through the C ABI with caller-owned device buffers (torch tensors here), twice in a row
with different inputs, and compared with the allocating entry point (pq_sort + pq_get_sa) on
the same reads.  Suffix arrays are integer data: the comparison is exact.  This file is
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


@pytest.mark.parametrize("width", [32, 64])
def test_static_sort_matches_allocating_sort_twice(width):
    import torch
    f = static_sort_fn(width)
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev)
    tdt = torch.int64 if width == 64 else torch.int32
    cases = [
        (synth.reads_for_coverage(synth.genome(30000, 0.41, 0.1, (0.01, 0.01), seed=3), 100, 25,
                                  0.005, seed=4), 63, 0),
        (synth.reads_for_coverage(synth.genome(20000, 0.5, seed=5), 60, 30, 0.0, seed=6), 31, 1),
    ]
    for reads, t, direction in cases:
        reads = np.ascontiguousarray(reads[: MAX_SUFFIXES // reads.shape[1]])
        n = reads.size
        d_reads = torch.from_numpy(reads).to(dev)
        d_sa = torch.full((n,), -1, dtype=tdt, device=dev)
        rc = f(d_reads.data_ptr(), reads.shape[0], reads.shape[1], direction, d_sa.data_ptr(),
               stream.cuda_stream)
        assert rc == 0
        torch.cuda.synchronize(dev)
        got = d_sa.cpu().numpy().view(np.uint64 if width == 64 else np.uint32)
        want = reference_sa(reads, t, width, direction)
        assert np.array_equal(got, want)


def test_static_sort_rejects_oversize():
    f = static_sort_fn(32)
    # rejected before any device access: the pointers are never dereferenced
    assert f(None, MAX_SUFFIXES // 100 + 1, 100, 0, None, None) == 6   # PQ_ERR_CAPACITY
