"""pq_host_alloc / pq_host_free: page-locked host buffers for reads in and graphs out, which
pq_set_reads and pq_get_graph copy with a kernel.  The reads and the graph that pass through such
buffers are the ones that pass through ordinary (pageable) numpy arrays."""
import numpy as np
import pytest

from conftest import load_golden
import pasqual_gb300 as pq

pytestmark = pytest.mark.gpu


def test_host_buffers_round_trip():
    g = load_golden("rep15k_L100_t63_u32")
    reads, t = g["reads"], int(g["t"])
    hr = pq.host_empty(reads.shape, np.uint8)
    assert hr.ctypes.data % 256 == 0
    hr[:] = reads
    with pq.Pasqual(32) as P:
        P.set_reads(reads, t)
        P.build_index()
        P.overlaps()
        want = P.graph()
        P.set_reads(hr, t)
        P.build_index()
        P.overlaps()
        out = pq.Graph(**{f: pq.host_empty((getattr(want, f).size,), getattr(want, f).dtype)
                          for f in ("num_B", "num_F", "olp_B", "olp_F", "edge_off", "dest", "length",
                                    "etype", "trans")})
        got = P.graph(out=out)
    for f in ("num_B", "num_F", "olp_B", "olp_F", "edge_off", "dest", "length", "etype", "trans"):
        assert np.array_equal(getattr(got, f), getattr(want, f)), f


def test_host_free_rejects_foreign_pointers():
    lib = pq.load_library(32)
    a = np.zeros(16, np.uint8)
    assert lib.pq_host_free(a.ctypes.data) == 1        # PQ_ERR_ARG: not from pq_host_alloc
    assert lib.pq_host_free(None) == 0
