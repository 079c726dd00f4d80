"""The reference's own entry points served by the GPU library: construct_index and
construct_string_graph called through their reference signatures, results read back through the
reference's struct layouts and compared with the oracle run on the same kept reads."""
import ctypes as ct
import gzip
import os

import numpy as np
import pytest

from conftest import GOLDEN, sha
import pasqual_gb300 as pq
from pasqual_gb300 import graph

pytestmark = pytest.mark.gpu


def structs(width):
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    P = ct.POINTER

    class Index(ct.Structure):
        _fields_ = [("bloom_array", ct.c_void_p), ("bloom_size", I), ("n_hashfunc", ct.c_int),
                    ("C", I * 6), ("suffix_count", I * 4), ("prefix_count", I * 4),
                    ("OCC_bitmap", P(ct.c_uint64) * 5), ("OCC_bitmap_bw", P(ct.c_uint64) * 5),
                    ("OCC_sample", P(I)), ("OCC_sample_bw", P(I)), ("reads_index", P(I)),
                    ("reads_index_bw", P(I)), ("interval_start", P(I)), ("interval_end", P(I)),
                    ("interval_depth", P(ct.c_uint16)), ("interval_start_bw", P(I)),
                    ("interval_end_bw", P(I)), ("interval_depth_bw", P(ct.c_uint16)),
                    ("read_lock", ct.c_void_p), ("reads", P(ct.c_uint8)), ("read_len", ct.c_uint16),
                    ("num_reads", I), ("min_overlap", ct.c_uint16), ("size_bw", I * 5),
                    ("offset_bw", I * 5), ("size_fw", I * 5), ("offset_fw", I * 5),
                    ("max_size_fw", I), ("max_size_bw", I)]

    class Path(ct.Structure):
        _fields_ = [("end", I), ("hop", I), ("len", ct.c_uint16), ("end_len", ct.c_uint16),
                    ("bubble_len", ct.c_uint16), ("trans", ct.c_int), ("updated", ct.c_char),
                    ("direction", ct.c_char), ("type", ct.c_char)]

    class PathQ(ct.Structure):
        _fields_ = [("path", P(Path)), ("max_F_endlen", ct.c_uint16),
                    ("max_B_endlen", ct.c_uint16), ("max_B_len", ct.c_uint16),
                    ("max_F_len", ct.c_uint16), ("max_F_trans", ct.c_int),
                    ("max_B_trans", ct.c_int)]

    class Edge(ct.Structure):
        _fields_ = [("dest", I), ("overlap_len", ct.c_uint16), ("type", ct.c_char)]

    class Node(ct.Structure):
        _fields_ = [("edges", P(Edge)), ("path_q", P(PathQ)), ("num_F", ct.c_uint16),
                    ("num_B", ct.c_uint16), ("max_F", ct.c_uint16), ("max_B", ct.c_uint16),
                    ("B_type", ct.c_uint8), ("F_type", ct.c_uint8), ("status", ct.c_uint8),
                    ("marked", ct.c_uint8)]

    class Graph(ct.Structure):
        _fields_ = [("read_len", ct.c_uint16), ("min_overlap", ct.c_uint16),
                    ("average_overlap", ct.c_double), ("num_reads", I), ("nodes", P(Node))]
    return I, Index, Graph


@pytest.mark.parametrize("width", [32, 64])
def test_reference_entry_points(tmp_path, width):
    from oracle import port
    fa = tmp_path / "import.fa"
    with gzip.open(os.path.join(GOLDEN, "import_L60.fa.gz"), "rb") as f:
        fa.write_bytes(f.read())
    z = np.load(os.path.join(GOLDEN, "import_L60.npz"))
    lib = pq.load_library(width)
    I, Index, Graph = structs(width)
    lib.construct_index.restype = ct.POINTER(Index)
    lib.construct_index.argtypes = [ct.c_char_p] * 5 + [ct.c_int] * 4
    lib.construct_string_graph.restype = ct.POINTER(Graph)
    lib.construct_string_graph.argtypes = [ct.POINTER(Index)]
    L, t = 60, 31
    ix = lib.construct_index(str(fa).encode(), None, None, None, None, t, L, 36, 2).contents
    nr = int(ix.num_reads)
    assert nr == int(z["kept%d" % width])
    reads = np.ctypeslib.as_array(ix.reads, shape=(nr * L,)).reshape(nr, L).copy()
    assert sha(reads) == str(z["sha_reads%d" % width])

    O = port.Port(width)
    oix = O.build_index(reads, t)
    assert list(ix.C) == [int(x) for x in oix["C"]]
    # sort-slot sizes of both directions (5 slots of 17 first-prefix ranks)
    from test_slot_sizes import direct_histogram
    for d, (szf, off_f, mxf) in enumerate((("size_fw", "offset_fw", "max_size_fw"),
                                           ("size_bw", "offset_bw", "max_size_bw"))):
        h = direct_histogram(reads, d)
        sizes = [int(h[17 * k:17 * k + 17].sum()) for k in range(5)]
        assert list(getattr(ix, szf)) == sizes
        assert list(getattr(ix, off_f)) == [sum(sizes[:k]) for k in range(5)]
        assert int(getattr(ix, mxf)) == max(sizes)
    n = nr * L
    rowlen = n // 64 + 1
    for d, (bmf, smpf, rif) in enumerate((("OCC_bitmap", "OCC_sample", "reads_index"),
                                          ("OCC_bitmap_bw", "OCC_sample_bw", "reads_index_bw"))):
        bm = np.concatenate([np.ctypeslib.as_array(getattr(ix, bmf)[c], shape=(rowlen,))
                             for c in range(5)])
        assert np.array_equal(bm, oix["bitmap%d" % d])
        assert np.array_equal(np.ctypeslib.as_array(getattr(ix, smpf), shape=(5 * rowlen,)),
                              oix["sample%d" % d])
        assert np.array_equal(np.ctypeslib.as_array(getattr(ix, rif), shape=(nr,)),
                              oix["reads_index%d" % d])
    ref = O.overlaps(oix)
    g = lib.construct_string_graph(ct.byref(ix)).contents
    assert int(g.num_reads) == nr
    off = ref.edge_off.astype(np.int64)
    nf = graph.node_fields(ref.num_B, ref.num_F, ref.olp_B, ref.olp_F)
    hp = graph.has_path_queue(ref.num_B, ref.num_F)
    total_len = 0
    for i in range(nr):
        nd = g.nodes[i]
        assert (nd.num_B, nd.num_F) == (int(ref.num_B[i]), int(ref.num_F[i]))
        assert [nd.B_type, nd.F_type, nd.status, nd.marked] == list(nf[i])
        m = nd.num_B + nd.num_F
        for j in range(m):
            e = nd.edges[j]
            k = off[i] + j
            assert (int(e.dest), int(e.overlap_len), ord(e.type)) == \
                (int(ref.dest[k]), int(ref.length[k]), int(ref.etype[k]))
            total_len += int(e.overlap_len)
        assert bool(nd.path_q) == bool(hp[i])
        if nd.path_q:
            for j in range(m):
                assert nd.path_q.contents.path[j].trans == int(ref.trans[off[i] + j])
    assert abs(g.average_overlap - total_len / max(len(ref.dest), 1)) < 1e-9
