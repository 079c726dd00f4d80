"""Node construction of construct_string_graph (src/string_graph.c:832-1017) on the host, through
pq_string_graph_from_csr: every node_t / edge_t / path_q_t field against the restatement in
pasqual_gb300/graph.py and a direct numpy statement, and the same result for any thread count."""
import ctypes as ct
import math

import numpy as np
import pytest

import pasqual_gb300 as pq
from pasqual_gb300 import graph
from conftest import golden_cases, idx_dtype, load_golden, sha
from test_gpu_dropin import structs


def random_csr(nr, seed, L=100):
    rng = np.random.default_rng(seed)
    nb = rng.choice([0, 0, 1, 1, 1, 2, 3, 7], nr).astype(np.uint16)
    nf = rng.choice([0, 1, 1, 1, 2, 4], nr).astype(np.uint16)
    olp_b = (nb * rng.integers(1, 4, nr)).astype(np.int32)
    olp_f = (nf * rng.integers(1, 9, nr)).astype(np.int32)
    off = np.zeros(nr + 1, np.uint64)
    off[1:] = np.cumsum(nb.astype(np.uint64) + nf)
    ne = int(off[-1])
    dest = rng.integers(0, max(nr, 1), ne)
    ln = rng.integers(30, L, ne).astype(np.uint16)
    et = rng.integers(0, 4, ne).astype(np.uint8)
    trans = rng.integers(0, 1000, ne).astype(np.int32)
    return nb, nf, olp_b, olp_f, off, dest, ln, et, trans


def call(lib, width, L, t, csr, threads):
    I, _, Graph = structs(width)
    nb, nf, ob, of, off, dest, ln, et, trans = csr
    idx = np.uint64 if width == 64 else np.uint32
    dest = np.ascontiguousarray(dest.astype(idx))
    f = lib.pq_string_graph_from_csr
    f.restype = ct.POINTER(Graph)
    f.argtypes = [I, ct.c_int, ct.c_int] + [ct.c_void_p] * 9 + [ct.c_int]
    p = lambda a: a.ctypes.data_as(ct.c_void_p)
    r = f(len(nb), L, t, p(nb), p(nf), p(ob), p(of), p(off), p(dest), p(ln), p(et), p(trans), threads)
    assert r
    return r.contents


def read_graph(g, nr):
    """Every field of the nodes, flattened to arrays."""
    node = np.zeros((nr, 8), np.int64)
    edges, paths, q = [], [], []
    for i in range(nr):
        nd = g.nodes[i]
        node[i] = (nd.num_B, nd.num_F, nd.max_B, nd.max_F, nd.B_type, nd.F_type, nd.status, nd.marked)
        m = nd.num_B + nd.num_F
        for j in range(m):
            e = nd.edges[j]
            edges.append((int(e.dest), e.overlap_len, ord(e.type)))
        if nd.path_q:
            pq_ = nd.path_q.contents
            q.append((i, pq_.max_F_endlen, pq_.max_B_endlen, pq_.max_B_len, pq_.max_F_len,
                      pq_.max_F_trans, pq_.max_B_trans))
            for j in range(m):
                x = pq_.path[j]
                paths.append((int(x.end), int(x.hop), x.len, x.end_len, x.bubble_len, x.trans,
                              ord(x.updated), ord(x.direction), ord(x.type)))
    return node, np.array(edges, np.int64).reshape(-1, 3), np.array(paths, np.int64).reshape(-1, 9), \
        np.array(q, np.int64).reshape(-1, 7)


@pytest.mark.parametrize("width", [32, 64])
def test_nodes_match_restatement(width):
    lib = pq.load_library(width)
    nr, L, t = 20000, 100, 55
    csr = random_csr(nr, 7 + width, L)
    nb, nf, ob, of, off, dest, ln, et, trans = csr
    g1 = call(lib, width, L, t, csr, 1)
    node, edges, paths, q = read_graph(g1, nr)
    assert (g1.num_reads, g1.read_len, g1.min_overlap) == (nr, L, t)
    assert np.array_equal(node[:, 0], nb) and np.array_equal(node[:, 1], nf)
    assert np.array_equal(node[:, 2], nb) and np.array_equal(node[:, 3], nf)
    assert np.array_equal(node[:, 4:8], graph.node_fields(nb, nf, ob, of))
    assert np.array_equal(edges, np.stack([dest, ln, et], 1))
    hp = graph.has_path_queue(nb, nf)
    assert np.array_equal(q[:, 0], np.nonzero(hp)[0])
    # path entries of the nodes with a path queue, in node order
    sel = np.concatenate([np.arange(off[i], off[i + 1]) for i in np.nonzero(hp)[0]]).astype(np.int64)
    is_b = np.concatenate([np.arange(int(nb[i]) + int(nf[i])) < nb[i] for i in np.nonzero(hp)[0]])
    direction = np.where(is_b, et[sel] == 3, et[sel] == 1).astype(np.int64)
    want = np.stack([dest[sel], dest[sel], np.ones_like(sel), L - ln[sel].astype(np.int64),
                     np.zeros_like(sel), trans[sel], np.zeros_like(sel), direction,
                     np.zeros_like(sel)], 1)
    assert np.array_equal(paths, want)
    # running maxima of trans in read order, B and F edges separately
    own_b = np.zeros(nr, np.int64)
    own_f = np.zeros(nr, np.int64)
    for i in range(nr):
        b0, b1 = int(off[i]), int(off[i]) + int(nb[i])
        if nb[i]:
            own_b[i] = trans[b0:b1].max()
        if nf[i]:
            own_f[i] = trans[b1:int(off[i + 1])].max()
    run_b = np.maximum.accumulate(own_b)
    run_f = np.maximum.accumulate(own_f)
    assert np.array_equal(q[:, 5], run_f[q[:, 0]]) and np.array_equal(q[:, 6], run_b[q[:, 0]])
    assert np.all(q[:, 1:5] == 0)
    assert g1.average_overlap == pytest.approx(ln.astype(np.float64).mean(), rel=0, abs=1e-12)
    # any thread count: the same graph, field for field
    for threads in (3, 5, 0):
        g = call(lib, width, L, t, csr, threads)
        for a, b in zip(read_graph(g, nr), (node, edges, paths, q)):
            assert np.array_equal(a, b)
        assert g.average_overlap == g1.average_overlap


def test_graph_without_edges():
    lib = pq.load_library(32)
    nr = 5000
    z16 = np.zeros(nr, np.uint16)
    z32 = np.zeros(nr, np.int32)
    csr = (z16, z16, z32, z32, np.zeros(nr + 1, np.uint64), np.zeros(0, np.int64),
           np.zeros(0, np.uint16), np.zeros(0, np.uint8), np.zeros(0, np.int32))
    g = call(lib, 32, 80, 41, csr, 2)
    node, edges, paths, q = read_graph(g, nr)
    assert np.all(node[:, 4:6] == 4) and np.all(node[:, 6] == 8) and np.all(node[:, 7] == 0)
    assert len(edges) == 0 and len(q) == 0
    assert math.isnan(g.average_overlap)
    g0 = call(lib, 32, 80, 41, tuple(a[:0] if k < 4 else (a[:1] if k == 4 else a)
                                     for k, a in enumerate(csr)), 0)
    assert g0.num_reads == 0 and math.isnan(g0.average_overlap)


def test_invalid_arguments_return_null():
    lib = pq.load_library(32)
    f = lib.pq_string_graph_from_csr
    f.restype = ct.c_void_p
    f.argtypes = [ct.c_uint32, ct.c_int, ct.c_int] + [ct.c_void_p] * 9 + [ct.c_int]
    nb, nf, ob, of, off, dest, ln, et, trans = random_csr(100, 3)
    dest = dest.astype(np.uint32)
    p = lambda a: a.ctypes.data_as(ct.c_void_p)
    good = [p(nb), p(nf), p(ob), p(of), p(off), p(dest), p(ln), p(et), p(trans)]
    assert f(100, 100, 55, *good, 1)                    # leaks one small graph; fine in a test
    assert not f(100, 0, 55, *good, 1)
    assert not f(100, 70000, 55, *good, 1)
    for k in range(9):
        args = list(good)
        args[k] = None
        assert not f(100, 100, 55, *args, 1), k
    z16, z32 = np.zeros(10, np.uint16), np.zeros(10, np.int32)
    zoff = np.zeros(11, np.uint64)
    assert f(10, 100, 55, p(z16), p(z16), p(z32), p(z32), p(zoff), None, None, None, None, 1)


@pytest.mark.parametrize("name", golden_cases())
def test_nodes_match_reference_digests(name):
    """The library's node build on the oracle's edge lists gives the reference's own node_t
    array: node types, status, SUSPECT marks, edges and path trans (-1 where a node has no path
    queue) hash to the digests the reference's construct_string_graph produced for the case."""
    from oracle import port
    port.build()
    g = load_golden(name)
    width, t = int(g["width"]), int(g["t"])
    reads = g["reads"]
    nr, L = reads.shape
    O = port.Port(width)
    ref = O.overlaps(O.build_index(reads, t, threads=4), threads=4)
    csr = (ref.num_B, ref.num_F, ref.olp_B, ref.olp_F, ref.edge_off, ref.dest, ref.length,
           ref.etype, ref.trans)
    gr = call(pq.load_library(width), width, L, t, csr, 0)
    node = np.zeros((nr, 4), np.uint8)
    dest, length, etype, trans = [], [], [], []
    for i in range(nr):
        nd = gr.nodes[i]
        node[i] = (nd.B_type, nd.F_type, nd.status, nd.marked)
        for j in range(nd.num_B + nd.num_F):
            e = nd.edges[j]
            dest.append(int(e.dest))
            length.append(e.overlap_len)
            etype.append(ord(e.type))
            trans.append(nd.path_q.contents.path[j].trans if nd.path_q else -1)
    assert sha(node) == str(g["sha_node_types"])
    assert sha(np.array(dest, idx_dtype(width))) == str(g["sha_dest"])
    assert sha(np.array(length, np.uint16)) == str(g["sha_length"])
    assert sha(np.array(etype, np.uint8)) == str(g["sha_etype"])
    assert sha(np.array(trans, np.int64)) == str(g["sha_trans"])
