"""Queued search over several read sets (own L, t and index pair each) in one persistent kernel,
plain and through a captured CUDA graph, and the autotuned plan: every read set's edges are the
reference's and those of its own single search."""
import numpy as np
import pytest

from conftest import load_golden, sha, idx_dtype
import pasqual_gb300 as pq
from pasqual_gb300 import graph

pytestmark = pytest.mark.gpu

FIELDS = ("edge_off", "dest", "length", "etype", "trans", "num_B", "num_F", "olp_B", "olp_F")

SETS = {
    32: ["iid8k_L50_t31_u32", "rep15k_L100_t63_u32", "iid5k_L60_t59_u32", "dinuc6k_L60_t20_u32",
         "iid3k_L40_t10_u32"],
    64: ["lowc12k_L150_t63_u64", "rep20k_L100_t63_u64"],
}


def _contexts(width, names, mode=1):
    ctxs, gold = [], []
    for n in names:
        g = load_golden(n)
        P = pq.Pasqual(width)
        P.set_reads(g["reads"], int(g["t"]))
        P.set_seed_mode(mode)
        P.build_index()
        ctxs.append(P)
        gold.append(g)
    return ctxs, gold


def _check(ctxs, gold, single):
    for P, g, s in zip(ctxs, gold, single):
        out = P.graph()
        for f in FIELDS:
            assert np.array_equal(getattr(out, f), getattr(s, f)), f
        assert sha(out.dest.astype(idx_dtype(g["width"]))) == str(g["sha_dest"])
        assert sha(graph.trans_with_mask(out.num_B, out.num_F, out.edge_off, out.trans)) == str(g["sha_trans"])


@pytest.mark.parametrize("width", [32, 64])
@pytest.mark.parametrize("use_graph", [False, True])
def test_batched_equals_single(width, use_graph):
    ctxs, gold = _contexts(width, SETS[width])
    try:
        single = [P.construct_string_graph() for P in ctxs]
        for _ in range(2):                   # the graph is captured on the first call, replayed next
            pq.overlaps_batched(ctxs, graph=use_graph)
            _check(ctxs, gold, single)
        st = ctxs[0].batch_stats()
        assert st["graph_used"] == (1 if use_graph else 0)
        assert st["kernel_ms"] > 0
    finally:
        for P in ctxs:
            P.close()


def test_batched_learned_mode():
    ctxs, gold = _contexts(32, ["iid8k_L50_t31_u32", "rep15k_L100_t63_u32"], mode=2)
    try:
        single = [P.construct_string_graph() for P in ctxs]
        pq.overlaps_batched(ctxs, graph=True)
        _check(ctxs, gold, single)
    finally:
        for P in ctxs:
            P.close()


def test_autotune_keeps_results_and_sets_plan():
    ctxs, gold = _contexts(32, SETS[32][:3])
    try:
        single = [P.construct_string_graph() for P in ctxs]
        ms = pq.autotune_batched(ctxs, graph=True)
        assert ms > 0
        st = ctxs[0].batch_stats()
        assert st["ctas_per_sm"] >= 2 and st["groups_per_item"] in (1, 2, 4) and st["edge_slots"] in (32, 64)
        _check(ctxs, gold, single)
        pq.overlaps_batched(ctxs, graph=True)          # the tuned plan, replayed
        _check(ctxs, gold, single)
    finally:
        for P in ctxs:
            P.close()


def test_batch_argument_errors():
    g = load_golden("iid8k_L50_t31_u32")
    with pq.Pasqual(32) as P:
        P.construct_index(g["reads"], int(g["t"]))
        with pytest.raises(pq.PQError):
            pq.overlaps_batched([P, P])                 # the same context twice
        with pytest.raises(pq.PQError):
            P.set_batch_plan(ctas_per_sm=2, groups_per_item=0)
