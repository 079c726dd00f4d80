"""The CUDA path at the benchmark workloads' own sizes against digests of the unmodified
reference (tests/golden/large/, made by tests/golden/make_golden.py): the 1 Mbp, 50 bp, 40x,
t = 31 workload in full (about 550 K reads kept), and the 50 Mbp, 100 bp, 30x, t = 63 workload at
1/10 genome size (about 1.4 M reads, 141 M suffixes per index).  At these sizes the paths that
only fire at scale run: hand-over from the lean to the fast and wide tiers, edge-pool regrowth,
14-base key groups of more than 1024 suffixes, chunked sorts.

Reads are regenerated by the committed generator (checked against the fixture) and imported by
the library's FASTA import with the reference's Bloom filter (kept reads checked).  Every array
is compared by SHA-256 with the reference's: both suffix arrays, both FM-indexes in the
reference layout, and the ordered edge lists with node fields, in every seed mode.  The reference
path being matched: src/test.c:364-370 (construct_index, construct_string_graph) and
src/string_graph.c:796-1025."""
import numpy as np
import pytest

from conftest import graph_digests_ok, large_cases, large_kept_reads, load_large, sha
import pasqual_gb300 as pq

pytestmark = pytest.mark.gpu


def check_index(P, g, what):
    for d in (0, 1):
        bm, smp, ri = P.index_ref(d)
        assert sha(bm) == str(g["sha_bitmap%d" % d]), "%s OCC_bitmap %d" % (what, d)
        assert sha(smp) == str(g["sha_sample%d" % d]), "%s OCC_sample %d" % (what, d)
        assert sha(ri) == str(g["sha_reads_index%d" % d]), "%s reads_index %d" % (what, d)


@pytest.mark.parametrize("name", large_cases())
def test_workload_matches_reference(tmp_path, name):
    g = load_large(name)
    reads, _ = large_kept_reads(g, tmp_path)
    t = int(g["t"])
    with pq.Pasqual(int(g["width"])) as P:
        P.set_reads(reads, t)
        C, sfx, pfx = P.counts()
        assert np.array_equal(C, g["C"])
        assert np.array_equal(sfx, g["suffix_count"]) and np.array_equal(pfx, g["prefix_count"])
        # suffix array alone (pq_sort), then the index build whose sort leaves BWT symbols and
        # inverse-SA entries for the FM build
        for d in (0, 1):
            P.sort(d)
            assert sha(P.get_sa(d)) == str(g["sha_sa%d" % d]), "suffix array %d" % d
        P.build_index()
        for d in (0, 1):
            assert sha(P.get_sa(d)) == str(g["sha_sa%d" % d]), "suffix array %d (index build)" % d
        check_index(P, g, "index build")
        probes = {}
        for mode in (0, 1, 2):
            P.set_seed_mode(mode)
            P.overlaps()
            out = P.graph()
            graph_digests_ok(out, g, "seed mode %d" % mode)
            probes[mode] = out.probes
    assert probes[1] < probes[0]


@pytest.mark.parametrize("name", large_cases())
def test_workload_chunked_sort_matches_reference(tmp_path, name):
    """The same reads sorted in chunks of 6-base buckets (at most n/7 suffixes a chunk): the
    reference's suffix arrays, FM-indexes and edges."""
    g = load_large(name)
    reads, _ = large_kept_reads(g, tmp_path)
    n = reads.size
    with pq.Pasqual(int(g["width"])) as P:
        P.set_reads(reads, int(g["t"]))
        P.set_sort_chunk(n // 7)
        P.build_index()
        for d in (0, 1):
            assert sha(P.get_sa(d)) == str(g["sha_sa%d" % d]), "chunked suffix array %d" % d
        check_index(P, g, "chunked")
        graph_digests_ok(P.construct_string_graph(), g, "chunked")
