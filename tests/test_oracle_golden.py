"""The C restatement (oracle) against the golden vectors made by the unmodified reference.

Pins every array of the hot path: both suffix arrays (canonical single-thread order), both
FM-indexes in the reference layout, and the per-read ordered edge lists with node fields.
"""
import os
import sys

import numpy as np
import pytest

from conftest import GOLDEN, ROOT, golden_cases, load_golden, sha, idx_dtype
from oracle import port
from pasqual_gb300 import graph


@pytest.fixture(scope="module")
def ports():
    port.build()
    return {32: port.Port(32), 64: port.Port(64)}


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference(name, ports):
    g = load_golden(name)
    P = ports[int(g["width"])]
    ix = P.build_index(g["reads"], int(g["t"]), threads=4)
    C, sfx, pfx = ix["C"], ix["suffix_count"], ix["prefix_count"]
    assert np.array_equal(C, g["C"]) and np.array_equal(sfx, g["suffix_count"])
    assert np.array_equal(pfx, g["prefix_count"])
    for k in ("sa0", "sa1", "bitmap0", "bitmap1", "sample0", "sample1", "reads_index0",
              "reads_index1"):
        assert sha(ix[k]) == str(g["sha_" + k]), k
    out = P.overlaps(ix, threads=4)
    dt = idx_dtype(g["width"])
    assert int(g["num_edges"]) == len(out.dest)
    assert sha(out.num_B) == str(g["sha_num_B"])
    assert sha(out.num_F) == str(g["sha_num_F"])
    assert sha(out.dest.astype(np.uint64).astype(dt)) == str(g["sha_dest"])
    assert sha(out.length) == str(g["sha_length"])
    assert sha(out.etype) == str(g["sha_etype"])
    assert sha(graph.trans_with_mask(out.num_B, out.num_F, out.edge_off, out.trans)) == \
        str(g["sha_trans"])
    nf = graph.node_fields(out.num_B, out.num_F, out.olp_B, out.olp_F)
    assert sha(nf) == str(g["sha_node_types"])


def test_oracle_seed_equivalence(ports):
    """Any exact seed interval gives the same edges (k-mer seeds vs depth-1 starts)."""
    g = load_golden("rep15k_L100_t63_u32")
    P = ports[32]
    ix = P.build_index(g["reads"], int(g["t"]), threads=4, seed_k=12)
    a = P.overlaps(ix, threads=4)
    b = P.overlaps(ix, threads=4, seeds=(ix["seed0"], ix["seed1"]))
    assert np.array_equal(a.dest, b.dest) and np.array_equal(a.trans, b.trans)
    assert b.probes < a.probes


def test_oracle_bounded_sample_equals_full(ports):
    """A read range gives the same per-read edges as the full run (used by the CPU baseline)."""
    g = load_golden("iid8k_L50_t31_u32")
    P = ports[32]
    ix = P.build_index(g["reads"], int(g["t"]), threads=4)
    full = P.overlaps(ix, threads=4)
    part = P.overlaps(ix, first=1000, count=500, threads=2)
    o = full.edge_off.astype(np.int64)
    assert np.array_equal(part.dest, full.dest[o[1000]:o[1500]])
    assert np.array_equal(part.num_F, full.num_F[1000:1500])


@pytest.mark.parametrize("name", golden_cases())
def test_golden_fixture_is_the_reference_on_its_reads(tmp_path, name):
    """Each committed fixture is what the reference gives today on the fixture's own reads: same
    kept reads, counts, digests of every array and full edge arrays.  The reads go back through
    the reference's import with a Bloom filter long enough that no read is lost to a false
    positive (the fixture's reads are already free of duplicates)."""
    import os
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    port.build(ref=True)
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    full = "full_dest" in z.files
    fresh = make_golden.reference_fixture(z["reads"], int(z["t"]), int(z["width"]), full,
                                          str(tmp_path), bloom_m=100000)
    assert set(fresh) == set(z.files)
    for k in z.files:
        assert np.array_equal(np.asarray(fresh[k]), z[k]), k


@pytest.mark.parametrize("name", ["iid3k_L40_t10_u32", "iid8k_L50_t31_u32", "rep12k_L250_t95_u32"])
def test_golden_generator_reproduces_fixture(tmp_path, name):
    """The generator's seeded reads still give these committed fixtures.  The fixtures with
    repeats or low-complexity runs came from an earlier version of the genome generator; they are
    pinned by their stored reads above."""
    import os
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
    import make_golden
    port.build(ref=True)
    fresh = make_golden.compute(name, str(tmp_path))
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    for k in z.files:
        assert np.array_equal(np.asarray(fresh[k]), z[k]), k


def test_oracle_matches_reference_at_workload_size(tmp_path):
    """The restatement at the full size of the 1 Mbp, 50 bp, 40x, t = 31 workload (800 K reads
    generated, about 550 K kept by the library's import with the reference's Bloom filter):
    both suffix arrays, both FM-indexes and every edge equal the reference's digests."""
    from conftest import graph_digests_ok, large_kept_reads, load_large
    g = load_large("c1_1Mbp_L50_40x_t31_u32")
    reads, _ = large_kept_reads(g, tmp_path)
    P = port.Port(32)
    cores = os.cpu_count() or 1
    ix = P.build_index(reads, int(g["t"]), threads=cores)
    for d in (0, 1):
        assert sha(ix["sa%d" % d]) == str(g["sha_sa%d" % d])
        assert sha(ix["bitmap%d" % d]) == str(g["sha_bitmap%d" % d])
        assert sha(ix["sample%d" % d]) == str(g["sha_sample%d" % d])
        assert sha(ix["reads_index%d" % d]) == str(g["sha_reads_index%d" % d])
    graph_digests_ok(P.overlaps(ix, threads=cores), g, "oracle")
