"""CUDA path (through the C ABI) against the golden vectors of the unmodified reference and
against the C restatement at larger sizes.  Integer work: every comparison is bit-exact."""
import numpy as np
import pytest

from conftest import golden_cases, load_golden, sha, idx_dtype
import pasqual_gb300 as pq
from pasqual_gb300 import graph, synth

pytestmark = pytest.mark.gpu


def gpu_ctx(width):
    return pq.Pasqual(width)


@pytest.mark.parametrize("name", golden_cases())
def test_sort_and_index_match_reference(name):
    g = load_golden(name)
    with gpu_ctx(int(g["width"])) as P:
        P.set_reads(g["reads"], int(g["t"]))
        C, sfx, pfx = P.counts()
        assert np.array_equal(C, g["C"])
        assert np.array_equal(sfx, g["suffix_count"]) and np.array_equal(pfx, g["prefix_count"])
        for d in (0, 1):
            P.sort(d)
            assert sha(P.get_sa(d)) == str(g["sha_sa%d" % d]), "suffix array %d" % d
            P.build_fm(d)
            bm, smp, ri = P.index_ref(d)
            assert sha(bm) == str(g["sha_bitmap%d" % d]), "OCC_bitmap %d" % d
            assert sha(smp) == str(g["sha_sample%d" % d]), "OCC_sample %d" % d
            assert sha(ri) == str(g["sha_reads_index%d" % d]), "reads_index %d" % d


@pytest.mark.parametrize("name", golden_cases())
def test_overlaps_match_reference(name):
    g = load_golden(name)
    dt = idx_dtype(g["width"])
    with gpu_ctx(int(g["width"])) as P:
        P.construct_index(g["reads"], int(g["t"]))
        out = P.construct_string_graph()
    assert len(out.dest) == int(g["num_edges"])
    assert sha(out.num_B) == str(g["sha_num_B"])
    assert sha(out.num_F) == str(g["sha_num_F"])
    assert sha(out.dest.astype(dt)) == str(g["sha_dest"])
    assert sha(out.length) == str(g["sha_length"])
    assert sha(out.etype) == str(g["sha_etype"])
    assert sha(graph.trans_with_mask(out.num_B, out.num_F, out.edge_off, out.trans)) == \
        str(g["sha_trans"])
    assert sha(graph.node_fields(out.num_B, out.num_F, out.olp_B, out.olp_F)) == \
        str(g["sha_node_types"])
    if "full_dest" in g:
        assert np.array_equal(out.dest.astype(np.uint64), g["full_dest"])


@pytest.mark.parametrize("name", ["iid8k_L50_t31_u32", "rep15k_L100_t63_u32", "rep20k_L100_t63_u64",
                                  "lowc12k_L150_t63_u64"])
def test_chunked_sort_matches_reference(name):
    """Sorting in chunks of 6-base buckets gives the reference's suffix arrays and edges."""
    g = load_golden(name)
    n = g["reads"].shape[0] * g["reads"].shape[1]
    with gpu_ctx(int(g["width"])) as P:
        P.set_reads(g["reads"], int(g["t"]))
        P.set_sort_chunk(max(n // 6, 2))
        try:
            P.sort(0)
        except pq.PQError as e:      # a low-complexity bucket larger than n/6: half the index
            assert e.code == 6
            P.set_sort_chunk(n // 2 + 1)
            P.sort(0)
        assert sha(P.get_sa(0)) == str(g["sha_sa0"])
        P.sort(1)
        assert sha(P.get_sa(1)) == str(g["sha_sa1"])
        P.build_fm(0)
        P.build_fm(1)
        out = P.construct_string_graph()
    assert sha(out.dest.astype(idx_dtype(g["width"]))) == str(g["sha_dest"])
    # the same through pq_build_index, whose chunked sorts also leave BWT symbols and inverse-SA
    # entries for the FM build
    with gpu_ctx(int(g["width"])) as P:
        P.set_reads(g["reads"], int(g["t"]))
        for chunk in (max(n // 6, 2), n // 2 + 1):
            P.set_sort_chunk(chunk)
            try:
                P.build_index()
                break
            except pq.PQError as e:
                assert e.code == 6
        for d in (0, 1):
            bm, smp, ri = P.index_ref(d)
            assert sha(bm) == str(g["sha_bitmap%d" % d]) and sha(smp) == str(g["sha_sample%d" % d])
            assert sha(ri) == str(g["sha_reads_index%d" % d])
        out = P.construct_string_graph()
    assert sha(out.dest.astype(idx_dtype(g["width"]))) == str(g["sha_dest"])
    assert sha(out.length) == str(g["sha_length"])


@pytest.mark.parametrize("parts", [3, 40])
def test_chunk_counts_both_paths(parts):
    """Chunked sorts with up to 16 chunks count their positions per tile with per-thread counters,
    with more with per-warp groups of equal chunks: both give the reference's suffix arrays."""
    g = load_golden("rep20k_L100_t63_u64")
    n = g["reads"].shape[0] * g["reads"].shape[1]
    with gpu_ctx(int(g["width"])) as P:
        P.set_reads(g["reads"], int(g["t"]))
        P.set_sort_chunk(max(n // parts, 2))
        for d in (0, 1):
            P.sort(d)
            assert sha(P.get_sa(d)) == str(g["sha_sa%d" % d])


@pytest.mark.parametrize("k", [1, 5, 10, 14])
def test_seed_depth_does_not_change_edges(k):
    g = load_golden("rep15k_L100_t63_u32")
    with gpu_ctx(32) as P:
        P.set_reads(g["reads"], int(g["t"]))
        P.set_seed_k(k)
        P.build_index()
        out = P.construct_string_graph()
    assert sha(out.dest.astype(np.uint32)) == str(g["sha_dest"])
    assert sha(out.num_F) == str(g["sha_num_F"])


@pytest.mark.parametrize("name", ["rep15k_L100_t63_u32", "lowc12k_L150_t63_u64", "iid3k_L40_t10_u32"])
def test_seed_modes_agree(name):
    """The reference's method (mode 0: walk + FM-index DFS) and the interval scan with sorted
    reduction (mode 1) give the reference's edges; mode 1 issues fewer probes."""
    g = load_golden(name)
    dt = idx_dtype(g["width"])
    probes = {}
    for mode in (0, 1):
        with gpu_ctx(int(g["width"])) as P:
            P.set_reads(g["reads"], int(g["t"]))
            P.set_seed_mode(mode)
            P.build_index()
            out = P.construct_string_graph()
        assert sha(out.dest.astype(dt)) == str(g["sha_dest"]), mode
        assert sha(out.num_B) == str(g["sha_num_B"]) and sha(out.num_F) == str(g["sha_num_F"])
        probes[mode] = out.probes
    assert probes[1] < probes[0]


@pytest.mark.parametrize("name", ["dinuc6k_L60_t20_u32", "lowc12k_L150_t63_u64"])
def test_handed_over_tiers_used_and_exact(name):
    """Dinucleotide runs give reads with hundreds of candidates on a side: the lean tier hands them
    to the fast tier, which hands the largest to the block tier (one CTA a read); the edges stay
    the reference's."""
    g = load_golden(name)
    with gpu_ctx(int(g["width"])) as P:
        P.construct_index(g["reads"], int(g["t"]))
        out = P.construct_string_graph()
        tiers = P.tier_stats()
    assert tiers["deferred"] > 0
    assert tiers["block"] + tiers["heavy"] + tiers["wide"] > 0, tiers
    assert sha(out.dest.astype(idx_dtype(g["width"]))) == str(g["sha_dest"])
    assert sha(out.num_B) == str(g["sha_num_B"]) and sha(out.num_F) == str(g["sha_num_F"])
    assert sha(graph.trans_with_mask(out.num_B, out.num_F, out.edge_off, out.trans)) == str(g["sha_trans"])


def test_block_tier_in_global_memory_matches_reference_method():
    """The 200 Mbp, 150 bp workload (2 % dinucleotide runs) at 1/100 genome: its run reads have
    thousands of candidates a side, more than the block tier holds in shared memory, so they are
    reduced by the global-memory block tier (sorted reduction).  Every edge field equals the
    reference's method on the GPU (seed mode 0: walk + FM-index DFS, no block tier), and no read
    reaches the heavy or wide tier."""
    _, rd, L, t = synth.make_workload("200Mbp_L150_20x_t63", scale=0.01)
    rd = synth.dedup(rd)
    out, tiers = {}, None
    for mode in (0, 1):
        with gpu_ctx(64) as P:
            P.set_reads(rd, t)
            P.set_seed_mode(mode)
            P.build_index()
            out[mode] = P.construct_string_graph()
            if mode == 1:
                tiers = P.tier_stats()
    assert tiers["block"] > 1000 and tiers["heavy"] == 0 and tiers["wide"] == 0, tiers
    for f in ("edge_off", "dest", "length", "etype", "trans", "num_B", "num_F", "olp_B", "olp_F"):
        assert np.array_equal(getattr(out[0], f), getattr(out[1], f)), f


def _oracle_run(reads, t, width):
    from oracle import port
    P = port.Port(width)
    ix = P.build_index(reads, t)
    return ix, P.overlaps(ix)


@pytest.mark.parametrize("width", [32, 64])
def test_against_oracle_config1_shape(width):
    """1 Mbp-shaped workload at 1/5 scale (200 kbp, L=50, 40x, t=31): GPU == oracle."""
    gen = synth.genome(200_000, 0.5, seed=21)
    rd = synth.reads_for_coverage(gen, 50, 40, 0.0, seed=22)
    rd = np.unique(rd, axis=0)          # distinct reads, as after de-duplication
    ix, ref = _oracle_run(rd, 31, width)
    with gpu_ctx(width) as P:
        P.construct_index(rd, 31)
        for d in (0, 1):
            assert np.array_equal(P.get_sa(d), ix["sa%d" % d])
            bm, smp, ri = P.index_ref(d)
            assert np.array_equal(bm, ix["bitmap%d" % d])
            assert np.array_equal(smp, ix["sample%d" % d])
            assert np.array_equal(ri, ix["reads_index%d" % d])
        out = P.construct_string_graph()
    assert np.array_equal(out.edge_off, ref.edge_off)
    assert np.array_equal(out.dest, ref.dest)
    assert np.array_equal(out.length, ref.length)
    assert np.array_equal(out.etype, ref.etype)
    assert np.array_equal(out.trans, ref.trans)
    assert np.array_equal(out.olp_B, ref.olp_B) and np.array_equal(out.olp_F, ref.olp_F)


def test_repeats_errors_long_reads_against_oracle():
    """L=150 reads with repeats, low-complexity runs and errors (U32): GPU == oracle."""
    gen = synth.genome(300_000, 0.40, 0.12, (0.005, 0.02), 0.02, seed=31)
    rd = np.unique(synth.reads_for_coverage(gen, 150, 20, 0.003, seed=32), axis=0)
    ix, ref = _oracle_run(rd, 63, 32)
    with gpu_ctx(32) as P:
        P.construct_index(rd, 63)
        assert np.array_equal(P.get_sa(0), ix["sa0"])
        assert np.array_equal(P.get_sa(1), ix["sa1"])
        out = P.construct_string_graph()
    assert np.array_equal(out.dest, ref.dest)
    assert np.array_equal(out.trans, ref.trans)
    assert np.array_equal(out.num_B, ref.num_B) and np.array_equal(out.num_F, ref.num_F)


@pytest.mark.parametrize("t", [31, 95])
def test_long_reads_against_oracle(t):
    """L = 180 (continuations up to 149 bases, DFS depth beyond the fast tier's frames) with
    repeats and errors: every seed mode equals the oracle."""
    gen = synth.genome(120_000, 0.45, 0.08, (0.01, 0.01), 0.0, seed=41 + t)
    rd = np.unique(synth.reads_for_coverage(gen, 180, 12, 0.005, seed=42 + t), axis=0)
    ix, ref = _oracle_run(rd, t, 32)
    for mode in (0, 1, 2):
        with gpu_ctx(32) as P:
            P.set_reads(rd, t)
            P.set_seed_mode(mode)
            P.build_index()
            out = P.construct_string_graph()
        assert np.array_equal(out.edge_off, ref.edge_off), mode
        assert np.array_equal(out.dest, ref.dest), mode
        assert np.array_equal(out.length, ref.length) and np.array_equal(out.etype, ref.etype)
        assert np.array_equal(out.trans, ref.trans), mode
        assert np.array_equal(out.olp_B, ref.olp_B) and np.array_equal(out.olp_F, ref.olp_F)


def test_empty_and_tiny_inputs():
    with gpu_ctx(32) as P:
        P.construct_index(np.zeros((0, 50), np.uint8), 31)
        out = P.construct_string_graph()
        assert len(out.dest) == 0 and len(out.num_B) == 0
    one = np.array([[1, 2, 3, 4] * 12 + [1, 2]], np.uint8)
    with gpu_ctx(32) as P:
        P.construct_index(one, 31)
        out = P.construct_string_graph()
        assert len(out.dest) == 0


def test_invalid_arguments_raise():
    with gpu_ctx(32) as P:
        with pytest.raises(pq.PQError):
            P.set_reads(np.ones((10, 50), np.uint8), 9)      # t must exceed SEQ_DEPTH (9)
        with pytest.raises(pq.PQError):
            P.set_reads(np.ones((10, 50), np.uint8), 50)     # t must be below L
        with pytest.raises(pq.PQError):
            P.overlaps()                                     # no index yet
        for bad in (0, 5, 78):                               # only base codes 1..4 (the import drops N)
            r = np.ones((40, 50), np.uint8)
            r[17, 33] = bad
            with pytest.raises(pq.PQError):
                P.set_reads(r, 20)
        r = np.random.default_rng(3).integers(1, 5, (40, 50), dtype=np.uint8)
        P.set_reads(r, 20)                                   # a valid set after a rejected one
        C, sfx, pfx = P.counts()
        assert int(C[5]) == r.size and int(sfx.sum()) == 40 and int(pfx.sum()) == 40


def test_graph_into_reused_arrays():
    """graph(out=...) fills an earlier result's arrays in place (views of the new lengths) and
    gives the same graph as fresh arrays; too-small or mistyped arrays are replaced."""
    big, small = load_golden("rep15k_L100_t63_u32"), load_golden("iid8k_L50_t31_u32")
    with gpu_ctx(32) as P:
        P.construct_index(big["reads"], int(big["t"]))
        g_big = P.construct_string_graph()
        P.construct_index(small["reads"], int(small["t"]))
        P.overlaps()
        fresh = P.graph()
        reused = P.graph(out=g_big)
        for name in ("num_B", "num_F", "olp_B", "olp_F", "edge_off", "dest", "length", "etype", "trans"):
            a, b = getattr(fresh, name), getattr(reused, name)
            assert np.array_equal(a, b), name
        if len(g_big.dest) >= len(fresh.dest):
            assert np.shares_memory(reused.dest, g_big.dest)
        assert len(reused.dest) == int(small["num_edges"])
        # arrays too short for the bigger graph are replaced, not overrun
        P.construct_index(big["reads"], int(big["t"]))
        P.overlaps()
        again = P.graph(out=reused)
        assert len(again.dest) == int(big["num_edges"])
        assert sha(again.dest) == str(big["sha_dest"])
