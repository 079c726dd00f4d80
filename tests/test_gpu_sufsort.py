"""The reference's suffix-sort entry points (src/sufsort.h:29-46) served by the library, and the
seed intervals the reference's sort records (index_t.interval_start/end/depth,
src/sufsort.c:178-209, 322-334), against the unmodified reference's digests:

* pq_get_sort_seeds on every golden case and at the workload sizes;
* transform_to_triplet[_reverse] -> initial_sort -> suf_sort over the five slots, driven exactly as
  build_idx drives them (src/index.c:495-502, 548-585): the slots concatenate to the reference's
  suffix array, the interval arrays end as the reference's, new_idx advances as the reference's;
* construct_index (src/index.h:63-68) leaves the reference's interval arrays in index_t.
Integer data: every comparison is exact."""
import ctypes as ct

import numpy as np
import pytest

from conftest import golden_cases, idx_dtype, large_cases, large_kept_reads, load_golden, load_large, sha
import pasqual_gb300 as pq
from pasqual_gb300 import synth

pytestmark = pytest.mark.gpu


def check_seeds(seeds, g, d, what):
    s, z, dp = seeds
    assert sha(s) == str(g["sha_seed_start%d" % d]), "%s interval_start %d" % (what, d)
    assert sha(z) == str(g["sha_seed_size%d" % d]), "%s interval_end %d" % (what, d)
    assert sha(dp) == str(g["sha_seed_depth%d" % d]), "%s interval_depth %d" % (what, d)


@pytest.mark.parametrize("name", golden_cases())
def test_sort_seeds_match_reference(name):
    g = load_golden(name)
    with pq.Pasqual(int(g["width"])) as P:
        P.set_reads(g["reads"], int(g["t"]))
        for d in (0, 1):
            P.sort(d)
            check_seeds(P.sort_seeds(d), g, d, name)


@pytest.mark.parametrize("name", large_cases())
def test_sort_seeds_match_reference_at_workload_size(tmp_path, name):
    g = load_large(name)
    reads, _ = large_kept_reads(g, tmp_path)
    with pq.Pasqual(int(g["width"])) as P:
        P.set_reads(reads, int(g["t"]))
        P.build_index()
        for d in (0, 1):
            check_seeds(P.sort_seeds(d), g, d, name)


class Bucket32(ct.Structure):
    _fields_ = [("freqs", ct.c_uint32 * 85), ("offs", ct.c_uint32 * 85)]


class Bucket64(ct.Structure):
    _fields_ = [("freqs", ct.c_uint64 * 85), ("offs", ct.c_uint64 * 85)]


def sufsort_lib(width):
    lib = pq.load_library(width)
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    B = Bucket64 if width == 64 else Bucket32
    vp = ct.c_void_p
    lib.transform_to_triplet.argtypes = [vp, ct.c_int, I]
    lib.transform_to_triplet_reverse.argtypes = [vp, ct.c_int, I]
    lib.initial_sort.argtypes = [vp, I, ct.POINTER(B), vp, vp, vp]
    lib.suf_sort.argtypes = [vp, vp, ct.c_int, vp, ct.POINTER(B), I, ct.c_int, vp, vp, vp, vp, I, ct.c_int]
    for f in ("transform_to_triplet", "transform_to_triplet_reverse", "initial_sort", "suf_sort"):
        getattr(lib, f).restype = None
    return lib, B


def drive_build_idx(reads, t, C, width, d):
    """src/index.c:495-585 for direction d: depth-1 seeds from C[], triplet recoding, initial_sort,
    then suf_sort slot by slot into one suffix array."""
    lib, B = sufsort_lib(width)
    dt = idx_dtype(width)
    nr, L = reads.shape
    n = nr * L
    ch = reads[:, L - 1] if d == 0 else reads[:, 0]
    C = np.asarray(C, dtype=np.int64)
    start = C[ch].astype(dt)
    size = (C[ch.astype(np.int64) + 1] - C[ch]).astype(dt)
    depth = np.ones(nr, np.uint16)
    text = np.ascontiguousarray(reads.reshape(-1).copy())
    (lib.transform_to_triplet_reverse if d else lib.transform_to_triplet)(text.ctypes.data, L, nr)
    bkt = B()
    bsize, boff, mx = np.zeros(5, dt), np.zeros(5, dt), np.zeros(1, dt)
    lib.initial_sort(text.ctypes.data, n, ct.byref(bkt), bsize.ctypes.data, boff.ctypes.data, mx.ctypes.data)
    new_idx = np.array(bkt.offs, dtype=dt)
    slots = []
    for j in range(5):
        sa = np.empty(max(int(bsize[j]), 1), dt)
        lib.suf_sort(sa.ctypes.data, text.ctypes.data, j, new_idx.ctypes.data, ct.byref(bkt), n, L,
                     start.ctypes.data, size.ctypes.data, depth.ctypes.data, None, int(boff[j]), t)
        slots.append(sa[:int(bsize[j])])
    freqs = np.array(bkt.freqs, dtype=dt)
    offs = np.array(bkt.offs, dtype=dt)
    return {"sa": np.concatenate(slots), "seeds": (start, size, depth), "new_idx": new_idx,
            "advanced": offs + freqs, "bsize": bsize, "boff": boff, "max_size": int(mx[0]), "freqs": freqs}


@pytest.mark.parametrize("name", ["iid8k_L50_t31_u32", "rep15k_L100_t63_u32", "lowc12k_L150_t63_u64",
                                  "dinuc6k_L60_t20_u32", "rep12k_L250_t95_u32"])
def test_sufsort_entry_points_drive_like_build_idx(name):
    g = load_golden(name)
    width = int(g["width"])
    for d in (0, 1):
        out = drive_build_idx(g["reads"], int(g["t"]), g["C"], width, d)
        assert sha(out["sa"]) == str(g["sha_sa%d" % d]), "suffix array %d" % d
        check_seeds(out["seeds"], g, d, name)
        assert np.array_equal(out["new_idx"], out["advanced"])
        assert int(out["bsize"].sum()) == g["reads"].size and out["max_size"] == int(out["bsize"].max())


def test_sufsort_second_text_is_sorted_afresh():
    """suf_sort keeps the last text's sort; another text (other reads, same sizes) is sorted again."""
    a = load_golden("iid8k_L50_t31_u32")
    ra = a["reads"]
    rb = np.ascontiguousarray(ra[::-1])              # same sizes, other text
    for reads in (ra, rb, ra):
        out = drive_build_idx(reads, int(a["t"]), a["C"], 32, 0)
        with pq.Pasqual(32) as P:
            P.set_reads(reads, int(a["t"]))
            P.sort(0)
            assert np.array_equal(out["sa"], P.get_sa(0))


@pytest.mark.parametrize("name", ["rep15k_L100_t63_u32", "rep20k_L100_t63_u64"])
def test_construct_index_interval_fields(tmp_path, name):
    from test_gpu_dropin import structs
    g = load_golden(name)
    width, t = int(g["width"]), int(g["t"])
    nr, L = g["reads"].shape
    fa = tmp_path / "reads.fa"
    synth.write_fasta(str(fa), g["reads"])
    lib = pq.load_library(width)
    I, Index, Graph = structs(width)
    lib.construct_index.restype = ct.POINTER(Index)
    lib.construct_index.argtypes = [ct.c_char_p] * 5 + [ct.c_int] * 4
    # a long Bloom filter: no stored read is lost to a false positive
    ix = lib.construct_index(str(fa).encode(), None, None, None, None, t, L, 100000, 2).contents
    assert int(ix.num_reads) == nr
    for d, (sf, zf, df) in enumerate((("interval_start", "interval_end", "interval_depth"),
                                       ("interval_start_bw", "interval_end_bw", "interval_depth_bw"))):
        seeds = (np.ctypeslib.as_array(getattr(ix, sf), shape=(nr,)),
                 np.ctypeslib.as_array(getattr(ix, zf), shape=(nr,)),
                 np.ctypeslib.as_array(getattr(ix, df), shape=(nr,)))
        check_seeds(seeds, g, d, "construct_index")
