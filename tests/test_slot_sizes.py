"""Sort-slot sizes of the drop-in index (index_t size/offset/max_size of both directions, the
reference's initial_sort bookkeeping): the parallel histogram of pasqual_gb300/csrc/pq_slots.h
against a direct count of every suffix's first-prefix rank.  Host code only: the header is
compiled into a small harness with the host compiler."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HARNESS = r"""
#include <cstdio>
#include <cstdlib>
#include <vector>
#include "pq_slots.h"
int main(int argc, char** argv) {
    // argv: reads file, num_reads, L, dir, threads; prints the 85-bin histogram
    const size_t nr = strtoull(argv[2], 0, 10);
    const int L = atoi(argv[3]), dir = atoi(argv[4]), threads = atoi(argv[5]);
    std::vector<uint8_t> reads(nr * L + 1);
    FILE* f = fopen(argv[1], "rb");
    if (nr * L && fread(reads.data(), 1, nr * L, f) != nr * L) return 1;
    fclose(f);
    uint64_t hist[85];
    pq_slots::prefix_rank_histogram(reads.data(), nr, L, dir, hist, threads);
    for (int i = 0; i < 85; ++i) printf("%llu\n", (unsigned long long)hist[i]);
    unsigned long long size[5], off[5], mx;
    pq_slots::slot_sizes<unsigned long long>(reads.data(), nr, L, dir, size, off, &mx, threads);
    for (int k = 0; k < 5; ++k) printf("%llu %llu\n", size[k], off[k]);
    printf("%llu\n", mx);
    return 0;
}
"""


def direct_histogram(reads, dir_):
    """rank of a suffix = sum over its first min(3, remaining) bases i of q_i * span(i + 1) + 1,
    spans (21, 5, 1): a string comes before its extensions"""
    span = (21, 5, 1)
    h = np.zeros(85, np.int64)
    seqs = reads[:, ::-1] if dir_ else reads
    L = reads.shape[1]
    for j in range(L):
        ln = min(3, L - j)
        r = np.zeros(reads.shape[0], np.int64)
        for i in range(ln):
            r += (seqs[:, j + i].astype(np.int64) - 1) * span[i] + 1
        h += np.bincount(r, minlength=85)
    return h


@pytest.fixture(scope="module")
def harness(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("no host C++ compiler")
    d = tmp_path_factory.mktemp("slots")
    src = d / "h.cpp"
    src.write_text(HARNESS)
    exe = d / "h"
    subprocess.run([gxx, "-O2", "-std=c++17", "-pthread", "-I", os.path.join(ROOT, "pasqual_gb300", "csrc"),
                    str(src), "-o", str(exe)], check=True)
    return str(exe), d


@pytest.mark.parametrize("L", [1, 2, 3, 4, 37, 100])
@pytest.mark.parametrize("threads", [1, 5])
def test_slot_histogram_matches_direct_count(harness, L, threads):
    exe, d = harness
    rng = np.random.default_rng(L * 7 + threads)
    reads = rng.integers(1, 5, (3001, L), dtype=np.uint8)
    path = d / ("r%d.bin" % L)
    path.write_bytes(reads.tobytes())
    for dir_ in (0, 1):
        out = subprocess.run([exe, str(path), str(reads.shape[0]), str(L), str(dir_), str(threads)],
                             capture_output=True, text=True, check=True).stdout.split("\n")
        hist = np.array([int(x) for x in out[:85]])
        want = direct_histogram(reads, dir_)
        assert np.array_equal(hist, want), (L, dir_)
        assert hist.sum() == reads.size
        sizes = [tuple(int(v) for v in ln.split()) for ln in out[85:90]]
        for k, (sz, off) in enumerate(sizes):
            assert sz == int(want[17 * k:17 * k + 17].sum())
            assert off == int(want[:17 * k].sum())
        assert int(out[90]) == max(s for s, _ in sizes)


@pytest.mark.parametrize("name", ["iid8k_L50_t31_u32", "lowc12k_L150_t63_u64"])
def test_slot_sizes_match_reference(harness, tmp_path, name):
    """The same sizes the reference's own initial_sort leaves in index_t, on a golden case's
    reads (fed back through the reference with a Bloom filter long enough to keep them all)."""
    from conftest import GOLDEN
    from oracle import port
    from pasqual_gb300 import synth
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    port.build(ref=True)
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    reads, t, width = z["reads"], int(z["t"]), int(z["width"])
    fa = tmp_path / "r.fa"
    synth.write_fasta(str(fa), reads)
    d = port.run_ref_dump(str(fa), reads.shape[1], t, str(tmp_path / "d"), width=width, bloom_m=100000)
    assert np.array_equal(d["reads"], reads)
    exe, _ = harness
    path = tmp_path / "r.bin"
    path.write_bytes(reads.tobytes())
    for dir_, tag in ((0, "fw"), (1, "bw")):
        out = subprocess.run([exe, str(path), str(reads.shape[0]), str(reads.shape[1]), str(dir_), "4"],
                             capture_output=True, text=True, check=True).stdout.split("\n")
        sizes = [tuple(int(v) for v in ln.split()) for ln in out[85:90]]
        assert [s for s, _ in sizes] == d["meta"]["size_" + tag]
        assert [o for _, o in sizes] == d["meta"]["offset_" + tag]
        assert int(out[90]) == d["meta"]["max_size_" + tag]
