"""Regenerate the golden fixtures in this folder from the UNMODIFIED reference.

Needs the reference sources (read where they lie) and an x86 host: it builds oracle/_ref with
oracle/Makefile, writes seeded synthetic reads as FASTA, runs oracle/_ref/ref_dump_uXX (which
drives the reference's construct_index / sufsort / construct_string_graph) and stores, per case:

* the reads the reference kept after its Bloom-filter de-duplication (codes 1..4),
* C[], suffix_count, prefix_count,
* SHA-256 digests of every array the hot path produces: both suffix arrays, both FM-indexes in
  the reference layout (OCC_bitmap, OCC_sample, reads_index), the per-node edge counts and node
  fields, and the ordered edge list (dest, overlap length, type, path trans),
* the full edge arrays for the small cases.

    python tests/golden/make_golden.py [CASE ...]     (CASE "seeds": add seed digests in place)

The fixtures with repeats or low-complexity runs (rep15k, rep20k, lowc12k, dinuc6k) were made
with an earlier version of the genome generator, so running this now writes different reads for
them.  Every fixture is pinned by its own stored reads: the tests feed them back through the
reference and compare every digest.
"""
from __future__ import annotations

import hashlib
import os
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from pasqual_gb300 import synth  # noqa: E402
from oracle import port  # noqa: E402

# name: genome length, gc, repeat fraction, divergence, low-complexity fraction, read length,
#       coverage, error rate, t, index width, keep full edge arrays
CASES = {
    "iid8k_L50_t31_u32": (8000, 0.50, 0.00, (0.0, 0.0), 0.00, 50, 30, 0.0, 31, 32, True),
    "rep15k_L100_t63_u32": (15000, 0.41, 0.10, (0.01, 0.01), 0.00, 100, 30, 0.005, 63, 32, True),
    "lowc12k_L150_t63_u64": (12000, 0.40, 0.12, (0.005, 0.02), 0.02, 150, 20, 0.003, 63, 64, True),
    "iid3k_L40_t10_u32": (3000, 0.50, 0.00, (0.0, 0.0), 0.00, 40, 40, 0.0, 10, 32, False),
    "iid5k_L60_t59_u32": (5000, 0.50, 0.00, (0.0, 0.0), 0.00, 60, 50, 0.0, 59, 32, False),
    "dinuc6k_L60_t20_u32": (6000, 0.45, 0.00, (0.0, 0.0), 0.50, 60, 30, 0.002, 20, 32, False),
    "rep20k_L100_t63_u64": (20000, 0.41, 0.10, (0.01, 0.01), 0.00, 100, 20, 0.005, 63, 64, False),
    # long reads: the sort's widest refinement words and the search's 8-word continuations
    "rep12k_L250_t95_u32": (12000, 0.45, 0.08, (0.01, 0.01), 0.00, 250, 25, 0.005, 95, 32, False),
}

DIGEST_KEYS = ["sa0", "sa1", "bitmap0", "bitmap1", "sample0", "sample1", "reads_index0",
               "reads_index1", "num_B", "num_F", "node_types", "dest", "length", "etype", "trans"]
# the per-read seed intervals the reference's sort records (index_t.interval_start/end/depth)
SEED_KEYS = ["seed_start0", "seed_size0", "seed_depth0", "seed_start1", "seed_size1", "seed_depth1"]

# Cases at the benchmark workloads' own sizes (pasqual_gb300.synth.WORKLOADS): digests only, kept
# in large/.  Their reads are not stored: a test regenerates them with the committed generator,
# checks the digest of the generated reads (sha_input), imports them through the library's FASTA
# import and checks the kept reads (sha_reads) before comparing anything else.
# name: workload, genome scale, index width
LARGE = {
    "c1_1Mbp_L50_40x_t31_u32": ("1Mbp_L50_40x_t31", 1.0, 32),
    "c2_50Mbp_L100_30x_t63_s0.1_u32": ("50Mbp_L100_30x_t63", 0.1, 32),
    # the learned-index workload's shape (2 % dinucleotide runs, 150 bp) and the large workload's
    # (15 % repeats at 0.5-2 %, t = 55), 64-bit index, at small genome scale
    "c4_200Mbp_L150_20x_t63_s0.002_u64": ("200Mbp_L150_20x_t63", 0.002, 64),
    "c5_250Mbp_L100_20x_t55_s0.002_u64": ("250Mbp_L100_20x_t55", 0.002, 64),
}
LARGE_DIR = os.path.join(HERE, "large")


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def case_reads(name: str) -> np.ndarray:
    g_len, gc, rep, div, lowc, L, cov, err, t, width, full = CASES[name]
    seed = sum(map(ord, name))
    g = synth.genome(g_len, gc, rep, div, lowc, seed=seed)
    return synth.reads_for_coverage(g, L, cov, err, seed=seed + 1)


def reference_fixture(reads: np.ndarray, t: int, width: int, full: bool, tmp: str,
                      bloom_m: int = 36) -> dict:
    """Write reads as FASTA, run the reference on them in `tmp` and return the fixture arrays."""
    L = reads.shape[1]
    fa = os.path.join(tmp, "reads.fa")
    synth.write_fasta(fa, reads)
    d = port.run_ref_dump(fa, L, t, os.path.join(tmp, "dump"), width=width, bloom_m=bloom_m)
    idt = np.uint64 if width == 64 else np.uint32
    d["dest"] = d["dest"].astype(idt)
    out = {"reads": d["reads"], "t": np.int64(t), "width": np.int64(width), "C": d["C"],
           "suffix_count": d["suffix_count"], "prefix_count": d["prefix_count"],
           "num_edges": np.int64(len(d["dest"]))}
    for k in DIGEST_KEYS:
        out["sha_" + k] = np.array(digest(d[k]))
    for dd in (0, 1):
        for j, k in enumerate(("start", "size", "depth")):
            out["sha_seed_%s%d" % (k, dd)] = np.array(digest(d["seed%d" % dd][j]))
    if full:
        for k in ("num_B", "num_F", "dest", "length", "etype", "trans"):
            out["full_" + k] = d[k]
    return out


def compute(name: str, tmp: str) -> dict:
    """The fixture of one case: its seeded reads through the reference, run in `tmp`."""
    g_len, gc, rep, div, lowc, L, cov, err, t, width, full = CASES[name]
    return reference_fixture(case_reads(name), t, width, full, tmp)


def make(name: str, tmp: str) -> None:
    out = compute(name, tmp)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)
    print("%-24s reads=%-6d edges=%-7d" % (name, out["reads"].shape[0], int(out["num_edges"])))


def add_seed_digests(name: str, tmp: str) -> None:
    """Add the digests of the reference's seed intervals to an existing fixture, computed from its
    own stored reads (the reads and every other entry stay as they are)."""
    p = os.path.join(HERE, name + ".npz")
    z = np.load(p)
    out = {k: z[k] for k in z.files}
    L = out["reads"].shape[1]
    fa = os.path.join(tmp, name + ".fa")
    synth.write_fasta(fa, out["reads"])
    d = port.run_ref_dump(fa, L, int(out["t"]), os.path.join(tmp, name), width=int(out["width"]),
                          bloom_m=100000)           # long filter: no read lost to a false positive
    assert np.array_equal(d["reads"], out["reads"])        # no read dropped on re-import
    for dd in (0, 1):
        for j, k in enumerate(("start", "size", "depth")):
            out["sha_seed_%s%d" % (k, dd)] = np.array(digest(d["seed%d" % dd][j]))
    np.savez_compressed(p, **out)
    print("%-24s seed digests added" % name)


def large_input(name: str) -> tuple[np.ndarray, int, int, int]:
    """Raw (not yet de-duplicated) reads of a workload-size case, L, t, index width."""
    workload, scale, width = LARGE[name]
    _, rd, L, t = synth.make_workload(workload, scale=scale)
    return rd, L, t, width


def make_large(name: str, tmp: str, threads: int = 0) -> None:
    """Digest-only fixture of a workload-size case, plus the contigs.fa digest of the reference's
    own CLI (OMP_NUM_THREADS=1) on the same FASTA."""
    import subprocess
    rd, L, t, width = large_input(name)
    fa = os.path.join(tmp, name + ".fa")
    synth.write_fasta(fa, rd)
    d = port.run_ref_dump(fa, L, t, os.path.join(tmp, name), width=width,
                          threads=threads or os.cpu_count() or 1)
    out = {"workload": np.array(LARGE[name][0]), "scale": np.float64(LARGE[name][1]),
           "read_len": np.int64(L), "t": np.int64(t), "width": np.int64(width),
           "raw_reads": np.int64(rd.shape[0]), "sha_input": np.array(digest(rd)),
           "num_reads": np.int64(d["reads"].shape[0]), "sha_reads": np.array(digest(d["reads"])),
           "C": d["C"], "suffix_count": d["suffix_count"], "prefix_count": d["prefix_count"],
           "num_edges": np.int64(len(d["dest"]))}
    idt = np.uint64 if width == 64 else np.uint32
    d["dest"] = d["dest"].astype(idt)
    for k in DIGEST_KEYS:
        out["sha_" + k] = np.array(digest(d[k]))
    for dd in (0, 1):
        for j, k in enumerate(("start", "size", "depth")):
            out["sha_seed_%s%d" % (k, dd)] = np.array(digest(d["seed%d" % dd][j]))
    run = os.path.join(tmp, name + "_cli")
    os.makedirs(run, exist_ok=True)
    exe = os.path.join(port.REF, "pasqual_omp_u%d" % width)
    subprocess.run([exe, "--singlereads", fa, "-l", str(L), "-t", str(t)], cwd=run, check=True,
                   env=dict(os.environ, OMP_NUM_THREADS="1"), stdout=subprocess.DEVNULL)
    with open(os.path.join(run, "contigs.fa"), "rb") as f:
        contigs = f.read()
    out["sha_contigs"] = np.array(hashlib.sha256(contigs).hexdigest())
    out["contigs"] = np.int64(contigs.count(b">"))
    os.makedirs(LARGE_DIR, exist_ok=True)
    np.savez_compressed(os.path.join(LARGE_DIR, name + ".npz"), **out)
    print("%-32s raw=%d kept=%d edges=%d contigs=%d" % (name, rd.shape[0], out["num_reads"],
                                                       out["num_edges"], out["contigs"]))


IMPORT_FASTA = "import_L60.fa.gz"


def make_import(tmp: str) -> None:
    """FASTA import + Bloom de-duplication: exact duplicates, reverse-complement duplicates,
    reads with N, lowercase bases; kept reads of both index widths (their Bloom hashes wrap in
    the index width, so the kept sets can differ)."""
    import gzip
    rng = np.random.default_rng(7)
    g = synth.genome(30000, 0.5, seed=77)
    rd = synth.reads(g, 60, 6000, 0.01, seed=78)
    seqs = [bytes(synth.ACGT[r]) for r in rd]
    extra = []
    for i in rng.choice(len(seqs), 400, replace=False):
        extra.append(seqs[i])                                        # exact duplicate
    for i in rng.choice(len(seqs), 400, replace=False):
        extra.append(bytes(synth.ACGT[synth.revcomp(rd[i])]))       # reverse complement
    for i in rng.choice(len(seqs), 100, replace=False):
        s = bytearray(seqs[i]); s[int(rng.integers(0, 60))] = ord("N"); extra.append(bytes(s))
    for i in rng.choice(len(seqs), 100, replace=False):
        extra.append(seqs[i].lower())                                # lowercase duplicate
    allseq = seqs + extra
    order = rng.permutation(len(allseq))
    text = b"".join(b">q%d\n%s\n" % (k, allseq[j]) for k, j in enumerate(order))
    with gzip.open(os.path.join(HERE, IMPORT_FASTA), "wb") as f:
        f.write(text)
    fa = os.path.join(tmp, "import.fa")
    with open(fa, "wb") as f:
        f.write(text)
    out = {"records": np.int64(len(allseq))}
    for width in (32, 64):
        d = port.run_ref_dump(fa, 60, 31, os.path.join(tmp, "imp%d" % width), width=width)
        out["kept%d" % width] = np.int64(d["reads"].shape[0])
        out["sha_reads%d" % width] = np.array(digest(d["reads"]))
    np.savez_compressed(os.path.join(HERE, "import_L60.npz"), **out)
    print("import: records=%d kept u32=%d u64=%d" % (len(allseq), out["kept32"], out["kept64"]))


if __name__ == "__main__":
    port.build(ref=True)
    with tempfile.TemporaryDirectory() as tmp:
        names = sys.argv[1:] or list(CASES) + ["import"] + list(LARGE)
        for name in names:
            if name == "import":
                make_import(tmp)
            elif name == "seeds":
                for c in CASES:
                    add_seed_digests(c, tmp)
            elif name in LARGE:
                make_large(name, tmp)
            else:
                make(name, tmp)
