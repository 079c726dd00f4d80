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

    python tests/golden/make_golden.py [CASE ...]

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
        names = sys.argv[1:] or list(CASES) + ["import"]
        for name in names:
            if name == "import":
                make_import(tmp)
            else:
                make(name, tmp)
