"""Seeded synthetic genomes and short reads with the shapes PASQUAL is benchmarked on.

The reference ships one small genome and a read simulator (``data/gen_reads-0.9.tgz``,
``gen_reads/gen_reads.c:109-231``): uniform start positions, 50 % of reads from the reverse-
complement strand, substitution errors spread evenly over the three other bases, fixed read
length.  This module restates those sampling rules with numpy's PCG64 generator (the reference
tool uses glibc ``rand()``, so reads are not byte-identical to its output, only identically
distributed) and adds the genome shapes the benchmark workloads name: GC content, repeat copies
of 1-5 kbp segments at a substitution divergence, and low-complexity dinucleotide runs.

Bases are returned as codes 1..4 (A, C, G, T), the alphabet the reference's index uses after
import (``src/index.c:282-303``).
"""
from __future__ import annotations

import numpy as np

ACGT = np.frombuffer(b"@ACGT", dtype=np.uint8)  # code -> ASCII, code 0 unused


def genome(length: int, gc: float = 0.5, repeat_frac: float = 0.0,
           divergence=(0.01, 0.01), lowcomplex_frac: float = 0.0, seed: int = 1) -> np.ndarray:
    """Return a genome of ``length`` bases as uint8 codes 1..4.

    i.i.d. bases at the given GC fraction; then uniform 1-5 kbp segments are copied to uniform
    positions, each copy mutated at a divergence drawn uniformly from ``divergence``, until
    ``repeat_frac`` of the length has been written; then dinucleotide runs (e.g. ACACAC...) of
    20-200 bp cover ``lowcomplex_frac`` of the length.
    """
    rng = np.random.default_rng(seed)
    p = [(1 - gc) / 2, gc / 2, gc / 2, (1 - gc) / 2]
    g = rng.choice(4, size=length, p=p).astype(np.uint8)
    target = int(repeat_frac * length)
    done = 0
    while done < target and length > 6000:
        seg_len = int(rng.integers(1000, 5001))
        src = int(rng.integers(0, length - seg_len))
        dst = int(rng.integers(0, length - seg_len))
        div = float(rng.uniform(divergence[0], divergence[1]))
        seg = g[src:src + seg_len].copy()
        mut = rng.random(seg_len) < div
        seg[mut] = (seg[mut] + rng.integers(1, 4, size=int(mut.sum()))) % 4
        g[dst:dst + seg_len] = seg
        done += seg_len
    target = int(lowcomplex_frac * length)
    done = 0
    while done < target and length > 400:
        run = int(rng.integers(20, 201))
        dst = int(rng.integers(0, length - run))
        a, b = rng.choice(4, size=2, replace=False)
        g[dst:dst + run] = np.where(np.arange(run) % 2 == 0, a, b)
        done += run
    return (g + 1).astype(np.uint8)


def revcomp(codes: np.ndarray) -> np.ndarray:
    """Reverse complement of code arrays along the last axis (A<->T, C<->G)."""
    return (5 - codes[..., ::-1]).astype(np.uint8)


def reads(g: np.ndarray, read_len: int, num_reads: int, error: float = 0.0,
          seed: int = 2) -> np.ndarray:
    """Sample ``num_reads`` fixed-length reads (uint8 codes, shape [num_reads, read_len]).

    Uniform start, strand chosen with probability 1/2 (reverse complement), and a substitution
    error at each base with probability ``error``, replaced by one of the three other bases with
    equal probability.
    """
    rng = np.random.default_rng(seed)
    G = g.shape[0]
    starts = rng.integers(0, G - read_len + 1, size=num_reads)
    rc = rng.random(num_reads) < 0.5
    r = np.empty((num_reads, read_len), dtype=np.uint8)
    ar = np.arange(read_len)
    chunk = 1 << 18
    for s in range(0, num_reads, chunk):
        e = min(num_reads, s + chunk)
        blk = g[starts[s:e, None] + ar]
        m = rc[s:e]
        blk[m] = revcomp(blk[m])
        r[s:e] = blk
    if error > 0 and r.size:
        # error positions: Binomial(total, error) distinct positions, uniform
        k = int(rng.binomial(r.size, error))
        pos = np.unique(rng.integers(0, r.size, size=k))
        flat = r.reshape(-1)
        shift = rng.integers(1, 4, size=pos.size).astype(np.uint8)
        flat[pos] = ((flat[pos] - 1 + shift) % 4) + 1
    return r


def reads_for_coverage(g: np.ndarray, read_len: int, coverage: float, error: float = 0.0,
                       seed: int = 2) -> np.ndarray:
    """Reads at ``coverage`` x: num_reads = genome_length * coverage / read_len."""
    n = int(g.shape[0] * coverage // read_len)
    return reads(g, read_len, n, error, seed)


def write_fasta(path: str, rd: np.ndarray) -> None:
    """Write reads as the 2-line FASTA the reference imports (``src/index.c:197-365``)."""
    seqs = ACGT[rd]
    n, L = seqs.shape
    buf = np.empty((n, L + 1), dtype=np.uint8)
    buf[:, :L] = seqs
    buf[:, L] = ord("\n")
    with open(path, "wb") as f:
        step = 1 << 18
        for s in range(0, n, step):
            block = buf[s:s + step]
            lines = [b">r%d\n" % (s + i) + bytes(block[i]) for i in range(block.shape[0])]
            f.write(b"".join(lines))


# Benchmark workload shapes, named by what they are (genome size, read length, coverage).
WORKLOADS = {
    "1Mbp_L50_40x_t31": dict(genome=1_000_000, gc=0.5, repeat=0.0, div=(0.0, 0.0), lowc=0.0,
                             L=50, cov=40, err=0.0, t=31),
    "50Mbp_L100_30x_t63": dict(genome=50_000_000, gc=0.41, repeat=0.10, div=(0.01, 0.01),
                               lowc=0.0, L=100, cov=30, err=0.005, t=63),
    # learned-index workload: 12 % repeats, 2 % dinucleotide runs; 64-bit index
    "200Mbp_L150_20x_t63": dict(genome=200_000_000, gc=0.40, repeat=0.12, div=(0.01, 0.01),
                                lowc=0.02, L=150, cov=20, err=0.003, t=63, index=64),
    # large single-GPU workload: 15 % repeats at 0.5-2 % divergence, 50 M reads, 64-bit index,
    # 5 G suffixes per index (sorted in chunks)
    "250Mbp_L100_20x_t55": dict(genome=250_000_000, gc=0.42, repeat=0.15, div=(0.005, 0.02),
                                lowc=0.0, L=100, cov=20, err=0.005, t=55, index=64),
}

# Queued-search workload: one genome, several read sets, each with its own read length (uniform
# in [75, 250]) and min overlap (from {31, 47, 63, 95}, below L - 4); together 25x coverage.
BATCHED = {
    "100Mbp_L75-250_25x_batched": dict(genome=100_000_000, gc=0.45, repeat=0.08, div=(0.01, 0.01),
                                       lowc=0.0, L=(75, 250), cov=25, err=0.005,
                                       t=(31, 47, 63, 95), batches=8),
}


def make_workload(name: str, scale: float = 1.0, seed: int = 11):
    """Genome and reads of a named workload; ``scale`` shrinks the genome (same coverage)."""
    w = WORKLOADS[name]
    glen = max(int(w["genome"] * scale), 4 * w["L"])
    gen = genome(glen, w["gc"], w["repeat"], w["div"], w["lowc"], seed=seed)
    rd = reads_for_coverage(gen, w["L"], w["cov"], w["err"], seed=seed + 1)
    return gen, rd, w["L"], w["t"]


def _hash_rows(codes: np.ndarray) -> np.ndarray:
    """64-bit hash per row of base codes (splitmix-style mixing over 2-bit packed words)."""
    n, L = codes.shape
    h = np.full(n, np.uint64(0x9E3779B97F4A7C15), dtype=np.uint64)
    m1, m2 = np.uint64(0xBF58476D1CE4E5B9), np.uint64(0x94D049BB133111EB)
    for s in range(0, L, 32):
        blk = codes[:, s:s + 32]
        k = blk.shape[1]
        pow4 = (np.uint64(4) ** np.arange(k - 1, -1, -1, dtype=np.uint64)).astype(np.uint64)
        w = (blk.astype(np.uint64) - np.uint64(1)) @ pow4
        w ^= np.uint64(k)
        h ^= w
        h ^= h >> np.uint64(30)
        h *= m1
        h ^= h >> np.uint64(27)
        h *= m2
        h ^= h >> np.uint64(31)
    return h


def dedup(rd: np.ndarray) -> np.ndarray:
    """Keep the first read of every group of reads that are equal or reverse complements of each
    other (the duplicates the reference's Bloom filter is there to drop, src/index.c:325-333,
    without its false positives).  Order of first occurrence is kept."""
    if rd.shape[0] == 0:
        return rd
    hf = _hash_rows(rd)
    hr = _hash_rows(revcomp(rd))
    key = np.minimum(hf, hr)
    _, first = np.unique(key, return_index=True)
    first.sort()
    return np.ascontiguousarray(rd[first])


def make_batches(name: str = "100Mbp_L75-250_25x_batched", scale: float = 1.0, seed: int = 31):
    """Read sets of a queued-search workload: [(reads, L, t)], de-duplicated."""
    w = BATCHED[name]
    glen = max(int(w["genome"] * scale), 4 * w["L"][1])
    gen = genome(glen, w["gc"], w["repeat"], w["div"], w["lowc"], seed=seed)
    rng = np.random.default_rng(seed + 1000)
    out = []
    for b in range(w["batches"]):
        L = int(rng.integers(w["L"][0], w["L"][1] + 1))
        ts = [x for x in w["t"] if x < L - 4]
        t = int(ts[int(rng.integers(0, len(ts)))])
        rd = reads_for_coverage(gen, L, w["cov"] / w["batches"], w["err"], seed=seed + 1 + b)
        out.append((dedup(rd), L, t))
    return out
