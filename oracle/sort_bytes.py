"""Algorithmic bytes of the suffix sort on a workload sample: per suffix, ceil(D_i / 4) bytes of
2-bit text, where D_i = min(length_i, max(LCP_i, LCP_{i+1}) + 1) is the prefix that tells suffix
i apart from its neighbours in suffix order (LCP_i = common prefix of rows i - 1 and i), plus one
suffix-array entry written.  Both directions, from the oracle's suffix arrays.

TEST INFRASTRUCTURE (CPU): run by hand to measure the per-suffix figure the benchmark's sort
roofline uses, e.g.

    python -m oracle.sort_bytes 250Mbp_L100_20x_t55 0.002

The figure is a property of the workload's shape (read length, coverage, repeat content), so a
sample of the genome gives it; the result is recorded in the profiles summary of the workload.
"""
from __future__ import annotations

import sys

import numpy as np

from oracle import port
from pasqual_gb300 import synth


def lcp_adjacent(text: np.ndarray, sa: np.ndarray, L: int) -> np.ndarray:
    """lcp[i] = common prefix (bases, within each read) of the suffixes at rows i - 1 and i."""
    n = len(sa)
    pos = sa.astype(np.int64)
    ln = L - pos % L
    a, b = pos[:-1], pos[1:]
    m = np.minimum(ln[:-1], ln[1:])
    lcp = np.zeros(n, np.int64)
    live = np.ones(n - 1, bool)
    cur = np.zeros(n - 1, np.int64)
    for j in range(L):
        idx = np.nonzero(live)[0]
        if idx.size == 0:
            break
        inside = j < m[idx]
        live[idx[~inside]] = False
        idx = idx[inside]
        ok = text[a[idx] + j] == text[b[idx] + j]
        cur[idx[ok]] += 1
        live[idx[~ok]] = False
    lcp[1:] = cur
    return lcp


def distinguishing_bytes(text: np.ndarray, sa: np.ndarray, L: int) -> float:
    """Mean ceil(D_i / 4) over the suffix array."""
    lcp = lcp_adjacent(text, sa, L)
    ln = L - sa.astype(np.int64) % L
    nxt = np.append(lcp[1:], 0)
    d = np.minimum(ln, np.maximum(lcp, nxt) + 1)
    return float(np.mean((d + 3) // 4))


def main(workload: str, scale: float) -> None:
    _, rd, L, t = synth.make_workload(workload, scale=scale)
    rd = synth.dedup(rd)
    width = synth.WORKLOADS[workload].get("index", 32)
    P = port.Port(width)
    ix = P.build_index(rd, t)
    per = []
    for d in (0, 1):
        text = (rd[:, ::-1] if d else rd).reshape(-1)
        per.append(distinguishing_bytes(np.ascontiguousarray(text), ix["sa%d" % d], L))
    idx_bytes = width // 8
    print("workload %s at scale %g: %d reads x %d, %d suffixes per index" % (workload, scale, rd.shape[0], L,
                                                                             rd.size))
    print("mean ceil(D/4) bytes per suffix: forward %.3f, backward %.3f" % tuple(per))
    print("sort_bytes_per_suffix = %.2f" % (sum(per) / 2 + idx_bytes))


if __name__ == "__main__":
    main(sys.argv[1], float(sys.argv[2]))
