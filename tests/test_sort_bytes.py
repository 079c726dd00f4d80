"""oracle/sort_bytes.py: the distinguishing prefix of every suffix (the sort's algorithmic bytes)
from the vectorised adjacent common prefixes, against a direct per-row comparison on small read
sets with repeats, identical reads and short reads."""
import numpy as np
import pytest

from oracle import port, sort_bytes
from pasqual_gb300 import synth


def direct(reads: np.ndarray, sa: np.ndarray, d: int) -> float:
    nr, L = reads.shape
    text = (reads[:, ::-1] if d else reads).reshape(-1)
    suf = [bytes(text[p:(p // L + 1) * L]) for p in sa.astype(np.int64)]
    total = 0
    for i, s in enumerate(suf):
        def lcp(a, b):
            n = 0
            while n < min(len(a), len(b)) and a[n] == b[n]:
                n += 1
            return n
        left = lcp(suf[i - 1], s) if i > 0 else 0
        right = lcp(s, suf[i + 1]) if i + 1 < len(suf) else 0
        dd = min(len(s), max(left, right) + 1)
        total += (dd + 3) // 4
    return total / len(suf)


@pytest.mark.parametrize("seed,L", [(1, 20), (2, 33), (3, 50)])
def test_distinguishing_bytes_match_direct(seed, L):
    gen = synth.genome(3000, 0.45, 0.2, (0.01, 0.01), 0.05, seed=seed)
    rd = synth.reads_for_coverage(gen, L, 8, 0.0, seed=seed + 10)
    rd = np.concatenate([rd, rd[:5]])            # identical reads: suffixes equal to the end
    P = port.Port(32)
    for d in (0, 1):
        sa = P.sort(rd, d, 1)
        text = np.ascontiguousarray((rd[:, ::-1] if d else rd).reshape(-1))
        assert sort_bytes.distinguishing_bytes(text, sa, L) == pytest.approx(direct(rd, sa, d), abs=1e-12)
