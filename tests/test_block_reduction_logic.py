"""The block tier's two ways to reduce one side's candidates, restated on the host and checked
against each other on random candidate sets rich in prefixes, equal continuations and repeated
read ids.

* Pairwise (the shared-memory variant, and `reduce_gathered` of the lean tier): a candidate is
  covered when another candidate's continuation is a proper prefix of its own; trans counts the
  continuations that start with its own; a second-kind candidate yields to a first-kind one with
  exactly its continuation; the emitted candidates are ordered by (continuation, read id) with a
  continuation before its extensions -- the order of the reference's DFS
  (src/string_graph.c:469-731).
* Sorted (the global-memory variant, `block_sorted_side` in pasqual_gb300/csrc/pq_search.cu):
  order by (continuation bases padded with A, length, read id), then one walk over the common
  prefixes of neighbours.

The GPU tests compare the kernels themselves with the reference's method; this pins the
algorithm the sorted variant relies on, on inputs far more adversarial than real reads.
"""
import random

import pytest

FIRST, SECOND = 0, 1


def pairwise(cands, self_id):
    """cands: (continuation tuple, kind, read id); returns [(index, trans)] in DFS order."""
    out = []
    for i, (c, kind, rid) in enumerate(cands):
        covered = False
        trans = 0
        first_same = False
        for (x, kx, _) in cands:
            if len(x) < len(c) and c[:len(x)] == x:
                covered = True
                break
            if len(x) >= len(c) and x[:len(c)] == c:
                trans += 1
                if len(x) == len(c) and kx == FIRST:
                    first_same = True
        if covered or rid == self_id or (kind != FIRST and first_same):
            continue
        out.append((i, trans))
    out.sort(key=lambda e: (cands[e[0]][0], cands[e[0]][2]))   # tuple order: a prefix first
    return out


def sorted_walk(cands, self_id, M):
    """The sorted variant as the kernel computes it."""
    order = sorted(range(len(cands)),
                   key=lambda i: (cands[i][0] + (0,) * (M - len(cands[i][0])), len(cands[i][0]),
                                  cands[i][2]))
    m = len(order)
    lens = [len(cands[i][0]) for i in order]
    lcp = [0] * m
    for k in range(1, m):
        a, b = cands[order[k - 1]][0], cands[order[k]][0]
        pa, pb = a + (0,) * (M - len(a)), b + (0,) * (M - len(b))
        n = 0
        while n < M and pa[n] == pb[n]:
            n += 1
        lcp[k] = min(n, lens[k - 1], lens[k])
    out = []
    i = 0
    while i < m:
        lr = lens[i]
        k = i + 1
        while k < m and lcp[k] >= lr and lens[k] == lr:
            k += 1
        eq_end = k
        while k < m and lcp[k] >= lr:
            k += 1
        trans = k - i
        first_same = any(cands[order[j]][1] == FIRST for j in range(i, eq_end))
        for j in range(i, eq_end):
            c = order[j]
            if cands[c][2] == self_id or (cands[c][1] != FIRST and first_same):
                continue
            out.append((c, trans))
        i = k
    return out


def random_side(rng, M):
    """Continuations drawn from a few periodic motifs (as in dinucleotide runs) and random ones,
    cut at random lengths, so prefixes, equal continuations and shared read ids are common."""
    motifs = [tuple(rng.choice([(0, 1), (2, 3), (0,), (1, 0, 2)]) * M)[:M] for _ in range(3)]
    motifs.append(tuple(rng.randrange(4) for _ in range(M)))
    cands = []
    for _ in range(rng.randrange(1, 90)):
        base = rng.choice(motifs)
        n = rng.randrange(1, M + 1)
        c = list(base[:n])
        if rng.random() < 0.3 and n > 1:
            c[rng.randrange(n)] = rng.randrange(4)
        cands.append((tuple(c), rng.choice([FIRST, SECOND]), rng.randrange(12)))
    return cands


@pytest.mark.parametrize("seed", range(300))
def test_sorted_walk_equals_pairwise(seed):
    rng = random.Random(seed)
    M = rng.choice([5, 13, 40, 87])
    cands = random_side(rng, M)
    self_id = rng.randrange(12)
    assert sorted_walk(cands, self_id, M) == pairwise(cands, self_id)
