"""The learned-index oracle pinned on the CPU: its analytic gradient against central differences,
its keys against a per-row loop over the text."""
import numpy as np

from oracle import learned


def _params(rng):
    H = learned.HIDDEN
    p = np.zeros(learned.STRIDE)
    p[:H] = rng.normal(1.0, 0.3, H)
    p[H:2 * H] = -rng.uniform(0.0, 1.0, H)
    p[2 * H:3 * H] = rng.normal(0.0, 0.2, H)
    p[3 * H] = 0.1
    return p


def test_gradient_matches_finite_differences():
    rng = np.random.default_rng(5)
    p = _params(rng)
    x = rng.uniform(0.0, 1.0, 300)
    dy = rng.normal(0.0, 1.0, 300)
    g = learned.mlp_backward(p, x, dy)
    fd = learned.finite_difference(p, x, dy)
    np.testing.assert_allclose(g, fd, rtol=1e-6, atol=1e-6 * np.abs(fd).max())


def test_keys_against_per_row_loop():
    rng = np.random.default_rng(6)
    reads = rng.integers(1, 5, size=(40, 21), dtype=np.uint8)
    L = reads.shape[1]
    for d in (0, 1):
        text = learned.text_of(reads, d)
        sa = rng.permutation(len(text))              # any row order: keys are per row
        got = learned.row_keys(reads, sa, d)
        for r, p in enumerate(sa):
            m = L - p % L
            k = 0
            for j in range(16):
                k = k * 4 + (int(text[p + j]) - 1 if j < m else 0)
            assert int(got[r]) == k


def test_distinct_keys_are_group_heads():
    reads = np.array([[1, 2, 3, 4, 1, 2, 3, 4, 1, 2, 3, 4, 1, 2, 3, 4, 1, 2],
                      [1, 2, 3, 4, 1, 2, 3, 4, 1, 2, 3, 4, 1, 2, 3, 4, 1, 2]], np.uint8)
    text = learned.text_of(reads, 0)
    L = reads.shape[1]
    # canonical order: suffix string with end-of-read lowest, ties by position
    sufs = [tuple(text[p:(p // L + 1) * L]) for p in range(len(text))]
    sa = np.array(sorted(range(len(text)), key=lambda p: (sufs[p], p)))
    keys, first = learned.distinct_keys(reads, sa, 0)
    assert np.all(np.diff(keys.astype(np.int64)) > 0)      # keys never decrease down the SA
    assert first[0] == 0 and len(np.unique(first)) == len(first)
