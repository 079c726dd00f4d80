"""Learned index on the GPU: the training kernels against the CPU oracle, the keys against the
oracle's, every present key inside its recorded window, and the overlap set of the learned search
against the plain search and the reference's golden vectors."""
import numpy as np
import pytest

from conftest import load_golden, sha, idx_dtype
import pasqual_gb300 as pq
from oracle import learned

pytestmark = pytest.mark.gpu

# fp32 kernels against the float64 oracle: relative to the largest gradient entry
GRAD_RTOL = 1e-4


def _params(rng):
    H = learned.HIDDEN
    p = np.zeros(learned.STRIDE, np.float32)
    p[:H] = rng.normal(1.0, 0.3, H)
    p[H:2 * H] = -rng.uniform(0.0, 1.0, H)
    p[2 * H:3 * H] = rng.normal(0.0, 0.2, H)
    p[3 * H] = 0.1
    return p


@pytest.mark.parametrize("n", [1, 200, 1000])
def test_mlp_kernels_match_oracle(n):
    rng = np.random.default_rng(n)
    p = _params(rng)
    x = rng.uniform(0.0, 1.0, n).astype(np.float32)
    dy = rng.normal(0.0, 1.0, n).astype(np.float32)
    y = pq.mlp_forward(p, x)
    np.testing.assert_allclose(y, learned.mlp_forward(p, x), rtol=1e-5, atol=1e-5)
    g = pq.mlp_backward(p, x, dy)
    ref = learned.mlp_backward(p, x, dy)
    np.testing.assert_allclose(g, ref, rtol=GRAD_RTOL, atol=GRAD_RTOL * np.abs(ref).max())


@pytest.mark.parametrize("step", [1, 7])
def test_adam_step_matches_oracle(step):
    """One step of the training's joint phase (all 193 parameters, w1 and b1 included): the GPU's
    mean-squared-error gradient and Adam update against the float64 oracle, twice in a row."""
    rng = np.random.default_rng(step)
    p = _params(rng)
    k = 3 * learned.HIDDEN + 1
    m1 = rng.normal(0.0, 1e-3, k).astype(np.float32)
    m2 = rng.uniform(1e-8, 1e-6, k).astype(np.float32)
    x = rng.uniform(0.0, 1.0, 256).astype(np.float32)
    tgt = rng.normal(0.0, 0.5, 256).astype(np.float32)
    gp, ga, gb = p, m1, m2
    rp, ra, rb = p.astype(np.float64), m1.astype(np.float64), m2.astype(np.float64)
    for t in (step, step + 1):
        gp, ga, gb = pq.mlp_adam_step(gp, ga, gb, x, tgt, t, 1e-3)
        rp, ra, rb = learned.adam_step(rp, ra, rb, x, tgt, t, 1e-3)
        np.testing.assert_allclose(ga, ra, rtol=GRAD_RTOL, atol=GRAD_RTOL * np.abs(ra).max())
        np.testing.assert_allclose(gb, rb, rtol=1e-3, atol=1e-3 * np.abs(rb).max())
        # parameters move by about lr a step: compare the moves
        np.testing.assert_allclose(gp[:k] - p[:k], rp[:k] - p[:k].astype(np.float64), rtol=1e-2, atol=2e-5)
    assert np.any(gp[:2 * learned.HIDDEN] != p[:2 * learned.HIDDEN])      # the first layer trains too


@pytest.mark.parametrize("name", ["rep15k_L100_t63_u32", "lowc12k_L150_t63_u64"])
def test_learned_keys_match_oracle(name):
    g = load_golden(name)
    with pq.Pasqual(int(g["width"])) as P:
        P.construct_index(g["reads"], int(g["t"]))
        for d in (0, 1):
            keys, first = P.learned_keys(d)
            rk, rf = learned.distinct_keys(g["reads"], P.get_sa(d), d)
            assert np.array_equal(keys, rk)
            assert np.array_equal(first.astype(np.int64), rf)


@pytest.mark.parametrize("name", ["rep15k_L100_t63_u32", "lowc12k_L150_t63_u64"])
def test_every_key_inside_its_window(name):
    """Each present key's whole row group lies in [pred - e_lo, pred + e_hi) of its segment, and
    training narrows the windows of the root alone."""
    g = load_golden(name)
    with pq.Pasqual(int(g["width"])) as P:
        P.construct_index(g["reads"], int(g["t"]))
        n = P.num_reads * P.read_len
        for d in (0, 1):
            P.learned_build(d, 400)
            info = P.learned_info(d)
            m = P.learned_export(d)
            keys, first = P.learned_keys(d)
            assert info["num_keys"] == len(keys)
            pred, seg = P.learned_predict(d, keys)
            end = np.append(first[1:].astype(np.int64), n)
            lo = pred - m["err"][seg, 0]
            hi = pred + m["err"][seg, 1]
            assert np.all(lo <= first.astype(np.int64)) and np.all(end <= hi)
            # segments are found by key: boundaries ascend and every key's segment starts at or below it
            assert np.all(np.diff(m["bnd"].astype(np.int64)) > 0)
            assert np.all(m["bnd"][seg] <= keys)
            assert info["mean_window"] < info["mean_window_root"]


@pytest.mark.parametrize("name", ["iid8k_L50_t31_u32", "rep15k_L100_t63_u32", "lowc12k_L150_t63_u64",
                                  "iid5k_L60_t59_u32", "rep20k_L100_t63_u64"])
def test_learned_search_matches_plain_and_reference(name):
    """Plain backward search (mode 0) is the yardstick: the learned search's edges are identical, and
    both are the reference's."""
    g = load_golden(name)
    dt = idx_dtype(g["width"])
    out = {}
    for mode in (0, 2):
        with pq.Pasqual(int(g["width"])) as P:
            P.set_reads(g["reads"], int(g["t"]))
            P.set_seed_mode(mode)
            P.build_index()
            out[mode] = P.construct_string_graph()
            if mode == 2:
                info = P.learned_info(0)
                assert info["queries"] == 4 * P.num_reads
                assert info["misses"] <= info["queries"]
    for f in ("edge_off", "dest", "length", "etype", "trans", "num_B", "num_F", "olp_B", "olp_F"):
        assert np.array_equal(getattr(out[0], f), getattr(out[2], f)), f
    assert sha(out[2].dest.astype(dt)) == str(g["sha_dest"])


def test_trained_network_gains_over_root():
    """What the trained network adds: narrower windows, so fewer probes for the same edges."""
    g = load_golden("rep15k_L100_t63_u32")
    res = {}
    for steps in (0, 400):
        with pq.Pasqual(32) as P:
            P.set_reads(g["reads"], int(g["t"]))
            P.set_seed_mode(2)
            P.build_index()
            P.learned_build(0, steps)
            P.learned_build(1, steps)
            out = P.construct_string_graph()
            res[steps] = (out.probes, P.learned_info(0)["mean_window"], sha(out.dest))
    assert res[400][2] == res[0][2] == str(g["sha_dest"])
    assert res[400][1] < res[0][1]
    assert res[400][0] < res[0][0]
