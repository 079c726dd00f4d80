"""How the learned-index workload's low-complexity reads grow with the genome (no GPU needed).

The 200 Mbp workload puts 2 % of its genome in dinucleotide runs.  A read inside a run overlaps
every read that starts inside a run of the same period anywhere in the genome, so the candidates
of such a read -- and, after transitive reduction, its irreducible edges -- grow in proportion to
the genome, not to the coverage.  The reference's method (the C restatement, which equals the
reference on every golden case) run on the workload at three small genome scales shows it: the
largest number of edges on one side of one read doubles when the genome doubles.  Extrapolated, a
read of the full 200 Mbp workload has hundreds of thousands of edges on a side, far beyond the
65,535 at which the reference aborts with "assembly failed. Try a larger min overlap length."
(src/string_graph.c:469-472); the library returns PQ_ERR_TOO_MANY_EDGES there, and the workload is
measured at the scales where the reference completes."""
import numpy as np

from pasqual_gb300 import synth


def side_maxima(scale):
    from oracle import port
    _, rd, L, t = synth.make_workload("200Mbp_L150_20x_t63", scale=scale)
    rd = synth.dedup(rd)
    P = port.Port(64)
    ix = P.build_index(rd, t, seed_k=12)
    g = P.overlaps(ix, seeds=(ix["seed0"], ix["seed1"]))
    edges = int(np.maximum(g.num_B, g.num_F).max())
    cands = int(np.maximum(g.olp_B, g.olp_F).max())
    return edges, cands


def test_low_complexity_edges_grow_with_the_genome():
    got = [side_maxima(s) for s in (0.0005, 0.001, 0.002)]
    for (e0, c0), (e1, c1) in zip(got, got[1:]):
        assert 1.4 < e1 / e0 < 2.8 and 1.4 < c1 / c0 < 2.8, got
    # edges per genome base at the largest scale, times the full genome: far past 65535
    e_full = got[-1][0] / 0.002
    assert e_full > 4 * 65535, got
