"""contigs.fa byte parity with the reference (its `OMP_NUM_THREADS=1` output) on the host side of
the drop-in path: the reference CLI run end to end against reads imported by this library, their
overlap graph from the oracle (which the GPU tests pin edge for edge to the CUDA search), nodes
built by pq_string_graph_from_csr and the reference's own assemble().  Needs the reference's
sources (x86), so it runs where the oracle recipe can compile them."""
import os
import subprocess
import sys

import pytest

from conftest import ROOT
from pasqual_gb300 import build, synth



@pytest.mark.parametrize("width,L,t,glen,cov,seed,lowc,err", [(32, 100, 63, 300000, 20, 5, 0.0, 0.003),
                                                              (64, 75, 41, 200000, 25, 6, 0.0, 0.003),
                                                              (32, 100, 55, 150000, 25, 9, 0.01, 0.01)])
def test_contigs_match_reference(tmp_path, width, L, t, glen, cov, seed, lowc, err):
    from oracle import port
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    build.build()
    port.build(ref=True)
    g = synth.genome(glen, 0.42, 0.08, (0.01, 0.03), lowc, seed=seed)
    rd = synth.reads_for_coverage(g, L, cov, err, seed=seed + 1)
    fa = tmp_path / "reads.fa"
    synth.write_fasta(str(fa), rd)
    env = dict(os.environ, OMP_NUM_THREADS="1")
    ref_dir, my_dir = tmp_path / "ref", tmp_path / "mine"
    ref_dir.mkdir()
    my_dir.mkdir()
    exe = os.path.join(ROOT, "oracle", "_ref", "pasqual_omp_u%d" % width)
    r = subprocess.run([exe, "--singlereads", str(fa), "-l", str(L), "-t", str(t)], cwd=str(ref_dir),
                       env=env, capture_output=True, text=True, timeout=600)
    assert r.returncode == 0, r.stderr
    m = subprocess.run([sys.executable, os.path.join(ROOT, "tests", "contigs_from_csr.py"), str(fa),
                        str(L), str(t), str(width)], cwd=str(my_dir), env=env, capture_output=True,
                       text=True, timeout=600)
    assert m.returncode == 0, m.stderr
    want = (ref_dir / "contigs.fa").read_bytes()
    got = (my_dir / "contigs.fa").read_bytes()
    assert want.count(b">") > 3            # a graph with several contigs, not a trivial one
    assert got == want
