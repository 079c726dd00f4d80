import glob
import hashlib
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def golden_cases():
    """Index/overlap golden cases (the FASTA-import case has its own test)."""
    names = (os.path.basename(p)[:-4] for p in glob.glob(os.path.join(GOLDEN, "*.npz")))
    return sorted(n for n in names if not n.startswith("import"))


def load_golden(name):
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return {k: z[k] for k in z.files}


def sha(a):
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()


def idx_dtype(width):
    return np.uint64 if int(width) == 64 else np.uint32


LARGE = os.path.join(GOLDEN, "large")


def large_cases():
    """Digest-only fixtures at the benchmark workloads' own sizes (tests/golden/large/)."""
    return sorted(os.path.basename(p)[:-4] for p in glob.glob(os.path.join(LARGE, "*.npz")))


def load_large(name):
    z = np.load(os.path.join(LARGE, name + ".npz"))
    return {k: z[k] for k in z.files}


def large_kept_reads(g, tmp_path):
    """Regenerate a workload-size case's reads with the committed generator, check them against
    the fixture, import them through the library's FASTA import (the reference's Bloom-filter
    de-duplication) and check the kept reads.  Returns them as uint8 [num_reads, L]."""
    from pasqual_gb300 import synth
    from test_dropin_host import import_fasta
    _, raw, L, t = synth.make_workload(str(g["workload"]), scale=float(g["scale"]))
    assert raw.shape[0] == int(g["raw_reads"]) and L == int(g["read_len"]) and t == int(g["t"])
    assert sha(raw) == str(g["sha_input"]), "the generator gave other reads on this host"
    fa = str(tmp_path / "reads.fa")
    synth.write_fasta(fa, raw)
    rc, err, kept, _ = import_fasta(int(g["width"]), fa, L)
    assert rc == 0, err
    assert kept.shape[0] == int(g["num_reads"]) and sha(kept) == str(g["sha_reads"])
    return kept, fa


def graph_digests_ok(out, g, what):
    """Assert that an overlap-search result (per-read counts and CSR edges) has the reference's
    digests: edge counts, ordered edge fields, path trans and node fields."""
    from pasqual_gb300 import graph
    dt = idx_dtype(g["width"])
    assert len(out.dest) == int(g["num_edges"]), what
    assert sha(out.num_B) == str(g["sha_num_B"]), what
    assert sha(out.num_F) == str(g["sha_num_F"]), what
    assert sha(out.dest.astype(dt)) == str(g["sha_dest"]), what
    assert sha(out.length) == str(g["sha_length"]), what
    assert sha(out.etype) == str(g["sha_etype"]), what
    assert sha(graph.trans_with_mask(out.num_B, out.num_F, out.edge_off, out.trans)) == \
        str(g["sha_trans"]), what
    assert sha(graph.node_fields(out.num_B, out.num_F, out.olp_B, out.olp_F)) == \
        str(g["sha_node_types"]), what
