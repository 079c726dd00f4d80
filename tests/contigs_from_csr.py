"""contigs.fa through this library's host side with no GPU: reads imported by pq_import_fasta, the
overlap graph's CSR from the oracle, node_t construction by pq_string_graph_from_csr, then the
reference's own assemble() (src/assemble.h:8-10, from the reference compiled by the oracle recipe)
writes ./contigs.fa into the working directory.  Run as a child process of the contigs test, with
OMP_NUM_THREADS=1 so that the reference's assemble stage runs in its deterministic order (the
oracle's own thread count is passed explicitly).

usage: python contigs_from_csr.py FASTA L T WIDTH
"""
import ctypes as ct
import os
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path[:0] = [ROOT, HERE]

import numpy as np  # noqa: E402

import pasqual_gb300 as pq  # noqa: E402
from oracle import port  # noqa: E402
from test_dropin_host import import_fasta  # noqa: E402
from test_node_build import call  # noqa: E402


def main(fasta, L, t, width):
    rc, err, reads, removed = import_fasta(width, fasta, L)
    assert rc == 0, err
    O = port.Port(width)
    cores = os.cpu_count() or 1       # the oracle's index and edges do not depend on its threads
    ix = O.build_index(reads, t, threads=cores)
    g = O.overlaps(ix, threads=cores)
    lib = pq.load_library(width)
    csr = (g.num_B, g.num_F, g.olp_B, g.olp_F, g.edge_off, g.dest, g.length, g.etype, g.trans)
    graph = call(lib, width, L, t, csr, 0)
    ref = ct.CDLL(os.path.join(ROOT, "oracle", "_ref", "libpasqual_ref_u%d.so" % width))
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    ref.assemble.restype = None
    ref.assemble.argtypes = [ct.c_void_p, ct.c_void_p, ct.POINTER(I), ct.POINTER(I)] + [ct.c_int] * 4
    num, total = I(), I()
    rd = np.ascontiguousarray(reads.reshape(-1))
    ref.assemble(ct.addressof(graph), rd.ctypes.data, ct.byref(num), ct.byref(total),
                 2 * L, 2 * L, 10, 2 * L // 5)        # the CLI's defaults (src/test.c:336-346)
    print("contigs %d total %d edges %d" % (num.value, total.value, len(g.dest)))


if __name__ == "__main__":
    main(sys.argv[1], int(sys.argv[2]), int(sys.argv[3]), int(sys.argv[4]))
