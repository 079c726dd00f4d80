"""The host halves of the library's sufsort.h entry points -- transform_to_triplet[_reverse] and
initial_sort (src/sufsort.c:80-151, 386-450) -- against the reference's own functions, compiled
from its sources by the oracle recipe (x86 only), on generated reads.  No GPU needed."""
import ctypes as ct
import os

import numpy as np
import pytest

from conftest import ROOT
import pasqual_gb300 as pq
from pasqual_gb300 import build, synth


@pytest.mark.parametrize("width,L", [(32, 50), (64, 100), (32, 13)])
def test_triplets_and_initial_sort_match_reference(width, L):
    from oracle import port
    from test_gpu_sufsort import Bucket32, Bucket64
    if not port.reference_buildable():
        pytest.skip("reference sources (x86) not present")
    build.build()
    port.build(ref=True)
    ref = ct.CDLL(os.path.join(ROOT, "oracle", "_ref", "libpasqual_ref_u%d.so" % width))
    mine = pq.load_library(width)
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    B = Bucket64 if width == 64 else Bucket32
    dt = np.uint64 if width == 64 else np.uint32
    for lib in (ref, mine):
        lib.transform_to_triplet.argtypes = [ct.c_void_p, ct.c_int, I]
        lib.transform_to_triplet_reverse.argtypes = [ct.c_void_p, ct.c_int, I]
        lib.initial_sort.argtypes = [ct.c_void_p, I, ct.POINTER(B), ct.c_void_p, ct.c_void_p, ct.c_void_p]
    reads = synth.reads_for_coverage(synth.genome(40000, 0.45, 0.1, (0.01, 0.01), 0.02, seed=L), L, 20,
                                     0.01, seed=L + 1)
    nr = reads.shape[0]
    for rev in (False, True):
        out = []
        for lib in (ref, mine):
            text = np.ascontiguousarray(reads.reshape(-1).copy())
            (lib.transform_to_triplet_reverse if rev else lib.transform_to_triplet)(text.ctypes.data, L, nr)
            bkt = B()
            bsize, boff, mx = np.zeros(5, dt), np.zeros(5, dt), np.zeros(1, dt)
            lib.initial_sort(text.ctypes.data, text.size, ct.byref(bkt), bsize.ctypes.data, boff.ctypes.data,
                             mx.ctypes.data)
            out.append((text, np.array(bkt.freqs), np.array(bkt.offs), bsize, boff, mx))
        for a, b in zip(*out):
            assert np.array_equal(a, b)
