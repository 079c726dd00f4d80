"""ctypes wrapper of the C restatement (oracle/pq_oracle.c) and of the reference dump tool.

TEST INFRASTRUCTURE: imported only by tests/, by ``__graft_entry__.smoke()`` and by the CPU
baseline leg of ``bench.py``, always as the oracle the GPU results are compared with or as the
timed CPU baseline, never as the product path.
"""
from __future__ import annotations

import ctypes as ct
import os
import subprocess
from dataclasses import dataclass

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
REF = os.path.join(HERE, "_ref")

# The reference checkout the recipes read (never written).  PASQUAL_REFERENCE overrides it; this
# is the one place that names the default.
REFERENCE = os.environ.get("PASQUAL_REFERENCE", "/root/reference")
REFERENCE_SRC = os.path.join(REFERENCE, "src")


def reference_buildable() -> bool:
    """The reference's sources are present and this host can compile them (x86: SSE4.2)."""
    return os.path.isdir(REFERENCE_SRC) and os.uname().machine == "x86_64"


def build(ref: bool = False) -> None:
    """Compile the restatement (and, when asked and available, the reference)."""
    subprocess.run(["make", "-s", "-C", HERE, "port"], check=True)
    if ref:
        subprocess.run(["make", "-s", "-C", HERE, "ref", "stage", "REF=" + REFERENCE], check=True)


def np_idx(width: int):
    return np.uint64 if width == 64 else np.uint32


class _Index(ct.Structure):
    pass


class _Graph(ct.Structure):
    pass


def _declare(width: int):
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    P = ct.POINTER
    _Index_w = type("_Index%d" % width, (ct.Structure,), {"_fields_": [
        ("reads", ct.c_void_p), ("num_reads", I), ("read_len", ct.c_int),
        ("min_overlap", ct.c_int), ("C", I * 6),
        ("bitmap", ct.c_void_p * 2), ("sample", ct.c_void_p * 2),
        ("reads_index", ct.c_void_p * 2), ("seed_start", ct.c_void_p * 2),
        ("seed_size", ct.c_void_p * 2), ("seed_depth", ct.c_void_p * 2)]})
    _Graph_w = type("_Graph%d" % width, (ct.Structure,), {"_fields_": [
        ("first", I), ("count", I), ("num_B", P(ct.c_uint16)), ("num_F", P(ct.c_uint16)),
        ("olp_B", P(ct.c_int32)), ("olp_F", P(ct.c_int32)), ("edge_off", P(ct.c_uint64)),
        ("edge_dest", P(I)), ("edge_len", P(ct.c_uint16)), ("edge_type", P(ct.c_uint8)),
        ("edge_trans", P(ct.c_int32)), ("num_edges", ct.c_uint64), ("probes", ct.c_uint64),
        ("status", ct.c_int), ("failed_read", I)]})
    return I, _Index_w, _Graph_w


@dataclass
class Graph:
    """Per-read overlap-search output in the reference's node order (B edges, then F)."""
    num_B: np.ndarray
    num_F: np.ndarray
    olp_B: np.ndarray
    olp_F: np.ndarray
    edge_off: np.ndarray
    dest: np.ndarray
    length: np.ndarray
    etype: np.ndarray
    trans: np.ndarray
    probes: int = 0


class Port:
    """The C restatement for one index width (32 or 64)."""

    def __init__(self, width: int = 32):
        self.width = width
        path = os.path.join(BUILD, "libpq_oracle_u%d.so" % width)
        if not os.path.exists(path):
            build()
        self.lib = ct.CDLL(path)
        self.I, self.Index, self.GraphS = _declare(width)
        self.dt = np_idx(width)
        L = self.lib
        vp = ct.c_void_p
        L.pqo_idx_bytes.restype = ct.c_int
        assert L.pqo_idx_bytes() * 8 == width
        L.pqo_counts.argtypes = [vp, self.I, ct.c_int, vp, vp, vp]
        L.pqo_sort.argtypes = [vp, self.I, ct.c_int, ct.c_int, vp, ct.c_int]
        L.pqo_build_occ.argtypes = [vp, self.I, ct.c_int, ct.c_int, vp, vp, vp, vp, vp]
        L.pqo_kmer_table.argtypes = [vp, self.I, ct.c_int, ct.c_int, vp, ct.c_int, vp, vp]
        L.pqo_seeds_from_kmers.argtypes = [vp, self.I, ct.c_int, ct.c_int, vp, vp, ct.c_int,
                                           vp, vp, vp]
        L.pqo_overlaps.argtypes = [ct.POINTER(self.Index), self.I, self.I, ct.c_int,
                                   ct.POINTER(self.GraphS)]
        L.pqo_graph_free.argtypes = [ct.POINTER(self.GraphS)]

    @staticmethod
    def _p(a: np.ndarray):
        return a.ctypes.data_as(ct.c_void_p)

    def counts(self, reads: np.ndarray):
        nr, L = reads.shape
        C = np.zeros(6, self.dt)
        sfx = np.zeros(4, self.dt)
        pfx = np.zeros(4, self.dt)
        self.lib.pqo_counts(self._p(reads), nr, L, self._p(C), self._p(sfx), self._p(pfx))
        return C, sfx, pfx

    def sort(self, reads: np.ndarray, direction: int, threads: int = 0) -> np.ndarray:
        nr, L = reads.shape
        sa = np.empty(nr * L, self.dt)
        rc = self.lib.pqo_sort(self._p(reads), nr, L, direction, self._p(sa), threads)
        assert rc == 0, rc
        return sa

    def build_occ(self, reads: np.ndarray, direction: int, sa: np.ndarray, fix: np.ndarray):
        nr, L = reads.shape
        n = nr * L
        rowlen = n // 64 + 1
        bm = np.empty(5 * rowlen, np.uint64)
        sample = np.empty(5 * rowlen, self.dt)
        ri = np.empty(max(nr, 1), self.dt)
        rc = self.lib.pqo_build_occ(self._p(reads), nr, L, direction, self._p(sa),
                                    self._p(np.ascontiguousarray(fix, self.dt)),
                                    self._p(bm), self._p(sample), self._p(ri))
        assert rc == 0, rc
        return bm, sample, ri[:nr]

    def kmer_table(self, reads, direction, sa, k):
        nr, L = reads.shape
        start = np.empty(4 ** k, self.dt)
        size = np.empty(4 ** k, self.dt)
        rc = self.lib.pqo_kmer_table(self._p(reads), nr, L, direction, self._p(sa), k,
                                     self._p(start), self._p(size))
        assert rc == 0, rc
        return start, size

    def seeds_from_kmers(self, reads, k, kstart, ksize, direction):
        nr, L = reads.shape
        s = np.empty(max(nr, 1), self.dt)
        z = np.empty(max(nr, 1), self.dt)
        d = np.empty(max(nr, 1), np.uint16)
        rc = self.lib.pqo_seeds_from_kmers(self._p(reads), nr, L, k, self._p(kstart),
                                           self._p(ksize), direction, self._p(s), self._p(z),
                                           self._p(d))
        assert rc == 0, rc
        return s[:nr], z[:nr], d[:nr]

    def build_index(self, reads: np.ndarray, t: int, threads: int = 0, seed_k: int = 0):
        """Full CPU index: counts, both suffix arrays, occ tables, optional k-mer seeds."""
        reads = np.ascontiguousarray(reads, np.uint8)
        C, sfx, pfx = self.counts(reads)
        ix = {"reads": reads, "t": t, "C": C, "suffix_count": sfx, "prefix_count": pfx}
        for d, fix in ((0, sfx), (1, pfx)):
            sa = self.sort(reads, d, threads)
            bm, sample, ri = self.build_occ(reads, d, sa, fix)
            ix["sa%d" % d] = sa
            ix["bitmap%d" % d] = bm
            ix["sample%d" % d] = sample
            ix["reads_index%d" % d] = ri
            if seed_k:
                ks, kz = self.kmer_table(reads, d, sa, seed_k)
                ix["seed%d" % d] = self.seeds_from_kmers(reads, seed_k, ks, kz, d)
        return ix

    def overlaps(self, ix: dict, first: int = 0, count: int | None = None, threads: int = 0,
                 seeds=None) -> Graph:
        """Overlap search.  ``seeds`` = ((start, size, depth) fw, (start, size, depth) bw) or
        None to start every F-B / B-F search at depth 1."""
        reads = ix["reads"]
        nr, L = reads.shape
        if count is None:
            count = nr - first
        keep = []

        def ptr(a):
            a = np.ascontiguousarray(a)
            keep.append(a)
            return self._p(a)

        s = self.Index()
        s.reads = ptr(reads)
        s.num_reads = nr
        s.read_len = L
        s.min_overlap = int(ix["t"])
        for c in range(6):
            s.C[c] = int(ix["C"][c])
        for d in range(2):
            s.bitmap[d] = ptr(ix["bitmap%d" % d])
            s.sample[d] = ptr(ix["sample%d" % d].astype(self.dt, copy=False))
            s.reads_index[d] = ptr(ix["reads_index%d" % d].astype(self.dt, copy=False))
            if seeds is not None:
                st, sz, dp = seeds[d]
                s.seed_start[d] = ptr(st.astype(self.dt, copy=False))
                s.seed_size[d] = ptr(sz.astype(self.dt, copy=False))
                s.seed_depth[d] = ptr(dp.astype(np.uint16, copy=False))
        g = self.GraphS()
        rc = self.lib.pqo_overlaps(ct.byref(s), first, count, threads, ct.byref(g))
        try:
            if rc != 0:
                raise RuntimeError("pqo_overlaps failed: status %d at read %d"
                                   % (rc, g.failed_read))
            ne = int(g.num_edges)

            def arr(p, n, dt):
                return np.ctypeslib.as_array(p, shape=(n,)).astype(dt, copy=True) if n else \
                    np.zeros(0, dt)
            return Graph(num_B=arr(g.num_B, count, np.uint16),
                         num_F=arr(g.num_F, count, np.uint16),
                         olp_B=arr(g.olp_B, count, np.int32), olp_F=arr(g.olp_F, count, np.int32),
                         edge_off=arr(g.edge_off, count + 1, np.uint64),
                         dest=arr(g.edge_dest, ne, self.dt), length=arr(g.edge_len, ne, np.uint16),
                         etype=arr(g.edge_type, ne, np.uint8),
                         trans=arr(g.edge_trans, ne, np.int32), probes=int(g.probes))
        finally:
            self.lib.pqo_graph_free(ct.byref(g))


# ------------------------------------------------------------------------- reference dumps

def ref_available() -> bool:
    return os.path.exists(os.path.join(REF, "ref_dump_u32"))


def run_ref_dump(fasta: str, L: int, t: int, outdir: str, width: int = 32, threads: int = 4,
                 bloom_m: int = 36, n_hashfunc: int = 2):
    """Run the unmodified reference (oracle/_ref/ref_dump_uXX) on a FASTA; return its dump."""
    exe = os.path.join(REF, "ref_dump_u%d" % width)
    subprocess.run([exe, fasta, str(L), str(t), outdir, str(threads), str(bloom_m), str(n_hashfunc)],
                   check=True, stdout=subprocess.DEVNULL)
    return load_dump(outdir)


def load_dump(outdir: str) -> dict:
    meta = {}
    with open(os.path.join(outdir, "meta.txt")) as f:
        for line in f:
            k, *v = line.split()
            meta[k] = [int(x) for x in v] if len(v) > 1 else int(v[0])
    dt = np.uint64 if meta["idx_bytes"] == 8 else np.uint32
    nr, L = meta["num_reads"], meta["read_len"]

    def rd(name, t):
        return np.fromfile(os.path.join(outdir, name), dtype=t)
    d = {"meta": meta, "t": meta["min_overlap"],
         "reads": rd("reads.bin", np.uint8).reshape(nr, L),
         "C": np.array(meta["C"], dt), "suffix_count": np.array(meta["suffix_count"], dt),
         "prefix_count": np.array(meta["prefix_count"], dt)}
    for d_, tag in ((0, "fw"), (1, "bw")):
        d["sa%d" % d_] = rd("sa_%s.bin" % tag, dt)
        d["bitmap%d" % d_] = rd("occ_bitmap_%s.bin" % tag, np.uint64)
        d["sample%d" % d_] = rd("occ_sample_%s.bin" % tag, dt)
        d["reads_index%d" % d_] = rd("reads_index_%s.bin" % tag, dt)
        d["seed%d" % d_] = (rd("seed_start_%s.bin" % tag, dt), rd("seed_size_%s.bin" % tag, dt),
                            rd("seed_depth_%s.bin" % tag, np.uint16))
    nodes = rd("nodes.bin", np.uint8).reshape(nr, 8)
    d["num_B"] = nodes[:, 0:2].copy().view(np.uint16).ravel()
    d["num_F"] = nodes[:, 2:4].copy().view(np.uint16).ravel()
    d["node_types"] = nodes[:, 4:8].copy()
    d["dest"] = rd("edges_dest.bin", np.uint64)
    d["length"] = rd("edges_len.bin", np.uint16)
    d["etype"] = rd("edges_type.bin", np.uint8)
    d["trans"] = rd("edges_trans.bin", np.int64)
    return d
