"""pasqual_gb300 — GB300 (sm_103a) build of PASQUAL's hot path behind a C ABI.

The product is the CUDA library ``pasqual_gb300/_build/libpasqual_gb300_u{32,64}.so`` (C ABI
declared in ``include/pasqual_gb300.h``).  This module is a thin ctypes host mirror of the
reference's two entry points on the path:

* :meth:`Pasqual.construct_index`        ~ ``construct_index`` (src/index.h:63-68) without the
  FASTA import: reads in, both FM-indexes built on the GPU;
* :meth:`Pasqual.construct_string_graph` ~ ``construct_string_graph`` (src/string_graph.h:139):
  per-read irreducible edges in the reference's node order.

There is no CPU fallback: if the CUDA library is missing or no GPU is present, these calls raise.
"""
from __future__ import annotations

import ctypes as ct
import os
import weakref
from dataclasses import dataclass

import numpy as np

from . import build as _build

__all__ = ["Pasqual", "Graph", "PQError", "load_library", "library_path", "EXPORTS", "mlp_forward",
           "mlp_backward", "mlp_adam_step", "LearnedInfo", "overlaps_batched", "autotune_batched",
           "host_empty"]

PQ_ERRORS = {1: "PQ_ERR_ARG", 2: "PQ_ERR_CUDA", 3: "PQ_ERR_NOMEM", 4: "PQ_ERR_TOO_MANY_EDGES",
             5: "PQ_ERR_STATE", 6: "PQ_ERR_CAPACITY", 7: "PQ_ERR_INTERNAL"}

# Every entry point of include/pasqual_gb300.h (checked against the header by the tests).
EXPORTS = ["pq_idx_bytes", "pq_create", "pq_destroy", "pq_last_error", "pq_set_reads",
           "pq_get_counts", "pq_sort", "pq_set_sa", "pq_get_sa", "pq_build_fm", "pq_build_index",
           "pq_get_index_ref", "pq_get_seeds", "pq_set_seed_k", "pq_set_seed_mode", "pq_overlaps",
           "pq_get_graph_sizes", "pq_get_graph", "pq_get_stage_ms", "pq_get_kernel_stats",
           "pq_suffix_sort_static", "pq_learned_build", "pq_learned_get_info", "pq_learned_export",
           "pq_learned_predict", "pq_learned_keys", "pq_mlp_forward", "pq_mlp_backward",
           "pq_overlaps_batched", "pq_set_batch_plan", "pq_get_batch_stats", "pq_autotune_batched",
           "pq_set_sort_chunk", "pq_get_search_traffic", "pq_get_sort_seeds", "pq_mlp_adam_step",
           "pq_get_tier_stats", "pq_host_alloc", "pq_host_free"]


# The reference's own entry points served by the same library (include/pasqual_gb300_dropin.h).
DROPIN_EXPORTS = ["construct_index", "construct_string_graph", "destroy_graph", "pq_import_fasta",
                  "pq_string_graph_from_csr", "transform_to_triplet", "transform_to_triplet_reverse",
                  "initial_sort", "suf_sort"]


class PQError(RuntimeError):
    def __init__(self, code: int, msg: str):
        super().__init__("%s: %s" % (PQ_ERRORS.get(code, "PQ_ERR_%d" % code), msg))
        self.code = code


def library_path(width: int = 32) -> str:
    return _build.lib_path(width)


_LIBS: dict = {}


def load_library(width: int = 32) -> ct.CDLL:
    """Load the CUDA library of one index width; raise if it was not built."""
    if width in _LIBS:
        return _LIBS[width]
    path = library_path(width)
    if not os.path.exists(path):
        raise RuntimeError("pasqual_gb300 CUDA library not built: %s (run "
                           "`python -c 'import __graft_entry__ as g; g.build()'`)" % path)
    lib = ct.CDLL(path)
    I = ct.c_uint64 if width == 64 else ct.c_uint32
    vp, c_int = ct.c_void_p, ct.c_int
    sig = {
        "pq_idx_bytes": (c_int, []),
        "pq_create": (c_int, [ct.POINTER(vp), c_int, vp]),
        "pq_destroy": (None, [vp]),
        "pq_last_error": (ct.c_char_p, [vp]),
        "pq_set_reads": (c_int, [vp, vp, I, c_int, c_int, c_int]),
        "pq_get_counts": (c_int, [vp, vp, vp, vp]),
        "pq_sort": (c_int, [vp, c_int]),
        "pq_set_sa": (c_int, [vp, c_int, vp, c_int]),
        "pq_get_sa": (c_int, [vp, c_int, vp]),
        "pq_build_fm": (c_int, [vp, c_int]),
        "pq_build_index": (c_int, [vp]),
        "pq_get_index_ref": (c_int, [vp, c_int, vp, vp, vp]),
        "pq_get_seeds": (c_int, [vp, c_int, vp, vp, vp]),
        "pq_set_seed_k": (c_int, [vp, c_int]),
        "pq_set_seed_mode": (c_int, [vp, c_int]),
        "pq_overlaps": (c_int, [vp]),
        "pq_get_graph_sizes": (c_int, [vp, vp, vp, vp]),
        "pq_get_graph": (c_int, [vp] + [vp] * 9),
        "pq_get_stage_ms": (c_int, [vp, vp, vp, vp]),
        "pq_get_kernel_stats": (c_int, [vp, vp, vp]),
        "pq_learned_build": (c_int, [vp, c_int, c_int]),
        "pq_learned_get_info": (c_int, [vp, c_int, vp]),
        "pq_learned_export": (c_int, [vp, c_int, vp, vp, vp, vp, vp]),
        "pq_learned_predict": (c_int, [vp, c_int, vp, ct.c_uint64, vp, vp]),
        "pq_learned_keys": (c_int, [vp, c_int, vp, vp, ct.c_uint64, vp]),
        "pq_mlp_forward": (c_int, [vp, vp, c_int, vp]),
        "pq_mlp_backward": (c_int, [vp, vp, vp, c_int, vp]),
        "pq_overlaps_batched": (c_int, [vp, c_int, c_int]),
        "pq_set_batch_plan": (c_int, [vp, c_int, c_int, c_int]),
        "pq_get_batch_stats": (c_int, [vp, vp, vp, vp, vp, vp]),
        "pq_autotune_batched": (c_int, [vp, c_int, c_int, vp]),
        "pq_set_sort_chunk": (c_int, [vp, ct.c_uint64]),
        "pq_get_search_traffic": (c_int, [vp, vp, vp]),
        "pq_get_sort_seeds": (c_int, [vp, c_int, vp, vp, vp]),
        "pq_mlp_adam_step": (c_int, [vp, vp, vp, vp, vp, c_int, c_int, ct.c_float]),
        "pq_get_tier_stats": (c_int, [vp, vp, vp]),
        "pq_host_alloc": (c_int, [ct.c_size_t, ct.POINTER(vp)]),
        "pq_host_free": (c_int, [vp]),
    }
    for name, (res, args) in sig.items():
        f = getattr(lib, name)
        f.restype = res
        f.argtypes = args
    if lib.pq_idx_bytes() * 8 != width:
        raise RuntimeError("library %s has the wrong index width" % path)
    _LIBS[width] = lib
    return lib


class LearnedInfo(ct.Structure):
    """pq_learned_info of include/pasqual_gb300.h."""
    _fields_ = [("num_keys", ct.c_uint64), ("segments", ct.c_int32), ("hidden", ct.c_int32),
                ("steps", ct.c_int32), ("keys_ms", ct.c_float), ("train_ms", ct.c_float),
                ("eval_ms", ct.c_float), ("mean_window", ct.c_double), ("mean_window_root", ct.c_double),
                ("max_window", ct.c_int64), ("max_window_root", ct.c_int64), ("queries", ct.c_uint64),
                ("misses", ct.c_uint64)]

    def as_dict(self) -> dict:
        return {k: getattr(self, k) for k, _ in self._fields_}


LX_STRIDE = 196      # floats per segment record: w1[64] b1[64] w2[64] b2, padded
LX_HIDDEN = 64


def mlp_forward(params: np.ndarray, x: np.ndarray, width: int = 32) -> np.ndarray:
    """The learned index's per-segment network on the GPU: y = mlp(x) (params: one record)."""
    lib = load_library(width)
    params = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    y = np.empty_like(x)
    rc = lib.pq_mlp_forward(_p(params), _p(x), len(x), _p(y))
    if rc != 0:
        raise PQError(rc, "pq_mlp_forward")
    return y


def mlp_backward(params: np.ndarray, x: np.ndarray, dy: np.ndarray, width: int = 32) -> np.ndarray:
    """Gradient of sum(dy * mlp(x)) with respect to (w1, b1, w2, b2), 193 values, on the GPU."""
    lib = load_library(width)
    params = np.ascontiguousarray(params, np.float32)
    x = np.ascontiguousarray(x, np.float32)
    dy = np.ascontiguousarray(dy, np.float32)
    g = np.empty(3 * LX_HIDDEN + 1, np.float32)
    rc = lib.pq_mlp_backward(_p(params), _p(x), _p(dy), len(x), _p(g))
    if rc != 0:
        raise PQError(rc, "pq_mlp_backward")
    return g


def mlp_adam_step(params: np.ndarray, m1: np.ndarray, m2: np.ndarray, x: np.ndarray, target: np.ndarray,
                  step: int, lr: float, width: int = 32):
    """One joint-phase training step of one network on the GPU; returns (params, m1, m2) updated."""
    lib = load_library(width)
    p = np.ascontiguousarray(params, np.float32).copy()
    a = np.ascontiguousarray(m1, np.float32).copy()
    b = np.ascontiguousarray(m2, np.float32).copy()
    x = np.ascontiguousarray(x, np.float32)
    t = np.ascontiguousarray(target, np.float32)
    rc = lib.pq_mlp_adam_step(_p(p), _p(a), _p(b), _p(x), _p(t), len(x), int(step), float(lr))
    if rc != 0:
        raise PQError(rc, "pq_mlp_adam_step")
    return p, a, b


def host_empty(shape, dtype=np.uint8, width: int = 32) -> np.ndarray:
    """A host array in page-locked memory (pq_host_alloc), for the buffers that cross to the device
    and back: pq_set_reads and pq_get_graph copy such buffers with a kernel that keeps the link's
    rate after a sort or search.  Released when the array and every view of it are gone."""
    lib = load_library(width)
    dt = np.dtype(dtype)
    count = int(np.prod(shape, dtype=np.int64))
    nbytes = max(count * dt.itemsize, 1)
    ptr = ct.c_void_p()
    rc = lib.pq_host_alloc(nbytes, ct.byref(ptr))
    if rc != 0:
        raise PQError(rc, "pq_host_alloc(%d bytes)" % nbytes)
    buf = (ct.c_uint8 * nbytes).from_address(ptr.value)
    weakref.finalize(buf, lib.pq_host_free, ptr.value)
    return np.frombuffer(buf, dtype=dt, count=count).reshape(shape)


BATCH_GRAPH = 1


def _handles(ctxs):
    if not ctxs:
        raise ValueError("empty batch")
    w = ctxs[0].width
    if any(c.width != w for c in ctxs):
        raise ValueError("all contexts of a batch must have the same index width")
    arr = (ct.c_void_p * len(ctxs))(*[c.h for c in ctxs])
    return ctxs[0], arr


def overlaps_batched(ctxs, graph: bool = False) -> None:
    """One persistent search over the read sets of several contexts (each with its own L and t)."""
    lead, arr = _handles(ctxs)
    lead._ck(lead.lib.pq_overlaps_batched(arr, len(ctxs), BATCH_GRAPH if graph else 0), "pq_overlaps_batched")


def autotune_batched(ctxs, graph: bool = False) -> float:
    """Time every launch plan on this batch set, keep the fastest; returns its kernel ms."""
    lead, arr = _handles(ctxs)
    ms = ct.c_float()
    lead._ck(lead.lib.pq_autotune_batched(arr, len(ctxs), BATCH_GRAPH if graph else 0, ct.byref(ms)),
             "pq_autotune_batched")
    return ms.value


@dataclass
class Graph:
    """Overlap-search output: per read (num_B, num_F, olp_B, olp_F, edge_off) and per edge
    (dest, length, etype, trans), B edges then F edges of each read, reference DFS order."""
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
    wide_reads: int = 0


def _p(a: np.ndarray) -> ct.c_void_p:
    return a.ctypes.data_as(ct.c_void_p)


class Pasqual:
    """One GPU context holding both FM-indexes of a read set (index width 32 or 64)."""

    def __init__(self, width: int = 32, device: int = 0, stream: int | None = None):
        self.width = width
        self.lib = load_library(width)
        self.dt = np.uint64 if width == 64 else np.uint32
        h = ct.c_void_p()
        rc = self.lib.pq_create(ct.byref(h), device, ct.c_void_p(stream) if stream else None)
        if rc != 0:
            raise PQError(rc, "pq_create failed (no CUDA device?)")
        self.h = h
        self.num_reads = 0
        self.read_len = 0

    def close(self) -> None:
        if getattr(self, "h", None):
            self.lib.pq_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def _ck(self, rc: int, what: str) -> None:
        if rc != 0:
            msg = self.lib.pq_last_error(self.h)
            raise PQError(rc, "%s: %s" % (what, msg.decode() if msg else ""))

    # -- construct_index -------------------------------------------------------------------
    def set_reads(self, reads: np.ndarray, min_overlap: int) -> None:
        reads = np.ascontiguousarray(reads, dtype=np.uint8)
        nr, L = reads.shape
        self._ck(self.lib.pq_set_reads(self.h, _p(reads), nr, L, int(min_overlap), 0),
                 "pq_set_reads")
        self.num_reads, self.read_len = nr, L

    def set_seed_k(self, k: int) -> None:
        self._ck(self.lib.pq_set_seed_k(self.h, int(k)), "pq_set_seed_k")

    def set_seed_mode(self, mode: int) -> None:
        """0: walk from the k-mer seed; 1: depth-t interval scan (default); 2: the scan with
        learned-index windows."""
        self._ck(self.lib.pq_set_seed_mode(self.h, int(mode)), "pq_set_seed_mode")

    def set_sort_chunk(self, max_suffixes: int) -> None:
        """Sort in chunks of at most this many suffixes (0: one pass up to 2^31 - 1)."""
        self._ck(self.lib.pq_set_sort_chunk(self.h, int(max_suffixes)), "pq_set_sort_chunk")

    def sort(self, direction: int) -> None:
        self._ck(self.lib.pq_sort(self.h, direction), "pq_sort")

    def set_sa(self, direction: int, sa: np.ndarray) -> None:
        sa = np.ascontiguousarray(sa, dtype=self.dt)
        self._ck(self.lib.pq_set_sa(self.h, direction, _p(sa), 0), "pq_set_sa")

    def get_sa(self, direction: int) -> np.ndarray:
        sa = np.empty(self.num_reads * self.read_len, self.dt)
        self._ck(self.lib.pq_get_sa(self.h, direction, _p(sa)), "pq_get_sa")
        return sa

    def build_fm(self, direction: int) -> None:
        self._ck(self.lib.pq_build_fm(self.h, direction), "pq_build_fm")

    def build_index(self) -> None:
        self._ck(self.lib.pq_build_index(self.h), "pq_build_index")

    def construct_index(self, reads: np.ndarray, min_overlap: int) -> None:
        """Reads (codes 1..4, [num_reads, read_len]) -> both FM-indexes on the GPU."""
        self.set_reads(reads, min_overlap)
        self.build_index()

    def counts(self):
        C = np.zeros(6, self.dt)
        s = np.zeros(4, self.dt)
        p = np.zeros(4, self.dt)
        self._ck(self.lib.pq_get_counts(self.h, _p(C), _p(s), _p(p)), "pq_get_counts")
        return C, s, p

    def index_ref(self, direction: int):
        """Reference-layout (OCC_bitmap[5] concatenated, OCC_sample, reads_index)."""
        n = self.num_reads * self.read_len
        rowlen = n // 64 + 1
        bm = np.empty(5 * rowlen, np.uint64)
        smp = np.empty(5 * rowlen, self.dt)
        ri = np.empty(max(self.num_reads, 1), self.dt)
        self._ck(self.lib.pq_get_index_ref(self.h, direction, _p(bm), _p(smp), _p(ri)),
                 "pq_get_index_ref")
        return bm, smp, ri[:self.num_reads]

    def seeds(self, direction: int):
        nr = max(self.num_reads, 1)
        s = np.empty(nr, self.dt)
        z = np.empty(nr, self.dt)
        d = np.empty(nr, np.uint16)
        self._ck(self.lib.pq_get_seeds(self.h, direction, _p(s), _p(z), _p(d)), "pq_get_seeds")
        return s[:self.num_reads], z[:self.num_reads], d[:self.num_reads]

    def sort_seeds(self, direction: int):
        """The seed intervals the reference's sort records: (start, size, depth) per read."""
        nr = max(self.num_reads, 1)
        s = np.empty(nr, self.dt)
        z = np.empty(nr, self.dt)
        d = np.empty(nr, np.uint16)
        self._ck(self.lib.pq_get_sort_seeds(self.h, direction, _p(s), _p(z), _p(d)), "pq_get_sort_seeds")
        return s[:self.num_reads], z[:self.num_reads], d[:self.num_reads]

    # -- construct_string_graph ------------------------------------------------------------
    def overlaps(self) -> None:
        self._ck(self.lib.pq_overlaps(self.h), "pq_overlaps")

    def graph(self, out: Graph | None = None) -> Graph:
        """The last overlap search's graph.  With `out` (an earlier result, or any Graph whose
        arrays are at least as long), the arrays are filled in place and views of the right
        lengths are returned: host buffers that are reused skip the page faults of fresh ones."""
        ne = ct.c_uint64()
        pr = ct.c_uint64()
        wr = ct.c_uint64()
        self._ck(self.lib.pq_get_graph_sizes(self.h, ct.byref(ne), ct.byref(pr), ct.byref(wr)),
                 "pq_get_graph_sizes")
        nr, m = self.num_reads, ne.value
        want = {"num_B": (nr, np.uint16), "num_F": (nr, np.uint16), "olp_B": (nr, np.int32),
                "olp_F": (nr, np.int32), "edge_off": (nr + 1, np.uint64), "dest": (m, self.dt),
                "length": (m, np.uint16), "etype": (m, np.uint8), "trans": (m, np.int32)}
        arrays = {}
        for name, (size, dt) in want.items():
            a = getattr(out, name, None) if out is not None else None
            if (a is None or a.dtype != np.dtype(dt) or a.ndim != 1 or len(a) < size
                    or not a.flags.c_contiguous or not a.flags.writeable):
                a = np.empty(size, dt)
            arrays[name] = a[:size]
        g = Graph(**arrays, probes=pr.value, wide_reads=wr.value)
        self._ck(self.lib.pq_get_graph(self.h, _p(g.num_B), _p(g.num_F), _p(g.olp_B), _p(g.olp_F),
                                       _p(g.edge_off), _p(g.dest), _p(g.length), _p(g.etype),
                                       _p(g.trans)), "pq_get_graph")
        return g

    def construct_string_graph(self) -> Graph:
        self.overlaps()
        return self.graph()

    def tier_stats(self) -> dict:
        """Reads the last overlap search handed from tier to tier, and each tier's time."""
        n = (ct.c_uint64 * 4)()
        ms = (ct.c_float * 4)()
        self._ck(self.lib.pq_get_tier_stats(self.h, n, ms), "pq_get_tier_stats")
        return {"deferred": n[0], "block": n[1], "heavy": n[2], "wide": n[3], "lean_fast_ms": ms[0],
                "block_ms": ms[1], "heavy_ms": ms[2], "wide_ms": ms[3]}

    def search_traffic(self):
        """(32-byte sectors of index data the last overlap search loaded, bytes of results it
        wrote): the search's algorithmic traffic is 32 * sectors + bytes."""
        sec, out = ct.c_uint64(), ct.c_uint64()
        self._ck(self.lib.pq_get_search_traffic(self.h, ct.byref(sec), ct.byref(out)),
                 "pq_get_search_traffic")
        return sec.value, out.value

    def kernel_stats(self):
        """(fast search kernel ms of the last overlap search, kernels launched so far)."""
        ms, n = ct.c_float(), ct.c_ulonglong()
        self._ck(self.lib.pq_get_kernel_stats(self.h, ct.byref(ms), ct.byref(n)),
                 "pq_get_kernel_stats")
        return ms.value, n.value

    # -- learned index -----------------------------------------------------------------------
    def learned_build(self, direction: int, steps: int = 400) -> None:
        self._ck(self.lib.pq_learned_build(self.h, direction, int(steps)), "pq_learned_build")

    def learned_info(self, direction: int) -> dict:
        info = LearnedInfo()
        self._ck(self.lib.pq_learned_get_info(self.h, direction, ct.byref(info)), "pq_learned_get_info")
        return info.as_dict()

    def learned_export(self, direction: int) -> dict:
        S = self.learned_info(direction)["segments"]
        out = {"bnd": np.empty(S, np.uint32), "base": np.empty(S + 1, self.dt),
               "params": np.empty((S, LX_STRIDE), np.float32), "err": np.empty((S, 2), np.int32),
               "err_root": np.empty((S, 2), np.int32)}
        self._ck(self.lib.pq_learned_export(self.h, direction, _p(out["bnd"]), _p(out["base"]),
                                            _p(out["params"]), _p(out["err"]), _p(out["err_root"])),
                 "pq_learned_export")
        return out

    def learned_predict(self, direction: int, keys: np.ndarray):
        keys = np.ascontiguousarray(keys, np.uint32)
        pred = np.empty(len(keys), np.int64)
        seg = np.empty(len(keys), np.int32)
        self._ck(self.lib.pq_learned_predict(self.h, direction, _p(keys), len(keys), _p(pred), _p(seg)),
                 "pq_learned_predict")
        return pred, seg

    def learned_keys(self, direction: int):
        """Distinct 16-base keys of the suffix array and the first row of each."""
        n = self.num_reads * self.read_len
        keys = np.empty(max(n, 1), np.uint32)
        first = np.empty(max(n, 1), self.dt)
        m = ct.c_uint64()
        self._ck(self.lib.pq_learned_keys(self.h, direction, _p(keys), _p(first), n, ct.byref(m)),
                 "pq_learned_keys")
        return keys[:m.value], first[:m.value]

    def set_batch_plan(self, ctas_per_sm: int = 0, groups_per_item: int = 1, edge_slots: int = 64) -> None:
        self._ck(self.lib.pq_set_batch_plan(self.h, ctas_per_sm, groups_per_item, edge_slots), "pq_set_batch_plan")

    def batch_stats(self) -> dict:
        ms, c, g, e, gr = ct.c_float(), ct.c_int(), ct.c_int(), ct.c_int(), ct.c_int()
        self._ck(self.lib.pq_get_batch_stats(self.h, ct.byref(ms), ct.byref(c), ct.byref(g), ct.byref(e),
                                             ct.byref(gr)), "pq_get_batch_stats")
        return {"kernel_ms": ms.value, "ctas_per_sm": c.value, "groups_per_item": g.value,
                "edge_slots": e.value, "graph_used": gr.value}

    def stage_ms(self):
        a, b, c = ct.c_float(), ct.c_float(), ct.c_float()
        self._ck(self.lib.pq_get_stage_ms(self.h, ct.byref(a), ct.byref(b), ct.byref(c)),
                 "pq_get_stage_ms")
        return a.value, b.value, c.value
