"""Build the CUDA library in-tree: pasqual_gb300/_build/libpasqual_gb300_{u32,u64}.so.

Each index width (the reference's INDEX_LENGTH=U32/U64 split) is one shared library compiled
from the same sources, sm_103a only.  Translation units compile in parallel; a rebuild is skipped
when every object is newer than its sources.
"""
from __future__ import annotations

import os
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
ROOT = os.path.dirname(HERE)
SOURCES = ["pq_index.cu", "pq_search.cu", "pq_sort.cu", "pq_api.cu", "pq_dropin.cu",
           "pq_sort_static.cu", "pq_learned.cu", "pq_seeds.cu",
           "pq_sufsort.cu"]
HEADERS = ["pq_common.cuh", "pq_index.cuh", "pq_sort.cuh", "pq_learned.cuh", "pq_learned_build.cuh", "pq_slots.h"]
PUBLIC = ["pasqual_gb300.h", "pasqual_gb300_dropin.h"]
NVCC = os.environ.get("NVCC", "/usr/local/cuda/bin/nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-fvisibility=hidden"]


def lib_path(width: int) -> str:
    return os.path.join(OUT, "libpasqual_gb300_u%d.so" % width)


def _stale(target: str, deps) -> bool:
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(widths=(32, 64), verbose: bool = False) -> None:
    os.makedirs(OUT, exist_ok=True)
    hdrs = [os.path.join(CSRC, h) for h in HEADERS] + [os.path.join(ROOT, "include", h) for h in PUBLIC]
    jobs = []
    for w in widths:
        defs = ["-DPQ_IDX64"] if w == 64 else []
        for s in SOURCES:
            src = os.path.join(CSRC, s)
            obj = os.path.join(OUT, "%s.u%d.o" % (s[:-3], w))
            if _stale(obj, [src] + hdrs):
                jobs.append([NVCC] + ARCH + FLAGS + defs + ["-c", src, "-o", obj])

    def run(cmd):
        if verbose:
            print(" ".join(cmd), file=sys.stderr)
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n%s\n%s" % (" ".join(cmd), r.stderr))
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 4))) as ex:
        list(ex.map(run, jobs))
    for w in widths:
        objs = [os.path.join(OUT, "%s.u%d.o" % (s[:-3], w)) for s in SOURCES]
        lib = lib_path(w)
        if _stale(lib, objs):
            run([NVCC] + ARCH + ["-shared", "-o", lib] + objs + ["-lcudart"])


if __name__ == "__main__":
    build(verbose=True)
    print("built", [lib_path(w) for w in (32, 64)])
