"""The C-ABI library builds for sm_103a, loads, and exports every symbol its header declares.

No compute calls: this runs without a GPU.
"""
import ctypes as ct
import os
import re
import subprocess

import pytest

from conftest import ROOT
import pasqual_gb300 as pq
from pasqual_gb300 import build


HEADERS = ("pasqual_gb300.h", "pasqual_gb300_dropin.h")


def header_symbols():
    """Every function an include/*.h header declares with PQ_API."""
    out = set()
    for h in HEADERS:
        txt = open(os.path.join(ROOT, "include", h)).read()
        out |= set(re.findall(r"^PQ_API\s+[\w\s\*]+?\b(\w+)\s*\(", txt, flags=re.M))
    return out


@pytest.fixture(scope="module")
def libs():
    build.build()
    return {w: pq.load_library(w) for w in (32, 64)}


def test_header_lists_entry_points():
    syms = header_symbols()
    assert "pq_overlaps" in syms and "pq_sort" in syms and "pq_build_index" in syms
    assert {"construct_index", "construct_string_graph", "destroy_graph"} <= syms
    assert syms == set(pq.EXPORTS) | set(pq.DROPIN_EXPORTS)


@pytest.mark.parametrize("width", [32, 64])
def test_library_exports_header_symbols(libs, width):
    lib = libs[width]
    for s in header_symbols():
        assert hasattr(lib, s), s
    assert lib.pq_idx_bytes() == width // 8
    nm = subprocess.run(["nm", "-D", "--defined-only", pq.library_path(width)],
                        capture_output=True, text=True, check=True).stdout
    exported = set(re.findall(r"\b[TDB] (\w+)", nm))
    assert header_symbols() <= exported
    assert "time_importreads" in exported      # src/index.c:20, read by the reference's main()


def test_create_without_gpu_fails_loudly(libs):
    """No silent CPU fallback: without a usable GPU the context cannot be created."""
    import torch
    if torch.cuda.is_available():
        pytest.skip("a GPU is present")
    with pytest.raises(pq.PQError):
        pq.Pasqual(32)


@pytest.mark.parametrize("width", [32, 64])
def test_product_never_links_the_oracle(libs, width):
    """The library and its Python binding neither link, load nor import the oracle (the C
    restatement or the reference build): no CPU fallback can stand in for the CUDA path."""
    out = subprocess.run(["readelf", "-d", pq.library_path(width)], capture_output=True, text=True,
                         check=True).stdout
    needed = re.findall(r"\(NEEDED\)\s+Shared library: \[([^\]]+)\]", out)
    assert needed and not [n for n in needed if "oracle" in n or "pasqual_ref" in n], needed
    pkg = os.path.join(ROOT, "pasqual_gb300")
    for dirpath, _, files in os.walk(pkg):
        for fn in files:
            if fn.endswith((".py", ".cu", ".cuh", ".h", ".cpp")):
                txt = open(os.path.join(dirpath, fn)).read()
                assert not re.search(r"^\s*(from|import)\s+oracle\b", txt, flags=re.M), fn
                assert "pq_oracle" not in txt and "libpasqual_ref" not in txt, fn
