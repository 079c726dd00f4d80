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
