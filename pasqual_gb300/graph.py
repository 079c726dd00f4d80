"""Node fields of the string graph from the per-read search output.

Restates the node construction of construct_string_graph (src/string_graph.c:832-889, 897-899)
on the CSR the CUDA search returns: node types from the edge counts, the SUSPECT mark from the
ratio of overlaps_B to overlaps_F, REMOVED for nodes without edges, and which nodes get a path
queue (their path_t.trans values are the per-edge ``trans`` the GPU returns).
"""
from __future__ import annotations

import numpy as np

# src/string_graph.h:20-40
ONE, BRANCH, ENDING = 1, 2, 4
DEFAULT, REMOVED = 0, 8
SUSPECT = 4


def node_fields(num_B: np.ndarray, num_F: np.ndarray, olp_B: np.ndarray, olp_F: np.ndarray) -> np.ndarray:
    """[num_reads, 4] uint8: B_type, F_type, status, marked (the reference's node_t fields)."""
    nB = num_B.astype(np.int64)
    nF = num_F.astype(np.int64)
    oB = olp_B.astype(np.int64)
    oF = olp_F.astype(np.int64)
    bt = np.where(nB == 1, ONE, np.where(nB > 1, BRANCH, ENDING))
    ft = np.where(nF == 1, ONE, np.where(nF > 1, BRANCH, ENDING))
    none = (nB == 0) & (nF == 0)
    bt = np.where(none, ENDING, bt)
    ft = np.where(none, ENDING, ft)
    status = np.where(none, REMOVED, DEFAULT)
    # ratio = |oB - oF| / max(oB, oF) in double, SUSPECT when > 0.6 (src/string_graph.c:843-854);
    # abs() is taken on the C int difference
    mx = np.maximum(oB, oF)
    diff = np.abs((oB - oF).astype(np.int32).astype(np.int64)).astype(np.float64)
    with np.errstate(divide="ignore", invalid="ignore"):
        ratio = np.where(mx == 0, 0.0, diff / np.where(mx == 0, 1, mx).astype(np.float64))
    marked = np.where(ratio > 0.6, SUSPECT, 0)
    return np.stack([bt, ft, status, marked], axis=1).astype(np.uint8)


def has_path_queue(num_B: np.ndarray, num_F: np.ndarray) -> np.ndarray:
    """Nodes for which the reference allocates path_q (src/string_graph.c:897-899)."""
    f = node_fields(num_B, num_F, np.zeros_like(num_B, dtype=np.int32),
                    np.zeros_like(num_B, dtype=np.int32))
    bt, ft = f[:, 0], f[:, 1]
    return ((bt == BRANCH) & (ft != ENDING)) | ((ft == BRANCH) & (bt != ENDING))


def trans_with_mask(num_B, num_F, edge_off, trans) -> np.ndarray:
    """Per-edge path trans as the reference exposes it: the value for nodes with a path queue,
    -1 elsewhere (int64)."""
    hp = has_path_queue(num_B, num_F)
    per_edge = np.repeat(hp, np.diff(edge_off.astype(np.int64)))
    return np.where(per_edge, trans.astype(np.int64), -1)
