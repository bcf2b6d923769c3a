"""Block-size autotuner of the FP64 contraction engine.

The reference multiplies every block pair with one DGEMM call
(tensor_su2_dmrg_src.cpp:977-1006), whatever the block sizes.  Here the
blocks of one H_eff application or environment update run as tiles of one
launch, and the tile shape is a choice: 64 x 64 tiles waste most of the FP64
tensor pipe's work on blocks of a few tens of rows (the padding is computed),
smaller tiles cost more operand staging per product.  The autotuner measures,
for each bucket of output-block sizes (M, N), the device time of the four tile
classes (64x64, 64x32, 32x64, 32x32) on a batch of independent block products
of that size (su2g_f64_tile_bench), keeps the fastest class per bucket, and
installs the table (su2g_f64_tile_table): plans built afterwards tile every
block by its size class.  The table persists as JSON; `load` installs a saved
one (the package ships the one measured on GB300, tile_table_gb300.json, and
installs it when the library loads).
"""
from __future__ import annotations

import ctypes
import json
import os

import numpy as np

from . import capi

EDGES = [8, 16, 24, 32, 48, 64, 96, 128]  # bucket upper edges; the last bucket is open-ended
CLASSES = [(64, 64), (64, 32), (32, 64), (32, 32)]
SHIPPED = os.path.join(os.path.dirname(os.path.abspath(__file__)), "tile_table_gb300.json")


def _rep(i: int) -> int:
    """A representative size of bucket i (its upper edge; 192 for the open one)."""
    return EDGES[i] if i < len(EDGES) else 192


def bench_class(M: int, N: int, K: int, cls: int, reps: int = 5, stream=None) -> float:
    """Device milliseconds per block of M x N x K block products in tiles of
    class cls, over enough blocks to fill the GPU."""
    tm, tn = CLASSES[cls]
    tiles_per_block = -(-M // tm) * -(-N // tn)
    nblocks = max(64, min(4096, 4000 // tiles_per_block))
    ms = ctypes.c_double()
    capi.check(capi.lib().su2g_f64_tile_bench(int(M), int(N), int(K), nblocks, int(cls), int(reps),
                                              ctypes.addressof(ms), capi.stream_handle(stream)))
    return ms.value / nblocks


def tune(K: int = 128, reps: int = 5) -> dict:
    """Measures every (M bucket, N bucket, class) and returns the table:
    {"m_edges", "n_edges", "cls" (row-major M x N buckets), "ms" (per class)}."""
    nb = len(EDGES) + 1
    ms = np.zeros((nb, nb, len(CLASSES)))
    for i in range(nb):
        for j in range(nb):
            for c in range(len(CLASSES)):
                ms[i, j, c] = bench_class(_rep(i), _rep(j), K, c, reps)
    cls = ms.argmin(axis=2)
    return {"m_edges": EDGES, "n_edges": EDGES, "cls": cls.ravel().tolist(), "K": K,
            "ms_per_block": ms.tolist(), "classes": CLASSES}


def install(table: dict) -> None:
    """Installs a table whose buckets are M <= m_edges[i] (and one more,
    open-ended bucket beyond the last edge), likewise N."""
    me = list(table["m_edges"]) + [2**31 - 1]
    ne = list(table["n_edges"]) + [2**31 - 1]
    if len(table["cls"]) != len(me) * len(ne):
        raise ValueError("tile table: cls must hold (len(m_edges) + 1) x (len(n_edges) + 1) classes")
    m = (ctypes.c_int * len(me))(*me)
    n = (ctypes.c_int * len(ne))(*ne)
    c = (ctypes.c_int * len(table["cls"]))(*table["cls"])
    capi.check(capi.lib().su2g_f64_tile_table(ctypes.addressof(m), len(me), ctypes.addressof(n), len(ne),
                                              ctypes.addressof(c)))


def reset() -> None:
    """Back to 64 x 64 tiles for every block."""
    install({"m_edges": [], "n_edges": [], "cls": [0]})


def save(table: dict, path: str) -> None:
    with open(path, "w") as f:
        json.dump(table, f, indent=1)


def load(path: str = SHIPPED) -> dict | None:
    """Installs a saved table; returns it (None when the file does not exist)."""
    if not os.path.exists(path):
        return None
    with open(path) as f:
        table = json.load(f)
    install(table)
    return table
