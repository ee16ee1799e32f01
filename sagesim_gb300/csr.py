"""Ragged adjacency -> CSR (host side).

Same results as sagesim/internal_utils.py:111-186 (build_csr_from_ragged,
build_csr_values_only): offsets int32[n+1], values int32 in each row's own
iteration order (set order for sets, insertion order for lists).
"""
from itertools import chain

import numpy as np


def _row_len(row):
    return len(row) if isinstance(row, (list, tuple, set, np.ndarray)) else 0


def build_csr_from_ragged(ragged_list):
    if len(ragged_list) == 0:
        return np.array([0], dtype=np.int32), np.array([], dtype=np.int32)
    lengths = np.fromiter((_row_len(r) for r in ragged_list), dtype=np.int64, count=len(ragged_list))
    offsets = np.zeros(len(lengths) + 1, dtype=np.int64)
    np.cumsum(lengths, out=offsets[1:])
    if offsets[-1] >= 2**31:
        raise ValueError("more than 2^31-1 CSR entries")
    values = build_csr_values_only(ragged_list, offsets)
    return offsets.astype(np.int32), values


def build_csr_values_only(ragged_list, offsets):
    total = int(offsets[-1])
    if all(isinstance(row, (set, list, tuple)) for row in ragged_list):
        # every row a Python container: one pass over their concatenation
        return np.fromiter(chain.from_iterable(ragged_list), dtype=np.int64, count=total).astype(np.int32)
    values = np.empty(total, dtype=np.int32)
    pos = 0
    for row in ragged_list:
        if isinstance(row, np.ndarray):
            k = row.size
            values[pos:pos + k] = row.astype(np.int32)
            pos += k
        elif isinstance(row, (set, list, tuple)):
            k = len(row)
            if k:
                values[pos:pos + k] = np.fromiter((int(v) for v in row), dtype=np.int64, count=k)
            pos += k
    return values
