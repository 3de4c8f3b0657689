"""Digests of AMG hierarchies and solutions for configuration-size golden files.

At the benchmark's sizes (2.1M unknowns, ~150M stored entries over the
hierarchy) the reference's hierarchy cannot be committed; its SHA-256 per
level can.  Both the generator (make_golden.py, run against the reference)
and the tests (run against this library) hash the same arrays in the same
layout: CSR row pointers and column indices as int32, values as float64,
labels as int32.
"""
from __future__ import annotations

import hashlib

import numpy as np

SAMPLES = 4096


def _sha(*arrays) -> str:
    h = hashlib.sha256()
    for a, dt in arrays:
        h.update(np.ascontiguousarray(a, dtype=dt).tobytes())
    return h.hexdigest()


def csr_sha(m) -> str:
    """SHA-256 of a CSR triple (indptr, indices, data)."""
    return _sha((m[0], np.int32), (m[1], np.int32), (m[2], np.float64))


def level_digest(level_getter, depth):
    """{name: sha} for every level: A, and for l > 0 labels, P and R.  level_getter(l) returns an
    object with attributes A, P, R (CSR triples) and labels."""
    out = {}
    for lv in range(depth):
        L = level_getter(lv)
        out[f"L{lv}_A"] = csr_sha(L.A)
        if lv > 0:
            out[f"L{lv}_labels"] = _sha((L.labels, np.int32))
            out[f"L{lv}_P"] = csr_sha(L.P)
            out[f"L{lv}_R"] = csr_sha(L.R)
    return out


def sample_index(n: int) -> np.ndarray:
    """A fixed subsample of about SAMPLES unknowns, spread evenly over 0..n-1."""
    return np.arange(0, n, max(1, n // SAMPLES), dtype=np.int64)
