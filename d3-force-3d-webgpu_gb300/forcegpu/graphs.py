"""Seeded synthetic inputs with the shape of the reference's own workloads.

  lcg_uniforms      the reference's LCG (src/lcg.js: a = 1664525, c = 1013904223, m = 2^32) as
                    uniforms in [0, 1), from any seed; vectorised by jump-ahead
  benchmark_links   the benchmark graph (examples/benchmark.html:86-93): a random tree, node i
                    linked to floor(u * i), then extra uniform random pairs; here the extras
                    reject self-loops and duplicates (undirected) until `extra` are found
  make_nodes        test/gpu-helpers.js:42-53 makeNodes: f32-exact coordinates in a cube
  phyllotaxis       src/simulation.js:79-107: the start of nodes without a position
"""
from __future__ import annotations

import math

import numpy as np

A, C, M = 1664525, 1013904223, 1 << 32


def _jump_tables(k):
    """s_j = A_j * s_0 + C_j (mod 2^32) for j = 1..k."""
    Aj = np.empty(k, np.uint64)
    Cj = np.empty(k, np.uint64)
    a, c = 1, 0
    for j in range(k):
        a, c = (A * a) % M, (A * c + C) % M
        Aj[j], Cj[j] = a, c
    return Aj, Cj


_TABLES = {}


class LCG:
    """The reference's LCG stream; draw(k) returns the next k uniforms s / 2^32."""

    def __init__(self, seed):
        self.s = int(seed) % M

    def draw(self, k):
        out = np.empty(k, np.float64)
        B = 4096
        if B not in _TABLES:
            _TABLES[B] = _jump_tables(B)
        Aj, Cj = _TABLES[B]
        done = 0
        mask = np.uint64(M - 1)
        while done < k:
            m = min(B, k - done)
            s = (Aj[:m] * np.uint64(self.s) + Cj[:m]) & mask
            out[done:done + m] = s.astype(np.float64) / M
            self.s = int(s[m - 1])
            done += m
        return out


def lcg_uniforms(seed, k):
    return LCG(seed).draw(k)


def benchmark_links(n, extra=None, seed=42):
    """(source, target) int32 arrays: n - 1 tree links then `extra` distinct random pairs."""
    if extra is None:
        extra = n // 2
    rng = LCG(seed)
    if n < 2:
        return np.zeros(0, np.int32), np.zeros(0, np.int32)
    i = np.arange(1, n, dtype=np.int64)
    tgt = np.floor(rng.draw(n - 1) * i).astype(np.int64)
    src = i
    keys = np.minimum(src, tgt) * n + np.maximum(src, tgt)
    seen = np.sort(keys)
    max_pairs = n * (n - 1) // 2 - (n - 1)
    extra = min(extra, max_pairs)
    es, et = [], []
    got = 0
    while got < extra:
        want = max(1024, 2 * (extra - got))
        u = rng.draw(2 * want)
        a = np.floor(u[0::2] * n).astype(np.int64)
        b = np.floor(u[1::2] * n).astype(np.int64)
        ok = a != b
        a, b = a[ok], b[ok]
        k = np.minimum(a, b) * n + np.maximum(a, b)
        _, first = np.unique(k, return_index=True)
        firstmask = np.zeros(len(k), bool)
        firstmask[first] = True
        pos = np.searchsorted(seen, k)
        pos[pos == len(seen)] = 0
        new = firstmask & (seen[pos] != k)
        a, b, k = a[new], b[new], k[new]
        take = min(len(a), extra - got)
        es.append(a[:take])
        et.append(b[:take])
        seen = np.sort(np.concatenate([seen, k[:take]]))
        got += take
    src = np.concatenate([src] + es).astype(np.int32)
    tgt = np.concatenate([tgt] + et).astype(np.int32)
    return src, tgt


def make_nodes(n, dims, size=200.0, seed=12345):
    """(n, 3) float64 array of f32-exact coordinates (test/gpu-helpers.js:42-53), unused axes 0."""
    u = np.float32(LCG(seed).draw(n * dims)).astype(np.float64).reshape(n, dims)
    xyz = np.zeros((n, 3))
    xyz[:, :dims] = np.float32((u - 0.5) * size)
    return xyz


def phyllotaxis(n, dims):
    """(n, 3) float64 start positions of src/simulation.js:79-107."""
    i = np.arange(n, dtype=np.float64)
    roll = i * (math.pi * (3 - math.sqrt(5)))
    yaw = i * (math.pi * 20 / (9 + math.sqrt(221)))
    out = np.zeros((n, 3))
    if dims == 1:
        out[:, 0] = 10 * i
    elif dims == 2:
        r = 10 * np.sqrt(0.5 + i)
        out[:, 0], out[:, 1] = r * np.cos(roll), r * np.sin(roll)
    else:
        r = 10 * np.cbrt(0.5 + i)
        out[:, 0] = r * np.sin(roll) * np.cos(yaw)
        out[:, 1] = r * np.cos(roll)
        out[:, 2] = r * np.sin(roll) * np.sin(yaw)
    return out


def link_defaults(n, src, dst):
    """count, bias and the default strength 1 / min(count) of src/link.js:30-32, :65-75."""
    count = np.bincount(src, minlength=n) + np.bincount(dst, minlength=n)
    cs, ct = count[src].astype(np.float64), count[dst].astype(np.float64)
    return cs / (cs + ct), 1.0 / np.minimum(cs, ct)
