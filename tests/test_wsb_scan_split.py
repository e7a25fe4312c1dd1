"""The warp split of the general-gap scan keeps the reference's tie rule (CPU).

GeneralGapCostSolver (solver.h:3138-3183) scans a cell's u + 1 vertical and v + 1 horizontal
candidates in order, a later one winning only when strictly better: the winner is the first
maximum.  wsb_kernel splits the scan over a warp -- lane l takes positions p = l + 32 r of both
phases, keeps each phase's first maximum, prefers the vertical one on a tie -- and combines
the lanes by the largest order-preserving key (-0 and +0 equal) and then the smallest
position holding it, taking the value from the lane that scanned that position.  This
restates that split on random scans, with -inf entries and signed-zero ties, and checks it
against the sequential rule bit for bit.
"""

import struct

import numpy as np


def _key(f):
    f = np.float32(0.0) if f == 0 else np.float32(f)
    b = struct.unpack("<I", struct.pack("<f", f))[0]
    return (~b) & 0xFFFFFFFF if b & 0x80000000 else b | 0x80000000


def _sequential(vals):
    best, pos = np.float32(-np.inf), None
    for q, x in enumerate(vals):
        if x > best:
            best, pos = x, q
    return best, pos


def _warp(vals, u, v):
    none = 2**31 - 1
    lanes = []
    for lane in range(32):
        bvv, bqv, bvh, bqh = np.float32(-np.inf), none, np.float32(-np.inf), none
        for p0 in range(0, max(u, v) + 1, 128):
            for r in range(4):
                p = p0 + lane + 32 * r
                if p <= u and vals[p] > bvv:
                    bvv, bqv = vals[p], p
                if p <= v and vals[u + 1 + p] > bvh:
                    bvh, bqh = vals[u + 1 + p], u + 1 + p
        lanes.append((bvh, bqh) if bvh > bvv else (bvv, bqv))
    keys = [_key(x) for x, _ in lanes]
    m = max(keys)
    qw = min(q if k == m else none for (_, q), k in zip(lanes, keys))
    owner = (qw if qw <= u else qw - u - 1) % 32
    return lanes[owner][0], qw


def test_warp_split_finds_the_first_maximum():
    rng = np.random.default_rng(7)
    for _ in range(600):
        u, v = int(rng.integers(0, 300)), int(rng.integers(0, 300))
        vals = rng.integers(-4, 4, u + v + 2).astype(np.float32)
        if rng.random() < 0.3:
            vals[rng.random(vals.size) < 0.2] = -np.inf
        if rng.random() < 0.3:
            vals[rng.random(vals.size) < 0.3] = np.float32(-0.0)
        want_v, want_q = _sequential(vals)
        got_v, got_q = _warp(vals, u, v)
        if want_q is None:
            assert got_q == 2**31 - 1 and got_v == -np.inf
        else:
            assert got_q == want_q, (u, v)
            assert struct.pack("<f", got_v) == struct.pack("<f", want_v), (u, v)
