"""The block reduction of the tile procedures (block_sum in
graphitethree_gb300/csrc/nlgb_core.cuh) shares the first two butterfly
levels of several values: at level 16 the half-warps swap values a and b,
at level 8 the quarter-warps swap the pairs (a, b) and (c, d).  Because
floating-point addition is commutative, each value must come out of that
packed tree bit for bit as it comes out of the plain 32-lane butterfly
(warp_sum), which the canonical reduction and the two-level election also
use; the executors' bit-identity rests on it.  This restates both trees
lane by lane in float64 and compares them on values spanning 16 decades.
(The GPU tests compare the executors themselves bit for bit.)"""
import numpy as np
import pytest

LANES = np.arange(32)


def shfl_xor(v, o):
    return v[LANES ^ o]


def warp_sum(v):
    """The plain butterfly: v += shfl_xor(v, o) for o = 16, 8, 4, 2, 1."""
    for o in (16, 8, 4, 2, 1):
        v = v + shfl_xor(v, o)
    return v


def packed_totals(vals):
    """The packed tree of block_sum for K = len(vals) values; returns the K
    warp totals as lane 0 collects them."""
    K = len(vals)
    if K == 1:
        return [warp_sum(vals[0])[0]]
    h16 = (LANES & 16) != 0
    u = np.where(h16, vals[1], vals[0]) + shfl_xor(np.where(h16, vals[0], vals[1]), 16)
    if K == 2:
        for o in (8, 4, 2, 1):
            u = u + shfl_xor(u, o)
        return [u[0], u[16]]
    v3 = vals[3] if K == 4 else np.zeros(32)
    u2 = np.where(h16, v3, vals[2]) + shfl_xor(np.where(h16, vals[2], v3), 16)
    h8 = (LANES & 8) != 0
    t = np.where(h8, u2, u) + shfl_xor(np.where(h8, u, u2), 8)
    for o in (4, 2, 1):
        t = t + shfl_xor(t, o)
    return [t[0], t[16], t[8], t[24]][:K]


@pytest.mark.parametrize("K", [1, 2, 3, 4])
def test_packed_butterfly_equals_plain_butterfly_bitwise(K):
    rng = np.random.default_rng(100 + K)
    for _ in range(3000):
        scale = 10.0 ** rng.integers(-8, 8, size=(K, 32))
        vals = [rng.standard_normal(32) * scale[k] for k in range(K)]
        ref = [warp_sum(v)[0] for v in vals]
        got = packed_totals(vals)
        assert [np.float64(x).tobytes() for x in got] == [np.float64(x).tobytes() for x in ref]


def test_every_lane_of_the_plain_butterfly_agrees():
    """The packed tree reads b's total from lane 16 (c from 8, d from 24):
    in an XOR butterfly every lane ends with the same bits, because each
    pair of partners adds the same two values."""
    rng = np.random.default_rng(7)
    for _ in range(1000):
        v = rng.standard_normal(32) * 10.0 ** rng.integers(-8, 8, size=32)
        out = warp_sum(v)
        assert len({x.tobytes() for x in out}) == 1
