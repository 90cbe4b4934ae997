"""The warp reduce-scatter of block_sum (hbtplus_gb300/csrc/loop.cu) adds the
same pairs in the same association as an xor butterfly, so its sums are
bit-identical to the butterfly's; and the lane-to-sum map it computes gives
every one of the K sums to exactly one lane.

This restates the kernel's steps (rs_step and the index tracking of
block_sum) over 32 simulated lanes in float64 and compares them with a
butterfly, for every K from 1 to 32 and values spread over 16 decades."""
import numpy as np
import pytest


def butterfly(v):
    """v[lane][k]: every lane ends with the same sums."""
    v = [list(r) for r in v]
    for o in (16, 8, 4, 2, 1):
        v = [[v[l][k] + v[l ^ o][k] for k in range(len(v[0]))] for l in range(32)]
    return v[0]


def reduce_scatter(v, K):
    cur, N = [list(r) for r in v], K
    for o in (16, 8, 4, 2, 1):  # rs_step<N>
        h = (N + 1) // 2
        nxt = []
        for l in range(32):
            up, p = bool(l & o), l ^ o
            row = []
            for j in range(h):
                lo, hi = cur[l][j], (cur[l][j + h] if j + h < N else 0.0)
                plo, phi = cur[p][j], (cur[p][j + h] if j + h < N else 0.0)
                recv = plo if (p & o) else phi  # the partner sends (upper ? lo : hi)
                row.append((hi if up else lo) + recv)
            nxt.append(row)
        cur, N = nxt, h
    out = {}
    for l in range(32):  # block_sum's index tracking
        base, n, N = 0, K, K
        for o in (16, 8, 4, 2, 1):
            h = (N + 1) // 2
            if l & o:
                base += h
                n = max(0, n - h)
            else:
                n = min(n, h)
            N = h
        if n >= 1:
            assert base not in out and 0 <= base < K, (K, l, base)
            out[base] = cur[l][0]
    assert sorted(out) == list(range(K))
    return [out[k] for k in range(K)]


@pytest.mark.parametrize("K", list(range(1, 33)))
def test_reduce_scatter_equals_butterfly(K):
    rng = np.random.default_rng(K)
    for _ in range(8):
        v = rng.standard_normal((32, K)) * 10.0 ** rng.integers(-8, 8, (32, K))
        a, b = butterfly(v.tolist()), reduce_scatter(v.tolist(), K)
        assert np.array(a, np.float64).tobytes() == np.array(b, np.float64).tobytes()
