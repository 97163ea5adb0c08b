"""CPU checks of the PRNG restatement and of the parallel-seeding algorithm
the GPU uses (no GPU needed).

The GPU computes state i as J^i s0, J the GF(2) matrix of vulkpy's jump
(_vkarray.cc:597-621), from precomputed powers J^(2^k).  Here that algorithm
is restated in numpy and compared with the oracle's serial seeding, which
follows the reference loop exactly.
"""
import numpy as np
import pytest

from oracle import ops as O

JUMP = [0x8764000B, 0xF542D2D3, 0x6FA035C3, 0x77F2DB5B]


def step(s):
    s = list(s)
    t = (s[1] << 9) & 0xFFFFFFFF
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3]; s[2] ^= t
    s[3] = ((s[3] << 11) | (s[3] >> 21)) & 0xFFFFFFFF
    return s


def ref_jump(s):
    acc = [0, 0, 0, 0]
    for w in JUMP:
        for b in range(32):
            if w >> b & 1:
                acc = [a ^ x for a, x in zip(acc, s)]
            s = step(s)
        s = list(acc)
    return s


def matrix_of(f):
    cols = []
    for p in range(128):
        e = [0, 0, 0, 0]
        e[p >> 5] = 1 << (p & 31)
        cols.append(f(e))
    return cols


def apply(m, x):
    r = [0, 0, 0, 0]
    for p in range(128):
        if x[p >> 5] >> (p & 31) & 1:
            r = [a ^ c for a, c in zip(r, m[p])]
    return r


def test_jump_is_linear_and_matrix_power_matches_serial_seeding():
    J = matrix_of(ref_jump)
    pows = [J]
    for _ in range(6):
        pows.append([apply(pows[-1], c) for c in pows[-1]])
    size = 70
    serial = O.Xoshiro128pp(seed=2023, size=size).state.reshape(size, 4)
    s0 = [int(v) for v in serial[0]]
    for i in (1, 2, 5, 33, 64, 69):
        x = s0
        for k in range(7):
            if i >> k & 1:
                x = apply(pows[k], x)
        assert x == [int(v) for v in serial[i]], i


def test_chunked_layout():
    """out[k] = next^(k // size)(state[k % size]); states persist across calls."""
    size = 5
    a = O.Xoshiro128pp(seed=9, size=size)
    b = O.Xoshiro128pp(seed=9, size=size)
    first = a.u32(13)
    second = a.u32(4)
    # one-state-at-a-time restatement from b's initial states
    st = b.state.reshape(size, 4).copy()
    def nxt(t):
        s = [int(v) for v in st[t]]
        r = ((((s[0] + s[3]) & 0xFFFFFFFF) << 7 | ((s[0] + s[3]) & 0xFFFFFFFF) >> 25) & 0xFFFFFFFF)
        r = (r + s[0]) & 0xFFFFFFFF
        st[t] = step(s)
        return r
    exp1 = [nxt(k % size) for k in range(13)]
    exp2 = [nxt(k % size) for k in range(4)]
    assert first.tolist() == exp1
    assert second.tolist() == exp2


def test_float_conversion_and_range():
    r = O.Xoshiro128pp(seed=0, size=64)
    u = r.f32(100000)
    assert u.min() >= 0.0 and u.max() < 1.0
    r2 = O.Xoshiro128pp(seed=0, size=64)
    raw = r2.u32(100000)
    conv = ((raw >> 9) | 0x3F800000).view(np.float32) - np.float32(1)
    np.testing.assert_array_equal(u, conv)


def test_randrange_bounds():
    r = O.Xoshiro128pp(seed=4, size=16)
    v = r.randrange(10000, 10, 1000)
    assert v.min() >= 10 and v.max() < 1000


@pytest.mark.parametrize("n", [0, 1, 2, 3, 4, 5, 17, 1000, 65536, 65537, 1 << 20])
def test_oracle_permutation_is_a_permutation(n):
    from oracle.ops import Xoshiro128pp
    p = Xoshiro128pp(7, 64).permutation(n)
    assert p.dtype == np.uint32 and p.shape == (n,)
    assert np.array_equal(np.sort(p), np.arange(n, dtype=np.uint32))
    # reproducible for a seed, different for another
    assert np.array_equal(p, Xoshiro128pp(7, 64).permutation(n))
    if n > 16:
        assert not np.array_equal(p, Xoshiro128pp(8, 64).permutation(n))
        assert not np.array_equal(p, np.arange(n))


def test_oracle_permutation_draws_four_keys():
    from oracle.ops import Xoshiro128pp
    a, b = Xoshiro128pp(3, 2), Xoshiro128pp(3, 2)
    a.permutation(10)
    b.u32(4)
    assert np.array_equal(a.state, b.state)
    c = Xoshiro128pp(3, 2)
    c.permutation(0)            # draws nothing
    assert np.array_equal(c.state, Xoshiro128pp(3, 2).state)
