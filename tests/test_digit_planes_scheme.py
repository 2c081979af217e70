"""The digit-plane scheme of the tensor-core products (htool_gb300/csrc/oz.cu),
restated on the CPU with Python integers: the properties its exactness rests
on, independent of the GPU.

* The balanced base-128 split (|lower digits| <= 64, top <= 2^(T - 49) + 1)
  and its carry-free form (bias 64 on every lower position) give the same
  digits, and reconstruct the fixed-point integer exactly.
* Every digit is exact in BF16 (at most 8 significant bits).
* With T = 54 (8 digits) a diagonal of the plane products adds at most
  28 800 per column, so 271 rows stay below 2^23; the worst case is reached
  by digits all of one sign at their bound.
* Dropping the pairs i + j >= S costs less than 2^-(7 S - 8) of the leading
  term."""
import random

import numpy as np


def split_seq(q, S):
    d = [0] * S
    for i in range(S - 1, 0, -1):
        lo = q & 127
        lo = lo - 128 if lo >= 64 else lo
        d[i] = lo
        q = (q - lo) >> 7
    d[0] = q
    return d


def split_bias(q, S):
    bias = sum(64 << (7 * i) for i in range(S - 1))
    u = q + bias
    return [u >> (7 * (S - 1))] + [((u >> (7 * (S - 1 - i))) & 127) - 64 for i in range(1, S)]


def value(d, S):
    return sum(di << (7 * (S - 1 - i)) for i, di in enumerate(d))


def bf16_exact(v):
    f = np.float32(v)
    b = f.view(np.uint32) & np.uint32(0xFFFF0000)
    return float(b.view(np.float32)) == float(v)


def test_splits_agree_and_reconstruct():
    rng = random.Random(5)
    for S in (8, 4):
        T = 5 + 7 * (S - 1)
        edge = [0, 1, -1, 63, 64, -64, -65, 2**T, -(2**T), 2**T - 1, -(2**T) + 1]
        for q in edge + [rng.randint(-(2**T), 2**T) for _ in range(20000)]:
            d = split_seq(q, S)
            assert d == split_bias(q, S)
            assert value(d, S) == q
            assert all(-64 <= x <= 63 for x in d[1:])
            assert abs(d[0]) <= 2 ** (T - 7 * (S - 1)) + 1
            assert all(bf16_exact(x) for x in d)


def test_diagonal_sums_stay_below_2_23():
    S, T = 8, 54
    top = 2 ** (T - 7 * (S - 1)) + 1  # 33
    per_column = max(sum((top if i == 0 else 64) * (top if D - i == 0 else 64) for i in range(D + 1)) for D in range(S))
    assert per_column == 2 * 33 * 64 + 6 * 64 * 64 == 28800
    assert per_column * 271 < 2**23
    # the adversarial operand of the GPU test: digits -31, -64, ..., -64
    q = -31 * 2**49 - 64 * ((2**49 - 1) // 127)
    d = split_seq(q, S)
    assert d == [-31] + [-64] * 7 and 2**53 <= -q < 2**54
    worst = max(sum(d[i] * d[D - i] for i in range(D + 1)) for D in range(S)) * 256
    assert worst == 7307264 < 2**23


def test_dropped_pairs_are_small():
    S = 8
    T = 5 + 7 * (S - 1)
    rng = random.Random(9)
    for _ in range(2000):
        a, b = rng.randint(-(2**T), 2**T), rng.randint(-(2**T), 2**T)
        da, db = split_seq(a, S), split_seq(b, S)
        kept = sum(da[i] * db[j] << (7 * (2 * S - 2 - i - j)) for i in range(S) for j in range(S) if i + j < S)
        assert abs(a * b - kept) <= 2 ** (2 * T - (7 * S - 8))
