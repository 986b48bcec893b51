"""The pre-split average's exact f32 sum, restated on the CPU: inside one
binade [2^E, 2^(E+1)) adding a >= 0 is integer arithmetic on the
significand, a block of elements maps to two increments (even / odd start)
composed by an associative rule with saturation at 2^25, and a block whose
composed effect leaves the binade is added element by element.  The chained
result equals numpy's strictly sequential float32 sum bit for bit."""
import numpy as np
import pytest

SAT = 1 << 25


def _elem(v, e):
    x = float(v) * 2.0 ** (23 - e)  # exact: a power-of-two scaling
    if not x < 16777216.0:
        return SAT, SAT
    m = int(np.floor(x))
    f = x - m
    if f < 0.5:
        return m, m
    if f > 0.5:
        return m + 1, m + 1
    return m + (m & 1), m + ((1 + m) & 1)  # a tie makes S + m + r even


def _then(a, b):
    g0 = min(a[0] + (b[1] if a[0] & 1 else b[0]), SAT)
    g1 = min(a[1] + (b[1] if (1 + a[1]) & 1 else b[0]), SAT)
    return g0, g1


def _chain(ha, block=64):
    s = np.float32(0.0)
    sequential = 0
    for b0 in range(0, len(ha), block):
        blk = ha[b0:b0 + block]
        bits = int(s.view(np.uint32))
        ex = (bits >> 23) & 0xFF
        if ex not in (0, 0xFF):
            eff = (0, 0)
            for v in blk:
                eff = _then(eff, _elem(v, ex - 127))
            S = (bits & 0x7FFFFF) | 0x800000
            S2 = S + (eff[1] if S & 1 else eff[0])
            if S2 < (1 << 24):
                s = np.uint32((ex << 23) | (S2 - (1 << 23))).view(np.float32)
                continue
        sequential += 1
        for v in blk:
            s = np.float32(s + v)
    return s, sequential


CASES = {
    "uniform": lambda r: r.uniform(0, 1, 4000),
    "lognormal": lambda r: r.lognormal(-9, 1.4, 4000),
    "integers": lambda r: r.integers(0, 1000, 3000).astype(np.float64),
    "ties": lambda r: np.concatenate([[2.0 ** 24], np.full(500, 1.0), np.full(500, 1.5), np.full(500, 3.0)]),
    "growing": lambda r: np.geomspace(1e-6, 1e4, 3000),
    "zeros_first": lambda r: np.concatenate([np.zeros(200), r.uniform(0, 1, 2000)]),
}


@pytest.mark.parametrize("case", list(CASES))
def test_chained_sum_equals_sequential(case):
    ha = CASES[case](np.random.default_rng(7)).astype(np.float32)
    want = np.add.accumulate(ha, dtype=np.float32)[-1]
    got, sequential = _chain(ha)
    assert got.view(np.uint32) == np.float32(want).view(np.uint32)
    assert sequential <= len(ha) // 64 + 1
