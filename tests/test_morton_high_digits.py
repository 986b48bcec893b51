"""The Morton sort's plan on the CPU: a stable sort on the high digits only
(U128: the high 64 bits; U64: bits 24-63), then every run of equal high
digits (at most 32 long) put in order of the remaining bits stably, gives
the stable order of the whole codes -- checked against the oracle's own
stable sort on inputs with many equal high digits."""
import numpy as np
import pytest

from oracle import oracle as O


def _high_then_runs(codes, precision, run_max=32):
    if precision:
        hi, lo = codes[:, 1], codes[:, 0]
    else:
        hi, lo = codes[:, 0] >> np.uint64(24), codes[:, 0] & np.uint64(0xFFFFFF)
    order = np.argsort(hi, kind="stable")
    h = hi[order]
    i, n = 0, len(order)
    while i < n:
        j = i + 1
        while j < n and h[j] == h[i]:
            j += 1
        if j - i > run_max:
            return None  # the device sorts the whole codes instead
        if j - i > 1:
            seg = order[i:j]
            order[i:j] = seg[np.argsort(lo[seg], kind="stable")]
        i = j
    return order


@pytest.mark.parametrize("precision", [0, 1])
def test_high_digits_then_runs_is_the_stable_order(precision):
    rng = np.random.default_rng(40 + precision)
    base = rng.uniform(-50, 50, size=(1500, 3))
    reps = rng.integers(1, 33, size=len(base))
    c = np.repeat(base, reps, axis=0)
    c = c + rng.uniform(-1, 1, size=c.shape) * (2e-3 if precision == 0 else 1e-5)
    c[::5] = np.repeat(base, reps, axis=0)[::5]
    c = c[rng.permutation(len(c))]
    a = np.concatenate([c - 1e-6, c + 1e-6], 1).astype(np.float32)
    codes, order = O.morton(a, precision)
    got = _high_then_runs(codes, precision)
    if got is None:
        pytest.skip("a run longer than 32: the whole codes are sorted")
    assert np.array_equal(got.astype(np.uint32), order)
