"""The pre-split set-up's average half area must equal the reference's
sequential f32 sum bit for bit (src/cwbvh/builder.rs:36-41): checked on
values chosen to hit rounding ties, binade crossings and saturation."""
import numpy as np
import pytest

from obvhs_gb300 import scenes as S
from obvhs_gb300 import test_util as T

pytestmark = pytest.mark.gpu


def tris_with_half_areas(v):
    """Flat triangles (0,0,0) (1,0,0) (0,v,0): AABB (1, v, 0), half area v."""
    v = np.asarray(v, np.float32)
    t = np.zeros((len(v), 9), np.float32)
    t[:, 3] = 1.0
    t[:, 7] = v
    return t


def expected(tris):
    a = T.tri_aabbs(tris)
    d = a[:, 3:] - a[:, :3]
    ha = (d[:, 0] + d[:, 1]) * d[:, 2] + d[:, 0] * d[:, 1]
    s = np.add.accumulate(ha, dtype=np.float32)[-1]  # strictly sequential
    avg = np.float32(s / np.float32(len(ha)))
    largest = np.float32(max(np.float32(0), ha.max()))
    hi = max(np.float32(avg * np.float32(4)), np.float32(avg * np.float32(0.9) + largest * np.float32(0.1)))
    return np.array([avg * np.float32(3), hi, avg, largest, s], np.float32)


CASES = {
    "uniform": lambda r: r.uniform(0, 1, 300_000),
    "lognormal": lambda r: r.lognormal(-9, 1.4, 500_000),
    "integers": lambda r: r.integers(0, 1000, 200_000).astype(np.float64),
    "powers_of_two": lambda r: 2.0 ** r.integers(-30, 4, 250_000),
    "outliers": lambda r: np.where(r.random(300_000) < 1e-4, 1e6, r.uniform(0, 1e-3, 300_000)),
    "saturating_ties": lambda r: np.concatenate([[2.0 ** 24], np.full(5000, 1.0), np.full(5000, 1.5),
                                                  np.full(5000, 3.0)]),
    "tiny_then_big": lambda r: np.concatenate([np.full(3000, 1e-30), r.uniform(0, 10, 100_000)]),
    "zeros_then_uniform": lambda r: np.concatenate([np.zeros(5000), r.uniform(0, 1, 60_000)]),
    "one": lambda r: np.array([0.375]),
    "ragged_tail": lambda r: r.uniform(0, 1, 256 * 129 + 77),
    "big_blocks": lambda r: r.uniform(1e5, 1e6, 200_000),
    "growing": lambda r: np.geomspace(1e-6, 1e4, 150_000),
    "near_min_normal": lambda r: r.uniform(1e-38, 1e-36, 100_000),
    "subnormal_start": lambda r: np.concatenate([np.full(700, 1e-40), r.uniform(1e-38, 1e-37, 40_000)]),
}


@pytest.mark.parametrize("case", list(CASES))
def test_sequential_sum_exact(case):
    import obvhs_gb300 as G

    r = np.random.default_rng(11)
    tris = tris_with_half_areas(CASES[case](r))
    got = G.split_thresholds(tris)
    want = expected(tris)
    assert got[:5].tobytes() == want.tobytes(), (got, want)


def test_sequential_sum_scene():
    import obvhs_gb300 as G

    tris = S.scene2_tris(400_000)
    got = G.split_thresholds(tris)
    assert got[:5].tobytes() == expected(tris).tobytes()
    # the block chaining stays parallel: only a few blocks are summed one by one
    assert got[5:6].view(np.uint32)[0] < 40
