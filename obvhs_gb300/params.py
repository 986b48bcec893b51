"""Build parameters mirroring obvhs's `BvhBuildParams` and its presets.

Reference: src/lib.rs:296-395 (struct + presets), src/ploc/mod.rs:530-561
(PlocSearchDistance) and :657-661 (SortPrecision).  Pure Python, no CUDA.
"""
from __future__ import annotations

import enum
from dataclasses import dataclass


class PlocSearchDistance(enum.IntEnum):
    """In PLOC, the number of nodes before and after the current one that are
    evaluated for pairing (src/ploc/mod.rs:534-548).  The integer value is the
    radius; `PlocBuilder.build_ploc` also accepts any radius 1..32 directly,
    like the reference's `build_ploc::<SEARCH_DISTANCE>`."""

    Minimum = 1
    VeryLow = 2
    Low = 6
    Medium = 14
    High = 24
    VeryHigh = 32

    @classmethod
    def from_u32(cls, value: int) -> "PlocSearchDistance":
        """`impl From<u32> for PlocSearchDistance` (src/ploc/mod.rs:550-561):
        any value outside the six variants is an error."""
        try:
            return cls(int(value))
        except ValueError:
            raise ValueError(f"Invalid value for PlocSearchDistance: {value}") from None


class SortPrecision(enum.IntEnum):
    """Bits used for the PLOC Morton sort (src/ploc/mod.rs:657-661)."""

    U64 = 0
    U128 = 1


@dataclass
class BvhBuildParams:
    """General build parameters for Bvh2 & CwBvh (src/lib.rs:296-319)."""

    pre_split: bool
    ploc_search_distance: int
    search_depth_threshold: int
    reinsertion_batch_ratio: float
    post_collapse_reinsertion_batch_ratio_multiplier: float
    sort_precision: int
    max_prims_per_leaf: int
    collapse_traversal_cost: float

    @staticmethod
    def fastest_build() -> "BvhBuildParams":
        return BvhBuildParams(False, PlocSearchDistance.Minimum, 0, 0.0, 0.0, SortPrecision.U64, 1, 1.0)

    @staticmethod
    def very_fast_build() -> "BvhBuildParams":
        return BvhBuildParams(False, PlocSearchDistance.Minimum, 0, 0.01, 0.0, SortPrecision.U64, 8, 3.0)

    @staticmethod
    def fast_build() -> "BvhBuildParams":
        return BvhBuildParams(False, PlocSearchDistance.Low, 2, 0.02, 0.0, SortPrecision.U64, 8, 3.0)

    @staticmethod
    def medium_build() -> "BvhBuildParams":
        return BvhBuildParams(False, PlocSearchDistance.Medium, 3, 0.05, 2.0, SortPrecision.U64, 8, 3.0)

    @staticmethod
    def slow_build() -> "BvhBuildParams":
        return BvhBuildParams(True, PlocSearchDistance.High, 2, 0.2, 2.0, SortPrecision.U128, 8, 3.0)

    @staticmethod
    def very_slow_build() -> "BvhBuildParams":
        return BvhBuildParams(True, PlocSearchDistance.Medium, 1, 1.0, 1.0, SortPrecision.U128, 8, 3.0)


#: The six presets in the order of the reference's BUILD_PARAM_SET (tests/mod.rs:25-32).
PRESETS = {
    "fastest": BvhBuildParams.fastest_build,
    "very_fast": BvhBuildParams.very_fast_build,
    "fast": BvhBuildParams.fast_build,
    "medium": BvhBuildParams.medium_build,
    "slow": BvhBuildParams.slow_build,
    "very_slow": BvhBuildParams.very_slow_build,
}
