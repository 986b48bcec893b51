"""Device-side waits that run out (needs a GPU).

Every wait in the library's kernels is bounded: a kernel that waits too long
sets a status bit and returns, and the call reports OBVHS_ERR_LIMIT instead of
hanging.  The radix sort's decoupled look-back (tiles waiting for the counts
of earlier tiles) takes its bound from the context, so a test can make it run
out: with a bound of 0 a tile gives up at its first wait.  The build must then
fail with OBVHS_ERR_LIMIT, touch nothing out of bounds, and the same context
must build the correct tree once the bound is back at its default.  The
reference has no counterpart (it has no device waits).
"""
import numpy as np
import pytest

from oracle import oracle as O
from obvhs_gb300 import scenes as S
from obvhs_gb300.params import BvhBuildParams

pytestmark = pytest.mark.gpu

ERR_LIMIT = -5  # OBVHS_ERR_LIMIT in include/obvhs_gb300.h


def test_sort_wait_bound_runs_out_then_the_context_recovers():
    import obvhs_gb300 as G
    from obvhs_gb300._native import ObvhsError

    tris = S.scene2_tris(1_000_000)
    # no pre-splits or reinsertion: the Morton sort is the only sort of the build
    p = BvhBuildParams(False, 14, 3, 0.0, 0.0, 0, 3, 3.0)
    ctx = G.Context()
    try:
        ctx.set_wait_limit(0)
        codes = []
        for _ in range(3):  # a tile of 1M keys almost always finds its predecessor busy
            try:
                G.build_cwbvh_from_tris(tris, p, ctx=ctx)
                codes.append(0)
            except ObvhsError as e:
                codes.append(e.code)
                if e.code == ERR_LIMIT:
                    break
        assert ERR_LIMIT in codes, codes
        assert set(codes) <= {0, ERR_LIMIT}, codes
        ctx.set_wait_limit()
        cw = G.build_cwbvh_from_tris(tris, p, ctx=ctx)
        nodes, prims = cw.download()
    finally:
        ctx.close()
    ob = O.build(tris=tris, params=p, nthreads=8, keep_intermediate=False)
    assert nodes.tobytes() == np.ascontiguousarray(ob.cw_nodes).tobytes()
    assert prims.tobytes() == np.ascontiguousarray(ob.cw_pidx).tobytes()
