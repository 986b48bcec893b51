"""Output memory (CWBVH nodes, primitive indices, attached triangles) of freed
BVHs stays in the device's output pool up to the reserve: a rebuild takes no
new device memory and gives the same bytes; a reserve of 0 hands the memory
back to the device."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MB = 1 << 20


def test_freed_outputs_reused_then_returned():
    import torch

    import obvhs_gb300 as G
    from obvhs_gb300 import scenes as S
    from obvhs_gb300.params import BvhBuildParams

    ctx = G.Context(0)
    p = BvhBuildParams.fast_build()
    d = torch.from_numpy(S.scene2_tris(400_000)).cuda()
    try:
        first = G.build_cwbvh_from_tris(d, p, ctx=ctx)
        nodes, pidx = first.download()
        n_nodes, n_prims, _ = first.info()
        out_bytes = n_nodes * 80 + n_prims * 4 + n_prims * 64  # nodes, indices, triangles
        first.free()
        ctx.synchronize()
        free_a = torch.cuda.mem_get_info()[0]
        again = G.build_cwbvh_from_tris(d, p, ctx=ctx)
        ctx.synchronize()
        free_b = torch.cuda.mem_get_info()[0]
        assert free_a - free_b <= 4 * MB  # the reserved memory was reused
        n2, p2 = again.download()
        assert np.array_equal(n2, nodes)
        assert np.array_equal(p2, pidx)
        again.free()
        ctx.synchronize()
        ctx.set_output_reserve(0)
        free_c = torch.cuda.mem_get_info()[0]
        assert free_c - free_a >= out_bytes - 8 * MB  # returned to the device
    finally:
        ctx.set_output_reserve()
