"""obvhs_morton_sort_noalloc, the entry point that allocates no device memory,
called through the C ABI on device buffers, against obvhs_morton_sort.

Morton codes and the sorted order are integers, so the comparison is bit for
bit.  Each test makes two calls in a row (a larger input, then a smaller one
with other values) because every call shares one fixed scratch array that
keeps the previous call's contents.  The file is named to run last and also
passes on its own in a fresh process.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_PRIMS = 262144  # OBVHS_NOALLOC_MAX_PRIMS in include/obvhs_gb300.h
ERR_INVALID_ARG = -1
ERR_TOO_LARGE = -7


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a CUDA device")
    import obvhs_gb300 as G
    from obvhs_gb300 import _native as N
    torch.cuda.set_device(0)
    return torch, G, N.load()


def _aabbs(n, seed, dup_every=0):
    rng = np.random.default_rng(seed)
    c = rng.uniform(-50, 50, size=(n, 3))
    if dup_every:  # runs of equal centres: equal codes, order decided by input position
        c[1::dup_every] = c[0::dup_every][: len(c[1::dup_every])]
    e = rng.uniform(0, 2, size=(n, 3))
    return np.concatenate([c - e, c + e], 1).astype(np.float32)


def _noalloc(env, a, precision, with_codes=True):
    torch, _, lib = env
    n = len(a)
    dev = torch.device("cuda:0")
    da = torch.from_numpy(a).to(dev)
    codes = torch.full((n, 2), -1, dtype=torch.int64, device=dev)
    order = torch.full((n,), -1, dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    rc = lib.obvhs_morton_sort_noalloc(da.data_ptr(), n, precision, codes.data_ptr() if with_codes else None,
                                       order.data_ptr(), stream.cuda_stream)
    assert rc == 0, rc
    return codes.cpu().numpy().view(np.uint64), order.cpu().numpy().view(np.uint32)


@pytest.mark.parametrize("precision", [0, 1])
def test_two_calls_match_the_allocating_entry_point(env, precision):
    _, G, _ = env
    for n, seed, dup in [(200_003, 11 + precision, 0), (70_001, 12 + precision, 3)]:
        a = _aabbs(n, seed, dup)
        codes, order = _noalloc(env, a, precision)
        ref_codes, ref_order = G.morton_sort(a, precision)
        assert codes.tobytes() == ref_codes.tobytes()
        assert order.tobytes() == ref_order.tobytes()


def test_capacity_edge_and_order_only(env):
    _, G, _ = env
    a = _aabbs(MAX_PRIMS, 21)
    _, order = _noalloc(env, a, 1, with_codes=False)
    _, ref_order = G.morton_sort(a, 1)
    assert order.tobytes() == ref_order.tobytes()
    b = _aabbs(5, 22)
    codes, order = _noalloc(env, b, 0)
    ref_codes, ref_order = G.morton_sort(b, 0)
    assert codes.tobytes() == ref_codes.tobytes()
    assert order.tobytes() == ref_order.tobytes()


def test_rejects_inputs_beyond_capacity(env):
    torch, _, lib = env
    dev = torch.device("cuda:0")
    da = torch.zeros((16, 6), dtype=torch.float32, device=dev)
    order = torch.zeros(16, dtype=torch.int32, device=dev)
    rc = lib.obvhs_morton_sort_noalloc(da.data_ptr(), MAX_PRIMS + 1, 0, None, order.data_ptr(), None)
    assert rc == ERR_TOO_LARGE
    assert lib.obvhs_morton_sort_noalloc(da.data_ptr(), 0, 0, None, order.data_ptr(), None) == 0


def test_rejects_host_memory_without_launching(env):
    """Buffers that are not memory of the current device are refused before
    any GPU work (the check reads pointer attributes only)."""
    torch, _, lib = env
    dev = torch.device("cuda:0")
    h_aabbs = torch.zeros((16, 6), dtype=torch.float32).pin_memory()
    d_aabbs = torch.zeros((16, 6), dtype=torch.float32, device=dev)
    h_order = torch.zeros(16, dtype=torch.int32).pin_memory()
    d_order = torch.zeros(16, dtype=torch.int32, device=dev)
    assert lib.obvhs_morton_sort_noalloc(h_aabbs.data_ptr(), 16, 0, None, d_order.data_ptr(), None) == ERR_INVALID_ARG
    assert lib.obvhs_morton_sort_noalloc(d_aabbs.data_ptr(), 16, 0, None, h_order.data_ptr(), None) == ERR_INVALID_ARG
    codes = np.zeros((16, 2), np.uint64)  # pageable host memory
    assert lib.obvhs_morton_sort_noalloc(d_aabbs.data_ptr(), 16, 0, codes.ctypes.data, d_order.data_ptr(),
                                         None) == ERR_INVALID_ARG


def test_call_leaves_free_device_memory_unchanged(env):
    """After a warm-up call (which loads the library's kernels), a second call
    leaves the device's free memory as it was: it allocates nothing.  The free
    figure only approximates "no allocation" (another process on the GPU
    could change it), so this is a check, not a proof."""
    torch, _, lib = env
    dev = torch.device("cuda:0")
    a = _aabbs(100_000, 31)
    da = torch.from_numpy(a).to(dev)
    codes = torch.empty((len(a), 2), dtype=torch.int64, device=dev)
    order = torch.empty((len(a),), dtype=torch.int32, device=dev)
    stream = torch.cuda.current_stream(dev)
    assert lib.obvhs_morton_sort_noalloc(da.data_ptr(), len(a), 1, codes.data_ptr(), order.data_ptr(),
                                         stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free0, _ = torch.cuda.mem_get_info(dev)
    assert lib.obvhs_morton_sort_noalloc(da.data_ptr(), len(a), 1, codes.data_ptr(), order.data_ptr(),
                                         stream.cuda_stream) == 0
    torch.cuda.synchronize()
    free1, _ = torch.cuda.mem_get_info(dev)
    assert free1 == free0
