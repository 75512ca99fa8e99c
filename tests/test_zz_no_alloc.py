"""cu_reorderDataAndFindCellStart_noalloc: the allocation-free sort + cell
ranges, for callers that may not call cudaMalloc (real-time loops that cannot
risk an allocation's latency or an out-of-memory failure mid-run, hosts whose
device memory an external pool owns).

It must give exactly what cu_reorderDataAndFindCellStart gives (integer work:
bit-exact), call after call, although every call reuses one fixed scratch
array inside the library whose contents the previous call left behind.  This
file is collected last so a failure here cannot hide another test's result.
"""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

MAX_ENTRIES = 262144


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, _lib
    build.build()
    return torch, _lib.lib()


def _run(torch, fn, keys, vals, ncell):
    n = keys.size
    # one spare entry so an empty call still passes real (non-null) pointers
    d = lambda a: torch.from_numpy(np.concatenate([a, [0xDEADBEEF]]).astype(np.uint32).view(np.int32)).cuda()
    dk, dv = d(keys), d(vals)
    dcs = torch.full((ncell,), 7, dtype=torch.int32, device="cuda")
    dce = torch.full((ncell,), 7, dtype=torch.int32, device="cuda")
    dsi = torch.zeros(max(n, 1), dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    rc = fn(p(dk), p(dv), p(dcs), p(dce), p(dsi), n, ncell)
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    return rc, u(dk)[:n], u(dv)[:n], u(dcs), u(dce), u(dsi)[:n]


def _scene_keys(n, ncell, seed, dup):
    rng = np.random.default_rng(seed)
    keys = (rng.integers(0, max(ncell // dup, 1), size=n) * dup % ncell).astype(np.uint32)
    return keys, np.arange(n, dtype=np.uint32)


def test_noalloc_matches_allocating_launcher_twice(env):
    torch, L = env
    # two calls in a row: a large one, then a smaller one with other keys, so
    # the second call runs over scratch the first one left behind
    for n, ncell, seed, dup in [(200000, 1 << 21, 1, 3), (70001, 128 ** 3, 2, 1)]:
        keys, vals = _scene_keys(n, ncell, seed, dup)
        ref = _run(torch, L.cu_reorderDataAndFindCellStart, keys, vals, ncell)
        new = _run(torch, L.cu_reorderDataAndFindCellStart_noalloc, keys, vals, ncell)
        assert ref[0] == 0 and new[0] == 0
        for a, b, name in zip(ref[1:], new[1:], ["hash", "index", "cstart", "cend", "sorted_index"]):
            assert np.array_equal(a, b), name
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(new[1], keys[order]) and np.array_equal(new[2], vals[order])


def test_noalloc_rejects_sizes_beyond_capacity(env):
    torch, L = env
    from xdynamics_dll_gb300 import types as T
    n = MAX_ENTRIES + 1
    keys, vals = _scene_keys(n, 4096, 3, 1)
    rc, k, v, cs, ce, _ = _run(torch, L.cu_reorderDataAndFindCellStart_noalloc, keys, vals, 4096)
    assert rc == T.XDEM_ERR_ARG
    # nothing was touched
    assert np.array_equal(k, keys) and np.array_equal(v, vals)
    assert np.all(cs == 7) and np.all(ce == 7)
    # the largest allowed size still works
    keys, vals = _scene_keys(MAX_ENTRIES, 1 << 20, 4, 1)
    rc, k, v, _, _, _ = _run(torch, L.cu_reorderDataAndFindCellStart_noalloc, keys, vals, 1 << 20)
    order = np.argsort(keys, kind="stable")
    assert rc == 0 and np.array_equal(k, keys[order]) and np.array_equal(v, vals[order])


def test_noalloc_every_pass_count_after_a_large_call(env):
    """The radix sort runs one pass per 8 bits of the cell count: an odd
    number of passes leaves the result in the scratch array (copied back),
    an even number leaves it in place, and fewer than two entries sort
    nothing.  A large call first fills the shared scratch with other data;
    each smaller call must still match the allocating launcher bit for bit."""
    torch, L = env
    big_keys, big_vals = _scene_keys(MAX_ENTRIES, 1 << 21, 11, 1)
    assert _run(torch, L.cu_reorderDataAndFindCellStart_noalloc, big_keys, big_vals, 1 << 21)[0] == 0
    cases = [(50000, 1 << 16, 12, 3),   # 16 bits: two passes, result in place
             (40000, 1 << 12, 13, 1),   # 12 bits: two passes
             (3000, 256, 14, 2),        # 8 bits: one pass, copied back
             (5, 1, 15, 1),             # one cell: one pass
             (1, 4096, 16, 1),          # one entry: nothing to sort
             (0, 4096, 17, 1)]          # empty: every cell empty
    for n, ncell, seed, dup in cases:
        keys, vals = _scene_keys(n, ncell, seed, dup)
        ref = _run(torch, L.cu_reorderDataAndFindCellStart, keys, vals, ncell)
        new = _run(torch, L.cu_reorderDataAndFindCellStart_noalloc, keys, vals, ncell)
        assert ref[0] == 0 and new[0] == 0, (n, ncell)
        for a, b, name in zip(ref[1:], new[1:], ["hash", "index", "cstart", "cend", "sorted_index"]):
            assert np.array_equal(a, b), (n, ncell, name)
        order = np.argsort(keys, kind="stable")
        assert np.array_equal(new[1], keys[order]) and np.array_equal(new[2], vals[order])
        if n == 0:
            assert np.all(new[3] == 0xFFFFFFFF) and np.all(new[4] == 0)
