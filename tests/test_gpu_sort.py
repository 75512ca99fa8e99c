"""The radix sort behind cu_reorderDataAndFindCellStart: stable, bit-exact
against a CPU stable sort, on sizes and key ranges the step meets."""
import ctypes as C

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def env():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from xdynamics_dll_gb300 import build, _lib
    build.build()
    return torch, _lib.lib()


@pytest.mark.parametrize("n,ncell,dup", [(1, 8, 1), (2, 8, 1), (5000, 128 ** 3, 1), (70001, 1 << 21, 64),
                                         (300000, 1 << 23, 7), (4096, 1, 1), (2049, 256, 256)])
def test_reorder_matches_stable_sort(env, n, ncell, dup):
    torch, L = env
    rng = np.random.default_rng(n + ncell)
    keys = rng.integers(0, max(ncell // dup, 1), size=n, dtype=np.uint64).astype(np.uint32) * dup % ncell
    vals = np.arange(n, dtype=np.uint32)
    order = np.argsort(keys, kind="stable")
    ks, vs = keys[order], vals[order]
    cstart = np.full(ncell, 0xFFFFFFFF, np.uint32)
    cend = np.zeros(ncell, np.uint32)
    first = np.r_[True, ks[1:] != ks[:-1]] if n else np.zeros(0, bool)
    cstart[ks[first]] = np.nonzero(first)[0]
    last = np.r_[ks[1:] != ks[:-1], True] if n else np.zeros(0, bool)
    cend[ks[last]] = np.nonzero(last)[0] + 1
    d = lambda a: torch.from_numpy(a.view(np.int32)).cuda()
    dk, dv = d(keys.copy()), d(vals.copy())
    dcs, dce = torch.zeros(ncell, dtype=torch.int32, device="cuda"), torch.zeros(ncell, dtype=torch.int32, device="cuda")
    dsi = torch.zeros(n, dtype=torch.int32, device="cuda")
    p = lambda t: C.c_void_p(t.data_ptr())
    assert L.cu_reorderDataAndFindCellStart(p(dk), p(dv), p(dcs), p(dce), p(dsi), n, ncell) == 0
    torch.cuda.synchronize()
    u = lambda t: t.cpu().numpy().view(np.uint32)
    assert np.array_equal(u(dk), ks)
    assert np.array_equal(u(dv), vs)
    assert np.array_equal(u(dsi), vs)
    assert np.array_equal(u(dcs), cstart)
    assert np.array_equal(u(dce), cend)
