"""The mixed kernel's integer-pipe conversions and float-pair arithmetic
(xdynamics_dll_gb300/csrc/xdem_df.cuh) against numpy's IEEE conversions and
FP64 arithmetic, through a small probe library built with nvcc.

  d2f_rn  double -> float, round to nearest even: bit-exact with numpy for
          every input of FP32 normal magnitude; smaller inputs flush to a
          signed zero; NaN stays NaN, overflow gives inf.
  f2d     float -> double: bit-exact for every float (subnormals included).
  split_d hi + lo represents the double to 2^-47 relative (|x| >= 2^-78).
  df_add, df_mul: float-pair results within 2^-44 relative of FP64.
"""
import ctypes as C
import os
import shutil
import subprocess
import tempfile

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

HERE = os.path.dirname(os.path.abspath(__file__))


@pytest.fixture(scope="module")
def probe():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    nvcc = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    out = os.path.join(tempfile.mkdtemp(prefix="xdem_df_"), "libdfprobe.so")
    subprocess.run([nvcc, "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-shared", "-Xcompiler", "-fPIC",
                    os.path.join(HERE, "gpu_df_probe.cu"), "-o", out], check=True)
    L = C.CDLL(out)
    L.df_probe.restype = C.c_int
    L.d2f_sweep.restype = C.c_int
    L.d2f_sweep.argtypes = [C.c_ulonglong, C.c_ulonglong, C.c_void_p]
    return L


def _run(L, x, f, a, b):
    n = x.size
    outs = [np.zeros(n, np.float32) for _ in range(7)]
    f2d = np.zeros(n, np.float64)
    p = lambda arr: arr.ctypes.data_as(C.c_void_p)
    rc = L.df_probe(p(x), p(f), p(a), p(b), C.c_int(n), p(outs[0]), p(f2d), *[p(o) for o in outs[1:]])
    assert rc == 0
    return outs[0], f2d, outs[1], outs[2], outs[3:5], outs[5:7]


def _inputs(n, seed):
    rng = np.random.default_rng(seed)
    # doubles over the whole exponent range, plus hand-picked edge cases
    bits = rng.integers(0, 2 ** 63, size=n, dtype=np.uint64) | (rng.integers(0, 2, size=n, dtype=np.uint64) << 63)
    x = bits.view(np.float64).copy()
    phys = rng.uniform(-2.0, 2.0, n // 2) * 10.0 ** rng.uniform(-12, 3, n // 2)
    x[: n // 2] = phys
    fmin = np.float64(np.finfo(np.float32).tiny)
    fmax = np.float64(np.finfo(np.float32).max)
    edge = [0.0, -0.0, np.inf, -np.inf, np.nan, 1.0, -1.0, fmin, -fmin, fmax, -fmax, fmax * (1 + 2 ** -25),
            fmax * (1 + 2 ** -23), 1 + 2 ** -24, 1 + 3 * 2 ** -24, 1 + 2 ** -24 + 2 ** -40, 2.0 ** -149, 1e-300,
            5e-324, 1.0 - 2 ** -25, 0.1, 1.0 / 3.0, 2.0 ** 127 * (2 - 2 ** -24)]
    x[-len(edge):] = edge
    # floats over the whole range including subnormals, inf and NaN
    fb = rng.integers(0, 2 ** 32, size=n, dtype=np.uint64).astype(np.uint32)
    f = fb.view(np.float32).copy()
    f[:8] = np.array([0.0, -0.0, np.inf, -np.inf, np.nan, 1e-45, -1e-40, 3.4e38], np.float32)
    # float pairs: (hi, lo) with |lo| <= ulp(hi) / 2
    def pairs():
        v = rng.uniform(-1, 1, n) * 10.0 ** rng.uniform(-6, 3, n)
        hi = v.astype(np.float32)
        lo = (v - hi.astype(np.float64) + rng.uniform(-1, 1, n) * np.abs(v) * 2 ** -30).astype(np.float32)
        return np.stack([hi, lo], 1).reshape(-1).astype(np.float32)
    return x, f, pairs(), pairs()


def test_conversions_and_float_pairs(probe):
    n = 1 << 16
    x, f, a, b = _inputs(n, 5)
    d2f, f2d, shi, slo, (sh, sl), (ph, pl) = _run(probe, x, f, a, b)

    # d2f_rn: bit-exact where the result is an FP32 normal or inf/NaN
    with np.errstate(over="ignore"):
        ref = x.astype(np.float32)
    tiny = np.finfo(np.float32).tiny
    normal = np.isfinite(ref) & (np.abs(x) >= tiny)
    assert np.array_equal(d2f[normal].view(np.uint32), ref[normal].view(np.uint32))
    sub = np.isfinite(x) & (np.abs(x) < tiny)
    assert np.all(d2f[sub] == 0.0) and np.array_equal(np.signbit(d2f[sub]), np.signbit(x[sub]))
    inf = np.isinf(ref) & ~np.isnan(x)
    assert np.array_equal(d2f[inf], ref[inf])
    assert np.all(np.isnan(d2f[np.isnan(x)]))

    # f2d: exact for every float
    nanf = np.isnan(f)
    assert np.array_equal(f2d[~nanf].view(np.uint64), f[~nanf].astype(np.float64).view(np.uint64))
    assert np.all(np.isnan(f2d[nanf]))

    # split_d: hi + lo within 2^-47 relative wherever the remainder is an
    # FP32 normal too (|x| >= 2^-78)
    rng_ok = np.isfinite(x) & (np.abs(x) >= 2.0 ** -78) & (np.abs(x) < 2.0 ** 127)
    rec = shi[rng_ok].astype(np.float64) + slo[rng_ok].astype(np.float64)
    assert np.all(np.abs(rec - x[rng_ok]) <= 2.0 ** -47 * np.abs(x[rng_ok]))

    # float-pair sum and product against FP64
    A = a[0::2].astype(np.float64) + a[1::2].astype(np.float64)
    B = b[0::2].astype(np.float64) + b[1::2].astype(np.float64)
    S = sh.astype(np.float64) + sl.astype(np.float64)
    P = ph.astype(np.float64) + pl.astype(np.float64)
    scale = np.abs(A) + np.abs(B)
    assert np.all(np.abs(S - (A + B)) <= 2.0 ** -44 * scale)
    assert np.all(np.abs(P - A * B) <= 2.0 ** -44 * np.abs(A * B))


def test_d2f_rebias_form_equals_field_form(probe):
    """d2f_rn (rebias and round on the bit pattern) against the field-by-field
    form it replaced, bit for bit, over 2^30 doubles of every exponent (half
    of them with their dropped bits at the rounding boundaries)."""
    bad = C.c_ulonglong(0)
    for seed in (1, 2, 3, 4):
        assert probe.d2f_sweep(seed * 0x1234567, 1 << 28, C.byref(bad)) == 0
        assert bad.value == 0, (seed, bad.value)
