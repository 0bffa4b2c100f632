"""Model check of the integer exact-sum shortcut used by the device kernels
(smartcore_gb300/csrc/exactsum.cuh): whenever the exponent-span condition
holds, the integer sum equals the reference's sequential f64 sum of the f32
squares (src/metrics/distance/euclidian.rs:56-63) bit for bit."""
import math

import numpy as np


def reference(a, b):
    s = 0.0
    for x, y in zip(a, b):
        r = np.float32(x) - np.float32(y)
        s += float(np.float32(r * r))
    return s


def shortcut(a, b):
    d = len(a)
    lg_d = max(0, math.ceil(math.log2(d))) if d > 1 else 0
    q = (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)
    q = (q * q).astype(np.float32)
    bits = q.view(np.uint32)
    nz = bits[bits != 0]
    if len(nz) == 0:
        return 0.0
    e = np.maximum(nz >> 23, 1).astype(np.int64)
    emin, emax = int(e.min()), int(e.max())
    if emax >= 255 or emax - emin > 29 - lg_d:
        return None
    m = (nz & 0x7FFFFF) | np.where((nz >> 23) != 0, 0x800000, 0).astype(np.uint32)
    S = sum(int(mi) << (int(ei) - emin) for mi, ei in zip(m, e))
    assert S < 2 ** 53
    return math.ldexp(float(S), emin - 150)


def test_shortcut_matches_sequential_sum():
    rng = np.random.default_rng(0)
    used = 0
    for trial in range(3000):
        d = int(rng.integers(1, 80))
        scale = 10.0 ** rng.uniform(-6, 6)
        a = (rng.normal(size=d) * scale).astype(np.float32)
        b = (rng.normal(size=d) * scale).astype(np.float32)
        if trial % 7 == 0:
            b[: d // 2] = a[: d // 2]  # exact zeros
        if trial % 11 == 0:
            b[0] = np.float32(a[0] + np.float32(1e-3) * scale)  # a small term
        got = shortcut(a, b)
        if got is not None:
            used += 1
            assert got == reference(a, b)
    assert used > 1000
