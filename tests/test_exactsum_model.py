"""Model check of the integer reproduction of the sequential f64 sum used by
the device kernels (smartcore_gb300/csrc/exactsum.cuh): whenever the
exponent-span condition holds, it equals the reference's sequential f64 sum
of the f32 squares (src/metrics/distance/euclidian.rs:56-63) bit for bit."""
import math

import numpy as np


def reference(a, b):
    s = 0.0
    for x, y in zip(a, b):
        r = np.float32(x) - np.float32(y)
        s += float(np.float32(r * r))
    return s


def seq_rounding(a, b):
    """Model of sqd_seq_f32_d32: exact integer running sum of the f32 squares
    in units of 2^(emin - 150), rounded to 53 significant bits (nearest, ties
    to even) after every term, as each f64 addition rounds; the span limit
    38 - ceil(log2 d) keeps the sum below 2^63."""
    q = (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)
    q = (q * q).astype(np.float32)
    bits = q.view(np.uint32)
    nz = bits[bits != 0]
    if len(nz) == 0:
        return 0.0
    e_all = np.maximum(nz >> 23, 1).astype(np.int64)
    emin, emax = int(e_all.min()), int(e_all.max())
    lg_d = max(0, math.ceil(math.log2(len(a)))) if len(a) > 1 else 0
    if emax >= 255 or emax - emin > 38 - lg_d:
        return None
    S = 0
    for u in bits:
        u = int(u)
        if u == 0:
            continue
        e = u >> 23
        m = (u & 0x7FFFFF) | (0x800000 if e else 0)
        S += m << (max(e, 1) - emin)
        assert S < 2 ** 63
        if S >> 53:
            drop = S.bit_length() - 53
            half = 1 << (drop - 1)
            rem = S & ((half << 1) - 1)
            qv = S >> drop
            if rem > half or (rem == half and (qv & 1)):
                qv += 1
            S = qv << drop
    return math.ldexp(float(S), emin - 150)


def test_sequential_rounding_matches_sequential_sum():
    rng = np.random.default_rng(1)
    used = 0
    for trial in range(4000):
        d = int(rng.integers(1, 81))
        span = rng.uniform(0, 7)
        scale = 10.0 ** rng.uniform(-span, span, size=d)
        a = (rng.normal(size=d) * scale).astype(np.float32)
        b = (rng.normal(size=d) * scale).astype(np.float32)
        if trial % 5 == 0:
            b = (a * np.float32(1.0 + 1e-6)).astype(np.float32)  # near-duplicates: tiny terms
        got = seq_rounding(a, b)
        if got is not None:
            used += 1
            assert got == reference(a, b), (trial, got, reference(a, b))
    assert used > 1000


def no_rounding_sum(a, b):
    """Model of the k-means++ row update's integer path: with the exponent
    span of the nonzero f32 squares at most 38 - ceil(log2 d), the integer sum
    S of the terms in units of 2^(emin - 150) stays below 2^62; when S < 2^53,
    every partial sum of the sequential f64 sum is an integer below 2^53, so
    no addition rounds and the terms may be added in any order (here: reversed
    halves, as lanes of a row are added by a shuffle tree)."""
    q = (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)
    q = (q * q).astype(np.float32)
    bits = [int(u) for u in q.view(np.uint32)]
    nz = [u for u in bits if u]
    if not nz:
        return 0.0
    e_all = [max(u >> 23, 1) for u in nz]
    emin, emax = min(e_all), max(e_all)
    lg_d = max(0, math.ceil(math.log2(len(a)))) if len(a) > 1 else 0
    if emax >= 255 or emax - emin > 38 - lg_d:
        return None
    terms = [((u & 0x7FFFFF) | (0x800000 if u >> 23 else 0)) << (max(u >> 23, 1) - emin) for u in nz]
    half = len(terms) // 2
    S = sum(reversed(terms[half:])) + sum(terms[:half])
    assert S < 2 ** 62
    if S >= 2 ** 53:
        return None
    return math.ldexp(float(S), emin - 150)


def test_integer_sum_without_rounding_matches_sequential_sum():
    rng = np.random.default_rng(2)
    used = 0
    for trial in range(3000):
        d = int(rng.integers(1, 129))
        span = rng.uniform(0, 5)
        scale = 10.0 ** rng.uniform(-span, span, size=d)
        a = (rng.normal(size=d) * scale).astype(np.float32)
        b = (rng.normal(size=d) * scale).astype(np.float32)
        if trial % 5 == 0:
            b = (a * np.float32(1.0 + 1e-6)).astype(np.float32)
        got = no_rounding_sum(a, b)
        if got is not None:
            used += 1
            assert got == reference(a, b), (trial, got, reference(a, b))
    assert used > 1000
