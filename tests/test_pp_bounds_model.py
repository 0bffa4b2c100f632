"""Model check of the k-means++ update's skip tests (smartcore_gb300/csrc/
exact.cu: pp_seed_gaps, pp_far32 and the BF16 bound of pp_draw_kernel): a row
the tests settle must keep its distance under the reference's own update
(kmeans.rs:368-379: `dist < d[i]`, dist = Euclidian::squared_distance with
f32 terms summed in f64).  Directed f32 roundings are modelled exactly from
f64 values (every f32 operation here is exact in f64 before its rounding).
Points are drawn near the boundary of each test so that it is exercised."""
import numpy as np

F32_MAX = np.float32(np.finfo(np.float32).max)


def ref_sqdist(a, b):
    """euclidian.rs:56-63: r = a - b and r * r in f32, summed in f64 in order."""
    r = (a.astype(np.float32) - b.astype(np.float32)).astype(np.float32)
    q = (r * r).astype(np.float32).astype(np.float64)
    s = 0.0
    for t in q:
        s += float(t)
    return s


def rd(v):
    """f64 value rounded down to f32."""
    f = np.float32(v)
    return f if float(f) <= v else np.nextafter(f, np.float32(-np.inf))


def ru(v):
    f = np.float32(v)
    return f if float(f) >= v else np.nextafter(f, np.float32(np.inf))


def gap_lo(xp, xa):
    """pp_seed_gaps for f32 rows (one lane per 32 features, then a tree)."""
    d = len(xp)
    g = (xp - xa).astype(np.float32)
    sq = (g * g).astype(np.float32)
    lanes = [np.float32(0)] * 32
    for t in range(d):
        lanes[t % 32] = np.float32(lanes[t % 32] + sq[t])
    while len(lanes) > 1:
        half = len(lanes) // 2
        lanes = [np.float32(lanes[i] + lanes[i + half]) for i in range(half)]
    s = lanes[0]
    rel = np.float32(1.0 - (d + 10) * 2.0 ** -23)
    lo = rd(float(rd(float(s) - d * 2.0 ** -149)) * float(rel))
    return max(np.float32(0), lo)


def far32(cc, d32, d):
    mul = np.float32(4.0 * (1.0 + 3.0 * 2.0 ** -22))
    a = np.float32(d * 2.0 ** -140)
    return float(cc) >= float(ru(float(mul) * float(ru(float(d32) + float(a)))))


def bf16_keep(x, c, d32):
    """The BF16 bound: x_h = x rounded to BF16; keep when (1 - eta) r_lo^2 - A >= d32."""
    d = len(x)
    u = x.astype(np.float32).view(np.uint32).astype(np.uint64)
    # round to nearest even BF16 (the split's __float2bfloat16_rn)
    rnd = ((u >> 16) & 1) + 0x7FFF
    xh = (((u + rnd) >> 16) << 16).astype(np.uint32).view(np.float32)
    r = (xh - c).astype(np.float32)
    sh = np.float32(0)
    for t in (r * r).astype(np.float32):
        sh = np.float32(sh + t)
    rel = np.float32(1.0 - (d + 8) * 2.0 ** -23)
    L = max(np.float32(0), rd(float(rd(float(sh) - d * 2.0 ** -147)) * float(rel)))
    xn = ru(np.sqrt(float(np.dot(x.astype(np.float64), x.astype(np.float64))))) + np.float32(0)
    xn = np.nextafter(xn, np.float32(np.inf))  # xnrm: one more ulp, as the prep kernel stores it
    sub = ru(float(ru(float(xn) * 2.0 ** -8)) + float(np.float32(np.sqrt(d) * 2.0 ** -133)))
    rlo = rd(float(rd(np.sqrt(float(L)))) - float(sub))
    if not rlo > 0:
        return False
    v = rd(float(rd(float(rd(float(rlo) * float(rlo))) * float(np.float32(1 - 2.0 ** -22)))) - d * 2.0 ** -140)
    return float(v) >= float(d32)


def test_far_and_bf16_tests_never_skip_an_update():
    rng = np.random.default_rng(11)
    checked_far = checked_bf16 = 0
    for trial in range(3000):
        d = int(rng.choice([1, 3, 8, 17, 32, 64]))
        scale = 10.0 ** rng.uniform(-3, 3)
        ca = (rng.normal(size=d) * scale).astype(np.float32)
        x = (ca + rng.normal(size=d) * scale * rng.uniform(0.01, 1.0)).astype(np.float32)
        D = ref_sqdist(x, ca)
        d32 = ru(D)
        # a new seed about twice the row's distance away from its seed: the far test's boundary
        direction = rng.normal(size=d)
        direction /= np.linalg.norm(direction)
        cn = (ca + direction * np.sqrt(D) * rng.uniform(1.95, 2.05)).astype(np.float32)
        D_new = ref_sqdist(x, cn)
        if far32(gap_lo(cn, ca), d32, d):
            checked_far += 1
            assert not D_new < D, (trial, D, D_new)
        # the BF16 bound against a seed at about the row's own distance
        cm = (x + direction * np.sqrt(D) * rng.uniform(0.98, 1.3)).astype(np.float32)
        if bf16_keep(x, cm, d32):
            checked_bf16 += 1
            assert not ref_sqdist(x, cm) < D, (trial,)
    assert checked_far > 200 and checked_bf16 > 200
