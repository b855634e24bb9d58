"""The mixed form's arithmetic restated in numpy (CPU): the exact-slice BF16 products of the
tensor-core step and Dyson kernels (slice4f, issue_product's 10 slice pairs on three
accumulation levels, sum3) and the float powers z^j of the mixed Fave (z_pow_f).  These pin
the precision the kernels rely on: ~sqrt(K) 2^-32 per element of a product of K terms (two
orders of magnitude below an FP32 product's error) and a few float ulp per power."""
import numpy as np

F32 = np.float32


def fma32(a, b, c):
    """fmaf: the float32 rounding of a*b + c (float32 products are exact in float64)."""
    return (np.float64(a) * np.float64(b) + np.float64(c)).astype(F32)


def slice4f(hi, lo):
    """Four slices at natural scale, x = 2^-8 (q0 + q1 + q2 + q3), as the kernels store them
    (q0 an integer, q_j an integer times 2^-8j: exact in BF16)."""
    q0 = np.rint(hi.astype(np.float64) * 256.0).astype(F32)
    d0 = fma32(hi, F32(256), -q0)
    q1 = np.rint(fma32(lo, F32(65536), d0 * F32(256)))
    d1 = fma32(d0, F32(256), -q1)
    q2 = np.rint(fma32(lo, F32(16777216), d1 * F32(256)))
    d2 = fma32(d1, F32(256), -q2)
    q3 = np.rint(fma32(lo, F32(4294967296), d2 * F32(256)))
    return [q0, q1 * F32(2.0**-8), q2 * F32(2.0**-16), q3 * F32(2.0**-24)]


def bf16_exact(x):
    """True when every value is a BF16 number (8 significant bits)."""
    m, _ = np.frexp(x.astype(np.float64))
    return np.all(np.abs(m * 256.0 - np.rint(m * 256.0)) == 0)


def f32_sum(products):
    """FP32 accumulation, one rounding per added product (sequential along K)."""
    acc = np.zeros(products.shape[:-1], dtype=F32)
    for k in range(products.shape[-1]):
        acc = (acc + products[..., k].astype(F32)).astype(F32)
    return acc


def sum3(a, b, c):
    """(hi, lo) of a + b + c: two two-sums, as tc::sum3."""
    s = (a + b).astype(F32)
    bb = (s - a).astype(F32)
    e = ((a - (s - bb)) + (b - bb)).astype(F32)
    s2 = (s + c).astype(F32)
    bb = (s2 - s).astype(F32)
    e = (e + ((s - (s2 - bb)) + (c - bb))).astype(F32)
    h = (s2 + e).astype(F32)
    return h, (e - (h - s2)).astype(F32)


def slice_product(xa, xb):
    """C = A B^T the way issue_product + the epilogue form it: pairs (i, j) with i + j <= 3,
    levels 0, 1 and 2+3 accumulated in FP32, sum3, scaled by 2^-16."""
    ha, la = xa.astype(F32), (xa - xa.astype(F32).astype(np.float64)).astype(F32)
    hb, lb = xb.astype(F32), (xb - xb.astype(F32).astype(np.float64)).astype(F32)
    qa, qb = slice4f(ha, la), slice4f(hb, lb)
    for q in qa + qb:
        assert bf16_exact(q)
    lev = [None, None, None]
    for i in range(4):
        for j in range(4):
            if i + j > 3:
                continue
            p = qa[i][:, None, :].astype(np.float64) * qb[j][None, :, :].astype(np.float64)  # exact
            L = min(i + j, 2)
            lev[L] = p if lev[L] is None else np.concatenate([lev[L], p], axis=-1)
    acc = [f32_sum(v) for v in lev]
    h, l = sum3(*acc)
    return (h.astype(np.float64) + l.astype(np.float64)) * 2.0**-16


def test_exact_slice_products_are_far_below_fp32_error():
    rng = np.random.default_rng(3)
    for b in (40, 56, 70):
        q, _ = np.linalg.qr(rng.standard_normal((b, b)))  # entries <= 1, as the kernels' operands
        r, _ = np.linalg.qr(rng.standard_normal((b, b)))
        exact = q @ r.T
        got = slice_product(q, r)
        err = np.max(np.abs(got - exact))
        f32 = (q.astype(F32) @ r.T.astype(F32)).astype(np.float64)
        err32 = np.max(np.abs(f32 - exact))
        # the dropped pairs (i + j >= 4) are ~2^-32 each, summed over K with random signs
        assert err <= 2 * np.sqrt(b) * 2.0**-32, (b, err)
        assert err * 100 < err32, (b, err, err32)


def test_slice_levels_zero_and_one_are_exact_in_fp32():
    """The products of the level-0 and level-1 pairs are integers times 2^-8l whose sums stay
    below 2^24 units for K <= 80: FP32 accumulates them exactly."""
    rng = np.random.default_rng(4)
    x = rng.uniform(-1, 1, (8, 80))
    h, l = x.astype(F32), (x - x.astype(F32).astype(np.float64)).astype(F32)
    q = slice4f(h, l)
    p0 = q[0][:, None, :].astype(np.float64) * q[0][None, :, :].astype(np.float64)
    np.testing.assert_array_equal(f32_sum(p0).astype(np.float64), p0.sum(axis=-1))
    p1 = np.concatenate([q[0][:, None, :].astype(np.float64) * q[1][None, :, :].astype(np.float64),
                         q[1][:, None, :].astype(np.float64) * q[0][None, :, :].astype(np.float64)], axis=-1)
    np.testing.assert_array_equal(f32_sum(p1).astype(np.float64), p1.sum(axis=-1))


def z_pow_f(a, bh, bl, j):
    """z^j for z = e^{a + i b}, b = bh + bl (floats), as the mixed Fave computes it."""
    P1, P2, P3 = F32(6.28125), F32(0.0019353071693331003), F32(1.0253131677018246e-11)
    jf = F32(j)
    p = (jf * bh).astype(F32)
    pe = fma32(jf, bh, -p)
    corr = fma32(jf, bl, pe)
    k = np.rint((p * F32(0.15915494)).astype(F32))
    r = fma32(-k, P1, p)
    r = fma32(-k, P2, r)
    r = (fma32(-k, P3, r) + corr).astype(F32)
    sn, cs = np.sin(r.astype(np.float64)).astype(F32), np.cos(r.astype(np.float64)).astype(F32)  # sincosf, ~1 ulp
    m = np.exp((jf * a).astype(F32).astype(np.float64)).astype(F32)
    return (m * cs).astype(F32), (m * sn).astype(F32)


def test_float_powers_of_z_within_a_few_ulp():
    rng = np.random.default_rng(5)
    b = rng.uniform(-2 * np.pi, 2 * np.pi, 4000)  # a difference of two principal arguments
    a = rng.uniform(-1e-3, 0, 4000)
    bh = b.astype(F32)
    bl = (b - bh.astype(np.float64)).astype(F32)
    af = a.astype(F32)
    worst = 0.0
    for j in (1, 2, 7, 21, 64):
        re, im = z_pow_f(af, bh, bl, j)
        z = np.exp(j * (af.astype(np.float64) + 1j * b))
        err = np.abs((re.astype(np.float64) + 1j * im.astype(np.float64)) - z) / np.abs(z)
        worst = max(worst, float(err.max()))
    assert worst < 8 * 2.0**-24, worst
