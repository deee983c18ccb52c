"""The numerical design of the split-precision paths, checked on the CPU by
emulating the kernels' fp32 / fp16 arithmetic with NumPy (the kernels
themselves are checked against FP64 on the GPU):

* the exact dominant product: every partial sum of A0.B0 over K = 128 with
  |A0| <= 127 q_A and |B0| <= 1023 q_B is an integer multiple of q_A q_B
  below 2^24, so fp32 accumulation (even truncating) is exact;
* the magic-number rounding (x + 1.5 2^23 q) - 1.5 2^23 q gives the nearest
  multiple of q;
* the driven kernel's per-step split of A(t) = Heff - c(t) mu from fp32
  hi/lo pairs in double-float arithmetic reproduces A(t) to ~2^-30 of the
  row bound (the undriven FP64 split: ~2^-29).
"""
import numpy as np

f32, f16 = np.float32, np.float16


def test_exact_dominant_product_bound():
    assert 127 * 1023 * 128 < 2 ** 24
    rng = np.random.default_rng(0)
    a0 = rng.integers(-127, 128, size=(64, 128)).astype(np.float32)
    b0 = rng.integers(-1023, 1024, size=(128, 32)).astype(np.float32)
    a0[0, :] = 127
    b0[:, 0] = 1023                      # the extreme partial sum
    acc = np.zeros((64, 32), dtype=np.float32)
    for k in range(128):                 # fp32 accumulation, one product at a time
        acc = (acc + a0[:, k:k + 1] * b0[k:k + 1, :]).astype(np.float32)
    assert np.array_equal(acc.astype(np.int64), a0.astype(np.int64) @ b0.astype(np.int64))


def test_magic_rounding_to_grid():
    rng = np.random.default_rng(1)
    for e in range(-6, 8):
        q = f32(2.0 ** e)
        magic = f32(1.5 * 2 ** 23) * q
        x = (rng.uniform(-1000, 1000, 2000) * float(q)).astype(np.float32)
        x0 = ((x + magic).astype(np.float32) - magic).astype(np.float32)
        k = x0 / q
        assert np.array_equal(k, np.round(k))                          # on the grid
        assert np.all(np.abs(x0 - x) <= q / 2)                         # nearest
        assert np.all(np.abs(x - x0) == np.abs((x.astype(np.float64) - x0.astype(np.float64))))


def _df_sub_prod(xh, xl, ch, cl, mh, ml):
    """x -= c m on fp32 pairs, as the driven kernel does (fma emulated in
    float64, where the fp32 products and sums are exact)."""
    d = np.float64
    ph = f32(ch * mh)
    pe = f32(d(ch) * d(mh) - d(ph))
    pl = f32(d(ch) * d(ml) + d(f32(d(cl) * d(mh) + d(pe))))
    sm = f32(xh - ph)
    bb = f32(sm - xh)
    er = f32(f32(xh - f32(sm - bb)) + f32(-ph - bb))
    return sm, f32(f32(xl - pl) + er)


def _split_a32(xh, xl, magic, qmax):
    v0 = f32(f32(xh + magic) - magic)
    v0 = f32(min(max(v0, -qmax), qmax))
    r = f32(f32(xh - v0) + xl)
    a1 = f16(r)
    a2 = f16(f32(r - f32(a1)))
    return float(f16(v0)), float(a1), float(a2), float(v0)


def test_driven_split_reconstruction():
    rng = np.random.default_rng(2)
    worst = 0.0
    sa = 2.0 ** 14
    for _ in range(3000):
        H, mu = rng.normal(0, 0.1), rng.normal(1, 0.1)
        c = 0.01 * np.cos(rng.uniform(0, 10))
        x = H - c * mu
        bound = (abs(H) + 0.01 * abs(mu)) * sa * rng.uniform(1, 3)   # the row's bound >= |x|
        e = int(np.floor(np.log2(bound)))
        q = 2.0 ** (e - 6)
        magic, qmax = f32(1.5 * 2 ** (e + 17)), f32(127 * q)
        hh, ch, mh = f32(H), f32(c), f32(mu)
        hl, cl, ml = f32(H - float(hh)), f32(c - float(ch)), f32(mu - float(mh))
        xh, xl = _df_sub_prod(hh, hl, ch, cl, mh, ml)
        a0, a1, a2, v0 = _split_a32(f32(xh * f32(sa)), f32(xl * f32(sa)), magic, qmax)
        assert a0 == v0 and abs(a0) <= 127 * q and a0 / q == round(a0 / q)   # fixed-point A0, exact in fp16
        worst = max(worst, abs((a0 + a1 + a2) / sa - x) / (bound / sa))
    assert worst < 2.0 ** -29, worst
