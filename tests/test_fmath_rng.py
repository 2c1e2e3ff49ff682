"""The shared elementary functions (ne_fmath.h) and random numbers (ne_rng.h) on the host.

ne_fmath replaces libm in both the oracle and the GPU kernels; here its host build is
checked against double-precision numpy within stated ulp bounds. The generator is checked
against the published Philox-4x32-10 known-answer vectors (Salmon et al., SC 2011,
Random123 distribution) and for range and uniformity. Bit equality of the device copies
is checked in test_gpu_parity.py.
"""
import numpy as np
import pytest


def ulp_err(got, ref):
    got = got.astype(np.float64)
    ref32 = ref.astype(np.float32)
    spacing = np.abs(np.spacing(ref32).astype(np.float64))
    spacing = np.maximum(spacing, np.finfo(np.float32).smallest_subnormal)
    return np.abs(got - ref) / spacing


@pytest.mark.parametrize("fn,gen,ref,max_ulp", [
    (0, lambda r: np.exp(r.uniform(-80, 80, 200000)), np.log, 2.0),
    (0, lambda r: 1.0 - r.random(200000) * (1 - 2 ** -24), np.log, 2.0),  # log(1 - u) of the tracking steps
    (1, lambda r: r.uniform(-80, 80, 200000), np.exp, 3.0),
    (2, lambda r: r.uniform(-7, 7, 200000), np.sin, 2.0),
    (3, lambda r: r.uniform(-7, 7, 200000), np.cos, 2.0),
    (4, lambda r: r.uniform(-1, 1, 200000), np.arccos, 2.0),
])
def test_fmath_accuracy(oracle_lib, fn, gen, ref, max_ulp):
    x = gen(np.random.default_rng(fn)).astype(np.float32)
    got = oracle_lib.fmath(fn, x)
    want = ref(x.astype(np.float64))
    if fn in (2, 3):
        # absolute error near zeros of sin/cos: compare against 2^-24 of the argument range
        err = np.abs(got.astype(np.float64) - want)
        assert err.max() < 2e-7, err.max()
    else:
        e = ulp_err(got, want)
        assert e.max() <= max_ulp, (fn, e.max(), x[np.argmax(e)])


def test_atan2_accuracy(oracle_lib):
    rng = np.random.default_rng(6)
    n = 200000
    yx = np.empty(2 * n, np.float32)
    yx[0::2] = rng.normal(size=n) * np.exp(rng.uniform(-8, 8, n))
    yx[1::2] = rng.normal(size=n) * np.exp(rng.uniform(-8, 8, n))
    got = oracle_lib.fmath(6, yx)[0::2]
    want = np.arctan2(yx[0::2].astype(np.float64), yx[1::2].astype(np.float64))
    e = ulp_err(got, want)
    assert e.max() <= 3.0, (e.max(), yx[2 * np.argmax(e)], yx[2 * np.argmax(e) + 1])


def test_atan2_quadrants_and_zeros(oracle_lib):
    y = np.array([0.0, -0.0, 0.0, -0.0, 1.0, -1.0, 1.0, -1.0, np.inf, np.inf, -np.inf, 2.0, 3.0], np.float32)
    x = np.array([0.0, 0.0, -0.0, -0.0, 0.0, 0.0, -1.0, -1.0, np.inf, -np.inf, 5.0, np.inf, -np.inf], np.float32)
    yx = np.empty(2 * len(y), np.float32)
    yx[0::2], yx[1::2] = y, x
    got = oracle_lib.fmath(6, yx)[0::2].astype(np.float64)
    want = np.arctan2(y.astype(np.float64), x.astype(np.float64))
    assert np.all(np.abs(got - want) <= 4e-7), (got, want)
    assert np.array_equal(np.signbit(got), np.signbit(want))


def test_log1m_draw_equals_log_on_every_draw(oracle_lib):
    """The tracking steps' log(1 - u) without log's special cases gives log's bits for all
    2^24 values a draw can take."""
    u = (np.arange(1 << 24, dtype=np.float64) * 2.0 ** -24).astype(np.float32)
    fast = oracle_lib.fmath(7, u)
    ref = oracle_lib.fmath(0, (np.float32(1) - u).astype(np.float32))
    assert np.array_equal(fast.view(np.uint32), ref.view(np.uint32))


def test_fmath_special_values(oracle_lib):
    log = oracle_lib.fmath(0, np.array([0.0, -1.0, np.inf, np.nan, 1.0, 2.0 ** -149], np.float32))
    assert log[0] == -np.inf and np.isnan(log[1]) and log[2] == np.inf and np.isnan(log[3]) and log[4] == 0.0
    assert abs(log[5] - np.log(2.0 ** -149)) < 1e-4
    ex = oracle_lib.fmath(1, np.array([0.0, 100.0, -200.0, -np.inf], np.float32))
    assert ex[0] == 1.0 and ex[1] == np.inf and ex[2] == 0.0 and ex[3] == 0.0
    ac = oracle_lib.fmath(4, np.array([1.0, -1.0, 0.0, 1.5], np.float32))
    assert ac[0] == 0.0 and abs(ac[1] - np.pi) < 1e-6 and abs(ac[2] - np.pi / 2) < 1e-7 and np.isnan(ac[3])
    p5 = oracle_lib.fmath(5, np.array([0.5, 1.0, 0.0, 2.0], np.float32))
    assert list(p5) == [0.03125, 1.0, 0.0, 32.0]


def test_philox_known_answers(oracle_lib):
    kat = [
        ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
        ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
        ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
         [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
    ]
    for ctr, key, want in kat:
        assert oracle_lib.philox(ctr, key) == want


def test_u01_range_and_uniformity(oracle_lib):
    n = 400000
    keys = np.stack([np.arange(n, dtype=np.uint32) % 1024, np.arange(n, dtype=np.uint32) // 1024], 1)
    dims = (np.arange(n, dtype=np.uint32) * 7) % 97
    u = oracle_lib.rng(0x4E415256, keys, dims)
    assert u.min() >= 0.0 and u.max() < 1.0
    hist, _ = np.histogram(u, bins=64, range=(0, 1))
    chi2 = ((hist - n / 64) ** 2 / (n / 64)).sum()
    assert chi2 < 130  # 63 degrees of freedom, p ~ 1e-6
    # consecutive draws of one path are uncorrelated
    k1 = np.zeros((n, 2), np.uint32)
    d = np.arange(n, dtype=np.uint32)
    s = oracle_lib.rng(1, k1, d)
    assert abs(np.corrcoef(s[:-1], s[1:])[0, 1]) < 0.01


def test_u01_is_a_function_of_the_key(oracle_lib):
    keys = np.array([[5, 3], [5, 3], [5, 4], [6, 3]], np.uint32)
    dims = np.array([9, 9, 9, 9], np.uint32)
    u = oracle_lib.rng(12, keys, dims)
    assert u[0] == u[1] and u[0] != u[2] and u[0] != u[3]
    assert oracle_lib.rng(13, keys, dims)[0] != u[0]
