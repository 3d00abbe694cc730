"""The tensor-core inference's sin/cos encoding (sincospi2 and the angle
doublings of tc_encode_pairs in sray_gb300/csrc/nrc.cu), emulated in numpy
with the kernel's own coefficients read from the source: every FP32
operation rounded as the kernel rounds it (products and sums of two FP32
values and FMAs are exact in float64 before the one rounding to FP32).  The
bounds are the ones the kernel's comments state: the base band within 8e-8
of sin(pi t) and cos(pi t), and after the three doublings 0.011 % of the
features rounding to another BF16 value than the exact ones'."""
import os
import re

import numpy as np

SRC = os.path.join(os.path.dirname(__file__), "..", "sray_gb300", "csrc", "nrc.cu")


def r32(a):
    return np.asarray(a, dtype=np.float64).astype(np.float32)


def fma(a, b, c):
    return r32(np.asarray(a, np.float64) * np.asarray(b, np.float64) + np.asarray(c, np.float64))


def mul(a, b):
    return r32(np.asarray(a, np.float64) * np.asarray(b, np.float64))


def add(a, b):
    return r32(np.asarray(a, np.float64) + np.asarray(b, np.float64))


def bf16(x):
    x = np.asarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    return (((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16).astype(np.uint32).view(np.float32)


def coefficients():
    """The polynomial coefficients in sincospi2, in the order they are used."""
    src = open(SRC).read()
    body = src[src.index("void sincospi2("):]
    body = body[:body.index("quarter_turns(sn.x")]
    vals = [float(v) for v in re.findall(r"make_float2\((-?[0-9.]+(?:e-?[0-9]+)?)f, \1f\)", body)]
    # MAGIC is not a make_float2 literal; -0.5 (the reduction), then P (3 terms
    # after the first pair), then Q; 1.0 closes the cosine
    return [np.float32(v) for v in vals]


def sincospi(t, c):
    # c: -0.5, p3, p2, p1, p0(pi), q3, q2, q1, q0, 1.0
    magic = np.float32(12582912.0)
    u = add(add(t, t), magic)
    n = add(u, -magic)
    r = fma(n, c[0], t)
    z = mul(r, r)
    p = fma(z, c[1], c[2])
    p = fma(p, z, c[3])
    p = fma(p, z, c[4])
    q = fma(z, c[5], c[6])
    q = fma(q, z, c[7])
    q = fma(q, z, c[8])
    s = mul(p, r)
    co = fma(q, z, c[9])
    k = u.view(np.uint32) & 3
    so = np.where(k & 1, co, s)
    cr = np.where(k & 1, s, co)
    so = np.where(k & 2, -so, so)
    cr = np.where((k + 1) & 2, -cr, cr)
    return so, cr


def test_coefficients_found():
    c = coefficients()
    assert len(c) == 10 and c[0] == np.float32(-0.5) and c[9] == np.float32(1.0)
    assert abs(float(c[4]) - np.pi) < 1e-6


def test_base_band_error():
    c = coefficients()
    t = np.linspace(-300.0, 300.0, 2000001).astype(np.float32)
    s, co = sincospi(t, c)
    a = np.pi * t.astype(np.float64)
    assert np.max(np.abs(s - np.sin(a))) < 8e-8
    assert np.max(np.abs(co - np.cos(a))) < 8e-8


def test_doubled_bands_round_like_exact_features():
    c = coefficients()
    rng = np.random.default_rng(5)
    x = np.concatenate([rng.uniform(0, 1, 200000), rng.uniform(-1, 1, 200000)]).astype(np.float32)
    flips = total = 0
    for k in range(3):
        s, co = sincospi(mul(x, np.float32(2.0 ** (4 * k))), c)
        for b in range(4):
            a = np.pi * (2.0 ** (4 * k + b)) * x.astype(np.float64)
            for got, want in ((s, np.sin(a)), (co, np.cos(a))):
                flips += np.count_nonzero(bf16(got) != bf16(r32(want)))
                total += got.size
            m = mul(s, np.float32(-2.0))
            s2 = mul(add(s, s), co)
            co = fma(m, s, np.float32(1.0))
            s = s2
    assert flips / total < 1.5e-4, flips / total
