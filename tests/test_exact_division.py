"""The division (div_by) and the integer-pipe multiply (mul_int) of fdf_exact.cuh restated step by
step in Python.  The division: FP32 steps in numpy float32 (round to nearest), integer steps in
Python integers with the kernel's 64-bit wrap, the reciprocal perturbed by up to 2^-22 (the
approximate reciprocal's 2 ulps) before its Newton step.  Checks the bounds the kernel relies
on (|Q1 - Q| < 2^11, |R1| < 2^65, R2 in (-mb, mb), the 32-bit top word of R1) and that the
result is Python's correctly rounded quotient.  The multiply: the 128-bit significand product
and its rounding, against Python's product, with short significands for exact ties.  The
conversions: double -> float and the (hi, lo) split by rounding the bit pattern, against
numpy's float32 rounding, and the split's 2^-48 |x| bound."""
import random
import struct
from fractions import Fraction

import numpy as np
import pytest

M64 = (1 << 64) - 1
F = np.float32


def _ub(x):
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _fb(u):
    return struct.unpack("<d", struct.pack("<Q", u & M64))[0]


def _u2f(u):
    return np.frombuffer(struct.pack("<I", u & 0xFFFFFFFF), dtype=np.float32)[0]


def _f2u(f):
    return struct.unpack("<I", np.float32(f).tobytes())[0]


def _fma(a, b, c):
    """fl32(a * b + c) with a single rounding."""
    v = Fraction(float(a)) * Fraction(float(b)) + Fraction(float(c))
    r = np.float32(float(v))
    cands = [r, np.nextafter(r, F(np.inf)), np.nextafter(r, F(-np.inf))]
    return min(cands, key=lambda c: (abs(Fraction(float(c)) - v), _f2u(c) & 1))


def _parts(m):
    hi = _u2f(0x3F800000 | ((m >> 29) & 0x7FFFFF))
    lo = F(F(_u2f(0x4B000000 | ((m >> 6) & 0x7FFFFF)) - F(8388608.0)) * F(2.0 ** -46))
    return hi, lo


def div_by(a, b, rcp_err):
    ua, ub = _ub(a), _ub(b)
    ea, eb = (ua >> 52) & 0x7FF, (ub >> 52) & 0x7FF
    de = ea - eb
    assert 0 < ea < 0x7FF and 0 < eb < 0x7FF and -1021 <= de <= 1021
    ma = (ua & ((1 << 52) - 1)) | (1 << 52)
    mb = (ub & ((1 << 52) - 1)) | (1 << 52)
    fbh, fbl = _parts(mb)
    r0 = F(float(F(1.0) / fbh) * (1.0 + rcp_err))
    r = _fma(r0, _fma(-fbh, r0, F(1.0)), r0)
    fah, fal = _parts(ma)
    qh = F(fah * r)
    p = F(qh * fbh)
    pe = _fma(qh, fbh, -p)
    rem = F(F(F(fah - p) - pe) + _fma(-qh, fbl, fal))
    ql = F(rem * r)
    ge = 1 if ma >= mb else 0
    s = 54 - ge
    qb = _f2u(qh)
    sh = s - 23 + ((qb >> 23) & 0xFF) - 127
    assert 29 <= sh <= 32
    x = F(ql * F(2.0 ** (42 + 1 - ge)))
    assert abs(float(x)) < 2 ** 31
    Q1 = (((qb & 0x7FFFFF) | 0x800000) << sh) + (int(np.rint(x)) << 11)
    Q = (ma << s) // mb
    assert abs(Q1 - Q) < 2 ** 11, (a, b, Q1 - Q)
    n_lo, n_hi = (ma << s) & M64, ma >> (64 - s)
    prod = Q1 * mb
    p_lo, p_hi = prod & M64, (prod >> 64) & M64
    r_lo = (n_lo - p_lo) & M64
    r_hi = (n_hi - p_hi - (1 if n_lo < p_lo else 0)) & M64
    R1 = (ma << s) - Q1 * mb
    assert abs(R1) < 2 ** 65
    t = ((r_hi << 29) | (r_lo >> 35)) & 0xFFFFFFFF
    t = t - (1 << 32) if t >= 1 << 31 else t
    assert t == R1 >> 35
    dl = int(np.rint(F(F(F(t) * r) * F(2.0 ** -17))))
    Qc = Q1 + dl
    r2 = (r_lo - ((dl * mb) & M64)) & M64
    r2 = r2 - (1 << 64) if r2 >= 1 << 63 else r2
    assert r2 == R1 - dl * mb and -mb < r2 < mb
    Qc -= 1 if r2 < 0 else 0
    assert Qc == Q
    qr = (Qc + 1) >> 1
    return _fb(((ua ^ ub) & (1 << 63)) | (((de + 1021 + ge) << 52) + qr))


def _cases(n, seed):
    rng = random.Random(seed)
    ext = [(1 << 53) - 1, 1 << 52, (1 << 52) + 1, (1 << 53) - 2]
    for i in range(n):
        a = rng.uniform(1, 2) * 2.0 ** rng.randint(-80, 80) * rng.choice([1, -1])
        b = rng.uniform(1, 2) * 2.0 ** rng.randint(-80, 80) * rng.choice([1, -1])
        if i % 3 == 0:
            b = 1.0 + rng.randint(-8, 8) * 2.0 ** -52          # a trilinear weight sum
        if i % 4 == 0:
            a = rng.choice(ext) * 2.0 ** rng.randint(-60, -40)
        if i % 5 == 0:
            b = rng.choice(ext) * 2.0 ** rng.randint(-60, -40)
        if i % 7 == 0:
            b = float(rng.randint(3, 1000))                  # a particle count
        yield a, b, rng.uniform(-2.0 ** -22, 2.0 ** -22)


@pytest.mark.parametrize("seed", [11, 12])
def test_division_restatement_is_correctly_rounded(seed):
    for a, b, e in _cases(4000, seed):
        q = div_by(a, b, e)
        assert _ub(q) == _ub(a / b), (a, b)


def test_division_extreme_reciprocal_errors():
    for a in (1.0, 2.0 - 2.0 ** -52, 1.0 + 2.0 ** -52, 1.5, 0.1, 1e-14, 1 / 3):
        for b in (1.0, 2.0 - 2.0 ** -52, 1.0 + 2.0 ** -52, 3.0, 0.1, 2e-14, 7.0):
            for e in (2.0 ** -22, -(2.0 ** -22), 0.0):
                assert _ub(div_by(a, b, e)) == _ub(a / b)


# ---- mul_int: the 53 x 53-bit significand product, exact in 128 bits, rounded to nearest even


def mul_int(a, b):
    """fdf_exact.cuh mul_int step by step (fast path: normal operands, normal product; zeros)."""
    ua, ub = _ub(a), _ub(b)
    sign = (ua ^ ub) & (1 << 63)
    ea, eb = (ua >> 52) & 0x7FF, (ub >> 52) & 0x7FF
    e = ea + eb - 1023
    if ea == 0 or eb == 0 or ea == 0x7FF or eb == 0x7FF or e < 1 or e > 2044:
        if ((ua & ((1 << 63) - 1)) == 0 and eb != 0x7FF) or ((ub & ((1 << 63) - 1)) == 0 and ea != 0x7FF):
            return _fb(sign)
        return None   # the hardware multiply
    ma = (ua & ((1 << 52) - 1)) | (1 << 52)
    mb = (ub & ((1 << 52) - 1)) | (1 << 52)
    prod = ma * mb
    lo, hi = prod & M64, prod >> 64
    top = (hi >> 41) & 1
    sh = 52 + top
    mant = ((hi << (64 - sh)) & M64) | (lo >> sh)
    assert (1 << 52) <= mant < (1 << 53)
    rem, half = lo & ((1 << sh) - 1), 1 << (sh - 1)
    up = 1 if (rem > half or (rem == half and (mant & 1))) else 0
    return _fb(sign | (((e - 1 + top) << 52) + mant + up))


def _short(x, rng):
    m = rng.randint(1, 53)
    keep = ~((1 << (53 - m)) - 1)
    return _fb(_ub(x) & (0xFFF0000000000000 | (keep & ((1 << 52) - 1))))


def test_mul_int_restatement_is_correctly_rounded():
    rng = random.Random(21)
    ties = 0
    for i in range(60000):
        a = rng.uniform(1, 2) * 2.0 ** rng.randint(-300, 300) * rng.choice([1, -1])
        b = rng.uniform(1, 2) * 2.0 ** rng.randint(-300, 300) * rng.choice([1, -1])
        if i % 2:
            a, b = _short(a, rng), _short(b, rng)   # short significands: exact products and ties
        if i % 11 == 0:
            b = 0.0 if i % 22 == 0 else -0.0
        q = mul_int(a, b)
        if q is None:
            continue
        want = a * b
        assert _ub(q) == _ub(want), (a, b, q, want)
        ua, ub = _ub(a), _ub(b)
        if a != 0 and b != 0:
            p = ((ua & ((1 << 52) - 1)) | (1 << 52)) * ((ub & ((1 << 52) - 1)) | (1 << 52))
            sh = 52 + ((p >> 105) & 1)
            ties += (p & ((1 << sh) - 1)) == 1 << (sh - 1)
    assert ties > 100   # the exact-half case is exercised


# ---- d2f_rn and split_rn: double -> float by rounding the bit pattern, and the (hi, lo) split


def d2f_rn(x):
    """fdf_exact.cuh d2f_rn, fast path ([2^-126, FLT_MAX) in magnitude); None for the rest."""
    b = _ub(x)
    mag = b & ((1 << 63) - 1)
    if not (0x3810000000000000 <= mag < 0x47EFFFFFE0000000):
        return None
    r = mag + 0x0FFFFFFF + ((mag >> 29) & 1)
    f = ((r >> 29) - ((1023 - 127) << 23)) & 0xFFFFFFFF
    return struct.unpack("<f", struct.pack("<I", f | ((b >> 32) & 0x80000000)))[0]


def split_rn(x):
    """fdf_exact.cuh split_rn, fast path (2^-74 <= |x| < 2^127); None for the rest."""
    b = _ub(x)
    mag = b & ((1 << 63) - 1)
    sgn = (b >> 32) & 0x80000000
    if not (0x3B50000000000000 <= mag < 0x47E0000000000000):
        return None
    r = mag + 0x0FFFFFFF + ((mag >> 29) & 1)
    hmag = r & ~0x1FFFFFFF
    hi = struct.unpack("<f", struct.pack("<I", (((r >> 29) - ((1023 - 127) << 23)) & 0xFFFFFFFF) | sgn))[0]
    units = mag - hmag
    assert abs(units) <= 1 << 28
    ulp = np.float32(2.0 ** ((mag >> 52) - 1075))
    lo = np.float32(np.float32(units) * ulp)          # one rounding of the exact integer, then exact scaling
    if units != 0 and sgn:
        lo = -lo
    return np.float32(hi), lo


def test_conversions_restatement_match_numpy():
    rng = random.Random(33)
    for i in range(40000):
        x = rng.uniform(1, 2) * 2.0 ** rng.randint(-140, 140) * rng.choice([1, -1])
        if i % 3 == 0:
            x = _short(x, rng)
        f = d2f_rn(x)
        if f is not None:
            assert struct.pack("<f", f) == np.float32(x).tobytes(), x
        sp = split_rn(x)
        if sp is not None:
            h = np.float32(x)
            lo = np.float32(x - float(h))   # x - h is exact in double
            assert sp[0].tobytes() == h.tobytes() and sp[1].tobytes() == lo.tobytes(), x
            assert abs(float(sp[0]) + float(sp[1]) - x) <= 2.0 ** -48 * abs(x)
