"""The integer arithmetic of the FP64 deterministic deposit, restated bit for
bit from its device functions (`puffin_gb300/csrc/rk4_fp64.cu`:
`mul_to_fix`, the exact product of a weight and a source term on the
128-bit fixed-point grid, and `fix_to_double`, the nearest double of a
128-bit sum scaled by 2^-E) and checked against exact rational arithmetic.
The GPU parity tests check the kernels that use them against the oracle;
these tests pin the two algorithms themselves, on the edge cases too
(overflow bound, truncation toward zero, ties to even, carries into a new
leading bit)."""
import random
import struct
from fractions import Fraction

M64 = (1 << 64) - 1


def _bits(v):
    return struct.unpack("<Q", struct.pack("<d", v))[0]


def _operand(v):
    """fix_operand: significand with its hidden bit, biased exponent, sign."""
    b = _bits(v)
    return (b & 0xFFFFFFFFFFFFF) | 0x10000000000000, (b >> 52) & 0x7FF, b >> 63


def mul_to_fix(x, y, e_scale, maxexp):
    (mx, ex, nx), (my, ey, ny) = x, y
    if ex == 0x7FF or ey == 0x7FF:
        return False, 0, 0
    if ex == 0 or ey == 0:
        return True, 0, 0
    prod = mx * my
    plo, phi = prod & M64, prod >> 64
    sh = ex + ey - 2150 + e_scale
    top = 106 if (phi >> 41) else 105
    if top + sh > maxexp:
        return False, 0, 0
    lo = hi = 0
    if sh >= 0:
        hi = ((phi << sh) | (plo >> (64 - sh))) & M64 if sh else phi
        lo = (plo << sh) & M64
    else:
        r = -sh
        if r >= 106:
            return True, 0, 0
        if r < 64:
            lo = ((plo >> r) | (phi << (64 - r))) & M64
            hi = phi >> r
        else:
            lo = phi >> (r - 64)
    if nx ^ ny:
        nlo = (~lo + 1) & M64
        hi = (~hi + (1 if lo == 0 else 0)) & M64
        lo = nlo
    return True, lo, hi


def fix_to_double(lo, hi, e_scale):
    neg = hi >> 63
    if neg:
        nlo = (~lo + 1) & M64
        hi = (~hi + (1 if lo == 0 else 0)) & M64
        lo = nlo
    if hi == 0 and lo == 0:
        return 0.0
    lz = 64 - hi.bit_length() if hi else 128 - lo.bit_length()
    if lz >= 64:
        nh, nl = (lo << (lz - 64)) & M64, 0
    elif lz > 0:
        nh, nl = ((hi << lz) | (lo >> (64 - lz))) & M64, (lo << lz) & M64
    else:
        nh, nl = hi, lo
    msb = 127 - lz
    m = nh >> 11
    rb = (nh >> 10) & 1
    sticky = ((nh & 0x3FF) | nl) != 0
    if rb and (sticky or (m & 1)):
        m += 1
    if m >> 53:
        m >>= 1
        msb += 1
    be = msb - e_scale + 1023
    assert 0 < be < 2047  # the device takes its FP64 route outside this range
    d = struct.unpack("<d", struct.pack("<Q", (be << 52) | (m & ((1 << 52) - 1))))[0]
    return -d if neg else d


def _as_int(lo, hi):
    v = (hi << 64) | lo
    return v - (1 << 128) if hi >> 63 else v


def test_mul_to_fix_is_the_truncated_exact_product():
    rng = random.Random(1)
    for t in range(20000):
        e_scale, maxexp = rng.randint(60, 110), rng.randint(95, 125)
        w = rng.random() if t % 3 else rng.choice([0.0, 1.0, 0.5, rng.random() * 1e-30])
        s = rng.choice([-1, 1]) * (rng.random() + 0.5) * 2.0 ** rng.randint(-60, 30)
        ok, lo, hi = mul_to_fix(_operand(w), _operand(s), e_scale, maxexp)
        exact = Fraction(w) * Fraction(s) * Fraction(2) ** e_scale
        if ok:
            assert abs(exact) < Fraction(2) ** maxexp
            assert _as_int(lo, hi) == int(exact)  # int() truncates toward zero
        else:
            # refused only where the bound 2^(bits + shift) reaches 2^maxexp
            assert abs(exact) >= Fraction(2) ** (maxexp - 1)


def test_mul_to_fix_special_operands():
    inf, nan = float("inf"), float("nan")
    assert mul_to_fix(_operand(inf), _operand(1.0), 80, 120)[0] is False
    assert mul_to_fix(_operand(0.5), _operand(nan), 80, 120)[0] is False
    assert mul_to_fix(_operand(0.0), _operand(3.0), 80, 120) == (True, 0, 0)
    assert mul_to_fix(_operand(5e-324), _operand(3.0), 80, 120) == (True, 0, 0)  # subnormal
    ok, lo, hi = mul_to_fix(_operand(-0.75), _operand(2.0), 4, 120)
    assert ok and _as_int(lo, hi) == -24


def test_fix_to_double_rounds_to_nearest_even():
    rng = random.Random(3)
    for t in range(20000):
        nb = rng.randint(1, 126)
        v = rng.getrandbits(nb)
        if t % 5 == 0:
            v = (v >> 20) << 20 | (1 << 19)  # ties below the 53rd bit
        if t % 7 == 0:
            v = (1 << nb) - 1  # all ones: the rounding carries into a new bit
        x = rng.choice([1, -1]) * v
        e_scale = rng.randint(-50, 120)
        w = x & ((1 << 128) - 1)
        got = fix_to_double(w & M64, w >> 64, e_scale)
        want = float(Fraction(x) / Fraction(2) ** e_scale)  # correctly rounded
        assert got == want, (x, e_scale)
