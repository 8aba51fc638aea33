"""Exact binary values with MPFR's representation, in plain Python ints.

An MpVal is sign * 0.d[n-1]...d[0] * 2^exp with 64-bit limbs (least
significant first) and a precision in bits -- the layout of an mpfr_t
(src/image_info.h embeds them by value) and of the mdzgpu_mpval struct the C
ABI takes.  Values round to nearest, ties to even, like MPFR's GMP_RNDN.
"""
from __future__ import annotations

import ctypes as C
import re
from dataclasses import dataclass
from fractions import Fraction

from .native import MpValStruct


def _round_shift(num: int, den: int, shift: int) -> int:
    """round(num/den * 2^shift) to nearest, ties to even (num, den > 0)."""
    if shift >= 0:
        n, d = num << shift, den
    else:
        n, d = num, den << (-shift)
    q, r = divmod(n, d)
    if 2 * r > d or (2 * r == d and (q & 1)):
        q += 1
    return q


@dataclass(frozen=True)
class MpVal:
    sign: int          # +1 / -1
    exp: int           # value = sign * M / 2^(64 n) * 2^exp
    mant: int          # M, the n*64-bit mantissa integer (0 = zero)
    prec: int

    @property
    def nlimbs(self) -> int:
        return (self.prec + 63) // 64

    @staticmethod
    def zero(prec: int = 64) -> "MpVal":
        return MpVal(1, 0, 0, prec)

    @staticmethod
    def from_fraction(x: Fraction | int | str, prec: int) -> "MpVal":
        if isinstance(x, str):
            x = parse_number(x)
        x = Fraction(x)
        if x == 0:
            return MpVal(1, 0, 0, prec)
        sign = -1 if x < 0 else 1
        a = abs(x)
        num, den = a.numerator, a.denominator
        e = num.bit_length() - den.bit_length()   # 2^(e-1) <= a < 2^(e+1)
        if Fraction(num, den) >= Fraction(2) ** e:
            e += 1
        # a in [2^(e-1), 2^e): M_p = round(a * 2^(prec - e))
        m = _round_shift(num, den, prec - e)
        if m == 1 << prec:
            m >>= 1
            e += 1
        n = (prec + 63) // 64
        return MpVal(sign, e, m << (64 * n - prec), prec)

    @staticmethod
    def from_limbs(prec: int, sign: int, exp: int, limbs: list[int]) -> "MpVal":
        mant = 0
        for i, l in enumerate(limbs):
            mant |= int(l) << (64 * i)
        return MpVal(1 if sign >= 0 else -1, int(exp), mant, int(prec))

    def to_fraction(self) -> Fraction:
        if self.mant == 0:
            return Fraction(0)
        return self.sign * Fraction(self.mant) * Fraction(2) ** (self.exp - 64 * self.nlimbs)

    def limbs(self) -> list[int]:
        return [(self.mant >> (64 * i)) & ((1 << 64) - 1) for i in range(self.nlimbs)]

    def struct(self):
        """(MpValStruct, keepalive) for the C ABI."""
        if self.mant == 0:
            s = MpValStruct(1, 0, 0, None)
            return s, None
        arr = (C.c_uint64 * self.nlimbs)(*self.limbs())
        s = MpValStruct(self.sign, self.nlimbs, self.exp, C.cast(arr, C.POINTER(C.c_uint64)))
        return s, arr

    def hex(self) -> str:
        return hexfloat(self.to_fraction())


_HEX = re.compile(r"^([+-]?)0x([0-9a-fA-F]*)(?:\.([0-9a-fA-F]*))?p([+-]?\d+)$")


def parse_number(s: str) -> Fraction:
    """Exact value of a decimal or hex-float ("-0x1.8p-3") string."""
    s = s.strip()
    m = _HEX.match(s)
    if m:
        sign, ip, fp, ex = m.groups()
        digits = (ip or "0") + (fp or "")
        v = Fraction(int(digits, 16), 16 ** len(fp or "")) * Fraction(2) ** int(ex)
        return -v if sign == "-" else v
    return Fraction(s)


def hexfloat(x: Fraction) -> str:
    """Exact hex-float string of a dyadic rational (mpfr_set_str base 0)."""
    x = Fraction(x)
    if x == 0:
        return "0x0p+0"
    sign = "-" if x < 0 else ""
    a = abs(x)
    if a.denominator & (a.denominator - 1):
        raise ValueError("not a dyadic rational")
    k = a.denominator.bit_length() - 1     # a = num / 2^k
    num = a.numerator
    return f"{sign}0x{num:x}p-{k}" if k else f"{sign}0x{num:x}p+0"


def round_to_double(x: Fraction) -> float:
    """Round to the nearest IEEE double (ties to even): mpfr_get_d RNDN."""
    return float(Fraction(x))
