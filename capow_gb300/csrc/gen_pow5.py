"""Writes pow5_table.h: for each decimal exponent q in [-342, 308], the 128-bit significand F of 5^q,
F = floor(5^q * 2^(127 - floor(log2 5^q))), so that 2^127 <= F < 2^128 (exact for 0 <= q <= 55,
truncated otherwise), as two uint64 words. Used by the catalogue reader's Eisel-Lemire path.

    python capow_gb300/csrc/gen_pow5.py > capow_gb300/csrc/pow5_table.h
"""
from fractions import Fraction

QMIN, QMAX = -342, 308


def floor_log2(fr: Fraction) -> int:
    n, d = fr.numerator, fr.denominator
    e = n.bit_length() - d.bit_length()
    if Fraction(n, d) < Fraction(2) ** e:
        e -= 1
    return e


def main() -> None:
    print("/* Generated by gen_pow5.py: 128-bit significands F of 5^q, q in [-342, 308],")
    print(" * F = floor(5^q 2^(127 - floor(log2 5^q))) in [2^127, 2^128), {high, low} words. */")
    print("#pragma once")
    print("#include <stdint.h>")
    print(f"#define POW5_QMIN ({QMIN})")
    print(f"#define POW5_QMAX {QMAX}")
    print("static const uint64_t pow5_128[%d][2] = {" % (QMAX - QMIN + 1))
    for q in range(QMIN, QMAX + 1):
        v = Fraction(5) ** q
        e = floor_log2(v)
        f = v * Fraction(2) ** (127 - e)
        F = f.numerator // f.denominator
        assert 2 ** 127 <= F < 2 ** 128
        print("    {0x%016xULL, 0x%016xULL}," % (F >> 64, F & (2 ** 64 - 1)))
    print("};")


if __name__ == "__main__":
    main()
