"""Writes exp2_table.cuh, the tables of the fixed-point exp of the Gaussian epilogues:
2^(-j/256), j = 0..255, rounded to integers in units of 2^-63; 256/ln2 in units of
2^-54; ln2/256 in units of 2^-116 (two 64-bit words).  All computed in 60-digit
decimal arithmetic.  Run once; the output is committed.

    python qml_gb300/csrc/gen_exp2_table.py > qml_gb300/csrc/exp2_table.cuh
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
TWO = Decimal(2)
LN2 = TWO.ln()


def main():
    print("// Fixed-point exp tables.  Written by gen_exp2_table.py.")
    print("#pragma once")
    q = [int((TWO ** (Decimal(-j) / 256) * TWO ** 63).to_integral_value()) for j in range(256)]
    print("// 2^(-j/256) in units of 2^-63 (j = 0 is 2^63)")
    print("__device__ const unsigned long long kExp2NegQ63[256] = {")
    for j in range(0, 256, 4):
        print("    " + ", ".join("0x%016xull" % v for v in q[j:j + 4]) + ",")
    print("};")
    c = int((Decimal(256) / LN2 * TWO ** 54).to_integral_value())
    l = int((LN2 / 256 * TWO ** 116).to_integral_value())
    print("constexpr unsigned long long kExpK256Q54 = 0x%016xull;  // 256/ln2 x 2^54" % c)
    print("constexpr unsigned long long kExpL256Hi = 0x%016xull;  // ln2/256 x 2^116, high word" % (l >> 64))
    print("constexpr unsigned long long kExpL256Lo = 0x%016xull;  // low word" % (l & (2 ** 64 - 1)))


if __name__ == "__main__":
    main()
