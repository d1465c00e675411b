"""Writes exp2_table.cuh: 2^(j/128), j = 0..127, as (lead, trail) FP64 pairs, with
lead = 2^(j/128) rounded to FP64 and trail = the remainder rounded to FP64, both
computed in 60-digit decimal arithmetic.  Run once; the output is committed.

    python qml_gb300/csrc/gen_exp2_table.py > qml_gb300/csrc/exp2_table.cuh
"""
from decimal import Decimal, getcontext

getcontext().prec = 60
TWO = Decimal(2)
LN2 = TWO.ln()


def to_double(d: Decimal) -> float:
    # nearest FP64 to a decimal (float(str) rounds correctly)
    return float(format(d, ".40e"))


def main():
    print("// 2^(j/128) for j = 0..127 as (lead, trail): lead = the value rounded to FP64,")
    print("// trail = (value - lead) rounded to FP64.  Written by gen_exp2_table.py.")
    print("#pragma once")
    print("__device__ const double2 kExp2Tab128[128] = {")
    for j in range(128):
        v = (LN2 * Decimal(j) / Decimal(128)).exp()
        lead = to_double(v)
        trail = to_double(v - Decimal(lead))
        print("    {%s, %s}," % (lead.hex(), trail.hex()))
    print("};")
    c = LN2 / Decimal(128)
    hi = to_double(c)
    lo = to_double(c - Decimal(hi))
    print("// ln2 / 128 as hi + lo; 128 / ln2")
    print("constexpr double kLn2Over128Hi = %s;" % hi.hex())
    print("constexpr double kLn2Over128Lo = %s;" % lo.hex())
    print("constexpr double k128OverLn2 = %s;" % to_double(Decimal(128) / LN2).hex())


if __name__ == "__main__":
    main()
