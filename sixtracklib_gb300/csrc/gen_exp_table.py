"""Write exp_table.h: the constants of the fast policy's exponential
(maps.cuh exp_fast), P. T. P. Tang's table-driven method (ACM Trans. Math.
Softw. 15 (1989) 144-157) with 256 table entries.

* 2^(j/256), j = 0..255, as a pair (hi, lo): hi the nearest double, lo the
  nearest double to the remainder;
* 256 / ln 2, and ln 2 / 256 split as L1 + L2 with L1's low 20 significand
  bits zero (n L1 exact for |n| < 2^20).

All values from 60-digit decimal arithmetic.  Run from this directory:
python gen_exp_table.py > exp_table.h
"""

import struct
from decimal import Decimal, getcontext

getcontext().prec = 60
N = 256


def bits(d: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", d))[0]


def from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b))[0]


def lit(d: float) -> str:
    return f"{d!r}" if d != 0 else "0.0"


def table():
    ln2 = Decimal(2).ln()
    hi, lo = [], []
    for j in range(N):
        v = (ln2 * j / N).exp()
        h = float(v)
        hi.append(h)
        lo.append(float(v - Decimal(h)))
    c = ln2 / N
    l1 = from_bits(bits(float(c)) & ~((1 << 20) - 1))
    l2 = float(c - Decimal(l1))
    inv = float(N / ln2)
    return hi, lo, l1, l2, inv


def main():
    hi, lo, l1, l2, inv = table()
    out = ["// exp_table.h -- written by gen_exp_table.py; do not edit.",
           "// 2^(j/256) as (hi, lo) pairs and the argument reduction constants of",
           "// exp_fast (maps.cuh).",
           "#pragma once", "",
           "namespace stg {", "",
           "constexpr int kExpTableBits = 8;",
           f"constexpr double kExpInvLn2N = {lit(inv)};  // 256 / ln 2",
           f"constexpr unsigned long long kExpL1Bits = 0x{bits(l1):016X}ull;  // ln 2 / 256, high part",
           f"constexpr unsigned long long kExpL2Bits = 0x{bits(l2):016X}ull;  // ln 2 / 256 - L1",
           "",
           "// [2 j] = hi, [2 j + 1] = lo of 2^(j/256)",
           "static __device__ const double kExpTable[512] = {"]
    for j in range(N):
        out.append(f"    {lit(hi[j])}, {lit(lo[j])},")
    out += ["};", "", "}  // namespace stg", ""]
    print("\n".join(out))


if __name__ == "__main__":
    main()
