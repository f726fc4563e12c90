"""Generates the constants of the table-driven exponential in ts_common.h:
2^(j/64) for j = 0..63 rounded to the nearest double, and ln(2)/64 split in
a high part (trailing zero bits) and a low remainder.  Exact decimal
arithmetic at 60 digits; Python's float() of a decimal string rounds
correctly."""
from decimal import Decimal, getcontext

getcontext().prec = 60
ln2 = Decimal(2).ln()
table = [float(str((Decimal(j) / 64 * ln2).exp())) for j in range(64)]
step = ln2 / 64
hi = float(str(step))
# keep 32 significant bits in the high part so k * hi is exact for |k| < 2^21
import struct
bits = struct.unpack("<Q", struct.pack("<d", hi))[0] & ~((1 << 21) - 1)
hi = struct.unpack("<d", struct.pack("<Q", bits))[0]
lo = float(str(step - Decimal(hi)))
inv = float(str(64 / ln2))
print("inv_step = %s;  // 64 / ln 2" % inv.hex())
print("step_hi = %s;  // ln 2 / 64, high bits" % hi.hex())
print("step_lo = %s;  // ln 2 / 64 - step_hi" % lo.hex())
for j in range(0, 64, 2):
    print("    %s, %s," % (table[j].hex(), table[j + 1].hex()))

# float-float constants of ts_weight_ff: ln2/64 = C1 + C2 + C3 with C1 of
# 9 significant bits (k * C1 exact for |k| < 2^15), 64/ln2 as a float, and
# 2^(j/64) as (hi, lo) float pairs.
import math
import struct


def f32(x):
    return struct.unpack("<f", struct.pack("<f", float(x)))[0]


C = ln2 / 64
m, e = math.frexp(float(C))
C1 = math.ldexp(round(m * 2 ** 11) / 2 ** 11, e)
C2 = f32(C - Decimal(C1))
C3 = f32(C - Decimal(C1) - Decimal(C2))
print("ff_inv = %sf; ff_c1 = %sf; ff_c2 = %sf; ff_c3 = %sf;" % (
    float(f32(64 / ln2)).hex(), C1.hex(), float(C2).hex(), float(C3).hex()))
for j in range(0, 64, 2):
    pair = []
    for jj in (j, j + 1):
        v = (Decimal(jj) / 64 * ln2).exp()
        hi = f32(v)
        lo = f32(v - Decimal(hi))
        pair += [float(hi).hex() + "f", float(lo).hex() + "f"]
    print("    %s, %s, %s, %s," % tuple(pair))
