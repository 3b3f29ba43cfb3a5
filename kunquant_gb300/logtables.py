"""Lookup tables of the table-driven logarithm (``cpp/KunSIMD/cpu/Math.hpp:20-93``).

Entry i belongs to the mantissa bin selected by the top five mantissa bits.
Bins 0-15 hold mantissas M in [1, 1.5); bins 16-31 hold M in [0.75, 1) (the
exponent is lowered by one).  ``r_i`` is the reciprocal of the bin centre
rounded to the nearest multiple of 1/32 (bins 0-15) or 1/16 (bins 16-31);
``logr_i = -log(r_i) - bias*ln2`` folds in the exponent bias (127 / 1023).

The values are frozen as exact hex literals so every machine that builds the
kernels (x86 or Arm, whatever its libm) gets the same bits; ``derive()``
recomputes them from the formula for the tests.
"""
import math

R = [1.0, 0.96875, 0.9375, 0.90625, 0.875, 0.84375, 0.84375, 0.8125, 0.78125, 0.78125,
     0.75, 0.75, 0.71875, 0.71875, 0.6875, 0.6875, 1.3125, 1.3125, 1.25, 1.25, 1.25,
     1.1875, 1.1875, 1.125, 1.125, 1.125, 1.125, 1.0625, 1.0625, 1.0625, 1.0, 1.0]

LOGR_F32 = [
    "-0x1.601e680000000p+6", "-0x1.5ffde40000000p+6", "-0x1.5fdc520000000p+6",
    "-0x1.5fb99a0000000p+6", "-0x1.5f95ac0000000p+6", "-0x1.5f706e0000000p+6",
    "-0x1.5f706e0000000p+6", "-0x1.5f49c80000000p+6", "-0x1.5f219e0000000p+6",
    "-0x1.5f219e0000000p+6", "-0x1.5ef7d20000000p+6", "-0x1.5ef7d20000000p+6",
    "-0x1.5ecc3c0000000p+6", "-0x1.5ecc3c0000000p+6", "-0x1.5e9eb80000000p+6",
    "-0x1.5e9eb80000000p+6", "-0x1.6134de0000000p+6", "-0x1.6134de0000000p+6",
    "-0x1.6102e80000000p+6", "-0x1.6102e80000000p+6", "-0x1.6102e80000000p+6",
    "-0x1.60ce620000000p+6", "-0x1.60ce620000000p+6", "-0x1.6097040000000p+6",
    "-0x1.6097040000000p+6", "-0x1.6097040000000p+6", "-0x1.6097040000000p+6",
    "-0x1.605c7c0000000p+6", "-0x1.605c7c0000000p+6", "-0x1.605c7c0000000p+6",
    "-0x1.601e680000000p+6", "-0x1.601e680000000p+6"]

LOGR_F64 = [
    "-0x1.628b76e3a7b61p+9", "-0x1.6287668c453c4p+9", "-0x1.628334174ce6fp+9",
    "-0x1.627edd3479097p+9", "-0x1.627a5f55258e3p+9", "-0x1.6275b7a33c61dp+9",
    "-0x1.6275b7a33c61dp+9", "-0x1.6270e2f66b2b3p+9", "-0x1.626bddc73b026p+9",
    "-0x1.626bddc73b026p+9", "-0x1.6266a41f854c6p+9", "-0x1.6266a41f854c6p+9",
    "-0x1.626131879944dp+9", "-0x1.626131879944dp+9", "-0x1.625b80ef3005ep+9",
    "-0x1.625b80ef3005ep+9", "-0x1.62ae459cff0d6p+9", "-0x1.62ae459cff0d6p+9",
    "-0x1.62a806db6f50bp+9", "-0x1.62a806db6f50bp+9", "-0x1.62a806db6f50bp+9",
    "-0x1.62a17614185dap+9", "-0x1.62a17614185dap+9", "-0x1.629a8a675ecb9p+9",
    "-0x1.629a8a675ecb9p+9", "-0x1.629a8a675ecb9p+9", "-0x1.629a8a675ecb9p+9",
    "-0x1.6293396fd7ba7p+9", "-0x1.6293396fd7ba7p+9", "-0x1.6293396fd7ba7p+9",
    "-0x1.628b76e3a7b61p+9", "-0x1.628b76e3a7b61p+9"]


def derive(dtype: str):
    """(r, logr) from the formula, as Python floats (logr before rounding to
    the dtype)."""
    bias = 127 if dtype == "float" else 1023
    r, lr = [], []
    for i in range(32):
        if i < 16:
            m, g = 1.0 + (i + 0.5) / 32.0, 32.0
        else:
            m, g = 0.5 * (1.0 + (i + 0.5) / 32.0), 16.0
        rv = math.floor(g / m + 0.5) / g
        r.append(rv)
        lr.append(-math.log(rv) + (-math.log(2) * bias))
    return r, lr


def table(dtype: str):
    """C literal lists (r, logr) for the code generator."""
    if dtype == "float":
        return [float(v).hex() + "f" for v in R], [h + "f" for h in LOGR_F32]
    return [float(v).hex() for v in R], list(LOGR_F64)
