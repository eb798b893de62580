"""Constants and tables of the FP64 exp and log (rr_math.h), computed with
60-digit arithmetic and printed as C hex literals.  Run it to regenerate the
block pasted into rr_math.h:  python gen_rr_math_tables.py"""
import mpmath as mp

mp.mp.dps = 60


def rn(v):
    """v rounded to the nearest double."""
    return float(v)


def hexf(x):
    return float(x).hex()


def short(v, bits):
    """v rounded to `bits` significant bits."""
    e = int(mp.floor(mp.log(abs(v), 2)))
    q = mp.mpf(2) ** (e - bits + 1)
    return mp.nint(v / q) * q


def grid(v, step_exp):
    """v rounded to a multiple of 2^step_exp."""
    q = mp.mpf(2) ** step_exp
    return mp.nint(v / q) * q


ln2 = mp.log(2)
L64 = ln2 / 64
c1 = short(L64, 36)                 # |k| < 2^17: k * C1 is exact
c2 = L64 - c1
print("/* exp: x = k ln2/64 + r; 64/ln2, ln2/64 = C1 + C2 (C1: 36 bits) */")
print(f"#define RR_EXP_INV_L64 {hexf(rn(1 / L64))}")
print(f"#define RR_EXP_C1 {hexf(rn(c1))}")
print(f"#define RR_EXP_C2 {hexf(rn(c2))}")
print("/* 1/n!, n = 2..6 */")
for n in range(2, 7):
    print(f"#define RR_EXP_F{n} {hexf(rn(1 / mp.factorial(n)))}")
print("/* 2^(j/64) = hi + lo, j = 0..63 */")
print("#define RR_EXP_TAB { \\")
for j in range(64):
    v = mp.mpf(2) ** (mp.mpf(j) / 64)
    h = rn(v)
    lo = rn(v - mp.mpf(h))
    print(f"  {{{hexf(h)}, {hexf(lo)}}}, \\")
print("}")
ln2_hi = grid(ln2, -42)
print("/* log: ln2 = HI + LO (HI a multiple of 2^-42) */")
print(f"#define RR_LOG_LN2_HI {hexf(rn(ln2_hi))}")
print(f"#define RR_LOG_LN2_LO {hexf(rn(ln2 - ln2_hi))}")
print("/* (-1)^(n+1) / n, n = 2..9 */")
for n in range(2, 10):
    print(f"#define RR_LOG_P{n} {hexf(rn(mp.mpf((-1) ** (n + 1)) / n))}")
print("/* c = 1 + j/64, j = -19..27: RN(1/c), log(c) = hi + lo (hi a multiple of 2^-42) */")
print("#define RR_LOG_TAB { \\")
for j in range(-19, 28):
    c = 1 + mp.mpf(j) / 64
    lc = mp.log(c)
    hi = grid(lc, -42)
    print(f"  {{{hexf(rn(1 / c))}, {hexf(rn(hi))}, {hexf(rn(lc - hi))}}}, \\")
print("}")
