"""Constants of the double-float elementary functions (df32.h): each value is
printed as the pair (hi, lo) of FP32 numbers nearest to it, hi = RN(v),
lo = RN(v - hi), computed with 60-digit arithmetic.  Run it to regenerate the
tables pasted into df32.h:  python gen_df32_tables.py"""
import mpmath as mp
import numpy as np

mp.mp.dps = 60


def df(v):
    hi = np.float32(float(v))
    lo = np.float32(float(v - mp.mpf(float(hi))))
    return float(hi), float(lo)


def split_bits(v, bits):
    """v rounded to `bits` significant bits (a float with a short significand)."""
    e = int(mp.floor(mp.log(abs(v), 2)))
    q = mp.mpf(2) ** (e - bits + 1)
    return mp.nint(v / q) * q


def f32(x):
    return repr(np.float32(x).item()) + "f"


ln2_32 = mp.log(2) / 32
c1 = split_bits(ln2_32, 11)
c2 = split_bits(ln2_32 - c1, 11)
c3 = mp.mpf(float(np.float32(float(ln2_32 - c1 - c2))))
c4 = mp.mpf(float(np.float32(float(ln2_32 - c1 - c2 - c3))))
print("/* ln 2 / 32 = C1 + C2 + C3 + C4 (+ %.1e) */" % float(ln2_32 - c1 - c2 - c3 - c4))
for name, v in (("C1", c1), ("C2", c2), ("C3", c3), ("C4", c4)):
    print(f"#define DF_LN2_32_{name} {f32(float(v))}")
print("/* 2^(j/32), j = 0..31 */")
for j in range(32):
    h, l = df(mp.mpf(2) ** (mp.mpf(j) / 32))
    print(f"  {{{f32(h)}, {f32(l)}}},")
print("/* c = 1 + j/64, j = -19..27: 1/c and log(c) */")
for j in range(-19, 28):
    c = 1 + mp.mpf(j) / 64
    r = df(1 / c)
    lg = df(mp.log(c))
    print(f"  {{{f32(r[0])}, {f32(r[1])}, {f32(lg[0])}, {f32(lg[1])}}},")
for name, v in (("1/3", mp.mpf(1) / 3), ("1/6", mp.mpf(1) / 6), ("1/120", mp.mpf(1) / 120),
                ("1/5040", mp.mpf(1) / 5040), ("1/362880", mp.mpf(1) / 362880), ("1/24", mp.mpf(1) / 24),
                ("1/720", mp.mpf(1) / 720), ("1/40320", mp.mpf(1) / 40320)):
    h, l = df(v)
    print(f"/* {name} */ {f32(h)}, {f32(l)}")
