/*
 * Double-float arithmetic ("df32"): a value is the unevaluated sum hi + lo of
 * two FP32 numbers with |lo| <= ulp(hi) / 2, about 48 significant bits over
 * FP32's exponent range.  It runs on the FP32 pipes, which on GB300 issue
 * 64 times as many operations per cycle as the FP64 pipe.
 *
 * Basic operations follow the double-word algorithms analysed by Joldes,
 * Muller and Popescu ("Tight and rigorous error bounds for basic building
 * blocks of double-word arithmetic", ACM TOMS 44(2), 2017): addition
 * (their Algorithm 6), addition of a float (Algorithm 4), multiplication
 * with FMA (Algorithm 12), division (Algorithm 17 form), the square root by
 * one Karp-Markstein correction of the FP32 root.  Elementary functions are
 * our own, table-driven: exp by reduction by ln 2 / 32 (four-part split,
 * exact leading products), 2^(j/32) from a table and a short polynomial whose
 * terms of order 4 and above are summed in FP32; log by m 2^e with
 * m in [sqrt(1/2), sqrt(2)), c = 1 + j/64 nearest to m, log m = log c +
 * log1p((m - c) / c) from a table of 1/c and log c and a short series (order
 * 5 and above in FP32); sin / cos by Cody-Waite reduction by pi / 2
 * (four-part split, |k| < 4096) and Taylor polynomials on |r| <= pi / 4 whose
 * high-order tails are summed in FP32.  Table entries and constants are the
 * double-floats nearest to their values (gen_df32_tables.py).  Relative
 * accuracy is about 1e-13 (absolute for results near zero, and only
 * absolute, about 1e-38, for magnitudes below 1e-31, where the low part
 * leaves FP32's normal range); arguments that the reductions do not cover
 * give NaN, so that a caller treats the value as not computed.
 *
 * Non-finite results carry lo = 0.  Host builds need -ffp-contract=off.
 */
#ifndef RR_DF32_H
#define RR_DF32_H

#include <math.h>

#if defined(__CUDACC__)
#define DFN static __host__ __device__ __forceinline__
#else
#define DFN static inline
#endif

#if defined(__CUDA_ARCH__)
#define DF_ADD(a, b) __fadd_rn((a), (b))
#define DF_SUB(a, b) __fsub_rn((a), (b))
#define DF_MUL(a, b) __fmul_rn((a), (b))
#define DF_DIV(a, b) __fdiv_rn((a), (b))
#define DF_FMA(a, b, c) __fmaf_rn((a), (b), (c))
#define DF_SQRT(a) __fsqrt_rn(a)
#else
#define DF_ADD(a, b) ((float)((a) + (b)))
#define DF_SUB(a, b) ((float)((a) - (b)))
#define DF_MUL(a, b) ((float)((a) * (b)))
#define DF_DIV(a, b) ((float)((a) / (b)))
#define DF_FMA(a, b, c) fmaf((a), (b), (c))
#define DF_SQRT(a) sqrtf(a)
#endif

/* an approximate reciprocal (within a few ulp; a Newton step follows every
 * use): the special-function unit's on the device; on the host the quotient
 * moved one ulp toward zero, so that host tests exercise the Newton step */
static
#if defined(__CUDACC__)
    __host__ __device__
#endif
    inline float df_rcp_approx(float y) {
#if defined(__CUDA_ARCH__)
  float r;
  asm("rcp.approx.ftz.f32 %0, %1;" : "=f"(r) : "f"(y));
  return r;
#else
  return nextafterf(1.0f / y, 0.0f);
#endif
}

typedef struct {
  float hi, lo;
} dfl;

DFN dfl dfl_make(float h, float l) {
  dfl r;
  r.hi = h;
  r.lo = l;
  return r;
}
DFN int dfl_finite(float x) { return x - x == 0.0f; }
#if defined(__CUDA_ARCH__)
DFN float dfl_nanf(void) { return __int_as_float(0x7fc00000); }
DFN float dfl_inff(void) { return __int_as_float(0x7f800000); }
/* 2^e for e in [-126, 127] */
DFN float dfl_pow2(int e) { return __int_as_float((e + 127) << 23); }
#else
DFN float dfl_nanf(void) { return NAN; }
DFN float dfl_inff(void) { return INFINITY; }
DFN float dfl_pow2(int e) { return ldexpf(1.0f, e); }
#endif

/* ---- error-free transformations ---- */
DFN dfl dfl_fast_two_sum(float a, float b) {
  const float s = DF_ADD(a, b);
  const float z = DF_SUB(s, a);
  return dfl_make(s, DF_SUB(b, z));
}
DFN dfl dfl_two_sum(float a, float b) {
  const float s = DF_ADD(a, b);
  const float ap = DF_SUB(s, b);
  const float bp = DF_SUB(s, ap);
  return dfl_make(s, DF_ADD(DF_SUB(a, ap), DF_SUB(b, bp)));
}
DFN dfl dfl_two_prod(float a, float b) {
  const float p = DF_MUL(a, b);
  return dfl_make(p, DF_FMA(a, b, -p));
}
/* a non-finite leading part, or a low part made non-finite by an overflow in
 * an intermediate, leaves the value as its leading part */
DFN dfl dfl_guard(dfl r, float lead) {
  if (!dfl_finite(lead)) return dfl_make(lead, 0.0f);
  if (!dfl_finite(r.hi)) return dfl_make(r.hi, 0.0f);
  if (!dfl_finite(r.lo)) r.lo = 0.0f;
  return r;
}

/* ---- conversions ---- */
DFN dfl dfl_from_double(double x) {
  const float h = (float)x;
  if (!dfl_finite(h)) return dfl_make(h, 0.0f);
  return dfl_make(h, (float)(x - (double)h));
}
DFN double dfl_to_double(dfl a) { return (double)a.hi + (double)a.lo; }

/* ---- arithmetic ---- */
DFN dfl dfl_add(dfl x, dfl y) {
  const float lead = DF_ADD(x.hi, y.hi);
  if (!dfl_finite(lead)) return dfl_make(lead, 0.0f);
  const dfl s = dfl_two_sum(x.hi, y.hi);
  const dfl t = dfl_two_sum(x.lo, y.lo);
  const float c = DF_ADD(s.lo, t.hi);
  const dfl v = dfl_fast_two_sum(s.hi, c);
  const float w = DF_ADD(t.lo, v.lo);
  return dfl_guard(dfl_fast_two_sum(v.hi, w), lead);
}
DFN dfl dfl_neg(dfl x) { return dfl_make(-x.hi, -x.lo); }
DFN dfl dfl_sub(dfl x, dfl y) { return dfl_add(x, dfl_neg(y)); }
DFN dfl dfl_mul(dfl x, dfl y) {
  const dfl c = dfl_two_prod(x.hi, y.hi);
  if (!dfl_finite(c.hi)) return dfl_make(c.hi, 0.0f);
  const float tl0 = DF_MUL(x.lo, y.lo);
  const float tl1 = DF_FMA(x.hi, y.lo, tl0);
  const float cl2 = DF_FMA(x.lo, y.hi, tl1);
  const float cl3 = DF_ADD(c.lo, cl2);
  return dfl_guard(dfl_fast_two_sum(c.hi, cl3), c.hi);
}
DFN dfl dfl_mul_f(dfl x, float y) {
  const dfl c = dfl_two_prod(x.hi, y);
  if (!dfl_finite(c.hi)) return dfl_make(c.hi, 0.0f);
  const float cl3 = DF_FMA(x.lo, y, c.lo);
  return dfl_guard(dfl_fast_two_sum(c.hi, cl3), c.hi);
}
DFN dfl dfl_div(dfl x, dfl y) {
  const float th = DF_DIV(x.hi, y.hi);
  if (!dfl_finite(th) || y.hi == 0.0f || th == 0.0f) return dfl_make(th, 0.0f);
  const dfl r = dfl_mul_f(y, th);
  const float pih = DF_SUB(x.hi, r.hi);
  const float dl = DF_SUB(x.lo, r.lo);
  const float d = DF_ADD(pih, dl);
  const float tl = DF_DIV(d, y.hi);
  return dfl_guard(dfl_fast_two_sum(th, tl), th);
}
DFN dfl dfl_sqrt(dfl x) {
  if (!(x.hi > 0.0f) || !dfl_finite(x.hi)) return dfl_make(DF_SQRT(x.hi), 0.0f);
  const float s = DF_SQRT(x.hi);
  const dfl e = dfl_sub(x, dfl_two_prod(s, s));
  const float c = DF_DIV(e.hi, DF_MUL(2.0f, s));
  return dfl_guard(dfl_fast_two_sum(s, c), s);
}
DFN dfl dfl_scale(dfl x, float p2) { return dfl_make(DF_MUL(x.hi, p2), DF_MUL(x.lo, p2)); }

/* ---- unguarded forms for finite operands (inside the elementary functions) ---- */
DFN dfl dfl_add_nc(dfl x, dfl y) {
  const dfl s = dfl_two_sum(x.hi, y.hi);
  const dfl t = dfl_two_sum(x.lo, y.lo);
  const float c = DF_ADD(s.lo, t.hi);
  const dfl v = dfl_fast_two_sum(s.hi, c);
  const float w = DF_ADD(t.lo, v.lo);
  return dfl_fast_two_sum(v.hi, w);
}
DFN dfl dfl_mul_nc(dfl x, dfl y) {
  const dfl c = dfl_two_prod(x.hi, y.hi);
  const float tl0 = DF_MUL(x.lo, y.lo);
  const float tl1 = DF_FMA(x.hi, y.lo, tl0);
  const float cl2 = DF_FMA(x.lo, y.hi, tl1);
  return dfl_fast_two_sum(c.hi, DF_ADD(c.lo, cl2));
}
/* x + a for a float a */
DFN dfl dfl_add_fl(dfl x, float a) {
  const dfl s = dfl_two_sum(x.hi, a);
  return dfl_fast_two_sum(s.hi, DF_ADD(x.lo, s.lo));
}
/* x * a for a float a */
DFN dfl dfl_mul_fl(dfl x, float a) {
  const dfl c = dfl_two_prod(x.hi, a);
  return dfl_fast_two_sum(c.hi, DF_FMA(x.lo, a, c.lo));
}
/* x / y for finite operands and a finite quotient: 1/y.hi from the
 * approximate reciprocal and one Newton step (relative error near 2^-44),
 * th = x.hi / y.hi rounded, then the remainder x - th y (its leading part
 * by FMA, exact for a faithful th) times 1/y.hi as the low part.  A
 * non-finite leading part means the guarded dfl_div has to run. */
DFN dfl dfl_div_nc(dfl x, dfl y) {
  const float r0 = df_rcp_approx(y.hi);
  const float r1 = DF_FMA(r0, DF_FMA(-y.hi, r0, 1.0f), r0);
  const float th = DF_MUL(x.hi, r1);
  const float rem = DF_ADD(DF_FMA(-th, y.lo, DF_FMA(-th, y.hi, x.hi)), x.lo);
  return dfl_fast_two_sum(th, DF_MUL(rem, r1));
}

/* ---- tables ---- */
#define DF_LN2_32_C1 0.02166748046875f
#define DF_LN2_32_C2 -6.631016731262207e-06f
#define DF_LN2_32_C3 -5.952044412893542e-11f
#define DF_LN2_32_C4 -2.7447449183091686e-18f
#define DFL_EXP2_TAB { \
  {1.0f, 0.0f}, \
  {1.0218971967697144f, -4.811559861650494e-08f}, \
  {1.0442737340927124f, 4.8334701574503924e-08f}, \
  {1.0671404600143433f, -5.9337519786595294e-08f}, \
  {1.0905077457427979f, -1.3077539939843064e-08f}, \
  {1.114386796951294f, -5.435540018083884e-08f}, \
  {1.1387885808944702f, 5.386222312608879e-08f}, \
  {1.1637248992919922f, -4.051441493402308e-08f}, \
  {1.1892070770263672f, 3.797635272917432e-08f}, \
  {1.215247392654419f, -3.267394887984665e-08f}, \
  {1.2418577671051025f, 4.496838101886169e-08f}, \
  {1.2690509557724f, 1.419333317542737e-09f}, \
  {1.2968395948410034f, -4.018999533172973e-08f}, \
  {1.3252366781234741f, -3.496373324196611e-08f}, \
  {1.3542555570602417f, -1.0123349269974824e-08f}, \
  {1.3839099407196045f, -5.875577357983275e-08f}, \
  {1.4142135381698608f, 2.4203234971764687e-08f}, \
  {1.4451807737350464f, 3.324199937537742e-08f}, \
  {1.4768261909484863f, -4.500898853621038e-08f}, \
  {1.5091644525527954f, -2.4959373234878512e-08f}, \
  {1.5422108173370361f, 8.070904833346049e-09f}, \
  {1.5759809017181396f, -5.661025426206834e-08f}, \
  {1.610490322113037f, 9.836217174097328e-09f}, \
  {1.6457555294036865f, -5.124972091152813e-08f}, \
  {1.6817928552627563f, -2.4755326677450284e-08f}, \
  {1.7186193466186523f, -4.8496175963919086e-08f}, \
  {1.7562521696090698f, -9.235770370707996e-09f}, \
  {1.7947090864181519f, -1.141504490931311e-08f}, \
  {1.8340080976486206f, -1.1239277952768134e-08f}, \
  {1.8741676807403564f, -4.663005626071026e-08f}, \
  {1.9152065515518188f, 9.845328108326612e-09f}, \
  {1.9571441411972046f, -1.7021804410433106e-08f}, \
}
#define DFL_LOG_TAB { \
  {1.4222222566604614f, -3.443824070359369e-08f, -0.3522205948829651f, 1.2936129945018138e-09f}, \
  {1.39130437374115f, -2.5915062096260044e-08f, -0.33024168014526367f, -6.725313195232729e-09f}, \
  {1.3617020845413208f, 4.311825207992115e-08f, -0.3087354898452759f, 8.195662815069227e-09f}, \
  {1.3333333730697632f, -3.973643103449831e-08f, -0.28768208622932434f, 1.3777543550475002e-08f}, \
  {1.3061224222183228f, 2.676126875655882e-08f, -0.267062783241272f, -2.0077732809653526e-09f}, \
  {1.2799999713897705f, 2.8610228852699038e-08f, -0.246860072016716f, -5.914809975138269e-09f}, \
  {1.2549020051956177f, -4.441130485588474e-08f, -0.22705745697021484f, 6.334868629664925e-09f}, \
  {1.2307692766189575f, -4.5849727570157484e-08f, -0.20763936638832092f, 1.610076405533789e-09f}, \
  {1.2075471878051758f, -1.7993855294662353e-08f, -0.18859116733074188f, -2.476808091955718e-09f}, \
  {1.185185194015503f, -8.830317810293309e-09f, -0.16989903151988983f, -5.275507586333106e-09f}, \
  {1.163636326789856f, 3.684650806690115e-08f, -0.15154990553855896f, 7.411358193820661e-09f}, \
  {1.1428571939468384f, -5.108969602929392e-08f, -0.133531391620636f, -1.0038866404826763e-09f}, \
  {1.1228070259094238f, -8.365564241330503e-09f, -0.11583181470632553f, -8.187961975103519e-10f}, \
  {1.1034482717514038f, 4.11066514161007e-09f, -0.09844007343053818f, 6.17285667026124e-10f}, \
  {1.0847457647323608f, -2.020496436827557e-09f, -0.08134564012289047f, 6.689380716018434e-10f}, \
  {1.0666667222976685f, -5.563100202721216e-08f, -0.06453852355480194f, 2.417230859919073e-09f}, \
  {1.049180269241333f, 5.862752061602805e-08f, -0.04800922051072121f, 1.3243606211688075e-09f}, \
  {1.0322580337524414f, 3.076368670917873e-08f, -0.0317486971616745f, -1.1529057708514756e-09f}, \
  {1.0158730745315552f, -5.865853935915766e-08f, -0.01574835740029812f, 4.3215894751647e-10f}, \
  {1.0f, 0.0f, 0.0f, 0.0f}, \
  {0.9846153855323792f, -9.169945358600273e-10f, 0.015504186972975731f, -4.3701048335620385e-10f}, \
  {0.9696969985961914f, -2.8899222570544225e-08f, 0.030771657824516296f, 8.422373909411363e-10f}, \
  {0.9552238583564758f, 2.224053829991135e-08f, 0.045809537172317505f, -1.1410232758635175e-09f}, \
  {0.9411764740943909f, -3.5061555880844253e-09f, 0.0606246218085289f, 7.905942393804377e-12f}, \
  {0.9275362491607666f, -1.7276708064173363e-08f, 0.0752234235405922f, -2.303004675852094e-09f}, \
  {0.9142857193946838f, -5.108969691747234e-09f, 0.08961215615272522f, 2.536961973831353e-09f}, \
  {0.9014084339141846f, 1.6790041357239716e-08f, 0.10379679501056671f, -1.328923193710807e-09f}, \
  {0.8888888955116272f, -6.622738357719982e-09f, 0.11778303235769272f, 3.2986906539633765e-09f}, \
  {0.8767123222351074f, 6.532015817128922e-09f, 0.13157635927200317f, -1.4832839401179854e-09f}, \
  {0.8648648858070374f, -2.0942172440641116e-08f, 0.14518201351165771f, -3.6671599090709606e-09f}, \
  {0.8533333539962769f, -2.0662943356342112e-08f, 0.15860502421855927f, 5.9580793632108e-09f}, \
  {0.8421052694320679f, -6.274173180997877e-09f, 0.1718502640724182f, -7.145759095550375e-09f}, \
  {0.8311688303947449f, 7.740862950633698e-10f, 0.18492233753204346f, 9.619685048534166e-10f}, \
  {0.8205128312110901f, -1.0698269825581974e-08f, 0.19782574474811554f, -1.4181956720094036e-09f}, \
  {0.8101266026496887f, -2.037120694353689e-08f, 0.2105647623538971f, 6.753452463925669e-09f}, \
  {0.800000011920929f, -1.1920929132713809e-08f, 0.2231435477733612f, 3.540848503291727e-09f}, \
  {0.790123462677002f, -5.886878540195539e-09f, 0.23556606471538544f, 6.597381307926753e-09f}, \
  {0.7804877758026123f, 2.907543716901273e-08f, 0.2478361576795578f, 6.225023607697722e-09f}, \
  {0.7710843086242676f, 2.8725130718498804e-08f, 0.25995752215385437f, 2.283071731667974e-09f}, \
  {0.761904776096344f, -1.419158213167293e-08f, 0.2719337046146393f, 1.086900258684409e-08f}, \
  {0.7529411911964417f, -1.4725853425545665e-08f, 0.2837681770324707f, -3.9018259734291405e-09f}, \
  {0.7441860437393188f, 2.772309048992838e-09f, 0.2954642176628113f, -4.768975436775236e-09f}, \
  {0.7356321811676025f, 2.740443427740047e-09f, 0.3070250451564789f, -9.86156667437399e-09f}, \
  {0.7272727489471436f, -2.167441692790817e-08f, 0.31845372915267944f, 1.9658552563583953e-09f}, \
  {0.7191011309623718f, -7.3668662281534125e-09f, 0.3297532796859741f, 6.686494025132106e-09f}, \
  {0.7111111283302307f, -1.7219120351796846e-08f, 0.3409265875816345f, -6.110413286464222e-10f}, \
  {0.7032967209815979f, -1.7684895325942307e-08f, 0.3519764244556427f, -1.2984645580971232e-09f}, \
}
/* a = j/32, j = -26..26: sin a and cos a */
#define DFL_SC_TAB { \
  {-0.7260086536407471f, -1.6199654950810327e-09f, 0.6876855492591858f, 1.2961319129090043e-08f}, \
  {-0.7041674852371216f, -2.6217412241180682e-08f, 0.7100338935852051f, -1.0019125085136693e-08f}, \
  {-0.681638777256012f, 1.723267750719515e-08f, 0.7316888570785522f, 1.1795268761716216e-08f}, \
  {-0.6584444046020508f, 4.691483201924029e-09f, 0.7526293992996216f, -2.6881554759938808e-08f}, \
  {-0.6346070766448975f, -3.37037175945909e-09f, 0.7728349566459656f, -1.0493494073671172e-08f}, \
  {-0.6101500988006592f, 2.1724867238503975e-08f, 0.7922858595848083f, 9.237019482633002e-11f}, \
  {-0.5850972533226013f, -1.9617861113374602e-08f, 0.8109630942344666f, 2.5270750825256982e-08f}, \
  {-0.5594731569290161f, 2.568164880756285e-08f, 0.8288484811782837f, 6.431041921217684e-09f}, \
  {-0.5333026647567749f, -8.779244886625293e-09f, 0.8459244966506958f, 2.5803721381834066e-09f}, \
  {-0.5066114664077759f, 1.1593518145502912e-08f, 0.8621744513511658f, 2.858371495051415e-08f}, \
  {-0.4794255495071411f, 1.0902938107903992e-08f, 0.8775825500488281f, 1.1841544633739431e-08f}, \
  {-0.45177146792411804f, -3.5675657983347264e-09f, 0.8921337127685547f, -1.3401559861847545e-08f}, \
  {-0.4236762523651123f, -4.838825784503342e-09f, 0.9058136940002441f, -1.0574307651722847e-08f}, \
  {-0.3951673209667206f, -9.274213397247877e-09f, 0.9186091423034668f, 1.3491451511526975e-08f}, \
  {-0.36627253890037537f, 9.814328016943819e-09f, 0.9305076003074646f, 2.1604849465006737e-08f}, \
  {-0.33702006936073303f, 3.384799662775606e-10f, 0.9414974451065063f, 1.8021374614818342e-08f}, \
  {-0.30743852257728577f, 7.996904471951893e-09f, 0.9515679478645325f, 1.8363972842383447e-10f}, \
  {-0.27755674719810486f, -4.448231560871818e-09f, 0.9607092142105103f, 2.880505078906026e-08f}, \
  {-0.24740396440029144f, 5.145768700032249e-09f, 0.9689124226570129f, -9.463682060228962e-10f}, \
  {-0.21700957417488098f, -6.920129358434224e-09f, 0.9761694669723511f, 6.896283988311325e-09f}, \
  {-0.186403289437294f, -7.324975737077466e-09f, 0.9824733138084412f, -7.071859209339948e-10f}, \
  {-0.15561498701572418f, -5.757831988972839e-09f, 0.9878177642822266f, 1.9534246220587193e-08f}, \
  {-0.1246747300028801f, -3.3823475131811165e-09f, 0.9921976923942566f, -2.516492791926339e-08f}, \
  {-0.09361273050308228f, -7.324306161571315e-10f, 0.9956086874008179f, -9.428161584779104e-10f}, \
  {-0.0624593161046505f, -1.737729737882887e-09f, 0.9980475306510925f, -1.9950993745965206e-08f}, \
  {-0.03124491311609745f, -8.69228633515462e-10f, 0.9995117783546448f, -1.9869508705028238e-08f}, \
  {0.0f, 0.0f, 1.0f, 0.0f}, \
  {0.03124491311609745f, 8.69228633515462e-10f, 0.9995117783546448f, -1.9869508705028238e-08f}, \
  {0.0624593161046505f, 1.737729737882887e-09f, 0.9980475306510925f, -1.9950993745965206e-08f}, \
  {0.09361273050308228f, 7.324306161571315e-10f, 0.9956086874008179f, -9.428161584779104e-10f}, \
  {0.1246747300028801f, 3.3823475131811165e-09f, 0.9921976923942566f, -2.516492791926339e-08f}, \
  {0.15561498701572418f, 5.757831988972839e-09f, 0.9878177642822266f, 1.9534246220587193e-08f}, \
  {0.186403289437294f, 7.324975737077466e-09f, 0.9824733138084412f, -7.071859209339948e-10f}, \
  {0.21700957417488098f, 6.920129358434224e-09f, 0.9761694669723511f, 6.896283988311325e-09f}, \
  {0.24740396440029144f, -5.145768700032249e-09f, 0.9689124226570129f, -9.463682060228962e-10f}, \
  {0.27755674719810486f, 4.448231560871818e-09f, 0.9607092142105103f, 2.880505078906026e-08f}, \
  {0.30743852257728577f, -7.996904471951893e-09f, 0.9515679478645325f, 1.8363972842383447e-10f}, \
  {0.33702006936073303f, -3.384799662775606e-10f, 0.9414974451065063f, 1.8021374614818342e-08f}, \
  {0.36627253890037537f, -9.814328016943819e-09f, 0.9305076003074646f, 2.1604849465006737e-08f}, \
  {0.3951673209667206f, 9.274213397247877e-09f, 0.9186091423034668f, 1.3491451511526975e-08f}, \
  {0.4236762523651123f, 4.838825784503342e-09f, 0.9058136940002441f, -1.0574307651722847e-08f}, \
  {0.45177146792411804f, 3.5675657983347264e-09f, 0.8921337127685547f, -1.3401559861847545e-08f}, \
  {0.4794255495071411f, -1.0902938107903992e-08f, 0.8775825500488281f, 1.1841544633739431e-08f}, \
  {0.5066114664077759f, -1.1593518145502912e-08f, 0.8621744513511658f, 2.858371495051415e-08f}, \
  {0.5333026647567749f, 8.779244886625293e-09f, 0.8459244966506958f, 2.5803721381834066e-09f}, \
  {0.5594731569290161f, -2.568164880756285e-08f, 0.8288484811782837f, 6.431041921217684e-09f}, \
  {0.5850972533226013f, 1.9617861113374602e-08f, 0.8109630942344666f, 2.5270750825256982e-08f}, \
  {0.6101500988006592f, -2.1724867238503975e-08f, 0.7922858595848083f, 9.237019482633002e-11f}, \
  {0.6346070766448975f, 3.37037175945909e-09f, 0.7728349566459656f, -1.0493494073671172e-08f}, \
  {0.6584444046020508f, -4.691483201924029e-09f, 0.7526293992996216f, -2.6881554759938808e-08f}, \
  {0.681638777256012f, -1.723267750719515e-08f, 0.7316888570785522f, 1.1795268761716216e-08f}, \
  {0.7041674852371216f, 2.6217412241180682e-08f, 0.7100338935852051f, -1.0019125085136693e-08f}, \
  {0.7260086536407471f, 1.6199654950810327e-09f, 0.6876855492591858f, 1.2961319129090043e-08f}, \
}
/* 1/6 */
#define DF_INV6_HI 0.1666666716337204f
#define DF_INV6_LO -4.967053879312289e-09f
#if defined(__CUDACC__)
static __device__ const float dfl_exp2_tab_d[32][2] = DFL_EXP2_TAB;  /* 2^(j/32) */
static __device__ const float dfl_log_tab_d[47][4] = DFL_LOG_TAB;    /* c = 1 + j/64, j = -19..27: 1/c, log c */
static __device__ const float dfl_sc_tab_d[53][4] = DFL_SC_TAB;      /* a = j/32, j = -26..26: sin a, cos a */
#endif
static const float dfl_exp2_tab_h[32][2] = DFL_EXP2_TAB;
static const float dfl_log_tab_h[47][4] = DFL_LOG_TAB;
static const float dfl_sc_tab_h[53][4] = DFL_SC_TAB;
#if defined(__CUDA_ARCH__)
#define DFL_EXP2(j, i) dfl_exp2_tab_d[j][i]
#define DFL_LOGT(j, i) dfl_log_tab_d[j][i]
#define DFL_SCT(j, i) dfl_sc_tab_d[j][i]
#else
#define DFL_EXP2(j, i) dfl_exp2_tab_h[j][i]
#define DFL_LOGT(j, i) dfl_log_tab_h[j][i]
#define DFL_SCT(j, i) dfl_sc_tab_h[j][i]
#endif

/* ---- comparisons (the semantics of the FP64 comparisons on hi + lo) ---- */
DFN int dfl_lt(dfl a, dfl b) { return a.hi < b.hi || (a.hi == b.hi && a.lo < b.lo); }
DFN int dfl_eq(dfl a, dfl b) { return a.hi == b.hi && a.lo == b.lo; }

/* ---- exp ---- */
DFN dfl dfl_exp(dfl x) {
  if (x.hi != x.hi) return dfl_make(dfl_nanf(), 0.0f);
  if (x.hi > 88.72f) return dfl_make(dfl_inff(), 0.0f);
  if (x.hi < -103.5f) return dfl_make(0.0f, 0.0f);
  const float kf = rintf(DF_MUL(x.hi, 46.16624130844683f)); /* 32 / ln 2; |k| < 2^13 */
  /* r = x - k ln2/32, |r| <= ln2/64: x.hi - k C1 is exact (C1 and C2 have 11
   * bits), the leading sums are exact two-sums, only terms below 2^-24 of r
   * are added rounded */
  const float a1 = DF_FMA(-kf, DF_LN2_32_C1, x.hi);
  const dfl a2 = dfl_two_sum(a1, DF_MUL(-kf, DF_LN2_32_C2));
  const dfl p3 = dfl_two_prod(-kf, DF_LN2_32_C3);
  const dfl a3 = dfl_two_sum(a2.hi, p3.hi);
  const dfl a4 = dfl_two_sum(a3.hi, x.lo);
  const float rlo = DF_ADD(DF_ADD(DF_ADD(a2.lo, a3.lo), DF_ADD(p3.lo, a4.lo)), DF_MUL(-kf, DF_LN2_32_C4));
  const dfl r = dfl_fast_two_sum(a4.hi, rlo);
  /* expm1(r) = r + z P, z = r^2, P = 1/2 + r/6 + z (1/24 + r/120 + z/720):
   * z and r/6 as unnormalised pairs, 1/2 + r/6 by an exact two-sum, the z
   * term of P in FP32 (below 5e-6) */
  const float zh = DF_MUL(r.hi, r.hi);
  const float zl = DF_FMA(DF_ADD(r.hi, r.hi), r.lo, DF_FMA(r.hi, r.hi, -zh));
  const float p6h = DF_MUL(r.hi, DF_INV6_HI);
  const float p6l = DF_FMA(r.lo, DF_INV6_HI, DF_FMA(r.hi, DF_INV6_LO, DF_FMA(r.hi, DF_INV6_HI, -p6h)));
  const float pz = DF_MUL(zh, DF_FMA(zh, 1.3888889225e-3f, DF_FMA(r.hi, 8.333333768e-3f, 4.166666791e-2f)));
  const dfl ph = dfl_two_sum(0.5f, p6h);
  const float pl = DF_ADD(ph.lo, DF_ADD(p6l, pz));
  const float zph = DF_MUL(zh, ph.hi);
  const float zpl = DF_FMA(zl, ph.hi, DF_FMA(zh, pl, DF_FMA(zh, ph.hi, -zph)));
  const dfl e0 = dfl_fast_two_sum(r.hi, zph); /* |z P| <= 0.0055 |r| */
  const float eml = DF_ADD(e0.lo, DF_ADD(r.lo, zpl));
  /* 2^(j/32) (1 + em) 2^m, k = 32 m + j */
  const int k = (int)kf;
  const int jj = k & 31, m = (k - jj) / 32;
  const dfl t = dfl_make(DFL_EXP2(jj, 0), DFL_EXP2(jj, 1));
  const float teh = DF_MUL(t.hi, e0.hi);
  const float tel = DF_FMA(t.lo, e0.hi, DF_FMA(t.hi, eml, DF_FMA(t.hi, e0.hi, -teh)));
  const dfl u = dfl_two_sum(t.hi, teh);
  dfl e = dfl_fast_two_sum(u.hi, DF_ADD(u.lo, DF_ADD(t.lo, tel)));
  /* times 2^m in two exact steps (m in [-150, 128]) */
  const int m1 = m / 2, m2 = m - m1;
  e = dfl_scale(e, dfl_pow2(m1));
  e = dfl_scale(e, dfl_pow2(m2));
  if (!dfl_finite(e.hi)) e.lo = 0.0f;
  return e;
}

/* ---- log ---- */
/* x = m 2^e with m in [sqrt(1/2), sqrt(2)); x finite, > 0 and normal */
DFN dfl dfl_split_exp(dfl x, int* e) {
#if defined(__CUDA_ARCH__)
  int ex = ((__float_as_int(x.hi) >> 23) & 0xff) - 127;
#else
  int ex;
  frexpf(x.hi, &ex);
  ex -= 1;
#endif
  dfl m = dfl_scale(x, dfl_pow2(-ex));
  if (m.hi > 1.41421353816986083984f) {
    m = dfl_scale(m, 0.5f);
    ex += 1;
  }
  *e = ex;
  return m;
}
DFN dfl dfl_log(dfl x) {
  if (x.hi != x.hi || x.hi < 0.0f) return dfl_make(dfl_nanf(), 0.0f);
  if (x.hi == 0.0f) return dfl_make(-dfl_inff(), 0.0f);
  if (!dfl_finite(x.hi)) return dfl_make(dfl_inff(), 0.0f);
  int shift = 0;
  if (x.hi < 1e-30f) {  /* keep m and its low part normal: log(x) = log(x 2^64) - 64 ln 2 */
    x = dfl_scale(x, 18446744073709551616.0f);
    shift = 64;
  }
  int e;
  const dfl m = dfl_split_exp(x, &e);
  /* c = 1 + j/64 nearest to m (j in [-19, 27]); t = (m - c) / c, |t| <= 0.011 */
  const float jf = rintf(DF_MUL(DF_SUB(m.hi, 1.0f), 64.0f));
  const int J = (int)jf + 19;
  /* t = (m - c)/c: m.hi - c is exact, m - c normalised by a two-sum, times
   * 1/c (a pair) */
  const float c = DF_FMA(jf, 0.015625f, 1.0f);
  const dfl d = dfl_two_sum(DF_SUB(m.hi, c), m.lo);
  const float ih = DFL_LOGT(J, 0), il = DFL_LOGT(J, 1);
  const float th0 = DF_MUL(d.hi, ih);
  const dfl t = dfl_fast_two_sum(th0, DF_FMA(d.lo, ih, DF_FMA(d.hi, il, DF_FMA(d.hi, ih, -th0))));
  /* log1p(t) = t + z Q, z = t^2, Q = -1/2 + t/3 - z/4 + t z (1/5 - t/6 + z/7 - t z/8 + z^2/9):
   * z and t/3 as unnormalised pairs, -1/2 + t/3 - z/4 by exact two-sums, the
   * t z term in FP32 (below 3e-7) */
  const float zh = DF_MUL(t.hi, t.hi);
  const float zl = DF_FMA(DF_ADD(t.hi, t.hi), t.lo, DF_FMA(t.hi, t.hi, -zh));
  const float p3h = DF_MUL(t.hi, 0.3333333432674408f);
  const float p3l = DF_FMA(t.lo, 0.3333333432674408f,
                           DF_FMA(t.hi, -9.934107758624577e-09f, DF_FMA(t.hi, 0.3333333432674408f, -p3h)));
  const dfl q1 = dfl_two_sum(-0.5f, p3h);
  const dfl q2 = dfl_two_sum(q1.hi, DF_MUL(-0.25f, zh));
  const float inner = DF_FMA(DF_FMA(DF_FMA(DF_FMA(t.hi, 0.1111111119389534f, -0.125f), t.hi, 0.1428571492433548f),
                                    t.hi, -0.1666666716337204f),
                             t.hi, 0.2f);
  const float qt = DF_MUL(DF_MUL(t.hi, zh), inner);
  const float ql = DF_ADD(DF_ADD(q1.lo, q2.lo), DF_ADD(DF_FMA(-0.25f, zl, p3l), qt));
  const float zqh = DF_MUL(zh, q2.hi);
  const float zql = DF_FMA(zl, q2.hi, DF_FMA(zh, ql, DF_FMA(zh, q2.hi, -zqh)));
  const dfl l0 = dfl_fast_two_sum(t.hi, zqh); /* |z Q| <= 0.0057 |t| */
  /* + log c + (e - shift) ln 2: the leading parts by exact steps */
  const float ef = (float)(e - shift);
  const dfl a = dfl_two_prod(ef, 0.6931471824645996f);
  const dfl b = dfl_two_sum(a.hi, DFL_LOGT(J, 2));
  const dfl s = dfl_two_sum(b.hi, l0.hi);
  const float lo = DF_ADD(DF_ADD(DF_ADD(s.lo, b.lo), DF_ADD(a.lo, DF_MUL(ef, -1.9046542121259336e-09f))),
                          DF_ADD(DFL_LOGT(J, 3), DF_ADD(l0.lo, DF_ADD(t.lo, zql))));
  return dfl_fast_two_sum(s.hi, lo);
}

/* ---- sin / cos ---- */
/* r = x - k pi/2 with pi/2 = P1 + P2 + P3 + P4 (P1, P2 of 12 bits); returns
 * the quadrant k mod 4, or -1 when |k| >= 4096 (the reduction is not exact
 * there).  x.hi - k P1 is exact (both are multiples of the smaller one's ulp
 * and the difference is below 0.8), k P2 and k P3 are exact products, the
 * sums of the leading parts are exact two-sums, and only terms below 2^-24
 * of r are added in rounded arithmetic. */
DFN int dfl_reduce_half_pi(dfl x, dfl* r) {
  const float k = rintf(DF_MUL(x.hi, 0.6366197466850281f));
  if (!(fabsf(k) < 4096.0f)) return -1;
  const float a1 = DF_FMA(-k, 1.57080078125f, x.hi);
  const dfl a2 = dfl_two_sum(a1, DF_MUL(k, 4.453584551811218e-06f));
  const dfl p3 = dfl_two_prod(-k, -8.705515752716053e-10f);
  const dfl a3 = dfl_two_sum(a2.hi, p3.hi);
  const dfl a4 = dfl_two_sum(a3.hi, x.lo);
  const float rl = DF_ADD(DF_ADD(DF_ADD(a2.lo, a3.lo), DF_ADD(p3.lo, a4.lo)), DF_MUL(-k, 5.721188916458728e-18f));
  *r = dfl_fast_two_sum(a4.hi, rl);
  const int ki = (int)k;
  return ki & 3;
}
/* sin(x + shift pi/2), shift 0 (sin) or 1 (cos), in one path for every
 * quadrant: x = k pi/2 + r, r = j/32 + s with |s| <= 1/64, sin(j/32) and
 * cos(j/32) from a table, and sin(x + shift pi/2) = A cos s + B sin s with
 * (A, B) = (S, C), (C, -S), (-S, -C), (-C, S) for the quadrant k + shift;
 * sin s = s + s q with q = -s^2/6 + s^4 (1/120 - s^2/5040) and cos s - 1 =
 * -s^2/2 + s^4 (1/24 - s^2/720).  Intermediates are unnormalised pairs: a
 * rounded leading part, and a low part gathering the exact product and sum
 * errors with the small terms (s^2/6 and s^2/2 carried as pairs, the s^4
 * terms in FP32); the relative weight of every rounded low-part term is
 * below 2^-40, so the result keeps about 2^-47. */
DFN dfl dfl_sincos(dfl x, int shift) {
  if (!dfl_finite(x.hi)) return dfl_make(dfl_nanf(), 0.0f);
  dfl r;
  const int q0 = dfl_reduce_half_pi(x, &r);
  if (q0 < 0) return dfl_make(dfl_nanf(), 0.0f);
  const int q = (q0 + shift) & 3;
  const float jf = rintf(DF_MUL(r.hi, 32.0f));
  const int J = (int)jf + 26;
  const dfl s = dfl_two_sum(DF_FMA(-jf, 0.03125f, r.hi), r.lo); /* r.hi - j/32 is exact */
  /* z = s^2 */
  const float zh = DF_MUL(s.hi, s.hi);
  const float zl = DF_FMA(DF_ADD(s.hi, s.hi), s.lo, DF_FMA(s.hi, s.hi, -zh));
  /* q = -z/6 + z^2 (1/120 - z/5040) */
  const float qh = DF_MUL(-zh, DF_INV6_HI);
  const float ql = DF_FMA(-zl, DF_INV6_HI, DF_FMA(-zh, DF_INV6_LO, DF_FMA(-zh, DF_INV6_HI, -qh)));
  const float q4 = DF_MUL(DF_MUL(zh, zh), DF_FMA(zh, -1.9841270113829523e-04f, 8.333333767950535e-03f));
  /* sin s = s + s q, |s q| <= 4.1e-5 |s| */
  const float sqh = DF_MUL(s.hi, qh);
  const float sql = DF_FMA(s.lo, qh, DF_FMA(s.hi, DF_ADD(ql, q4), DF_FMA(s.hi, qh, -sqh)));
  const dfl sn = dfl_fast_two_sum(s.hi, sqh);
  const float snl = DF_ADD(sn.lo, DF_ADD(s.lo, sql));
  /* cos s - 1 = ch + cl */
  const float ch = DF_MUL(-0.5f, zh);
  const float cl = DF_FMA(-0.5f, zl, DF_MUL(DF_MUL(zh, zh), DF_FMA(zh, -1.3888889225199819e-03f, 4.1666667908430099e-02f)));
  const dfl S = dfl_make(DFL_SCT(J, 0), DFL_SCT(J, 1)), C = dfl_make(DFL_SCT(J, 2), DFL_SCT(J, 3));
  dfl A = (q & 1) ? C : S, B = (q & 1) ? S : C;
  if (q & 2) A = dfl_neg(A);
  if ((q + 1) & 2) B = dfl_neg(B);
  /* T = A (cos s - 1) + B sin s, then A + T */
  const float ah = DF_MUL(A.hi, ch);
  const float al = DF_FMA(A.lo, ch, DF_FMA(A.hi, cl, DF_FMA(A.hi, ch, -ah)));
  const float bh = DF_MUL(B.hi, sn.hi);
  const float bl = DF_FMA(B.lo, sn.hi, DF_FMA(B.hi, snl, DF_FMA(B.hi, sn.hi, -bh)));
  const dfl t = dfl_two_sum(bh, ah);
  const float tl = DF_ADD(t.lo, DF_ADD(al, bl));
  const dfl u = dfl_two_sum(A.hi, t.hi);
  return dfl_fast_two_sum(u.hi, DF_ADD(u.lo, DF_ADD(A.lo, tl)));
}
DFN dfl dfl_sin(dfl x) { return dfl_sincos(x, 0); }
DFN dfl dfl_cos(dfl x) { return dfl_sincos(x, 1); }

#endif
