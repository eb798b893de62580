// Batched mixed-precision fitness path.
//
// Same contract as the plain path (tune_constants + fitness of
// rils_rols_cpp.cpp:445-541 for every candidate of a round), different
// arithmetic:
//   gram pass     X row tiles are staged in shared memory by TMA bulk copies
//                 (cp.async.bulk + mbarrier) and shared by every candidate of
//                 a work unit; one warp interprets one candidate's factor
//                 programs on 4 rows per lane in FP32 and accumulates the
//                 factor Gram matrix, the factor sums and X^T y as exact
//                 products (FMA TwoProduct) added into double-float (hi, lo)
//                 pairs; warps reduce with double-float shuffles and write
//                 one partial per tile;
//   solve         one warp per candidate: FP64 reduction of the tile partials,
//                 symmetric-pivoted Cholesky in FP64 (pivot = largest
//                 remaining column norm, as in column-pivoted QR), one step of
//                 iterative refinement; ill-conditioned systems are queued for
//                 the FP64 QR path;
//   residual pass re-evaluates the factors in FP32 and forms the rebuilt sum
//                 sum_i c_i f_i (drop / snap rules of rils_rols_cpp.cpp:488-517)
//                 in double-float arithmetic against a double-float y; the
//                 squared residuals are summed with compensation per lane and
//                 in FP64 across tiles (finalize_kernel).
#include <cfloat>
#include <cstdint>

#include "../common/rr_math.h"
#include "common.cuh"
#include "mixed.cuh"
#include "plain.cuh"
#include "reduce.cuh"

namespace rrd {

namespace {

// ---------------------------------------------------------------- PTX ----
__device__ __forceinline__ uint32_t smem_u32(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* bar, uint32_t parity) {
  uint32_t ok;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}\n"
      : "=r"(ok)
      : "r"(smem_u32(bar)), "r"(parity)
      : "memory");
  return ok != 0;
}
// 1-D TMA bulk copy global -> shared, completion counted on `bar`.
// dst, src 16-byte aligned; bytes a multiple of 16.
__device__ __forceinline__ void tma_bulk_g2s(void* dst, const void* src, uint32_t bytes, uint64_t* bar) {
  asm volatile(
      "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(smem_u32(dst)),
      "l"(src), "r"(bytes), "r"(smem_u32(bar))
      : "memory");
}
__device__ __forceinline__ void fence_proxy_async() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

// Bounded wait: about 2^24 polls (seconds), then the caller reports ST_WAIT_TIMEOUT.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* bar, uint32_t parity) {
  for (uint32_t it = 0; it < (1u << 24); ++it) {
    if (mbar_try_wait(bar, parity)) return true;
    if (it > 64) __nanosleep(64);
  }
  return false;
}

// ------------------------------------------------------ FP32 arithmetic ----
__device__ __forceinline__ float bin32(int base, float a, float b) {
  switch (base) {
    case RRG_ADD: return __fadd_rn(a, b);
    case RRG_SUB: return __fsub_rn(a, b);
    case RRG_MUL: return __fmul_rn(a, b);
    case RRG_DIV: return __fdiv_rn(a, b);
    case RRG_POW: return powf(a, b);
    case RRG_LT: return a < b ? 1.f : 0.f;
    case RRG_EQ: return a == b ? 1.f : 0.f;
    case RRG_NE: return a != b ? 1.f : 0.f;
    case RRG_MIN: return a < b ? a : b;
    case RRG_MAX: return a > b ? a : b;
    default: return __int_as_float(0x7fc00000);
  }
}

#define V4(expr_x, expr_y, expr_z, expr_w) make_float4(expr_x, expr_y, expr_z, expr_w)
#define MAP4(f, v) V4(f((v).x), f((v).y), f((v).z), f((v).w))
#define ZIP4(base, a, b) V4(bin32(base, (a).x, (b).x), bin32(base, (a).y, (b).y), bin32(base, (a).z, (b).z), bin32(base, (a).w, (b).w))

__device__ __forceinline__ float sqr32(float a) { return __fmul_rn(a, a); }

// sin / cos in FP32: Cody-Waite reduction by pi/2 with a three-term split
// of pi/2 (each product folded in by one FMA), then the Taylor polynomials
// of sin (to r^11) and cos (to r^10) on |r| <= pi/4.  About 1 ulp for
// |x| up to ~1e6; beyond that an FP32 argument no longer determines the
// FP64 result anyway, and the reduction simply degrades (no slow path).
__device__ __forceinline__ void sincos_kernel32(float r, float& s, float& c) {
  const float r2 = __fmul_rn(r, r);
  float ps = __fmaf_rn(r2, -2.5052108385441720e-08f, 2.7557319223985893e-06f);
  ps = __fmaf_rn(r2, ps, -1.9841269841269841e-04f);
  ps = __fmaf_rn(r2, ps, 8.3333333333333333e-03f);
  ps = __fmaf_rn(r2, ps, -1.6666666666666667e-01f);
  s = __fmaf_rn(__fmul_rn(r2, r), ps, r);
  float pc = __fmaf_rn(r2, -2.7557319223985891e-07f, 2.4801587301587302e-05f);
  pc = __fmaf_rn(r2, pc, -1.3888888888888889e-03f);
  pc = __fmaf_rn(r2, pc, 4.1666666666666667e-02f);
  pc = __fmaf_rn(r2, pc, -0.5f);
  c = __fmaf_rn(r2, pc, 1.0f);
}
__device__ __forceinline__ int reduce_half_pi(float x, float& r) {
  const float k = rintf(__fmul_rn(x, 0.63661977236758134f));
  r = __fmaf_rn(-k, 1.5707963705062866f, x);
  r = __fmaf_rn(-k, -4.371138828673793e-08f, r);
  r = __fmaf_rn(-k, -1.7151245100058819e-15f, r);
  // quadrant k mod 4 (exact for |k| < 2^24; larger k only picks a sign)
  const float k4 = __fsub_rn(k, __fmul_rn(4.0f, floorf(__fmul_rn(k, 0.25f))));
  return (int)k4 & 3;
}
__device__ __forceinline__ float sin32(float x) {
  float r, s, c;
  const int q = reduce_half_pi(x, r);
  sincos_kernel32(r, s, c);
  const float v = (q & 1) ? c : s;
  return (q & 2) ? -v : v;
}
__device__ __forceinline__ float cos32(float x) {
  float r, s, c;
  const int q = reduce_half_pi(x, r);
  sincos_kernel32(r, s, c);
  const float v = (q & 1) ? s : c;
  return ((q + 1) & 2) ? -v : v;
}
__device__ __forceinline__ float sqrt32(float a) { return __fsqrt_rn(a); }

// double-float helpers (Knuth TwoSum, Dekker Fast2Sum, FMA TwoProduct)
struct DF {
  float hi, lo;
};
__device__ __forceinline__ DF two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  const float bb = __fsub_rn(s, a);
  const float e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bb)), __fsub_rn(b, bb));
  return DF{s, e};
}
__device__ __forceinline__ DF fast_two_sum(float a, float b) {
  const float s = __fadd_rn(a, b);
  return DF{s, __fsub_rn(b, __fsub_rn(s, a))};
}
__device__ __forceinline__ DF df_add(DF x, DF y) {
  DF s = two_sum(x.hi, y.hi);
  s.lo = __fadd_rn(s.lo, __fadd_rn(x.lo, y.lo));
  return fast_two_sum(s.hi, s.lo);
}
__device__ __forceinline__ DF df_mul_f(float chi, float clo, float f) {
  const float p = __fmul_rn(chi, f);
  float e = __fmaf_rn(chi, f, -p);
  e = __fmaf_rn(clo, f, e);
  return fast_two_sum(p, e);
}
__device__ __forceinline__ void kahan(float& s, float& c, float x) {
  const float y = __fsub_rn(x, c);
  const float t = __fadd_rn(s, y);
  c = __fsub_rn(__fsub_rn(t, s), y);
  s = t;
}
// (hi, lo) += a * b exactly rounded into a double-float: TwoProduct by FMA,
// TwoSum of the high parts, low parts added plainly.
__device__ __forceinline__ void acc_prod(float& hi, float& lo, float a, float b) {
  const float p = __fmul_rn(a, b);
  const float e = __fmaf_rn(a, b, -p);
  const DF s = two_sum(hi, p);
  hi = s.hi;
  lo = __fadd_rn(lo, __fadd_rn(s.lo, e));
}
__device__ __forceinline__ void acc_sum(float& hi, float& lo, float a) {
  const DF s = two_sum(hi, a);
  hi = s.hi;
  lo = __fadd_rn(lo, s.lo);
}

template <int MMAX>
struct GramSize {
  static constexpr int G = MMAX * (MMAX + 1) / 2;
  static constexpr int E = G + 2 * MMAX;
};

// ----------------------------------------------------------- evaluator ----
// Interprets one candidate's code on 4 consecutive rows per lane (row offset
// `r` inside the staged tile); factor slot s lands in f[s].
template <int MMAX>
__device__ __forceinline__ bool eval4(const uint32_t* code, int len, const float* __restrict__ K,
                                      const float* xs, int tile, int r, float4* st, float4 (&f)[MMAX]) {
  float4 tos = make_float4(0.f, 0.f, 0.f, 0.f);
  int sp = 0;
  if (len <= 0) return true;
  uint32_t w = code[0];
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t wn = pc + 1 < len ? code[pc + 1] : 0u;
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = *reinterpret_cast<const float4*>(xs + (size_t)arg * tile + r); break;
      case RRG_OP_LDC: { const float k = __ldg(K + arg); tos = make_float4(k, k, k, k); } break;
      case RRG_OP_PSV:
        if (sp >= kMixedStackCap) return false;
        st[32 * sp++] = tos;
        tos = *reinterpret_cast<const float4*>(xs + (size_t)arg * tile + r);
        break;
      case RRG_OP_PSC: {
        if (sp >= kMixedStackCap) return false;
        st[32 * sp++] = tos;
        const float k = __ldg(K + arg);
        tos = make_float4(k, k, k, k);
      } break;
      case RRG_OP_SIN: tos = MAP4(sin32, tos); break;
      case RRG_OP_COS: tos = MAP4(cos32, tos); break;
      case RRG_OP_LN: tos = MAP4(logf, tos); break;
      case RRG_OP_EXP: tos = MAP4(expf, tos); break;
      case RRG_OP_SQRT: tos = MAP4(sqrt32, tos); break;
      case RRG_OP_SQR: tos = MAP4(sqr32, tos); break;
      case RRG_OP_EMIT:
#pragma unroll
        for (int s = 0; s < MMAX; ++s)
          if ((int)arg == s) f[s] = tos;
        sp = 0;
        break;
      default: {
        const int kk = op - RRG_OP_BIN;
        const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
        float4 o;
        if (src == RRG_SRC_S) {
          if (sp <= 0) return false;
          o = st[32 * --sp];
        } else if (src == RRG_SRC_V) {
          o = *reinterpret_cast<const float4*>(xs + (size_t)arg * tile + r);
        } else {
          const float k = __ldg(K + arg);
          o = make_float4(k, k, k, k);
        }
        tos = dir == RRG_DIR_N ? ZIP4(base, o, tos) : ZIP4(base, tos, o);
      }
    }
    w = wn;
  }
  return true;
}

// --------------------------------------------------------- tile staging ----
struct TileSmem {
  float* xs;       // d columns x tile rows
  float* yh;       // tile rows
  float* yl;       // tile rows (residual pass)
  float4* stacks;  // [warp][kMixedStackCap][32]
  uint32_t* codes; // [warp][kMixedCodeCap]
  uint64_t* bar;
  int* counter;
  int* abort_flag;
};

__device__ __forceinline__ TileSmem carve(unsigned char* smem, int d, int tile, int nwarps, bool resid) {
  TileSmem t;
  size_t off = 0;
  t.bar = reinterpret_cast<uint64_t*>(smem + off);
  off += 16;
  t.counter = reinterpret_cast<int*>(smem + off);
  off += 16;
  t.abort_flag = reinterpret_cast<int*>(smem + off);
  off += 96;  // keep 128-byte alignment of what follows
  t.xs = reinterpret_cast<float*>(smem + off);
  off += sizeof(float) * (size_t)d * tile;
  t.yh = reinterpret_cast<float*>(smem + off);
  off += sizeof(float) * tile;
  t.yl = reinterpret_cast<float*>(smem + off);
  if (resid) off += sizeof(float) * tile;
  t.stacks = reinterpret_cast<float4*>(smem + off);
  off += sizeof(float4) * kMixedStackCap * 32 * nwarps;
  t.codes = reinterpret_cast<uint32_t*>(smem + off);
  return t;
}

// thread 0: issue the TMA bulk copies of tile q (X columns, y hi [, y lo])
__device__ __forceinline__ void issue_tile(const TileSmem& t, const DevData& ds, int q, int tile, bool resid) {
  const int64_t row0 = (int64_t)q * tile;
  const int64_t rows = min((int64_t)tile, ds.n_pad - row0);
  const uint32_t bytes = (uint32_t)(rows * sizeof(float));
  const uint32_t total = bytes * (ds.d + 1 + (resid ? 1 : 0));
  fence_proxy_async();
  mbar_expect_tx(t.bar, total);
  for (int j = 0; j < ds.d; ++j) tma_bulk_g2s(t.xs + (size_t)j * tile, ds.X32 + (int64_t)j * ds.n_pad + row0, bytes, t.bar);
  tma_bulk_g2s(t.yh, ds.y32 + row0, bytes, t.bar);
  if (resid) tma_bulk_g2s(t.yl, ds.y32lo + row0, bytes, t.bar);
}

}  // namespace

// ------------------------------------------------------------ kernels ----
template <int MMAX, int NWARPS, bool RESID>
__global__ void __launch_bounds__(NWARPS * 32, 1) mixed_pass_kernel(MixedArgs a) {
  extern __shared__ __align__(128) unsigned char smem_raw[];
  constexpr int E = GramSize<MMAX>::E;
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int tile = a.tile;
  TileSmem t = carve(smem_raw, a.ds.d, tile, NWARPS, RESID);
  if (threadIdx.x == 0) {
    mbar_init(t.bar, 1);
    *t.abort_flag = 0;
  }
  fence_proxy_async();
  __syncthreads();
  float4* st = t.stacks + (size_t)warp * kMixedStackCap * 32 + lane;
  uint32_t* code_w = t.codes + (size_t)warp * kMixedCodeCap;
  uint32_t phase = 0;

  for (int unit = blockIdx.x; unit < a.n_units; unit += gridDim.x) {
    const int q = unit % a.n_tiles, g = unit / a.n_tiles;
    if (threadIdx.x == 0) {
      *t.counter = 0;
      issue_tile(t, a.ds, q, tile, RESID);
    }
    // every thread waits on the tile (bounded)
    if (!mbar_wait_bounded(t.bar, phase)) atomicExch(t.abort_flag, 1);
    phase ^= 1;
    __syncthreads();
    if (*t.abort_flag) {
      if (threadIdx.x == 0) atomicOr(a.status, ST_WAIT_TIMEOUT);
      return;
    }
    const int64_t row0 = (int64_t)q * tile;
    const int rows_here = (int)min((int64_t)tile, a.ds.n_pad - row0);
    const int c_lo = g * a.group, c_hi = min(a.n_list, c_lo + a.group);
    for (;;) {
      int li = 0;
      if (lane == 0) li = atomicAdd(t.counter, 1);
      li = __shfl_sync(0xffffffffu, li, 0) + c_lo;
      if (li >= c_hi) break;
      const int c = a.list[li];
      const rrg_cand cd = a.b.cands[c];
      const bool tuned = cd.mode == RRG_TUNED;
      // stage the candidate's code for this warp
      const uint32_t* code = a.b.code + cd.code_offset;
      if (cd.code_len <= kMixedCodeCap) {
        for (int i = lane; i < cd.code_len; i += 32) code_w[i] = code[i];
        __syncwarp();
        code = code_w;
      }
      float4 f[MMAX];
#pragma unroll
      for (int s = 0; s < MMAX; ++s) f[s] = make_float4(0.f, 0.f, 0.f, 0.f);

      if (!RESID) {
        // exact products (FMA TwoProduct) accumulated in double-float (hi, lo)
        float acc_h[E], acc_l[E];
#pragma unroll
        for (int e = 0; e < E; ++e) acc_h[e] = acc_l[e] = 0.f;
        for (int r = lane * 4; r < rows_here; r += 128) {
          if (!eval4<MMAX>(code, cd.code_len, a.b.consts32, t.xs, tile, r, st, f)) {
            atomicOr(a.status, ST_STACK);
            break;
          }
          float4 yv = *reinterpret_cast<const float4*>(t.yh + r);
          const int64_t gr = row0 + r;
          const bool m0 = gr < a.ds.n, m1 = gr + 1 < a.ds.n, m2 = gr + 2 < a.ds.n, m3 = gr + 3 < a.ds.n;
#pragma unroll
          for (int s = 0; s < MMAX; ++s) {
            f[s].x = m0 ? f[s].x : 0.f;
            f[s].y = m1 ? f[s].y : 0.f;
            f[s].z = m2 ? f[s].z : 0.f;
            f[s].w = m3 ? f[s].w : 0.f;
          }
          {
            // remember the first row with a NaN factor value (the solve
            // re-evaluates that row in FP64 to tell a domain error from an
            // FP32 breakdown)
            bool nan_any = false;
            int first = 4;
#pragma unroll
            for (int s = 0; s < MMAX; ++s) {
              if (f[s].w != f[s].w) first = 3;
              if (f[s].z != f[s].z) first = 2;
              if (f[s].y != f[s].y) first = 1;
              if (f[s].x != f[s].x) first = 0;
            }
            nan_any = first < 4;
            if (nan_any && a.nanrow) atomicMin(reinterpret_cast<unsigned long long*>(a.nanrow + c),
                                               (unsigned long long)(gr + first));
          }
          yv.x = m0 ? yv.x : 0.f;
          yv.y = m1 ? yv.y : 0.f;
          yv.z = m2 ? yv.z : 0.f;
          yv.w = m3 ? yv.w : 0.f;
          int e = 0;
#pragma unroll
          for (int i = 0; i < MMAX; ++i) {
#pragma unroll
            for (int j = i; j < MMAX; ++j) {
              acc_prod(acc_h[e], acc_l[e], f[i].x, f[j].x);
              acc_prod(acc_h[e], acc_l[e], f[i].y, f[j].y);
              acc_prod(acc_h[e], acc_l[e], f[i].z, f[j].z);
              acc_prod(acc_h[e], acc_l[e], f[i].w, f[j].w);
              ++e;
            }
          }
#pragma unroll
          for (int i = 0; i < MMAX; ++i) {
            constexpr int G = GramSize<MMAX>::G;
            acc_sum(acc_h[G + i], acc_l[G + i], f[i].x);
            acc_sum(acc_h[G + i], acc_l[G + i], f[i].y);
            acc_sum(acc_h[G + i], acc_l[G + i], f[i].z);
            acc_sum(acc_h[G + i], acc_l[G + i], f[i].w);
            acc_prod(acc_h[G + MMAX + i], acc_l[G + MMAX + i], f[i].x, yv.x);
            acc_prod(acc_h[G + MMAX + i], acc_l[G + MMAX + i], f[i].y, yv.y);
            acc_prod(acc_h[G + MMAX + i], acc_l[G + MMAX + i], f[i].z, yv.z);
            acc_prod(acc_h[G + MMAX + i], acc_l[G + MMAX + i], f[i].w, yv.w);
          }
        }
        // double-float warp reduction
        float2* out = a.gram + ((size_t)li * a.n_tiles + q) * E;
#pragma unroll
        for (int e = 0; e < E; ++e) {
          DF v = fast_two_sum(acc_h[e], acc_l[e]);
#pragma unroll
          for (int o = 16; o > 0; o >>= 1) {
            DF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
            v = df_add(v, w);
          }
          if (lane == (e & 31)) out[e] = make_float2(v.hi, v.lo);
        }
      } else {
        // residual pass: coefficients (double-float) and term kinds
        const MixedTerm& tm = a.terms[c];
        const int m = cd.n_factors;
        float ssum = 0.f, scomp = 0.f;
        for (int r = lane * 4; r < rows_here; r += 128) {
          if (!eval4<MMAX>(code, cd.code_len, a.b.consts32, t.xs, tile, r, st, f)) {
            atomicOr(a.status, ST_STACK);
            break;
          }
          const float4 yh = *reinterpret_cast<const float4*>(t.yh + r);
          const float4 yl = *reinterpret_cast<const float4*>(t.yl + r);
          const int64_t gr = row0 + r;
          float sq4 = 0.f;
#pragma unroll
          for (int u = 0; u < 4; ++u) {
            DF yp{0.f, 0.f};
            if (tuned) {
              bool have = false;
#pragma unroll
              for (int i = 0; i <= MMAX; ++i) {
                if (i > m) break;
                const int kd = tm.kind[i];
                if (kd == 0) continue;
                float fv = 0.f;
#pragma unroll
                for (int s = 0; s < MMAX; ++s)
                  if (s == i) fv = u == 0 ? f[s].x : (u == 1 ? f[s].y : (u == 2 ? f[s].z : f[s].w));
                DF term;
                if (kd == 1) term = DF{tm.hi[i], tm.lo[i]};
                else if (kd == 2) term = DF{fv, 0.f};
                else term = df_mul_f(tm.hi[i], tm.lo[i], fv);
                yp = have ? df_add(yp, term) : term;
                have = true;
              }
            } else {
              yp.hi = u == 0 ? f[0].x : (u == 1 ? f[0].y : (u == 2 ? f[0].z : f[0].w));
            }
            const float yhu = u == 0 ? yh.x : (u == 1 ? yh.y : (u == 2 ? yh.z : yh.w));
            const float ylu = u == 0 ? yl.x : (u == 1 ? yl.y : (u == 2 ? yl.z : yl.w));
            const DF e = df_add(DF{yhu, ylu}, DF{-yp.hi, -yp.lo});
            const float ev = __fadd_rn(e.hi, e.lo);
            const float sq = gr + u < a.ds.n ? __fmul_rn(ev, ev) : 0.f;
            sq4 = __fadd_rn(sq4, sq);
          }
          kahan(ssum, scomp, sq4);
        }
        DF v{ssum, -scomp};
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
          DF w{__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o)};
          v = df_add(v, w);
        }
        if (lane == 0) a.sse[(size_t)c * a.n_tiles + q] = (double)v.hi + (double)v.lo;
      }
      __syncwarp();
    }
    __syncthreads();  // the tile buffer is reused by the next unit
  }
}

template <int MM>
__device__ bool probe_eval64(const uint32_t* code, int len, const double* K, const DevData& ds, int64_t row,
                             double (&f)[MM]);

// One warp per candidate: FP64 reduction of the Gram partials; tuned
// candidates get a symmetric-pivoted Cholesky solve with one refinement step.
// Every candidate then gets its SSE from the Gram identity
//     SSE = y'y - 2 c'b + c'Gc      (c: coefficients after the drop / snap rules)
// when its bound  u * (y'y + 2|c|'|b| + |c|'|G||c|)  is below pass2_tol * SSE;
// otherwise it is flagged for the residual pass.
__global__ void __launch_bounds__(128) mixed_solve_kernel(SolveArgs a) {
  __shared__ double red[4][GramSize<kMixedMaxM>::E];
  const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
  const int li = blockIdx.x * 4 + warp;
  if (li >= a.n_list) return;
  const int mmax = a.mmax;
  const int Gn = mmax * (mmax + 1) / 2, E = Gn + 2 * mmax;
  const float2* part = a.gram + (size_t)li * a.n_tiles * E;
  for (int e = lane; e < E; e += 32) {
    double s = 0.0;
    for (int q = 0; q < a.n_tiles; ++q) {
      const float2 p = part[(size_t)q * E + e];
      s = __dadd_rn(s, __dadd_rn((double)p.x, (double)p.y));
    }
    red[warp][e] = s;
  }
  __syncwarp();
  if (lane != 0) return;
  const int c = a.list[li];
  const rrg_cand cd = a.b.cands[c];
  const double* ent = red[warp];
  const double yy = a.ds.yy;
  const double kU = 1e-11;  // relative accuracy of the double-float Gram sums
  auto queue_fallback = [&](int why) {
    const int slot = atomicAdd(a.fallback, 1);
    if (slot < a.fallback_cap) a.fallback[1 + slot] = c;
    if (a.reasons) atomicAdd(a.reasons + why, 1u);
  };
  const ProbeOut pr = a.probe[c];
  const double n_d = (double)a.ds.n;
  // certification: bound on the relative error of the penalised fitness
  // (1 + loss)(1 + rmse)(1 + size * cp) caused by FP32 evaluation, from the
  // per-row bound E on the error of the rebuilt sum (independent of cp)
  auto cert_bound = [&](double sse, double E) {
    if (!(sse >= 0.0) || !(E >= 0.0)) return 1e300;
    const double dsse = 2.0 * sqrt(sse * n_d) * E + n_d * E * E;
    const double loss = sse / a.ds.sst, rmse = sqrt(sse / n_d);
    const double rl = (dsse / a.ds.sst) / (1.0 + loss);
    const double rr = (sqrt((sse + dsse) / n_d) - rmse) / (1.0 + rmse);
    return rl + rr;
  };
  // per-row error bound of factor i: the largest probed deviation with a
  // safety factor (exact maximum when every row was probed)
  const double safety = pr.all_rows ? 1.5 : 8.0;
  auto ferr = [&](int i) { return safety * (double)pr.dev[i] + 1e-7 * (double)pr.rms[i]; };
  if (cd.mode != RRG_TUNED) {
    // yp = f: SSE = y'y - 2 f'y + f'f
    const double ff = ent[0], fs = ent[Gn], fy = ent[Gn + mmax];
    const bool nan = ff != ff || fs != fs || fy != fy;
    const bool inf = !nan && (fabs(ff) > DBL_MAX || fabs(fs) > DBL_MAX || fabs(fy) > DBL_MAX);
    uint32_t confirmed = pr.nan64;
    if (nan && !(confirmed & 1u) && a.nanrow && a.nanrow[c] >= 0 && a.nanrow[c] < a.ds.n) {
      double f64[kMixedMaxM];
      for (int i = 0; i < kMixedMaxM; ++i) f64[i] = 0.0;
      if (probe_eval64<kMixedMaxM>(a.b.code + cd.code_offset, cd.code_len, a.b.consts, a.ds, a.nanrow[c], f64) &&
          f64[0] != f64[0])
        confirmed |= 1u;
    }
    uint8_t p2 = 0;
    double sse;
    if (pr.bad32 || pr.inf64 || inf || (nan && !(confirmed & 1u))) {
      // FP32 broke down, FP64 overflows, or an FP32 NaN that the FP64 probe
      // does not confirm: the FP64 path scores it
      queue_fallback(pr.bad32 ? FB_PROBE_NONFINITE
                              : (pr.inf64 ? FB_FP64_INF : (inf ? FB_FP32_OVERFLOW : FB_OTHER_NAN)));
      sse = -1.0;
    } else if (nan || (pr.nan64 & 1u)) {
      sse = __longlong_as_double(0x7ff8000000000000ll);
    } else {
      sse = __dadd_rn(__dsub_rn(yy, __dmul_rn(2.0, fy)), ff);
      const double bound = kU * (yy + 2.0 * fabs(fy) + ff);
      if (!(sse > 0.0 && bound <= a.pass2_tol * sse)) {
        if (a.certify) queue_fallback(FB_ONE_PASS);
        else p2 = 1;
        sse = -1.0;
      } else if (a.certify && cert_bound(sse, ferr(0)) > a.cert_tol) {
        queue_fallback(FB_CERT);
        sse = -1.0;
      }
    }
    a.sse1[c] = sse;
    a.pass2[c] = p2;
    a.res[c].rank = 0;
    return;
  }
  const int m = cd.n_factors, k = m + 1;
  double G[kMixedMaxM + 1][kMixedMaxM + 1], L[kMixedMaxM + 1][kMixedMaxM + 1], bvec[kMixedMaxM + 1];
  int e = 0;
  for (int i = 0; i < mmax; ++i)
    for (int j = i; j < mmax; ++j, ++e)
      if (i < m && j < m) G[i][j] = G[j][i] = ent[e];
  for (int i = 0; i < m; ++i) {
    G[i][m] = G[m][i] = ent[Gn + i];
    bvec[i] = ent[Gn + mmax + i];
  }
  G[m][m] = (double)a.ds.n;
  bvec[m] = a.ds.ysum;
  // Non-finite sums: NaN (a domain error in some factor) gives NaN
  // coefficients and so the fitness sentinel, as the reference's QR does;
  // +-inf without NaN (FP32 overflow) is re-solved by the FP64 path.
  bool has_nan = false, has_inf = false;
  for (int i = 0; i < k; ++i) {
    for (int j = 0; j < k; ++j) {
      has_nan |= G[i][j] != G[i][j];
      has_inf |= fabs(G[i][j]) > DBL_MAX;
    }
    has_nan |= bvec[i] != bvec[i];
    has_inf |= fabs(bvec[i]) > DBL_MAX;
  }
  // factors whose own sums are NaN (a domain error on some row); the cross
  // sums of a NaN factor are NaN for every partner, so only the diagonal,
  // the factor sum and the factor-y sum identify it
  uint32_t nanmask = 0, infmask = 0;
  for (int i = 0; i < m; ++i) {
    const double d = G[i][i], sf = G[i][m], sy = bvec[i];
    if (d != d || sf != sf || sy != sy) nanmask |= 1u << i;
    else if (fabs(d) > DBL_MAX || fabs(sf) > DBL_MAX || fabs(sy) > DBL_MAX) infmask |= 1u << i;
  }
  const uint32_t fullmask = (m >= 32) ? 0xffffffffu : ((1u << m) - 1u);
  uint32_t confirmed = pr.nan64;
  if ((nanmask & ~confirmed) && a.nanrow && a.nanrow[c] >= 0 && a.nanrow[c] < a.ds.n) {
    // FP32 NaN outside the probe rows: evaluate the first such row in FP64
    double f64[kMixedMaxM];
    for (int i = 0; i < kMixedMaxM; ++i) f64[i] = 0.0;
    if (probe_eval64<kMixedMaxM>(a.b.code + cd.code_offset, cd.code_len, a.b.consts, a.ds, a.nanrow[c], f64))
      for (int i = 0; i < m; ++i)
        if (f64[i] != f64[i]) confirmed |= 1u << i;
  }
  nanmask |= pr.nan64 & fullmask;
  if (pr.bad32 || pr.inf64 || infmask || (nanmask & ~confirmed) ||
      (!nanmask && (has_nan || has_inf))) {
    // FP32 broke down where FP64 did not, FP64 overflow, FP32 overflow, an
    // FP32 NaN the FP64 probe does not confirm, or a non-finite sum outside
    // the factor columns: the FP64 path scores it
    queue_fallback(pr.bad32 ? FB_PROBE_NONFINITE
                            : (pr.inf64 ? FB_FP64_INF : (infmask ? FB_FP32_OVERFLOW : FB_OTHER_NAN)));
    a.sse1[c] = -1.0;
    a.pass2[c] = 0;
    a.res[c].rank = 0;
    return;
  }
  if (nanmask) {
    // A NaN factor column makes the reference's QR return NaN coefficients
    // (the sentinel) unless a rank cut among the other columns happens before
    // the QR reaches it.  Full, well-conditioned rank of the other columns
    // rules that out; otherwise the FP64 path decides.
    int idx[kMixedMaxM + 1], kk2 = 0;
    for (int i = 0; i < k; ++i)
      if (i == m || !((nanmask >> i) & 1u)) idx[kk2++] = i;
    double H[kMixedMaxM + 1][kMixedMaxM + 1];
    for (int i = 0; i < kk2; ++i)
      for (int j = 0; j < kk2; ++j) H[i][j] = G[idx[i]][idx[j]];
    bool full = true;
    double hmax = 0.0;
    for (int i = 0; i < kk2; ++i) hmax = fmax(hmax, H[i][i]);
    for (int s2 = 0; s2 < kk2 && full; ++s2) {
      int p = s2;
      for (int j = s2 + 1; j < kk2; ++j)
        if (H[j][j] > H[p][p]) p = j;
      if (!(H[p][p] > 1e-6 * hmax)) {
        full = false;
        break;
      }
      if (p != s2) {
        for (int j = 0; j < kk2; ++j) { const double t2 = H[s2][j]; H[s2][j] = H[p][j]; H[p][j] = t2; }
        for (int j = 0; j < kk2; ++j) { const double t2 = H[j][s2]; H[j][s2] = H[j][p]; H[j][p] = t2; }
      }
      const double l = sqrt(H[s2][s2]);
      for (int i = s2 + 1; i < kk2; ++i) H[i][s2] /= l;
      for (int i = s2 + 1; i < kk2; ++i)
        for (int j = s2 + 1; j <= i; ++j) {
          H[i][j] -= H[i][s2] * H[j][s2];
          H[j][i] = H[i][j];
        }
    }
    double* out = a.coefs + cd.coef_offset;
    for (int i = 0; i < k; ++i) out[i] = __longlong_as_double(0x7ff8000000000000ll);
    if (full) {
      a.sse1[c] = __longlong_as_double(0x7ff8000000000000ll);
    } else {
      queue_fallback(FB_NAN_RANK);
      a.sse1[c] = -1.0;
    }
    a.pass2[c] = 0;
    a.res[c].rank = 0;
    return;
  }
  // symmetric pivoted Cholesky (pivot = largest remaining diagonal, i.e. the
  // largest remaining column norm of the design, as column-pivoted QR picks)
  int piv[kMixedMaxM + 1];
  double d0[kMixedMaxM + 1];
  double maxd = 0.0;
  for (int i = 0; i < k; ++i) {
    piv[i] = i;
    d0[i] = G[i][i];
    if (G[i][i] > maxd) maxd = G[i][i];
    for (int j = 0; j < k; ++j) L[i][j] = G[i][j];
  }
  int rank = k;
  double min_ratio = 1.0;
  const bool finite = !has_nan && !has_inf;
  for (int s2 = 0; s2 < k && finite; ++s2) {
    int p = s2;
    for (int j = s2 + 1; j < k; ++j)
      if (L[j][j] > L[p][p]) p = j;
    const double dp = L[p][p];
    if (!(dp > a.rank_tol * maxd)) {
      rank = s2;
      break;
    }
    if (p != s2) {
      for (int j = 0; j < k; ++j) { const double t2 = L[s2][j]; L[s2][j] = L[p][j]; L[p][j] = t2; }
      for (int j = 0; j < k; ++j) { const double t2 = L[j][s2]; L[j][s2] = L[j][p]; L[j][p] = t2; }
      const int t3 = piv[s2]; piv[s2] = piv[p]; piv[p] = t3;
    }
    const double ratio = dp / d0[piv[s2]];
    if (ratio < min_ratio) min_ratio = ratio;
    const double lss = sqrt(dp);
    L[s2][s2] = lss;
    for (int i = s2 + 1; i < k; ++i) L[i][s2] = L[i][s2] / lss;
    for (int i = s2 + 1; i < k; ++i)
      for (int j = s2 + 1; j <= i; ++j) {
        L[i][j] = L[i][j] - L[i][s2] * L[j][s2];
        L[j][i] = L[i][j];
      }
  }
  double coef[kMixedMaxM + 1];
  for (int i = 0; i < k; ++i) coef[i] = 0.0;
  uint32_t flags = 0;
  if (!finite) {
    for (int i = 0; i < k; ++i) coef[i] = __longlong_as_double(0x7ff8000000000000ll);
    rank = 0;
  } else if (rank > 0) {
    // solve L L^T z = P b on the leading `rank` block, then one refinement step
    double z[kMixedMaxM + 1], rhs[kMixedMaxM + 1];
    for (int i = 0; i < rank; ++i) rhs[i] = bvec[piv[i]];
    for (int pass = 0; pass < 2; ++pass) {
      for (int i = 0; i < rank; ++i) {
        double v = rhs[i];
        for (int j = 0; j < i; ++j) v -= L[i][j] * z[j];
        z[i] = v / L[i][i];
      }
      for (int i = rank - 1; i >= 0; --i) {
        double v = z[i];
        for (int j = i + 1; j < rank; ++j) v -= L[j][i] * z[j];
        z[i] = v / L[i][i];
      }
      for (int i = 0; i < rank; ++i) coef[piv[i]] += z[i];
      if (pass == 0) {
        for (int i = 0; i < rank; ++i) {
          const int pi = piv[i];
          double v = bvec[pi];
          for (int j = 0; j < k; ++j) v -= G[pi][j] * coef[j];
          rhs[i] = v;
        }
      }
    }
  }
  if (rank < k) flags |= RRG_F_RANK_DEFICIENT;
  // Decisions the FP64 path must take itself: a rank cut (the reference's
  // rule works at eps^2 of the column norms), ill-conditioning, and
  // coefficients inside the ambiguity band of the drop (|c| < 1e-12) and
  // snap (|c - 1| < 1e-12) rules of the rebuilt tree.
  const double yrms = sqrt(yy / n_d);
  int why = -1;
  if (!finite) why = FB_OTHER_NAN;
  else if (rank < k && a.certify) why = FB_RANK;
  else if (rank == k && min_ratio < a.fallback_tol) why = FB_ILL_COND;
  for (int i = 0; i < k && why < 0 && a.certify; ++i) {
    const double ci = coef[i];
    const double scale = i == m ? 1.0 : fmax((double)pr.rms[i], 1e-300);
    if (fabs(ci - 1.0) < 1e-4 && i < m) why = FB_SNAP;
    else if (fabs(ci) * scale < 1e-6 * yrms) why = FB_DROP;
  }
  double* out = a.coefs + cd.coef_offset;
  MixedTerm& tm = a.terms[c];
  double ceff[kMixedMaxM + 1];
  for (int i = 0; i < k; ++i) {
    out[i] = coef[i];
    const double ci = coef[i];
    tm.hi[i] = (float)ci;
    tm.lo[i] = (float)(ci - (double)tm.hi[i]);
    const int kind = fabs(ci) < kEps12 ? 0 : (i == m ? 1 : (fabs(ci - 1) < kEps12 ? 2 : 3));
    tm.kind[i] = (int8_t)kind;
    ceff[i] = kind == 0 ? 0.0 : (kind == 2 ? 1.0 : ci);
  }
  double sse;
  uint8_t p2 = 0;
  if (has_nan || !finite) {
    sse = has_nan ? __longlong_as_double(0x7ff8000000000000ll) : -1.0;
  } else {
    double lin = 0.0, quad = 0.0, mag = yy;
    for (int i = 0; i < k; ++i) {
      lin += ceff[i] * bvec[i];
      mag += 2.0 * fabs(ceff[i] * bvec[i]);
      for (int j = 0; j < k; ++j) {
        quad += ceff[i] * ceff[j] * G[i][j];
        mag += fabs(ceff[i] * ceff[j] * G[i][j]);
      }
    }
    sse = yy - 2.0 * lin + quad;
    double E = 0.0;
    for (int i = 0; i < m; ++i) E += fabs(ceff[i]) * ferr(i);
    if (why < 0 && !(sse > 0.0 && kU * mag <= a.pass2_tol * sse)) {
      if (a.certify) why = FB_ONE_PASS;
      else p2 = 1;
    }
    if (why < 0 && a.certify && cert_bound(sse, E) > a.cert_tol) why = FB_CERT;
  }
  const bool fallback = why >= 0;
  if (fallback) {
    queue_fallback(why);
    p2 = 0;
    sse = -1.0;
  } else if (p2) {
    sse = -1.0;
  }
  a.sse1[c] = sse;
  a.pass2[c] = p2;
  a.res[c].rank = rank;
  a.res[c].flags |= flags;
}

// ------------------------------------------------------------- probe ----
// Scalar interpreters for the probe: the FP64 one has the semantics of the
// plain path (rr_math functions), the FP32 one those of eval4.
template <int MM>
__device__ bool probe_eval64(const uint32_t* code, int len, const double* K, const DevData& ds, int64_t row,
                             double (&f)[MM]) {
  double st[RRG_MAX_STACK];
  double tos = 0.0;
  int sp = 0;
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = ds.X64[(int64_t)arg * ds.n_pad + row]; break;
      case RRG_OP_LDC: tos = K[arg]; break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = ds.X64[(int64_t)arg * ds.n_pad + row];
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = K[arg];
        break;
      case RRG_OP_SIN: tos = rr_sin(tos); break;
      case RRG_OP_COS: tos = rr_cos(tos); break;
      case RRG_OP_LN: tos = rr_log(tos); break;
      case RRG_OP_EXP: tos = rr_exp(tos); break;
      case RRG_OP_SQRT: tos = __dsqrt_rn(tos); break;
      case RRG_OP_SQR: tos = __dmul_rn(tos, tos); break;
      case RRG_OP_EMIT:
#pragma unroll
        for (int s = 0; s < MM; ++s)
          if ((int)arg == s) f[s] = tos;
        sp = 0;
        break;
      default: {
        const int kk = op - RRG_OP_BIN;
        const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
        double o;
        if (src == RRG_SRC_S) {
          if (sp <= 0) return false;
          o = st[--sp];
        } else if (src == RRG_SRC_V) {
          o = ds.X64[(int64_t)arg * ds.n_pad + row];
        } else {
          o = K[arg];
        }
        const double a = dir == RRG_DIR_N ? o : tos, b = dir == RRG_DIR_N ? tos : o;
        switch (base) {
          case RRG_ADD: tos = __dadd_rn(a, b); break;
          case RRG_SUB: tos = __dsub_rn(a, b); break;
          case RRG_MUL: tos = __dmul_rn(a, b); break;
          case RRG_DIV: tos = __ddiv_rn(a, b); break;
          case RRG_POW: tos = rr_pow(a, b); break;
          case RRG_LT: tos = a < b ? 1.0 : 0.0; break;
          case RRG_EQ: tos = a == b ? 1.0 : 0.0; break;
          case RRG_NE: tos = a != b ? 1.0 : 0.0; break;
          case RRG_MIN: tos = a < b ? a : b; break;
          default: tos = a > b ? a : b; break;
        }
      }
    }
  }
  return true;
}

template <int MM>
__device__ bool probe_eval32(const uint32_t* code, int len, const float* K, const DevData& ds, int64_t row,
                             float (&f)[MM]) {
  float st[RRG_MAX_STACK];
  float tos = 0.f;
  int sp = 0;
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: tos = ds.X32[(int64_t)arg * ds.n_pad + row]; break;
      case RRG_OP_LDC: tos = K[arg]; break;
      case RRG_OP_PSV:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = ds.X32[(int64_t)arg * ds.n_pad + row];
        break;
      case RRG_OP_PSC:
        if (sp >= RRG_MAX_STACK) return false;
        st[sp++] = tos;
        tos = K[arg];
        break;
      case RRG_OP_SIN: tos = sin32(tos); break;
      case RRG_OP_COS: tos = cos32(tos); break;
      case RRG_OP_LN: tos = logf(tos); break;
      case RRG_OP_EXP: tos = expf(tos); break;
      case RRG_OP_SQRT: tos = sqrt32(tos); break;
      case RRG_OP_SQR: tos = sqr32(tos); break;
      case RRG_OP_EMIT:
#pragma unroll
        for (int s = 0; s < MM; ++s)
          if ((int)arg == s) f[s] = tos;
        sp = 0;
        break;
      default: {
        const int kk = op - RRG_OP_BIN;
        const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
        float o;
        if (src == RRG_SRC_S) {
          if (sp <= 0) return false;
          o = st[--sp];
        } else if (src == RRG_SRC_V) {
          o = ds.X32[(int64_t)arg * ds.n_pad + row];
        } else {
          o = K[arg];
        }
        tos = dir == RRG_DIR_N ? bin32(base, o, tos) : bin32(base, tos, o);
      }
    }
  }
  return true;
}

// One warp per candidate: both interpreters on kProbeRows rows spread evenly
// over the dataset; per factor the largest FP32 deviation, the FP64 RMS and
// the non-finite patterns.
__global__ void __launch_bounds__(128) mixed_probe_kernel(DevBatch b, DevData ds, const int32_t* list,
                                                          int32_t n_list, ProbeOut* out) {
  const int lane = threadIdx.x & 31;
  const int li = blockIdx.x * 4 + (threadIdx.x >> 5);
  if (li >= n_list) return;
  const int c = list[li];
  const rrg_cand cd = b.cands[c];
  const int nf = cd.n_factors;
  const uint32_t* code = b.code + cd.code_offset;
  const int P = ds.n < kProbeRows ? (int)ds.n : kProbeRows;
  float dev[kMixedMaxM];
  double ss[kMixedMaxM];
  int cnt[kMixedMaxM];
  uint32_t nan64 = 0, inf64 = 0, bad32 = 0;
#pragma unroll
  for (int i = 0; i < kMixedMaxM; ++i) {
    dev[i] = 0.f;
    ss[i] = 0.0;
    cnt[i] = 0;
  }
  for (int p = lane; p < P; p += 32) {
    const int64_t row = ds.n < kProbeRows ? p : ((2 * (int64_t)p + 1) * ds.n) / (2 * kProbeRows);
    double f64[kMixedMaxM];
    float f32[kMixedMaxM];
#pragma unroll
    for (int i = 0; i < kMixedMaxM; ++i) {
      f64[i] = 0.0;
      f32[i] = 0.f;
    }
    if (!probe_eval64<kMixedMaxM>(code, cd.code_len, b.consts, ds, row, f64) ||
        !probe_eval32<kMixedMaxM>(code, cd.code_len, b.consts32, ds, row, f32)) {
      bad32 = 0xffffffffu;
      continue;
    }
#pragma unroll
    for (int i = 0; i < kMixedMaxM; ++i) {
      if (i >= nf) break;
      const double v = f64[i];
      const float u = f32[i];
      const bool n64 = v != v, i64 = !n64 && fabs(v) > DBL_MAX;
      const bool n32 = u != u, i32 = !n32 && fabsf(u) > FLT_MAX;
      if (n64) nan64 |= 1u << i;
      if (i64) inf64 |= 1u << i;
      if (n64 != n32 || (i32 && !i64) || (i64 && !i32)) bad32 |= 1u << i;
      if (!n64 && !i64 && !n32 && !i32) {
        const float dv = (float)fabs((double)u - v);
        dev[i] = fmaxf(dev[i], dv);
        ss[i] = __fma_rn(v, v, ss[i]);
        cnt[i] += 1;
      }
    }
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    nan64 |= __shfl_xor_sync(0xffffffffu, nan64, o);
    inf64 |= __shfl_xor_sync(0xffffffffu, inf64, o);
    bad32 |= __shfl_xor_sync(0xffffffffu, bad32, o);
#pragma unroll
    for (int i = 0; i < kMixedMaxM; ++i) {
      dev[i] = fmaxf(dev[i], __shfl_xor_sync(0xffffffffu, dev[i], o));
      ss[i] += __shfl_xor_sync(0xffffffffu, ss[i], o);
      cnt[i] += __shfl_xor_sync(0xffffffffu, cnt[i], o);
    }
  }
  if (lane == 0) {
    ProbeOut r;
    for (int i = 0; i < kMixedMaxM; ++i) {
      r.dev[i] = dev[i];
      r.rms[i] = cnt[i] > 0 ? (float)sqrt(ss[i] / (double)cnt[i]) : 0.f;
    }
    r.nan64 = nan64;
    r.inf64 = inf64;
    r.bad32 = bad32;
    r.all_rows = P == ds.n ? 1u : 0u;
    out[c] = r;
  }
}

__global__ void to_f32_kernel(const double* src, float* dst, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x)
    dst[i] = (float)src[i];
}
__global__ void split_f32_kernel(const double* src, float* hi, float* lo, int64_t n) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
    const float h = (float)src[i];
    hi[i] = h;
    lo[i] = (float)(src[i] - (double)h);
  }
}

// ----------------------------------------------------------- launchers ----
int mixed_threads(int mmax) { return mmax <= 2 ? 1024 : (mmax == 4 ? 512 : 256); }
int mixed_gram_entries(int mmax) { return mmax * (mmax + 1) / 2 + 2 * mmax; }

size_t mixed_smem(int mmax, int d, int tile, bool resid) {
  const int nw = mixed_threads(mmax) / 32;
  return 128 + sizeof(float) * (size_t)(d + (resid ? 2 : 1)) * tile + sizeof(float4) * kMixedStackCap * 32 * nw +
         sizeof(uint32_t) * kMixedCodeCap * nw;
}

template <int MMAX>
struct Warps {
  static constexpr int NW = MMAX <= 2 ? 32 : (MMAX == 4 ? 16 : 8);
};

template <int MMAX, bool RESID>
static bool launch_one(const MixedArgs& a, int grid, size_t smem, cudaStream_t st) {
  constexpr int NW = Warps<MMAX>::NW;
  mixed_pass_kernel<MMAX, NW, RESID><<<grid, NW * 32, smem, st>>>(a);
  return cudaGetLastError() == cudaSuccess;
}

bool launch_gram(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st) {
  switch (mmax) {
    case 1: return launch_one<1, false>(a, grid, smem, st);
    case 2: return launch_one<2, false>(a, grid, smem, st);
    case 4: return launch_one<4, false>(a, grid, smem, st);
    case 8: return launch_one<8, false>(a, grid, smem, st);
    default: return false;
  }
}
bool launch_resid(int mmax, const MixedArgs& a, int grid, size_t smem, cudaStream_t st) {
  switch (mmax) {
    case 1: return launch_one<1, true>(a, grid, smem, st);
    case 2: return launch_one<2, true>(a, grid, smem, st);
    case 4: return launch_one<4, true>(a, grid, smem, st);
    case 8: return launch_one<8, true>(a, grid, smem, st);
    default: return false;
  }
}
bool launch_probe(const DevBatch& b, const DevData& ds, const int32_t* list, int32_t n_list, ProbeOut* out,
                  cudaStream_t st) {
  if (n_list <= 0) return true;
  mixed_probe_kernel<<<(n_list + 3) / 4, 128, 0, st>>>(b, ds, list, n_list, out);
  return cudaGetLastError() == cudaSuccess;
}
bool launch_solve(const SolveArgs& a, cudaStream_t st) {
  mixed_solve_kernel<<<(a.n_list + 3) / 4, 128, 0, st>>>(a);
  return cudaGetLastError() == cudaSuccess;
}
bool launch_to_f32(const double* src, float* dst, int64_t n, cudaStream_t st) {
  to_f32_kernel<<<1024, 256, 0, st>>>(src, dst, n);
  return cudaGetLastError() == cudaSuccess;
}
bool launch_split_f32(const double* src, float* hi, float* lo, int64_t n, cudaStream_t st) {
  split_f32_kernel<<<1024, 256, 0, st>>>(src, hi, lo, n);
  return cudaGetLastError() == cudaSuccess;
}

template <int MMAX, bool RESID>
static bool allow_smem() {
  constexpr int NW = Warps<MMAX>::NW;
  return cudaFuncSetAttribute(mixed_pass_kernel<MMAX, NW, RESID>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                              227 * 1024) == cudaSuccess;
}
bool mixed_allow_smem() {
  return allow_smem<1, false>() && allow_smem<2, false>() && allow_smem<4, false>() && allow_smem<8, false>() &&
         allow_smem<1, true>() && allow_smem<2, true>() && allow_smem<4, true>() && allow_smem<8, true>();
}

}  // namespace rrd
