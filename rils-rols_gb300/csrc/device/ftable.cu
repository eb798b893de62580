// Factor table of a mixed round: double-float evaluation of the distinct
// factor programs, Gram sums per distinct pair, and the residual pass.
//
//   fac_eval      block = (group of factors, row chunk).  Every factor of
//                 the group is interpreted on the chunk in double-float
//                 arithmetic, 4 rows per thread for short shallow programs
//                 and 2 for the others, with the semantics of
//                 node::evaluate_inner (node.cpp:23-95); X and y (high and
//                 low parts) are read from L2, where they stay resident
//                 (staging each chunk in shared memory by TMA bulk copies
//                 was measured slower: the shared memory it takes costs
//                 more occupancy than the loads it saves).
//                 Values go to the table F in HBM (rows >= n set to 0); the
//                 self sums  sum f*f, sum f, sum f*y  of the chunk are formed
//                 on the way;
//   pair_sum      block = (factor a with its partners b, row block): a's
//                 values stay in registers, each partner column is streamed
//                 once, sum a*b in double-float arithmetic;
//   pair_reduce   FP64 totals of the partials, in chunk order;
//   ftab_resid    the rebuilt sum  sum_i c_i f_i  (drop / snap rules of
//                 rils_rols_cpp.cpp:488-517) from the table, its residual
//                 against y and the squared residuals, all double-float.
#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "common.cuh"
#include "dfeval.cuh"
#include "ftable.cuh"

namespace rrd {

namespace {

constexpr int kPairPerThread = kPairRows / (2 * kPairThreads);  // row pairs per thread (8)

__device__ __forceinline__ dfl shfl_dfl(dfl v, int o) {
  return dfl_make(__shfl_xor_sync(0xffffffffu, v.hi, o), __shfl_xor_sync(0xffffffffu, v.lo, o));
}
__device__ __forceinline__ dfl warp_dfl_sum(dfl v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v = dfl_add(v, shfl_dfl(v, o));
  return v;
}

// Running sum s += p + e in the manner of Sum2 (Ogita, Rump and Oishi, 2005):
// p joins the high part by an exact two-sum (Knuth), its rounding error and
// the small term e join the low part, which is not renormalised per step.
__device__ __forceinline__ void acc2(dfl& s, float p, float e) {
  const float t = DF_ADD(s.hi, p);
  const float bp = DF_SUB(t, s.hi);
  const float err = DF_ADD(DF_SUB(s.hi, DF_SUB(t, bp)), DF_SUB(p, bp));
  s.hi = t;
  s.lo = DF_ADD(s.lo, DF_ADD(err, e));
}
// hi + lo as a normalised double-float (|lo| small against |hi|, or hi = 0);
// non-finite parts pass through
__device__ __forceinline__ dfl dfl_renorm(dfl s) {
  if (!dfl_finite(s.hi) || !dfl_finite(s.lo)) return s;
  const float t = DF_ADD(s.hi, s.lo);
  return dfl_make(t, DF_SUB(s.lo, DF_SUB(t, s.hi)));
}

// One table program on 2 consecutive rows (r, r + 1 of the chunk); X column
// j has its high parts at xh + j * ldx and its low parts at xl + j * ldx;
// table column t (an earlier level) at tb + t * ldtab.
__device__ __forceinline__ bool eval_fac2(const uint32_t* code, int len, const float* __restrict__ K,
                                          const float* __restrict__ Klo, const float* xh, const float* xl,
                                          int64_t ldx, const float2* tb, int64_t ldtab, int r, float4* st,
                                          dfl& o0, dfl& o1) {
  dfl t0 = dfl_make(0.f, 0.f), t1 = t0;
  int sp = 0;
  auto ldv = [&](uint32_t j, dfl& u0, dfl& u1) {
    const float2 h = *reinterpret_cast<const float2*>(xh + (int64_t)j * ldx + r);
    const float2 l = *reinterpret_cast<const float2*>(xl + (int64_t)j * ldx + r);
    u0 = dfl_make(h.x, l.x);
    u1 = dfl_make(h.y, l.y);
  };
  auto ldt = [&](uint32_t t, dfl& u0, dfl& u1) {
    const float4 v = *reinterpret_cast<const float4*>(tb + (int64_t)t * ldtab + r);
    u0 = dfl_make(v.x, v.y);
    u1 = dfl_make(v.z, v.w);
  };
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: ldv(arg, t0, t1); break;
      case RRG_OP_LDC: t0 = t1 = dfl_make(__ldg(K + arg), __ldg(Klo + arg)); break;
      case RRG_OP_PSV:
        if (sp >= kMixedStackCap) return false;
        st[32 * sp++] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo);
        ldv(arg, t0, t1);
        break;
      case RRG_OP_PSC:
        if (sp >= kMixedStackCap) return false;
        st[32 * sp++] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo);
        t0 = t1 = dfl_make(__ldg(K + arg), __ldg(Klo + arg));
        break;
      case kOpLDT: ldt(arg, t0, t1); break;
      case kOpPST:
        if (sp >= kMixedStackCap) return false;
        st[32 * sp++] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo);
        ldt(arg, t0, t1);
        break;
      case RRG_OP_EMIT:
        o0 = t0;
        o1 = t1;
        sp = 0;
        break;
      default:
        if (op >= RRG_OP_SIN && op <= RRG_OP_SQR) {
          df_unary2(op, t0, t1);
        } else {
          const int kk = op - RRG_OP_BIN;
          const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
          dfl u0, u1;
          if (src == RRG_SRC_S) {
            if (sp <= 0) return false;
            const float4 v = st[32 * --sp];
            u0 = dfl_make(v.x, v.y);
            u1 = dfl_make(v.z, v.w);
          } else if (src == RRG_SRC_V) {
            ldv(arg, u0, u1);
          } else if (src == kSrcT) {
            ldt(arg, u0, u1);
          } else {
            u0 = u1 = dfl_make(__ldg(K + arg), __ldg(Klo + arg));
          }
          if (dir == RRG_DIR_N) df_bin2(base, u0, t0, u1, t1, t0, t1);
          else df_bin2(base, t0, u0, t1, u1, t0, t1);
        }
    }
  }
  return true;
}

// One table program on 4 consecutive rows (r .. r + 3 of the chunk), as two
// pairs A (r, r + 1) and B (r + 2, r + 3) sharing one dispatch; X column j has
// its high parts at xh + j * ldx and its low parts at xl + j * ldx; table
// column t (an earlier level) at tb + t * ldtab.  A spill level holds the
// four values in two float4 slots.
__device__ __forceinline__ bool eval_fac4(const uint32_t* code, int len, const float* __restrict__ K,
                                          const float* __restrict__ Klo, const float* xh, const float* xl,
                                          int64_t ldx, const float2* tb, int64_t ldtab, int r, float4* st,
                                          dfl (&o)[4]) {
  dfl t0 = dfl_make(0.f, 0.f), t1 = t0, t2 = t0, t3 = t0;
  int sp = 0;
  auto ldv = [&](uint32_t j, dfl& u0, dfl& u1, dfl& u2, dfl& u3) {
    const float4 h = *reinterpret_cast<const float4*>(xh + (int64_t)j * ldx + r);
    const float4 l = *reinterpret_cast<const float4*>(xl + (int64_t)j * ldx + r);
    u0 = dfl_make(h.x, l.x);
    u1 = dfl_make(h.y, l.y);
    u2 = dfl_make(h.z, l.z);
    u3 = dfl_make(h.w, l.w);
  };
  auto ldt = [&](uint32_t t, dfl& u0, dfl& u1, dfl& u2, dfl& u3) {
    const float4 v = *reinterpret_cast<const float4*>(tb + (int64_t)t * ldtab + r);
    const float4 w = *reinterpret_cast<const float4*>(tb + (int64_t)t * ldtab + r + 2);
    u0 = dfl_make(v.x, v.y);
    u1 = dfl_make(v.z, v.w);
    u2 = dfl_make(w.x, w.y);
    u3 = dfl_make(w.z, w.w);
  };
  auto push = [&]() {
    st[32 * (2 * sp)] = make_float4(t0.hi, t0.lo, t1.hi, t1.lo);
    st[32 * (2 * sp + 1)] = make_float4(t2.hi, t2.lo, t3.hi, t3.lo);
    ++sp;
  };
  for (int pc = 0; pc < len; ++pc) {
    const uint32_t w = code[pc];
    const int op = (int)(w & 0xffu);
    const uint32_t arg = w >> 8;
    switch (op) {
      case RRG_OP_LDV: ldv(arg, t0, t1, t2, t3); break;
      case RRG_OP_LDC: t0 = t1 = t2 = t3 = dfl_make(__ldg(K + arg), __ldg(Klo + arg)); break;
      case RRG_OP_PSV:
        if (sp >= kMixedStackCap) return false;
        push();
        ldv(arg, t0, t1, t2, t3);
        break;
      case RRG_OP_PSC:
        if (sp >= kMixedStackCap) return false;
        push();
        t0 = t1 = t2 = t3 = dfl_make(__ldg(K + arg), __ldg(Klo + arg));
        break;
      case kOpLDT: ldt(arg, t0, t1, t2, t3); break;
      case kOpPST:
        if (sp >= kMixedStackCap) return false;
        push();
        ldt(arg, t0, t1, t2, t3);
        break;
      case RRG_OP_EMIT:
        o[0] = t0;
        o[1] = t1;
        o[2] = t2;
        o[3] = t3;
        sp = 0;
        break;
      default:
        if (op >= RRG_OP_SIN && op <= RRG_OP_SQR) {
          df_unary2(op, t0, t1);
          df_unary2(op, t2, t3);
        } else {
          const int kk = op - RRG_OP_BIN;
          const int base = kk >> 3, src = (kk & 7) >> 1, dir = kk & 1;
          dfl u0, u1, u2, u3;
          if (src == RRG_SRC_S) {
            if (sp <= 0) return false;
            --sp;
            const float4 v = st[32 * (2 * sp)];
            const float4 v2 = st[32 * (2 * sp + 1)];
            u0 = dfl_make(v.x, v.y);
            u1 = dfl_make(v.z, v.w);
            u2 = dfl_make(v2.x, v2.y);
            u3 = dfl_make(v2.z, v2.w);
          } else if (src == RRG_SRC_V) {
            ldv(arg, u0, u1, u2, u3);
          } else if (src == kSrcT) {
            ldt(arg, u0, u1, u2, u3);
          } else {
            u0 = u1 = u2 = u3 = dfl_make(__ldg(K + arg), __ldg(Klo + arg));
          }
          if (dir == RRG_DIR_N) {
            df_bin2(base, u0, t0, u1, t1, t0, t1);
            df_bin2(base, u2, t2, u3, t3, t2, t3);
          } else {
            df_bin2(base, t0, u0, t1, u1, t0, t1);
            df_bin2(base, t2, u2, t3, u3, t2, t3);
          }
        }
    }
  }
  return true;
}

// shared-memory layout of fac_eval
constexpr size_t kFacRedOff = 128;                                   // [warp][6] floats
constexpr size_t kFacCodeOff = kFacRedOff + 256;
constexpr size_t kFacStackOff = kFacCodeOff + sizeof(uint32_t) * kFacCodeSmem;
constexpr size_t kFacXOff = kFacStackOff + sizeof(float4) * (kFacThreads / 32) * kMixedStackCap * 32 * 2;  // end
// staged form: the copy barrier, then the staged rows (hi of every slot, lo
// of every slot, y hi, y lo; `chunk` floats each)
constexpr size_t kFacBarOff = kFacXOff;
constexpr size_t kFacStageOff = kFacXOff + 128;

__device__ __forceinline__ uint32_t smem_addr(const void* p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}
__device__ __forceinline__ void mbar_init(uint64_t* m, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_addr(m)), "r"(count) : "memory");
}
// the barrier's initialisation visible to the tensor-copy (async) proxy
__device__ __forceinline__ void mbar_init_fence() { asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory"); }
__device__ __forceinline__ void mbar_expect_tx(uint64_t* m, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_addr(m)), "r"(bytes) : "memory");
}
__device__ __forceinline__ bool mbar_try_wait(uint64_t* m, uint32_t parity) {
  uint32_t done;
  asm volatile(
      "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
      : "=r"(done)
      : "r"(smem_addr(m)), "r"(parity)
      : "memory");
  return done != 0;
}
// Waits for the barrier's phase `parity` to complete, at most `tries` times.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t* m, uint32_t parity, int tries) {
  for (int i = 0; i < tries; ++i)
    if (mbar_try_wait(m, parity)) return true;
  return false;
}
// Tensor copy of the box at (x, y) of `map` into dst, completing on m.
__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, int x, int y, uint64_t* m) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          smem_addr(dst)),
      "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_addr(m))
      : "memory");
}
constexpr int kStageWaitTries = 1 << 20;  // bounded wait for the staged rows

}  // namespace

// R = 4 rows per thread for short, shallow programs (one dispatch per op for
// four rows), R = 2 for the others (less spill traffic per thread).
template <int R, bool STAGED>
__global__ void __launch_bounds__(kFacThreads) fac_eval_kernel(const __grid_constant__ FacEvalArgs a) {
  extern __shared__ __align__(128) unsigned char smem[];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int2 grp = a.groups[blockIdx.x];
  const int q = blockIdx.y;
  const int64_t n = a.ds.n, n_pad = a.ds.n_pad;
  const int64_t row0 = (int64_t)q * a.chunk;
  const int rows = (int)min((int64_t)a.chunk, n_pad - row0);  // a multiple of 256
  float* red = reinterpret_cast<float*>(smem + kFacRedOff);
  uint32_t* code_s = reinterpret_cast<uint32_t*>(smem + kFacCodeOff);
  float4* stk = reinterpret_cast<float4*>(smem + kFacStackOff);
  const float* xh = a.ds.X32 + row0;
  const float* xl = a.ds.X32lo + row0;
  int64_t ldx = n_pad;
  const float* yh = a.ds.y32 + row0;
  const float* yl = a.ds.y32lo + row0;
  int f0 = 0, nf = 0;
  if constexpr (STAGED) {
    // the chunk's rows of the group's features and of y into shared memory:
    // one thread arms the barrier with the byte count and issues the tensor
    // copies; every thread waits for them (a bounded wait)
    f0 = a.gfeat_off[blockIdx.x];
    nf = a.gfeat_off[blockIdx.x + 1] - f0;
    uint64_t* bar = reinterpret_cast<uint64_t*>(smem + kFacBarOff);
    float* stg = reinterpret_cast<float*>(smem + kFacStageOff);
    if (tid == 0) {
      mbar_init(bar, 1);
      mbar_init_fence();
    }
    __syncthreads();
    if (tid == 0) {
      mbar_expect_tx(bar, (uint32_t)((2 * nf + 2) * rows * (int)sizeof(float)));
      for (int b = 0; b < rows; b += kTmaRows) {
        const int x = (int)(row0 + b);  // a multiple of kTmaRows: 16-byte aligned
        for (int s = 0; s < nf; ++s) {
          const int j = a.gfeat[f0 + s];
          tma_load_2d(stg + (size_t)s * rows + b, &a.tm_xh, x, j, bar);
          tma_load_2d(stg + (size_t)(nf + s) * rows + b, &a.tm_xl, x, j, bar);
        }
        tma_load_2d(stg + (size_t)(2 * nf) * rows + b, &a.tm_yh, x, 0, bar);
        tma_load_2d(stg + (size_t)(2 * nf + 1) * rows + b, &a.tm_yl, x, 0, bar);
      }
    }
    if (!mbar_wait_bounded(bar, 0, kStageWaitTries)) {
      // the copies did not complete: report it, give them a second bounded
      // wait (they write this block's shared memory) and leave
      if (tid == 0) atomicOr(a.status, ST_WAIT_TIMEOUT);
      mbar_wait_bounded(bar, 0, kStageWaitTries);
      return;
    }
    xh = stg;
    xl = stg + (size_t)nf * rows;
    ldx = rows;
    yh = stg + (size_t)(2 * nf) * rows;
    yl = stg + (size_t)(2 * nf + 1) * rows;
  }
  // the group's programs are contiguous: stage them (staged form: feature
  // operands renumbered to their shared-memory slots)
  const int base = a.meta[grp.x].x;
  const int2 last = a.meta[grp.x + grp.y - 1];
  const int total = last.x + last.y - base;
  for (int i = tid; i < total; i += kFacThreads) {
    uint32_t w = a.code[base + i];
    if constexpr (STAGED) {
      const int op = (int)(w & 0xffu);
      const bool feat = op == RRG_OP_LDV || op == RRG_OP_PSV ||
                        (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_V);
      if (feat) {
        const int j = (int)(w >> 8);
        int slot = 0;
        for (int s = 0; s < nf; ++s)
          if (a.gfeat[f0 + s] == j) slot = s;
        w = (w & 0xffu) | ((uint32_t)slot << 8);
      }
    }
    code_s[i] = w;
  }
  __syncthreads();
  const float2* tb = a.F + row0;
  const bool tail = row0 + rows > n;  // the chunk holds padding rows (set to 0)
  float4* st = stk + (size_t)warp * kMixedStackCap * 32 * 2 + lane;
  for (int i = 0; i < grp.y; ++i) {
    const int f = grp.x + i;
    const int64_t fw = a.wcol ? a.wcol[f] : f;  // the column it writes
    const int2 mt = a.meta[f];
    const uint32_t* code = code_s + (mt.x - base);
    dfl ff = dfl_make(0.f, 0.f), fs = ff, fy = ff;
    unsigned long long first = ~0ull;
    bool ok = true;
    for (int r = R * tid; r < rows; r += R * kFacThreads) {
      dfl v[4];
      if constexpr (R == 4) {
        ok = eval_fac4(code, mt.y, a.K, a.Klo, xh, xl, ldx, tb, n_pad, r, st, v) && ok;
      } else {
        ok = eval_fac2(code, mt.y, a.K, a.Klo, xh, xl, ldx, tb, n_pad, r, st, v[0], v[1]) && ok;
        v[2] = v[3] = dfl_make(0.f, 0.f);
      }
      const int64_t gr = row0 + r;
      if (tail) {
#pragma unroll
        for (int u = 0; u < R; ++u)
          if (gr + u >= n) v[u] = dfl_make(0.f, 0.f);
      }
      *reinterpret_cast<float4*>(a.F + fw * n_pad + gr) = make_float4(v[0].hi, v[0].lo, v[1].hi, v[1].lo);
      if constexpr (R == 4)
        *reinterpret_cast<float4*>(a.F + fw * n_pad + gr + 2) = make_float4(v[2].hi, v[2].lo, v[3].hi, v[3].lo);
      dfl y[4];
      if constexpr (R == 4) {
        const float4 yhv = *reinterpret_cast<const float4*>(yh + r);
        const float4 ylv = *reinterpret_cast<const float4*>(yl + r);
        y[0] = dfl_make(yhv.x, ylv.x);
        y[1] = dfl_make(yhv.y, ylv.y);
        y[2] = dfl_make(yhv.z, ylv.z);
        y[3] = dfl_make(yhv.w, ylv.w);
      } else {
        const float2 yhv = *reinterpret_cast<const float2*>(yh + r);
        const float2 ylv = *reinterpret_cast<const float2*>(yl + r);
        y[0] = dfl_make(yhv.x, ylv.x);
        y[1] = dfl_make(yhv.y, ylv.y);
        y[2] = y[3] = dfl_make(0.f, 0.f);
      }
      bool fin = dfl_finite(ff.hi) && dfl_finite(fs.hi) && dfl_finite(fy.hi);
#pragma unroll
      for (int u = 0; u < R; ++u) fin = fin && dfl_finite(v[u].hi);
      if (__all_sync(0xffffffffu, fin)) {
        // finite values (the common case): each product's high part joins
        // the running high part by an exact two-sum; its low part and the
        // two-sum's error join the low part (renormalised after the loop)
#pragma unroll
        for (int u = 0; u < R; ++u) {
          const float p2 = DF_MUL(v[u].hi, v[u].hi);
          acc2(ff, p2, DF_FMA(DF_ADD(v[u].hi, v[u].hi), v[u].lo, DF_FMA(v[u].hi, v[u].hi, -p2)));
          acc2(fs, v[u].hi, v[u].lo);
          const float py = DF_MUL(v[u].hi, y[u].hi);
          acc2(fy, py, DF_FMA(v[u].lo, y[u].hi, DF_FMA(v[u].hi, y[u].lo, DF_FMA(v[u].hi, y[u].hi, -py))));
        }
      } else {
        // a non-finite value in the warp: guarded sums, and the first NaN row
#pragma unroll
        for (int u = 0; u < R; ++u) {
          if (v[u].hi != v[u].hi) first = min(first, (unsigned long long)(gr + u));
          ff = dfl_add(ff, dfl_mul(v[u], v[u]));
          fs = dfl_add(fs, v[u]);
          fy = dfl_add(fy, dfl_mul(v[u], y[u]));
        }
      }
    }
    if (!ok) atomicOr(a.status, ST_STACK);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const unsigned long long other = __shfl_xor_sync(0xffffffffu, first, o);
      first = other < first ? other : first;
    }
    if (lane == 0 && first != ~0ull) atomicMin(a.fnan + fw, first);
    const dfl s0 = warp_dfl_sum(dfl_renorm(ff)), s1 = warp_dfl_sum(dfl_renorm(fs)), s2 = warp_dfl_sum(dfl_renorm(fy));
    if (lane == 0) {
      float* rw = red + warp * 6;
      rw[0] = s0.hi; rw[1] = s0.lo;
      rw[2] = s1.hi; rw[3] = s1.lo;
      rw[4] = s2.hi; rw[5] = s2.lo;
    }
    __syncthreads();
    if (tid < 3) {
      dfl s = dfl_make(0.f, 0.f);
      for (int w = 0; w < kFacThreads / 32; ++w) s = dfl_add(s, dfl_make(red[w * 6 + 2 * tid], red[w * 6 + 2 * tid + 1]));
      a.P[(size_t)q * a.n_pairs + 3 * (size_t)f + tid] = make_float2(s.hi, s.lo);
    }
    __syncthreads();
  }
}

// low part of the double-float product (ah, al) x (bh, bl), symmetric in the
// two operands: fma(ah, bh, -ah*bh) + (ah*bl + al*bh)
__device__ __forceinline__ float pair_lo(float ah, float al, float bh, float bl) {
  const float p = DF_MUL(ah, bh);
  return DF_ADD(DF_FMA(ah, bh, -p), DF_ADD(DF_MUL(ah, bl), DF_MUL(al, bh)));
}

__global__ void __launch_bounds__(kPairThreads) pair_sum_kernel(PairArgs a) {
  __shared__ float red[kPairBatch][kPairThreads / 32][2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int u = blockIdx.x % a.n_units;
  const int qs = blockIdx.x / a.n_units;
  const int4 U = a.units[u];
  const int64_t row0 = (int64_t)qs * kPairRows;
  const int rows = (int)min((int64_t)kPairRows, a.n_pad - row0);
  const float2* fa = a.F + (int64_t)U.x * a.n_pad + row0;
  float4 av[kPairPerThread];
#pragma unroll
  for (int s = 0; s < kPairPerThread; ++s) {
    const int r = 2 * tid + 2 * kPairThreads * s;
    av[s] = r < rows ? *reinterpret_cast<const float4*>(fa + r) : make_float4(0.f, 0.f, 0.f, 0.f);
  }
  for (int p0 = U.y; p0 < U.z; p0 += kPairBatch) {
    const int nb = min(kPairBatch, U.z - p0);
    for (int j = 0; j < nb; ++j) {
      const float2* fb = a.F + (int64_t)a.partner[p0 + j] * a.n_pad + row0;
      dfl acc = dfl_make(0.f, 0.f);
#pragma unroll
      for (int s = 0; s < kPairPerThread; ++s) {
        const int r = 2 * tid + 2 * kPairThreads * s;
        if (r < rows) {
          const float4 bv = *reinterpret_cast<const float4*>(fb + r);
          // without the non-finite guards: a non-finite factor value turns the
          // sum NaN instead of +-inf, and the solve sends every candidate with a
          // non-finite cross sum (NaN or inf alike) to the FP64 path.  The
          // product is symmetric in its operands (the exact error of hi x hi,
          // then the rounded sum of the two rounded cross products), so a
          // pair's sum is the same bits whichever factor a unit holds
          acc2(acc, DF_MUL(av[s].x, bv.x), pair_lo(av[s].x, av[s].y, bv.x, bv.y));
          acc2(acc, DF_MUL(av[s].z, bv.z), pair_lo(av[s].z, av[s].w, bv.z, bv.w));
        }
      }
      const dfl v = warp_dfl_sum(dfl_renorm(acc));
      if (lane == 0) {
        red[j][warp][0] = v.hi;
        red[j][warp][1] = v.lo;
      }
    }
    __syncthreads();
    if (tid < nb) {
      dfl s = dfl_make(0.f, 0.f);
      for (int w = 0; w < kPairThreads / 32; ++w) s = dfl_add(s, dfl_make(red[tid][w][0], red[tid][w][1]));
      a.P[(size_t)qs * a.n_pairs + a.cross0 + p0 + tid] = make_float2(s.hi, s.lo);
    }
    __syncthreads();
  }
}

// psum[p] = sum over chunks q (in order) of P[q][p], in FP64.
__global__ void pair_reduce_kernel(const float2* P, int32_t n_pairs, int32_t n_chunks, int32_t p0, int32_t p1,
                                   double* psum, const int32_t* smap, const int32_t* omap) {
  const int p = p0 + blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= p1) return;
  double s = 0.0;
  for (int q = 0; q < n_chunks; ++q) {
    const float2 v = P[(size_t)q * n_pairs + p];
    s = __dadd_rn(s, __dadd_rn((double)v.x, (double)v.y));
  }
  psum[omap ? (int64_t)omap[p] : (smap ? 3 * (int64_t)smap[p / 3] + p % 3 : (int64_t)p)] = s;
}

__global__ void fill_slots_kernel(const int32_t* idx, int32_t n, unsigned long long* dst, int words,
                                  unsigned long long v) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n)
    for (int w = 0; w < words; ++w) dst[(int64_t)idx[i] * words + w] = v;
}

// The candidates of the residual pass have finite table values (the solve sends
// every non-finite one to the FP64 path), so the unguarded operations apply.
__device__ __forceinline__ void ftab_resid_item(const ResidArgs& a, int i, int qs);

// Items (candidate i of list2, row block qs), i = item % n2, qs = item / n2,
// walked by the grid in any shape: each item's partial sum is the same.
__global__ void __launch_bounds__(kResidThreads) ftab_resid_kernel(ResidArgs a) {
  const int n2 = a.n2_dev ? min(*a.n2_dev, a.n2) : a.n2;
  const int64_t items = (int64_t)n2 * a.n_chunks;
  for (int64_t w = blockIdx.x; w < items; w += gridDim.x) ftab_resid_item(a, (int)(w % n2), (int)(w / n2));
}

__device__ __forceinline__ void ftab_resid_item(const ResidArgs& a, int i, int qs) {
  __shared__ float red[kResidThreads / 32][2];
  const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
  const int li = a.list2[i];
  const int c = a.mlist[li];
  const rrg_cand cd = a.b.cands[c];
  const bool tuned = cd.mode == RRG_TUNED;
  const int m = tuned ? cd.n_factors : 1;
  const MixedTerm& tm = a.terms[c];
  const int64_t n = a.ds.n, n_pad = a.ds.n_pad;
  const int64_t row0 = (int64_t)qs * kPairRows;
  const int rows = (int)min((int64_t)kPairRows, n_pad - row0);
  const float2* col[kMixedMaxM];
#pragma unroll
  for (int s = 0; s < kMixedMaxM; ++s)
    col[s] = s < m ? a.F + (int64_t)a.cand_col[(size_t)li * kMixedMaxM + s] * n_pad + row0 : nullptr;
  dfl acc = dfl_make(0.f, 0.f);
  for (int r = 2 * tid; r < rows; r += 2 * kResidThreads) {
    const int64_t gr = row0 + r;
    float4 fv[kMixedMaxM];
#pragma unroll
    for (int s = 0; s < kMixedMaxM; ++s)
      fv[s] = s < m ? *reinterpret_cast<const float4*>(col[s] + r) : make_float4(0.f, 0.f, 0.f, 0.f);
    const float2 yh = *reinterpret_cast<const float2*>(a.ds.y32 + gr);
    const float2 yl = *reinterpret_cast<const float2*>(a.ds.y32lo + gr);
#pragma unroll
    for (int u = 0; u < 2; ++u) {
      // the rebuilt sum in term order, Sum2-style (each term's high part by
      // an exact two-sum, the errors and low parts gathered), then normalised
      dfl yp = dfl_make(0.f, 0.f);
      if (tuned) {
#pragma unroll
        for (int t = 0; t <= kMixedMaxM; ++t) {
          if (t > m) break;
          const int kd = tm.kind[t];
          if (kd == 0) continue;
          dfl f = dfl_make(0.f, 0.f);
#pragma unroll
          for (int s = 0; s < kMixedMaxM; ++s)
            if (s == t) f = u == 0 ? dfl_make(fv[s].x, fv[s].y) : dfl_make(fv[s].z, fv[s].w);
          const dfl cf = dfl_make(tm.hi[t], tm.lo[t]);
          if (kd == 3) {
            const float p = DF_MUL(cf.hi, f.hi);
            acc2(yp, p, DF_FMA(cf.lo, f.hi, DF_FMA(cf.hi, f.lo, DF_FMA(cf.hi, f.hi, -p))));
          } else {
            const dfl term = kd == 1 ? cf : f;
            acc2(yp, term.hi, term.lo);
          }
        }
        yp = dfl_two_sum(yp.hi, yp.lo);
      } else {
        yp = u == 0 ? dfl_make(fv[0].x, fv[0].y) : dfl_make(fv[0].z, fv[0].w);
      }
      const dfl y = u == 0 ? dfl_make(yh.x, yl.x) : dfl_make(yh.y, yl.y);
      // e = y - yp (exact two-sum of the high parts), e^2 into the running sum
      const dfl dh = dfl_two_sum(y.hi, -yp.hi);
      const dfl e = dfl_fast_two_sum(dh.hi, DF_ADD(dh.lo, DF_SUB(y.lo, yp.lo)));
      if (gr + u < n) {
        const float p = DF_MUL(e.hi, e.hi);
        acc2(acc, p, DF_FMA(DF_ADD(e.hi, e.hi), e.lo, DF_FMA(e.hi, e.hi, -p)));
      }
    }
  }
  const dfl v = warp_dfl_sum(dfl_renorm(acc));
  if (lane == 0) {
    red[warp][0] = v.hi;
    red[warp][1] = v.lo;
  }
  __syncthreads();
  if (tid == 0) {
    dfl s = dfl_make(0.f, 0.f);
    for (int w = 0; w < kResidThreads / 32; ++w) s = dfl_add(s, dfl_make(red[w][0], red[w][1]));
    a.sse[(size_t)c * a.n_chunks + qs] = (double)s.hi + (double)s.lo;
  }
  __syncthreads();  // red is reused by the block's next item
}

// ----------------------------------------------------------- launchers ----
size_t fac_eval_smem() { return kFacXOff; }
size_t fac_eval_smem_staged(int chunk, int slots) {
  return kFacStageOff + sizeof(float) * (size_t)(2 * slots + 2) * (size_t)chunk;
}
bool fac_allow_smem() {
  const int big = 227 * 1024;
  return cudaFuncSetAttribute(fac_eval_kernel<4, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ==
             cudaSuccess &&
         cudaFuncSetAttribute(fac_eval_kernel<2, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ==
             cudaSuccess &&
         cudaFuncSetAttribute(fac_eval_kernel<4, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ==
             cudaSuccess &&
         cudaFuncSetAttribute(fac_eval_kernel<2, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, big) ==
             cudaSuccess;
}

namespace {
using EncodeTiledFn = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*,
                                   const cuuint64_t*, const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave,
                                   CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);
EncodeTiledFn encode_tiled() {
  static EncodeTiledFn fn = [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess) {
      cudaGetLastError();
      return (EncodeTiledFn) nullptr;
    }
    return reinterpret_cast<EncodeTiledFn>(p);
  }();
  return fn;
}
// a [rows_dim][n_pad] float array (rows of n_pad floats) as a 2D tensor with
// boxes of kTmaRows x 1
bool encode_2d(CUtensorMap* m, const float* base, int64_t n_pad, int64_t outer) {
  EncodeTiledFn fn = encode_tiled();
  if (!fn || !base || (reinterpret_cast<uintptr_t>(base) & 15) || (n_pad * 4) % 16 != 0) return false;
  const cuuint64_t dims[2] = {(cuuint64_t)n_pad, (cuuint64_t)outer};
  const cuuint64_t strides[1] = {(cuuint64_t)n_pad * sizeof(float)};
  const cuuint32_t box[2] = {(cuuint32_t)kTmaRows, 1};
  const cuuint32_t estr[2] = {1, 1};
  return fn(m, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 2, const_cast<float*>(base), dims, strides, box, estr,
            CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
            CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}
}  // namespace

bool fac_stage_maps(FacEvalArgs& a, const DevData& ds) {
  return encode_2d(&a.tm_xh, ds.X32, ds.n_pad, std::max(ds.d, 1)) &&
         encode_2d(&a.tm_xl, ds.X32lo, ds.n_pad, std::max(ds.d, 1)) && encode_2d(&a.tm_yh, ds.y32, ds.n_pad, 1) &&
         encode_2d(&a.tm_yl, ds.y32lo, ds.n_pad, 1);
}

bool launch_fac_eval(const FacEvalArgs& a, int n_groups, int n_chunks, bool light, cudaStream_t st) {
  if (n_groups <= 0 || n_chunks <= 0) return true;
  if (a.stage) {
    const size_t sm = fac_eval_smem_staged(a.chunk, a.stage_slots);
    if (light) fac_eval_kernel<4, true><<<dim3(n_groups, n_chunks), kFacThreads, sm, st>>>(a);
    else fac_eval_kernel<2, true><<<dim3(n_groups, n_chunks), kFacThreads, sm, st>>>(a);
    return launch_ok("launch_fac_eval");
  }
  const size_t sm = fac_eval_smem();
  if (light) fac_eval_kernel<4, false><<<dim3(n_groups, n_chunks), kFacThreads, sm, st>>>(a);
  else fac_eval_kernel<2, false><<<dim3(n_groups, n_chunks), kFacThreads, sm, st>>>(a);
  return launch_ok("launch_fac_eval");
}
int pair_row_blocks(int64_t n_pad) { return (int)((n_pad + kPairRows - 1) / kPairRows); }
bool launch_pair_sum(const PairArgs& a, int n_super, cudaStream_t st) {
  if (a.n_units <= 0 || n_super <= 0) return true;
  pair_sum_kernel<<<a.n_units * n_super, kPairThreads, 0, st>>>(a);
  return launch_ok("launch_pair_sum");
}
bool launch_pair_reduce(const float2* P, int32_t n_pairs, int32_t n_chunks, int32_t p0, int32_t p1, double* psum,
                        cudaStream_t st, const int32_t* smap, const int32_t* omap) {
  if (p1 <= p0) return true;
  pair_reduce_kernel<<<(p1 - p0 + 255) / 256, 256, 0, st>>>(P, n_pairs, n_chunks, p0, p1, psum, smap, omap);
  return launch_ok("launch_pair_reduce");
}
bool launch_fill_slots(const int32_t* idx, int32_t n, unsigned long long* dst, int words, unsigned long long v,
                       cudaStream_t st) {
  if (n <= 0) return true;
  fill_slots_kernel<<<(n + 255) / 256, 256, 0, st>>>(idx, n, dst, words, v);
  return launch_ok("launch_fill_slots");
}
bool launch_ftab_resid(const ResidArgs& a, cudaStream_t st, int max_blocks) {
  if (a.n2 <= 0 || a.n_chunks <= 0) return true;
  const int64_t items = (int64_t)a.n2 * a.n_chunks;
  const int grid = (int)(max_blocks > 0 ? std::min<int64_t>(items, max_blocks) : items);
  ftab_resid_kernel<<<grid, kResidThreads, 0, st>>>(a);
  return launch_ok("launch_ftab_resid");
}

}  // namespace rrd
