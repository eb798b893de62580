// Device runtime and C ABI of the GB300 fitness path (include/rils_rols_gb300.h).
//
// A context owns one CUDA stream, pinned staging buffers and device arenas
// that only grow.  A round is: validate the batch on the host, pack it into
// pinned staging, one host-to-device copy, the kernels of the chosen
// precision (plain.cu or mixed.cu), one device-to-host copy of the results,
// and an event that rrg_round_wait polls with a bounded wait.
#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include "../common/error.h"
#include "../common/df32.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "ftable.cuh"
#include "mixed.cuh"
#include "plain.cuh"
#include "qr_chunk.cuh"
#include "runtime.cuh"

using namespace rrd;

namespace {

bool cuda_ok(cudaError_t e, const char* what) {
  if (e == cudaSuccess) return true;
  rrc::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}

#define RRG_CUDA(call)                                   \
  do {                                                   \
    if (!cuda_ok((call), #call)) return RRG_E_CUDA;      \
  } while (0)

}  // namespace

// ------------------------------------------------------------- buffers ----
bool DevBuf::reserve(size_t bytes) {
  if (bytes <= cap) return true;
  if (frozen && *frozen) return false;  // an allocation would become part of the captured graph
  if (ptr) {
    if (st) {
      cudaFreeAsync(ptr, st);  // after the queued kernels that may still use it
    } else {
      cudaDeviceSynchronize();  // queued kernels may still use the old buffer
      cudaFree(ptr);
    }
  }
  ptr = nullptr;
  cap = 0;
  size_t want = round_up((int64_t)bytes, 1 << 20);
  auto alloc = [&](size_t b) { return (st ? cudaMallocAsync(&ptr, b, st) : cudaMalloc(&ptr, b)) == cudaSuccess; };
  if (!alloc(want)) {
    cudaGetLastError();
    if (!alloc(bytes)) {
      cudaGetLastError();
      ptr = nullptr;
      return false;
    }
    want = bytes;
  }
  cap = want;
  return true;
}
bool DevBuf::grow_keep(size_t bytes, size_t keep) {
  if (bytes <= cap) return true;
  if (frozen && *frozen) return false;
  size_t want = round_up((int64_t)bytes, 1 << 20);
  void* np = nullptr;
  auto alloc = [&](size_t b) { return (st ? cudaMallocAsync(&np, b, st) : cudaMalloc(&np, b)) == cudaSuccess; };
  if (!alloc(want)) {
    cudaGetLastError();
    if (!alloc(bytes)) {
      cudaGetLastError();
      return false;
    }
    want = bytes;
  }
  if (ptr) {
    keep = std::min(keep, cap);
    if (keep && cudaMemcpyAsync(np, ptr, keep, cudaMemcpyDeviceToDevice, st) != cudaSuccess) {
      cudaGetLastError();
      if (st) cudaFreeAsync(np, st);
      else cudaFree(np);
      return false;
    }
    if (st) {
      cudaFreeAsync(ptr, st);
    } else {
      cudaDeviceSynchronize();
      cudaFree(ptr);
    }
  }
  ptr = np;
  cap = want;
  return true;
}

void DevBuf::release() {
  if (ptr) {
    if (st) cudaFreeAsync(ptr, st);
    else cudaFree(ptr);
  }
  ptr = nullptr;
  cap = 0;
}
bool HostBuf::reserve(size_t bytes) {
  if (bytes <= cap) return true;
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  cap = 0;
  size_t want = round_up((int64_t)std::max(bytes, (size_t)(1 << 16)), 1 << 16);
  if (cudaMallocHost(&ptr, want) != cudaSuccess) {
    cudaGetLastError();
    ptr = nullptr;
    return false;
  }
  cap = want;
  return true;
}
void HostBuf::release() {
  if (ptr) cudaFreeHost(ptr);
  ptr = nullptr;
  cap = 0;
}

// --------------------------------------------------------------- timing ----
namespace rrd {
bool launch_ok(const char* what) {
  const cudaError_t e = cudaGetLastError();
  if (e == cudaSuccess) return true;
  rrc::set_error(std::string(what) + ": " + cudaGetErrorString(e));
  return false;
}
}  // namespace rrd

cudaEvent_t rrg_context::mark_begin() {
  if (!timing) return nullptr;
  if (event_next >= event_pool.size()) {
    cudaEvent_t e;
    if (cudaEventCreate(&e) != cudaSuccess) return nullptr;
    event_pool.push_back(e);
  }
  cudaEvent_t e = event_pool[event_next++];
  cudaEventRecord(e, stream);
  return e;
}
void rrg_context::mark_end(int phase, cudaEvent_t begin) {
  if (!timing || !begin) return;
  cudaEvent_t e = mark_begin();
  if (e) marks.push_back({phase, {begin, e}});
}

// ----------------------------------------------------------- validation ----
// Every instruction is checked on the host so that kernels never index out of
// bounds: opcodes, feature and constant indices, factor slots, and the spill
// depth of every program.
static rrg_status validate(const rrg_batch* b, int32_t d, int64_t* n_coefs_out) {
  if (!b || b->n_cand < 0 || b->n_factors < 0 || b->n_code < 0 || b->n_consts < 0) return RRG_E_INVALID;
  if (b->n_cand > 0 && (!b->cands || !b->factors || !b->code)) return RRG_E_INVALID;
  int64_t n_coefs = 0;
  for (int32_t c = 0; c < b->n_cand; ++c) {
    const rrg_cand& cd = b->cands[c];
    if (cd.code_offset < 0 || cd.code_len < 0 || (int64_t)cd.code_offset + cd.code_len > b->n_code) return RRG_E_INVALID;
    if (cd.code_len == 0 && !(cd.mode == RRG_TUNED && cd.n_factors == 0)) return RRG_E_INVALID;
    if (cd.first_factor < 0 || cd.n_factors < 0 || (int64_t)cd.first_factor + cd.n_factors > b->n_factors)
      return RRG_E_INVALID;
    if (cd.mode == RRG_TUNED) {
      if (cd.n_factors + 1 > RRG_MAX_TERMS) return RRG_E_TOO_LARGE;
      if (cd.coef_offset < 0) return RRG_E_INVALID;
      n_coefs = std::max(n_coefs, (int64_t)cd.coef_offset + cd.n_factors + 1);
    } else if (cd.mode == RRG_UNTUNED) {
      if (cd.n_factors != 1) return RRG_E_INVALID;
    } else {
      return RRG_E_INVALID;
    }
    if (cd.stack_need < 0 || cd.stack_need > RRG_MAX_STACK) return RRG_E_TOO_LARGE;
    int sp = 0, depth = 0, emitted = 0;
    bool live = false;
    for (int32_t pc = 0; pc < cd.code_len; ++pc) {
      const uint32_t w = b->code[cd.code_offset + pc];
      const int op = (int)(w & 0xffu);
      const uint32_t arg = w >> 8;
      switch (op) {
        case RRG_OP_LDV: case RRG_OP_PSV:
          if ((int64_t)arg >= d) return RRG_E_INVALID;
          break;
        case RRG_OP_LDC: case RRG_OP_PSC:
          if ((int64_t)arg >= b->n_consts) return RRG_E_INVALID;
          break;
        default: break;
      }
      if (op == RRG_OP_LDV || op == RRG_OP_LDC) {
        if (live) return RRG_E_INVALID;
        live = true;
      } else if (op == RRG_OP_PSV || op == RRG_OP_PSC) {
        if (!live) return RRG_E_INVALID;
        if (++sp > RRG_MAX_STACK) return RRG_E_TOO_LARGE;
        depth = std::max(depth, sp);
      } else if (op >= RRG_OP_SIN && op <= RRG_OP_SQR) {
        if (!live) return RRG_E_INVALID;
      } else if (op == RRG_OP_EMIT) {
        if (!live || (int)arg != emitted || sp != 0) return RRG_E_INVALID;
        ++emitted;
        live = false;
      } else if (op >= RRG_OP_BIN) {
        const int k = op - RRG_OP_BIN;
        if (k >= 8 * RRG_N_BASE || (k & 7) >= 6 || !live) return RRG_E_INVALID;
        const int src = (k & 7) >> 1;
        if (src == RRG_SRC_S) {
          if (--sp < 0) return RRG_E_INVALID;
        } else if (src == RRG_SRC_V) {
          if ((int64_t)arg >= d) return RRG_E_INVALID;
        } else if ((int64_t)arg >= b->n_consts) {
          return RRG_E_INVALID;
        }
      } else {
        return RRG_E_INVALID;
      }
    }
    if (live || emitted != cd.n_factors || depth > cd.stack_need) return RRG_E_INVALID;
  }
  *n_coefs_out = n_coefs;
  return RRG_OK;
}

// -------------------------------------------------------------- context ----
rrg_status rrg_context::stage_batch(const rrg_batch* b) {
  const size_t sz_c = sizeof(rrg_cand) * b->n_cand, sz_f = sizeof(rrg_factor) * b->n_factors;
  const size_t sz_k = sizeof(uint32_t) * b->n_code, sz_d = sizeof(double) * b->n_consts;
  const size_t sz_s = sizeof(float) * b->n_consts;
  off_c = 0;
  off_f = round_up(off_c + sz_c, 256);
  off_k = round_up(off_f + sz_f, 256);
  off_d = round_up(off_k + sz_k, 256);
  off_s = round_up(off_d + sz_d, 256);
  off_sl = round_up(off_s + sz_s, 256);
  batch_bytes = round_up(off_sl + sz_s + 8, 256);
  if (!h_batch.reserve(batch_bytes) || !d_batch.reserve(batch_bytes)) {
    rrc::set_error("cannot reserve batch staging");
    return RRG_E_OOM;
  }
  char* h = static_cast<char*>(h_batch.ptr);
  if (sz_c) std::memcpy(h + off_c, b->cands, sz_c);
  if (sz_f) std::memcpy(h + off_f, b->factors, sz_f);
  if (sz_k) std::memcpy(h + off_k, b->code, sz_k);
  if (sz_d) std::memcpy(h + off_d, b->consts, sz_d);
  // constants as double-floats (high part: the FP32 rounding)
  float* c32 = reinterpret_cast<float*>(h + off_s);
  float* c32lo = reinterpret_cast<float*>(h + off_sl);
  for (int32_t i = 0; i < b->n_consts; ++i) {
    const dfl v = dfl_from_double(b->consts[i]);
    c32[i] = v.hi;
    c32lo[i] = v.lo;
  }
  char* d = static_cast<char*>(d_batch.ptr);
  dev.cands = reinterpret_cast<const rrg_cand*>(d + off_c);
  dev.factors = reinterpret_cast<const rrg_factor*>(d + off_f);
  dev.code = reinterpret_cast<const uint32_t*>(d + off_k);
  dev.consts = reinterpret_cast<const double*>(d + off_d);
  dev.consts32 = reinterpret_cast<const float*>(d + off_s);
  dev.consts32lo = reinterpret_cast<const float*>(d + off_sl);
  dev.n_cand = b->n_cand;
  dev.n_factors = b->n_factors;
  dev.n_code = b->n_code;
  dev.n_consts = b->n_consts;
  host_cands.assign(b->cands, b->cands + b->n_cand);
  if (!cuda_ok(cudaMemcpyAsync(d_batch.ptr, h_batch.ptr, batch_bytes, cudaMemcpyHostToDevice, stream),
               "batch upload"))
    return RRG_E_CUDA;
  return RRG_OK;
}

// The values of candidate 0 (one untuned program) on every row, into d_A.
rrg_status rrg_context::run_predict(const rrg_dataset* ds) {
  const DevData dd = ds->view();
  std::vector<PlainCand> pcs(host_cands.size());
  pcs[0] = PlainCand{0, 0, 0, 1, 0};
  const size_t pc_bytes = sizeof(PlainCand) * pcs.size();
  if (!d_A.reserve((size_t)ds->n_pad * sizeof(double)) || !d_pc.reserve(pc_bytes) || !h_pc.reserve(pc_bytes)) {
    rrc::set_error("device scratch allocation failed");
    return RRG_E_OOM;
  }
  // h_pc may still feed a copy queued by an earlier call of this round
  if (h_pc.used_in == round_seq) RRG_CUDA(cudaStreamSynchronize(stream));
  h_pc.used_in = round_seq;
  std::memcpy(h_pc.ptr, pcs.data(), pc_bytes);
  RRG_CUDA(cudaMemcpyAsync(d_pc.ptr, h_pc.ptr, pc_bytes, cudaMemcpyHostToDevice, stream));
  const int nb = (int)std::max<int64_t>(1, std::min<int64_t>(4LL * sm_count, (ds->n + 1023) / 1024));
  cudaEvent_t t0 = mark_begin();
  plain_eval_kernel<<<dim3(nb, 1), 256, plain_eval_smem(), stream>>>(dev, dd, static_cast<const PlainCand*>(d_pc.ptr),
                                                                      nullptr, 0, static_cast<double*>(d_A.ptr),
                                                                      static_cast<uint32_t*>(d_status.ptr), nullptr);
  mark_end(P_PLAIN_EVAL, t0);
  ++launches;
  RRG_CUDA(cudaGetLastError());
  return RRG_OK;
}

// dup_of[c]: the first candidate with c's mode and factor list (c itself
// when none comes before); reps: those that are their own.
void rrg_context::dedup_candidates(std::vector<int32_t>& reps) {
  const int32_t n = (int32_t)host_cands.size();
  dup_of.assign(n, 0);
  reps.clear();
  // key: the mode and the factor ids in order; a 64-bit hash picks earlier
  // candidates, a comparison of the id lists decides
  std::unordered_map<uint64_t, int32_t> seen;  // hash -> latest representative with it
  std::vector<int32_t> next_same(n, -1);       // earlier representatives with the same hash
  seen.reserve((size_t)n * 2 + 16);
  auto same = [&](int32_t a, int32_t b) {
    const int32_t la = ft.cand_off[a + 1] - ft.cand_off[a], lb = ft.cand_off[b + 1] - ft.cand_off[b];
    return host_cands[a].mode == host_cands[b].mode && la == lb &&
           std::equal(ft.ids.begin() + ft.cand_off[a], ft.ids.begin() + ft.cand_off[a + 1],
                      ft.ids.begin() + ft.cand_off[b]);
  };
  for (int32_t c = 0; c < n; ++c) {
    uint64_t h = 0x9e3779b97f4a7c15ull ^ (uint64_t)(uint32_t)host_cands[c].mode;
    for (int32_t i = ft.cand_off[c]; i < ft.cand_off[c + 1]; ++i) {
      h = (h ^ (uint64_t)(uint32_t)ft.ids[i]) * 0x100000001b3ull;
      h ^= h >> 29;
    }
    auto it = seen.find(h);
    int32_t r = it == seen.end() ? -1 : it->second;
    while (r >= 0 && !same(r, c)) r = next_same[r];
    if (r < 0) {
      next_same[c] = it == seen.end() ? -1 : it->second;
      seen[h] = c;
      dup_of[c] = c;
      reps.push_back(c);
    } else {
      dup_of[c] = r;
    }
  }
}

rrg_status rrg_context::submit(rrg_dataset* ds, const rrg_batch* b, int32_t precision, rrg_result* results,
                               double* coefs) {
  if (in_flight) {
    rrc::set_error("a round is already in flight on this context");
    return RRG_E_INVALID;
  }
  int64_t n_coefs = 0;
  rrg_status st = validate(b, ds->d, &n_coefs);
  if (st != RRG_OK) {
    rrc::set_error("rrg_round_submit: malformed or oversized batch");
    return st;
  }
  if (precision != RRG_PLAIN_FP64 && precision != RRG_MIXED && precision != RRG_MIXED_CERTIFIED)
    return RRG_E_INVALID;
  if (n_coefs > 0 && !coefs) return RRG_E_INVALID;
  RRG_CUDA(cudaSetDevice(device));
  last_graph = false;
  if (graph_rounds && !timing) {
    // the round's work captured from the context stream (and the side
    // streams it forks) into a graph, then launched as one; the graph of the
    // previous round is updated in place when the shapes allow.  A round
    // that cannot be captured (a host wait inside it: a launch-shape trial,
    // a reused staging buffer, table sub-rounds) is enqueued directly.
    cudaGraph_t g = nullptr;
    rrg_status cst = RRG_E_CUDA;
    // the previous lane's columns go into the FP64 cache before the capture
    // (storing them may grow the cache's arena, which a capture refuses)
    const rrg_status sst = store_lane_columns();
    if (sst != RRG_OK) {
      clear_caches();
      return sst;
    }
    if (cudaStreamBeginCapture(stream, cudaStreamCaptureModeRelaxed) == cudaSuccess) {
      capturing = true;
      cst = enqueue_round(ds, b, precision, n_coefs);
      capturing = false;
      const cudaError_t ec = cudaStreamEndCapture(stream, &g);
      if (ec != cudaSuccess) cst = RRG_E_CUDA;
    }
    bool launched = false;
    if (cst == RRG_OK && g) {
      bool ready = false;
      if (graph_exec) {
        cudaGraphExecUpdateResultInfo info;
        ready = cudaGraphExecUpdate(graph_exec, g, &info) == cudaSuccess;
        if (!ready) {
          cudaGetLastError();
          cudaGraphExecDestroy(graph_exec);
          graph_exec = nullptr;
        }
      }
      if (!ready) ready = cudaGraphInstantiate(&graph_exec, g, 0) == cudaSuccess;
      launched = ready && cudaGraphLaunch(graph_exec, stream) == cudaSuccess;
    }
    if (g) cudaGraphDestroy(g);
    if (launched) {
      last_graph = true;
      st = RRG_OK;
    } else {
      cudaGetLastError();
      ++graph_fallbacks;
      // the captured work never ran: the columns it was to leave are not there
      clear_caches();
      st = enqueue_round(ds, b, precision, n_coefs);
    }
  } else {
    st = enqueue_round(ds, b, precision, n_coefs);
  }
  if (st != RRG_OK) {
    clear_caches();  // a round that failed part-way may have left slots unwritten
    return st;
  }
  RRG_CUDA(cudaEventRecord(done, stream));
  in_flight = true;
  out_results = results;
  out_coefs = coefs;
  out_n = b->n_cand;
  out_ncoef = n_coefs;
  return RRG_OK;
}

// The device work of one round on the context stream: batch upload, the
// precision's kernels, the results back into pinned staging.  Everything
// that reaches the device goes through the stream (or side streams forked
// from it), so it can run under stream capture.
rrg_status rrg_context::enqueue_round(rrg_dataset* ds, const rrg_batch* b, int32_t precision, int64_t n_coefs) {
  rrg_status st = RRG_OK;
  // an error another library left pending on this thread is not this
  // round's: clear it so the launch checks below see only their own
  cudaGetLastError();
  ++round_seq;
  fbstat_pending = false;
  launches = 0;
  last_plain_routed = last_fallback = last_pass2 = last_sentinel = 0;
  last_cache_hits = last_cache_evals = last_cache64_hits = last_cache64_evals = 0;
  last_pair_hits = last_pair_evals = 0;
  for (double& v : phase_bytes) v = 0.0;
  for (auto& r : last_reasons) r = 0;
  marks.clear();
  event_next = 0;
  // columns the previous round's re-scoring lane evaluated go into the FP64
  // column cache before anything of this round is queued
  st = store_lane_columns();
  if (st != RRG_OK) return st;
  st = stage_batch(b);
  if (st != RRG_OK) return st;
  const size_t res_bytes = sizeof(rrg_result) * std::max(1, b->n_cand);
  const size_t coef_bytes = sizeof(double) * std::max<int64_t>(1, n_coefs);
  if (!d_res.reserve(res_bytes) || !d_coefs.reserve(coef_bytes) || !d_status.reserve(64) ||
      !h_res.reserve(res_bytes) || !h_coefs.reserve(coef_bytes) || !h_status.reserve(64)) {
    rrc::set_error("cannot reserve result buffers");
    return RRG_E_OOM;
  }
  RRG_CUDA(cudaMemsetAsync(d_res.ptr, 0, res_bytes, stream));
  RRG_CUDA(cudaMemsetAsync(d_coefs.ptr, 0, coef_bytes, stream));
  RRG_CUDA(cudaMemsetAsync(d_status.ptr, 0, 64, stream));
  // distinct factor programs, and candidates with identical factor lists
  // (same programs, same order, same mode) scored once
  build_factor_table(host_cands.data(), b->n_cand, b->code, b->consts, ft);
  std::vector<int32_t> reps;
  dedup_candidates(reps);
  last_distinct = (int64_t)reps.size();
  last_tiled = false;
  // on small datasets the mixed form's probes, pair sums and read-backs cost
  // more than the FP64 arithmetic they replace: such rounds run in FP64
  // (exact, so within any certified bound).  So do rounds on a constant y
  // (SST = 0): R2 = 1 - SSE/SST is then decided by whether the SSE is exactly
  // zero (0/0 gives the NaN sentinel), which only the exact path settles.
  if (precision == RRG_PLAIN_FP64 || ds->n < mixed_min_rows || !(ds->sst > 0.0)) {
    st = run_fp64_table(ds, reps, 0u);
  } else {
    st = run_mixed(ds, reps, precision == RRG_MIXED_CERTIFIED);
  }
  if (st != RRG_OK) return st;
  RRG_CUDA(cudaMemcpyAsync(h_res.ptr, d_res.ptr, res_bytes, cudaMemcpyDeviceToHost, stream));
  RRG_CUDA(cudaMemcpyAsync(h_coefs.ptr, d_coefs.ptr, coef_bytes, cudaMemcpyDeviceToHost, stream));
  RRG_CUDA(cudaMemcpyAsync(h_status.ptr, d_status.ptr, 64, cudaMemcpyDeviceToHost, stream));
  return RRG_OK;
}

rrg_status rrg_context::wait(int32_t timeout_ms) {
  if (!in_flight) return RRG_OK;
  const auto t0 = std::chrono::steady_clock::now();
  for (;;) {
    cudaError_t e = cudaEventQuery(done);
    if (e == cudaSuccess) break;
    if (e != cudaErrorNotReady) {
      in_flight = false;
      clear_caches();
      cuda_ok(e, "round execution");
      return RRG_E_CUDA;
    }
    if (timeout_ms >= 0 &&
        std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(timeout_ms)) {
      rrc::set_error("rrg_round_wait: timed out");
      return RRG_E_TIMEOUT;
    }
    std::this_thread::yield();
  }
  in_flight = false;
  const uint32_t dev_status = *static_cast<uint32_t*>(h_status.ptr);
  if (dev_status != 0) {
    clear_caches();  // columns of a round that reported an error are not kept
    char msg[128];
    std::snprintf(msg, sizeof msg, "device reported error status 0x%x", dev_status);
    rrc::set_error(msg);
    return RRG_E_DEVICE_FAULT;
  }
  last_sentinel = static_cast<const uint32_t*>(h_status.ptr)[rrd::kStatusSentinel];
  for (int i = 0; i < P_COUNT; ++i) last_phase_bytes[i] = phase_bytes[i];
  if (fbstat_pending) {
    // statistics of a mixed round whose second half the device decided
    const int32_t* hs = static_cast<const int32_t*>(h_fbstat.ptr);
    last_fallback += hs[0];
    last_pass2 += hs[1];
    for (int i = 0; i < kFbReasons && i < 16; ++i) last_reasons[i] += static_cast<const uint32_t*>(h_fbstat.ptr)[2 + i];
    int64_t cols = 0;
    for (int32_t L = 0; L < fbstat_levels; ++L) cols += hs[2 + kFbReasons + L];
    last_phase_bytes[P_PLAIN_EVAL] += fbstat_rows * 8.0 * (double)(fbstat_d + cols);
    fbstat_pending = false;
  }
  {
    unsigned long long qb = 0;
    std::memcpy(&qb, static_cast<const uint32_t*>(h_status.ptr) + rrd::kStatusQrBytes, sizeof qb);
    last_phase_bytes[P_PLAIN_QR] += (double)qb;
  }
  for (int i = 0; i < P_COUNT; ++i) {
    phase_ms[i] = 0;
    phase_launches[i] = 0;
  }
  for (auto& mk : marks) {
    float ms = 0;
    if (cudaEventElapsedTime(&ms, mk.second.first, mk.second.second) == cudaSuccess) {
      phase_ms[mk.first] += ms;
      phase_launches[mk.first] += 1;
    }
  }
  if (out_results) std::memcpy(out_results, h_res.ptr, sizeof(rrg_result) * out_n);
  if (out_coefs && out_ncoef > 0) std::memcpy(out_coefs, h_coefs.ptr, sizeof(double) * out_ncoef);
  // candidates scored through an identical one
  for (int32_t c = 0; c < out_n && c < (int32_t)dup_of.size(); ++c) {
    const int32_t r = dup_of[c];
    if (r == c) continue;
    if (out_results) out_results[c] = out_results[r];
    const rrg_cand& cd = host_cands[c];
    if (out_coefs && cd.mode == RRG_TUNED)
      std::memcpy(out_coefs + cd.coef_offset, out_coefs + host_cands[r].coef_offset,
                  sizeof(double) * (size_t)(cd.n_factors + 1));
  }
  last_launches = launches;
  return RRG_OK;
}

std::vector<DevBuf*> rrg_context::all_bufs() {
  return {&d_batch, &d_A, &d_pc, &d_partial, &d_list, &d_qrs, &d_terms, &d_fallback, &d_sse1, &d_probe,
          &d_nanrow, &d_cert_e, &d_ft, &d_ftp, &d_ft64, &d_F, &d_P, &d_Pc, &d_psum, &d_F64, &d_M,
          &d_gram, &d_rlist2, &d_fbpack, &d_fbneed, &d_fbcols, &d_fbF64, &d_fbcst, &d_fbgram, &d_fbblist,
          &d_fbM, &d_fbctr, &d_cself, &d_cprobe, &d_cfnan, &d_ccst, &d_slots, &d_store, &d_res, &d_coefs, &d_status};
}

// Persistent grid of the chunked QR's passes for `items` candidate x chunk items.
int rrg_context::qr_blocks(int max_cols, int64_t items) {
  const int w = max_cols - 1;
  const int g = w <= 4 ? 0 : (w <= 8 ? 1 : 2);
  if (!qr_bps[g]) qr_bps[g] = qr_chunk_blocks_per_sm(max_cols);
  const int64_t cap = (int64_t)sm_count * qr_bps[g];
  return (int)std::max<int64_t>(1, std::min<int64_t>(cap, items));
}

int64_t rrg_context::device_bytes() {
  int64_t t = 0;
  for (DevBuf* b : all_bufs()) t += (int64_t)b->cap;
  return t;
}

namespace {

// the dataset's device columns, freed in the order of `st`
void release_dataset_memory(rrg_dataset* ds, cudaStream_t st) {
  for (void** p : {(void**)&ds->X64, (void**)&ds->X32, (void**)&ds->X32lo, (void**)&ds->y64, (void**)&ds->y32,
                   (void**)&ds->y32lo}) {
    if (*p) cudaFreeAsync(*p, st);
    *p = nullptr;
  }
}

// a dataset whose context was destroyed first has no device data left
bool detached_ok(const rrg_dataset* ds) {
  if (ds->ctx) return true;
  rrc::set_error("the dataset's context was destroyed");
  return false;
}

}  // namespace

rrg_context::~rrg_context() {
  if (in_flight) cudaEventSynchronize(done);
  for (rrg_dataset* ds : datasets) {
    release_dataset_memory(ds, stream);
    ds->ctx = nullptr;
  }
  datasets.clear();
  if (graph_exec) cudaGraphExecDestroy(graph_exec);
  for (DevBuf* bf : all_bufs()) bf->release();
  h_mlist.release();
  h_fallback.release();
  h_list.release();
  h_fbpack.release();
  h_fbstat.release();
  h_fbneed.release();
  h_store.release();
  h_ft.release();
  h_ftp.release();
  h_ft64.release();
  h_batch.release();
  h_res.release();
  h_coefs.release();
  h_status.release();
  h_pc.release();
  for (cudaEvent_t e : event_pool) cudaEventDestroy(e);
  if (done) cudaEventDestroy(done);
  if (stream) cudaStreamDestroy(stream);
  if (fork_ev) cudaEventDestroy(fork_ev);
  for (cudaEvent_t e : tune_ev)
    if (e) cudaEventDestroy(e);
  for (int i = 0; i < kSide; ++i) {
    if (join_ev[i]) cudaEventDestroy(join_ev[i]);
    if (side[i]) cudaStreamDestroy(side[i]);
  }
}

rrg_status rrg_context::trial_error() {
  rrc::set_error(std::string("launch-shape trial: ") + cudaGetErrorString(cudaGetLastError()));
  return RRG_E_CUDA;
}

DevData rrg_dataset::view() const {
  DevData v;
  v.X64 = X64;
  v.X32 = X32;
  v.X32lo = X32lo;
  v.y64 = y64;
  v.y32 = y32;
  v.y32lo = y32lo;
  v.ysum = ysum;
  v.yy = yy;
  v.n = n;
  v.n_pad = n_pad;
  v.d = d;
  v.ymean = ymean;
  v.sst = sst;
  return v;
}

// ------------------------------------------------------------------ ABI ----
namespace {

// X given row-major (n x d) into the padded column layout (rows >= n zero)
__global__ void rows_to_cols_kernel(const double* __restrict__ rows, int64_t n, int32_t d, int64_t n_pad,
                                    double* __restrict__ cols) {
  for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n_pad; i += (int64_t)gridDim.x * blockDim.x)
    for (int32_t j = 0; j < d; ++j) cols[(int64_t)j * n_pad + i] = i < n ? rows[i * d + j] : 0.0;
}

// Shared part of the two entry points: device buffers, the copies queued by
// `upload` on the context stream, the FP32 splits, and meanwhile the sums of
// y in the fixed CSUM order on the host.
template <class Upload>
rrg_status make_dataset(rrg_context* ctx, const double* y, int64_t n, int32_t d, rrg_dataset** out, Upload upload) {
  *out = nullptr;
  RRG_CUDA(cudaSetDevice(ctx->device));
  rrg_dataset* ds = new rrg_dataset();
  ds->ctx = ctx;
  ds->uid = ++ctx->next_uid;
  ctx->datasets.push_back(ds);
  ds->n = n;
  ds->d = d;
  ds->n_pad = round_up(n, 256);
  const int64_t cols = std::max(d, 1);
  const size_t b64 = sizeof(double) * ds->n_pad * cols, b32 = sizeof(float) * ds->n_pad * cols;
  const size_t y64b = sizeof(double) * ds->n_pad, y32b = sizeof(float) * ds->n_pad;
  // stream-ordered on the context stream (no device-wide wait when a
  // dataset comes or goes while other contexts' rounds run)
  cudaStream_t st = ctx->stream;
  auto alloc = [&](void** p, size_t b) { return cudaMallocAsync(p, b, st) == cudaSuccess; };
  if (!alloc((void**)&ds->X64, b64) || !alloc((void**)&ds->X32, b32) || !alloc((void**)&ds->X32lo, b32) ||
      !alloc((void**)&ds->y64, y64b) || !alloc((void**)&ds->y32, y32b) || !alloc((void**)&ds->y32lo, y32b)) {
    cudaGetLastError();
    rrg_dataset_destroy(ds);
    rrc::set_error("rrg_dataset_create: out of device memory");
    return RRG_E_OOM;
  }
  bool ok = cudaMemsetAsync(ds->X64, 0, b64, st) == cudaSuccess && upload(ds, st) &&
            cudaMemcpyAsync(ds->y64, y, sizeof(double) * n, cudaMemcpyHostToDevice, st) == cudaSuccess &&
            cudaMemsetAsync(ds->y64 + n, 0, sizeof(double) * (ds->n_pad - n), st) == cudaSuccess &&
            launch_split_f32(ds->X64, ds->X32, ds->X32lo, ds->n_pad * cols, st) &&
            launch_split_f32(ds->y64, ds->y32, ds->y32lo, ds->n_pad, st);
  // mean and total sum of squares of y (rils_rols_cpp.cpp:41-43) in the fixed
  // CSUM order, while the copies run
  ds->ysum = rr_csum(y, (long)n);
  ds->ymean = ds->ysum / (double)n;
  rr_csum_acc acc;
  rr_csum_init(&acc);
  for (int64_t i = 0; i < n; ++i) rr_csum_add(&acc, (y[i] - ds->ymean) * (y[i] - ds->ymean));
  ds->sst = rr_csum_total(&acc);
  rr_csum_init(&acc);
  for (int64_t i = 0; i < n; ++i) rr_csum_add(&acc, y[i] * y[i]);
  ds->yy = rr_csum_total(&acc);
  ok = ok && cudaStreamSynchronize(st) == cudaSuccess;
  if (!ok) {
    cuda_ok(cudaGetLastError(), "dataset upload");
    rrg_dataset_destroy(ds);
    return RRG_E_CUDA;
  }
  *out = ds;
  return RRG_OK;
}

bool dataset_args_ok(rrg_context* ctx, const double* X, const double* y, int64_t n, int32_t d, rrg_dataset** out) {
  if (!ctx || !out || !y || n <= 0 || d < 0 || (d > 0 && !X) || n > (int64_t)1 << 40) {
    rrc::set_error("rrg_dataset_create: invalid arguments");
    return false;
  }
  return true;
}

}  // namespace

extern "C" {

rrg_status rrg_context_create(int32_t device, rrg_context** out) {
  if (!out) return RRG_E_INVALID;
  *out = nullptr;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || count <= device || device < 0) {
    cudaGetLastError();
    rrc::set_error("no CUDA device available for the GB300 fitness path");
    return RRG_E_NO_DEVICE;
  }
  RRG_CUDA(cudaSetDevice(device));
  cudaDeviceProp prop;
  RRG_CUDA(cudaGetDeviceProperties(&prop, device));
  if (prop.major < 10) {
    rrc::set_error("the GB300 fitness path needs a Blackwell (sm_10x) device");
    return RRG_E_NO_DEVICE;
  }
  rrg_context* ctx = new rrg_context();
  ctx->device = device;
  ctx->sm_count = prop.multiProcessorCount;
  size_t free_b = 0, total_b = 0;
  cudaMemGetInfo(&free_b, &total_b);
  ctx->scratch_budget_bytes = std::min<size_t>((size_t)64 << 30, free_b / 3);
  // the double-float table is also the column cache of the rounds: a search
  // at n = 1M keeps about 8K factor columns in 64 GiB (about 84% of a round's
  // factors are then read instead of evaluated)
  ctx->table_budget_bytes = std::min<size_t>((size_t)64 << 30, free_b / 4);
  bool side_ok = cudaEventCreateWithFlags(&ctx->fork_ev, cudaEventDisableTiming) == cudaSuccess;
  side_ok = side_ok && cudaEventCreate(&ctx->tune_ev[0]) == cudaSuccess && cudaEventCreate(&ctx->tune_ev[1]) == cudaSuccess;
  for (int i = 0; i < rrg_context::kSide && side_ok; ++i)
    side_ok = cudaStreamCreateWithFlags(&ctx->side[i], cudaStreamNonBlocking) == cudaSuccess &&
              cudaEventCreateWithFlags(&ctx->join_ev[i], cudaEventDisableTiming) == cudaSuccess;
  if (!side_ok || cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking) != cudaSuccess ||
      cudaEventCreateWithFlags(&ctx->done, cudaEventDisableTiming) != cudaSuccess) {
    cuda_ok(cudaGetLastError(), "stream creation");
    delete ctx;
    return RRG_E_CUDA;
  }
  if (cudaFuncSetAttribute(plain_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)plain_eval_smem()) !=
          cudaSuccess ||
      !rrd::fac_allow_smem()) {
    cuda_ok(cudaGetLastError(), "kernel attributes");
    delete ctx;
    return RRG_E_CUDA;
  }
  // scratch from the device's memory pool, ordered on the context stream:
  // growing a buffer or freeing it never waits for the device (other
  // contexts' rounds keep running); the pool keeps freed memory for reuse
  // by this process instead of returning it at every synchronisation
  cudaMemPool_t pool;
  if (cudaDeviceGetDefaultMemPool(&pool, device) == cudaSuccess) {
    uint64_t keep = UINT64_MAX;
    cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    for (DevBuf* b : ctx->all_bufs()) {
      b->st = ctx->stream;
      b->frozen = &ctx->capturing;
    }
  }
  cudaGetLastError();
  *out = ctx;
  return RRG_OK;
}

rrg_status rrg_context_destroy(rrg_context* ctx) {
  if (!ctx) return RRG_E_INVALID;
  cudaSetDevice(ctx->device);
  delete ctx;
  return RRG_OK;
}


rrg_status rrg_dataset_create(rrg_context* ctx, const double* X_col, const double* y, int64_t n, int32_t d,
                              rrg_dataset** out) {
  if (!dataset_args_ok(ctx, X_col, y, n, d, out)) return RRG_E_INVALID;
  // each column straight into its padded place (one 2-D copy)
  return make_dataset(ctx, y, n, d, out, [&](rrg_dataset* ds, cudaStream_t st) {
    return d == 0 || cudaMemcpy2DAsync(ds->X64, sizeof(double) * ds->n_pad, X_col, sizeof(double) * n,
                                       sizeof(double) * n, d, cudaMemcpyHostToDevice, st) == cudaSuccess;
  });
}

rrg_status rrg_dataset_create_rows(rrg_context* ctx, const double* X_rows, const double* y, int64_t n, int32_t d,
                                   rrg_dataset** out) {
  if (!dataset_args_ok(ctx, X_rows, y, n, d, out)) return RRG_E_INVALID;
  // the rows as given, then transposed on the device (a stream-ordered
  // temporary)
  return make_dataset(ctx, y, n, d, out, [&](rrg_dataset* ds, cudaStream_t st) {
    if (d == 0) return true;
    void* raw = nullptr;
    const size_t bytes = sizeof(double) * (size_t)n * d;
    if (cudaMallocAsync(&raw, bytes, st) != cudaSuccess) return false;
    bool ok = cudaMemcpyAsync(raw, X_rows, bytes, cudaMemcpyHostToDevice, st) == cudaSuccess;
    if (ok) {
      const int64_t blocks = std::min<int64_t>((ds->n_pad + 255) / 256, 8LL * ctx->sm_count);
      rows_to_cols_kernel<<<(int)blocks, 256, 0, st>>>(static_cast<const double*>(raw), n, d, ds->n_pad, ds->X64);
      ok = cudaGetLastError() == cudaSuccess;
    }
    return cudaFreeAsync(raw, st) == cudaSuccess && ok;
  });
}

rrg_status rrg_dataset_destroy(rrg_dataset* ds) {
  if (!ds) return RRG_E_INVALID;
  rrg_context* ctx = ds->ctx;
  if (ctx) {
    cudaSetDevice(ctx->device);
    if (ctx->in_flight) cudaEventSynchronize(ctx->done);
    // freed behind the context stream's queued work (every round of this
    // dataset ran on that stream or joined it)
    release_dataset_memory(ds, ctx->stream);
    // its kept columns go with it
    if (ctx->fcache.uid() == ds->uid) ctx->fcache.bind(0);
    if (ctx->pcache.uid() == ds->uid) ctx->pcache.bind(0);
    if (ctx->pairc.uid() == ds->uid) ctx->pairc.bind(0);
    auto it = std::find(ctx->datasets.begin(), ctx->datasets.end(), ds);
    if (it != ctx->datasets.end()) ctx->datasets.erase(it);
  }
  delete ds;
  return RRG_OK;
}

rrg_status rrg_round_submit(rrg_dataset* ds, const rrg_batch* batch, int32_t precision, rrg_result* results,
                            double* coefs) {
  if (!ds || !batch || (!results && batch->n_cand > 0)) return RRG_E_INVALID;
  if (!detached_ok(ds)) return RRG_E_INVALID;
  return ds->ctx->submit(ds, batch, precision, results, coefs);
}

rrg_status rrg_round_wait(rrg_context* ctx, int32_t timeout_ms) {
  if (!ctx) return RRG_E_INVALID;
  return ctx->wait(timeout_ms);
}

rrg_status rrg_eval(rrg_dataset* ds, const rrg_batch* batch, int32_t precision, rrg_result* results, double* coefs) {
  rrg_status st = rrg_round_submit(ds, batch, precision, results, coefs);
  if (st != RRG_OK) return st;
  return ds->ctx->wait(-1);
}

rrg_status rrg_predict(rrg_dataset* ds, const rrg_batch* batch, double* values) {
  if (!ds || !batch || !values || batch->n_cand < 1) return RRG_E_INVALID;
  if (!detached_ok(ds)) return RRG_E_INVALID;
  rrg_context* ctx = ds->ctx;
  if (ctx->in_flight) return RRG_E_INVALID;
  int64_t n_coefs = 0;
  rrg_batch one = *batch;
  one.n_cand = 1;
  rrg_status st = validate(&one, ds->d, &n_coefs);
  if (st != RRG_OK || one.cands[0].mode != RRG_UNTUNED) {
    rrc::set_error("rrg_predict: candidate 0 must be a valid untuned program");
    return RRG_E_INVALID;
  }
  RRG_CUDA(cudaSetDevice(ctx->device));
  cudaGetLastError();  // not this call's: an error left pending on this thread by other code
  ++ctx->round_seq;
  st = ctx->stage_batch(&one);
  if (st != RRG_OK) return st;
  if (!ctx->d_status.reserve(64) || !ctx->h_status.reserve(64)) return RRG_E_OOM;
  RRG_CUDA(cudaMemsetAsync(ctx->d_status.ptr, 0, 64, ctx->stream));
  st = ctx->run_predict(ds);
  if (st != RRG_OK) return st;
  RRG_CUDA(cudaMemcpyAsync(ctx->h_status.ptr, ctx->d_status.ptr, 64, cudaMemcpyDeviceToHost, ctx->stream));
  RRG_CUDA(cudaMemcpyAsync(values, ctx->d_A.ptr, sizeof(double) * ds->n, cudaMemcpyDeviceToHost, ctx->stream));
  RRG_CUDA(cudaStreamSynchronize(ctx->stream));
  if (*static_cast<uint32_t*>(ctx->h_status.ptr) != 0) {
    rrc::set_error("rrg_predict: device reported an error status");
    return RRG_E_DEVICE_FAULT;
  }
  return RRG_OK;
}

rrg_status rrg_batch_validate(const rrg_batch* batch, int32_t d) {
  int64_t n_coefs = 0;
  rrg_status st = validate(batch, d, &n_coefs);
  if (st != RRG_OK) rrc::set_error("rrg_batch_validate: malformed or oversized batch");
  return st;
}

int64_t rrg_dataset_rows(const rrg_dataset* ds) { return ds ? ds->n : -1; }
int32_t rrg_dataset_cols(const rrg_dataset* ds) { return ds ? ds->d : -1; }
int64_t rrg_last_round_launches(const rrg_context* ctx) { return ctx ? ctx->last_launches : -1; }

int32_t rrg_last_round_stats(const rrg_context* ctx, int64_t* out, int32_t n) {
  if (!ctx || !out || n <= 0) return 0;
  int64_t v[14 + kFbReasons] = {ctx->last_launches, ctx->last_plain_routed, ctx->last_fallback, ctx->last_pass2};
  for (int i = 0; i < kFbReasons; ++i) v[4 + i] = ctx->last_reasons[i];
  v[4 + kFbReasons] = ctx->last_sentinel;
  v[5 + kFbReasons] = ctx->last_distinct;
  v[6 + kFbReasons] = ctx->last_tiled ? 1 : 0;
  v[7 + kFbReasons] = ctx->last_graph ? 1 : 0;
  v[8 + kFbReasons] = ctx->last_cache_hits;
  v[9 + kFbReasons] = ctx->last_cache_evals;
  v[10 + kFbReasons] = ctx->last_cache64_hits;
  v[11 + kFbReasons] = ctx->last_cache64_evals;
  v[12 + kFbReasons] = ctx->last_pair_hits;
  v[13 + kFbReasons] = ctx->last_pair_evals;
  const int32_t k = n < 14 + kFbReasons ? n : 14 + kFbReasons;
  for (int32_t i = 0; i < k; ++i) out[i] = v[i];
  return k;
}

void* rrg_context_stream(const rrg_context* ctx) { return ctx ? (void*)ctx->stream : nullptr; }

rrg_status rrg_context_set_timing(rrg_context* ctx, int32_t on) {
  if (!ctx) return RRG_E_INVALID;
  ctx->timing = on != 0;
  return RRG_OK;
}

int64_t rrg_context_memory(rrg_context* ctx) { return ctx ? ctx->device_bytes() : -1; }

rrg_status rrg_context_set_graph(rrg_context* ctx, int32_t on) {
  if (!ctx) return RRG_E_INVALID;
  if (ctx->in_flight) {
    rrc::set_error("rrg_context_set_graph: a round is in flight");
    return RRG_E_INVALID;
  }
  ctx->graph_rounds = on != 0;
  return RRG_OK;
}

rrg_status rrg_context_set_column_cache(rrg_context* ctx, int32_t on) {
  if (!ctx) return RRG_E_INVALID;
  if (ctx->in_flight) {
    rrc::set_error("rrg_context_set_column_cache: a round is in flight");
    return RRG_E_INVALID;
  }
  ctx->cache_on = on != 0;
  ctx->clear_caches();
  return RRG_OK;
}

rrg_status rrg_context_clear_column_cache(rrg_context* ctx) {
  if (!ctx) return RRG_E_INVALID;
  if (ctx->in_flight) {
    rrc::set_error("rrg_context_clear_column_cache: a round is in flight");
    return RRG_E_INVALID;
  }
  ctx->clear_caches();
  return RRG_OK;
}

rrg_status rrg_context_set_async(rrg_context* ctx, int32_t on) {
  if (!ctx) return RRG_E_INVALID;
  if (ctx->in_flight) {
    rrc::set_error("rrg_context_set_async: a round is in flight");
    return RRG_E_INVALID;
  }
  ctx->async_rounds = on != 0;
  return RRG_OK;
}

rrg_status rrg_context_set_mixed_min_rows(rrg_context* ctx, int64_t rows) {
  if (!ctx || rows < 0) {
    rrc::set_error("rrg_context_set_mixed_min_rows: invalid arguments");
    return RRG_E_INVALID;
  }
  ctx->mixed_min_rows = rows;
  return RRG_OK;
}

rrg_status rrg_context_set_limits(rrg_context* ctx, int64_t scratch_bytes, int64_t table_bytes) {
  if (!ctx || scratch_bytes < (1 << 20) || table_bytes < (1 << 20)) {
    rrc::set_error("rrg_context_set_limits: invalid arguments (each limit at least 1 MiB)");
    return RRG_E_INVALID;
  }
  ctx->scratch_budget_bytes = (size_t)scratch_bytes;
  ctx->table_budget_bytes = (size_t)table_bytes;
  return RRG_OK;
}

rrg_status rrg_device_memory(int32_t device, int64_t* free_bytes, int64_t* total_bytes) {
  if (!free_bytes || !total_bytes) return RRG_E_INVALID;
  int count = 0;
  if (cudaGetDeviceCount(&count) != cudaSuccess || device < 0 || device >= count) {
    cudaGetLastError();
    rrc::set_error("no CUDA device available for the GB300 fitness path");
    return RRG_E_NO_DEVICE;
  }
  RRG_CUDA(cudaSetDevice(device));
  size_t f = 0, t = 0;
  RRG_CUDA(cudaMemGetInfo(&f, &t));
  *free_bytes = (int64_t)f;
  *total_bytes = (int64_t)t;
  return RRG_OK;
}

int32_t rrg_last_round_bytes(const rrg_context* ctx, double* bytes, int32_t n) {
  if (!ctx || !bytes || n <= 0) return 0;
  const int32_t k = n < (int32_t)rrg_context::P_COUNT ? n : (int32_t)rrg_context::P_COUNT;
  for (int32_t i = 0; i < k; ++i) bytes[i] = ctx->last_phase_bytes[i];
  return k;
}

int32_t rrg_last_round_timing(const rrg_context* ctx, double* ms, int64_t* launches, int32_t n) {
  if (!ctx || !ms || n <= 0) return 0;
  const int32_t k = n < (int32_t)rrg_context::P_COUNT ? n : (int32_t)rrg_context::P_COUNT;
  for (int32_t i = 0; i < k; ++i) {
    ms[i] = ctx->phase_ms[i];
    if (launches) launches[i] = ctx->phase_launches[i];
  }
  return k;
}

}  // extern "C"
