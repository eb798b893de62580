// Context and dataset objects behind the C ABI (runtime.cu).
#pragma once
#include <cstdint>
#include <vector>

#include "../host/colcache.h"
#include "common.cuh"

// Device allocation that only grows.  With an owner stream, allocation and
// release are stream-ordered (the device's memory pool, kept cached): the
// old allocation is freed behind the work already queued on that stream and
// nothing waits for the device; the owner's side streams only touch it
// after forking from that stream.
struct DevBuf {
  void* ptr = nullptr;
  size_t cap = 0;
  cudaStream_t st = nullptr;      // owner stream (nullptr: plain cudaMalloc / cudaFree)
  const bool* frozen = nullptr;   // while *frozen (a graph capture), growth is refused
  bool reserve(size_t bytes);
  // grows to `bytes` keeping the first `keep` bytes (a stream-ordered copy)
  bool grow_keep(size_t bytes, size_t keep);
  void release();
};
// Pinned host allocation that only grows.
struct HostBuf {
  void* ptr = nullptr;
  size_t cap = 0;
  uint64_t used_in = 0;  // round sequence number of its last upload (0: none)
  bool reserve(size_t bytes);
  void release();
};

struct rrg_dataset {
  rrg_context* ctx = nullptr;
  uint64_t uid = 0;  // unique on its context: the column caches' entries belong to it
  int64_t n = 0, n_pad = 0;
  int32_t d = 0;
  double* X64 = nullptr;
  float* X32 = nullptr;
  float* X32lo = nullptr;
  double* y64 = nullptr;
  float* y32 = nullptr;
  float* y32lo = nullptr;
  double ymean = 0, sst = 0, ysum = 0, yy = 0;
  rrd::DevData view() const;
};

// Distinct factor programs of a round's batch (host side), shared by the
// candidates that use them.
struct FactorTable {
  std::vector<uint32_t> code;      // programs in id order, each ending in EMIT 0
  std::vector<int2> meta;          // [f] (code offset, length)
  std::vector<int32_t> stack;      // [f] spill depth
  std::vector<int32_t> occ;        // [f] factor instances in the batch
  std::vector<int32_t> cand_off;   // [c] first entry of candidate c in ids (n_cand + 1 entries)
  std::vector<int32_t> ids;        // factor id of every factor slot, candidates in order
};
void build_factor_table(const rrg_cand* cands, int32_t n_cand, const uint32_t* code, const double* consts,
                        FactorTable& ft);

struct rrg_context {
  int device = 0;
  int sm_count = 0;
  size_t scratch_budget_bytes = 0;  // FP64 tables and QR working columns
  size_t table_budget_bytes = 0;    // FP32 factor table of a mixed round
  cudaStream_t stream = nullptr;
  cudaEvent_t done = nullptr;
  // side streams: QR launches of different register buckets run side by side
  static constexpr int kSide = 4;
  cudaStream_t side[kSide] = {nullptr};
  cudaEvent_t fork_ev = nullptr, join_ev[kSide] = {nullptr};
  cudaEvent_t tune_ev[2] = {nullptr, nullptr};  // launch-shape trials (timing events)
  // batch staging
  HostBuf h_batch;
  DevBuf d_batch;
  size_t off_c = 0, off_f = 0, off_k = 0, off_d = 0, off_s = 0, off_sl = 0, batch_bytes = 0;
  rrd::DevBatch dev{};
  std::vector<rrg_cand> host_cands;
  // plain scratch
  DevBuf d_A, d_pc, d_partial, d_list;
  // chunked-QR state and chunk totals (qr_chunk.cu); blocks per SM of its
  // passes by column group (0: not asked yet)
  DevBuf d_qrs;
  int qr_bps[3] = {0, 0, 0};
  int qr_blocks(int max_cols, int64_t items);
  HostBuf h_pc, h_list;
  // mixed scratch
  DevBuf d_terms, d_fallback, d_sse1, d_probe, d_nanrow, d_cert_e;
  HostBuf h_mlist, h_fallback;
  // device-decided second half of a mixed round (residual-pass list, FP64
  // re-scoring lane): its buffers, and the read-back of its statistics
  DevBuf d_rlist2, d_fbpack, d_fbneed, d_fbcols, d_fbF64, d_fbcst, d_fbgram, d_fbblist, d_fbM, d_fbctr;
  HostBuf h_fbpack, h_fbstat;
  bool fbstat_pending = false;
  int32_t fbstat_levels = 0;
  double fbstat_rows = 0.0;
  int32_t fbstat_d = 0;
  bool async_rounds = true;  // mixed rounds decide their second half on the device
  uint64_t round_seq = 0;    // rounds submitted on this context
  // CUDA graph form of a round (rrg_context_set_graph)
  bool graph_rounds = false;
  bool capturing = false;            // the context stream is being captured: no host waits
  bool last_graph = false;           // the last round ran as a graph
  int64_t graph_fallbacks = 0;       // rounds that could not be captured
  cudaGraphExec_t graph_exec = nullptr;
  // factor tables
  FactorTable ft;
  HostBuf h_ft, h_ftp, h_ft64;
  DevBuf d_ft, d_ftp, d_ft64, d_F, d_P, d_Pc, d_psum, d_F64, d_M, d_gram;
  // factor columns kept across rounds of one dataset (colcache.h): the
  // double-float columns of mixed rounds (arena d_F, with per slot the three
  // self sums d_cself, the probe record d_cprobe and the first NaN row
  // d_cfnan) and the FP64 columns of the FP64 table (arena d_F64, column
  // statistics d_ccst)
  bool cache_on = true;
  ColumnCache fcache, pcache;
  FactorRegistry freg;  // factor ids of the pair cache
  PairCache pairc;      // cross-pair sums kept across rounds (slots of d_psum)
  DevBuf d_cself, d_cprobe, d_cfnan, d_ccst, d_slots;
  int64_t fcache_npad = 0, pcache_npad = 0;  // the row padding the arenas' slots are sized for
  uint64_t next_uid = 0;
  int64_t last_cache_hits = 0, last_cache_evals = 0, last_cache64_hits = 0, last_cache64_evals = 0;
  int64_t last_pair_hits = 0, last_pair_evals = 0;
  // the factor programs of the last re-scoring lane whose columns it may
  // have evaluated (its marks come back in h_fbneed with the round), stored
  // into the FP64 cache when the next round starts
  struct LaneStore {
    bool valid = false;
    uint64_t uid = 0;
    int64_t n_pad = 0;
    std::vector<uint32_t> code;
    std::vector<int2> meta;
    std::vector<double> consts;
    std::vector<int32_t> col;  // the lane table column of each program
  } lane_store;
  HostBuf h_fbneed, h_store;
  DevBuf d_store;
  rrg_status store_lane_columns();
  void clear_caches() {
    fcache.clear();
    pcache.clear();
    pairc.clear();
    lane_store.valid = false;
  }
  // results
  DevBuf d_res, d_coefs, d_status;
  HostBuf h_res, h_coefs, h_status;
  // round in flight
  bool in_flight = false;
  rrg_result* out_results = nullptr;
  double* out_coefs = nullptr;
  int32_t out_n = 0;
  int64_t out_ncoef = 0;
  int64_t launches = 0, last_launches = 0;
  // mixed-round statistics of the last round
  int64_t last_fallback = 0, last_plain_routed = 0, last_pass2 = 0, last_sentinel = 0;
  int64_t last_distinct = 0;  // candidates scored after merging identical factor lists
  bool last_tiled = false;    // always false: every round's QR is the direct one
  int64_t last_reasons[16] = {0};
  // certified bound on the relative fitness error of a mixed result; larger
  // bounds are re-scored by the FP64 path
  double cert_tol = 5e-7;
  // datasets with fewer rows run mixed-precision rounds in FP64 (at 569 rows
  // a 600-candidate round takes 1.4 ms in FP64 against 3.0 ms mixed; the
  // mixed form wins from about 7000 rows)
  int64_t mixed_min_rows = 8192;
  // optional per-phase device timing (CUDA events on the context stream)
  bool timing = false;
  enum Phase { P_GRAM = 0, P_SOLVE, P_RESID, P_FINAL, P_PLAIN_EVAL, P_PLAIN_QR, P_PLAIN_RESID, P_PAIRS, P_COUNT };
  std::vector<std::pair<int, std::pair<cudaEvent_t, cudaEvent_t>>> marks;
  std::vector<cudaEvent_t> event_pool;
  size_t event_next = 0;
  double phase_ms[P_COUNT] = {0};
  int64_t phase_launches[P_COUNT] = {0};
  double phase_bytes[P_COUNT] = {0};      // algorithmic bytes (host-counted phases)
  double last_phase_bytes[P_COUNT] = {0};
  cudaEvent_t mark_begin();
  void mark_end(int phase, cudaEvent_t begin);
  // device milliseconds of the launches fn() makes on the context stream
  // (the host waits for them): one shape of a launch-shape trial
  template <class F>
  rrg_status time_trial(F&& fn, float& ms) {
    if (cudaEventRecord(tune_ev[0], stream) != cudaSuccess) return trial_error();
    fn();
    if (cudaEventRecord(tune_ev[1], stream) != cudaSuccess || cudaEventSynchronize(tune_ev[1]) != cudaSuccess ||
        cudaEventElapsedTime(&ms, tune_ev[0], tune_ev[1]) != cudaSuccess)
      return trial_error();
    return RRG_OK;
  }
  rrg_status trial_error();

  rrg_status stage_batch(const rrg_batch* b);
  // the values of candidate 0 (an untuned program) on every row, into d_A
  rrg_status run_predict(const rrg_dataset* ds);
  // mixed round over the shared FP32 factor table; FP64 re-scoring of the
  // candidates it cannot decide
  rrg_status run_mixed(const rrg_dataset* ds, const std::vector<int32_t>& cands, bool certify);
  // async: decide the residual-pass list and the FP64 re-scoring on the
  // device (no read-back); returns with *async_done = false when this
  // sub-round could not (then the re-scored candidates are in fb_all)
  rrg_status mixed_subround(const rrg_dataset* ds, const int32_t* list, int32_t cnt, const std::vector<int32_t>& lf,
                            const std::vector<int32_t>& lid, bool certify, std::vector<int32_t>& fb_all,
                            bool async, bool* async_done);
  // plain FP64 arithmetic over a shared FP64 factor table with the direct QR
  // per candidate (bit-identical to run_plain's direct QR)
  rrg_status run_fp64_table(const rrg_dataset* ds, const std::vector<int32_t>& list, uint32_t flags_or);
  // candidates with identical factor lists: dup_of[c] = the one scored for c
  std::vector<int32_t> dup_of;
  void dedup_candidates(std::vector<int32_t>& reps);
  rrg_status submit(rrg_dataset* ds, const rrg_batch* b, int32_t precision, rrg_result* results, double* coefs);
  rrg_status enqueue_round(rrg_dataset* ds, const rrg_batch* b, int32_t precision, int64_t n_coefs);
  rrg_status wait(int32_t timeout_ms);
  // datasets created on this context and not yet destroyed: destroying the
  // context first releases their device memory and leaves their handles
  // detached (rrg_dataset_destroy then only frees the handle)
  std::vector<rrg_dataset*> datasets;
  std::vector<DevBuf*> all_bufs();  // every device buffer the context owns
  int64_t device_bytes();           // device memory they hold
  ~rrg_context();
};
