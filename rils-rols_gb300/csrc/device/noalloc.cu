// Allocation-free scoring of one candidate on the plain FP64 path:
// rrg_eval_plain_noalloc (declared in include/rils_rols_gb300.h).
//
// Who needs it: callers that may not allocate device memory themselves or
// have a library do it for them.  A host framework that hands out every byte
// of device memory from its own pool cannot have a cudaMalloc happen behind
// its back (it would break the framework's accounting and fragment the pool),
// and a latency-bound caller cannot take the device-wide synchronisation that
// cudaFree implies.  rrg_context_create / rrg_dataset_create / rrg_eval
// allocate (a context, pinned staging, scratch arenas that grow with the
// round); this entry point allocates nothing: the caller passes device
// buffers it already owns, and the scratch is one file-scope device array of
// fixed size that CUDA reserves when it loads this file's device code on a
// device (at library load, or at the first call on that device when modules
// load lazily).  The first call on each device also looks up the scratch's
// address (cudaGetSymbolAddress): make it before any stream capture begins
// on that device.
//
// Costs and limits: every device this file's code is loaded on holds
// kNoAllocScratchBytes (32 MiB) for the life of the process.  A call that
// needs more (about (2k + 1) * ld * 8 bytes for k OLS columns and leading
// dimension ld) is rejected with RRG_E_TOO_LARGE.  All calls on a device
// share the one array, so calls that overlap on the GPU (two streams, two
// host threads) race on it; serialise them.
#include <algorithm>
#include <cstdio>
#include <mutex>
#include <string>

#include "../common/error.h"
#include "../common/rr_sum.h"
#include "common.cuh"
#include "plain.cuh"
#include "reduce.cuh"

using namespace rrd;

namespace {

constexpr size_t kNoAllocScratchBytes = size_t(32) << 20;  // 32 MiB per device, whole process
constexpr int kNoAllocMaxDevices = 64;

// The scratch.  In host code this name is only a handle for the symbol; its
// device address comes from cudaGetSymbolAddress.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

std::mutex g_setup_mutex;
unsigned char* g_scratch_ptr[kNoAllocMaxDevices] = {nullptr};

// Device address of the scratch on `device` (the current device), looked up
// by the first call on that device.
bool scratch_address(int device, unsigned char** out) {
  if (device < 0 || device >= kNoAllocMaxDevices) {
    rrc::set_error("rrg_eval_plain_noalloc: device index out of range");
    return false;
  }
  std::lock_guard<std::mutex> lock(g_setup_mutex);
  if (!g_scratch_ptr[device]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      rrc::set_error(std::string("rrg_eval_plain_noalloc: cudaGetSymbolAddress failed: ") + cudaGetErrorString(e));
      return false;
    }
    const cudaError_t a = cudaFuncSetAttribute(plain_eval_kernel, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                               (int)plain_eval_smem());
    if (a != cudaSuccess) {
      rrc::set_error(std::string("rrg_eval_plain_noalloc: kernel attribute setup failed: ") + cudaGetErrorString(a));
      return false;
    }
    g_scratch_ptr[device] = static_cast<unsigned char*>(p);
  }
  *out = g_scratch_ptr[device];
  return true;
}

// A caller buffer must be device (or managed) memory of the current device:
// a host pointer handed to a kernel would fault the GPU, so it is refused here.
bool on_device(const void* p, int device) {
  cudaPointerAttributes at;
  if (cudaPointerGetAttributes(&at, p) != cudaSuccess) {
    cudaGetLastError();
    return false;
  }
  if (at.type == cudaMemoryTypeManaged) return true;
  return at.type == cudaMemoryTypeDevice && at.device == device;
}

// Block j: RR256 sum of chunk j of y (rows [j*RR_CHUNK, (j+1)*RR_CHUNK)).
__global__ void __launch_bounds__(256) noalloc_ysum_kernel(const double* y, int64_t n, double* part) {
  __shared__ double red[8];
  const int64_t r0 = (int64_t)blockIdx.x * RR_CHUNK, r1 = min(n, r0 + (int64_t)RR_CHUNK);
  double acc = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) acc = __dadd_rn(acc, y[r]);
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) part[blockIdx.x] = s;
}

// Block j: the mean from the chunk sums (added in order from chunk 0), then
// the RR256 sum of (y - mean)^2 over chunk j.
__global__ void __launch_bounds__(256) noalloc_ydev_kernel(const double* y, int64_t n, const double* part, int nb,
                                                           double* part2) {
  __shared__ double red[8];
  double total = 0.0;
  for (int j = 0; j < nb; ++j) total = __dadd_rn(total, part[j]);
  const double mean = __ddiv_rn(total, (double)n);
  const int64_t r0 = (int64_t)blockIdx.x * RR_CHUNK, r1 = min(n, r0 + (int64_t)RR_CHUNK);
  double acc = 0.0;
  for (int64_t r = r0 + threadIdx.x; r < r1; r += blockDim.x) {
    const double e = __dsub_rn(y[r], mean);
    acc = __dadd_rn(acc, __dmul_rn(e, e));
  }
  const double s = block_sum(acc, red);
  if (threadIdx.x == 0) part2[blockIdx.x] = s;
}

// out = {sum(y), mean(y), sum((y - mean)^2)}: the CSUM order that
// rrg_dataset_create uses on the host (csrc/common/rr_sum.h).
__global__ void noalloc_ystats_kernel(const double* part, const double* part2, int nb, int64_t n, double* out) {
  if (threadIdx.x != 0) return;
  double total = 0.0, sst = 0.0;
  for (int j = 0; j < nb; ++j) total = __dadd_rn(total, part[j]);
  for (int j = 0; j < nb; ++j) sst = __dadd_rn(sst, part2[j]);
  out[0] = total;
  out[1] = __ddiv_rn(total, (double)n);
  out[2] = sst;
}

rrg_status cuda_fail(const char* what, cudaError_t e) {
  rrc::set_error(std::string("rrg_eval_plain_noalloc: ") + what + ": " + cudaGetErrorString(e));
  return RRG_E_CUDA;
}

}  // namespace

extern "C" rrg_status rrg_eval_plain_noalloc(const double* X_col, int64_t ld, const double* y, int64_t n, int32_t d,
                                             const rrg_batch* batch, rrg_result* result, double* coefs,
                                             void* stream_handle) {
  if (!X_col || !y || !batch || !result || n <= 0 || d <= 0 || ld < n || batch->n_cand != 1 || !batch->cands) {
    rrc::set_error("rrg_eval_plain_noalloc: invalid arguments (needs device X (ld >= n), y and result, "
                   "and a batch of exactly one candidate)");
    return RRG_E_INVALID;
  }
  const rrg_status vst = rrg_batch_validate(batch, d);
  if (vst != RRG_OK) return vst;
  const rrg_cand cd = batch->cands[0];
  if (cd.mode == RRG_TUNED && !coefs) {
    rrc::set_error("rrg_eval_plain_noalloc: a tuned candidate needs a device coefficient output");
    return RRG_E_INVALID;
  }
  // an error another library left pending on this thread is not this
  // call's: clear it so the launch checks below see only their own
  cudaGetLastError();
  int device = 0;
  cudaError_t e = cudaGetDevice(&device);
  if (e != cudaSuccess) {
    rrc::set_error("rrg_eval_plain_noalloc: no current CUDA device");
    return RRG_E_NO_DEVICE;
  }
  if (!on_device(X_col, device) || !on_device(y, device) || !on_device(result, device) ||
      (coefs && !on_device(coefs, device))) {
    rrc::set_error("rrg_eval_plain_noalloc: X, y, result and coefs must be device memory of the current device");
    return RRG_E_INVALID;
  }

  // scratch layout, every piece 256-byte aligned
  const int64_t k = cd.mode == RRG_TUNED ? (int64_t)cd.n_factors + 1 : 1;
  const int nb_res = (int)((n + RR_CHUNK - 1) / RR_CHUNK);
  auto up = [](size_t v) { return (v + 255) / 256 * 256; };
  size_t off = 0;
  const size_t o_cand = off;    off += up(sizeof(rrg_cand));
  const size_t o_fact = off;    off += up(sizeof(rrg_factor) * (size_t)std::max(1, cd.n_factors));
  const size_t o_code = off;    off += up(sizeof(uint32_t) * (size_t)std::max(1, cd.code_len));
  const size_t o_const = off;   off += up(sizeof(double) * (size_t)std::max(1, batch->n_consts));
  const size_t o_pc = off;      off += up(sizeof(PlainCand));
  const size_t o_status = off;  off += up(sizeof(uint32_t));
  const size_t o_ystats = off;  off += up(sizeof(double) * 3);
  const size_t o_ypart = off;   off += up(sizeof(double) * (size_t)nb_res);
  const size_t o_ypart2 = off;  off += up(sizeof(double) * (size_t)nb_res);
  const size_t o_partial = off; off += up(sizeof(double) * (size_t)nb_res);
  const size_t o_coefs = off;   off += up(sizeof(double) * (size_t)k);
  const size_t o_arena = off;
  const double arena_bytes = 8.0 * (double)(2 * k + 1) * (double)ld;
  if ((double)o_arena + arena_bytes > (double)kNoAllocScratchBytes) {
    char msg[320];
    std::snprintf(msg, sizeof msg,
                  "rrg_eval_plain_noalloc: n=%lld (ld=%lld) with %lld OLS columns needs %.0f bytes of scratch; "
                  "the fixed scratch holds %zu bytes (about (2k+1)*ld*8 must fit): use rrg_eval for this size",
                  (long long)n, (long long)ld, (long long)k, (double)o_arena + arena_bytes, kNoAllocScratchBytes);
    rrc::set_error(msg);
    return RRG_E_TOO_LARGE;
  }
  unsigned char* base = nullptr;
  if (!scratch_address(device, &base)) return RRG_E_CUDA;
  cudaStream_t st = static_cast<cudaStream_t>(stream_handle);

  // descriptors rebased to this single candidate, built on the stack
  rrg_cand c0 = cd;
  c0.code_offset = 0;
  c0.first_factor = 0;
  c0.coef_offset = 0;
  PlainCand pc;
  pc.a_col = 0;
  pc.m_col = k;
  pc.s_off = 0;
  pc.k = (int32_t)k;
  pc.pad = 0;
  // The scratch keeps the previous call's contents: the candidate, program,
  // constants and placement are overwritten below; what the kernels
  // accumulate into must start at zero (the status word, which kernels only
  // OR into, and the result record, whose rank and flags the QR kernel sets
  // and the finalize kernel extends).  Arena, partial sums and y statistics
  // are fully written before they are read.
  if ((e = cudaMemcpyAsync(base + o_cand, &c0, sizeof c0, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_fail("staging copy", e);
  if (cd.n_factors > 0 &&
      (e = cudaMemcpyAsync(base + o_fact, batch->factors + cd.first_factor, sizeof(rrg_factor) * cd.n_factors,
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_fail("staging copy", e);
  if (cd.code_len > 0 &&
      (e = cudaMemcpyAsync(base + o_code, batch->code + cd.code_offset, sizeof(uint32_t) * cd.code_len,
                           cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_fail("staging copy", e);
  if (batch->n_consts > 0 &&
      (e = cudaMemcpyAsync(base + o_const, batch->consts, sizeof(double) * batch->n_consts, cudaMemcpyHostToDevice,
                           st)) != cudaSuccess)
    return cuda_fail("staging copy", e);
  if ((e = cudaMemcpyAsync(base + o_pc, &pc, sizeof pc, cudaMemcpyHostToDevice, st)) != cudaSuccess)
    return cuda_fail("staging copy", e);
  if ((e = cudaMemsetAsync(base + o_status, 0, sizeof(uint32_t), st)) != cudaSuccess ||
      (e = cudaMemsetAsync(result, 0, sizeof(rrg_result), st)) != cudaSuccess)
    return cuda_fail("clearing the status and result", e);

  // y statistics on the device in the fixed order (the dataset's own sums)
  double* ypart = reinterpret_cast<double*>(base + o_ypart);
  double* ypart2 = reinterpret_cast<double*>(base + o_ypart2);
  double* ystats_d = reinterpret_cast<double*>(base + o_ystats);
  noalloc_ysum_kernel<<<nb_res, 256, 0, st>>>(y, n, ypart);
  noalloc_ydev_kernel<<<nb_res, 256, 0, st>>>(y, n, ypart, nb_res, ypart2);
  noalloc_ystats_kernel<<<1, 32, 0, st>>>(ypart, ypart2, nb_res, n, ystats_d);
  double ystats[3] = {0.0, 0.0, 0.0};
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(ystats, ystats_d, sizeof ystats, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return cuda_fail("y statistics", e);

  DevBatch db;
  db.cands = reinterpret_cast<const rrg_cand*>(base + o_cand);
  db.factors = reinterpret_cast<const rrg_factor*>(base + o_fact);
  db.code = reinterpret_cast<const uint32_t*>(base + o_code);
  db.consts = reinterpret_cast<const double*>(base + o_const);
  db.consts32 = nullptr;
  db.consts32lo = nullptr;
  db.n_cand = 1;
  db.n_factors = cd.n_factors;
  db.n_code = cd.code_len;
  db.n_consts = batch->n_consts;
  DevData dd;
  dd.X64 = X_col;
  dd.X32 = nullptr;
  dd.X32lo = nullptr;
  dd.y64 = y;
  dd.y32 = nullptr;
  dd.y32lo = nullptr;
  dd.n = n;
  dd.n_pad = ld;
  dd.d = d;
  dd.ysum = ystats[0];
  dd.ymean = ystats[1];
  dd.sst = ystats[2];
  dd.yy = 0.0;  // used by the mixed path only
  const PlainCand* dpc = reinterpret_cast<const PlainCand*>(base + o_pc);
  uint32_t* status = reinterpret_cast<uint32_t*>(base + o_status);
  double* arena = reinterpret_cast<double*>(base + o_arena);
  double* partial = reinterpret_cast<double*>(base + o_partial);
  double* cf = coefs ? coefs : reinterpret_cast<double*>(base + o_coefs);

  // the plain FP64 kernels (factor evaluation, direct column-pivoted QR,
  // residual, fitness), pointed at the scratch
  const int nb_eval = (int)std::min<int64_t>(1024, std::max<int64_t>(1, (n + 1023) / 1024));
  plain_eval_kernel<<<dim3(nb_eval, 1), 256, plain_eval_smem(), st>>>(db, dd, dpc, nullptr, 0, arena, status,
                                                                       nullptr);
  if ((e = cudaGetLastError()) != cudaSuccess) return cuda_fail("factor evaluation launch", e);
  // launch_plain_qr reads (and so clears) the launch error itself: a failed
  // QR launch is only visible through its return value
  if (!launch_plain_qr((int)k + 1, 1, st, db, dd, dpc, nullptr, 0, arena, arena, cf, result, status, nullptr))
    return cuda_fail("QR launch", cudaErrorLaunchFailure);
  plain_resid_kernel<<<dim3(nb_res, 1), 256, 0, st>>>(db, dd, dpc, nullptr, 0, arena, cf, partial, nullptr);
  finalize_kernel<<<1, 128, 0, st>>>(db, dd, nullptr, 0, 1, partial, nb_res, cf, result, 0u, nullptr);
  uint32_t dev_status = 0;
  if ((e = cudaGetLastError()) != cudaSuccess ||
      (e = cudaMemcpyAsync(&dev_status, status, sizeof dev_status, cudaMemcpyDeviceToHost, st)) != cudaSuccess ||
      (e = cudaStreamSynchronize(st)) != cudaSuccess)
    return cuda_fail("scoring", e);
  if (dev_status != 0) {
    char msg[96];
    std::snprintf(msg, sizeof msg, "rrg_eval_plain_noalloc: device reported error status 0x%x", dev_status);
    rrc::set_error(msg);
    return RRG_E_DEVICE_FAULT;
  }
  return RRG_OK;
}
