// Launch-shape tuner: process-wide choices keyed by (knob, column bucket, row
// class), optionally kept in the file named by RRG_TUNE_CACHE.  The knobs are
// result-invariant launch shapes (tune.cuh), so the tuner never changes a
// result bit.  No counterpart in the reference (single-threaded CPU code).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <tuple>
#include <vector>

#include "../common/error.h"
#include "common.cuh"
#include "plain.cuh"
#include "tune.cuh"

namespace rrd {
namespace {

struct Trial {
  int value;
  float ms;
};
struct Entry {
  int value = 0;
  std::vector<Trial> trials;  // empty when loaded from the cache file
};
using Key = std::tuple<int, int, int>;  // knob, bucket, row class

struct Tuner {
  std::mutex mu;
  int mode = RRG_TUNE_ON;
  bool loaded = false;
  std::map<Key, Entry> chosen;
  std::map<std::pair<int, int>, int> pinned;  // (knob, bucket) -> value
};

Tuner& tuner() {
  static Tuner t;
  return t;
}

const char* cache_path() {
  const char* p = std::getenv("RRG_TUNE_CACHE");
  return (p && *p) ? p : nullptr;
}

void load_locked(Tuner& t) {
  if (t.loaded) return;
  t.loaded = true;
  const char* path = cache_path();
  if (!path) return;
  FILE* f = std::fopen(path, "r");
  if (!f) return;
  int knob, bucket, rc, value;
  char tag[16];
  if (std::fscanf(f, "%15s %d", tag, &value) == 2 && std::string(tag) == "rrg-tune" && value == 1) {
    while (std::fscanf(f, "%d %d %d %d", &knob, &bucket, &rc, &value) == 4) {
      int v[4];
      const int nv = tune_variants(knob, bucket, v);
      for (int i = 0; i < nv; ++i)
        if (v[i] == value) t.chosen[Key(knob, bucket, rc)].value = value;
    }
  }
  std::fclose(f);
}

void save_locked(const Tuner& t) {
  const char* path = cache_path();
  if (!path) return;
  const std::string tmp = std::string(path) + ".tmp";
  FILE* f = std::fopen(tmp.c_str(), "w");
  if (!f) return;
  std::fprintf(f, "rrg-tune 1\n");
  for (const auto& kv : t.chosen)
    std::fprintf(f, "%d %d %d %d\n", std::get<0>(kv.first), std::get<1>(kv.first), std::get<2>(kv.first),
                 kv.second.value);
  std::fclose(f);
  std::rename(tmp.c_str(), path);
}

const char* knob_name(int knob) {
  switch (knob) {
    case TK_EVAL_WAVES: return "eval_waves";
    case TK_FAC_GROUP: return "fac_group";
    case TK_PAIR_UNIT: return "pair_unit";
    default: return "fac_stage";
  }
}

}  // namespace

int tune_variants(int knob, int bucket, int* out) {
  if (knob == TK_EVAL_WAVES && bucket == 0) {
    out[0] = 4;
    out[1] = 2;
    out[2] = 8;
    out[3] = 16;
    return 4;
  }
  if (knob == TK_FAC_GROUP && bucket == 0) {
    out[0] = 64;
    out[1] = 32;
    out[2] = 16;
    return 3;
  }
  if (knob == TK_FAC_STAGE && bucket >= 1 && bucket <= 64) {
    out[0] = 1;  // X and y read from global memory (L2) (the first shape)
    out[1] = 2;  // staged in shared memory by tensor copies
    return 2;
  }
  if (knob == TK_PAIR_UNIT && bucket == 0) {
    out[0] = 1 << 16;  // a factor's whole partner list in one block (the first shape)
    out[1] = 512;
    out[2] = 128;
    return 3;
  }
  return 0;
}

int tune_row_class(int64_t n) {
  int c = 0;
  while (c < 62 && (int64_t(1) << (c + 1)) <= n) ++c;
  return c;
}

int tune_pick(int knob, int bucket, int64_t n, bool* trial) {
  Tuner& t = tuner();
  std::lock_guard<std::mutex> lk(t.mu);
  *trial = false;
  int v[4];
  if (tune_variants(knob, bucket, v) == 0) return 0;
  auto pin = t.pinned.find({knob, bucket});
  if (pin != t.pinned.end()) return pin->second;
  if (t.mode == RRG_TUNE_OFF) return v[0];
  load_locked(t);
  auto it = t.chosen.find(Key(knob, bucket, tune_row_class(n)));
  if (it != t.chosen.end()) return it->second.value;
  *trial = true;
  return v[0];
}

void tune_store(int knob, int bucket, int64_t n, const int* vals, const float* ms, int cnt) {
  if (cnt <= 0) return;
  Tuner& t = tuner();
  std::lock_guard<std::mutex> lk(t.mu);
  Entry e;
  int best = 0;
  for (int i = 0; i < cnt; ++i) {
    e.trials.push_back({vals[i], ms[i]});
    if (ms[i] < ms[best]) best = i;
  }
  e.value = vals[best];
  t.chosen[Key(knob, bucket, tune_row_class(n))] = e;
  save_locked(t);
}

}  // namespace rrd

using namespace rrd;

extern "C" {

rrg_status rrg_tune_set_mode(int32_t mode) {
  if (mode != RRG_TUNE_OFF && mode != RRG_TUNE_ON) {
    rrc::set_error("rrg_tune_set_mode: mode must be RRG_TUNE_OFF or RRG_TUNE_ON");
    return RRG_E_INVALID;
  }
  Tuner& t = tuner();
  std::lock_guard<std::mutex> lk(t.mu);
  t.mode = mode;
  return RRG_OK;
}

rrg_status rrg_tune_pin(int32_t knob, int32_t bucket, int32_t value) {
  int v[4];
  const int nv = tune_variants(knob, bucket, v);
  if (nv == 0) {
    rrc::set_error("rrg_tune_pin: unknown knob or bucket");
    return RRG_E_INVALID;
  }
  bool ok = value == 0;
  for (int i = 0; i < nv; ++i) ok = ok || v[i] == value;
  if (!ok) {
    rrc::set_error("rrg_tune_pin: the kernel is not built for this value");
    return RRG_E_INVALID;
  }
  Tuner& t = tuner();
  std::lock_guard<std::mutex> lk(t.mu);
  if (value == 0)
    t.pinned.erase({knob, bucket});
  else
    t.pinned[{knob, bucket}] = value;
  return RRG_OK;
}

rrg_status rrg_tune_reset(void) {
  Tuner& t = tuner();
  std::lock_guard<std::mutex> lk(t.mu);
  t.chosen.clear();
  t.pinned.clear();
  t.loaded = true;  // a reset forgets the cache file's choices too
  return RRG_OK;
}

int64_t rrg_tune_report(char* buf, int64_t cap) {
  Tuner& t = tuner();
  std::string s;
  {
    std::lock_guard<std::mutex> lk(t.mu);
    char line[256];
    for (const auto& kv : t.chosen) {
      std::snprintf(line, sizeof line, "%s bucket=%d row_class=%d value=%d", knob_name(std::get<0>(kv.first)),
                    std::get<1>(kv.first), std::get<2>(kv.first), kv.second.value);
      s += line;
      if (!kv.second.trials.empty()) {
        s += " ms=";
        for (size_t i = 0; i < kv.second.trials.size(); ++i) {
          std::snprintf(line, sizeof line, "%s%d:%.4f", i ? "," : "", kv.second.trials[i].value,
                        (double)kv.second.trials[i].ms);
          s += line;
        }
      }
      s += "\n";
    }
    for (const auto& kv : t.pinned) {
      std::snprintf(line, sizeof line, "%s bucket=%d pinned=%d\n", knob_name(kv.first.first), kv.first.second,
                    kv.second);
      s += line;
    }
  }
  if (buf && cap > 0) {
    const size_t n = std::min<size_t>((size_t)cap - 1, s.size());
    std::memcpy(buf, s.data(), n);
    buf[n] = 0;
  }
  return (int64_t)s.size() + 1;
}

}  // extern "C"
