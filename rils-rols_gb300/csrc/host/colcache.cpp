// Host bookkeeping of the device column cache (colcache.h).
#include "colcache.h"

#include <algorithm>
#include <cstring>

#include "../../../include/rils_rols_gb300.h"

void ColumnCache::reset(int64_t limit) {
  slot_.clear();
  free_.clear();
  map_.clear();
  limit_ = limit;
  pinned_ = 0;
}

void ColumnCache::clear() {
  pinned_ = 0;
  map_.clear();
  free_.clear();
  for (int32_t s = (int32_t)slot_.size() - 1; s >= 0; --s) {
    slot_[s].key.clear();
    slot_[s].last = -1;
    free_.push_back(s);
  }
}

int32_t ColumnCache::find(const std::string& key) {
  auto it = map_.find(key);
  if (it == map_.end()) return -1;
  Slot& sl = slot_[it->second];
  if (sl.last != stamp_) ++pinned_;
  sl.last = stamp_;
  return it->second;
}

bool ColumnCache::take(int64_t count, std::vector<int32_t>& out) {
  out.clear();
  if (count <= 0) return true;
  if (available() < count) return false;
  while ((int64_t)out.size() < count && !free_.empty()) {
    out.push_back(free_.back());
    free_.pop_back();
  }
  if ((int64_t)out.size() < count && (int64_t)slot_.size() < limit_) {
    // grow by at least the number of slots so far (fewer arena growths)
    const int64_t want = count - (int64_t)out.size();
    const int64_t grow = std::min(limit_ - (int64_t)slot_.size(), std::max(want, (int64_t)slot_.size()));
    const int32_t s0 = (int32_t)slot_.size();
    slot_.resize(slot_.size() + (size_t)grow);
    for (int32_t s = s0; s < (int32_t)slot_.size(); ++s) {
      if ((int64_t)out.size() < count) out.push_back(s);
      else free_.push_back(s);
    }
  }
  if ((int64_t)out.size() < count) {
    // least recently used entries not pinned by this sub-round (ties by slot)
    std::vector<std::pair<int64_t, int32_t>> old;
    for (int32_t s = 0; s < (int32_t)slot_.size(); ++s)
      if (!slot_[s].key.empty() && slot_[s].last < stamp_) old.push_back({slot_[s].last, s});
    const size_t need = (size_t)(count - (int64_t)out.size());
    std::partial_sort(old.begin(), old.begin() + need, old.end());
    for (size_t i = 0; i < need; ++i) {
      Slot& sl = slot_[old[i].second];
      map_.erase(sl.key);
      sl.key.clear();
      out.push_back(old[i].second);
    }
  }
  for (int32_t s : out) slot_[s].last = stamp_;
  pinned_ += count;
  return true;
}

void ColumnCache::insert(const std::string& key, int32_t s) {
  slot_[s].key = key;
  slot_[s].last = stamp_;
  map_[key] = s;
}

void ColumnCache::give_back(const std::vector<int32_t>& s) {
  for (int32_t v : s) {
    slot_[v].key.clear();
    free_.push_back(v);
  }
}

std::string factor_key(const uint32_t* code, int len, const double* consts) {
  std::string k;
  k.reserve((size_t)len * 5);
  for (int i = 0; i < len; ++i) {
    const uint32_t w = code[i];
    const int op = (int)(w & 0xffu);
    const bool c = op == RRG_OP_LDC || op == RRG_OP_PSC ||
                   (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_C);
    if (c) {
      uint64_t bits;
      std::memcpy(&bits, consts + (w >> 8), sizeof bits);
      k.push_back((char)op);
      k.append(reinterpret_cast<const char*>(&bits), sizeof bits);
    } else {
      k.append(reinterpret_cast<const char*>(&w), sizeof w);
    }
  }
  return k;
}
