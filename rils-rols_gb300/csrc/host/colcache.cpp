// Host bookkeeping of the device column cache (colcache.h).
#include "colcache.h"

#include <algorithm>
#include <cstring>

#include "../../../include/rils_rols_gb300.h"

namespace {

bool const_operand(int op) {
  return op == RRG_OP_LDC || op == RRG_OP_PSC || (op >= RRG_OP_BIN && (((op - RRG_OP_BIN) & 7) >> 1) == RRG_SRC_C);
}

uint64_t const_bits(const double* consts, uint32_t w) {
  uint64_t b;
  std::memcpy(&b, consts + (w >> 8), sizeof b);
  return b;
}

// the key words of one code word: itself, or (bit 63 | opcode, value bits)
// for a constant operand (code words have bit 63 clear)
template <class F>
void key_words(uint32_t w, const double* consts, F&& out) {
  const int op = (int)(w & 0xffu);
  if (const_operand(op)) {
    out((1ull << 63) | (uint64_t)op);
    out(const_bits(consts, w));
  } else {
    out((uint64_t)w);
  }
}

}  // namespace

uint64_t FactorProg::hash() const {
  uint64_t h = 0xcbf29ce484222325ull;
  for (int i = 0; i < len; ++i)
    key_words(code[i], consts, [&](uint64_t v) {
      h ^= v;
      h *= 0x100000001b3ull;
      h ^= h >> 31;
    });
  return h;
}

void ColumnCache::reset(int64_t limit) {
  slot_.clear();
  free_.clear();
  head_.clear();
  limit_ = limit;
  pinned_ = 0;
}

void ColumnCache::clear() {
  pinned_ = 0;
  head_.clear();
  free_.clear();
  for (int32_t s = (int32_t)slot_.size() - 1; s >= 0; --s) {
    Slot& sl = slot_[s];
    sl.held = false;
    sl.next = -1;
    sl.last = -1;
    free_.push_back(s);
  }
}

bool ColumnCache::matches(const Slot& s, const FactorProg& p) const {
  size_t k = 0;
  bool ok = true;
  for (int i = 0; i < p.len && ok; ++i)
    key_words(p.code[i], p.consts, [&](uint64_t v) {
      ok = ok && k < s.key.size() && s.key[k] == v;
      ++k;
    });
  return ok && k == s.key.size();
}

int32_t ColumnCache::find(const FactorProg& p, uint64_t h) {
  auto it = head_.find(h);
  if (it == head_.end()) return -1;
  for (int32_t s = it->second; s >= 0; s = slot_[s].next) {
    Slot& sl = slot_[s];
    if (!matches(sl, p)) continue;
    if (sl.last != stamp_) ++pinned_;
    sl.last = stamp_;
    return s;
  }
  return -1;
}

void ColumnCache::forget(int32_t s) {
  Slot& sl = slot_[s];
  if (!sl.held) return;
  auto it = head_.find(sl.hash);
  if (it != head_.end()) {
    if (it->second == s) {
      if (sl.next >= 0) it->second = sl.next;
      else head_.erase(it);
    } else {
      for (int32_t q = it->second; q >= 0; q = slot_[q].next)
        if (slot_[q].next == s) {
          slot_[q].next = sl.next;
          break;
        }
    }
  }
  sl.held = false;
  sl.next = -1;
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
      if (slot_[s].held && slot_[s].last < stamp_) old.push_back({slot_[s].last, s});
    const size_t need = (size_t)(count - (int64_t)out.size());
    std::partial_sort(old.begin(), old.begin() + need, old.end());
    for (size_t i = 0; i < need; ++i) {
      forget(old[i].second);
      out.push_back(old[i].second);
    }
  }
  for (int32_t s : out) slot_[s].last = stamp_;
  pinned_ += count;
  return true;
}

void ColumnCache::insert(const FactorProg& p, uint64_t h, int32_t s) {
  Slot& sl = slot_[s];
  sl.key.clear();
  for (int i = 0; i < p.len; ++i) key_words(p.code[i], p.consts, [&](uint64_t v) { sl.key.push_back(v); });
  sl.hash = h;
  sl.held = true;
  sl.last = stamp_;
  auto it = head_.find(h);
  sl.next = it == head_.end() ? -1 : it->second;
  head_[h] = s;
}

void ColumnCache::give_back(const std::vector<int32_t>& s) {
  for (int32_t v : s) {
    forget(v);
    free_.push_back(v);
  }
}

uint32_t FactorRegistry::id(const FactorProg& p, uint64_t h) {
  auto it = head_.find(h);
  int32_t first = it == head_.end() ? -1 : it->second;
  for (int32_t q = first; q >= 0; q = e_[q].next) {
    const std::vector<uint64_t>& k = e_[q].key;
    size_t j = 0;
    bool ok = true;
    for (int i = 0; i < p.len && ok; ++i)
      key_words(p.code[i], p.consts, [&](uint64_t v) {
        ok = ok && j < k.size() && k[j] == v;
        ++j;
      });
    if (ok && j == k.size()) return (uint32_t)q;
  }
  Entry en;
  for (int i = 0; i < p.len; ++i) key_words(p.code[i], p.consts, [&](uint64_t v) { en.key.push_back(v); });
  en.next = first;
  e_.push_back(std::move(en));
  head_[h] = (int32_t)e_.size() - 1;
  return (uint32_t)e_.size() - 1;
}

void PairCache::clear() {
  pinned_ = 0;
  map_.clear();
  free_.clear();
  for (int32_t s = (int32_t)slot_.size() - 1; s >= 0; --s) {
    slot_[s].held = false;
    slot_[s].last = -1;
    free_.push_back(s);
  }
}

int32_t PairCache::find(uint64_t key) {
  auto it = map_.find(key);
  if (it == map_.end()) return -1;
  Slot& sl = slot_[it->second];
  if (sl.last != stamp_) ++pinned_;
  sl.last = stamp_;
  return it->second;
}

bool PairCache::take(int64_t count, std::vector<int32_t>& out) {
  out.clear();
  if (count <= 0) return true;
  if (available() < count) return false;
  while ((int64_t)out.size() < count && !free_.empty()) {
    out.push_back(free_.back());
    free_.pop_back();
  }
  if ((int64_t)out.size() < count && (int64_t)slot_.size() < limit_) {
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
    std::vector<std::pair<int64_t, int32_t>> old;
    for (int32_t s = 0; s < (int32_t)slot_.size(); ++s)
      if (slot_[s].held && slot_[s].last < stamp_) old.push_back({slot_[s].last, s});
    const size_t need = (size_t)(count - (int64_t)out.size());
    std::partial_sort(old.begin(), old.begin() + need, old.end());
    for (size_t i = 0; i < need; ++i) {
      Slot& sl = slot_[old[i].second];
      map_.erase(sl.key);
      sl.held = false;
      out.push_back(old[i].second);
    }
  }
  for (int32_t s : out) slot_[s].last = stamp_;
  pinned_ += count;
  return true;
}

void PairCache::insert(uint64_t key, int32_t s) {
  Slot& sl = slot_[s];
  sl.key = key;
  sl.held = true;
  sl.last = stamp_;
  map_[key] = s;
}
