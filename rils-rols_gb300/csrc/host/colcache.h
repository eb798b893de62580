// Factor columns kept on the device across rounds: the host-side map from a
// factor program to the slot of a column arena that holds its values.
//
// The candidates of a local-search round are perturbations of the current
// model, and consecutive rounds perturb mostly the same model: the terms a
// round leaves unchanged, and their perturbations, come back in the next
// round.  A factor column is a function of its program (constants by value)
// and of the dataset only, so the column a round evaluated can be read by a
// later round on the same dataset instead of being evaluated again.  The
// columns of the current sub-round are pinned; the others are reused least
// recently used first.  Which slot a column sits in changes no value.
//
// Entries are found by a 64-bit hash of the program and confirmed word by
// word against the program kept with the slot, so a lookup allocates nothing.
#pragma once
#include <cstdint>
#include <unordered_map>
#include <vector>

// A factor program as the cache sees it: code words ending in EMIT, whose
// constant operands are compared by value.
struct FactorProg {
  const uint32_t* code;
  int len;
  const double* consts;
  uint64_t hash() const;
};

// Persistent ids of the factor programs seen on one dataset (found by hash,
// confirmed word by word): the keys of the pair cache.
class FactorRegistry {
 public:
  void clear() {
    e_.clear();
    head_.clear();
  }
  size_t size() const { return e_.size(); }
  uint32_t id(const FactorProg& p, uint64_t h);

 private:
  struct Entry {
    std::vector<uint64_t> key;
    int32_t next = -1;
  };
  std::vector<Entry> e_;
  std::unordered_map<uint64_t, int32_t> head_;
};

// Pair sums kept across rounds: a map from a pair of factor ids to a slot
// of a device array, least recently used slots replaced (the bookkeeping
// of ColumnCache with exact 64-bit keys).
class PairCache {
 public:
  void reset(int64_t limit) {
    slot_.clear();
    free_.clear();
    map_.clear();
    limit_ = limit;
    pinned_ = 0;
  }
  void clear();
  void bind(uint64_t ds_uid) {
    if (ds_uid != uid_) clear();
    uid_ = ds_uid;
  }
  uint64_t uid() const { return uid_; }
  int64_t limit() const { return limit_; }
  int64_t size() const { return (int64_t)slot_.size(); }
  void begin() {
    ++stamp_;
    pinned_ = 0;
  }
  int32_t find(uint64_t key);
  int64_t available() const { return limit_ - pinned_; }
  bool take(int64_t count, std::vector<int32_t>& out);
  void insert(uint64_t key, int32_t s);

 private:
  struct Slot {
    uint64_t key = 0;
    bool held = false;
    int64_t last = -1;
  };
  std::vector<Slot> slot_;
  std::vector<int32_t> free_;
  std::unordered_map<uint64_t, int32_t> map_;
  int64_t limit_ = 0, stamp_ = 0, pinned_ = 0;
  uint64_t uid_ = 0;
};

class ColumnCache {
 public:
  // Forget every entry and allow up to `limit` slots.
  void reset(int64_t limit);
  // Forget every entry (the slots stay allocated).
  void clear();
  // Entries belong to one dataset (by its unique id): another forgets them.
  void bind(uint64_t ds_uid) {
    if (ds_uid != uid_) clear();
    uid_ = ds_uid;
  }
  uint64_t uid() const { return uid_; }
  int64_t limit() const { return limit_; }
  // slots handed out so far (the arena must hold that many columns)
  int64_t size() const { return (int64_t)slot_.size(); }
  // a new sub-round: nothing pinned
  void begin() {
    ++stamp_;
    pinned_ = 0;
  }
  // the slot holding the column of `p` (hash h), pinned for this sub-round, or -1
  int32_t find(const FactorProg& p, uint64_t h);
  // slots that take() can still hand out in this sub-round
  int64_t available() const { return limit_ - pinned_; }
  // `count` slots for new columns, pinned: free ones first, then new ones up
  // to the limit, then the least recently used entries (forgotten).  False,
  // with nothing taken, when fewer are available.
  bool take(int64_t count, std::vector<int32_t>& out);
  // slot `s` (from take) now holds the column of `p` (hash h)
  void insert(const FactorProg& p, uint64_t h, int32_t s);
  // slots from take that hold no entry (scratch columns) back to the free list
  void give_back(const std::vector<int32_t>& s);

 private:
  struct Slot {
    std::vector<uint64_t> key;  // the program: words, a constant as its opcode and value bits
    uint64_t hash = 0;
    int32_t next = -1;   // next slot with the same hash
    bool held = false;   // holds an entry
    int64_t last = -1;   // sub-round stamp of its last use
  };
  bool matches(const Slot& s, const FactorProg& p) const;
  void forget(int32_t s);
  std::vector<Slot> slot_;
  std::vector<int32_t> free_;
  std::unordered_map<uint64_t, int32_t> head_;  // hash -> first slot with it
  int64_t limit_ = 0;
  int64_t stamp_ = 0;
  int64_t pinned_ = 0;  // slots used in this sub-round
  uint64_t uid_ = 0;
};
