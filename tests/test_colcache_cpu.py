"""Host bookkeeping of the column cache (csrc/host/colcache.cpp), compiled
with a small C++ harness: lookups confirm the program word by word (equal
hashes do not alias), constants compare by value, the sub-round's columns
are pinned, the least recently used entries go first, scratch slots come
back, a new dataset forgets every entry; the factor registry and the pair
cache behind the kept pair sums likewise (CPU only)."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
SRC = ROOT / "rils-rols_gb300" / "csrc" / "host" / "colcache.cpp"

HARNESS = r'''
#include <cassert>
#include <cstdio>
#include <vector>
#include "colcache.h"
#include "rils_rols_gb300.h"

static std::vector<uint32_t> prog(int feature, int cidx) {
  // x[feature] * K[cidx], EMIT
  return {RRG_INSN(RRG_OP_LDV, (uint32_t)feature), RRG_INSN(RRG_BIN_OP(RRG_MUL, RRG_SRC_C, RRG_DIR_R), (uint32_t)cidx),
          RRG_INSN(RRG_OP_EMIT, 0)};
}
#define CHECK(c) do { if (!(c)) { std::printf("FAIL line %d: %s\n", __LINE__, #c); return 1; } } while (0)

int main() {
  const double consts[4] = {2.5, 2.5, 3.0, -1.0};
  ColumnCache cc;
  cc.reset(4);
  cc.bind(7);
  std::vector<std::vector<uint32_t>> p = {prog(0, 0), prog(0, 1), prog(1, 2), prog(2, 3), prog(3, 2), prog(4, 2)};
  auto fp = [&](int i) { return FactorProg{p[i].data(), (int)p[i].size(), consts}; };
  // constants by value: programs 0 and 1 read different pool entries holding 2.5
  CHECK(fp(0).hash() == fp(1).hash());
  CHECK(fp(0).hash() != fp(2).hash());
  std::vector<int32_t> out;
  cc.begin();
  CHECK(cc.find(fp(0), fp(0).hash()) < 0);
  CHECK(cc.take(2, out) && out.size() == 2);
  cc.insert(fp(0), fp(0).hash(), out[0]);
  cc.insert(fp(2), fp(2).hash(), out[1]);
  CHECK(cc.find(fp(1), fp(1).hash()) == out[0]);  // same factor, other pool index
  // an equal hash does not alias a different program
  CHECK(cc.find(fp(3), fp(2).hash()) < 0);
  const int32_t s0 = out[0], s2 = out[1];
  // sub-round 2: program 3 and 4 new, 0 used (pinned)
  cc.begin();
  CHECK(cc.find(fp(0), fp(0).hash()) == s0);
  CHECK(cc.available() == 3);
  CHECK(cc.take(2, out));
  cc.insert(fp(3), fp(3).hash(), out[0]);
  cc.insert(fp(4), fp(4).hash(), out[1]);
  CHECK(cc.size() == 4);
  // sub-round 3: all four slots taken, 5 new -> the least recently used (2) goes
  cc.begin();
  CHECK(cc.find(fp(0), fp(0).hash()) == s0);
  CHECK(cc.find(fp(3), fp(3).hash()) >= 0);
  CHECK(cc.find(fp(4), fp(4).hash()) >= 0);
  CHECK(cc.take(1, out) && out[0] == s2);
  cc.insert(fp(5), fp(5).hash(), out[0]);
  CHECK(cc.find(fp(2), fp(2).hash()) < 0);
  // nothing left to hand out while all four are pinned
  CHECK(cc.available() == 0);
  CHECK(!cc.take(1, out));
  // scratch slots: taken, given back, taken again
  cc.begin();
  CHECK(cc.take(1, out));
  const int32_t sc = out[0];
  CHECK(cc.find(fp(5), fp(5).hash()) >= 0 || sc == s2);
  cc.give_back(out);
  cc.begin();
  CHECK(cc.take(1, out) && out[0] == sc);
  cc.give_back(out);
  // colliding hashes chain: insert two programs under one hash value
  cc.begin();
  CHECK(cc.take(2, out));
  cc.insert(fp(2), 99, out[0]);
  cc.insert(fp(3), 99, out[1]);
  CHECK(cc.find(fp(2), 99) == out[0] && cc.find(fp(3), 99) == out[1]);
  cc.give_back({out[0]});
  CHECK(cc.find(fp(2), 99) < 0 && cc.find(fp(3), 99) == out[1]);
  // another dataset forgets every entry
  cc.bind(8);
  cc.begin();
  CHECK(cc.find(fp(0), fp(0).hash()) < 0 && cc.find(fp(3), 99) < 0);
  CHECK(cc.available() == 4);

  // factor registry: one id per program content, colliding hashes kept apart
  FactorRegistry reg;
  const uint32_t i0 = reg.id(fp(0), fp(0).hash());
  CHECK(reg.id(fp(1), fp(1).hash()) == i0);  // same factor, other pool index
  const uint32_t i2 = reg.id(fp(2), 5), i3 = reg.id(fp(3), 5);
  CHECK(i2 != i3 && i2 != i0 && reg.id(fp(2), 5) == i2 && reg.id(fp(3), 5) == i3 && reg.size() == 3);

  // pair cache: exact keys, pinning, least recently used replaced, rebinding
  PairCache pc;
  pc.reset(3);
  pc.bind(1);
  pc.begin();
  CHECK(pc.find(11) < 0 && pc.take(2, out));
  pc.insert(11, out[0]);
  pc.insert(12, out[1]);
  const int32_t k11 = out[0], k12 = out[1];
  pc.begin();
  CHECK(pc.find(12) == k12 && pc.take(1, out));
  pc.insert(13, out[0]);
  pc.begin();
  CHECK(pc.find(13) >= 0 && pc.find(12) == k12);
  CHECK(pc.available() == 1 && pc.take(1, out) && out[0] == k11);  // 11 was used longest ago
  pc.insert(14, out[0]);
  CHECK(pc.find(11) < 0 && pc.find(14) == k11);
  CHECK(pc.available() == 0 && !pc.take(1, out));
  pc.bind(2);
  pc.begin();
  CHECK(pc.find(12) < 0 && pc.find(14) < 0 && pc.available() == 3);
  std::printf("ok\n");
  return 0;
}
'''


@pytest.mark.skipif(shutil.which("g++") is None, reason="needs g++")
def test_column_cache_bookkeeping(tmp_path):
    (tmp_path / "h.cpp").write_text(HARNESS)
    exe = tmp_path / "h"
    subprocess.run(["g++", "-std=c++17", "-O1", "-I", str(SRC.parent), "-I", str(ROOT / "include"),
                    str(tmp_path / "h.cpp"), str(SRC), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    assert r.returncode == 0 and r.stdout.strip() == "ok", r.stdout + r.stderr
