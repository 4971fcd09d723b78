// Seeded synthetic pair generator for the benchmark workloads (wfg_generate in
// include/wfa_gpu.h). Integer arithmetic only (no libm), so x86-64 and aarch64 hosts
// produce the same bytes for the same seed.
//
// Decisions (the workloads name error rates, not an edit model):
//   * an error rate r over a pattern of L bases means round(r * L) edit EVENTS; each event
//     is a substitution (a different base), an insertion or a deletion; indel lengths are
//     drawn separately (1 for workloads 1-2, geometric for 3-4), so bases changed can
//     exceed round(r * L);
//   * event positions are uniform over the pattern, sorted, and applied left to right in
//     one pass (an event landing inside an earlier deletion moves to its end);
//   * "log-uniform length in [100, 10000]" is sampled exactly over the integers with
//     P(L) proportional to 1/L (rejection from the uniform), and the per-pair error rate
//     "uniform in 1-10 %" is drawn on a 0.1 % grid (10..100 per mille);
//   * workload 5 picks workload 1, 2 or 3 with probability 1/3 each per pair.
// Every pair i draws from its own stream seeded by splitmix64(seed, i).
#include <cstdint>
#include <cstring>
#include <vector>

#include "../../include/wfa_gpu.h"

namespace {

inline uint64_t splitmix64(uint64_t& x) {
  uint64_t z = (x += 0x9e3779b97f4a7c15ull);
  z = (z ^ (z >> 30)) * 0xbf58476d1ce4e5b9ull;
  z = (z ^ (z >> 27)) * 0x94d049bb133111ebull;
  return z ^ (z >> 31);
}

// xoshiro256** (Blackman & Vigna, 2018)
struct Rng {
  uint64_t s[4];
  explicit Rng(uint64_t seed) {
    uint64_t x = seed;
    for (auto& v : s) v = splitmix64(x);
  }
  static inline uint64_t rotl(uint64_t v, int k) { return (v << k) | (v >> (64 - k)); }
  uint64_t next() {
    const uint64_t r = rotl(s[1] * 5, 7) * 9;
    const uint64_t t = s[1] << 17;
    s[2] ^= s[0]; s[3] ^= s[1]; s[1] ^= s[2]; s[0] ^= s[3];
    s[2] ^= t;
    s[3] = rotl(s[3], 45);
    return r;
  }
  // uniform integer in [0, n)
  uint64_t below(uint64_t n) { return (uint64_t)(((unsigned __int128)next() * n) >> 64); }
};

const char kBases[4] = {'A', 'C', 'G', 'T'};

struct PairSpec {
  int len;
  int edits;
  int geo_mean;     // 0: indels of length 1
  int sub_w, ins_w, del_w;
};

PairSpec draw_spec(int workload, Rng& r) {
  PairSpec p{};
  switch (workload) {
    case 1: p.len = 1000; p.edits = 50; p.geo_mean = 0; p.sub_w = p.ins_w = p.del_w = 1; break;
    case 2: p.len = 150; p.edits = 3; p.geo_mean = 0; p.sub_w = p.ins_w = p.del_w = 1; break;
    case 3: {
      int L;
      for (;;) {  // P(L) ~ 1/L on [100, 10000]
        L = 100 + (int)r.below(9901);
        if (r.below((uint64_t)L) < 100) break;
      }
      const int permille = 10 + (int)r.below(91);
      p.len = L;
      p.edits = (int)(((int64_t)permille * L + 500) / 1000);
      p.geo_mean = 2;
      p.sub_w = p.ins_w = p.del_w = 1;
      break;
    }
    case 4: {
      p.len = 50000 + (int)r.below(50001);
      p.edits = (int)(((int64_t)120 * p.len + 500) / 1000);
      p.geo_mean = 3;
      p.sub_w = 2; p.ins_w = 1; p.del_w = 1;
      break;
    }
    default: break;
  }
  return p;
}

int geometric(Rng& r, int mean) {  // P(k) = (1/m)(1-1/m)^(k-1), k >= 1
  if (mean <= 1) return 1;
  int k = 1;
  while (r.below((uint64_t)mean) != 0 && k < 1000000) ++k;
  return k;
}

struct Event { int pos; int type; int len; };

// Builds pattern and text of one pair into out (pattern then text); returns lengths.
void make_pair(const PairSpec& sp, Rng& r, std::vector<char>& pat, std::vector<char>& txt) {
  pat.resize((size_t)sp.len);
  for (int i = 0; i < sp.len; ++i) pat[(size_t)i] = kBases[r.below(4)];
  std::vector<Event> ev((size_t)sp.edits);
  const int wsum = sp.sub_w + sp.ins_w + sp.del_w;
  for (auto& e : ev) {
    e.pos = (int)r.below((uint64_t)sp.len);
    const int t = (int)r.below((uint64_t)wsum);
    e.type = (t < sp.sub_w) ? 0 : (t < sp.sub_w + sp.ins_w) ? 1 : 2;
    e.len = (e.type == 0) ? 1 : geometric(r, sp.geo_mean);
  }
  // insertion sort by position (stable; counts are small except workload 4)
  std::vector<Event> sorted;
  sorted.reserve(ev.size());
  {
    // counting sort by position keeps it O(L + E) and stable
    std::vector<int> cnt((size_t)sp.len + 1, 0);
    for (auto& e : ev) cnt[(size_t)e.pos + 1]++;
    for (int i = 0; i < sp.len; ++i) cnt[(size_t)i + 1] += cnt[(size_t)i];
    sorted.resize(ev.size());
    for (auto& e : ev) sorted[(size_t)cnt[(size_t)e.pos]++] = e;
  }
  txt.clear();
  txt.reserve((size_t)sp.len + (size_t)sp.edits * 4 + 16);
  int cursor = 0;
  for (const auto& e : sorted) {
    int pos = e.pos < cursor ? cursor : e.pos;
    if (pos > sp.len) pos = sp.len;
    while (cursor < pos) txt.push_back(pat[(size_t)cursor++]);
    if (e.type == 0) {
      if (pos >= sp.len) continue;
      const char orig = pat[(size_t)pos];
      int b = (int)r.below(3);
      int code = 0;
      while (kBases[code] != orig) ++code;
      if (b >= code) ++b;
      txt.push_back(kBases[b]);
      cursor = pos + 1;
    } else if (e.type == 1) {
      for (int j = 0; j < e.len; ++j) txt.push_back(kBases[r.below(4)]);
    } else {
      cursor = pos + e.len > sp.len ? sp.len : pos + e.len;
    }
  }
  while (cursor < sp.len) txt.push_back(pat[(size_t)cursor++]);
}

}  // namespace

extern "C" int wfg_generate(int workload, int n, uint64_t seed, char* seq, int64_t* seq_len_out, int64_t* p_off,
                            int* plen, int64_t* t_off, int* tlen) {
  if (workload < 1 || workload > 5 || n < 0 || !seq_len_out) return WF_STATUS_UNSUPPORTED;
  std::vector<char> pat, txt;
  int64_t cur = 0;
  for (int i = 0; i < n; ++i) {
    uint64_t x = seed ^ (0xa0761d6478bd642full * (uint64_t)(i + 1));
    Rng r(splitmix64(x));
    int w = workload;
    if (w == 5) w = 1 + (int)r.below(3);
    const PairSpec sp = draw_spec(w, r);
    make_pair(sp, r, pat, txt);
    if (seq) {
      memcpy(seq + cur, pat.data(), pat.size());
      p_off[i] = cur; plen[i] = (int)pat.size();
      cur += (int64_t)pat.size();
      memcpy(seq + cur, txt.data(), txt.size());
      t_off[i] = cur; tlen[i] = (int)txt.size();
      cur += (int64_t)txt.size();
    } else {
      cur += (int64_t)pat.size() + (int64_t)txt.size();
    }
  }
  *seq_len_out = cur;
  return WF_STATUS_ALG_COMPLETED;
}
