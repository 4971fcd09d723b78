// GB300 (sm_103a) bidirectional WFA, end-to-end: score + CIGAR on the device, for the
// gap-affine distance and the edit, indel, gap-linear and two-piece gap-affine ones.
//
// A group of G warps (G = 1 for most pairs, 4 or 8 for wide ones) owns one pair at a time;
// groups pull pair indices from a global work queue (one atomicAdd per pair) so a single
// persistent launch drains a whole uneven batch. Within a pair, threads split the diagonals
// of every wavefront; all control state (scores, breakpoints, recursion) is group-uniform.
//
// Semantics follow WFA2-lib v2.3 exactly (paths relative to WFA2-lib/):
//   compute      wavefront/wavefront_compute_affine.c:44-86, 229-260; wavefront_compute.c:40-104, 306-632;
//                wavefront_compute_affine2p.c:44-104, 334-368; wavefront_compute_edit.c;
//                wavefront_compute_linear.c
//   extend       wavefront/wavefront_extend.c:86-211; wavefront_extend_kernels.c:68-152
//   termination  wavefront/wavefront_termination.c:37-114
//   breakpoint   wavefront/wavefront_bialign.c:189-519
//   recursion    wavefront/wavefront_bialign.c:520-730
//   leaf         wavefront/wavefront_bialign.c:155-185; wavefront_unialign.c:54-273
//   backtrace    wavefront/wavefront_backtrace.c:41-219, 320-529
//   rescoring    alignment/cigar.c:244-342
#include <climits>
#include <cstdint>
#include <cuda_runtime.h>

#include "wfg_internal.h"

namespace wfg {
namespace {

constexpr int32_t kNull = INT32_MIN / 2;   // WAVEFRONT_OFFSET_NULL
constexpr int kAbsent = INT32_MAX;         // lo of a wavefront that does not exist
constexpr unsigned kFull = 0xffffffffu;
constexpr int kMaxScope = WFG_MAX_SCOPE;       // score scope cap of the usual kernels (32)
constexpr int kMaxScope2p = WFG_MAX_SCOPE_2P;  // the cap of the large-scope and two-piece kernels (64)
#ifndef WFG_G1_GROUPS
#define WFG_G1_GROUPS 1
#endif
#ifndef WFG_G1_WARPS3
#define WFG_G1_WARPS3 32
#endif
#ifndef WFG_G1_WARPS5
#define WFG_G1_WARPS5 28
#endif
#ifndef WFG_STEP_UNROLL
#define WFG_STEP_UNROLL 2
#endif
// Single-warp shape: kG1Groups pairs (warps) per block; resident warps per SM fix the register
// cap. The three-component kernels keep 32 warps per SM (64 registers), the two-piece one 28
// (72 registers). Measured (same GB300, identical results) against 28 warps for all: gap-affine
// mixture 1.3 % faster, uneven pairs 1.6 %, edit mixture 5.4 % faster, 150 bp pairs 2.6 %
// slower, two-piece mixture 7.9 % slower (its step spills at 64 registers); 36 warps (56
// registers) 4 % and 40 warps (48 registers) 15 % slower on the gap-affine mixture. One warp
// per block (measured equal to four: 2,457 vs 2,459 ms) lets each warp retire on its own when
// its queue drains, so a launch that follows on another stream takes over warp slots at once
// instead of waiting for whole blocks.
constexpr int kG1Groups = WFG_G1_GROUPS;
template <bool TWO>
constexpr int g1_min_blocks() { return (TWO ? WFG_G1_WARPS5 : WFG_G1_WARPS3) / kG1Groups; }
#ifndef WFG_LEAF_UNROLL
#define WFG_LEAF_UNROLL 1
#endif
constexpr int kStepUnroll = WFG_STEP_UNROLL;        // diagonals per thread per step iteration (rings)
// The same for the leaf store (narrower steps). One diagonal per thread there, measured against
// two at 32 warps per SM (same GB300, identical results): gap-affine mixture 3.2 % faster,
// 1 kbp pairs 6.7 %, 150 bp pairs 4.3 %, uneven pairs 2.4 %, two-piece equal, edit 2.8 %
// slower; three diagonals 3.5 % slower on the mixture. In the ring steps two per thread stay
// best (one 4.3 %, three 8.7 % slower). The multi-warp shapes keep two in the leaf steps (the
// 50-100 kbp pairs on 8-warp groups measured 1.5 % slower with one).
constexpr int kLeafUnroll = WFG_LEAF_UNROLL;
constexpr int ST_OK = -1, ST_END_REACHED = -2, ST_END_UNREACHABLE = -3;
constexpr int CM = 0, CI = 1, CI2 = 2, CD = 3, CD2 = 4;  // components (affine2p_matrix_type values)
constexpr int kFallbackMinScore = 250, kFallbackMinLength = 100, kRecoveryMinScore = 500;
constexpr int BT_M = 9, BT_D2_EXT = 8, BT_D2_OPEN = 7, BT_D_EXT = 6, BT_D_OPEN = 5, BT_I2_EXT = 4, BT_I2_OPEN = 3,
              BT_I_EXT = 2, BT_I_OPEN = 1;

// Storage index of a component: M, I1, D1 (0-2, every gap distance), then the second gap
// piece's I2, D2 (3-4, two-piece gap-affine only), kept in a separate region so that the
// three-component layout does not change.
__device__ __forceinline__ int comp_index(int c) {
  return c == CM ? 0 : c == CI ? 1 : c == CD ? 2 : c == CI2 ? 3 : 4;
}

// A view of one stored wavefront. Offsets for diagonal k live at base[(k - kbase) & mask]:
// rings use kbase = 0 and a power-of-two mask (circular over diagonals), the leaf store
// uses kbase = the allocation's first diagonal and mask = ~0.
struct WfRef {
  int lo, hi;
  int32_t* base;
  int kbase;
  uint32_t mask;
  __device__ __forceinline__ bool present() const { return lo != kAbsent; }
  __device__ __forceinline__ bool nonnull() const { return lo <= hi; }
  __device__ __forceinline__ int32_t at(int k) const { return base[(uint32_t)(k - kbase) & mask]; }
  __device__ __forceinline__ void put(int k, int32_t v) const { base[(uint32_t)(k - kbase) & mask] = v; }
  __device__ __forceinline__ int32_t get(int k) const { return (k >= lo && k <= hi) ? at(k) : kNull; }
};

__device__ __forceinline__ WfRef absent_ref() {
  WfRef r;
  r.lo = kAbsent; r.hi = INT_MIN; r.base = nullptr; r.kbase = 0; r.mask = 0;
  return r;
}

// Internal penalties. metric: kMetricAffine, kMetricEdit, kMetricIndel, kMetricLinear (o =
// indel, e = 0) or kMetricAffine2p (o, e the first gap piece; the second, o2/e2, is carried by
// DirCfg so that the other distances' functions keep their register budget); go: the
// gap-opening adjust of the overlap and its stop conditions (o for gap-affine, max(o, o2) for
// two-piece gap-affine, 0 otherwise, wavefront/wavefront_bialign.c:396-410).
struct Pen { int x, o, e, scope, metric, go; };
constexpr int kMetricAffine = 0, kMetricEdit = 1, kMetricIndel = 2, kMetricLinear = 3, kMetricAffine2p = 4;

// Oriented window over packed words (forward arrays for the forward aligner and the
// leaf, reversed arrays for the reverse aligner). bshift = log2(bits per character).
struct SeqView {
  const uint32_t* pw;
  const uint32_t* tw;
  int p0, t0;
  int plen, tlen;
  int bshift;
};

#ifndef WFG_SEQ_SMEM_WORDS
#define WFG_SEQ_SMEM_WORDS 0
#endif
// Shared-memory words per single-warp group for its pair's packed sequences (0: none, the
// default). A 2-bit pair whose four arrays fit is copied there (cp.async) when the group takes
// it, and its windows are read from shared memory; other pairs read global memory. Measured on
// the 1M-pair mixture (same GB300, identical results): 512 words 1.9 %, 768 words 1.6 % and
// 1,280 words 6.9 % slower than global windows through the read-only path — the windows of a
// pair mostly hit L1 already, the loads become generic, and the slots shrink L1.
constexpr int kSeqSmemWords = WFG_SEQ_SMEM_WORDS;

// One packed word. With shared-memory staging the pointer may address either space (a
// generic load); otherwise global memory through the read-only path. The packed words are
// read-only while the alignment kernel runs.
__device__ __forceinline__ uint32_t seq_word(const uint32_t* w, uint32_t i) {
  if (kSeqSmemWords > 0) return w[i];
  return __ldg(w + i);
}

// 32-bit window of packed characters starting at character pos (first char in the low bits).
__device__ __forceinline__ uint32_t win32(const uint32_t* w, int pos, int bshift) {
  const uint32_t bit = (uint32_t)pos << bshift;
  const uint32_t wi = bit >> 5;
  return __funnelshift_r(seq_word(w, wi), seq_word(w, wi + 1), bit & 31u);
}

#ifndef WFG_LCP64
#define WFG_LCP64 0
#endif
#ifndef WFG_ALIGN_START
#define WFG_ALIGN_START 0
#endif
// 8-warp shape with HBM rings (the retry passes, the sorted schedule's longest pairs): blocks
// per SM. Four (32 warps, 64 registers) measured on the 2,000 pairs of 50-100 kbp at 12 %
// (same GB300, identical results): 23.2 s, against 25.4 s with three (80 registers) and 28.9 s
// with two (127 registers, no spills).
#ifndef WFG_G8_MIN_BLOCKS
#define WFG_G8_MIN_BLOCKS 4
#endif

#if WFG_LCP64 >= 1
// 64-bit window (32 bases of a 2-bit pair, 8 bytes of an 8-bit one) starting at character
// pos: three words, two funnel shifts. Reads at most word (pos >> (5 - bshift)) + 2, inside
// the array's two words of padding for every pos < the array's length.
__device__ __forceinline__ uint64_t win64(const uint32_t* w, int pos, int bshift) {
  const uint32_t bit = (uint32_t)pos << bshift;
  const uint32_t wi = bit >> 5, sh = bit & 31u;
  const uint32_t a = seq_word(w, wi), b = seq_word(w, wi + 1), c = seq_word(w, wi + 2);
  return ((uint64_t)__funnelshift_r(b, c, sh) << 32) | __funnelshift_r(a, b, sh);
}
__device__ __forceinline__ int first_set(uint64_t x) { return __ffsll((long long)x) - 1; }
#endif
// Window of the LCP loop: 0 — 32-bit windows throughout (the default); 1 — the first window
// 32-bit (most extensions of noisy pairs end inside it), the following ones 64-bit; 2 — 64-bit
// throughout. Measured on the 1M-pair mixture (same GB300, identical results): 1 is 4 % and 2 is
// 6 % slower than 0 — most extensions end within 16 bases, and the wider windows cost loads and
// registers (the step's spills double).
#if WFG_LCP64 == 2
typedef uint64_t lcpw_t;
#else
typedef uint32_t lcpw_t;
#endif

__device__ __forceinline__ int first_set(uint32_t x) { return __ffs((int)x) - 1; }

// The LCP in two parts, so that the first windows of several diagonals load together:
// lcp_first() is the XOR of the first windows (0 when nothing can match), lcp_rest()
// continues from it.
__device__ __forceinline__ lcpw_t lcp_first(const SeqView& s, int v, int h) {
  if (min(s.plen - v, s.tlen - h) <= 0) return 0u;
#if WFG_LCP64 == 2
  return win64(s.pw, s.p0 + v, s.bshift) ^ win64(s.tw, s.t0 + h, s.bshift);
#else
  return win32(s.pw, s.p0 + v, s.bshift) ^ win32(s.tw, s.t0 + h, s.bshift);
#endif
}

__device__ __forceinline__ int lcp_rest(const SeqView& s, int v, int h, lcpw_t x) {
  const int maxn = min(s.plen - v, s.tlen - h);
  if (maxn <= 0) return 0;
  if (x) return min(first_set(x) >> s.bshift, maxn);
  int n = (8 * (int)sizeof(lcpw_t)) >> s.bshift;
#if WFG_LCP64 >= 1
  const int cpw = 64 >> s.bshift;
  for (; n < maxn; n += cpw) {
    const uint64_t y = win64(s.pw, s.p0 + v + n, s.bshift) ^ win64(s.tw, s.t0 + h + n, s.bshift);
    if (y) { n += first_set(y) >> s.bshift; break; }
  }
#else
  const int cpw = 32 >> s.bshift;
  for (; n < maxn; n += cpw) {
    const uint32_t y = win32(s.pw, s.p0 + v + n, s.bshift) ^ win32(s.tw, s.t0 + h + n, s.bshift);
    if (y) { n += first_set(y) >> s.bshift; break; }
  }
#endif
  return min(n, maxn);
}

// Longest common extension of P[v..] and T[h..] inside the window: the sentinel-bounded
// blockwise compare of wavefront_extend_matches_kernel_blockwise, with explicit bounds.
__device__ __forceinline__ int lcp(const SeqView& s, int v, int h) { return lcp_rest(s, v, h, lcp_first(s, v, h)); }

// A group of G warps that owns one pair. G == 1: warp-synchronous; G > 1: the warps meet
// at named barrier `bar` (one per group in a block) and reduce through `red` (shared memory,
// >= 8*G + 4 ints).
template <int G>
struct Grp {
  int tid;      // 0 .. 32*G-1
  int bar;
  int* red;
  __device__ __forceinline__ int lane() const { return tid & 31; }
  __device__ __forceinline__ int warp() const { return tid >> 5; }
  __device__ __forceinline__ void sync() const {
    if (G == 1) __syncwarp();
    else asm volatile("bar.sync %0, %1;" ::"r"(bar), "r"(G * 32) : "memory");
  }
  // min/max of up to 8 values at once (slot j of each warp in red[warp*8 + j])
  template <int N>
  __device__ __forceinline__ void minmax(int (&v)[N], const bool (&is_max)[N]) const {
    #pragma unroll
    for (int j = 0; j < N; ++j) v[j] = is_max[j] ? __reduce_max_sync(kFull, v[j]) : __reduce_min_sync(kFull, v[j]);
    if (G == 1) return;
    if (lane() == 0) {
      #pragma unroll
      for (int j = 0; j < N; ++j) red[warp() * 8 + j] = v[j];
    }
    sync();
    #pragma unroll
    for (int j = 0; j < N; ++j) {
      int r = red[j];
      for (int w = 1; w < G; ++w) r = is_max[j] ? max(r, red[w * 8 + j]) : min(r, red[w * 8 + j]);
      v[j] = r;
    }
    sync();
  }
  // value of thread `src_tid` to every thread of the group
  __device__ __forceinline__ int bcast(int v, int src_tid) const {
    if (G == 1) return __shfl_sync(kFull, v, src_tid);
    if (tid == src_tid) red[8 * G] = v;
    sync();
    const int r = red[8 * G];
    sync();
    return r;
  }
};

// Storage configuration of one direction, fixed for the kernel's lifetime; functions copy
// it into registers once per call.
struct DirCfg {
  int leaf;          // 0: modular ring (breakpoint search), 1: full store (leaf)
  int scope;
  uint32_t magic;    // floor(2^32 / scope) + 1: slot = s - scope * umulhi(s, magic), s < 2^27
  int W;             // ring width (power of two)
  int nphys;         // physical ring buffers (round-robin over non-null steps)
  int lmax;          // leaf descriptor capacity (scores)
  int nc;            // stored components: 3 (M, I1, D1) or 5 (+ I2, D2)
  int o2, e2;        // second gap piece, internal (two-piece gap-affine)
  int2* rdesc;       // ring descriptors [scope*3] (shared memory)
  int2* rdesc2;      // I2/D2 ring descriptors [scope*2] (warp arena; nc == 5 only)
  int* rphys;        // physical buffer of each ring slot [scope] (shared memory)
  int32_t* rdata;    // ring storage [nphys*3][W], then I2/D2 [nphys*2][W] when nc == 5
  int4* ldesc;       // leaf descriptors [(lmax+1)*3] {lo, hi, data_off, kbase}, then I2/D2 [(lmax+1)*2]
  int32_t* ldata;
};

// One direction of WFA over one window (a wavefront_aligner_t in WFA2). Lives in shared
// memory; every thread of the group updates its fields with identical values. A field that
// a call reads is written by that call only after a group barrier (G > 1).
struct Dir {
  DirCfg cfg;
  int lcap, lused;
  int next_phys;
  SeqView sv;
  int cb, ce;
  int num_null, status, status_score, end_k;
};

__device__ __forceinline__ int slot_of(const DirCfg& c, int score) {
  return score - c.scope * (int)__umulhi((uint32_t)score, c.magic);
}

// MODE: 0 ring, 1 leaf store, -1 read from the configuration (callers that serve both).
// An absent ring reference keeps the ring's base, kbase and mask (never dereferenced: its
// range is empty), so that every ring reference of a step shares them.
template <int MODE = -1>
__device__ __forceinline__ WfRef ref_raw(const DirCfg& c, int score, int ci) {
  WfRef r;
  const bool leaf = MODE < 0 ? (c.leaf != 0) : (MODE == 1);
  if (!leaf) {
    r.kbase = 0; r.mask = (uint32_t)c.W - 1u;
    if (score < 0) { r.lo = kAbsent; r.hi = INT_MIN; r.base = c.rdata; return r; }
    const int slot = slot_of(c, score);
    const int2 ds = ci < 3 ? c.rdesc[slot * 3 + ci] : c.rdesc2[slot * 2 + (ci - 3)];
    r.lo = ds.x; r.hi = ds.y;
    const int buf = ci < 3 ? c.rphys[slot] * 3 + ci : c.nphys * 3 + c.rphys[slot] * 2 + (ci - 3);
    r.base = c.rdata + (size_t)buf * (size_t)c.W;
  } else {
    if (score < 0 || score > c.lmax) return absent_ref();
    const int4 ds = ci < 3 ? c.ldesc[score * 3 + ci] : c.ldesc[(c.lmax + 1) * 3 + score * 2 + (ci - 3)];
    r.lo = ds.x; r.hi = ds.y;
    r.base = c.ldata + ds.z;
    r.kbase = ds.w; r.mask = 0xffffffffu;
  }
  return r;
}
// Input fetch: absent when the score is negative, the slot is empty or the wavefront is
// null (wavefront_compute_get_*wavefront).
template <int MODE = -1>
__device__ __forceinline__ WfRef fetch(const DirCfg& c, int score, int ci) {
  WfRef r = ref_raw<MODE>(c, score, ci);
  if (!r.nonnull()) { r.lo = kAbsent; r.hi = INT_MIN; }
  return r;
}
template <int MODE = -1>
__device__ __forceinline__ void set_desc(const DirCfg& c, int score, int ci, int lo, int hi, int data_off, int kbase) {
  const bool leaf = MODE < 0 ? (c.leaf != 0) : (MODE == 1);
  if (!leaf) {
    if (ci < 3) c.rdesc[slot_of(c, score) * 3 + ci] = make_int2(lo, hi);
    else c.rdesc2[slot_of(c, score) * 2 + (ci - 3)] = make_int2(lo, hi);
  } else {
    if (ci < 3) c.ldesc[score * 3 + ci] = make_int4(lo, hi, data_off, kbase);
    else c.ldesc[(c.lmax + 1) * 3 + score * 2 + (ci - 3)] = make_int4(lo, hi, data_off, kbase);
  }
}

// The five-component (two-piece gap-affine) form of dir_init's storage reset.
__device__ __noinline__ void dir_init_5(const DirCfg& c, int cbi) {
  if (!c.leaf) {
    for (int i = 0; i < c.scope * 3; ++i) c.rdesc[i] = make_int2(kAbsent, INT_MIN);
    for (int i = 0; i < c.scope * 2; ++i) c.rdesc2[i] = make_int2(kAbsent, INT_MIN);
    for (int i = 0; i < c.scope; ++i) c.rphys[i] = 0;
    set_desc<0>(c, 0, cbi, 0, 0, 0, 0);
    // diagonal 0 of score 0 (physical buffer 0)
    c.rdata[(size_t)(cbi < 3 ? cbi : c.nphys * 3 + (cbi - 3)) * c.W] = 0;
  } else {
    for (int ci = 0; ci < c.nc; ++ci) set_desc<1>(c, 0, ci, kAbsent, INT_MIN, 0, 0);
    set_desc<1>(c, 0, cbi, 0, 0, 0, 0);
    c.ldata[0] = 0;
  }
}

// wavefront_aligner_init / init_wf (wavefront/wavefront_aligner.c:251-417). The caller
// has passed a group barrier since the last read of d. TWO: two-piece gap-affine storage
// (five components); the kernel is specialised on it so the three-component path carries
// no trace of the other.
template <bool TWO>
__device__ void dir_init(Dir& d, const SeqView& sv, int cb, int ce) {
  const DirCfg c = d.cfg;
  d.sv = sv; d.cb = cb; d.ce = ce;
  d.num_null = 0; d.status = ST_OK; d.status_score = 0; d.end_k = INT_MAX;
  const int cbi = comp_index(cb);
  if (TWO) {
    dir_init_5(c, cbi);
    if (!c.leaf) d.next_phys = 1 % c.nphys;
    else d.lused = 1;
    return;
  }
  if (!c.leaf) {
    for (int i = 0; i < c.scope * 3; ++i) c.rdesc[i] = make_int2(kAbsent, INT_MIN);
    for (int i = 0; i < c.scope; ++i) c.rphys[i] = 0;
    c.rdesc[cbi] = make_int2(0, 0);
    c.rdata[(size_t)cbi * c.W] = 0;  // diagonal 0 of score 0 (physical buffer 0)
    d.next_phys = 1 % c.nphys;
  } else {
    d.lused = 1;
    for (int ci = 0; ci < 3; ++ci) c.ldesc[ci] = make_int4(kAbsent, INT_MIN, 0, 0);
    c.ldesc[cbi] = make_int4(0, 0, 0, 0);
    c.ldata[0] = 0;
  }
}

// wavefront_extend_end2end(_max) + wavefront_termination_end2end. Returns 1 when the
// direction is finished (end reached or unreachable).
template <int G>
__device__ __noinline__ int dir_extend(Dir& d, int s, const Grp<G> g, int* max_ak_out) {
  const DirCfg c = d.cfg;
  if (max_ak_out) *max_ak_out = 0;
  const WfRef m = ref_raw(c, s, 0);
  if (!m.present()) {
    if (d.num_null > c.scope) { d.status = ST_END_UNREACHABLE; d.status_score = s; return 1; }
    return 0;
  }
  const SeqView sv = d.sv;
  const int ce = d.ce;
  int my[1] = {0};
  for (int k = m.lo + g.tid; k <= m.hi; k += 32 * G) {
    int32_t off = m.at(k);
    if (off == kNull) continue;
    off += lcp(sv, off - k, off);
    m.put(k, off);
    my[0] = max(my[0], 2 * off - k);
  }
  const bool mx1[1] = {true};
  g.minmax(my, mx1);
  g.sync();
  const int ak = sv.tlen - sv.plen;
  const WfRef t = (ce == CM) ? m : ref_raw(c, s, comp_index(ce));
  const bool done = (t.lo <= ak && ak <= t.hi) && (t.at(ak) >= sv.tlen);
  if (done) { d.status = ST_END_REACHED; d.status_score = s; d.end_k = ak; return 1; }
  if (max_ak_out) *max_ak_out = my[0];
  return 0;
}

// One score step of a direction: wavefront_compute_affine(s) followed by
// wavefront_extend_end2end(_max)(s) and the termination check, fused into one pass over the
// diagonals. Extending diagonal k depends only on M[k] and the sequences, and the trimmed
// range is fixed by which M[k] are in bounds before extension, so the extended offset is
// written once. Returns -1 on scratch overflow, 1 when the direction is finished (end
// reached or unreachable), 0 otherwise; *max_ak receives the extension's max antidiagonal.
// The edit and indel step: wavefront_compute_edit (wavefront/wavefront_compute_edit.c:329-374)
// with the edit / indel kernels (:41-79), trim, the exact pruning of edit
// (wavefront_compute_edit_exact_prune, :199-275), then extension and termination as in
// dir_step. One component (M); the output is [prev.lo-1, prev.hi+1] from the previous score's
// M wavefront (reads outside its range are null). The component-1 buffer of the output slot
// keeps the pre-extension offsets the pruning reads.
template <int G, int MODE>
__device__ __noinline__ int dir_step_linear(Dir& d, const Pen p, int s, const Grp<G> g, int* max_ak_out) {
  const DirCfg c = d.cfg;
  constexpr bool kLeaf = MODE == 1;
  const int used = d.lused, nphys = d.next_phys;
  const SeqView sv = d.sv;
  const uint32_t tl = (uint32_t)sv.tlen, pl = (uint32_t)sv.plen;
  const bool edit = p.metric == kMetricEdit;
  *max_ak_out = 0;
  if (kLeaf && s > c.lmax) return -1;
  const WfRef pv = ref_raw<MODE>(c, s - 1, 0);  // the previous M wavefront (possibly null)
  const int lo = pv.lo - 1, hi = pv.hi + 1;
  const int width = hi - lo + 1;
  WfRef om, os;  // output M, pre-extension scratch
  int offm = 0, need = 0;
  if (!kLeaf) {
    if (width > c.W) return -1;
    om.base = c.rdata + (size_t)(nphys * 3 + 0) * c.W;
    os.base = om.base + c.W;
    om.kbase = os.kbase = 0;
    om.mask = os.mask = (uint32_t)c.W - 1u;
  } else {
    need = 2 * width;
    if (used + need > d.lcap) return -1;
    offm = used;
    om.base = c.ldata + offm; os.base = om.base + width;
    om.kbase = os.kbase = lo;
    om.mask = os.mask = 0xffffffffu;
  }
  const int ak = sv.tlen - sv.plen;
  // r: trimmed lo/hi, max antidiagonal of the extended offsets, min worst-case score
  int r[4] = {INT_MAX, INT_MIN, 0, INT_MAX};
  for (int k = lo + g.tid; k <= hi; k += 32 * G) {
    int32_t m;
    if (edit) m = max(pv.get(k + 1), max(pv.get(k - 1), pv.get(k)) + 1);
    else m = max(pv.get(k + 1), pv.get(k - 1) + 1);
    if ((uint32_t)m > tl || (uint32_t)(m - k) > pl) m = kNull;
    os.put(k, m);
    if (m != kNull) {
      r[0] = min(r[0], k); r[1] = max(r[1], k);
      r[3] = min(r[3], max((int)pl - (m - k), (int)tl - m));  // wf_compute_edit_worst_score
      m += lcp(sv, m - k, m);
      r[2] = max(r[2], 2 * m - k);
    }
    om.put(k, m);
  }
  const bool mm[4] = {false, true, true, false};
  g.minmax(r, mm);
  g.sync();
  int nlo = r[0], nhi = r[1];
  if (nlo > nhi) { nlo = lo; nhi = lo - 1; }  // trimmed to null
  int max_ak = r[2];
  if (edit && nhi - nlo + 1 >= 1000) {
    // Exact pruning. The best case of diagonal k is |k - ak| whatever its offset, the worst
    // case max(|P| - v, |T| - h); sample the middle diagonal's worst case first.
    const int sk = nlo + (nhi - nlo) / 2;
    const int32_t so = os.at(sk);
    const int smax = (so < 0) ? INT_MAX : max((int)pl - (so - sk), (int)tl - so);
    if (so >= 0 && (abs(nlo - ak) > smax || abs(nhi - ak) > smax)) {
      const int mw = r[3];
      int lo_r, hi_r;
      const int a = max(nlo, ak - mw), b = min(nhi, ak + mw);
      lo_r = (a <= b) ? a : nhi + 1;
      if (lo_r >= nhi) hi_r = nhi;
      else hi_r = (b > lo_r) ? b : lo_r;
      if (lo_r != nlo || hi_r != nhi) {
        // the extension's max antidiagonal covers the pruned range only
        int q[1] = {0};
        for (int k = lo_r + g.tid; k <= hi_r; k += 32 * G) {
          const int32_t m = om.at(k);
          if (m != kNull) q[0] = max(q[0], 2 * m - k);
        }
        const bool mq[1] = {true};
        g.minmax(q, mq);
        max_ak = q[0];
        nlo = lo_r; nhi = hi_r;
      }
    }
  }
  g.sync();
  d.num_null = 0;
  if (kLeaf) d.lused = used + need;
  else { c.rphys[slot_of(c, s)] = nphys; d.next_phys = (nphys + 1 == c.nphys) ? 0 : nphys + 1; }
  set_desc<MODE>(c, s, 0, nlo, nhi, offm, lo);
  set_desc<MODE>(c, s, 1, kAbsent, INT_MIN, 0, 0);
  set_desc<MODE>(c, s, 2, kAbsent, INT_MIN, 0, 0);
  // wavefront_termination_end2end on M
  if (nlo <= ak && ak <= nhi && om.at(ak) >= sv.tlen) {
    d.status = ST_END_REACHED; d.status_score = s; d.end_k = ak; return 1;
  }
  *max_ak_out = max_ak;
  return 0;
}

// The two-piece gap-affine step: wavefront_compute_affine2p (wavefront/wavefront_compute_affine2p.c:
// 334-368) with the idm kernel (:44-104), then extension and termination as in dir_step.
// Seven inputs (M[s-x], M[s-o1-e1], I1/D1[s-e1], M[s-o2-e2], I2/D2[s-e2]); the output range
// covers all of them; I1/D1/I2/D2 outputs exist when one of their inputs does
// (wavefront_compute_allocate_output, wavefront/wavefront_compute.c:450-494). One diagonal
// per thread per iteration: the nine input reads already keep enough loads in flight.
template <int G, int MODE>
__device__ __noinline__ int dir_step_2p(Dir& d, const Pen p, int s, const Grp<G> g, int* max_ak_out) {
  const DirCfg c = d.cfg;
  constexpr bool kLeaf = MODE == 1;
  const int nn = d.num_null, used = d.lused, nphys = d.next_phys, ce = d.ce;
  const SeqView sv = d.sv;
  const uint32_t tl = (uint32_t)sv.tlen, pl = (uint32_t)sv.plen;
  *max_ak_out = 0;
  if (kLeaf && s > c.lmax) return -1;
  const WfRef mx = fetch<MODE>(c, s - p.x, 0);
  const WfRef mo1 = fetch<MODE>(c, s - p.o - p.e, 0);
  const WfRef ie1 = fetch<MODE>(c, s - p.e, 1);
  const WfRef de1 = fetch<MODE>(c, s - p.e, 2);
  const WfRef mo2 = fetch<MODE>(c, s - c.o2 - c.e2, 0);
  const WfRef ie2 = fetch<MODE>(c, s - c.e2, 3);
  const WfRef de2 = fetch<MODE>(c, s - c.e2, 4);
  const bool hx = mx.nonnull(), ho1 = mo1.nonnull(), hie1 = ie1.nonnull(), hde1 = de1.nonnull();
  const bool ho2 = mo2.nonnull(), hie2 = ie2.nonnull(), hde2 = de2.nonnull();
  if (!hx && !ho1 && !hie1 && !hde1 && !ho2 && !hie2 && !hde2) {
    if (G > 1) g.sync();
    d.num_null = nn + 1;
    #pragma unroll
    for (int ci = 0; ci < 5; ++ci) set_desc<MODE>(c, s, ci, kAbsent, INT_MIN, 0, 0);
    if (nn + 1 > c.scope) { d.status = ST_END_UNREACHABLE; d.status_score = s; return 1; }
    return 0;
  }
  // wavefront_compute_limits_input over the seven inputs
  int lo = hx ? mx.lo : 1, hi = hx ? mx.hi : -1;
  lo = min(lo, (ho1 ? mo1.lo : 1) - 1);   hi = max(hi, (ho1 ? mo1.hi : -1) + 1);
  lo = min(lo, (hie1 ? ie1.lo : 1) + 1);  hi = max(hi, (hie1 ? ie1.hi : -1) + 1);
  lo = min(lo, (hde1 ? de1.lo : 1) - 1);  hi = max(hi, (hde1 ? de1.hi : -1) - 1);
  lo = min(lo, (ho2 ? mo2.lo : 1) - 1);   hi = max(hi, (ho2 ? mo2.hi : -1) + 1);
  lo = min(lo, (hie2 ? ie2.lo : 1) + 1);  hi = max(hi, (hie2 ? ie2.hi : -1) + 1);
  lo = min(lo, (hde2 ? de2.lo : 1) - 1);  hi = max(hi, (hde2 ? de2.hi : -1) - 1);
  const bool ai1 = ho1 || hie1, ad1 = ho1 || hde1, ai2 = ho2 || hie2, ad2 = ho2 || hde2;
  const int width = hi - lo + 1;
  WfRef om, oi1, od1, oi2, od2;
  int offm = 0, offi1 = 0, offd1 = 0, offi2 = 0, offd2 = 0, need = 0;
  if (!kLeaf) {
    if (width > c.W) return -1;
    om.base = c.rdata + (size_t)(nphys * 3 + 0) * c.W;
    oi1.base = om.base + c.W;
    od1.base = oi1.base + c.W;
    oi2.base = c.rdata + (size_t)(c.nphys * 3 + nphys * 2) * c.W;
    od2.base = oi2.base + c.W;
    om.kbase = oi1.kbase = od1.kbase = oi2.kbase = od2.kbase = 0;
    om.mask = oi1.mask = od1.mask = oi2.mask = od2.mask = (uint32_t)c.W - 1u;
  } else {
    need = width * (1 + (ai1 ? 1 : 0) + (ad1 ? 1 : 0) + (ai2 ? 1 : 0) + (ad2 ? 1 : 0));
    if (used + need > d.lcap) return -1;
    offm = used;
    offi1 = offm + width;
    offd1 = offi1 + (ai1 ? width : 0);
    offi2 = offd1 + (ad1 ? width : 0);
    offd2 = offi2 + (ai2 ? width : 0);
    om.base = c.ldata + offm; oi1.base = c.ldata + offi1; od1.base = c.ldata + offd1;
    oi2.base = c.ldata + offi2; od2.base = c.ldata + offd2;
    om.kbase = oi1.kbase = od1.kbase = oi2.kbase = od2.kbase = lo;
    om.mask = oi1.mask = od1.mask = oi2.mask = od2.mask = 0xffffffffu;
  }
  // ra: M, I1, D1 trimmed lo/hi; rb: I2, D2 trimmed lo/hi, then the max antidiagonal of the
  // extended M (two reductions of at most 8 values each)
  int ra[6] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN};
  int rb[5] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, 0};
  for (int k = lo + g.tid; k <= hi; k += 32 * G) {
    const int32_t i1 = max(mo1.get(k - 1), ie1.get(k - 1)) + 1;
    const int32_t i2 = max(mo2.get(k - 1), ie2.get(k - 1)) + 1;
    const int32_t d1 = max(mo1.get(k + 1), de1.get(k + 1));
    const int32_t d2 = max(mo2.get(k + 1), de2.get(k + 1));
    int32_t m = max(max(mx.get(k) + 1, max(i1, i2)), max(d1, d2));
    if ((uint32_t)m > tl || (uint32_t)(m - k) > pl) m = kNull;
    if (m != kNull) {
      ra[0] = min(ra[0], k); ra[1] = max(ra[1], k);
      m += lcp(sv, m - k, m);
      rb[4] = max(rb[4], 2 * m - k);
    }
    om.put(k, m);
    if (ai1) {
      oi1.put(k, i1);
      if ((uint32_t)i1 <= tl && (uint32_t)(i1 - k) <= pl) { ra[2] = min(ra[2], k); ra[3] = max(ra[3], k); }
    }
    if (ad1) {
      od1.put(k, d1);
      if ((uint32_t)d1 <= tl && (uint32_t)(d1 - k) <= pl) { ra[4] = min(ra[4], k); ra[5] = max(ra[5], k); }
    }
    if (ai2) {
      oi2.put(k, i2);
      if ((uint32_t)i2 <= tl && (uint32_t)(i2 - k) <= pl) { rb[0] = min(rb[0], k); rb[1] = max(rb[1], k); }
    }
    if (ad2) {
      od2.put(k, d2);
      if ((uint32_t)d2 <= tl && (uint32_t)(d2 - k) <= pl) { rb[2] = min(rb[2], k); rb[3] = max(rb[3], k); }
    }
  }
  const bool ma[6] = {false, true, false, true, false, true};
  const bool mb[5] = {false, true, false, true, true};
  g.minmax(ra, ma);
  g.minmax(rb, mb);
  g.sync();
  d.num_null = 0;
  if (kLeaf) d.lused = used + need;
  else { c.rphys[slot_of(c, s)] = nphys; d.next_phys = (nphys + 1 == c.nphys) ? 0 : nphys + 1; }
  if (ra[0] <= ra[1]) set_desc<MODE>(c, s, 0, ra[0], ra[1], offm, lo); else set_desc<MODE>(c, s, 0, lo, lo - 1, offm, lo);
  const bool alloc[4] = {ai1, ad1, ai2, ad2};
  const int tlo[4] = {ra[2], ra[4], rb[0], rb[2]}, thi[4] = {ra[3], ra[5], rb[1], rb[3]};
  const int toff[4] = {offi1, offd1, offi2, offd2};
  #pragma unroll
  for (int j = 0; j < 4; ++j) {
    if (!alloc[j]) set_desc<MODE>(c, s, j + 1, kAbsent, INT_MIN, 0, 0);
    else if (tlo[j] <= thi[j]) set_desc<MODE>(c, s, j + 1, tlo[j], thi[j], toff[j], lo);
    else set_desc<MODE>(c, s, j + 1, lo, lo - 1, toff[j], lo);
  }
  // wavefront_termination_end2end on component_end at score s
  const int ak = sv.tlen - sv.plen;
  bool done;
  if (ce == CM) {
    done = (ra[0] <= ak && ak <= ra[1]) && (om.at(ak) >= sv.tlen);
  } else {
    const int j = (ce == CI) ? 0 : (ce == CD) ? 1 : (ce == CI2) ? 2 : 3;
    const WfRef& t = (j == 0) ? oi1 : (j == 1) ? od1 : (j == 2) ? oi2 : od2;
    done = alloc[j] && (tlo[j] <= ak && ak <= thi[j]) && (t.at(ak) >= sv.tlen);
  }
  if (done) { d.status = ST_END_REACHED; d.status_score = s; d.end_k = ak; return 1; }
  *max_ak_out = rb[4];
  return 0;
}

template <int G, int MODE, bool TWO>
__device__ __noinline__ int dir_step(Dir& d, const Pen p, int s, const Grp<G> g, int* max_ak_out) {
  if (TWO) return dir_step_2p<G, MODE>(d, p, s, g, max_ak_out);
  if (p.metric == kMetricEdit || p.metric == kMetricIndel) return dir_step_linear<G, MODE>(d, p, s, g, max_ak_out);
  const DirCfg c = d.cfg;
  constexpr bool kLeaf = MODE == 1;  // the leaf store (else the modular rings)
  // gap-linear (wavefront_compute_linear, wavefront/wavefront_compute_linear.c:166-195): the
  // same step with M inputs only (mismatch at s-x, indel at s-o) and an M output
  const bool lin = p.metric == kMetricLinear;
  const int nn = d.num_null, used = d.lused, nphys = d.next_phys, ce = d.ce;
  const SeqView sv = d.sv;
  const uint32_t tl = (uint32_t)sv.tlen, pl = (uint32_t)sv.plen;
  *max_ak_out = 0;
  if (kLeaf && s > c.lmax) return -1;
  const WfRef mx = fetch<MODE>(c, s - p.x, 0);
  const WfRef mo = fetch<MODE>(c, s - p.o - p.e, 0);
  const WfRef ie = lin ? absent_ref() : fetch<MODE>(c, s - p.e, 1);
  const WfRef de = lin ? absent_ref() : fetch<MODE>(c, s - p.e, 2);
  const bool hx = mx.nonnull(), ho = mo.nonnull(), hie = ie.nonnull(), hde = de.nonnull();
  if (!hx && !ho && !hie && !hde) {
    // null step: no wavefront; the extension finds no M (wavefront_extend_end2end)
    if (G > 1) g.sync();
    d.num_null = nn + 1;
    set_desc<MODE>(c, s, 0, kAbsent, INT_MIN, 0, 0);
    set_desc<MODE>(c, s, 1, kAbsent, INT_MIN, 0, 0);
    set_desc<MODE>(c, s, 2, kAbsent, INT_MIN, 0, 0);
    if (nn + 1 > c.scope) { d.status = ST_END_UNREACHABLE; d.status_score = s; return 1; }
    return 0;
  }
  int lo = hx ? mx.lo : 1, hi = hx ? mx.hi : -1;
  lo = min(lo, (ho ? mo.lo : 1) - 1);   hi = max(hi, (ho ? mo.hi : -1) + 1);
  if (!lin) {  // wavefront_compute_limits_input stops after M for gap-linear
    lo = min(lo, (hie ? ie.lo : 1) + 1);  hi = max(hi, (hie ? ie.hi : -1) + 1);
    lo = min(lo, (hde ? de.lo : 1) - 1);  hi = max(hi, (hde ? de.hi : -1) - 1);
  }
  const bool ai = !lin && (ho || hie), ad = !lin && (ho || hde);
  const int width = hi - lo + 1;
  WfRef om, oi, od;
  int offm = 0, offi = 0, offd = 0, need = 0;
  if (!kLeaf) {
    if (width > c.W) return -1;
    om.base = c.rdata + (size_t)(nphys * 3 + 0) * c.W;
    oi.base = om.base + c.W;
    od.base = oi.base + c.W;
    om.kbase = oi.kbase = od.kbase = 0;
    om.mask = oi.mask = od.mask = (uint32_t)c.W - 1u;
  } else {
    need = width * (1 + (ai ? 1 : 0) + (ad ? 1 : 0));
    if (used + need > d.lcap) return -1;
    offm = used;
    offi = offm + width;
    offd = offi + (ai ? width : 0);
    om.base = c.ldata + offm; oi.base = c.ldata + offi; od.base = c.ldata + offd;
    om.kbase = oi.kbase = od.kbase = lo;
    om.mask = oi.mask = od.mask = 0xffffffffu;
  }
  // r: M, I, D trimmed lo/hi, then the max antidiagonal of the extended M
  int r[7] = {INT_MAX, INT_MIN, INT_MAX, INT_MIN, INT_MAX, INT_MIN, 0};
  // U diagonals per thread per iteration, so that their loads are in flight together. For
  // k > hi every input read falls outside its input's [lo, hi] (the output range covers
  // them), so those lanes read nothing and store nothing.
  constexpr int U = kLeaf ? (G == 1 ? kLeafUnroll : 2) : kStepUnroll;
  // ALIGN: ring steps start at the 32-diagonal boundary below lo, so each warp-wide access of
  // a row covers whole 128-byte lines (lanes below lo read and write nothing).
  constexpr bool ALIGN = !kLeaf && WFG_ALIGN_START;
  const int k0 = ALIGN ? (lo & ~31) : lo;
  for (int kb = k0 + g.tid; kb <= hi; kb += U * 32 * G) {
    int32_t mv[U], iv[U], dv[U];
    lcpw_t xw[U];
    #pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = kb + u * 32 * G;
      iv[u] = max(mo.get(k - 1), ie.get(k - 1)) + 1;
      dv[u] = max(mo.get(k + 1), de.get(k + 1));
      int32_t m = max(dv[u], max(mx.get(k) + 1, iv[u]));
      if (k > hi || (ALIGN && k < lo) || (uint32_t)m > tl || (uint32_t)(m - k) > pl) m = kNull;
      mv[u] = m;
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = kb + u * 32 * G;
      xw[u] = (mv[u] != kNull) ? lcp_first(sv, mv[u] - k, mv[u]) : 1u;
    }
    #pragma unroll
    for (int u = 0; u < U; ++u) {
      const int k = kb + u * 32 * G;
      if (k > hi) break;
      if (ALIGN && k < lo) continue;
      int32_t m = mv[u];
      if (m != kNull) {
        r[0] = min(r[0], k); r[1] = max(r[1], k);
        m += lcp_rest(sv, m - k, m, xw[u]);
        r[6] = max(r[6], 2 * m - k);
      }
      om.put(k, m);
      const int32_t ins = iv[u], del = dv[u];
      if (ai) {
        oi.put(k, ins);
        if ((uint32_t)ins <= tl && (uint32_t)(ins - k) <= pl) { r[2] = min(r[2], k); r[3] = max(r[3], k); }
      }
      if (ad) {
        od.put(k, del);
        if ((uint32_t)del <= tl && (uint32_t)(del - k) <= pl) { r[4] = min(r[4], k); r[5] = max(r[5], k); }
      }
    }
  }
  const bool mm[7] = {false, true, false, true, false, true, true};
  g.minmax(r, mm);
  g.sync();
  d.num_null = 0;
  if (kLeaf) d.lused = used + need;
  else { c.rphys[slot_of(c, s)] = nphys; d.next_phys = (nphys + 1 == c.nphys) ? 0 : nphys + 1; }
  if (r[0] <= r[1]) set_desc<MODE>(c, s, 0, r[0], r[1], offm, lo); else set_desc<MODE>(c, s, 0, lo, lo - 1, offm, lo);
  if (ai) { if (r[2] <= r[3]) set_desc<MODE>(c, s, 1, r[2], r[3], offi, lo); else set_desc<MODE>(c, s, 1, lo, lo - 1, offi, lo); }
  else set_desc<MODE>(c, s, 1, kAbsent, INT_MIN, 0, 0);
  if (ad) { if (r[4] <= r[5]) set_desc<MODE>(c, s, 2, r[4], r[5], offd, lo); else set_desc<MODE>(c, s, 2, lo, lo - 1, offd, lo); }
  else set_desc<MODE>(c, s, 2, kAbsent, INT_MIN, 0, 0);
  // wavefront_termination_end2end on component_end at score s
  const int ak = sv.tlen - sv.plen;
  bool done;
  if (ce == CM) {
    done = (r[0] <= ak && ak <= r[1]) && (om.at(ak) >= sv.tlen);
  } else {
    const bool alloc = (ce == CI) ? ai : ad;
    const WfRef& t = (ce == CI) ? oi : od;
    const int tlo = (ce == CI) ? r[2] : r[4], thi = (ce == CI) ? r[3] : r[5];
    done = alloc && (tlo <= ak && ak <= thi) && (t.at(ak) >= sv.tlen);
  }
  if (done) { d.status = ST_END_REACHED; d.status_score = s; d.end_k = ak; return 1; }
  *max_ak_out = r[6];
  return 0;
}

struct BP { int score, sf, sr, kf, kr, of, orv, comp; };

// wavefront_bialign_breakpoint_indel2indel / _m2m: the first k0 (ascending) that meets,
// found with a ballot per 32 diagonals (and the lowest hitting warp for G > 1).
template <int G>
__device__ void bp_scan(bool is_m, bool fwd, int s0, int s1, const WfRef& w0, const WfRef& w1,
                        int plen, int tlen, int go, int comp, BP& bp, const Grp<G> g) {
  const int lo0 = w0.lo, hi0 = w0.hi;
  const int lo1 = tlen - plen - w1.hi, hi1 = tlen - plen - w1.lo;
  if (hi1 < lo0 || hi0 < lo1) return;
  const int cand = is_m ? s0 + s1 : s0 + s1 - go;
  if (!(cand < bp.score)) return;
  const int min_hi = min(hi0, hi1), max_lo = max(lo0, lo1);
  for (int kb = max_lo; kb <= min_hi; kb += 32 * G) {
    const int k0 = kb + g.tid;
    bool hit = false;
    int32_t o0 = 0, o1 = 0;
    if (k0 <= min_hi) {
      const int k1 = tlen - plen - k0;
      o0 = w0.at(k0); o1 = w1.at(k1);
      hit = (o0 + o1 >= tlen);
      if (hit && !is_m) {
        const int v = fwd ? o0 - k0 : o1 - k1;
        const int h = fwd ? o0 : o1;
        if (v > plen || h > tlen) hit = false;
      }
    }
    const unsigned b = __ballot_sync(kFull, hit);
    int src;
    if (G == 1) {
      if (!b) continue;
      src = __ffs((int)b) - 1;
    } else {
      int first[1] = {b ? g.warp() * 32 + __ffs((int)b) - 1 : INT_MAX};
      const bool mn[1] = {false};
      g.minmax(first, mn);
      if (first[0] == INT_MAX) continue;
      src = first[0];
    }
    const int hk0 = g.bcast(k0, src);
    const int32_t h0 = g.bcast(o0, src);
    const int32_t h1 = g.bcast(o1, src);
    const int hk1 = tlen - plen - hk0;
    if (fwd) { bp.sf = s0; bp.sr = s1; bp.kf = hk0; bp.kr = hk1; bp.of = h0; bp.orv = h1; }
    else     { bp.sf = s1; bp.sr = s0; bp.kf = hk1; bp.kr = hk0; bp.of = h1; bp.orv = h0; }
    bp.score = cand;
    bp.comp = comp;
    return;
  }
}

// wavefront_bialign_overlap (wavefront/wavefront_bialign.c:314-392), two-piece gap-affine: the
// I2/D2 pairs first (gap-open o2), then I1/D1 (o1), then M.
template <int G>
__device__ __noinline__ void overlap_2p(const Dir& d0, const Dir& d1, int s0, int s1, bool fwd, BP& bp, const Pen p,
                                        const Grp<G> g) {
  const DirCfg c0 = d0.cfg, c1 = d1.cfg;
  const int plen = d0.sv.plen, tlen = d0.sv.tlen, o2 = c0.o2;
  const WfRef m0 = ref_raw<0>(c0, s0, 0);
  if (!m0.present()) return;
  for (int i = 0; i < p.scope; ++i) {
    const int si = s1 - i;
    if (si < 0) break;
    if (s0 + si - o2 >= bp.score) continue;
    const WfRef dd20 = ref_raw<0>(c0, s0, 4), dd21 = ref_raw<0>(c1, si, 4);
    if (dd20.present() && dd21.present()) bp_scan<G>(false, fwd, s0, si, dd20, dd21, plen, tlen, o2, CD2, bp, g);
    const WfRef ii20 = ref_raw<0>(c0, s0, 3), ii21 = ref_raw<0>(c1, si, 3);
    if (ii20.present() && ii21.present()) bp_scan<G>(false, fwd, s0, si, ii20, ii21, plen, tlen, o2, CI2, bp, g);
    if (s0 + si - p.o >= bp.score) continue;
    const WfRef dd0 = ref_raw<0>(c0, s0, 2), dd1 = ref_raw<0>(c1, si, 2);
    if (dd0.present() && dd1.present()) bp_scan<G>(false, fwd, s0, si, dd0, dd1, plen, tlen, p.o, CD, bp, g);
    const WfRef ii0 = ref_raw<0>(c0, s0, 1), ii1 = ref_raw<0>(c1, si, 1);
    if (ii0.present() && ii1.present()) bp_scan<G>(false, fwd, s0, si, ii0, ii1, plen, tlen, p.o, CI, bp, g);
    if (s0 + si >= bp.score) continue;
    const WfRef mm1 = ref_raw<0>(c1, si, 0);
    if (mm1.present()) bp_scan<G>(true, fwd, s0, si, m0, mm1, plen, tlen, p.o, CM, bp, g);
  }
}

// wavefront_bialign_overlap (wavefront/wavefront_bialign.c:314-392): I/D pairs (gap-affine),
// then M (every distance).
template <int G, bool TWO>
__device__ __noinline__ void overlap(const Dir& d0, const Dir& d1, int s0, int s1, bool fwd, BP& bp, const Pen p,
                                     const Grp<G> g) {
  if (TWO) { overlap_2p<G>(d0, d1, s0, s1, fwd, bp, p, g); return; }
  const DirCfg c0 = d0.cfg, c1 = d1.cfg;
  const int plen = d0.sv.plen, tlen = d0.sv.tlen;
  const WfRef m0 = ref_raw<0>(c0, s0, 0);
  if (!m0.present()) return;
  const WfRef dd0 = ref_raw<0>(c0, s0, 2);
  const WfRef ii0 = ref_raw<0>(c0, s0, 1);
  for (int i = 0; i < p.scope; ++i) {
    const int si = s1 - i;
    if (si < 0) break;
    if (s0 + si - p.go >= bp.score) continue;
    const WfRef dd1 = ref_raw<0>(c1, si, 2);
    if (dd0.present() && dd1.present()) bp_scan<G>(false, fwd, s0, si, dd0, dd1, plen, tlen, p.o, CD, bp, g);
    const WfRef ii1 = ref_raw<0>(c1, si, 1);
    if (ii0.present() && ii1.present()) bp_scan<G>(false, fwd, s0, si, ii0, ii1, plen, tlen, p.o, CI, bp, g);
    if (s0 + si >= bp.score) continue;
    const WfRef mm1 = ref_raw<0>(c1, si, 0);
    if (mm1.present()) bp_scan<G>(true, fwd, s0, si, m0, mm1, plen, tlen, p.o, CM, bp, g);
  }
}

struct PairSeqs {
  const uint32_t* pf; const uint32_t* tf; const uint32_t* pr; const uint32_t* tr;
  int plen, tlen, bshift;
};

__device__ __forceinline__ SeqView fwd_view(const PairSeqs& q, int pb, int pe, int tb, int te) {
  SeqView v; v.pw = q.pf; v.tw = q.tf; v.p0 = pb; v.t0 = tb; v.plen = pe - pb; v.tlen = te - tb; v.bshift = q.bshift;
  return v;
}
__device__ __forceinline__ SeqView rev_view(const PairSeqs& q, int pb, int pe, int tb, int te) {
  SeqView v; v.pw = q.pr; v.tw = q.tr; v.p0 = q.plen - pe; v.t0 = q.tlen - te;
  v.plen = pe - pb; v.tlen = te - tb; v.bshift = q.bshift;
  return v;
}

// Upper bound on the optimal score of a window (a guard against runaway loops).
__device__ __forceinline__ int score_guard(const Pen& p, int plen, int tlen) {
  const int mn = min(plen, tlen), df = abs(plen - tlen);
  const int ge = (p.metric == kMetricLinear) ? p.o : p.e;  // cost of one more gap base
  const long long b = (long long)p.x * mn + (long long)(p.o + p.e) + (long long)ge * df + 4LL * p.scope + 16;
  return (int)min(b, (long long)INT_MAX / 4);
}

// wavefront_bialign_find_breakpoint
template <int G, bool TWO>
__device__ __noinline__ int find_breakpoint(Dir& F, Dir& R, const PairSeqs& q, int pb, int pe, int tb, int te,
                                            int cb, int ce, const Pen p, int max_steps, BP& bp, const Grp<G> g) {
  g.sync();
  dir_init<TWO>(F, fwd_view(q, pb, pe, tb, te), cb, ce);
  dir_init<TWO>(R, rev_view(q, pb, pe, tb, te), ce, cb);
  g.sync();
  const int plen = pe - pb, tlen = te - tb;
  const int max_antidiag = plen + tlen - 1;
  const int guard = score_guard(p, plen, tlen);
  int sf = 0, sr = 0, fmax = 0, rmax = 0, ak = 0;
  bp.score = INT_MAX;
  if (dir_extend<G>(F, sf, g, &fmax)) return F.status;
  if (dir_extend<G>(R, sr, g, &rmax)) return R.status;
  bool last_fwd = false;
  for (;;) {
    if (fmax + rmax >= max_antidiag) break;
    ++sf;
    const int qf = dir_step<G, 0, TWO>(F, p, sf, g, &ak);
    if (qf < 0) return WFG_ST_SCRATCH_OVERFLOW;
    if (fmax < ak) fmax = ak;
    last_fwd = true;
    if (qf) return F.status;
    if (fmax + rmax >= max_antidiag) break;
    ++sr;
    const int qr = dir_step<G, 0, TWO>(R, p, sr, g, &ak);
    if (qr < 0) return WFG_ST_SCRATCH_OVERFLOW;
    if (rmax < ak) rmax = ak;
    last_fwd = false;
    if (qr) return R.status;
    if (sr + sf >= max_steps) return WFG_ST_MAX_STEPS;
    if (sf > guard) return WFG_ST_UNATTAINABLE;
  }
  for (;;) {
    if (last_fwd) {
      const int min_sr = (sr > p.scope - 1) ? sr - (p.scope - 1) : 0;
      if (sf + min_sr - p.go >= bp.score) break;
      overlap<G, TWO>(F, R, sf, sr, true, bp, p, g);
      ++sr;
      const int q = dir_step<G, 0, TWO>(R, p, sr, g, &ak);
      if (q < 0) return WFG_ST_SCRATCH_OVERFLOW;
      if (q) return R.status;
    }
    const int min_sf = (sf > p.scope - 1) ? sf - (p.scope - 1) : 0;
    if (min_sf + sr - p.go >= bp.score) break;
    overlap<G, TWO>(R, F, sr, sf, false, bp, p, g);
    ++sf;
    const int q = dir_step<G, 0, TWO>(F, p, sf, g, &ak);
    if (q < 0) return WFG_ST_SCRATCH_OVERFLOW;
    if (q) return F.status;
    if (sr + sf >= max_steps) return WFG_ST_MAX_STEPS;
    if (sf > guard + 2 * p.scope || sr > guard + 2 * p.scope) return WFG_ST_UNATTAINABLE;
    last_fwd = true;
  }
  return ST_OK;
}

// Forward run list of the pair (the CIGAR being assembled), with the open run in registers.
struct RunOut {
  uint32_t* buf;
  int n, cap;
  int cur_op, cur_len;
  bool overflow;
  __device__ __forceinline__ void flush() {
    if (cur_len > 0) {
      if (n < cap) buf[n] = ((uint32_t)cur_len << 4) | (uint32_t)cur_op; else overflow = true;
      ++n;
    }
    cur_len = 0;
  }
  __device__ __forceinline__ void emit(int op, int len) {
    if (len <= 0) return;
    if (op == cur_op && cur_len > 0) { cur_len += len; return; }
    flush();
    cur_op = op; cur_len = len;
  }
};

// wavefront_backtrace_affine: packed (offset<<4)|type source of one step, or the
// unshifted null when the source is absent or out of range.
__device__ __forceinline__ long long bt_src(const DirCfg& B, int score, int ci, int kk, int add, int type) {
  if (score < 0) return (long long)kNull;
  const WfRef w = ref_raw<1>(B, score, ci);
  if (w.lo <= kk && kk <= w.hi) return (long long)(w.at(kk) + add) * 16LL + type;
  return (long long)kNull;
}

// wavefront_backtrace_affine (wavefront/wavefront_backtrace.c:320-529; TWO: the two-piece
// distance's I2/D2 sources) or wavefront_backtrace_linear (:223-319) over the leaf store, from
// (end_k, tlen) at score s in component ce; appends the leaf's ops to out.
template <bool TWO>
__device__ __forceinline__ int leaf_backtrace(const Dir& B, const Pen p, int s, int ce, RunOut& out, uint32_t* lruns,
                                              int lruns_cap) {
  const DirCfg bc = B.cfg;
  // Backtrace from (end_k, tlen) in component ce; runs are produced end -> begin. Every
  // thread of the group walks the same path (uniform loads, identical writes).
  const int plen = B.sv.plen, tlen = B.sv.tlen;
  int nrev = 0; int rop = -1, rlen = 0; bool rover = false;
  auto push = [&](int op, int len) {
    if (len <= 0) return;
    if (op == rop && rlen > 0) { rlen += len; return; }
    if (rlen > 0) { if (nrev < lruns_cap) lruns[nrev] = ((uint32_t)rlen << 4) | (uint32_t)rop; else rover = true; ++nrev; }
    rop = op; rlen = len;
  };
  const bool lin = !TWO && p.metric != kMetricAffine;
  constexpr bool two = TWO;
  int matrix = ce, score = s, k = B.end_k;
  int32_t off = tlen;
  int h = off, v = off - k;
  if (ce == CM) {
    if (v < plen) push(WFG_OP_DEL, plen - v);
    if (h < tlen) push(WFG_OP_INS, tlen - h);
  }
  int iters = 0;
  while (v > 0 && h > 0 && score > 0) {
    if (++iters > plen + tlen + 8) return WFG_ST_UNATTAINABLE;
    // gap-affine: wavefront_backtrace_affine; edit/indel: wavefront_backtrace_linear
    // (wavefront/wavefront_backtrace.c:223-319): M sources only, gap-open = o, no mismatch
    // source for indel
    const int mm = score - p.x, go = score - p.o - (lin ? 0 : p.e), ge = score - p.e;
    const int go2 = score - bc.o2 - bc.e2, ge2 = score - bc.e2;  // second gap piece (two-piece only)
    long long max_all;
    if (matrix == CM) {
      const long long mis = (p.metric == kMetricIndel) ? (long long)kNull : bt_src(bc, mm, 0, k, 1, BT_M);
      const long long io = bt_src(bc, go, 0, k - 1, 1, BT_I_OPEN);
      const long long ix = lin ? (long long)kNull : bt_src(bc, ge, 1, k - 1, 1, BT_I_EXT);
      const long long dop = bt_src(bc, go, 0, k + 1, 0, BT_D_OPEN);
      const long long dx = lin ? (long long)kNull : bt_src(bc, ge, 2, k + 1, 0, BT_D_EXT);
      long long mi = io >= ix ? io : ix;
      long long md = dop >= dx ? dop : dx;
      if (two) {
        const long long io2 = bt_src(bc, go2, 0, k - 1, 1, BT_I2_OPEN);
        const long long ix2 = bt_src(bc, ge2, 3, k - 1, 1, BT_I2_EXT);
        const long long dop2 = bt_src(bc, go2, 0, k + 1, 0, BT_D2_OPEN);
        const long long dx2 = bt_src(bc, ge2, 4, k + 1, 0, BT_D2_EXT);
        const long long mi2 = io2 >= ix2 ? io2 : ix2;
        const long long md2 = dop2 >= dx2 ? dop2 : dx2;
        mi = mi >= mi2 ? mi : mi2;
        md = md >= md2 ? md : md2;
      }
      const long long mid = mi >= md ? mi : md;
      max_all = mis >= mid ? mis : mid;
    } else if (matrix == CI) {
      const long long io = bt_src(bc, go, 0, k - 1, 1, BT_I_OPEN);
      const long long ix = bt_src(bc, ge, 1, k - 1, 1, BT_I_EXT);
      max_all = io >= ix ? io : ix;
    } else if (!TWO || matrix == CD) {
      const long long dop = bt_src(bc, go, 0, k + 1, 0, BT_D_OPEN);
      const long long dx = bt_src(bc, ge, 2, k + 1, 0, BT_D_EXT);
      max_all = dop >= dx ? dop : dx;
    } else if (matrix == CI2) {
      const long long io = bt_src(bc, go2, 0, k - 1, 1, BT_I2_OPEN);
      const long long ix = bt_src(bc, ge2, 3, k - 1, 1, BT_I2_EXT);
      max_all = io >= ix ? io : ix;
    } else {
      const long long dop = bt_src(bc, go2, 0, k + 1, 0, BT_D2_OPEN);
      const long long dx = bt_src(bc, ge2, 4, k + 1, 0, BT_D2_EXT);
      max_all = dop >= dx ? dop : dx;
    }
    if (max_all < 0) break;
    if (matrix == CM) {
      const int max_off = (int)(max_all >> 4);
      push(WFG_OP_EQ, off - max_off);
      off = max_off;
      v = off - k; h = off;
      if (v <= 0 || h <= 0) break;
    }
    const int type = (int)(max_all & 15);
    if (type == BT_M) { score = mm; matrix = CM; push(WFG_OP_X, 1); --off; }
    else if (type == BT_I_OPEN) { score = go; matrix = CM; push(WFG_OP_INS, 1); --k; --off; }
    else if (type == BT_I_EXT) { score = ge; matrix = CI; push(WFG_OP_INS, 1); --k; --off; }
    else if (type == BT_D_OPEN) { score = go; matrix = CM; push(WFG_OP_DEL, 1); ++k; }
    else if (!TWO || type == BT_D_EXT) { score = ge; matrix = CD; push(WFG_OP_DEL, 1); ++k; }
    else if (type == BT_I2_OPEN) { score = go2; matrix = CM; push(WFG_OP_INS, 1); --k; --off; }
    else if (type == BT_I2_EXT) { score = ge2; matrix = CI2; push(WFG_OP_INS, 1); --k; --off; }
    else if (type == BT_D2_OPEN) { score = go2; matrix = CM; push(WFG_OP_DEL, 1); ++k; }
    else { score = ge2; matrix = CD2; push(WFG_OP_DEL, 1); ++k; }
    v = off - k; h = off;
  }
  if (matrix == CM) {
    if (v > 0 && h > 0) {
      const int nm = min(v, h);
      push(WFG_OP_EQ, nm);
      v -= nm; h -= nm;
    }
    if (v > 0) push(WFG_OP_DEL, v);
    if (h > 0) push(WFG_OP_INS, h);
  } else if (v != 0 || h != 0 || score != 0) {
    return WFG_ST_UNATTAINABLE;  // WFA2 aborts here ("I?/D?-Beginning backtrace error")
  }
  if (rlen > 0) { if (nrev < lruns_cap) lruns[nrev] = ((uint32_t)rlen << 4) | (uint32_t)rop; else rover = true; ++nrev; }
  if (rover) return WFG_ST_SCRATCH_OVERFLOW;
  for (int i = nrev - 1; i >= 0; --i) {
    const uint32_t r = lruns[i];
    out.emit((int)(r & 15u), (int)(r >> 4));
  }
  return ST_OK;
}

__device__ __noinline__ int leaf_backtrace_2p(const Dir& B, const Pen p, int s, int ce, RunOut& out, uint32_t* lruns,
                                             int lruns_cap) {
  return leaf_backtrace<true>(B, p, s, ce, out, lruns, lruns_cap);
}

// Leaf: wavefront_bialign_base -> unialign -> backtrace. Appends the leaf's ops to out.
template <int G, bool TWO>
__device__ __noinline__ int leaf_align(Dir& B, const PairSeqs& q, int pb, int pe, int tb, int te, int cb, int ce,
                                       const Pen p, int max_steps, RunOut& out, uint32_t* lruns, int lruns_cap,
                                       const Grp<G> g, int* max_leaf_score) {
  g.sync();
  dir_init<TWO>(B, fwd_view(q, pb, pe, tb, te), cb, ce);
  g.sync();
  const int guard = score_guard(p, pe - pb, te - tb);
  int s = 0, ak = 0;
  if (!dir_extend<G>(B, s, g, nullptr)) {
    for (;;) {
      ++s;
      // wavefront_unialign_reached_limits checks the step count after compute, before extend
      if (s >= max_steps) return WFG_ST_UNATTAINABLE;
      if (s > guard) return WFG_ST_UNATTAINABLE;
      const int q = dir_step<G, 1, TWO>(B, p, s, g, &ak);
      if (q < 0) return WFG_ST_SCRATCH_OVERFLOW;
      if (q) break;
    }
  }
  if (*max_leaf_score < s) *max_leaf_score = s;
  if (B.status != ST_END_REACHED) return WFG_ST_UNATTAINABLE;
  if (TWO) return leaf_backtrace_2p(B, p, s, ce, out, lruns, lruns_cap);
  return leaf_backtrace<false>(B, p, s, ce, out, lruns, lruns_cap);
}

// cigar_score_gap_affine (alignment/cigar.c:277-303), cigar_score_gap_affine2p (:304-342: per
// gap run the cheaper piece), cigar_score_gap_linear (:260-276; o is the indel penalty), or
// cigar_score_edit (:244-259) for the edit and indel distances. The runs are maximal (adjacent
// runs of one op are merged when emitted).
__device__ __forceinline__ int rescore_runs(const uint32_t* runs, int n, int metric, int match, int x, int o, int e,
                                            int o2, int e2) {
  int score = 0;
  for (int i = 0; i < n; ++i) {
    const int op = (int)(runs[i] & 15u), len = (int)(runs[i] >> 4);
    if (metric == kMetricEdit || metric == kMetricIndel) { if (op != WFG_OP_EQ) score += len; continue; }
    if (metric == kMetricLinear) { score -= (op == WFG_OP_EQ ? match : op == WFG_OP_X ? x : o) * len; continue; }
    if (op == WFG_OP_EQ) score -= match * len;
    else if (op == WFG_OP_X) score -= x * len;
    else if (metric == kMetricAffine2p) score -= min(o + e * len, o2 + e2 * len);
    else score -= o + e * len;
  }
  return score;
}

__device__ __forceinline__ int classic_score(int metric, int match_o, int plen, int tlen, int wf_score) {
  if (metric == kMetricEdit || metric == kMetricIndel) return wf_score;  // the distance itself
  const int swg_match = -match_o;
  if (swg_match == 0) return -wf_score;
  return (swg_match * (plen + tlen) - wf_score) / 2;
}

}  // namespace

// Shared memory per group: three directions, ring descriptors and buffer map, reduction
// scratch (dynamic shared memory holds the rings themselves when ring_in_smem). MS: the score
// scope cap of the instantiation.
template <int MS>
struct GroupSmem {
  Dir dir[3];
  int2 rdesc[2][MS * 3];
  int rphys[2][MS];
  int red[8 * 8 + 8];
};

// G warps per pair, GROUPS groups per block. RING_SMEM: the two rings of each group live
// in dynamic shared memory (sized by the host for ring_w); otherwise in the warp arena.
// TWO: the two-piece gap-affine distance (five wavefront components); the other distances
// run in the TWO = false instantiations. MS: the score scope cap (shared-memory ring
// descriptors), 32 for the usual penalties and 64 for larger ones.
template <int G, int GROUPS, bool RING_SMEM, int MINB, bool TWO, int MS>
__global__ void __launch_bounds__(G * GROUPS * 32, MINB) biwfa_persistent_kernel(KernelParams P) {
  __shared__ GroupSmem<MS> s_grp[GROUPS];
  extern __shared__ __align__(16) int32_t s_ring_dyn[];
  const int gib = threadIdx.x / (32 * G);
  GroupSmem<MS>& S = s_grp[gib];
  Grp<G> g;
  g.tid = threadIdx.x % (32 * G);
  g.bar = 1 + gib;
  g.red = S.red;
  const long long ggroup = (long long)blockIdx.x * GROUPS + gib;
  const int nphys = P.ring_nphys > 0 ? P.ring_nphys : P.scope;
  const int nc = TWO ? 5 : 3;
  const ArenaLayout L = wfg_arena_layout(RING_SMEM ? 0 : nphys, P.ring_w, P.leaf_max_score, P.leaf_words,
                                         P.run_cap, P.leaf_run_cap, P.stack_cap, nc);
  uint8_t* arena = P.arena + ggroup * P.arena_bytes;
  const size_t ring_dir = (size_t)nphys * nc * P.ring_w;
  int32_t* ring = RING_SMEM ? s_ring_dyn + (size_t)gib * 2 * ring_dir : (int32_t*)(arena + L.ring_off);
  int4* ldesc = (int4*)(arena + L.ldesc_off);
  int32_t* ldata = (int32_t*)(arena + L.ldata_off);
  uint32_t* runs = (uint32_t*)(arena + L.runs_off);
  uint32_t* lruns = (uint32_t*)(arena + L.lruns_off);
  int* stack = (int*)(arena + L.stack_off);

  Dir& F = S.dir[0];
  Dir& R = S.dir[1];
  Dir& B = S.dir[2];
  const uint32_t magic = (uint32_t)(0xffffffffu / (uint32_t)P.scope) + 1u;
  DirCfg fc{};
  int2* rdesc2 = (int2*)(arena + L.rdesc2_off);  // I2/D2 ring descriptors of both directions
  fc.leaf = 0; fc.scope = P.scope; fc.magic = magic; fc.W = P.ring_w; fc.nphys = nphys; fc.lmax = 0; fc.nc = nc;
  fc.o2 = P.o2; fc.e2 = P.e2;
  fc.rdesc = S.rdesc[0]; fc.rdesc2 = rdesc2; fc.rphys = S.rphys[0]; fc.rdata = ring;
  DirCfg rc = fc;
  rc.rdesc = S.rdesc[1]; rc.rdesc2 = rdesc2 + kMaxScope2p * 2; rc.rphys = S.rphys[1]; rc.rdata = ring + ring_dir;
  DirCfg bcfg{};
  bcfg.leaf = 1; bcfg.scope = P.scope; bcfg.magic = magic; bcfg.W = 0; bcfg.nphys = 1; bcfg.lmax = P.leaf_max_score;
  bcfg.nc = nc; bcfg.o2 = P.o2; bcfg.e2 = P.e2;
  bcfg.ldesc = ldesc; bcfg.ldata = ldata;
  F.cfg = fc; R.cfg = rc; B.cfg = bcfg;
  F.lcap = R.lcap = 0; F.lused = R.lused = 0;
  B.lcap = P.leaf_words; B.lused = 0;
  g.sync();
  const int go = P.metric == kMetricAffine ? P.o : P.metric == kMetricAffine2p ? max(P.o, P.o2) : 0;
  const Pen pen = {P.x, P.o, P.e, P.scope, P.metric, go};

  const unsigned long long num_pairs =
      P.num_pairs_ptr ? *P.num_pairs_ptr : (unsigned long long)P.num_pairs;
  for (;;) {
    int widx_i = 0;
    if (g.tid == 0) {
      const unsigned long long w = atomicAdd(P.queue_head, 1ull);
      widx_i = w >= num_pairs ? -1 : (int)w;
    }
    widx_i = g.bcast(widx_i, 0);
    if (widx_i < 0) break;
    const int pi = P.order[widx_i];
    const PairDesc pd = P.pairs[pi];
    PairSeqs q;
    q.pf = P.words + pd.word_off;
    q.tf = q.pf + pd.pw_len;
    q.pr = q.tf + pd.tw_len;
    q.tr = q.pr + pd.pw_len;
    q.plen = pd.plen; q.tlen = pd.tlen; q.bshift = (pd.bits == 2) ? 1 : 3;
    if (G == 1 && kSeqSmemWords > 0 && pd.bits == 2) {
      // The four 2-bit arrays, each with the two words of padding the windows may read, into
      // this group's shared-memory slot: [P fwd][T fwd][P rev][T rev]. The group's reads of
      // the previous pair ended at its last group barrier.
      const int pw2 = (pd.plen + 15) / 16 + 2, tw2 = (pd.tlen + 15) / 16 + 2;
      if (2 * (pw2 + tw2) <= kSeqSmemWords) {
        uint32_t* slot = reinterpret_cast<uint32_t*>(s_ring_dyn) + (size_t)gib * kSeqSmemWords;
        const uint32_t* src[4] = {q.pf, q.tf, q.pr, q.tr};
        const int len[4] = {pw2, tw2, pw2, tw2};
        uint32_t* dst = slot;
        #pragma unroll
        for (int a = 0; a < 4; ++a) {
          for (int i = g.tid; i < len[a]; i += 32) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(dst + i);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(sa), "l"(src[a] + i) : "memory");
          }
          dst += len[a];
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        __syncwarp();
        q.pf = slot; q.tf = slot + pw2; q.pr = q.tf + tw2; q.tr = q.pr + pw2;
      }
    }
    {
      // Rings sized to the pair: every wavefront of the pair (and of its sub-windows) lies on
      // diagonals [-plen-1, tlen+1], so a ring of next_pow2(plen+tlen+8) <= ring_w diagonals
      // never overflows; the two directions' rings are packed back to back at that width
      // (a smaller footprint per warp for short pairs).
      const uint32_t need = (uint32_t)(pd.plen + pd.tlen + 8);
      const int wp = min(P.ring_w, max(64, (int)(1u << (32 - __clz((int)need - 1)))));
      F.cfg.W = wp; R.cfg.W = wp;
      F.cfg.rdata = ring;
      R.cfg.rdata = ring + (size_t)nphys * nc * wp;
    }
    int status = ST_OK;
    int score = 0;
    int nsteps = 0, max_leaf = -1, max_depth = 0;
    RunOut out; out.buf = runs; out.n = 0; out.cap = P.run_cap; out.cur_op = -1; out.cur_len = 0; out.overflow = false;

    if (P.score_only) {
      // wavefront_bialign_compute_score (wavefront/wavefront_bialign.c:662-699)
      BP bp;
      const int st = find_breakpoint<G, TWO>(F, R, q, 0, q.plen, 0, q.tlen, CM, CM, pen, P.max_steps, bp, g);
      if (st == ST_OK || st == ST_END_REACHED) {
        const int wf = (st == ST_END_REACHED) ? (F.status == ST_END_REACHED ? F.status_score : R.status_score) : bp.score;
        score = classic_score(P.metric, P.match_o, q.plen, q.tlen, wf);
        status = WFG_ST_COMPLETED;
      } else {
        status = st;
      }
    } else {
      // wavefront_bialign (wavefront/wavefront_bialign.c:703-730) with the recursion of
      // wavefront_bialign_alignment unrolled onto an explicit stack (half_0 before half_1).
      const bool min_len = max(q.plen, q.tlen) <= kFallbackMinLength;
      int sp = 0;
      auto push = [&](int pb, int pe, int tb, int te, int cb, int ce, int rem, int lvl) -> bool {
        if (sp >= P.stack_cap) return false;
        int* e = stack + sp * 8;
        e[0] = pb; e[1] = pe; e[2] = tb; e[3] = te; e[4] = cb; e[5] = ce; e[6] = rem; e[7] = lvl;
        ++sp;
        return true;
      };
      push(0, q.plen, 0, q.tlen, CM, CM, min_len ? 0 : INT_MAX, 0);
      while (sp > 0 && status == ST_OK) {
        --sp;
        const int* e = stack + sp * 8;
        const int pb = e[0], pe = e[1], tb = e[2], te = e[3], cb = e[4], ce = e[5], rem = e[6], lvl = e[7];
        if (lvl > max_depth) max_depth = lvl;
        const int pl = pe - pb, tl = te - tb;
        if (tl == 0) { out.emit(WFG_OP_DEL, pl); continue; }
        if (pl == 0) { out.emit(WFG_OP_INS, tl); continue; }
        if (rem <= kFallbackMinScore) {
          const int st = leaf_align<G, TWO>(B, q, pb, pe, tb, te, cb, ce, pen, P.max_steps, out, lruns, P.leaf_run_cap, g,
                                       &max_leaf);
          if (st != ST_OK) status = st;
          continue;
        }
        BP bp;
        const int st = find_breakpoint<G, TWO>(F, R, q, pb, pe, tb, te, cb, ce, pen, P.max_steps, bp, g);
        if (st != ST_OK) {
          if (st == ST_END_REACHED) {
            const int reached = (F.status == ST_END_REACHED) ? F.status_score : R.status_score;
            if (reached <= kRecoveryMinScore) {
              const int st2 = leaf_align<G, TWO>(B, q, pb, pe, tb, te, cb, ce, pen, P.max_steps, out, lruns,
                                            P.leaf_run_cap, g, &max_leaf);
              if (st2 != ST_OK) status = st2;
            } else {
              status = WFG_ST_UNATTAINABLE;
            }
          } else if (st == WFG_ST_SCRATCH_OVERFLOW || st == WFG_ST_MAX_STEPS || st == WFG_ST_OOM) {
            status = st;
          } else {
            status = WFG_ST_UNATTAINABLE;
          }
          continue;
        }
        const int bh = bp.of, bv = bp.of - bp.kf;
        if (!push(pb + bv, pe, tb + bh, te, bp.comp, ce, bp.sr, lvl + 1) ||
            !push(pb, pb + bv, tb, tb + bh, cb, bp.comp, bp.sf, lvl + 1)) {
          status = WFG_ST_SCRATCH_OVERFLOW;
        }
      }
      out.flush();
      if (status == ST_OK && out.overflow) status = WFG_ST_SCRATCH_OVERFLOW;
      if (status == ST_OK) status = WFG_ST_COMPLETED;
      g.sync();
      if (status == WFG_ST_COMPLETED) {
        score = (out.n > 0) ? rescore_runs(runs, out.n, P.metric, P.match_o, P.x_o, P.o_o, P.e_o, P.o2_o, P.e2_o) : 0;
        int base_lo = 0, base_hi = 0;
        if (g.tid == 0) {
          const unsigned long long b = atomicAdd(P.out_head, (unsigned long long)out.n);
          base_lo = (int)(b & 0xffffffffull);
          base_hi = (int)(b >> 32);
        }
        base_lo = g.bcast(base_lo, 0);
        base_hi = g.bcast(base_hi, 0);
        const long long base = (long long)(((unsigned long long)(unsigned)base_hi << 32) | (unsigned)base_lo);
        if (base + out.n > P.out_cap) {
          status = WFG_ST_OUTPUT_OVERFLOW;
        } else {
          for (int i = g.tid; i < out.n; i += 32 * G) P.out_runs[base + i] = runs[i];
          if (g.tid == 0) { P.run_off[pi] = (int64_t)base; P.run_len[pi] = out.n; }
        }
      }
    }
    if (status == WFG_ST_SCRATCH_OVERFLOW && P.retry_out != nullptr) {
      // Hand the pair to the next pass (larger arena); its results are written there.
      if (g.tid == 0) {
        const unsigned long long slot = atomicAdd(P.retry_count, 1ull);
        P.retry_out[slot] = pi;
      }
      g.sync();
      continue;
    }
    if (g.tid == 0) {
      P.scores[pi] = score;
      P.status[pi] = status;
      if (status != WFG_ST_COMPLETED || P.score_only) { P.run_off[pi] = 0; P.run_len[pi] = 0; }
      if (P.stats) {
        P.stats[pi * 4 + 0] = nsteps;
        P.stats[pi * 4 + 1] = max_leaf;
        P.stats[pi * 4 + 2] = max_depth;
        P.stats[pi * 4 + 3] = 0;
      }
    }
    g.sync();
  }
}

// Pack ASCII pairs into the four word arrays per pair; pure ACGT pairs use 2 bits per base,
// anything else keeps 8 bits so the comparison stays exact for every byte value.
__global__ void pack_pairs_kernel(int n, const uint8_t* __restrict__ ascii, PairDesc* __restrict__ pairs,
                                  uint32_t* __restrict__ words) {
  const int lane = threadIdx.x & 31;
  const int warps_per_block = blockDim.x >> 5;
  const long long first = (long long)blockIdx.x * warps_per_block + (threadIdx.x >> 5);
  const long long stride = (long long)gridDim.x * warps_per_block;
  for (long long i = first; i < n; i += stride) {
    PairDesc pd = pairs[i];
    const uint8_t* P = ascii + pd.p_off;
    const uint8_t* T = ascii + pd.t_off;
    bool ok = true;
    for (int j = lane; j < pd.plen; j += 32) { const uint8_t c = P[j]; ok &= (c == 'A' || c == 'C' || c == 'G' || c == 'T'); }
    for (int j = lane; j < pd.tlen; j += 32) { const uint8_t c = T[j]; ok &= (c == 'A' || c == 'C' || c == 'G' || c == 'T'); }
    ok = __all_sync(kFull, ok);
    const int bits = ok ? 2 : 8;
    const int cpw = 32 / bits;
    uint32_t* base = words + pd.word_off;
    for (int a = 0; a < 4; ++a) {
      const uint8_t* src = (a & 1) ? T : P;
      const int len = (a & 1) ? pd.tlen : pd.plen;
      const bool rev = a >= 2;
      const int region = (a & 1) ? pd.tw_len : pd.pw_len;
      uint32_t* dst = base + ((a == 0) ? 0 : (a == 1) ? pd.pw_len : (a == 2) ? pd.pw_len + pd.tw_len : 2 * pd.pw_len + pd.tw_len);
      for (int w = lane; w < region; w += 32) {
        uint32_t word = 0;
        const int c0 = w * cpw;
        for (int j = 0; j < cpw; ++j) {
          const int c = c0 + j;
          if (c >= len) break;
          const uint8_t ch = rev ? src[len - 1 - c] : src[c];
          const uint32_t code = (bits == 2) ? (uint32_t)((ch >> 1) & 3u) : (uint32_t)ch;
          word |= code << (j * bits);
        }
        dst[w] = word;
      }
    }
    if (lane == 0) pairs[i].bits = bits;
  }
}

// ------------------------------------------------------------------ host launchers
namespace {

// Execution shapes: (warps per pair, groups per block, rings in shared memory), each in three
// instantiations: three components with a score scope up to 32 (the usual penalties), three
// components up to 64, and five components (two-piece gap-affine) up to 64.
// Dynamic shared memory of the single-warp shape: the groups' packed-sequence slots.
constexpr size_t kSeqSmemBytesG1 = (size_t)kG1Groups * kSeqSmemWords * sizeof(uint32_t);

template <int G, int GROUPS, bool RS, int MINB, bool TWO, int MS>
cudaError_t launch_shape(const KernelParams& p, int grid, cudaStream_t stream) {
  const size_t dyn = RS ? (size_t)GROUPS * 2 * (size_t)(p.ring_nphys > 0 ? p.ring_nphys : p.scope) * (TWO ? 5 : 3) *
                              (size_t)p.ring_w * sizeof(int32_t)
                        : (G == 1 ? kSeqSmemBytesG1 : 0);
  if (dyn > 0) {
    const cudaError_t e = cudaFuncSetAttribute(biwfa_persistent_kernel<G, GROUPS, RS, MINB, TWO, MS>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  biwfa_persistent_kernel<G, GROUPS, RS, MINB, TWO, MS><<<grid, G * GROUPS * 32, dyn, stream>>>(p);
  return cudaGetLastError();
}

template <int G, int GROUPS, bool RS, int MINB, bool TWO, int MS>
cudaError_t occupancy_of(size_t dyn, int* blocks_per_sm) {
  if (dyn > 0) {
    const cudaError_t e = cudaFuncSetAttribute(biwfa_persistent_kernel<G, GROUPS, RS, MINB, TWO, MS>,
                                               cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn);
    if (e != cudaSuccess) return e;
  }
  return cudaOccupancyMaxActiveBlocksPerMultiprocessor(blocks_per_sm,
                                                       biwfa_persistent_kernel<G, GROUPS, RS, MINB, TWO, MS>,
                                                       G * GROUPS * 32, dyn);
}

template <bool TWO, int MS>
cudaError_t occupancy_shape(int gw, int ring_in_smem, size_t dyn, int* blocks_per_sm) {
  if (gw <= 1) return occupancy_of<1, kG1Groups, false, g1_min_blocks<TWO>(), TWO, MS>(kSeqSmemBytesG1, blocks_per_sm);
  if (gw == 8) {
    if (ring_in_smem) return occupancy_of<8, 1, true, 1, TWO, MS>(dyn, blocks_per_sm);
    return occupancy_of<8, 1, false, WFG_G8_MIN_BLOCKS, TWO, MS>(0, blocks_per_sm);
  }
  if (ring_in_smem) return occupancy_of<4, 1, true, 1, TWO, MS>(dyn, blocks_per_sm);
  return occupancy_of<4, 1, false, 3, TWO, MS>(0, blocks_per_sm);
}

template <bool TWO, int MS>
cudaError_t launch_kernel(const KernelParams& p, int grid, cudaStream_t stream) {
  const int gw = p.group_warps > 0 ? p.group_warps : 1;
  if (gw == 1) return launch_shape<1, kG1Groups, false, g1_min_blocks<TWO>(), TWO, MS>(p, grid, stream);
  if (gw == 8) {
    if (p.ring_in_smem) return launch_shape<8, 1, true, 1, TWO, MS>(p, grid, stream);
    return launch_shape<8, 1, false, WFG_G8_MIN_BLOCKS, TWO, MS>(p, grid, stream);
  }
  if (gw == 4) {
    if (p.ring_in_smem) return launch_shape<4, 1, true, 1, TWO, MS>(p, grid, stream);
    return launch_shape<4, 1, false, 3, TWO, MS>(p, grid, stream);
  }
  return cudaErrorInvalidValue;
}

}  // namespace

int biwfa_warps_per_block() { return kG1Groups; }

cudaError_t biwfa_occupancy(int* blocks_per_sm) {
  return occupancy_of<1, kG1Groups, false, g1_min_blocks<false>(), false, kMaxScope>(kSeqSmemBytesG1, blocks_per_sm);
}

// The kernel instantiation of a launch: 0 three components (scope <= 32), 1 three components
// (scope <= 64), 2 two-piece gap-affine (scope <= 64).
int biwfa_kernel_kind(int metric, int scope) {
  return metric == kMetricAffine2p ? 2 : (scope > kMaxScope ? 1 : 0);
}

// Resident blocks per SM of a shape (dyn: its dynamic shared memory in bytes; kind: as
// biwfa_kernel_kind).
cudaError_t biwfa_occupancy_shape(int gw, int ring_in_smem, size_t dyn, int* blocks_per_sm, int kind) {
  if (kind == 2) return occupancy_shape<true, kMaxScope2p>(gw, ring_in_smem, dyn, blocks_per_sm);
  if (kind == 1) return occupancy_shape<false, kMaxScope2p>(gw, ring_in_smem, dyn, blocks_per_sm);
  return occupancy_shape<false, kMaxScope>(gw, ring_in_smem, dyn, blocks_per_sm);
}

// Groups (pairs in flight) per block of a shape.
int biwfa_groups_per_block(int group_warps, int ring_in_smem) {
  (void)ring_in_smem;
  return group_warps <= 1 ? kG1Groups : 1;
}

cudaError_t launch_biwfa(const KernelParams& p, int grid, cudaStream_t stream) {
  const int kind = biwfa_kernel_kind(p.metric, p.scope);
  if (kind == 2) return launch_kernel<true, kMaxScope2p>(p, grid, stream);
  if (kind == 1) return launch_kernel<false, kMaxScope2p>(p, grid, stream);
  return launch_kernel<false, kMaxScope>(p, grid, stream);
}

cudaError_t launch_pack(int n, const uint8_t* ascii, PairDesc* pairs, uint32_t* words, int num_sms,
                        cudaStream_t stream) {
  if (n <= 0) return cudaSuccess;
  const int wpb = 8;
  long long blocks = ((long long)n + wpb - 1) / wpb;
  const long long cap = (long long)num_sms * 16;
  if (blocks > cap) blocks = cap;
  pack_pairs_kernel<<<(int)blocks, wpb * 32, 0, stream>>>(n, ascii, pairs, words);
  return cudaGetLastError();
}

}  // namespace wfg
