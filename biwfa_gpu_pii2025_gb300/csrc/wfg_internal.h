// Shared host/device definitions of the GB300 BiWFA engine.
//
// Layout in HBM for one batch (all device buffers are owned by a wfg_context_t):
//   seq_ascii   : the batch's raw pattern/text bytes, concatenated (uploaded once per batch)
//   seq_words   : per pair, four packed arrays [P fwd | T fwd | P rev | T rev], each
//                 ceil(len*bits/32)+2 uint32 words (2 zero pad words so a 64-bit window
//                 read never leaves the array). bits = 2 for pure ACGT pairs, else 8.
//   arena       : one private scratch slab per resident warp (rings, leaf store, runs, stack)
//   out_runs    : dense CIGAR output, uint32 (len<<4 | op) SAM-style ops, one contiguous
//                 span per pair reserved with one atomicAdd when the pair finishes
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define WFG_HD __host__ __device__
#else
#define WFG_HD
#endif

#ifdef __cplusplus
namespace wfg {
#endif

// SAM BAM op codes used in the output runs (op '=' is a match, 'X' a mismatch).
enum { WFG_OP_INS = 1, WFG_OP_DEL = 2, WFG_OP_EQ = 7, WFG_OP_X = 8 };

// Internal per-pair statuses beyond WFA2's public ones.
enum {
  WFG_ST_COMPLETED = 0,
  WFG_ST_MAX_STEPS = -100,
  WFG_ST_OOM = -200,              // WFA2's WF_STATUS_OOM
  WFG_ST_UNATTAINABLE = -300,
  WFG_ST_SCRATCH_OVERFLOW = -210, // the pair needs a larger per-warp arena (retried by the host)
  WFG_ST_OUTPUT_OVERFLOW = -220,  // the dense output span could not be reserved
};

struct PairDesc {
  int64_t word_off;   // first word of this pair's packed arrays in seq_words
  int64_t p_off;      // pattern / text byte offsets in seq_ascii
  int64_t t_off;
  int plen, tlen;
  int pw_len, tw_len; // words per packed pattern / text array (incl. 2 pad words)
  int bits;           // 2 or 8 (set by the pack kernel)
  int pad;
};

struct KernelParams {
  // penalties: internal (transformed when match < 0) and the caller's for rescoring
  int x, o, e, scope;
  int o2, e2;                // second gap piece (two-piece gap-affine), internal
  int match_o, x_o, o_o, e_o;
  int o2_o, e2_o;            // second gap piece as the caller gave it
  int metric;                // 0 gap-affine, 1 edit, 2 indel, 3 gap-linear, 4 two-piece gap-affine
                             // (x, o, e, scope already set for it)
  int score_only;
  int max_steps;
  // pairs
  int num_pairs;             // used when num_pairs_ptr is null
  const unsigned long long* num_pairs_ptr; // device count (retry passes read the previous pass's count)
  const PairDesc* pairs;
  const int* order;          // processing order (work-stealing queue)
  int* retry_out;            // pairs that overflowed the arena are appended here (null: final pass)
  unsigned long long* retry_count;  // append cursor of retry_out
  unsigned long long* queue_head;   // work-queue cursor of this pass
  const uint32_t* words;
  // per-warp arena
  uint8_t* arena;
  int64_t arena_bytes;       // bytes per warp
  int ring_w;                // ring width (power of two, diagonals per wavefront slot)
  int leaf_words;            // int32 capacity of the leaf wavefront store
  int leaf_max_score;        // capacity of the leaf descriptor table (scores)
  int run_cap;               // uint32 capacity of the per-pair run list
  int leaf_run_cap;          // uint32 capacity of the leaf reverse-run buffer
  int stack_cap;             // recursion stack entries
  // outputs
  int* scores;
  int* status;
  int64_t* run_off;
  int* run_len;
  uint32_t* out_runs;
  int64_t out_cap;
  unsigned long long* out_head;  // dense output cursor (shared by all passes)
  // statistics (optional, may be null): per pair {n_steps, max_leaf_score, max_depth, n_cells}
  int* stats;
  // execution shape (0 = defaults): warps cooperating on one pair, rings in shared memory,
  // physical ring buffers per direction (<= scope; see ring_buffers())
  int group_warps;
  int ring_in_smem;
  int ring_nphys;
};

// Score scope caps (max(x, o+e[, o2+e2]) + 1 after the match transform): the ring descriptors
// live in shared memory, sized for the cap of each kernel instantiation (32 for the usual
// penalties; 64 for larger ones and for two-piece gap-affine).
#define WFG_MAX_SCOPE 32
#define WFG_MAX_SCOPE_2P 64

// Physical ring buffers a direction needs: scores that can hold a wavefront are multiples of
// g = gcd(x, o+e, e), so any window of `scope` consecutive scores holds at most ceil(scope/g)
// live wavefronts, and round-robin buffers of that count are never overwritten while needed.
WFG_HD constexpr inline int wfg_gcd(int a, int b) { return b == 0 ? a : wfg_gcd(b, a % b); }
WFG_HD constexpr inline int wfg_ring_buffers(int x, int o, int e) {
  return ((o + e > x ? o + e : x) + 1 + wfg_gcd(wfg_gcd(x, o + e), e) - 1) / wfg_gcd(wfg_gcd(x, o + e), e);
}
// The same for two gap pieces: g = gcd(x, o1+e1, e1, o2+e2, e2) over scope = max(x, o1+e1,
// o2+e2) + 1.
WFG_HD constexpr inline int wfg_ring_buffers_2p(int x, int o1, int e1, int o2, int e2) {
  return ((o1 + e1 > x ? (o1 + e1 > o2 + e2 ? o1 + e1 : o2 + e2) : (x > o2 + e2 ? x : o2 + e2)) + 1 +
          wfg_gcd(wfg_gcd(wfg_gcd(x, o1 + e1), wfg_gcd(e1, o2 + e2)), e2) - 1) /
         wfg_gcd(wfg_gcd(wfg_gcd(x, o1 + e1), wfg_gcd(e1, o2 + e2)), e2);
}

// Per-warp arena carving (bytes); all offsets 256-byte aligned.
struct ArenaLayout {
  int64_t ring_off, ring_bytes;     // 2 directions x buffers x ncomp components x ring_w int32
  int64_t ldesc_off, ldesc_bytes;   // (leaf_max_score+1) x ncomp x int4
  int64_t ldata_off, ldata_bytes;   // leaf_words int32
  int64_t runs_off, runs_bytes;     // run_cap uint32
  int64_t lruns_off, lruns_bytes;   // leaf_run_cap uint32
  int64_t stack_off, stack_bytes;   // stack_cap x 8 int32
  int64_t rdesc2_off, rdesc2_bytes; // I2/D2 ring descriptors, 2 directions x WFG_MAX_SCOPE_2P
                                    // scores x 2 x int2 (ncomp == 5 only)
  int64_t total;
};

WFG_HD constexpr inline int64_t wfg_align256(int64_t v) { return (v + 255) & ~(int64_t)255; }

// ncomp: 3 (M, I1, D1) or 5 (two-piece gap-affine: + I2, D2).
WFG_HD constexpr inline ArenaLayout wfg_arena_layout(int scope, int ring_w, int leaf_max_score, int leaf_words,
                                           int run_cap, int leaf_run_cap, int stack_cap, int ncomp = 3) {
  ArenaLayout L{};
  int64_t off = 0;
  L.ring_off = off; L.ring_bytes = wfg_align256((int64_t)2 * scope * ncomp * ring_w * 4); off += L.ring_bytes;
  L.ldesc_off = off; L.ldesc_bytes = wfg_align256((int64_t)(leaf_max_score + 1) * ncomp * 16); off += L.ldesc_bytes;
  L.ldata_off = off; L.ldata_bytes = wfg_align256((int64_t)leaf_words * 4); off += L.ldata_bytes;
  L.runs_off = off; L.runs_bytes = wfg_align256((int64_t)run_cap * 4); off += L.runs_bytes;
  L.lruns_off = off; L.lruns_bytes = wfg_align256((int64_t)leaf_run_cap * 4); off += L.lruns_bytes;
  L.stack_off = off; L.stack_bytes = wfg_align256((int64_t)stack_cap * 8 * 4); off += L.stack_bytes;
  L.rdesc2_off = off;
  L.rdesc2_bytes = ncomp == 5 ? wfg_align256((int64_t)2 * WFG_MAX_SCOPE_2P * 2 * 8) : 0;
  off += L.rdesc2_bytes;
  L.total = off;
  return L;
}

#ifdef __cplusplus
}  // namespace wfg
#endif
