/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT.
 *
 * A plain-C restatement of WFA2-lib v2.3's bidirectional WFA (BiWFA) for the
 * gap-affine distance with match = 0 (or match < 0 through Eizenga's transform), and for
 * the edit, indel, gap-linear and two-piece gap-affine distances,
 * end-to-end form, no heuristic, "ultralow" memory mode. Only tests/, the smoke
 * check and bench.py's CPU-baseline leg may load it, and only as the checker
 * or the timed CPU baseline. The GPU product never calls it.
 *
 * Parity is pinned two ways (see tests/test_oracle.py):
 *   1. against WFA2-lib's own golden files for these paths
 *      (tests/wfa.utest.check/test.biwfa.affine*.alg, test.biwfa.score.affine*.alg,
 *      test.biwfa{,.score}.{edit,indel,affine2p}.alg), carried as fixtures under tests/golden/;
 *   2. against the real WFA2-lib compiled from the reference sources
 *      (oracle/_ref/libwfa2_ref.so) on seeded random inputs.
 */
#ifndef BIWFA_ORACLE_H_
#define BIWFA_ORACLE_H_

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Status codes as in WFA2-lib wavefront/wfa.h:46-55. */
#define ORC_STATUS_ALG_COMPLETED      0
#define ORC_STATUS_ALG_PARTIAL        1
#define ORC_STATUS_MAX_STEPS_REACHED  (-100)
#define ORC_STATUS_OOM                (-200)
#define ORC_STATUS_UNATTAINABLE       (-300)

/* Distances (WFA2-lib's gap_affine, edit, indel, gap_linear); edit and indel ignore the
 * penalties, gap-linear reads (match, mismatch, indel) from (match, mismatch, gap_open). */
#define ORC_METRIC_AFFINE 0
#define ORC_METRIC_EDIT   1
#define ORC_METRIC_INDEL  2
#define ORC_METRIC_LINEAR 3
#define ORC_METRIC_AFFINE2P 4  /* two-piece gap-affine: penalties (match, x, o1, e1, o2, e2) */

typedef struct {
  int status;          /* final WFA2 status (0 = completed) */
  int score;           /* full mode: cigar_score_gap_affine() of the ops, -1 if the CIGAR is empty
                          (what align_benchmark prints); score-only mode: cigar->score */
  int cigar_score;     /* the value WFA2 leaves in cigar->score (INT32_MIN when unset) */
  int ops_len;         /* number of operations written to ops */
  int64_t n_cells;     /* sum over every compute step of 3*(hi-lo+1) */
  int64_t n_ext;       /* sum over every extended diagonal of (matched chars + 1) */
  int64_t n_steps;     /* number of compute steps (all directions, all levels) */
  int max_leaf_score;  /* largest score reached inside a unidirectional leaf (-1 if none) */
  int max_depth;       /* deepest recursion level reached */
} orc_result_t;

/* Align one pair. ops must hold at least plen + tlen + 1 bytes (full mode).
 * Returns the status (same as res->status). */
int orc_biwfa_align(const char* pattern, int plen, const char* text, int tlen,
                    int match, int mismatch, int gap_open, int gap_ext,
                    int score_only, char* ops, int ops_cap, orc_result_t* res);

/* The same for a given distance (ORC_METRIC_*). For edit and indel, score is the distance
 * (cigar_score_edit in full mode, as align_benchmark prints it). */
int orc_wfa_align(int metric, const char* pattern, int plen, const char* text, int tlen,
                  int match, int mismatch, int gap_open, int gap_ext,
                  int score_only, char* ops, int ops_cap, orc_result_t* res);

/* Any distance with the full penalty set pen = {match, mismatch, gap_open1, gap_ext1,
 * gap_open2, gap_ext2} (the last two read by ORC_METRIC_AFFINE2P only). */
int orc_wfa_align_pen(int metric, const char* pattern, int plen, const char* text, int tlen, const int pen[6],
                      int score_only, char* ops, int ops_cap, orc_result_t* res);

/* Align a batch with nthreads POSIX threads (static interleaved partition).
 * Sequences are concatenated: pattern i is pat[pat_off[i] .. pat_off[i]+plen[i]).
 * ops for pair i go to ops[ops_off[i] ..] (capacity plen+tlen+1 each).
 * scores[i] / status[i] / ops_len[i] receive the per-pair results.
 * Returns total wall-clock seconds of the align loop (excluding thread start-up is not attempted). */
double orc_biwfa_align_batch(int n, const char* pat, const int64_t* pat_off, const int* plen,
                             const char* txt, const int64_t* txt_off, const int* tlen,
                             int match, int mismatch, int gap_open, int gap_ext, int score_only,
                             char* ops, const int64_t* ops_off,
                             int* scores, int* status, int* ops_len, int nthreads);
double orc_wfa_align_batch(int metric, int n, const char* pat, const int64_t* pat_off, const int* plen,
                           const char* txt, const int64_t* txt_off, const int* tlen,
                           int match, int mismatch, int gap_open, int gap_ext, int score_only,
                           char* ops, const int64_t* ops_off,
                           int* scores, int* status, int* ops_len, int nthreads);
double orc_wfa_align_batch_pen(int metric, int n, const char* pat, const int64_t* pat_off, const int* plen,
                               const char* txt, const int64_t* txt_off, const int* tlen, const int pen[6],
                               int score_only, char* ops, const int64_t* ops_off,
                               int* scores, int* status, int* ops_len, int nthreads);

/* Compares pair i's operations (ops[ops_off[i] ..], ops_len[i] bytes of M/X/I/D) with the
 * run-length list runs[run_off[i] ..], run_len[i] uint32 of (len << 4 | SAM op 7 '=', 8 X, 1 I,
 * 2 D). bad[i] = 1 where they differ; returns the number of differing pairs. */
int64_t orc_compare_runs(int n, const char* ops, const int64_t* ops_off, const int* ops_len, const uint32_t* runs,
                         const int64_t* run_off, const int* run_len, uint8_t* bad);

#ifdef __cplusplus
}
#endif
#endif
