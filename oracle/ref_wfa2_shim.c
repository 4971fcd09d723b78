/*
 * Test infrastructure only: a thin shim over the real WFA2-lib v2.3 API, compiled
 * together with the WFA2-lib sources into oracle/_ref/libwfa2_ref.so. It is used to
 * pin the C restatement in oracle/biwfa_oracle.c and to generate golden fixtures.
 * Nothing in the product links or calls it.
 *
 * The attribute set is the exact BiWFA configuration of the hot path:
 *   distance_metric = gap_affine, penalties {match, x, o, e},
 *   memory_mode = wavefront_memory_ultralow, heuristic = wf_heuristic_none,
 *   alignment_scope = compute_alignment (or compute_score).
 * This is the configuration align_benchmark uses for
 * `-a gap-affine-wfa --wfa-memory=ultralow` (tools/align_benchmark/align_benchmark.c:155-241).
 */
#include <string.h>
#include "wavefront/wavefront_align.h"
#include "alignment/cigar.h"

/* Returns the WFA2 status. On success writes:
 *   *cigar_score_out : wf_aligner->cigar->score as WFA2 leaves it
 *   *rescore_out     : cigar_score_gap_affine() of the ops (what align_benchmark prints)
 *   ops_out[0..*ops_len) : raw operations (M/X/I/D)
 * ops_cap must be >= plen + tlen + 1. */
int ref_biwfa_align(const char* pattern, int plen, const char* text, int tlen,
                    int match, int mismatch, int gap_open, int gap_ext, int score_only,
                    int* cigar_score_out, int* rescore_out,
                    char* ops_out, int ops_cap, int* ops_len) {
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_affine;
  attr.affine_penalties.match = match;
  attr.affine_penalties.mismatch = mismatch;
  attr.affine_penalties.gap_opening = gap_open;
  attr.affine_penalties.gap_extension = gap_ext;
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = score_only ? compute_score : compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  const int status = wavefront_align(wf, pattern, plen, text, tlen);
  cigar_t* const cigar = wf->cigar;
  *cigar_score_out = cigar->score;
  *ops_len = 0;
  *rescore_out = -1;
  if (!score_only && cigar->begin_offset < cigar->end_offset) {
    const int n = cigar->end_offset - cigar->begin_offset;
    if (n < ops_cap) {
      memcpy(ops_out, cigar->operations + cigar->begin_offset, n);
      ops_out[n] = '\0';
      *ops_len = n;
    }
    affine_penalties_t pen = {match, mismatch, gap_open, gap_ext};
    *rescore_out = cigar_score_gap_affine(cigar, &pen);
  }
  wavefront_aligner_delete(wf);
  return status;
}

/* The same for the edit and indel distances (metric 1: edit, 2: indel; penalties unused):
 * *rescore_out is cigar_score_edit() of the ops, as align_benchmark prints it. */
int ref_wfa_align_linear(int metric, const char* pattern, int plen, const char* text, int tlen, int score_only,
                         int* cigar_score_out, int* rescore_out, char* ops_out, int ops_cap, int* ops_len) {
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = (metric == 1) ? edit : indel;
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = score_only ? compute_score : compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  const int status = wavefront_align(wf, pattern, plen, text, tlen);
  cigar_t* const cigar = wf->cigar;
  *cigar_score_out = cigar->score;
  *ops_len = 0;
  *rescore_out = -1;
  if (!score_only && cigar->begin_offset < cigar->end_offset) {
    const int n = cigar->end_offset - cigar->begin_offset;
    if (n < ops_cap) {
      memcpy(ops_out, cigar->operations + cigar->begin_offset, n);
      ops_out[n] = '\0';
      *ops_len = n;
    }
    *rescore_out = cigar_score_edit(cigar);
  }
  wavefront_aligner_delete(wf);
  return status;
}

/* The same for the gap-linear distance (penalties match, mismatch, indel):
 * *rescore_out is cigar_score_gap_linear() of the ops, as align_benchmark prints it. */
int ref_wfa_align_gap_linear(const char* pattern, int plen, const char* text, int tlen, int match, int mismatch,
                             int indel, int score_only, int* cigar_score_out, int* rescore_out, char* ops_out,
                             int ops_cap, int* ops_len) {
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_linear;
  attr.linear_penalties.match = match;
  attr.linear_penalties.mismatch = mismatch;
  attr.linear_penalties.indel = indel;
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = score_only ? compute_score : compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  const int status = wavefront_align(wf, pattern, plen, text, tlen);
  cigar_t* const cigar = wf->cigar;
  *cigar_score_out = cigar->score;
  *ops_len = 0;
  *rescore_out = -1;
  if (!score_only && cigar->begin_offset < cigar->end_offset) {
    const int n = cigar->end_offset - cigar->begin_offset;
    if (n < ops_cap) {
      memcpy(ops_out, cigar->operations + cigar->begin_offset, n);
      ops_out[n] = '\0';
      *ops_len = n;
    }
    linear_penalties_t pen = {match, mismatch, indel};
    *rescore_out = cigar_score_gap_linear(cigar, &pen);
  }
  wavefront_aligner_delete(wf);
  return status;
}

/* The same for the two-piece gap-affine distance (penalties match, mismatch, o1, e1, o2, e2):
 * *rescore_out is cigar_score_gap_affine2p() of the ops, as align_benchmark prints it. */
int ref_wfa_align_affine2p(const char* pattern, int plen, const char* text, int tlen, const int pen6[6],
                           int score_only, int* cigar_score_out, int* rescore_out, char* ops_out, int ops_cap,
                           int* ops_len) {
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_affine_2p;
  attr.affine2p_penalties.match = pen6[0];
  attr.affine2p_penalties.mismatch = pen6[1];
  attr.affine2p_penalties.gap_opening1 = pen6[2];
  attr.affine2p_penalties.gap_extension1 = pen6[3];
  attr.affine2p_penalties.gap_opening2 = pen6[4];
  attr.affine2p_penalties.gap_extension2 = pen6[5];
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = score_only ? compute_score : compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  const int status = wavefront_align(wf, pattern, plen, text, tlen);
  cigar_t* const cigar = wf->cigar;
  *cigar_score_out = cigar->score;
  *ops_len = 0;
  *rescore_out = -1;
  if (!score_only && cigar->begin_offset < cigar->end_offset) {
    const int n = cigar->end_offset - cigar->begin_offset;
    if (n < ops_cap) {
      memcpy(ops_out, cigar->operations + cigar->begin_offset, n);
      ops_out[n] = '\0';
      *ops_len = n;
    }
    *rescore_out = cigar_score_gap_affine2p(cigar, &attr.affine2p_penalties);
  }
  wavefront_aligner_delete(wf);
  return status;
}

/* Timing helper: aligns n pairs (concatenated sequences, offsets and lengths as in the
 * oracle's batch call) with ONE WFA2-lib aligner reused across pairs, as align_benchmark does
 * per thread; full CIGAR, gap-affine penalties. Returns the wall-clock seconds of the loop and
 * writes the printed scores (cigar_score_gap_affine of the CIGAR) to scores[]. */
#include <time.h>
double ref_biwfa_batch_time(int n, const char* seq, const long long* p_off, const int* plen, const long long* t_off,
                            const int* tlen, int match, int mismatch, int gap_open, int gap_ext, int* scores) {
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_affine;
  attr.affine_penalties.match = match;
  attr.affine_penalties.mismatch = mismatch;
  attr.affine_penalties.gap_opening = gap_open;
  attr.affine_penalties.gap_extension = gap_ext;
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  affine_penalties_t pen = {match, mismatch, gap_open, gap_ext};
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int i = 0; i < n; ++i) {
    wavefront_align(wf, seq + p_off[i], plen[i], seq + t_off[i], tlen[i]);
    scores[i] = (wf->cigar->begin_offset < wf->cigar->end_offset) ? cigar_score_gap_affine(wf->cigar, &pen) : -1;
  }
  clock_gettime(CLOCK_MONOTONIC, &t1);
  wavefront_aligner_delete(wf);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

/* The timed CPU baseline: n pairs on nthreads POSIX threads, static interleaved partition, ONE
 * WFA2-lib aligner per thread reused across its pairs (align_benchmark's per-thread use,
 * tools/align_benchmark/align_benchmark.c:521-551), BiWFA gap-affine, full CIGAR. Writes each
 * pair's status, printed score (cigar_score_gap_affine, -1 for an empty CIGAR) and, when ops is
 * not NULL, its operations to ops[ops_off[i] ..] (capacity plen + tlen + 1) with their count in
 * ops_len[i]. Returns the wall-clock seconds of the align loops (threads started and joined
 * inside). */
#include <pthread.h>
typedef struct {
  int tid, nthreads, n;
  const char* seq; const long long* p_off; const int* plen; const long long* t_off; const int* tlen;
  int pen[4];
  char* ops; const long long* ops_off;
  int* scores; int* status; int* ops_len;
} ref_job_t;

static void* ref_batch_worker(void* arg) {
  ref_job_t* j = (ref_job_t*)arg;
  wavefront_aligner_attr_t attr = wavefront_aligner_attr_default;
  attr.distance_metric = gap_affine;
  attr.affine_penalties.match = j->pen[0];
  attr.affine_penalties.mismatch = j->pen[1];
  attr.affine_penalties.gap_opening = j->pen[2];
  attr.affine_penalties.gap_extension = j->pen[3];
  attr.memory_mode = wavefront_memory_ultralow;
  attr.heuristic.strategy = wf_heuristic_none;
  attr.alignment_scope = compute_alignment;
  wavefront_aligner_t* const wf = wavefront_aligner_new(&attr);
  affine_penalties_t pen = {j->pen[0], j->pen[1], j->pen[2], j->pen[3]};
  for (int i = j->tid; i < j->n; i += j->nthreads) {
    j->status[i] = wavefront_align(wf, j->seq + j->p_off[i], j->plen[i], j->seq + j->t_off[i], j->tlen[i]);
    cigar_t* const cg = wf->cigar;
    const int nops = cg->end_offset - cg->begin_offset;
    j->scores[i] = nops > 0 ? cigar_score_gap_affine(cg, &pen) : -1;
    if (j->ops != NULL) {
      const int cap = j->plen[i] + j->tlen[i] + 1;
      const int m = (nops > 0 && nops <= cap) ? nops : 0;
      if (m > 0) memcpy(j->ops + j->ops_off[i], cg->operations + cg->begin_offset, (size_t)m);
      j->ops_len[i] = m;
    }
  }
  wavefront_aligner_delete(wf);
  return NULL;
}

double ref_biwfa_align_batch_mt(int n, const char* seq, const long long* p_off, const int* plen,
                                const long long* t_off, const int* tlen, const int pen4[4], int nthreads, char* ops,
                                const long long* ops_off, int* scores, int* status, int* ops_len) {
  if (nthreads < 1) nthreads = 1;
  pthread_t th[256];
  ref_job_t jobs[256];
  if (nthreads > 256) nthreads = 256;
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nthreads; ++t) {
    ref_job_t jb = {t, nthreads, n, seq, p_off, plen, t_off, tlen, {pen4[0], pen4[1], pen4[2], pen4[3]},
                    ops, ops_off, scores, status, ops_len};
    jobs[t] = jb;
    pthread_create(&th[t], NULL, ref_batch_worker, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}
