/*
 * TEST INFRASTRUCTURE — NOT PART OF THE PRODUCT (see biwfa_oracle.h).
 *
 * Plain-C restatement of WFA2-lib v2.3 BiWFA, end-to-end, no heuristic, for the gap-affine,
 * two-piece gap-affine, gap-linear, edit and indel distances.
 * Every function names the WFA2-lib function (path:line, relative to WFA2-lib/) it
 * restates. Semantics that matter for bit-exact CIGARs and are easy to lose:
 *   - an absent or null input wavefront contributes lo = 1, hi = -1 to the output
 *     limits (the shared null wavefront, wavefront/wavefront.c:110-140);
 *   - reads outside [lo,hi] of a wavefront give OFFSET_NULL (init_ends,
 *     wavefront/wavefront_compute.c:498-575);
 *   - only M offsets are bounds-checked inside the recurrence; I/D keep
 *     out-of-bounds interior values, only their ends are trimmed
 *     (wavefront_compute_affine.c:65-85, wavefront_compute.c:579-613);
 *   - the overlap scan order and strict "<" (wavefront_bialign.c:189-392);
 *   - backtrace source priority via (offset<<4)|type with an UNSHIFTED null for
 *     out-of-range sources (wavefront_backtrace.c:41-219, 320-529).
 */
#include "biwfa_oracle.h"

#include <limits.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#define OFF_NULL (INT32_MIN / 2)            /* wavefront/wavefront_offset.h:45 */
#define FALLBACK_MIN_SCORE 250              /* wavefront/wavefront_bialign.c:48 */
#define FALLBACK_MIN_LENGTH 100             /* wavefront/wavefront_bialign.c:49 */
#define RECOVERY_MIN_SCORE 500              /* wavefront/wavefront_bialign.c:50 */

/* Internal statuses (wavefront/wfa.h:52-54) */
#define ST_OK (-1)
#define ST_END_REACHED (-2)
#define ST_END_UNREACHABLE (-3)

/* Components (alignment/affine2p_penalties.h:51-57) */
enum { C_M = 0, C_I = 1, C_I2 = 2, C_D = 3, C_D2 = 4 };

/* Backtrace types (wavefront/wavefront_backtrace.c:49-59) */
enum { BT_M = 9, BT_D2_EXT = 8, BT_D2_OPEN = 7, BT_D_EXT = 6, BT_D_OPEN = 5, BT_I2_EXT = 4, BT_I2_OPEN = 3,
       BT_I_EXT = 2, BT_I_OPEN = 1 };

/* ---------------------------------------------------------------- wavefronts */
typedef struct {
  int present;   /* the slot holds a wavefront (a non-NULL pointer in WFA2) */
  int lo, hi;    /* effective range; lo > hi means null (trimmed empty) */
  int base, cap; /* storage covers k in [base, base + cap) */
  int32_t* off;
} wf_t;

static inline int wf_null(const wf_t* w) { return !w->present || w->lo > w->hi; }
static inline int32_t wf_get(const wf_t* w, int k) {
  return (w != NULL && w->present && w->lo <= k && k <= w->hi) ? w->off[k - w->base] : OFF_NULL;
}
static void wf_reserve(wf_t* w, int lo, int hi) {
  if (w->off != NULL && lo >= w->base && hi < w->base + w->cap) return;
  int len = hi - lo + 1;
  int pad = len / 2 + 16;
  free(w->off);
  w->base = lo - pad;
  w->cap = len + 2 * pad;
  w->off = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
}
/* Make k in [need_lo, need_hi] readable without range checks: values outside the
 * wavefront's [lo, hi] read as OFF_NULL (the init_ends of
 * wavefront/wavefront_compute.c:498-575). Returns a k-indexed pointer. */
static const int32_t* wf_padded(wf_t* w, int need_lo, int need_hi) {
  if (need_lo < w->base || need_hi >= w->base + w->cap) {
    const int lo = need_lo < w->lo ? need_lo : w->lo, hi = need_hi > w->hi ? need_hi : w->hi;
    const int len = hi - lo + 1, pad = len / 2 + 16;
    int32_t* nb = (int32_t*)malloc(sizeof(int32_t) * (size_t)(len + 2 * pad));
    const int nbase = lo - pad;
    if (w->lo <= w->hi)
      memcpy(nb + (w->lo - nbase), w->off + (w->lo - w->base), sizeof(int32_t) * (size_t)(w->hi - w->lo + 1));
    free(w->off);
    w->off = nb; w->base = nbase; w->cap = len + 2 * pad;
  }
  int32_t* p = w->off - w->base;
  for (int k = need_lo; k < w->lo && k <= need_hi; ++k) p[k] = OFF_NULL;
  for (int k = (w->hi + 1 > need_lo ? w->hi + 1 : need_lo); k <= need_hi; ++k) p[k] = OFF_NULL;
  return p;
}

typedef struct {
  int metric;         /* ORC_METRIC_AFFINE, _AFFINE2P, _LINEAR, _EDIT or _INDEL */
  int o2, e2;         /* second gap piece (two-piece affine; wavefront_penalties.c:132-172) */
  int x, o, e;        /* internal (possibly transformed) penalties; gap-linear: x, indel, 0;
                         edit: 1, 1, -; indel: -1, 1, - (wavefront/wavefront_penalties.c:39-94) */
  int go_adj;         /* gap-opening adjust of the overlap (wavefront_bialign.c:396-410): o, or 0 */
  int scope;          /* max_score_scope: max(o+e, x) + 1, or 2 for edit/indel (wavefront_components.c:45-93) */
  int max_steps;      /* system.max_alignment_steps */
} pen_t;

typedef struct {
  int64_t n_cells, n_ext, n_steps;
  int max_leaf_score, max_depth;
} counters_t;

/* One direction of WFA over one window (a wavefront_aligner_t in WFA2). */
typedef struct {
  const pen_t* pen;
  counters_t* cnt;
  int modular;              /* ring of `scope` slots (score-only sub-aligners) or one slot per score */
  int nslots;
  wf_t* M; wf_t* I; wf_t* D; wf_t* I2; wf_t* D2;
  const char* pat; const char* txt; /* oriented window */
  int plen, tlen;
  int comp_begin, comp_end;
  int num_null_steps;
  int status, status_score;
  int end_k, end_off;
  wf_t nullw;               /* all-NULL storage standing in for absent inputs */
  wf_t victim;              /* write-only sink for outputs that are not kept */
} dir_t;

static void dir_alloc(dir_t* d, const pen_t* pen, counters_t* cnt, int modular, int nslots) {
  memset(d, 0, sizeof(*d));
  d->pen = pen; d->cnt = cnt; d->modular = modular; d->nslots = nslots;
  d->M = (wf_t*)calloc((size_t)nslots, sizeof(wf_t));
  d->I = (wf_t*)calloc((size_t)nslots, sizeof(wf_t));
  d->D = (wf_t*)calloc((size_t)nslots, sizeof(wf_t));
  d->I2 = (wf_t*)calloc((size_t)nslots, sizeof(wf_t));
  d->D2 = (wf_t*)calloc((size_t)nslots, sizeof(wf_t));
}
static void dir_grow(dir_t* d, int nslots) {
  if (nslots <= d->nslots) return;
  d->M = (wf_t*)realloc(d->M, sizeof(wf_t) * (size_t)nslots);
  d->I = (wf_t*)realloc(d->I, sizeof(wf_t) * (size_t)nslots);
  d->D = (wf_t*)realloc(d->D, sizeof(wf_t) * (size_t)nslots);
  d->I2 = (wf_t*)realloc(d->I2, sizeof(wf_t) * (size_t)nslots);
  d->D2 = (wf_t*)realloc(d->D2, sizeof(wf_t) * (size_t)nslots);
  memset(d->I2 + d->nslots, 0, sizeof(wf_t) * (size_t)(nslots - d->nslots));
  memset(d->D2 + d->nslots, 0, sizeof(wf_t) * (size_t)(nslots - d->nslots));
  memset(d->M + d->nslots, 0, sizeof(wf_t) * (size_t)(nslots - d->nslots));
  memset(d->I + d->nslots, 0, sizeof(wf_t) * (size_t)(nslots - d->nslots));
  memset(d->D + d->nslots, 0, sizeof(wf_t) * (size_t)(nslots - d->nslots));
  d->nslots = nslots;
}
static void dir_free(dir_t* d) {
  for (int i = 0; i < d->nslots; ++i) {
    free(d->M[i].off); free(d->I[i].off); free(d->D[i].off); free(d->I2[i].off); free(d->D2[i].off);
  }
  free(d->nullw.off);
  free(d->victim.off);
  free(d->M); free(d->I); free(d->D); free(d->I2); free(d->D2);
}
static inline int dir_slot(const dir_t* d, int score) {
  return d->modular ? score % d->pen->scope : score;
}

/* wavefront_aligner_init + init_wf (wavefront/wavefront_aligner.c:251-417) */
static void dir_init(dir_t* d, const char* pat, int plen, const char* txt, int tlen, int cb, int ce) {
  d->pat = pat; d->plen = plen; d->txt = txt; d->tlen = tlen;
  d->comp_begin = cb; d->comp_end = ce;
  d->num_null_steps = 0;
  d->status = ST_OK; d->status_score = 0;
  d->end_k = INT_MAX; d->end_off = OFF_NULL;
  const int n = d->modular ? d->pen->scope : 1;
  for (int i = 0; i < n && i < d->nslots; ++i)
    d->M[i].present = d->I[i].present = d->D[i].present = d->I2[i].present = d->D2[i].present = 0;
  wf_t* w = (cb == C_M) ? &d->M[0] : (cb == C_I) ? &d->I[0] : (cb == C_D) ? &d->D[0] : (cb == C_I2) ? &d->I2[0]
                                                                                                 : &d->D2[0];
  wf_reserve(w, 0, 0);
  w->present = 1; w->lo = 0; w->hi = 0; w->off[0 - w->base] = 0;
}

/* Fetch an input wavefront: NULL when score < 0, the slot is empty or the wavefront
 * is null (wavefront_compute_get_*wavefront, wavefront/wavefront_compute.c:249-285). */
static inline wf_t* fetch(const dir_t* d, wf_t* comp, int score) {
  if (score < 0) return NULL;
  int s = score;
  if (d->modular && s > 0) s = s % d->pen->scope;
  if (!d->modular && s >= d->nslots) return NULL;
  wf_t* w = &comp[s];
  return wf_null(w) ? NULL : w;
}

/* k-indexed all-NULL array covering [need_lo, need_hi] (the shared null wavefront). */
static const int32_t* null_padded(dir_t* d, int need_lo, int need_hi) {
  wf_t* w = &d->nullw;
  if (w->off == NULL || need_lo < w->base || need_hi >= w->base + w->cap) {
    const int lo = (w->off && w->base < need_lo) ? w->base : need_lo;
    const int hi = (w->off && w->base + w->cap - 1 > need_hi) ? w->base + w->cap - 1 : need_hi;
    const int len = hi - lo + 1, pad = len / 2 + 64;
    free(w->off);
    w->base = lo - pad; w->cap = len + 2 * pad;
    w->off = (int32_t*)malloc(sizeof(int32_t) * (size_t)w->cap);
    for (int i = 0; i < w->cap; ++i) w->off[i] = OFF_NULL;
  }
  return w->off - w->base;
}

/* Trim out-of-bounds ends (wavefront_compute_trim_ends, wavefront/wavefront_compute.c:579-613). */
static void trim_ends(const dir_t* d, wf_t* w) {
  const uint32_t tl = (uint32_t)d->tlen, pl = (uint32_t)d->plen;
  int k;
  for (k = w->hi; k >= w->lo; --k) {
    const int32_t off = w->off[k - w->base];
    if ((uint32_t)off <= tl && (uint32_t)(off - k) <= pl) break;
  }
  w->hi = k;
  for (k = w->lo; k <= w->hi; ++k) {
    const int32_t off = w->off[k - w->base];
    if ((uint32_t)off <= tl && (uint32_t)(off - k) <= pl) break;
  }
  w->lo = k;
}

/* wf_compute_edit_best_score / _worst_score (wavefront/wavefront_compute_edit.c:199-218) */
static inline int edit_best(int plen, int tlen, int k, int32_t off) {
  const int left_v = plen - (off - k), left_h = tlen - off;
  return left_v >= left_h ? left_v - left_h : left_h - left_v;
}
static inline int edit_worst(int plen, int tlen, int k, int32_t off) {
  const int left_v = plen - (off - k), left_h = tlen - off;
  return left_v > left_h ? left_v : left_h;
}

/* wavefront_compute_edit_exact_prune (wavefront/wavefront_compute_edit.c:219-275): on
 * wavefronts of 1,000 diagonals or more, drop end diagonals whose best case cannot beat the
 * best worst case. */
static void edit_prune(const dir_t* d, wf_t* w) {
  const int plen = d->plen, tlen = d->tlen, lo = w->lo, hi = w->hi;
  if (hi - lo + 1 < 1000) return;
  const int32_t* offs = w->off - w->base;
  const int sample_k = lo + (hi - lo) / 2;
  if (offs[sample_k] < 0) return;
  const int smax_sample = edit_worst(plen, tlen, sample_k, offs[sample_k]);
  if (edit_best(plen, tlen, lo, offs[lo]) <= smax_sample && edit_best(plen, tlen, hi, offs[hi]) <= smax_sample) return;
  int min_worst = INT_MAX;
  for (int k = lo; k <= hi; ++k) {
    if (offs[k] < 0) continue;
    const int sw = edit_worst(plen, tlen, k, offs[k]);
    if (sw < min_worst) min_worst = sw;
  }
  int lo_r = lo;
  for (int k = lo; k <= hi; ++k) {
    if (edit_best(plen, tlen, k, offs[k]) <= min_worst) break;
    ++lo_r;
  }
  int hi_r = hi;
  for (int k = hi; k > lo_r; --k) {
    if (edit_best(plen, tlen, k, offs[k]) <= min_worst) break;
    --hi_r;
  }
  w->lo = lo_r; w->hi = hi_r;
}

/* wavefront_compute_edit (wavefront/wavefront_compute_edit.c:329-374) with the edit and
 * indel kernels (:41-79): the previous M wavefront, read NULL-padded over [lo-1, hi+1],
 * gives M over [prev.lo-1, prev.hi+1]; trimmed, then pruned (edit only). */
static void dir_compute_edit(dir_t* d, int score) {
  if (!d->modular && score >= d->nslots) dir_grow(d, score + 1 > 2 * d->nslots ? score + 1 : 2 * d->nslots);
  wf_t* prev = &d->M[dir_slot(d, score - 1)];
  wf_t* om = &d->M[dir_slot(d, score)];
  d->cnt->n_steps++;
  const int lo = prev->lo - 1, hi = prev->hi + 1;
  const int32_t* pp = wf_padded(prev, lo - 1, hi + 1);
  wf_reserve(om, lo, hi); om->present = 1; om->lo = lo; om->hi = hi;
  d->cnt->n_cells += (int64_t)(hi - lo + 1);
  const uint32_t tl = (uint32_t)d->tlen, pl = (uint32_t)d->plen;
  int32_t* q = om->off - om->base;
  const int edit = d->pen->metric == ORC_METRIC_EDIT;
  for (int k = lo; k <= hi; ++k) {
    int32_t m;
    if (edit) {
      const int32_t ins = pp[k - 1], del = pp[k + 1], mis = pp[k];
      const int32_t im = (ins >= mis ? ins : mis) + 1;
      m = del >= im ? del : im;
    } else {
      const int32_t ins = pp[k - 1] + 1, del = pp[k + 1];
      m = del >= ins ? del : ins;
    }
    if ((uint32_t)m > tl || (uint32_t)(m - k) > pl) m = OFF_NULL;
    q[k] = m;
  }
  trim_ends(d, om);
  if (edit) edit_prune(d, om);
}

/* wavefront_compute_affine2p (wavefront/wavefront_compute_affine2p.c:334-368) with the idm
 * kernel (:44-104): two gap pieces (I1/D1 from M[s-o1-e1] and I1/D1[s-e1], I2/D2 likewise),
 * limits over all seven inputs, outputs allocated as wavefront_compute_allocate_output does
 * (wavefront/wavefront_compute.c:450-494), every output trimmed. */
static void dir_compute_2p(dir_t* d, int score) {
  const pen_t* p = d->pen;
  if (!d->modular && score >= d->nslots) dir_grow(d, score + 1 > 2 * d->nslots ? score + 1 : 2 * d->nslots);
  wf_t* mx = fetch(d, d->M, score - p->x);
  wf_t* mo1 = fetch(d, d->M, score - p->o - p->e);
  wf_t* ie1 = fetch(d, d->I, score - p->e);
  wf_t* de1 = fetch(d, d->D, score - p->e);
  wf_t* mo2 = fetch(d, d->M, score - p->o2 - p->e2);
  wf_t* ie2 = fetch(d, d->I2, score - p->e2);
  wf_t* de2 = fetch(d, d->D2, score - p->e2);
  const int slot = dir_slot(d, score);
  wf_t* om = &d->M[slot]; wf_t* oi1 = &d->I[slot]; wf_t* od1 = &d->D[slot];
  wf_t* oi2 = &d->I2[slot]; wf_t* od2 = &d->D2[slot];
  d->cnt->n_steps++;
  if (!mx && !mo1 && !ie1 && !de1 && !mo2 && !ie2 && !de2) {
    d->num_null_steps++;
    om->present = oi1->present = od1->present = oi2->present = od2->present = 0;
    return;
  }
  d->num_null_steps = 0;
  int lo = mx ? mx->lo : 1, hi = mx ? mx->hi : -1, t;
  t = (mo1 ? mo1->lo : 1) - 1; if (lo > t) lo = t;
  t = (mo1 ? mo1->hi : -1) + 1; if (hi < t) hi = t;
  t = (ie1 ? ie1->lo : 1) + 1; if (lo > t) lo = t;
  t = (ie1 ? ie1->hi : -1) + 1; if (hi < t) hi = t;
  t = (de1 ? de1->lo : 1) - 1; if (lo > t) lo = t;
  t = (de1 ? de1->hi : -1) - 1; if (hi < t) hi = t;
  t = (mo2 ? mo2->lo : 1) - 1; if (lo > t) lo = t;
  t = (mo2 ? mo2->hi : -1) + 1; if (hi < t) hi = t;
  t = (ie2 ? ie2->lo : 1) + 1; if (lo > t) lo = t;
  t = (ie2 ? ie2->hi : -1) + 1; if (hi < t) hi = t;
  t = (de2 ? de2->lo : 1) - 1; if (lo > t) lo = t;
  t = (de2 ? de2->hi : -1) - 1; if (hi < t) hi = t;
  const int a_i1 = mo1 || ie1, a_d1 = mo1 || de1, a_i2 = mo2 || ie2, a_d2 = mo2 || de2;
  wf_reserve(om, lo, hi); om->present = 1; om->lo = lo; om->hi = hi;
  wf_t* outs[4] = {oi1, od1, oi2, od2};
  const int alloc[4] = {a_i1, a_d1, a_i2, a_d2};
  for (int j = 0; j < 4; ++j) {
    if (alloc[j]) { wf_reserve(outs[j], lo, hi); outs[j]->present = 1; outs[j]->lo = lo; outs[j]->hi = hi; }
    else outs[j]->present = 0;
  }
  d->cnt->n_cells += 5 * (int64_t)(hi - lo + 1);
  const uint32_t tl = (uint32_t)d->tlen, pl = (uint32_t)d->plen;
  /* NULL-padded k-indexed inputs over [lo-1, hi+1] (two inputs may be the same wavefront) */
  wf_t* ins[7] = {mx, mo1, ie1, de1, mo2, ie2, de2};
  const int32_t* pin[7];
  for (int j = 0; j < 7; ++j) {
    int shared = -1;
    for (int q = 0; q < j; ++q) if (ins[j] != NULL && ins[q] == ins[j]) shared = q;
    pin[j] = ins[j] ? (shared >= 0 ? pin[shared] : wf_padded(ins[j], lo - 1, hi + 1)) : null_padded(d, lo - 1, hi + 1);
  }
  for (int j = 0; j < 7; ++j) if (!ins[j]) pin[j] = null_padded(d, lo - 1, hi + 1);
  wf_reserve(&d->victim, lo, hi);
  int32_t* const vic = d->victim.off - d->victim.base;
  int32_t* qm = om->off - om->base;
  int32_t* q[4];
  for (int j = 0; j < 4; ++j) q[j] = alloc[j] ? outs[j]->off - outs[j]->base : vic;
  for (int k = lo; k <= hi; ++k) {
    const int32_t i1o = pin[1][k - 1], i1e = pin[2][k - 1];
    const int32_t ins1 = (i1o >= i1e ? i1o : i1e) + 1;
    const int32_t i2o = pin[4][k - 1], i2e = pin[5][k - 1];
    const int32_t ins2 = (i2o >= i2e ? i2o : i2e) + 1;
    const int32_t ins = ins1 >= ins2 ? ins1 : ins2;
    const int32_t d1o = pin[1][k + 1], d1e = pin[3][k + 1];
    const int32_t del1 = d1o >= d1e ? d1o : d1e;
    const int32_t d2o = pin[4][k + 1], d2e = pin[6][k + 1];
    const int32_t del2 = d2o >= d2e ? d2o : d2e;
    const int32_t del = del1 >= del2 ? del1 : del2;
    const int32_t mis = pin[0][k] + 1;
    int32_t m = mis >= ins ? mis : ins;
    m = del >= m ? del : m;
    if ((uint32_t)m > tl || (uint32_t)(m - k) > pl) m = OFF_NULL;
    q[0][k] = ins1; q[1][k] = del1; q[2][k] = ins2; q[3][k] = del2;
    qm[k] = m;
  }
  trim_ends(d, om);
  for (int j = 0; j < 4; ++j) if (alloc[j]) trim_ends(d, outs[j]);
}

/* wavefront_compute_affine (wavefront/wavefront_compute_affine.c:229-260) with
 * fetch_input (wavefront_compute.c:306-352), limits_input (:40-104),
 * allocate_output(_null) (:382-494), the idm kernel (compute_affine.c:44-86)
 * and process_ends (:614-632). */
static void dir_compute(dir_t* d, int score) {
  const pen_t* p = d->pen;
  if (p->metric == ORC_METRIC_EDIT || p->metric == ORC_METRIC_INDEL) { dir_compute_edit(d, score); return; }
  if (p->metric == ORC_METRIC_AFFINE2P) { dir_compute_2p(d, score); return; }
  /* gap-linear (wavefront_compute_linear, wavefront/wavefront_compute_linear.c:166-195): the
   * same step with M inputs only (mismatch at s-x, indel at s-o) and an M output */
  const int lin = p->metric == ORC_METRIC_LINEAR;
  if (!d->modular && score >= d->nslots) dir_grow(d, score + 1 > 2 * d->nslots ? score + 1 : 2 * d->nslots);
  wf_t* mx = fetch(d, d->M, score - p->x);
  wf_t* mo = fetch(d, d->M, score - p->o - p->e);
  wf_t* ie = lin ? NULL : fetch(d, d->I, score - p->e);
  wf_t* de = lin ? NULL : fetch(d, d->D, score - p->e);
  const int slot = dir_slot(d, score);
  wf_t* om = &d->M[slot]; wf_t* oi = &d->I[slot]; wf_t* od = &d->D[slot];
  d->cnt->n_steps++;
  if (!mx && !mo && !ie && !de) {
    d->num_null_steps++;
    om->present = oi->present = od->present = 0;
    return;
  }
  d->num_null_steps = 0;
  /* Limits: a missing input is the shared null wavefront with lo=1, hi=-1. */
  int lo = mx ? mx->lo : 1, hi = mx ? mx->hi : -1, t;
  t = (mo ? mo->lo : 1) - 1; if (lo > t) lo = t;
  t = (mo ? mo->hi : -1) + 1; if (hi < t) hi = t;
  if (!lin) {  /* wavefront_compute_limits_input stops after M for gap-linear */
    t = (ie ? ie->lo : 1) + 1; if (lo > t) lo = t;
    t = (ie ? ie->hi : -1) + 1; if (hi < t) hi = t;
    t = (de ? de->lo : 1) - 1; if (lo > t) lo = t;
    t = (de ? de->hi : -1) - 1; if (hi < t) hi = t;
  }
  const int alloc_i = !lin && ((mo != NULL) || (ie != NULL));
  const int alloc_d = !lin && ((mo != NULL) || (de != NULL));
  wf_reserve(om, lo, hi); om->present = 1; om->lo = lo; om->hi = hi;
  if (alloc_i) { wf_reserve(oi, lo, hi); oi->present = 1; oi->lo = lo; oi->hi = hi; } else oi->present = 0;
  if (alloc_d) { wf_reserve(od, lo, hi); od->present = 1; od->lo = lo; od->hi = hi; } else od->present = 0;
  d->cnt->n_cells += 3 * (int64_t)(hi - lo + 1);
  const uint32_t tl = (uint32_t)d->tlen, pl = (uint32_t)d->plen;
  /* NULL-padded k-indexed inputs (mx and mo may be the same wavefront when x == o + e). */
  const int32_t *pmx, *pmo;
  if (mx != NULL && mx == mo) {
    pmx = pmo = wf_padded(mx, lo - 1, hi + 1);
  } else {
    pmo = mo ? wf_padded(mo, lo - 1, hi + 1) : null_padded(d, lo - 1, hi + 1);
    pmx = mx ? wf_padded(mx, lo, hi) : null_padded(d, lo - 1, hi + 1);
  }
  const int32_t* pie = ie ? wf_padded(ie, lo - 1, hi - 1) : null_padded(d, lo - 1, hi + 1);
  const int32_t* pde = de ? wf_padded(de, lo + 1, hi + 1) : null_padded(d, lo - 1, hi + 1);
  /* Outputs that WFA2 sends to its victim wavefront go to a scratch array here, so the
   * loop below has no branches (wavefront_compute.c:382-494). */
  wf_reserve(&d->victim, lo, hi);
  int32_t* qm = om->off - om->base;
  int32_t* qi = alloc_i ? oi->off - oi->base : d->victim.off - d->victim.base;
  int32_t* qd = alloc_d ? od->off - od->base : d->victim.off - d->victim.base;
  for (int k = lo; k <= hi; ++k) {
    const int32_t ins_o = pmo[k - 1], ins_e = pie[k - 1];
    const int32_t ins = (ins_o >= ins_e ? ins_o : ins_e) + 1;
    const int32_t del_o = pmo[k + 1], del_e = pde[k + 1];
    const int32_t del = (del_o >= del_e ? del_o : del_e);
    const int32_t mis = pmx[k] + 1;
    int32_t m = mis >= ins ? mis : ins;
    m = del >= m ? del : m;
    if ((uint32_t)m > tl || (uint32_t)(m - k) > pl) m = OFF_NULL;
    qi[k] = ins;
    qd[k] = del;
    qm[k] = m;
  }
  trim_ends(d, om);
  if (alloc_i) trim_ends(d, oi);
  if (alloc_d) trim_ends(d, od);
}

/* Longest common extension from (v, h): the sentinel comparison of
 * wavefront_extend_matches_kernel_blockwise (wavefront_extend_kernels.c:68-92)
 * written with explicit window bounds instead of EOS characters. */
static inline int lcp(const char* P, int plen, const char* T, int tlen, int v, int h) {
  const int maxn = (plen - v < tlen - h) ? plen - v : tlen - h;
  const char* p = P + v;
  const char* t = T + h;
  int n = 0;
  while (n + 8 <= maxn) {
    uint64_t a, b;
    memcpy(&a, p + n, 8); memcpy(&b, t + n, 8);
    const uint64_t x = a ^ b;
    if (x) return n + (__builtin_ctzll(x) >> 3);
    n += 8;
  }
  while (n < maxn && p[n] == t[n]) ++n;
  return n;
}

/* wavefront_termination_end2end (wavefront/wavefront_termination.c:37-114) */
static int termination(dir_t* d, int score) {
  const int ak = d->tlen - d->plen;
  const int aoff = d->tlen;
  const int slot = dir_slot(d, score);
  const wf_t* w = (d->comp_end == C_M) ? &d->M[slot] : (d->comp_end == C_I) ? &d->I[slot]
                 : (d->comp_end == C_D) ? &d->D[slot] : (d->comp_end == C_I2) ? &d->I2[slot] : &d->D2[slot];
  if (!w->present || w->lo > ak || ak > w->hi) return 0;
  if (w->off[ak - w->base] < aoff) return 0;
  d->end_k = ak; d->end_off = aoff;
  return 1;
}

/* wavefront_extend_end2end(_max) (wavefront/wavefront_extend.c:86-121, 173-211) */
static int dir_extend(dir_t* d, int score, int* max_ak_out) {
  if (max_ak_out) *max_ak_out = 0;
  const int slot = dir_slot(d, score);
  wf_t* m = &d->M[slot];
  if (!m->present) {
    if (d->num_null_steps > d->pen->scope) {
      d->status = ST_END_UNREACHABLE; d->status_score = score; return 1;
    }
    return 0;
  }
  int max_ak = 0;
  int32_t* const offs = m->off - m->base;
  const char* const P = d->pat;
  const char* const T = d->txt;
  const int plen = d->plen, tlen = d->tlen, lo = m->lo, hi = m->hi;
  int64_t ext = 0;
  for (int k = lo; k <= hi; ++k) {
    int32_t off = offs[k];
    if (off == OFF_NULL) continue;
    const int n = lcp(P, plen, T, tlen, off - k, off);
    ext += n + 1;
    off += n;
    offs[k] = off;
    const int ak = 2 * off - k;
    if (max_ak < ak) max_ak = ak;
  }
  d->cnt->n_ext += ext;
  if (termination(d, score)) {
    d->status = ST_END_REACHED; d->status_score = score; return 1;
  }
  if (max_ak_out) *max_ak_out = max_ak;
  return 0;
}

/* ---------------------------------------------------------------- BiWFA */
typedef struct {
  int score, score_fwd, score_rev, k_fwd, k_rev, off_fwd, off_rev, comp;
} bp_t; /* wf_bialign_breakpoint_t (wavefront/wavefront_bialigner.h:43-54) */

typedef struct {
  pen_t pen;
  int match_orig, x_orig, o_orig, e_orig, o2_orig, e2_orig;
  const char* P; const char* T; /* forward full sequences */
  char* rP; char* rT;           /* reversed full sequences */
  int plen_full, tlen_full;
  dir_t fwd, rev, base;
  char* ops; int ops_len, ops_cap;
  char* leaf;                   /* leaf backtrace buffer (written backwards) */
  int leaf_cap;
  int cigar_score;
  counters_t cnt;
} ctx_t;

/* wavefront_bialign_breakpoint_indel2indel (wavefront/wavefront_bialign.c:189-256) */
static void bp_indel(int go, int plen, int tlen, int fwd, int s0, int s1,
                     const wf_t* w0, const wf_t* w1, int comp, bp_t* bp) {
  const int lo0 = w0->lo, hi0 = w0->hi;
  const int lo1 = tlen - plen - w1->hi, hi1 = tlen - plen - w1->lo;
  if (hi1 < lo0 || hi0 < lo1) return;
  const int min_hi = hi0 < hi1 ? hi0 : hi1;
  const int max_lo = lo0 > lo1 ? lo0 : lo1;
  for (int k0 = max_lo; k0 <= min_hi; ++k0) {
    const int k1 = tlen - plen - k0;
    const int32_t d0 = w0->off[k0 - w0->base], d1 = w1->off[k1 - w1->base];
    if (d0 + d1 >= tlen && s0 + s1 - go < bp->score) {
      if (fwd) {
        const int v = d0 - k0, h = d0;
        if (v > plen || h > tlen) continue;
        bp->score_fwd = s0; bp->score_rev = s1; bp->k_fwd = k0; bp->k_rev = k1;
        bp->off_fwd = d0; bp->off_rev = d1;
      } else {
        const int v = d1 - k1, h = d1;
        if (v > plen || h > tlen) continue;
        bp->score_fwd = s1; bp->score_rev = s0; bp->k_fwd = k1; bp->k_rev = k0;
        bp->off_fwd = d1; bp->off_rev = d0;
      }
      bp->score = s0 + s1 - go;
      bp->comp = comp;
      return;
    }
  }
}

/* wavefront_bialign_breakpoint_m2m (wavefront/wavefront_bialign.c:257-310) */
static void bp_m2m(int plen, int tlen, int fwd, int s0, int s1,
                   const wf_t* w0, const wf_t* w1, bp_t* bp) {
  const int lo0 = w0->lo, hi0 = w0->hi;
  const int lo1 = tlen - plen - w1->hi, hi1 = tlen - plen - w1->lo;
  if (hi1 < lo0 || hi0 < lo1) return;
  const int min_hi = hi0 < hi1 ? hi0 : hi1;
  const int max_lo = lo0 > lo1 ? lo0 : lo1;
  for (int k0 = max_lo; k0 <= min_hi; ++k0) {
    const int k1 = tlen - plen - k0;
    const int32_t m0 = w0->off[k0 - w0->base], m1 = w1->off[k1 - w1->base];
    if (m0 + m1 >= tlen && s0 + s1 < bp->score) {
      if (fwd) {
        bp->score_fwd = s0; bp->score_rev = s1; bp->k_fwd = k0; bp->k_rev = k1;
        bp->off_fwd = m0; bp->off_rev = m1;
      } else {
        bp->score_fwd = s1; bp->score_rev = s0; bp->k_fwd = k1; bp->k_rev = k0;
        bp->off_fwd = m1; bp->off_rev = m0;
      }
      bp->score = s0 + s1;
      bp->comp = C_M;
      return;
    }
  }
}

/* wavefront_bialign_overlap (wavefront/wavefront_bialign.c:314-392): the second gap
 * piece's I2/D2 pairs first (gap-open o2), then I1/D1 (o1), then M. */
static void overlap(const ctx_t* c, const dir_t* d0, const dir_t* d1, int s0, int s1, int fwd, bp_t* bp) {
  const int scope = c->pen.scope, go = c->pen.go_adj;
  const int plen = d0->plen, tlen = d0->tlen;
  const int sm0 = s0 % scope;
  const wf_t* m0 = &d0->M[sm0];
  if (!m0->present) return;
  const int two = c->pen.metric == ORC_METRIC_AFFINE2P;
  const wf_t* dd0 = &d0->D[sm0];
  const wf_t* ii0 = &d0->I[sm0];
  const wf_t* dd20 = two ? &d0->D2[sm0] : NULL;
  const wf_t* ii20 = two ? &d0->I2[sm0] : NULL;
  for (int i = 0; i < scope; ++i) {
    const int si = s1 - i;
    if (si < 0) break;
    const int smi = si % scope;
    if (two) {
      if (s0 + si - c->pen.o2 >= bp->score) continue;
      const wf_t* dd21 = &d1->D2[smi];
      if (dd20->present && dd21->present) bp_indel(c->pen.o2, plen, tlen, fwd, s0, si, dd20, dd21, C_D2, bp);
      const wf_t* ii21 = &d1->I2[smi];
      if (ii20->present && ii21->present) bp_indel(c->pen.o2, plen, tlen, fwd, s0, si, ii20, ii21, C_I2, bp);
    }
    if (s0 + si - (two ? c->pen.o : go) >= bp->score) continue;
    const wf_t* dd1 = &d1->D[smi];
    if (dd0->present && dd1->present) bp_indel(c->pen.o, plen, tlen, fwd, s0, si, dd0, dd1, C_D, bp);
    const wf_t* ii1 = &d1->I[smi];
    if (ii0->present && ii1->present) bp_indel(c->pen.o, plen, tlen, fwd, s0, si, ii0, ii1, C_I, bp);
    if (s0 + si >= bp->score) continue;
    const wf_t* mm1 = &d1->M[smi];
    if (mm1->present) bp_m2m(plen, tlen, fwd, s0, si, m0, mm1, bp);
  }
}

/* Window set-up: wavefront_bialigner_set_sequences_bounds (wavefront_bialigner.c:107-121)
 * and wavefront_sequences_set_bounds (wavefront_sequences.c:274-309). */
static void set_windows(ctx_t* c, int pb, int pe, int tb, int te, int cb, int ce) {
  dir_init(&c->fwd, c->P + pb, pe - pb, c->T + tb, te - tb, cb, ce);
  dir_init(&c->rev, c->rP + (c->plen_full - pe), pe - pb, c->rT + (c->tlen_full - te), te - tb, ce, cb);
}

/* wavefront_bialign_find_breakpoint (wavefront/wavefront_bialign.c:411-519) */
static int find_breakpoint(ctx_t* c, int pb, int pe, int tb, int te, int cb, int ce, bp_t* bp) {
  dir_t* F = &c->fwd; dir_t* R = &c->rev;
  set_windows(c, pb, pe, tb, te, cb, ce);
  const int plen = pe - pb, tlen = te - tb;
  const int max_steps = c->pen.max_steps;
  const int max_antidiag = plen + tlen - 1;
  int sf = 0, sr = 0, fmax = 0, rmax = 0, ak;
  bp->score = INT_MAX;
  if (dir_extend(F, sf, &fmax)) return F->status;
  if (dir_extend(R, sr, &rmax)) return R->status;
  int last_fwd = 0;
  for (;;) {
    if (fmax + rmax >= max_antidiag) break;
    ++sf; dir_compute(F, sf);
    const int qf = dir_extend(F, sf, &ak);
    if (fmax < ak) fmax = ak;
    last_fwd = 1;
    if (qf) return F->status;
    if (fmax + rmax >= max_antidiag) break;
    ++sr; dir_compute(R, sr);
    const int qr = dir_extend(R, sr, &ak);
    if (rmax < ak) rmax = ak;
    last_fwd = 0;
    if (qr) return R->status;
    if (sr + sf >= max_steps) return ORC_STATUS_MAX_STEPS_REACHED;
  }
  const int scope = c->pen.scope, go = c->pen.go_adj;
  for (;;) {
    if (last_fwd) {
      const int min_sr = (sr > scope - 1) ? sr - (scope - 1) : 0;
      if (sf + min_sr - go >= bp->score) break;
      overlap(c, F, R, sf, sr, 1, bp);
      ++sr; dir_compute(R, sr);
      if (dir_extend(R, sr, NULL)) return R->status;
    }
    const int min_sf = (sf > scope - 1) ? sf - (scope - 1) : 0;
    if (min_sf + sr - go >= bp->score) break;
    overlap(c, R, F, sr, sf, 0, bp);
    ++sf; dir_compute(F, sf);
    if (dir_extend(F, sf, NULL)) return F->status;
    if (sr + sf >= max_steps) return ORC_STATUS_MAX_STEPS_REACHED;
    last_fwd = 1;
  }
  return ST_OK;
}

/* Backtrace source fetchers (wavefront/wavefront_backtrace.c:64-219). An absent or
 * out-of-range source is the UNSHIFTED null; an in-range source is (offset<<4)|type. */
static inline int64_t bt_src(const dir_t* d, const wf_t* comp, int score, int kk, int add, int type) {
  if (score < 0 || score >= d->nslots) return OFF_NULL;
  const wf_t* w = &comp[score];
  if (w->present && w->lo <= kk && kk <= w->hi) {
    return (int64_t)((uint64_t)(int64_t)(w->off[kk - w->base] + add) << 4) | type;
  }
  return OFF_NULL;
}
static inline int64_t max64(int64_t a, int64_t b) { return a >= b ? a : b; }

/* wavefront_backtrace_affine (wavefront/wavefront_backtrace.c:320-529), gap-affine and
 * two-piece gap-affine.
 * Writes the ops of the leaf into c->leaf backwards; returns the first index. */
static int backtrace_affine(ctx_t* c, const dir_t* d, int score_end, int k, int32_t off) {
  const pen_t* p = &c->pen;
  char* ops = c->leaf;
  int pos = c->leaf_cap - 1; /* next write position (backwards) */
  int matrix = d->comp_end;
  int score = score_end;
  int h = off, v = off - k;
  if (d->comp_end == C_M) {
    if (v < d->plen) { for (int i = d->plen - v; i > 0; --i) ops[pos--] = 'D'; }
    if (h < d->tlen) { for (int i = d->tlen - h; i > 0; --i) ops[pos--] = 'I'; }
  }
  while (v > 0 && h > 0 && score > 0) {
    const int mm = score - p->x, go = score - p->o - p->e, ge = score - p->e;
    const int go2 = score - p->o2 - p->e2, ge2 = score - p->e2;
    int64_t max_all;
    if (matrix == C_M) {
      const int64_t mis = bt_src(d, d->M, mm, k, 1, BT_M);
      const int64_t io = bt_src(d, d->M, go, k - 1, 1, BT_I_OPEN);
      const int64_t ix = bt_src(d, d->I, ge, k - 1, 1, BT_I_EXT);
      const int64_t dop = bt_src(d, d->M, go, k + 1, 0, BT_D_OPEN);
      const int64_t dx = bt_src(d, d->D, ge, k + 1, 0, BT_D_EXT);
      if (p->metric == ORC_METRIC_AFFINE2P) {
        const int64_t io2 = bt_src(d, d->M, go2, k - 1, 1, BT_I2_OPEN);
        const int64_t ix2 = bt_src(d, d->I2, ge2, k - 1, 1, BT_I2_EXT);
        const int64_t dop2 = bt_src(d, d->M, go2, k + 1, 0, BT_D2_OPEN);
        const int64_t dx2 = bt_src(d, d->D2, ge2, k + 1, 0, BT_D2_EXT);
        const int64_t ins = max64(max64(io, ix), max64(io2, ix2));
        const int64_t del = max64(max64(dop, dx), max64(dop2, dx2));
        max_all = max64(mis, max64(ins, del));
      } else {
        max_all = max64(mis, max64(max64(io, ix), max64(dop, dx)));
      }
    } else if (matrix == C_I) {
      max_all = max64(bt_src(d, d->M, go, k - 1, 1, BT_I_OPEN), bt_src(d, d->I, ge, k - 1, 1, BT_I_EXT));
    } else if (matrix == C_I2) {
      max_all = max64(bt_src(d, d->M, go2, k - 1, 1, BT_I2_OPEN), bt_src(d, d->I2, ge2, k - 1, 1, BT_I2_EXT));
    } else if (matrix == C_D) {
      max_all = max64(bt_src(d, d->M, go, k + 1, 0, BT_D_OPEN), bt_src(d, d->D, ge, k + 1, 0, BT_D_EXT));
    } else {
      max_all = max64(bt_src(d, d->M, go2, k + 1, 0, BT_D2_OPEN), bt_src(d, d->D2, ge2, k + 1, 0, BT_D2_EXT));
    }
    if (max_all < 0) break;
    if (matrix == C_M) {
      const int max_off = (int)(max_all >> 4);
      const int nm = off - max_off;
      for (int i = 0; i < nm; ++i) ops[pos--] = 'M';
      off = max_off;
      v = off - k; h = off;
      if (v <= 0 || h <= 0) break;
    }
    const int type = (int)(max_all & 0xF);
    switch (type) {
      case BT_M: score = mm; matrix = C_M; break;
      case BT_I_OPEN: score = go; matrix = C_M; break;
      case BT_I_EXT: score = ge; matrix = C_I; break;
      case BT_D_OPEN: score = go; matrix = C_M; break;
      case BT_D_EXT: score = ge; matrix = C_D; break;
      case BT_I2_OPEN: score = go2; matrix = C_M; break;
      case BT_I2_EXT: score = ge2; matrix = C_I2; break;
      case BT_D2_OPEN: score = go2; matrix = C_M; break;
      default: score = ge2; matrix = C_D2; break; /* BT_D2_EXT */
    }
    if (type == BT_M) { ops[pos--] = 'X'; --off; }
    else if (type == BT_I_OPEN || type == BT_I_EXT || type == BT_I2_OPEN || type == BT_I2_EXT) {
      ops[pos--] = 'I'; --k; --off;
    }
    else { ops[pos--] = 'D'; ++k; }
    v = off - k; h = off;
  }
  if (matrix == C_M) {
    if (v > 0 && h > 0) {
      const int nm = v < h ? v : h;
      for (int i = 0; i < nm; ++i) ops[pos--] = 'M';
      v -= nm; h -= nm;
    }
    while (v > 0) { ops[pos--] = 'D'; --v; }
    while (h > 0) { ops[pos--] = 'I'; --h; }
  }
  return pos + 1;
}

/* wavefront_backtrace_linear (wavefront/wavefront_backtrace.c:223-319), edit and indel:
 * sources M[s-x][k] (mismatch, edit only), M[s-o][k-1] (insertion), M[s-o][k+1] (deletion). */
static int backtrace_linear(ctx_t* c, const dir_t* d, int score_end, int k, int32_t off) {
  const pen_t* p = &c->pen;
  char* ops = c->leaf;
  int pos = c->leaf_cap - 1;
  int score = score_end;
  int h = off, v = off - k;
  if (v < d->plen) { for (int i = d->plen - v; i > 0; --i) ops[pos--] = 'D'; }
  if (h < d->tlen) { for (int i = d->tlen - h; i > 0; --i) ops[pos--] = 'I'; }
  while (v > 0 && h > 0 && score > 0) {
    const int mm = score - p->x, go = score - p->o;
    const int64_t mis = (p->metric != ORC_METRIC_INDEL) ? bt_src(d, d->M, mm, k, 1, BT_M) : (int64_t)OFF_NULL;
    const int64_t ins = bt_src(d, d->M, go, k - 1, 1, BT_I_OPEN);
    const int64_t del = bt_src(d, d->M, go, k + 1, 0, BT_D_OPEN);
    const int64_t max_all = max64(mis, max64(ins, del));
    if (max_all < 0) break;
    const int max_off = (int)(max_all >> 4);
    for (int i = off - max_off; i > 0; --i) ops[pos--] = 'M';
    off = max_off;
    v = off - k; h = off;
    if (v <= 0 || h <= 0) break;
    const int type = (int)(max_all & 0xF);
    if (type == BT_M) { score = mm; ops[pos--] = 'X'; --off; }
    else if (type == BT_I_OPEN) { score = go; ops[pos--] = 'I'; --k; --off; }
    else { score = go; ops[pos--] = 'D'; ++k; }
    v = off - k; h = off;
  }
  if (v > 0 && h > 0) {
    const int nm = v < h ? v : h;
    for (int i = 0; i < nm; ++i) ops[pos--] = 'M';
    v -= nm; h -= nm;
  }
  while (v > 0) { ops[pos--] = 'D'; --v; }
  while (h > 0) { ops[pos--] = 'I'; --h; }
  return pos + 1;
}

static void append_ops(ctx_t* c, const char* src, int n) {
  if (c->ops != NULL && c->ops_len + n <= c->ops_cap) memcpy(c->ops + c->ops_len, src, (size_t)n);
  c->ops_len += n;
}
static void append_run(ctx_t* c, char op, int n) {
  for (int i = 0; i < n; ++i) {
    if (c->ops != NULL && c->ops_len < c->ops_cap) c->ops[c->ops_len] = op;
    c->ops_len++;
  }
}

/* wavefront_bialign_base (wavefront/wavefront_bialign.c:155-185) ->
 * wavefront_unialign_init / wavefront_unialign / wavefront_unialign_terminate
 * (wavefront/wavefront_unialign.c:54-94, 147-273). */
static int bialign_base(ctx_t* c, int pb, int pe, int tb, int te, int cb, int ce) {
  dir_t* B = &c->base;
  dir_init(B, c->P + pb, pe - pb, c->T + tb, te - tb, cb, ce);
  int score = 0;
  for (;;) {
    if (dir_extend(B, score, NULL)) break;
    ++score;
    dir_compute(B, score);
    if (score >= c->pen.max_steps) return ORC_STATUS_UNATTAINABLE;
  }
  if (c->cnt.max_leaf_score < score) c->cnt.max_leaf_score = score;
  if (B->status != ST_END_REACHED) return ORC_STATUS_UNATTAINABLE;
  const int need = 2 * (B->plen + B->tlen) + 8;
  if (c->leaf_cap < need) { free(c->leaf); c->leaf_cap = need; c->leaf = (char*)malloc((size_t)need); }
  if (B->end_off != OFF_NULL) {
    const int first = (c->pen.metric == ORC_METRIC_AFFINE || c->pen.metric == ORC_METRIC_AFFINE2P) ? backtrace_affine(c, B, score, B->end_k, B->end_off)
                                                             : backtrace_linear(c, B, score, B->end_k, B->end_off);
    append_ops(c, c->leaf + first, c->leaf_cap - first);
  }
  return ST_OK;
}

static int classic_score(const ctx_t* c, int plen, int tlen, int wf_score) {
  /* wavefront_compute_classic_score (wavefront/wavefront_compute.c:108-120) */
  const int swg_match = -c->match_orig;
  if (c->pen.metric == ORC_METRIC_EDIT || c->pen.metric == ORC_METRIC_INDEL) return wf_score;  /* the distance */
  if (swg_match == 0) return -wf_score;
  return (swg_match * (plen + tlen) - wf_score) / 2; /* WF_SCORE_TO_SW_SCORE */
}

/* wavefront_bialign_alignment (wavefront/wavefront_bialign.c:581-658) */
static int bialign_alignment(ctx_t* c, int pb, int pe, int tb, int te, int cb, int ce, int rem, int level) {
  const int plen = pe - pb, tlen = te - tb;
  if (c->cnt.max_depth < level) c->cnt.max_depth = level;
  if (tlen == 0) { append_run(c, 'D', plen); return ST_OK; }
  if (plen == 0) { append_run(c, 'I', tlen); return ST_OK; }
  if (rem <= FALLBACK_MIN_SCORE) return bialign_base(c, pb, pe, tb, te, cb, ce);
  bp_t bp;
  int st = find_breakpoint(c, pb, pe, tb, te, cb, ce, &bp);
  if (st != ST_OK) {
    /* wavefront_bialign_find_breakpoint_exception (:520-547) */
    if (st == ST_END_REACHED) {
      const int reached = (c->fwd.status == ST_END_REACHED) ? c->fwd.status_score : c->rev.status_score;
      if (reached <= RECOVERY_MIN_SCORE) return bialign_base(c, pb, pe, tb, te, cb, ce);
      return ST_END_UNREACHABLE;
    }
    return st;
  }
  const int bh = bp.off_fwd, bv = bp.off_fwd - bp.k_fwd;
  st = bialign_alignment(c, pb, pb + bv, tb, tb + bh, cb, bp.comp, bp.score_fwd, level + 1);
  if (st != ST_OK) return st;
  st = bialign_alignment(c, pb + bv, pe, tb + bh, te, bp.comp, ce, bp.score_rev, level + 1);
  if (st != ST_OK) return st;
  if (level == 0) c->cigar_score = classic_score(c, plen, tlen, bp.score);
  return ST_OK;
}

/* cigar_score_gap_affine2p (alignment/cigar.c:304-342: per run of I or D the cheaper piece,
 * min(o1 + e1*L, o2 + e2*L)),
 * cigar_score_gap_affine (alignment/cigar.c:277-303) with the caller's penalties,
 * cigar_score_gap_linear (:260-276, o = indel) or cigar_score_edit (:244-259) for the edit and
 * indel distances. */
static int rescore(int metric, const char* ops, int n, int match, int x, int o, int e, int o2, int e2) {
  char last = 0; int score = 0;
  if (metric == ORC_METRIC_AFFINE2P) {
    for (int i = 0; i < n;) {
      int j = i;
      while (j < n && ops[j] == ops[i]) ++j;
      const int len = j - i;
      if (ops[i] == 'M') score -= match * len;
      else if (ops[i] == 'X') score -= x * len;
      else { const int a = o + e * len, b = o2 + e2 * len; score -= a < b ? a : b; }
      i = j;
    }
    return score;
  }
  if (metric == ORC_METRIC_EDIT || metric == ORC_METRIC_INDEL) {
    for (int i = 0; i < n; ++i) score += (ops[i] != 'M');
    return score;
  }
  if (metric == ORC_METRIC_LINEAR) {
    for (int i = 0; i < n; ++i) score -= (ops[i] == 'M') ? match : (ops[i] == 'X') ? x : o;
    return score;
  }
  for (int i = 0; i < n; ++i) {
    switch (ops[i]) {
      case 'M': score -= match; break;
      case 'X': score -= x; break;
      case 'D': score -= e + (last == 'D' ? 0 : o); break;
      case 'I': score -= e + (last == 'I' ? 0 : o); break;
      default: break;
    }
    last = ops[i];
  }
  return score;
}

static void ctx_init(ctx_t* c, int metric, int match, int x, int o, int e, int o2, int e2) {
  memset(c, 0, sizeof(*c));
  c->match_orig = match; c->x_orig = x; c->o_orig = o; c->e_orig = e; c->o2_orig = o2; c->e2_orig = e2;
  c->pen.metric = metric;
  if (metric == ORC_METRIC_EDIT || metric == ORC_METRIC_INDEL) {
    /* wavefront_penalties_set_edit / _indel and wavefront_components_dimensions_edit */
    c->pen.x = metric == ORC_METRIC_EDIT ? 1 : -1; c->pen.o = 1; c->pen.e = -1;
    c->pen.go_adj = 0;
    c->pen.scope = 2;
  } else if (metric == ORC_METRIC_LINEAR) {
    /* wavefront_penalties_set_linear (wavefront/wavefront_penalties.c:63-94), indel in o;
     * wavefront_components_dimensions_linear (wavefront_components.c:61-78) */
    if (match < 0) { c->pen.x = 2 * x - 2 * match; c->pen.o = 2 * o - match; }
    else { c->pen.x = x; c->pen.o = o; }
    c->pen.e = 0;
    c->pen.scope = (c->pen.x > c->pen.o ? c->pen.x : c->pen.o) + 1;
    c->pen.go_adj = 0;
  } else if (metric == ORC_METRIC_AFFINE2P) {
    /* wavefront_penalties_set_affine2p (wavefront/wavefront_penalties.c:132-173);
     * wavefront_components_dimensions_affine2p (wavefront_components.c:97-116);
     * wavefront_bialign_overlap_gopen_adjust (wavefront_bialign.c:396-410) */
    if (match < 0) {
      c->pen.x = 2 * x - 2 * match; c->pen.o = 2 * o; c->pen.e = 2 * e - match;
      c->pen.o2 = 2 * o2; c->pen.e2 = 2 * e2 - match;
    } else {
      c->pen.x = x; c->pen.o = o; c->pen.e = e; c->pen.o2 = o2; c->pen.e2 = e2;
    }
    int sc = c->pen.x;
    if (sc < c->pen.o + c->pen.e) sc = c->pen.o + c->pen.e;
    if (sc < c->pen.o2 + c->pen.e2) sc = c->pen.o2 + c->pen.e2;
    c->pen.scope = sc + 1;
    c->pen.go_adj = c->pen.o > c->pen.o2 ? c->pen.o : c->pen.o2;
  } else {
    /* wavefront_penalties_set_affine (wavefront/wavefront_penalties.c:95-130) */
    if (match < 0) {
      c->pen.x = 2 * x - 2 * match; c->pen.o = 2 * o; c->pen.e = 2 * e - match;
    } else {
      c->pen.x = x; c->pen.o = o; c->pen.e = e;
    }
    const int oe = c->pen.o + c->pen.e;
    c->pen.scope = (oe > c->pen.x ? oe : c->pen.x) + 1;
    c->pen.go_adj = c->pen.o;
  }
  c->pen.max_steps = INT_MAX;
  c->cnt.max_leaf_score = -1;
  dir_alloc(&c->fwd, &c->pen, &c->cnt, 1, c->pen.scope);
  dir_alloc(&c->rev, &c->pen, &c->cnt, 1, c->pen.scope);
  dir_alloc(&c->base, &c->pen, &c->cnt, 0, 64);
}
static void ctx_free(ctx_t* c) {
  dir_free(&c->fwd); dir_free(&c->rev); dir_free(&c->base);
  free(c->rP); free(c->rT); free(c->leaf);
}

static int validate(int metric, int match, int x, int o, int e, int o2, int e2) {
  if (metric == ORC_METRIC_EDIT || metric == ORC_METRIC_INDEL) return 1;
  if (metric == ORC_METRIC_LINEAR) return !(match > 0 || x <= 0 || o <= 0);
  if (metric == ORC_METRIC_AFFINE2P) return !(match > 0 || x <= 0 || o < 0 || e <= 0 || o2 < 0 || e2 <= 0);
  if (metric != ORC_METRIC_AFFINE) return 0;
  return !(match > 0 || x <= 0 || o < 0 || e <= 0);
}

static int align_one(ctx_t* c, const char* pattern, int plen, const char* text, int tlen,
                     int score_only, char* ops, int ops_cap, orc_result_t* res) {
  c->P = pattern; c->T = text; c->plen_full = plen; c->tlen_full = tlen;
  c->rP = (char*)realloc(c->rP, (size_t)plen + 1);
  c->rT = (char*)realloc(c->rT, (size_t)tlen + 1);
  for (int i = 0; i < plen; ++i) c->rP[i] = pattern[plen - 1 - i];
  for (int i = 0; i < tlen; ++i) c->rT[i] = text[tlen - 1 - i];
  c->ops = ops; c->ops_cap = ops_cap; c->ops_len = 0;
  c->cigar_score = INT32_MIN;
  memset(&c->cnt, 0, sizeof(c->cnt));
  c->cnt.max_leaf_score = -1;
  int st, final_status;
  if (score_only) {
    /* wavefront_bialign_compute_score (wavefront/wavefront_bialign.c:662-699) */
    bp_t bp;
    st = find_breakpoint(c, 0, plen, 0, tlen, C_M, C_M, &bp);
    if (st == ST_OK || st == ST_END_REACHED) {
      if (st == ST_END_REACHED)
        bp.score = (c->fwd.status == ST_END_REACHED) ? c->fwd.status_score : c->rev.status_score;
      c->cigar_score = classic_score(c, plen, tlen, bp.score);
      st = ST_OK;
    }
  } else {
    /* wavefront_bialign (wavefront/wavefront_bialign.c:703-730) */
    const int min_len = (plen > tlen ? plen : tlen) <= FALLBACK_MIN_LENGTH;
    st = bialign_alignment(c, 0, plen, 0, tlen, C_M, C_M, min_len ? 0 : INT_MAX, 0);
  }
  if (st == ST_OK) final_status = ORC_STATUS_ALG_COMPLETED;
  else if (st == ORC_STATUS_MAX_STEPS_REACHED || st == ORC_STATUS_OOM) final_status = st;
  else final_status = ORC_STATUS_UNATTAINABLE;
  if (res) {
    res->status = final_status;
    res->cigar_score = c->cigar_score;
    res->ops_len = score_only ? 0 : c->ops_len;
    if (score_only) res->score = c->cigar_score;
    else res->score = (c->ops_len > 0 && c->ops_len <= ops_cap)
        ? rescore(c->pen.metric, ops, c->ops_len, c->match_orig, c->x_orig, c->o_orig, c->e_orig, c->o2_orig,
                  c->e2_orig)
        : -1;
    res->n_cells = c->cnt.n_cells; res->n_ext = c->cnt.n_ext; res->n_steps = c->cnt.n_steps;
    res->max_leaf_score = c->cnt.max_leaf_score; res->max_depth = c->cnt.max_depth;
  }
  return final_status;
}

int orc_wfa_align_pen(int metric, const char* pattern, int plen, const char* text, int tlen, const int pen[6],
                      int score_only, char* ops, int ops_cap, orc_result_t* res) {
  if (!validate(metric, pen[0], pen[1], pen[2], pen[3], pen[4], pen[5]) || plen < 0 || tlen < 0) {
    if (res) { memset(res, 0, sizeof(*res)); res->status = ORC_STATUS_UNATTAINABLE; res->score = -1; }
    return ORC_STATUS_UNATTAINABLE;
  }
  ctx_t c;
  ctx_init(&c, metric, pen[0], pen[1], pen[2], pen[3], pen[4], pen[5]);
  const int st = align_one(&c, pattern, plen, text, tlen, score_only, ops, ops_cap, res);
  ctx_free(&c);
  return st;
}

int orc_wfa_align(int metric, const char* pattern, int plen, const char* text, int tlen,
                  int match, int mismatch, int gap_open, int gap_ext,
                  int score_only, char* ops, int ops_cap, orc_result_t* res) {
  const int pen[6] = {match, mismatch, gap_open, gap_ext, 0, 1};
  return orc_wfa_align_pen(metric, pattern, plen, text, tlen, pen, score_only, ops, ops_cap, res);
}

int orc_biwfa_align(const char* pattern, int plen, const char* text, int tlen,
                    int match, int mismatch, int gap_open, int gap_ext,
                    int score_only, char* ops, int ops_cap, orc_result_t* res) {
  return orc_wfa_align(ORC_METRIC_AFFINE, pattern, plen, text, tlen, match, mismatch, gap_open, gap_ext, score_only,
                       ops, ops_cap, res);
}

/* ---------------------------------------------------------------- batch (CPU baseline) */
typedef struct {
  int tid, nthreads, n;
  const char* pat; const int64_t* pat_off; const int* plen;
  const char* txt; const int64_t* txt_off; const int* tlen;
  int metric, match, x, o, e, o2, e2, score_only;
  char* ops; const int64_t* ops_off;
  int* scores; int* status; int* ops_len;
} job_t;

static void* batch_worker(void* arg) {
  job_t* j = (job_t*)arg;
  ctx_t c;
  ctx_init(&c, j->metric, j->match, j->x, j->o, j->e, j->o2, j->e2);
  for (int i = j->tid; i < j->n; i += j->nthreads) {
    orc_result_t r;
    const int cap = j->plen[i] + j->tlen[i] + 1;
    char* ops = j->score_only ? NULL : j->ops + j->ops_off[i];
    align_one(&c, j->pat + j->pat_off[i], j->plen[i], j->txt + j->txt_off[i], j->tlen[i],
              j->score_only, ops, cap, &r);
    j->scores[i] = r.score; j->status[i] = r.status; j->ops_len[i] = r.ops_len;
  }
  ctx_free(&c);
  return NULL;
}

double orc_wfa_align_batch_pen(int metric, int n, const char* pat, const int64_t* pat_off, const int* plen,
                               const char* txt, const int64_t* txt_off, const int* tlen, const int pen[6],
                               int score_only, char* ops, const int64_t* ops_off,
                               int* scores, int* status, int* ops_len, int nthreads) {
  if (nthreads < 1) nthreads = 1;
  const int match = pen[0], mismatch = pen[1], gap_open = pen[2], gap_ext = pen[3], o2 = pen[4], e2 = pen[5];
  if (!validate(metric, match, mismatch, gap_open, gap_ext, o2, e2)) return -1.0;
  pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)nthreads);
  job_t* jobs = (job_t*)malloc(sizeof(job_t) * (size_t)nthreads);
  struct timespec t0, t1;
  clock_gettime(CLOCK_MONOTONIC, &t0);
  for (int t = 0; t < nthreads; ++t) {
    job_t j = {t, nthreads, n, pat, pat_off, plen, txt, txt_off, tlen, metric, match, mismatch, gap_open, gap_ext,
               o2, e2, score_only, ops, ops_off, scores, status, ops_len};
    jobs[t] = j;
    pthread_create(&th[t], NULL, batch_worker, &jobs[t]);
  }
  for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
  clock_gettime(CLOCK_MONOTONIC, &t1);
  free(th); free(jobs);
  return (double)(t1.tv_sec - t0.tv_sec) + 1e-9 * (double)(t1.tv_nsec - t0.tv_nsec);
}

double orc_wfa_align_batch(int metric, int n, const char* pat, const int64_t* pat_off, const int* plen,
                           const char* txt, const int64_t* txt_off, const int* tlen,
                           int match, int mismatch, int gap_open, int gap_ext, int score_only,
                           char* ops, const int64_t* ops_off,
                           int* scores, int* status, int* ops_len, int nthreads) {
  const int pen[6] = {match, mismatch, gap_open, gap_ext, 0, 1};
  return orc_wfa_align_batch_pen(metric, n, pat, pat_off, plen, txt, txt_off, tlen, pen, score_only, ops, ops_off,
                                 scores, status, ops_len, nthreads);
}

double orc_biwfa_align_batch(int n, const char* pat, const int64_t* pat_off, const int* plen,
                             const char* txt, const int64_t* txt_off, const int* tlen,
                             int match, int mismatch, int gap_open, int gap_ext, int score_only,
                             char* ops, const int64_t* ops_off,
                             int* scores, int* status, int* ops_len, int nthreads) {
  return orc_wfa_align_batch(ORC_METRIC_AFFINE, n, pat, pat_off, plen, txt, txt_off, tlen, match, mismatch, gap_open,
                             gap_ext, score_only, ops, ops_off, scores, status, ops_len, nthreads);
}

/* ---------------------------------------------------------------- whole-batch comparison */
/* Compares each pair's operations ops[ops_off[i] .. ops_off[i] + ops_len[i]) (M/X/I/D bytes, as
 * the batch functions above write them) with a run-length list runs[run_off[i] .. run_off[i] +
 * run_len[i]) of uint32 (len << 4 | SAM op: 7 '=' -> M, 8 X, 1 I, 2 D; the GPU's output form).
 * bad[i] = 1 where they differ. Returns the number of differing pairs. */
int64_t orc_compare_runs(int n, const char* ops, const int64_t* ops_off, const int* ops_len, const uint32_t* runs,
                         const int64_t* run_off, const int* run_len, uint8_t* bad) {
  int64_t nbad = 0;
  for (int i = 0; i < n; ++i) {
    const char* o = ops + ops_off[i];
    const int len = ops_len[i];
    int pos = 0, ok = 1;
    for (int r = 0; r < run_len[i] && ok; ++r) {
      const uint32_t v = runs[run_off[i] + r];
      const int op = (int)(v & 15u), rl = (int)(v >> 4);
      const char ch = op == 7 ? 'M' : op == 8 ? 'X' : op == 1 ? 'I' : op == 2 ? 'D' : '?';
      if (ch == '?' || rl <= 0 || pos + rl > len) { ok = 0; break; }
      for (int k = 0; k < rl; ++k)
        if (o[pos + k] != ch) { ok = 0; break; }
      pos += rl;
    }
    if (pos != len) ok = 0;
    bad[i] = (uint8_t)(ok ? 0 : 1);
    nbad += ok ? 0 : 1;
  }
  return nbad;
}
