// WFA2-lib compatible aligner API (include/wfa_gpu.h, first surface) on top of the
// wfg_* batch runtime. Every alignment runs on the GPU; there is no CPU alignment path.
#include <algorithm>
#include <climits>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wfa_gpu.h"

namespace {

struct AlignerImpl {
  wfg_context_t* ctx = nullptr;
  wavefront_aligner_attr_t attr;
  int unsupported = 0;
  std::string reason;
  // last batch
  int n = 0;
  std::vector<int64_t> run_off;
  std::vector<int> run_len;
  std::vector<uint32_t> runs;
  // single-pair result buffers behind wf_aligner->cigar
  std::vector<char> ops;
  std::vector<uint32_t> sam;
  // staging
  std::vector<char> seq;
  std::vector<int64_t> p_off, t_off;
  std::vector<int> plen, tlen, scores, statuses;
};

AlignerImpl* impl_of(wavefront_aligner_t* wf) { return static_cast<AlignerImpl*>(wf->bialigner); }

void check_config(AlignerImpl* im) {
  const wavefront_aligner_attr_t& a = im->attr;
  const affine_penalties_t& p = a.affine_penalties;
  im->unsupported = 1;
  if (a.distance_metric != gap_affine && a.distance_metric != edit && a.distance_metric != indel &&
      a.distance_metric != gap_linear && a.distance_metric != gap_affine_2p) {
    im->reason = "unknown distance metric"; return;
  }
  const affine2p_penalties_t& q = a.affine2p_penalties;
  if (a.distance_metric == gap_affine_2p &&
      (q.match > 0 || q.mismatch <= 0 || q.gap_opening1 < 0 || q.gap_extension1 <= 0 || q.gap_opening2 < 0 ||
       q.gap_extension2 <= 0)) {
    im->reason = "two-piece penalties must satisfy match <= 0, mismatch > 0, o1 >= 0, e1 > 0, o2 >= 0, e2 > 0";
    return;
  }
  if (a.distance_metric == gap_linear && (a.linear_penalties.match > 0 || a.linear_penalties.mismatch <= 0 ||
                                          a.linear_penalties.indel <= 0)) {
    im->reason = "gap-linear penalties must satisfy match <= 0, mismatch > 0, indel > 0"; return;
  }
  if (a.memory_mode != wavefront_memory_ultralow) {
    im->reason = "only wavefront_memory_ultralow (BiWFA) is supported"; return;
  }
  if (a.heuristic.strategy != wf_heuristic_none) { im->reason = "heuristics are not supported (use wf_heuristic_none)"; return; }
  if (a.alignment_form.span != alignment_end2end || a.alignment_form.extension ||
      a.alignment_form.pattern_begin_free || a.alignment_form.pattern_end_free ||
      a.alignment_form.text_begin_free || a.alignment_form.text_end_free) {
    im->reason = "BiWFA supports end-to-end alignment only"; return;
  }
  if (a.distance_metric == gap_affine && (p.match > 0 || p.mismatch <= 0 || p.gap_opening < 0 || p.gap_extension <= 0)) {
    im->reason = "penalties must satisfy match <= 0, mismatch > 0, gap_opening >= 0, gap_extension > 0"; return;
  }
  im->unsupported = 0;
  im->reason.clear();
}

wfg_config_t config_of(const AlignerImpl* im) {
  wfg_config_t c{};
  c.match = im->attr.affine_penalties.match;
  c.mismatch = im->attr.affine_penalties.mismatch;
  c.gap_opening = im->attr.affine_penalties.gap_opening;
  c.gap_extension = im->attr.affine_penalties.gap_extension;
  c.score_only = im->attr.alignment_scope == compute_score;
  c.max_alignment_steps = im->attr.system.max_alignment_steps;
  c.metric = (im->attr.distance_metric == edit) ? WFG_METRIC_EDIT
           : (im->attr.distance_metric == indel) ? WFG_METRIC_INDEL
           : (im->attr.distance_metric == gap_linear) ? WFG_METRIC_GAP_LINEAR
           : (im->attr.distance_metric == gap_affine_2p) ? WFG_METRIC_GAP_AFFINE_2P : WFG_METRIC_GAP_AFFINE;
  if (c.metric == WFG_METRIC_GAP_LINEAR) {
    c.match = im->attr.linear_penalties.match;
    c.mismatch = im->attr.linear_penalties.mismatch;
    c.gap_opening = im->attr.linear_penalties.indel;
    c.gap_extension = 0;
  }
  if (c.metric == WFG_METRIC_GAP_AFFINE_2P) {
    const affine2p_penalties_t& q = im->attr.affine2p_penalties;
    c.match = q.match; c.mismatch = q.mismatch;
    c.gap_opening = q.gap_opening1; c.gap_extension = q.gap_extension1;
    c.gap_opening2 = q.gap_opening2; c.gap_extension2 = q.gap_extension2;
  }
  return c;
}

char op_char(uint32_t op) {
  switch (op) {
    case 7: return 'M';
    case 8: return 'X';
    case 1: return 'I';
    default: return 'D';
  }
}

}  // namespace

extern "C" {

// Defaults of WFA2-lib (wavefront/wavefront_attributes.c:38-100).
wavefront_aligner_attr_t wavefront_aligner_attr_default = {
    gap_affine,
    compute_alignment,
    {alignment_end2end, false, 0, 0, 0, 0},
    {0, 4, 2},
    {0, 4, 6, 2},
    {0, 4, 6, 2, 24, 1},
    {wf_heuristic_wfadaptive, 1, 0, 0, 10, 50, 0, 0, 0, 0, 0, 0, 0},
    wavefront_memory_high,
    NULL,
    {false, 2000, 0},
    {INT_MAX, 3000, 6000, 0, (uint64_t)-1, (uint64_t)-1, UINT64_MAX, 0, false, {}, 1, 500},
};

// The GPU context is created by the first alignment (device WFG_DEVICE, default 0), so an
// aligner exists, and reports its configuration errors, on a machine without a GPU.
wavefront_aligner_t* wavefront_aligner_new(wavefront_aligner_attr_t* attributes) {
  if (attributes == NULL) attributes = &wavefront_aligner_attr_default;
  AlignerImpl* im = new AlignerImpl();
  im->attr = *attributes;
  check_config(im);
  wavefront_aligner_t* wf = (wavefront_aligner_t*)calloc(1, sizeof(wavefront_aligner_t));
  wf->bialigner = im;
  wf->align_mode = attributes->memory_mode == wavefront_memory_ultralow ? 1 : 0;  // wf_align_biwfa / _regular
  wf->alignment_scope = attributes->alignment_scope;
  wf->alignment_form = attributes->alignment_form;
  wf->heuristic = attributes->heuristic;
  wf->memory_mode = attributes->memory_mode;
  wf->mm_allocator = attributes->mm_allocator;
  wf->system = attributes->system;
  wf->cigar = (cigar_t*)calloc(1, sizeof(cigar_t));
  wf->cigar->score = INT32_MIN;
  wf->cigar->end_v = wf->cigar->end_h = -1;
  wf->align_status.status = WF_STATUS_OK;
  return wf;
}

void wavefront_aligner_delete(wavefront_aligner_t* const wf) {
  if (!wf) return;
  AlignerImpl* im = impl_of(wf);
  if (im->ctx) wfg_context_destroy(im->ctx);
  delete im;
  free(wf->cigar);
  free(wf);
}

void wavefront_aligner_set_alignment_end_to_end(wavefront_aligner_t* const wf) {
  AlignerImpl* im = impl_of(wf);
  im->attr.alignment_form.span = alignment_end2end;
  im->attr.alignment_form.extension = false;
  wf->alignment_form = im->attr.alignment_form;
  check_config(im);
}

void wavefront_aligner_set_heuristic_none(wavefront_aligner_t* const wf) {
  AlignerImpl* im = impl_of(wf);
  im->attr.heuristic.strategy = wf_heuristic_none;
  check_config(im);
}

void wavefront_aligner_set_max_alignment_steps(wavefront_aligner_t* const wf, const int max_alignment_steps) {
  impl_of(wf)->attr.system.max_alignment_steps = max_alignment_steps;
}

int wavefront_align_batch(wavefront_aligner_t* const wf, const int n, const char* const* patterns,
                          const int* plens, const char* const* texts, const int* tlens, int* scores, int* statuses) {
  AlignerImpl* im = impl_of(wf);
  if (im->unsupported) {
    fprintf(stderr, "[WFA-GB300] %s\n", im->reason.c_str());
    for (int i = 0; i < n; ++i) { if (scores) scores[i] = 0; if (statuses) statuses[i] = WF_STATUS_UNSUPPORTED; }
    wf->align_status.status = WF_STATUS_UNSUPPORTED;
    return WF_STATUS_UNSUPPORTED;
  }
  if (im->ctx == NULL) {
    const char* dev = getenv("WFG_DEVICE");
    im->ctx = wfg_context_create(dev ? atoi(dev) : 0);
    if (im->ctx == NULL) {
      fprintf(stderr, "[WFA-GB300] no usable CUDA device\n");
      for (int i = 0; i < n; ++i) { if (scores) scores[i] = 0; if (statuses) statuses[i] = WF_STATUS_DEVICE_ERROR; }
      wf->align_status.status = WF_STATUS_DEVICE_ERROR;
      return WF_STATUS_DEVICE_ERROR;
    }
  }
  int64_t total = 0;
  for (int i = 0; i < n; ++i) total += (int64_t)plens[i] + tlens[i];
  im->seq.resize((size_t)std::max<int64_t>(total, 1));
  im->p_off.resize(n); im->t_off.resize(n); im->plen.assign(plens, plens + n); im->tlen.assign(tlens, tlens + n);
  int64_t cur = 0;
  for (int i = 0; i < n; ++i) {
    im->p_off[i] = cur; memcpy(im->seq.data() + cur, patterns[i], (size_t)plens[i]); cur += plens[i];
    im->t_off[i] = cur; memcpy(im->seq.data() + cur, texts[i], (size_t)tlens[i]); cur += tlens[i];
  }
  im->n = n;
  im->scores.resize(n); im->statuses.resize(n); im->run_off.resize(n); im->run_len.resize(n);
  im->runs.resize((size_t)std::max<int64_t>(total + n, 1));
  const wfg_config_t cfg = config_of(im);
  int64_t nruns = 0;
  const int st = wfg_align_host(im->ctx, &cfg, WFG_SCHED_SORTED, n, im->seq.data(), total, im->p_off.data(),
                                im->plen.data(), im->t_off.data(), im->tlen.data(), im->scores.data(),
                                im->statuses.data(), im->run_off.data(), im->run_len.data(), im->runs.data(),
                                (int64_t)im->runs.size(), &nruns);
  if (st != WF_STATUS_ALG_COMPLETED) {
    fprintf(stderr, "[WFA-GB300] %s\n", wfg_last_error(im->ctx));
    wf->align_status.status = st;
    return st;
  }
  for (int i = 0; i < n; ++i) {
    if (scores) scores[i] = im->scores[i];
    if (statuses) statuses[i] = im->statuses[i];
  }
  wf->align_status.status = WF_STATUS_ALG_COMPLETED;
  return WF_STATUS_ALG_COMPLETED;
}

int wavefront_batch_cigar(wavefront_aligner_t* const wf, const int pair, const uint32_t** runs, int* num_runs) {
  AlignerImpl* im = impl_of(wf);
  if (pair < 0 || pair >= im->n) return WF_STATUS_UNSUPPORTED;
  *runs = im->runs.data() + im->run_off[pair];
  *num_runs = im->run_len[pair];
  return im->statuses[pair];
}

int wavefront_align(wavefront_aligner_t* const wf, const char* const pattern, const int plen,
                    const char* const text, const int tlen) {
  AlignerImpl* im = impl_of(wf);
  cigar_t* cg = wf->cigar;
  cg->begin_offset = cg->end_offset = 0;
  cg->score = INT32_MIN;
  cg->end_v = cg->end_h = -1;
  cg->cigar_length = 0;
  const char* ps[1] = {pattern};
  const char* ts[1] = {text};
  int score = 0, status = 0;
  const int st = wavefront_align_batch(wf, 1, ps, &plen, ts, &tlen, &score, &status);
  if (st != WF_STATUS_ALG_COMPLETED) return st;
  wf->align_status.status = status;
  wf->align_status.score = score;
  if (status != WF_STATUS_ALG_COMPLETED) return status;
  // Expand the runs into WFA2-lib's operation string.
  int64_t nops = 0;
  for (int r = 0; r < im->run_len[0]; ++r) nops += im->runs[(size_t)(im->run_off[0] + r)] >> 4;
  im->ops.resize((size_t)nops + 1);
  int64_t pos = 0;
  for (int r = 0; r < im->run_len[0]; ++r) {
    const uint32_t run = im->runs[(size_t)(im->run_off[0] + r)];
    memset(im->ops.data() + pos, op_char(run & 15u), run >> 4);
    pos += run >> 4;
  }
  im->ops[(size_t)nops] = '\0';
  cg->operations = im->ops.data();
  cg->max_operations = (int)nops + 1;
  cg->begin_offset = 0;
  cg->end_offset = (int)nops;
  cg->score = score;
  cg->end_v = plen;
  cg->end_h = tlen;
  return status;
}

char* wavefront_align_strerror(const int code) {
  switch (code) {
    case WF_STATUS_ALG_COMPLETED: return (char*)"[WFA] Alignment completed successfully";
    case WF_STATUS_ALG_PARTIAL: return (char*)"[WFA] Alignment extension computed (partial alignment)";
    case WF_STATUS_MAX_STEPS_REACHED: return (char*)"[WFA] Alignment failed. Maximum WFA-steps limit reached";
    case WF_STATUS_OOM: return (char*)"[WFA] Alignment failed. Maximum memory limit reached";
    case WF_STATUS_UNATTAINABLE: return (char*)"[WFA] Alignment failed. Unattainable under configured heuristics";
    case WF_STATUS_END_REACHED: return (char*)"[WFA] Alignment end reached";
    case WF_STATUS_END_UNREACHABLE:
      return (char*)"[WFA] Alignment end unreachable under current configuration (due to heuristics like Z-drop)";
    case WF_STATUS_UNSUPPORTED: return (char*)"[WFA-GB300] Configuration not supported by the GPU BiWFA aligner";
    case WF_STATUS_DEVICE_ERROR: return (char*)"[WFA-GB300] CUDA device error";
    default: return (char*)"[WFA] Unknown error code";
  }
}

char* wavefront_align_strerror_short(const int code) {
  switch (code) {
    case WF_STATUS_ALG_COMPLETED: return (char*)"OK.Full";
    case WF_STATUS_ALG_PARTIAL: return (char*)"OK.Partial";
    case WF_STATUS_MAX_STEPS_REACHED: return (char*)"FAILED.MaxWFASteps";
    case WF_STATUS_OOM: return (char*)"FAILED.OOM";
    case WF_STATUS_UNATTAINABLE: return (char*)"FAILED.Unattainable";
    case WF_STATUS_END_REACHED: return (char*)"INTERNAL.Reached";
    case WF_STATUS_END_UNREACHABLE: return (char*)"INTERNAL.Dropped";
    case WF_STATUS_UNSUPPORTED: return (char*)"FAILED.Unsupported";
    case WF_STATUS_DEVICE_ERROR: return (char*)"FAILED.Device";
    default: return (char*)"Unknown";
  }
}

// cigar_sprint (alignment/cigar.c:706-740): run-length text over the operations.
int cigar_sprint(char* const buffer, const cigar_t* const cigar, const bool print_matches) {
  if (cigar->begin_offset >= cigar->end_offset) { buffer[0] = '\0'; return 0; }
  const char* ops = cigar->operations;
  char last = ops[cigar->begin_offset];
  int len = 1, cursor = 0;
  for (int i = cigar->begin_offset + 1; i < cigar->end_offset; ++i) {
    if (ops[i] == last) { ++len; continue; }
    if (print_matches || last != 'M') cursor += sprintf(buffer + cursor, "%d%c", len, last);
    last = ops[i];
    len = 1;
  }
  if (print_matches || last != 'M') cursor += sprintf(buffer + cursor, "%d%c", len, last);
  buffer[cursor] = '\0';
  return cursor;
}

// cigar_score_gap_affine (alignment/cigar.c:277-303)
int cigar_score_gap_affine(const cigar_t* const cigar, const affine_penalties_t* const pen) {
  char last = '\0';
  int score = 0;
  for (int i = cigar->begin_offset; i < cigar->end_offset; ++i) {
    const char op = cigar->operations[i];
    if (op == 'M') score -= pen->match;
    else if (op == 'X') score -= pen->mismatch;
    else if (op == 'D') score -= pen->gap_extension + (last == 'D' ? 0 : pen->gap_opening);
    else if (op == 'I') score -= pen->gap_extension + (last == 'I' ? 0 : pen->gap_opening);
    last = op;
  }
  return score;
}

// cigar_score_edit (alignment/cigar.c:244-259): every operation but a match counts one.
int cigar_score_edit(const cigar_t* const cigar) {
  int score = 0;
  for (int i = cigar->begin_offset; i < cigar->end_offset; ++i) score += cigar->operations[i] != 'M';
  return score;
}

// cigar_score_gap_linear (alignment/cigar.c:260-276)
int cigar_score_gap_linear(const cigar_t* const cigar, const linear_penalties_t* const pen) {
  int score = 0;
  for (int i = cigar->begin_offset; i < cigar->end_offset; ++i) {
    const char op = cigar->operations[i];
    score -= op == 'M' ? pen->match : op == 'X' ? pen->mismatch : pen->indel;
  }
  return score;
}

// cigar_score_gap_affine2p (alignment/cigar.c:304-342): each maximal run of one operation at
// once, a gap run at the cheaper of the two pieces. An empty CIGAR scores 0 here (WFA2-lib
// aborts on it).
int cigar_score_gap_affine2p(const cigar_t* const cigar, const affine2p_penalties_t* const pen) {
  int score = 0;
  int i = cigar->begin_offset;
  while (i < cigar->end_offset) {
    const char op = cigar->operations[i];
    int j = i;
    while (j < cigar->end_offset && cigar->operations[j] == op) ++j;
    const int len = j - i;
    if (op == 'M') score -= pen->match * len;
    else if (op == 'X') score -= pen->mismatch * len;
    else {
      const int a = pen->gap_opening1 + pen->gap_extension1 * len;
      const int b = pen->gap_opening2 + pen->gap_extension2 * len;
      score -= a < b ? a : b;
    }
    i = j;
  }
  return score;
}

// cigar_get_CIGAR / cigar_compute_CIGAR (alignment/cigar.c:181-235). The buffer is owned
// by the aligner that produced the cigar (valid until its next alignment).
void cigar_get_CIGAR(cigar_t* const cigar, const bool show_mismatches, uint32_t** const cigar_buffer,
                     int* const cigar_length) {
  static thread_local std::vector<uint32_t> tls;
  std::vector<uint32_t>& out = tls;
  out.clear();
  if (cigar->begin_offset < cigar->end_offset) {
    auto code = [&](char op) -> uint32_t {
      if (op == 'M') return show_mismatches ? 7u : 0u;
      if (op == 'X') return 8u;
      if (op == 'I') return 1u;
      if (op == 'D') return 2u;
      return 15u;
    };
    char last = cigar->operations[cigar->begin_offset];
    if (!show_mismatches && last == 'X') last = 'M';
    uint32_t len = 1;
    for (int i = cigar->begin_offset + 1; i < cigar->end_offset; ++i) {
      char op = cigar->operations[i];
      if (!show_mismatches && op == 'X') op = 'M';
      if (op == last) { ++len; continue; }
      out.push_back((len << 4) | code(last));
      last = op;
      len = 1;
    }
    out.push_back((len << 4) | code(last));
  }
  cigar->cigar_buffer = out.data();
  cigar->cigar_length = (int)out.size();
  cigar->has_misms = show_mismatches;
  *cigar_buffer = out.data();
  *cigar_length = (int)out.size();
}

}  // extern "C"
