/*
 * C++ aligner classes over the C ABI of libbiwfa_gb300.so (wfa_gpu.h), with the names,
 * signatures and error behaviour of WFA2-lib's C++ binding (WFA2-lib/bindings/cpp/
 * WFAligner.hpp:48-262, WFAligner.cpp), so that code written against wfa::WFAligner
 * compiles and runs unchanged for the configuration this library computes on the GPU:
 *
 *   wfa::WFAlignerGapAffine aligner(4, 6, 2, wfa::WFAligner::Alignment,
 *                                   wfa::WFAligner::MemoryUltralow);
 *   aligner.alignEnd2End(pattern, text);
 *   int score = aligner.getAlignmentScore();          // e.g. -8
 *   std::string cigar = aligner.getCIGAR(true);        // e.g. "14=1I86="
 *
 * Header-only; link with -lbiwfa_gb300. Configurations the GPU aligner does not compute
 * (memory models other than MemoryUltralow, heuristics, ends-free and extension forms,
 * the two-piece affine distance, 2-bit packed or lambda sequences) return
 * StatusUnsupported (WF_STATUS_UNSUPPORTED) from the align call instead of computing
 * something different. Like WFA2-lib's, the class is not copyable and not thread-safe:
 * use one aligner per thread. alignEnd2EndBatch() is this library's addition: many pairs
 * in one GPU launch.
 */
#ifndef WFA_GPU_WFALIGNER_HPP_
#define WFA_GPU_WFALIGNER_HPP_

#include <algorithm>
#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

#include "wfa_gpu.h"

namespace wfa {

class WFAligner {
 public:
  enum MemoryModel { MemoryHigh, MemoryMed, MemoryLow, MemoryUltralow };
  enum AlignmentScope { Score, Alignment };
  enum AlignmentStatus {
    StatusAlgCompleted = WF_STATUS_ALG_COMPLETED,
    StatusAlgPartial = WF_STATUS_ALG_PARTIAL,
    StatusMaxStepsReached = WF_STATUS_MAX_STEPS_REACHED,
    StatusOOM = WF_STATUS_OOM,
    StatusUnattainable = WF_STATUS_UNATTAINABLE,
    StatusUnsupported = WF_STATUS_UNSUPPORTED,
    StatusDeviceError = WF_STATUS_DEVICE_ERROR,
  };

  // ---- end-to-end (WFAligner.cpp alignEnd2End)
  AlignmentStatus alignEnd2End(const char* const pattern, const int patternLength, const char* const text,
                               const int textLength) {
    if (unsupported_) return unsupported();
    wavefront_aligner_set_alignment_end_to_end(wfAligner);
    return (AlignmentStatus)wavefront_align(wfAligner, pattern, patternLength, text, textLength);
  }
  AlignmentStatus alignEnd2End(const std::string& pattern, const std::string& text) {
    return alignEnd2End(pattern.c_str(), (int)pattern.length(), text.c_str(), (int)text.length());
  }
  AlignmentStatus alignEnd2End(const uint8_t* const, const int, const uint8_t* const, const int) {
    return unsupported();  // 2-bit packed input (wavefront_align_packed2bits)
  }
  AlignmentStatus alignEnd2End(int (*)(int, int, void*), void*, const int, const int) {
    return unsupported();  // custom match function (wavefront_align_lambda)
  }
  // Many pairs in one GPU batch; per-pair statuses/scores in the output vectors. The CIGAR
  // of pair i is then available through getBatchCIGAR(i).
  AlignmentStatus alignEnd2EndBatch(const std::vector<std::string>& patterns, const std::vector<std::string>& texts,
                                    std::vector<int>* scores, std::vector<int>* statuses) {
    if (unsupported_) return unsupported();
    const int n = (int)std::min(patterns.size(), texts.size());
    std::vector<const char*> ps((size_t)n), ts((size_t)n);
    std::vector<int> pl((size_t)n), tl((size_t)n);
    for (int i = 0; i < n; ++i) {
      ps[(size_t)i] = patterns[(size_t)i].c_str(); pl[(size_t)i] = (int)patterns[(size_t)i].length();
      ts[(size_t)i] = texts[(size_t)i].c_str(); tl[(size_t)i] = (int)texts[(size_t)i].length();
    }
    scores->assign((size_t)n, 0);
    statuses->assign((size_t)n, 0);
    return (AlignmentStatus)wavefront_align_batch(wfAligner, n, ps.data(), pl.data(), ts.data(), tl.data(),
                                                  scores->data(), statuses->data());
  }
  std::string getBatchCIGAR(const int pair) {
    const uint32_t* runs = nullptr;
    int nruns = 0;
    if (wavefront_batch_cigar(wfAligner, pair, &runs, &nruns) != WF_STATUS_ALG_COMPLETED) return std::string();
    return sam_string(runs, nruns);
  }

  // ---- ends-free and extension: not computed by BiWFA (WFA2-lib exits on this misuse)
  AlignmentStatus alignEndsFree(const char* const, const int, const int, const int, const char* const, const int,
                                const int, const int) {
    return unsupported();
  }
  AlignmentStatus alignEndsFree(const std::string&, const int, const int, const std::string&, const int, const int) {
    return unsupported();
  }
  AlignmentStatus alignEndsFree(const uint8_t* const, const int, const int, const int, const uint8_t* const,
                                const int, const int, const int) {
    return unsupported();
  }
  AlignmentStatus alignEndsFree(int (*)(int, int, void*), void*, const int, const int, const int, const int,
                                const int, const int) {
    return unsupported();
  }
  AlignmentStatus alignExtension(const char* const, const int, const char* const, const int) { return unsupported(); }
  AlignmentStatus alignExtension(std::string&, std::string&) { return unsupported(); }
  AlignmentStatus alignExtension(const uint8_t* const, const int, const uint8_t* const, const int) {
    return unsupported();
  }
  AlignmentStatus alignExtension(int (*)(int, int, void*), void*, const int, const int) { return unsupported(); }

  // ---- heuristics: only none is computed exactly; any other marks the aligner unsupported
  void setHeuristicNone() {
    wavefront_aligner_set_heuristic_none(wfAligner);
    attributes.heuristic.strategy = wf_heuristic_none;
    heuristic_unsupported_ = false;
    refresh();
  }
  void setHeuristicBandedStatic(const int, const int) { heuristic_unsupported_ = true; refresh(); }
  void setHeuristicBandedAdaptive(const int, const int, const int = 1) { heuristic_unsupported_ = true; refresh(); }
  void setHeuristicWFadaptive(const int, const int, const int = 1) { heuristic_unsupported_ = true; refresh(); }
  void setHeuristicWFmash(const int, const int, const int = 1) { heuristic_unsupported_ = true; refresh(); }
  void setHeuristicXDrop(const int, const int = 1) { heuristic_unsupported_ = true; refresh(); }
  void setHeuristicZDrop(const int, const int = 1) { heuristic_unsupported_ = true; refresh(); }

  // ---- limits
  void setMaxAlignmentSteps(const int maxAlignmentSteps) {
    wavefront_aligner_set_max_alignment_steps(wfAligner, maxAlignmentSteps);
  }
  void setMaxMemory(const uint64_t, const uint64_t) {}  // scratch is sized per batch on the device
  void setMaxNumThreads(const int) {}                   // one GPU per aligner

  // ---- accessors (WFAligner.cpp:282-320)
  int getAlignmentStatus() { return wfAligner->align_status.status; }
  int getAlignmentScore() { return wfAligner->cigar->score; }
  void getAlignment(char** const cigarOperations, int* cigarLength) {
    *cigarOperations = wfAligner->cigar->operations + wfAligner->cigar->begin_offset;
    *cigarLength = wfAligner->cigar->end_offset - wfAligner->cigar->begin_offset;
  }
  std::string getAlignment() {
    const int len = wfAligner->cigar->end_offset - wfAligner->cigar->begin_offset;
    if (len <= 0) return std::string();
    return std::string(wfAligner->cigar->operations + wfAligner->cigar->begin_offset, (size_t)len);
  }
  void getCIGAR(const bool showMismatches, uint32_t** const cigarOperations, int* const numCigarOperations) {
    cigar_get_CIGAR(wfAligner->cigar, showMismatches, cigarOperations, numCigarOperations);
  }
  // SAM CIGAR text (cigar_sprint_SAM_CIGAR, alignment/cigar.c:755-779): "=" / "X" when
  // showMismatches, "M" for both otherwise.
  std::string getCIGAR(const bool showMismatches) {
    if (wfAligner->cigar->end_offset - wfAligner->cigar->begin_offset <= 0) return std::string();
    uint32_t* ops = nullptr;
    int n = 0;
    cigar_get_CIGAR(wfAligner->cigar, showMismatches, &ops, &n);
    return sam_string(ops, n);
  }

  // ---- display / misc
  void printPretty(FILE* const stream, const char* const, const int, const char* const, const int) {
    const std::string ops = getAlignment();
    fprintf(stream, "%s\n", ops.c_str());
  }
  char* strStatus(const AlignmentStatus status) { return wavefront_align_strerror((int)status); }
  void debugTag(char* const) {}

 protected:
  wavefront_aligner_attr_t attributes;
  wavefront_aligner_t* wfAligner = nullptr;

  WFAligner(const AlignmentScope alignmentScope, const MemoryModel memoryModel = MemoryHigh) {
    attributes = wavefront_aligner_attr_default;
    switch (memoryModel) {
      case MemoryMed: attributes.memory_mode = wavefront_memory_med; break;
      case MemoryLow: attributes.memory_mode = wavefront_memory_low; break;
      case MemoryUltralow: attributes.memory_mode = wavefront_memory_ultralow; break;
      default: attributes.memory_mode = wavefront_memory_high; break;
    }
    attributes.alignment_scope = (alignmentScope == Score) ? compute_score : compute_alignment;
  }
  ~WFAligner() { wavefront_aligner_delete(wfAligner); }
  // Called by the derived constructors once the distance and penalties are set.
  void create() {
    wfAligner = wavefront_aligner_new(&attributes);
    heuristic_unsupported_ = attributes.heuristic.strategy != wf_heuristic_none;  // the default is wf-adaptive
    refresh();
  }

 private:
  bool unsupported_ = false;            // the attributes name something the GPU aligner does not compute
  bool heuristic_unsupported_ = false;  // a heuristic other than none was requested

  void refresh() {
    unsupported_ = heuristic_unsupported_ || attributes.memory_mode != wavefront_memory_ultralow;
  }
  AlignmentStatus unsupported() {
    if (wfAligner) {
      wfAligner->align_status.status = WF_STATUS_UNSUPPORTED;
      wfAligner->cigar->begin_offset = wfAligner->cigar->end_offset = 0;
    }
    return StatusUnsupported;
  }
  static std::string sam_string(const uint32_t* runs, int n) {
    static const char kOps[] = "MIDN---=X";
    std::string s;
    char buf[24];
    for (int i = 0; i < n; ++i) {
      const uint32_t op = runs[i] & 0xfu;
      snprintf(buf, sizeof(buf), "%u%c", runs[i] >> 4, op <= 8 ? kOps[op] : '?');
      s += buf;
    }
    return s;
  }
  WFAligner(const WFAligner&) = delete;
  WFAligner& operator=(const WFAligner&) = delete;
};

// The other distances keep WFA2-lib's class names; all of them (indel, edit, gap-linear,
// gap-affine, two-piece gap-affine) run on the GPU.
class WFAlignerIndel : public WFAligner {
 public:
  WFAlignerIndel(const AlignmentScope alignmentScope, const MemoryModel memoryModel = MemoryHigh)
      : WFAligner(alignmentScope, memoryModel) {
    attributes.distance_metric = indel;
    create();
  }
};

class WFAlignerEdit : public WFAligner {
 public:
  WFAlignerEdit(const AlignmentScope alignmentScope, const MemoryModel memoryModel = MemoryHigh)
      : WFAligner(alignmentScope, memoryModel) {
    attributes.distance_metric = edit;
    create();
  }
};

class WFAlignerGapLinear : public WFAligner {
 public:
  WFAlignerGapLinear(const int mismatch, const int indel, const AlignmentScope alignmentScope,
                     const MemoryModel memoryModel = MemoryHigh)
      : WFAlignerGapLinear(0, mismatch, indel, alignmentScope, memoryModel) {}
  WFAlignerGapLinear(const int match, const int mismatch, const int indel, const AlignmentScope alignmentScope,
                     const MemoryModel memoryModel = MemoryHigh)
      : WFAligner(alignmentScope, memoryModel) {
    attributes.distance_metric = gap_linear;
    attributes.linear_penalties.match = match;
    attributes.linear_penalties.mismatch = mismatch;
    attributes.linear_penalties.indel = indel;
    create();
  }
};

class WFAlignerGapAffine : public WFAligner {
 public:
  WFAlignerGapAffine(const int mismatch, const int gapOpening, const int gapExtension,
                     const AlignmentScope alignmentScope, const MemoryModel memoryModel = MemoryHigh)
      : WFAlignerGapAffine(0, mismatch, gapOpening, gapExtension, alignmentScope, memoryModel) {}
  WFAlignerGapAffine(const int match, const int mismatch, const int gapOpening, const int gapExtension,
                     const AlignmentScope alignmentScope, const MemoryModel memoryModel = MemoryHigh)
      : WFAligner(alignmentScope, memoryModel) {
    attributes.distance_metric = gap_affine;
    attributes.affine_penalties.match = match;
    attributes.affine_penalties.mismatch = mismatch;
    attributes.affine_penalties.gap_opening = gapOpening;
    attributes.affine_penalties.gap_extension = gapExtension;
    create();
  }
};

class WFAlignerGapAffine2Pieces : public WFAligner {
 public:
  WFAlignerGapAffine2Pieces(const int mismatch, const int gapOpening1, const int gapExtension1,
                            const int gapOpening2, const int gapExtension2, const AlignmentScope alignmentScope,
                            const MemoryModel memoryModel = MemoryHigh)
      : WFAlignerGapAffine2Pieces(0, mismatch, gapOpening1, gapExtension1, gapOpening2, gapExtension2,
                                  alignmentScope, memoryModel) {}
  WFAlignerGapAffine2Pieces(const int match, const int mismatch, const int gapOpening1, const int gapExtension1,
                            const int gapOpening2, const int gapExtension2, const AlignmentScope alignmentScope,
                            const MemoryModel memoryModel = MemoryHigh)
      : WFAligner(alignmentScope, memoryModel) {
    attributes.distance_metric = gap_affine_2p;
    attributes.affine2p_penalties.match = match;
    attributes.affine2p_penalties.mismatch = mismatch;
    attributes.affine2p_penalties.gap_opening1 = gapOpening1;
    attributes.affine2p_penalties.gap_extension1 = gapExtension1;
    attributes.affine2p_penalties.gap_opening2 = gapOpening2;
    attributes.affine2p_penalties.gap_extension2 = gapExtension2;
    create();
  }
};

}  // namespace wfa

#endif  // WFA_GPU_WFALIGNER_HPP_
