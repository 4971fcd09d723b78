// Reads "pattern<TAB>text" lines from stdin, aligns each pair with wfa::WFAlignerGapAffine
// (match 0, mismatch 4, gap-open 6, gap-extend 2, MemoryUltralow) and prints
// "status<TAB>score<TAB>SAM-CIGAR<TAB>ops" per pair, then the same pairs through one
// alignEnd2EndBatch call as "batch<TAB>status<TAB>score<TAB>SAM-CIGAR". With --config-only
// it reports what the unsupported configurations return, which needs no GPU.
#include <iostream>
#include <string>
#include <vector>

#include "WFAligner.hpp"

int main(int argc, char** argv) {
  using wfa::WFAligner;
  if (argc > 1 && std::string(argv[1]) == "--config-only") {
    wfa::WFAlignerGapAffine high(4, 6, 2, WFAligner::Alignment);  // default MemoryHigh
    wfa::WFAlignerGapAffine2Pieces affine2p(4, 6, 2, 24, 1, WFAligner::Alignment);  // default MemoryHigh
    wfa::WFAlignerGapAffine dflt(4, 6, 2, WFAligner::Alignment, WFAligner::MemoryUltralow);
    wfa::WFAlignerGapAffine ul(4, 6, 2, WFAligner::Alignment, WFAligner::MemoryUltralow);
    ul.setHeuristicNone();
    std::cout << "default_heuristic\t" << dflt.alignEnd2End("ACGT", "ACGA") << "\n";
    std::cout << "no_device\t" << ul.alignEnd2End("", "") << "\n";
    ul.setHeuristicWFadaptive(10, 50);
    std::cout << "high\t" << high.alignEnd2End("ACGT", "ACGA") << "\n";
    std::cout << "affine2p\t" << affine2p.alignEnd2End("ACGT", "ACGA") << "\n";
    std::cout << "heuristic\t" << ul.alignEnd2End("ACGT", "ACGA") << "\n";
    std::cout << "endsfree\t" << ul.alignEndsFree("ACGT", 0, 0, "ACGA", 0, 0) << "\n";
    std::cout << "status_text\t" << ul.strStatus(WFAligner::StatusUnsupported) << "\n";
    std::cout << "cigar_after_refusal\t[" << ul.getCIGAR(true) << "]\n";
    return 0;
  }
  // --affine2p: the two-piece distance (0,4,6,2,24,1); otherwise gap-affine (0,4,6,2)
  const bool two = argc > 1 && std::string(argv[1]) == "--affine2p";
  wfa::WFAlignerGapAffine affine(4, 6, 2, WFAligner::Alignment, WFAligner::MemoryUltralow);
  wfa::WFAlignerGapAffine2Pieces affine2p(4, 6, 2, 24, 1, WFAligner::Alignment, WFAligner::MemoryUltralow);
  WFAligner& aligner = two ? static_cast<WFAligner&>(affine2p) : static_cast<WFAligner&>(affine);
  aligner.setHeuristicNone();  // WFA2-lib's default attributes carry the wf-adaptive heuristic
  std::vector<std::string> ps, ts;
  std::string line;
  while (std::getline(std::cin, line)) {
    const size_t tab = line.find('\t');
    if (tab == std::string::npos) continue;
    ps.push_back(line.substr(0, tab));
    ts.push_back(line.substr(tab + 1));
  }
  for (size_t i = 0; i < ps.size(); ++i) {
    const int st = aligner.alignEnd2End(ps[i], ts[i]);
    std::cout << st << "\t" << aligner.getAlignmentScore() << "\t" << aligner.getCIGAR(true) << "\t"
              << aligner.getAlignment() << "\n";
  }
  std::vector<int> scores, statuses;
  const int st = aligner.alignEnd2EndBatch(ps, ts, &scores, &statuses);
  for (size_t i = 0; i < ps.size(); ++i)
    std::cout << "batch\t" << (st == 0 ? statuses[i] : st) << "\t" << scores[i] << "\t"
              << aligner.getBatchCIGAR((int)i) << "\n";
  return 0;
}
