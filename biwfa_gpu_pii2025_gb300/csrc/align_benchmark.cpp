// align_benchmark-compatible command-line front end of the GPU BiWFA aligner.
//
// Reads WFA2-lib's .seq input (a pattern line starting with '>' then a text line starting
// with '<', WFA2-lib/tools/align_benchmark/align_benchmark.c:313-340), aligns the pairs in
// GPU batches through the wfg_* C ABI and writes align_benchmark's output lines:
//   --output PATH       "score<TAB>CIGAR" (benchmark_utils.c:103-117; "-1<TAB>-" when the
//                       CIGAR is empty; score-only prints cigar->score and "-")
//   --output-full PATH  "plen<TAB>tlen<TAB>score<TAB>pattern<TAB>text<TAB>CIGAR" (:118-142)
// The score of a full alignment is the CIGAR rescored with the gap-affine penalties
// (cigar_score_gap_affine), with the two-piece penalties for gap-affine2p-wfa
// (cigar_score_gap_affine2p), with the linear penalties for gap-linear-wfa
// (cigar_score_gap_linear), or its number of edits for edit-wfa / indel-wfa
// (cigar_score_edit), as align_benchmark prints it. Options follow align_benchmark_params.c;
// configurations other than BiWFA without heuristics for those five distances are refused
// with exit status 1, as align_benchmark refuses bad options.
#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "../../include/wfa_gpu.h"

namespace {

struct Options {
  std::string algorithm = "gap-affine-wfa";
  std::string input, output;
  bool output_full = false;
  int match = 0, mismatch = 4, gap_opening = 6, gap_extension = 2;
  int lin_match = 0, lin_mismatch = 4, lin_indel = 2;  // --linear-penalties (align_benchmark defaults)
  int p2[6] = {0, 4, 6, 2, 24, 1};                     // --affine2p-penalties (align_benchmark defaults)
  bool score_only = false;
  std::string span = "global", memory = "ultralow", heuristic = "none";
  int max_steps = 0;
  int batch_size = 100000;
  int device = 0;
  bool quiet = false;
};

[[noreturn]] void usage_exit(const char* msg) {
  if (msg) fprintf(stderr, "%s\n", msg);
  fprintf(stderr,
          "USE: align_benchmark -i PATH [-o PATH | --output-full PATH] [options]\n"
          "      --algorithm|a gap-affine-wfa | gap-affine2p-wfa | gap-linear-wfa | edit-wfa | indel-wfa\n"
          "      --affine-penalties|g M,X,O,E          (default 0,4,6,2)\n"
          "      --affine2p-penalties M,X,O1,E1,O2,E2  (default 0,4,6,2,24,1)\n"
          "      --linear-penalties|p M,X,I             (default 0,4,2)\n"
          "      --wfa-score-only\n"
          "      --wfa-span global   --wfa-memory ultralow   --wfa-heuristic none\n"
          "      --wfa-max-steps INT\n"
          "      --batch-size INT                       (pairs per GPU batch, default 100000)\n"
          "      --device INT   --quiet|q   --help|h\n");
  exit(msg ? 1 : 0);
}

const char* need_value(int& i, int argc, char** argv) {
  if (i + 1 >= argc) usage_exit((std::string("option ") + argv[i] + " needs a value").c_str());
  return argv[++i];
}

Options parse(int argc, char** argv) {
  Options o;
  for (int i = 1; i < argc; ++i) {
    const std::string a = argv[i];
    if (a == "-a" || a == "--algorithm") o.algorithm = need_value(i, argc, argv);
    else if (a == "-i" || a == "--input") o.input = need_value(i, argc, argv);
    else if (a == "-o" || a == "--output") { o.output = need_value(i, argc, argv); o.output_full = false; }
    else if (a == "--output-full") { o.output = need_value(i, argc, argv); o.output_full = true; }
    else if (a == "-g" || a == "--affine-penalties") {
      const char* v = need_value(i, argc, argv);
      if (sscanf(v, "%d,%d,%d,%d", &o.match, &o.mismatch, &o.gap_opening, &o.gap_extension) != 4)
        usage_exit("--affine-penalties expects M,X,O,E");
    } else if (a == "--affine2p-penalties") {
      const char* v = need_value(i, argc, argv);
      if (sscanf(v, "%d,%d,%d,%d,%d,%d", &o.p2[0], &o.p2[1], &o.p2[2], &o.p2[3], &o.p2[4], &o.p2[5]) != 6)
        usage_exit("--affine2p-penalties expects M,X,O1,E1,O2,E2");
    } else if (a == "-p" || a == "--linear-penalties") {
      const char* v = need_value(i, argc, argv);
      if (sscanf(v, "%d,%d,%d", &o.lin_match, &o.lin_mismatch, &o.lin_indel) != 3)
        usage_exit("--linear-penalties expects M,X,I");
    } else if (a == "--wfa-score-only") o.score_only = true;
    else if (a == "--wfa-span") o.span = need_value(i, argc, argv);
    else if (a == "--wfa-memory") o.memory = need_value(i, argc, argv);
    else if (a == "--wfa-heuristic") o.heuristic = need_value(i, argc, argv);
    else if (a == "--wfa-max-steps") o.max_steps = atoi(need_value(i, argc, argv));
    else if (a == "--batch-size") o.batch_size = atoi(need_value(i, argc, argv));
    else if (a == "--device") o.device = atoi(need_value(i, argc, argv));
    else if (a == "-q" || a == "--quiet") o.quiet = true;
    else if (a == "-h" || a == "--help") usage_exit(nullptr);
    else usage_exit((std::string("unknown option ") + a).c_str());
  }
  if (o.algorithm != "gap-affine-wfa" && o.algorithm != "gap-affine2p-wfa" && o.algorithm != "gap-linear-wfa" &&
      o.algorithm != "edit-wfa" && o.algorithm != "indel-wfa")
    usage_exit("only --algorithm gap-affine-wfa, gap-affine2p-wfa, gap-linear-wfa, edit-wfa or indel-wfa runs on "
               "the GPU aligner");
  if (o.memory != "ultralow") usage_exit("only --wfa-memory ultralow (BiWFA) runs on the GPU aligner");
  if (o.heuristic != "none") usage_exit("only --wfa-heuristic none runs on the GPU aligner");
  if (o.span != "global") usage_exit("BiWFA aligns end-to-end only (--wfa-span global)");
  if (o.input.empty()) usage_exit("--input is required");
  if (o.batch_size <= 0) usage_exit("--batch-size must be positive");
  return o;
}

// One batch of pairs in one byte buffer.
struct Batch {
  std::vector<char> seq;
  std::vector<int64_t> p_off, t_off;
  std::vector<int> plen, tlen;
  void clear() { seq.clear(); p_off.clear(); t_off.clear(); plen.clear(); tlen.clear(); }
  int n() const { return (int)plen.size(); }
};

// Strip the record marker and the end of line as align_benchmark_read_input does.
void strip(std::string& s) {
  while (!s.empty() && (s.back() == '\n' || s.back() == '\r')) s.pop_back();
  if (!s.empty()) s.erase(0, 1);
}

bool read_line(FILE* f, std::string& out) {
  out.clear();
  char buf[1 << 16];
  while (fgets(buf, sizeof(buf), f)) {
    out += buf;
    if (!out.empty() && out.back() == '\n') return true;
  }
  return !out.empty();
}

void print_cigar(std::string& line, const uint32_t* runs, int n) {
  char tmp[24];
  for (int r = 0; r < n; ++r) {
    const uint32_t op = runs[r] & 15u;
    const char c = op == 7 ? 'M' : op == 8 ? 'X' : op == 1 ? 'I' : 'D';
    snprintf(tmp, sizeof(tmp), "%u%c", runs[r] >> 4, c);
    line += tmp;
  }
}

}  // namespace

int main(int argc, char** argv) {
  const Options opt = parse(argc, argv);
  FILE* in = fopen(opt.input.c_str(), "r");
  if (!in) { fprintf(stderr, "cannot open %s\n", opt.input.c_str()); return 1; }
  FILE* out = nullptr;
  if (!opt.output.empty()) {
    out = fopen(opt.output.c_str(), "w");
    if (!out) { fprintf(stderr, "cannot open %s\n", opt.output.c_str()); return 1; }
  }
  wfg_context_t* ctx = wfg_context_create(opt.device);
  if (!ctx) { fprintf(stderr, "no usable CUDA device %d\n", opt.device); return 1; }
  const int metric = opt.algorithm == "edit-wfa" ? WFG_METRIC_EDIT
                   : opt.algorithm == "indel-wfa" ? WFG_METRIC_INDEL
                   : opt.algorithm == "gap-linear-wfa" ? WFG_METRIC_GAP_LINEAR
                   : opt.algorithm == "gap-affine2p-wfa" ? WFG_METRIC_GAP_AFFINE_2P : WFG_METRIC_GAP_AFFINE;
  wfg_config_t cfg{opt.match, opt.mismatch, opt.gap_opening, opt.gap_extension, opt.score_only ? 1 : 0,
                   opt.max_steps, metric, 0, 0};
  if (metric == WFG_METRIC_GAP_AFFINE_2P) {
    cfg.match = opt.p2[0]; cfg.mismatch = opt.p2[1]; cfg.gap_opening = opt.p2[2]; cfg.gap_extension = opt.p2[3];
    cfg.gap_opening2 = opt.p2[4]; cfg.gap_extension2 = opt.p2[5];
  }
  if (metric == WFG_METRIC_GAP_LINEAR) {
    cfg.match = opt.lin_match; cfg.mismatch = opt.lin_mismatch; cfg.gap_opening = opt.lin_indel; cfg.gap_extension = 0;
  }
  Batch b;
  std::vector<int> scores, statuses, run_len;
  std::vector<int64_t> run_off;
  std::vector<uint32_t> runs;
  std::string l1, l2, line;
  long long total = 0, failed = 0;
  double align_s = 0.0;
  const auto t_begin = std::chrono::steady_clock::now();
  bool eof = false;
  while (!eof) {
    b.clear();
    while (b.n() < opt.batch_size) {
      if (!read_line(in, l1) || !read_line(in, l2)) { eof = true; break; }
      strip(l1); strip(l2);
      b.p_off.push_back((int64_t)b.seq.size()); b.plen.push_back((int)l1.size());
      b.seq.insert(b.seq.end(), l1.begin(), l1.end());
      b.t_off.push_back((int64_t)b.seq.size()); b.tlen.push_back((int)l2.size());
      b.seq.insert(b.seq.end(), l2.begin(), l2.end());
    }
    const int n = b.n();
    if (n == 0) break;
    scores.assign((size_t)n, 0); statuses.assign((size_t)n, 0);
    run_off.assign((size_t)n, 0); run_len.assign((size_t)n, 0);
    runs.resize(b.seq.size() + (size_t)n + 16);  // a CIGAR has at most |P| + |T| runs
    int64_t nruns = 0;
    const auto t0 = std::chrono::steady_clock::now();
    const int st = wfg_align_host(ctx, &cfg, WFG_SCHED_SORTED, n, b.seq.data(), (int64_t)b.seq.size(), b.p_off.data(),
                                  b.plen.data(), b.t_off.data(), b.tlen.data(), scores.data(), statuses.data(),
                                  run_off.data(), run_len.data(), runs.data(), (int64_t)runs.size(), &nruns);
    align_s += std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
    if (st != WF_STATUS_ALG_COMPLETED) {
      fprintf(stderr, "alignment failed (%d): %s\n", st, wfg_last_error(ctx));
      wfg_context_destroy(ctx);
      return 1;
    }
    for (int i = 0; i < n; ++i) {
      if (statuses[i] != WF_STATUS_ALG_COMPLETED) ++failed;
      if (!out) continue;
      const bool has_cigar = !opt.score_only && statuses[i] == WF_STATUS_ALG_COMPLETED && run_len[i] > 0;
      const int score = opt.score_only ? scores[i] : (has_cigar ? scores[i] : -1);
      line.clear();
      if (opt.output_full) {
        line += std::to_string(b.plen[(size_t)i]) + "\t" + std::to_string(b.tlen[(size_t)i]) + "\t" +
                std::to_string(score) + "\t";
        line.append(b.seq.data() + b.p_off[(size_t)i], (size_t)b.plen[(size_t)i]);
        line += "\t";
        line.append(b.seq.data() + b.t_off[(size_t)i], (size_t)b.tlen[(size_t)i]);
        line += "\t";
      } else {
        line += std::to_string(score) + "\t";
      }
      if (has_cigar) print_cigar(line, runs.data() + run_off[(size_t)i], run_len[(size_t)i]);
      else line += "-";
      line += "\n";
      fwrite(line.data(), 1, line.size(), out);
    }
    total += n;
  }
  const double wall_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_begin).count();
  if (!opt.quiet) {
    fprintf(stderr, "[Benchmark]\n=> Total.reads            %lld\n", total);
    fprintf(stderr, "=> Time.Benchmark        %.3f s\n", wall_s);
    fprintf(stderr, "  => Time.Alignment      %.3f s (%.0f pairs/s)\n", align_s,
            align_s > 0 ? (double)total / align_s : 0.0);
    if (failed) fprintf(stderr, "=> Failed.pairs           %lld\n", failed);
  }
  if (out) fclose(out);
  fclose(in);
  wfg_context_destroy(ctx);
  return 0;
}
