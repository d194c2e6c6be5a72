// sgns_train -- command-line trainer over walk files, the drop-in for the embedding step
// huge_walk runs after its walks (src/examples/huge_walk.cpp:67,133).  It takes the
// trainer flags of include/dsgl.hpp:1495-1535 (-size -window -negative -batch-size
// -sample -alpha -min-count -iter -threads -debug -binary -eoutput), one -train <walk
// file or wildcard pattern> per walk file (" %u" per vertex, one walk per line,
// include/path.hpp:92-110),
// and writes the text embedding of my_saveModel (dsgl.hpp:1443-1461).
//
// Additional flags: -vertices V (vocabulary size; default max id + 1), -storage fp32|bf16,
// -engine plain|persistent, -mode hogwild|exact, -workers N, -warps-per-cta N, -table-size N,
// -seed N, -device N, -loss 0|1.
#include <glob.h>

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include "sgns.h"

// A -train argument with a wildcard (huge_walk writes one walk file per worker) expands to
// its matches in sorted order; one without a match is an error.
static bool expand_train(const char* arg, std::vector<std::string>* out) {
  if (!std::strpbrk(arg, "*?[")) {
    out->push_back(arg);
    return true;
  }
  glob_t g;
  const int rc = glob(arg, 0, nullptr, &g);
  if (rc != 0) {
    if (rc != GLOB_NOMATCH) globfree(&g);
    return false;
  }
  for (size_t i = 0; i < g.gl_pathc; i++) out->push_back(g.gl_pathv[i]);
  globfree(&g);
  return true;
}

int main(int argc, char** argv) {
  std::vector<std::string> train_paths;
  std::vector<const char*> train;
  const char* out = nullptr;
  long long V = 0;
  for (int a = 1; a < argc; a++) {
    if (!std::strcmp(argv[a], "-train") && a + 1 < argc && !expand_train(argv[a + 1], &train_paths)) {
      fprintf(stderr, "error: no walk file matches %s\n", argv[a + 1]);
      return 1;
    }
    if (!std::strcmp(argv[a], "-eoutput") && a + 1 < argc) out = argv[a + 1];
    if (!std::strcmp(argv[a], "-vertices") && a + 1 < argc) V = atoll(argv[a + 1]);
  }
  for (const std::string& t : train_paths) train.push_back(t.c_str());
  if (train.empty()) {
    fprintf(stderr,
            "usage: %s -train <walk file> [-train ...] [-eoutput <embedding file>] [-size d] [-window w]\n"
            "          [-negative K] [-batch-size B] [-sample s] [-alpha a] [-min-count m] [-iter n]\n"
            "          [-threads t] [-debug n] [-binary 0|1] [-vertices V] [-storage fp32|bf16]\n"
            "          [-engine plain|persistent] [-mode hogwild|exact] [-workers N] [-warps-per-cta N]\n"
            "          [-table-size N] [-seed N] [-device N] [-loss 0|1]\n",
            argv[0]);
    return 2;
  }
  sgns_options opt;
  sgns_default_options(&opt);
  if (sgns_options_from_args(&opt, argc, argv) != SGNS_OK) {
    fprintf(stderr, "error: %s\n", sgns_last_error(nullptr));
    return 1;
  }
  sgns_handle* h = nullptr;
  if (sgns_create(&opt, &h) != SGNS_OK) {
    fprintf(stderr, "error: %s\n", sgns_last_error(nullptr));
    return 1;
  }
  int rc = 0;
  if (sgns_train_walk_files(h, train.data(), (int32_t)train.size(), V) != SGNS_OK) {
    fprintf(stderr, "error: %s\n", sgns_last_error(h));
    rc = 1;
  } else {
    sgns_stats st;
    sgns_get_stats(h, &st);
    if (opt.debug > 0)
      printf("vertices %lld  steps %llu  pairs %llu  words %llu  %.3f ms  %.3f Mpairs/s  alpha %f\n",
             (long long)sgns_vocab_size(h), (unsigned long long)st.steps, (unsigned long long)st.pairs,
             (unsigned long long)st.word_count_actual, st.train_ms,
             st.train_ms > 0 ? st.pairs / (st.train_ms * 1e3) : 0.0, st.final_alpha);
    if (out && sgns_save_text(h, out) != SGNS_OK) {
      fprintf(stderr, "error: %s\n", sgns_last_error(h));
      rc = 1;
    }
  }
  sgns_destroy(h);
  return rc;
}
