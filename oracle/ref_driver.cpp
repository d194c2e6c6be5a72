// Harness that runs the reference's own DSGL trainer (include/dsgl.hpp, compiled
// unmodified) on a corpus file and dumps its final matrices.  Test infrastructure:
// it produces the golden vectors that pin the oracle (tests/golden/make_golden.py) and
// is never part of the product.
//
// Three stand-ins make a run deterministic without touching dsgl.hpp:
//   * omp_get_wtime (used only by the model-sync thread, dsgl.hpp:568-576) returns 0
//     while compute threads run, so no sync round races with them; once every compute
//     thread has returned it jumps ahead so the sync thread takes its exit branch
//     (dsgl.hpp:773).
//   * _mm_malloc/_mm_free are tracked so a compute thread's exit (it frees its first
//     buffer, inputM, at dsgl.hpp:1409) is observable, and so the free of the
//     never-initialised `stream` pointer (dsgl.hpp:1422) is ignored.
//   * rand (used only by the sync thread, to pick one row per block of equal counts,
//     dsgl.hpp:705) returns 0, so the pick is each block's first row.  The reference reads
//     sync_ind[0] of a still empty vector when its pick in the first block is not row 0
//     (dsgl.hpp:700-711), which crashes whenever the largest count is shared; the first row
//     never triggers that read.  The round only runs after training, on one rank, where it
//     copies rows out and back unchanged (allreduce of one rank, division by 1).
//
// usage: dsgl_ref <corpus.i32> <V> <out_prefix> [dsgl flags: -size -window ...]
#include <omp.h>
#include <xmmintrin.h>

// every standard header dsgl.hpp and util.hpp include, before the rand stand-in below
#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <random>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <set>
#include <string>
#include <vector>

#include "type.hpp"

template <typename A, typename B>
class WalkEngine {
 public:
  std::vector<int> local_corpus;
};

static std::atomic<int> g_compute_running{1};
static std::mutex g_alloc_mx;
static std::set<void*> g_live;
static thread_local void* tl_first_alloc = nullptr;

double shim_wtime() { return g_compute_running.load() > 0 ? 0.0 : 1.0e6; }
void* shim_mm_malloc(size_t n, size_t align) {
  void* p = nullptr;
  if (align < sizeof(void*)) align = sizeof(void*);
  if (posix_memalign(&p, align, n ? n : 1) != 0) return nullptr;
  {
    std::lock_guard<std::mutex> g(g_alloc_mx);
    g_live.insert(p);
  }
  if (!tl_first_alloc && omp_in_parallel() && omp_get_thread_num() != 0) tl_first_alloc = p;
  return p;
}
void shim_mm_free(void* p) {
  {
    std::lock_guard<std::mutex> g(g_alloc_mx);
    if (!g_live.count(p)) return;
    g_live.erase(p);
  }
  if (p == tl_first_alloc) {
    tl_first_alloc = nullptr;
    g_compute_running--;
  }
  free(p);
}

int shim_rand() { return 0; }

#define omp_get_wtime shim_wtime
#define rand shim_rand
#define _mm_malloc shim_mm_malloc
#define _mm_free shim_mm_free
#include "dsgl.hpp"
#undef _mm_free
#undef _mm_malloc
#undef rand
#undef omp_get_wtime

int main(int argc, char** argv) {
  if (argc < 4) {
    fprintf(stderr, "usage: %s corpus.i32 V out_prefix [dsgl flags]\n", argv[0]);
    return 2;
  }
  FILE* f = fopen(argv[1], "rb");
  if (!f) return 3;
  fseek(f, 0, SEEK_END);
  long nbytes = ftell(f);
  fseek(f, 0, SEEK_SET);
  WalkEngine<real_t, uint32_t> graph_stub;
  graph_stub.local_corpus.resize(nbytes / 4);
  if (fread(graph_stub.local_corpus.data(), 4, graph_stub.local_corpus.size(), f) !=
      graph_stub.local_corpus.size())
    return 3;
  fclose(f);
  long V = atol(argv[2]);
  std::vector<int> vertex_cn(V, 0);
  for (int t : graph_stub.local_corpus)
    if (t >= 0) vertex_cn[t]++;  // path.hpp:98
  std::vector<vertex_id_t> identity(V);
  for (long i = 0; i < V; i++) identity[i] = (vertex_id_t)i;

  std::vector<char*> args;
  args.push_back(argv[0]);
  int threads = 12;  // dsgl.hpp:69 default
  for (int a = 4; a < argc; a++) {
    args.push_back(argv[a]);
    if (std::string(argv[a]) == "-threads" && a + 1 < argc) threads = atoi(argv[a + 1]);
  }
  args.push_back(nullptr);
  g_compute_running = threads - 1;
  dsgl((int)args.size() - 1, args.data(), &vertex_cn, &identity, &graph_stub);

  std::string pre = argv[3];
  FILE* fw = fopen((pre + ".wih").c_str(), "wb");
  fwrite(Wih, sizeof(float), vocab_size * hidden_size, fw);
  fclose(fw);
  FILE* fo = fopen((pre + ".woh").c_str(), "wb");
  fwrite(Woh, sizeof(float), vocab_size * hidden_size, fo);
  fclose(fo);
  FILE* fr = fopen((pre + ".order").c_str(), "wb");
  for (size_t r = 0; r < vocab_size; r++) fwrite(&v_vocab[r].id, sizeof(uint32_t), 1, fr);
  fclose(fr);
  if (getenv("DSGL_REF_DUMP_TABLES")) {
    FILE* fe = fopen((pre + ".exp").c_str(), "wb");
    fwrite(expTable, sizeof(float), EXP_TABLE_SIZE + 1, fe);
    fclose(fe);
    FILE* ft = fopen((pre + ".table").c_str(), "wb");
    fwrite(table, sizeof(int), table_size, ft);
    fclose(ft);
  }
  return 0;
}
