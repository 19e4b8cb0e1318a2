// Stage profiler: CUDA events recorded on the launching stream at the stage
// boundaries of pvdb_train_step and pvdb_renderer_render. Events of up to
// max_steps calls are kept, so the timed loop never synchronises; the totals
// are read once at the end.
#include <atomic>
#include <mutex>
#include <vector>

#include "pvdb_internal.cuh"

namespace pvdb {

static std::atomic<unsigned long long> g_launches{0};
void count_launches(int n) { g_launches.fetch_add((unsigned long long)n, std::memory_order_relaxed); }
uint64_t launch_counter() { return g_launches.load(); }

namespace {
struct Prof {
  bool on = false;
  int max_steps = 0;
  int step = -1;  // index of the call being recorded
  std::vector<cudaEvent_t> ev;  // [max_steps][kProfMarks]
  std::vector<uint8_t> rec;     // recorded flags
};
Prof g_prof;
std::mutex g_prof_mu;
}  // namespace

void prof_begin_call() {
  if (!g_prof.on) return;
  if (g_prof.step + 1 >= g_prof.max_steps) {
    g_prof.on = false;  // ring full: stop recording
    return;
  }
  ++g_prof.step;
}

void prof_mark(cudaStream_t st, int id) {
  if (!g_prof.on || g_prof.step < 0 || id < 0 || id >= kProfMarks) return;
  const size_t k = size_t(g_prof.step) * kProfMarks + id;
  cudaEventRecord(g_prof.ev[k], st);
  g_prof.rec[k] = 1;
}

}  // namespace pvdb

using namespace pvdb;

extern "C" {

uint64_t pvdb_launch_count(void) { return g_launches.load(); }

int pvdb_profile_begin(int32_t max_steps) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_prof_mu);
  PVDB_REQUIRE(max_steps > 0 && max_steps <= 100000, "max_steps must be in 1..100000");
  for (cudaEvent_t e : g_prof.ev) cudaEventDestroy(e);
  g_prof.ev.assign(size_t(max_steps) * kProfMarks, nullptr);
  g_prof.rec.assign(g_prof.ev.size(), 0);
  for (auto& e : g_prof.ev) PVDB_CHECK_CUDA(cudaEventCreate(&e));
  g_prof.max_steps = max_steps;
  g_prof.step = -1;
  g_prof.on = true;
  return PVDB_OK;
}

int pvdb_profile_end(float* ms, int32_t n_marks, int32_t* n_calls) {
  clear_error();
  std::lock_guard<std::mutex> lk(g_prof_mu);
  PVDB_REQUIRE(ms && n_marks > 0 && n_marks <= kProfMarks, "bad output");
  g_prof.on = false;
  for (int i = 0; i < n_marks; ++i) ms[i] = 0.f;
  const int calls = g_prof.step + 1;
  for (int s = 0; s < calls; ++s) {
    int prev = -1;
    for (int i = 0; i < kProfMarks; ++i) {
      const size_t k = size_t(s) * kProfMarks + i;
      if (!g_prof.rec[k]) continue;
      if (prev >= 0) {
        PVDB_CHECK_CUDA(cudaEventSynchronize(g_prof.ev[k]));
        float t = 0.f;
        PVDB_CHECK_CUDA(cudaEventElapsedTime(&t, g_prof.ev[size_t(s) * kProfMarks + prev], g_prof.ev[k]));
        if (i < n_marks) ms[i] += t;
      }
      prev = i;
    }
  }
  if (n_calls) *n_calls = calls;
  for (cudaEvent_t e : g_prof.ev) cudaEventDestroy(e);
  g_prof.ev.clear();
  g_prof.rec.clear();
  g_prof.step = -1;
  return PVDB_OK;
}

}  // extern "C"
