// Launch accounting and per-kernel CUDA-event timing of the library's own kernels.
#include "internal.h"

namespace fg {

Profiler::~Profiler() {
  for (auto& p : pending_) {
    cudaEventDestroy(p.a);
    cudaEventDestroy(p.b);
  }
  for (auto e : pool_) cudaEventDestroy(e);
}

void Profiler::reset() {
  stats.clear();
  for (auto& p : pending_) {
    pool_.push_back(p.a);
    pool_.push_back(p.b);
  }
  pending_.clear();
}

cudaEvent_t Profiler::get_event() {
  if (!pool_.empty()) {
    cudaEvent_t e = pool_.back();
    pool_.pop_back();
    return e;
  }
  cudaEvent_t e = nullptr;
  cudaEventCreate(&e);
  return e;
}

int Profiler::begin(cudaStream_t st) {
  ++launches;
  if (!on) return -1;
  Pending p;
  p.a = get_event();
  p.b = get_event();
  p.bytes = 0.0;
  cudaEventRecord(p.a, st);
  pending_.push_back(p);
  return (int)pending_.size() - 1;
}

void Profiler::end(int slot, cudaStream_t st, const char* name, double bytes) {
  if (slot < 0) return;
  Pending& p = pending_[slot];
  p.name = name;
  p.bytes = bytes;
  cudaEventRecord(p.b, st);
}

void Profiler::idle(const char* name, int64_t n) {
  if (!on || n <= 0) return;
  for (auto& q : stats)
    if (q.name == name) q.idle += n;
}

int Profiler::flush() {
  for (auto& p : pending_) {
    float ms = 0.0f;
    if (cudaEventElapsedTime(&ms, p.a, p.b) != cudaSuccess) {
      set_error("profiler: event timing failed");
      return FREHG_ERR_CUDA;
    }
    Stat* s = nullptr;
    for (auto& q : stats)
      if (q.name == p.name) s = &q;
    if (!s) {
      stats.push_back(Stat());
      s = &stats.back();
      s->name = p.name;
    }
    s->launches += 1;
    s->ms += ms;
    s->bytes = p.bytes;
    pool_.push_back(p.a);
    pool_.push_back(p.b);
  }
  pending_.clear();
  return FREHG_OK;
}

}  // namespace fg
