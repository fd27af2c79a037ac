// engine_host.cu - process-wide GPU resources of the engine (see engine_host.h).
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>

#include "engine_host.h"

namespace tl {

void* DevBuf::need(size_t bytes) {
  if (bytes == 0) bytes = 16;
  if (bytes > n) {
    if (p) cudaFree(p);
    p = nullptr;
    size_t want = bytes + bytes / 4;
    if (cudaMalloc(&p, want) != cudaSuccess) {
      p = nullptr;
      n = 0;
      fprintf(stderr, "liblcirs: cudaMalloc of %zu bytes failed\n", want);
      return nullptr;
    }
    n = want;
  }
  return p;
}

Engine& Engine::get() {
  static Engine* e = new Engine();
  return *e;
}

Engine::Engine() {
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    fprintf(stderr, "liblcirs: no CUDA device available; this library has no CPU path\n");
    abort();
  }
  check(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
  upload_trig_tables();
  if (const char* c = getenv("TL_FILL_CAP_LOG2")) want_cap_log2_ = atoi(c);
  if (const char* c = getenv("TL_TRACE")) {
    tracing = atoi(c) != 0;
    sync_steps = atoi(c) >= 2;
  }
  if (const char* c = getenv("TL_FILL_CTAS")) want_ctas_ = atoi(c);
}

void Engine::trace(const char* what) {
  if (!tracing) return;
  static const auto t0 = std::chrono::steady_clock::now();
  const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  fprintf(stderr, "[tl %10.4f] %s\n", t, what);
  fflush(stderr);
}

bool Engine::check(cudaError_t e) {
  if (e != cudaSuccess) {
    fprintf(stderr, "liblcirs: CUDA error %s\n", cudaGetErrorString(e));
    last_error = 1;
    return false;
  }
  return true;
}

void Engine::set_fill_config(int ctas, int cap_log2, int threads) {
  if (ctas > 0) want_ctas_ = ctas;
  if (cap_log2 > 0) want_cap_log2_ = cap_log2;
  if (threads > 0) threads_ = threads;
  if (fs_.keys && (fs_.ctas != want_ctas_ || fs_.cap_log2 != want_cap_log2_)) {
    cudaStreamSynchronize(stream);
    cudaFree(fill_base_);
    fill_base_ = nullptr;
    fs_ = FillScratch{};
  }
}

void Engine::ensure_fill_scratch() {
  if (fs_.keys) return;
  const int ctas = want_ctas_ > 0 ? want_ctas_ : fill_default_ctas();
  const int cap = want_cap_log2_;
  fill_bytes_ = fill_scratch_bytes(ctas, cap);
  if (!check(cudaMalloc(&fill_base_, fill_bytes_))) return;
  fill_scratch_init(&fs_, fill_base_, ctas, cap, stream);
  check(cudaStreamSynchronize(stream));
}

Run Engine::prepare(size_t np, size_t ntraj, size_t njobs, bool dump) {
  last_error = 0;
  Run R;
  R.trajs = (Traj*)trajs_.need(sizeof(Traj) * ntraj);
  R.jobs = (SeedJob*)jobs_.need(sizeof(SeedJob) * njobs);
  R.points = (PointIn*)points_.need(sizeof(PointIn) * np);
  R.seeds = (int32_t*)seeds_.need(sizeof(int32_t) * 2 * kMaxSeeds * np);
  R.out = (PointOut*)out_.need(sizeof(PointOut) * np);
  R.dump = nullptr;
  R.dump_count = nullptr;
  R.dump_cap = 0;
  if (dump) {
    const size_t cap = 1u << 22;  // tiles
    char* b = (char*)dump_.need(sizeof(uint32_t) * kDumpWords * cap + 16);
    R.dump_count = (unsigned*)b;
    R.dump = (uint32_t*)(b + 16);
    R.dump_cap = (unsigned)cap;
    check(cudaMemsetAsync(R.dump_count, 0, sizeof(unsigned), stream));
  }
  return R;
}

void Engine::fill(const Run& R, size_t np, const DevLens* d_lenses, int mode) {
  fill_on(R, np, d_lenses, mode, stream);
}

void Engine::fill_on(const Run& R, size_t np, const DevLens* d_lenses, int mode, cudaStream_t st) {
  ensure_fill_scratch();
  FillScratch s = fs_;
  s.dump = R.dump;
  s.dump_count = R.dump_count;
  s.dump_cap = R.dump_cap;
  launch_fill(R.points, (int)np, d_lenses, R.seeds, R.out, s, mode, threads_, st);
  check(cudaGetLastError());
}

}  // namespace tl
