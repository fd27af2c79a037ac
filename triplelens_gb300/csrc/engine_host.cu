// engine_host.cu - process-wide GPU resources of the engine (see engine_host.h).
#include <cuda_runtime.h>

#include <unistd.h>

#include <atomic>
#include <thread>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <string>

#include "engine_host.h"

namespace tl {

void* DevBuf::need(size_t bytes, cudaStream_t st) {
  if (bytes == 0) bytes = 16;
  if (bytes > n) {
    release(st);
    size_t want = bytes + bytes / 4;
    const cudaError_t e = st ? cudaMallocAsync(&p, want, st) : cudaMalloc(&p, want);
    if (e != cudaSuccess) {
      p = nullptr;
      n = 0;
      fprintf(stderr, "liblcirs: device allocation of %zu bytes failed\n", want);
      return nullptr;
    }
    pooled = st != nullptr;
    n = want;
  }
  return p;
}

void DevBuf::release(cudaStream_t st) {
  if (p) {
    if (pooled)
      cudaFreeAsync(p, st);
    else
      cudaFree(p);
  }
  p = nullptr;
  n = 0;
  pooled = false;
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
  check(cudaEventCreateWithFlags(&fill_done_, cudaEventDisableTiming));
  // freed pool memory stays with the process (stream-ordered buffers of
  // objects are released and taken again without a trip to the driver)
  {
    int dev = 0;
    cudaMemPool_t pool;
    if (cudaGetDevice(&dev) == cudaSuccess && cudaDeviceGetDefaultMemPool(&pool, dev) == cudaSuccess) {
      uint64_t keep = ~0ull;
      cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
    }
  }
  upload_trig_tables();
  if (const char* c = getenv("TL_FILL_CAP_LOG2")) want_cap_log2_ = atoi(c);
  if (const char* c = getenv("TL_TRACE")) {
    tracing = atoi(c) != 0;
    sync_steps = atoi(c) >= 2;
  }
  if (const char* c = getenv("TL_FILL_CTAS")) want_ctas_ = atoi(c);
  if (const char* c = getenv("TL_FILL_OCC")) set_fill_occupancy(atoi(c));
  // TL_FILL_BIG: CTAs with the large level-0 tables (0: none)
  if (const char* c = getenv("TL_FILL_BIG")) want_big_ctas_ = atoi(c);
  // TL_FILL_LEVELS=1 disables the overflow retries (and their tables)
  if (const char* c = getenv("TL_FILL_LEVELS")) levels_ = atoi(c);
  if (const char* c = getenv("TL_FILL_PROFILE")) profiling = atoi(c) != 0;
  if (const char* c = getenv("TL_FILL_KERNEL")) warp_fill_ = std::string(c) == "cta" ? 0 : 1;
  if (const char* c = getenv("TL_WFILL_THR")) wfill_thr_ = (unsigned)atoi(c);
  if (const char* c = getenv("TL_BLOCK_H")) {
    const int b = atoi(c);
    if (b == 8 || b == 16 || b == 32) block_h_ = b;
  }
}

void Engine::trace(const char* what) {
  if (!tracing) return;
  static const auto t0 = std::chrono::steady_clock::now();
  const double t = std::chrono::duration<double>(std::chrono::steady_clock::now() - t0).count();
  fprintf(stderr, "[tl %10.4f t%zx] %s\n", t,
          (size_t)std::hash<std::thread::id>()(std::this_thread::get_id()) & 0xfff, what);
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

void Engine::set_fill_config(int ctas, int cap_log2, int threads, int block_h, int occ) {
  if (ctas > 0) want_ctas_ = ctas;
  if (cap_log2 > 0) want_cap_log2_ = cap_log2;
  if (threads > 0) threads_ = threads;
  if (occ >= 2 && occ <= 4) set_fill_occupancy(occ);
  const bool bh_changed = (block_h == 8 || block_h == 16 || block_h == 32) && block_h != block_h_;
  if (bh_changed) block_h_ = block_h;
  const int ctas0 = want_ctas_ > 0 ? want_ctas_ : fill_default_ctas();
  for (int level = 0; level < kFillLevels; level++) {
    if (!fs_[level].keys) continue;
    if (bh_changed || (level == 0 && (fs_[0].ctas != ctas0 ||
                                      fs_[0].cap_log2 + (block_h_ == 32 ? 2 : (block_h_ == 16 ? 1 : 0)) !=
                                          want_cap_log2_))) {
      cudaStreamSynchronize(stream);
      cudaEventSynchronize(fill_done_);   // a fill may run on another stream
      cudaFree(fill_base_[level]);
      fill_base_[level] = nullptr;
      fs_[level] = FillScratch{};
    }
  }
}

bool Engine::ensure_fill_scratch(int level) {
  if (fs_[level].keys) return true;
  int ctas, cap;
  if (level == 0) {
    ctas = want_ctas_ > 0 ? want_ctas_ : fill_default_ctas();
    cap = want_cap_log2_;
  } else {
    ctas = kFillLevelCtas[level];
    cap = kFillLevelLog2[level];
  }
  // capacities are counted in 32x8 tiles; a block holds block_h/8 of them
  for (int b = block_h_; b > 8; b >>= 1) cap--;
  // level 0: the first CTAs own 4x larger tables and take the points
  // predicted largest (those that would overflow the others' tables)
  int big = 0, big_log2 = cap;
  if (level == 0) {
    big = want_big_ctas_ >= 0 ? want_big_ctas_ : (ctas >= 256 ? 64 : ctas / 4);
    big = big > ctas ? ctas : big;
    big_log2 = cap + 2;
    // predicted size (units of 1024 rays) from which a point goes to them:
    // 0.6 of the usable 3/4 of a regular table
    big_units_ = (unsigned)(0.45 * (double)((size_t)1 << cap) * block_h_ / 32.0);
  }
  const size_t bytes = fill_scratch_bytes(ctas, cap, block_h_, big, big_log2);
  if (!check(cudaMalloc(&fill_base_[level], bytes))) return false;
  fill_scratch_init(&fs_[level], fill_base_[level], ctas, cap, block_h_, stream, big, big_log2);
  check(cudaStreamSynchronize(stream));
  return true;
}

bool Engine::ensure_wscratch() {
  if (ws_.keys) return true;
  const int warps = wfill_default_warps();
  if (!check(cudaMalloc(&wfill_base_, wscratch_bytes(warps)))) return false;
  wscratch_init(&ws_, wfill_base_, warps, stream);
  check(cudaStreamSynchronize(stream));
  return true;
}

Run RunBufs::prepare(size_t np, size_t ntraj, size_t njobs, bool dump, size_t nscan,
                     cudaStream_t st) {
  Run R;
  R.trajs = (Traj*)trajs.need(sizeof(Traj) * ntraj, st);
  R.jobs = (SeedJob*)jobs.need(sizeof(SeedJob) * njobs, st);
  R.scan_jobs = nscan ? (SeedJob*)scan.need(sizeof(SeedJob) * nscan, st) : nullptr;
  R.prep = nscan ? (PointPrep*)prep.need(sizeof(PointPrep) * np, st) : nullptr;
  R.points = (PointIn*)points.need(sizeof(PointIn) * np, st);
  R.seeds = (int32_t*)seeds.need(sizeof(int32_t) * 2 * kMaxSeeds * np, st);
  R.out = (PointOut*)out.need(sizeof(PointOut) * np, st);
  R.trials = (TrialList*)trials.need(sizeof(TrialList) * np, st);
  R.dump = nullptr;
  R.dump_count = nullptr;
  R.dump_cap = 0;
  if (dump) {
    const size_t cap = 1u << 22;  // tiles
    char* b = (char*)this->dump.need(sizeof(uint32_t) * kDumpWords * cap + 16, st);
    R.dump_count = (unsigned*)b;
    R.dump = (uint32_t*)(b + 16);
    R.dump_cap = (unsigned)cap;
    cudaMemsetAsync(R.dump_count, 0, sizeof(unsigned), st);
  }
  return R;
}

Run Engine::prepare(size_t np, size_t ntraj, size_t njobs, bool dump, size_t nscan) {
  last_error = 0;
  return run_.prepare(np, ntraj, njobs, dump, nscan, stream);
}

void Engine::fill(const Run& R, size_t np, const DevLens* d_lenses, int mode) {
  fill_on(R, np, d_lenses, mode, stream);
}

void Engine::fill_on(const Run& R, size_t np, const DevLens* d_lenses, int mode, cudaStream_t st) {
  if (!ensure_fill_scratch(0)) return;
  if (warp_fill_ && !ensure_wscratch()) return;
  // the tables are shared: start after the previous fill, on any stream (a
  // graph being captured is ordered at its launch instead)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  check(cudaStreamIsCapturing(st, &cap));
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  if (!capturing) fill_after(st);
  FillScratch s = fs_[0];
  // largest points first; the head of the list goes to the large tables
  char* ob = (char*)order_.need(sizeof(int32_t) * np + 1024);
  unsigned* order_meta = (unsigned*)ob;
  int32_t* order_list = (int32_t*)(ob + 1024);
  launch_order(R.points, (int)np, order_list, order_meta, big_units_, st);
  s.nbig = order_meta + 1;
  s.dump = R.dump;
  s.dump_count = R.dump_count;
  s.dump_cap = R.dump_cap;
  unsigned long long* prof = nullptr;
  if (profiling) {
    prof = (unsigned long long*)prof_.need(8 * sizeof(unsigned long long));
    cudaMemsetAsync(prof, 0, 8 * sizeof(unsigned long long), st);
    s.prof = prof;
  }
  if (heartbeat_words_ == 0 && getenv("TL_HEARTBEAT")) {
    heartbeat_words_ = 1 << 16;
    cudaHostAlloc((void**)&heartbeat_host_, heartbeat_words_ * 8, cudaHostAllocMapped);
    cudaHostGetDevicePointer((void**)&heartbeat_dev_, heartbeat_host_, 0);
  }
  s.heartbeat = heartbeat_dev_;
  if (warp_fill_) {
    // one warp per point for every point up to wfill_thr_ predicted blocks;
    // the larger ones, and those whose warp table fills up, come back with
    // status bit 4 and go to the CTA fill below (all its levels)
    WScratch w = ws_;
    w.wthr = wfill_thr_;
    w.dump = R.dump;
    w.dump_count = R.dump_count;
    w.dump_cap = R.dump_cap;
    launch_wfill(R.points, (int)np, d_lenses, R.seeds, R.out, w, mode, st, order_list,
                 order_meta);
  } else {
    launch_fill(R.points, (int)np, d_lenses, R.seeds, R.out, s, mode, threads_, st, order_list,
                order_meta);
  }
  if (heartbeat_host_) {
    // a side thread reports the warps' phases while the stream is busy; the
    // caller keeps blocking as usual
    const int nw = s.ctas * (threads_ / 32);
    unsigned long long* hb = heartbeat_host_;
    std::atomic<bool> done(false);
    std::thread watch([hb, nw, &done]() {
      for (int it = 1; !done.load() && it < 600; it++) {
        for (int k = 0; k < 20 && !done.load(); k++) usleep(100000);
        if (done.load()) break;
        int hist[16] = {0};
        for (int w = 0; w < nw; w++) hist[(hb[w] >> 56) & 15]++;
        fprintf(stderr, "[tl hb] %ds phases:", 2 * it);
        for (int k = 0; k < 9; k++) fprintf(stderr, " %d:%d", k, hist[k]);
        fprintf(stderr, "\n");
        int shown = 0;
        for (int w = 0; w < nw && shown < 16; w++) {
          const unsigned long long v = hb[w];
          const int ph = (int)((v >> 56) & 15);
          if (ph != 0 && ph != 8) {
            fprintf(stderr, "   warp %d cta %d phase %d point %llu step %llu\n", w, w / 8, ph,
                    (v >> 24) & 0xffffffffull, v & 0xffffffull);
            shown++;
          }
        }
      }
    });
    cudaStreamSynchronize(st);
    done.store(true);
    watch.join();
  }
  if (profiling) {
    unsigned long long h[8];
    cudaMemcpyAsync(h, prof, sizeof(h), cudaMemcpyDeviceToHost, st);
    cudaStreamSynchronize(st);
    fprintf(stderr,
            "[tl prof] tiles %llu  cyc/tile %.0f  idle polls %llu  work-loop cyc %llu  "
            "supertiles %llu  cyc/supertile %.0f  eval cyc/tile %.0f  push cyc/tile %.0f\n",
            h[0], h[0] ? (double)h[1] / h[0] : 0.0, h[2], h[3], h[4],
            h[4] ? (double)h[5] / h[4] : 0.0, h[0] ? (double)h[6] / h[0] : 0.0,
            h[0] ? (double)h[7] / h[0] : 0.0);
  }
  // points whose tile table overflowed run again with larger tables; the
  // retry launches read their point count on the device, so no host round
  // trip is needed (a retry with an empty list exits at once)
  char* rb = (char*)retry_.need(sizeof(int32_t) * np + 64);
  int32_t* list = (int32_t*)(rb + 64);
  unsigned* count = (unsigned*)rb;
  for (int level = warp_fill_ ? 0 : 1; level < kFillLevels && level < levels_ + warp_fill_;
       level++) {
    if (!ensure_fill_scratch(level)) break;
    FillScratch sl = fs_[level];
    sl.nbig = nullptr;   // a retry list is not size-ordered: every CTA takes from it
    sl.dump = R.dump;
    sl.dump_count = R.dump_count;
    sl.dump_cap = R.dump_cap;
    launch_collect_overflow(R.out, (int)np, list, count, st);
    launch_fill(R.points, (int)np, d_lenses, R.seeds, R.out, sl, mode, threads_, st, list, count);
  }
  if (!capturing) fill_mark(st);
  check(cudaGetLastError());
}

void Engine::fill_after(cudaStream_t st) { check(cudaStreamWaitEvent(st, fill_done_, 0)); }
void Engine::fill_mark(cudaStream_t st) { check(cudaEventRecord(fill_done_, st)); }

}  // namespace tl
