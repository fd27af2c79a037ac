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

std::atomic<unsigned long long> g_copy_h2d{0}, g_copy_d2h{0};

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
  // TL_FILL_LEVELS: CTA-fill table levels used (1: the warp fill's overflow
  // goes to level 0 only; with TL_FILL_KERNEL=cta, no retries)
  if (const char* c = getenv("TL_FILL_LEVELS")) levels_ = atoi(c);
  if (const char* c = getenv("TL_FILL_PROFILE")) profiling = atoi(c) != 0;
  if (const char* c = getenv("TL_FILL_KERNEL")) warp_fill_ = std::string(c) == "cta" ? 0 : 1;
  if (const char* c = getenv("TL_WFILL_THR")) wfill_thr_ = (unsigned)atoi(c);
  // TL_WFILL_WARPS: warps of the warp fill (default 32 per SM; each owns a
  // 5.5 MB table)
  if (const char* c = getenv("TL_WFILL_WARPS")) want_wfill_warps_ = atoi(c);
  // TL_TEAM_FILL=0: no team fill (the CTA fill takes the warp fill's leftovers);
  // TL_TEAMS: teams of 8 warps (default 2 per SM)
  if (const char* c = getenv("TL_TEAM_FILL")) team_fill_ = atoi(c) != 0;
  // TL_PIPE_CTAS: warp-fill CTAs per SM beside the chain (1..7)
  if (const char* c = getenv("TL_PIPE_CTAS")) pipe_ctas_ = atoi(c);
  if (const char* c = getenv("TL_TEAMS")) want_teams_ = atoi(c);
  // TL_WFILL_CAP_LOG2: slots per warp table (log2, 10..16; the threshold follows)
  if (const char* c = getenv("TL_WFILL_CAP_LOG2")) {
    wfill_cap_log2_ = atoi(c);
    if (!getenv("TL_WFILL_THR"))
      wfill_thr_ = (unsigned)(0.43 * (double)(1u << (wfill_cap_log2_ < 10 ? 10 : wfill_cap_log2_)));
  }
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
  const int warps = want_wfill_warps_ > 0 ? want_wfill_warps_ : wfill_default_warps();
  int cap = wfill_cap_log2_;
  cap = cap < kWCapLog2Min ? kWCapLog2Min : (cap > kWCapLog2 ? kWCapLog2 : cap);
  if (!check(cudaMalloc(&wfill_base_, wscratch_bytes(warps, cap)))) return false;
  wscratch_init(&ws_, wfill_base_, warps, cap, stream);
  check(cudaStreamSynchronize(stream));
  return true;
}

bool Engine::ensure_tscratch() {
  if (ts_.keys) return true;
  const int teams = want_teams_ > 0 ? want_teams_ : tfill_default_teams();
  const int cap = kTeamCapLog2;
  const unsigned inbox = 1u << 13;
  if (!check(cudaMalloc(&tfill_base_, tscratch_bytes(teams, cap, inbox)))) return false;
  tscratch_init(&ts_, tfill_base_, teams, cap, inbox, stream);
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
  R.ok = R.trajs && R.jobs && R.points && R.seeds && R.out && R.trials &&
         (!nscan || (R.scan_jobs && R.prep));
  if (dump && R.ok) {
    const size_t cap = 1u << 22;  // tiles
    char* b = (char*)this->dump.need(sizeof(uint32_t) * kDumpWords * cap + 16, st);
    if (!b) {
      R.ok = false;
      return R;
    }
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

bool Engine::fill(const Run& R, size_t np, const DevLens* d_lenses, int mode) {
  return fill_on(R, np, d_lenses, mode, stream);
}

bool Engine::fill_on(const Run& R, size_t np, const DevLens* d_lenses, int mode, cudaStream_t st) {
  NvtxRange range("tl fill");
  const bool warp = warp_fill_ != 0;
  const bool team = warp && team_fill_ != 0;
  if (!R.ok) return false;
  if (warp && !ensure_wscratch()) return false;
  if (team && !ensure_tscratch()) return false;
  if (!team && !ensure_fill_scratch(0)) return false;
  // the tables are shared: start after the previous fill, on any stream (a
  // graph being captured is ordered at its launch instead)
  cudaStreamCaptureStatus cap = cudaStreamCaptureStatusNone;
  check(cudaStreamIsCapturing(st, &cap));
  const bool capturing = cap != cudaStreamCaptureStatusNone;
  if (!capturing) fill_after(st);
  // largest points first; in the CTA fill the head of the list goes to its
  // large tables
  char* ob = (char*)order_.need(sizeof(int32_t) * np + 1024);
  if (!ob || !retry_.need(sizeof(int32_t) * np + 64)) return false;
  unsigned* order_meta = (unsigned*)ob;
  int32_t* order_list = (int32_t*)(ob + 1024);
  launch_order(R.points, (int)np, order_list, order_meta, big_units_, st);
  cudaEvent_t pe[3] = {nullptr, nullptr, nullptr};
  if (profiling && warp) {
    for (auto& e : pe) cudaEventCreate(&e);
    cudaEventRecord(pe[0], st);
  }
  if (warp) {
    // one warp per point for every point up to wfill_thr_ predicted blocks
    WScratch w = ws_;
    w.wthr = wfill_thr_;
    w.dump = R.dump;
    w.dump_count = R.dump_count;
    w.dump_cap = R.dump_cap;
    unsigned long long* wprof = nullptr;
    if (profiling) {
      wprof = (unsigned long long*)wprof_.need(8 * sizeof(unsigned long long));
      if (wprof) {
        cudaMemsetAsync(wprof, 0, 8 * sizeof(unsigned long long), st);
        w.prof = wprof;
      }
    }
    {
      NvtxRange stage("tl warp fill");
      launch_wfill(R.points, (int)np, d_lenses, R.seeds, R.out, w, mode, st, order_list,
                   order_meta);
    }
    if (profiling && wprof) {
      cudaEventRecord(pe[1], st);
      unsigned long long h[8];
      cudaMemcpyAsync(h, wprof, sizeof(h), cudaMemcpyDeviceToHost, st);
      cudaStreamSynchronize(st);
      fprintf(stderr,
              "[tl wprof] points %llu  visits %llu  first visits %llu  super-tiles %llu  "
              "probe rounds %llu  inserted %llu  whole %llu  ray-by-ray weights %llu\n",
              h[7], h[0], h[1], h[2], h[3], h[4], h[5], h[6]);
    }
  } else {
    FillScratch s = fs_[0];
    s.nbig = order_meta + 1;
    s.dump = R.dump;
    s.dump_count = R.dump_count;
    s.dump_cap = R.dump_cap;
    unsigned long long* prof = nullptr;
    if (profiling) {
      prof = (unsigned long long*)prof_.need(8 * sizeof(unsigned long long));
      if (prof) {
        cudaMemsetAsync(prof, 0, 8 * sizeof(unsigned long long), st);
        s.prof = prof;
      }
    }
    {
      NvtxRange stage("tl cta fill");
      launch_fill(R.points, (int)np, d_lenses, R.seeds, R.out, s, mode, threads_, st,
                  order_list, order_meta);
    }
    if (profiling && prof) {
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
  }
  if (profiling && warp) cudaEventRecord(pe[2], st);
  fill_rest(R, np, d_lenses, mode, st, warp, team);
  if (profiling && warp) {
    cudaEvent_t e3;
    cudaEventCreate(&e3);
    cudaEventRecord(e3, st);
    cudaEventSynchronize(e3);
    float a = 0.f, b = 0.f, c = 0.f;
    cudaEventElapsedTime(&a, pe[0], pe[1]);
    cudaEventElapsedTime(&b, pe[1], pe[2]);
    cudaEventElapsedTime(&c, pe[2], e3);
    fprintf(stderr, "[tl wprof] warp fill %.1f ms, then %.1f ms, team fill and CTA-fill levels %.1f ms\n",
            a, b, c);
    for (auto& e : pe) cudaEventDestroy(e);
    cudaEventDestroy(e3);
  }
  if (!capturing) fill_mark(st);
  check(cudaGetLastError());
  return true;
}

void Engine::fill_rest(const Run& R, size_t np, const DevLens* d_lenses, int mode,
                       cudaStream_t st, bool warp, bool team) {
  // points left over by one stage (status bit 4) are listed for the next;
  // the launches read their point count on the device, so no host round trip
  // is needed (a launch with an empty list exits at once)
  char* rb = (char*)retry_.need(sizeof(int32_t) * np + 64);
  if (!rb) return;   // allocated by the caller already: not reached
  int32_t* list = (int32_t*)(rb + 64);
  unsigned* count = (unsigned*)rb;
  if (warp && team) {
    // the larger points (and those whose warp table filled up): 8 warps each
    WScratch t = ts_;
    t.dump = R.dump;
    t.dump_count = R.dump_count;
    t.dump_cap = R.dump_cap;
    NvtxRange stage("tl team fill");
    launch_collect_overflow(R.out, (int)np, list, count, st);
    launch_tfill(R.points, (int)np, d_lenses, R.seeds, R.out, t, mode, st, list, count);
  }
  // points whose table overflowed run again with larger tables (CTA fill;
  // level 0 only when neither the team fill nor the CTA fill has run)
  for (int level = warp && !team ? 0 : 1; level < kFillLevels && level < levels_; level++) {
    if (!ensure_fill_scratch(level)) break;
    FillScratch sl = fs_[level];
    sl.nbig = nullptr;   // a retry list is not size-ordered: every CTA takes from it
    sl.dump = R.dump;
    sl.dump_count = R.dump_count;
    sl.dump_cap = R.dump_cap;
    NvtxRange stage(level == 0 ? "tl cta fill" : level == 1 ? "tl cta fill level 1"
                                                             : "tl cta fill level 2");
    launch_collect_overflow(R.out, (int)np, list, count, st);
    launch_fill(R.points, (int)np, d_lenses, R.seeds, R.out, sl, mode, threads_, st, list, count);
  }
}

bool Engine::pipeline_exact(const Run& R, size_t np, const Pipeline& P, int mode,
                            cudaStream_t st) {
  NvtxRange range("tl seeds and fill");
  const bool team = team_fill_ != 0;
  if (!R.ok || !P.prep || !P.chains) return false;
  if (!ensure_wscratch()) return false;
  if (team && !ensure_tscratch()) return false;
  if (!team && !ensure_fill_scratch(0)) return false;
  if (!retry_.need(sizeof(int32_t) * np + 64)) return false;
  if (!side_ && !check(cudaStreamCreateWithFlags(&side_, cudaStreamNonBlocking))) return false;
  while ((int)seg_ev_.size() < P.nseg + 1) {
    cudaEvent_t e;
    if (!check(cudaEventCreateWithFlags(&e, cudaEventDisableTiming))) return false;
    seg_ev_.push_back(e);
  }
  fill_after(st);
  launch_seeds_prep(P.scan, P.nscan, R.trajs, P.lenses, P.ca, R.trials, P.prep, st);
  if (P.reset_chains) launch_chain_reset(R.trajs, P.ntraj, P.lenses, P.chains, st);
  WScratch w = ws_;
  w.wthr = wfill_thr_;
  w.dump = R.dump;
  w.dump_count = R.dump_count;
  w.dump_cap = R.dump_cap;
  // TL_FILL_PROFILE: event times of the chain segments and the fills
  std::vector<cudaEvent_t> tc, tf;
  cudaEvent_t t0 = nullptr, tend = nullptr;
  if (profiling) {
    cudaEventCreate(&t0);
    cudaEventCreate(&tend);
    cudaEventRecord(t0, st);
    tc.resize(P.nseg);
    tf.resize(P.nseg);
    for (int s = 0; s < P.nseg; s++) {
      cudaEventCreate(&tc[s]);
      cudaEventCreate(&tf[s]);
    }
  }
  for (int s = 0; s < P.nseg; s++) {
    NvtxRange segment("tl chain segment and its warp fill");
    launch_chain(P.segjobs + P.segjob0[s], P.segjob0[s + 1] - P.segjob0[s], R.trajs, P.lenses,
                 R.points, R.seeds, R.out, R.trials, P.prep, P.chains, st);
    if (profiling) cudaEventRecord(tc[s], st);
    check(cudaEventRecord(seg_ev_[s], st));
    check(cudaStreamWaitEvent(side_, seg_ev_[s], 0));
    // wfill_ctas_ CTAs per SM: every SM keeps room for the next segment's
    // chain warp
    launch_wfill(R.points, (int)np, P.lenses, R.seeds, R.out, w, mode, side_,
                 P.seglist + P.segoff[s], P.segn + s, pipe_ctas_);
    if (profiling) cudaEventRecord(tf[s], side_);
  }
  check(cudaEventRecord(seg_ev_[P.nseg], side_));
  check(cudaStreamWaitEvent(st, seg_ev_[P.nseg], 0));
  fill_rest(R, np, P.lenses, mode, st, true, team);
  fill_mark(st);
  if (profiling) {
    cudaEventRecord(tend, st);
    cudaEventSynchronize(tend);
    fprintf(stderr, "[tl pipe] chain segments end at");
    for (int s = 0; s < P.nseg; s++) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, tc[s]);
      fprintf(stderr, " %.0f", ms);
    }
    fprintf(stderr, " ms; fills end at");
    for (int s = 0; s < P.nseg; s++) {
      float ms = 0.f;
      cudaEventElapsedTime(&ms, t0, tf[s]);
      fprintf(stderr, " %.0f", ms);
    }
    float ms = 0.f;
    cudaEventElapsedTime(&ms, t0, tend);
    fprintf(stderr, " ms; all %.0f ms\n", ms);
    for (int s = 0; s < P.nseg; s++) {
      cudaEventDestroy(tc[s]);
      cudaEventDestroy(tf[s]);
    }
    cudaEventDestroy(t0);
    cudaEventDestroy(tend);
  }
  check(cudaGetLastError());
  return true;
}

void Engine::fill_after(cudaStream_t st) { check(cudaStreamWaitEvent(st, fill_done_, 0)); }
void Engine::fill_mark(cudaStream_t st) { check(cudaEventRecord(fill_done_, st)); }

}  // namespace tl
