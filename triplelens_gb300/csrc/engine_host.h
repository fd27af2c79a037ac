// engine_host.h - process-wide GPU resources of liblcirs.so: one stream, grow-only
// device buffers and the fill kernel's per-CTA tile tables.  Calls into the
// engine are serialised by `mu` (the reference's objects are not thread-safe
// either; the engine is shared by every object of the process).
#pragma once

#include <cuda_runtime.h>
#include <nvtx3/nvToolsExt.h>

#include <atomic>
#include <cstdio>
#include <mutex>
#include <vector>

#include "engine.h"

struct LightCurveIRS;

namespace tl {

// Bytes moved host -> device and device -> host by the C ABIs' own copies
// (lcirs_*, tlb_*), process-wide totals for end-to-end accounting.
extern std::atomic<unsigned long long> g_copy_h2d, g_copy_d2h;

// NVTX range over a host scope (header-only NVTX 3; a no-op unless a
// profiler is attached): the kernels launched inside it carry its name, so
// `ncu --nvtx --nvtx-include "<name>/"` selects one stage of the pipeline.
struct NvtxRange {
  explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
  ~NvtxRange() { nvtxRangePop(); }
  NvtxRange(const NvtxRange&) = delete;
  NvtxRange& operator=(const NvtxRange&) = delete;
};

// cudaMemcpyAsync with the same arguments, counted.
inline cudaError_t copy_async(void* dst, const void* src, size_t bytes, cudaMemcpyKind kind,
                              cudaStream_t st = 0) {
  if (kind == cudaMemcpyHostToDevice) g_copy_h2d.fetch_add(bytes, std::memory_order_relaxed);
  if (kind == cudaMemcpyDeviceToHost) g_copy_d2h.fetch_add(bytes, std::memory_order_relaxed);
  return cudaMemcpyAsync(dst, src, bytes, kind, st);
}

// Grow-only device buffer.  With a stream, the buffer comes from the
// device's stream-ordered pool (cudaMallocAsync / cudaFreeAsync on that
// stream), which neither waits for the device nor returns memory to the
// system between calls; objects created and freed while a fill runs on
// another stream then do not stall behind it.
struct DevBuf {
  void* p = nullptr;
  size_t n = 0;
  bool pooled = false;
  void* need(size_t bytes, cudaStream_t st = nullptr);
  void release(cudaStream_t st = nullptr);
};

struct Run {
  Traj* trajs;
  SeedJob* jobs;
  SeedJob* scan_jobs;      // exact chain: point chunks of the scan and the prep
  PointPrep* prep;         // exact chain: per-point coefficients and cold roots
  PointIn* points;
  int32_t* seeds;
  PointOut* out;
  TrialList* trials;
  uint32_t* dump;
  unsigned* dump_count;
  unsigned dump_cap;
  bool ok = true;          // every buffer the run needs was allocated
};

// The per-call device buffers of a run (grow-only).  The engine keeps one
// set; every LightCurveIRS object keeps its own, so that the seeds of
// different objects run concurrently (only the fill shares the engine's
// tables).
struct RunBufs {
  DevBuf trajs, jobs, scan, prep, points, seeds, out, trials, dump;
  // sizes the buffers for npoints points, ntraj curves, njobs jobs (and nscan
  // scan chunks for the exact chain); clears the dump counter on st
  Run prepare(size_t npoints, size_t ntraj, size_t njobs, bool dump, size_t nscan,
              cudaStream_t st);
};

// device copy of an object's lens, grid and limb darkening (lcirs_abi.cu)
const DevLens* object_device_lens(const LightCurveIRS* lc);
// the device an object's buffers live on (-1 before its set-up)
int object_device(const LightCurveIRS* lc);

class Engine {
 public:
  static Engine& get();
  std::mutex mu;
  cudaStream_t stream = nullptr;
  int last_error = 0;
  DevBuf scratch_specs, scratch_amp;

  // sizes the per-call buffers for npoints points, ntraj curves, njobs jobs
  // (and nscan scan chunks for the exact chain)
  Run prepare(size_t npoints, size_t ntraj, size_t njobs, bool dump, size_t nscan = 0);
  // runs the fill kernel over the points of R.  Fills share the engine's
  // tables: each fill waits (on the device) for the previous one, whatever
  // stream either was launched on.  Call with `mu` held.
  // Both return false, with nothing launched, when the fill's tables or
  // work lists could not be allocated.
  bool fill(const Run& R, size_t npoints, const DevLens* d_lenses, int mode);
  bool fill_on(const Run& R, size_t npoints, const DevLens* d_lenses, int mode, cudaStream_t st);
  // seeds (exact chain, in segments) and fill overlapped on st and a side
  // stream; the result is ordered on st (false as fill_on)
  bool pipeline_exact(const Run& R, size_t np, const Pipeline& P, int mode, cudaStream_t st);
  // order work that uses the fill tables outside fill_on (a graph replay):
  // fill_after makes st wait for the last fill, fill_mark records st's work
  // as the last fill
  void fill_after(cudaStream_t st);
  void fill_mark(cudaStream_t st);
  bool check(cudaError_t e);
  // TL_TRACE=1: print every host step with a timestamp to stderr
  void trace(const char* what);
  bool tracing = false;
  bool sync_steps = false;  // TL_TRACE=2: also synchronise after every launch
  bool profiling = false;   // TL_FILL_PROFILE=1: fill-kernel cycle counters
  int fill_ctas() const { return fs_[0].ctas; }
  int fill_cap_log2() const { return fs_[0].cap_log2; }
  // fill launch shape; values <= 0 keep the current setting; block_h is the
  // rows per block (8, 16 or 32), occ the resident CTAs per SM (2, 3 or 4)
  void set_fill_config(int ctas, int cap_log2, int threads, int block_h = 0, int occ = 0);
  int block_h() const { return block_h_; }
  // which stage takes which points: warp fill up to thr predicted blocks,
  // then the team fill (team) or the CTA fill; warp = false: CTA fill alone
  void set_fill_paths(bool warp, bool team, unsigned thr) {
    warp_fill_ = warp ? 1 : 0;
    team_fill_ = team ? 1 : 0;
    if (thr > 0) wfill_thr_ = thr;
  }

 private:
  Engine();
  bool ensure_fill_scratch(int level);
  bool ensure_wscratch();
  void* wfill_base_ = nullptr;
  WScratch ws_{};
  // 1: the warp fill takes every point up to wfill_thr_ predicted blocks and
  // the CTA fill the rest (TL_FILL_KERNEL=cta: the CTA fill alone)
  int warp_fill_ = 1;
  unsigned wfill_thr_ = 7000;
  int want_wfill_warps_ = 0;
  int wfill_cap_log2_ = 14;
  // the team fill (8 warps per point) takes the points the warp fill leaves
  bool ensure_tscratch();
  // the leftovers of the warp fill (status bit 4): team fill, then the
  // CTA-fill levels; rb: the retry buffer
  void fill_rest(const Run& R, size_t np, const DevLens* d_lenses, int mode, cudaStream_t st,
                 bool warp, bool team);
  cudaStream_t side_ = nullptr;
  int pipe_ctas_ = 7;
  std::vector<cudaEvent_t> seg_ev_;
  void* tfill_base_ = nullptr;
  WScratch ts_{};
  int team_fill_ = 1;
  int want_teams_ = 0;
  static constexpr int kTeamCapLog2 = 15;   // slots per team warp's table
  RunBufs run_;
  DevBuf retry_, prof_, order_, wprof_;
  cudaEvent_t fill_done_ = nullptr;   // the last fill launched
  int want_big_ctas_ = -1;   // -1: 64 when there are >= 256 CTAs, else a quarter
  unsigned big_units_ = 0;
  void* fill_base_[kFillLevels] = {};
  FillScratch fs_[kFillLevels]{};
  int want_ctas_ = 0, want_cap_log2_ = 17, threads_ = 256;
  int levels_ = kFillLevels;
  size_t heartbeat_words_ = 0;
  unsigned long long* heartbeat_host_ = nullptr;
  unsigned long long* heartbeat_dev_ = nullptr;
  int block_h_ = 32;
};

}  // namespace tl
