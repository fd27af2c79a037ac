// batch_abi.cu - batched light curves (include/tl_batch.h): many lenses,
// many trajectories, one seeds launch and one persistent fill launch.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <mutex>
#include <stdexcept>
#include <vector>

#include "batch_internal.h"
#include "engine.h"
#include "engine_host.h"
#include "plan.h"
#include "tl_batch.h"

using tl::cx;

namespace {

cudaStream_t pick(void* s) {
  return s ? (cudaStream_t)s : tl::Engine::get().stream;
}

// Runs an entry point's body; an exception (host memory exhausted) does not
// cross the C ABI but returns `fail`, as a CUDA failure does.
template <class R, class F>
R guarded(R fail, F body) {
  try {
    return body();
  } catch (const std::exception& ex) {
    fprintf(stderr, "tl_batch: %s\n", ex.what());
    return fail;
  }
}

}  // namespace

extern "C" {

tl_batch* tlb_new(void) {
  tl::Engine::get();
  return new tl_batch();
}

void tlb_delete(tl_batch* b) {
  if (!b) return;
  if (b->graph) cudaGraphExecDestroy(b->graph);
  for (tl::DevBuf* d : {&b->specs, &b->lenses, &b->cc, &b->ca, &b->trajs, &b->jobs, &b->points,
                        &b->seeds, &b->out, &b->amp, &b->trials, &b->scan, &b->prep})
    if (d->p) cudaFree(d->p);
  delete b;
}

static int set_lenses_body(tl_batch* b, int nlens, const double* p8) {
  if (!b || nlens <= 0 || !p8) return -1;
  // rows the lens set-up cannot use (as lcirs_new's bad input): non-finite
  // values, rho <= 0, rays per radius outside 1..2^31-1
  for (int i = 0; i < nlens; i++) {
    const double* q = p8 + 8 * (size_t)i;
    for (int k = 0; k < 8; k++)
      if (!std::isfinite(q[k])) return -1;
    if (!(q[5] > 0.0) || q[7] < 1.0 || q[7] > 2147483647.0) return -1;
  }
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  std::vector<tl::LensSpec> specs(nlens);
  for (int i = 0; i < nlens; i++) {
    const double* q = p8 + 8 * (size_t)i;
    double A, B, I;
    if (q[6] >= 0.0) {  // limbdarkeningmodel.cc:18-28
      const double v = q[6];
      const double i0 = 1.0 / ((1.0 - v / 3.0));
      A = i0 * (1.0 - v);
      B = i0 * v;
      I = 1.0;
    } else {  // limbdarkeningmodel.cc:8-15
      A = 0.6;
      B = 0.4;
      I = 1.0 / (A + 2.0 / 3.0 * B);
    }
    specs[i] = tl::make_lens_spec(q[0], q[1], q[2], q[3], q[4], q[5], (long)q[7], A, B, I);
  }
  b->nlens = nlens;
  void* ds = b->specs.need(sizeof(tl::LensSpec) * nlens);
  void* dl = b->lenses.need(sizeof(tl::DevLens) * nlens);
  void* dcc = b->cc.need(sizeof(cx) * tl::kBranches * tl::kCCLen * nlens);
  void* dca = b->ca.need(sizeof(cx) * tl::kBranches * tl::kCCLen * nlens);
  if (!ds || !dl || !dcc || !dca) return -2;
  if (!E.check(tl::copy_async(ds, specs.data(), sizeof(tl::LensSpec) * nlens,
                               cudaMemcpyHostToDevice, E.stream)))
    return -2;
  tl::launch_lens_setup((const tl::LensSpec*)ds, nlens, (tl::DevLens*)dl, (cx*)dcc, (cx*)dca,
                        E.stream);
  b->hlens.resize(nlens);
  E.check(tl::copy_async(b->hlens.data(), dl, sizeof(tl::DevLens) * nlens,
                          cudaMemcpyDeviceToHost, E.stream));
  if (!E.check(cudaStreamSynchronize(E.stream))) return -2;
  return nlens;
}

// segments of an exact chain for tlb_run_device phase 4
constexpr int kSegments = 8;

static long set_trajectories_body(tl_batch* b, int ntraj, const double* t4,
                                  const int32_t* lens_idx, const uint32_t* n) {
  if (!b || ntraj <= 0 || !t4 || !lens_idx || !n || b->nlens <= 0) return -1;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  b->htraj.resize(ntraj);
  std::vector<tl::SeedJob> jobs, scan;
  long base = 0;
  for (int i = 0; i < ntraj; i++) {
    if (lens_idx[i] < 0 || lens_idx[i] >= b->nlens) return -1;
    tl::Traj& T = b->htraj[i];
    T.x0 = t4[4 * (size_t)i];
    T.y0 = t4[4 * (size_t)i + 1];
    T.x1 = t4[4 * (size_t)i + 2];
    T.y1 = t4[4 * (size_t)i + 3];
    T.n = n[i];
    T.lens = lens_idx[i];
    T.point_base = base;
    const long np = (long)n[i] + 1;
    tl::plan_jobs(&jobs, i, np, b->chain, -1);
    if (b->chain <= 0) tl::plan_jobs(&scan, i, np, tl::kChainChunk, -1);
    base += np;
  }
  if (base >= (1L << 31)) return -1;
  b->ntraj = ntraj;
  b->npoints = base;
  b->njobs = (int)jobs.size();
  void* dt = b->trajs.need(sizeof(tl::Traj) * ntraj);
  void* dj = b->jobs.need(sizeof(tl::SeedJob) * jobs.size());
  void* dp = b->points.need(sizeof(tl::PointIn) * base);
  void* dsd = b->seeds.need(sizeof(int32_t) * 2 * tl::kMaxSeeds * base);
  void* dout = b->out.need(sizeof(tl::PointOut) * base);
  void* dtr = b->trials.need(sizeof(tl::TrialList) * base);
  if (!dt || !dj || !dp || !dsd || !dout || !dtr) return -2;
  b->nscan = (int)scan.size();
  if (!scan.empty()) {
    void* dsc = b->scan.need(sizeof(tl::SeedJob) * scan.size());
    void* dpr = b->prep.need(sizeof(tl::PointPrep) * base);
    if (!dsc || !dpr) return -2;
    E.check(tl::copy_async(dsc, scan.data(), sizeof(tl::SeedJob) * scan.size(),
                            cudaMemcpyHostToDevice, E.stream));
  }
  E.check(tl::copy_async(dt, b->htraj.data(), sizeof(tl::Traj) * ntraj, cudaMemcpyHostToDevice,
                          E.stream));
  E.check(tl::copy_async(dj, jobs.data(), sizeof(tl::SeedJob) * jobs.size(),
                          cudaMemcpyHostToDevice, E.stream));
  // the exact chain in kSegments segments: jobs, point lists and counts
  b->nseg = 0;
  if (b->chain <= 0) {
    const int S = kSegments;
    std::vector<tl::SeedJob> sj;
    std::vector<int32_t> sl;
    std::vector<unsigned> sn;
    std::vector<int64_t> pb(ntraj);
    std::vector<uint32_t> nn(ntraj);
    for (int i = 0; i < ntraj; i++) {
      pb[i] = b->htraj[i].point_base;
      nn[i] = b->htraj[i].n;
    }
    tl::plan_segments(S, ntraj, pb.data(), nn.data(), &sj, &sl, &sn, &b->segjob0, &b->segoff);
    void* dsj = b->segjobs.need(sizeof(tl::SeedJob) * sj.size());
    void* dsl = b->seglist.need(sizeof(int32_t) * sl.size());
    void* dsn = b->segn.need(sizeof(unsigned) * S);
    void* dch = b->chains.need(sizeof(tl::RootChain) * ntraj);
    if (!dsj || !dsl || !dsn || !dch) return -2;
    E.check(tl::copy_async(dsj, sj.data(), sizeof(tl::SeedJob) * sj.size(),
                            cudaMemcpyHostToDevice, E.stream));
    E.check(tl::copy_async(dsl, sl.data(), sizeof(int32_t) * sl.size(), cudaMemcpyHostToDevice,
                            E.stream));
    E.check(tl::copy_async(dsn, sn.data(), sizeof(unsigned) * S, cudaMemcpyHostToDevice,
                            E.stream));
    b->nseg = S;
  }
  if (!E.check(cudaStreamSynchronize(E.stream))) return -2;
  return base;
}

int tlb_run_device(tl_batch* b, int phase, void* stream) {
  if (!b || b->npoints <= 0) return -1;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  cudaStream_t st = pick(stream);
  if ((phase & 1) && b->nscan > 0)
    tl::launch_seeds_exact((const tl::SeedJob*)b->scan.p, b->nscan, (const tl::SeedJob*)b->jobs.p,
                           b->njobs, (const tl::Traj*)b->trajs.p, (const tl::DevLens*)b->lenses.p,
                           (const cx*)b->ca.p, (tl::PointIn*)b->points.p, (int32_t*)b->seeds.p,
                           (tl::PointOut*)b->out.p, (tl::TrialList*)b->trials.p,
                           (tl::PointPrep*)b->prep.p, nullptr, st);
  else if (phase & 1)
    tl::launch_seeds((const tl::SeedJob*)b->jobs.p, b->njobs, (const tl::Traj*)b->trajs.p,
                     (const tl::DevLens*)b->lenses.p, (const cx*)b->ca.p, (tl::PointIn*)b->points.p,
                     (int32_t*)b->seeds.p, (tl::PointOut*)b->out.p, (tl::TrialList*)b->trials.p,
                     nullptr, st);
  if ((phase & 4) && b->nscan > 0 && b->nseg > 0) {
    // seeds and fill overlapped: the chain of segment s+1 runs while the
    // warp fill works segment s
    tl::Run R;
    R.trajs = (tl::Traj*)b->trajs.p;
    R.jobs = (tl::SeedJob*)b->jobs.p;
    R.points = (tl::PointIn*)b->points.p;
    R.seeds = (int32_t*)b->seeds.p;
    R.out = (tl::PointOut*)b->out.p;
    R.trials = (tl::TrialList*)b->trials.p;
    R.dump = nullptr;
    R.dump_count = nullptr;
    R.dump_cap = 0;
    tl::Pipeline P;
    P.lenses = (const tl::DevLens*)b->lenses.p;
    P.ca = (const cx*)b->ca.p;
    P.scan = (const tl::SeedJob*)b->scan.p;
    P.nscan = b->nscan;
    P.ntraj = b->ntraj;
    P.segjobs = (const tl::SeedJob*)b->segjobs.p;
    P.segjob0 = b->segjob0.data();
    P.seglist = (const int32_t*)b->seglist.p;
    P.segoff = b->segoff.data();
    P.segn = (const unsigned*)b->segn.p;
    P.nseg = b->nseg;
    P.prep = (tl::PointPrep*)b->prep.p;
    P.chains = (tl::RootChain*)b->chains.p;
    if (!E.pipeline_exact(R, (size_t)b->npoints, P, b->precision, st)) return -2;
    return E.check(cudaGetLastError()) ? 0 : -2;
  }
  if (phase & 2) {
    tl::Run R;
    R.trajs = (tl::Traj*)b->trajs.p;
    R.jobs = (tl::SeedJob*)b->jobs.p;
    R.points = (tl::PointIn*)b->points.p;
    R.seeds = (int32_t*)b->seeds.p;
    R.out = (tl::PointOut*)b->out.p;
    R.trials = (tl::TrialList*)b->trials.p;
    R.dump = nullptr;
    R.dump_count = nullptr;
    R.dump_cap = 0;
    if (!E.fill_on(R, (size_t)b->npoints, (const tl::DevLens*)b->lenses.p, b->precision, st))
      return -2;
  }
  return E.check(cudaGetLastError()) ? 0 : -2;
}

static int download_body(tl_batch* b, double* amp, uint64_t* counts, uint32_t* status,
                         void* stream) {
  if (!b || b->npoints <= 0) return -1;
  tl::Engine& E = tl::Engine::get();
  cudaStream_t st = pick(stream);
  std::vector<tl::PointOut> h(b->npoints);
  // wait before the pageable copy: a copy that waits for kernels holds the
  // driver's staging path and stalls other threads' copies
  if (!E.check(cudaStreamSynchronize(st))) return -2;
  if (!E.check(tl::copy_async(h.data(), b->out.p, sizeof(tl::PointOut) * b->npoints,
                               cudaMemcpyDeviceToHost, st)))
    return -2;
  if (!E.check(cudaStreamSynchronize(st))) return -2;
  for (int k = 0; k < 4; k++) b->stats[k] = 0;
  for (int t = 0; t < b->ntraj; t++) {
    const tl::Traj& T = b->htraj[t];
    const double scale = b->hlens[T.lens].g.amp_scale;
    for (long i = 0; i <= (long)T.n; i++) {
      const tl::PointOut& o = h[T.point_base + i];
      if (amp) amp[T.point_base + i] = ((double)o.wsum_fx / tl::kWsumScale) * scale;
      if (counts) counts[T.point_base + i] = o.count;
      if (status) status[T.point_base + i] = o.status;
      b->stats[0] += o.rays_eval;
      b->stats[1] += o.rays_fp64;
      b->stats[2] += o.tiles;
      b->stats[3] += o.count;
    }
  }
  return 0;
}

static long run_host_body(tl_batch* b, int ntraj, const double* t4, const int32_t* lens_idx,
                          const uint32_t* n, double* amp, uint64_t* counts, uint32_t* status,
                          void* stream) {
  long np = tlb_set_trajectories(b, ntraj, t4, lens_idx, n);
  if (np < 0) return np;
  int r = tlb_run_device(b, 3, stream);
  if (r < 0) return r;
  r = tlb_download(b, amp, counts, status, stream);
  return r < 0 ? r : np;
}

int tlb_stats(tl_batch* b, uint64_t* out4) {
  if (!b || !out4) return -1;
  for (int k = 0; k < 4; k++) out4[k] = b->stats[k];
  return 0;
}

int tlb_set_chain(tl_batch* b, int points) {
  if (!b) return -1;
  b->chain = points;
  return 0;
}

int tlb_configure(tl_batch* b, int precision, int fill_ctas, int table_log2, int threads,
                  int block_h) {
  if (!b) return -1;
  if (precision >= 0) b->precision = precision;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  E.set_fill_config(fill_ctas, table_log2, threads, block_h);
  return 0;
}

int tlb_autotune(tl_batch* b, long sample_points, int32_t* chosen3, float* times_ms) {
  if (!b || b->npoints <= 0 || !chosen3) return -1;
  tl::Engine& E = tl::Engine::get();
  const long np = sample_points > 0 && sample_points < b->npoints ? sample_points : b->npoints;
  // seeds of every point once; candidates time the fill of the first np
  if (tlb_run_device(b, 1, nullptr) < 0) return -2;
  // where the points go, by predicted size: one warp per point up to a
  // threshold (blocks of 32 x 32 rays), then 8 warps per point (team fill)
  // or the CTA fill; {threshold, team} (threshold 0: the CTA fill alone)
  const int cand[5][2] = {{7000, 1}, {3000, 1}, {1500, 1}, {7000, 0}, {0, 0}};
  float msk[5];
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  int k = 0;
  for (const auto& c : cand) {
    float ms = -1.f;
    {
      std::lock_guard<std::mutex> g(E.mu);
      E.set_fill_paths(c[0] > 0, c[1] != 0, (unsigned)c[0]);
      tl::Run R;
      R.trajs = (tl::Traj*)b->trajs.p;
      R.jobs = (tl::SeedJob*)b->jobs.p;
      R.points = (tl::PointIn*)b->points.p;
      R.seeds = (int32_t*)b->seeds.p;
      R.out = (tl::PointOut*)b->out.p;
      R.trials = (tl::TrialList*)b->trials.p;
      R.dump = nullptr;
      R.dump_count = nullptr;
      R.dump_cap = 0;
      for (int rep = 0; rep < 2; rep++) {   // the first run allocates the tables
        cudaEventRecord(e0, E.stream);
        const bool ran =
            E.fill_on(R, (size_t)np, (const tl::DevLens*)b->lenses.p, b->precision, E.stream);
        cudaEventRecord(e1, E.stream);
        if (!E.check(cudaEventSynchronize(e1)) || !ran) {
          ms = -1.f;   // a candidate that cannot run is not chosen
          break;
        }
        cudaEventElapsedTime(&ms, e0, e1);
      }
    }
    if (times_ms) times_ms[k] = ms;
    msk[k++] = ms;
  }
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  // the first candidate (the default) stays unless the fastest beats it by 5 %
  const int pick = tl::pick_candidate(msk, 5, 0.05f);
  const int best_thr = cand[pick][0], best_team = cand[pick][1];
  {
    std::lock_guard<std::mutex> g(E.mu);
    E.set_fill_paths(best_thr > 0, best_team != 0, (unsigned)best_thr);
  }
  chosen3[0] = best_thr;
  chosen3[1] = best_team;
  chosen3[2] = (int32_t)np;
  return 0;
}

int tlb_set_fill_stages(tl_batch* b, int warp_threshold_blocks, int team) {
  if (!b || warp_threshold_blocks < 0) return -1;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  const bool warp = warp_threshold_blocks > 0;
  E.set_fill_paths(warp, warp && team != 0, (unsigned)warp_threshold_blocks);
  return 0;
}

int tlb_graph_capture(tl_batch* b) {
  if (!b || b->npoints <= 0) return -1;
  tl::Engine& E = tl::Engine::get();
  if (b->graph) {
    cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
  }
  // a warm run allocates every buffer and table level the run touches, so
  // the captured run allocates nothing
  if (tlb_run_device(b, 3, nullptr) < 0) return -2;
  if (!E.check(cudaStreamSynchronize(E.stream))) return -2;
  cudaGraph_t graph = nullptr;
  if (!E.check(cudaStreamBeginCapture(E.stream, cudaStreamCaptureModeThreadLocal))) return -2;
  const int r = tlb_run_device(b, 3, nullptr);
  const cudaError_t ce = cudaStreamEndCapture(E.stream, &graph);
  if (r < 0 || ce != cudaSuccess || !graph) {
    if (graph) cudaGraphDestroy(graph);
    cudaGetLastError();
    return -2;
  }
  const cudaError_t ie = cudaGraphInstantiate(&b->graph, graph, 0);
  cudaGraphDestroy(graph);
  if (ie != cudaSuccess) {
    b->graph = nullptr;
    cudaGetLastError();
    return -2;
  }
  b->graph_points = b->npoints;
  b->graph_jobs = b->njobs;
  return 0;
}

int tlb_graph_launch(tl_batch* b, void* stream) {
  if (!b || !b->graph) return -1;
  if (b->npoints != b->graph_points || b->njobs != b->graph_jobs) return -1;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  cudaStream_t st = pick(stream);
  E.fill_after(st);
  const bool ok = E.check(cudaGraphLaunch(b->graph, st));
  E.fill_mark(st);
  return ok ? 0 : -2;
}

static long point_lc_body(tl_batch* b, double* amp) {
  if (!b || b->ntraj <= 0 || !amp) return -1;
  tl::Engine& E = tl::Engine::get();
  std::lock_guard<std::mutex> g(E.mu);
  // point-source sampling uses n points per curve (t = i/(n-1)); reuse the
  // IRS layout (n+1 slots per curve) and leave the last slot unused
  std::vector<tl::SeedJob> jobs;
  for (int t = 0; t < b->ntraj; t++) tl::plan_jobs(&jobs, t, (long)b->htraj[t].n, b->chain, -1);
  tl::DevBuf dj;
  void* djp = dj.need(sizeof(tl::SeedJob) * jobs.size());
  double* da = (double*)b->amp.need(sizeof(double) * b->npoints);
  if (!djp || !da) {
    if (djp) cudaFree(djp);
    return -2;
  }
  E.check(cudaMemsetAsync(da, 0, sizeof(double) * b->npoints, E.stream));
  E.check(tl::copy_async(djp, jobs.data(), sizeof(tl::SeedJob) * jobs.size(),
                          cudaMemcpyHostToDevice, E.stream));
  if (b->chain <= 0)
    tl::launch_point_lc_exact((const tl::Traj*)b->trajs.p, (const tl::SeedJob*)djp,
                              (int)jobs.size(), (const tl::DevLens*)b->lenses.p, da, nullptr,
                              E.stream);
  else
    tl::launch_point_lc((const tl::Traj*)b->trajs.p, (const tl::SeedJob*)djp, (int)jobs.size(),
                        (const tl::DevLens*)b->lenses.p, da, nullptr, E.stream);
  E.check(cudaStreamSynchronize(E.stream));
  E.check(tl::copy_async(amp, da, sizeof(double) * b->npoints, cudaMemcpyDeviceToHost, E.stream));
  bool ok = E.check(cudaStreamSynchronize(E.stream));
  cudaFree(djp);
  return ok ? b->npoints : -2;
}

// entry points that allocate host memory
int tlb_set_lenses(tl_batch* b, int nlens, const double* p8) {
  return guarded(-2, [&] { return set_lenses_body(b, nlens, p8); });
}

long tlb_set_trajectories(tl_batch* b, int ntraj, const double* t4, const int32_t* lens_idx,
                          const uint32_t* n) {
  return guarded(-2L, [&] { return set_trajectories_body(b, ntraj, t4, lens_idx, n); });
}

int tlb_download(tl_batch* b, double* amp, uint64_t* counts, uint32_t* status, void* stream) {
  return guarded(-2, [&] { return download_body(b, amp, counts, status, stream); });
}

long tlb_run_host(tl_batch* b, int ntraj, const double* t4, const int32_t* lens_idx,
                  const uint32_t* n, double* amp, uint64_t* counts, uint32_t* status,
                  void* stream) {
  return guarded(-2L, [&] {
    return run_host_body(b, ntraj, t4, lens_idx, n, amp, counts, status, stream);
  });
}

long tlb_point_lc(tl_batch* b, double* amp) {
  return guarded(-2L, [&] { return point_lc_body(b, amp); });
}

}  // extern "C"
