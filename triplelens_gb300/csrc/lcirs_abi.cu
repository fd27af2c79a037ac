// lcirs_abi.cu - LightCurveIRS class and the reference's C ABI on top of the
// GPU engine (seeds.cu, fill.cu).
//
// Reference interface replaced: src/LightCurves/lcirs.cc:515-609 (extern "C"
// block) and the LightCurveIRS class (src/LightCurves/lcirs.h:30-116).
// Everything numeric runs on the GPU: critical curve/caustics/grid
// (lens_setup_kernel), images and seeds (seeds_kernel), the amoeba fill
// (fill_kernel).  The host builds descriptors, moves data and prints the
// reference's per-point lines.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <fstream>
#include <iostream>
#include <chrono>
#include <condition_variable>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "engine.h"
#include "engine_host.h"
#include "plan.h"
#include "lcirs.hpp"

using tl::cx;

struct LightCurveIRS::Impl {
  tl::LensSpec spec;
  tl::DevLens lens;         // host copy
  tl::DevLens* d_lens = nullptr;
  cx* d_cc = nullptr;
  cx* d_ca = nullptr;
  // the image solver's warm-start state, carried from call to call as the
  // reference's ImgPoint member carries it (imgpoint.h:104-110)
  tl::RootChain* d_chain = nullptr;
  std::vector<double> lcFull;  // n+1 magnifications
  // the object's own stream and buffers: objects used from different host
  // threads set up and seed concurrently; their fills take turns on the
  // engine's tables
  cudaStream_t st = nullptr;
  int dev = -1;             // the device current when the object was set up
  tl::RunBufs bufs;
  tl::DevBuf specbuf, ampbuf;
  bool failed = false;
  bool fresh = true;        // no get_lc_irs yet
  // parameters the lens set-up cannot use (status 32, bad input), or a
  // set-up whose device memory could not be had (0x100): the object runs
  // nothing on the GPU, and its calls report invalid_status on every point
  bool invalid = false;
  uint32_t invalid_status = tl::kStBadInput;
  bool ck(cudaError_t e) {
    if (e != cudaSuccess) {
      fprintf(stderr, "liblcirs: CUDA error %s\n", cudaGetErrorString(e));
      failed = true;
      return false;
    }
    return true;
  }
};

namespace {

// objects that have not run get_lc_irs yet: while there are any, a batch
// waits longer for callers (they are likely on their way)
std::atomic<int> g_fresh{0};
// constructors running now (their lens set-up takes tens of ms): a batch
// keeps gathering while there are any, within its time cap
std::atomic<int> g_constructing{0};

void setup_object(LightCurveIRS* o) {
  tl::Engine& E = tl::Engine::get();
  E.trace("setup_object: lens set-up");
  auto* I = o->impl;
  I->spec = tl::make_lens_spec(o->a, o->b, o->th, o->m2, o->m3, o->sourceRadius,
                               o->pointsPerRadius, o->ldA, o->ldB, o->intensityCoeff);
  if (!I->d_lens) {
    I->ck(cudaGetDevice(&I->dev));
    I->ck(cudaStreamCreateWithFlags(&I->st, cudaStreamNonBlocking));
    I->ck(cudaMallocAsync(&I->d_lens, sizeof(tl::DevLens), I->st));
    I->ck(cudaMallocAsync(&I->d_cc, sizeof(cx) * tl::kBranches * tl::kCCLen, I->st));
    I->ck(cudaMallocAsync(&I->d_ca, sizeof(cx) * tl::kBranches * tl::kCCLen, I->st));
    I->ck(cudaMallocAsync(&I->d_chain, sizeof(tl::RootChain), I->st));
  }
  tl::LensSpec* d_spec = (tl::LensSpec*)I->specbuf.need(sizeof(tl::LensSpec), I->st);
  if (I->failed || !I->d_lens || !I->d_cc || !I->d_ca || !I->d_chain || !d_spec) {
    // no stream or device memory for the set-up: kept off the GPU
    I->invalid = true;
    I->invalid_status = 0x100u;
    return;
  }
  I->ck(tl::copy_async(d_spec, &I->spec, sizeof(tl::LensSpec), cudaMemcpyHostToDevice, I->st));
  {
    tl::NvtxRange range("tl lens set-up");
    tl::launch_lens_setup(d_spec, 1, I->d_lens, I->d_cc, I->d_ca, I->st);
  }
  // every copy into pageable host memory waits for its stream first: such a
  // copy holds the driver's staging path while it waits, and would stall the
  // copies of every other host thread behind a long kernel
  I->ck(cudaStreamSynchronize(I->st));
  I->ck(tl::copy_async(&I->lens, I->d_lens, sizeof(tl::DevLens), cudaMemcpyDeviceToHost, I->st));
  I->ck(cudaStreamSynchronize(I->st));
  // a fresh object's solver: no roots yet, the constructor's heap state
  tl::RootChain ch;
  tl::chain_reset(&ch, I->lens.heap0);
  I->ck(tl::copy_async(I->d_chain, &ch, sizeof(ch), cudaMemcpyHostToDevice, I->st));
  I->ck(cudaStreamSynchronize(I->st));
  E.trace("setup_object: done");
  const tl::Grid& g2 = I->lens.g;
  o->grid[0] = g2.corner_x;
  o->grid[1] = g2.corner_y;
  o->grid[2] = g2.top_x;
  o->grid[3] = g2.top_y;
  o->grid[4] = g2.size_double;
  o->grid[5] = g2.h;
  o->grid[6] = g2.amp_scale;
  o->grid[7] = (double)g2.n;
}

}  // namespace

LightCurveIRS::LightCurveIRS(double a_, double b_, double th_, double m2_, double m3_,
                             double sourceSize, unsigned int lcLength_, long ppr)
    : a(a_), b(b_), th(th_), m1(1.0 - m2_ - m3_), m2(m2_), m3(m3_), sourceRadius(sourceSize),
      lcLength(lcLength_), pointsPerRadius(ppr) {
  impl = new Impl();
  // default limb darkening A = 0.6, B = 0.4 (limbdarkeningmodel.cc:8-15)
  ldA = 0.6;
  ldB = 0.4;
  intensityCoeff = 1.0 / (ldA + 2.0 / 3.0 * ldB);
  lcVec.assign(lcLength, 0.0);
  impl->lcFull.assign((size_t)lcLength + 1, 0.0);
  for (double& g : grid) g = 0.0;
  // a non-finite parameter, a source radius <= 0 or a ray density outside
  // 1..2^31-1 would give the lens set-up no usable grid (the reference's
  // arithmetic is undefined there): such an object exists, as the
  // reference's does, but never reaches the GPU
  if (!(std::isfinite(a_) && std::isfinite(b_) && std::isfinite(th_) && std::isfinite(m2_) &&
        std::isfinite(m3_) && std::isfinite(sourceSize) && sourceSize > 0.0 && ppr >= 1 &&
        ppr <= 2147483647L)) {
    impl->invalid = true;
    impl->fresh = false;
    lastStatus = tl::kStBadInput;
    return;
  }
  // counted from the start of its construction until its first get_lc_irs
  // (batching window): objects still in their lens set-up (tens of ms) when
  // another object calls are on their way too; counted only after it, a
  // first caller could find none and run alone
  g_fresh.fetch_add(1);
  g_constructing.fetch_add(1);
  setup_object(this);
  g_constructing.fetch_sub(1);
  if (impl->invalid) {   // the set-up could not run
    lastStatus = impl->invalid_status;
    impl->fresh = false;
    g_fresh.fetch_sub(1);
  }
}

LightCurveIRS::~LightCurveIRS() {
  if (impl && !impl->invalid) tl::Engine::get().trace("delete object");
  if (impl && impl->fresh) g_fresh.fetch_sub(1);
  if (impl) {
    // stream-ordered releases: no wait for work on other streams
    cudaStream_t st = impl->st;
    for (void* q : {(void*)impl->d_lens, (void*)impl->d_cc, (void*)impl->d_ca,
                    (void*)impl->d_chain})
      if (q) cudaFreeAsync(q, st);
    for (tl::DevBuf* d : {&impl->bufs.trajs, &impl->bufs.jobs, &impl->bufs.scan, &impl->bufs.prep,
                          &impl->bufs.points, &impl->bufs.seeds, &impl->bufs.out,
                          &impl->bufs.trials, &impl->bufs.dump, &impl->specbuf, &impl->ampbuf})
      d->release(st);
    if (st) {
      cudaStreamSynchronize(st);
      cudaStreamDestroy(st);
    }
    delete impl;
  }
}

void LightCurveIRS::setLimbDarkening(const std::string& model, double v) {
  if (!impl->invalid) tl::Engine::get().trace("setLimbDarkening");
  // limbdarkeningmodel.cc:18-28 ("linear") and 8-15 (anything else)
  setLimbDarkeningModel(model == "linear" ? LimbDarkeningModel(v) : LimbDarkeningModel());
}

void LightCurveIRS::setLimbDarkeningModel(LimbDarkeningModel ldm) {
  applyLimbDarkening(ldm.getParA(), ldm.getParB(), ldm.intensityCoeff);
}

void LightCurveIRS::applyLimbDarkening(double A, double B, double intensity) {
  ldA = A;
  ldB = B;
  intensityCoeff = intensity;
  // _ampScale = intensityCoeff/pi/ppr^2 (lcirs.cc:94-101)
  const double ppr = (double)(int)pointsPerRadius;
  grid[6] = intensityCoeff / 3.14159265358979323846 / (ppr * ppr);
  impl->lens.g.amp_scale = grid[6];
  impl->lens.ld_a = ldA;
  impl->lens.ld_b = ldB;
  impl->spec.ld_a = ldA;
  impl->spec.ld_b = ldB;
  impl->spec.intensity = intensityCoeff;
  if (impl->invalid) return;   // no device lens
  impl->ck(tl::copy_async(impl->d_lens, &impl->lens, sizeof(tl::DevLens), cudaMemcpyHostToDevice,
                           impl->st));
  impl->ck(cudaStreamSynchronize(impl->st));
}

void LightCurveIRS::setAmoebaPrintOut(bool on, std::string amoebaFilename,
                                      std::string parFilename) {
  amoebaPrintOut_ = on;
  amoebaFilename_ = amoebaFilename;
  parFilename_ = parFilename;
}

// lcirs.cc:479-512 (including the reference's "m3" field written with m2)
void LightCurveIRS::printOutLCParameters() {
  std::ofstream f(parFilename_);
  const char* ind = "\t";
  f << "{" << '\n';
  f << ind << "\"sourceRadius\": " << sourceRadius << ",\n";
  f << ind << "\"pointsPerRadius\": " << (int)pointsPerRadius << ",\n";
  f << ind << "\"imgPlaneSize\": " << impl->lens.g.n << ",\n";
  f << ind << "\"imgPlaneSizeDouble\": " << impl->lens.g.size_double << ",\n";
  f << ind << "\"bottomLeftCornerImgX\": " << impl->lens.g.corner_x << ",\n";
  f << ind << "\"bottomLeftCornerImgY\": " << impl->lens.g.corner_y << ",\n";
  f << ind << "\"topRightCornerImgX\": " << impl->lens.g.top_x << ",\n";
  f << ind << "\"topRightCornerImgY\": " << impl->lens.g.top_y << ",\n";
  f << ind << "\"a\": " << a << ",\n";
  f << ind << "\"b\": " << b << ",\n";
  f << ind << "\"th\": " << th << ",\n";
  f << ind << "\"m1\": " << m1 << ",\n";
  f << ind << "\"m2\": " << m2 << ",\n";
  f << ind << "\"m3\": " << m2 << ",\n";
  f << ind << "\"z1x\": " << 0.0 << ",\n";
  f << ind << "\"z1y\": " << 0.0 << ",\n";
  f << ind << "\"z2x\": " << impl->lens.L.z2.re << ",\n";
  f << ind << "\"z2y\": " << impl->lens.L.z2.im << ",\n";
  f << ind << "\"z3x\": " << impl->lens.L.z3.re << ",\n";
  f << ind << "\"z3y\": " << impl->lens.L.z3.im << "\n";
  f << "}";
}

namespace {

// Per-point results of a curve (its n+1 PointOut records) into the object:
// counts, status, magnifications, statistics, and the reference's per-point
// stdout lines (lcirs.cc:121-122, 176-177).
void absorb_results(LightCurveIRS* o, std::complex<double> s, std::complex<double> e,
                    const tl::PointOut* hout, bool failed) {
  const uint32_t n = o->lcLength;
  const size_t np = (size_t)n + 1;
  o->counts.resize(np);
  o->status.resize(np);
  o->diag.resize(np);
  o->nseeds.resize(np);
  o->lastStatus = failed ? 0x100u : 0u;
  o->stats[0] = o->stats[1] = o->stats[2] = 0;
  const double scale = o->impl->lens.g.amp_scale;
  for (size_t i = 0; i < np; i++) {
    o->counts[i] = hout[i].count;
    o->status[i] = hout[i].status;
    o->diag[i] = hout[i].diag;
    o->nseeds[i] = (int32_t)hout[i].nseeds;
    o->lastStatus |= hout[i].status;
    o->stats[0] += hout[i].rays_eval;
    o->stats[1] += hout[i].rays_fp64;
    o->stats[2] += hout[i].tiles;
    const double wsum = (double)hout[i].wsum_fx / tl::kWsumScale;
    o->impl->lcFull[i] = wsum * scale;
  }
  for (size_t i = 0; i < n; i++) o->lcVec[i] = o->impl->lcFull[i];
  if (o->verbose) {
    std::cout << "IRS called with imgPlaneSize:" << o->impl->lens.g.n << "\n";
    for (size_t i = 0; i < np; i++) {
      const double t = double(i) / double(n);
      const double px = s.real() + (e.real() - s.real()) * t;
      const double py = s.imag() + (e.imag() - s.imag()) * t;
      std::cout << "started pos:" << i << ", (" << px << "," << py << ")\n";
      std::cout << "irs amplification: " << o->impl->lcFull[i] << " and the count "
                << o->counts[i] << " and amp scale " << scale << "\n";
    }
  }
}

// ---------------------------------------------------------------------------
// Dynamic batching of concurrent get_lc_irs calls.
//
// The fill kernel is persistent and occupies every SM, so objects that run
// their own launches from different host threads mostly wait for each
// other.  Instead, a call queues its request; the first caller that finds no
// batch running becomes the leader, waits until requests stop arriving (a
// gap of 3 ms, 15 ms while objects exist that have not called yet, and no
// object still in its constructor; at most 300 ms), and runs every queued
// request with its chain and precision
// settings as one batch: the seeds (a chain per curve; the exact chain in
// segments overlapped with the fill) and the fill, on the batcher's stream.
// Every caller then finds its results in its object, exactly as a lone call
// would leave them.  A lone caller pays the 3 ms window once.
// ---------------------------------------------------------------------------
struct Request {
  LightCurveIRS* obj;
  std::complex<double> s, e;
  int chain;       // 0: exact chain, else chunk length
  int precision;
  bool done = false;
};

struct Batcher {
  std::mutex mu;
  std::condition_variable cv;
  std::vector<Request*> pending;
  bool running = false;
  uint64_t arrivals = 0;
  cudaStream_t st = nullptr;
  tl::RunBufs bufs;
  tl::DevBuf lenses, ca, chains, segjobs, seglist, segn;
  std::vector<tl::PointOut> hout;
  std::vector<int32_t> hseeds;
};

Batcher& batcher() {
  static Batcher* b = new Batcher();
  return *b;
}

// Runs one batch of requests that share chain mode and precision.
// segments of the exact chain in a batch (each segment's fill overlaps the
// next segment's chain)
constexpr int kBatchSegments = 8;

void run_batch(Batcher& B, const std::vector<Request*>& reqs) {
  tl::NvtxRange range("tl object batch");
  tl::Engine& E = tl::Engine::get();
  if (!B.st) cudaStreamCreateWithFlags(&B.st, cudaStreamNonBlocking);
  const int k = (int)reqs.size();
  const int chain = reqs[0]->chain, precision = reqs[0]->precision;
  bool failed = false;
  auto ck = [&](cudaError_t err) {
    if (err != cudaSuccess) {
      fprintf(stderr, "liblcirs: CUDA error %s\n", cudaGetErrorString(err));
      failed = true;
    }
  };
  std::vector<tl::Traj> trajs(k);
  std::vector<tl::SeedJob> jobs, scan;
  std::vector<size_t> base(k + 1, 0);
  for (int i = 0; i < k; i++) {
    LightCurveIRS* o = reqs[i]->obj;
    tl::Traj& T = trajs[i];
    T.x0 = reqs[i]->s.real();
    T.y0 = reqs[i]->s.imag();
    T.x1 = reqs[i]->e.real();
    T.y1 = reqs[i]->e.imag();
    T.n = o->lcLength;
    T.lens = i;
    T.point_base = (int64_t)base[i];
    const long np = (long)o->lcLength + 1;
    tl::plan_jobs(&jobs, i, np, chain, i);
    if (chain <= 0) tl::plan_jobs(&scan, i, np, tl::kChainChunk, -1);
    base[i + 1] = base[i] + (size_t)np;
  }
  const size_t total = base[k];
  tl::Run R = B.bufs.prepare(total, k, jobs.size(), false, scan.size(), B.st);
  auto* dl = (tl::DevLens*)B.lenses.need(sizeof(tl::DevLens) * k, B.st);
  auto* dca = (cx*)B.ca.need(sizeof(cx) * tl::kBranches * tl::kCCLen * k, B.st);
  auto* dch = (tl::RootChain*)B.chains.need(sizeof(tl::RootChain) * k, B.st);
  if (!R.ok || !dl || !dca || !dch) {   // device memory exhausted: launch nothing
    fprintf(stderr, "liblcirs: device allocation for a batch of %d curves failed\n", k);
    for (Request* q : reqs) q->obj->lastStatus = 0x100u;
    return;
  }
  // gather the objects' lenses, caustics and warm-start chains
  for (int i = 0; i < k; i++) {
    const LightCurveIRS::Impl* I = reqs[i]->obj->impl;
    ck(tl::copy_async(dl + i, I->d_lens, sizeof(tl::DevLens), cudaMemcpyDeviceToDevice, B.st));
    ck(tl::copy_async(dca + (size_t)i * tl::kBranches * tl::kCCLen, I->d_ca,
                       sizeof(cx) * tl::kBranches * tl::kCCLen, cudaMemcpyDeviceToDevice, B.st));
    ck(tl::copy_async(dch + i, I->d_chain, sizeof(tl::RootChain), cudaMemcpyDeviceToDevice,
                       B.st));
  }
  ck(tl::copy_async(R.trajs, trajs.data(), sizeof(tl::Traj) * k, cudaMemcpyHostToDevice, B.st));
  ck(tl::copy_async(R.jobs, jobs.data(), sizeof(tl::SeedJob) * jobs.size(),
                     cudaMemcpyHostToDevice, B.st));
  if (chain <= 0) {
    // the exact chain in segments, each segment's fill beside the next
    // segment's chain; every curve continues from its object's chain state
    ck(tl::copy_async(R.scan_jobs, scan.data(), sizeof(tl::SeedJob) * scan.size(),
                       cudaMemcpyHostToDevice, B.st));
    const int S = kBatchSegments;
    std::vector<tl::SeedJob> sj;
    std::vector<int32_t> sl;
    std::vector<unsigned> sn;
    std::vector<int> segoff, segjob0;
    std::vector<int64_t> pb(k);
    std::vector<uint32_t> nn(k);
    for (int i = 0; i < k; i++) {
      pb[i] = (int64_t)base[i];
      nn[i] = trajs[i].n;
    }
    tl::plan_segments(S, k, pb.data(), nn.data(), &sj, &sl, &sn, &segjob0, &segoff);
    auto* dsj = (tl::SeedJob*)B.segjobs.need(sizeof(tl::SeedJob) * sj.size(), B.st);
    auto* dsl = (int32_t*)B.seglist.need(sizeof(int32_t) * sl.size(), B.st);
    auto* dsn = (unsigned*)B.segn.need(sizeof(unsigned) * S, B.st);
    if (!dsj || !dsl || !dsn) {
      fprintf(stderr, "liblcirs: device allocation for a batch of %d curves failed\n", k);
      for (Request* q : reqs) q->obj->lastStatus = 0x100u;
      return;
    }
    ck(tl::copy_async(dsj, sj.data(), sizeof(tl::SeedJob) * sj.size(), cudaMemcpyHostToDevice,
                       B.st));
    ck(tl::copy_async(dsl, sl.data(), sizeof(int32_t) * sl.size(), cudaMemcpyHostToDevice,
                       B.st));
    ck(tl::copy_async(dsn, sn.data(), sizeof(unsigned) * S, cudaMemcpyHostToDevice, B.st));
    tl::Pipeline P;
    P.lenses = dl;
    P.ca = dca;
    P.scan = R.scan_jobs;
    P.nscan = (int)scan.size();
    P.ntraj = k;
    P.segjobs = dsj;
    P.segjob0 = segjob0.data();
    P.seglist = dsl;
    P.segoff = segoff.data();
    P.segn = dsn;
    P.nseg = S;
    P.prep = R.prep;
    P.chains = dch;
    P.reset_chains = false;
    std::lock_guard<std::mutex> g(E.mu);
    if (!E.pipeline_exact(R, total, P, precision, B.st)) failed = true;
  } else {
    tl::launch_seeds(R.jobs, (int)jobs.size(), R.trajs, dl, dca, R.points, R.seeds, R.out,
                     R.trials, dch, B.st);
    std::lock_guard<std::mutex> g(E.mu);
    if (!E.fill_on(R, total, dl, precision, B.st)) failed = true;
  }
  // the chains go back to their objects
  for (int i = 0; i < k; i++)
    ck(tl::copy_async(reqs[i]->obj->impl->d_chain, dch + i, sizeof(tl::RootChain),
                       cudaMemcpyDeviceToDevice, B.st));
  B.hout.resize(total);
  B.hseeds.resize(total * 2 * tl::kMaxSeeds);
  ck(cudaStreamSynchronize(B.st));   // before the pageable copies (see setup_object)
  ck(tl::copy_async(B.hout.data(), R.out, sizeof(tl::PointOut) * total, cudaMemcpyDeviceToHost,
                     B.st));
  ck(tl::copy_async(B.hseeds.data(), R.seeds, sizeof(int32_t) * 2 * tl::kMaxSeeds * total,
                     cudaMemcpyDeviceToHost, B.st));
  ck(cudaStreamSynchronize(B.st));
  for (int i = 0; i < k; i++) {
    LightCurveIRS* o = reqs[i]->obj;
    const size_t np = base[i + 1] - base[i];
    o->seeds.assign(B.hseeds.begin() + (ptrdiff_t)(base[i] * 2 * tl::kMaxSeeds),
                    B.hseeds.begin() + (ptrdiff_t)(base[i + 1] * 2 * tl::kMaxSeeds));
    (void)np;
    absorb_results(o, reqs[i]->s, reqs[i]->e, B.hout.data() + base[i], failed);
  }
}

}  // namespace

void LightCurveIRS::runBatched(std::complex<double> s, std::complex<double> e) {
  Batcher& B = batcher();
  Request r;
  r.obj = this;
  r.s = s;
  r.e = e;
  r.chain = chainPoints <= 0 ? 0 : chainPoints;
  r.precision = precision;
  std::unique_lock<std::mutex> lk(B.mu);
  B.pending.push_back(&r);
  B.arrivals++;
  B.cv.notify_all();
  while (!r.done) {
    if (!B.running) {
      B.running = true;
      // gather callers: until a quiet gap of 3 ms (15 ms while objects that
      // have not called yet exist) with no constructor running, at most
      // 300 ms
      tl::gather_callers(lk, B.cv, B.arrivals, g_fresh, g_constructing);
      std::vector<Request*> mine, rest;
      for (Request* q : B.pending)
        (q->chain == r.chain && q->precision == r.precision ? mine : rest).push_back(q);
      B.pending.swap(rest);
      lk.unlock();
      tl::Engine& E = tl::Engine::get();
      if (E.tracing) {
        char msg[96];
        snprintf(msg, sizeof msg, "batch of %zu curves (%zu left queued)", mine.size(),
                 B.pending.size());
        E.trace(msg);
      }
      try {
        run_batch(B, mine);
      } catch (const std::exception& ex) {
        // host allocation failure: the callers get the error bit, and the
        // batcher stays usable (no caller is left waiting on this batch)
        fprintf(stderr, "liblcirs: batch of %zu curves failed: %s\n", mine.size(), ex.what());
        for (Request* q : mine) q->obj->lastStatus = 0x100u;
      }
      E.trace("batch done");
      lk.lock();
      for (Request* q : mine) q->done = true;
      B.running = false;
      B.cv.notify_all();
    } else {
      B.cv.wait(lk);
    }
  }
}

void LightCurveIRS::unusableResults() {
  const size_t np = (size_t)lcLength + 1;
  counts.assign(np, 0);
  status.assign(np, impl->invalid_status);
  diag.assign(np, 0);
  nseeds.assign(np, 0);
  seeds.assign(np * 2 * tl::kMaxSeeds, 0);
  for (double& v : lcVec) v = 0.0;
  for (double& v : impl->lcFull) v = 0.0;
  stats[0] = stats[1] = stats[2] = 0;
  lastStatus = impl->invalid_status;
}

void LightCurveIRS::runFill(std::complex<double> s, std::complex<double> e,
                            const int32_t* extSeeds, const int32_t* extN) {
  if (impl->invalid) {
    unusableResults();
    return;
  }
  tl::Engine& E = tl::Engine::get();
  auto* I = impl;
  I->failed = false;
  const uint32_t n = lcLength;
  const size_t np = (size_t)n + 1;
  tl::Traj T;
  T.x0 = s.real();
  T.y0 = s.imag();
  T.x1 = e.real();
  T.y1 = e.imag();
  T.n = n;
  T.lens = 0;
  T.point_base = 0;
  std::vector<tl::SeedJob> jobs, scan;
  tl::plan_jobs(&jobs, 0, (long)np, chainPoints, 0);
  if (chainPoints <= 0) tl::plan_jobs(&scan, 0, (long)np, tl::kChainChunk, -1);
  E.trace("runFill: prepare");
  tl::Run R = I->bufs.prepare(np, 1, jobs.size(), amoebaPrintOut_, scan.size(), I->st);
  if (!R.ok) {   // device memory exhausted: launch nothing
    I->failed = true;
    lastStatus = 0x100u;
    return;
  }
  I->ck(tl::copy_async(R.trajs, &T, sizeof(T), cudaMemcpyHostToDevice, I->st));
  I->ck(tl::copy_async(R.jobs, jobs.data(), sizeof(tl::SeedJob) * jobs.size(),
                          cudaMemcpyHostToDevice, I->st));
  if (chainPoints <= 0) {
    I->ck(tl::copy_async(R.scan_jobs, scan.data(), sizeof(tl::SeedJob) * scan.size(),
                            cudaMemcpyHostToDevice, I->st));
    tl::launch_seeds_exact(R.scan_jobs, (int)scan.size(), R.jobs, (int)jobs.size(), R.trajs,
                           impl->d_lens, impl->d_ca, R.points, R.seeds, R.out, R.trials, R.prep,
                           impl->d_chain, I->st);
  } else {
    tl::launch_seeds(R.jobs, (int)jobs.size(), R.trajs, impl->d_lens, impl->d_ca, R.points,
                     R.seeds, R.out, R.trials, impl->d_chain, I->st);
  }
  if (extSeeds) {
    // replace the seeds with the caller's, keep the positions
    std::vector<tl::PointOut> hout(np);
    I->ck(cudaStreamSynchronize(I->st));
    I->ck(tl::copy_async(hout.data(), R.out, sizeof(tl::PointOut) * np, cudaMemcpyDeviceToHost,
                            I->st));
    I->ck(cudaStreamSynchronize(I->st));
    for (size_t i = 0; i < np; i++) {
      hout[i].nseeds = (uint32_t)std::max(0, std::min(extN[i], tl::kMaxSeeds));
      hout[i].status = 0;
    }
    I->ck(tl::copy_async(R.out, hout.data(), sizeof(tl::PointOut) * np, cudaMemcpyHostToDevice,
                            I->st));
    I->ck(tl::copy_async(R.seeds, extSeeds, sizeof(int32_t) * 2 * tl::kMaxSeeds * np,
                            cudaMemcpyHostToDevice, I->st));
  }
  E.trace("runFill: seeds launched");
  if (E.sync_steps) {
    I->ck(cudaStreamSynchronize(I->st));
    E.trace("runFill: seeds done");
  }
  {
    // the fill tables are the engine's: one launch sequence at a time
    std::lock_guard<std::mutex> g(E.mu);
    if (!E.fill_on(R, np, impl->d_lens, precision, I->st)) I->failed = true;
  }
  E.trace("runFill: fill launched");
  if (E.sync_steps) {
    I->ck(cudaStreamSynchronize(I->st));
    E.trace("runFill: fill done");
  }
  I->ck(cudaStreamSynchronize(I->st));   // before the pageable copies (see setup_object)
  std::vector<tl::PointOut> hout(np);
  I->ck(tl::copy_async(hout.data(), R.out, sizeof(tl::PointOut) * np, cudaMemcpyDeviceToHost,
                          I->st));
  seeds.resize(np * 2 * tl::kMaxSeeds);
  nseeds.resize(np);
  I->ck(tl::copy_async(seeds.data(), R.seeds, sizeof(int32_t) * 2 * tl::kMaxSeeds * np,
                          cudaMemcpyDeviceToHost, I->st));
  std::vector<uint32_t> dump;
  unsigned ndump = 0;
  if (amoebaPrintOut_) {
    I->ck(tl::copy_async(&ndump, R.dump_count, sizeof(unsigned), cudaMemcpyDeviceToHost,
                            I->st));
  }
  I->ck(cudaStreamSynchronize(I->st));
  if (amoebaPrintOut_) {
    if (ndump > R.dump_cap) {
      std::cout << "amoeba dump truncated: " << ndump << " tiles, capacity " << R.dump_cap << "\n";
      ndump = R.dump_cap;
    }
    dump.resize((size_t)ndump * tl::kDumpWords);
    I->ck(cudaMemcpy(dump.data(), R.dump, sizeof(uint32_t) * dump.size(),
                       cudaMemcpyDeviceToHost));
  }
  E.trace("runFill: results copied");
  absorb_results(this, s, e, hout.data(), I->failed);
  if (amoebaPrintOut_) {
    // rows of every point from its tile masks: maximal runs, merged across
    // neighbouring tiles (amoeba.cc:90-108 writes "ny,xleft,xright")
    std::vector<std::vector<std::pair<int64_t, std::pair<int64_t, int64_t>>>> per(np);
    for (unsigned d = 0; d < ndump; d++) {
      const uint32_t* r = &dump[(size_t)d * tl::kDumpWords];
      const uint32_t p = r[0];
      if (p >= np) continue;
      const int64_t tx = r[1], ty = r[2];
      for (int row = 0; row < 8; row++) {
        uint32_t m = r[3 + row];
        while (m) {
          const int lo = __builtin_ctz(m);
          const uint32_t sh = m >> lo;
          const int len = (~sh == 0u) ? 32 - lo : __builtin_ctz(~sh);
          per[p].push_back({ty * 8 + row, {tx * 32 + lo, tx * 32 + lo + len - 1}});
          m &= (len + lo >= 32) ? 0u : ~((1u << (lo + len)) - 1u);
        }
      }
    }
    for (size_t i = 0; i < np; i++) {
      auto& v = per[i];
      std::sort(v.begin(), v.end());
      std::ofstream f(amoebaFilename_ + std::to_string(i));
      for (size_t k = 0; k < v.size();) {
        const int64_t ny = v[k].first;
        int64_t xl = v[k].second.first, xr = v[k].second.second;
        size_t q = k + 1;
        while (q < v.size() && v[q].first == ny && v[q].second.first == xr + 1) {
          xr = v[q].second.second;
          q++;
        }
        f << ny << "," << xl << "," << xr << "\n";
        k = q;
      }
    }
  }
}

void LightCurveIRS::getLCIRS(std::complex<double> s, std::complex<double> e) {
  if (impl->fresh) {
    impl->fresh = false;
    g_fresh.fetch_sub(1);
  }
  if (impl->invalid) {
    unusableResults();
    return;
  }
  if (amoebaPrintOut_) {
    printOutLCParameters();
    runFill(s, e, nullptr, nullptr);   // the amoeba dump needs the object's own run
  } else {
    runBatched(s, e);
  }
}

void LightCurveIRS::getLC(std::complex<double> s, std::complex<double> e) {
  auto* I = impl;
  const uint32_t n = lcLength;
  if (I->invalid) {
    for (double& v : lcVec) v = 0.0;
    for (double& v : I->lcFull) v = 0.0;
    lastStatus = I->invalid_status;
    return;
  }
  if (n == 0) return;
  tl::Traj T;
  T.x0 = s.real();
  T.y0 = s.imag();
  T.x1 = e.real();
  T.y1 = e.imag();
  T.n = n;
  T.lens = 0;
  T.point_base = 0;
  std::vector<tl::SeedJob> jobs;
  tl::plan_jobs(&jobs, 0, (long)n, chainPoints, 0);
  tl::Run R = I->bufs.prepare(n, 1, jobs.size(), false, 0, I->st);
  if (!R.ok) {   // device memory exhausted: launch nothing
    lastStatus = 0x100u;
    return;
  }
  I->ck(tl::copy_async(R.trajs, &T, sizeof(T), cudaMemcpyHostToDevice, I->st));
  I->ck(tl::copy_async(R.jobs, jobs.data(), sizeof(tl::SeedJob) * jobs.size(),
                          cudaMemcpyHostToDevice, I->st));
  double* d_amp = (double*)I->ampbuf.need(sizeof(double) * n, I->st);
  if (!d_amp) {   // device memory exhausted: launch nothing
    lastStatus = 0x100u;
    return;
  }
  if (chainPoints <= 0)
    tl::launch_point_lc_exact(R.trajs, R.jobs, (int)jobs.size(), impl->d_lens, d_amp,
                              impl->d_chain, I->st);
  else
    tl::launch_point_lc(R.trajs, R.jobs, (int)jobs.size(), impl->d_lens, d_amp, impl->d_chain,
                        I->st);
  I->ck(cudaStreamSynchronize(I->st));   // before the pageable copy (see setup_object)
  I->ck(tl::copy_async(lcVec.data(), d_amp, sizeof(double) * n, cudaMemcpyDeviceToHost,
                          I->st));
  I->ck(cudaStreamSynchronize(I->st));
  for (size_t i = 0; i < n; i++) impl->lcFull[i] = lcVec[i];
}

// ---------------------------------------------------------------------------
// C ABI (src/LightCurves/lcirs.cc:515-609 and additive entry points)
// ---------------------------------------------------------------------------
namespace tl {
const DevLens* object_device_lens(const LightCurveIRS* lc) { return lc->impl->d_lens; }
int object_device(const LightCurveIRS* lc) { return lc->impl->dev; }
}  // namespace tl

extern "C" {

LightCurveIRS* lcirs_new(double a, double b, double th, double m2, double m3, double sourceSize,
                         unsigned int lcLength, long pointsPerRadius) {
  return new LightCurveIRS(a, b, th, m2, m3, sourceSize, lcLength, pointsPerRadius);
}

void get_lc(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY) {
  lc->getLC({iniX, iniY}, {finX, finY});
}

void get_lc_irs(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY) {
  lc->getLCIRS({iniX, iniY}, {finX, finY});
}

void copy_lc(LightCurveIRS* lc, double* out) {
  const size_t n = lc->lcVec.size();
  for (size_t i = 0; i < n; i++) out[i] = lc->lcVec[i];
}

void set_limb_darkening(LightCurveIRS* lc, const char* model, double v) {
  if (strcmp(model, "linear") == 0) {
    std::cout << "model is linear\n";
    lc->setLimbDarkening("linear", v);
  } else {
    std::cout << "model is default\n";
    lc->setLimbDarkening("default", v);
  }
}

void set_amoeba_printout(LightCurveIRS* lc, const char* amoebaFilename, const char* parFilename) {
  lc->setAmoebaPrintOut(true, std::string(amoebaFilename), std::string(parFilename));
}

void lcirs_delete(LightCurveIRS* lc) { delete lc; }

unsigned int lcirs_last_status(LightCurveIRS* lc) { return lc->lastStatus; }

void lcirs_copy_counts(LightCurveIRS* lc, uint64_t* out) {
  for (size_t i = 0; i < lc->counts.size(); i++) out[i] = lc->counts[i];
}

void lcirs_copy_lc_full(LightCurveIRS* lc, double* out) {
  for (size_t i = 0; i <= lc->lcLength; i++) out[i] = lc->impl->lcFull[i];
}

void lcirs_copy_status(LightCurveIRS* lc, uint32_t* out) {
  for (size_t i = 0; i < lc->status.size(); i++) out[i] = lc->status[i];
}

void lcirs_set_verbose(LightCurveIRS* lc, int v) { lc->verbose = v; }

void lcirs_grid(LightCurveIRS* lc, double* out8) {
  for (int k = 0; k < 8; k++) out8[k] = lc->grid[k];
}

void lcirs_copy_seeds(LightCurveIRS* lc, int32_t* seeds, int32_t* nseeds) {
  for (size_t i = 0; i < lc->seeds.size(); i++) seeds[i] = lc->seeds[i];
  for (size_t i = 0; i < lc->nseeds.size(); i++) nseeds[i] = lc->nseeds[i];
}

void lcirs_fill_from_seeds(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY,
                           const int32_t* seeds, const int32_t* nseeds) {
  lc->runFill({iniX, iniY}, {finX, finY}, seeds, nseeds);
}

void lcirs_copy_stats(LightCurveIRS* lc, uint64_t* out3) {
  for (int k = 0; k < 3; k++) out3[k] = lc->stats[k];
}

void lcirs_copy_transfer_bytes(uint64_t* out2) {
  if (!out2) return;
  out2[0] = tl::g_copy_h2d.load();
  out2[1] = tl::g_copy_d2h.load();
}

void lcirs_set_precision(LightCurveIRS* lc, int mode) { lc->precision = mode; }

void lcirs_set_chain(LightCurveIRS* lc, int points) { lc->chainPoints = points; }

void lcirs_copy_diag(LightCurveIRS* lc, uint32_t* out) {
  for (size_t i = 0; i < lc->diag.size(); i++) out[i] = lc->diag[i];
}

}  // extern "C"
