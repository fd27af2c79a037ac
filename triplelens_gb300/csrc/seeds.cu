// seeds.cu - FP64 lens set-up, image seeding and point-source kernels.
//
// Compiled with --fmad=false: every FP64 operation below is a separately
// rounded IEEE operation, like the host build of tl_math.h, so roots, caustic
// samples, grid parameters and seed pixels are bit-identical between the
// device and a -ffp-contract=off host build.
//
//   lens_setup_kernel  one warp per lens: critical curve (500 phase samples,
//                      warm-started, six roots polished on six lanes),
//                      caustics, caustic boxes, image-plane grid.
//                      (ccc.cc:42-203, lcirs.cc:39-92)
//   caustic_scan_kernel  one warp per chunk: caustic-segment tests of every
//                      point (lanes over segments), trial points in order
//   seeds_kernel       one thread per chunk of kChainChunk consecutive points
//                      of a curve: point images through the warm-started
//                      Laguerre chain, then the images of the crossing trial
//                      points (lcirs.cc:117-174, imgpoint.cc:160-286)
//   point_lc_kernel    point-source magnification curve (lcbase.cc:17-52)
#include <cuda_runtime.h>
#include <math.h>
#include <stdio.h>

#include <algorithm>

#include "engine.h"

namespace tl {

__constant__ TrigTable c_trig;
__constant__ double c_phase_cos[kCCLen];
__constant__ double c_phase_sin[kCCLen];

// Host tables: cos(i)/sin(i) for the Laguerre fallback step (laguerre.cc:77)
// and the phase samples phi_j = 2*3.14159265359*j/500 (ccc.cc:57), both from
// the host libm so that host and device agree.
void upload_trig_tables() {
  static TrigTable t;
  static double pc[kCCLen], ps[kCCLen];
  for (int i = 0; i <= kMaxIt; i++) {
    t.c[i] = cos(1.0 * i);
    t.s[i] = sin(1.0 * i);
  }
  for (unsigned j = 0; j < (unsigned)kCCLen; j++) {
    double phi = 2.0 * 3.14159265359 * j / kCCLen;
    pc[j] = cos(phi);
    ps[j] = sin(phi);
  }
  cudaMemcpyToSymbol(c_trig, &t, sizeof(t));
  upload_chain_tables(t);
  cudaMemcpyToSymbol(c_phase_cos, pc, sizeof(pc));
  cudaMemcpyToSymbol(c_phase_sin, ps, sizeof(ps));
}

LensSpec make_lens_spec(double a, double b, double th, double m2, double m3, double rho,
                        long ppr, double ld_a, double ld_b, double intensity) {
  LensSpec s;
  s.m1 = 1.0 - m2 - m3;
  s.m2 = m2;
  s.m3 = m3;
  s.z2x = a;
  s.z3x = b * cos(th);
  s.z3y = b * sin(th);
  s.rho = rho;
  s.ld_a = ld_a;
  s.ld_b = ld_b;
  s.intensity = intensity;
  s.ppr = ppr;
  s.is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0) ? 1 : 0;
  s.pad = 0;
  return s;
}

// ---------------------------------------------------------------------------
// lens set-up
// ---------------------------------------------------------------------------
constexpr int kSetupWarps = 4;

__device__ __forceinline__ void minmax_acc(cx v, cx* mn, cx* mx) {
  if (v.re < mn->re) mn->re = v.re;
  if (v.im < mn->im) mn->im = v.im;
  if (v.re > mx->re) mx->re = v.re;
  if (v.im > mx->im) mx->im = v.im;
}

__global__ void __launch_bounds__(kSetupWarps * 32)
lens_setup_kernel(const LensSpec* specs, int nlens, DevLens* lenses, cx* cc_out, cx* ca_out) {
  __shared__ cx s_roots[kSetupWarps][8];
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int li = blockIdx.x * kSetupWarps + warp;
  if (li >= nlens) return;
  const LensSpec sp = specs[li];
  Lens L;
  L.m1 = sp.m1;
  L.m2 = sp.m2;
  L.m3 = sp.m3;
  L.z1 = mk(0.0, 0.0);
  L.z2 = mk(sp.z2x, 0.0);
  L.z3 = mk(sp.z3x, sp.z3y);
  L.is_binary_img = sp.is_binary_img;
  lens_finish(&L);
  cx* cc = cc_out + (size_t)li * kBranches * kCCLen;
  cx* ca = ca_out + (size_t)li * kBranches * kCCLen;

  // critical curve: ccc.cc:55-94
  cx root = mk(0.0, 0.0);
  for (int j = 0; j < kCCLen; j++) {
    cx c[7];
    cc_poly(L, mk(c_phase_cos[j], c_phase_sin[j]), c);
    if (j == 0) {
      if (lane == 0) {
        cx r6[6];
        solve_roots(c, 6, nullptr, r6, &c_trig);
        for (int k = 0; k < 6; k++) s_roots[warp][k] = r6[k];
      }
    } else {
      if (lane < 6) {
        laguerre(c, 6, &root, &c_trig);  // polishRoots: each root on its own
        s_roots[warp][lane] = root;
      }
      __syncwarp();
      if (lane == 0) {
        cx r6[6];
        for (int k = 0; k < 6; k++) r6[k] = s_roots[warp][k];
        if (!check_roots(c, 6, r6)) {
          solve_roots(c, 6, nullptr, r6, &c_trig);
          for (int k = 0; k < 6; k++) s_roots[warp][k] = r6[k];
        }
      }
    }
    __syncwarp();
    if (lane < 6) {
      root = s_roots[warp][lane];
      cc[lane * kCCLen + j] = root;
    }
    __syncwarp();
  }
  __syncwarp();
  // caustics: ccc.cc:182-200
  for (int i = lane; i < kBranches * kCCLen; i += 32) ca[i] = caustic_point(L, cc[i]);
  __syncwarp();
  if (lane != 0) return;

  DevLens D;
  D.L = L;
  // caustic boxes, accumulated and including the origin (lcirs.cc:39-48)
  cx mn = mk(0.0, 0.0), mx = mk(0.0, 0.0);
  for (int k = 0; k < kBranches; k++) {
    for (int j = 0; j < kCCLen; j++) minmax_acc(ca[k * kCCLen + j], &mn, &mx);
    D.box_min[k] = mn;
    D.box_max[k] = mx;
  }
  // image plane (lcirs.cc:51-92)
  mn = mk(0.0, 0.0);
  mx = mk(0.0, 0.0);
  for (int i = 0; i < kBranches * kCCLen; i++) minmax_acc(cc[i], &mn, &mx);
  double half = mx.re - mn.re;
  if (mx.im - mn.im > half) half = mx.im - mn.im;
  half *= 3.0 / 2.0;
  const double cxr = (mx.re + mn.re) / 2.0, cxi = (mx.im + mn.im) / 2.0;
  Grid g;
  g.top_x = cxr + half;
  g.top_y = cxi + half;
  g.corner_x = cxr - half;
  g.corner_y = cxi - half;
  const int ppr = (int)sp.ppr;
  g.n = (int64_t)(2 * half / sp.rho * (double)ppr);
  g.size_double = 2 * half;
  g.amp_scale = sp.intensity / 3.14159265358979323846 / ((double)ppr * (double)ppr);
  g.h = g.size_double / ((double)g.n - 1.0);
  D.g = g;
  D.rho = sp.rho;
  D.rho2 = sp.rho * sp.rho;
  D.ld_a = sp.ld_a;
  D.ld_b = sp.ld_b;
  D.ray_binary = (sp.m3 == 0.0) ? 1 : 0;
  D.ppr = ppr;
  for (int k = 0; k < 5; k++) D.heap0[k] = cc[k * kCCLen + 10];
  lenses[li] = D;
}

void launch_lens_setup(const LensSpec* d_specs, int nlens, DevLens* d_lenses, cx* d_cc, cx* d_ca,
                       cudaStream_t st) {
  if (nlens <= 0) return;
  int blocks = (nlens + kSetupWarps - 1) / kSetupWarps;
  lens_setup_kernel<<<blocks, kSetupWarps * 32, 0, st>>>(d_specs, nlens, d_lenses, d_cc, d_ca);
}

// ---------------------------------------------------------------------------
// seeds
// ---------------------------------------------------------------------------
constexpr int kSeedThreads = 32;   // one warp per block: chains are latency-bound
constexpr int kScanWarps = 4;

// point i of a curve (t = i/n); a curve of length n = 0 is the single
// position (x0, y0)
__device__ __forceinline__ cx traj_pos(const Traj& T, uint32_t i) {
  double t = T.n ? (double)i / (double)T.n : 0.0;
  cx s = mk(T.x0, T.y0), e = mk(T.x1, T.y1);
  return add(s, scale(sub(e, s), t));
}

__device__ __forceinline__ int32_t clamp_px(int64_t v, uint32_t* status) {
  if (v < -(int64_t)1 << 30 || v > ((int64_t)1 << 30)) {
    *status |= kStEdge;
    return v < 0 ? -(1 << 30) : (1 << 30);
  }
  return (int32_t)v;
}

// lane 0: append the seed pixels of n images
__device__ __forceinline__ void emit_seeds(const Grid& g, const cx* imgs, int n, int32_t* seeds,
                                           uint32_t* nseed, uint32_t* status) {
  for (int k = 0; k < n; k++) {
    int32_t px = clamp_px(x_to_nx(g, imgs[k].re), status);
    int32_t py = clamp_px(y_to_ny(g, imgs[k].im), status);
    if (*nseed < (uint32_t)kMaxSeeds) {
      seeds[2 * *nseed] = px;
      seeds[2 * *nseed + 1] = py;
    } else {
      *status |= kStSeedOverflow;
    }
    (*nseed)++;
  }
}

// Caustic-segment tests (lcirs.cc:131-165, 195-255): one warp per chunk, the
// 32 lanes over consecutive segments of a branch whose box overlaps the
// source; a warp ballot marks the first segment of every run of hits
// (pointTaken), whose trial point is appended in segment order.
__global__ void __launch_bounds__(kScanWarps * 32)
caustic_scan_kernel(const SeedJob* jobs, int njobs, const Traj* trajs, const DevLens* lenses,
                    const cx* ca_all, TrialList* trials) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const int ji = blockIdx.x * kScanWarps + warp;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const DevLens& D = lenses[T.lens];
  const double rho = D.rho;
  const cx* ca = ca_all + (size_t)T.lens * kBranches * kCCLen;
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const int64_t p = T.point_base + i;
    const cx pos = traj_pos(T, i);
    TrialList* tl = &trials[p];
    uint32_t nt = 0;
    if (isfinite(pos.re) && isfinite(pos.im)) {
      for (int k = 0; k < kBranches; k++) {
        if (!(pos.re + rho >= D.box_min[k].re && pos.re - rho <= D.box_max[k].re &&
              pos.im + rho >= D.box_min[k].im && pos.im - rho <= D.box_max[k].im))
          continue;
        const cx* br = ca + k * kCCLen;
        unsigned carry = 0;  // was the previous segment a hit
        for (int base = 0; base < kCCLen - 1; base += 32) {
          const int j = base + lane;
          cx trial = mk(0.0, 0.0);
          bool hit = false;
          if (j < kCCLen - 1) hit = intersection_check(rho, pos, br[j], br[j + 1], &trial);
          const unsigned m = __ballot_sync(0xffffffffu, hit);
          const unsigned starts = m & ~((m << 1) | carry);
          carry = (m >> 31) & 1u;
          if ((starts >> lane) & 1u) {
            const uint32_t slot = nt + __popc(starts & ((1u << lane) - 1u));
            if (slot < (uint32_t)kMaxTrials) tl->t[slot] = trial;
          }
          nt += __popc(starts);
        }
      }
    }
    if (lane == 0) tl->n = nt;
  }
}

// One thread per chunk: the warm-start chain is serial within a chunk, and
// independent across chunks, so 32 chunks share a warp's FP64 instructions.
__global__ void __launch_bounds__(kSeedThreads)
seeds_kernel(const SeedJob* jobs, int njobs, const Traj* trajs, const DevLens* lenses,
             PointIn* points, int32_t* seeds_all, PointOut* out, const TrialList* trials,
             RootChain* chains) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const DevLens& D = lenses[T.lens];
  const Lens L = D.L;
  const Grid g = D.g;

  // a chain starts from a saved state, or from the one the reference's
  // constructor leaves
  RootChain ch;
  if (job.chain >= 0)
    ch = chains[job.chain];
  else
    chain_reset(&ch, D.heap0);
  cx imgs[10];
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const int64_t p = T.point_base + i;
    const cx pos = traj_pos(T, i);
    int32_t* seeds = seeds_all + (size_t)p * 2 * kMaxSeeds;
    uint32_t nseed = 0, status = 0;
    if (!(isfinite(pos.re) && isfinite(pos.im))) status |= kStBadInput;
    PointIn pi;
    pi.sx = pos.re;
    pi.sy = pos.im;
    pi.lens = T.lens;
    pi.est_blocks = 0;
    if (!(status & kStBadInput)) {
      int n = chain_images(L, &ch, pos, imgs, &c_trig);
      if (wrong_count(L, n)) status |= kStImageCount;
      emit_seeds(g, imgs, n, seeds, &nseed, &status);
      SeedList sl;
      seed_list_start(&sl, n);
      // predicted fill size, for the fill's largest-first order: the
      // point-source magnification tracks the finite-source one closely
      // (rays ~ A pi ppr^2), plus the boundary blocks
      double a = 0.0;
      for (int k = 0; k < n; k++) a += image_amp(L, imgs[k]);
      const double est = a * 3.14159265358979 * (double)D.ppr * (double)D.ppr / 1024.0 * 1.15;
      pi.est_blocks = (uint32_t)fmin(fmax(est, 0.0), 4.0e9);
      // caustic-crossing seeds (lcirs.cc:131-165): the images of the trial
      // points found by caustic_scan_kernel, in the reference's order
      const TrialList& tl = trials[p];
      const uint32_t ntr = tl.n < (uint32_t)kMaxTrials ? tl.n : (uint32_t)kMaxTrials;
      if (tl.n > (uint32_t)kMaxTrials) status |= kStSeedOverflow;
      for (uint32_t t = 0; t < ntr; t++) {
        const int nt = chain_images(L, &ch, tl.t[t], imgs, &c_trig);
        for (int k = 0; k < nt; k++) seed_list_push(&ch, &sl, imgs[k]);
        emit_seeds(g, imgs, nt, seeds, &nseed, &status);
      }
      seed_list_end(&ch, &sl);
    }
    points[p] = pi;
    PointOut o;
    o.count = 0;
    o.wsum_fx = 0;
    o.status = status;
    o.nseeds = nseed < (uint32_t)kMaxSeeds ? nseed : (uint32_t)kMaxSeeds;
    o.tiles = 0;
    o.diag = 0;
    o.rays_eval = 0;
    o.rays_fp64 = 0;
    out[p] = o;
  }
  if (job.chain >= 0) chains[job.chain] = ch;
}

void launch_seeds(const SeedJob* d_jobs, int njobs, const Traj* d_trajs, const DevLens* d_lenses,
                  const cx* d_ca, PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                  TrialList* d_trials, RootChain* d_chains, cudaStream_t st) {
  if (njobs <= 0) return;
  launch_caustic_scan(d_jobs, njobs, d_trajs, d_lenses, d_ca, d_trials, st);
  const int blocks = (njobs + kSeedThreads - 1) / kSeedThreads;
  seeds_kernel<<<blocks, kSeedThreads, 0, st>>>(d_jobs, njobs, d_trajs, d_lenses, d_points, d_seeds,
                                                d_out, d_trials, d_chains);
}

void launch_caustic_scan(const SeedJob* d_jobs, int njobs, const Traj* d_trajs,
                         const DevLens* d_lenses, const cx* d_ca, TrialList* d_trials,
                         cudaStream_t st) {
  if (njobs <= 0) return;
  caustic_scan_kernel<<<(njobs + kScanWarps - 1) / kScanWarps, kScanWarps * 32, 0, st>>>(
      d_jobs, njobs, d_trajs, d_lenses, d_ca, d_trials);
}

// ---------------------------------------------------------------------------
// point-source light curve (lcbase.cc:40-52): t = i/(n-1), i = 0..n-1
// ---------------------------------------------------------------------------
__global__ void point_lc_kernel(const Traj* trajs, const SeedJob* jobs, int njobs,
                                const DevLens* lenses, double* amp, RootChain* chains) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const Lens L = lenses[T.lens].L;
  RootChain ch;
  if (job.chain >= 0)
    ch = chains[job.chain];
  else
    chain_reset(&ch, lenses[T.lens].heap0);
  cx imgs[10];
  const cx s = mk(T.x0, T.y0), e = mk(T.x1, T.y1);
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const double t = i / ((double)T.n - 1.0);
    const cx pos = add(s, scale(sub(e, s), t));
    int n = chain_images(L, &ch, pos, imgs, &c_trig);
    double a = 0.0;
    for (int k = 0; k < n; k++) a += image_amp(L, imgs[k]);
    amp[T.point_base + i] = a;
  }
  if (job.chain >= 0) chains[job.chain] = ch;
}

void launch_point_lc(const Traj* d_trajs, const SeedJob* d_jobs, int njobs, const DevLens* d_lenses,
                     double* d_amp, RootChain* d_chains, cudaStream_t st) {
  if (njobs <= 0) return;
  point_lc_kernel<<<(njobs + 63) / 64, 64, 0, st>>>(d_trajs, d_jobs, njobs, d_lenses, d_amp,
                                                   d_chains);
}

void plan_jobs(std::vector<SeedJob>* jobs, int traj, long np, int chunk, int chain) {
  const long step = chunk > 0 ? chunk : (np > 0 ? np : 1);
  for (long f = 0; f < np; f += step) {
    SeedJob j;
    j.traj = traj;
    j.first = (int32_t)f;
    j.count = (int32_t)std::min<long>(step, np - f);
    j.chain = chunk > 0 ? -1 : chain;
    jobs->push_back(j);
  }
}

}  // namespace tl
