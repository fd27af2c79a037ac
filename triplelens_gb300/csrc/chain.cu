// chain.cu - the image solver's warm-start chain in the reference's order,
// one warp per light curve.
//
// The reference solves the images of a curve's points one after the other,
// each solve warm-started from the roots of the previous one
// (ImgPoint::getRootsPrecalculated, src/Images/imgpoint.cc:160-205; the
// trajectory loop, src/LightCurves/lcirs.cc:117-165).  Whether an image next
// to a small-mass lens passes the 1e-6 filter depends on the last bits of
// those roots, and those bits depend on the whole history of the chain, so
// the chain is serial within a curve.  On GB300 one FP64 warp instruction
// occupies a sub-partition's FP64 unit for 64 cycles whatever the number of
// active lanes, and a correctly rounded FP64 division or square root for
// about 600, so a serial chain is bound by its FP64 instruction count.  The
// kernels here cut that count without changing a single rounding:
//
//   prep_kernel   (thread per point, history-free work, run in parallel)
//                 the polynomial coefficients of every point and its cold
//                 solve (Laguerre from (EPS, EPS)), which the chain needs
//                 whenever checkRoots fails or the image count is wrong;
//   chain_kernel  (warp per curve) the warm-started solves: the three
//                 Horner recurrences of a Laguerre step on three lanes, every
//                 |b_j| of its error bound on its own lane, the two quotients
//                 f/b and 2s/b on two lanes, the ten polishes on ten lanes,
//                 the image filter on ten lanes.
//
// Every value is produced by exactly the operations of tl::laguerre /
// tl::solve_roots (tl_math.h) in the same order - only the lane that computes
// it changes - so the roots, seeds and ray counts are bit-identical to the
// serial chain and to the reference.  Compiled with --fmad=false.
#include <cuda_runtime.h>
#include <math.h>

#include <algorithm>

#include "engine.h"

namespace tl {

namespace {

__constant__ TrigTable k_trig;
constexpr unsigned kFull = 0xffffffffu;
constexpr int kPrepThreads = 64;

__device__ __forceinline__ cx shfl(cx v, int src) {
  return mk(__shfl_sync(kFull, v.re, src), __shfl_sync(kFull, v.im, src));
}
__device__ __forceinline__ cx shfl_up1(cx v) {
  return mk(__shfl_up_sync(kFull, v.re, 1), __shfl_up_sync(kFull, v.im, 1));
}

// Out-of-line copies of the heavy FP64 helpers: one warp runs this code
// serially, so a small instruction footprint matters more than call overhead
// (each call wraps a divide or square root of ~600 cycles).
__device__ __noinline__ double abs_c(cx a) { return cabs(a); }
__device__ __noinline__ cx div_c(cx a, cx b) { return div(a, b); }
__device__ __noinline__ cx sqrt_c(cx a) { return csqrt(a); }
__device__ __noinline__ void poly_c(const Lens& L, cx zeta, cx* c) { lens_poly(L, zeta, c); }
__device__ __noinline__ bool polish_c(const cx* poly, cx* r) { return laguerre(poly, 10, r, &k_trig); }
__device__ __noinline__ bool check_c(const cx* poly, const cx* roots) {
  return check_roots(poly, 10, roots);
}
__device__ __noinline__ bool img_check_c(const Lens& L, cx img, cx src) {
  return img_check(L, img, src, 1.0e-6);
}
__device__ __noinline__ double amp_c(const Lens& L, cx img) { return image_amp(L, img); }

// per-warp scratch of the cooperative solver
struct WarpScratch {
  cx poly[11];    // polynomial of the current solve
  cx temp[11];    // its deflated copy
  cx bv[11];      // Horner values b_j of one Laguerre step
  double h[12];   // |b_j|, j = 0..m, and |x| at m + 1
  cx roots[10];
  cx imgs[10];
};

// laguerre.cc:18-99 for one root of poly[0..m] on a whole warp.  Every lane
// leaves with the same *px and result.
__device__ bool laguerre_warp(const cx* poly, int m, cx* px, WarpScratch* sh) {
  const int lane = threadIdx.x & 31;
  cx x = *px;
  if (m == 1) {
    if (abs_c(poly[1]) != 0.0) {
      *px = neg(div_c(poly[0], poly[1]));
      return true;
    }
    *px = mk(999.0, 999.0);
    return false;
  }
  const double md = (double)m;
  for (int i = 1; i <= kMaxIt; i++) {
    // Horner, laguerre.cc:49-56: lane 0 carries b, lane 1 f, lane 2 s; each
    // step reads the lower lane's value from before the step
    cx v = lane == 0 ? poly[m] : mk(0.0, 0.0);
    if (lane == 0) sh->bv[m] = v;
    for (int j = m - 1; j >= 0; j--) {
      const cx prev = shfl_up1(v);
      v = add(mul(x, v), lane == 0 ? poly[j] : prev);
      if (lane == 0) sh->bv[j] = v;
    }
    __syncwarp();
    // |b_m| .. |b_0| and |x| (the reference takes |x| once per term: the
    // same value), one per lane
    const cx w = lane <= m ? sh->bv[lane < 11 ? lane : 0] : x;
    const double hv = abs_c(w);
    if (lane <= m + 1) sh->h[lane] = hv;
    __syncwarp();
    const double ax = sh->h[m + 1];
    double err = sh->h[m];
    for (int j = m - 1; j >= 0; j--) err = sh->h[j] + ax * err;
    err *= kEps;
    const double ab = sh->h[0];
    __syncwarp();
    if (ab <= err) {
      *px = x;
      return true;
    }
    const cx b = shfl(v, 0), f = shfl(v, 1), s = shfl(v, 2);
    // g = f/b on lane 1, 2s/b on lane 2
    const cx q = div_c(lane == 1 ? f : scale(s, 2.0), b);
    const cx g = shfl(q, 1), t = shfl(q, 2);
    const cx h = sub(mul(g, g), t);
    const cx sq = sqrt_c(scale(sub(scale(h, md), mul(g, g)), md - 1.0));
    cx gp = add(g, sq);
    const cx gm = sub(g, sq);
    // |gp| on lane 0, |gm| on lane 1
    const double a = abs_c(lane == 0 ? gp : gm);
    const double agp = __shfl_sync(kFull, a, 0), agm = __shfl_sync(kFull, a, 1);
    double asel = agp;
    if (agp < agm) {
      gp = gm;
      asel = agm;
    }
    cx dx;
    if (asel > 0.0)
      dx = div_c(mk(md, 0.0), gp);
    else
      dx = scale(mk(k_trig.c[i], k_trig.s[i]), 1.0 + ax);
    const cx x1 = sub(x, dx);
    if (x.re == x1.re && x.im == x1.im) {
      *px = x;
      return true;
    }
    if (i % kMT)
      x = x1;
    else
      x = sub(x, scale(dx, frac_step(i / kMT)));
  }
  *px = x;
  return false;
}

// laguerre.cc:103-167 on a whole warp: sh->poly holds the polynomial;
// init == nullptr is the cold start.  Roots land in sh->roots.
__device__ void solve_warp(const cx* init, WarpScratch* sh) {
  const int lane = threadIdx.x & 31;
  if (lane < 11) sh->temp[lane] = sh->poly[lane];
  __syncwarp();
  for (int j = 10; j >= 1; j--) {
    cx x = init ? init[j] : mk(kEps, kEps);
    if (!laguerre_warp(sh->temp, j, &x, sh)) {
      if (init) x = mk(kEps, kEps);
    }
    if (lane == 0) {
      sh->roots[10 - j] = x;
      // deflation (laguerre.cc:147-157)
      cx b = sh->temp[j];
      for (int jj = j - 1; jj >= 0; jj--) {
        const cx c = sh->temp[jj];
        sh->temp[jj] = b;
        b = add(mul(x, b), c);
      }
    }
    __syncwarp();
  }
  // polish every root on the full polynomial (laguerre.cc:160-164), one lane
  // per root
  if (lane < 10) {
    cx r = sh->roots[lane];
    polish_c(sh->poly, &r);
    sh->roots[lane] = r;
  }
  __syncwarp();
}

// getRootsPrecalculated (imgpoint.cc:160-205) for a position whose
// coefficients are in sh->poly; cold: its cold-solve roots, or nullptr to
// solve them here.
__device__ void roots_warp(RootChain* ch, const cx* cold, bool force, WarpScratch* sh) {
  auto take_cold = [&]() {
    if (cold) {
      for (int k = 0; k < 10; k++) ch->roots[k] = cold[k];
    } else {
      solve_warp(nullptr, sh);
      for (int k = 0; k < 10; k++) ch->roots[k] = sh->roots[k];
    }
    chain_replace_roots(ch);
  };
  if (!ch->have || force) {
    take_cold();
    ch->have = 1;
  } else {
    solve_warp(ch->roots, sh);
    for (int k = 0; k < 10; k++) ch->roots[k] = sh->roots[k];
    chain_replace_roots(ch);
    if (!check_c(sh->poly, ch->roots)) take_cold();
  }
}

// the image filter (imgpoint.cc:72-90, 218-231) on ten lanes; images in root
// order into sh->imgs
__device__ int filter_warp(const Lens& L, RootChain* ch, cx zeta, WarpScratch* sh) {
  const int lane = threadIdx.x & 31;
  const bool acc = lane < 10 && img_check_c(L, ch->roots[lane < 10 ? lane : 0], zeta);
  const unsigned m = __ballot_sync(kFull, acc);
  if (acc) sh->imgs[__popc(m & ((1u << lane) - 1u))] = ch->roots[lane];
  __syncwarp();
  const int n = __popc(m);
  if (n >= 9 && !ch->imgs_big) {  // the image list outgrows capacity 8
    heap_take(ch);
    ch->imgs_big = 1;
  }
  return n;
}

// getImages (imgpoint.cc:208-274) through the chain; sh->poly must hold the
// position's coefficients
__device__ int images_warp(const Lens& L, RootChain* ch, cx zeta, const cx* cold,
                           WarpScratch* sh) {
  roots_warp(ch, cold, false, sh);
  int n = filter_warp(L, ch, zeta, sh);
  if (wrong_count(L, n)) {
    roots_warp(ch, cold, true, sh);
    n = filter_warp(L, ch, zeta, sh);
  }
  return n;
}

__device__ __forceinline__ cx traj_point(const Traj& T, uint32_t i) {
  double t = T.n ? (double)i / (double)T.n : 0.0;
  cx s = mk(T.x0, T.y0), e = mk(T.x1, T.y1);
  return add(s, scale(sub(e, s), t));
}

__device__ __forceinline__ int32_t clamp_pixel(int64_t v, uint32_t* status) {
  if (v < -(int64_t)1 << 30 || v > ((int64_t)1 << 30)) {
    *status |= kStEdge;
    return v < 0 ? -(1 << 30) : (1 << 30);
  }
  return (int32_t)v;
}

__device__ void put_seeds(const Grid& g, const cx* imgs, int n, int32_t* seeds, uint32_t* nseed,
                          uint32_t* status) {
  for (int k = 0; k < n; k++) {
    const int32_t px = clamp_pixel(x_to_nx(g, imgs[k].re), status);
    const int32_t py = clamp_pixel(y_to_ny(g, imgs[k].im), status);
    if (*nseed < (uint32_t)kMaxSeeds) {
      seeds[2 * *nseed] = px;
      seeds[2 * *nseed + 1] = py;
    } else {
      *status |= kStSeedOverflow;
    }
    (*nseed)++;
  }
}

// Coefficients and cold-solve roots of every point (history-free), one
// thread per point chunk (the chunks of the caustic scan).
__global__ void __launch_bounds__(kPrepThreads)
prep_kernel(const SeedJob* jobs, int njobs, const Traj* trajs, const DevLens* lenses,
            PointPrep* prep) {
  const int ji = blockIdx.x * blockDim.x + threadIdx.x;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const Lens& L = lenses[T.lens].L;
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const cx pos = traj_point(T, i);
    PointPrep* P = &prep[T.point_base + i];
    if (!(isfinite(pos.re) && isfinite(pos.im))) continue;
    cx c[11], r[10];
    lens_poly(L, pos, c);
    solve_roots(c, 10, nullptr, r, &k_trig);
    for (int k = 0; k < 11; k++) P->coef[k] = c[k];
    for (int k = 0; k < 10; k++) P->cold[k] = r[k];
  }
}

// One warp per curve job: the seeds of its points in the reference's order
// (lcirs.cc:117-165): the point's images, then the images of its caustic-
// crossing trial points (from caustic_scan_kernel), all through one chain.
__global__ void __launch_bounds__(32)
chain_kernel(const SeedJob* jobs, int njobs, const Traj* trajs, const DevLens* lenses,
             PointIn* points, int32_t* seeds_all, PointOut* out, const TrialList* trials,
             const PointPrep* prep, RootChain* chains) {
  __shared__ WarpScratch sh;
  const int lane = threadIdx.x & 31;
  const int ji = blockIdx.x;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const DevLens& D = lenses[T.lens];
  const Lens L = D.L;
  const Grid g = D.g;
  RootChain ch;
  if (job.chain >= 0)
    ch = chains[job.chain];
  else
    chain_reset(&ch, D.heap0);
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const int64_t p = T.point_base + i;
    const cx pos = traj_point(T, i);
    int32_t* seeds = seeds_all + (size_t)p * 2 * kMaxSeeds;
    uint32_t nseed = 0, status = 0;
    if (!(isfinite(pos.re) && isfinite(pos.im))) status |= kStBadInput;
    PointIn pi;
    pi.sx = pos.re;
    pi.sy = pos.im;
    pi.lens = T.lens;
    pi.est_blocks = 0;
    if (!(status & kStBadInput)) {
      const PointPrep& P = prep[p];
      if (lane < 11) sh.poly[lane] = P.coef[lane];
      __syncwarp();
      const int n = images_warp(L, &ch, pos, P.cold, &sh);
      if (wrong_count(L, n)) status |= kStImageCount;
      // predicted fill size for the fill's largest-first order
      const double am = lane < n ? amp_c(L, sh.imgs[lane < 10 ? lane : 0]) : 0.0;
      double a = am;
      for (int o = 16; o > 0; o >>= 1) a += __shfl_xor_sync(kFull, a, o);
      const double est = a * 3.14159265358979 * (double)D.ppr * (double)D.ppr / 1024.0 * 1.15;
      pi.est_blocks = (uint32_t)fmin(fmax(est, 0.0), 4.0e9);
      if (lane == 0) put_seeds(g, sh.imgs, n, seeds, &nseed, &status);
      SeedList sl;
      seed_list_start(&sl, n);
      const TrialList& tl = trials[p];
      const uint32_t ntr = tl.n < (uint32_t)kMaxTrials ? tl.n : (uint32_t)kMaxTrials;
      if (tl.n > (uint32_t)kMaxTrials) status |= kStSeedOverflow;
      for (uint32_t t = 0; t < ntr; t++) {
        const cx tz = tl.t[t];
        __syncwarp();
        if (lane == 0) poly_c(L, tz, sh.poly);
        __syncwarp();
        const int nt = images_warp(L, &ch, tz, nullptr, &sh);
        for (int k = 0; k < nt; k++) seed_list_push(&ch, &sl, sh.imgs[k]);
        if (lane == 0) put_seeds(g, sh.imgs, nt, seeds, &nseed, &status);
      }
      seed_list_end(&ch, &sl);
    }
    if (lane == 0) {
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
    __syncwarp();
  }
  if (job.chain >= 0 && lane == 0) chains[job.chain] = ch;
}

// Point-source curve (lcbase.cc:40-52: t = i/(n-1)) through one chain per
// job, one warp per job; cold solves are made in the chain.
__global__ void __launch_bounds__(32)
point_chain_kernel(const SeedJob* jobs, int njobs, const Traj* trajs, const DevLens* lenses,
                   double* amp, RootChain* chains) {
  __shared__ WarpScratch sh;
  const int lane = threadIdx.x & 31;
  const int ji = blockIdx.x;
  if (ji >= njobs) return;
  const SeedJob job = jobs[ji];
  const Traj T = trajs[job.traj];
  const DevLens& D = lenses[T.lens];
  const Lens L = D.L;
  RootChain ch;
  if (job.chain >= 0)
    ch = chains[job.chain];
  else
    chain_reset(&ch, D.heap0);
  const cx s = mk(T.x0, T.y0), e = mk(T.x1, T.y1);
  for (int q = 0; q < job.count; q++) {
    const uint32_t i = (uint32_t)(job.first + q);
    const double t = i / ((double)T.n - 1.0);
    const cx pos = add(s, scale(sub(e, s), t));
    __syncwarp();
    if (lane == 0) poly_c(L, pos, sh.poly);
    __syncwarp();
    const int n = images_warp(L, &ch, pos, nullptr, &sh);
    double a = 0.0;
    for (int k = 0; k < n; k++) a += amp_c(L, sh.imgs[k]);
    if (lane == 0) amp[T.point_base + i] = a;
  }
  if (job.chain >= 0 && lane == 0) chains[job.chain] = ch;
}

}  // namespace

void upload_chain_tables(const TrigTable& t) { cudaMemcpyToSymbol(k_trig, &t, sizeof(t)); }

void launch_point_lc_exact(const Traj* d_trajs, const SeedJob* d_jobs, int njobs,
                           const DevLens* d_lenses, double* d_amp, RootChain* d_chains,
                           cudaStream_t st) {
  if (njobs <= 0) return;
  point_chain_kernel<<<njobs, 32, 0, st>>>(d_jobs, njobs, d_trajs, d_lenses, d_amp, d_chains);
}

namespace {
// every curve's chain in the lens's construction state
__global__ void chain_reset_kernel(const Traj* trajs, int ntraj, const DevLens* lenses,
                                   RootChain* chains) {
  const int t = blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= ntraj) return;
  RootChain ch;
  chain_reset(&ch, lenses[trajs[t].lens].heap0);
  chains[t] = ch;
}
}  // namespace

void launch_seeds_prep(const SeedJob* d_scan_jobs, int nscan, const Traj* d_trajs,
                       const DevLens* d_lenses, const cx* d_ca, TrialList* d_trials,
                       PointPrep* d_prep, cudaStream_t st) {
  if (nscan <= 0) return;
  launch_caustic_scan(d_scan_jobs, nscan, d_trajs, d_lenses, d_ca, d_trials, st);
  prep_kernel<<<(nscan + kPrepThreads - 1) / kPrepThreads, kPrepThreads, 0, st>>>(
      d_scan_jobs, nscan, d_trajs, d_lenses, d_prep);
}

void launch_chain_reset(const Traj* d_trajs, int ntraj, const DevLens* d_lenses,
                        RootChain* d_chains, cudaStream_t st) {
  if (ntraj <= 0) return;
  chain_reset_kernel<<<(ntraj + 127) / 128, 128, 0, st>>>(d_trajs, ntraj, d_lenses, d_chains);
}

void launch_chain(const SeedJob* d_chain_jobs, int nchain, const Traj* d_trajs,
                  const DevLens* d_lenses, PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                  const TrialList* d_trials, const PointPrep* d_prep, RootChain* d_chains,
                  cudaStream_t st) {
  if (nchain <= 0) return;
  chain_kernel<<<nchain, 32, 0, st>>>(d_chain_jobs, nchain, d_trajs, d_lenses, d_points, d_seeds,
                                      d_out, d_trials, d_prep, d_chains);
}

void launch_seeds_exact(const SeedJob* d_scan_jobs, int nscan, const SeedJob* d_chain_jobs,
                        int nchain, const Traj* d_trajs, const DevLens* d_lenses, const cx* d_ca,
                        PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                        TrialList* d_trials, PointPrep* d_prep, RootChain* d_chains,
                        cudaStream_t st) {
  if (nscan <= 0 || nchain <= 0) return;
  launch_caustic_scan(d_scan_jobs, nscan, d_trajs, d_lenses, d_ca, d_trials, st);
  prep_kernel<<<(nscan + kPrepThreads - 1) / kPrepThreads, kPrepThreads, 0, st>>>(
      d_scan_jobs, nscan, d_trajs, d_lenses, d_prep);
  chain_kernel<<<nchain, 32, 0, st>>>(d_chain_jobs, nchain, d_trajs, d_lenses, d_points, d_seeds,
                                      d_out, d_trials, d_prep, d_chains);
}

}  // namespace tl
