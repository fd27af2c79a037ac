// engine.h - data layout and host entry points of the GB300 IRS engine.
//
// Device data (all in HBM, one copy per engine):
//   DevLens[nlens]          lens, grid, limb darkening, caustic boxes
//   caustics[nlens][6][500] caustic samples (tl::cx), branch-major
//   Traj[ntraj]             light curves: lens index, end points, length
//   SeedJob[njobs]          chunks of consecutive points of one curve
//   PointIn[npoints]        source position + lens index of every point
//   seeds[npoints][kMaxSeeds] seed pixels (int32 x, y)
//   PointOut[npoints]       ray count, fixed-point weight sum, status, stats
//   fill scratch            per resident CTA: tile hash table, work ring
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <vector>

#include "tl_math.h"

namespace tl {

constexpr int kMaxSeeds = 64;     // seed pixels kept per point
constexpr int kChainChunk = 4;    // points per warm-start chain in the fast mode

// status bits of a point (PointOut::status)
enum : uint32_t {
  kStSeedOverflow = 1u << 0,   // more than kMaxSeeds seeds: surplus dropped
  kStEdge = 1u << 1,           // fill touched column 1 or N-1 (plane edge)
  kStTableFull = 1u << 2,      // tile table full: point was not completed
  kStTimeout = 1u << 3,        // a bounded wait ran out
  kStImageCount = 1u << 4,     // wrong image count after the cold retry
  kStBadInput = 1u << 5,       // non-finite source position or grid
};

struct DevLens {
  Lens L;
  Grid g;
  double rho, rho2;
  double ld_a, ld_b;       // weight = ld_a + ld_b * sqrt(1 - r^2/rho^2)
  cx box_min[kBranches];   // caustic boxes (lcirs.cc:39-48, accumulated)
  cx box_max[kBranches];
  int32_t ray_binary;      // m3 == 0: two-lens ray map (lcirs.cc:28-36)
  int32_t ppr;
  cx heap0[5];             // sample 10 of critical-curve branches 0..4: the
                           // warm-start chain's heap state after construction
};

struct LensSpec {          // host-side input of the lens set-up kernel
  double m1, m2, m3;       // m1 = 1 - m2 - m3 (lens.cc:13)
  double z2x;              // z2 = (a, 0)
  double z3x, z3y;         // z3 = (b cos th, b sin th), host libm (lens.cc:38)
  double rho;
  double ld_a, ld_b, intensity;
  int64_t ppr;
  int32_t is_binary_img;   // a == 0 || b == 0 || m3 == 0
  int32_t pad;
};

// Host-side construction of a LensSpec from the reference's constructor
// arguments (lens.cc:4-18, limbdarkeningmodel.cc:8-28).
LensSpec make_lens_spec(double a, double b, double th, double m2, double m3, double rho,
                        long ppr, double ld_a, double ld_b, double intensity);

struct Traj {
  double x0, y0, x1, y1;
  uint32_t n;              // IRS points at t = i/n, i = 0..n (n+1 points)
  int32_t lens;
  int64_t point_base;      // flat index of point 0
};

struct SeedJob {
  int32_t traj;
  int32_t first;           // first point index within the curve
  int32_t count;
  int32_t chain;           // >= 0: start from and save back chains[chain];
                           // -1: start from the lens's construction state
};

// Jobs of one curve of np points: chunk > 0 restarts the warm-start chain
// every chunk points (parallel, fast); chunk <= 0 runs the whole curve as one
// chain, the reference's order (exact).  chain: see SeedJob.
void plan_jobs(std::vector<SeedJob>* jobs, int traj, long np, int chunk, int chain);

struct PointIn {
  double sx, sy;
  int32_t lens;
  uint32_t est_blocks;     // predicted rays / 1024 (point-source magnification)
};

struct PointOut {
  uint64_t count;          // accepted rays
  int64_t wsum_fx;         // sum of weights, fixed point (units of 2^-32)
  uint32_t status;
  uint32_t nseeds;
  uint32_t tiles;          // 32x8 tiles visited
  uint32_t diag;           // bits 0-15: max passes over one tile; 16: pass
                           // limit hit; 17: dequeue limit hit; 24-31: state
  uint64_t rays_eval;      // rays evaluated (FP32 path + FP64 path)
  uint64_t rays_fp64;      // rays evaluated in FP64
};

constexpr double kWsumScale = 4294967296.0;  // 2^32

// ---------------------------------------------------------------------------
// kernels' host launchers (seeds.cu, fill.cu)
// ---------------------------------------------------------------------------
void upload_trig_tables();  // Laguerre kick table + phase samples, once per device

void launch_lens_setup(const LensSpec* d_specs, int nlens, DevLens* d_lenses, cx* d_cc,
                       cx* d_ca, cudaStream_t st);

// caustic-crossing trial points of one point, in the reference's order
// (branch, then segment); n counts every run start, the first kMaxTrials are kept
constexpr int kMaxTrials = 16;
struct TrialList {
  uint32_t n;
  uint32_t pad;
  cx t[kMaxTrials];
};

// seeds of every point: caustic_scan_kernel (warp per chunk, lanes over
// caustic segments) into d_trials, then seeds_kernel (thread per chunk, the
// warm-start chain over the points and their trial points)
void launch_seeds(const SeedJob* d_jobs, int njobs, const Traj* d_trajs, const DevLens* d_lenses,
                  const cx* d_ca, PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                  TrialList* d_trials, RootChain* d_chains, cudaStream_t st);

// caustic-crossing trial points of the points of the given chunks
void launch_caustic_scan(const SeedJob* d_jobs, int njobs, const Traj* d_trajs,
                         const DevLens* d_lenses, const cx* d_ca, TrialList* d_trials,
                         cudaStream_t st);

// history-free part of a point's solve: its polynomial and its cold-start
// roots (the chain takes them whenever the reference solves cold)
struct PointPrep {
  cx coef[11];
  cx cold[10];
};

// Seeds with one warm-start chain per curve, the reference's order
// (chain.cu): the caustic scan and PointPrep over the point chunks of
// scan_jobs, then one warp per chain job.
void launch_seeds_exact(const SeedJob* d_scan_jobs, int nscan, const SeedJob* d_chain_jobs,
                        int nchain, const Traj* d_trajs, const DevLens* d_lenses, const cx* d_ca,
                        PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                        TrialList* d_trials, PointPrep* d_prep, RootChain* d_chains,
                        cudaStream_t st);
void upload_chain_tables(const TrigTable& t);
// the two parts of launch_seeds_exact, for chains run in segments: the
// caustic scan and PointPrep of the scan jobs; the chain jobs (a job with
// chain >= 0 starts from chains[chain] and leaves its state there)
void launch_seeds_prep(const SeedJob* d_scan_jobs, int nscan, const Traj* d_trajs,
                       const DevLens* d_lenses, const cx* d_ca, TrialList* d_trials,
                       PointPrep* d_prep, cudaStream_t st);
void launch_chain(const SeedJob* d_chain_jobs, int nchain, const Traj* d_trajs,
                  const DevLens* d_lenses, PointIn* d_points, int32_t* d_seeds, PointOut* d_out,
                  const TrialList* d_trials, const PointPrep* d_prep, RootChain* d_chains,
                  cudaStream_t st);
// chains[t] = the construction state of curve t's lens
void launch_chain_reset(const Traj* d_trajs, int ntraj, const DevLens* d_lenses,
                        RootChain* d_chains, cudaStream_t st);
// point-source curve with one warm-start chain per job (chain.cu)
void launch_point_lc_exact(const Traj* d_trajs, const SeedJob* d_jobs, int njobs,
                           const DevLens* d_lenses, double* d_amp, RootChain* d_chains,
                           cudaStream_t st);

void launch_point_lc(const Traj* d_trajs, const SeedJob* d_jobs, int njobs,
                     const DevLens* d_lenses, double* d_amp, RootChain* d_chains,
                     cudaStream_t st);

struct FillScratch {
  uint64_t* keys;          // [ctas << cap_log2]
  uint32_t* recs;          // [ctas << cap_log2][32 words]
  uint32_t* ring;          // [ctas << cap_log2]
  uint32_t* used;          // [ctas << cap_log2]
  // super-tile expansion table (split-precision ray map), per CTA
  uint64_t* skeys;         // [ctas << kSuperLog2]
  uint32_t* sents;         // [ctas << kSuperLog2][32 words]
  uint32_t* sused;         // [ctas << kSuperLog2]
  unsigned* next_point;    // work counters: [0] the point list, [1] its large-point head
  int ctas;
  int cap_log2;
  // the first big_ctas CTAs own tables of 2^big_log2 blocks and take the
  // head of a size-ordered point list (its first *nbig entries) first
  int big_ctas;
  int big_log2;
  const unsigned* nbig;
  int block_h;             // rows per block (8, 16 or 32)
  int rec_words;           // 32-bit words per block record
  // optional export of the filled masks: records of kDumpWords words
  // (point, tx, ty, F[8]); nullptr disables it
  uint32_t* dump;
  unsigned* dump_count;
  unsigned dump_cap;
  // optional profiling counters (8 x u64): tiles, cycles in tiles, idle
  // polls, cycles in work loops, super-tiles, cycles building super-tiles,
  // cycles evaluating rays, cycles pushing
  unsigned long long* prof;
  // optional heartbeat in host-mapped memory: one 64-bit word per warp,
  // (phase << 56) | (point << 24) | step (debugging of slow points)
  unsigned long long* heartbeat;
};
constexpr int kDumpWords = 11;
constexpr int kSuperLog2 = 12;   // super-tile table capacity per CTA (entries)

int block_rec_words(int bh);
size_t fill_scratch_bytes(int ctas, int cap_log2, int bh, int big_ctas = 0, int big_log2 = 0);
void fill_scratch_init(FillScratch* s, void* base, int ctas, int cap_log2, int bh,
                       cudaStream_t st, int big_ctas = 0, int big_log2 = 0);

// Size-ordered work list for the fill: points by decreasing predicted size
// (PointIn::est_blocks, from the point-source magnification).  meta[0] =
// number of points, meta[1] = number of points predicted at or above
// big_units blocks of 1024 rays (the list's head); meta needs 2 + 2*64 words.
void launch_order(const PointIn* d_points, int npoints, int32_t* d_list, unsigned* d_meta,
                  unsigned big_units, cudaStream_t st);

enum FillMode : int { kFillFp64 = 0, kFillSplit = 1 };

// d_list/d_count (optional): process only the listed points
void launch_fill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                 const int32_t* d_seeds, PointOut* d_out, const FillScratch& s, int mode,
                 int threads, cudaStream_t st, const int32_t* d_list = nullptr,
                 const unsigned* d_count = nullptr);

void launch_collect_overflow(PointOut* d_out, int npoints, int32_t* d_list, unsigned* d_count,
                             cudaStream_t st);

// block-table sizes tried in turn for points whose table overflows:
// (CTAs, log2 of the table's capacity in 32x8 tiles); CTAs <= 0 means two
// per SM.  A table of 2^k tiles holds 2^k / (BH/8) blocks.
constexpr int kFillLevels = 3;
constexpr int kFillLevelCtas[kFillLevels] = {0, 64, 16};
constexpr int kFillLevelLog2[kFillLevels] = {17, 20, 22};

int fill_default_ctas();        // SMs x fill_occupancy()
void set_fill_occupancy(int occ);  // 2, 3 or 4 resident fill CTAs per SM
int fill_occupancy();

// ---------------------------------------------------------------------------
// Warp fill (fill.cu, wfill_kernel): one warp fills one point alone.  Its
// blocks of 32 x 32 rays live in the warp's own hash table in HBM (key,
// 16-word header with the entry masks, the filled border and the state, and
// a 64-word body with the accepted and filled rows); its work stack,
// super-tile expansions and seed pixels in shared memory.  No warp waits for
// another.  Points predicted above `wthr` blocks, and points whose table
// fills up, come back with status bit 4 for the CTA fill's levels.
// ---------------------------------------------------------------------------
constexpr int kWCapLog2 = 16;                 // largest warp table (log2 of its slots)
constexpr int kWCapLog2Min = 10;
constexpr int kWHdrWords = 16;
struct WScratch {
  uint64_t* keys;          // [warps << cap_log2]
  uint32_t* hdr;           // [warps << cap_log2][kWHdrWords]
  uint32_t* body;          // [warps << cap_log2][64]
  uint32_t* used;          // [warps << cap_log2] slots used by the current point
  uint32_t* spill;         // [warps << cap_log2] work stack beyond its shared part
  unsigned* next_point;
  int warps;
  int cap_log2;            // slots per warp table (log2), kWCapLog2Min..kWCapLog2
  uint32_t wthr;           // points predicted above this many blocks go to the CTA fill
  uint32_t* dump;          // optional amoeba export, as FillScratch
  unsigned* dump_count;
  unsigned dump_cap;
  // optional counters (8 x u64): block visits, first visits, super-tile
  // expansions computed, probe rounds, slots inserted, visits filled whole
  // by the simple-region test, visits with ray-by-ray weights, points
  unsigned long long* prof;
  // team fill only: message inboxes [teams][2][8][inbox_cap]
  uint4* inbox;
  unsigned inbox_cap;
};
int wfill_default_warps();      // SMs x resident warp-fill warps per SM
size_t wscratch_bytes(int warps, int cap_log2);
void wscratch_init(WScratch* s, void* base, int warps, int cap_log2, cudaStream_t st);
// Team fill (fill.cu, tfill_kernel): 8 warps of a CTA fill one large point
// in rounds; each warp owns the blocks of its share of the super-tiles (its
// own table, laid out as the warp fill's: teams x 8 tables) and sends the
// entries into other shares as messages, read at the next round.
int tfill_default_teams();      // 2 per SM
size_t tscratch_bytes(int teams, int cap_log2, unsigned inbox_cap);
void tscratch_init(WScratch* s, void* base, int teams, int cap_log2, unsigned inbox_cap,
                   cudaStream_t st);
void launch_tfill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                  const int32_t* d_seeds, PointOut* d_out, const WScratch& s, int mode,
                  cudaStream_t st, const int32_t* d_list = nullptr,
                  const unsigned* d_count = nullptr);
// d_list/d_count (optional): process only the listed points.  ctas_per_sm
// (1..7, 0: all 8) caps the resident CTAs per SM and leaves room for a
// one-warp kernel of up to 255 registers beside them (the exact chain).
void launch_wfill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                  const int32_t* d_seeds, PointOut* d_out, const WScratch& s, int mode,
                  cudaStream_t st, const int32_t* d_list = nullptr,
                  const unsigned* d_count = nullptr, int ctas_per_sm = 0);

// Seeds and fill of an exact chain overlapped (Engine::pipeline_exact): the
// chain runs in nseg segments (segjobs[segjob0[s] .. segjob0[s+1]) carry
// every curve's state in chains), and while segment s+1's chain runs the
// warp fill works segment s's points (seglist[segoff[s] ..), segn[s] on the
// device).
struct Pipeline {
  const DevLens* lenses;
  const cx* ca;
  const SeedJob* scan;
  int nscan;
  int ntraj;
  const SeedJob* segjobs;
  const int* segjob0;      // host, nseg + 1
  const int32_t* seglist;
  const int* segoff;       // host, nseg + 1
  const unsigned* segn;    // device, nseg
  int nseg;
  PointPrep* prep;
  RootChain* chains;
  bool reset_chains = true;   // false: chains hold each curve's state already (objects)
};

}  // namespace tl
