// fill.cu - persistent amoeba kernel: the filled set of every source
// position, grown as a frontier of 32x8 ray tiles.
//
// What it computes (lcirs.cc:171-174 + lineFloodFill lcirs.cc:381-466 +
// Amoeba amoeba.cc:15-82): the union of the 4-connected components (same row
// neighbours, same column in the rows above/below) of the accepted rays
// {r^2 < rho^2} that contain a seed pixel, over columns 1..N-1 and rows
// 0..N-1 (seeds only on rows 1..N-1).  Per point: number of rays in that set
// and the sum of their limb-darkened weights.
//
// Layout:
//   * one CTA works on one source position at a time, taking positions from
//     a global counter (persistent grid, a few CTAs per SM);
//   * per CTA a tile table in HBM: 64-bit tile keys (open addressing,
//     linear probing) and 128-byte tile records holding the pending entry
//     bits (seeds, bottom row, top row, left/right columns), the tile state
//     (QUEUED/BUSY), the accepted mask H (8 rows x 32 bits) and the filled
//     mask F;
//   * per CTA a work ring of tile slots; counters live in shared memory.
// A warp processes one tile: lane = column, 8 rows per lane; __ballot_sync
// builds the 8 row masks; the closure of the entry bits inside the tile is a
// bit-parallel run fill (carry propagation) plus shuffles between rows;
// newly filled border bits are pushed to the four neighbour tiles.  Closure
// distributes over union, so the order in which tiles and entries are
// processed does not change the result.
//
// Every wait is bounded: an expired wait sets kStTimeout on the point and the
// CTA abandons that point.  A full table sets kStTableFull.
#include <cuda_runtime.h>
#include <stdint.h>

#include "engine.h"

namespace tl {

namespace {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr int kRecWords = 32;
// record layout (32-bit words)
constexpr int kRSeed = 0;    // [0..7]  seed entry bits per row
constexpr int kRBot = 8;     // entries into row 0 from the tile below
constexpr int kRTop = 9;     // entries into row 7 from the tile above
constexpr int kRLR = 10;     // bits 0-7: column 0 per row; bits 8-15: column 31
constexpr int kRState = 11;  // kQueued | kBusy
constexpr int kRHDone = 12;  // H computed
constexpr int kRH = 16;      // [16..23] accepted mask
constexpr int kRF = 24;      // [24..31] filled mask
constexpr uint32_t kQueued = 1u, kBusy = 2u;

constexpr unsigned kIdleSpinLimit = 1u << 21;   // x ~100 ns sleeps
constexpr unsigned long long kPointDeadlineNs = 20ull * 1000000000ull;  // per point

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}
constexpr unsigned kEntrySpinLimit = 1u << 20;

struct Ctx {
  double sx, sy;
  double cx0, cy0, h;
  double rho, rho2, ld_a, ld_b;
  double m1, m2, m3;
  double z2x, z3x, z3y;
  int64_t n;
  int32_t binary;
  int32_t txmax, tymax;
  int32_t split;      // 1: FP32 split-precision ray map with FP64 guard band
  int32_t slog2;      // super-tile edge = 2^slog2 pixels
  float hf, rho2f, inv_rho2f, ldaf, ldbf;
};

struct Shared {
  Ctx c;
  unsigned head, tail, pending, used, sused;
  unsigned abort_, status;
  unsigned long long count, wsum, rays_eval, rays_fp64;
  unsigned long long t0;
  unsigned dbg_again, dbg_state, dbg_slot, dbg_deq, max_pass;
  int point;
};

__device__ __forceinline__ uint32_t ldcg32(const uint32_t* p) { return __ldcg(p); }
__device__ __forceinline__ uint64_t ldcg64(const uint64_t* p) {
  return (uint64_t)__ldcg((const unsigned long long*)p);
}

__device__ __forceinline__ uint64_t tile_key(int tx, int ty) {
  return ((uint64_t)(uint32_t)ty << 32) | (uint32_t)tx;
}

__device__ __forceinline__ uint32_t hash_key(uint64_t k) {
  k ^= k >> 31;
  k *= 0x7fb5d329728ea185ull;
  k ^= k >> 27;
  k *= 0x81dadef4bc2dd44dull;
  k ^= k >> 33;
  return (uint32_t)k;
}

// FP64 ray map in the reference's irsSIMD lane order (lcirs.cc:290-341):
// lanes (z3, z2, z1, zeta_s); every operation separately rounded.
__device__ __forceinline__ double irs_exact(const Ctx& c, double x, double y) {
  if (c.binary) {
    // irsBinary (lcirs.cc:345-353) with the naive complex division
    cx img = mk(x, y);
    cx w1 = mk(__dsub_rn(img.re, 0.0), __dsub_rn(img.im, 0.0));
    double d1 = __dadd_rn(__dmul_rn(w1.re, w1.re), __dmul_rn(w1.im, w1.im));
    // m1 / conj(w1) = (m1*w1.re + 0*(-w1.im))/d1 , (0*w1.re - m1*(-w1.im))/d1
    double q1r = __ddiv_rn(__dadd_rn(__dmul_rn(c.m1, w1.re), __dmul_rn(0.0, -w1.im)), d1);
    double q1i = __ddiv_rn(__dsub_rn(__dmul_rn(0.0, w1.re), __dmul_rn(c.m1, -w1.im)), d1);
    cx w2 = mk(__dsub_rn(img.re, c.z2x), __dsub_rn(img.im, 0.0));
    double d2 = __dadd_rn(__dmul_rn(w2.re, w2.re), __dmul_rn(w2.im, w2.im));
    double q2r = __ddiv_rn(__dadd_rn(__dmul_rn(c.m2, w2.re), __dmul_rn(0.0, -w2.im)), d2);
    double q2i = __ddiv_rn(__dsub_rn(__dmul_rn(0.0, w2.re), __dmul_rn(c.m2, -w2.im)), d2);
    double tr = __dsub_rn(__dsub_rn(img.re, q1r), q2r);
    double ti = __dsub_rn(__dsub_rn(img.im, q1i), q2i);
    double er = __dsub_rn(tr, c.sx), ei = __dsub_rn(ti, c.sy);
    return __dadd_rn(__dmul_rn(er, er), __dmul_rn(ei, ei));
  }
  const double wr0 = __dsub_rn(c.z3x, x), wr1 = __dsub_rn(c.z2x, x), wr2 = __dsub_rn(0.0, x),
               wr3 = __dsub_rn(c.sx, x);
  const double wi0 = __dsub_rn(c.z3y, y), wi1 = __dsub_rn(0.0, y), wi2 = __dsub_rn(0.0, y),
               wi3 = __dsub_rn(c.sy, y);
  const double n0 = __dadd_rn(__dmul_rn(wr0, wr0), __dmul_rn(wi0, wi0));
  const double n1 = __dadd_rn(__dmul_rn(wr1, wr1), __dmul_rn(wi1, wi1));
  const double n2 = __dadd_rn(__dmul_rn(wr2, wr2), __dmul_rn(wi2, wi2));
  const double c0 = __ddiv_rn(c.m3, n0), c1 = __ddiv_rn(c.m2, n1), c2 = __ddiv_rn(c.m1, n2);
  const double tr0 = __dmul_rn(wr0, c0), tr1 = __dmul_rn(wr1, c1), tr2 = __dmul_rn(wr2, c2),
               tr3 = -wr3;
  const double ti0 = __dmul_rn(wi0, c0), ti1 = __dmul_rn(wi1, c1), ti2 = __dmul_rn(wi2, c2),
               ti3 = -wi3;
  const double sr0 = __dadd_rn(tr0, tr2), sr1 = __dadd_rn(tr1, tr3);
  const double si0 = __dadd_rn(ti0, ti2), si1 = __dadd_rn(ti1, ti3);
  const double sr = __dadd_rn(sr0, sr1), si = __dadd_rn(si0, si1);
  return __dadd_rn(__dmul_rn(sr, sr), __dmul_rn(si, si));
}

// limb-darkened weight of an accepted ray (lcirs.cc:406-407,
// limbdarkeningmodel.cc:45-49)
__device__ __forceinline__ double ray_weight(const Ctx& c, double rsq) {
  const double q = __ddiv_rn(rsq, c.rho2);
  return __dadd_rn(c.ld_a, __dmul_rn(c.ld_b, __dsqrt_rn(__dsub_rn(1.0, q))));
}

__device__ __forceinline__ double grid_x(const Ctx& c, int64_t nx) {
  return __dadd_rn(c.cx0, __dmul_rn(c.h, (double)nx));
}
__device__ __forceinline__ double grid_y(const Ctx& c, int64_t ny) {
  return __dadd_rn(c.cy0, __dmul_rn(c.h, (double)ny));
}

// Runs of h that contain a bit of s (s is first restricted to h):
// carry propagation fills towards the high bits, the bit-reversed version
// towards the low bits.
__device__ __forceinline__ uint32_t run_fill(uint32_t s, uint32_t h) {
  s &= h;
  const uint32_t up = ((s + h) ^ h) & h;
  const uint32_t rs = __brev(s), rh = __brev(h);
  const uint32_t dn = __brev(((rs + rh) ^ rh) & rh);
  return s | up | dn;
}

struct Table {
  uint64_t* keys;
  uint32_t* recs;
  uint32_t* ring;
  uint32_t* used;
  uint32_t mask;
  uint64_t* skeys;
  uint32_t* sents;
  uint32_t* sused;
  uint32_t smask;
};

__device__ __forceinline__ void set_abort(Shared& S, uint32_t st) {
  atomicOr(&S.status, st);
  atomicExch(&S.abort_, 1u);
}

// find or insert tile (tx, ty); returns the slot or -1 (table full / abort)
__device__ int find_or_insert(Shared& S, const Table& T, int tx, int ty) {
  const uint64_t key = tile_key(tx, ty);
  uint32_t i = hash_key(key) & T.mask;
  for (uint32_t probe = 0; probe <= T.mask; probe++, i = (i + 1) & T.mask) {
    uint64_t k = ldcg64(&T.keys[i]);
    if (k == key) return (int)i;
    if (k == kEmptyKey) {
      unsigned long long old =
          atomicCAS((unsigned long long*)&T.keys[i], (unsigned long long)kEmptyKey,
                    (unsigned long long)key);
      if (old == kEmptyKey) {
        const unsigned u = atomicAdd(&S.used, 1u);
        __stcg(&T.used[u], i);  // u < capacity: at most mask+1 slots exist
        if (u >= (T.mask + 1) / 4 * 3) set_abort(S, kStTableFull);
        return (int)i;
      }
      if (old == key) return (int)i;
    }
  }
  set_abort(S, kStTableFull);
  return -1;
}

__device__ __forceinline__ void enqueue(Shared& S, const Table& T, int slot) {
  atomicAdd(&S.pending, 1u);
  const unsigned t = atomicAdd(&S.tail, 1u);
  atomicExch(&T.ring[t & T.mask], (uint32_t)slot + 1u);
}

// one lane: OR entry bits into word `w` of tile (tx, ty) and queue it
__device__ void push(Shared& S, const Table& T, int tx, int ty, int w, uint32_t bits) {
  if (!bits) return;
  if (tx < 0 || ty < 0 || tx > S.c.txmax || ty > S.c.tymax) return;
  if (S.abort_) return;
  const int slot = find_or_insert(S, T, tx, ty);
  if (slot < 0) return;
  uint32_t* rec = T.recs + (size_t)slot * kRecWords;
  // entries that are already filled add nothing
  if (w == kRBot) {
    bits &= ~ldcg32(&rec[kRF + 0]);
  } else if (w == kRTop) {
    bits &= ~ldcg32(&rec[kRF + 7]);
  } else if (w == kRLR) {
    uint32_t keep = 0;
    for (int r = 0; r < 8; r++) {
      const uint32_t f = ldcg32(&rec[kRF + r]);
      if (((bits >> r) & 1u) && !(f & 1u)) keep |= 1u << r;
      if (((bits >> (8 + r)) & 1u) && !(f & 0x80000000u)) keep |= 1u << (8 + r);
    }
    bits = keep;
  } else {
    bits &= ~ldcg32(&rec[kRF + (w - kRSeed)]);
  }
  if (!bits) return;
  atomicOr(&rec[w], bits);
  __threadfence_block();
  const uint32_t old = atomicOr(&rec[kRState], kQueued);
  if (old == 0u) enqueue(S, T, slot);
}

// lane 0: take one slot from the ring; -1 if the ring is empty
__device__ int try_dequeue(Shared& S, const Table& T) {
  for (unsigned spin = 0;; spin++) {
    if (spin > (1u << 22)) {
      atomicAdd(&S.dbg_deq, 1u);
      set_abort(S, kStTimeout);
      return -1;
    }
    const unsigned h = *(volatile unsigned*)&S.head;
    const unsigned t = *(volatile unsigned*)&S.tail;
    if (h == t) return -1;
    if (atomicCAS(&S.head, h, h + 1u) == h) {
      unsigned v;
      unsigned it = 0;
      while ((v = atomicExch(&T.ring[h & T.mask], 0u)) == 0u) {
        if (++it > kEntrySpinLimit) {
          set_abort(S, kStTimeout);
          return -1;
        }
        __nanosleep(32);
      }
      return (int)(v - 1u);
    }
  }
}

// Evaluates the 8 rays of this lane's column in tile (tx, ty) in FP64.
// Returns the 8 row masks (uniform) and keeps each ray's weight in w[].
__device__ __forceinline__ void eval_tile_fp64(const Ctx& c, int tx, int ty, int lane,
                                               uint32_t* H, double* w, unsigned* nrays) {
  const int64_t nx = (int64_t)tx * 32 + lane;
  const bool col_ok = nx >= 1 && nx <= c.n - 1;
  const double x = grid_x(c, nx);
  unsigned evaluated = 0;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int64_t ny = (int64_t)ty * 8 + r;
    bool hit = false;
    w[r] = 0.0;
    if (col_ok && ny <= c.n - 1) {
      const double rsq = irs_exact(c, x, grid_y(c, ny));
      evaluated++;
      hit = rsq < c.rho2;
      if (hit) w[r] = ray_weight(c, rsq);
    }
    H[r] = __ballot_sync(0xffffffffu, hit);
  }
  *nrays = evaluated;
}

// ---------------------------------------------------------------------------
// Split-precision ray map.
//
// The image plane is cut into super-tiles of 2^slog2 x 2^slog2 pixels.  For
// each super-tile a warp computes once, in FP64, the mapped offset of its
// centre pixel from the source, D0 = zeta(Zc) - zeta_s, and the expansion of
// the deflection around Zc in eps = conj(delta):
//   alpha(Zc + delta) - alpha(Zc) = sum_n c_n eps^n,
//   c_n = (-1)^n sum_i m_i u_i^(n+1),   u_i = 1/conj(Zc - z_i).
// A ray at pixel offset delta from the centre then maps in FP32 to
//   s = D0 + delta - sum_{n<=K} c_n eps^n,      r^2 = |s|^2,
// every quantity of size rho, so FP32 rounding is relative to rho, not to
// the coordinates.  K (<= 8) is the smallest order whose tail bound
//   T_K = sum_i m_i |u_i| q_i^(K+1) / (1 - q_i),  q_i = |u_i| |delta|max
// is below u*rho/2; where no K qualifies, the exact difference form
//   s = D0 + delta + sum_i m_i conj(delta / ((W_i + delta) W_i))
// is used in FP32, and where a lens lies inside the super-tile, FP64.
// From the magnitudes of the terms the super-tile also gets an error bound E
// on s and a band B = 4 rho E + 4 E^2 + 4 u rho^2 on r^2: a ray with
// |r^2 - rho^2| <= B is classified by the exact FP64 map (irs_exact), so the
// accepted set is exactly the reference's.
// ---------------------------------------------------------------------------
constexpr float kU32 = 5.9604645e-8f;  // 2^-24
// super-tile entry (32 words)
constexpr int kSState = 0, kSMode = 1, kSK = 2, kSD0x = 3, kSD0y = 4, kSBand = 5, kSC = 6;
constexpr int kSEntryWords = 32;
constexpr uint32_t kModeTaylor = 0, kModeExact32 = 1, kModeFp64 = 2;

struct SuperTile {
  int mode, K;
  int nxc, nyc;
  float d0x, d0y, band;
  float cr[8], ci[8];   // Taylor coefficients c_1..c_K, or W_i (mode 1)
};

__device__ __forceinline__ double shfl_d(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// whole warp: computes the entry of super-tile (sx, sy) into `ent`
__device__ void compute_supertile(const Ctx& c, int sxi, int syi, int lane, uint32_t* ent) {
  const int half = 1 << (c.slog2 - 1);
  const int64_t nxc = ((int64_t)sxi << c.slog2) + half;
  const int64_t nyc = ((int64_t)syi << c.slog2) + half;
  const double zx = c.cx0 + c.h * (double)nxc;
  const double zy = c.cy0 + c.h * (double)nyc;
  const double dmax = c.h * (double)half * 1.4142135623730951;
  // lanes 0..2: one lens each (z1 = 0, z2 = (a, 0), z3)
  double wx = 0.0, wy = 0.0, mi = 0.0;
  if (lane == 0) { wx = zx; wy = zy; mi = c.m1; }
  if (lane == 1) { wx = zx - c.z2x; wy = zy; mi = c.m2; }
  if (lane == 2) { wx = zx - c.z3x; wy = zy - c.z3y; mi = c.m3; }
  const double nw = wx * wx + wy * wy;
  const double inv = lane < 3 ? 1.0 / nw : 0.0;
  const double ux = wx * inv, uy = wy * inv;          // u = 1/conj(W) = W/|W|^2
  double ax = mi * ux, ay = mi * uy;                  // m u
  ax += shfl_d(ax, 1) + shfl_d(ax, 2);
  ay += shfl_d(ay, 1) + shfl_d(ay, 2);
  const double d0x = (zx - c.sx) - shfl_d(ax, 0);
  const double d0y = (zy - c.sy) - shfl_d(ay, 0);
  const double wabs = sqrt(nw);
  const double uabs = lane < 3 ? 1.0 / wabs : 0.0;
  const double q = uabs * dmax;
  // Taylor coefficients in FP32 (relative accuracy suffices): lane i holds
  // m_i u_i^(n+1), reduced over the three lanes
  const float fux = (float)ux, fuy = (float)uy;
  float pr = (float)(mi * ux), pi = (float)(mi * uy);   // m u^1
  float cr[8], ci[8];
#pragma unroll
  for (int n = 0; n < 8; n++) {
    const float tr = pr * fux - pi * fuy, ti = pr * fuy + pi * fux;  // m u^(n+2)
    pr = tr;
    pi = ti;
    float sr = lane < 3 ? pr : 0.f, si = lane < 3 ? pi : 0.f;
    sr += __shfl_sync(0xffffffffu, sr, 1) + __shfl_sync(0xffffffffu, sr, 2);
    si += __shfl_sync(0xffffffffu, si, 1) + __shfl_sync(0xffffffffu, si, 2);
    const float sg = (n & 1) ? 1.f : -1.f;   // (-1)^(n+1) for c_(n+1)
    cr[n] = sg * __shfl_sync(0xffffffffu, sr, 0);
    ci[n] = sg * __shfl_sync(0xffffffffu, si, 0);
  }
  // tail bounds and mode (uniform; computed from lanes 0..2)
  double qmax = 0.0, wmin = 1e300, ex1 = 0.0;
  double tk[9];
  for (int K = 1; K <= 8; K++) {
    double t = 0.0;
    if (lane < 3 && q < 1.0) t = mi * uabs * pow(q, (double)(K + 1)) / (1.0 - q);
    else if (lane < 3) t = 1e300;
    t += shfl_d(t, 1) + shfl_d(t, 2);
    tk[K] = shfl_d(t, 0);
  }
  {
    double a = lane < 3 ? q : 0.0, b = lane < 3 ? wabs : 1e300;
    double e = (lane < 3 && wabs > dmax) ? mi * dmax / (wabs * (wabs - dmax)) : (lane < 3 ? 1e300 : 0.0);
    a = fmax(a, fmax(shfl_d(a, 1), shfl_d(a, 2)));
    b = fmin(b, fmin(shfl_d(b, 1), shfl_d(b, 2)));
    e += shfl_d(e, 1) + shfl_d(e, 2);
    qmax = shfl_d(a, 0);
    wmin = shfl_d(b, 0);
    ex1 = shfl_d(e, 0);
  }
  const double u = (double)kU32;
  const double d0abs = sqrt(d0x * d0x + d0y * d0y);
  int mode = kModeFp64, K = 0;
  double E = 0.0;
  if (qmax < 0.5) {
    for (int k = 1; k <= 8; k++)
      if (tk[k] <= 0.5 * u * c.rho) { K = k; break; }
  }
  if (K > 0) {
    double sc = 0.0, dp = dmax;
    for (int n = 0; n < K; n++) {
      sc += sqrt((double)cr[n] * cr[n] + (double)ci[n] * ci[n]) * dp;
      dp *= dmax;
    }
    E = 2.0 * (u * (3.0 * d0abs + 4.0 * dmax + (4.0 * K + 6.0) * sc) + tk[K]);
    mode = kModeTaylor;
  } else if (wmin > 2.0 * dmax) {
    E = 2.0 * (u * (3.0 * d0abs + 4.0 * dmax) + 12.0 * u * ex1);
    mode = kModeExact32;
  }
  const double band = 4.0 * c.rho * E + 4.0 * E * E + 4.0 * u * c.rho2;
  if (lane == 0) {
    __stcg(&ent[kSMode], (uint32_t)mode);
    __stcg(&ent[kSK], (uint32_t)K);
    __stcg(&ent[kSD0x], __float_as_uint((float)d0x));
    __stcg(&ent[kSD0y], __float_as_uint((float)d0y));
    __stcg(&ent[kSBand], __float_as_uint((float)(band * 1.0001)));
    if (mode == kModeTaylor) {
      for (int n = 0; n < 8; n++) {
        __stcg(&ent[kSC + 2 * n], __float_as_uint(cr[n]));
        __stcg(&ent[kSC + 2 * n + 1], __float_as_uint(ci[n]));
      }
    }
  }
  if (mode == kModeExact32 && lane < 3) {  // W_i in FP32
    __stcg(&ent[kSC + 2 * lane], __float_as_uint((float)wx));
    __stcg(&ent[kSC + 2 * lane + 1], __float_as_uint((float)wy));
  }
  __threadfence();
  __syncwarp();
}

// find-or-compute the super-tile holding tile (tx, ty); whole warp
__device__ bool get_supertile(Shared& S, const Table& T, int tx, int ty, int lane,
                              SuperTile* st) {
  const Ctx& c = S.c;
  const int sh = c.slog2;
  const int sxi = (int)(((int64_t)tx * 32) >> sh);
  const int syi = (int)(((int64_t)ty * 8) >> sh);
  const uint64_t key = tile_key(sxi, syi);
  int slot = -1, mine = 0;
  if (lane == 0) {
    uint32_t i = hash_key(key ^ 0x5bd1e995ull) & T.smask;
    for (uint32_t probe = 0; probe <= T.smask; probe++, i = (i + 1) & T.smask) {
      uint64_t k = ldcg64(&T.skeys[i]);
      if (k == key) { slot = (int)i; break; }
      if (k == kEmptyKey) {
        unsigned long long old = atomicCAS((unsigned long long*)&T.skeys[i],
                                           (unsigned long long)kEmptyKey, (unsigned long long)key);
        if (old == kEmptyKey) {
          const unsigned u = atomicAdd(&S.sused, 1u);
          __stcg(&T.sused[u], i);
          if (u >= (T.smask + 1) / 4 * 3) set_abort(S, kStTableFull);
          slot = (int)i;
          mine = 1;
          break;
        }
        if (old == key) { slot = (int)i; break; }
      }
    }
    if (slot < 0) set_abort(S, kStTableFull);
  }
  slot = __shfl_sync(0xffffffffu, slot, 0);
  mine = __shfl_sync(0xffffffffu, mine, 0);
  if (slot < 0) return false;
  uint32_t* ent = T.sents + (size_t)slot * kSEntryWords;
  if (mine) {
    compute_supertile(c, sxi, syi, lane, ent);
    if (lane == 0) atomicExch(&ent[kSState], 2u);
  } else {
    uint32_t ready = 0;
    if (lane == 0) {
      for (unsigned it = 0; it < (1u << 18); it++) {
        if (atomicAdd(&ent[kSState], 0u) == 2u) { ready = 1; break; }
        __nanosleep(64);
      }
    }
    ready = __shfl_sync(0xffffffffu, ready, 0);
    if (!ready) {  // the computing warp is slow: compute the same values here
      compute_supertile(c, sxi, syi, lane, ent);
      if (lane == 0) atomicExch(&ent[kSState], 2u);
    }
    __threadfence();
  }
  st->mode = (int)ldcg32(&ent[kSMode]);
  st->K = (int)ldcg32(&ent[kSK]);
  st->d0x = __uint_as_float(ldcg32(&ent[kSD0x]));
  st->d0y = __uint_as_float(ldcg32(&ent[kSD0y]));
  st->band = __uint_as_float(ldcg32(&ent[kSBand]));
#pragma unroll
  for (int n = 0; n < 8; n++) {
    st->cr[n] = __uint_as_float(ldcg32(&ent[kSC + 2 * n]));
    st->ci[n] = __uint_as_float(ldcg32(&ent[kSC + 2 * n + 1]));
  }
  const int half = 1 << (sh - 1);
  st->nxc = (sxi << sh) + half;
  st->nyc = (syi << sh) + half;
  return true;
}

template <int K>
__device__ __forceinline__ void taylor_rows(const SuperTile& st, float ex, float bx,
                                            const float* dyr, float* r2) {
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const float ey = -dyr[r];
    float pr = st.cr[K - 1], pi = st.ci[K - 1];
#pragma unroll
    for (int n = K - 2; n >= 0; n--) {
      const float tr = fmaf(pr, ex, fmaf(-pi, ey, st.cr[n]));
      const float ti = fmaf(pr, ey, fmaf(pi, ex, st.ci[n]));
      pr = tr;
      pi = ti;
    }
    const float qr = fmaf(pr, ex, -pi * ey);
    const float qi = fmaf(pr, ey, pi * ex);
    const float sx = bx - qr;
    const float sy = (st.d0y + dyr[r]) - qi;
    r2[r] = fmaf(sx, sx, sy * sy);
  }
}

__device__ __forceinline__ void exact32_rows(const Ctx& c, const SuperTile& st, float dx,
                                             float bx, const float* dyr, float* r2) {
  const float ms[3] = {(float)c.m1, (float)c.m2, (float)c.m3};
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const float dy = dyr[r];
    float sx = bx, sy = st.d0y + dy;
#pragma unroll
    for (int i = 0; i < 3; i++) {
      const float wx = st.cr[i], wy = st.ci[i];
      const float vx = wx + dx, vy = wy + dy;
      const float px = vx * wx - vy * wy, py = vx * wy + vy * wx;   // P = V W
      const float inv = __frcp_rn(fmaf(px, px, py * py));
      const float qx = (dx * px + dy * py) * inv, qy = (dy * px - dx * py) * inv;  // delta/P
      sx = fmaf(ms[i], qx, sx);
      sy = fmaf(-ms[i], qy, sy);   // + m conj(delta/P)
    }
    r2[r] = fmaf(sx, sx, sy * sy);
  }
}

// Evaluates the 8 rays of this lane's column in tile (tx, ty) with the
// split-precision map; rays inside the guard band go through irs_exact.
__device__ __forceinline__ void eval_tile_split(const Ctx& c, const SuperTile& st, int tx, int ty,
                                                int lane, uint32_t* H, float* w, unsigned* nrays,
                                                unsigned* nfp64) {
  const int64_t nx = (int64_t)tx * 32 + lane;
  const bool col_ok = nx >= 1 && nx <= c.n - 1;
  const float dx = c.hf * (float)(int)(nx - st.nxc);
  const float bx = st.d0x + dx;
  float dyr[8], r2[8];
#pragma unroll
  for (int r = 0; r < 8; r++) dyr[r] = c.hf * (float)(int)((int64_t)ty * 8 + r - st.nyc);
  if (st.mode == kModeTaylor) {
    switch (st.K) {
      case 1: taylor_rows<1>(st, dx, bx, dyr, r2); break;
      case 2: taylor_rows<2>(st, dx, bx, dyr, r2); break;
      case 3: taylor_rows<3>(st, dx, bx, dyr, r2); break;
      case 4: taylor_rows<4>(st, dx, bx, dyr, r2); break;
      case 5: taylor_rows<5>(st, dx, bx, dyr, r2); break;
      case 6: taylor_rows<6>(st, dx, bx, dyr, r2); break;
      case 7: taylor_rows<7>(st, dx, bx, dyr, r2); break;
      default: taylor_rows<8>(st, dx, bx, dyr, r2); break;
    }
  } else {
    exact32_rows(c, st, dx, bx, dyr, r2);
  }
  unsigned ev = 0, e64 = 0;
  const float lo = c.rho2f - st.band, hi = c.rho2f + st.band;
#pragma unroll
  for (int r = 0; r < 8; r++) {
    const int64_t ny = (int64_t)ty * 8 + r;
    bool hit = false;
    w[r] = 0.f;
    if (col_ok && ny <= c.n - 1) {
      ev++;
      if (r2[r] < lo) {
        hit = true;
        w[r] = fmaf(c.ldbf, sqrtf(fmaxf(0.f, fmaf(-r2[r], c.inv_rho2f, 1.f))), c.ldaf);
      } else if (r2[r] <= hi) {
        const double rsq = irs_exact(c, grid_x(c, nx), grid_y(c, ny));
        e64++;
        hit = rsq < c.rho2;
        if (hit) w[r] = (float)ray_weight(c, rsq);
      }
    }
    H[r] = __ballot_sync(0xffffffffu, hit);
  }
  *nrays = ev;
  *nfp64 = e64;
}

// FP32 weight of one accepted ray (re-visit of a tile whose rays are no
// longer in registers)
__device__ __forceinline__ float weight_split(const Ctx& c, const SuperTile& st, int64_t nx,
                                              int64_t ny) {
  const float dx = c.hf * (float)(int)(nx - st.nxc);
  float dyr[8], r2[8];
  for (int r = 0; r < 8; r++) dyr[r] = c.hf * (float)(int)(ny - st.nyc);
  const float bx = st.d0x + dx;
  if (st.mode == kModeTaylor) {
    switch (st.K) {
      case 1: taylor_rows<1>(st, dx, bx, dyr, r2); break;
      case 2: taylor_rows<2>(st, dx, bx, dyr, r2); break;
      case 3: taylor_rows<3>(st, dx, bx, dyr, r2); break;
      case 4: taylor_rows<4>(st, dx, bx, dyr, r2); break;
      case 5: taylor_rows<5>(st, dx, bx, dyr, r2); break;
      case 6: taylor_rows<6>(st, dx, bx, dyr, r2); break;
      case 7: taylor_rows<7>(st, dx, bx, dyr, r2); break;
      default: taylor_rows<8>(st, dx, bx, dyr, r2); break;
    }
  } else {
    exact32_rows(c, st, dx, bx, dyr, r2);
  }
  return fmaf(c.ldbf, sqrtf(fmaxf(0.f, fmaf(-r2[0], c.inv_rho2f, 1.f))), c.ldaf);
}

__device__ __forceinline__ double warp_sum(double v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// processes one queued tile (whole warp)
__device__ void process_tile(Shared& S, const Table& T, int slot, int lane) {
  const Ctx& c = S.c;
  const uint64_t key = ldcg64(&T.keys[slot]);
  const int tx = (int)(uint32_t)(key & 0xffffffffu);
  const int ty = (int)(uint32_t)(key >> 32);
  uint32_t* rec = T.recs + (size_t)slot * kRecWords;
  double w[8];
  bool have_w = false;
  SuperTile st;
  bool have_st = false;
  unsigned long long local_count = 0, local_eval = 0, local_fp64 = 0;
  double local_wsum = 0.0;
  uint32_t edge = 0;
  for (int pass = 0;; pass++) {
    if (pass > 4096) {  // a tile re-queued without end: give up on the point
      if (lane == 0) {
        set_abort(S, kStTimeout);
        atomicAdd(&S.dbg_again, 1u);
        S.dbg_state = atomicAdd(&rec[kRState], 0u);
        S.dbg_slot = (unsigned)slot;
      }
      break;
    }
    if (lane == 0) atomicExch(&rec[kRState], kBusy);
    __syncwarp();
    __threadfence_block();
    uint32_t ew = 0;
    if (lane < 11) ew = atomicExch(&rec[lane], 0u);
    const uint32_t ebot = __shfl_sync(0xffffffffu, ew, kRBot);
    const uint32_t etop = __shfl_sync(0xffffffffu, ew, kRTop);
    const uint32_t elr = __shfl_sync(0xffffffffu, ew, kRLR);
    // this lane's row (lanes 0..7)
    uint32_t e_row = 0;
    if (lane < 8) {
      e_row = ew | (lane == 0 ? ebot : 0u) | (lane == 7 ? etop : 0u) | ((elr >> lane) & 1u) |
              (((elr >> (8 + lane)) & 1u) << 31);
    }
    uint32_t Hrow[8];
    uint32_t hdone = 0;
    if (lane == 0) hdone = ldcg32(&rec[kRHDone]);
    hdone = __shfl_sync(0xffffffffu, hdone, 0);
    if (!hdone) {
      unsigned nr, n64;
      if (c.split && !have_st) have_st = get_supertile(S, T, tx, ty, lane, &st);
      if (c.split && have_st && st.mode != kModeFp64) {
        float wf[8];
        eval_tile_split(c, st, tx, ty, lane, Hrow, wf, &nr, &n64);
#pragma unroll
        for (int r = 0; r < 8; r++) w[r] = wf[r];
      } else {
        eval_tile_fp64(c, tx, ty, lane, Hrow, w, &nr);
        n64 = nr;
      }
      have_w = true;
      local_eval += warp_sum_u(nr);
      local_fp64 += warp_sum_u(n64);
      if (lane < 8) __stcg(&rec[kRH + lane], Hrow[lane]);
      __threadfence_block();
      if (lane == 0) __stcg(&rec[kRHDone], 1u);
    } else {
      uint32_t hv = lane < 8 ? ldcg32(&rec[kRH + lane]) : 0u;
#pragma unroll
      for (int r = 0; r < 8; r++) Hrow[r] = __shfl_sync(0xffffffffu, hv, r);
    }
    uint32_t h_lane = 0;  // Hrow is uniform; lane r < 8 keeps row r
#pragma unroll
    for (int r = 0; r < 8; r++)
      if (lane == r) h_lane = Hrow[r];
    const uint32_t f_old = lane < 8 ? ldcg32(&rec[kRF + lane]) : 0u;
    const uint32_t hp = h_lane & ~f_old;  // accepted, not yet filled
    uint32_t f = e_row & hp;
    if (__ballot_sync(0xffffffffu, f != 0u)) {
      // closure inside the tile: rows exchange with the rows above/below
      for (int it = 0; it < 64; it++) {
        uint32_t below = __shfl_up_sync(0xffffffffu, f, 1);
        uint32_t above = __shfl_down_sync(0xffffffffu, f, 1);
        if (lane == 0) below = 0u;
        if (lane >= 7) above = 0u;
        uint32_t nf = lane < 8 ? run_fill(f | ((below | above) & hp), hp) : 0u;
        const unsigned changed = __ballot_sync(0xffffffffu, nf != f);
        f = nf;
        if (!changed) break;
      }
      if (lane < 8) __stcg(&rec[kRF + lane], f_old | f);
      uint32_t nw[8];
#pragma unroll
      for (int r = 0; r < 8; r++) nw[r] = __shfl_sync(0xffffffffu, f, r);
      // weights and count of the newly filled rays
      double acc = 0.0;
      unsigned cnt = 0;
      unsigned re_eval = 0;
      const int64_t nx = (int64_t)tx * 32 + lane;
      if (!have_w && c.split && !have_st) have_st = get_supertile(S, T, tx, ty, lane, &st);
#pragma unroll
      for (int r = 0; r < 8; r++) {
        cnt += __popc(nw[r]);
        if ((nw[r] >> lane) & 1u) {
          if (have_w) {
            acc += w[r];
          } else if (c.split && have_st && st.mode != kModeFp64) {
            acc += (double)weight_split(c, st, nx, (int64_t)ty * 8 + r);
            re_eval++;
          } else {
            const double rsq = irs_exact(c, grid_x(c, nx), grid_y(c, (int64_t)ty * 8 + r));
            acc += ray_weight(c, rsq);
            re_eval++;
          }
        }
      }
      acc = warp_sum(acc);
      re_eval = warp_sum_u(re_eval);
      local_eval += re_eval;
      if (!c.split) local_fp64 += re_eval;
      local_count += cnt;
      local_wsum += acc;
      // plane edge: columns 1 and N-1 are where the reference's row scan
      // stops differently (lcirs.cc:413-440)
      {
        const int64_t c0 = (int64_t)tx * 32;
        uint32_t colmask = 0;
        if (1 >= c0 && 1 < c0 + 32) colmask |= 1u << (1 - c0);
        if (c.n - 1 >= c0 && c.n - 1 < c0 + 32) colmask |= 1u << (c.n - 1 - c0);
        uint32_t any = 0;
#pragma unroll
        for (int r = 0; r < 8; r++) any |= nw[r];
        if (any & colmask) edge = 1;
      }
      // neighbours
      if (lane == 0) {
        push(S, T, tx, ty + 1, kRBot, nw[7]);
      } else if (lane == 1) {
        push(S, T, tx, ty - 1, kRTop, nw[0]);
      } else if (lane == 2) {
        uint32_t b = 0;
#pragma unroll
        for (int r = 0; r < 8; r++) b |= (nw[r] & 1u) << r;
        push(S, T, tx - 1, ty, kRLR, b << 8);  // enters the left tile at its column 31
      } else if (lane == 3) {
        uint32_t b = 0;
#pragma unroll
        for (int r = 0; r < 8; r++) b |= (nw[r] >> 31) << r;
        push(S, T, tx + 1, ty, kRLR, b);  // enters the right tile at its column 0
      }
      __syncwarp();
    }
    __threadfence_block();
    uint32_t again = 0;
    if (lane == 0) again = atomicCAS(&rec[kRState], kBusy, 0u) != kBusy;
    again = __shfl_sync(0xffffffffu, again, 0);
    if (!again) {
      if (lane == 0) atomicMax(&S.max_pass, (unsigned)pass);
      break;
    }
  }
  if (lane == 0) {
    if (local_count) atomicAdd(&S.count, local_count);
    if (local_wsum != 0.0)
      atomicAdd(&S.wsum, (unsigned long long)(long long)llrint(local_wsum * kWsumScale));
    atomicAdd(&S.rays_eval, local_eval);
    atomicAdd(&S.rays_fp64, local_fp64);
    if (edge) atomicOr(&S.status, kStEdge);
  }
}

}  // namespace

__global__ void __launch_bounds__(256)
fill_kernel(const PointIn* points, int npoints, const DevLens* lenses, const int32_t* seeds,
            PointOut* out, FillScratch sc, int split_mode) {
  __shared__ Shared S;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  const size_t cap = (size_t)1 << sc.cap_log2;
  Table T;
  T.keys = sc.keys + (size_t)blockIdx.x * cap;
  T.recs = sc.recs + (size_t)blockIdx.x * cap * kRecWords;
  T.ring = sc.ring + (size_t)blockIdx.x * cap;
  T.used = sc.used + (size_t)blockIdx.x * cap;
  T.mask = (uint32_t)(cap - 1);
  const size_t scap = (size_t)1 << kSuperLog2;
  T.skeys = sc.skeys + (size_t)blockIdx.x * scap;
  T.sents = sc.sents + (size_t)blockIdx.x * scap * kSEntryWords;
  T.sused = sc.sused + (size_t)blockIdx.x * scap;
  T.smask = (uint32_t)(scap - 1);

  for (;;) {
    if (threadIdx.x == 0) {
      S.point = (int)atomicAdd(sc.next_point, 1u);
      S.head = S.tail = S.pending = S.used = S.sused = 0;
      S.abort_ = 0;
      S.count = S.wsum = S.rays_eval = S.rays_fp64 = 0;
      S.status = 0;
      S.t0 = globaltimer();
      S.dbg_again = S.dbg_state = S.dbg_slot = S.dbg_deq = S.max_pass = 0;
      if (S.point < npoints) {
        const PointIn pi = points[S.point];
        const DevLens& D = lenses[pi.lens];
        Ctx& c = S.c;
        c.sx = pi.sx;
        c.sy = pi.sy;
        c.cx0 = D.g.corner_x;
        c.cy0 = D.g.corner_y;
        c.h = D.g.h;
        c.n = D.g.n;
        c.rho = D.rho;
        c.rho2 = D.rho2;
        c.ld_a = D.ld_a;
        c.ld_b = D.ld_b;
        c.m1 = D.L.m1;
        c.m2 = D.L.m2;
        c.m3 = D.L.m3;
        c.z2x = D.L.z2.re;
        c.z3x = D.L.z3.re;
        c.z3y = D.L.z3.im;
        c.binary = D.ray_binary;
        c.txmax = (int)((c.n - 1) >> 5);
        c.tymax = (int)((c.n - 1) >> 3);
        c.split = split_mode;
        // super-tile edge: 2^9 pixels when h is small, down to 2^7 when the
        // grid is coarse (the expansion's ratio |delta|/|W| stays ~1e-3)
        int sl = 9;
        while (sl > 7 && c.h * (double)(1 << sl) > 1.5e-3) sl--;
        c.slog2 = sl;
        c.hf = (float)c.h;
        c.rho2f = (float)c.rho2;
        c.inv_rho2f = (float)(1.0 / c.rho2);
        c.ldaf = (float)c.ld_a;
        c.ldbf = (float)c.ld_b;
        if (!(c.n > 2 && c.n < ((int64_t)1 << 31))) S.status |= kStBadInput;
        if (out[S.point].status & kStBadInput) S.status |= kStBadInput;
      }
    }
    __syncthreads();
    const int p = S.point;
    if (p >= npoints) break;
    const bool skip = (S.status & kStBadInput) != 0;
    // seeds (lcirs.cc:171-174; seed rows must satisfy 0 < ny < N, 386-391)
    if (!skip && warp == 0) {
      const unsigned ns = out[p].nseeds;
      for (unsigned k = lane; k < ns; k += 32) {
        const int32_t sx = seeds[((size_t)p * kMaxSeeds + k) * 2];
        const int32_t sy = seeds[((size_t)p * kMaxSeeds + k) * 2 + 1];
        if (sy <= 0 || (int64_t)sy >= S.c.n) continue;
        if (sx < 1 || (int64_t)sx > S.c.n - 1) {
          atomicOr(&S.status, kStEdge);
          continue;
        }
        push(S, T, sx >> 5, sy >> 3, kRSeed + (sy & 7), 1u << (sx & 31));
      }
    }
    __syncthreads();
    // work loop
    if (!skip) {
      unsigned spins = 0;
      for (;;) {
        int slot = -1;
        if (lane == 0) slot = try_dequeue(S, T);
        slot = __shfl_sync(0xffffffffu, slot, 0);
        if (slot < 0) {
          const unsigned pend = *(volatile unsigned*)&S.pending;
          const unsigned ab = *(volatile unsigned*)&S.abort_;
          if (pend == 0u || ab) break;
          if (++spins > kIdleSpinLimit) {
            if (lane == 0) set_abort(S, kStTimeout);
            break;
          }
          __nanosleep(100);
          continue;
        }
        spins = 0;
        if (lane == 0 && globaltimer() - S.t0 > kPointDeadlineNs) set_abort(S, kStTimeout);
        if (!*(volatile unsigned*)&S.abort_) process_tile(S, T, slot, lane);
        if (lane == 0) atomicSub(&S.pending, 1u);
      }
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      PointOut o = out[p];
      o.count = S.count;
      o.wsum_fx = (int64_t)S.wsum;
      o.status |= S.status;
      o.tiles = S.used;
      o.diag = S.max_pass | (S.dbg_again ? 0x10000u : 0u) | (S.dbg_deq ? 0x20000u : 0u) |
              ((S.dbg_state & 0xffu) << 24);
      o.rays_eval = S.rays_eval;
      o.rays_fp64 = S.rays_fp64;
      out[p] = o;
    }
    // clear the slots this point used (tables start every point empty)
    const unsigned nused = S.used < cap ? S.used : (unsigned)cap;
    for (unsigned u = threadIdx.x; u < nused; u += blockDim.x) {
      const uint32_t slot = __ldcg(&T.used[u]);
      if (sc.dump) {
        uint32_t fm[8], any = 0;
        for (int r = 0; r < 8; r++) any |= (fm[r] = ldcg32(&T.recs[(size_t)slot * kRecWords + kRF + r]));
        if (any) {
          const unsigned d = atomicAdd(sc.dump_count, 1u);
          if (d < sc.dump_cap) {
            const uint64_t key = ldcg64(&T.keys[slot]);
            uint32_t* o = sc.dump + (size_t)d * kDumpWords;
            o[0] = (uint32_t)p;
            o[1] = (uint32_t)(key & 0xffffffffu);
            o[2] = (uint32_t)(key >> 32);
            for (int r = 0; r < 8; r++) o[3 + r] = fm[r];
          }
        }
      }
      __stcg((unsigned long long*)&T.keys[slot], (unsigned long long)kEmptyKey);
      uint4* r4 = (uint4*)(T.recs + (size_t)slot * kRecWords);
#pragma unroll
      for (int q = 0; q < kRecWords / 4; q++) __stcg(&r4[q], make_uint4(0u, 0u, 0u, 0u));
    }
    const unsigned nsu = S.sused < scap ? S.sused : (unsigned)scap;
    for (unsigned u = threadIdx.x; u < nsu; u += blockDim.x) {
      const uint32_t slot = __ldcg(&T.sused[u]);
      __stcg((unsigned long long*)&T.skeys[slot], (unsigned long long)kEmptyKey);
      uint4* r4 = (uint4*)(T.sents + (size_t)slot * kSEntryWords);
#pragma unroll
      for (int q = 0; q < kSEntryWords / 4; q++) __stcg(&r4[q], make_uint4(0u, 0u, 0u, 0u));
    }
    if (S.abort_) {
      const unsigned nt = S.tail < cap ? S.tail : (unsigned)cap;
      for (unsigned u = threadIdx.x; u < nt; u += blockDim.x) __stcg(&T.ring[u], 0u);
    }
    // the next point reads these words through L2 (ld.cg and atomics): the
    // clears must have reached L2 before any thread of the block goes on
    __threadfence();
    __syncthreads();
  }
}

size_t fill_scratch_bytes(int ctas, int cap_log2) {
  const size_t cap = (size_t)1 << cap_log2;
  const size_t scap = (size_t)1 << kSuperLog2;
  return (size_t)ctas * cap * (8 + kRecWords * 4 + 4 + 4) +
         (size_t)ctas * scap * (8 + kSEntryWords * 4 + 4) + 256;
}

void fill_scratch_init(FillScratch* s, void* base, int ctas, int cap_log2, cudaStream_t st) {
  const size_t cap = (size_t)1 << cap_log2;
  char* p = (char*)base;
  s->ctas = ctas;
  s->cap_log2 = cap_log2;
  s->keys = (uint64_t*)p;
  p += (size_t)ctas * cap * 8;
  s->recs = (uint32_t*)p;
  p += (size_t)ctas * cap * kRecWords * 4;
  s->ring = (uint32_t*)p;
  p += (size_t)ctas * cap * 4;
  s->used = (uint32_t*)p;
  p += (size_t)ctas * cap * 4;
  const size_t scap = (size_t)1 << kSuperLog2;
  s->skeys = (uint64_t*)p;
  p += (size_t)ctas * scap * 8;
  s->sents = (uint32_t*)p;
  p += (size_t)ctas * scap * kSEntryWords * 4;
  s->sused = (uint32_t*)p;
  p += (size_t)ctas * scap * 4;
  s->next_point = (unsigned*)p;
  s->dump = nullptr;
  s->dump_count = nullptr;
  s->dump_cap = 0;
  cudaMemsetAsync(s->keys, 0xff, (size_t)ctas * cap * 8, st);
  cudaMemsetAsync(s->recs, 0, (size_t)ctas * cap * kRecWords * 4, st);
  cudaMemsetAsync(s->ring, 0, (size_t)ctas * cap * 4, st);
  cudaMemsetAsync(s->skeys, 0xff, (size_t)ctas * scap * 8, st);
  cudaMemsetAsync(s->sents, 0, (size_t)ctas * scap * kSEntryWords * 4, st);
}

int fill_default_ctas() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms * 2 : 2;
}

void launch_fill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                 const int32_t* d_seeds, PointOut* d_out, const FillScratch& s, int mode,
                 int threads, cudaStream_t st) {
  if (npoints <= 0) return;
  cudaMemsetAsync(s.next_point, 0, sizeof(unsigned), st);
  const int ctas = s.ctas;
  fill_kernel<<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out, s,
                                        mode == kFillSplit ? 1 : 0);
}

}  // namespace tl
