// fill.cu - persistent amoeba kernel: the filled set of every source
// position, grown as a frontier of ray blocks (32 columns x BH rows, made of
// BH/8 tiles of 32x8 rays; BH in {8, 16, 32} is chosen by the autotuner).
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
//     a size-ordered list, largest first (persistent grid, 2-4 CTAs per SM;
//     the first CTAs own 4x larger tables and take the list's head);
//   * per CTA a block table in HBM: 64-bit block keys (open addressing,
//     linear probing, one CAS per probe) and block records holding the
//     pending entry bits (seed rows, bottom row, top row, left and right
//     columns), a state word (queued | busy | accepted-mask-done), the
//     accepted mask H (BH rows x 32 bits), the filled mask F and the F
//     column summaries used to filter pushes;
//   * per CTA a work ring of block slots; counters in shared memory.
// A warp processes one block: lane = column, BH rays per lane, hits kept
// as a per-lane column mask and turned into row masks by one ballot per row;
// lane r < BH then holds row r, and the
// closure of the entry bits is a bit-parallel run fill (carry propagation)
// with shuffles between neighbouring rows; newly filled border bits are
// pushed to the four neighbour blocks.  Closure distributes over union, so
// the processing order of blocks and entries does not change the result.
//
// Every wait is bounded: an expired wait sets kStTimeout on the point and the
// CTA abandons that point.  A full table sets kStTableFull (the host retries
// those points with larger tables).
#include <cuda_runtime.h>

#include <algorithm>
#include <stdint.h>

#include <cmath>

#include "engine.h"

namespace tl {

namespace {

constexpr uint64_t kEmptyKey = ~0ull;
constexpr uint32_t kQ = 1u, kB = 2u, kD = 4u;   // queued, busy, H done

template <int BH>
struct Lo {
  static constexpr int kBot = BH, kTop = BH + 1, kLeft = BH + 2, kRight = BH + 3;
  static constexpr int kState = BH + 4, kFl = BH + 5, kFr = BH + 6;
  static constexpr int kH = BH + 8, kF = 2 * BH + 8;
  static constexpr int kWords = (3 * BH + 8) <= 32 ? 32 : ((3 * BH + 8) <= 64 ? 64 : 128);
};

constexpr unsigned kIdleSpinLimit = 1u << 21;   // x ~100 ns sleeps
constexpr unsigned kEntrySpinLimit = 1u << 20;
constexpr unsigned long long kPointDeadlineNs = 5ull * 1000000000ull;  // per point

__device__ __forceinline__ unsigned long long globaltimer() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

__device__ __forceinline__ void beat(unsigned long long* hb, int phase, int point, unsigned step) {
  if (hb) {
    const int w = blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
    *(volatile unsigned long long*)&hb[w] =
        ((unsigned long long)phase << 56) | ((unsigned long long)(point & 0xffffffff) << 24) |
        (step & 0xffffff);
  }
}

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
  unsigned dbg_again, dbg_deq, max_pass, profiling, dbg_where;
  unsigned long long prof[8];  // profiling counters (sc.prof != nullptr)
  unsigned long long* hb;
  int point;
};

// true (and the point aborted, with `where` recorded) once the point has run
// past its deadline
__device__ __forceinline__ bool overdue(Shared& S, unsigned where) {
  if (globaltimer() - S.t0 <= kPointDeadlineNs) return false;
  atomicCAS(&S.dbg_where, 0u, where);
  atomicOr(&S.status, kStTimeout);
  atomicExch(&S.abort_, 1u);
  return true;
}

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

// m / conj(w) for real m, as complex<double>(m) / conj(w) divides in a strict
// IEEE build: Smith's algorithm (R. L. Smith, CACM 5(8), 1962) with the
// numerator's zero imaginary part kept in every operation
__device__ __forceinline__ void rdiv_conj(double m, double wr, double wi, double* qr, double* qi) {
  const double br = wr, bi = -wi;
  if (fabs(br) < fabs(bi)) {
    const double r = __ddiv_rn(br, bi), den = __dadd_rn(__dmul_rn(br, r), bi);
    if (fabs(r) > 2.2250738585072014e-308) {
      *qr = __ddiv_rn(__dadd_rn(__dmul_rn(m, r), 0.0), den);
      *qi = __ddiv_rn(__dsub_rn(__dmul_rn(0.0, r), m), den);
    } else {
      *qr = __ddiv_rn(__dadd_rn(__dmul_rn(br, __ddiv_rn(m, bi)), 0.0), den);
      *qi = __ddiv_rn(__dsub_rn(__dmul_rn(br, __ddiv_rn(0.0, bi)), m), den);
    }
  } else {
    const double r = __ddiv_rn(bi, br), den = __dadd_rn(__dmul_rn(bi, r), br);
    if (fabs(r) > 2.2250738585072014e-308) {
      *qr = __ddiv_rn(__dadd_rn(__dmul_rn(0.0, r), m), den);
      *qi = __ddiv_rn(__dsub_rn(0.0, __dmul_rn(m, r)), den);
    } else {
      *qr = __ddiv_rn(__dadd_rn(m, __dmul_rn(bi, __ddiv_rn(0.0, br))), den);
      *qi = __ddiv_rn(__dsub_rn(0.0, __dmul_rn(bi, __ddiv_rn(m, br))), den);
    }
  }
}

// FP64 ray map in the reference's irsSIMD lane order (lcirs.cc:290-341):
// lanes (z3, z2, z1, zeta_s); every operation separately rounded.
__device__ __noinline__ double irs_exact(const Ctx& c, double x, double y) {
  if (c.binary) {
    // irsBinary (lcirs.cc:345-353): img - m1/conj(img - z1) - m2/conj(img - z2),
    // each quotient by Smith's complex division (the strict build's __divdc3)
    double q1r, q1i, q2r, q2i;
    rdiv_conj(c.m1, __dsub_rn(x, 0.0), __dsub_rn(y, 0.0), &q1r, &q1i);
    rdiv_conj(c.m2, __dsub_rn(x, c.z2x), __dsub_rn(y, 0.0), &q2r, &q2i);
    const double tr = __dsub_rn(__dsub_rn(x, q1r), q2r);
    const double ti = __dsub_rn(__dsub_rn(y, q1i), q2i);
    const double er = __dsub_rn(tr, c.sx), ei = __dsub_rn(ti, c.sy);
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
  int rec_words;
  uint64_t* skeys;
  uint32_t* sents;
  uint32_t* sused;
  uint32_t smask;
};

__device__ __forceinline__ void set_abort(Shared& S, uint32_t st) {
  atomicOr(&S.status, st);
  atomicExch(&S.abort_, 1u);
}

// find or insert block (bx, by): one CAS per probe; -1 if the table is full
__device__ __noinline__ int find_or_insert(Shared& S, const Table& T, int bx, int by) {
  const uint64_t key = tile_key(bx, by);
  uint32_t i = hash_key(key) & T.mask;
  for (uint32_t probe = 0; probe <= T.mask; probe++, i = (i + 1) & T.mask) {
    if ((probe & 255) == 255 && overdue(S, 1)) return -1;
    const unsigned long long old = atomicCAS((unsigned long long*)&T.keys[i],
                                             (unsigned long long)kEmptyKey,
                                             (unsigned long long)key);
    if (old == kEmptyKey) {
      const unsigned u = atomicAdd(&S.used, 1u);
      __stcg(&T.used[u], i);  // u < capacity: at most mask+1 slots exist
      if (u >= (T.mask + 1) / 4 * 3) set_abort(S, kStTableFull);
      return (int)i;
    }
    if (old == key) return (int)i;
  }
  set_abort(S, kStTableFull);
  return -1;
}

__device__ __forceinline__ void enqueue(Shared& S, const Table& T, int slot) {
  atomicAdd(&S.pending, 1u);
  const unsigned t = atomicAdd(&S.tail, 1u);
  atomicExch(&T.ring[t & T.mask], (uint32_t)slot + 1u);
}

enum PushKind { kPushSeed = 0, kPushBot, kPushTop, kPushLeft, kPushRight };

// one lane: post entry bits into block (bx, by) and queue it.  `row` is the
// row of a seed entry.  Bits that the target has already filled are dropped
// (the F rows and the F column summaries are read for that).
template <int BH>
__device__ __noinline__ void push(Shared& S, const Table& T, int bx, int by, int kind, int row,
                                  uint32_t bits) {
  using L = Lo<BH>;
  if (!bits) return;
  if (bx < 0 || by < 0 || bx > S.c.txmax || by > S.c.tymax) return;
  if (S.abort_) return;
  const int slot = find_or_insert(S, T, bx, by);
  if (slot < 0) return;
  uint32_t* rec = T.recs + (size_t)slot * T.rec_words;
  int w;
  uint32_t filled;
  switch (kind) {
    case kPushBot: w = L::kBot; filled = ldcg32(&rec[L::kF + 0]); break;
    case kPushTop: w = L::kTop; filled = ldcg32(&rec[L::kF + BH - 1]); break;
    case kPushLeft: w = L::kLeft; filled = ldcg32(&rec[L::kFl]); break;
    case kPushRight: w = L::kRight; filled = ldcg32(&rec[L::kFr]); break;
    default: w = row; filled = ldcg32(&rec[L::kF + row]); break;
  }
  bits &= ~filled;
  if (!bits) return;
  atomicOr(&rec[w], bits);
  __threadfence_block();
  const uint32_t old = atomicOr(&rec[L::kState], kQ);
  if ((old & (kQ | kB)) == 0u) enqueue(S, T, slot);
}

// lane 0: take one slot from the ring; -1 if the ring is empty
__device__ __noinline__ int try_dequeue(Shared& S, const Table& T) {
  for (unsigned spin = 0;; spin++) {
    if (spin > (1u << 22)) {
      atomicAdd(&S.dbg_deq, 1u);
      set_abort(S, kStTimeout);
      return -1;
    }
    if ((spin & 1023) == 1023 && overdue(S, 2)) return -1;
    const unsigned h = *(volatile unsigned*)&S.head;
    const unsigned t = *(volatile unsigned*)&S.tail;
    if (h == t) return -1;
    if (atomicCAS(&S.head, h, h + 1u) == h) {
      unsigned v;
      unsigned it = 0;
      while ((v = atomicExch(&T.ring[h & T.mask], 0u)) == 0u) {
        if ((it & 255) == 255 && overdue(S, 3)) return -1;
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

__device__ __forceinline__ float warp_sum_f(float v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

__device__ __forceinline__ unsigned warp_sum_u(unsigned v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
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
// the coordinates.  The expansion is used where some order K <= 4 has a tail
// bound
//   T_K = sum_i m_i |u_i| q_i^(K+1) / (1 - q_i),  q_i = |u_i| |delta|max
// below u*rho/2, and then always with K = 4 terms (one compiled variant);
// where no K qualifies, the exact difference form
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
  float cr[4], ci[4];   // Taylor coefficients c_1..c_K, or W_i (mode 1)
};

__device__ __forceinline__ double shfl_d(double v, int src) {
  return __shfl_sync(0xffffffffu, v, src);
}

// whole warp: the expansion of super-tile (sx, sy) (every lane leaves with
// the same values)
__device__ __noinline__ void supertile_values(const Ctx& c, int sxi, int syi, int lane,
                                              SuperTile* out) {
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
  float cr[4], ci[4];
#pragma unroll
  for (int n = 0; n < 4; n++) {
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
  double tk[5];
  {
    const double tail0 = (lane < 3 && q < 1.0) ? mi * uabs / (1.0 - q) : 0.0;
    double qp = q;
    for (int K = 1; K <= 4; K++) {
      qp *= q;   // q^(K+1)
      double t = 0.0;
      if (lane < 3 && q < 1.0) t = tail0 * qp;
      else if (lane < 3) t = 1e300;
      t += shfl_d(t, 1) + shfl_d(t, 2);
      tk[K] = shfl_d(t, 0);
    }
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
    for (int k = 1; k <= 4; k++)
      if (tk[k] <= 0.5 * u * c.rho) { K = k; break; }
  }
  // one compiled order keeps the kernels' hot code small (instruction fetch
  // is their largest stall): every expansion uses 4 terms (more terms only
  // shrink the tail; the bound E below is the one of 4 terms)
  if (K > 0) K = 4;
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
  out->mode = mode;
  out->K = K;
  out->d0x = (float)d0x;
  out->d0y = (float)d0y;
  out->band = (float)(band * 1.0001);
  // the exact-difference form keeps W_i (FP32) where the expansion keeps c_n
  const float w0x = (float)__shfl_sync(0xffffffffu, wx, 0);
  const float w0y = (float)__shfl_sync(0xffffffffu, wy, 0);
  const float w1x = (float)__shfl_sync(0xffffffffu, wx, 1);
  const float w1y = (float)__shfl_sync(0xffffffffu, wy, 1);
  const float w2x = (float)__shfl_sync(0xffffffffu, wx, 2);
  const float w2y = (float)__shfl_sync(0xffffffffu, wy, 2);
#pragma unroll
  for (int n = 0; n < 4; n++) {
    out->cr[n] = mode == kModeTaylor ? cr[n] : 0.f;
    out->ci[n] = mode == kModeTaylor ? ci[n] : 0.f;
  }
  if (mode == kModeExact32) {
    out->cr[0] = w0x;
    out->ci[0] = w0y;
    out->cr[1] = w1x;
    out->ci[1] = w1y;
    out->cr[2] = w2x;
    out->ci[2] = w2y;
  }
  out->nxc = (int)nxc;
  out->nyc = (int)nyc;
}

// whole warp: computes the entry of super-tile (sx, sy) into `ent`
__device__ __noinline__ void compute_supertile(const Ctx& c, int sxi, int syi, int lane, uint32_t* ent) {
  SuperTile v;
  supertile_values(c, sxi, syi, lane, &v);
  if (lane == 0) {
    __stcg(&ent[kSMode], (uint32_t)v.mode);
    __stcg(&ent[kSK], (uint32_t)v.K);
    __stcg(&ent[kSD0x], __float_as_uint(v.d0x));
    __stcg(&ent[kSD0y], __float_as_uint(v.d0y));
    __stcg(&ent[kSBand], __float_as_uint(v.band));
    if (v.mode == kModeTaylor) {
      for (int n = 0; n < 4; n++) {
        __stcg(&ent[kSC + 2 * n], __float_as_uint(v.cr[n]));
        __stcg(&ent[kSC + 2 * n + 1], __float_as_uint(v.ci[n]));
      }
    }
    if (v.mode == kModeExact32) {  // W_i in FP32
      for (int n = 0; n < 3; n++) {
        __stcg(&ent[kSC + 2 * n], __float_as_uint(v.cr[n]));
        __stcg(&ent[kSC + 2 * n + 1], __float_as_uint(v.ci[n]));
      }
    }
  }
  __threadfence();
  __syncwarp();
}

// find-or-compute the super-tile holding tile (tx, ty); whole warp
__device__ __noinline__ bool get_supertile(Shared& S, const Table& T, int64_t nx0, int64_t ny0,
                                           int lane, SuperTile* st) {
  const Ctx& c = S.c;
  const int sh = c.slog2;
  const int sxi = (int)(nx0 >> sh);
  const int syi = (int)(ny0 >> sh);
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
    const long long c0 = clock64();
    compute_supertile(c, sxi, syi, lane, ent);
    if (lane == 0) atomicExch(&ent[kSState], 2u);
    if (lane == 0 && S.profiling) atomicAdd(&S.prof[5], (unsigned long long)(clock64() - c0));
  } else {
    uint32_t ready = 0;
    if (lane == 0) {
      for (unsigned it = 0; it < (1u << 18); it++) {
        if (atomicAdd(&ent[kSState], 0u) == 2u) { ready = 1; break; }
        if ((it & 255) == 255 && overdue(S, 4)) break;
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
  for (int n = 0; n < 4; n++) {
    st->cr[n] = __uint_as_float(ldcg32(&ent[kSC + 2 * n]));
    st->ci[n] = __uint_as_float(ldcg32(&ent[kSC + 2 * n + 1]));
  }
  const int half = 1 << (sh - 1);
  st->nxc = (sxi << sh) + half;
  st->nyc = (syi << sh) + half;
  return true;
}

template <int K>
__device__ __forceinline__ float taylor_r2(const SuperTile& st, float ex, float bx, float dy) {
  const float ey = -dy;
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
  const float sy = (st.d0y + dy) - qi;
  return fmaf(sx, sx, sy * sy);
}

__device__ __forceinline__ float exact32_r2(const Ctx& c, const SuperTile& st, float dx, float bx,
                                            float dy) {
  float sx = bx, sy = st.d0y + dy;
#pragma unroll
  for (int i = 0; i < 3; i++) {
    const float mi = i == 0 ? (float)c.m1 : (i == 1 ? (float)c.m2 : (float)c.m3);
    const float wx = st.cr[i], wy = st.ci[i];
    const float vx = wx + dx, vy = wy + dy;
    const float px = vx * wx - vy * wy, py = vx * wy + vy * wx;   // P = V W
    const float inv = __frcp_rn(fmaf(px, px, py * py));
    const float qx = (dx * px + dy * py) * inv, qy = (dy * px - dx * py) * inv;  // delta/P
    sx = fmaf(mi, qx, sx);
    sy = fmaf(-mi, qy, sy);   // + m conj(delta/P)
  }
  return fmaf(sx, sx, sy * sy);
}

template <int K>
__device__ __forceinline__ float split_r2(const Ctx& c, const SuperTile& st, float dx, float bx,
                                          float dy) {
  if (K == 0) return exact32_r2(c, st, dx, bx, dy);
  return taylor_r2<(K > 0 ? K : 1)>(st, dx, bx, dy);
}

// single-instruction square root (relative error ~2^-22; weights only)
__device__ __forceinline__ float sqrt_fast(float x) {
  float y;
  asm("sqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
  return y;
}

__device__ __forceinline__ float ld_weight_f(const Ctx& c, float r2) {
  return fmaf(c.ldbf, sqrt_fast(fmaxf(0.f, fmaf(-r2, c.inv_rho2f, 1.f))), c.ldaf);
}

// Rays of this lane's column in block (bx, by), split-precision map with the
// FP64 guard band.  Returns the accepted mask of row `lane` (lane < BH) and
// adds the weights of this lane's accepted rays to *wsum.
// The FP32 pass is branch-free: eight independent rows per iteration, hits
// and guard-band rays collected as per-lane column masks; the rare band rays
// are decided in FP64 afterwards, and 32 ballots turn the column masks into
// row masks.
template <int BH, int K>
__device__ __forceinline__ uint32_t classify_block(const Ctx& c, const SuperTile st, int bx,
                                                   int by, int lane, float* wsum, unsigned* ev,
                                                   unsigned* e64) {
  // per-block constants kept in registers across the row loop
  const float hf = c.hf;
  const int64_t n = c.n;
  const int64_t nx = (int64_t)bx * 32 + lane;
  const bool col_ok = nx >= 1 && nx <= n - 1;
  const float dx = hf * (float)(int)(nx - st.nxc);
  const float bxo = st.d0x + dx;
  const float lo = c.rho2f - st.band, hi = c.rho2f + st.band;
  const float inv_rho2 = c.inv_rho2f, lda = c.ldaf, ldb = c.ldbf;
  const int64_t ny0 = (int64_t)by * BH;
  const int rows_ok = col_ok ? (int)max((int64_t)0, min((int64_t)BH, n - ny0)) : 0;  // rows <= N-1
  const int dy0 = (int)(ny0 - st.nyc);
  uint32_t hitm = 0, bandm = 0;
  float ws = 0.f;
#pragma unroll 1
  for (int r0 = 0; r0 < BH; r0 += 8) {
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int r = r0 + q;
      const float dy = hf * (float)(dy0 + r);
      const float r2 = split_r2<K>(c, st, dx, bxo, dy);
      const bool ok = r < rows_ok;
      const bool hit = ok && r2 < lo;
      const bool band = ok && r2 >= lo && r2 <= hi;
      const float w = fmaf(ldb, sqrt_fast(fmaxf(0.f, fmaf(-r2, inv_rho2, 1.f))), lda);
      ws += hit ? w : 0.f;
      hitm |= (uint32_t)hit << r;
      bandm |= (uint32_t)band << r;
    }
  }
  unsigned n64 = 0;
  while (bandm) {  // rays within the guard band of the limb: FP64
    const int r = __ffs(bandm) - 1;
    bandm &= bandm - 1u;
    const double rsq = irs_exact(c, grid_x(c, nx), grid_y(c, ny0 + r));
    n64++;
    if (rsq < c.rho2) {
      hitm |= 1u << r;
      ws += (float)ray_weight(c, rsq);
    }
  }
  uint32_t hl = 0;
#pragma unroll
  for (int r = 0; r < BH; r++) {
    const uint32_t b = __ballot_sync(0xffffffffu, (hitm >> r) & 1u);
    if (lane == r) hl = b;
  }
  *wsum += ws;
  *ev += rows_ok;
  *e64 += n64;
  return hl;
}

template <int BH>
__device__ __forceinline__ uint32_t classify_block_fp64(const Ctx& c, int bx, int by, int lane,
                                                        float* wsum, unsigned* ev,
                                                        unsigned* e64) {
  const int64_t nx = (int64_t)bx * 32 + lane;
  const bool col_ok = nx >= 1 && nx <= c.n - 1;
  const double x = grid_x(c, nx);
  const int64_t ny0 = (int64_t)by * BH;
  uint32_t hl = 0;
  float ws = 0.f;
  unsigned nev = 0;
#pragma unroll 1
  for (int r = 0; r < BH; r++) {
    const int64_t ny = ny0 + r;
    bool hit = false;
    if (col_ok && ny <= c.n - 1) {
      const double rsq = irs_exact(c, x, grid_y(c, ny));
      nev++;
      hit = rsq < c.rho2;
      if (hit) ws += (float)ray_weight(c, rsq);
    }
    const uint32_t b = __ballot_sync(0xffffffffu, hit);
    if (lane == r) hl = b;
  }
  *wsum += ws;
  *ev += nev;
  *e64 += nev;
  return hl;
}

// weight of one accepted ray evaluated again (blocks filled over several
// passes: their rays are no longer in registers)
__device__ __noinline__ float weight_again(const Ctx& c, const SuperTile& st, bool split,
                                           int64_t nx, int64_t ny) {
  if (!split || st.mode == kModeFp64) {
    return (float)ray_weight(c, irs_exact(c, grid_x(c, nx), grid_y(c, ny)));
  }
  const float dx = c.hf * (float)(int)(nx - st.nxc);
  const float dy = c.hf * (float)(int)(ny - st.nyc);
  const float bx = st.d0x + dx;
  float r2;
  if (st.mode == kModeTaylor) {
    r2 = taylor_r2<4>(st, dx, bx, dy);
  } else {
    r2 = exact32_r2(c, st, dx, bx, dy);
  }
  return ld_weight_f(c, r2);
}

// Weights of the rays of f (lane r: row r's mask) in block (bx, by) of
// super-tile st, one lane per column: the split map once per filled ray,
// the same formula and summation order as weight_again over the rows.
template <int K>
__device__ __forceinline__ float partial_weights(const Ctx& c, const SuperTile& st, int bx,
                                                 int by, int lane, uint32_t f, unsigned* nre) {
  const float hf = c.hf;
  const int64_t nx = (int64_t)bx * 32 + lane;
  const float dx = hf * (float)(int)(nx - st.nxc);
  const float bxo = st.d0x + dx;
  const int dy0 = (int)((int64_t)by * 32 - st.nyc);
  float acc = 0.f;
  unsigned re = 0;
#pragma unroll 1
  for (int r = 0; r < 32; r++) {
    const uint32_t nwr = __shfl_sync(0xffffffffu, f, r);
    if (nwr == 0u) continue;   // the same in every lane
    const bool on = (nwr >> lane) & 1u;
    const float dy = hf * (float)(dy0 + r);
    const float w = ld_weight_f(c, split_r2<K>(c, st, dx, bxo, dy));
    acc += on ? w : 0.f;
    re += on ? 1u : 0u;
  }
  *nre = re;
  return acc;
}

// weights of the rays of f in a 32 x 32 block (whole warp): inline for the
// split map, ray by ray in FP64 otherwise (as weight_again)
__device__ __forceinline__ float block_weights(const Ctx& c, const SuperTile& st, bool split,
                                               int bx, int by, int lane, uint32_t f,
                                               unsigned* nre) {
  if (split && st.mode == kModeTaylor)
    return partial_weights<4>(c, st, bx, by, lane, f, nre);
  if (split && st.mode == kModeExact32) return partial_weights<0>(c, st, bx, by, lane, f, nre);
  float acc = 0.f;
  unsigned re = 0;
  const int64_t nx = (int64_t)bx * 32 + lane;
#pragma unroll 1
  for (int r = 0; r < 32; r++) {
    const uint32_t nwr = __shfl_sync(0xffffffffu, f, r);
    if ((nwr >> lane) & 1u) {
      acc += weight_again(c, st, split, nx, (int64_t)by * 32 + r);
      re++;
    }
  }
  *nre = re;
  return acc;
}

// Whole warp: true when hp (lane r: row r's mask) is 4-connected by a simple
// test: one run per row, its non-empty rows consecutive, each row's run
// overlapping the next row's.  A fill entering such a set anywhere fills
// all of it.
__device__ __forceinline__ bool simple_region(uint32_t hp, int lane) {
  const bool one_run = (hp & (hp + (hp & (0u - hp)))) == 0u;
  const uint32_t nxt = __shfl_down_sync(0xffffffffu, hp, 1);
  const bool link = lane == 31 || hp == 0u || nxt == 0u || (hp & nxt) != 0u;
  const uint32_t nz = __ballot_sync(0xffffffffu, hp != 0u);
  const bool rows = (nz & (nz + (nz & (0u - nz)))) == 0u;
  return __all_sync(0xffffffffu, one_run && link) && rows;
}

// per-warp cache of the last super-tile used
struct WarpST {
  uint64_t key;
  bool valid;
  SuperTile st;
};

template <int BH>
__device__ __forceinline__ bool warp_supertile(Shared& S, const Table& T, int bx, int by,
                                               int lane, WarpST& ws) {
  const int sh = S.c.slog2;
  const int64_t nx0 = (int64_t)bx * 32, ny0 = (int64_t)by * BH;
  const uint64_t key = tile_key((int)(nx0 >> sh), (int)(ny0 >> sh));
  if (ws.valid && ws.key == key) return true;
  ws.valid = get_supertile(S, T, nx0, ny0, lane, &ws.st);
  ws.key = key;
  return ws.valid;
}

// processes one queued block (whole warp)
template <int BH>
__device__ void process_block(Shared& S, const Table& T, int slot, int lane, WarpST& wst) {
  using L = Lo<BH>;
  const Ctx& c = S.c;
  const uint64_t key = ldcg64(&T.keys[slot]);
  const int bx = (int)(uint32_t)(key & 0xffffffffu);
  const int by = (int)(uint32_t)(key >> 32);
  uint32_t* rec = T.recs + (size_t)slot * T.rec_words;
  unsigned long long local_count = 0, local_eval = 0, local_fp64 = 0;
  long long local_fx = 0;  // weight sum, units of 2^-16
  uint32_t edge = 0;
  // dequeued: queued set, busy clear -> clear queued, set busy
  uint32_t st0 = 0;
  if (lane == 0) {
    st0 = atomicXor(&rec[L::kState], kQ | kB);
    __threadfence_block();
  }
  st0 = __shfl_sync(0xffffffffu, st0, 0);
  bool hdone = (st0 & kD) != 0;
  uint32_t h_row = 0, f_cur = 0;  // lane r < BH: row r
  if (lane < BH) {
    f_cur = ldcg32(&rec[L::kF + lane]);
    if (hdone) h_row = ldcg32(&rec[L::kH + lane]);
  }
  for (int pass = 0;; pass++) {
    if (lane == 0) beat(S.hb, 3, S.point, (unsigned)pass);
    unsigned late = 0;
    if (lane == 0) late = overdue(S, 5);
    if (__shfl_sync(0xffffffffu, late, 0)) break;
    if (pass > 4096) {  // a block re-queued without end: give up on the point
      if (lane == 0) {
        set_abort(S, kStTimeout);
        atomicAdd(&S.dbg_again, 1u);
      }
      break;
    }
    __threadfence_block();
    uint32_t e_row = lane < BH ? atomicExch(&rec[lane], 0u) : 0u;
    uint32_t eside = lane < 4 ? atomicExch(&rec[BH + lane], 0u) : 0u;
    const uint32_t ebot = __shfl_sync(0xffffffffu, eside, 0);
    const uint32_t etop = __shfl_sync(0xffffffffu, eside, 1);
    const uint32_t eleft = __shfl_sync(0xffffffffu, eside, 2);
    const uint32_t eright = __shfl_sync(0xffffffffu, eside, 3);
    if (lane < BH) {
      e_row |= (lane == 0 ? ebot : 0u) | (lane == BH - 1 ? etop : 0u) | ((eleft >> lane) & 1u) |
               (((eright >> lane) & 1u) << 31);
    }
    bool fresh = false;
    float wall = 0.f;
    if (!hdone) {
      unsigned nr = 0, n64 = 0;
      if (lane == 0) beat(S.hb, 7, S.point, 0);
      const long long e0 = clock64();
      const bool have = c.split && warp_supertile<BH>(S, T, bx, by, lane, wst);
      if (have && wst.st.mode != kModeFp64) {
        const SuperTile stc = wst.st;  // by value: the coefficients stay in registers
        const int K = stc.mode == kModeTaylor ? stc.K : 0;
        if (K == 0) h_row = classify_block<BH, 0>(c, stc, bx, by, lane, &wall, &nr, &n64);
        else h_row = classify_block<BH, 4>(c, stc, bx, by, lane, &wall, &nr, &n64);
      } else {
        h_row = classify_block_fp64<BH>(c, bx, by, lane, &wall, &nr, &n64);
      }
      if (S.profiling && lane == 0) atomicAdd(&S.prof[6], (unsigned long long)(clock64() - e0));
      local_eval += warp_sum_u(nr);
      local_fp64 += warp_sum_u(n64);
      if (lane < BH) __stcg(&rec[L::kH + lane], h_row);
      hdone = true;
      fresh = true;
    }
    const uint32_t hp = h_row & ~f_cur;  // accepted, not yet filled
    uint32_t f = e_row & hp;
    if (__ballot_sync(0xffffffffu, f != 0u)) {
      // closure inside the block: rows exchange with the rows above/below
      // every iteration that changes anything fills at least one more run,
      // so 32 rows x 16 runs bounds it
      if (lane == 0) beat(S.hb, 4, S.point, 0);
      const bool whole = simple_region(hp, lane);   // filled whole by any entry
      if (whole) f = hp;
      for (int it = 0; it < 1024 && !whole; it++) {
        if ((it & 63) == 63) {
          unsigned late = 0;
          if (lane == 0) late = overdue(S, 6);
          if (__shfl_sync(0xffffffffu, late, 0)) break;
        }
        uint32_t below = __shfl_up_sync(0xffffffffu, f, 1);
        uint32_t above = __shfl_down_sync(0xffffffffu, f, 1);
        if (lane == 0) below = 0u;
        if (lane >= BH - 1) above = 0u;
        const uint32_t nf = lane < BH ? run_fill(f | ((below | above) & hp), hp) : 0u;
        const unsigned changed = __ballot_sync(0xffffffffu, nf != f);
        f = nf;
        if (!changed) break;
      }
      const uint32_t f_new = f_cur | f;
      if (lane < BH) __stcg(&rec[L::kF + lane], f_new);
      const uint32_t fl = __ballot_sync(0xffffffffu, lane < BH && (f_new & 1u));
      const uint32_t fr = __ballot_sync(0xffffffffu, lane < BH && (f_new >> 31));
      if (lane == 0) {
        __stcg(&rec[L::kFl], fl);
        __stcg(&rec[L::kFr], fr);
      }
      // weights of the newly filled rays: the whole evaluated block when this
      // pass filled all of its accepted rays, otherwise ray by ray
      float acc;
      const bool all = fresh && __ballot_sync(0xffffffffu, lane < BH && f != h_row) == 0u;
      if (all) {
        acc = wall;
      } else {
        acc = 0.f;
        unsigned re = 0;
        const int64_t nx = (int64_t)bx * 32 + lane;
        if (c.split) warp_supertile<BH>(S, T, bx, by, lane, wst);
        if (BH == 32) {
          acc = block_weights(c, wst.st, c.split && wst.valid, bx, by, lane, f, &re);
        } else {
#pragma unroll 1
          for (int r = 0; r < BH; r++) {
            const uint32_t nwr = __shfl_sync(0xffffffffu, f, r);
            if ((nwr >> lane) & 1u) {
              acc += weight_again(c, wst.st, c.split && wst.valid, nx, (int64_t)by * BH + r);
              re++;
            }
          }
        }
        local_eval += warp_sum_u(re);
      }
      f_cur = f_new;
      local_count += warp_sum_u(lane < BH ? __popc(f) : 0u);
      // a block's sum is below 1024 * 1.5: 2^-16 resolution fits an int32
      local_fx += (long long)__float2int_rn(warp_sum_f(acc) * 65536.f);
      // plane edge: columns 1 and N-1 are where the reference's row scan
      // stops differently (lcirs.cc:413-440)
      {
        const int64_t c0 = (int64_t)bx * 32;
        uint32_t colmask = 0;
        if (1 >= c0 && 1 < c0 + 32) colmask |= 1u << (1 - c0);
        if (c.n - 1 >= c0 && c.n - 1 < c0 + 32) colmask |= 1u << (c.n - 1 - c0);
        const uint32_t any = __reduce_or_sync(0xffffffffu, lane < BH ? f : 0u);
        if (any & colmask) edge = 1;
      }
      // neighbours
      const long long p0 = clock64();
      if (lane == 0) beat(S.hb, 5, S.point, 0);
      const uint32_t top = __shfl_sync(0xffffffffu, f, BH - 1);
      const uint32_t bot = __shfl_sync(0xffffffffu, f, 0);
      const uint32_t lcol = __ballot_sync(0xffffffffu, lane < BH && (f & 1u));
      const uint32_t rcol = __ballot_sync(0xffffffffu, lane < BH && (f >> 31));
      if (lane == 0) {
        push<BH>(S, T, bx, by + 1, kPushBot, 0, top);
      } else if (lane == 1) {
        push<BH>(S, T, bx, by - 1, kPushTop, 0, bot);
      } else if (lane == 2) {
        push<BH>(S, T, bx - 1, by, kPushRight, 0, lcol);  // enters the left block at column 31
      } else if (lane == 3) {
        push<BH>(S, T, bx + 1, by, kPushLeft, 0, rcol);   // enters the right block at column 0
      }
      __syncwarp();
      if (S.profiling && lane == 0) atomicAdd(&S.prof[7], (unsigned long long)(clock64() - p0));
    }
    // release: H and F (stored by every lane) must be visible before the
    // state says so
    if (lane == 0) beat(S.hb, 6, S.point, 0);
    __threadfence_block();
    __syncwarp();
    uint32_t again = 0;
    if (lane == 0) {
      const uint32_t old = atomicCAS(&rec[L::kState], kB | (fresh ? 0u : kD), kD);
      if (old != (kB | (fresh ? 0u : kD))) {
        // queued again while busy (and, after a fresh evaluation, D not yet
        // set): keep busy, clear queued, mark H done
        atomicAnd(&rec[L::kState], ~kQ);
        atomicOr(&rec[L::kState], kD);
        again = 1;
      }
    }
    again = __shfl_sync(0xffffffffu, again, 0);
    if (!again) {
      if (lane == 0) atomicMax(&S.max_pass, (unsigned)pass);
      break;
    }
  }
  if (lane == 0) {
    if (local_count) atomicAdd(&S.count, local_count);
    if (local_fx) atomicAdd(&S.wsum, (unsigned long long)(local_fx << 16));
    atomicAdd(&S.rays_eval, local_eval);
    atomicAdd(&S.rays_fp64, local_fp64);
    if (edge) atomicOr(&S.status, kStEdge);
  }
}

}  // namespace

// MINB: resident CTAs per SM the register budget is cut for (2, 3 or 4)
template <int BH, int MINB>
__global__ void __launch_bounds__(256, MINB)
fill_kernel(const PointIn* points, int npoints, const DevLens* lenses, const int32_t* seeds,
            PointOut* out, FillScratch sc, int split_mode, const int32_t* list,
            const unsigned* list_count) {
  __shared__ Shared S;
  // with a point list (overflow retry) the work is list[0 .. *list_count)
  const int nwork = list ? (int)*list_count : npoints;
  const int lane = threadIdx.x & 31;
  const int warp = threadIdx.x >> 5;
  // table of this CTA: the first big_ctas CTAs own the larger tables
  const bool big_cta = (int)blockIdx.x < sc.big_ctas;
  const size_t cap = (size_t)1 << (big_cta ? sc.big_log2 : sc.cap_log2);
  const size_t tbase = big_cta ? (size_t)blockIdx.x * cap
                               : ((size_t)sc.big_ctas << sc.big_log2) +
                                     (size_t)(blockIdx.x - sc.big_ctas) * cap;
  const int nbig = (list && sc.nbig && big_cta) ? (int)*sc.nbig : 0;
  const int nbig_all = (list && sc.nbig && sc.big_ctas > 0) ? (int)*sc.nbig : 0;
  bool big_left = nbig > 0;
  Table T;
  T.keys = sc.keys + tbase;
  T.recs = sc.recs + tbase * sc.rec_words;
  T.ring = sc.ring + tbase;
  T.used = sc.used + tbase;
  T.mask = (uint32_t)(cap - 1);
  T.rec_words = sc.rec_words;
  const size_t scap = (size_t)1 << kSuperLog2;
  T.skeys = sc.skeys + (size_t)blockIdx.x * scap;
  T.sents = sc.sents + (size_t)blockIdx.x * scap * kSEntryWords;
  T.sused = sc.sused + (size_t)blockIdx.x * scap;
  T.smask = (uint32_t)(scap - 1);
  WarpST wst;
  wst.valid = false;
  wst.key = 0;

  for (;;) {
    if (threadIdx.x == 0) {
      {
        // large CTAs drain the list's head (largest points) first; all CTAs
        // then share the rest, largest first
        int w = -1;
        if (big_left) {
          w = (int)atomicAdd(&sc.next_point[1], 1u);
          if (w >= nbig) {
            big_left = false;
            w = -1;
          }
        }
        if (w < 0) w = nbig_all + (int)atomicAdd(&sc.next_point[0], 1u);
        S.point = w < nwork ? (list ? list[w] : w) : npoints;
      }
      S.head = S.tail = S.pending = S.used = S.sused = 0;
      S.abort_ = 0;
      S.count = S.wsum = S.rays_eval = S.rays_fp64 = 0;
      S.status = 0;
      S.t0 = globaltimer();
      S.dbg_again = S.dbg_deq = S.max_pass = S.dbg_where = 0;
      S.profiling = sc.prof != nullptr;
      S.hb = sc.heartbeat;
      for (int q = 0; q < 8; q++) S.prof[q] = 0;
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
        c.tymax = (int)((c.n - 1) / BH);
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
    wst.valid = false;
    const bool skip = (S.status & kStBadInput) != 0;
    // seeds (lcirs.cc:171-174; seed rows must satisfy 0 < ny < N, 386-391)
    if (!skip && warp == 0) {
      // at most kMaxSeeds pixels per point exist, whatever the count says
      const unsigned ns = min(out[p].nseeds, (unsigned)kMaxSeeds);
      for (unsigned k = lane; k < ns; k += 32) {
        const int32_t sx = seeds[((size_t)p * kMaxSeeds + k) * 2];
        const int32_t sy = seeds[((size_t)p * kMaxSeeds + k) * 2 + 1];
        if (sy <= 0 || (int64_t)sy >= S.c.n) continue;
        if (sx < 1 || (int64_t)sx > S.c.n - 1) {
          atomicOr(&S.status, kStEdge);
          continue;
        }
        push<BH>(S, T, sx >> 5, sy / BH, kPushSeed, sy % BH, 1u << (sx & 31));
      }
    }
    __syncthreads();
    // work loop
    const long long wl0 = clock64();
    if (!skip) {
      unsigned spins = 0;
      for (;;) {
        int slot = -1;
        if (lane == 0) beat(S.hb, 1, p, spins);
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
          if ((spins & 255) == 255) {
            unsigned late = 0;
            if (lane == 0) late = overdue(S, 7);
            if (__shfl_sync(0xffffffffu, late, 0)) break;
          }
          if (S.profiling && lane == 0) atomicAdd(&S.prof[2], 1ull);
          __nanosleep(100);
          continue;
        }
        spins = 0;
        if (lane == 0) overdue(S, 8);
        const long long c0 = clock64();
        if (lane == 0) beat(S.hb, 2, p, (unsigned)slot);
        if (!*(volatile unsigned*)&S.abort_) process_block<BH>(S, T, slot, lane, wst);
        if (S.profiling && lane == 0) {
          atomicAdd(&S.prof[0], 1ull);
          atomicAdd(&S.prof[1], (unsigned long long)(clock64() - c0));
        }
        if (lane == 0) atomicSub(&S.pending, 1u);
      }
    }
    if (S.profiling && lane == 0) atomicAdd(&S.prof[3], (unsigned long long)(clock64() - wl0));
    if (lane == 0) beat(S.hb, 8, p, 0);
    __syncthreads();
    if (S.profiling && threadIdx.x == 0) {
      S.prof[4] = S.sused;
      for (int q = 0; q < 8; q++) atomicAdd(&sc.prof[q], S.prof[q]);
    }
    if (threadIdx.x == 0) {
      PointOut o = out[p];
      o.count = S.count;
      o.wsum_fx = (int64_t)S.wsum;
      o.status |= S.status;
      o.tiles = S.used;
      o.diag = S.max_pass | (S.dbg_again ? 0x10000u : 0u) | (S.dbg_deq ? 0x20000u : 0u) |
               (S.dbg_where << 24);
      o.rays_eval = S.rays_eval;
      o.rays_fp64 = S.rays_fp64;
      out[p] = o;
    }
    // clear the slots this point used (tables start every point empty)
    const unsigned nused = S.used < cap ? S.used : (unsigned)cap;
    for (unsigned u = threadIdx.x; u < nused; u += blockDim.x) {
      const uint32_t slot = __ldcg(&T.used[u]);
      uint32_t* rec = T.recs + (size_t)slot * T.rec_words;
      if (sc.dump && !S.abort_) {  // an aborted point is retried and dumped then
        uint32_t any = 0;
        for (int r = 0; r < BH; r++) any |= ldcg32(&rec[Lo<BH>::kF + r]);
        if (any) {
          const uint64_t key = ldcg64(&T.keys[slot]);
          const int bxk = (int)(uint32_t)(key & 0xffffffffu), byk = (int)(uint32_t)(key >> 32);
          for (int t8 = 0; t8 < BH / 8; t8++) {  // one record per 32x8 tile
            uint32_t fm[8], a8 = 0;
            for (int r = 0; r < 8; r++) a8 |= (fm[r] = ldcg32(&rec[Lo<BH>::kF + 8 * t8 + r]));
            if (!a8) continue;
            const unsigned d = atomicAdd(sc.dump_count, 1u);
            if (d < sc.dump_cap) {
              uint32_t* o = sc.dump + (size_t)d * kDumpWords;
              o[0] = (uint32_t)p;
              o[1] = (uint32_t)bxk;
              o[2] = (uint32_t)(byk * (BH / 8) + t8);
              for (int r = 0; r < 8; r++) o[3 + r] = fm[r];
            }
          }
        }
      }
      __stcg((unsigned long long*)&T.keys[slot], (unsigned long long)kEmptyKey);
      uint4* r4 = (uint4*)rec;
      for (int q = 0; q < T.rec_words / 4; q++) __stcg(&r4[q], make_uint4(0u, 0u, 0u, 0u));
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

// ===========================================================================
// Warp fill.  One warp fills one point alone, points taken from the
// size-ordered list (largest first).  The point's blocks of 32 x 32 rays sit
// in the warp's own open-addressing table in HBM; the work stack (spilling
// into HBM past kWStack entries), the last super-tile expansions and the
// seed pixels in shared memory; a slot's header says whether it is queued.  Each visit of a block
// does what process_block does (classification, closure, weights, edge
// test), and the warp is the only writer of its table: no atomics on the
// table and no waits on other warps.  A block's four neighbours are looked
// up by four groups of 8 lanes, each probing 8 slots with one load.
// ===========================================================================
namespace {

constexpr int kWThreads = 128;                   // 4 warps per CTA
constexpr int kWWarps = kWThreads / 32;
constexpr int kWOcc = 8;                         // resident CTAs per SM (32 warps)
constexpr int kWStack = 512;                     // work-stack entries in shared memory
constexpr int kWStCache = 8;                     // super-tile expansions kept per warp
constexpr unsigned kFull = 0xffffffffu;
// header words
constexpr int kHEb = 0, kHEt = 1, kHEl = 2, kHEr = 3;   // entry masks: bottom/top row, left/right column
constexpr int kHFb = 4, kHFt = 5, kHFl = 6, kHFr = 7;   // filled border: row 0, row 31, column 0, column 31
constexpr int kHState = 8, kHBx = 9, kHBy = 10;
// state: H and F valid; holds a seed pixel; on the work stack
constexpr uint32_t kWCls = 1u, kWSeed = 2u, kWQueued = 4u;

struct WarpSh {
  Ctx c;
  SuperTile st[kWStCache];
  uint64_t sttag[kWStCache];
  uint32_t stack[kWStack];
  int32_t seedx[kMaxSeeds], seedy[kMaxSeeds];
  unsigned top, used, nseed;
};

struct WTable {
  uint64_t* keys;
  uint32_t* hdr;
  uint32_t* body;
  uint32_t* used;
  uint32_t* spill;
  uint32_t mask;      // slots - 1
  unsigned usable;    // table load limit (blocks per point): 3/4 of the slots
};

struct WAcc {
  unsigned long long count, eval, fp64;
  long long fx;       // weight sum, units of 2^-16 (lane 0's value is used)
  unsigned edge;
  unsigned prof[8];   // optional counters (WScratch::prof), lane 0's values
};

// one lane: put `slot` on the work stack (its header's state says queued
// from now until its visit writes the header back)
__device__ __forceinline__ void w_push_stack(WarpSh& W, const WTable& T, uint32_t slot) {
  const unsigned pos = atomicAdd(&W.top, 1u);
  if (pos < (unsigned)kWStack) W.stack[pos] = slot;
  else __stcg(&T.spill[pos], slot);   // pos < number of queued slots <= slots
}

// Whole warp.  The 8 lanes of group g = lane / 8 look up block (bx, by) when
// `act` (uniform in the group) and insert it when absent; every lane of the
// group returns the slot (-1: inactive, or no free slot) and *ins = inserted
// now.  Groups that pick the same free slot in one round: the lower group
// takes it, the other reads its window again.
__device__ __noinline__ int w_find4(const WTable& T, bool act, int bx, int by, int lane,
                                    bool* ins, unsigned* rounds) {
  const int g = lane >> 3, j = lane & 7;
  const uint64_t key = tile_key(bx, by);
  const uint32_t h0 = hash_key(key) & T.mask;
  int slot = -1;
  bool done = !act, inserted = false;
  uint32_t r = 0;
  const int iters = 4 * (int)(T.mask / 8u + 2u);
  for (int it = 0; it < iters; it++) {
    const bool live = !done;
    if (!__any_sync(kFull, live)) break;
    ++*rounds;
    const uint32_t base = h0 + r * 8u;
    uint64_t k = 0;
    if (live) k = ldcg64(&T.keys[(base + (uint32_t)j) & T.mask]);
    const uint32_t mm = __ballot_sync(kFull, live && k == key);
    const uint32_t me = __ballot_sync(kFull, live && k == kEmptyKey);
    const uint32_t gm = (mm >> (8 * g)) & 0xffu, ge = (me >> (8 * g)) & 0xffu;
    uint32_t want = kFull;
    if (live && gm == 0u && ge != 0u) want = (base + (uint32_t)(__ffs(ge) - 1)) & T.mask;
    const uint32_t w0 = __shfl_sync(kFull, want, 0);
    const uint32_t w1 = __shfl_sync(kFull, want, 8);
    const uint32_t w2 = __shfl_sync(kFull, want, 16);
    const bool lose = want != kFull && ((g > 0 && want == w0) || (g > 1 && want == w1) ||
                                        (g > 2 && want == w2));
    bool take = false;
    if (live) {
      if (gm != 0u) {
        slot = (int)((base + (uint32_t)(__ffs(gm) - 1)) & T.mask);
        done = true;
      } else if (want != kFull) {
        if (!lose) {
          slot = (int)want;
          inserted = true;
          take = true;
          done = true;
        }
      } else {
        r++;
        if (r > T.mask / 8u) done = true;   // every window holds other keys: no slot
      }
    }
    if (take && j == 0) __stcg((unsigned long long*)&T.keys[slot], (unsigned long long)key);
    __syncwarp();
  }
  *ins = inserted;
  return slot;
}

// group of 8 lanes: header of a slot inserted now (entries and border zero),
// and its place in the used list
__device__ __forceinline__ void w_init_slot(WarpSh& W, const WTable& T, int slot, int bx, int by,
                                            int lane) {
  const int j = lane & 7;
  uint32_t* h = T.hdr + (size_t)slot * kWHdrWords;
  for (int q = j; q < kWHdrWords; q += 8)
    __stcg(&h[q], q == kHBx ? (uint32_t)bx : (q == kHBy ? (uint32_t)by : 0u));
  if (j == 0) {
    const unsigned u = atomicAdd(&W.used, 1u);
    if (u <= T.mask) __stcg(&T.used[u], (uint32_t)slot);
  }
}

// whole warp: cache index of the expansion of the super-tile holding block
// (bx, by), computed on a miss
__device__ __noinline__ int w_supertile(WarpSh& W, int bx, int by, int lane, unsigned* misses) {
  const int sh = W.c.slog2 - 5;
  const int sxi = bx >> sh, syi = by >> sh;
  const uint64_t key = tile_key(sxi, syi);
  const int idx = (int)(hash_key(key) & (uint32_t)(kWStCache - 1));
  if (W.sttag[idx] != key) {
    ++*misses;
    SuperTile v;
    supertile_values(W.c, sxi, syi, lane, &v);
    __syncwarp();
    if (lane == 0) {
      W.st[idx] = v;
      W.sttag[idx] = key;
    }
    __syncwarp();
  }
  return idx;
}

// A team of kTeamWarps warps filling one point together (tfill_kernel):
// each warp owns the blocks of its share of the super-tiles; entries into a
// block of another share go to that warp's inbox as messages (block, side,
// bits), read at the start of the next round.
constexpr int kTeamWarps = 8;
struct WTeam {
  uint4* inbox;            // this team's inboxes: [2 buffers][kTeamWarps][cap]
  unsigned* inbox_n;       // shared counters [2][kTeamWarps]
  unsigned* abort_;        // shared: status bits that end the point
  unsigned cap;            // messages per inbox
  int me;                  // this warp's share
  int post;                // buffer taking this round's messages
  int sh;                  // log2 of the super-tile edge in blocks
};

__device__ __forceinline__ int team_owner(int bx, int by, int sh) {
  return (int)(hash_key(tile_key(bx >> sh, by >> sh)) & (uint32_t)(kTeamWarps - 1));
}

// entry and filled-border words of a block side (side 0: bottom row, from
// the block below; 1: top row; 2: column 31; 3: column 0)
__device__ __forceinline__ void side_words(int side, int* ew, int* fw) {
  *ew = side == 0 ? kHEb : (side == 1 ? kHEt : (side == 2 ? kHEr : kHEl));
  *fw = side == 0 ? kHFb : (side == 1 ? kHFt : (side == 2 ? kHFr : kHFl));
}

// one lane: entry bits into slot s (inserted now: header zero), less what it
// has filled; queued if new bits arrived and it is not queued yet
__device__ __forceinline__ void w_enter(WarpSh& W, const WTable& T, int s, bool ins, int side,
                                        uint32_t bits) {
  int ew, fw;
  side_words(side, &ew, &fw);
  uint32_t* nh = T.hdr + (size_t)s * kWHdrWords;
  const uint32_t filled = ins ? 0u : ldcg32(&nh[fw]);
  const uint32_t old = ins ? 0u : ldcg32(&nh[ew]);
  const uint32_t nst = ins ? 0u : ldcg32(&nh[kHState]);
  const uint32_t nb = bits & ~filled;
  if (nb) {
    __stcg(&nh[ew], old | nb);
    if (!(nst & kWQueued)) {
      __stcg(&nh[kHState], nst | kWQueued);
      w_push_stack(W, T, (uint32_t)s);
    }
  }
}

// whole warp: one visit of the block in `slot`; tm: the warp's team (null
// for the warp fill, where every block is the warp's own)
__device__ __noinline__ void w_block(WarpSh& W, const WTable& T, uint32_t slot, int lane,
                                     WAcc& A, const WTeam* tm) {
  const Ctx& c = W.c;
  uint32_t* hdr = T.hdr + (size_t)slot * kWHdrWords;
  uint32_t* body = T.body + (size_t)slot * 64;
  const uint32_t hw = lane < kWHdrWords ? ldcg32(&hdr[lane]) : 0u;
  const uint32_t hb = ldcg32(&body[lane]);
  const uint32_t fb = ldcg32(&body[32 + lane]);
  const uint32_t eb = __shfl_sync(kFull, hw, kHEb), et = __shfl_sync(kFull, hw, kHEt);
  const uint32_t el = __shfl_sync(kFull, hw, kHEl), er = __shfl_sync(kFull, hw, kHEr);
  const uint32_t state = __shfl_sync(kFull, hw, kHState);
  const int bx = (int)__shfl_sync(kFull, hw, kHBx), by = (int)__shfl_sync(kFull, hw, kHBy);
  const bool cls = (state & kWCls) != 0u;
  uint32_t h_row = cls ? hb : 0u;
  const uint32_t f_cur = cls ? fb : 0u;
  uint32_t e_row = (lane == 0 ? eb : 0u) | (lane == 31 ? et : 0u) | ((el >> lane) & 1u) |
                   (((er >> lane) & 1u) << 31);
  // seed pixels of this block (lcirs.cc:171-174), applied on every visit
  if (state & kWSeed) {
    for (unsigned k = 0; k < W.nseed; k++) {
      const int32_t px = W.seedx[k], py = W.seedy[k];
      if ((px >> 5) == bx && (py >> 5) == by && (py & 31) == lane) e_row |= 1u << (px & 31);
    }
  }
  bool fresh = false;
  float wall = 0.f;
  int sti = -1;
  if (!cls) {
    unsigned nr = 0, n64 = 0;
    if (c.split) sti = w_supertile(W, bx, by, lane, &A.prof[2]);
    if (sti >= 0 && W.st[sti].mode != kModeFp64) {
      const SuperTile stc = W.st[sti];   // by value: the coefficients stay in registers
      const int K = stc.mode == kModeTaylor ? stc.K : 0;
      if (K == 0) h_row = classify_block<32, 0>(c, stc, bx, by, lane, &wall, &nr, &n64);
      else h_row = classify_block<32, 4>(c, stc, bx, by, lane, &wall, &nr, &n64);
    } else {
      h_row = classify_block_fp64<32>(c, bx, by, lane, &wall, &nr, &n64);
    }
    A.eval += warp_sum_u(nr);
    A.fp64 += warp_sum_u(n64);
    fresh = true;
    A.prof[1]++;
  }
  A.prof[0]++;
  const uint32_t hp = h_row & ~f_cur;   // accepted, not yet filled
  uint32_t f = e_row & hp;
  uint32_t f_new = f_cur;
  const bool any = __ballot_sync(kFull, f != 0u) != 0u;
  uint32_t top = 0, bot = 0, lcol = 0, rcol = 0;
  if (any) {
    // closure inside the block (as process_block); a simply connected hp is
    // filled whole by any entry
    const bool whole = simple_region(hp, lane);
    if (whole) {
      f = hp;
      A.prof[5]++;
    }
    for (int it = 0; it < 1024 && !whole; it++) {
      uint32_t below = __shfl_up_sync(kFull, f, 1);
      uint32_t above = __shfl_down_sync(kFull, f, 1);
      if (lane == 0) below = 0u;
      if (lane == 31) above = 0u;
      const uint32_t nf = run_fill(f | ((below | above) & hp), hp);
      const unsigned changed = __ballot_sync(kFull, nf != f);
      f = nf;
      if (!changed) break;
    }
    f_new = f_cur | f;
    // weights of the newly filled rays: the whole block when this visit
    // filled all of its accepted rays at its evaluation, else ray by ray
    float acc;
    const bool all = fresh && __ballot_sync(kFull, f != h_row) == 0u;
    if (all) {
      acc = wall;
    } else {
      unsigned re = 0;
      A.prof[6]++;
      if (c.split && sti < 0) sti = w_supertile(W, bx, by, lane, &A.prof[2]);
      const SuperTile stw = sti >= 0 ? W.st[sti] : SuperTile{};
      acc = block_weights(c, stw, c.split && sti >= 0, bx, by, lane, f, &re);
      A.eval += warp_sum_u(re);
    }
    A.count += warp_sum_u(__popc(f));
    // a block's sum is below 1024 * 1.5: 2^-16 resolution fits an int32
    A.fx += (long long)__float2int_rn(warp_sum_f(acc) * 65536.f);
    // plane edge: columns 1 and N-1 (lcirs.cc:413-440)
    {
      const int64_t c0 = (int64_t)bx * 32;
      uint32_t colmask = 0;
      if (1 >= c0 && 1 < c0 + 32) colmask |= 1u << (1 - c0);
      if (c.n - 1 >= c0 && c.n - 1 < c0 + 32) colmask |= 1u << (c.n - 1 - c0);
      if (__reduce_or_sync(kFull, f) & colmask) A.edge = 1u;
    }
    top = __shfl_sync(kFull, f, 31);
    bot = __shfl_sync(kFull, f, 0);
    lcol = __ballot_sync(kFull, f & 1u);
    rcol = __ballot_sync(kFull, f >> 31);
  }
  // write back: rows, entries consumed, filled border, state (a first visit
  // writes F as well: the body still holds an earlier point's rows)
  if (fresh) __stcg(&body[lane], h_row);
  if (any || fresh) __stcg(&body[32 + lane], f_new);
  const uint32_t flb = __ballot_sync(kFull, f_new & 1u), frb = __ballot_sync(kFull, f_new >> 31);
  const uint32_t fr0 = __shfl_sync(kFull, f_new, 0), fr31 = __shfl_sync(kFull, f_new, 31);
  if (lane <= kHState) {
    uint32_t v = 0u;
    if (lane == kHFb) v = fr0;
    else if (lane == kHFt) v = fr31;
    else if (lane == kHFl) v = flb;
    else if (lane == kHFr) v = frb;
    else if (lane == kHState) v = (state | kWCls) & ~kWQueued;
    __stcg(&hdr[lane], v);
  }
  __syncwarp();
  if (!any) return;
  // neighbours: group 0 the block above (its bottom row), 1 below (its top
  // row), 2 left (its column 31), 3 right (its column 0)
  const int g = lane >> 3, j = lane & 7;
  int nbx = bx, nby = by;
  uint32_t bits;
  if (g == 0) { nby = by + 1; bits = top; }
  else if (g == 1) { nby = by - 1; bits = bot; }
  else if (g == 2) { nbx = bx - 1; bits = lcol; }
  else { nbx = bx + 1; bits = rcol; }
  const bool inplane = bits != 0u && nbx >= 0 && nby >= 0 && nbx <= c.txmax && nby <= c.tymax;
  int owner = 0;
  if (tm && inplane) owner = team_owner(nbx, nby, tm->sh);
  const bool remote = tm && inplane && owner != tm->me;
  const bool act = inplane && !remote;
  bool ins = false;
  const int s = w_find4(T, act, nbx, nby, lane, &ins, &A.prof[3]);
  if (s >= 0 && ins) w_init_slot(W, T, s, nbx, nby, lane);
  A.prof[4] += (unsigned)__popc(__ballot_sync(kFull, s >= 0 && ins && j == 0));
  __syncwarp();
  if (s >= 0 && j == 0) w_enter(W, T, s, ins, g, bits);
  if (remote && j == 0) {
    const unsigned k = atomicAdd(&tm->inbox_n[tm->post * kTeamWarps + owner], 1u);
    if (k < tm->cap) {
      // the bits word last, after a CTA-scope fence: the owner may read the
      // message in this round as soon as it sees bits (never 0 in a message)
      uint32_t* mw = (uint32_t*)&tm->inbox[((size_t)tm->post * kTeamWarps + owner) * tm->cap + k];
      __stcg(&mw[0], (uint32_t)nbx);
      __stcg(&mw[1], (uint32_t)nby);
      __stcg(&mw[2], (uint32_t)g);
      __threadfence_block();
      __stcg(&mw[3], bits);
    } else {
      atomicOr(tm->abort_, (unsigned)kStTableFull);
    }
  }
  __syncwarp();
}

// lane 0 sets the warp's point context (the CTA fill's Ctx, 32-row blocks);
// whole warp clears the super-tile cache
__device__ __forceinline__ void w_context(WarpSh& W, const PointIn& pi, const DevLens* lenses,
                                          int split_mode, int lane) {
  if (lane == 0) {
    const DevLens& D = lenses[pi.lens];
    Ctx& c = W.c;
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
    c.tymax = (int)((c.n - 1) >> 5);
    c.split = split_mode;
    // super-tile edge as the CTA fill: 2^9 pixels, down to 2^7 as h grows
    int sl = 9;
    while (sl > 7 && c.h * (double)(1 << sl) > 1.5e-3) sl--;
    c.slog2 = sl;
    c.hf = (float)c.h;
    c.rho2f = (float)c.rho2;
    c.inv_rho2f = (float)(1.0 / c.rho2);
    c.ldaf = (float)c.ld_a;
    c.ldbf = (float)c.ld_b;
    W.top = 0;
    W.used = 0;
    W.nseed = 0;
  }
  if (lane < kWStCache) W.sttag[lane] = kEmptyKey;
  __syncwarp();
}

// whole warp: the point's seed pixels (lcirs.cc:171-174; seed rows must
// satisfy 0 < ny < N, 386-391) into W.seedx/seedy; returns kStEdge when a
// seed lies outside columns 1..N-1
__device__ __forceinline__ uint32_t w_load_seeds(WarpSh& W, int p, const int32_t* seeds,
                                                 const PointOut* out, int lane) {
  const int64_t n = W.c.n;
  uint32_t status = 0;
  const unsigned ns = min(out[p].nseeds, (unsigned)kMaxSeeds);
  for (unsigned k0 = 0; k0 < ns; k0 += 32) {
    const unsigned k = k0 + (unsigned)lane;
    int32_t px = 0, py = 0;
    bool ok = false, edge = false;
    if (k < ns) {
      px = seeds[((size_t)p * kMaxSeeds + k) * 2];
      py = seeds[((size_t)p * kMaxSeeds + k) * 2 + 1];
      if (py > 0 && (int64_t)py < n) {
        if (px < 1 || (int64_t)px > n - 1) edge = true;
        else ok = true;
      }
    }
    if (__any_sync(kFull, edge)) status |= kStEdge;
    const uint32_t okm = __ballot_sync(kFull, ok);
    if (ok) {
      const unsigned pos = W.nseed + (unsigned)__popc(okm & ((1u << lane) - 1u));
      W.seedx[pos] = px;
      W.seedy[pos] = py;
    }
    __syncwarp();
    if (lane == 0) W.nseed += (unsigned)__popc(okm);
    __syncwarp();
  }
  return status;
}

// whole warp: the amoeba export (32 x 8 tiles of F, as the CTA fill) of
// the point's blocks when `complete`, and the clearing of the slots used
__device__ __forceinline__ void w_finish(const WTable& T, const WScratch& sc, int p,
                                         unsigned nused, bool complete, int lane) {
  for (unsigned u = (unsigned)lane; u < nused; u += 32) {
    const uint32_t slot = ldcg32(&T.used[u]);
    if (sc.dump && complete) {
      const uint32_t* h = T.hdr + (size_t)slot * kWHdrWords;
      if (ldcg32(&h[kHState]) & kWCls) {
        const uint32_t* b = T.body + (size_t)slot * 64;
        const uint32_t bxk = ldcg32(&h[kHBx]), byk = ldcg32(&h[kHBy]);
        for (int t8 = 0; t8 < 4; t8++) {
          uint32_t fm[8], a8 = 0;
          for (int r = 0; r < 8; r++) a8 |= (fm[r] = ldcg32(&b[32 + 8 * t8 + r]));
          if (!a8) continue;
          const unsigned d = atomicAdd(sc.dump_count, 1u);
          if (d < sc.dump_cap) {
            uint32_t* o = sc.dump + (size_t)d * kDumpWords;
            o[0] = (uint32_t)p;
            o[1] = bxk;
            o[2] = byk * 4u + (uint32_t)t8;
            for (int r = 0; r < 8; r++) o[3 + r] = fm[r];
          }
        }
      }
    }
    __stcg((unsigned long long*)&T.keys[slot], (unsigned long long)kEmptyKey);
  }
}

// the warp's table inside a WScratch
__device__ __forceinline__ WTable w_table(const WScratch& sc, size_t gw) {
  WTable T;
  const size_t slots = (size_t)1 << sc.cap_log2;
  T.keys = sc.keys + gw * slots;
  T.hdr = sc.hdr + gw * slots * kWHdrWords;
  T.body = sc.body + gw * slots * 64;
  T.used = sc.used + gw * slots;
  T.spill = sc.spill + gw * slots;
  T.mask = (uint32_t)(slots - 1);
  T.usable = (unsigned)(slots / 4 * 3);
  return T;
}

}  // namespace

template <int MINB>
__global__ void __launch_bounds__(kWThreads, MINB)
wfill_kernel(const PointIn* points, int npoints, const DevLens* lenses, const int32_t* seeds,
             PointOut* out, WScratch sc, int split_mode, const int32_t* list,
             const unsigned* list_count) {
  __shared__ WarpSh wsh[kWWarps];
  const int lane = threadIdx.x & 31;
  WarpSh& W = wsh[threadIdx.x >> 5];
  const size_t gw = (size_t)blockIdx.x * kWWarps + (threadIdx.x >> 5);
  if (gw >= (size_t)sc.warps) return;   // whole warps; the kernel has no block barrier
  const WTable T = w_table(sc, gw);
  const size_t slots = (size_t)T.mask + 1;
  const unsigned pop_limit = 16u * (unsigned)slots;   // bound on block visits per point
  const unsigned nwork = list ? *list_count : (unsigned)npoints;
  for (;;) {
    unsigned w = 0;
    if (lane == 0) w = atomicAdd(sc.next_point, 1u);
    w = __shfl_sync(kFull, w, 0);
    if (w >= nwork) break;
    const int p = list ? list[w] : (int)w;
    const PointIn pi = points[p];
    w_context(W, pi, lenses, split_mode, lane);
    const int64_t n = W.c.n;
    uint32_t status = 0;
    if (!(n > 2 && n < ((int64_t)1 << 31)) || (out[p].status & kStBadInput)) status |= kStBadInput;
    else if (pi.est_blocks > sc.wthr) status |= kStTableFull;   // left to the CTA fill
    WAcc A = {0ull, 0ull, 0ull, 0ll, 0u, {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u}};
    unsigned pops = 0;
    if (!status) {
      status |= w_load_seeds(W, p, seeds, out, lane);
      // seed blocks: found or inserted by group 0, marked and queued
      const unsigned nsd = W.nseed;
      for (unsigned k = 0; k < nsd; k++) {
        const int sbx = W.seedx[k] >> 5, sby = W.seedy[k] >> 5;
        bool ins = false;
        unsigned rounds = 0;
        const int s = w_find4(T, lane < 8, sbx, sby, lane, &ins, &rounds);
        if (lane < 8 && s >= 0 && ins) w_init_slot(W, T, s, sbx, sby, lane);
        __syncwarp();
        if (lane == 0 && s >= 0) {
          uint32_t* h = T.hdr + (size_t)s * kWHdrWords;
          const uint32_t st0 = ldcg32(&h[kHState]);
          __stcg(&h[kHState], st0 | kWSeed | kWQueued);
          if (!(st0 & kWQueued)) w_push_stack(W, T, (uint32_t)s);
        }
        __syncwarp();
        const int sl0 = __shfl_sync(kFull, s, 0);
        if (sl0 < 0 || W.used > T.usable) {
          status |= kStTableFull;
          break;
        }
      }
      // blocks, last queued first
      while (!(status & (kStTableFull | kStTimeout))) {
        const unsigned t = W.top;
        if (t == 0u) break;
        const uint32_t slot = t - 1u < (unsigned)kWStack ? W.stack[t - 1u] : ldcg32(&T.spill[t - 1u]);
        __syncwarp();
        if (lane == 0) W.top = t - 1u;
        __syncwarp();
        w_block(W, T, slot, lane, A, nullptr);
        if (W.used > T.usable) status |= kStTableFull;
        if (++pops > pop_limit) status |= kStTimeout;
      }
    }
    const unsigned nused = min(W.used, (unsigned)slots);
    if (sc.prof && lane == 0) {
      A.prof[7] = 1u;
      for (int q = 0; q < 8; q++) atomicAdd(&sc.prof[q], (unsigned long long)A.prof[q]);
    }
    if (lane == 0) {
      PointOut o = out[p];
      o.count = A.count;
      o.wsum_fx = A.fx * 65536ll;
      o.status |= status | (A.edge ? (uint32_t)kStEdge : 0u);
      o.tiles = nused;
      o.diag = (status & kStTimeout) ? 0x10000u : 0u;
      o.rays_eval = A.eval;
      o.rays_fp64 = A.fp64;
      out[p] = o;
    }
    // amoeba export and the clearing of the slots used (the table starts
    // every point empty)
    w_finish(T, sc, p, nused, !(status & (kStTableFull | kStTimeout | kStBadInput)), lane);
    __syncwarp();
  }
}

// ===========================================================================
// Team fill: kTeamWarps warps of one CTA fill one large point together, in
// rounds.  Each warp owns the blocks of its share of the super-tiles
// (team_owner) in its own table and works them as the warp fill does; an
// entry into a block of another share is a message in that warp's inbox.
// A round: every warp reads the previous round's messages into its table,
// the CTA meets at a barrier, every warp works its stack empty, the CTA
// meets again, and another round runs while any message was sent.  The only
// waits are these barriers, which every warp reaches once per round.
// ===========================================================================
namespace {
constexpr int kTThreads = 32 * kTeamWarps;
constexpr int kTeamRounds = 1 << 16;

struct TeamSh {
  WarpSh w[kTeamWarps];
  unsigned inbox_n[2 * kTeamWarps];    // messages reserved per inbox
  unsigned inbox_rd[2 * kTeamWarps];   // messages read by the owner
  unsigned abort_;          // kStTableFull / kStTimeout: the point ends
  int point;
  unsigned long long count, eval, fp64;
  unsigned long long fx;    // two's complement sum of the warps' 2^-16 units
  unsigned tiles, status;
};
}  // namespace

// whole warp: the messages of inbox buffer b that this warp has not read,
// in order, up to the first one not yet written; returns how many it took.
// Each message is looked up by group 0 and applied by one lane; its bits
// word is cleared (the slot reads "unwritten" when the buffer is reused).
__device__ __noinline__ unsigned team_drain(TeamSh& S, WarpSh& W, const WTable& T,
                                            const WTeam& tm, int b, int wid, int lane) {
  uint4* box = tm.inbox + ((size_t)b * kTeamWarps + wid) * tm.cap;
  unsigned* rd = &S.inbox_rd[b * kTeamWarps + wid];
  unsigned took = 0;
  for (;;) {
    unsigned k = 0, n = 0, ab = 0;
    if (lane == 0) {
      k = *(volatile unsigned*)rd;
      n = min(*(volatile unsigned*)&S.inbox_n[b * kTeamWarps + wid], tm.cap);
      ab = *(volatile unsigned*)&S.abort_;
    }
    k = __shfl_sync(kFull, k, 0);
    n = __shfl_sync(kFull, n, 0);
    if (__shfl_sync(kFull, ab, 0) || k >= n) break;
    uint32_t* mw = (uint32_t*)&box[k];
    uint32_t bits = 0, mx = 0, my = 0, side = 0;
    if (lane == 0) {
      bits = __ldcg(&mw[3]);   // from L2: the sender's stores go there
      if (bits) {
        __threadfence_block();
        mx = __ldcg(&mw[0]);
        my = __ldcg(&mw[1]);
        side = __ldcg(&mw[2]);
      }
    }
    bits = __shfl_sync(kFull, bits, 0);
    if (!bits) break;   // reserved, not written yet: read in a later pass
    mx = __shfl_sync(kFull, mx, 0);
    my = __shfl_sync(kFull, my, 0);
    side = __shfl_sync(kFull, side, 0);
    bool ins = false;
    unsigned rounds = 0;
    const int s = w_find4(T, lane < 8, (int)mx, (int)my, lane, &ins, &rounds);
    if (lane < 8 && s >= 0 && ins) w_init_slot(W, T, s, (int)mx, (int)my, lane);
    __syncwarp();
    if (lane == 0) {
      if (s >= 0) w_enter(W, T, s, ins, (int)side, bits);
      __stcg(&mw[3], 0u);
      *rd = k + 1u;
    }
    __syncwarp();
    took++;
    const int sl0 = __shfl_sync(kFull, s, 0);
    if (sl0 < 0 || W.used > T.usable) {
      if (lane == 0) atomicOr(&S.abort_, (unsigned)kStTableFull);
      break;
    }
  }
  return took;
}

template <int MINB>
__global__ void __launch_bounds__(kTThreads, MINB)
tfill_kernel(const PointIn* points, int npoints, const DevLens* lenses, const int32_t* seeds,
             PointOut* out, WScratch sc, int split_mode, const int32_t* list,
             const unsigned* list_count) {
  __shared__ TeamSh S;
  const int lane = threadIdx.x & 31;
  const int wid = threadIdx.x >> 5;
  WarpSh& W = S.w[wid];
  const WTable T = w_table(sc, (size_t)blockIdx.x * kTeamWarps + wid);
  const size_t slots = (size_t)T.mask + 1;
  const unsigned pop_limit = 16u * (unsigned)slots;   // block visits per warp and point
  const unsigned nwork = list ? *list_count : (unsigned)npoints;
  WTeam tm;
  tm.inbox = sc.inbox + (size_t)blockIdx.x * 2 * kTeamWarps * sc.inbox_cap;
  tm.inbox_n = S.inbox_n;
  tm.abort_ = &S.abort_;
  tm.cap = sc.inbox_cap;
  tm.me = wid;
  tm.post = 1;
  tm.sh = 0;
  for (;;) {
    if (threadIdx.x == 0) {
      const unsigned w = atomicAdd(sc.next_point, 1u);
      S.point = w < nwork ? (list ? list[w] : (int)w) : -1;
      S.abort_ = 0u;
      S.count = S.eval = S.fp64 = S.fx = 0ull;
      S.tiles = 0u;
      S.status = 0u;
    }
    if (threadIdx.x < 2 * kTeamWarps) {
      S.inbox_n[threadIdx.x] = 0u;
      S.inbox_rd[threadIdx.x] = 0u;
    }
    __syncthreads();
    const int p = S.point;
    if (p < 0) break;
    const PointIn pi = points[p];
    w_context(W, pi, lenses, split_mode, lane);
    tm.sh = W.c.slog2 - 5;
    const int64_t n = W.c.n;
    const bool skip = !(n > 2 && n < ((int64_t)1 << 31)) || (out[p].status & kStBadInput);
    uint32_t status = skip ? (uint32_t)kStBadInput : 0u;
    WAcc A = {0ull, 0ull, 0ull, 0ll, 0u, {0u, 0u, 0u, 0u, 0u, 0u, 0u, 0u}};
    if (!skip) {
      status |= w_load_seeds(W, p, seeds, out, lane);
      // the seed blocks of this warp's share
      const unsigned nsd = W.nseed;
      for (unsigned k = 0; k < nsd; k++) {
        const int sbx = W.seedx[k] >> 5, sby = W.seedy[k] >> 5;
        if (team_owner(sbx, sby, tm.sh) != wid) continue;
        bool ins = false;
        unsigned rounds = 0;
        const int s = w_find4(T, lane < 8, sbx, sby, lane, &ins, &rounds);
        if (lane < 8 && s >= 0 && ins) w_init_slot(W, T, s, sbx, sby, lane);
        __syncwarp();
        if (lane == 0 && s >= 0) {
          uint32_t* h = T.hdr + (size_t)s * kWHdrWords;
          const uint32_t st0 = ldcg32(&h[kHState]);
          __stcg(&h[kHState], st0 | kWSeed | kWQueued);
          if (!(st0 & kWQueued)) w_push_stack(W, T, (uint32_t)s);
        }
        __syncwarp();
        const int sl0 = __shfl_sync(kFull, s, 0);
        if (sl0 < 0 || W.used > T.usable) {
          if (lane == 0) atomicOr(&S.abort_, (unsigned)kStTableFull);
          break;
        }
      }
    }
    unsigned pops = 0;
    int round = 0;
    for (;; round++) {
      const int pin = round & 1;   // buffer holding the previous round's messages
      tm.post = pin ^ 1;
      // the previous round's messages not read yet (all written: the
      // barrier that ended the round orders them)
      if (round > 0 && !skip) team_drain(S, W, T, tm, pin, wid, lane);
      __syncthreads();
      // the buffer is read out: it takes the next round's messages
      if (threadIdx.x < kTeamWarps) {
        S.inbox_n[pin * kTeamWarps + threadIdx.x] = 0u;
        S.inbox_rd[pin * kTeamWarps + threadIdx.x] = 0u;
      }
      // this warp's blocks, last queued first, and the messages other warps
      // send it meanwhile, until both run dry
      for (;;) {
        while (!skip) {
          unsigned ab = 0;
          if (lane == 0) ab = *(volatile unsigned*)&S.abort_;
          if (__shfl_sync(kFull, ab, 0)) break;
          const unsigned t = W.top;
          if (t == 0u) break;
          const uint32_t slot =
              t - 1u < (unsigned)kWStack ? W.stack[t - 1u] : ldcg32(&T.spill[t - 1u]);
          __syncwarp();
          if (lane == 0) W.top = t - 1u;
          __syncwarp();
          w_block(W, T, slot, lane, A, &tm);
          ++pops;
          if (lane == 0) {
            if (W.used > T.usable) atomicOr(&S.abort_, (unsigned)kStTableFull);
            if (pops > pop_limit) atomicOr(&S.abort_, (unsigned)kStTimeout);
          }
        }
        if (skip || team_drain(S, W, T, tm, tm.post, wid, lane) == 0u) break;
      }
      __syncthreads();
      const bool ab = S.abort_ != 0u;
      const int more = __syncthreads_or(lane == 0 && S.inbox_n[tm.post * kTeamWarps + wid] >
                                                         S.inbox_rd[tm.post * kTeamWarps + wid]);
      if (ab || !more) break;
      if (round + 1 >= kTeamRounds) {
        if (threadIdx.x == 0) atomicOr(&S.abort_, (unsigned)kStTimeout);
        break;
      }
    }
    // the point's totals
    if (lane == 0) {
      atomicAdd(&S.count, A.count);
      atomicAdd(&S.eval, A.eval);
      atomicAdd(&S.fp64, A.fp64);
      atomicAdd(&S.fx, (unsigned long long)A.fx);
      atomicAdd(&S.tiles, min(W.used, (unsigned)slots));
      atomicOr(&S.status, status | (A.edge ? (uint32_t)kStEdge : 0u));
    }
    __syncthreads();
    const uint32_t fin = S.status | S.abort_;
    // a point given up on may leave messages unread (and its counters
    // reset): every slot of the team's inboxes reads "unwritten" again
    if (S.abort_) {
      uint32_t* all = (uint32_t*)tm.inbox;
      const size_t nslot = (size_t)2 * kTeamWarps * tm.cap;
      for (size_t q = threadIdx.x; q < nslot; q += blockDim.x) __stcg(&all[4 * q + 3], 0u);
    }
    if (threadIdx.x == 0) {
      PointOut o = out[p];
      o.count = S.count;
      o.wsum_fx = (int64_t)S.fx * 65536ll;
      o.status |= fin;
      o.tiles = S.tiles;
      // rounds (bits 0-15) and the time limit (bit 16)
      o.diag = (uint32_t)min(round + 1, 0xffff) | ((S.abort_ & kStTimeout) ? 0x10000u : 0u);
      o.rays_eval = S.eval;
      o.rays_fp64 = S.fp64;
      out[p] = o;
    }
    w_finish(T, sc, p, min(W.used, (unsigned)slots),
             !(fin & (kStTableFull | kStTimeout | kStBadInput)), lane);
    __syncthreads();
  }
}

int tfill_default_teams() {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms * 2;
}

size_t tscratch_bytes(int teams, int cap_log2, unsigned inbox_cap) {
  return wscratch_bytes(teams * kTeamWarps, cap_log2) +
         (size_t)teams * 2 * kTeamWarps * inbox_cap * sizeof(uint4) + 256;
}

void tscratch_init(WScratch* s, void* base, int teams, int cap_log2, unsigned inbox_cap,
                   cudaStream_t st) {
  wscratch_init(s, base, teams * kTeamWarps, cap_log2, st);
  const size_t wb = wscratch_bytes(teams * kTeamWarps, cap_log2);
  s->inbox = (uint4*)(((uintptr_t)base + wb + 255) / 256 * 256);
  s->inbox_cap = inbox_cap;
  // every message slot reads "unwritten" (bits 0) until a sender writes it
  cudaMemsetAsync(s->inbox, 0, (size_t)teams * 2 * kTeamWarps * inbox_cap * sizeof(uint4), st);
}

void launch_tfill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                  const int32_t* d_seeds, PointOut* d_out, const WScratch& s, int mode,
                  cudaStream_t st, const int32_t* d_list, const unsigned* d_count) {
  if (npoints <= 0 || s.warps < kTeamWarps) return;
  cudaMemsetAsync(s.next_point, 0, sizeof(unsigned), st);
  tfill_kernel<2><<<s.warps / kTeamWarps, kTThreads, 0, st>>>(
      d_points, npoints, d_lenses, d_seeds, d_out, s, mode == kFillSplit ? 1 : 0, d_list,
      d_count);
}

int wfill_default_warps() {
  int dev = 0, sms = 152;
  if (cudaGetDevice(&dev) == cudaSuccess)
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms * kWOcc * kWWarps;
}

size_t wscratch_bytes(int warps, int cap_log2) {
  const size_t ent = (size_t)warps << cap_log2;
  return ent * (8 + (size_t)kWHdrWords * 4 + 64 * 4 + 4 + 4) + 256;
}

void wscratch_init(WScratch* s, void* base, int warps, int cap_log2, cudaStream_t st) {
  const size_t ent = (size_t)warps << cap_log2;
  char* p = (char*)base;
  s->warps = warps;
  s->cap_log2 = cap_log2;
  s->keys = (uint64_t*)p;
  p += ent * 8;
  s->hdr = (uint32_t*)p;
  p += ent * (size_t)kWHdrWords * 4;
  s->body = (uint32_t*)p;
  p += ent * 64 * 4;
  s->used = (uint32_t*)p;
  p += ent * 4;
  s->spill = (uint32_t*)p;
  p += ent * 4;
  s->next_point = (unsigned*)p;
  s->wthr = 14000;
  s->dump = nullptr;
  s->dump_count = nullptr;
  s->dump_cap = 0;
  s->prof = nullptr;
  s->inbox = nullptr;
  s->inbox_cap = 0;
  // keys empty (all ones); headers are written when a slot is taken, bodies
  // are read only once their state says so
  cudaMemsetAsync(s->keys, 0xff, ent * 8, st);
  cudaMemsetAsync(s->next_point, 0, 256, st);
}

void launch_wfill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                  const int32_t* d_seeds, PointOut* d_out, const WScratch& s, int mode,
                  cudaStream_t st, const int32_t* d_list, const unsigned* d_count,
                  int ctas_per_sm) {
  if (npoints <= 0 || s.warps <= 0) return;
  cudaMemsetAsync(s.next_point, 0, sizeof(unsigned), st);
  int ctas = (s.warps + kWWarps - 1) / kWWarps;
  size_t pad = 0;
  if (ctas_per_sm > 0 && ctas_per_sm < kWOcc) {
    int dev = 0, sms = 152, smem = 228 * 1024;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    cudaDeviceGetAttribute(&smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev);
    int reserve = 1024;
    cudaDeviceGetAttribute(&reserve, cudaDevAttrReservedSharedMemoryPerBlock, dev);
    ctas = std::min(ctas, sms * ctas_per_sm);
    // unused dynamic shared memory so that no SM takes more CTAs than that:
    // (ctas_per_sm + 1) of them would exceed the SM's shared memory
    const size_t per = (size_t)smem / (size_t)(ctas_per_sm + 1) + 1;
    const size_t used = sizeof(WarpSh) * kWWarps + (size_t)reserve;
    pad = per > used ? per - used : 0;
    static bool carveout = false;
    if (!carveout) {
      cudaFuncSetAttribute(wfill_kernel<kWOcc>, cudaFuncAttributePreferredSharedMemoryCarveout,
                           100);
      carveout = true;
    }
  }
  wfill_kernel<kWOcc><<<ctas, kWThreads, pad, st>>>(d_points, npoints, d_lenses, d_seeds, d_out,
                                                    s, mode == kFillSplit ? 1 : 0, d_list,
                                                    d_count);
}

int block_rec_words(int bh) {
  return bh == 8 ? Lo<8>::kWords : (bh == 16 ? Lo<16>::kWords : Lo<32>::kWords);
}

namespace {
// block-table entries over all CTAs
size_t table_entries(int ctas, int cap_log2, int big_ctas, int big_log2) {
  big_ctas = big_ctas < 0 ? 0 : (big_ctas > ctas ? ctas : big_ctas);
  return ((size_t)big_ctas << big_log2) + ((size_t)(ctas - big_ctas) << cap_log2);
}
}  // namespace

size_t fill_scratch_bytes(int ctas, int cap_log2, int bh, int big_ctas, int big_log2) {
  const size_t ent = table_entries(ctas, cap_log2, big_ctas, big_log2);
  const size_t scap = (size_t)1 << kSuperLog2;
  return ent * (8 + (size_t)block_rec_words(bh) * 4 + 4 + 4) +
         (size_t)ctas * scap * (8 + kSEntryWords * 4 + 4) + 256;
}

void fill_scratch_init(FillScratch* s, void* base, int ctas, int cap_log2, int bh,
                       cudaStream_t st, int big_ctas, int big_log2) {
  big_ctas = big_ctas < 0 ? 0 : (big_ctas > ctas ? ctas : big_ctas);
  const size_t ent = table_entries(ctas, cap_log2, big_ctas, big_log2);
  const int rw = block_rec_words(bh);
  char* p = (char*)base;
  s->ctas = ctas;
  s->cap_log2 = cap_log2;
  s->big_ctas = big_ctas;
  s->big_log2 = big_ctas > 0 ? big_log2 : cap_log2;
  s->nbig = nullptr;
  s->block_h = bh;
  s->rec_words = rw;
  s->keys = (uint64_t*)p;
  p += ent * 8;
  s->recs = (uint32_t*)p;
  p += ent * rw * 4;
  s->ring = (uint32_t*)p;
  p += ent * 4;
  s->used = (uint32_t*)p;
  p += ent * 4;
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
  s->prof = nullptr;
  s->heartbeat = nullptr;
  cudaMemsetAsync(s->keys, 0xff, ent * 8, st);
  cudaMemsetAsync(s->recs, 0, ent * rw * 4, st);
  cudaMemsetAsync(s->ring, 0, ent * 4, st);
  cudaMemsetAsync(s->skeys, 0xff, (size_t)ctas * scap * 8, st);
  cudaMemsetAsync(s->sents, 0, (size_t)ctas * scap * kSEntryWords * 4, st);
}

namespace {
int g_fill_occ = 4;   // resident fill CTAs per SM (measured: 2 -> 56k, 3 -> 63k, 4 -> 64.5k points/s)
}  // namespace

void set_fill_occupancy(int occ) {
  if (occ >= 2 && occ <= 4) g_fill_occ = occ;
}

int fill_occupancy() { return g_fill_occ; }

int fill_default_ctas() {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  return sms > 0 ? sms * g_fill_occ : 2;
}

void launch_fill(const PointIn* d_points, int npoints, const DevLens* d_lenses,
                 const int32_t* d_seeds, PointOut* d_out, const FillScratch& s, int mode,
                 int threads, cudaStream_t st, const int32_t* d_list, const unsigned* d_count) {
  if (npoints <= 0) return;
  cudaMemsetAsync(s.next_point, 0, 2 * sizeof(unsigned), st);
  const int ctas = s.ctas;
  const int split = mode == kFillSplit ? 1 : 0;
  switch (s.block_h) {
    case 8:
      fill_kernel<8, 2><<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out, s,
                                                 split, d_list, d_count);
      break;
    case 16:
      fill_kernel<16, 2><<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out, s,
                                                  split, d_list, d_count);
      break;
    default:
      if (g_fill_occ == 4)
        fill_kernel<32, 4><<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out,
                                                     s, split, d_list, d_count);
      else if (g_fill_occ == 3)
        fill_kernel<32, 3><<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out,
                                                     s, split, d_list, d_count);
      else
        fill_kernel<32, 2><<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out,
                                                     s, split, d_list, d_count);
      break;
  }
}

// ---------------------------------------------------------------------------
// size-ordered work list (counting sort on half-octave buckets of the
// predicted size, largest first)
// ---------------------------------------------------------------------------
constexpr int kOrderBuckets = 64;

__device__ __forceinline__ int order_bucket(uint32_t est) {
  const int b = (int)(2.f * __log2f((float)est + 1.f));
  return b < 0 ? 0 : (b >= kOrderBuckets ? kOrderBuckets - 1 : b);
}

int order_bucket_host(unsigned est) {
  const int b = (int)(2.0 * std::log2((double)est + 1.0));
  return b < 0 ? 0 : (b >= kOrderBuckets ? kOrderBuckets - 1 : b);
}

__global__ void order_hist_kernel(const PointIn* pts, int n, unsigned* hist) {
  __shared__ unsigned h[kOrderBuckets];
  if (threadIdx.x < kOrderBuckets) h[threadIdx.x] = 0;
  __syncthreads();
  for (int p = blockIdx.x * blockDim.x + threadIdx.x; p < n; p += gridDim.x * blockDim.x)
    atomicAdd(&h[order_bucket(pts[p].est_blocks)], 1u);
  __syncthreads();
  if (threadIdx.x < kOrderBuckets && h[threadIdx.x]) atomicAdd(&hist[threadIdx.x], h[threadIdx.x]);
}

// meta: [0] points, [1] list head (buckets >= big_bucket), [2..66) histogram,
// [66..130) cursors
__global__ void order_scan_kernel(int n, unsigned* meta, int big_bucket) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const unsigned* hist = meta + 2;
  unsigned* cur = meta + 2 + kOrderBuckets;
  unsigned acc = 0, head = 0;
  for (int b = kOrderBuckets - 1; b >= 0; b--) {
    cur[b] = acc;
    acc += hist[b];
    if (b >= big_bucket) head = acc;
  }
  meta[0] = (unsigned)n;
  meta[1] = head;
}

__global__ void order_scatter_kernel(const PointIn* pts, int n, unsigned* meta, int32_t* list) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const unsigned pos = atomicAdd(&meta[2 + kOrderBuckets + order_bucket(pts[p].est_blocks)], 1u);
  if (pos < (unsigned)n) list[pos] = p;
}

void launch_order(const PointIn* d_points, int npoints, int32_t* d_list, unsigned* d_meta,
                  unsigned big_units, cudaStream_t st) {
  cudaMemsetAsync(d_meta, 0, sizeof(unsigned) * (2 + 2 * kOrderBuckets), st);
  if (npoints <= 0) return;
  const int blocks = (npoints + 255) / 256;
  order_hist_kernel<<<blocks < 1024 ? blocks : 1024, 256, 0, st>>>(d_points, npoints,
                                                                  d_meta + 2);
  order_scan_kernel<<<1, 32, 0, st>>>(npoints, d_meta, order_bucket_host(big_units));
  order_scatter_kernel<<<blocks, 256, 0, st>>>(d_points, npoints, d_meta, d_list);
}

// Points whose block table overflowed: clear their transient status bits and
// list them for a retry with a larger table.
__global__ void collect_overflow_kernel(PointOut* out, int npoints, int32_t* list,
                                        unsigned* count) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= npoints) return;
  const uint32_t st = out[p].status;
  if (st & kStTableFull) {
    out[p].status = st & ~(kStTableFull | kStTimeout);
    list[atomicAdd(count, 1u)] = p;
  }
}

void launch_collect_overflow(PointOut* d_out, int npoints, int32_t* d_list, unsigned* d_count,
                             cudaStream_t st) {
  if (npoints <= 0) return;
  cudaMemsetAsync(d_count, 0, sizeof(unsigned), st);
  collect_overflow_kernel<<<(npoints + 255) / 256, 256, 0, st>>>(d_out, npoints, d_list, d_count);
}

}  // namespace tl
