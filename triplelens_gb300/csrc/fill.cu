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

constexpr unsigned kIdleSpinLimit = 1u << 24;   // x ~100 ns sleeps
constexpr unsigned kEntrySpinLimit = 1u << 22;

struct Ctx {
  double sx, sy;
  double cx0, cy0, h;
  double rho2, ld_a, ld_b;
  double m1, m2, m3;
  double z2x, z3x, z3y;
  int64_t n;
  int32_t binary;
  int32_t txmax, tymax;
};

struct Shared {
  Ctx c;
  unsigned head, tail, pending, used;
  unsigned abort_, status;
  unsigned long long count, wsum, rays_eval, rays_fp64;
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
        T.used[u] = i;  // u < capacity: at most mask+1 slots exist
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
  for (;;) {
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
  unsigned long long local_count = 0, local_eval = 0, local_fp64 = 0;
  double local_wsum = 0.0;
  uint32_t edge = 0;
  for (;;) {
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
      unsigned nr;
      eval_tile_fp64(c, tx, ty, lane, Hrow, w, &nr);
      have_w = true;
      local_eval += warp_sum_u(nr);
      local_fp64 += warp_sum_u(nr);
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
#pragma unroll
      for (int r = 0; r < 8; r++) {
        cnt += __popc(nw[r]);
        if ((nw[r] >> lane) & 1u) {
          if (have_w) {
            acc += w[r];
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
      local_fp64 += re_eval;
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
    if (!again) break;
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
            PointOut* out, FillScratch sc) {
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

  for (;;) {
    if (threadIdx.x == 0) {
      S.point = (int)atomicAdd(sc.next_point, 1u);
      S.head = S.tail = S.pending = S.used = 0;
      S.abort_ = 0;
      S.count = S.wsum = S.rays_eval = S.rays_fp64 = 0;
      S.status = 0;
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
      o.rays_eval = S.rays_eval;
      o.rays_fp64 = S.rays_fp64;
      out[p] = o;
    }
    // clear the slots this point used (tables start every point empty)
    const unsigned nused = S.used < cap ? S.used : (unsigned)cap;
    for (unsigned u = threadIdx.x; u < nused; u += blockDim.x) {
      const uint32_t slot = T.used[u];
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
      T.keys[slot] = kEmptyKey;
      uint4* r4 = (uint4*)(T.recs + (size_t)slot * kRecWords);
#pragma unroll
      for (int q = 0; q < kRecWords / 4; q++) r4[q] = make_uint4(0u, 0u, 0u, 0u);
    }
    if (S.abort_) {
      const unsigned nt = S.tail < cap ? S.tail : (unsigned)cap;
      for (unsigned u = threadIdx.x; u < nt; u += blockDim.x) T.ring[u] = 0u;
    }
    __threadfence_block();
    __syncthreads();
  }
}

size_t fill_scratch_bytes(int ctas, int cap_log2) {
  const size_t cap = (size_t)1 << cap_log2;
  return (size_t)ctas * cap * (8 + kRecWords * 4 + 4 + 4) + 256;
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
  s->next_point = (unsigned*)p;
  s->dump = nullptr;
  s->dump_count = nullptr;
  s->dump_cap = 0;
  cudaMemsetAsync(s->keys, 0xff, (size_t)ctas * cap * 8, st);
  cudaMemsetAsync(s->recs, 0, (size_t)ctas * cap * kRecWords * 4, st);
  cudaMemsetAsync(s->ring, 0, (size_t)ctas * cap * 4, st);
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
  (void)mode;
  if (npoints <= 0) return;
  cudaMemsetAsync(s.next_point, 0, sizeof(unsigned), st);
  const int ctas = s.ctas;
  fill_kernel<<<ctas, threads, 0, st>>>(d_points, npoints, d_lenses, d_seeds, d_out, s);
}

}  // namespace tl
