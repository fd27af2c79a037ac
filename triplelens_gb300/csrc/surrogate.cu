// surrogate.cu - the learned finite-source correction (include/tl_surrogate.h).
//
// A small MLP maps features of a source position (lens geometry, rho, limb
// darkening, point-source magnification, offset from the nearest caustic
// sample) to y = ln(A_finite / A_point).  It is trained on magnifications
// from the GPU IRS and evaluated as an ensemble; points whose members
// disagree, or that lie close to a caustic, are sent back to the IRS.
//
//   features_kernel     one thread per position: cold FP64 image solve
//                       (tl_math.h), A_point (lcbase.cc:17-38), nearest of
//                       the 3000 caustic samples, 14 features
//   gemm_bf16_kernel    C = A B on the tensor cores (mma.sync m16n8k16, BF16
//                       in, FP32 accumulate) with strided operands, so the
//                       forward product, both backward products and the
//                       split-K weight gradient share one kernel; epilogues:
//                       bias + SiLU (BF16 Z and H), SiLU backward, FP32 atomic
//   out_layer_kernel    256 -> 1 output, loss and its gradient, dw5/db5
//   adam_kernel         FP32 Adam on the master parameters + BF16 mirror
//   gate_kernel         ensemble mean/std, gating, A = A_point exp(mean)
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>

#include "batch_internal.h"
#include "engine.h"
#include "engine_host.h"
#include "tl_surrogate.h"

namespace tl {
namespace sur {

constexpr int kIn = TLS_FEATURES;   // 14 features
constexpr int kInPad = 16;          // padded to one k16 step
constexpr int kW = 256;             // hidden width
constexpr int kHidden = 4;          // hidden layers (SiLU)

// parameter layout of one member (floats): W1[256][16] b1[256]
// (W_l[256][256] b_l[256]) for l = 2..4, w5[256] b5[1]
constexpr size_t kOffW1 = 0;
constexpr size_t kOffB1 = kOffW1 + (size_t)kW * kInPad;
constexpr size_t kOffW2 = kOffB1 + kW;
constexpr size_t kLayerHH = (size_t)kW * kW + kW;
constexpr size_t kOffW5 = kOffW2 + 3 * kLayerHH;
constexpr size_t kOffB5 = kOffW5 + kW;
constexpr size_t kParams = kOffB5 + 1;

__host__ __device__ constexpr size_t off_w(int l) {  // l = 1..4
  return l == 1 ? kOffW1 : kOffW2 + (size_t)(l - 2) * kLayerHH;
}
__host__ __device__ constexpr size_t off_b(int l) {
  return l == 1 ? kOffB1 : off_w(l) + (size_t)kW * kW;
}

// ---------------------------------------------------------------------------
// features
// ---------------------------------------------------------------------------
// cos(i), sin(i) for the Laguerre fallback step, from the host libm
__constant__ TrigTable s_trig;

bool upload_trig() {
  static bool done = false;
  if (done) return true;
  TrigTable t;
  for (int i = 0; i <= kMaxIt; i++) {
    t.c[i] = cos(1.0 * i);
    t.s[i] = sin(1.0 * i);
  }
  done = cudaMemcpyToSymbol(s_trig, &t, sizeof(t)) == cudaSuccess;
  return done;
}

__global__ void __launch_bounds__(64)
features_kernel(int n, const double* xy, const int32_t* lens_idx, const DevLens* lenses,
                const cx* ca_all, float* feat, double* aps, float* dc_rho) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  const int li = lens_idx[p];
  const DevLens& D = lenses[li];
  const Lens L = D.L;
  const cx src = mk(xy[2 * (size_t)p], xy[2 * (size_t)p + 1]);
  // point-source images, cold start (imgpoint.cc:208-274)
  RootChain ch;
  chain_reset(&ch, nullptr);
  cx imgs[10];
  const int ni = chain_images(L, &ch, src, imgs, &s_trig);
  // A_point over the images on the IRS image plane (the IRS sees no others);
  // an image whose disc may reach the plane's edge marks the point for the
  // IRS (its magnification there is the truncated one)
  const Grid& g = D.g;
  double a = 0.0;
  bool edge = false;
  for (int k = 0; k < ni; k++) {
    const double ak = image_amp(L, imgs[k]);
    const double nx = (imgs[k].re - g.corner_x) / g.h, ny = (imgs[k].im - g.corner_y) / g.h;
    const double r = 4.0 * sqrt(fmax(ak, 1.0)) * (double)D.ppr + 8.0;   // pixels
    const double lo = 1.0, hi = (double)(g.n - 1);
    if (nx >= lo && nx <= hi && ny >= lo && ny <= hi) a += ak;
    if (nx - r < lo || nx + r > hi || ny - r < lo || ny + r > hi) {
      if (!(nx + r < lo || nx - r > hi || ny + r < lo || ny - r > hi)) edge = true;
    }
  }
  // nearest caustic sample and the local tangent of its branch
  const cx* ca = ca_all + (size_t)li * kBranches * kCCLen;
  float best = 3.0e38f;
  int bk = 0, bj = 0;
  const float sx = (float)src.re, sy = (float)src.im;
  for (int k = 0; k < kBranches; k++) {
    for (int j = 0; j < kCCLen; j++) {
      const float dx = (float)ca[k * kCCLen + j].re - sx, dy = (float)ca[k * kCCLen + j].im - sy;
      const float d2 = dx * dx + dy * dy;
      if (d2 < best) {
        best = d2;
        bk = k;
        bj = j;
      }
    }
  }
  // nearest point of the two polyline segments at that sample (samples are
  // far apart at small rho), and the segment's direction there
  const cx c0 = ca[bk * kCCLen + bj];
  const cx cp = ca[bk * kCCLen + (bj + 1) % kCCLen];
  const cx cm = ca[bk * kCCLen + (bj + kCCLen - 1) % kCCLen];
  double qx = c0.re, qy = c0.im, tx = cp.re - cm.re, ty = cp.im - cm.im;
  double dist = sqrt((src.re - c0.re) * (src.re - c0.re) + (src.im - c0.im) * (src.im - c0.im));
  for (int side = 0; side < 2; side++) {
    const cx e = side ? cp : cm;
    const double ex = e.re - c0.re, ey = e.im - c0.im;
    const double l2 = ex * ex + ey * ey;
    if (!(l2 > 0.0)) continue;
    const double u = fmin(fmax(((src.re - c0.re) * ex + (src.im - c0.im) * ey) / l2, 0.0), 1.0);
    const double px = c0.re + u * ex, py = c0.im + u * ey;
    const double dd = sqrt((src.re - px) * (src.re - px) + (src.im - py) * (src.im - py));
    if (dd < dist) {
      dist = dd;
      qx = px;
      qy = py;
      tx = ex;
      ty = ey;
    }
  }
  const double tn = sqrt(tx * tx + ty * ty);
  tx = tn > 0.0 ? tx / tn : 1.0;
  ty = tn > 0.0 ? ty / tn : 0.0;
  const double ox = src.re - qx, oy = src.im - qy;
  const double on = -ty * ox + tx * oy;   // normal component
  const double rho = D.rho;
  const double v = D.ld_b / (D.ld_a + D.ld_b);   // linear LD coefficient
  const double a_lens = L.z2.re, b_lens = sqrt(norm(L.z3));
  float* f = feat + (size_t)p * kIn;
  f[0] = (float)log10(fmax(a_lens, 1e-6));
  f[1] = (float)log10(fmax(b_lens, 1e-6));
  f[2] = (float)(b_lens > 0.0 ? L.z3.re / b_lens : 1.0);
  f[3] = (float)(b_lens > 0.0 ? L.z3.im / b_lens : 0.0);
  f[4] = (float)log10(fmax(L.m2, 1e-9));
  f[5] = (float)log10(fmax(L.m3, 1e-9));
  f[6] = (float)log10(rho);
  f[7] = (float)v;
  f[8] = (float)log10(fmax(a, 1e-3));
  f[9] = (float)ni / 10.f;
  f[10] = (float)fmin(fmax(log10(fmax(dist / rho, 1e-9)), -3.0), 6.0);
  f[11] = (float)(dist > 0.0 ? on / dist : 0.0);
  f[12] = (float)tanh(on / (3.0 * rho));
  f[13] = (float)log10(fmax(dist, 1e-12));
  aps[p] = a;
  dc_rho[p] = edge ? 0.f : (float)(dist / rho);
}

__global__ void caustic_points_kernel(int n, const int32_t* lens_idx, const int32_t* branch,
                                      const int32_t* index, const cx* ca_all, int nlens,
                                      double* xy) {
  const int p = blockIdx.x * blockDim.x + threadIdx.x;
  if (p >= n) return;
  int li = lens_idx[p], k = branch[p], j = index[p];
  li = li < 0 ? 0 : (li >= nlens ? nlens - 1 : li);
  k = k < 0 ? 0 : (k >= kBranches ? kBranches - 1 : k);
  j = j < 0 ? 0 : (j >= kCCLen ? kCCLen - 1 : j);
  const cx c = ca_all[((size_t)li * kBranches + k) * kCCLen + j];
  xy[2 * (size_t)p] = c.re;
  xy[2 * (size_t)p + 1] = c.im;
}

// ---------------------------------------------------------------------------
// BF16 GEMM on the tensor cores
// ---------------------------------------------------------------------------
enum Epi : int { kEpiFwd = 0, kEpiFwdInf = 1, kEpiAtomic = 2, kEpiBwdSilu = 3 };

__device__ __forceinline__ float silu_f(float z) { return z / (1.f + __expf(-z)); }
__device__ __forceinline__ float dsilu_f(float z) {
  const float s = 1.f / (1.f + __expf(-z));
  return s * (1.f + z * (1.f - s));
}

__device__ __forceinline__ void mma_bf16(float* d, const uint32_t* a, const uint32_t* b) {
  asm volatile(
      "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, "
      "{%8,%9}, {%0,%1,%2,%3};\n"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b[0]), "r"(b[1]));
}

constexpr int kBM = 64, kBN = 64, kBK = 32, kPitch = kBK + 8;

// Stages the 64 x 32 tile T(r, c) = P[(r0 + r) * s_r + (c0 + c) * s_c] (zero
// outside r < rmax, c < cmax) into S[r][c] with 128 threads.  16-byte loads
// along whichever direction is contiguous when the rows (or columns) are
// 16-byte aligned and the tile is whole in that direction; element loads
// otherwise.
__device__ __forceinline__ void stage_tile(uint16_t (*S)[kPitch], const uint16_t* P, long s_r,
                                           long s_c, int r0, int rmax, int c0, int cmax,
                                           int tid) {
  const bool aligned = ((uintptr_t)P & 15) == 0;
  if (aligned && s_c == 1 && (s_r & 7) == 0 && c0 + kBK <= cmax) {
    // 4 vectors per row along c
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int e = tid + i * 128;
      const int r = e >> 2, q = e & 3;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (r0 + r < rmax) v = *reinterpret_cast<const uint4*>(P + (long)(r0 + r) * s_r + c0 + q * 8);
      *reinterpret_cast<uint4*>(&S[r][q * 8]) = v;
    }
    return;
  }
  if (aligned && s_r == 1 && (s_c & 7) == 0 && r0 + kBM <= rmax) {
    // 8 vectors per column along r, scattered into the rows
#pragma unroll
    for (int i = 0; i < 2; i++) {
      const int e = tid + i * 128;
      const int c = e >> 3, q = e & 7;
      uint4 v = make_uint4(0, 0, 0, 0);
      if (c0 + c < cmax) v = *reinterpret_cast<const uint4*>(P + (long)(c0 + c) * s_c + r0 + q * 8);
      const uint32_t w[4] = {v.x, v.y, v.z, v.w};
#pragma unroll
      for (int j = 0; j < 4; j++) {
        S[q * 8 + 2 * j][c] = (uint16_t)(w[j] & 0xffffu);
        S[q * 8 + 2 * j + 1][c] = (uint16_t)(w[j] >> 16);
      }
    }
    return;
  }
  for (int e = tid; e < kBM * kBK; e += 128) {
    int r, c;
    if (s_c == 1) { r = e / kBK; c = e % kBK; } else { c = e / kBM; r = e % kBM; }
    const int m = r0 + r, k = c0 + c;
    S[r][c] = (m < rmax && k < cmax) ? P[(long)m * s_r + (long)k * s_c] : (uint16_t)0;
  }
}

// C[m][n] = sum_k A(m,k) B(k,n), A(m,k) = A[m*a_sm + k*a_sk], B(k,n) =
// B[k*b_sk + n*b_sn]; blockIdx.z splits k into chunks of k_split.
template <int EPI>
__global__ void __launch_bounds__(128)
gemm_bf16_kernel(int M, int N, int K, const __nv_bfloat16* A, long a_sm, long a_sk,
                 const __nv_bfloat16* B, long b_sk, long b_sn, const float* bias,
                 __nv_bfloat16* out0, __nv_bfloat16* out1, float* outf, long ldo,
                 const __nv_bfloat16* zprev, long ldz, int k_split) {
  __shared__ __align__(16) uint16_t As[kBM][kPitch];   // [m][k]
  __shared__ __align__(16) uint16_t Bs[kBN][kPitch];   // [n][k]
  const int m0 = blockIdx.y * kBM, n0 = blockIdx.x * kBN;
  const int kbeg = blockIdx.z * k_split;
  const int kend = min(K, kbeg + k_split);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const int wm = (warp >> 1) * 32, wn = (warp & 1) * 32;
  const int g = lane >> 2, t = lane & 3;
  const uint16_t* Au = reinterpret_cast<const uint16_t*>(A);
  const uint16_t* Bu = reinterpret_cast<const uint16_t*>(B);
  float acc[2][4][4];
#pragma unroll
  for (int i = 0; i < 2; i++)
#pragma unroll
    for (int j = 0; j < 4; j++)
#pragma unroll
      for (int q = 0; q < 4; q++) acc[i][j][q] = 0.f;

  for (int k0 = kbeg; k0 < kend; k0 += kBK) {
    stage_tile(As, Au, a_sm, a_sk, m0, M, k0, kend, tid);
    stage_tile(Bs, Bu, b_sn, b_sk, n0, N, k0, kend, tid);
    __syncthreads();
#pragma unroll
    for (int kk = 0; kk < kBK; kk += 16) {
      uint32_t af[2][4], bfr[4][2];
#pragma unroll
      for (int i = 0; i < 2; i++) {
        const int row = wm + i * 16 + g;
        af[i][0] = *reinterpret_cast<const uint32_t*>(&As[row][kk + 2 * t]);
        af[i][1] = *reinterpret_cast<const uint32_t*>(&As[row + 8][kk + 2 * t]);
        af[i][2] = *reinterpret_cast<const uint32_t*>(&As[row][kk + 2 * t + 8]);
        af[i][3] = *reinterpret_cast<const uint32_t*>(&As[row + 8][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int j = 0; j < 4; j++) {
        const int col = wn + j * 8 + g;
        bfr[j][0] = *reinterpret_cast<const uint32_t*>(&Bs[col][kk + 2 * t]);
        bfr[j][1] = *reinterpret_cast<const uint32_t*>(&Bs[col][kk + 2 * t + 8]);
      }
#pragma unroll
      for (int i = 0; i < 2; i++)
#pragma unroll
        for (int j = 0; j < 4; j++) mma_bf16(acc[i][j], af[i], bfr[j]);
    }
    __syncthreads();
  }
  // epilogue: acc[i][j] = rows (g, g+8), columns (2t, 2t+1) of an m16n8 tile
#pragma unroll
  for (int i = 0; i < 2; i++) {
#pragma unroll
    for (int j = 0; j < 4; j++) {
#pragma unroll
      for (int q = 0; q < 4; q++) {
        const int r = m0 + wm + i * 16 + g + (q >= 2 ? 8 : 0);
        const int c = n0 + wn + j * 8 + 2 * t + (q & 1);
        if (r >= M || c >= N) continue;
        const float v = acc[i][j][q];
        const long o = (long)r * ldo + c;
        if (EPI == kEpiFwd || EPI == kEpiFwdInf) {
          const float z = v + bias[c];
          if (EPI == kEpiFwd) out0[o] = __float2bfloat16_rn(z);
          out1[o] = __float2bfloat16_rn(silu_f(z));
        } else if (EPI == kEpiAtomic) {
          atomicAdd(&outf[o], v);
        } else {  // dZ_prev = dH_prev * silu'(Z_prev)
          const float z = __bfloat162float(zprev[(long)r * ldz + c]);
          out0[o] = __float2bfloat16_rn(v * dsilu_f(z));
        }
      }
    }
  }
}

template <int EPI>
void gemm(int M, int N, int K, const __nv_bfloat16* A, long a_sm, long a_sk,
          const __nv_bfloat16* B, long b_sk, long b_sn, const float* bias, __nv_bfloat16* out0,
          __nv_bfloat16* out1, float* outf, long ldo, const __nv_bfloat16* zprev, long ldz,
          int splits, cudaStream_t st) {
  int k_split = (K + splits - 1) / splits;
  k_split = (k_split + kBK - 1) / kBK * kBK;
  splits = (K + k_split - 1) / k_split;
  dim3 grid((N + kBN - 1) / kBN, (M + kBM - 1) / kBM, splits);
  gemm_bf16_kernel<EPI><<<grid, 128, 0, st>>>(M, N, K, A, a_sm, a_sk, B, b_sk, b_sn, bias, out0,
                                              out1, outf, ldo, zprev, ldz, k_split);
}

// ---------------------------------------------------------------------------
// elementwise and small kernels
// ---------------------------------------------------------------------------
// normalised features -> BF16 input rows (16 wide, zero padded)
__global__ void input_kernel(int M, const float* feat, const float* mean, const float* inv_std,
                             __nv_bfloat16* x) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * kInPad) return;
  const int m = i / kInPad, c = i % kInPad;
  float v = 0.f;
  if (c < kIn) v = (feat[(size_t)m * kIn + c] - mean[c]) * inv_std[c];
  x[i] = __float2bfloat16_rn(v);
}

// y = H4 w5 + b5 (warp per row); training: loss, dy, dZ4 = dy w5 silu'(Z4),
// dw5 and db5 (block sums, one atomic per block)
__global__ void __launch_bounds__(256)
out_layer_kernel(int M, const __nv_bfloat16* H4, const __nv_bfloat16* Z4, const float* w5,
                 const float* b5, const float* target, float* y, __nv_bfloat16* dZ4, float* gw5,
                 float* gb5, float* loss) {
  __shared__ float s_gw[kW];
  __shared__ float s_gb, s_loss;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const bool train = target != nullptr;
  if (train) {
    for (int k = threadIdx.x; k < kW; k += blockDim.x) s_gw[k] = 0.f;
    if (threadIdx.x == 0) s_gb = s_loss = 0.f;
    __syncthreads();
  }
  const int rows_per_block = 8 * 4;
  for (int rr = 0; rr < 4; rr++) {
    const int m = blockIdx.x * rows_per_block + warp * 4 + rr;
    if (m >= M) break;
    float h[8], s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; q++) {
      const int k = lane * 8 + q;
      h[q] = __bfloat162float(H4[(size_t)m * kW + k]);
      s += h[q] * w5[k];
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
    const float yv = s + b5[0];
    if (lane == 0) y[m] = yv;
    if (train) {
      const float diff = yv - target[m];
      const float dy = 2.f * diff / (float)M;
#pragma unroll
      for (int q = 0; q < 8; q++) {
        const int k = lane * 8 + q;
        const float z = __bfloat162float(Z4[(size_t)m * kW + k]);
        dZ4[(size_t)m * kW + k] = __float2bfloat16_rn(dy * w5[k] * dsilu_f(z));
        atomicAdd(&s_gw[k], dy * h[q]);
      }
      if (lane == 0) {
        atomicAdd(&s_gb, dy);
        atomicAdd(&s_loss, diff * diff / (float)M);
      }
    }
  }
  if (train) {
    __syncthreads();
    for (int k = threadIdx.x; k < kW; k += blockDim.x) atomicAdd(&gw5[k], s_gw[k]);
    if (threadIdx.x == 0) {
      atomicAdd(gb5, s_gb);
      atomicAdd(loss, s_loss);
    }
  }
}

// db[n] = sum_m dZ[m][n]
__global__ void bias_grad_kernel(int M, const __nv_bfloat16* dZ, float* gb) {
  const int c = threadIdx.x;   // 256 threads, one column each
  const int r0 = blockIdx.x * 64;
  float s = 0.f;
  for (int r = r0; r < min(M, r0 + 64); r++) s += __bfloat162float(dZ[(size_t)r * kW + c]);
  atomicAdd(&gb[c], s);
}

__global__ void adam_kernel(int n, float* p, const float* g, float* m1, float* m2,
                            __nv_bfloat16* pb, float lr, float b1, float b2, float eps,
                            float c1, float c2) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float gi = g[i];
  const float a = b1 * m1[i] + (1.f - b1) * gi;
  const float b = b2 * m2[i] + (1.f - b2) * gi * gi;
  m1[i] = a;
  m2[i] = b;
  const float v = p[i] - lr * (a / c1) / (sqrtf(b / c2) + eps);
  p[i] = v;
  pb[i] = __float2bfloat16_rn(v);
}

__global__ void to_bf16_kernel(int n, const float* p, __nv_bfloat16* pb) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) pb[i] = __float2bfloat16_rn(p[i]);
}

// ensemble mean/std of y, gating, magnification of the points the surrogate
// keeps
__global__ void gate_kernel(int M, int members, const float* ys, long ys_stride,
                            const double* aps, const float* dc_rho, float max_std,
                            float min_dc_rho, float far_dc_rho, float* mean, float* stdv,
                            double* mag, int32_t* gated) {
  const int m = blockIdx.x * blockDim.x + threadIdx.x;
  if (m >= M) return;
  float s = 0.f, s2 = 0.f;
  for (int k = 0; k < members; k++) {
    const float v = ys[(size_t)k * ys_stride + m];
    s += v;
    s2 += v * v;
  }
  const float mu0 = s / members;
  const float var = fmaxf(0.f, s2 / members - mu0 * mu0);
  const float sd = sqrtf(var);
  // shrink a correction the members do not resolve towards 0 (A_point)
  const float snr2 = mu0 * mu0 / fmaxf(var, 1e-30f);
  const bool far = dc_rho[m] >= far_dc_rho;   // A_point alone suffices there
  const float mu = (far || snr2 <= 1.f) ? 0.f : mu0 * (1.f - 1.f / snr2);
  mean[m] = mu;
  stdv[m] = sd;
  const bool g = (!(sd <= max_std) && !far) || !(dc_rho[m] >= min_dc_rho) || !isfinite(aps[m]);
  gated[m] = g ? 1 : 0;
  mag[m] = g ? 0.0 : aps[m] * exp((double)mu);
}

}  // namespace sur
}  // namespace tl

using namespace tl;
using namespace tl::sur;

struct tls_model {
  int members = 0;
  std::vector<float*> p, g, m1, m2;          // FP32 master, gradients, Adam moments
  std::vector<__nv_bfloat16*> pb;           // BF16 mirror
  float* mean = nullptr;                     // feature normalisation (14 + 14 floats)
  float* inv_std = nullptr;
  std::vector<int> steps;
  // activations for up to cap rows
  int cap = 0;
  __nv_bfloat16 *x = nullptr, *Z[kHidden] = {}, *H[kHidden] = {}, *dA = nullptr, *dB = nullptr;
  float *y = nullptr, *loss = nullptr;
  float* ys = nullptr;   // members x cap predictions
};

namespace {

bool ok(cudaError_t e, const char* what) {
  if (e != cudaSuccess) {
    fprintf(stderr, "tls: %s: %s\n", what, cudaGetErrorString(e));
    return false;
  }
  return true;
}

bool ensure_rows(tls_model* s, int M) {
  if (M <= s->cap) return true;
  int cap = 1024;
  while (cap < M) cap *= 2;
  auto fr = [](void* q) { if (q) cudaFree(q); };
  fr(s->x);
  for (int l = 0; l < kHidden; l++) {
    fr(s->Z[l]);
    fr(s->H[l]);
  }
  fr(s->dA);
  fr(s->dB);
  fr(s->y);
  fr(s->ys);
  bool good = ok(cudaMalloc(&s->x, sizeof(__nv_bfloat16) * (size_t)cap * kInPad), "alloc x");
  for (int l = 0; l < kHidden; l++) {
    good = good && ok(cudaMalloc(&s->Z[l], sizeof(__nv_bfloat16) * (size_t)cap * kW), "alloc Z");
    good = good && ok(cudaMalloc(&s->H[l], sizeof(__nv_bfloat16) * (size_t)cap * kW), "alloc H");
  }
  good = good && ok(cudaMalloc(&s->dA, sizeof(__nv_bfloat16) * (size_t)cap * kW), "alloc dA");
  good = good && ok(cudaMalloc(&s->dB, sizeof(__nv_bfloat16) * (size_t)cap * kW), "alloc dB");
  good = good && ok(cudaMalloc(&s->y, sizeof(float) * (size_t)cap), "alloc y");
  good = good && ok(cudaMalloc(&s->ys, sizeof(float) * (size_t)cap * s->members), "alloc ys");
  s->cap = good ? cap : 0;
  return good;
}

cudaStream_t stream_of(void* st) { return (cudaStream_t)st; }

// forward pass of one member over M rows of features; keep = store Z
void forward(tls_model* s, int k, int M, const float* feat, bool keep, cudaStream_t st) {
  input_kernel<<<(M * kInPad + 255) / 256, 256, 0, st>>>(M, feat, s->mean, s->inv_std, s->x);
  const float* P = s->p[k];
  const __nv_bfloat16* PB = s->pb[k];
  const __nv_bfloat16* in = s->x;
  int kin = kInPad;
  for (int l = 1; l <= kHidden; l++) {
    const __nv_bfloat16* W = PB + off_w(l);   // [256][kin]
    const float* b = P + off_b(l);
    if (keep)
      gemm<kEpiFwd>(M, kW, kin, in, kin, 1, W, 1, kin, b, s->Z[l - 1], s->H[l - 1], nullptr, kW,
                    nullptr, 0, 1, st);
    else
      gemm<kEpiFwdInf>(M, kW, kin, in, kin, 1, W, 1, kin, b, nullptr, s->H[l - 1], nullptr, kW,
                       nullptr, 0, 1, st);
    in = s->H[l - 1];
    kin = kW;
  }
}

// gradients of one member into s->g[k] (zeroed here); returns nothing, loss in s->loss
void backward(tls_model* s, int k, int M, const float* feat, const float* target,
              cudaStream_t st) {
  float* G = s->g[k];
  const float* P = s->p[k];
  const __nv_bfloat16* PB = s->pb[k];
  cudaMemsetAsync(G, 0, sizeof(float) * kParams, st);
  cudaMemsetAsync(s->loss, 0, sizeof(float), st);
  forward(s, k, M, feat, true, st);
  out_layer_kernel<<<(M + 31) / 32, 256, 0, st>>>(M, s->H[kHidden - 1], s->Z[kHidden - 1],
                                                 P + kOffW5, P + kOffB5, target, s->y, s->dA,
                                                 G + kOffW5, G + kOffB5, s->loss);
  __nv_bfloat16* dz = s->dA;   // dZ of layer l
  __nv_bfloat16* dn = s->dB;
  const int splits = M >= 8192 ? 32 : (M >= 1024 ? 8 : 1);
  for (int l = kHidden; l >= 1; l--) {
    const int kin = l == 1 ? kInPad : kW;
    const __nv_bfloat16* Xin = l == 1 ? s->x : s->H[l - 2];
    // dW_l[n][kk] = sum_m dZ[m][n] X[m][kk]
    gemm<kEpiAtomic>(kW, kin, M, dz, 1, kW, Xin, kin, 1, nullptr, nullptr, nullptr, G + off_w(l),
                     kin, nullptr, 0, splits, st);
    bias_grad_kernel<<<(M + 63) / 64, kW, 0, st>>>(M, dz, G + off_b(l));
    if (l > 1) {
      // dZ_{l-1}[m][kk] = (sum_n dZ[m][n] W_l[n][kk]) silu'(Z_{l-1}[m][kk])
      gemm<kEpiBwdSilu>(M, kW, kW, dz, kW, 1, PB + off_w(l), kW, 1, nullptr, dn, nullptr, nullptr,
                        kW, s->Z[l - 2], kW, 1, st);
      __nv_bfloat16* t = dz;
      dz = dn;
      dn = t;
    }
  }
}

}  // namespace

extern "C" {

int tls_param_count(void) { return (int)kParams; }

tls_model* tls_new(int members) {
  if (members <= 0 || members > 16) return nullptr;
  tl::Engine::get();
  tls_model* s = new tls_model();
  s->members = members;
  bool good = true;
  for (int k = 0; k < members; k++) {
    float *p = nullptr, *g = nullptr, *a = nullptr, *b = nullptr;
    __nv_bfloat16* pb = nullptr;
    good = good && ok(cudaMalloc(&p, sizeof(float) * kParams), "alloc params");
    good = good && ok(cudaMalloc(&g, sizeof(float) * kParams), "alloc grads");
    good = good && ok(cudaMalloc(&a, sizeof(float) * kParams), "alloc m1");
    good = good && ok(cudaMalloc(&b, sizeof(float) * kParams), "alloc m2");
    good = good && ok(cudaMalloc(&pb, sizeof(__nv_bfloat16) * kParams), "alloc bf16 params");
    s->p.push_back(p);
    s->g.push_back(g);
    s->m1.push_back(a);
    s->m2.push_back(b);
    s->pb.push_back(pb);
    s->steps.push_back(0);
    if (good) {
      cudaMemset(p, 0, sizeof(float) * kParams);
      cudaMemset(a, 0, sizeof(float) * kParams);
      cudaMemset(b, 0, sizeof(float) * kParams);
      cudaMemset(pb, 0, sizeof(__nv_bfloat16) * kParams);
    }
  }
  good = good && ok(cudaMalloc(&s->mean, sizeof(float) * 2 * kIn), "alloc norm");
  good = good && ok(cudaMalloc(&s->loss, sizeof(float)), "alloc loss");
  if (good) {
    s->inv_std = s->mean + kIn;
    std::vector<float> h(2 * kIn, 0.f);
    for (int c = 0; c < kIn; c++) h[kIn + c] = 1.f;
    cudaMemcpy(s->mean, h.data(), sizeof(float) * 2 * kIn, cudaMemcpyHostToDevice);
  }
  if (!good) {
    tls_delete(s);
    return nullptr;
  }
  return s;
}

void tls_delete(tls_model* s) {
  if (!s) return;
  for (int k = 0; k < (int)s->p.size(); k++) {
    cudaFree(s->p[k]);
    cudaFree(s->g[k]);
    cudaFree(s->m1[k]);
    cudaFree(s->m2[k]);
    cudaFree(s->pb[k]);
  }
  cudaFree(s->mean);
  cudaFree(s->loss);
  cudaFree(s->x);
  for (int l = 0; l < kHidden; l++) {
    cudaFree(s->Z[l]);
    cudaFree(s->H[l]);
  }
  cudaFree(s->dA);
  cudaFree(s->dB);
  cudaFree(s->y);
  cudaFree(s->ys);
  delete s;
}

int tls_set_params(tls_model* s, int member, const float* host) {
  if (!s || member < 0 || member >= s->members || !host) return -1;
  if (!ok(cudaMemcpy(s->p[member], host, sizeof(float) * kParams, cudaMemcpyHostToDevice),
          "set params"))
    return -2;
  to_bf16_kernel<<<(int)((kParams + 255) / 256), 256>>>((int)kParams, s->p[member], s->pb[member]);
  cudaMemset(s->m1[member], 0, sizeof(float) * kParams);
  cudaMemset(s->m2[member], 0, sizeof(float) * kParams);
  s->steps[member] = 0;
  return ok(cudaDeviceSynchronize(), "set params") ? 0 : -2;
}

int tls_get_params(tls_model* s, int member, float* host) {
  if (!s || member < 0 || member >= s->members || !host) return -1;
  return ok(cudaMemcpy(host, s->p[member], sizeof(float) * kParams, cudaMemcpyDeviceToHost),
            "get params")
             ? 0
             : -2;
}

int tls_set_normalisation(tls_model* s, const float* mean14, const float* std14) {
  if (!s || !mean14 || !std14) return -1;
  std::vector<float> h(2 * kIn);
  for (int c = 0; c < kIn; c++) {
    h[c] = mean14[c];
    h[kIn + c] = std14[c] > 0.f ? 1.f / std14[c] : 1.f;
  }
  return ok(cudaMemcpy(s->mean, h.data(), sizeof(float) * 2 * kIn, cudaMemcpyHostToDevice),
            "set normalisation")
             ? 0
             : -2;
}

int tls_train_step(tls_model* s, int member, int M, const float* feat, const float* target,
                   float lr, float* loss_out, void* stream) {
  if (!s || member < 0 || member >= s->members || M <= 0 || !feat || !target) return -1;
  if (!ensure_rows(s, M)) return -2;
  cudaStream_t st = stream_of(stream);
  backward(s, member, M, feat, target, st);
  const int t = ++s->steps[member];
  const float b1 = 0.9f, b2 = 0.999f;
  const float c1 = 1.f - powf(b1, (float)t), c2 = 1.f - powf(b2, (float)t);
  adam_kernel<<<(int)((kParams + 255) / 256), 256, 0, st>>>(
      (int)kParams, s->p[member], s->g[member], s->m1[member], s->m2[member], s->pb[member], lr, b1,
      b2, 1e-8f, c1, c2);
  if (loss_out) cudaMemcpyAsync(loss_out, s->loss, sizeof(float), cudaMemcpyDeviceToDevice, st);
  return ok(cudaGetLastError(), "train step") ? 0 : -2;
}

int tls_gradients(tls_model* s, int member, int M, const float* feat, const float* target,
                  float* host_grads, float* host_loss) {
  if (!s || member < 0 || member >= s->members || M <= 0 || !feat || !target || !host_grads)
    return -1;
  if (!ensure_rows(s, M)) return -2;
  backward(s, member, M, feat, target, 0);
  if (!ok(cudaMemcpy(host_grads, s->g[member], sizeof(float) * kParams, cudaMemcpyDeviceToHost),
          "gradients"))
    return -2;
  if (host_loss) cudaMemcpy(host_loss, s->loss, sizeof(float), cudaMemcpyDeviceToHost);
  return 0;
}

int tls_forward(tls_model* s, int member, int M, const float* feat, float* y, void* stream) {
  if (!s || member < 0 || member >= s->members || M <= 0 || !feat || !y) return -1;
  if (!ensure_rows(s, M)) return -2;
  cudaStream_t st = stream_of(stream);
  forward(s, member, M, feat, false, st);
  out_layer_kernel<<<(M + 31) / 32, 256, 0, st>>>(M, s->H[kHidden - 1], nullptr,
                                                 s->p[member] + kOffW5, s->p[member] + kOffB5,
                                                 nullptr, y, nullptr, nullptr, nullptr, nullptr);
  return ok(cudaGetLastError(), "forward") ? 0 : -2;
}

int tls_predict(tls_model* s, int M, const float* feat, const double* aps, const float* dc_rho,
                float max_std, float min_dc_rho, float far_dc_rho, float* mean, float* stdv,
                double* mag, int32_t* gated, void* stream) {
  if (!s || M <= 0 || !feat || !aps || !dc_rho || !mean || !stdv || !mag || !gated) return -1;
  if (!ensure_rows(s, M)) return -2;
  cudaStream_t st = stream_of(stream);
  for (int k = 0; k < s->members; k++) {
    forward(s, k, M, feat, false, st);
    out_layer_kernel<<<(M + 31) / 32, 256, 0, st>>>(M, s->H[kHidden - 1], nullptr,
                                                   s->p[k] + kOffW5, s->p[k] + kOffB5, nullptr,
                                                   s->ys + (size_t)k * s->cap, nullptr, nullptr,
                                                   nullptr, nullptr);
  }
  gate_kernel<<<(M + 255) / 256, 256, 0, st>>>(M, s->members, s->ys, s->cap, aps, dc_rho, max_std,
                                               min_dc_rho, far_dc_rho, mean, stdv, mag, gated);
  return ok(cudaGetLastError(), "predict") ? 0 : -2;
}

int tls_features(tl_batch* b, int M, const double* xy, const int32_t* lens_idx, float* feat,
                 double* aps, float* dc_rho, void* stream) {
  if (!b || b->nlens <= 0 || M <= 0 || !xy || !lens_idx || !feat || !aps || !dc_rho) return -1;
  if (!upload_trig()) return -2;
  cudaStream_t st = stream_of(stream);
  features_kernel<<<(M + 63) / 64, 64, 0, st>>>(M, xy, lens_idx, (const DevLens*)b->lenses.p,
                                                (const cx*)b->ca.p, feat, aps, dc_rho);
  return ok(cudaGetLastError(), "features") ? 0 : -2;
}

int tlb_caustic_points(tl_batch* b, int n, const int32_t* lens_idx, const int32_t* branch,
                       const int32_t* index, double* xy, void* stream) {
  if (!b || b->nlens <= 0 || n <= 0 || !lens_idx || !branch || !index || !xy) return -1;
  cudaStream_t st = stream_of(stream);
  caustic_points_kernel<<<(n + 255) / 256, 256, 0, st>>>(n, lens_idx, branch, index,
                                                         (const cx*)b->ca.p, b->nlens, xy);
  return ok(cudaGetLastError(), "caustic points") ? 0 : -2;
}

}  // extern "C"
