// noalloc_abi.cu - lcirs_fill_device_noalloc: the amoeba fill of an existing
// lens object on caller-provided device arrays, with every scratch byte taken
// from one static device array instead of cudaMalloc.
//
// Who needs it: programs that cannot allocate device memory at the time they
// compute magnifications.  A host application that reserves (nearly) all of
// the GPU's memory for its own pool at start-up sees cudaMalloc fail or
// bypass its accounting; a latency-bound loop cannot take the device-wide
// synchronisation that cudaFree (and often cudaMalloc) performs, which would
// also stall every other stream of the process.  The other entry points grow
// their buffers with cudaMalloc on demand; this one allocates nothing.
//
// Limits: at most kMaxPoints points per call, and a block table of
// 2^kCapLog2 blocks of 32 x 32 rays per point (about 16.8 million rays around
// the images, 3/4 of it usable: magnifications up to ~100 at 200 rays per
// source radius, ~15 at 500).  kCtas fill CTAs work on one point each at a
// time.  A point whose images need more comes back with status bit 4 (table
// full) and an incomplete magnification; the allocating entry points retry
// such points with larger tables, this one cannot.
#include <cuda_runtime.h>

#include <cstdio>
#include <mutex>

#include "engine.h"
#include "engine_host.h"
#include "lcirs.hpp"

namespace {

constexpr int kMaxPoints = LCIRS_NOALLOC_MAX_POINTS;
constexpr int kCtas = 8;         // fill CTAs (each owns one block table)
constexpr int kCapLog2 = 14;     // blocks per CTA table (log2)
constexpr int kBlockH = 32;      // rows per block
constexpr int kThreads = 256;
constexpr int kMaxDevices = 64;

constexpr size_t align256(size_t b) { return (b + 255) / 256 * 256; }
constexpr size_t kPointsOff = 0;
constexpr size_t kOutOff = align256(kPointsOff + sizeof(tl::PointIn) * kMaxPoints);
constexpr size_t kFillOff = align256(kOutOff + sizeof(tl::PointOut) * kMaxPoints);
// 80 MiB: the point arrays (576 KiB) and the fill tables (70.4 MiB: 8 CTAs x
// (16384 block records of 528 bytes + 4096 super-tile entries of 140 bytes)),
// checked against fill_scratch_bytes() at set-up
constexpr size_t kScratchBytes = (size_t)80 << 20;

// The one scratch array.  Every GPU that loads this file's device code holds
// it until the process exits; all calls on a device share it.
static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

std::mutex g_mu;
char* g_base[kMaxDevices] = {};   // device address of the array, per device

// the array's device address on the current device; the first call on a
// device looks it up (this loads the file's device code there)
char* scratch_base(int* err) {
  int dev = -1;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
    fprintf(stderr, "lcirs_fill_device_noalloc: no usable current device (%s)\n",
            cudaGetErrorString(e));
    *err = -2;
    return nullptr;
  }
  std::lock_guard<std::mutex> g(g_mu);
  if (!g_base[dev]) {
    if (tl::fill_scratch_bytes(kCtas, kCapLog2, kBlockH) > kScratchBytes - kFillOff) {
      fprintf(stderr, "lcirs_fill_device_noalloc: fill tables exceed the static scratch\n");
      *err = -2;
      return nullptr;
    }
    void* p = nullptr;
    e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      fprintf(stderr, "lcirs_fill_device_noalloc: cudaGetSymbolAddress failed on device %d: %s\n",
              dev, cudaGetErrorString(e));
      *err = -2;
      return nullptr;
    }
    g_base[dev] = (char*)p;
  }
  return g_base[dev];
}

// caller's positions and seed counts -> the fill kernel's point records
__global__ void noalloc_pack_kernel(int npoints, const double* xy, const int32_t* nseeds,
                                    tl::PointIn* points, tl::PointOut* out) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npoints) return;
  const double x = xy[2 * (size_t)i], y = xy[2 * (size_t)i + 1];
  tl::PointIn p;
  p.sx = x;
  p.sy = y;
  p.lens = 0;
  p.est_blocks = 0;
  points[i] = p;
  tl::PointOut o;
  o.count = 0;
  o.wsum_fx = 0;
  o.status = (isfinite(x) && isfinite(y)) ? 0u : (uint32_t)tl::kStBadInput;
  const int32_t n = nseeds[i];
  o.nseeds = (uint32_t)(n < 0 ? 0 : (n > tl::kMaxSeeds ? tl::kMaxSeeds : n));
  o.tiles = 0;
  o.diag = 0;
  o.rays_eval = 0;
  o.rays_fp64 = 0;
  out[i] = o;
}

// point records -> caller's magnifications, counts and status words
__global__ void noalloc_unpack_kernel(int npoints, const tl::PointOut* out, double amp_scale,
                                      double* mag, uint64_t* counts, uint32_t* status) {
  const int i = blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= npoints) return;
  const tl::PointOut o = out[i];
  mag[i] = ((double)o.wsum_fx / tl::kWsumScale) * amp_scale;
  if (counts) counts[i] = o.count;
  if (status) status[i] = o.status;
}

}  // namespace

extern "C" int lcirs_fill_device_noalloc(LightCurveIRS* lc, int npoints, const double* src_xy,
                                         const int32_t* seeds, const int32_t* nseeds,
                                         double* mag, uint64_t* counts, uint32_t* status,
                                         void* stream) {
  if (!lc || npoints <= 0 || !src_xy || !seeds || !nseeds || !mag) return -1;
  if (npoints > kMaxPoints) {
    fprintf(stderr,
            "lcirs_fill_device_noalloc: %d points exceed the static scratch's maximum of %d "
            "points per call; split the call\n",
            npoints, kMaxPoints);
    return -3;
  }
  // the object's lens lives on the device it was created on; launching on
  // another device would read foreign addresses
  int cur = -1;
  if (cudaGetDevice(&cur) != cudaSuccess) return -2;
  if (tl::object_device(lc) != cur) {
    fprintf(stderr,
            "lcirs_fill_device_noalloc: the object lives on device %d, the current device is "
            "%d\n",
            tl::object_device(lc), cur);
    return -1;
  }
  int err = 0;
  char* base = scratch_base(&err);
  if (!base) return err;
  const cudaStream_t st = (cudaStream_t)stream;
  tl::PointIn* points = (tl::PointIn*)(base + kPointsOff);
  tl::PointOut* out = (tl::PointOut*)(base + kOutOff);
  // the tables keep the previous call's contents: clear them (memsets on the
  // stream, no allocation)
  tl::FillScratch fs;
  tl::fill_scratch_init(&fs, base + kFillOff, kCtas, kCapLog2, kBlockH, st);
  const int grid = (npoints + 255) / 256;
  noalloc_pack_kernel<<<grid, 256, 0, st>>>(npoints, src_xy, nseeds, points, out);
  tl::launch_fill(points, npoints, tl::object_device_lens(lc), seeds, out, fs, lc->precision,
                  kThreads, st);
  noalloc_unpack_kernel<<<grid, 256, 0, st>>>(npoints, out, lc->grid[6], mag, counts, status);
  const cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) {
    fprintf(stderr, "lcirs_fill_device_noalloc: %s\n", cudaGetErrorString(e));
    return -2;
  }
  return 0;
}
