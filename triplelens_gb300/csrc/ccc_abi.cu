// ccc_abi.cu - libccc.so: critical curves and caustics behind the reference's
// ccc_* C ABI (src/CCC/ccc.cc:244-348, bound by Examples/ctypes_classes.py:
// 13-75), computed on the GPU.
//
// Compiled with --fmad=false, like seeds.cu: every FP64 operation is a
// separately rounded IEEE operation.
//
//   ccc_kernel  one warp per object: the phase samples phi_j = 2 pi j / L
//               (pi as 3.14159265359, ccc.cc:57) walked in order; sample 0
//               solved cold, every later sample polished from the previous
//               roots (one root per lane) and re-solved when checkRoots
//               fails, so the branches keep the reference's continuation;
//               then the caustic of every critical-curve point.
//               Triple lens: degree-6 polynomial (ccc.cc:42-98).  m3 == 0:
//               the binary degree-4 polynomial with the origin shifted to
//               the first lens (ccc.cc:101-158) and the binary caustic map
//               (ccc.cc:176-196).
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>
#include <string>
#include <vector>

#include "ccc.h"
#include "tl_math.h"

using tl::cx;

namespace {

__constant__ tl::TrigTable k_trig;
constexpr int kMaxOff = 256;   // phase samples whose polish failed, recorded

struct CccSpec {
  tl::Lens L;
  double a;
  int cc_binary;   // critical curve from the binary degree-4 polynomial
  int deg;         // critical-curve branches (4 or 6)
  int ca_binary;   // binary caustic map (ccc.cc:186-189)
  int ca_branches; // caustic branches (the reference's _polOrder)
  int len;
  int do_cc;       // 0: the critical curve is already in cc
};

// binary critical-curve coefficients (ccc.cc:118-124)
__device__ void bin_poly(double a, double m, cx e, cx* c) {
  c[4] = tl::mk(1.0, 0.0);
  c[3] = tl::mk(0.0, 0.0);
  c[2] = tl::sub(tl::neg(e), tl::mk(a * a / 2.0, 0.0));
  c[1] = tl::scale(tl::scale(e, a), 2.0 * m - 1.0);
  const cx t = tl::sub(tl::mk(a * a, 0.0), tl::scale(e, 4.0));
  c[0] = tl::scale(tl::scale(t, a * a), 1.0 / 16.0);
}

__global__ void ccc_kernel(CccSpec sp, const double* pc, const double* ps, cx* cc, cx* ca,
                           int* roots_off) {
  __shared__ cx s_roots[8];
  const int lane = threadIdx.x & 31;
  const int deg = sp.deg, len = sp.len;
  const double m = 1.0 - sp.L.m2 - sp.L.m3;
  cx root = tl::mk(0.0, 0.0);
  for (int j = 0; sp.do_cc && j < len; j++) {
    cx c[7];
    const cx e = tl::mk(pc[j], ps[j]);
    if (sp.cc_binary)
      bin_poly(sp.a, m, e, c);
    else
      tl::cc_poly(sp.L, e, c);
    if (j == 0) {
      if (lane == 0) {
        cx r[6];
        tl::solve_roots(c, deg, nullptr, r, &k_trig);
        for (int k = 0; k < deg; k++) s_roots[k] = r[k];
      }
    } else {
      if (lane < deg) {
        tl::laguerre(c, deg, &root, &k_trig);   // polishRoots: each root on its own
        s_roots[lane] = root;
      }
      __syncwarp();
      if (lane == 0) {
        cx r[6];
        for (int k = 0; k < deg; k++) r[k] = s_roots[k];
        if (!tl::check_roots(c, deg, r)) {
          // recorded for the reference's "Roots off for j = ..." line
          const int n_off = roots_off[0]++;
          if (n_off < kMaxOff) roots_off[1 + n_off] = j;
          tl::solve_roots(c, deg, nullptr, r, &k_trig);
          for (int k = 0; k < deg; k++) s_roots[k] = r[k];
        }
      }
    }
    __syncwarp();
    if (lane < deg) {
      root = s_roots[lane];
      // binary: origin shifted to z1 (ccc.cc:152)
      cc[lane * len + j] = sp.cc_binary ? tl::add(root, tl::mk(sp.a / 2.0, 0.0)) : root;
    }
    __syncwarp();
  }
  __syncwarp();
  for (int i = lane; i < sp.ca_branches * len; i += 32) {
    const cx s = cc[i];
    if (sp.ca_binary) {
      cx t = tl::sub(s, tl::rdiv(m, tl::conj(s)));
      t = tl::sub(t, tl::rdiv(sp.L.m2, tl::conj(tl::sub(s, tl::mk(sp.a, 0.0)))));
      ca[i] = t;
    } else {
      ca[i] = tl::caustic_point(sp.L, s);
    }
  }
}

bool g_trig_ok = false;

bool upload_trig() {
  if (g_trig_ok) return true;
  tl::TrigTable t;
  for (int i = 0; i <= tl::kMaxIt; i++) {
    t.c[i] = cos(1.0 * i);
    t.s[i] = sin(1.0 * i);
  }
  g_trig_ok = cudaMemcpyToSymbol(k_trig, &t, sizeof(t)) == cudaSuccess;
  return g_trig_ok;
}

void minmax(const cx& v, cx* mn, cx* mx) {
  if (v.re < mn->re) mn->re = v.re;
  if (v.im < mn->im) mn->im = v.im;
  if (v.re > mx->re) mx->re = v.re;
  if (v.im > mx->im) mx->im = v.im;
}

// utils.h:31-46
void make_square(cx* mn, cx* mx, double scale) {
  const double cre = (mx->re + mn->re) / 2.0, cim = (mx->im + mn->im) / 2.0;
  double half = mx->re - mn->re;
  if (mx->im - mn->im > half) half = mx->im - mn->im;
  half *= scale / 2.0;
  *mx = tl::mk(cre + half, cim + half);
  *mn = tl::mk(cre - half, cim - half);
}

}  // namespace

// The reference's object state (ccc.h:43-60): get_cc always solves the
// triple polynomial; get_ca solves the critical curve first when there is
// none (binary polynomial when m3 == 0) and maps its first _polOrder branches.
struct CriticalCurveCaustic {
  double a, b, th, m2, m3;
  tl::Lens L;
  int len = 500;
  int order = 6;          // _polOrder: 4 for a binary lens
  bool binary = false;
  int cc_branches = 0;    // 0: no critical curve yet
  bool cc_binary = false;
  int ca_branches = 0;    // 0: no caustic yet
  std::vector<cx> cc, ca;   // [branch][sample]

  // run the kernel: solve the critical curve (binary polynomial or not) if
  // `solve`, then map `ca_n` branches to the caustic
  bool run(bool solve, bool solve_binary, int ca_n) {
    if (len <= 0 || !upload_trig()) return false;
    const int deg = solve ? (solve_binary ? 4 : 6) : cc_branches;
    std::vector<double> pc(len), ps(len);
    for (int j = 0; j < len; j++) {
      const double phi = 2.0 * 3.14159265359 * j / len;   // ccc.cc:57
      pc[j] = cos(phi);
      ps[j] = sin(phi);
    }
    CccSpec sp;
    sp.L = L;
    sp.a = a;
    sp.cc_binary = solve_binary ? 1 : 0;
    sp.deg = deg;
    sp.ca_binary = binary ? 1 : 0;
    sp.ca_branches = ca_n;
    sp.len = len;
    sp.do_cc = solve ? 1 : 0;
    double *dpc = nullptr, *dps = nullptr;
    cx *dcc = nullptr, *dca = nullptr;
    int* doff = nullptr;
    const size_t n = (size_t)6 * len;
    bool ok = cudaMalloc(&dpc, sizeof(double) * len) == cudaSuccess &&
              cudaMalloc(&dps, sizeof(double) * len) == cudaSuccess &&
              cudaMalloc(&dcc, sizeof(cx) * n) == cudaSuccess &&
              cudaMalloc(&dca, sizeof(cx) * n) == cudaSuccess &&
              cudaMalloc(&doff, sizeof(int) * (1 + kMaxOff)) == cudaSuccess;
    int off[1 + kMaxOff] = {0};
    if (ok) {
      cudaMemcpy(dpc, pc.data(), sizeof(double) * len, cudaMemcpyHostToDevice);
      cudaMemcpy(dps, ps.data(), sizeof(double) * len, cudaMemcpyHostToDevice);
      cudaMemset(doff, 0, sizeof(int) * (1 + kMaxOff));
      if (!solve)
        cudaMemcpy(dcc, cc.data(), sizeof(cx) * (size_t)cc_branches * len,
                   cudaMemcpyHostToDevice);
      ccc_kernel<<<1, 32>>>(sp, dpc, dps, dcc, dca, doff);
      if (solve) cc.resize((size_t)deg * len);
      ca.resize((size_t)ca_n * len);
      ok = (!solve || cudaMemcpy(cc.data(), dcc, sizeof(cx) * cc.size(),
                                 cudaMemcpyDeviceToHost) == cudaSuccess) &&
           (ca_n == 0 || cudaMemcpy(ca.data(), dca, sizeof(cx) * ca.size(),
                                    cudaMemcpyDeviceToHost) == cudaSuccess) &&
           cudaMemcpy(off, doff, sizeof(int) * (1 + kMaxOff), cudaMemcpyDeviceToHost) ==
               cudaSuccess;
    }
    cudaFree(dpc);
    cudaFree(dps);
    cudaFree(dcc);
    cudaFree(dca);
    cudaFree(doff);
    if (!ok) {
      fprintf(stderr, "libccc: CUDA error: %s\n", cudaGetErrorString(cudaGetLastError()));
      return false;
    }
    for (int k = 0; k < off[0] && k < kMaxOff; k++) printf("Roots off for j = %d\n", off[1 + k]);
    fflush(stdout);
    if (solve) {
      cc_branches = deg;
      cc_binary = solve_binary;
    }
    ca_branches = ca_n;
    return true;
  }

  // ccc.cc:42-98 (get_cc solves the triple polynomial whatever m3 is)
  bool get_cc() { return run(true, false, 0); }

  // ccc.cc:160-203
  bool get_ca() {
    if (cc_branches == 0) return run(true, binary, order);
    return run(false, cc_binary, order < cc_branches ? order : cc_branches);
  }
};

extern "C" {

CriticalCurveCaustic* ccc_new(double a, double b, double th, double m2, double m3,
                              int cccLength) {
  auto* o = new CriticalCurveCaustic();
  o->a = a;
  o->b = b;
  o->th = th;
  o->m2 = m2;
  o->m3 = m3;
  // lens.cc:4-18, 35-40
  o->L.m1 = 1.0 - m2 - m3;
  o->L.m2 = m2;
  o->L.m3 = m3;
  o->L.z1 = tl::mk(0.0, 0.0);
  o->L.z2 = tl::mk(a, 0.0);
  o->L.z3 = tl::mk(b * cos(th), b * sin(th));
  o->L.is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0) ? 1 : 0;
  o->len = cccLength > 0 ? cccLength : 0;
  // ccc.cc:21-25
  o->binary = m3 == 0.0;
  o->order = o->binary ? 4 : 6;
  return o;
}

void get_cc(CriticalCurveCaustic* ccc) { ccc->get_cc(); }

void get_ca(CriticalCurveCaustic* ccc) { ccc->get_ca(); }

// Where the reference reads branches it does not have (a caustic not yet
// computed, or fewer caustic than critical-curve branches after get_cc on a
// binary lens: undefined behaviour there), zeros are written here.
static cx branch_value(const std::vector<cx>& v, int branches, int len, int j, int i) {
  return j < branches ? v[(size_t)j * len + i] : tl::mk(0.0, 0.0);
}

void print_ccc(CriticalCurveCaustic* ccc, char* fileName) {
  FILE* f = fopen(fileName, "w");
  if (!f) return;
  const int p = ccc->order;   // ostream precision = polynomial order (ccc.cc:206)
  fprintf(f, "#Critical Curve and Caustic\n");
  fprintf(f, "# (a,b,theta,m2,m3) = (%.*g, %.*g, %.*g, %.*g, %.*g)\n", p, ccc->a, p, ccc->b, p,
          ccc->th, p, ccc->m2, p, ccc->m3);
  for (int s = 0; s < 2; s++) {
    const std::vector<cx>& v = s ? ccc->ca : ccc->cc;
    const int nb = s ? ccc->ca_branches : ccc->cc_branches;
    if (s) fprintf(f, "\n###########\n");
    for (int i = 0; i < ccc->len; i++) {
      for (int j = 0; j < ccc->order; j++) {
        const cx z = branch_value(v, nb, ccc->len, j, i);
        fprintf(f, "%.*g %.*g ", p, z.re, p, z.im);
      }
      fprintf(f, "\n");
    }
  }
  fclose(f);
}

// ccc.cc:277-291: as many branches as the critical curve has
void copy_cc_ca(CriticalCurveCaustic* ccc, double* cc, double* ca) {
  const int len = ccc->len;
  for (int j = 0; j < ccc->cc_branches; j++) {
    for (int i = 0; i < len; i++) {
      const size_t idx = (size_t)j * len + i;
      const cx z = branch_value(ccc->cc, ccc->cc_branches, len, j, i);
      const cx w = branch_value(ccc->ca, ccc->ca_branches, len, j, i);
      cc[2 * idx] = z.re;
      cc[2 * idx + 1] = z.im;
      ca[2 * idx] = w.re;
      ca[2 * idx + 1] = w.im;
    }
  }
}

void copy_lenses(CriticalCurveCaustic* ccc, double* lensPos) {
  const cx z[3] = {ccc->L.z1, ccc->L.z2, ccc->L.z3};
  for (int k = 0; k < 3; k++) {
    lensPos[2 * k] = z[k].re;
    lensPos[2 * k + 1] = z[k].im;
  }
}

double* get_lens_pos(CriticalCurveCaustic* ccc) {
  static double pos[6];
  copy_lenses(ccc, pos);
  return pos;
}

void get_bounding_box(CriticalCurveCaustic* ccc, double* ccMin, double* ccMax, double* caMin,
                      double* caMax, double scale) {
  cx bmn[2] = {tl::mk(1.0e10, 1.0e10), tl::mk(1.0e10, 1.0e10)};
  cx bmx[2] = {tl::mk(-1.0e10, -1.0e10), tl::mk(-1.0e10, -1.0e10)};
  const cx lz[3] = {ccc->L.z1, ccc->L.z2, ccc->L.z3};
  for (int s = 0; s < 2; s++) {
    for (const cx& z : s ? ccc->ca : ccc->cc) minmax(z, &bmn[s], &bmx[s]);
    for (int k = 0; k < 3; k++) minmax(lz[k], &bmn[s], &bmx[s]);
    make_square(&bmn[s], &bmx[s], scale);
  }
  ccMin[0] = bmn[0].re;
  ccMin[1] = bmn[0].im;
  ccMax[0] = bmx[0].re;
  ccMax[1] = bmx[0].im;
  caMin[0] = bmn[1].re;
  caMin[1] = bmn[1].im;
  caMax[0] = bmx[1].re;
  caMax[1] = bmx[1].im;
}

void ccc_delete(CriticalCurveCaustic* ccc) { delete ccc; }

}  // extern "C"
