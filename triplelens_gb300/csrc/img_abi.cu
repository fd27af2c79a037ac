// img_abi.cu - libimg.so: point-source images of one source position behind
// the reference's img_* C ABI (src/Images/imgpoint.cc:297-351, bound by
// Examples/ctypes_classes.py:78-125), solved on the GPU.
//
// Compiled with --fmad=false.  The object keeps the reference's state:
// the warm-start roots of its previous position (imgpoint.h:104-110), so a
// sequence of set_pos / get_images calls follows the same root continuation
// as ImgPoint (getRootsPrecalculated, imgpoint.cc:160-205; getImages,
// imgpoint.cc:208-274).  Each call runs one GPU thread (img_kernel) on the
// object's state.
#include <cuda_runtime.h>

#include <cmath>
#include <cstdio>

#include "img.h"
#include "tl_math.h"

using tl::cx;

namespace {

__constant__ tl::TrigTable k_trig;

struct ImgState {
  tl::Lens L;
  cx pos;
  tl::RootChain ch;
  int roots_available;
  int is_img[10];
  int n_img;
  int wrong_after_check;   // image count still wrong after the cold retry
};

// op 0: get_roots (always solves, warm-started); op 1: get_images
__global__ void img_kernel(ImgState* s, int op) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const tl::Lens L = s->L;
  if (op == 0 || !s->roots_available) {
    tl::chain_roots(L, &s->ch, s->pos, false, &k_trig);
    s->roots_available = 1;
  }
  if (op == 0) return;
  for (int pass = 0; pass < 2; pass++) {
    int n = 0;
    for (int k = 0; k < 10; k++) {
      s->is_img[k] = tl::img_check(L, s->ch.roots[k], s->pos, 1.0e-6) ? 1 : 0;
      n += s->is_img[k];
    }
    s->n_img = n;
    s->wrong_after_check = 0;
    if (!tl::wrong_count(L, n)) return;
    if (pass == 0) {
      tl::chain_roots(L, &s->ch, s->pos, true, &k_trig);   // cold retry
    } else {
      s->wrong_after_check = 1;
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

}  // namespace

struct ImgPoint {
  ImgState s;
  ImgState* d = nullptr;

  bool run(int op) {
    if (!upload_trig()) return false;
    if (!d && cudaMalloc(&d, sizeof(ImgState)) != cudaSuccess) {
      d = nullptr;
      return false;
    }
    if (cudaMemcpy(d, &s, sizeof(ImgState), cudaMemcpyHostToDevice) != cudaSuccess) return false;
    img_kernel<<<1, 1>>>(d, op);
    if (cudaMemcpy(&s, d, sizeof(ImgState), cudaMemcpyDeviceToHost) != cudaSuccess) {
      fprintf(stderr, "libimg: CUDA error: %s\n", cudaGetErrorString(cudaGetLastError()));
      return false;
    }
    if (op == 1 && s.wrong_after_check) {
      printf("Wrong number of images after the check: %d\n", s.n_img);   // imgpoint.cc:252
      fflush(stdout);
    }
    return true;
  }
};

extern "C" {

ImgPoint* img_new(double a, double b, double th, double m2, double m3, double posX,
                  double posY) {
  auto* o = new ImgPoint();
  // lens.cc:4-18, 35-40; imgpoint.cc:64
  o->s.L.m1 = 1.0 - m2 - m3;
  o->s.L.m2 = m2;
  o->s.L.m3 = m3;
  o->s.L.z1 = tl::mk(0.0, 0.0);
  o->s.L.z2 = tl::mk(a, 0.0);
  o->s.L.z3 = tl::mk(b * cos(th), b * sin(th));
  o->s.L.is_binary_img = (a == 0.0 || b == 0.0 || m3 == 0.0) ? 1 : 0;
  tl::lens_finish(&o->s.L);
  o->s.pos = tl::mk(posX, posY);
  // a lone ImgPoint starts with no cached 256-byte chunks: its warm starts
  // read a zeroed slot past the roots
  tl::chain_reset(&o->s.ch, nullptr);
  o->s.roots_available = 0;
  o->s.n_img = 0;
  o->s.wrong_after_check = 0;
  for (int k = 0; k < 10; k++) o->s.is_img[k] = 0;
  return o;
}

void get_roots(ImgPoint* img) { img->run(0); }

void get_images(ImgPoint* img) { img->run(1); }

void set_pos(ImgPoint* img, double posX, double posY) {
  // imgpoint.cc:93-102: invalidates the roots, keeps the warm-start roots
  img->s.pos = tl::mk(posX, posY);
  img->s.roots_available = 0;
}

void copy_images(ImgPoint* img, double* roots, bool* isImg) {
  for (int k = 0; k < 10; k++) {
    roots[2 * k] = img->s.ch.roots[k].re;
    roots[2 * k + 1] = img->s.ch.roots[k].im;
    isImg[k] = img->s.is_img[k] != 0;
  }
}

void img_delete(ImgPoint* img) {
  if (!img) return;
  if (img->d) cudaFree(img->d);
  delete img;
}

}  // extern "C"
