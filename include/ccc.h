/*
 * ccc.h - C ABI of libccc.so: critical curves and caustics of a triple (or,
 * with m3 == 0, binary) lens, computed on the GPU.  The entry points keep the
 * reference's ctypes ABI (src/CCC/ccc.cc:244-348, bound by
 * Examples/ctypes_classes.py:13-75).  Complex arrays are std::complex<double>
 * layout: (re, im) pairs of doubles.  Results are identical to the reference
 * up to FP64 rounding, with the branches in the reference's order.
 */
#ifndef TL_CCC_H
#define TL_CCC_H

#ifdef __cplusplus
extern "C" {
#endif

typedef struct CriticalCurveCaustic CriticalCurveCaustic;

/* Replaces ccc_new (ccc.cc:243-258 -> ccc.cc:4-26): z1 = 0, z2 = (a, 0),
 * z3 = b e^{i th}; cccLength phase samples; m3 == 0 selects the binary
 * degree-4 polynomial. */
CriticalCurveCaustic* ccc_new(double a, double b, double th, double m2, double m3, int cccLength);

/* Replaces get_cc (ccc.cc:260-263 -> 42-98, 101-158). */
void get_cc(CriticalCurveCaustic* ccc);

/* Replaces get_ca (ccc.cc:265-268 -> 160-203). */
void get_ca(CriticalCurveCaustic* ccc);

/* Replaces print_ccc (ccc.cc:270-273 -> 205-237): text file, values with as
 * many significant digits as the polynomial order. */
void print_ccc(CriticalCurveCaustic* ccc, char* fileName);

/* Replaces copy_cc_ca (ccc.cc:277-291): order x cccLength complex values
 * each, branch-major. */
void copy_cc_ca(CriticalCurveCaustic* ccc, double* cc, double* ca);

/* Replaces copy_lenses (ccc.cc:297-304): z1, z2, z3. */
void copy_lenses(CriticalCurveCaustic* ccc, double* lensPos);

/* Replaces get_lens_pos (ccc.cc:306-313): pointer to a static array of three
 * complex values. */
double* get_lens_pos(CriticalCurveCaustic* ccc);

/* Replaces get_bounding_box (ccc.cc:315-345): square boxes (edge scaled by
 * `scale`) around the critical curve and the caustic, lens positions
 * included. */
void get_bounding_box(CriticalCurveCaustic* ccc, double* ccMin, double* ccMax, double* caMin,
                      double* caMax, double scale);

/* Frees an object (additive; the reference has no destroy export). */
void ccc_delete(CriticalCurveCaustic* ccc);

#ifdef __cplusplus
}
#endif
#endif
