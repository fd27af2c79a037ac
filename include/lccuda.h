/*
 * lccuda.h - C ABI of liblccuda.so: the reference's LC_cuda interface
 * (src/Cuda/cudalc.cc:486-542, bound by Examples/ctypes_classes.py:196-270)
 * routed to this engine.  The library also exports get_lc and copy_lc with
 * the meaning they have in lcirs.h.  get_lc_cuda computes the IRS
 * magnifications of get_lc_irs: the reference's CPU result, not its CUDA
 * estimator's (which uses 8 x 8 sub-grids and a 1.4 rho^2 envelope).
 */
#ifndef TL_LCCUDA_H
#define TL_LCCUDA_H

#include "lcirs.h"

#ifdef __cplusplus
extern "C" {
#endif

/* Replaces lccuda_new (cudalc.cc:488-506). */
LightCurveIRS* lccuda_new(double a, double b, double th, double m2, double m3, double sourceSize,
                          unsigned int lcLength, long pointsPerRadius);

/* Replaces get_lc_cuda (cudalc.cc:509-518): extended-source curve. */
void get_lc_cuda(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY);

/* Replaces set_limb_darkening_cuda (cudalc.cc:521-540). */
void set_limb_darkening_cuda(LightCurveIRS* lc, const char* model, double v);

#ifdef __cplusplus
}
#endif
#endif
