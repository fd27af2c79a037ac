// lccuda_abi.cu - liblccuda.so: the reference's CUDA light-curve ABI
// (src/Cuda/cudalc.cc:486-542, bound by Examples/ctypes_classes.py:196-270)
// routed to this engine.  The reference's CUDA estimator (8 x 8 sub-grids,
// a 1.4 rho^2 envelope) differs from its CPU IRS; here get_lc_cuda returns
// the IRS magnifications of get_lc_irs (the reference's CPU result), so
// scripts written for LC_cuda get the CPU reference's numbers at GPU speed.
// get_lc and copy_lc come from lcirs_abi.cu.
#include "lccuda.h"
#include "lcirs.h"

extern "C" {

LightCurveIRS* lccuda_new(double a, double b, double th, double m2, double m3, double sourceSize,
                          unsigned int lcLength, long pointsPerRadius) {
  return lcirs_new(a, b, th, m2, m3, sourceSize, lcLength, pointsPerRadius);
}

void get_lc_cuda(LightCurveIRS* lc, double iniX, double iniY, double finX, double finY) {
  get_lc_irs(lc, iniX, iniY, finX, finY);
}

void set_limb_darkening_cuda(LightCurveIRS* lc, const char* model, double v) {
  set_limb_darkening(lc, model, v);
}

}  // extern "C"
