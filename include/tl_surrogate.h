/*
 * tl_surrogate.h - the learned finite-source correction of liblcirs.so
 * (additive; no counterpart in the reference, whose magnifications always
 * come from inverse-ray shooting, src/LightCurves/lcirs.cc:103-191).
 *
 * A source position is described by 14 features (lens geometry, rho, the
 * linear limb-darkening coefficient, the point-source magnification
 * A_point and the offset from the nearest caustic sample).  An ensemble of
 * MLPs (14 -> 256 x 4 SiLU -> 1, BF16 tensor-core GEMMs with FP32
 * accumulation, FP32 Adam) predicts y = ln(A_finite / A_point).  The
 * ensemble mean is shrunk towards 0 (A_point) where it is not larger than the
 * members' spread.  Points whose members disagree, or that lie within a
 * given number of source radii of the caustic polyline, are flagged for the
 * IRS.
 *
 * Device pointers throughout (features, targets, outputs); `stream` is a
 * cudaStream_t or NULL.  Returns 0, -1 bad argument, -2 CUDA error.
 * Parameter layout of one member (floats): W1[256][16] (inputs 14, 15 are
 * zero padding), b1[256], then W_l[256][256], b_l[256] for l = 2..4, then
 * w5[256], b5.
 */
#ifndef TL_SURROGATE_H
#define TL_SURROGATE_H

#include <stdint.h>

#include "tl_batch.h"

#ifdef __cplusplus
extern "C" {
#endif

#define TLS_FEATURES 14

typedef struct tls_model tls_model;

int tls_param_count(void);
tls_model* tls_new(int members);
void tls_delete(tls_model* s);
int tls_set_params(tls_model* s, int member, const float* host_params);
int tls_get_params(tls_model* s, int member, float* host_params);
/* feature standardisation applied before the first layer */
int tls_set_normalisation(tls_model* s, const float* mean14, const float* std14);

/* One Adam step of one member on M rows (features M x 14, targets M);
 * loss (mean squared error before the step) written to loss_out (device,
 * may be NULL). */
int tls_train_step(tls_model* s, int member, int M, const float* feat, const float* target,
                   float lr, float* loss_out, void* stream);
/* Gradients of the mean squared error w.r.t. one member's parameters, to a
 * host array of tls_param_count() floats (synchronous; for checks). */
int tls_gradients(tls_model* s, int member, int M, const float* feat, const float* target,
                  float* host_grads, float* host_loss);
/* One member's predictions y (M floats). */
int tls_forward(tls_model* s, int member, int M, const float* feat, float* y, void* stream);
/* Ensemble: mean (shrunk: mean * (1 - var/mean^2) when mean^2 > var, else 0;
 * 0 from far_dc_rho source radii on, where A_point alone is kept) and spread
 * of y; gated[i] = 1 when the source lies within min_dc_rho source radii of
 * the caustic polyline, or closer than far_dc_rho with a spread > max_std
 * (those points need the IRS); otherwise mag[i] = A_point * exp(mean). */
int tls_predict(tls_model* s, int M, const float* feat, const double* aps, const float* dc_rho,
                float max_std, float min_dc_rho, float far_dc_rho, float* mean, float* stdv,
                double* mag, int32_t* gated, void* stream);

/* Features of M source positions (xy: M x 2 doubles, lens_idx: lenses of
 * the batch): feat (M x 14), point-source magnification aps over the images
 * that fall on the IRS image plane, and the distance to the caustic polyline
 * (near its nearest sample) in source radii dc_rho (0 when an image may reach
 * the plane's edge: such points need the IRS). */
int tls_features(tl_batch* b, int M, const double* xy, const int32_t* lens_idx, float* feat,
                 double* aps, float* dc_rho, void* stream);
/* Caustic sample (lens, branch 0..5, index 0..499) positions of the batch's
 * lenses, n x 2 doubles. */
int tlb_caustic_points(tl_batch* b, int n, const int32_t* lens_idx, const int32_t* branch,
                       const int32_t* index, double* xy, void* stream);

#ifdef __cplusplus
}
#endif
#endif
