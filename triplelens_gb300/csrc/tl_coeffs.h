// tl_coeffs.h - coefficients of the degree-10 triple-lens polynomial, in
// the reference's evaluation order (shared by host and device code).
//
// The reference builds the polynomial of ImgPoint::getRootsPrecalculated
// (TripleLens src/Images/imgpoint.cc:160-176) from two machine-generated
// expression trees: the part free of the source position,
// ImgPoint::getCoeffsOptNoZ (src/Images/imgpointcoeff.cc:223-278), computed
// once per lens, and the part linear-to-cubic in the source position,
// ImgPoint::getCoeffsOptJustZ (imgpointcoeff.cc:280-447), computed for every
// solve; the two are added term by term.  The warm-started Laguerre iteration
// that follows resolves the roots next to a small-mass lens only to the
// rounding of these coefficients, and the 1e-6 image filter turns those last
// bits into whole images, so the expressions keep the reference's temporaries
// and operation order exactly: every product and sum below rounds as the
// corresponding std::complex<double> operation of a strict IEEE build does.
// Checked bit for bit against the reference build on 1.1e6 coefficients.
//
// C() lifts a real temporary to a complex one (the reference declares those
// temporaries complex<double>); the operators are tl_math.h's.
#pragma once

#include "tl_math.h"

namespace tl {

// imgpointcoeff.cc:223-278: out[k] = coefficient of z^k, source-free part
TL_HD void coeffs_nozeta(double m2, double m3, cx z2, cx z3, cx* out) {
  const cx z3c = conj(z3);
  const cx a10zl = C(0.0);
  const double t1 = -m2 - m3;
  const cx a9zl = C(t1 * z3c * z2);
  const double t3 = 0.3e1 * m3;
  const double t4 = 0.2e1 * m2;
  const cx t7 = C(z2 * z2);
  const double t9 = 0.2e1 * m3;
  const double t10 = 0.3e1 * m2;
  const cx t16 = C(z3c * m3);
  const cx a8zl = C((t3 + t4) * z3c * t7 + ((t9 + t10) * z3c * z3 + m2) * z2 + t16);
  const cx t19 = C(t7 * z2);
  const cx t30 = C(z3 * z3);
  const double t32 = m2 * m3;
  const cx a7zl = C((-t3 - m2) * z3c * t19 + (0.6e1 * t1 * z3c * z3 + m2 * (-0.2e1 + m2)) * t7 + ((-t10 - m3) * z3c * t30 + (m3 - t10 + t32) * z3 + (m2 - t3 + t32) * z3c) * z2 + m3 * (-0.2e1 + m3) * z3c * z3);
  const cx t43 = C(t7 * t7);
  const cx t44 = C(t43 * z3c);
  const double t46 = 0.6e1 * m3;
  const double t50 = m2 - 0.1e1;
  const double t51 = m2 * t50;
  const double t54 = 0.6e1 * m2;
  const double t58 = m2 * m2;
  const double t59 = 0.3e1 * t58;
  const cx t62 = C(0.2e1 * t32);
  const cx t68 = C(t30 * z3);
  const cx t69 = C(z3c * m2 * t68);
  const double t70 = m3 * m3;
  const cx t73 = C(0.3e1 * t70);
  const cx t79 = C(-0.1e1 + m3);
  const cx t80 = C(m3 * t79);
  const cx t83 = C(m3 * z3);
  const cx a6zl = C(t44 * m3 + ((t46 + t10) * z3c * z3 - t51) * t19 + ((t54 + t3) * z3c * t30 + (-t59 + t54 - t3 - t32) * z3 + (-t4 + t58 - t62 + t3) * z3c) * t7 + (t69 + (t10 - t9 - t62 + t70) * t30 + (-t32 + t46 - t10 - t73) * z3c * z3 - m2) * z2 - t80 * z3c * t30 - t83);
  const double t91 = m2 - m3;
  const cx a5zl = C(-0.2e1 * t44 * t83 + (0.3e1 * t1 * z3c * t30 + (t3 - t10 + t59 - t32) * z3 - t50 * t91 * z3c) * t19 + (-0.2e1 * t69 + (t46 + t59 + t62 - t54 - t73) * t30 + (-t46 + t62 + t54 + t73 - t59) * z3c * z3 - 0.2e1 * t51) * t7 + (t79 * t91 * t68 + (-t3 - t32 + t73 + t10) * z3c * t30 + (t10 + t3 - 0.4e1 * t32) * z3) * z2 - 0.2e1 * t80 * t30);
  const cx t127 = C(t50 * t50);
  const cx t136 = C(0.8e1 * t32);
  const cx t137 = C(t58 * m3);
  const cx t139 = C(0.6e1 * t58);
  const cx t145 = C(z3c * t68);
  const cx t147 = C(0.6e1 * t70);
  const double t148 = m2 * t70;
  const cx t154 = C(t79 * t79);
  const cx a4zl = C((t16 * t30 + m3 * t50 * z3) * t43 + (t69 + (t73 + t62 - t46 + t10 - t59) * t30 + (-t70 + t9 + t59 - t32 - t10) * z3c * z3 - m2 * t127) * t19 + ((t4 - t3 - t32 - t58 + t73) * t68 + (t62 + t3 - t73 - t54 + t59) * z3c * t30 + (t136 - t3 - t54 - 0.3e1 * t137 + t139) * z3) * t7 + (m2 * t79 * t145 + (-t10 + t147 - 0.3e1 * t148 + t136 - t46) * t30) * z2 - m3 * t154 * t68);
  const cx t166 = C(0.3e1 * t32);
  const cx a3zl = C(-m3 * (m3 - 0.2e1 + t4) * t30 * t43 + ((-t32 + t3 - m2 - t73 + t58) * t68 + (-m3 - t59 + t70 - t32 + t10) * z3c * t30 + t50 * (t59 - t10 + t166 - m3) * z3) * t19 + (-m2 * (m2 + t9 - 0.2e1) * t145 + (0.6e1 * t148 - 0.16e2 * t32 - t147 - t139 + t54 + 0.6e1 * t137 + t46) * t30) * t7 + t79 * (t73 + t166 - t3 - m2) * t68 * z2);
  const double t186 = -0.1e1 + m2 + m3;
  const cx a2zl = C(t68 * t186 * m3 * t43 + (t186 * z3c * m2 * t68 - t186 * (t166 - t10 + t59 - t9) * t30) * t19 - t186 * (t73 + t166 - t3 - t4) * t68 * t7);
  const cx t202 = C(t186 * t186);
  const cx a1zl = C(-t202 * t1 * t68 * t19);
  const cx a0zl = C(0.0);
  out[0] = a0zl;
  out[1] = a1zl;
  out[2] = a2zl;
  out[3] = a3zl;
  out[4] = a4zl;
  out[5] = a5zl;
  out[6] = a6zl;
  out[7] = a7zl;
  out[8] = a8zl;
  out[9] = a9zl;
  out[10] = a10zl;
}

// imgpointcoeff.cc:280-447: out[k] = coefficient of z^k, source part
TL_HD void coeffs_zeta(double m2, double m3, cx z2, cx z3, cx zeta, cx* out) {
  const cx z3c = conj(z3);
  const cx zetac = conj(zeta);
  const cx t1 = C(zetac * z3c);
  const cx t2 = C(zetac * zetac);
  const cx t3 = C(-t1 + t2);
  const cx t5 = C(t2 * zetac);
  const cx t6 = C(t2 * z3c);
  const cx a10 = C(t3 * z2 - t5 + t6);
  const cx t7 = C(-t3);
  const cx t8 = C(0.3e1 * t7);
  const cx t9 = C(z2 * z2);
  const cx t12 = C(0.3e1 * zetac);
  const cx t15 = C(zetac * (-t12 + zeta) * z3c);
  const cx t16 = C(zeta * zetac);
  const cx t17 = C(0.3e1 * t2);
  const cx t22 = C(-t6 + t5);
  const cx t23 = C(0.3e1 * t22);
  const cx a9 = C(t8 * t9 + (t8 * z3 + t15 + zetac * (-t16 + t17 + m2 + 0.1e1)) * z2 + t23 * z3 + zetac * (0.1e1 - t16 + m3) * z3c + t2 * (t16 - 0.2e1));
  const cx t30 = C(-t8);
  const cx t31 = C(t9 * z2);
  const cx t33 = C(0.9e1 * t3);
  const cx t37 = C(zetac * (-zetac + zeta) * z3c);
  const cx t38 = C(0.3e1 * t37);
  const cx t39 = C(0.3e1 * t16);
  const cx t44 = C(z3 * z3);
  const cx t46 = C(0.3e1 * t15);
  const cx t47 = C(0.9e1 * t2);
  const cx t48 = C(0.2e1 * m3);
  const cx t49 = C(0.3e1 * m2);
  const cx t54 = C(zetac * m2);
  const cx t55 = C(0.2e1 * t54);
  const cx t56 = C(zeta * t2);
  const cx t57 = C(0.3e1 * t56);
  const cx t58 = C(zetac * m3);
  const cx t59 = C(0.3e1 * t58);
  const cx t62 = C(0.6e1 * zetac);
  const cx t63 = C(0.3e1 * t54);
  const cx t64 = C(0.2e1 * zeta);
  const cx t79 = C(t16 * z3c);
  const cx a8 = C(t30 * t31 + (t33 * z3 - t38 - zetac * (t17 - t39 + 0.3e1 + m2)) * t9 + (t30 * t44 + (-t46 - zetac * (t47 - t39 - t48 + t49 + 0.3e1)) * z3 + (zeta + t55 + t57 - t59 - t12) * z3c - zetac * (t57 - t62 + t63 + t64)) * z2 - t23 * t44 + (-zetac * (-t39 + m3 + 0.3e1) * z3c - 0.3e1 * t2 * (t16 + m3 - 0.2e1)) * z3 - 0.2e1 * t79 + zetac * (t39 - 0.1e1));
  const cx t83 = C(t9 * t9);
  const cx t85 = C(-t33);
  const cx t87 = C(0.3e1 * zeta);
  const cx t90 = C(zetac * (-zetac + t87) * z3c);
  const cx t96 = C(0.9e1 * t37);
  const cx t102 = C(m2 * zeta);
  const cx t103 = C(0.4e1 * t54);
  const cx t106 = C(0.6e1 * t54);
  const cx t107 = C(0.2e1 * t102);
  const cx t108 = C(0.6e1 * zeta);
  const cx t113 = C(t44 * z3);
  const cx t115 = C(0.4e1 * m3);
  const cx t120 = C(0.9e1 * zetac);
  const cx t121 = C(zeta * m3);
  const cx t122 = C(0.9e1 * t56);
  const cx t125 = C(0.18e2 * zetac);
  const cx t126 = C(0.9e1 * t58);
  const cx t127 = C(0.9e1 * t54);
  const cx t128 = C(0.2e1 * t121);
  const cx t133 = C(-0.3e1 + m2);
  const cx t134 = C(t133 * z3c);
  const cx t137 = C(t56 * m2);
  const cx t138 = C(0.3e1 * t137);
  const cx t150 = C(m3 - 0.3e1);
  const cx t151 = C(t150 * z3c);
  const cx t154 = C(t16 * m3);
  const cx t156 = C(0.9e1 * t16);
  const cx a7 = C(t7 * t83 + (t85 * z3 + t90 - zetac * (-t2 + t39 - 0.3e1 + m2)) * t31 + (t85 * t44 + (t96 + 0.3e1 * zetac * (t17 - t39 - t48 + 0.3e1 + m2)) * z3 + (t102 - t103 - t57 + t12 - t87 + t59) * z3c - zetac * (-t57 - t106 + t62 + t107 - t108)) * t9 + (t7 * t113 + (t46 + zetac * (t47 - t39 + t49 + 0.3e1 - t115)) * t44 + ((t120 + t121 - t87 - t106 - t122 + t59) * z3c + zetac * (t122 - t125 + t126 + t127 - t128 + t108)) * z3 - 0.2e1 * t16 * t134 - t122 - zeta + t138 - t103 + t12) * z2 + t22 * t113 + (-zetac * (t39 + m3 - 0.3e1) * z3c + 0.3e1 * t2 * (t16 + t48 - 0.2e1)) * t44 + (-0.2e1 * t16 * t151 + zetac * (0.3e1 * t154 - t156 + 0.3e1 - t115)) * z3 - zeta * z3c + t39);
  const cx t175 = C(0.2e1 * zetac);
  const cx t176 = C(0.4e1 * t102);
  const cx t187 = C(0.12e2 * t54);
  const cx t188 = C(0.9e1 * zeta);
  const cx t189 = C(0.3e1 * t102);
  const cx t190 = C(0.3e1 * t121);
  const cx t198 = C(0.2e1 * m2);
  const cx t199 = C(-0.3e1 + t198);
  const cx t203 = C(m2 * m2);
  const cx t204 = C(zetac * t203);
  const cx t205 = C(0.3e1 * t204);
  const cx t206 = C(0.8e1 * t54);
  const cx t207 = C(0.6e1 * t137);
  const cx t208 = C(t30 * t113 + (-t96 - 0.3e1 * zetac * (t17 - t39 + m2 - t115 + 0.3e1)) * t44 + ((t187 + t188 - t120 + t122 - t189 - t190 - t59) * z3c + 0.3e1 * zetac * (-t57 + t62 - t59 - t106 - t108 + t128 + t107)) * z3 + 0.2e1 * t16 * t199 * z3c - t12 - t107 + t87 - t205 + t122 + t206 - t207);
  const cx t217 = C(0.4e1 * t121);
  const cx t226 = C(t54 * m3);
  const cx t227 = C(0.6e1 * t226);
  const cx t228 = C(0.9e1 * t137);
  const cx t229 = C(0.27e2 * t56);
  const cx t230 = C(t56 * m3);
  const cx t231 = C(0.9e1 * t230);
  const cx t232 = C(0.12e2 * t58);
  const cx t244 = C(0.3e1 * m3);
  const cx t249 = C(t48 - 0.3e1);
  const cx t254 = C(m3 * m3);
  const cx t255 = C(0.3e1 * t254);
  const cx a6 = C((t30 * z3 - t79 + zetac * (t16 + m2 - 0.1e1)) * t83 + (t33 * t44 + (-0.3e1 * t90 + 0.3e1 * zetac * (-t2 + t39 + m2 - 0.3e1 + t48)) * z3 + (-zetac - t58 + t87 + t55 + t56 - t107) * z3c + zetac * (-t56 + t175 - t63 - t108 + t176)) * t31 + t208 * t9 + ((-t15 - zetac * (t17 - t16 + 0.1e1 - t48 + m2)) * t113 + ((-t128 + t122 + t87 + t106 - t120 + t59) * z3c - zetac * (t122 - t125 + 0.18e2 * t58 + t127 - t217 + t108)) * t44 + (0.6e1 * t16 * (m3 + m2 - 0.3e1) * z3c - t120 - t227 + t187 - t228 + t229 - t231 + t232 - t128 + t87) * z3 - zeta * t199 * z3c + 0.3e1 * t16 * t199) * z2 + (zetac * (t16 - 0.1e1 + m3) * z3c - t2 * (t16 + t244 - 0.2e1)) * t113 + (0.2e1 * t16 * t249 * z3c - zetac * (-t156 + 0.6e1 * t154 + t255 + 0.3e1 - 0.8e1 * m3)) * t44 + (-zeta * t249 * z3c + 0.3e1 * t16 * t249) * z3 + zeta);
  const cx t268 = C(0.3e1 * t79);
  const cx t273 = C(m2 - 0.1e1);
  const cx t274 = C(zeta * t273);
  const cx t286 = C(0.6e1 * t102);
  const cx t301 = C(0.6e1 * m3);
  const cx t306 = C(0.6e1 * t121);
  const cx t319 = C(0.12e2 * t226);
  const cx t320 = C(t102 * m3);
  const cx t321 = C(0.2e1 * t320);
  const cx t322 = C(0.24e2 * t54);
  const cx t323 = C(0.18e2 * t137);
  const cx t324 = C(0.9e1 * t204);
  const cx t325 = C(-0.6e1 * t16 * (m3 + t198 - 0.3e1) * z3c + t120 - t188 + t286 + t319 - t229 - t321 + t231 - t232 - t322 + t306 + t323 + t324);
  const cx t343 = C(zeta * t254);
  const cx t344 = C(zetac * t254);
  const cx t345 = C(0.9e1 * t344);
  const cx t346 = C(0.24e2 * t58);
  const cx t347 = C(0.18e2 * t230);
  const cx t348 = C(-0.6e1 * t16 * (m2 - 0.3e1 + t48) * z3c + t217 - t343 - t87 + t120 - t187 + t345 - t346 + t228 + t319 + t347 - t229);
  const cx t350 = C(m2 * m3);
  const cx t351 = C(0.2e1 * t350);
  const cx t352 = C(0.6e1 * m2);
  const cx t353 = C(0.9e1 + t351 - t352 - t301);
  const cx t363 = C(-0.1e1 + m3);
  const cx t372 = C(zeta * t363);
  const cx a5 = C((t8 * t44 + (t268 - zetac * (t39 + t49 + t48 - 0.3e1)) * z3 + t274 * z3c - 0.2e1 * t16 * t273) * t83 + (t8 * t113 + (0.3e1 * t90 - 0.3e1 * zetac * (-t2 + t39 + m2 - 0.3e1 + t115)) * t44 + ((-t188 + t58 - t106 - t57 + t286 + t190 + t12) * z3c - 0.3e1 * zetac * (-t56 - t58 - t63 + t175 + t128 - t108 + t176)) * z3 - 0.2e1 * t16 * t273 * z3c - t273 * (-t63 + t102 - t57 - t87 + zetac)) * t31 + ((t38 + zetac * (t17 - t39 - t301 + m2 + 0.3e1)) * t113 + ((t306 - t59 - t122 + t120 - t188 + t189 - t187) * z3c - 0.3e1 * zetac * (-t57 - t106 + t62 - 0.6e1 * t58 - t108 + t217 + t107)) * t44 + t325 * z3 - t274 * t134 + 0.3e1 * t16 * t273 * t133) * t9 + (((t12 - zeta + t121 - t59 - t57 - t55) * z3c + zetac * (t57 - t62 + t63 + t126 - t128 + t64)) * t113 + t348 * t44 + (-zeta * t353 * z3c + 0.3e1 * t16 * t353) * z3 + 0.3e1 * t274) * z2 + (-0.2e1 * t16 * t363 * z3c + t363 * zetac * (t244 + t39 - 0.1e1)) * t113 + (-t372 * t151 + 0.3e1 * t16 * t363 * t150) * t44 + 0.3e1 * t372 * z3);
  const cx t386 = C(t49 + m3 - 0.3e1);
  const cx t393 = C(t273 * t273);
  const cx t394 = C(zeta * t393);
  const cx t409 = C(t386 * z3c);
  const cx t412 = C(0.12e2 * t102);
  const cx t413 = C(0.4e1 * t320);
  const cx t417 = C(0.3e1 * t203 * zeta);
  const cx t418 = C(0.2e1 * t16 * t409 + t188 - t324 - t412 - t227 + t122 + t413 - 0.3e1 * t230 + 0.4e1 * t58 - t12 - t306 + t417 + t187 - t228);
  const cx t435 = C(0.12e2 * t121);
  const cx t437 = C(0.3e1 * t343);
  const cx t438 = C(0.6e1 * t16 * (t198 + t48 - 0.3e1) * z3c + t346 - t286 - t345 - t435 - t323 + t413 + t229 - 0.24e2 * t226 - t120 - t324 + t437 - t347 + t188 + t322);
  const cx t440 = C(0.3e1 * t203);
  const cx t441 = C(0.4e1 * t350);
  const cx t442 = C(0.12e2 * m2);
  const cx t443 = C(0.9e1 - t301 + t440 + t441 - t442);
  const cx t453 = C(-0.3e1 + t244 + m2);
  const cx t454 = C(t453 * z3c);
  const cx t457 = C(0.2e1 * t16 * t454 - t138 - t231 - t227 + t122 - t12 + t232 - t345 + t103 + zeta - t128 + t343);
  const cx t459 = C(0.12e2 * m3);
  const cx t460 = C(0.9e1 - t459 + t441 - t352 + t255);
  const cx t467 = C(t351 - t49 + 0.3e1 - t244);
  const cx t473 = C(t363 * t363);
  const cx t474 = C(zeta * t473);
  const cx a4 = C((t3 * t113 + (-t268 + zetac * (t39 - 0.3e1 + t115 + t49)) * t44 + (-zeta * t386 * z3c + 0.2e1 * t16 * t386) * z3 + t394) * t83 + ((-t90 + zetac * (-t2 + t39 + m2 - 0.3e1 + t301)) * t113 + ((t57 - t306 + t58 - t12 + t188 + t106 - t286) * z3c + 0.3e1 * zetac * (-t56 - t63 - 0.2e1 * t58 + t175 - t108 + t217 + t176)) * t44 + t418 * z3 + t394 * z3c - 0.3e1 * t16 * t393) * t31 + (((t57 + t103 - t102 + t59 + t87 - t190 - t12) * z3c + zetac * (-t57 + t62 - t106 - t126 - t108 + t306 + t107)) * t113 + t438 * t44 + (zeta * t443 * z3c - 0.3e1 * t16 * t443) * z3 + 0.3e1 * t394) * t9 + (t457 * t113 + (zeta * t460 * z3c - 0.3e1 * t16 * t460) * t44 + 0.3e1 * zeta * t467 * z3) * z2 + (t474 * z3c - 0.3e1 * t16 * t473) * t113 + 0.3e1 * t474 * t44);
  const cx t486 = C(t48 + t49 - 0.3e1);
  const cx t503 = C(t486 * z3c);
  const cx t510 = C(-0.2e1 * t16 * t503 - 0.8e1 * t58 + t412 + 0.3e1 * t344 + t319 + t228 - 0.8e1 * t320 - t122 + 0.6e1 * t230 + t12 + t324 - t417 - t187 + t435 - t437 - t188);
  const cx t522 = C(t198 - 0.3e1 + t244);
  const cx t523 = C(t522 * z3c);
  const cx t526 = C(-0.2e1 * t16 * t523 + t319 - t437 + t107 - t122 + t231 + t207 + t12 + t205 + t345 - t206 - t232 - t87 + t306 - t321);
  const cx t529 = C(t440 + 0.9e1 + 0.8e1 * t350 + t255 - t442 - t459);
  const cx t536 = C(t350 - t49 - t244 + 0.3e1);
  const cx a3 = C(((t79 - zetac * (t16 + m2 - 0.1e1 + t48)) * t113 + (zeta * t486 * z3c - 0.2e1 * t16 * t486) * t44 - t274 * t486 * z3) * t83 + (((-t87 - t55 - t58 + t190 + t107 + zetac - t56) * z3c - zetac * (-t56 + t175 - t63 - t59 - t108 + t176 + t306)) * t113 + t510 * t44 + (-t274 * t503 + 0.3e1 * t16 * t273 * t486) * z3 + zeta * t393 * t273) * t31 + (t526 * t113 + (-zeta * t529 * z3c + 0.3e1 * t16 * t529) * t44 + 0.3e1 * t274 * t536 * z3) * t9 + ((-t372 * t523 + 0.3e1 * t16 * t363 * t522) * t113 + 0.3e1 * t372 * t536 * t44) * z2 + zeta * t473 * t363 * t113);
  const cx t556 = C(-0.1e1 + m2 + m3);
  const cx t557 = C(t556 * zeta);
  const cx a2 = C(((-t557 * z3c + 0.2e1 * t557 * zetac) * t113 + t557 * t386 * t44) * t83 + ((0.2e1 * t557 * t1 + t556 * (-t63 + t190 - t59 - t57 - t87 + zetac + t102)) * t113 + (t557 * t409 - 0.3e1 * t557 * zetac * t386) * t44 - 0.3e1 * t557 * t393 * z3) * t31 + ((t557 * t454 - 0.3e1 * t557 * zetac * t453) * t113 - 0.3e1 * t557 * t467 * t44) * t9 - 0.3e1 * t557 * t473 * t113 * z2);
  const cx t600 = C(t556 * t556);
  const cx t603 = C(zeta * t600);
  const cx a1 = C(-zeta * t113 * t600 * t83 + ((-t603 * z3c + 0.3e1 * t603 * zetac) * t113 + 0.3e1 * t603 * t273 * t44) * t31 + 0.3e1 * t603 * t363 * t113 * t9);
  const cx a0 = C(-zeta * t31 * t113 * t600 * t556);
  out[0] = a0;
  out[1] = a1;
  out[2] = a2;
  out[3] = a3;
  out[4] = a4;
  out[5] = a5;
  out[6] = a6;
  out[7] = a7;
  out[8] = a8;
  out[9] = a9;
  out[10] = a10;
}

}  // namespace tl
