/*
 * lens_coeffs.c - coefficients of the degree-10 triple-lens polynomial in
 * the reference's own operation order.  TEST INFRASTRUCTURE ONLY (part of the
 * oracle library; the product never links it).
 *
 * The reference evaluates the coefficients as two machine-generated
 * expression trees: a part that does not depend on the source position
 * (ImgPoint::getCoeffsOptNoZ, src/Images/imgpointcoeff.cc:223-278), computed
 * once per lens, and a part that does (ImgPoint::getCoeffsOptJustZ,
 * imgpointcoeff.cc:280-447); getRootsPrecalculated (imgpoint.cc:160-176) adds
 * them term by term.  The Laguerre iteration that follows is sensitive to the
 * last bit of every coefficient (it decides which roots near a small-mass
 * lens pass the 1e-6 image filter), so the expressions below keep the
 * reference's temporaries and evaluation order exactly.  Any other algebraic
 * form of the same polynomial rounds differently.
 *
 * Arithmetic: C11 double _Complex, compiled -ffp-contract=off.  Products and
 * sums of complex values lower to the same real operations as std::complex
 * (a*b = (ac - bd, ad + bc); a real operand scales or shifts componentwise),
 * and there is no complex division here.
 */
#include <complex.h>

typedef double _Complex zc;

/* imgpointcoeff.cc:223-278.  out[0..10] = a0zl..a10zl */
void orc_coeffs_nozeta(double m2, double m3, const double z2xy[2], const double z3xy[2],
                       zc out[11]) {
  const zc z2 = z2xy[0] + z2xy[1] * I, z3 = z3xy[0] + z3xy[1] * I;
  zc z3c = conj(z3);

  zc a10zl = 0.0;
  double t1 = -m2 - m3;
  zc a9zl = t1 * z3c * z2;
  double t3 = 0.3e1 * m3;
  double t4 = 0.2e1 * m2;
  zc t7 = z2 * z2;
  double t9 = 0.2e1 * m3;
  double t10 = 0.3e1 * m2;
  zc t16 = z3c * m3;
  zc a8zl = (t3 + t4) * z3c * t7 + ((t9 + t10) * z3c * z3 + m2) * z2 + t16;
  zc t19 = t7 * z2;
  zc t30 = z3 * z3;
  double t32 = m2 * m3;
  zc a7zl = (-t3 - m2) * z3c * t19 + (0.6e1 * t1 * z3c * z3 + m2 * (-0.2e1 + m2)) * t7 +
            ((-t10 - m3) * z3c * t30 + (m3 - t10 + t32) * z3 + (m2 - t3 + t32) * z3c) * z2 +
            m3 * (-0.2e1 + m3) * z3c * z3;
  zc t43 = t7 * t7;
  zc t44 = t43 * z3c;
  double t46 = 0.6e1 * m3;
  double t50 = m2 - 0.1e1;
  double t51 = m2 * t50;
  double t54 = 0.6e1 * m2;
  double t58 = m2 * m2;
  double t59 = 0.3e1 * t58;
  zc t62 = 0.2e1 * t32;
  zc t68 = t30 * z3;
  zc t69 = z3c * m2 * t68;
  double t70 = m3 * m3;
  zc t73 = 0.3e1 * t70;
  zc t79 = -0.1e1 + m3;
  zc t80 = m3 * t79;
  zc t83 = m3 * z3;
  zc a6zl = t44 * m3 + ((t46 + t10) * z3c * z3 - t51) * t19 +
            ((t54 + t3) * z3c * t30 + (-t59 + t54 - t3 - t32) * z3 + (-t4 + t58 - t62 + t3) * z3c) *
                t7 +
            (t69 + (t10 - t9 - t62 + t70) * t30 + (-t32 + t46 - t10 - t73) * z3c * z3 - m2) * z2 -
            t80 * z3c * t30 - t83;
  double t91 = m2 - m3;
  zc a5zl = -0.2e1 * t44 * t83 +
            (0.3e1 * t1 * z3c * t30 + (t3 - t10 + t59 - t32) * z3 - t50 * t91 * z3c) * t19 +
            (-0.2e1 * t69 + (t46 + t59 + t62 - t54 - t73) * t30 +
             (-t46 + t62 + t54 + t73 - t59) * z3c * z3 - 0.2e1 * t51) *
                t7 +
            (t79 * t91 * t68 + (-t3 - t32 + t73 + t10) * z3c * t30 + (t10 + t3 - 0.4e1 * t32) * z3) *
                z2 -
            0.2e1 * t80 * t30;
  zc t127 = t50 * t50;
  zc t136 = 0.8e1 * t32;
  zc t137 = t58 * m3;
  zc t139 = 0.6e1 * t58;
  zc t145 = z3c * t68;
  zc t147 = 0.6e1 * t70;
  double t148 = m2 * t70;
  zc t154 = t79 * t79;
  zc a4zl = (t16 * t30 + m3 * t50 * z3) * t43 +
            (t69 + (t73 + t62 - t46 + t10 - t59) * t30 + (-t70 + t9 + t59 - t32 - t10) * z3c * z3 -
             m2 * t127) *
                t19 +
            ((t4 - t3 - t32 - t58 + t73) * t68 + (t62 + t3 - t73 - t54 + t59) * z3c * t30 +
             (t136 - t3 - t54 - 0.3e1 * t137 + t139) * z3) *
                t7 +
            (m2 * t79 * t145 + (-t10 + t147 - 0.3e1 * t148 + t136 - t46) * t30) * z2 -
            m3 * t154 * t68;
  zc t166 = 0.3e1 * t32;
  zc a3zl = -m3 * (m3 - 0.2e1 + t4) * t30 * t43 +
            ((-t32 + t3 - m2 - t73 + t58) * t68 + (-m3 - t59 + t70 - t32 + t10) * z3c * t30 +
             t50 * (t59 - t10 + t166 - m3) * z3) *
                t19 +
            (-m2 * (m2 + t9 - 0.2e1) * t145 +
             (0.6e1 * t148 - 0.16e2 * t32 - t147 - t139 + t54 + 0.6e1 * t137 + t46) * t30) *
                t7 +
            t79 * (t73 + t166 - t3 - m2) * t68 * z2;
  double t186 = -0.1e1 + m2 + m3;
  zc a2zl = t68 * t186 * m3 * t43 +
            (t186 * z3c * m2 * t68 - t186 * (t166 - t10 + t59 - t9) * t30) * t19 -
            t186 * (t73 + t166 - t3 - t4) * t68 * t7;
  zc t202 = t186 * t186;
  zc a1zl = -t202 * t1 * t68 * t19;
  zc a0zl = 0.0;

  out[0] = a0zl; out[1] = a1zl; out[2] = a2zl; out[3] = a3zl; out[4] = a4zl;
  out[5] = a5zl; out[6] = a6zl; out[7] = a7zl; out[8] = a8zl; out[9] = a9zl;
  out[10] = a10zl;
}

/* imgpointcoeff.cc:280-447.  out[0..10] = a0..a10 for source position zeta */
void orc_coeffs_zeta(double m2, double m3, const double z2xy[2], const double z3xy[2],
                     double zx, double zy, zc out[11]) {
  const zc z2 = z2xy[0] + z2xy[1] * I, z3 = z3xy[0] + z3xy[1] * I;
  zc z3c = conj(z3);
  zc zeta = zx + zy * I;
  zc zetac = conj(zeta);

  zc t1 = zetac * z3c;
  zc t2 = zetac * zetac;
  zc t3 = -t1 + t2;
  zc t5 = t2 * zetac;
  zc t6 = t2 * z3c;
  zc a10 = t3 * z2 - t5 + t6;
  zc t7 = -t3;
  zc t8 = 0.3e1 * t7;
  zc t9 = z2 * z2;
  zc t12 = 0.3e1 * zetac;
  zc t15 = zetac * (-t12 + zeta) * z3c;
  zc t16 = zeta * zetac;
  zc t17 = 0.3e1 * t2;
  zc t22 = -t6 + t5;
  zc t23 = 0.3e1 * t22;
  zc a9 = t8 * t9 + (t8 * z3 + t15 + zetac * (-t16 + t17 + m2 + 0.1e1)) * z2 + t23 * z3 +
          zetac * (0.1e1 - t16 + m3) * z3c + t2 * (t16 - 0.2e1);
  zc t30 = -t8;
  zc t31 = t9 * z2;
  zc t33 = 0.9e1 * t3;
  zc t37 = zetac * (-zetac + zeta) * z3c;
  zc t38 = 0.3e1 * t37;
  zc t39 = 0.3e1 * t16;
  zc t44 = z3 * z3;
  zc t46 = 0.3e1 * t15;
  zc t47 = 0.9e1 * t2;
  zc t48 = 0.2e1 * m3;
  zc t49 = 0.3e1 * m2;
  zc t54 = zetac * m2;
  zc t55 = 0.2e1 * t54;
  zc t56 = zeta * t2;
  zc t57 = 0.3e1 * t56;
  zc t58 = zetac * m3;
  zc t59 = 0.3e1 * t58;
  zc t62 = 0.6e1 * zetac;
  zc t63 = 0.3e1 * t54;
  zc t64 = 0.2e1 * zeta;
  zc t79 = t16 * z3c;
  zc a8 = t30 * t31 + (t33 * z3 - t38 - zetac * (t17 - t39 + 0.3e1 + m2)) * t9 +
          (t30 * t44 + (-t46 - zetac * (t47 - t39 - t48 + t49 + 0.3e1)) * z3 +
           (zeta + t55 + t57 - t59 - t12) * z3c - zetac * (t57 - t62 + t63 + t64)) *
              z2 -
          t23 * t44 +
          (-zetac * (-t39 + m3 + 0.3e1) * z3c - 0.3e1 * t2 * (t16 + m3 - 0.2e1)) * z3 -
          0.2e1 * t79 + zetac * (t39 - 0.1e1);
  zc t83 = t9 * t9;
  zc t85 = -t33;
  zc t87 = 0.3e1 * zeta;
  zc t90 = zetac * (-zetac + t87) * z3c;
  zc t96 = 0.9e1 * t37;
  zc t102 = m2 * zeta;
  zc t103 = 0.4e1 * t54;
  zc t106 = 0.6e1 * t54;
  zc t107 = 0.2e1 * t102;
  zc t108 = 0.6e1 * zeta;
  zc t113 = t44 * z3;
  zc t115 = 0.4e1 * m3;
  zc t120 = 0.9e1 * zetac;
  zc t121 = zeta * m3;
  zc t122 = 0.9e1 * t56;
  zc t125 = 0.18e2 * zetac;
  zc t126 = 0.9e1 * t58;
  zc t127 = 0.9e1 * t54;
  zc t128 = 0.2e1 * t121;
  zc t133 = -0.3e1 + m2;
  zc t134 = t133 * z3c;
  zc t137 = t56 * m2;
  zc t138 = 0.3e1 * t137;
  zc t150 = m3 - 0.3e1;
  zc t151 = t150 * z3c;
  zc t154 = t16 * m3;
  zc t156 = 0.9e1 * t16;
  zc a7 = t7 * t83 + (t85 * z3 + t90 - zetac * (-t2 + t39 - 0.3e1 + m2)) * t31 +
          (t85 * t44 + (t96 + 0.3e1 * zetac * (t17 - t39 - t48 + 0.3e1 + m2)) * z3 +
           (t102 - t103 - t57 + t12 - t87 + t59) * z3c -
           zetac * (-t57 - t106 + t62 + t107 - t108)) *
              t9 +
          (t7 * t113 + (t46 + zetac * (t47 - t39 + t49 + 0.3e1 - t115)) * t44 +
           ((t120 + t121 - t87 - t106 - t122 + t59) * z3c +
            zetac * (t122 - t125 + t126 + t127 - t128 + t108)) *
               z3 -
           0.2e1 * t16 * t134 - t122 - zeta + t138 - t103 + t12) *
              z2 +
          t22 * t113 +
          (-zetac * (t39 + m3 - 0.3e1) * z3c + 0.3e1 * t2 * (t16 + t48 - 0.2e1)) * t44 +
          (-0.2e1 * t16 * t151 + zetac * (0.3e1 * t154 - t156 + 0.3e1 - t115)) * z3 -
          zeta * z3c + t39;
  zc t175 = 0.2e1 * zetac;
  zc t176 = 0.4e1 * t102;
  zc t187 = 0.12e2 * t54;
  zc t188 = 0.9e1 * zeta;
  zc t189 = 0.3e1 * t102;
  zc t190 = 0.3e1 * t121;
  zc t198 = 0.2e1 * m2;
  zc t199 = -0.3e1 + t198;
  zc t203 = m2 * m2;
  zc t204 = zetac * t203;
  zc t205 = 0.3e1 * t204;
  zc t206 = 0.8e1 * t54;
  zc t207 = 0.6e1 * t137;
  zc t208 = t30 * t113 + (-t96 - 0.3e1 * zetac * (t17 - t39 + m2 - t115 + 0.3e1)) * t44 +
            ((t187 + t188 - t120 + t122 - t189 - t190 - t59) * z3c +
             0.3e1 * zetac * (-t57 + t62 - t59 - t106 - t108 + t128 + t107)) *
                z3 +
            0.2e1 * t16 * t199 * z3c - t12 - t107 + t87 - t205 + t122 + t206 - t207;
  zc t217 = 0.4e1 * t121;
  zc t226 = t54 * m3;
  zc t227 = 0.6e1 * t226;
  zc t228 = 0.9e1 * t137;
  zc t229 = 0.27e2 * t56;
  zc t230 = t56 * m3;
  zc t231 = 0.9e1 * t230;
  zc t232 = 0.12e2 * t58;
  zc t244 = 0.3e1 * m3;
  zc t249 = t48 - 0.3e1;
  zc t254 = m3 * m3;
  zc t255 = 0.3e1 * t254;
  zc a6 = (t30 * z3 - t79 + zetac * (t16 + m2 - 0.1e1)) * t83 +
          (t33 * t44 + (-0.3e1 * t90 + 0.3e1 * zetac * (-t2 + t39 + m2 - 0.3e1 + t48)) * z3 +
           (-zetac - t58 + t87 + t55 + t56 - t107) * z3c +
           zetac * (-t56 + t175 - t63 - t108 + t176)) *
              t31 +
          t208 * t9 +
          ((-t15 - zetac * (t17 - t16 + 0.1e1 - t48 + m2)) * t113 +
           ((-t128 + t122 + t87 + t106 - t120 + t59) * z3c -
            zetac * (t122 - t125 + 0.18e2 * t58 + t127 - t217 + t108)) *
               t44 +
           (0.6e1 * t16 * (m3 + m2 - 0.3e1) * z3c - t120 - t227 + t187 - t228 + t229 - t231 +
            t232 - t128 + t87) *
               z3 -
           zeta * t199 * z3c + 0.3e1 * t16 * t199) *
              z2 +
          (zetac * (t16 - 0.1e1 + m3) * z3c - t2 * (t16 + t244 - 0.2e1)) * t113 +
          (0.2e1 * t16 * t249 * z3c -
           zetac * (-t156 + 0.6e1 * t154 + t255 + 0.3e1 - 0.8e1 * m3)) *
              t44 +
          (-zeta * t249 * z3c + 0.3e1 * t16 * t249) * z3 + zeta;
  zc t268 = 0.3e1 * t79;
  zc t273 = m2 - 0.1e1;
  zc t274 = zeta * t273;
  zc t286 = 0.6e1 * t102;
  zc t301 = 0.6e1 * m3;
  zc t306 = 0.6e1 * t121;
  zc t319 = 0.12e2 * t226;
  zc t320 = t102 * m3;
  zc t321 = 0.2e1 * t320;
  zc t322 = 0.24e2 * t54;
  zc t323 = 0.18e2 * t137;
  zc t324 = 0.9e1 * t204;
  zc t325 = -0.6e1 * t16 * (m3 + t198 - 0.3e1) * z3c + t120 - t188 + t286 + t319 - t229 -
            t321 + t231 - t232 - t322 + t306 + t323 + t324;
  zc t343 = zeta * t254;
  zc t344 = zetac * t254;
  zc t345 = 0.9e1 * t344;
  zc t346 = 0.24e2 * t58;
  zc t347 = 0.18e2 * t230;
  zc t348 = -0.6e1 * t16 * (m2 - 0.3e1 + t48) * z3c + t217 - t343 - t87 + t120 - t187 +
            t345 - t346 + t228 + t319 + t347 - t229;
  zc t350 = m2 * m3;
  zc t351 = 0.2e1 * t350;
  zc t352 = 0.6e1 * m2;
  zc t353 = 0.9e1 + t351 - t352 - t301;
  zc t363 = -0.1e1 + m3;
  zc t372 = zeta * t363;
  zc a5 = (t8 * t44 + (t268 - zetac * (t39 + t49 + t48 - 0.3e1)) * z3 + t274 * z3c -
           0.2e1 * t16 * t273) *
              t83 +
          (t8 * t113 +
           (0.3e1 * t90 - 0.3e1 * zetac * (-t2 + t39 + m2 - 0.3e1 + t115)) * t44 +
           ((-t188 + t58 - t106 - t57 + t286 + t190 + t12) * z3c -
            0.3e1 * zetac * (-t56 - t58 - t63 + t175 + t128 - t108 + t176)) *
               z3 -
           0.2e1 * t16 * t273 * z3c - t273 * (-t63 + t102 - t57 - t87 + zetac)) *
              t31 +
          ((t38 + zetac * (t17 - t39 - t301 + m2 + 0.3e1)) * t113 +
           ((t306 - t59 - t122 + t120 - t188 + t189 - t187) * z3c -
            0.3e1 * zetac * (-t57 - t106 + t62 - 0.6e1 * t58 - t108 + t217 + t107)) *
               t44 +
           t325 * z3 - t274 * t134 + 0.3e1 * t16 * t273 * t133) *
              t9 +
          (((t12 - zeta + t121 - t59 - t57 - t55) * z3c +
            zetac * (t57 - t62 + t63 + t126 - t128 + t64)) *
               t113 +
           t348 * t44 + (-zeta * t353 * z3c + 0.3e1 * t16 * t353) * z3 + 0.3e1 * t274) *
              z2 +
          (-0.2e1 * t16 * t363 * z3c + t363 * zetac * (t244 + t39 - 0.1e1)) * t113 +
          (-t372 * t151 + 0.3e1 * t16 * t363 * t150) * t44 + 0.3e1 * t372 * z3;
  zc t386 = t49 + m3 - 0.3e1;
  zc t393 = t273 * t273;
  zc t394 = zeta * t393;
  zc t409 = t386 * z3c;
  zc t412 = 0.12e2 * t102;
  zc t413 = 0.4e1 * t320;
  zc t417 = 0.3e1 * t203 * zeta;
  zc t418 = 0.2e1 * t16 * t409 + t188 - t324 - t412 - t227 + t122 + t413 - 0.3e1 * t230 +
            0.4e1 * t58 - t12 - t306 + t417 + t187 - t228;
  zc t435 = 0.12e2 * t121;
  zc t437 = 0.3e1 * t343;
  zc t438 = 0.6e1 * t16 * (t198 + t48 - 0.3e1) * z3c + t346 - t286 - t345 - t435 - t323 +
            t413 + t229 - 0.24e2 * t226 - t120 - t324 + t437 - t347 + t188 + t322;
  zc t440 = 0.3e1 * t203;
  zc t441 = 0.4e1 * t350;
  zc t442 = 0.12e2 * m2;
  zc t443 = 0.9e1 - t301 + t440 + t441 - t442;
  zc t453 = -0.3e1 + t244 + m2;
  zc t454 = t453 * z3c;
  zc t457 = 0.2e1 * t16 * t454 - t138 - t231 - t227 + t122 - t12 + t232 - t345 + t103 + zeta -
            t128 + t343;
  zc t459 = 0.12e2 * m3;
  zc t460 = 0.9e1 - t459 + t441 - t352 + t255;
  zc t467 = t351 - t49 + 0.3e1 - t244;
  zc t473 = t363 * t363;
  zc t474 = zeta * t473;
  zc a4 = (t3 * t113 + (-t268 + zetac * (t39 - 0.3e1 + t115 + t49)) * t44 +
           (-zeta * t386 * z3c + 0.2e1 * t16 * t386) * z3 + t394) *
              t83 +
          ((-t90 + zetac * (-t2 + t39 + m2 - 0.3e1 + t301)) * t113 +
           ((t57 - t306 + t58 - t12 + t188 + t106 - t286) * z3c +
            0.3e1 * zetac * (-t56 - t63 - 0.2e1 * t58 + t175 - t108 + t217 + t176)) *
               t44 +
           t418 * z3 + t394 * z3c - 0.3e1 * t16 * t393) *
              t31 +
          (((t57 + t103 - t102 + t59 + t87 - t190 - t12) * z3c +
            zetac * (-t57 + t62 - t106 - t126 - t108 + t306 + t107)) *
               t113 +
           t438 * t44 + (zeta * t443 * z3c - 0.3e1 * t16 * t443) * z3 + 0.3e1 * t394) *
              t9 +
          (t457 * t113 + (zeta * t460 * z3c - 0.3e1 * t16 * t460) * t44 +
           0.3e1 * zeta * t467 * z3) *
              z2 +
          (t474 * z3c - 0.3e1 * t16 * t473) * t113 + 0.3e1 * t474 * t44;
  zc t486 = t48 + t49 - 0.3e1;
  zc t503 = t486 * z3c;
  zc t510 = -0.2e1 * t16 * t503 - 0.8e1 * t58 + t412 + 0.3e1 * t344 + t319 + t228 -
            0.8e1 * t320 - t122 + 0.6e1 * t230 + t12 + t324 - t417 - t187 + t435 - t437 - t188;
  zc t522 = t198 - 0.3e1 + t244;
  zc t523 = t522 * z3c;
  zc t526 = -0.2e1 * t16 * t523 + t319 - t437 + t107 - t122 + t231 + t207 + t12 + t205 +
            t345 - t206 - t232 - t87 + t306 - t321;
  zc t529 = t440 + 0.9e1 + 0.8e1 * t350 + t255 - t442 - t459;
  zc t536 = t350 - t49 - t244 + 0.3e1;
  zc a3 = ((t79 - zetac * (t16 + m2 - 0.1e1 + t48)) * t113 +
           (zeta * t486 * z3c - 0.2e1 * t16 * t486) * t44 - t274 * t486 * z3) *
              t83 +
          (((-t87 - t55 - t58 + t190 + t107 + zetac - t56) * z3c -
            zetac * (-t56 + t175 - t63 - t59 - t108 + t176 + t306)) *
               t113 +
           t510 * t44 + (-t274 * t503 + 0.3e1 * t16 * t273 * t486) * z3 + zeta * t393 * t273) *
              t31 +
          (t526 * t113 + (-zeta * t529 * z3c + 0.3e1 * t16 * t529) * t44 +
           0.3e1 * t274 * t536 * z3) *
              t9 +
          ((-t372 * t523 + 0.3e1 * t16 * t363 * t522) * t113 + 0.3e1 * t372 * t536 * t44) * z2 +
          zeta * t473 * t363 * t113;
  zc t556 = -0.1e1 + m2 + m3;
  zc t557 = t556 * zeta;
  zc a2 = ((-t557 * z3c + 0.2e1 * t557 * zetac) * t113 + t557 * t386 * t44) * t83 +
          ((0.2e1 * t557 * t1 + t556 * (-t63 + t190 - t59 - t57 - t87 + zetac + t102)) * t113 +
           (t557 * t409 - 0.3e1 * t557 * zetac * t386) * t44 - 0.3e1 * t557 * t393 * z3) *
              t31 +
          ((t557 * t454 - 0.3e1 * t557 * zetac * t453) * t113 - 0.3e1 * t557 * t467 * t44) * t9 -
          0.3e1 * t557 * t473 * t113 * z2;
  zc t600 = t556 * t556;
  zc t603 = zeta * t600;
  zc a1 = -zeta * t113 * t600 * t83 +
          ((-t603 * z3c + 0.3e1 * t603 * zetac) * t113 + 0.3e1 * t603 * t273 * t44) * t31 +
          0.3e1 * t603 * t363 * t113 * t9;
  zc a0 = -zeta * t31 * t113 * t600 * t556;

  out[0] = a0; out[1] = a1; out[2] = a2; out[3] = a3; out[4] = a4; out[5] = a5;
  out[6] = a6; out[7] = a7; out[8] = a8; out[9] = a9; out[10] = a10;
}
