/*
 * img.h - C ABI of libimg.so: point-source images of a triple lens for one
 * source position, solved on the GPU.  The entry points keep the
 * reference's ctypes ABI (src/Images/imgpoint.cc:297-351, bound by
 * Examples/ctypes_classes.py:78-125).  Complex arrays are
 * std::complex<double> layout: (re, im) pairs of doubles.
 */
#ifndef TL_IMG_H
#define TL_IMG_H

#include <stdbool.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct ImgPoint ImgPoint;

/* Replaces img_new (imgpoint.cc:299-316): lens as in lcirs_new, source at
 * (posX, posY). */
ImgPoint* img_new(double a, double b, double th, double m2, double m3, double posX, double posY);

/* Replaces get_roots (imgpoint.cc:318-321): the 10 roots of the lens
 * polynomial, warm-started from the object's previous roots
 * (getRootsPrecalculated, imgpoint.cc:160-205; the degree-10 polynomial is
 * used for m3 = 0 as well). */
void get_roots(ImgPoint* img);

/* Replaces get_images (imgpoint.cc:323-326 -> 208-274): roots, the 1e-6
 * image filter, one cold retry on a wrong image count (and the reference's
 * "Wrong number of images after the check" line when it is still wrong). */
void get_images(ImgPoint* img);

/* Replaces set_pos (imgpoint.cc:328-333). */
void set_pos(ImgPoint* img, double posX, double posY);

/* Replaces copy_images (imgpoint.cc:337-349): 10 roots and their image flags. */
void copy_images(ImgPoint* img, double* roots, bool* isImg);

/* Frees an object (additive; the reference has no destroy export). */
void img_delete(ImgPoint* img);

#ifdef __cplusplus
}
#endif
#endif
