// lcirs.hpp - C++ class view of liblcirs.so, mirroring the reference's
// LightCurveIRS public interface (src/LightCurves/lcirs.h:30-116):
// constructor (a, b, th, m2, m3, sourceSize, lcLength, pointsPerRadius),
// getLCIRS / getLC over a straight trajectory, limb darkening, amoeba dump,
// and the light curve in lcVec.  The work runs on the GPU engine.
#pragma once

#include <cmath>
#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "lcirs.h"

// Limb-darkening model, the reference's LimbDarkeningModel
// (src/LimbDarkening/limbdarkeningmodel.h, .cc:8-49): a source pixel at
// radius r (in source radii) has brightness A + B sqrt(1 - r^2); intensityCoeff
// scales the ray sum so that a source of any profile has the flux of a
// uniform one.
struct LimbDarkeningModel {
  enum limbDarkeningModel { linear, linearNormalized, kurucz };
  limbDarkeningModel model;
  double intensityCoeff;

  // A = 0.6, B = 0.4
  LimbDarkeningModel() : model(linear), A_(0.6), B_(0.4) {
    intensityCoeff = 1.0 / (A_ + 2.0 / 3.0 * B_);
  }
  // normalised linear model: I0 (1 - v (1 - sqrt(1 - r^2))), I0 = 1/(1 - v/3)
  explicit LimbDarkeningModel(double v) : model(linearNormalized), intensityCoeff(1.0) {
    const double i0 = 1.0 / ((1.0 - v / 3.0));
    A_ = i0 * (1.0 - v);
    B_ = i0 * v;
  }
  // linear model with central intensity i0
  LimbDarkeningModel(double i0, double v) : model(linear), A_(i0 * (1.0 - v)), B_(i0 * v) {
    intensityCoeff = 1.0 / (i0 * (1.0 - v / 3.0));
  }
  double sourceBrightness(double r) const;
  double sourceBrightnessRSq(double rsq) const { return A_ + B_ * std::sqrt(1.0 - rsq); }
  double getParA() const { return A_; }
  double getParB() const { return B_; }

 private:
  double A_, B_;
};

inline double LimbDarkeningModel::sourceBrightness(double r) const {
  return A_ + B_ * std::sqrt(1.0 - r * r);
}

struct LightCurveIRS {
  LightCurveIRS(double a, double b, double th, double m2, double m3, double sourceSize,
                unsigned int lcLength = 100, long pointsPerRadius = 300);
  ~LightCurveIRS();

  // extended-source curve, n+1 points at t = i/n (lcirs.cc:103-191)
  void getLCIRS(std::complex<double> startPos, std::complex<double> endPos);
  // point-source curve, n points at t = i/(n-1) (lcbase.cc:40-52)
  void getLC(std::complex<double> startPos, std::complex<double> endPos);
  // "linear" -> v-normalised linear model; anything else -> A=0.6, B=0.4
  void setLimbDarkening(const std::string& model, double v);
  // the reference's setter (lcirs.cc:94-101): any of the model's forms
  void setLimbDarkeningModel(LimbDarkeningModel ldm);
  void setAmoebaPrintOut(bool amoebaPrintOut, std::string amoebaFilename,
                         std::string parFilename);

  std::vector<double> lcVec;          // n entries visible (copy_lc), n+1 stored
  std::vector<uint64_t> counts;       // rays per point of the last IRS curve
  std::vector<uint32_t> status;       // status bits per point
  std::vector<uint32_t> diag;         // fill-kernel diagnostics per point
  std::vector<int32_t> seeds;         // (n+1) x 64 x 2
  std::vector<int32_t> nseeds;        // n+1
  uint64_t stats[3] = {0, 0, 0};      // rays evaluated, FP64 rays, tiles
  unsigned int lastStatus = 0;
  int verbose = 1;
  int precision = 1;
  // warm-start chain of the image solver: 0 = one chain carried over the
  // object's life (the reference), k > 0 = restart every k points
  int chainPoints = 0;

  // lens and grid (host copies)
  double a, b, th, m1, m2, m3;
  double sourceRadius;
  unsigned int lcLength;
  long pointsPerRadius;
  double ldA, ldB, intensityCoeff;
  double grid[8];                     // corner x/y, top x/y, size, h, ampScale, N

  struct Impl;
  Impl* impl;

  // IRS over the trajectory; with extSeeds != nullptr the caller's seed
  // pixels ((n+1) x 64 x 2, counts in extN) replace the computed ones.
  void runFill(std::complex<double> s, std::complex<double> e, const int32_t* extSeeds,
               const int32_t* extN);
  // getLCIRS without the amoeba dump: joins concurrent calls of other objects
  // into one launch (same results as runFill)
  void runBatched(std::complex<double> s, std::complex<double> e);
  // results of an object kept off the GPU (parameters the lens set-up cannot
  // use, or a set-up without device memory): zero counts and magnifications,
  // its status (32 or 0x100) on every point
  void unusableResults();

 private:
  // A, B and the intensity coefficient into the object and its device lens;
  // the amplitude scale follows (lcirs.cc:94-101)
  void applyLimbDarkening(double A, double B, double intensity);
  void printOutLCParameters();
  bool amoebaPrintOut_ = false;
  std::string amoebaFilename_, parFilename_;
};
