// lcirs.hpp - C++ class view of liblcirs.so, mirroring the reference's
// LightCurveIRS public interface (src/LightCurves/lcirs.h:30-116):
// constructor (a, b, th, m2, m3, sourceSize, lcLength, pointsPerRadius),
// getLCIRS / getLC over a straight trajectory, limb darkening, amoeba dump,
// and the light curve in lcVec.  The work runs on the GPU engine.
#pragma once

#include <complex>
#include <cstdint>
#include <string>
#include <vector>

#include "lcirs.h"

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

 private:
  void printOutLCParameters();
  bool amoebaPrintOut_ = false;
  std::string amoebaFilename_, parFilename_;
};
