// plan.h - host-side planning (no CUDA; included by the batched API and the
// object batcher, and compiled alone by the CPU tests): the exact warm-start
// chain in segments, the autotuner's choice among timed candidates, and the
// object batcher's gathering of concurrent callers.
//
// Segments: every curve's n+1 points are cut into nseg consecutive shares of
// ceil((n+1)/nseg) points (the last shares of a short curve may be empty).
// Segment s holds one job per curve that has points in it, in curve order,
// with the curve's index as its chain (the chain state goes from segment to
// segment), and lists those points' flat indices in the same order.
#pragma once

#include <stdint.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <vector>

namespace tl {

// Job: any type with int32_t fields traj, first, count, chain (SeedJob).
// jobs/list are filled in segment order; job0[s] and off[s] (nseg + 1
// entries) are where segment s starts in jobs and list; count[s] = the
// number of points of segment s.
template <class Job>
void plan_segments(int nseg, int ncurves, const int64_t* point_base, const uint32_t* n,
                   std::vector<Job>* jobs, std::vector<int32_t>* list,
                   std::vector<unsigned>* count, std::vector<int>* job0,
                   std::vector<int>* off) {
  jobs->clear();
  list->clear();
  count->assign((size_t)nseg, 0u);
  job0->assign((size_t)nseg + 1, 0);
  off->assign((size_t)nseg + 1, 0);
  for (int s = 0; s < nseg; s++) {
    (*job0)[s] = (int)jobs->size();
    (*off)[s] = (int)list->size();
    for (int i = 0; i < ncurves; i++) {
      const long np = (long)n[i] + 1;
      const long len = (np + nseg - 1) / nseg;
      const long first = (long)s * len;
      const long cnt = std::min(len, np - first);
      if (cnt <= 0) continue;
      Job j;
      j.traj = i;
      j.first = (int32_t)first;
      j.count = (int32_t)cnt;
      j.chain = i;   // the curve's chain, carried from segment to segment
      jobs->push_back(j);
      for (long q = 0; q < cnt; q++) list->push_back((int32_t)(point_base[i] + first + q));
    }
    (*count)[s] = (unsigned)(list->size() - (size_t)(*off)[s]);
  }
  (*job0)[nseg] = (int)jobs->size();
  (*off)[nseg] = (int)list->size();
}

// The autotuner's choice: ms[k] is candidate k's time (<= 0: it failed), and
// candidate 0 is the default.  The fastest candidate wins only if it beats
// the default by more than `margin` (a fraction): timings on a sample vary
// by a few per cent from run to run.  A failed default loses to the fastest
// candidate that ran; if none ran, the default stays.
inline int pick_candidate(const float* ms, int n, float margin) {
  int best = -1;
  for (int k = 0; k < n; k++)
    if (ms[k] > 0.f && (best < 0 || ms[k] < ms[best])) best = k;
  if (best < 0) return 0;
  if (ms[0] > 0.f && ms[best] >= (1.f - margin) * ms[0]) return 0;
  return best;
}

// The object batcher's gathering of concurrent callers (called by the
// leader with `lk` held on the mutex `cv` waits with): waits until requests
// stop arriving - a quiet gap of 3 ms, 15 ms while objects exist that have
// not called yet (`fresh`), with no object still in its constructor
// (`constructing`) - or max_ms have passed.  `arrivals` counts requests and
// is read under the lock.
template <class Lock, class Cv>
void gather_callers(Lock& lk, Cv& cv, const uint64_t& arrivals, const std::atomic<int>& fresh,
                    const std::atomic<int>& constructing, int max_ms = 300) {
  const auto t0 = std::chrono::steady_clock::now();
  uint64_t seen = arrivals;
  for (;;) {
    const int gap = fresh.load() > 0 ? 15 : 3;
    cv.wait_for(lk, std::chrono::milliseconds(gap));
    if ((arrivals == seen && constructing.load() == 0) ||
        std::chrono::steady_clock::now() - t0 > std::chrono::milliseconds(max_ms))
      break;
    seen = arrivals;
  }
}

}  // namespace tl
