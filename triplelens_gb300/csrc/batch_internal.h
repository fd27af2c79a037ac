// batch_internal.h - the batch object behind include/tl_batch.h, shared by
// batch_abi.cu and surrogate.cu.
#pragma once

#include <cstdint>
#include <vector>

#include "engine.h"
#include "engine_host.h"

struct tl_batch {
  int nlens = 0;
  tl::DevBuf specs, lenses, cc, ca;
  std::vector<tl::DevLens> hlens;
  int ntraj = 0;
  long npoints = 0;
  int njobs = 0;
  tl::DevBuf trajs, jobs, points, seeds, out, amp, trials, scan, prep;
  int nscan = 0;                 // exact chain: point chunks of the scan/prep
  // exact chain in segments (tlb_run_device phase 4): segment s holds one
  // job per curve over its s-th share of points; its points are listed in
  // seglist[segoff[s] .. segoff[s+1]) and counted in segn[s] (device)
  int nseg = 0;
  std::vector<int> segoff, segjob0;
  tl::DevBuf segjobs, seglist, segn, chains;
  std::vector<tl::Traj> htraj;
  int precision = 1;
  int chain = tl::kChainChunk;   // warm-start chain length (<= 0: whole curve)
  uint64_t stats[4] = {0, 0, 0, 0};
  // captured seeds + fill of the current trajectories (tlb_graph_capture)
  cudaGraphExec_t graph = nullptr;
  long graph_points = 0;
  int graph_jobs = 0;
};
