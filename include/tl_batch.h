/*
 * tl_batch.h - batched entry points of liblcirs.so (additive; no counterpart
 * in the reference, whose API computes one light curve per call through
 * lcirs_new/get_lc_irs, src/LightCurves/lcirs.cc:515-562).
 *
 * A batch holds many lenses and many straight trajectories (each on one of
 * the lenses).  One run computes, for every trajectory with length n, the
 * n+1 extended-source magnifications at t = i/n (the reference's
 * getLCIRS sampling, lcirs.cc:117-120), in one seeds launch and one
 * persistent fill launch.  Results are identical to calling get_lc_irs on
 * each lens object.
 *
 * Lens parameter rows (8 doubles): a, b, th, m2, m3, rho, ld_v, ppr, where
 * ld_v >= 0 selects the v-normalised linear limb darkening ("linear", v)
 * and ld_v < 0 the reference's default model (A = 0.6, B = 0.4).
 * Trajectory rows (4 doubles): x0, y0, x1, y1.  A trajectory of length
 * n = 0 is one source position (x0, y0) (one point, its own chain).
 *
 * Return values: >= 0 success (number of points for runs), < 0 error
 * (-1 bad argument, -2 CUDA error or host memory exhausted; no C++
 * exception leaves these functions).
 */
#ifndef TL_BATCH_H
#define TL_BATCH_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct tl_batch tl_batch;

tl_batch* tlb_new(void);
void tlb_delete(tl_batch* b);

/* Lens set-up on the GPU (critical curves, caustics, grids).  -1, before
 * any GPU work, if a row holds a non-finite value, rho <= 0 or rays per
 * radius outside 1..2^31-1. */
int tlb_set_lenses(tl_batch* b, int nlens, const double* params8);

/* Uploads trajectories (host arrays) into device memory and plans the
 * chunks; returns the number of points (sum of n+1). */
long tlb_set_trajectories(tl_batch* b, int ntraj, const double* traj4, const int32_t* lens_idx,
                          const uint32_t* n);

/* Runs on device-resident inputs.  phase: 1 seeds kernel, 2 fill kernel,
 * 3 both.  stream: a cudaStream_t or NULL for the engine's stream.  No host
 * synchronisation. */
int tlb_run_device(tl_batch* b, int phase, void* stream);

/* Copies results to host arrays of size (number of points); any pointer may
 * be NULL.  Synchronises the stream. */
int tlb_download(tl_batch* b, double* amp, uint64_t* counts, uint32_t* status, void* stream);

/* End to end from host buffers: set trajectories, run, download. */
long tlb_run_host(tl_batch* b, int ntraj, const double* traj4, const int32_t* lens_idx,
                  const uint32_t* n, double* amp, uint64_t* counts, uint32_t* status,
                  void* stream);

/* Totals of the last run: rays evaluated, rays evaluated in FP64, tiles
 * visited, accepted rays (4 x uint64). */
int tlb_stats(tl_batch* b, uint64_t* out4);

/* Ray-map precision (0 FP64 everywhere, 1 FP32 + FP64 guard band) and fill
 * launch shape: CTAs, log2 of the first block table's capacity in 32x8
 * tiles, threads per CTA, rows per frontier block (8, 16 or 32).  Values
 * <= 0 keep the current setting. */
int tlb_configure(tl_batch* b, int precision, int fill_ctas, int table_log2, int threads,
                  int block_h);

/* Warm-start chain of the image solver.  points > 0: the chain restarts
 * from the lens's construction state every `points` points of a curve, so
 * chunks of a curve run in parallel (default 4); the result is the one the
 * reference would give with the same restarts, and it differs from the
 * reference's single chain at points whose image decisions depend on the
 * last bits of the warm start.  points <= 0: one chain per curve, the
 * reference's order, bit-exact with it on every point (serial per curve).
 * Takes effect at the next tlb_set_trajectories. */
int tlb_set_chain(tl_batch* b, int points);

/* Point-source magnifications (reference get_lc sampling t = i/(n-1)) of the
 * current trajectories, n points each, written to amp (host). */
long tlb_point_lc(tl_batch* b, double* amp);

/* Autotuner: runs the seeds of the current trajectories, then times the
 * fill over their first sample_points points (all if <= 0) for five ways of
 * sharing the points among the fill's stages by predicted size (blocks of
 * 32 x 32 rays): one warp per point up to 7000, 3000 or 1500 blocks and a
 * team of 8 warps per larger point; one warp up to 7000 and the CTA fill for
 * larger points; the CTA fill alone.  Keeps the fastest for later runs of the
 * process if it beats the first (the default) by more than 5 %, else the
 * default.  chosen3 = {warp-fill threshold in blocks (0: CTA fill alone), 1 if
 * the team fill takes the larger points, points timed}; times_ms (5 floats,
 * may be NULL) the fill times in that order.  Results do not depend
 * on the choice (the filled sets are exact). */
int tlb_autotune(tl_batch* b, long sample_points, int32_t* chosen3, float* times_ms);

/* Sets how the fill's stages share the points, as tlb_autotune chooses (to
 * reapply a saved choice): warp_threshold_blocks > 0 sends each point up to
 * that many predicted blocks of 32 x 32 rays to one warp and larger points
 * to the team fill (team != 0) or the CTA fill; 0 sends every point to the
 * CTA fill.  Process-wide, like the autotuner's choice; results do not
 * depend on it.  -1 on a negative threshold. */
int tlb_set_fill_stages(tl_batch* b, int warp_threshold_blocks, int team);

/* Captures seeds + fill of the current trajectories (one warm run first,
 * so the captured run allocates nothing) into a CUDA graph on the engine's
 * stream.  tlb_graph_launch replays it on `stream` (NULL: the engine's);
 * the trajectories may be replaced through tlb_set_trajectories between
 * replays if their counts stay the same.  Results are read with
 * tlb_download as after tlb_run_device. */
int tlb_graph_capture(tl_batch* b);
int tlb_graph_launch(tl_batch* b, void* stream);

#ifdef __cplusplus
}
#endif
#endif
