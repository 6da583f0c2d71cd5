/*
 * gcvt_gb300.h -- C ABI of libgcvt_gb300.so, the GB300 (sm_103a) engine for
 * the centroidal Voronoi tessellation (CVT) hot path of Surface-Remesher.
 *
 * Conventions shared with the reference (source/gcvt.h:26-27):
 *   - a grid of size n holds pixel (x, y) at index y*n + x;
 *   - a site / label grid holds two int16 per pixel, x then y (the memory
 *     layout of CUDA's short2); MARKER (-32768) marks "no site";
 *   - density is float32, 0 outside the domain; the mask is one byte per
 *     pixel, nonzero = fixed (constraint) site.
 *
 * Every function returns GCVT_OK (0) or a GCVT_ERR_* status; none exits the
 * process.  The only exception is the reference's own C++ entry point gCVT()
 * declared at the end, which keeps the reference's void signature and exits
 * with a message on failure as the reference does (gcvt.cu:41-47).
 *
 * Pointers tagged `mem` are host pointers when mem == GCVT_MEM_HOST and
 * device pointers (on the context's device) when mem == GCVT_MEM_DEVICE.
 */
#ifndef GCVT_GB300_H
#define GCVT_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GCVT_MARKER (-32768)

enum gcvt_status {
    GCVT_OK = 0,
    GCVT_ERR_ARGUMENT = 1, /* null pointer or invalid enum value              */
    GCVT_ERR_SIZE = 2,     /* grid size outside the supported set             */
    GCVT_ERR_CUDA = 3,     /* a CUDA runtime call failed                      */
    GCVT_ERR_INPUT = 4,    /* invalid input data (see each call)              */
    GCVT_ERR_STATE = 5,    /* call order: no problem loaded                   */
    GCVT_ERR_ALLOC = 6     /* device or host allocation failed                */
};

enum gcvt_mem { GCVT_MEM_HOST = 0, GCVT_MEM_DEVICE = 1 };

typedef struct gcvt_ctx gcvt_ctx;

typedef struct {
    int iterations;        /* Lloyd iterations run so far (gcvtIterations)    */
    int levels;            /* resolution levels run by the last gcvt_ctx_run  */
    float omega;           /* current over-relaxation factor (pbaOmega)       */
    double energy;         /* CVT energy of the most recent iteration         */
    double sampled_energy; /* energy sampled by the schedule (iter % 10 == 0) */
} gcvt_run_info;

/* Launch choices of a context (gcvt_ctx_autotune, gcvt_ctx_set_tuning).
 * None changes any result: they only change how fast it is reached. */
typedef struct {
    int cell_blocks_per_sm; /* persistent Lloyd grid: blocks (warps) per SM, 0 = all that fit */
    int hint_slack;         /* a site's next window: 2 R + hint_slack pixels              */
    int jfa_tail_halo;      /* jump flooding: steps <= halo/2 fused in one launch (8/16/32;
                               0, the default: every step its own launch) */
    float lloyd_ms;         /* autotune: best time of one Lloyd iteration (ms)           */
    float jfa_ms;           /* autotune: best time of one jump-flooding labelling (ms)   */
    int cell_mode;          /* Lloyd cells: 0 = one site per warp up to 8192 sites, else
                               one per lane; 1 = one per lane; 2 = one per warp (up to
                               8192 sites; a learned step's two passes run one per lane) */
} gcvt_tuning;

/* Human-readable text of a status code. */
const char *gcvt_status_string(int status);

/* Library version as 10000*major + 100*minor + patch. */
int gcvt_version(void);

/* ---- context API ------------------------------------------------------- */

/* Create a context on the current CUDA device for grids up to n_max (a
 * multiple of 256 in [256, 8192]).  Device buffers live in the context;
 * nothing is allocated per call afterwards.  Replaces the per-call
 * allocation of gcvtInitialization (gcvt.cu:840-875). */
int gcvt_ctx_create(int n_max, gcvt_ctx **out);

/* Free the context and its device buffers (pbaCVDDeinitialization,
 * gcvt.cu:878-903). */
int gcvt_ctx_destroy(gcvt_ctx *ctx);

/* Run subsequent work on `stream` (a cudaStream_t); NULL restores the
 * context's own stream. */
int gcvt_ctx_set_stream(gcvt_ctx *ctx, void *stream);

/* Load a problem of size n: site grid (2*n*n int16), density (n*n float),
 * mask (n*n bytes, may be NULL for "no fixed sites").  Replaces
 * pba2DInitializeInput + the site upload (gcvt.cu:906-914, 1102).  The grid is
 * checked where it is used: calls that work at full resolution return
 * GCVT_ERR_INPUT when a non-MARKER pixel does not hold its own (x, y), and
 * gcvt_ctx_run checks the coarse grid that depth > 1 reads from the first
 * (n >> (depth-1))^2 entries (gcvt.cu:1099-1103). */
int gcvt_ctx_load(gcvt_ctx *ctx, int n, const int16_t *voronoi, const float *density,
                  const uint8_t *mask, int mem);

/* Label every pixel with its nearest current site (2*n*n int16), bit-
 * identical to pba2DCompute (gcvt.cu:967-978). */
int gcvt_ctx_label(gcvt_ctx *ctx, int16_t *labels, int mem);

/* Run `iterations` plain Lloyd iterations (label, centroid, update;
 * gcvt.cu:1114-1123) with the reference's omega schedule and no stop rule. */
int gcvt_ctx_iterate(gcvt_ctx *ctx, int iterations);

/* Full gCVT schedule from the loaded site grid (restarting from it, with a
 * fresh schedule): `depth` pyramid levels, the energy stop rule and the
 * maxIter cap (gcvt.cu:1087-1147).  Follow with gcvt_ctx_label for the final
 * label grid (gcvt.cu:1149-1152).  The loaded size must be a power of two. */
int gcvt_ctx_run(gcvt_ctx *ctx, int depth, int max_iter, gcvt_run_info *info);

/* Current site grid (2*n*n int16; sites hold their coordinates, MARKER
 * elsewhere) -- the state kernelUpdateSites leaves (gcvt.cu:1030-1033). */
int gcvt_ctx_sites(gcvt_ctx *ctx, int16_t *voronoi, int mem);

/* Per-site moments of the current sites without moving them: four n*n
 * double planes W, X, Y, E (density sum, x- and y-weighted sums, energy sum
 * rho*|site-p|^2) at each site pixel, 0 elsewhere.  The reference keeps the
 * same sums in pbaTotalW/X/Y after kernelScan_Y (gcvt.cu:1008-1023). */
int gcvt_ctx_moments(gcvt_ctx *ctx, double *out4, int mem);

/* Run `iterations` plain Lloyd iterations as separate launches, each
 * followed by a labelling pass, then as many jump-flooding labellings of the
 * final sites, and return in ms3 the mean duration (ms) of [0] one Lloyd
 * iteration (site list + cells), [1] one exact labelling pass (column
 * summaries + rows), [2] one jump-flooding labelling (its step launches and
 * fused tail) -- timed with CUDA events on the context's stream.  The sites advance as in gcvt_ctx_iterate.  No reference
 * counterpart: the reference times nothing (gcvt.cu:27 includes a timer
 * header it never uses). */
int gcvt_ctx_time_kernels(gcvt_ctx *ctx, int iterations, float *ms3);

/* Jump-flooding labels of the current sites (approximate; no reference
 * counterpart -- the reference labels exactly with PBA+): steps n/2 ... 1
 * (from the largest power of two <= n/2) plus one more step of 1, each pixel
 * taking the nearest of the nine labels
 * at offsets (dx, dy) * k, ties to the smaller x, then y.  labels (may be
 * NULL) receives the n*n label grid.  stats (may be NULL) receives, against
 * the exact labels of gcvt_ctx_label: [0] pixels whose label differs,
 * [1] pixels whose label is strictly farther than the exact one's, [2] n*n. */
int gcvt_ctx_jfa_label(gcvt_ctx *ctx, int16_t *labels, unsigned long long *stats, int mem);

/* Autotuner (no reference counterpart; the reference's fixed band tables,
 * gcvt.cu:842-847, are its closest analogue): times the Lloyd iteration for
 * persistent grids of 16, 24 and 32 blocks per SM and hint slacks 1, 2, 3,
 * and the jump-flooding labelling for fusion depths 8, 16 and 32, on the
 * loaded problem, restores every state it touched, and keeps the fastest
 * choices (written to *out if not NULL). */
int gcvt_ctx_autotune(gcvt_ctx *ctx, gcvt_tuning *out);

/* Set the launch choices directly. */
int gcvt_ctx_set_tuning(gcvt_ctx *ctx, const gcvt_tuning *tuning);

/* ---- learned steps ------------------------------------------------------
 * No reference counterpart.  A per-site MLP (10 -> 64 -> 64 -> 2, ReLU,
 * bfloat16 weights and activations, FP32 accumulation) maps a site's last
 * four Lloyd displacements -- the pending one (its cell's centroid minus the
 * site, not yet rounded) and the last three applied moves -- and the density
 * gradient over the density at the site, all in units of the mean cell
 * radius r, to a predicted displacement (in r) of the site towards the
 * converged tessellation.  A learned step proposes, in place of a plain
 * Lloyd step from the sites S, the jumped sites L = S + prediction; the
 * plain Lloyd iteration of L measures E(L) and the step stands only if
 * E(L) < E(S); otherwise the plain step's sites are taken, exactly as
 * without the jump -- the plain method is both fallback and judge.  An
 * accepted step costs no extra cell pass (the iteration of L is the next
 * Lloyd iteration); a rejected one costs one. */

/* Number of MLP parameters: W1[10][64], b1[64], W2[64][64], b2[64], W3[64][2], b3[2]. */
int gcvt_mlp_param_count(void);

/* Histories (and, with track_ids, per-site ids for training data) on or off;
 * allocates 16 (+8) bytes per pixel of n_max^2.  Takes effect at the next
 * level start (load, run, iterate). */
int gcvt_ctx_learning(gcvt_ctx *ctx, int enable, int track_ids);

/* The MLP parameters (FP32 host array of gcvt_mlp_param_count() floats). */
int gcvt_ctx_set_mlp(gcvt_ctx *ctx, const float *params, int count);

/* Features of the current sites in list order: 10 floats each (host), and
 * optionally their ids (track_ids) and pixel positions (x, y).  Writes up to
 * capacity sites; *count = the number of sites. */
int gcvt_ctx_features(gcvt_ctx *ctx, float *feat, int *ids, int *xy, int capacity, int *count);

/* `iterations` Lloyd iterations in rounds of jump_every - 1 plain iterations
 * and one learned step (two iterations when its jump stands, one when it
 * does not); the run ends after exactly `iterations` iterations, or earlier
 * at a target energy (gcvt_ctx_set_target_energy).  *tried / *kept (may be
 * NULL) count the jumps. */
int gcvt_ctx_iterate_learned(gcvt_ctx *ctx, int iterations, int jump_every, int *tried,
                             int *kept);

/* Time-to-energy runs: with target > 0 every later run of this context at
 * full resolution (gcvt_ctx_iterate, gcvt_ctx_iterate_learned, gcvt_ctx_run,
 * batches) also stops after the first iteration whose energy is at most
 * `target`; 0 turns it off.  No reference counterpart (gCVT's own stop rule,
 * gcvt.cu:1125-1142, is unchanged beside it). */
int gcvt_ctx_set_target_energy(gcvt_ctx *ctx, double target);

/* The MLP on host feature vectors (count x 10) -> predictions (count x 2):
 * tensor_cores != 0 runs layers 1 and 2 as tcgen05.mma (bfloat16 operands in
 * shared memory, FP32 accumulators in tensor memory), 0 on the CUDA cores
 * (the same bfloat16 rounding).  Jumps use the tensor-core path. */
int gcvt_mlp_forward(const float *params, const float *feat, int count, float *out,
                     int tensor_cores);

/* Train the MLP on the GPU (hand-written forward, backward and Adam kernels):
 * samples are count x 12 floats (10 features, 2 targets), mean squared error,
 * `steps` Adam steps of `batch` samples drawn by a hash of (seed, step,
 * slot).  params: initial FP32 parameters in, trained ones out; loss (may be
 * NULL) receives the mean loss of every step. */
int gcvt_mlp_train(const float *samples, long long count, float *params, int steps, int batch,
                   float lr, unsigned long long seed, float *loss);

/* One backward pass of the trainer without the Adam step: the gradient
 * (gcvt_mlp_param_count() floats, host) of the mean loss 0.5 |out - target|^2
 * over the `batch` samples gcvt_mlp_train draws at step `step` with `seed`,
 * with respect to the FP32 parameters `params`; the forward rounds weights
 * and activations to bfloat16 and the backward passes through those
 * roundings unchanged.  loss (may be NULL) receives the batch's mean loss.
 * Gradients are summed across blocks with FP32 atomics, so the last bits can
 * differ run to run. */
int gcvt_mlp_gradient(const float *samples, long long count, const float *params, int batch,
                      unsigned long long seed, int step, float *grad, float *loss);

/* Schedule state (iterations, omega, energies). */
int gcvt_ctx_info(gcvt_ctx *ctx, gcvt_run_info *info);

/* The CDT's input points from the current sites, as delaunayInput collects
 * them (delaunay.h:46-57) from the label grid: every site that is not fixed,
 * in x-major then y order, as the FP64 pair (x * scale + left,
 * y * scale + lower).  Writes min(count, capacity) points (2 doubles each)
 * to xy and the number of points to *count.  Computed on the GPU from the
 * site bitmap, so no label grid leaves the device. */
int gcvt_ctx_extract_points(gcvt_ctx *ctx, double scale, double left, double lower, double *xy,
                            int capacity, int *count, int mem);

/* The Delaunay triangulation of the current free sites (the points of
 * gcvt_ctx_extract_points, same order), computed on the GPU: the Delaunay
 * half of the CDT stage (main.cpp:229-236, gDel2D's GpuDel::compute on
 * delaunayInput's points) without the constraint points and segments.  Sites are lattice points, so the
 * predicates are exact integers; four or more co-circular sites are split by
 * a fixed symbolic perturbation (rank y * n + x).  Writes min(count,
 * capacity) triangles (3 point indices each, counter-clockwise) to
 * triangles and their number to *count; capacity 0 only counts.  Fewer than
 * three sites, or all collinear: no triangles.  GCVT_ERR_INPUT when a site
 * has more than 64 Delaunay neighbours. */
int gcvt_ctx_delaunay(gcvt_ctx *ctx, int32_t *triangles, int capacity, int *count, int mem);

/* The constrained Delaunay triangulation of the CDT stage (main.cpp:229-236:
 * gDel2D's GpuDel::compute, gDel2D/GPU/GpuDelaunay.cu:46, on
 * delaunayInput's points and segments, delaunay.h:30-79), on the GPU.
 * Points: the current free sites, in gcvt_ctx_extract_points' order
 * (indices 0 .. F-1), then the num_cpoints constraint points (FP64 pairs
 * in the frame x * scale + left, y * scale + lower of the sites; indices
 * F .. F + num_cpoints - 1).  segments: num_segments index pairs into that
 * list, each made an edge of the result (gDel2D's constraintVec; a segment
 * with points exactly inside it becomes the chain of edges between them).
 * Writes
 * min(count, capacity) triangles (3 point indices, counter-clockwise, each
 * starting at its smallest index, ordered by that index and then the
 * second) to triangles and their number to *count.  Predicates are exact:
 * sites on their pixel lattice, constraint points rounded to 2^-15 of a
 * pixel (snapped coordinates beyond 2^14 pixels from the grid are
 * rejected); co-circular points are split by the symbolic perturbation of
 * gcvt_ctx_delaunay, constraint points ranking above every site.
 * GCVT_ERR_INPUT (with *detail, may be NULL, set to a reason mask: 1
 * coordinate range, 2 a constraint point on another point, 16 two
 * segments crossing, or a bad index pair) when the input cannot be
 * triangulated so; GCVT_ERR_CUDA (detail 4, 8, 32, 64) when an internal
 * bound ran out.  Host-synchronous. */
int gcvt_ctx_cdt(gcvt_ctx *ctx, double scale, double left, double lower, const double *cpoints,
                 int num_cpoints, const int32_t *segments, int num_segments, int32_t *triangles,
                 int capacity, int *count, int *detail, int mem);

/* ---- batches: many charts, one launch pair per iteration ---------------
 * No reference counterpart: the reference runs one chart per gCVT call.  A
 * batch groups loaded contexts (any mix of sizes, one device); its
 * iterations run every member's Lloyd iteration in one site-list launch and
 * one persistent cell launch, the charts' 32-site groups handed out from one
 * work queue.  Each chart keeps its own schedule (omega, energy, stop), so a
 * chart's results are the same as from its own context.  Level 0 only
 * (depth 1); the members are read and written through their contexts
 * (gcvt_ctx_label, gcvt_ctx_sites, gcvt_ctx_info ...) once the batch call
 * has returned. */
typedef struct gcvt_batch gcvt_batch;

int gcvt_batch_create(int count, gcvt_ctx *const *charts, gcvt_batch **out);
int gcvt_batch_destroy(gcvt_batch *batch);
/* Stream for the batch's work (a cudaStream_t; NULL = its own stream). */
int gcvt_batch_set_stream(gcvt_batch *batch, void *stream);
/* `iterations` plain Lloyd iterations of every member (fixed count). */
int gcvt_batch_iterate(gcvt_batch *batch, int iterations);
/* The MLP parameters of the batch's learned steps (FP32 host array of
 * gcvt_mlp_param_count() floats); one network for every chart. */
int gcvt_batch_set_mlp(gcvt_batch *batch, const float *params, int count);
/* gcvt_ctx_iterate_learned over every member at once (each must have
 * learned steps enabled, gcvt_ctx_learning): per round one site-list and
 * one persistent cell launch per plain iteration, and for the learned step
 * one MLP launch over all charts' sites; every chart judges its own jumps,
 * so its result is its solo learned run's.  *tried / *kept sum the charts. */
int gcvt_batch_iterate_learned(gcvt_batch *batch, int iterations, int jump_every, int *tried,
                               int *kept);
/* gCVT's schedule on every member at depth 1: each chart runs until its own
 * stop rule or max_iter (gcvt.cu:1105-1147); infos (may be NULL) receives
 * one gcvt_run_info per member. */
int gcvt_batch_run(gcvt_batch *batch, int max_iter, gcvt_run_info *infos);

/* ---- one-call forms ---------------------------------------------------- */

/* gCVT with a status code: host buffers in, label grid out in `voronoi`
 * (gcvt.cu:1087-1156).  size is a power of two in [256, 8192]. */
int gcvt_compute(int16_t *voronoi, const float *density, const uint8_t *mask, int size,
                 int depth, int max_iter);

/* Initial sites as the reference's centroidalVoronoi makes them
 * (gcvt.h:76-122), host buffers: every mask pixel becomes a fixed site, every
 * other pixel MARKER, then `num` distinct free pixels are drawn by rejection
 * against the density from the reference's generator (gcvt.h:57-73).
 * state: the generator's four 64-bit words (z, w, jsr, jcong), updated; NULL
 * uses the library's own generator, which starts at zero like the
 * reference's unseeded globals and carries over between calls.  mask may be
 * NULL (no fixed sites).  Returns GCVT_ERR_ARGUMENT when num exceeds the free
 * pixels of positive density (the reference would loop forever) and
 * GCVT_ERR_INPUT when a draw budget of 1000 n^2 + 10^6 runs out. */
int gcvt_seed_sites(int16_t *voronoi, const float *density, const uint8_t *mask, int num,
                    int size, uint64_t *state);

/* centroidalVoronoi (gcvt.h:124-139) with a status code: gcvt_seed_sites
 * with the library's generator, then gcvt_compute; labels out in voronoi. */
int gcvt_centroidal_voronoi(int16_t *voronoi, float *density, const uint8_t *mask, int vertices,
                            int size, int depth, int max_iter);

/* Label a site grid once (pba2DCompute on a given grid). */
int gcvt_label_grid(const int16_t *sites, int16_t *labels, int n, int mem);

/* Rasterise a triangle mesh into a density grid, pixel for pixel equal to
 * kernelDiscretization (discretization.cu:57-85): pixel (tx, ty) samples
 * (tx*scale, ty*scale); the first triangle (index order) whose three FP64
 * barycentric weights are all >= 0 gives sum w_i * weight[v_i], else 0.
 * points: 2*num_point doubles, weight: num_point doubles, triangle:
 * 3*num_tri vertex indices, density: n*n floats; n a multiple of 16.
 * Replaces discretization_d (discretization.cu:87-120). */
int gcvt_rasterize(const double *points, const double *weight, int num_point,
                   const int32_t *triangle, int num_tri, float *density, double scale, int n,
                   int mem);

/* Lift parameter-space points onto the surface: recover() (recover.h:98-157).
 * The mesh: num_vertex vertices with parameter-space coordinates uv
 * (2 doubles each) and surface positions xyz (3 doubles each), num_tri faces
 * (3 vertex indices each, listed in the order vertices_around_face visits
 * them).  points: 2*num_points doubles, the CDT's input points -- the free
 * points first, then num_fixed constraint points, which are the mesh vertices
 * fixed_vertex[0..num_fixed) (delaunay.h:61-67).  For each free point: the
 * first face in index order whose FP64 barycentric weights (recover.h:30-52)
 * are all >= 0 (out_face, may be NULL) and the weighted sum of its vertices'
 * xyz (out_xyz, 3 doubles per point); a point that no face holds keeps the
 * previous point's face and weights as in the reference (out_face -1, out_xyz
 * the nearest earlier located free point's, NaN when there is none).  A
 * constraint point's out_xyz is its vertex's xyz (out_face -1).  keep[t]
 * (num_cdt bytes) is 1 when the centroid of CDT triangle t (3 point indices
 * in cdt) lies in a face, the reference's condition for emitting it.  Results
 * equal the reference's bit for bit.  GCVT_ERR_ARGUMENT on an index out of
 * range (the other outputs are then unspecified). */
int gcvt_lift(const double *uv, const double *xyz, int num_vertex, const int32_t *triangle,
              int num_tri, const double *points, int num_points, int num_fixed,
              const int32_t *fixed_vertex, const int32_t *cdt, int num_cdt, double *out_xyz,
              int32_t *out_face, uint8_t *keep, int mem);

/* Per-vertex density weights: weighting_vertices_with_area (weighting.h:38-97).
 * weight[v] = (sum of the surface areas of the faces at v) / (sum of their
 * parameter-space areas), both summed in face order; ratios above 1e10 take
 * the largest ratio that is not (0 when none is positive).  Same mesh arrays
 * as gcvt_lift; weight: num_vertex doubles. */
int gcvt_vertex_weights(const double *uv, const double *xyz, int num_vertex,
                        const int32_t *triangle, int num_tri, double *weight, int mem);

/* The same labelling for callers that cannot allocate device memory -- code
 * handed pre-allocated buffers by a host that owns all device memory, or a
 * loop that must not allocate after start-up.  No counterpart in the
 * reference.  `sites` and `labels` are device pointers (2*n*n int16 each) on
 * the current device; `stream` is a cudaStream_t (NULL: the legacy default
 * stream).  Nothing is allocated: the scratch lives in one static device
 * array sized for n <= 2048 (about 0.8 MB, held by every device that loads the
 * library until exit); larger n returns GCVT_ERR_SIZE.  Every call is
 * synchronous: it reads back an error flag and waits for `stream` before it
 * returns, so it cannot be captured into a CUDA graph, and it fails while
 * another thread captures in global mode.  Calls share the array, so calls
 * that overlap on the GPU race.
 * A site pixel that does not hold its own (x, y) is detected on the GPU while
 * the labelling runs: the call then returns GCVT_ERR_INPUT and the contents
 * of `labels` are unspecified (gcvt_label_grid returns before writing). */
int gcvt_label_grid_static(const int16_t *sites, int16_t *labels, int n, void *stream);

#ifdef __cplusplus
} /* extern "C" */

/* The reference's entry point, same signature and C++ symbol (gcvt.h:29,
 * gcvt.cu:1087), so source/main.cpp links against this library unchanged. */
extern void gCVT(short *Voronoi, float *density_d, bool *mask, int size, int depth,
                 int maxIter);

/* The reference's rasteriser entry point, same signature and C++ symbol
 * (discretization.h:66, discretization.cu:87). */
extern void discretization_d(double *points, double *weight, int num_point, int *triangle,
                             int num_tri, float *density, double scale, int n);
#endif

#endif /* GCVT_GB300_H */
