/*
 * gcvt_oracle.h -- CPU oracle for the CVT hot path (TEST INFRASTRUCTURE ONLY).
 *
 * This library restates, on the host, the algorithm of the reference's gCVT
 * (source/gcvt.cu) and rasteriser (source/discretization.cu).  The tests
 * compare the CUDA path with it, and it is the CPU baseline timed beside it; the product
 * library never links or calls it.  Only tests/, __graft_entry__.smoke() and
 * bench.py's cpu_baseline / --impl reference legs may load it.
 *
 * Grid conventions (gcvt.h:26-27): pixel (x, y) lives at index y*n + x; a
 * label/site grid holds two int16 per pixel (x then y, the memory layout of
 * the reference's short2); MARKER = -32768 marks "no site".
 */
#ifndef GCVT_ORACLE_H
#define GCVT_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define ORC_MARKER (-32768)

/* Labelling ----------------------------------------------------------------*/

/* Literal restatement of PBA+ as launched by pba2DCompute (gcvt.cu:77-479,
 * 920-978) with the band tables of gcvtInitialization (gcvt.cu:842-847).
 * sites: 2*n*n int16 (site pixels hold their own (x, y), all others MARKER).
 * labels: 2*n*n int16 output.  n must be a power of two in [256, 8192].
 * Returns 0 on success, negative on bad arguments. */
int orc_pba_label(const int16_t *sites, int16_t *labels, int n);

/* Pointwise restatement of the same labelling (see gcvt_oracle.c for the
 * derivation): nearest site in Euclidean distance; ties go to the smaller
 * site x; a remaining mirror pair (x, r-k)/(x, r+k) goes to the lower site
 * (r+k) only when it lies in the same 64-row band as the pixel's row r.
 * Computed with the separable column pass + exact lower envelope.  Any n in
 * [1, 16384]. */
int orc_spec_label(const int16_t *sites, int16_t *labels, int n);

/* Same rule by brute force over all sites (O(n^2 * sites)); tiny cases. */
int orc_brute_label(const int16_t *sites, int16_t *labels, int n);

/* Lloyd loop ----------------------------------------------------------------*/

enum {
    ORC_MODE_FAITHFUL = 0, /* FP32 prefix-sum centroids and FP32 energy in
                              the reference's operation order (gcvt.cu:497-
                              832), including its energy-reduction quirk. */
    ORC_MODE_EXACT = 1     /* FP64 moments/energy straight from the labels;
                              the same integer update rule.  This is the
                              contract of the GB300 path. */
};

typedef struct {
    int iterations;       /* Lloyd iterations executed (gcvtIterations)    */
    int levels;           /* resolution levels run (after depth clamping)   */
    double last_energy;   /* last energy sampled by the schedule            */
    float omega;          /* over-relaxation factor at exit                 */
} orc_stats;

/* Restatement of gCVT (gcvt.cu:1087-1156): host buffers in, label grid out.
 * voronoi: 2*size*size int16 in/out; density: size*size float; mask: size*size
 * bytes (nonzero = fixed site).  fixed_iters > 0 replaces the energy stop rule
 * by exactly that many iterations (omega schedule unchanged).  threads <= 0
 * uses all OpenMP threads.  Returns 0 or a negative error. */
int orc_gcvt(int16_t *voronoi, const float *density, const uint8_t *mask,
             int size, int depth, int max_iter, int mode, int fixed_iters,
             int threads, orc_stats *stats);

/* One Lloyd step on a site grid at level resolution n (no schedule): label,
 * moments, update.  Exposes the per-iteration pieces for parity tests.
 *   sites_in  : 2*n*n int16 site grid
 *   labels_out: 2*n*n int16 labels of sites_in (may be NULL)
 *   moments   : 3*n*n double (W, X, Y at each site pixel, 0 elsewhere; may be NULL)
 *   energy    : sum(rho * d^2) / n^2 in FP64 (may be NULL)
 *   sites_out : 2*n*n int16 updated site grid (may be NULL)
 * Uses ORC_MODE_EXACT arithmetic. */
int orc_lloyd_step(const int16_t *sites_in, const float *density,
                   const uint8_t *mask, int n, float omega,
                   int16_t *labels_out, double *moments, double *energy,
                   int16_t *sites_out);

/* One faithful step (the reference's FP32 prefix-sum centroids): labels,
 * W/X/Y totals (3*n*n floats, valid at site pixels) and updated sites. */
int orc_faithful_step(const int16_t *sites_in, const float *density, const uint8_t *mask, int n,
                      float omega, int16_t *labels_out, float *totals3, int16_t *sites_out);

/* Faithful FP32 energy of a label grid (kernelCalcEnergy + kernelReduce
 * sequence, gcvt.cu:788-832, 1059-1083), scale factor 4^level included. */
float orc_faithful_energy(const int16_t *labels, const float *density, int n,
                          int level);

/* Rasteriser -----------------------------------------------------------------*/

/* Restatement of kernelDiscretization (discretization.cu:32-85): pixel (tx,
 * ty) samples (tx*scale, ty*scale); the first triangle in index order whose
 * three barycentric weights are all >= 0 gives density = sum w_i*weight[v_i]
 * (FP64, stored as float); no triangle gives 0. */
int orc_rasterize(const double *points, const double *weight, int num_point,
                  const int32_t *triangle, int num_tri, float *density,
                  double scale, int n, int threads);

/* Lift and weighting (recover.h, weighting.h) --------------------------------*/

/* Restatement of recover (recover.h:98-157) with locate (recover.h:64-85) and
 * barycentric (recover.h:30-52), host arithmetic (no fused multiply-add):
 * free points [0, num_points - num_fixed) are located by testing every face
 * in index order; an unlocated point keeps the previous location (NaN lift
 * when there is none); constraint points take xyz[fixed_vertex[k]]; keep[t]
 * says whether CDT triangle t's centroid locates.  out_face may be NULL. */
int orc_lift(const double *uv, const double *xyz, int num_vertex, const int32_t *triangle,
             int num_tri, const double *points, int num_points, int num_fixed,
             const int32_t *fixed_vertex, const int32_t *cdt, int num_cdt, double *out_xyz,
             int32_t *out_face, uint8_t *keep, int threads);

/* Restatement of weighting_vertices_with_area (weighting.h:38-97) with CGAL's
 * face_area for the surface areas. */
int orc_vertex_weights(const double *uv, const double *xyz, int num_vertex,
                       const int32_t *triangle, int num_tri, double *weight);

/* Seeding (gcvt.h:56-122) ----------------------------------------------------*/

/* putConstrains + randomPoints with the reference's Marsaglia generator in its
 * LP64 form (unsigned long = 64 bits).  seed < 0 keeps the generator's zero
 * initial state (the reference never calls randinit); otherwise randinit(seed).
 * Returns the number of sites placed or a negative error. */
int orc_seed_sites(int16_t *voronoi, const float *density, const uint8_t *mask,
                   int num, int size, long long seed);

#ifdef __cplusplus
}
#endif

#endif
