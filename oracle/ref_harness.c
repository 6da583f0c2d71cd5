/*
 * ref_harness.c -- runs the reference's own CUDA kernels (TEST INFRASTRUCTURE
 * ONLY; never linked into the product).
 *
 * oracle/build_oracle.py compiles the reference's source/gcvt.cu and
 * source/discretization.cu, where they lie in the reference checkout, into
 * cubins under oracle/_ref/.  This file is a restatement of the reference's
 * host code (gcvt.cu:840-1156, discretization.cu:87-120) over the CUDA driver
 * API: it allocates the same buffers, launches the reference kernels with the
 * reference's grid/block shapes in the reference's order, and copies results
 * back.  Two deliberate deviations, both for memory safety of the harness:
 *   - pbaMargin gets 2*m1*n entries (kernelPropagateInterband writes up to
 *     index 2*m1*n - 1, gcvt.cu:133, while gcvt.cu:861 allocates m1*n);
 *   - the energy texture gets 1024 spare floats after n*n.
 * Kernel symbols are the C++ names of the reference's kernels.
 */
#include <cuda.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#define MK (-32768)

static CUcontext g_ctx;
static CUmodule g_mod, g_rmod;
static int g_ready;

enum {
    F_FILL, F_FDOWN, F_FUP, F_PROP, F_UPV, F_PROX, F_FWD, F_MERGE, F_D2S, F_COLOR,
    F_ZOOM, F_DSCALE, F_PREFIX, F_V1D, F_TOTX, F_SCANY, F_UPD, F_ENERGY, F_REDUCE, F_COUNT
};
static const char *kNames[F_COUNT] = {
    "_Z15kernelFillShortP6short2si",
    "_Z15kernelFloodDownP6short2S0_ii",
    "_Z13kernelFloodUpP6short2S0_ii",
    "_Z24kernelPropagateInterbandP6short2S0_ii",
    "_Z20kernelUpdateVerticalP6short2S0_S0_ii",
    "_Z21kernelProximatePointsP6short2S0_ii",
    "_Z27kernelCreateForwardPointersP6short2S0_ii",
    "_Z16kernelMergeBandsP6short2S0_S0_ii",
    "_Z24kernelDoubleToSingleListP6short2S0_S0_i",
    "_Z11kernelColorP6short2S0_i",
    "_Z12kernelZoomInP6short2S0_ii",
    "_Z20kernelDensityScalingPfS_i",
    "_Z28kernelComputeWeightedPrefixXPfS_S_S_i",
    "_Z15kernelVoronoi1DP6short2Pii",
    "_Z13kernelTotal_XP6short2PfS1_S1_S1_S1_S1_i",
    "_Z12kernelScan_YPsPfS0_S0_i",
    "_Z17kernelUpdateSitesPsPfS0_S0_S0_P6short2Pbif",
    "_Z16kernelCalcEnergyP6short2PfS1_i",
    "_Z12kernelReduceILj512EEvPfS0_j",
};
static CUfunction g_fn[F_COUNT];
static CUfunction g_raster;

#define CHK(x)                                                             \
    do {                                                                   \
        CUresult r_ = (x);                                                 \
        if (r_ != CUDA_SUCCESS) {                                          \
            const char *s_ = 0;                                            \
            cuGetErrorString(r_, &s_);                                     \
            fprintf(stderr, "ref_harness: %s -> %s (line %d)\n", #x,       \
                    s_ ? s_ : "?", __LINE__);                              \
            return -(int)r_ - 1000;                                        \
        }                                                                  \
    } while (0)

int refh_init(const char *gcvt_cubin, const char *raster_cubin) {
    if (g_ready) return 0;
    CUdevice dev;
    CHK(cuInit(0));
    CHK(cuDeviceGet(&dev, 0));
    CHK(cuDevicePrimaryCtxRetain(&g_ctx, dev));
    CHK(cuCtxSetCurrent(g_ctx));
    CHK(cuModuleLoad(&g_mod, gcvt_cubin));
    for (int i = 0; i < F_COUNT; ++i) CHK(cuModuleGetFunction(&g_fn[i], g_mod, kNames[i]));
    if (raster_cubin) {
        CHK(cuModuleLoad(&g_rmod, raster_cubin));
        CHK(cuModuleGetFunction(&g_raster, g_rmod,
                                "_Z20kernelDiscretizationPdS_PiiPfdi"));
    }
    g_ready = 1;
    return 0;
}

static int launch(int f, unsigned gx, unsigned gy, unsigned bx, unsigned by, unsigned smem,
                  void **args) {
    CHK(cuLaunchKernel(g_fn[f], gx, gy, 1, bx, by, 1, smem, 0, args, 0));
    return 0;
}

/* ---- the reference's globals (gcvt.cu:50-62) and tables (842-847) ---- */
typedef struct {
    CUdeviceptr tex[2], margin, density[10], prefixX[10], prefixY[10], prefixW[10];
    CUdeviceptr totalX, totalY, totalW, energyTex, mask;
    int texSize, buffer, scale;
    CUdeviceptr voronoi, temp;
    float omega;
} RefState;

static int m1_of(int n) {
    switch (n) { case 256: return 4; case 512: return 8; case 1024: return 16;
                 case 2048: return 32; case 4096: return 64; case 8192: return 128; }
    return 0;
}
static int m3_of(int n) {
    switch (n) { case 256: return 16; case 512: return 16; case 1024: return 16;
                 case 2048: return 8; case 4096: return 8; case 8192: return 4; }
    return 0;
}

/* gcvtInitialization (gcvt.cu:840-875) */
static int ref_alloc(RefState *s, int size) {
    memset(s, 0, sizeof *s);
    size_t nn = (size_t)size * size;
    s->texSize = size;
    CHK(cuMemAlloc(&s->tex[0], nn * 4));
    CHK(cuMemAlloc(&s->tex[1], nn * 4));
    CHK(cuMemAlloc(&s->margin, 2 * (size_t)m1_of(size) * size * 4));
    CHK(cuMemAlloc(&s->totalX, nn * 4));
    CHK(cuMemAlloc(&s->totalY, nn * 4));
    CHK(cuMemAlloc(&s->totalW, nn * 4));
    CHK(cuMemAlloc(&s->energyTex, nn * 4 + 4096));
    CHK(cuMemsetD8(s->energyTex, 0, nn * 4 + 4096));
    CHK(cuMemAlloc(&s->mask, nn));
    for (int i = 0; i < 10; ++i) {
        int ni = size >> i;
        if (ni < 256) break;
        size_t b = (size_t)ni * ni * 4;
        CHK(cuMemAlloc(&s->density[i], b));
        CHK(cuMemAlloc(&s->prefixX[i], b));
        CHK(cuMemAlloc(&s->prefixY[i], b));
        CHK(cuMemAlloc(&s->prefixW[i], b));
    }
    return 0;
}

static void ref_free(RefState *s) {
    cuMemFree(s->tex[0]); cuMemFree(s->tex[1]); cuMemFree(s->margin);
    cuMemFree(s->totalX); cuMemFree(s->totalY); cuMemFree(s->totalW);
    cuMemFree(s->energyTex); cuMemFree(s->mask);
    for (int i = 0; i < 10; ++i) {
        if (s->density[i]) cuMemFree(s->density[i]);
        if (s->prefixX[i]) cuMemFree(s->prefixX[i]);
        if (s->prefixY[i]) cuMemFree(s->prefixY[i]);
        if (s->prefixW[i]) cuMemFree(s->prefixW[i]);
    }
}

/* pba2DCompute (gcvt.cu:920-978) at the current texSize */
static int ref_pba(RefState *s) {
    int n = s->texSize, m1 = m1_of(n), m2 = 32, m3 = m3_of(n);
    int b = s->buffer, bs;
    CUdeviceptr t0 = s->tex[b], t1 = s->tex[1 ^ b];
    /* phase 1 */
    bs = n / m1;
    { void *a[] = {&t0, &t0, &n, &bs}; if (launch(F_FDOWN, n / 64, m1, 64, 1, 0, a)) return -1; }
    { void *a[] = {&t0, &t0, &n, &bs}; if (launch(F_FUP, n / 64, m1, 64, 1, 0, a)) return -1; }
    { void *a[] = {&t0, &s->margin, &n, &bs}; if (launch(F_PROP, n / 64, m1, 64, 1, 0, a)) return -1; }
    { void *a[] = {&t0, &s->margin, &t1, &n, &bs}; if (launch(F_UPV, n / 64, m1, 64, 1, 0, a)) return -1; }
    /* phase 2 */
    bs = n / m2;
    { void *a[] = {&t1, &t0, &n, &bs}; if (launch(F_PROX, n / 64, m2, 64, 1, 0, a)) return -1; }
    { void *a[] = {&t0, &t0, &n, &bs}; if (launch(F_FWD, n / 64, m2, 64, 1, 0, a)) return -1; }
    for (int noBand = m2; noBand > 1; noBand /= 2) {
        int bsz = n / noBand;
        void *a[] = {&t1, &t0, &t0, &n, &bsz};
        if (launch(F_MERGE, n / 64, noBand / 2, 64, 1, 0, a)) return -1;
    }
    { void *a[] = {&t1, &t0, &t0, &n}; if (launch(F_D2S, n / 64, n, 64, 1, 0, a)) return -1; }
    /* phase 3 */
    { void *a[] = {&t0, &t1, &n}; if (launch(F_COLOR, n / 64, 1, 64, m3, 0, a)) return -1; }
    s->voronoi = t1;
    s->temp = t0;
    s->buffer = 1 ^ b;
    return 0;
}

int refh_pba_label(const int16_t *sites, int16_t *labels, int n) {
    if (!g_ready || !m1_of(n)) return -1;
    RefState s;
    int rc = ref_alloc(&s, n);
    if (rc) return rc;
    size_t bytes = (size_t)n * n * 4;
    CHK(cuMemcpyHtoD(s.tex[0], sites, bytes));
    s.buffer = 0;
    rc = ref_pba(&s);
    if (!rc) {
        CHK(cuCtxSynchronize());
        CHK(cuMemcpyDtoH(labels, s.voronoi, bytes));
    }
    ref_free(&s);
    return rc;
}

/* pbaCVDCalcEnergy (gcvt.cu:1059-1083) on s->voronoi */
static int ref_energy(RefState *s, float *out) {
    int n = s->texSize;
    void *a[] = {&s->voronoi, &s->density[s->scale], &s->energyTex, &n};
    if (launch(F_ENERGY, n / 16, n / 16, 16, 16, 0, a)) return -1;
    unsigned cnt = (unsigned)n * n;
    int blocks;
    do {
        double c = ceil((1.0 * cnt) / 512);
        blocks = c < 32768 ? (int)c : 32768;
        void *r[] = {&s->energyTex, &s->energyTex, &cnt};
        if (launch(F_REDUCE, blocks, 1, 512, 1, 0, r)) return -1;
        cnt = blocks;
    } while (cnt > 512);
    if (cnt > 1) {
        void *r[] = {&s->energyTex, &s->energyTex, &cnt};
        if (launch(F_REDUCE, 1, 1, 512, 1, 0, r)) return -1;
    }
    float e;
    CHK(cuMemcpyDtoH(&e, s->energyTex, sizeof(float)));
    *out = e * powf(2.0f, (float)(s->scale * 2.0));
    return 0;
}

int refh_energy(const int16_t *labels, const float *density, int n, float *e) {
    if (!g_ready || !m1_of(n)) return -1;
    RefState s;
    int rc = ref_alloc(&s, n);
    if (rc) return rc;
    CHK(cuMemcpyHtoD(s.tex[0], labels, (size_t)n * n * 4));
    CHK(cuMemcpyHtoD(s.density[0], density, (size_t)n * n * 4));
    s.voronoi = s.tex[0];
    s.scale = 0;
    rc = ref_energy(&s, e);
    ref_free(&s);
    return rc;
}

/* pbaCVDComputeCentroid + pbaCVDUpdateSites (gcvt.cu:1008-1034) */
static int ref_centroid_update(RefState *s) {
    int n = s->texSize;
    CUdeviceptr pX = s->prefixX[s->scale], pY = s->prefixY[s->scale], pW = s->prefixW[s->scale];
    { void *a[] = {&s->voronoi, &s->temp, &n}; if (launch(F_V1D, n, 1, 64, 1, n * 2, a)) return -1; }
    { void *a[] = {&s->voronoi, &pX, &pY, &pW, &s->totalX, &s->totalY, &s->totalW, &n};
      if (launch(F_TOTX, n, 1, 64, 1, 0, a)) return -1; }
    { void *a[] = {&s->temp, &s->totalX, &s->totalY, &s->totalW, &n};
      if (launch(F_SCANY, n / 64, n / 64, 64, 1, 0, a)) return -1; }
    short mk = MK;
    { void *a[] = {&s->voronoi, &mk, &n}; if (launch(F_FILL, n / 16, n / 16, 16, 16, 0, a)) return -1; }
    { void *a[] = {&s->temp, &s->totalX, &s->totalY, &s->totalW, &s->density[s->scale],
                   &s->voronoi, &s->mask, &n, &s->omega};
      if (launch(F_UPD, n / 16, n / 16, 16, 16, 0, a)) return -1; }
    return 0;
}

/* One Lloyd step from a given site grid at level 0 with a given omega:
 * labels, the totals at site pixels (W, X, Y as the reference leaves them
 * after kernelScan_Y) and the updated site grid. */
int refh_lloyd_step(const int16_t *sites, const float *density, const uint8_t *mask, int n,
                    float omega, int16_t *labels_out, float *totals3, int16_t *sites_out) {
    if (!g_ready || !m1_of(n)) return -1;
    RefState s;
    int rc = ref_alloc(&s, n);
    if (rc) return rc;
    size_t nn = (size_t)n * n;
    CHK(cuMemcpyHtoD(s.tex[0], sites, nn * 4));
    CHK(cuMemcpyHtoD(s.density[0], density, nn * 4));
    CHK(cuMemcpyHtoD(s.mask, mask, nn));
    s.buffer = 0;
    s.scale = 0;
    s.omega = omega;
    int ns = 64 * 3 * 4;
    { void *a[] = {&s.prefixW[0], &s.prefixX[0], &s.prefixY[0], &s.density[0], &n};
      if (launch(F_PREFIX, n, 1, 64, 1, ns, a)) { ref_free(&s); return -1; } }
    rc = ref_pba(&s);
    if (!rc && labels_out) {
        CHK(cuCtxSynchronize());
        CHK(cuMemcpyDtoH(labels_out, s.voronoi, nn * 4));
    }
    if (!rc) rc = ref_centroid_update(&s);
    if (!rc) {
        CHK(cuCtxSynchronize());
        if (totals3) {
            CHK(cuMemcpyDtoH(totals3, s.totalW, nn * 4));
            CHK(cuMemcpyDtoH(totals3 + nn, s.totalX, nn * 4));
            CHK(cuMemcpyDtoH(totals3 + 2 * nn, s.totalY, nn * 4));
        }
        if (sites_out) CHK(cuMemcpyDtoH(sites_out, s.voronoi, nn * 4));
    }
    ref_free(&s);
    return rc;
}

/* gCVT (gcvt.cu:1087-1156).  fixed_iters > 0 runs exactly that many
 * iterations per level without the stop rule (the omega schedule still runs);
 * energies (may be NULL) receives each sampled energy in order (cap
 * max_energies); stats: [0] = iterations, [1] = number of energies,
 * [2] = the final omega (pbaOmega) as float bits.
 * times_ms (may be NULL): [0] = whole call, [1] = the Lloyd loop only. */
int refh_gcvt(int16_t *voronoi, const float *density, const uint8_t *mask, int size, int depth,
              int max_iter, int fixed_iters, float *energies, int max_energies, int *stats,
              float *times_ms) {
    if (!g_ready || !m1_of(size) || depth < 1) return -1;
    CUevent e0, e1, e2, e3;
    CHK(cuEventCreate(&e0, CU_EVENT_DEFAULT));
    CHK(cuEventCreate(&e1, CU_EVENT_DEFAULT));
    CHK(cuEventCreate(&e2, CU_EVENT_DEFAULT));
    CHK(cuEventCreate(&e3, CU_EVENT_DEFAULT));
    CHK(cuEventRecord(e0, 0));
    RefState s;
    int rc = ref_alloc(&s, size);
    if (rc) return rc;
    for (int i = 0; i < depth; ++i)
        if ((s.texSize >> i) < 256) { depth = i; break; }
    size_t nn = (size_t)size * size;
    CHK(cuMemcpyHtoD(s.density[0], density, nn * 4));
    CHK(cuMemcpyHtoD(s.mask, mask, nn));
    s.voronoi = s.tex[0];
    s.temp = s.tex[1];
    s.buffer = 0;
    for (int i = 1; i < depth; ++i) {
        int ni = size >> i;
        void *a[] = {&s.density[i - 1], &s.density[i], &ni};
        if (launch(F_DSCALE, ni / 16, ni / 16, 16, 16, 0, a)) return -1;
    }
    for (int i = 0; i < depth; ++i) {
        int ni = size >> i, ns = 64 * 3 * 4;
        void *a[] = {&s.prefixW[i], &s.prefixX[i], &s.prefixY[i], &s.density[i], &ni};
        if (launch(F_PREFIX, ni, 1, 64, 1, ns, a)) return -1;
        CHK(cuCtxSynchronize());
    }
    s.scale = 0;
    int iters = 0, ne = 0;
    s.texSize >>= depth;
    s.texSize <<= 1;
    CHK(cuMemcpyHtoD(s.voronoi, voronoi, (size_t)s.texSize * s.texSize * 4));
    s.texSize >>= 1;
    float Energy = 0.0f, lastEnergy = (float)1e18, diffEnergy, gradientEnergy;
    s.omega = 2.0f;
    CHK(cuEventRecord(e1, 0));
    for (s.scale = depth - 1; s.scale >= 0; --s.scale) {
        s.texSize <<= 1;
        int level_iters = 0;
        do {
            if (ref_pba(&s)) return -1;
            if (iters % 10 == 0) {
                if (ref_energy(&s, &Energy)) return -1;
                if (energies && ne < max_energies) energies[ne] = Energy;
                ++ne;
            }
            if (ref_centroid_update(&s)) return -1;
            ++iters;
            ++level_iters;
            if (iters % 10 == 0) {
                diffEnergy = lastEnergy - Energy;
                gradientEnergy = (float)((double)diffEnergy / 10.0);
                s.omega = (float)fmin(2.0, 1.0 + (double)diffEnergy);
                if (fixed_iters <= 0) {
                    if (s.scale) { if ((double)gradientEnergy < 3e-1) break; }
                    else if ((double)gradientEnergy < 1e-5) break;
                }
                lastEnergy = Energy;
            }
        } while (fixed_iters > 0 ? level_iters < fixed_iters : iters < max_iter);
        if (s.scale) {
            /* pbaCVDZoomIn (gcvt.cu:1036-1051) */
            int n2 = s.texSize << 1, one = 1, n = s.texSize;
            short mk = MK;
            { void *a[] = {&s.temp, &mk, &n2}; if (launch(F_FILL, n2 / 16, n2 / 16, 16, 16, 0, a)) return -1; }
            { void *a[] = {&s.voronoi, &s.temp, &n, &one}; if (launch(F_ZOOM, n / 16, n / 16, 16, 16, 0, a)) return -1; }
            s.buffer = 1 ^ s.buffer;
            CUdeviceptr t = s.voronoi; s.voronoi = s.temp; s.temp = t;
        }
    }
    if (ref_pba(&s)) return -1;
    CHK(cuEventRecord(e2, 0));
    CHK(cuCtxSynchronize());
    CHK(cuMemcpyDtoH(voronoi, s.voronoi, nn * 4));
    ref_free(&s);
    CHK(cuEventRecord(e3, 0));
    CHK(cuEventSynchronize(e3));
    if (times_ms) {
        CHK(cuEventElapsedTime(&times_ms[0], e0, e3));
        CHK(cuEventElapsedTime(&times_ms[1], e1, e2));
    }
    cuEventDestroy(e0); cuEventDestroy(e1); cuEventDestroy(e2); cuEventDestroy(e3);
    if (stats) {
        stats[0] = iters;
        stats[1] = ne;
        memcpy(&stats[2], &s.omega, sizeof(float)); /* pbaOmega at the end */
    }
    return 0;
}

/* discretization_d (discretization.cu:87-120) */
int refh_rasterize(const double *points, const double *weight, int num_point,
                   const int32_t *triangle, int num_tri, float *density, double scale, int n,
                   float *time_ms) {
    if (!g_ready || !g_raster) return -1;
    CUdeviceptr pd, wd, td, dd;
    CHK(cuMemAlloc(&pd, (size_t)num_point * 16));
    CHK(cuMemAlloc(&wd, (size_t)num_point * 8));
    CHK(cuMemAlloc(&td, (size_t)num_tri * 12));
    CHK(cuMemAlloc(&dd, (size_t)n * n * 4));
    CHK(cuMemcpyHtoD(pd, points, (size_t)num_point * 16));
    CHK(cuMemcpyHtoD(wd, weight, (size_t)num_point * 8));
    CHK(cuMemcpyHtoD(td, triangle, (size_t)num_tri * 12));
    CUevent a0, a1;
    CHK(cuEventCreate(&a0, CU_EVENT_DEFAULT));
    CHK(cuEventCreate(&a1, CU_EVENT_DEFAULT));
    CHK(cuEventRecord(a0, 0));
    void *args[] = {&pd, &wd, &td, &num_tri, &dd, &scale, &n};
    CHK(cuLaunchKernel(g_raster, n / 16, n / 16, 1, 16, 16, 1, 0, 0, args, 0));
    CHK(cuEventRecord(a1, 0));
    CHK(cuEventSynchronize(a1));
    if (time_ms) CHK(cuEventElapsedTime(time_ms, a0, a1));
    CHK(cuMemcpyDtoH(density, dd, (size_t)n * n * 4));
    cuMemFree(pd); cuMemFree(wd); cuMemFree(td); cuMemFree(dd);
    cuEventDestroy(a0); cuEventDestroy(a1);
    return 0;
}
