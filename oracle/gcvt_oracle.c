/*
 * gcvt_oracle.c -- CPU oracle for the CVT hot path.  TEST INFRASTRUCTURE ONLY:
 * what the tests compare the CUDA path with, and the CPU baseline timed beside it.  Never
 * linked into the product library.
 *
 * Every function cites the reference file:line it restates.  "Reference" means
 * orzzzjq/Surface-Remesher, paths relative to its repository root.
 *
 * Parallelism: OpenMP over independent columns / bands / rows only, so every
 * result is identical for any thread count.
 */
#include "gcvt_oracle.h"

#include <math.h>
#include <stddef.h>
#include <stdlib.h>
#include <string.h>
#include <limits.h>
#ifdef _OPENMP
#include <omp.h>
#endif

typedef struct { int16_t x, y; } s2;

#define MK ORC_MARKER
#define IDX(x, y, n) ((ptrdiff_t)(y) * (ptrdiff_t)(n) + (ptrdiff_t)(x))

static inline s2 S2(int x, int y) { s2 r; r.x = (int16_t)x; r.y = (int16_t)y; return r; }
static inline int iabs(int v) { return v < 0 ? -v : v; }
static inline int imax(int a, int b) { return a > b ? a : b; }

/* Band tables of gcvtInitialization (gcvt.cu:842-847). */
static int tab_m1(int n) {
    switch (n) { case 256: return 4; case 512: return 8; case 1024: return 16;
                 case 2048: return 32; case 4096: return 64; case 8192: return 128; }
    return 0;
}
static int tab_m2(int n) { return tab_m1(n) ? 32 : 0; }
static int tab_m3(int n) {
    switch (n) { case 256: return 16; case 512: return 16; case 1024: return 16;
                 case 2048: return 8; case 4096: return 8; case 8192: return 4; }
    return 0;
}

/* ============================================================================
 * PBA+ literal restatement (gcvt.cu:77-479).  Each CUDA thread of the
 * reference owns one (column, band); here the same per-thread sequential
 * loops run with the thread state held in arrays, bands in parallel.
 * ==========================================================================*/

/* kernelFloodDown (gcvt.cu:77-95), in place. */
static void pba_flood_down(s2 *tex, int n, int bs, int m1) {
    #pragma omp parallel
    {
        s2 *p1 = (s2 *)malloc(sizeof(s2) * (size_t)n);
        #pragma omp for schedule(static)
        for (int b = 0; b < m1; ++b) {
            for (int tx = 0; tx < n; ++tx) p1[tx] = S2(MK, MK);
            for (int i = 0; i < bs; ++i) {
                s2 *row = tex + IDX(0, b * bs + i, n);
                for (int tx = 0; tx < n; ++tx) {
                    s2 p2 = row[tx];
                    if (p2.x != MK) p1[tx] = p2;
                    row[tx] = p1[tx];
                }
            }
        }
        free(p1);
    }
}

/* kernelFloodUp (gcvt.cu:97-119), in place; strict '<' keeps the carried
 * (lower) site on a tie. */
static void pba_flood_up(s2 *tex, int n, int bs, int m1) {
    #pragma omp parallel
    {
        s2 *p1 = (s2 *)malloc(sizeof(s2) * (size_t)n);
        #pragma omp for schedule(static)
        for (int b = 0; b < m1; ++b) {
            int ty = (b + 1) * bs - 1;
            for (int tx = 0; tx < n; ++tx) p1[tx] = S2(MK, MK);
            for (int i = 0; i < bs; ++i) {
                s2 *row = tex + IDX(0, ty - i, n);
                for (int tx = 0; tx < n; ++tx) {
                    int dist1 = iabs(p1[tx].y - ty + i);
                    s2 p2 = row[tx];
                    int dist2 = iabs(p2.y - ty + i);
                    if (dist2 < dist1) p1[tx] = p2;
                    row[tx] = p1[tx];
                }
            }
        }
        free(p1);
    }
}

/* kernelPropagateInterband (gcvt.cu:121-170).  margin holds 2*m1*n entries:
 * the reference writes bottom margins at tid + n*n/bandSize (gcvt.cu:133),
 * i.e. up to 2*m1*n, although gcvtInitialization allocates m1*n
 * (gcvt.cu:861). */
static void pba_propagate_interband(const s2 *in, s2 *out, int n, int bs, int m1) {
    ptrdiff_t inc = (ptrdiff_t)bs * n;
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < m1; ++b) {
        for (int tx = 0; tx < n; ++tx) {
            int ty = b * bs;
            ptrdiff_t topId = IDX(tx, ty, n);
            ptrdiff_t bottomId = IDX(tx, ty + bs - 1, n);
            ptrdiff_t tid = (ptrdiff_t)b * n + tx;
            ptrdiff_t bid = tid + (ptrdiff_t)n * n / bs;
            s2 pixel = in[topId];
            int myDist = iabs(pixel.y - ty);
            out[tid] = pixel;
            for (ptrdiff_t nid = bottomId - inc; nid >= 0; nid -= inc) {
                pixel = in[nid];
                if (pixel.x != MK) {
                    int nDist = iabs(pixel.y - ty);
                    if (nDist < myDist) out[tid] = pixel;
                    break;
                }
            }
            ty = ty + bs - 1;
            pixel = in[bottomId];
            myDist = iabs(pixel.y - ty);
            out[bid] = pixel;
            ptrdiff_t nid = topId + inc;
            for (int ny = ty + 1; ny < n; ny += bs, nid += inc) {
                pixel = in[nid];
                if (pixel.x != MK) {
                    int nDist = iabs(pixel.y - ty);
                    if (nDist < myDist) out[bid] = pixel;
                    break;
                }
            }
        }
    }
}

/* kernelUpdateVertical (gcvt.cu:172-216): merge with margins (strict '<'),
 * write transposed with (x, y) swapped. */
static void pba_update_vertical(const s2 *color, const s2 *margin, s2 *out, int n,
                                int bs, int m1) {
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < m1; ++b) {
        for (int tx = 0; tx < n; ++tx) {
            s2 top = margin[(ptrdiff_t)b * n + tx];
            s2 bottom = margin[(ptrdiff_t)(b + m1) * n + tx];
            for (int ty = b * bs; ty < (b + 1) * bs; ++ty) {
                s2 pixel = color[IDX(tx, ty, n)];
                int myDist = iabs(pixel.y - ty);
                int dist = iabs(top.y - ty);
                if (dist < myDist) { myDist = dist; pixel = top; }
                dist = iabs(bottom.y - ty);
                if (dist < myDist) pixel = bottom;
                out[IDX(ty, tx, n)] = S2(pixel.y, pixel.x);
            }
        }
    }
}

/* dominate (gcvt.cu:219-224): 64-bit exact lower-envelope test. */
static inline int pba_dominate(long long x1, long long y1, long long x2, long long y2,
                               long long x3, long long y3, long long x0) {
    long long k1 = y2 - y1, k2 = y3 - y2;
    return (k1 * (y1 + y2) + (x2 - x1) * ((x1 + x2) - (x0 << 1))) * k2 >
           (k2 * (y2 + y3) + (x3 - x2) * ((x2 + x3) - (x0 << 1))) * k1;
}

/* kernelProximatePoints (gcvt.cu:227-261). */
static void pba_proximate_points(const s2 *input, s2 *stack, int n, int bs, int m2) {
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < m2; ++b) {
        for (int tx = 0; tx < n; ++tx) {
            int ty = b * bs;
            ptrdiff_t id = IDX(tx, ty, n);
            int lasty = -1;
            s2 last1 = S2(0, -1), last2 = S2(0, -1), current;
            for (int i = 0; i < bs; i++, id += n) {
                current = input[id];
                if (current.x != MK) {
                    while (last2.y >= 0) {
                        if (!pba_dominate(last1.x, last2.y, last2.x, lasty, current.x,
                                          current.y, tx))
                            break;
                        lasty = last2.y; last2 = last1;
                        if (last1.y >= 0) last1 = stack[IDX(tx, last1.y, n)];
                    }
                    last1 = last2; last2 = S2(current.x, lasty); lasty = current.y;
                    stack[id] = last2;
                }
            }
            if (lasty != ty + bs - 1) stack[IDX(tx, ty + bs - 1, n)] = S2(MK, lasty);
        }
    }
}

/* kernelCreateForwardPointers (gcvt.cu:263-291), in place. */
static void pba_forward_pointers(s2 *tex, int n, int bs, int m2) {
    #pragma omp parallel for schedule(static)
    for (int b = 0; b < m2; ++b) {
        for (int tx = 0; tx < n; ++tx) {
            int ty = (b + 1) * bs - 1;
            ptrdiff_t id = IDX(tx, ty, n);
            int lasty = -1, nexty;
            s2 current = tex[id];
            nexty = (current.x == MK) ? current.y : ty;
            for (int i = 0; i < bs; i++, id -= n)
                if (ty - i == nexty) {
                    current = S2(lasty, tex[id].y);
                    tex[id] = current;
                    lasty = nexty;
                    nexty = current.y;
                }
            if (lasty != ty - bs + 1) tex[id + n] = S2(lasty, MK);
        }
    }
}

/* kernelMergeBands (gcvt.cu:293-410); link and output are the same buffer. */
static void pba_merge_bands(const s2 *color, s2 *link, int n, int bs, int npairs) {
    #define CL(yy) S2(color[IDX(tx, (yy), n)].x, link[IDX(tx, (yy), n)].y)
    #define LC(yy) S2(link[IDX(tx, (yy), n)].x, color[IDX(tx, (yy), n)].x)
    #pragma omp parallel for schedule(static)
    for (int p = 0; p < npairs; ++p) {
        for (int tx = 0; tx < n; ++tx) {
            int band1 = p * 2, band2 = band1 + 1;
            int firsty, lasty;
            s2 last1 = S2(0, -1), last2, current;
            lasty = band2 * bs - 1;
            last2 = CL(lasty);
            if (last2.x == MK) {
                lasty = last2.y;
                if (lasty >= 0) last2 = CL(lasty);
                else last2 = S2(MK, MK);
            }
            if (last2.y >= 0) last1 = CL(last2.y);
            firsty = band2 * bs;
            current = LC(firsty);
            if (current.y == MK) {
                firsty = current.x;
                if (firsty >= 0) current = LC(firsty);
                else current = S2(MK, MK);
            }
            int top = 0;
            while (top < 2 && current.y >= 0) {
                while (last2.y >= 0) {
                    if (!pba_dominate(last1.x, last2.y, last2.x, lasty, current.y, firsty, tx))
                        break;
                    lasty = last2.y; last2 = last1;
                    top--;
                    if (last1.y >= 0) last1 = CL(last1.y);
                }
                link[IDX(tx, firsty, n)] = S2(current.x, lasty);
                if (lasty >= 0) link[IDX(tx, lasty, n)] = S2(firsty, last2.y);
                last1 = last2; last2 = S2(current.y, lasty); lasty = firsty;
                firsty = current.x;
                top = imax(1, top + 1);
                if (firsty >= 0) current = LC(firsty);
                else current = S2(MK, MK);
            }
            firsty = band1 * bs;
            lasty = band2 * bs;
            current = link[IDX(tx, firsty, n)];
            if (current.y == MK && current.x < 0) {
                last1 = link[IDX(tx, lasty, n)];
                if (last1.y == MK) current.x = last1.x;
                else current.x = (int16_t)lasty;
                link[IDX(tx, firsty, n)] = current;
            }
            firsty = band1 * bs + bs - 1;
            lasty = band2 * bs + bs - 1;
            current = link[IDX(tx, lasty, n)];
            if (current.x == MK && current.y < 0) {
                last1 = link[IDX(tx, firsty, n)];
                if (last1.x == MK) current.y = last1.y;
                else current.y = (int16_t)firsty;
                link[IDX(tx, lasty, n)] = current;
            }
        }
    }
    #undef CL
    #undef LC
}

/* kernelDoubleToSingleList (gcvt.cu:412-419), in place on link. */
static void pba_double_to_single(const s2 *color, s2 *link, int n) {
    ptrdiff_t nn = (ptrdiff_t)n * n;
    #pragma omp parallel for schedule(static)
    for (ptrdiff_t id = 0; id < nn; ++id) link[id] = S2(color[id].x, link[id].y);
}

/* kernelColor (gcvt.cu:421-479): each of the m3 threads of a column walks the
 * stack on its own; '>' break lets a tie advance to the lower-index entry.
 * Writes the transposed-back label grid.  A column whose stack is empty (no
 * site anywhere) makes the reference read before the texture (lasty = -1);
 * here that column is labelled MARKER. */
static void pba_color(const s2 *input, s2 *out, int n, int m3) {
    #pragma omp parallel for schedule(static)
    for (int tx = 0; tx < n; ++tx) {
        for (int tid = 0; tid < m3; ++tid) {
            int lasty = n - 1;
            s2 last1 = S2(0, -1), last2 = input[IDX(tx, lasty, n)];
            if (last2.x == MK) {
                lasty = last2.y;
                if (lasty < 0) {
                    for (int ty = n - 1 - tid; ty >= 0; ty -= m3) out[IDX(ty, tx, n)] = S2(MK, MK);
                    continue;
                }
                last2 = input[IDX(tx, lasty, n)];
            }
            if (last2.y >= 0) last1 = input[IDX(tx, last2.y, n)];
            int nstep = n / 64;
            for (int step = 0; step < nstep; ++step) {
                int y_start = n - step * 64 - 1;
                int y_end = n - (step + 1) * 64;
                for (int ty = y_start - tid; ty >= y_end; ty -= m3) {
                    int dx = last2.x - tx, dy = lasty - ty;
                    unsigned int best, dist;
                    best = dist = (unsigned int)(dx * dx + dy * dy);
                    while (last2.y >= 0) {
                        dx = last1.x - tx; dy = last2.y - ty;
                        dist = (unsigned int)(dx * dx + dy * dy);
                        if (dist > best) break;
                        best = dist; lasty = last2.y; last2 = last1;
                        if (last2.y >= 0) last1 = input[IDX(tx, last2.y, n)];
                    }
                    out[IDX(ty, tx, n)] = S2(lasty, last2.x);
                }
            }
        }
    }
}

/* pba2DCompute (gcvt.cu:920-978) on a private copy of the site grid. */
static int pba_compute(const s2 *sites, s2 *labels, int n) {
    int m1 = tab_m1(n), m2 = tab_m2(n), m3 = tab_m3(n);
    if (!m1) return -1;
    size_t nn = (size_t)n * n;
    s2 *t0 = (s2 *)malloc(sizeof(s2) * nn);
    s2 *t1 = (s2 *)malloc(sizeof(s2) * nn);
    s2 *margin = (s2 *)malloc(sizeof(s2) * 2 * (size_t)m1 * n);
    if (!t0 || !t1 || !margin) { free(t0); free(t1); free(margin); return -2; }
    memcpy(t0, sites, sizeof(s2) * nn);
    /* phase 1 (gcvt.cu:921-933) */
    int bs = n / m1;
    pba_flood_down(t0, n, bs, m1);
    pba_flood_up(t0, n, bs, m1);
    pba_propagate_interband(t0, margin, n, bs, m1);
    pba_update_vertical(t0, margin, t1, n, bs, m1);
    /* phase 2 (gcvt.cu:936-956): color = t1, stack/link = t0 */
    bs = n / m2;
    pba_proximate_points(t1, t0, n, bs, m2);
    pba_forward_pointers(t0, n, bs, m2);
    for (int noBand = m2; noBand > 1; noBand /= 2)
        pba_merge_bands(t1, t0, n, n / noBand, noBand / 2);
    pba_double_to_single(t1, t0, n);
    /* phase 3 (gcvt.cu:959-965) */
    pba_color(t0, t1, n, m3);
    memcpy(labels, t1, sizeof(s2) * nn);
    free(t0); free(t1); free(margin);
    return 0;
}

int orc_pba_label(const int16_t *sites, int16_t *labels, int n) {
    if (!sites || !labels) return -1;
    return pba_compute((const s2 *)sites, (s2 *)labels, n);
}

/* ============================================================================
 * Pointwise statement of the PBA+ labelling.
 *
 * Phase 1 gives, per column x and row r, the vertically nearest site of that
 * column; with a above-or-at r and b below r at equal distance, FloodUp's
 * strict '<' (gcvt.cu:114) keeps b inside a 64-row band (bandSize =
 * n/m1 = 64 for every table entry), while the margin merges of
 * UpdateVertical (gcvt.cu:197-200) only replace on strict '<', so b wins
 * exactly when it lies in r's band.  Phase 2 keeps the lower envelope of the
 * resulting parabolas (its band merges do not change the envelope), and the
 * colour walk (gcvt.cu:457) advances on ties toward the smaller column.
 * Hence: nearest site; ties to smaller x; a mirror pair (x, r-k)/(x, r+k) to
 * r+k iff (r+k)/64 == r/64.  Tests check this against the literal
 * restatement above and against the reference kernels themselves.
 * ==========================================================================*/

#define NONE_Y (-32768)

/* Column pass: cy[r*n + x] = row of the vertically nearest site in column x
 * (band tie rule), or NONE_Y. */
static void spec_columns(const s2 *sites, int16_t *cy, int n) {
    #pragma omp parallel
    {
        int *ys = (int *)malloc(sizeof(int) * (size_t)n);
        #pragma omp for schedule(static)
        for (int x = 0; x < n; ++x) {
            int k = 0;
            for (int y = 0; y < n; ++y)
                if (sites[IDX(x, y, n)].x != MK) ys[k++] = y;
            int j = 0; /* ys[j] = first site row > r */
            for (int r = 0; r < n; ++r) {
                while (j < k && ys[j] <= r) ++j;
                int a = j > 0 ? ys[j - 1] : NONE_Y;
                int b = j < k ? ys[j] : NONE_Y;
                int c;
                if (a == NONE_Y && b == NONE_Y) c = NONE_Y;
                else if (a == NONE_Y) c = b;
                else if (b == NONE_Y) c = a;
                else {
                    int da = r - a, db = b - r;
                    if (da < db) c = a;
                    else if (db < da) c = b;
                    else c = ((b >> 6) == (r >> 6)) ? b : a;
                }
                cy[IDX(x, r, n)] = (int16_t)c;
            }
        }
        free(ys);
    }
}

static inline long long floordiv_ll(long long a, long long b) { /* b > 0 */
    long long q = a / b;
    if ((a % b != 0) && (a < 0)) --q;
    return q;
}

/* Row pass: lower envelope of the column candidates, exact integer
 * breakpoints, ties to the smaller column. */
static void spec_rows(const int16_t *cy, s2 *labels, int n) {
    #pragma omp parallel
    {
        int *hx = (int *)malloc(sizeof(int) * (size_t)n);
        long long *hb = (long long *)malloc(sizeof(long long) * (size_t)n);
        #pragma omp for schedule(static)
        for (int r = 0; r < n; ++r) {
            int K = 0;
            const int16_t *row = cy + IDX(0, r, n);
            for (int x = 0; x < n; ++x) {
                if (row[x] == NONE_Y) continue;
                long long g = (long long)row[x] - r;
                long long B = (long long)x * x + g * g;
                while (K >= 2) {
                    long long ox = hx[K - 2], oB = hb[K - 2], ax = hx[K - 1], aB = hb[K - 1];
                    long long cr = (ax - ox) * (B - oB) - (aB - oB) * ((long long)x - ox);
                    if (cr > 0) break;
                    --K;
                }
                hx[K] = x; hb[K] = B; ++K;
            }
            s2 *out = labels + IDX(0, r, n);
            if (K == 0) {
                for (int x = 0; x < n; ++x) out[x] = S2(MK, MK);
                continue;
            }
            int j = 0;
            for (int x0 = 0; x0 < n; ++x0) {
                while (j + 1 < K) {
                    long long start = floordiv_ll(hb[j + 1] - hb[j], 2LL * (hx[j + 1] - hx[j])) + 1;
                    if (start <= x0) ++j; else break;
                }
                out[x0] = S2(hx[j], row[hx[j]]);
            }
        }
        free(hx); free(hb);
    }
}

int orc_spec_label(const int16_t *sites, int16_t *labels, int n) {
    if (!sites || !labels || n < 1 || n > 16384) return -1;
    int16_t *cy = (int16_t *)malloc(sizeof(int16_t) * (size_t)n * n);
    if (!cy) return -2;
    spec_columns((const s2 *)sites, cy, n);
    spec_rows(cy, (s2 *)labels, n);
    free(cy);
    return 0;
}

/* 1 if site (sx, sy) is preferred over (tx, ty) for pixel (px, r). */
static inline int spec_better(int sx, int sy, int tx, int ty, int px, int r) {
    long long ds = (long long)(sx - px) * (sx - px) + (long long)(sy - r) * (sy - r);
    long long dt = (long long)(tx - px) * (tx - px) + (long long)(ty - r) * (ty - r);
    if (ds != dt) return ds < dt;
    if (sx != tx) return sx < tx;
    int below = sy > ty ? sy : ty;
    int pick = ((below >> 6) == (r >> 6)) ? below : (sy + ty - below);
    return sy == pick && ty != pick;
}

int orc_brute_label(const int16_t *sites, int16_t *labels, int n) {
    if (!sites || !labels || n < 1 || n > 16384) return -1;
    const s2 *s = (const s2 *)sites;
    s2 *out = (s2 *)labels;
    size_t nn = (size_t)n * n, m = 0;
    for (size_t i = 0; i < nn; ++i) if (s[i].x != MK) ++m;
    int *px = (int *)malloc(sizeof(int) * (m + 1)), *py = (int *)malloc(sizeof(int) * (m + 1));
    m = 0;
    for (int y = 0; y < n; ++y)
        for (int x = 0; x < n; ++x)
            if (s[IDX(x, y, n)].x != MK) { px[m] = x; py[m] = y; ++m; }
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
        for (int x0 = 0; x0 < n; ++x0) {
            int bx = MK, by = MK;
            for (size_t k = 0; k < m; ++k) {
                if (bx == MK || spec_better(px[k], py[k], bx, by, x0, r)) { bx = px[k]; by = py[k]; }
            }
            out[IDX(x0, r, n)] = S2(bx, by);
        }
    }
    free(px); free(py);
    return 0;
}

/* ============================================================================
 * Lloyd loop pieces (gcvt.cu:485-832, 985-1083).
 * ==========================================================================*/

/* Conversion used by kernelUpdateSites (gcvt.cu:772): float -> short is a
 * round-toward-zero conversion that saturates and maps NaN to 0; the clamp to
 * [0, n-1] (gcvt.cu:774-775) follows. */
static inline int upd_coord(float v, int n) {
    int c;
    if (v != v) c = 0;
    else if (v >= 32767.0f) c = 32767;
    else if (v <= -32768.0f) c = -32768;
    else c = (int)v; /* C truncates toward zero */
    if (c > n - 1) c = n - 1;
    if (c < 0) c = 0;
    return c;
}

/* kernelUpdateSites' position rule (gcvt.cu:770-777) given a float centroid:
 * nvcc contracts 'tx + (_x - tx) * omega' into one fused multiply-add. */
static inline void upd_rule(float cx, float cy, int tx, int ty, float omega, int n,
                            int fixed, const float *density, int *ox, int *oy) {
    float fx = fmaf(cx - (float)tx, omega, (float)tx) + 0.5f;
    float fy = fmaf(cy - (float)ty, omega, (float)ty) + 0.5f;
    int rx = upd_coord(fx, n), ry = upd_coord(fy, n);
    if (fixed || density[IDX(rx, ry, n)] == 0.0f) { rx = tx; ry = ty; }
    *ox = rx; *oy = ry;
}

/* kernelDensityScaling (gcvt.cu:497-511): x-outer, y-inner FP32 sums. */
static void density_scale(const float *in, float *out, int n) {
    #pragma omp parallel for schedule(static)
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            float d = 0.0f;
            for (int x = tx * 2; x < tx * 2 + 2; ++x)
                for (int y = ty * 2; y < ty * 2 + 2; ++y) d += in[IDX(x, y, 2 * n)];
            out[IDX(tx, ty, n)] = (float)((double)d / 4.0);
        }
}

/* kernelComputeWeightedPrefixX (gcvt.cu:515-560): 64-wide Hillis-Steele
 * blocks with a carry held only by thread 0. */
static void faithful_prefix(const float *density, float *pW, float *pX, float *pY, int n) {
    #pragma omp parallel for schedule(static)
    for (int ty = 0; ty < n; ++ty) {
        float lastX = 0.0f, lastY = 0.0f, lastW = 0.0f;
        float tW[64], tX[64], tY[64], nW[64], nX[64], nY[64];
        for (int xx = 0; xx < n; xx += 64) {
            for (int tid = 0; tid < 64; ++tid) {
                int tx = xx + tid;
                float w = density[IDX(tx, ty, n)];
                float lx = tid == 0 ? lastX : 0.0f, ly = tid == 0 ? lastY : 0.0f,
                      lw = tid == 0 ? lastW : 0.0f;
                tX[tid] = fmaf((float)tx, w, lx);
                tY[tid] = fmaf((float)ty, w, ly);
                tW[tid] = lw + w;
            }
            for (int step = 1; step < 64; step *= 2) {
                for (int tid = 0; tid < 64; ++tid) {
                    nW[tid] = tW[tid]; nX[tid] = tX[tid]; nY[tid] = tY[tid];
                    if (tid >= step) {
                        nW[tid] = tW[tid] + tW[tid - step];
                        nX[tid] = tX[tid] + tX[tid - step];
                        nY[tid] = tY[tid] + tY[tid - step];
                    }
                }
                memcpy(tW, nW, sizeof tW); memcpy(tX, nX, sizeof tX); memcpy(tY, nY, sizeof tY);
            }
            for (int tid = 0; tid < 64; ++tid) {
                pX[IDX(xx + tid, ty, n)] = tX[tid];
                pY[IDX(xx + tid, ty, n)] = tY[tid];
                pW[IDX(xx + tid, ty, n)] = tW[tid];
            }
            lastX = tX[63]; lastY = tY[63]; lastW = tW[63];
        }
    }
}

/* kernelCalcEnergy + kernelReduce<512> as driven by pbaCVDCalcEnergy
 * (gcvt.cu:788-832, 1059-1083).  Each pass runs in place; the reduction reads
 * input[i + 512] without a bound check, so the final single-block pass adds
 * the stale entries [512, 512 + n) left by the first pass.  Blocks are assumed
 * to read before any block writes. */
float orc_faithful_energy(const int16_t *labels, const float *density, int n, int level) {
    const s2 *lab = (const s2 *)labels;
    size_t nn = (size_t)n * n;
    size_t cap = nn > 65536 ? nn : 65536;
    float *tex = (float *)calloc(cap + 1024, sizeof(float));
    if (!tex) return NAN;
    #pragma omp parallel for schedule(static)
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            s2 site = lab[IDX(tx, ty, n)];
            float dx = (float)(site.x - tx) * 1.0f / (float)n;
            float dy = (float)(site.y - ty) * 1.0f / (float)n;
            float dist = fmaf(dx, dx, dy * dy);
            tex[IDX(tx, ty, n)] = density[IDX(tx, ty, n)] * dist;
        }
    const unsigned bsz = 512;
    unsigned cnt = (unsigned)nn;
    float *outv = (float *)malloc(sizeof(float) * 32768);
    int final_pass = 0;
    for (;;) {
        unsigned blocks;
        if (!final_pass) {
            double c = ceil((1.0 * cnt) / bsz);
            blocks = (unsigned)(c < 32768.0 ? c : 32768.0);
        } else {
            blocks = 1;
        }
        unsigned gridSize = bsz * 2 * blocks;
        #pragma omp parallel for schedule(static)
        for (unsigned b = 0; b < blocks; ++b) {
            float sd[512];
            for (unsigned tid = 0; tid < bsz; ++tid) {
                float acc = 0.0f;
                for (unsigned i = b * (bsz * 2) + tid; i < cnt; i += gridSize)
                    acc += tex[i] + tex[i + bsz];
                sd[tid] = acc;
            }
            for (unsigned s = 256; s >= 64; s >>= 1)
                for (unsigned tid = 0; tid < s; ++tid) sd[tid] += sd[tid + s];
            for (unsigned s = 32; s >= 1; s >>= 1) {
                float nv[32];
                for (unsigned tid = 0; tid < 32; ++tid) nv[tid] = sd[tid] + sd[tid + s];
                for (unsigned tid = 0; tid < 32; ++tid) sd[tid] = nv[tid];
            }
            outv[b] = sd[0];
        }
        for (unsigned b = 0; b < blocks; ++b) tex[b] = outv[b];
        if (final_pass) break;
        cnt = blocks;
        if (cnt > bsz) continue;
        if (cnt > 1) { final_pass = 1; continue; }
        break;
    }
    float e = tex[0];
    free(outv);
    free(tex);
    return e * powf(2.0f, (float)(level * 2.0));
}

/* FP64 moments and energy straight from a label grid (exact mode).  Summation
 * runs in row-major pixel order, so the result is thread-count independent. */
static void exact_moments(const s2 *lab, const float *density, int n, double *W, double *X,
                          double *Y, double *energy) {
    size_t nn = (size_t)n * n;
    memset(W, 0, sizeof(double) * nn);
    memset(X, 0, sizeof(double) * nn);
    memset(Y, 0, sizeof(double) * nn);
    double e = 0.0;
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            s2 s = lab[IDX(tx, ty, n)];
            double rho = density[IDX(tx, ty, n)];
            if (s.x == MK) continue;
            ptrdiff_t sid = IDX(s.x, s.y, n);
            W[sid] += rho;
            X[sid] += (double)tx * rho;
            Y[sid] += (double)ty * rho;
            double dx = s.x - tx, dy = s.y - ty;
            e += rho * (dx * dx + dy * dy);
        }
    if (energy) *energy = e / ((double)n * (double)n);
}

/* Site update shared by both modes: fill with MARKER (kernelFillShort,
 * gcvt.cu:65-71), then scatter each site's new position (gcvt.cu:753-781);
 * sites that land on the same pixel merge. */
static void update_sites(const s2 *lab, const float *cxs, const float *cys, const float *density,
                         const uint8_t *mask, int n, float omega, s2 *out) {
    size_t nn = (size_t)n * n;
    for (size_t i = 0; i < nn; ++i) out[i] = S2(MK, MK);
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            ptrdiff_t id = IDX(tx, ty, n);
            s2 s = lab[id];
            if (s.x != tx || s.y != ty) continue; /* a site pixel labels itself */
            int rx, ry;
            upd_rule(cxs[id], cys[id], tx, ty, omega, n, mask[id] != 0, density, &rx, &ry);
            out[IDX(rx, ry, n)] = S2(rx, ry);
        }
}

int orc_lloyd_step(const int16_t *sites_in, const float *density, const uint8_t *mask, int n,
                   float omega, int16_t *labels_out, double *moments, double *energy,
                   int16_t *sites_out) {
    if (!sites_in || !density || !mask || n < 1 || n > 16384) return -1;
    size_t nn = (size_t)n * n;
    s2 *lab = (s2 *)malloc(sizeof(s2) * nn);
    double *W = (double *)malloc(sizeof(double) * nn * 3);
    float *cx = (float *)malloc(sizeof(float) * nn), *cyv = (float *)malloc(sizeof(float) * nn);
    if (!lab || !W || !cx || !cyv) { free(lab); free(W); free(cx); free(cyv); return -2; }
    double *X = W + nn, *Y = W + 2 * nn;
    orc_spec_label(sites_in, (int16_t *)lab, n);
    exact_moments(lab, density, n, W, X, Y, energy);
    for (size_t i = 0; i < nn; ++i) {
        cx[i] = (float)(X[i] / W[i]);
        cyv[i] = (float)(Y[i] / W[i]);
    }
    if (sites_out) update_sites(lab, cx, cyv, density, mask, n, omega, (s2 *)sites_out);
    if (labels_out) memcpy(labels_out, lab, sizeof(s2) * nn);
    if (moments) memcpy(moments, W, sizeof(double) * nn * 3);
    free(lab); free(W); free(cx); free(cyv);
    return 0;
}

/* Faithful centroid pass: kernelVoronoi1D + kernelTotal_X + kernelScan_Y
 * (gcvt.cu:564-732) in FP32 with the reference's operation order; the
 * column atomics of Scan_Y are applied in window order (the reference's
 * order varies from run to run). */
static void faithful_centroids(const s2 *lab, const float *pW, const float *pX, const float *pY,
                               int n, float *tW, float *tX, float *tY, int16_t *tmp) {
    /* kernelVoronoi1D: tmp[r][site.x] = site.y */
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
        int16_t *row = tmp + IDX(0, r, n);
        for (int x = 0; x < n; ++x) row[x] = MK;
        for (int x = 0; x < n; ++x) {
            s2 p = lab[IDX(x, r, n)];
            if (p.x >= 0 && p.x < n) row[p.x] = p.y;
        }
    }
    /* kernelTotal_X: per row run of each site, prefix differences */
    #pragma omp parallel for schedule(static)
    for (int r = 0; r < n; ++r) {
        for (int x = 0; x < n;) {
            s2 me = lab[IDX(x, r, n)];
            int e = x;
            while (e + 1 < n && lab[IDX(e + 1, r, n)].x == me.x) ++e;
            if (me.x >= 0 && me.x < n) {
                float lw = 0.0f, lx = 0.0f, ly = 0.0f;
                if (x > 0) { lw = pW[IDX(x - 1, r, n)]; lx = pX[IDX(x - 1, r, n)]; ly = pY[IDX(x - 1, r, n)]; }
                ptrdiff_t o = IDX(me.x, r, n);
                tX[o] = pX[IDX(e, r, n)] - lx;
                tY[o] = pY[IDX(e, r, n)] - ly;
                tW[o] = pW[IDX(e, r, n)] - lw;
            }
            x = e + 1;
        }
    }
    /* kernelScan_Y: per column, 64-row windows, run-length groups */
    #pragma omp parallel for schedule(static)
    for (int tx = 0; tx < n; ++tx) {
        for (int w = 0; w < n / 64; ++w) {
            int last = MK;
            float ax = 0.0f, ay = 0.0f, aw = 0.0f;
            for (int i = 0; i < 64; ++i) {
                int ty = w * 64 + i;
                int pixel = tmp[IDX(tx, ty, n)];
                if (pixel != last) {
                    if (last != MK) {
                        ptrdiff_t t = IDX(tx, last, n);
                        tX[t] += ax; tY[t] += ay; tW[t] += aw;
                    }
                    ax = ay = aw = 0.0f;
                    last = pixel;
                }
                if (pixel != MK && pixel != ty) {
                    ptrdiff_t id = IDX(tx, ty, n);
                    ax += tX[id]; ay += tY[id]; aw += tW[id];
                }
            }
            if (last != MK) {
                ptrdiff_t t = IDX(tx, last, n);
                tX[t] += ax; tY[t] += ay; tW[t] += aw;
            }
        }
    }
}

/* One faithful Lloyd step (gcvt.cu:995-1034 with pba2DCompute): FP32 prefix
 * sums, PBA+ labels, Total_X / Scan_Y totals, update.  totals3 receives the
 * W, X, Y totals (n*n floats each) as the reference leaves them, meaningful
 * at site pixels. */
int orc_faithful_step(const int16_t *sites_in, const float *density, const uint8_t *mask, int n,
                      float omega, int16_t *labels_out, float *totals3, int16_t *sites_out) {
    if (!sites_in || !density || !mask || !tab_m1(n)) return -1;
    size_t nn = (size_t)n * n;
    s2 *lab = (s2 *)malloc(sizeof(s2) * nn);
    float *buf = (float *)malloc(sizeof(float) * nn * 8);
    int16_t *t1d = (int16_t *)malloc(sizeof(int16_t) * nn);
    if (!lab || !buf || !t1d) { free(lab); free(buf); free(t1d); return -2; }
    float *pW = buf, *pX = buf + nn, *pY = buf + 2 * nn, *tW = buf + 3 * nn, *tX = buf + 4 * nn,
          *tY = buf + 5 * nn, *cx = buf + 6 * nn, *cyv = buf + 7 * nn;
    memset(tW, 0, sizeof(float) * nn * 3);
    faithful_prefix(density, pW, pX, pY, n);
    pba_compute((const s2 *)sites_in, lab, n);
    faithful_centroids(lab, pW, pX, pY, n, tW, tX, tY, t1d);
    for (size_t i = 0; i < nn; ++i) {
        cx[i] = tX[i] / tW[i];
        cyv[i] = tY[i] / tW[i];
    }
    if (sites_out) update_sites(lab, cx, cyv, density, mask, n, omega, (s2 *)sites_out);
    if (labels_out) memcpy(labels_out, lab, sizeof(s2) * nn);
    if (totals3) {
        memcpy(totals3, tW, sizeof(float) * nn);
        memcpy(totals3 + nn, tX, sizeof(float) * nn);
        memcpy(totals3 + 2 * nn, tY, sizeof(float) * nn);
    }
    free(lab); free(buf); free(t1d);
    return 0;
}

/* kernelZoomIn after kernelFillShort (gcvt.cu:485-495, 1036-1051). */
static void zoom_in(const s2 *in, s2 *out, int n) {
    size_t n2 = (size_t)(2 * n) * (2 * n);
    for (size_t i = 0; i < n2; ++i) out[i] = S2(MK, MK);
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            s2 p = in[IDX(tx, ty, n)];
            out[IDX(tx << 1, ty << 1, 2 * n)] = (p.x == MK) ? S2(MK, MK) : S2(p.x << 1, p.y << 1);
        }
}

/* gCVT (gcvt.cu:1087-1156). */
int orc_gcvt(int16_t *voronoi, const float *density, const uint8_t *mask, int size, int depth,
             int max_iter, int mode, int fixed_iters, int threads, orc_stats *stats) {
    if (!voronoi || !density || !mask) return -1;
    if (!tab_m1(size)) return -2;
    if (depth < 1) return -3;
    if (mode != ORC_MODE_FAITHFUL && mode != ORC_MODE_EXACT) return -4;
#ifdef _OPENMP
    int saved_threads = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    for (int i = 0; i < depth; ++i)
        if ((size >> i) < 256) { depth = i; break; }
    size_t nn = (size_t)size * size;
    float *dens[16] = {0};
    uint8_t *masks[16] = {0};
    dens[0] = (float *)malloc(sizeof(float) * nn);
    memcpy(dens[0], density, sizeof(float) * nn);
    for (int i = 1; i < depth; ++i) {
        int ni = size >> i;
        dens[i] = (float *)malloc(sizeof(float) * (size_t)ni * ni);
        density_scale(dens[i - 1], dens[i], ni);
    }
    /* the mask is indexed with the level's own row pitch (gcvt.cu:777) */
    for (int i = 0; i < depth; ++i) masks[i] = (uint8_t *)mask;
    s2 *grid = (s2 *)malloc(sizeof(s2) * nn);
    s2 *lab = (s2 *)malloc(sizeof(s2) * nn);
    s2 *tmpg = (s2 *)malloc(sizeof(s2) * nn);
    float *cx = (float *)malloc(sizeof(float) * nn), *cyv = (float *)malloc(sizeof(float) * nn);
    double *W = NULL, *X = NULL, *Y = NULL;
    float *pW = NULL, *pX = NULL, *pY = NULL, *tW = NULL, *tX = NULL, *tY = NULL;
    int16_t *t1d = NULL;
    if (mode == ORC_MODE_EXACT) {
        W = (double *)malloc(sizeof(double) * nn); X = (double *)malloc(sizeof(double) * nn);
        Y = (double *)malloc(sizeof(double) * nn);
    } else {
        pW = (float *)malloc(sizeof(float) * nn); pX = (float *)malloc(sizeof(float) * nn);
        pY = (float *)malloc(sizeof(float) * nn); tW = (float *)malloc(sizeof(float) * nn);
        tX = (float *)malloc(sizeof(float) * nn); tY = (float *)malloc(sizeof(float) * nn);
        t1d = (int16_t *)malloc(sizeof(int16_t) * nn);
    }
    /* the initial grid is the first (size >> (depth-1))^2 entries of the
     * caller's array (gcvt.cu:1099-1103) */
    int n = size >> (depth - 1);
    memcpy(grid, voronoi, sizeof(s2) * (size_t)n * n);

    int iters = 0, levels = 0;
    float omega = 2.0f;
    double E = 0.0, lastE = 1e18;
    float Ef = 0.0f, lastEf = (float)1e18;
    for (int level = depth - 1; level >= 0; --level) {
        n = size >> level;
        ++levels;
        const float *d = dens[level];
        if (mode == ORC_MODE_FAITHFUL) faithful_prefix(d, pW, pX, pY, n);
        int level_iters = 0;
        do {
            pba_compute(grid, lab, n);
            if (mode == ORC_MODE_EXACT) {
                double e;
                exact_moments(lab, d, n, W, X, Y, &e);
                if (iters % 10 == 0) E = e * pow(4.0, level);
                size_t m = (size_t)n * n;
                for (size_t i = 0; i < m; ++i) {
                    cx[i] = (float)(X[i] / W[i]);
                    cyv[i] = (float)(Y[i] / W[i]);
                }
            } else {
                if (iters % 10 == 0) Ef = orc_faithful_energy((const int16_t *)lab, d, n, level);
                faithful_centroids(lab, pW, pX, pY, n, tW, tX, tY, t1d);
                size_t m = (size_t)n * n;
                for (size_t i = 0; i < m; ++i) {
                    if (lab[i].x == (int16_t)(i % n) && lab[i].y == (int16_t)(i / n)) {
                        cx[i] = tX[i] / tW[i];
                        cyv[i] = tY[i] / tW[i];
                    }
                }
            }
            update_sites(lab, cx, cyv, d, masks[level], n, omega, grid);
            ++iters;
            ++level_iters;
            if (iters % 10 == 0) {
                if (mode == ORC_MODE_EXACT) {
                    double diff = lastE - E;
                    double grad = diff / 10.0;
                    omega = (float)fmin(2.0, 1.0 + diff);
                    if (fixed_iters <= 0) {
                        if (level) { if (grad < 3e-1) break; }
                        else if (grad < 1e-5) break;
                    }
                    lastE = E;
                } else {
                    float diff = lastEf - Ef;
                    float grad = (float)((double)diff / 10.0);
                    omega = (float)fmin(2.0, 1.0 + (double)diff);
                    if (fixed_iters <= 0) {
                        if (level) { if ((double)grad < 3e-1) break; }
                        else if ((double)grad < 1e-5) break;
                    }
                    lastEf = Ef;
                }
            }
        } while (fixed_iters > 0 ? level_iters < fixed_iters : iters < max_iter);
        if (level) {
            zoom_in(grid, tmpg, n);
            s2 *t = grid; grid = tmpg; tmpg = t;
        }
    }
    pba_compute(grid, lab, size);
    memcpy(voronoi, lab, sizeof(s2) * nn);
    if (stats) {
        stats->iterations = iters;
        stats->levels = levels;
        stats->last_energy = mode == ORC_MODE_EXACT ? E : (double)Ef;
        stats->omega = omega;
    }
    for (int i = 0; i < depth; ++i) free(dens[i]);
    free(grid); free(lab); free(tmpg); free(cx); free(cyv);
    free(W); free(X); free(Y); free(pW); free(pX); free(pY); free(tW); free(tX); free(tY); free(t1d);
#ifdef _OPENMP
    omp_set_num_threads(saved_threads);
#endif
    return 0;
}

/* ============================================================================
 * Rasteriser (discretization.cu:28-85).  FP64 in the source's operation
 * order, written with explicit fused multiply-adds where nvcc contracts.
 * ==========================================================================*/

static inline void bary(double x1, double y1, double x2, double y2, double x3, double y3,
                        double x0, double y0, double *w3, double *w1, double *w2) {
    double v0x = x2 - x1, v0y = y2 - y1;
    double v1x = x3 - x1, v1y = y3 - y1;
    double v2x = x0 - x1, v2y = y0 - y1;
    double d00 = fma(v0x, v0x, v0y * v0y);
    double d01 = fma(v0x, v1x, v0y * v1y);
    double d11 = fma(v1x, v1x, v1y * v1y);
    double d20 = fma(v2x, v0x, v2y * v0y);
    double d21 = fma(v2x, v1x, v2y * v1y);
    double denom = fma(d00, d11, -(d01 * d01));
    if (denom == 0) { *w1 = *w2 = *w3 = -1; return; }
    *w1 = fma(d11, d20, -(d01 * d21)) / denom;
    *w2 = fma(d00, d21, -(d01 * d20)) / denom;
    *w3 = 1.0 - *w1 - *w2;
}

int orc_rasterize(const double *points, const double *weight, int num_point,
                  const int32_t *triangle, int num_tri, float *density, double scale, int n,
                  int threads) {
    if (!points || !weight || !triangle || !density || n < 1 || num_tri < 0) return -1;
    (void)num_point;
#ifdef _OPENMP
    int saved_threads = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    #pragma omp parallel for schedule(dynamic, 4)
    for (int ty = 0; ty < n; ++ty)
        for (int tx = 0; tx < n; ++tx) {
            double x = tx * scale, y = ty * scale;
            float res = 0.0f;
            for (int i = 0; i < num_tri; ++i) {
                int p1 = triangle[i * 3], p2 = triangle[i * 3 + 1], p3 = triangle[i * 3 + 2];
                double w1, w2, w3;
                bary(points[p1 << 1], points[p1 << 1 | 1], points[p2 << 1], points[p2 << 1 | 1],
                     points[p3 << 1], points[p3 << 1 | 1], x, y, &w1, &w2, &w3);
                if (w1 < 0 || w2 < 0 || w3 < 0) continue;
                /* w1*weight[p1] + w2*weight[p2] + w3*weight[p3] as nvcc contracts it */
                res = (float)fma(w3, weight[p3], fma(w1, weight[p1], w2 * weight[p2]));
                goto done;
            }
            res = 0.0f;
        done:
            density[IDX(tx, ty, n)] = res;
        }
#ifdef _OPENMP
    omp_set_num_threads(saved_threads);
#endif
    return 0;
}

/* ============================================================================
 * Lift (recover.h:30-157) and weighting (weighting.h:29-97).  Compiled with
 * -ffp-contract=off: every product and sum is rounded on its own, as in the
 * reference's host build.
 * ==========================================================================*/

static double dot2(double x1, double y1, double x2, double y2) { return x1 * x2 + y1 * y2; }

/* barycentric (recover.h:30-52); w[0..2] = the caller's _w[0..2]. */
static void lift_bary(double x1, double y1, double x2, double y2, double x3, double y3,
                      double x0, double y0, double w[3]) {
    double v0x = x2 - x1, v0y = y2 - y1;
    double v1x = x3 - x1, v1y = y3 - y1;
    double v2x = x0 - x1, v2y = y0 - y1;
    double d00 = dot2(v0x, v0y, v0x, v0y);
    double d01 = dot2(v0x, v0y, v1x, v1y);
    double d11 = dot2(v1x, v1y, v1x, v1y);
    double d20 = dot2(v2x, v2y, v0x, v0y);
    double d21 = dot2(v2x, v2y, v1x, v1y);
    double denom = d00 * d11 - d01 * d01;
    if (denom == 0) { w[0] = w[1] = w[2] = -1; return; }
    w[1] = (d11 * d20 - d01 * d21) / denom;
    w[2] = (d00 * d21 - d01 * d20) / denom;
    w[0] = 1.0 - w[1] - w[2];
}

/* locate (recover.h:64-85): first face, index order, all weights >= 0. */
static int lift_locate(const double *uv, const int32_t *tri, int nt, double px, double py,
                       double w[3]) {
    for (int f = 0; f < nt; ++f) {
        const int32_t *t = tri + 3 * f;
        double bc[3];
        lift_bary(uv[2 * t[0]], uv[2 * t[0] + 1], uv[2 * t[1]], uv[2 * t[1] + 1],
                  uv[2 * t[2]], uv[2 * t[2] + 1], px, py, bc);
        if (bc[0] < 0 || bc[1] < 0 || bc[2] < 0) continue;
        w[0] = bc[0], w[1] = bc[1], w[2] = bc[2];
        return f;
    }
    return -1;
}

int orc_lift(const double *uv, const double *xyz, int num_vertex, const int32_t *triangle,
             int num_tri, const double *points, int num_points, int num_fixed,
             const int32_t *fixed_vertex, const int32_t *cdt, int num_cdt, double *out_xyz,
             int32_t *out_face, uint8_t *keep, int threads) {
    if (num_vertex < 0 || num_tri < 0 || num_points < 0 || num_fixed < 0 || num_cdt < 0 ||
        num_fixed > num_points)
        return -1;
    for (long i = 0; i < 3L * num_tri; ++i)
        if (triangle[i] < 0 || triangle[i] >= num_vertex) return -1;
    for (int i = 0; i < num_fixed; ++i)
        if (fixed_vertex[i] < 0 || fixed_vertex[i] >= num_vertex) return -1;
    for (long i = 0; i < 3L * num_cdt; ++i)
        if (cdt[i] < 0 || cdt[i] >= num_points) return -1;
    const int nfree = num_points - num_fixed;
    int32_t *face = out_face ? out_face : (int32_t *)malloc(sizeof(int32_t) * (nfree + 1));
    if (!face) return -2;
#ifdef _OPENMP
    int saved_threads = omp_get_max_threads();
    if (threads > 0) omp_set_num_threads(threads);
#else
    (void)threads;
#endif
    /* recover.h:120-134: lift each free point with its face's vertices */
    #pragma omp parallel for schedule(dynamic, 16)
    for (int i = 0; i < nfree; ++i) {
        double w[3];
        int f = lift_locate(uv, triangle, num_tri, points[2 * i], points[2 * i + 1], w);
        face[i] = f;
        if (f < 0) continue;
        const int32_t *t = triangle + 3 * f;
        for (int d = 0; d < 3; ++d) {
            double s = 0.0;
            for (int j = 0; j < 3; ++j) s += xyz[3 * t[j] + d] * w[j];
            out_xyz[3 * i + d] = s;
        }
    }
    /* recover.h:141-156: keep the triangles whose centroid locates */
    #pragma omp parallel for schedule(dynamic, 16)
    for (int t = 0; t < num_cdt; ++t) {
        const int32_t *c = cdt + 3 * t;
        double cx = (points[2 * c[0]] + points[2 * c[1]] + points[2 * c[2]]) / 3;
        double cy = (points[2 * c[0] + 1] + points[2 * c[1] + 1] + points[2 * c[2] + 1]) / 3;
        double w[3];
        keep[t] = lift_locate(uv, triangle, num_tri, cx, cy, w) >= 0;
    }
#ifdef _OPENMP
    omp_set_num_threads(saved_threads);
#endif
    /* an unlocated point reuses the last successful location */
    int last = -1;
    for (int i = 0; i < nfree; ++i) {
        if (face[i] >= 0) { last = i; continue; }
        for (int d = 0; d < 3; ++d) out_xyz[3 * i + d] = last >= 0 ? out_xyz[3 * last + d] : NAN;
    }
    /* recover.h:137-139: constraint points keep their vertex's position */
    for (int k = 0; k < num_fixed; ++k) {
        int i = nfree + k;
        for (int d = 0; d < 3; ++d) out_xyz[3 * i + d] = xyz[3 * fixed_vertex[k] + d];
        if (out_face) out_face[i] = -1;
    }
    if (!out_face) free(face);
    return 0;
}

int orc_vertex_weights(const double *uv, const double *xyz, int num_vertex,
                       const int32_t *triangle, int num_tri, double *weight) {
    if (num_vertex < 0 || num_tri < 0) return -1;
    for (long i = 0; i < 3L * num_tri; ++i)
        if (triangle[i] < 0 || triangle[i] >= num_vertex) return -1;
    double *a3 = (double *)calloc((size_t)num_vertex + 1, sizeof(double));
    double *a2 = (double *)calloc((size_t)num_vertex + 1, sizeof(double));
    uint8_t *over = (uint8_t *)calloc((size_t)num_vertex + 1, 1);
    if (!a3 || !a2 || !over) { free(a3); free(a2); free(over); return -2; }
    /* weighting.h:53-60: CGAL face_area of (source(h), target(h), target(next(h))) */
    for (int f = 0; f < num_tri; ++f) {
        const int32_t *t = triangle + 3 * f;
        const double *p = xyz + 3 * t[2], *q = xyz + 3 * t[0], *r = xyz + 3 * t[1];
        double dqx = q[0] - p[0], dqy = q[1] - p[1], dqz = q[2] - p[2];
        double drx = r[0] - p[0], dry = r[1] - p[1], drz = r[2] - p[2];
        double vx = dqy * drz - dqz * dry, vy = dqz * drx - dqx * drz, vz = dqx * dry - dqy * drx;
        double area = sqrt((vx * vx + vy * vy + vz * vz) / 4);
        for (int j = 0; j < 3; ++j) a3[t[j]] += area;
    }
    /* weighting.h:62-75: get_area (weighting.h:29-36) */
    for (int f = 0; f < num_tri; ++f) {
        const int32_t *t = triangle + 3 * f;
        double ax = uv[2 * t[0]], ay = uv[2 * t[0] + 1];
        double bx = uv[2 * t[1]] - ax, by = uv[2 * t[1] + 1] - ay;
        double cx = uv[2 * t[2]] - ax, cy = uv[2 * t[2] + 1] - ay;
        double area = fabs(bx * cy - cx * by) / 2.;
        for (int j = 0; j < 3; ++j) a2[t[j]] += area;
    }
    /* weighting.h:77-92 */
    double mx = 0;
    for (int v = 0; v < num_vertex; ++v) {
        double w = a3[v] / a2[v];
        if (w > 1e10) { over[v] = 1; continue; }
        weight[v] = w;
        if (w > mx) mx = w;
    }
    for (int v = 0; v < num_vertex; ++v)
        if (over[v]) weight[v] = mx;
    free(a3); free(a2); free(over);
    return 0;
}

/* ============================================================================
 * Seeding (gcvt.h:56-122).  Marsaglia's KISS-style generator with unsigned
 * long taken as 64 bits (LP64).
 * ==========================================================================*/

typedef struct { unsigned long long z, w, jsr, jcong; } orc_rng;

static unsigned long long rng_int(orc_rng *g) {
    g->z = 36969ULL * (g->z & 0xffffULL) + (g->z >> 16);
    g->w = 18000ULL * (g->w & 0xffffULL) + (g->w >> 16);
    unsigned long long mwc = (g->z << 16) + g->w;
    g->jcong = 69069ULL * g->jcong + 1234567ULL;
    g->jsr ^= (g->jsr << 17); g->jsr ^= (g->jsr >> 13); g->jsr ^= (g->jsr << 5);
    return (mwc ^ g->jcong) + g->jsr;
}
static double rng_unit(orc_rng *g) {
    return (double)rng_int(g) / ((double)ULLONG_MAX + 1);
}

int orc_seed_sites(int16_t *voronoi, const float *density, const uint8_t *mask, int num,
                   int size, long long seed) {
    if (!voronoi || !density || !mask || size < 1 || num < 0) return -1;
    s2 *v = (s2 *)voronoi;
    /* putConstrains (gcvt.h:106-122) */
    for (int i = 0; i < size; ++i)
        for (int j = 0; j < size; ++j)
            v[IDX(i, j, size)] = mask[IDX(i, j, size)] ? S2(i, j) : S2(MK, MK);
    /* randomPoints (gcvt.h:76-104) */
    double mx = 0, avg = 0, cnt = 0;
    size_t nn = (size_t)size * size;
    for (size_t i = 0; i < nn; ++i) {
        if (density[i] > mx) mx = density[i];
        if (density[i] != 0) { cnt += 1; avg += density[i]; }
    }
    if (cnt == 0) return num == 0 ? 0 : -2;
    mx = fmin(mx, avg / cnt * 100.);
    orc_rng g;
    unsigned long long s0 = seed < 0 ? 0ULL : (unsigned long long)seed;
    g.z = g.w = g.jsr = g.jcong = s0;
    long long budget = 1000LL * (long long)nn + 1000000LL;
    for (int i = 0; i < num; ++i) {
        int x, y;
        double z;
        do {
            if (--budget < 0) return -3;
            x = (int)(rng_unit(&g) * size);
            y = (int)(rng_unit(&g) * size);
            z = rng_unit(&g) * mx;
        } while (v[IDX(x, y, size)].x != MK || density[IDX(x, y, size)] <= z);
        v[IDX(x, y, size)] = S2(x, y);
    }
    return num;
}
