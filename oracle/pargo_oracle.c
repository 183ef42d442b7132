/*
 * pargo_oracle.c -- CPU restatement of the PaRGO focal hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Only tests/, __graft_entry__.smoke() and the
 * bench's CPU-baseline / reference arms may load this library, and only as the
 * checker or the timed CPU baseline; the product never links or calls it.
 *
 * Every function restates a reference operator in plain C, in double
 * precision, following the reference source line by line (citations below are
 * paths inside the PaRGO project).  Pinning: tests/test_oracle.py compares each
 * function bit-for-bit against the reference operators themselves, compiled
 * unmodified into oracle/_ref/ (oracle/build.py) and against the committed
 * fixtures in tests/golden/ that those operators produced.
 *
 * Layout conventions (same as the reference CellSpace, gpro/cellSpace.h:117-234):
 * row-major, index = row * cols + col; the work rectangle of a Moore (3x3)
 * neighbourhood is rows 1..rows-2, cols 1..cols-2 (gpro/neighborhood.h:447-448);
 * output cells outside it keep the layer's initial value, which copyLayerInfo
 * sets to nodata (gpro/rasterLayer.h:739-745).
 *
 * Build with -ffp-contract=off: the reference is plain IEEE double arithmetic
 * with no fused multiply-add.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define ORC_EPS_SLOPE 0.0000001 /* apps/morphology/slope/slopeOperator.h:13 */
#define ORC_EPS_HYDRO 0.000001  /* d8Operator.cpp:3, pitRemoveOperator.h:13, scaOperator.cpp:3 */

static inline double orc_get(const void* p, int f64, size_t i) {
    return f64 ? ((const double*)p)[i] : (double)((const float*)p)[i];
}

static void orc_fill_ring(double* out, int rows, int cols, double v) {
    for (int j = 0; j < cols; j++) { out[j] = v; out[(size_t)(rows - 1) * cols + j] = v; }
    for (int i = 0; i < rows; i++) { out[(size_t)i * cols] = v; out[(size_t)i * cols + cols - 1] = v; }
}

/* ---------------------------------------------------------------- slope --
 * apps/morphology/slope/slopeOperator.cpp:51-139.  method follows SlopeAlgor
 * (slopeOperator.h:18-26): 0 FD (Horn), 1 FFD, 2 MD, 3 SD, 4 SFD, 5 TFD, 6 TFDW.
 * cellsize is the float MetaData::cellSize (gpro/metaData.h:56) widened to double. */
int orc_slope(const void* dem, int dem_f64, int rows, int cols, double nodata, float cellsize_f,
              int method, int threads, double* out) {
    if (rows < 3 || cols < 3 || method < 0 || method > 6) return 1;
    const double cellSize = (double)cellsize_f;
    orc_fill_ring(out, rows, cols, nodata);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static) if (threads > 1)
#endif
    for (int iRow = 1; iRow < rows - 1; iRow++) {
        for (int iCol = 1; iCol < cols - 1; iCol++) {
            double d[9];
            int k = 0, tag = 0;
            for (int r = iRow - 1; r <= iRow + 1; r++)          /* :65-73 */
                for (int c = iCol - 1; c <= iCol + 1; c++) {
                    d[k] = orc_get(dem, dem_f64, (size_t)r * cols + c);
                    if (fabs(d[k] - nodata) < ORC_EPS_SLOPE) tag = 1;
                    k++;
                }
            double* o = out + (size_t)iRow * cols + iCol;
            if (tag) { *o = nodata; continue; }               /* :75-78 */
            double dx, dy;
            switch (method) {
            case 0: /* FD :84-86 */
                dx = (d[8] + 2 * d[5] + d[2] - d[6] - 2 * d[3] - d[0]) / (8.0 * cellSize);
                dy = (d[2] + 2 * d[1] + d[0] - d[6] - 2 * d[7] - d[8]) / (8.0 * cellSize);
                *o = sqrt(dx * dx + dy * dy);
                break;
            case 1: /* FFD :88-90 */
                dx = (d[8] - d[6] + d[2] - d[0]) / (4.0 * cellSize);
                dy = (d[0] - d[6] + d[2] - d[8]) / (4.0 * cellSize);
                *o = sqrt(dx * dx + dy * dy);
                break;
            case 2: { /* MD :92-103; the distance is that of the LAST neighbour visited */
                double max_diff = 0.0, hori_dist = cellSize;
                for (int r = iRow - 1; r <= iRow + 1; r++)
                    for (int c = iCol - 1; c <= iCol + 1; c++) {
                        if (r == iRow && c == iCol) continue;
                        double v = orc_get(dem, dem_f64, (size_t)r * cols + c);
                        if (max_diff < d[4] - v) max_diff = d[4] - v;
                        hori_dist = cellSize * sqrt((double)((r - iRow) * (r - iRow) + (c - iCol) * (c - iCol)));
                    }
                *o = max_diff / hori_dist;
                break;
            }
            case 3: /* SD :122-124 */
                dx = (d[4] - d[3]) / cellSize;
                dy = (d[4] - d[7]) / cellSize;
                *o = sqrt(dx * dx + dy * dy);
                break;
            case 4: /* SFD :126-128 */
                dx = (d[5] - d[3]) / (2.0 * cellSize);
                dy = (d[1] - d[7]) / (2.0 * cellSize);
                *o = sqrt(dx * dx + dy * dy);
                break;
            case 5: /* TFD :130-132 (dy uses d[6] twice, as the reference does) */
                dx = (d[8] + d[5] + d[2] - d[0] - d[3] - d[6]) / (6.0 * cellSize);
                dy = (d[2] + d[1] + d[0] - d[6] - d[7] - d[6]) / (6.0 * cellSize);
                *o = sqrt(dx * dx + dy * dy);
                break;
            default: /* TFDW :134-136 */
                dx = (d[8] + sqrt(2.0) * d[5] + d[2] - d[6] - sqrt(2.0) * d[3] - d[0]) / ((4.0 + sqrt(8.0)) * cellSize);
                dy = (d[2] + sqrt(2.0) * d[1] + d[0] - d[6] - sqrt(2.0) * d[7] - d[8]) / ((4.0 + sqrt(8.0)) * cellSize);
                *o = sqrt(dx * dx + dy * dy);
                break;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------- D8 --
 * apps/hydrology/flowdird8/d8Operator.cpp:28-101.  Codes are the row-major
 * 3x3 window index of the receiver (0..8 without 4); -1 flat/pit; nodata when
 * the window holds nodata.  dir_type 8 picks the middle tied index, any other
 * value gives the ArcGIS-style bit sum (:96-97). */
static double orc_d8_cell(const double d[9], int dir_type) {
    int valid[9] = {0};
    double max = 0.0, diff[9];
    for (int i = 0; i < 9; i++) {                          /* :64-72 */
        diff[i] = d[4] - d[i];
        if (i == 0 || i == 2 || i == 6 || i == 8) diff[i] = diff[i] / sqrt(2.0);
        if (diff[i] > max) max = diff[i];
    }
    if (max < ORC_EPS_HYDRO) return -1;                    /* :73-76 */
    if (dir_type == 8) {                                   /* :78-88 */
        int dirs[9], len = 0;
        for (int i = 0; i < 9; i++)
            if (fabs(diff[i] - max) < ORC_EPS_HYDRO) dirs[len++] = i;
        return dirs[len >> 1];
    }
    for (int i = 0; i < 9; i++)                            /* :90-97 */
        if (fabs(diff[i] - max) < ORC_EPS_HYDRO) valid[i] = 1;
    return valid[5] * 1.0 + valid[8] * 2.0 + valid[7] * 4.0 + valid[6] * 8.0 + valid[3] * 16.0 +
           valid[0] * 32.0 + valid[1] * 64.0 + valid[2] * 128.0;
}

int orc_d8(const void* dem, int dem_f64, int rows, int cols, double nodata, int dir_type, int threads,
           double* out) {
    if (rows < 3 || cols < 3) return 1;
    orc_fill_ring(out, rows, cols, nodata);
#ifdef _OPENMP
    if (threads > 0) omp_set_num_threads(threads);
#pragma omp parallel for schedule(static) if (threads > 1)
#endif
    for (int iRow = 1; iRow < rows - 1; iRow++) {
        for (int iCol = 1; iCol < cols - 1; iCol++) {
            double d[9];
            int k = 0, ok = 1;
            for (int r = iRow - 1; r <= iRow + 1; r++)          /* :41-52 */
                for (int c = iCol - 1; c <= iCol + 1; c++) {
                    d[k] = orc_get(dem, dem_f64, (size_t)r * cols + c);
                    if (fabs(d[k] - nodata) < ORC_EPS_HYDRO) ok = 0;
                    k++;
                }
            out[(size_t)iRow * cols + iCol] = ok ? orc_d8_cell(d, dir_type) : nodata;
        }
    }
    return 0;
}

/* ----------------------------------------------------------- pit removal --
 * apps/hydrology/pitremove/pitRemoveOperator.cpp:26-72 driven by the serial
 * Work() loop (gpro/rasterOperator.h:169-219): sweep 1 sets the water level
 * (init_level on valid cells, nodata elsewhere); later sweeps relax in raster
 * order, in place, until a sweep changes nothing.  *sweeps counts Work()
 * iterations like the reference loop (setup sweep + changing sweeps + the
 * final quiet sweep).  gap is 0.0005 in the reference (:36) and init_level is
 * 10000.0 (:41).  Returns 2 if max_sweeps is reached first. */
int orc_fill_gs(const float* dem, int rows, int cols, double nodata, double gap, double init_level,
                int max_sweeps, double* w, int* sweeps) {
    if (rows < 3 || cols < 3) return 1;
    orc_fill_ring(w, rows, cols, nodata);
    for (int i = 1; i < rows - 1; i++)
        for (int j = 1; j < cols - 1; j++) {
            size_t c = (size_t)i * cols + j;
            w[c] = fabs((double)dem[c] - nodata) > ORC_EPS_HYDRO ? init_level : nodata;
        }
    int n = 1, changed = 1;
    while (changed) {
        if (n >= max_sweeps) { *sweeps = n; return 2; }
        changed = 0;
        n++;
        for (int iRow = 1; iRow < rows - 1; iRow++)
            for (int iCol = 1; iCol < cols - 1; iCol++) {
                size_t c = (size_t)iRow * cols + iCol;
                double z = (double)dem[c];
                if (fabs(z - nodata) <= ORC_EPS_HYDRO || w[c] <= z) continue; /* :53-55 */
                for (int r = iRow - 1; r <= iRow + 1; r++)                      /* :57-68 */
                    for (int q = iCol - 1; q <= iCol + 1; q++) {
                        double wn = w[(size_t)r * cols + q];
                        if (z >= wn + gap || fabs(wn - nodata) < ORC_EPS_HYDRO) {
                            w[c] = z;
                            changed = 1;
                        } else if (w[c] > wn + gap) {
                            w[c] = wn + gap;
                            changed = 1;
                        }
                    }
            }
    }
    *sweeps = n;
    return 0;
}

/* Same fixpoint by priority flood.  The relaxation above is monotone
 * (levels only fall), so every visiting order reaches the same fixpoint:
 *   W(c) = min(init_level, max(dem(c), min_n (W(n) + gap)))  for valid c,
 * with W(n) + gap rounded to double exactly as the reference adds it, and a
 * nodata W neighbour (interior nodata, or the nodata ring) forcing W(c) = dem(c).
 * Popping cells in increasing W order settles each cell the first time one of
 * its neighbours is popped, in O(N log N) instead of O(N * sweeps). */
typedef struct { double key; int64_t idx; } orc_item;
typedef struct { orc_item* a; int64_t n, cap; } orc_heap;

static int orc_push(orc_heap* h, double key, int64_t idx) {
    if (h->n == h->cap) {
        int64_t nc = h->cap ? h->cap * 2 : 1024;
        orc_item* na = (orc_item*)realloc(h->a, (size_t)nc * sizeof(orc_item));
        if (!na) return 1;
        h->a = na; h->cap = nc;
    }
    int64_t i = h->n++;
    while (i > 0) {
        int64_t p = (i - 1) >> 2;
        if (h->a[p].key <= key) break;
        h->a[i] = h->a[p];
        i = p;
    }
    h->a[i].key = key; h->a[i].idx = idx;
    return 0;
}
static orc_item orc_pop(orc_heap* h) {
    orc_item top = h->a[0], last = h->a[--h->n];
    int64_t i = 0;
    for (;;) {
        int64_t c = 4 * i + 1, best = -1;
        if (c >= h->n) break;
        double bk = last.key;
        for (int64_t k = c; k < c + 4 && k < h->n; k++)
            if (h->a[k].key < bk) { bk = h->a[k].key; best = k; }
        if (best < 0) break;
        h->a[i] = h->a[best];
        i = best;
    }
    h->a[i] = last;
    return top;
}

int orc_fill_pf(const float* dem, int rows, int cols, double nodata, double gap, double init_level, double* w) {
    if (rows < 3 || cols < 3) return 1;
    size_t N = (size_t)rows * cols;
    unsigned char* done = (unsigned char*)calloc(N, 1);
    if (!done) return 3;
    orc_heap h = {0, 0, 0};
    orc_fill_ring(w, rows, cols, nodata);
    for (int i = 1; i < rows - 1; i++)
        for (int j = 1; j < cols - 1; j++) {
            size_t c = (size_t)i * cols + j;
            double z = (double)dem[c];
            int valid = fabs(z - nodata) > ORC_EPS_HYDRO;
            w[c] = valid ? init_level : nodata;
            if (!valid || init_level <= z) done[c] = 1; /* never updated by the reference (:53-55) */
        }
    /* sources: valid cells with a nodata water-level neighbour */
    for (int i = 1; i < rows - 1; i++)
        for (int j = 1; j < cols - 1; j++) {
            size_t c = (size_t)i * cols + j;
            if (done[c]) continue;
            int outlet = 0;
            for (int r = i - 1; r <= i + 1 && !outlet; r++)
                for (int q = j - 1; q <= j + 1; q++) {
                    size_t n = (size_t)r * cols + q;
                    int ring = (r == 0 || q == 0 || r == rows - 1 || q == cols - 1);
                    double wn = ring ? nodata : w[n];
                    if (fabs(wn - nodata) < ORC_EPS_HYDRO) { outlet = 1; break; }
                }
            if (outlet) {
                w[c] = (double)dem[c];
                done[c] = 1;
                if (orc_push(&h, w[c], (int64_t)c)) { free(done); free(h.a); return 3; }
            }
        }
    while (h.n > 0) {
        orc_item it = orc_pop(&h);
        int64_t c = it.idx;
        int i = (int)(c / cols), j = (int)(c % cols);
        double up = w[c] + gap;
        for (int r = i - 1; r <= i + 1; r++)
            for (int q = j - 1; q <= j + 1; q++) {
                if (r < 1 || q < 1 || r > rows - 2 || q > cols - 2) continue;
                size_t n = (size_t)r * cols + q;
                if (done[n]) continue;
                double z = (double)dem[n];
                double v = z >= up ? z : up;
                if (v > init_level) v = init_level;
                w[n] = v;
                done[n] = 1;
                if (orc_push(&h, v, (int64_t)n)) { free(done); free(h.a); return 3; }
            }
    }
    free(done);
    free(h.a);
    return 0;
}

/* ------------------------------------------------------------------- SCA --
 * apps/hydrology/scad8/scaOperator.cpp:37-131 on a float64 D8 raster (codes as
 * the reference D8 writes them).  The degree layer starts as nodata everywhere
 * (copyLayerInfo, scaOperator.cpp:14), the output as nodata.
 * orc_sca_sweeps runs the reference phases in raster order, in place:
 * max_accum_sweeps = 1 is the shipped operator (it stops after one
 * accumulation sweep, :126); larger values keep sweeping while any in-degree
 * is positive (the converged contract).  *sweeps = accumulation sweeps run. */
int orc_sca_sweeps(const double* d8, int rows, int cols, double nodata, int max_accum_sweeps, double* sca,
                   int* sweeps) {
    if (rows < 3 || cols < 3) return 1;
    size_t N = (size_t)rows * cols;
    double* deg = (double*)malloc(N * sizeof(double));
    if (!deg) return 3;
    for (size_t c = 0; c < N; c++) { deg[c] = nodata; sca[c] = nodata; }
    const int maxRow = rows - 2, maxCol = cols - 2;
    for (int i = 1; i <= maxRow; i++)                                  /* phase 0 :46-63 */
        for (int j = 1; j <= maxCol; j++) {
            size_t c = (size_t)i * cols + j;
            if (fabs(d8[c] - nodata) < ORC_EPS_HYDRO) { deg[c] = -2; sca[c] = nodata; }
            else { deg[c] = 0; sca[c] = 1; }
        }
    for (int i = 1; i <= maxRow; i++)                                  /* phase 1 :65-84 */
        for (int j = 1; j <= maxCol; j++) {
            size_t c = (size_t)i * cols + j;
            int dir = 8;
            for (int r = i - 1; r <= i + 1; r++)
                for (int q = j - 1; q <= j + 1; q++) {
                    double t = d8[(size_t)r * cols + q];
                    if (t == dir && (dir + d8[c] != 8) && dir != 4 && fabs(d8[c] - nodata) > ORC_EPS_HYDRO)
                        deg[c]++;
                    dir--;
                }
        }
    int n = 0;
    for (;;) {                                                          /* phase 2 :86-128 */
        n++;
        for (int i = 1; i <= maxRow; i++)
            for (int j = 1; j <= maxCol; j++) {
                size_t c = (size_t)i * cols + j;
                int last = (i == maxRow && j == maxCol);
                if (deg[c] <= 0 && !last) continue;
                int dir = 8;
                for (int r = i - 1; r <= i + 1; r++)
                    for (int q = j - 1; q <= j + 1; q++) {
                        size_t t = (size_t)r * cols + q;
                        if ((deg[t] == 0 || deg[t] == -1) && d8[t] == dir) {
                            if ((dir + d8[c] != 8) && dir != 4) {
                                sca[c] += sca[t];
                                deg[c]--;
                                if (deg[c] == 0) deg[c] = -1;
                            }
                            if (deg[t] == -1) deg[t] = -2;
                        }
                        dir--;
                    }
                if (last) {
                    for (int a = 1; a <= maxRow; a++)
                        for (int b = 1; b <= maxCol; b++) {
                            size_t e = (size_t)a * cols + b;
                            if (deg[e] == 0) deg[e] = -2;
                            else if (deg[e] == -1) deg[e] = 0;
                        }
                }
            }
        if (n >= max_accum_sweeps) break;
        int left = 0;
        for (int i = 1; i <= maxRow && !left; i++)
            for (int j = 1; j <= maxCol; j++)
                if (deg[(size_t)i * cols + j] > 0) { left = 1; break; }
        if (!left) break;
    }
    if (sweeps) *sweeps = n;
    free(deg);
    return 0;
}

/* SCA by topological accumulation (Kahn order), for both contracts at once.
 *
 * In-degrees follow the reference phase-1 rule (scaOperator.cpp:65-84): a
 * neighbour p counts for c when p's code points at c, c does not point back at
 * p, and c is valid.  conv (may be NULL) receives the converged upslope count:
 * the reference rule iterated until every in-degree is consumed.  shipped (may
 * be NULL) receives what the shipped operator's single raster-order
 * accumulation sweep (:86-128) produces, in closed form:
 *   p is pulled by its receiver c  iff  p is a source (in-degree 0), or p lies
 *   before c in raster order and p is done;
 *   p is done                      iff  every inflow of p was pulled by p;
 *   shipped(c) = 1 + sum of conv(p) over the pulled inflows p of c.
 * Both reproduce the last-cell quirk: the last work cell is processed even when
 * its degree is not positive (:86), so when it is nodata it adds its pulled
 * inflows onto the nodata value.  Returns 4 if some in-degree is never consumed
 * (a cycle, or an inflow from the ring, whose degree the reference never
 * releases); the cells concerned keep their partial sums. */
int orc_sca_topo(const double* d8, int rows, int cols, double nodata, double* conv, double* shipped) {
    if (rows < 3 || cols < 3) return 1;
    size_t N = (size_t)rows * cols;
    int32_t* deg = (int32_t*)calloc(N, sizeof(int32_t));
    int64_t* q = (int64_t*)malloc(N * sizeof(int64_t));
    double* cv = (double*)malloc(N * sizeof(double));
    double* sh = (double*)malloc(N * sizeof(double));
    unsigned char* src = (unsigned char*)calloc(N, 1);
    unsigned char* notdone = (unsigned char*)calloc(N, 1);
    if (!deg || !q || !cv || !sh || !src || !notdone) {
        free(deg); free(q); free(cv); free(sh); free(src); free(notdone);
        return 3;
    }
    for (size_t c = 0; c < N; c++) { cv[c] = nodata; sh[c] = nodata; }
    const int maxRow = rows - 2, maxCol = cols - 2;
    const size_t last = (size_t)maxRow * cols + maxCol;
    int64_t qh = 0, qt = 0, valid = 0;
    for (int i = 1; i <= maxRow; i++)
        for (int j = 1; j <= maxCol; j++) {
            size_t c = (size_t)i * cols + j;
            if (fabs(d8[c] - nodata) < ORC_EPS_HYDRO) continue;
            valid++;
            cv[c] = 1;
            sh[c] = 1;
            int dir = 8;
            for (int r = i - 1; r <= i + 1; r++)
                for (int s = j - 1; s <= j + 1; s++) {
                    if (d8[(size_t)r * cols + s] == dir && (dir + d8[c] != 8) && dir != 4) deg[c]++;
                    dir--;
                }
        }
    for (int i = 1; i <= maxRow; i++)
        for (int j = 1; j <= maxCol; j++) {
            size_t c = (size_t)i * cols + j;
            if (fabs(d8[c] - nodata) >= ORC_EPS_HYDRO && deg[c] == 0) { q[qt++] = (int64_t)c; src[c] = 1; }
        }
    while (qh < qt) {
        int64_t p = q[qh++];
        double code = d8[p];
        int k = (int)code;
        if ((double)k != code || k < 0 || k > 8 || k == 4) continue; /* -1 (flat) and other codes drain nowhere */
        int r = (int)(p / cols) + k / 3 - 1, s = (int)(p % cols) + k % 3 - 1;
        if (r < 1 || s < 1 || r > maxRow || s > maxCol) continue;
        size_t c = (size_t)r * cols + s;
        int pulled = src[p] || ((size_t)p < c && !notdone[p]);
        if (fabs(d8[c] - nodata) < ORC_EPS_HYDRO) {
            if (c == last) { /* last-cell quirk: the nodata value accumulates */
                cv[c] += cv[p];
                if (pulled) sh[c] += cv[p];
            }
            continue;
        }
        if ((double)k + d8[c] == 8) continue; /* c drains back into p: excluded (:71) */
        cv[c] += cv[p];
        if (pulled) sh[c] += cv[p];
        else notdone[c] = 1;
        if (--deg[c] == 0) q[qt++] = (int64_t)c;
    }
    int rc = (qt == valid) ? 0 : 4;
    if (conv) memcpy(conv, cv, N * sizeof(double));
    if (shipped) memcpy(shipped, sh, N * sizeof(double));
    free(deg); free(q); free(cv); free(sh); free(src); free(notdone);
    return rc;
}

/* Topographic wetness index, restating TWIOperator::Operator
 * (apps/hydrology/twi/TWIOperator.cpp:42-69): on work cells (the 3x3 window
 * inside the raster) the result is nodata when any value of the window, in
 * the SCA or the slope layer, equals the SCA layer's nodata exactly (:51-55);
 * otherwise ln(sca / slope) with slope raised to Eps = 1e-7 when below it
 * (:61-65).  Ring cells keep the output layer's initial value, which
 * copyLayerInfo(slopeLayer) sets to nodata (pTWI.cpp:66); here out_nodata. */
int orc_twi(const double* slope, const double* sca, int rows, int cols, double sca_nodata, double out_nodata,
            double* twi) {
    if (rows < 0 || cols < 0) return 1;
    for (int r = 0; r < rows; r++)
        for (int c = 0; c < cols; c++) {
            const size_t i = (size_t)r * cols + c;
            if (r < 1 || c < 1 || r > rows - 2 || c > cols - 2) {
                twi[i] = out_nodata;
                continue;
            }
            int nd = 0;
            for (int a = -1; a <= 1 && !nd; a++)
                for (int b = -1; b <= 1; b++) {
                    const size_t j = (size_t)(r + a) * cols + (c + b);
                    if (sca[j] == sca_nodata || slope[j] == sca_nodata) {
                        nd = 1;
                        break;
                    }
                }
            if (nd) {
                twi[i] = sca_nodata;
                continue;
            }
            double s = slope[i];
            if (s < 0.0000001) s = 0.0000001;
            twi[i] = log(sca[i] / s);
        }
    return 0;
}

/* MFD-md flow partition weights, restating MFDOperator::Operator
 * (apps/hydrology/flowdirmfdmd/mfdOperator.cpp:36-123).  w holds 8 layers of
 * rows*cols doubles; layer i is the window position i (i < 4) or i + 1
 * (i >= 4) seen from the cell, as pMFDmd.cpp:132-137 names the files.  Work
 * cells: all 8 weights nodata when the cell is nodata (|z - nd| <= 1e-6, :60);
 * else drops to strictly lower, valid neighbours -- (z - zn) / (1.414 cs) on
 * diagonals with contour length 0.354 cs, (z - zn) / cs with 0.5 cs on
 * cardinals (:83-92) -- the exponent pe = (1 - e) min(max drop, 1) + e
 * (:100-103) and w_i = drop_i^pe l_i / sum over the window (:104-116).
 * Ring cells keep the layers' initial nodata (copyLayerInfo, pMFDmd.cpp:138). */
int orc_mfd(const void* dem, int dem_f64, int rows, int cols, double nodata, float cellsize_f, double slp_exp,
            double* w) {
    if (rows < 0 || cols < 0) return 1;
    const double cs = (double)cellsize_f;
    const size_t n = (size_t)rows * cols;
    for (size_t i = 0; i < 8 * n; i++) w[i] = nodata;
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++) {
            const size_t i = (size_t)r * cols + c;
            const double z = dem_f64 ? ((const double*)dem)[i] : (double)((const float*)dem)[i];
            if (fabs(z - nodata) <= 0.000001) continue;  /* all 8 stay nodata */
            double diff[9], l[9], maxd = 0.0;
            int dir = 0;
            for (int a = -1; a <= 1; a++)
                for (int b = -1; b <= 1; b++, dir++) {
                    const size_t j = (size_t)(r + a) * cols + (c + b);
                    const double zn = dem_f64 ? ((const double*)dem)[j] : (double)((const float*)dem)[j];
                    if (fabs(zn - nodata) <= 0.000001 || z <= zn) {
                        diff[dir] = 0.0;
                        l[dir] = 0.0;
                    } else {
                        if (dir == 0 || dir == 2 || dir == 6 || dir == 8) {
                            diff[dir] = (z - zn) / (1.414 * cs);
                            l[dir] = 0.354 * cs;
                        } else {
                            diff[dir] = (z - zn) / cs;
                            l[dir] = 0.5 * cs;
                        }
                        if (diff[dir] > maxd) maxd = diff[dir];
                    }
                }
            if (maxd > 1) maxd = 1;
            const double pe = (1 - slp_exp) * maxd + slp_exp;
            double sum = 0.0;
            for (int k = 0; k < 9; k++) sum += pow(diff[k], pe) * l[k];
            for (int k = 0; k < 8; k++) w[(size_t)k * n + i] = 0.0;
            if (sum > 0)
                for (int k = 0; k < 9; k++) {
                    if (k == 4) continue;
                    w[(size_t)(k < 4 ? k : k - 1) * n + i] = (pow(diff[k], pe) * l[k]) / sum;
                }
        }
    return 0;
}

/* MFD specific catchment area, restating the scamfdmd SCAOperator
 * (apps/hydrology/scamfdmd/scaOperator.cpp:42-113) as the reference runs it:
 * one raster sweep to initialise (sca = 1, degree 0; nodata when weight layer
 * 0 is within 1e-6 of nodata: degree -1), one to count in-degrees (neighbours
 * whose weight towards the cell is > 0), then ONE accumulation sweep in raster
 * order: a cell with degree > 0 adds sca(n) w(n -> cell) for each neighbour n
 * whose degree is 0 at that moment, in window order, and decrements its own
 * degree.  Ring cells stay nodata; the degree layer's ring holds nodata. */
int orc_sca_mfd(const double* w, int rows, int cols, double nodata, double* sca) {
    if (rows < 0 || cols < 0) return 1;
    const size_t n = (size_t)rows * cols;
    double* deg = (double*)malloc(n * sizeof(double));
    if (!deg) return 2;
    for (size_t i = 0; i < n; i++) {
        sca[i] = nodata;
        deg[i] = nodata;
    }
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++) {
            const size_t i = (size_t)r * cols + c;
            if (fabs(w[i] - nodata) < 0.000001) {
                deg[i] = -1;
                sca[i] = nodata;
            } else {
                deg[i] = 0;
                sca[i] = 1;
            }
        }
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++) {
            const size_t i = (size_t)r * cols + c;
            int dir = 8;
            for (int a = -1; a <= 1; a++)
                for (int b = -1; b <= 1; b++, dir--) {
                    const size_t j = (size_t)(r + a) * cols + (c + b);
                    if (dir > 4 && w[(size_t)(dir - 1) * n + j] > 0) deg[i]++;
                    if (dir < 4 && w[(size_t)dir * n + j] > 0) deg[i]++;
                }
        }
    for (int r = 1; r < rows - 1; r++)
        for (int c = 1; c < cols - 1; c++) {
            const size_t i = (size_t)r * cols + c;
            if (deg[i] <= 0) continue;
            int dir = 8;
            for (int a = -1; a <= 1; a++)
                for (int b = -1; b <= 1; b++, dir--) {
                    const size_t j = (size_t)(r + a) * cols + (c + b);
                    if (dir > 4 && deg[j] == 0 && w[(size_t)(dir - 1) * n + j] > 0) {
                        sca[i] += sca[j] * w[(size_t)(dir - 1) * n + j];
                        deg[i]--;
                    }
                    if (dir < 4 && deg[j] == 0 && w[(size_t)dir * n + j] > 0) {
                        sca[i] += sca[j] * w[(size_t)dir * n + j];
                        deg[i]--;
                    }
                }
        }
    free(deg);
    return 0;
}

/* Compute-intensity layer, restating ComputeLayer::_init (gpro/computeLayer.h:
 * 210-262: ceil(work rows / grain) x ceil(work cols / grain) cells, all 0) and
 * the intensity-ratio Transformation::Operator (gpro/transformation.h:155-197)
 * for a 3x3 data neighbourhood (data work rectangle [1, rows-2] x [1, cols-2]):
 * compute cell (r, c) sums, data row by data row, valid_load for a data cell
 * with |v - nodata| > 1e-7 and nodata_load otherwise, over rows
 * r*grain + 1 .. (r+1)*grain and columns c*grain + 1 .. (c+1)*grain, skipping
 * cells past the raster's last row / column.  With compute_ring the compute
 * layer has a 3x3 neighbourhood of its own and its ring cells stay 0.
 * data: float (is_f64 = 0) or double.  `layers` data rasters are summed in turn. */
int orc_compute_load(const void* data, int is_f64, int layers, int rows, int cols, double nodata, int grain,
                     double nodata_load, double valid_load, int compute_ring, double* load) {
    if (rows < 3 || cols < 3 || grain < 1 || layers < 1) return 1;
    const int crows = (rows - 2 + grain - 1) / grain, ccols = (cols - 2 + grain - 1) / grain;
    const size_t n = (size_t)rows * cols;
    for (size_t i = 0; i < (size_t)crows * ccols; i++) load[i] = 0.0;
    const int r0 = compute_ring ? 1 : 0, r1 = compute_ring ? crows - 2 : crows - 1;
    const int c0 = compute_ring ? 1 : 0, c1 = compute_ring ? ccols - 2 : ccols - 1;
    for (int cr = r0; cr <= r1; cr++)
        for (int cc = c0; cc <= c1; cc++) {
            double acc = 0.0;
            for (int l = 0; l < layers; l++)
                for (int dr = cr * grain + 1; dr < (cr + 1) * grain + 1; dr++)
                    for (int dc = cc * grain + 1; dc < (cc + 1) * grain + 1; dc++) {
                        if (dr > rows - 1 || dc > cols - 1) continue;
                        const size_t i = (size_t)l * n + (size_t)dr * cols + dc;
                        const double v = is_f64 ? ((const double*)data)[i] : (double)((const float*)data)[i];
                        acc += fabs(v - nodata) > 0.0000001 ? valid_load : nodata_load;
                    }
            load[(size_t)cr * ccols + cc] = acc;
        }
    return 0;
}

/* Row-wise decomposition of a compute layer by load, restating
 * DeComposition::valRowDcmp (gpro/deComposition.h:305-393) -- per-row loads
 * (cells above -9999 and above nodata by more than 1e-7, summed left to
 * right), then nparts-1 greedy cuts, each closing a part at the row where the
 * running load passes the current average or just before it, whichever is
 * nearer -- and the mapping of ComputeLayer::getCompuLoad
 * (gpro/computeLayer.h:402-430) to data rows of a 3x3 data neighbourhood:
 * part i starts at (int)(first compute row * data_rows / compute rows + 1).
 * comp_rows[2i], [2i+1]: compute rows of part i; bounds[4i..4i+3]: its data
 * rectangle {minRow, minCol, maxRow, maxCol}.  Returns 2 when the cuts run out
 * of rows (the reference then indexes past its part list). */
int orc_load_decompose(const double* load, int crows, int ccols, double nodata, int compute_ring, int data_rows,
                       int data_cols, int nparts, int* comp_rows, int* bounds) {
    const int work_rows = compute_ring ? crows - 2 : crows;
    if (nparts < 1 || nparts > work_rows) return 1;
    double* row_load = (double*)malloc(sizeof(double) * (size_t)(crows > 0 ? crows : 1));
    if (!row_load) return 3;
    double total = 0.0;
    for (int r = 0; r < crows; r++) {
        row_load[r] = 0.0;
        for (int c = 0; c < ccols; c++) {
            const double v = load[(size_t)r * ccols + c];
            if ((v + 9999) > 0.0000001 && (v - nodata) > 0.0000001) row_load[r] += v;
        }
        total += row_load[r];
    }
    double aver = total / nparts, accu = 0.0;
    int begin = 0, end = 0, k = 0;
    for (int i = 0; i < nparts - 1; i++) {
        double sub = 0.0, min_diff = 0.0;
        int cut = 0;
        for (int r = begin; r < crows; r++) {
            sub += row_load[r];
            accu += row_load[r];
            if (sub <= aver && crows - 1 - r > nparts - 1 - i) {
                if (fabs(min_diff) < 0.0000001 || (aver - sub) < min_diff) min_diff = aver - sub;
            } else {
                if (fabs(min_diff) < 0.0000001 || (sub - aver) <= min_diff || crows - 1 - r == nparts - 1 - i) {
                    end = r;
                    comp_rows[2 * k] = begin;
                    comp_rows[2 * k + 1] = end;
                    k++;
                    aver = (total - accu) / (nparts - i - 1);
                    begin = r + 1;
                } else {
                    end = r - 1;
                    accu -= row_load[r];
                    comp_rows[2 * k] = begin;
                    comp_rows[2 * k + 1] = end;
                    k++;
                    sub -= row_load[r];
                    aver = (total - accu) / (nparts - i - 1);
                    begin = r;
                }
                cut = 1;
                break;
            }
        }
        if (!cut) {
            free(row_load);
            return 2;
        }
    }
    comp_rows[2 * k] = begin;
    comp_rows[2 * k + 1] = crows - 1;
    free(row_load);
    /* data rows */
    const double convert = data_rows / (double)crows;
    const int wmin_r = 1, wmax_r = data_rows - 2, wmin_c = 1, wmax_c = data_cols - 2;
    int sub_begin = wmin_r, sub_end = wmin_r - 1, i = 0;
    for (; i < nparts - 1; i++) {
        sub_begin = (int)(comp_rows[2 * i] * convert + wmin_r);
        sub_end = (int)(comp_rows[2 * (i + 1)] * convert + wmin_r - 1);
        bounds[4 * i] = sub_begin;
        bounds[4 * i + 1] = wmin_c;
        bounds[4 * i + 2] = sub_end;
        bounds[4 * i + 3] = wmax_c;
    }
    bounds[4 * i] = sub_end + 1;
    bounds[4 * i + 1] = wmin_c;
    bounds[4 * i + 2] = wmax_r;
    bounds[4 * i + 3] = wmax_c;
    return 0;
}
