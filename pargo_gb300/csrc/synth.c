/*
 * synth.c -- seeded synthetic DEM generator for the benchmark and test workloads.
 *
 * Fractional-Brownian surfaces by diamond-square midpoint displacement, plus the
 * workload-specific edits (nodata border, lowered pit cells, a random-walk
 * nodata blob, a Gaussian-like perturbation).  The output depends only on the
 * arguments: the random numbers come from a counter-based hash of
 * (seed, stream, i, j), every level is computed from the previous one only (so
 * the OpenMP row split does not change the result), and the arithmetic is
 * plain IEEE double with no library transcendental calls (2^-H is evaluated by
 * a fixed series), so x86-64 and aarch64 builds give identical bytes when
 * compiled with -ffp-contract=off.
 */
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

static inline uint64_t syn_mix(uint64_t x) {
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
static inline uint64_t syn_hash4(uint64_t seed, uint64_t stream, uint64_t i, uint64_t j) {
    return syn_mix(syn_mix(syn_mix(syn_mix(seed) ^ stream) ^ i) ^ j);
}
/* uniform in [0, 1) with 53 random bits */
static inline double syn_u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }

double pargo_synth_u01(uint64_t seed, uint64_t stream, uint64_t i, uint64_t j) {
    return syn_u01(syn_hash4(seed, stream, i, j));
}

/* 2^-h for 0 <= h <= 4 by the exponential series of -h*ln2 (fixed term count). */
static double syn_exp2_neg(double h) {
    const double ln2 = 0.69314718055994530942;
    double x = -h * ln2, term = 1.0, sum = 1.0;
    for (int n = 1; n < 40; n++) {
        term = term * x / (double)n;
        sum += term;
    }
    return sum;
}

/* Diamond-square fBm on the (2^k+1)^2 grid that covers rows x cols, cropped to
 * rows x cols and rescaled linearly to [lo, hi]; written as float32. */
int pargo_synth_fbm(uint64_t seed, double hurst, double lo, double hi, int rows, int cols, float* out) {
    if (rows < 2 || cols < 2 || !out) return 1;
    int need = rows > cols ? rows : cols;
    int64_t m = 2;
    while (m + 1 < need) m *= 2;
    m += 1;
    float* g = (float*)malloc((size_t)m * (size_t)m * sizeof(float));
    if (!g) return 3;
#define G(i, j) g[(size_t)(i) * (size_t)m + (size_t)(j)]
    const double decay = syn_exp2_neg(hurst);
    G(0, 0) = (float)syn_u01(syn_hash4(seed, 1, 0, 0));
    G(0, m - 1) = (float)syn_u01(syn_hash4(seed, 1, 0, m - 1));
    G(m - 1, 0) = (float)syn_u01(syn_hash4(seed, 1, m - 1, 0));
    G(m - 1, m - 1) = (float)syn_u01(syn_hash4(seed, 1, m - 1, m - 1));
    double amp = 0.5;
    for (int64_t s = m - 1; s > 1; s /= 2) {
        int64_t h = s / 2;
        uint64_t stream = 2 + (uint64_t)s;
        int64_t nsq = (m - 1) / s;
        /* diamond: centres of the s x s squares */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t a = 0; a < nsq; a++) {
            int64_t i = a * s + h;
            for (int64_t j = h; j < m; j += s) {
                double avg = ((double)G(i - h, j - h) + (double)G(i - h, j + h) + (double)G(i + h, j - h) +
                              (double)G(i + h, j + h)) * 0.25;
                double u = syn_u01(syn_hash4(seed, stream, (uint64_t)i, (uint64_t)j));
                G(i, j) = (float)(avg + amp * (2.0 * u - 1.0));
            }
        }
        /* square: edge midpoints, averaging the 3 or 4 existing neighbours */
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
        for (int64_t i = 0; i < m; i += h) {
            int64_t j0 = ((i / h) % 2 == 0) ? h : 0;
            for (int64_t j = j0; j < m; j += s) {
                double sum = 0.0;
                int n = 0;
                if (i - h >= 0) { sum += (double)G(i - h, j); n++; }
                if (i + h < m) { sum += (double)G(i + h, j); n++; }
                if (j - h >= 0) { sum += (double)G(i, j - h); n++; }
                if (j + h < m) { sum += (double)G(i, j + h); n++; }
                double u = syn_u01(syn_hash4(seed, stream + 0x100000000ull, (uint64_t)i, (uint64_t)j));
                G(i, j) = (float)(sum / (double)n + amp * (2.0 * u - 1.0));
            }
        }
        amp *= decay;
    }
    double mn = 1e300, mx = -1e300;
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            double v = (double)G(i, j);
            if (v < mn) mn = v;
            if (v > mx) mx = v;
        }
    double scale = mx > mn ? (hi - lo) / (mx - mn) : 0.0;
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            out[(size_t)i * cols + j] = (float)(lo + ((double)G(i, j) - mn) * scale);
#undef G
    free(g);
    return 0;
}

/* Set a border of `width` cells to nodata. */
void pargo_synth_border(float* dem, int rows, int cols, int width, float nodata) {
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++)
            if (i < width || j < width || i >= rows - width || j >= cols - width)
                dem[(size_t)i * cols + j] = nodata;
}

/* Lower a seeded `fraction` of the cells by U(0, depth): artificial pits. */
void pargo_synth_pits(float* dem, int rows, int cols, uint64_t seed, double fraction, double depth, float nodata) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            size_t c = (size_t)i * cols + j;
            if (dem[c] == nodata) continue;
            if (syn_u01(syn_hash4(seed, 0x5157ull, (uint64_t)i, (uint64_t)j)) < fraction) {
                double u = syn_u01(syn_hash4(seed, 0x5158ull, (uint64_t)i, (uint64_t)j));
                dem[c] = (float)((double)dem[c] - depth * u);
            }
        }
}

/* Irregular nodata blob: a seeded random walk with a 3x3 brush, started at a
 * seeded cell, until `fraction` of the raster is nodata (or a step cap).
 * Returns the number of nodata cells written. */
int64_t pargo_synth_blob(float* dem, int rows, int cols, uint64_t seed, double fraction, float nodata) {
    int64_t target = (int64_t)(fraction * (double)rows * (double)cols);
    int64_t count = 0;
    for (size_t c = 0; c < (size_t)rows * cols; c++) count += (dem[c] == nodata);
    int64_t r = (int64_t)(syn_u01(syn_hash4(seed, 0xB10Bull, 0, 0)) * rows);
    int64_t q = (int64_t)(syn_u01(syn_hash4(seed, 0xB10Bull, 0, 1)) * cols);
    int64_t cap = (int64_t)rows * cols * 64;
    static const int dr[8] = {-1, -1, -1, 0, 0, 1, 1, 1}, dc[8] = {-1, 0, 1, -1, 1, -1, 0, 1};
    for (int64_t step = 0; count < target && step < cap; step++) {
        for (int a = -1; a <= 1; a++)
            for (int b = -1; b <= 1; b++) {
                int64_t rr = r + a, qq = q + b;
                if (rr < 0 || qq < 0 || rr >= rows || qq >= cols) continue;
                float* p = &dem[(size_t)rr * cols + qq];
                if (*p != nodata) { *p = nodata; count++; }
            }
        uint64_t h = syn_hash4(seed, 0xB10Cull, (uint64_t)step, 0);
        int k = (int)(h % 8);
        r += dr[k];
        q += dc[k];
        if (r < 0) r = 0;
        if (q < 0) q = 0;
        if (r >= rows) r = rows - 1;
        if (q >= cols) q = cols - 1;
    }
    return count;
}

/* Add sigma * (Irwin-Hall sum of 12 uniforms - 6): a seeded, nearly Gaussian
 * N(0, sigma^2) perturbation, to every non-nodata cell. */
void pargo_synth_perturb(const float* dem, float* out, int rows, int cols, uint64_t seed, double sigma, float nodata) {
#ifdef _OPENMP
#pragma omp parallel for schedule(static)
#endif
    for (int i = 0; i < rows; i++)
        for (int j = 0; j < cols; j++) {
            size_t c = (size_t)i * cols + j;
            if (dem[c] == nodata) { out[c] = nodata; continue; }
            double s = 0.0;
            for (int k = 0; k < 12; k++)
                s += syn_u01(syn_hash4(seed, 0x6A05ull + (uint64_t)k, (uint64_t)i, (uint64_t)j));
            out[c] = (float)((double)dem[c] + sigma * (s - 6.0));
        }
}
