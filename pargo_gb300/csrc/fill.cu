// fill.cu -- Planchon-Darboux pit removal (epsilon filling) by tiled
// relaxation with worklists.
//
// Reference: PitRemoveOperator::Operator (apps/hydrology/pitremove/
// pitRemoveOperator.cpp:26-72) swept by RasterOperator::Work
// (gpro/rasterOperator.h:169-219) until a sweep changes nothing.  Per valid
// cell c with level W(c) > dem(c), one visit computes
//     W(c) <- dem(c)                      if some neighbour n has a nodata level
//                                         or dem(c) >= W(n) + gap,
//     W(c) <- min(W(c), min_n W(n) + gap) otherwise,
// with W(n) + gap rounded to double exactly as the reference adds it.  The
// update is monotone (levels only fall) so every visiting order -- the
// reference's raster-order Gauss-Seidel, Jacobi, or this chaotic tiled order --
// ends at the same fixpoint, bit for bit.
//
// GPU structure
//  * init: levels = +inf on the nodata ring and on nodata cells (standing for
//    the reference's nodata level), init_level on valid cells, and dem(c) at
//    once on valid cells next to a nodata level (their first visit does that).
//    Only tiles holding such outlet cells start on the worklist: every other
//    tile is stable until a neighbour's border moves and requests it.
//  * rounds: a worklist of 32 x 32 tiles.  A CTA claims a tile, loads its
//    levels plus a one-cell halo into shared memory, relaxes the tile until it
//    is stable against that halo, writes back the cells that changed and puts
//    the neighbour tiles whose halo changed on the next worklist.  Rounds run
//    until the worklist is empty (a device-side count the host reads after a
//    CUDA graph of rounds).  The persistent form runs the same visits in one
//    launch over a device ring of tile ids.
//  * levels are kept as double bit patterns in an order-preserving integer
//    key, so min/compare run on the integer pipes; W + gap is done on the bit
//    pattern with a per-binade step table (the exact double sum while the sum
//    stays in the binade) and with a real double add otherwise.

#include <math.h>

#include <map>
#include <mutex>

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kT = 32;            // tile side
constexpr int kH = kT + 2;        // with halo
constexpr int kLS = kH + 1;       // 35: row stride of the level tile (odd, conflict-free both ways)
constexpr int kZS = kT + 1;       // 33: row stride of the DEM-key tile
constexpr int kThreads = 256;     // threads per tile
constexpr int kRun = kT * kT / kThreads;  // 4: cells of a thread's run (a row run, then a column run)
constexpr int kRunsPerLine = kT / kRun;   // 8
constexpr int kLocalCap = 4096;   // relaxation sweeps per visit before the tile re-queues itself
constexpr int64_t kKeyInf = 0x7FF0000000000000LL;  // key of +inf
// FillScratch::q slots of the persistent form
constexpr int kQHead = 0, kQTail = 1, kQPending = 2, kQProgress = 3, kQError = 4;
constexpr int kQErrPop = 1, kQErrPush = 2, kQErrState = 3;
constexpr uint32_t kHaloAll = 0x80000000u;  // halo_chg corner-word flag: relax every cell of the tile

// Per biased exponent e: fl64(x + gap) - x in ulps of x's binade when that
// is the same for every x of the binade, else -1 (subnormals, inf/nan, a sum
// that can leave the binade, and the binade in which gap is an odd number of
// half-ulps, where the tie rounds by the parity of x): those use the double add.
// In constant memory: the cells a warp relaxes together mostly share a
// binade, so the lookup is a broadcast (8192^2 fill 12.7 -> 12.3 ms against
// a global-memory table).
__constant__ int64_t g_step[2048];

__device__ __forceinline__ int64_t dkey(double x) {
    int64_t b = __double_as_longlong(x);
    return b ^ ((b >> 63) & 0x7FFFFFFFFFFFFFFFLL);
}
__device__ __forceinline__ double dval(int64_t k) { return __longlong_as_double(k ^ ((k >> 63) & 0x7FFFFFFFFFFFFFFFLL)); }

// key of fl64(x + gap) for x = dval(k)
__device__ __forceinline__ int64_t add_gap(int64_t k, double gap) {
    if (k >= 0 && k < kKeyInf) {
        const int e = (int)(k >> 52);
        const int64_t st = g_step[e];
        if (st >= 0) {
            const int64_t y = k + st;
            if ((int)(y >> 52) == e) return y;
        }
    }
    return dkey(__dadd_rn(dval(k), gap));
}

// The DEM value at (r, c) as an order-preserving key of its double value,
// from the bits: a float DEM widened to double and compared in double would
// cost conversions and compares on the FP64 pipe (a narrow pipe on this part)
// for every cell a visit loads.
__device__ __forceinline__ int64_t dem_key(const FillParams& p, int64_t r, int64_t c) {
    const char* row = reinterpret_cast<const char*>(p.dem) + r * p.dem_pitch;
    return p.dem_f64 ? dkey(reinterpret_cast<const double*>(row)[c]) : fkey64(reinterpret_cast<const float*>(row)[c]);
}

// A level into a filled-DEM output, nodata levels (+inf) as the output's
// nodata; float output rounded on the integer pipes.
__device__ __forceinline__ void put_level(const OutView& o, int64_t r, int64_t c, double w, bool nd, float nd_f) {
    char* row = o.base + r * o.pitch;
    if (o.dtype == PARGO_F32) reinterpret_cast<float*>(row)[c] = nd ? nd_f : dbl2flt_rn(w);
    else put_value(o, r, c, nd ? o.nodata : w);
}

// Tile bookkeeping: every ring slot empty, every tile idle with no halo
// changes, the counters zero.
__global__ void fill_init_tiles_kernel(const FillParams p, FillScratch s) {
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
        s.list_a[t] = -1;  // ring positions 0 .. ntiles-1
        s.list_b[t] = -1;  // and ntiles .. 2 ntiles-1
        s.queued[t] = 0;
#pragma unroll
        for (int k = 0; k < 5; k++) s.halo_chg[t * 5 + k] = 0u;
    }
    if (blockIdx.x == 0 && threadIdx.x < 4) s.counts[threadIdx.x] = 0;
    if (blockIdx.x == 0 && threadIdx.x < 5) s.q[threadIdx.x] = 0;
}

// Levels: +inf on the nodata ring and nodata cells, init_level on valid
// cells, dem(c) at once on valid cells next to a nodata level (their first
// visit does that).  A tile holding such an outlet cell is marked for a first
// visit that relaxes every cell; any other tile is stable as initialised
// (its cells see init_level or +inf around them, and init_level + gap is
// above init_level) until a neighbour's border moves and requests it.
// A block works tile by tile: it stages the tile's 34 x 34 window of DEM keys
// and nodata flags (each DEM value read about 1.13 times; the earlier
// row-band form read every value nine times, 0.42 ms per 8192^2 launch),
// writes the tile's 32 x 32 levels and marks the tile when it holds an
// outlet cell.
__global__ void __launch_bounds__(256) fill_init_tile_kernel(const FillParams p, FillScratch s) {
    __shared__ int64_t zk[kH * kH];
    __shared__ uint8_t ndf[kH * kH];  // 1: a nodata level (nodata DEM value, the ring, beyond the raster)
    const int tid = threadIdx.x;
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    const int64_t kinit = dkey(p.init_level);
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t y0 = (t / p.tiles_x) * kT - 1, x0 = (t % p.tiles_x) * kT - 1;  // window origin
        // the window's DEM values, every load of a thread issued before the
        // first is converted (one memory round trip per tile)
        constexpr int kPer = (kH * kH + 255) / 256;  // 5
        int64_t raw[kPer];
        bool in[kPer];
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int i = tid + q * 256;
            const int64_t r = y0 + i / kH, c = x0 + i % kH;
            in[q] = i < kH * kH && r > 0 && c > 0 && r < p.rows - 1 && c < p.cols - 1;
            raw[q] = 0;
            if (in[q]) {
                const char* row = reinterpret_cast<const char*>(p.dem) + r * p.dem_pitch;
                raw[q] = p.dem_f64 ? reinterpret_cast<const long long*>(row)[c]
                                   : (long long)reinterpret_cast<const unsigned*>(row)[c];
            }
        }
#pragma unroll
        for (int q = 0; q < kPer; q++) {
            const int i = tid + q * 256;
            if (i >= kH * kH) continue;
            bool nd = true;
            int64_t k = kKeyInf;
            if (in[q]) {
                if (p.dem_f64) {
                    k = dkey(__longlong_as_double(raw[q]));
                    nd = k >= dkey(p.nd6d.lo) && k <= dkey(p.nd6d.hi);  // an empty band has lo > hi: its keys too
                } else {
                    const float f = __uint_as_float((unsigned)raw[q]);
                    k = fkey64(f);
                    nd = p.nd6f.has(f);
                }
            }
            zk[i] = k;
            ndf[i] = nd ? 1 : 0;
        }
        __syncthreads();
        int outlet_here = 0;
        for (int i = tid; i < kT * kT; i += 256) {
            const int lr = i / kT, lc = i % kT;
            const int64_t r = y0 + 1 + lr, c = x0 + 1 + lc;
            if (r >= p.rows || c >= p.cols) continue;
            const int w0 = lr * kH + lc;  // the window's top-left in the staged arrays
            double w = INFINITY;
            if (!ndf[w0 + kH + 1]) {      // a valid work cell (the ring and nodata are flagged)
                const int64_t kz = zk[w0 + kH + 1];
                w = p.init_level;
                if (kinit > kz) {
                    const bool outlet = ndf[w0] | ndf[w0 + 1] | ndf[w0 + 2] | ndf[w0 + kH] | ndf[w0 + kH + 2] |
                                        ndf[w0 + 2 * kH] | ndf[w0 + 2 * kH + 1] | ndf[w0 + 2 * kH + 2];
                    if (outlet) {
                        w = dval(kz);
                        outlet_here = 1;
                    }
                }
            }
            p.w[r * p.w_stride + c] = w;
        }
        if (__syncthreads_or(outlet_here) && tid == 0) s.halo_chg[t * 5 + 4] = kHaloAll;
    }
}

// The first worklist (and ring): the tiles marked by fill_init_tile_kernel.
__global__ void fill_seed_kernel(const FillParams p, FillScratch s) {
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < ntiles; t += (int64_t)gridDim.x * blockDim.x) {
        if (!(s.halo_chg[t * 5 + 4] & kHaloAll)) continue;
        s.queued[t] = 1;
        s.list_a[atomicAdd(&s.counts[0], 1)] = (int32_t)t;
        atomicAdd(&s.q[kQTail], 1ULL);
        atomicAdd(&s.q[kQPending], 1ULL);
    }
}

__device__ __forceinline__ void enqueue(const FillScratch& s, int32_t* next, int32_t* next_count, int64_t ty, int64_t tx,
                                        const FillParams& p) {
    if (ty < 0 || tx < 0 || ty >= p.tiles_y || tx >= p.tiles_x) return;
    const int32_t t = (int32_t)(ty * p.tiles_x + tx);
    if (atomicExch(&s.queued[t], 1) == 0) next[atomicAdd(next_count, 1)] = t;
}

// ---- persistent form: one launch, a ring of tile ids ----------------------
// The ring has 2 * ntiles slots (-1 = empty).  A tile is in the ring at most
// once (its queued flag is set from its push until a visitor takes it), so
// fewer than ntiles slots are ever full and a pusher finds its slot empty or
// about to be emptied by the visitor that claimed that position.  q[kQPending]
// counts tiles pushed and not yet finished: it is raised before a push and
// lowered only after a visit has pushed its neighbours, so it reaches 0 only
// when the ring is empty and no visit is in flight -- the device-side
// convergence flag.  Every wait gives up after `patience` cycles without a
// finished visit anywhere (or without its slot emptying), sets q[kQError] and
// returns; the host reports that as a device timeout.

__device__ __forceinline__ unsigned long long vload64(const unsigned long long* a) {
    return *((const volatile unsigned long long*)a);
}

__device__ void ring_push(const FillScratch& s, int32_t t, long long patience) {
    atomicAdd(&s.q[kQPending], 1ULL);
    const unsigned long long pos = atomicAdd(&s.q[kQTail], 1ULL);
    int32_t* slot = &s.ring[pos % (unsigned long long)s.ring_cap];
    const long long t0 = clock64();
    unsigned ns = 32;
    while (atomicCAS(slot, -1, t) != -1) {
        if (vload64(&s.q[kQError]) != 0) return;
        if (clock64() - t0 > patience) {
            atomicCAS(&s.q[kQError], 0ULL, (unsigned long long)kQErrPush);
            return;
        }
        __nanosleep(ns);
        if (ns < 1024) ns *= 2;
    }
}

// Next tile to visit, or -1 once the work is done (or a wait gave up).  The
// slot is taken by exchanging it with -1: an empty slot stays empty, a full
// one is taken by exactly one of the visitors that share it.
__device__ int32_t ring_pop(const FillScratch& s, long long patience) {
    const unsigned long long pos = atomicAdd(&s.q[kQHead], 1ULL);
    int32_t* slot = &s.ring[pos % (unsigned long long)s.ring_cap];
    unsigned long long seen = vload64(&s.q[kQProgress]);
    long long t0 = clock64();
    unsigned ns = 32;
    for (;;) {
        const int32_t v = atomicExch(slot, -1);
        if (v >= 0) return v;
        if (vload64(&s.q[kQPending]) == 0 || vload64(&s.q[kQError]) != 0) return -1;
        const unsigned long long pr = vload64(&s.q[kQProgress]);
        if (pr != seen) {
            seen = pr;
            t0 = clock64();
        } else if (clock64() - t0 > patience) {
            atomicCAS(&s.q[kQError], 0ULL, (unsigned long long)kQErrPop);
            return -1;
        }
        __nanosleep(ns);
        if (ns < 2048) ns *= 2;
    }
}

// Tile states of the persistent form (in FillScratch::queued).  A tile has at
// most one visitor: a request for a running tile only marks it dirty, and the
// visitor queues it again when it finishes, so a visit that read a halo
// before a neighbour's write is always followed by one that reads after it.
constexpr int32_t kIdle = 0, kQueued = 1, kRunning = 2, kRunningDirty = 3;

__device__ void request_tile(const FillScratch& s, int32_t t, long long patience) {
    int32_t st = kIdle;  // the common state: the first CAS either queues the tile or returns its state
    for (int guard = 0; guard < 64; guard++) {  // each failed CAS means another thread moved the state
        int32_t want;
        if (st == kIdle) want = kQueued;
        else if (st == kRunning) want = kRunningDirty;
        else return;  // already queued, or will be queued by its visitor
        const int32_t old = atomicCAS(&s.queued[t], st, want);
        if (old == st) {
            if (want == kQueued) ring_push(s, t, patience);
            return;
        }
        st = old;
    }
    atomicCAS(&s.q[kQError], 0ULL, (unsigned long long)kQErrState);
}

// Record, in tile (ty, tx)'s halo-change words, cells of its halo that this
// visit changed (word k, bits); ignored outside the raster's tiles.
__device__ __forceinline__ void mark_halo(const FillScratch& s, const FillParams& p, int64_t ty, int64_t tx, int k,
                                          uint32_t bits) {
    if (ty < 0 || tx < 0 || ty >= p.tiles_y || tx >= p.tiles_x || !bits) return;
    atomicOr(&s.halo_chg[(ty * p.tiles_x + tx) * 5 + k], bits);
}

template <bool PERSIST>
__device__ __forceinline__ void put_tile(const FillScratch& s, int32_t* next, int32_t* next_count, int64_t ty, int64_t tx,
                                         const FillParams& p, long long patience) {
    if (!PERSIST) {
        enqueue(s, next, next_count, ty, tx, p);
        return;
    }
    if (ty < 0 || tx < 0 || ty >= p.tiles_y || tx >= p.tiles_x) return;
    request_tile(s, (int32_t)(ty * p.tiles_x + tx), patience);
}

// One CTA visits one 32 x 32 tile at a time: claim, load levels + halo into
// shared memory, relax to stability against the halo, write back what changed
// and queue the neighbours whose halo moved.  PERSIST = false: one round of
// the current worklist (a launch per round).  PERSIST = true: the whole fill
// in one launch over the ring; a tile requested again while it was being
// visited is visited again at once by the same CTA, which still holds its
// interior and reloads only the halo.
// 8 CTAs of 256 threads per SM (full warp occupancy, 32 registers): the
// visits are latency bound, and occupancy measured worth more than the few
// registers spilled at this bound (8192^2: 25.0 -> 22.8 ms).  Runs of 8 cells
// (128 threads, 12 CTAs per SM) took fewer passes but more visits and more
// time (19.9 ms against 12.8); fewer resident CTAs took fewer visits but
// more time (6 per SM: 13.4 ms).
template <bool PERSIST>
__global__ void __launch_bounds__(kThreads, 8) fill_tiles_kernel(const FillParams p, FillScratch s, int parity,
                                                              long long patience) {
    // Levels with the halo and the tile's DEM keys, both with odd row strides
    // (35 and 33 words of 8 bytes): a warp reading row runs or column runs
    // touches every bank pair equally, so neither mapping conflicts.
    __shared__ int64_t lv[kH * kLS];
    __shared__ int64_t zs[kT * kZS];
    __shared__ uint32_t dirty[kT];      // bit c of word r: cell (r, c) changed during this visit
    __shared__ uint32_t stale[kT];      // bit c of word r: a neighbour of (r, c) changed since (r, c) was last relaxed
    __shared__ uint32_t hmask[5];       // this visit's halo-change words
    __shared__ uint32_t colmask[2];     // changed cells of tile column 0 and 31 (bit = row)
    __shared__ int32_t claim;
    __shared__ int chase;               // the claimed tile is the one just visited (interior still held)
    __shared__ int edges;  // bit 0 top, 1 bottom, 2 left, 3 right, 4 tl, 5 tr, 6 bl, 7 br
    __shared__ bool last_block;
    int32_t* cur = parity ? s.list_b : s.list_a;
    int32_t* next = parity ? s.list_a : s.list_b;
    int32_t* cur_count = &s.counts[parity];
    int32_t* next_count = &s.counts[parity ^ 1];
    const int32_t ncur = PERSIST ? 0 : *((volatile int32_t*)cur_count);
    const int tid = threadIdx.x;
    if (!PERSIST && blockIdx.x == 0 && tid == 0 && ncur > 0) atomicAdd(s.active, 1ULL);
    unsigned long long st_visits = 0, st_iters = 0, st_changed = 0;  // thread 0's tallies
    if (tid == 0) chase = 0;

    for (;;) {
        if (tid == 0) {
            if (!chase) {
                if (PERSIST) {
                    claim = ring_pop(s, patience);
                } else {
                    const int32_t k = atomicAdd(&s.counts[2], 1);
                    claim = k < ncur ? cur[k] : -1;
                }
                if (claim >= 0) atomicExch(&s.queued[claim], PERSIST ? kRunning : 0);
            }
            edges = 0;
        }
        __syncthreads();
        const int32_t t = claim;
        if (t < 0) break;
        const bool held = chase;
        // Take the halo changes (one word per thread of five) before the halo
        // is read: a change recorded after this is followed by another request.
        if (tid < 5) {
            hmask[tid] = atomicExch(&s.halo_chg[(int64_t)t * 5 + tid], 0u);
            __threadfence();
        }
        __syncthreads();
        const int64_t ty = t / p.tiles_x, tx = t % p.tiles_x;
        const int64_t y0 = ty * kT - 1, x0 = tx * kT - 1;  // global coords of lv[0][0]
        if (!held) {
            // Every load of a thread is issued before the first is used (one
            // memory round trip per visit instead of one per loop trip).
            constexpr int kLvPer = (kH * kH + kThreads - 1) / kThreads;  // 5
            constexpr int kZPer = kT * kT / kThreads;                    // 4
            double wv[kLvPer];
#pragma unroll
            for (int q = 0; q < kLvPer; q++) {
                const int i = tid + q * kThreads;
                const int64_t r = y0 + i / kH, c = x0 + i % kH;
                wv[q] = INFINITY;  // key kKeyInf: beyond the raster
                if (i < kH * kH && r >= 0 && c >= 0 && r < p.rows && c < p.cols)
                    wv[q] = ((volatile double*)p.w)[r * p.w_stride + c];
            }
#pragma unroll
            for (int q = 0; q < kLvPer; q++) {
                const int i = tid + q * kThreads;
                if (i < kH * kH) lv[(i / kH) * kLS + i % kH] = dkey(wv[q]);
            }
            // DEM keys; kKeyInf where a level never moves (the raster's ring, beyond the raster)
            int64_t zk[kZPer];
#pragma unroll
            for (int q = 0; q < kZPer; q++) {
                const int i = tid + q * kThreads;
                const int64_t gr = y0 + 1 + i / kT, gc = x0 + 1 + i % kT;
                zk[q] = kKeyInf;
                if (gr > 0 && gc > 0 && gr < p.rows - 1 && gc < p.cols - 1) zk[q] = dem_key(p, gr, gc);
            }
#pragma unroll
            for (int q = 0; q < kZPer; q++) {
                const int i = tid + q * kThreads;
                zs[(i / kT) * kZS + i % kT] = zk[q];
            }
        } else if (tid < 4 * kH - 4) {
            // The same tile again: only its halo can have moved (this CTA
            // wrote its interior).  Rows 0 and 33, then columns 0 and 33.
            int a, b;
            if (tid < 2 * kH) {
                a = tid < kH ? 0 : kH - 1;
                b = tid < kH ? tid : tid - kH;
            } else {
                const int k = tid - 2 * kH;
                a = 1 + (k >> 1);
                b = (k & 1) ? kH - 1 : 0;
            }
            const int64_t r = y0 + a, c = x0 + b;
            int64_t k = kKeyInf;
            if (r >= 0 && c >= 0 && r < p.rows && c < p.cols) k = dkey(((volatile double*)p.w)[r * p.w_stride + c]);
            lv[a * kLS + b] = k;
        }
        if (tid < kT) {
            // Cells next to a halo cell that changed since the last visit (or
            // every cell on a first visit): between visits only the halo moves,
            // and the last visit left the tile stable against the halo it read.
            dirty[tid] = 0u;
            uint32_t st;
            if (hmask[4] & kHaloAll) {
                st = 0xFFFFFFFFu;
            } else {
                const uint32_t L = hmask[2] | (hmask[2] << 1) | (hmask[2] >> 1);
                const uint32_t Rr = hmask[3] | (hmask[3] << 1) | (hmask[3] >> 1);
                st = ((L >> tid) & 1u) | (((Rr >> tid) & 1u) << 31);
                if (tid == 0) st |= hmask[0] | (hmask[0] << 1) | (hmask[0] >> 1) | (hmask[4] & 1u) | (((hmask[4] >> 1) & 1u) << 31);
                if (tid == kT - 1)
                    st |= hmask[1] | (hmask[1] << 1) | (hmask[1] >> 1) | ((hmask[4] >> 2) & 1u) | (((hmask[4] >> 3) & 1u) << 31);
            }
            stale[tid] = st;
        }
        if (tid < 2) colmask[tid] = 0u;
        __syncthreads();
        // Local relaxation until a whole pass changes nothing; a pass skips the
        // cells none of whose neighbours moved since they were last relaxed
        // (the `stale` marks), so only the moving front is recomputed.  Passes
        // alternate between row runs and column runs (a thread owns 4
        // consecutive cells of one row, then of one column), and every second
        // pair of passes walks its run backwards, so a front crosses 4 cells per
        // pass in each of the four directions; within a run the update is in
        // place (Gauss-Seidel).  The marks are shared-memory atomics seen at
        // once by the other threads of the pass, which carries a front further
        // in one pass: marks gathered per warp by ballot and published once per
        // pass (no per-cell atomics or fences) measured 1.6x more passes per
        // visit and a slower fill (8192^2: 17.3 -> 27.5 ms).
        int it = 0;
        const int u = tid / kRunsPerLine, v0 = (tid % kRunsPerLine) * kRun;
        for (;;) {
            const bool colrun = it & 1, rev = (it >> 1) & 1;
            int changed = 0;
#pragma unroll
            for (int jj = 0; jj < kRun; jj++) {
                const int j = rev ? kRun - 1 - jj : jj;
                const int r = colrun ? v0 + j : u, c = colrun ? u : v0 + j;
                const uint32_t bit = 1u << c;
                if (!(stale[r] & bit)) continue;  // no neighbour moved since its last relaxation
                // Clear the mark before reading the neighbours: a neighbour that
                // changes after this (its write fenced before it marks this
                // cell) leaves the cell marked for another relaxation.
                atomicAnd(&stale[r], ~bit);
                __threadfence_block();
                const int64_t z = zs[r * kZS + c];
                const int64_t* w0 = lv + r * kLS + c;  // (a-1, b-1) of halo cell (a, b) = (r+1, c+1)
                const int64_t cur_v = w0[kLS + 1];
                if (!(cur_v > z && cur_v < kKeyInf)) continue;  // at its DEM, nodata, or never moves
                int64_t m = min(min(w0[0], w0[1]), w0[2]);
                m = min(m, min(w0[kLS], w0[kLS + 2]));
                m = min(m, min(min(w0[2 * kLS], w0[2 * kLS + 1]), w0[2 * kLS + 2]));
                const int64_t up = add_gap(m, p.gap);
                const int64_t nv = up <= z ? z : (up < cur_v ? up : cur_v);
                if (nv != cur_v) {
                    lv[(r + 1) * kLS + c + 1] = nv;
                    changed = 1;
                    atomicOr(&dirty[r], bit);
                    __threadfence_block();  // the new level before the marks
                    const uint32_t nb = bit | (bit << 1) | (bit >> 1);  // columns c-1 .. c+1 inside the tile
                    if (r > 0) atomicOr(&stale[r - 1], nb);
                    atomicOr(&stale[r], nb & ~bit);
                    if (r < kT - 1) atomicOr(&stale[r + 1], nb);
                }
            }
            it++;
            if (!__syncthreads_or(changed) || it >= kLocalCap) break;
        }
        // Write back the changed cells (row mapping) and note which borders moved.
        int e = 0;
        {
            const int r = u;
            const uint32_t d = dirty[r];
            const int64_t gr = y0 + 1 + r;
#pragma unroll
            for (int j = 0; j < kRun; j++) {
                const int c = v0 + j;
                if (!((d >> c) & 1u)) continue;
                p.w[gr * p.w_stride + (x0 + 1 + c)] = dval(lv[(r + 1) * kLS + c + 1]);
                if (r == 0) e |= 1;
                if (r == kT - 1) e |= 2;
                if (c == 0) e |= 4;
                if (c == kT - 1) e |= 8;
                if (r == 0 && c == 0) e |= 16;
                if (r == 0 && c == kT - 1) e |= 32;
                if (r == kT - 1 && c == 0) e |= 64;
                if (r == kT - 1 && c == kT - 1) e |= 128;
                if (c == 0) atomicOr(&colmask[0], 1u << r);
                if (c == kT - 1) atomicOr(&colmask[1], 1u << r);
            }
        }
        const int any = __syncthreads_or(e != 0);
        if (e) atomicOr(&edges, e);
        __syncthreads();
        // Neighbour d (one lane of warp 0 each, in parallel): record which of
        // its halo cells moved, then queue it.  Every lane fences first, which
        // orders the whole CTA's writes (seen through the barrier) before its marks.
        if (tid < 32) {
            const int ed = edges;
            if (any || it >= kLocalCap) __threadfence();
            if (tid < 8 && ((ed >> tid) & 1)) {
                const int64_t ny = ty + (tid == 0 || tid == 4 || tid == 5 ? -1 : (tid == 1 || tid == 6 || tid == 7 ? 1 : 0));
                const int64_t nx = tx + (tid == 2 || tid == 4 || tid == 6 ? -1 : (tid == 3 || tid == 5 || tid == 7 ? 1 : 0));
                const int word = tid == 0 ? 1 : tid == 1 ? 0 : tid == 2 ? 3 : tid == 3 ? 2 : 4;
                const uint32_t bits = tid == 0 ? dirty[0] : tid == 1 ? dirty[kT - 1] : tid == 2 ? colmask[0]
                                    : tid == 3 ? colmask[1] : (8u >> (tid - 4));  // corners: BR, BL, TR, TL of the neighbour
                mark_halo(s, p, ny, nx, word, bits);
                __threadfence();  // the mark before the request
                put_tile<PERSIST>(s, next, next_count, ny, nx, p, patience);
            }
            __syncwarp();
            if (tid == 0) {
                const bool capped = it >= kLocalCap;
                if (capped) mark_halo(s, p, ty, tx, 4, kHaloAll);  // stopped early: relax every cell next time
                if (!PERSIST && capped) put_tile<PERSIST>(s, next, next_count, ty, tx, p, patience);
                st_visits++;
                st_iters += (unsigned long long)it;
                st_changed += any ? 1ull : 0ull;
                if (PERSIST) {
                    // Back to idle, or queued again if it stopped at the cap; a
                    // request that came during the visit (running-and-requested)
                    // is served here at once: the tile goes back to running and
                    // this CTA visits it again, still counted as pending.
                    const int32_t old = atomicCAS(&s.queued[t], kRunning, capped ? kQueued : kIdle);
                    chase = old != kRunning;
                    if (chase) atomicExch(&s.queued[t], kRunning);  // only this visitor moves it out of kRunningDirty
                    else if (capped) ring_push(s, t, patience);
                    __threadfence();
                    atomicAdd(&s.q[kQProgress], 1ULL);
                    if (!chase) atomicAdd(&s.q[kQPending], ~0ULL);  // minus one, after the pushes above (the warp synced)
                }
            }
        }
        __syncthreads();
    }
    if (tid == 0) {  // this CTA's statistics, once
        if (st_visits) atomicAdd(s.visits, st_visits);
        if (st_iters) atomicAdd(s.iters, st_iters);
        if (st_changed) atomicAdd(s.changed, st_changed);
    }
    if (PERSIST) return;
    // The last CTA to finish resets the consumed list and the claim cursor.
    if (tid == 0) {
        __threadfence();
        const int32_t done = atomicAdd(&s.counts[3], 1);
        last_block = done == (int32_t)gridDim.x - 1;
    }
    __syncthreads();
    if (last_block && tid == 0) {
        *cur_count = 0;
        s.counts[2] = 0;
        s.counts[3] = 0;
        __threadfence();
    }
}

__device__ __forceinline__ bool level_is_inf(double w) {
    return (__double_as_longlong(w) & 0x7FFFFFFFFFFFFFFFLL) == 0x7FF0000000000000LL;
}

__global__ void fill_finish_kernel(const FillParams p, const OutView out, unsigned long long* raised) {
    const float nd_f = (float)out.nodata;
    unsigned long long cnt = 0;
    for (int64_t r = blockIdx.y; r < p.rows; r += gridDim.y) {
        for (int64_t c = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; c < p.cols; c += (int64_t)gridDim.x * blockDim.x) {
            const double w = p.w[r * p.w_stride + c];
            const bool nd = level_is_inf(w);
            if (!nd && dkey(w) > dem_key(p, r, c)) cnt++;
            put_level(out, r, c, w, nd, nd_f);
        }
    }
    cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
    if (raised && (threadIdx.x & 31) == 0 && cnt) atomicAdd(raised, cnt);
}

// ---- batched form: many rasters packed into one mosaic ------------------
// Every raster of a batch is copied into its own rectangle of one mosaic
// DEM; the raster's ring and its nodata cells become the mosaic's nodata, as
// does every mosaic cell outside the rasters.  A ring cell's level is nodata
// in the reference (rasterLayer copyLayerInfo) whatever its DEM value, so two
// rasters side by side meet at two rows (or columns) of nodata levels: no
// level of one is ever a neighbour of a level of the other, and the mosaic's
// fixpoint is every raster's own fixpoint.  One persistent relaxation then
// serves the whole batch.

__global__ void fill_mosaic_clear_kernel(void* mosaic, int64_t n, int f64, double nd) {
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        if (f64) reinterpret_cast<double*>(mosaic)[i] = nd;
        else reinterpret_cast<float*>(mosaic)[i] = (float)nd;
    }
}

// blockIdx.y = raster; the block's threads stride over the raster's cells.
__global__ void fill_mosaic_pack_kernel(const FillBatchItem* items, void* mosaic, int64_t mstride, int f64, double nd) {
    const FillBatchItem it = items[blockIdx.y];
    const int64_t n = it.rows * it.cols;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / it.cols, c = i - r * it.cols;
        const char* row = reinterpret_cast<const char*>(it.dem) + r * it.pitch;
        const bool ring = r == 0 || c == 0 || r == it.rows - 1 || c == it.cols - 1;
        const int64_t m = (it.oy + r) * mstride + it.ox + c;
        if (f64) {
            const double z = reinterpret_cast<const double*>(row)[c];
            reinterpret_cast<double*>(mosaic)[m] = (ring || it.nd6d.has(z)) ? nd : z;
        } else {
            const float z = reinterpret_cast<const float*>(row)[c];
            reinterpret_cast<float*>(mosaic)[m] = (ring || it.nd6f.has(z)) ? (float)nd : z;
        }
    }
}

// The levels of each raster's rectangle into its own output (nodata levels:
// the output's nodata), and the count of raised cells over the batch.
__global__ void fill_mosaic_finish_kernel(const FillParams p, const FillBatchItem* items, unsigned long long* raised) {
    const FillBatchItem it = items[blockIdx.y];
    const int64_t n = it.rows * it.cols;
    unsigned long long cnt = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / it.cols, c = i - r * it.cols;
        const double w = p.w[(it.oy + r) * p.w_stride + it.ox + c];
        const bool nd = level_is_inf(w);
        if (!nd && dkey(w) > dem_key(p, it.oy + r, it.ox + c)) cnt++;
        put_level(it.out, r, c, w, nd, (float)it.out.nodata);
    }
    cnt = __reduce_add_sync(0xffffffffu, (unsigned)cnt);
    if (raised && (threadIdx.x & 31) == 0 && cnt) atomicAdd(raised, cnt);
}

}  // namespace

cudaError_t fill_mosaic_pack(const FillBatchItem* items, int count, int64_t max_cells, void* mosaic, int64_t mrows,
                             int64_t mstride, int f64, double nd, cudaStream_t st) {
    const int64_t n = mrows * mstride;
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    fill_mosaic_clear_kernel<<<(unsigned)blocks, 256, 0, st>>>(mosaic, n, f64, nd);
    int64_t bx = (max_cells + 255) / 256;
    if (bx > 64) bx = 64;
    fill_mosaic_pack_kernel<<<dim3((unsigned)bx, (unsigned)count), 256, 0, st>>>(items, mosaic, mstride, f64, nd);
    return cudaGetLastError();
}

cudaError_t fill_mosaic_finish(const FillParams& p, const FillBatchItem* items, int count, int64_t max_cells,
                               unsigned long long* raised, cudaStream_t st) {
    int64_t bx = (max_cells + 255) / 256;
    if (bx > 64) bx = 64;
    fill_mosaic_finish_kernel<<<dim3((unsigned)bx, (unsigned)count), 256, 0, st>>>(p, items, raised);
    return cudaGetLastError();
}

int fill_tile_rows() { return kT; }
int fill_tile_cols() { return kT; }

// Host: per-binade step table for the gap, exact: for the binade starting at
// x = 2^(e-1023), (x + gap) - x is exact (both in the binade) and, divided by
// the binade's ulp, is the integer step that fl64(y + gap) adds to any y of the
// binade whose sum stays in it.
static cudaError_t upload_steps(double gap, cudaStream_t st) {
    // The table lives in each device's memory: remember the gap per device.
    static std::mutex mu;
    static std::map<int, double> uploaded;
    int dev = 0;
    cudaError_t err = cudaGetDevice(&dev);
    if (err != cudaSuccess) return err;
    std::lock_guard<std::mutex> lock(mu);
    auto it = uploaded.find(dev);
    if (it != uploaded.end() && it->second == gap) return cudaSuccess;
    int64_t tab[2048];
    for (int e = 0; e < 2048; e++) {
        tab[e] = -1;
        if (e == 0 || e >= 2047 || !(gap >= 0.0)) continue;
        const double x = ldexp(1.0, e - 1023);
        const double ulp = ldexp(1.0, e - 1023 - 52);
        const volatile double s0 = x + gap;  // one IEEE double add, even x
        const volatile double x1 = x + ulp;
        const volatile double s1 = x1 + gap;  // odd x
        const int64_t d0 = (int64_t)((s0 - x) / ulp);
        const int64_t d1 = (int64_t)((s1 - x1) / ulp);
        // Same step for even and odd x: no tie in this binade.  A sum that
        // leaves the binade is caught on the device by the result's exponent.
        if (!(s0 < 2.0 * x) || d0 != d1) continue;
        tab[e] = d0;
    }
    // Pageable source: staged at once, copied in stream order.
    err = cudaMemcpyToSymbolAsync(g_step, tab, sizeof(tab), 0, cudaMemcpyHostToDevice, st);
    if (err == cudaSuccess) uploaded[dev] = gap;
    return err;
}

cudaError_t fill_init(const FillParams& p, const FillScratch& s, cudaStream_t st) {
    cudaError_t e = upload_steps(p.gap, st);
    if (e != cudaSuccess) return e;
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    int64_t tblocks = (ntiles + 255) / 256;
    if (tblocks > 4096) tblocks = 4096;
    fill_init_tiles_kernel<<<(unsigned)tblocks, 256, 0, st>>>(p, s);
    int64_t iblocks = ntiles;
    if (iblocks > 16384) iblocks = 16384;
    fill_init_tile_kernel<<<(unsigned)iblocks, 256, 0, st>>>(p, s);
    fill_seed_kernel<<<(unsigned)tblocks, 256, 0, st>>>(p, s);
    return cudaGetLastError();
}

cudaError_t fill_round(const FillParams& p, const FillScratch& s, int parity, int num_sms, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_tiles_kernel<false>, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    if (grid > ntiles) grid = ntiles;
    fill_tiles_kernel<false><<<(unsigned)grid, kThreads, 0, st>>>(p, s, parity, 0);
    return cudaGetLastError();
}

cudaError_t fill_persistent(const FillParams& p, const FillScratch& s, long long patience, int num_sms, cudaStream_t st) {
    int per_sm = 0;
    cudaError_t e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fill_tiles_kernel<true>, kThreads, 0);
    if (e != cudaSuccess) return e;
    if (per_sm < 1) per_sm = 1;
    int64_t grid = (int64_t)num_sms * per_sm;  // every CTA resident
    const int64_t ntiles = p.tiles_y * p.tiles_x;
    if (grid > ntiles) grid = ntiles;
    fill_tiles_kernel<true><<<(unsigned)grid, kThreads, 0, st>>>(p, s, 0, patience);
    return cudaGetLastError();
}

cudaError_t fill_finish(const FillParams& p, const OutView& out, unsigned long long* raised, cudaStream_t st) {
    int64_t bx = (p.cols + 255) / 256;
    if (bx > 64) bx = 64;
    const int64_t by = p.rows < 4096 / bx ? p.rows : 4096 / bx;
    const dim3 grid((unsigned)bx, (unsigned)by);
    fill_finish_kernel<<<grid, 256, 0, st>>>(p, out, raised);
    return cudaGetLastError();
}

}  // namespace pargo
