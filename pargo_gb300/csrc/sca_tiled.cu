// sca_tiled.cu -- D8 specific catchment area as subtree sums over the flow
// forest, tiled so that the long serial chains stay in shared memory.
//
// Reference: SCAOperator::Operator (apps/hydrology/scad8/scaOperator.cpp:37-131).
// Flow forest: the parent of a valid work cell c is the cell its code names,
// when that cell is a valid work cell that does not name c back (a mutual
// pair is no inflow, :71).  Converged SCA = subtree size (counts are integers:
// exact in any summation order).  The shipped single raster-order sweep pulls
// the inflow p -> c when p is a source or p precedes c and p is "done"; p is
// done exactly when no cell u of p's subtree has a non-source inflow q that
// follows u in raster order ("bad" cells), so done is an OR over the subtree
// -- a second subtree reduction -- and shipped(c) = 1 + the pulled children's
// subtree sizes, gathered in the output pass.
//
// Phases (one launch each):
//  1. per 64 x 64 tile (codes with a 2-cell halo in shared memory): the in-tile
//     forest (from byte inflow masks), stored as one word per cell for phase
//     4; every cell's path end by pointer jumping; the in-tile subtree of an
//     exit (a cell whose parent lies in another tile) is the set of cells
//     whose path ends at it, so its sum and bad flag are counts and ORs over
//     them, with no walk.  Exits record their in-tile sum and the entry cell
//     they feed; every border cell records the exit its path reaches.
//  2. the exit forest: exit x's parent is the exit reached from the entry x
//     feeds; its feeding counts, added into the parents' packed words.
//  3. subtree sums over the exit forest (its leaves marked first, then a
//     global-memory walk, again one atomic per step; chains are as long as the
//     tiles a river crosses); each exit adds its total to the inflow of the
//     entry it feeds.
//  4. per tile again, from the stored forest: the in-tile sums with the
//     entries' inflows added, by a shared-memory topological walk (one atomic
//     add per step on the parent's word of pending children, bad-child count
//     and sum; the last contributor continues); converged contract: the
//     output itself, then a one-thread kernel for the reference's last-cell
//     quirk (a nodata last work cell accumulates what flows into it).
//  5. shipped contract only: the output pass over the final counts and flags.
// Cycles (inside a tile or across tiles) and inflows from the raster's ring,
// which the reference never releases, leave cells or exits uncompleted; the
// host compares the completion counts.

#include <type_traits>

#include "common.cuh"
#include "kernels.h"

namespace pargo {

namespace {

constexpr int kT = kScaTile;       // tile side
constexpr int kH = kT + 4;         // codes with a 2-cell halo
constexpr int kM = kT + 2;         // inflow masks with a 1-cell halo
constexpr int kCells = kT * kT;
constexpr int kThreads = 256;
constexpr int8_t kNodata = -1, kNoFlow = -2;

// A D8 value as a code: 0-8 but 4, kNoFlow for any other number, kNodata
// for the nodata value (scaOperator.cpp:48: within Eps for floating input).
__device__ __forceinline__ int8_t classify8(const ScaParams& p, double v) {
    const bool nd = (p.d8.dtype == PARGO_F64 || p.d8.dtype == PARGO_F32) ? fabs(v - p.nodata) < kEpsHydro
                                                                        : v == p.nodata;
    if (nd) return kNodata;
    const int k = (int)v;
    return ((double)k == v && k >= 0 && k <= 8 && k != 4) ? (int8_t)k : kNoFlow;
}

template <typename V>
__device__ __forceinline__ double d8_value(const ScaParams& p, int64_t r, int64_t c) {
    return (double)reinterpret_cast<const V*>(p.d8.base + r * p.d8.pitch)[c];
}

__device__ __forceinline__ int8_t decode8(const ScaParams& p, int64_t r, int64_t c) {
    if (r < 0 || c < 0 || r >= p.rows || c >= p.cols) return kNodata;
    double v;
    switch (p.d8.dtype) {
        case PARGO_F64: v = d8_value<double>(p, r, c); break;
        case PARGO_F32: v = d8_value<float>(p, r, c); break;
        case PARGO_I8: v = d8_value<int8_t>(p, r, c); break;
        case PARGO_I16: v = d8_value<int16_t>(p, r, c); break;
        default: v = d8_value<int32_t>(p, r, c); break;
    }
    return classify8(p, v);
}

// The int8 codes of the window at (r0, c0) of kH x kH cells into cd, the
// loads of a thread issued in two groups before their first use.
__device__ __forceinline__ void load_codes_i8(const ScaParams& p, int64_t r0, int64_t c0, int8_t* cd, int tid) {
    constexpr int kPer = (kH * kH + 255) / 256;  // 19
    constexpr int kHalf = (kPer + 1) / 2;          // two groups of loads in flight
    // An int8 value equals the nodata value exactly when the nodata value is
    // that integer: the classification stays on the integer pipes.
    const int ndv = (p.nodata == floor(p.nodata) && p.nodata >= -128.0 && p.nodata <= 127.0) ? (int)p.nodata : 1000;
#pragma unroll
    for (int h = 0; h < 2; h++) {
        int v[kHalf];
#pragma unroll
        for (int q = 0; q < kHalf; q++) {
            const int i = tid + (h * kHalf + q) * 256;
            const int64_t r = r0 + i / kH, c = c0 + i % kH;
            v[q] = ndv;  // outside the raster: nodata
            if (i < kH * kH && r >= 0 && c >= 0 && r < p.rows && c < p.cols)
                v[q] = reinterpret_cast<const int8_t*>(p.d8.base + r * p.d8.pitch)[c];
        }
#pragma unroll
        for (int q = 0; q < kHalf; q++) {
            const int i = tid + (h * kHalf + q) * 256;
            const int x = v[q];
            const int8_t k = x == ndv ? kNodata : ((x >= 0 && x <= 8 && x != 4) ? (int8_t)x : kNoFlow);
            if (i < kH * kH) cd[i] = k;
        }
        asm volatile("" ::: "memory");
    }
}

__device__ __forceinline__ bool in_work(const ScaParams& p, int64_t r, int64_t c) {
    return r >= 1 && c >= 1 && r <= p.rows - 2 && c <= p.cols - 2;
}

// Border slot of tile-local (lr, lc) in a th x tw tile, or -1 inside.
__device__ __forceinline__ int slot_of(int lr, int lc, int th, int tw) {
    if (lr == 0) return lc;
    if (lr == th - 1) return tw + lc;
    if (lc == 0) return 2 * tw + (lr - 1);
    if (lc == tw - 1) return 2 * tw + (th - 2) + (lr - 1);
    return -1;
}

// Shared state of one tile.  Each cell's accumulator word packs, from the
// top: a 4-bit count of in-tile children not yet folded in, a 4-bit count of
// folded children whose subtree holds a "bad" cell, and the sum of the folded
// subtree sizes (plus, in the final pass, the inflow from other tiles).  A
// child folds itself into its parent with one atomic add (its size, one more
// bad child if its subtree is bad, one child fewer) and the return value
// tells it whether it was the last child; the last one continues the walk
// from the value it computed, so no walk step waits for another read.  A
// completed cell's word is rewritten as 0xF in the count field (no real count
// reaches 15: a cell has at most 8 children), its subtree-bad bit and its
// subtree size.  First pass: 32-bit words (4 + 4 + 24 bits; an in-tile sum is
// at most 4096); final pass: 64-bit (4 + 4 + 56).  Static flags are bytes
// packed four to a word, written before the walk: 1 valid work cell, 2 "bad"
// (a non-source inflow follows it in raster order), 8 in-tile leaf, 16 an
// inflow from another tile was not pulled.
template <bool FINAL>
struct TileSmem {
    using Acc = typename std::conditional<FINAL, unsigned long long, unsigned int>::type;
    static constexpr int kDegShift = FINAL ? 60 : 28;
    static constexpr int kBadShift = FINAL ? 56 : 24;
    static constexpr Acc kSum = ((Acc)1 << kBadShift) - 1;
    static constexpr Acc kOne = (Acc)1 << kDegShift;   // one child in the count field
    static constexpr Acc kBadOne = (Acc)1 << kBadShift;
    static constexpr Acc kDone = (Acc)0xF << kDegShift;
    // first pass only: the codes, (a, b) = (r - r0 + 2, c - c0 + 2), and the
    // inflow masks of the tile and a 1-cell ring, (a, b) = (r - r0 + 1, c - c0 + 1)
    // in-tile parent, -1 none, -2 outside the tile; in the final pass packed
    // with the flags the walk reads: parent + 2 (bits 0-12), valid (13), bad
    // or fed by a not-pulled inflow (14), in-tile leaf (15)
    alignas(16) int16_t lpar[kCells];
    Acc acc[kCells];
    uint32_t flagw[FINAL ? 1 : kCells / 4];  // first pass: a byte of static flags per cell
    int8_t cd[FINAL ? 1 : kH * kH];
    uint8_t im[FINAL ? 1 : kM * kM];
    unsigned long long cnt[3];   // valid, completed, ring inflows
    int next;                    // the walk's next cell to look at for a leaf
    int16_t slotcell[FINAL ? kScaSlots : 1];  // final pass: the valid cell at each border slot, -1 none
    __device__ __forceinline__ unsigned flag(int i) const { return (flagw[i >> 2] >> (8 * (i & 3))) & 0xFFu; }
    // the final pass's packed parent and flags
    __device__ __forceinline__ unsigned packed(int i) const { return (unsigned)(uint16_t)lpar[i]; }
    __device__ __forceinline__ int parent(int i) const { return (int)(packed(i) & 0x1FFFu) - 2; }
    __device__ __forceinline__ bool p_valid(int i) const { return (packed(i) >> 13) & 1u; }
    __device__ __forceinline__ bool p_bad(int i) const { return (packed(i) >> 14) & 1u; }
    __device__ __forceinline__ bool p_leaf(int i) const { return (packed(i) >> 15) & 1u; }
    __device__ __forceinline__ bool done(int i) const { return (acc[i] & kDone) == kDone; }
    __device__ __forceinline__ Acc total(int i) const { return acc[i] & kSum; }
    __device__ __forceinline__ unsigned sub_bad(int i) const { return (unsigned)((acc[i] >> kBadShift) & 1u); }
};

// Whether the neighbour at (a, b) of the cell at codes position (ca, cb)
// flows into it: its code names the cell and the cell does not name it back.
template <class S_t>
__device__ __forceinline__ bool flows_in(const S_t& S, int ca, int cb, int a, int b) {
    const int k = (a + 1) * 3 + (b + 1);  // window index of the neighbour seen from the cell
    const int8_t q = S.cd[(ca + a) * kH + (cb + b)];
    return q == 8 - k && S.cd[ca * kH + cb] != k;
}

// An exit's word in the exit forest: from the top, a 12-bit count of exits
// still to feed it (at most 5 per border cell of its tile), a 12-bit count
// of fed exits whose total holds a "bad" cell (its own in-tile subtree's bad
// bit counts as one), and a 40-bit sum of cells.
constexpr int kXCountShift = 52, kXBadShift = 40;
constexpr unsigned long long kXCountMask = 0xFFFULL;
constexpr unsigned long long kXOne = 1ULL << kXCountShift, kXBadOne = 1ULL << kXBadShift;
constexpr unsigned long long kXSum = kXBadOne - 1;
__device__ __forceinline__ unsigned long long xpack(unsigned long long total, unsigned bad) {
    return total | (bad ? kXBadOne : 0ULL);
}

// The IEEE double of a count below 2^53, built on the integer pipes.
__device__ __forceinline__ unsigned long long count_bits(unsigned long long x) {
    if (x == 0) return 0;
    const int e = 63 - __clzll((long long)x);  // x = 1.m * 2^e
    const unsigned long long m = (x << (52 - e)) & 0xFFFFFFFFFFFFFULL;
    return ((unsigned long long)(1023 + e) << 52) | m;
}

// A cell's in-tile forest as one word: flags (1 valid work cell, 2 "bad"),
// in-tile children (bits 4-7) and parent + 2 (bits 8-20: -2 .. 4095).
__device__ __forceinline__ uint32_t pack_forest(unsigned f, int deg, int lp) {
    return (f & 3u) | ((uint32_t)deg << 4) | ((uint32_t)(lp + 2) << 8);
}

// Bit of the neighbour at offset (a, b) in an inflow mask (window index k =
// (a + 1) * 3 + b + 1 without the centre).
__device__ __forceinline__ int mask_bit(int k) { return k < 4 ? k : k - 1; }

// Reference in-degree of the cell at codes position (ca, cb) is zero.
template <class S_t>
__device__ __forceinline__ bool is_source(const S_t& S, int ca, int cb) {
#pragma unroll
    for (int a = -1; a <= 1; a++)
#pragma unroll
        for (int b = -1; b <= 1; b++)
            if ((a || b) && flows_in(S, ca, cb, a, b)) return false;
    return true;
}

template <bool FINAL>
__global__ void __launch_bounds__(kThreads, FINAL ? 5 : 6) sca_tile_kernel(const ScaParams p, ScaScratch s, ScaTiles T) {
    extern __shared__ __align__(16) unsigned char sca_smem[];
    using Smem = TileSmem<FINAL>;
    Smem& S = *reinterpret_cast<Smem*>(sca_smem);
    const int tid = threadIdx.x;
    const int64_t ntiles = T.tiles_x * T.tiles_y;
    for (int64_t t = blockIdx.x; t < ntiles; t += gridDim.x) {
        const int64_t r0 = (t / T.tiles_x) * kT, c0 = (t % T.tiles_x) * kT;
        const int th = (int)min((int64_t)kT, p.rows - r0), tw = (int)min((int64_t)kT, p.cols - c0);
        if (tid < 3) S.cnt[tid] = 0;
        // Final pass: the inflows from other tiles, loaded now and added to
        // their cells after the forest is built.
        unsigned long long xin = 0;
        uint32_t xinb = 0;
        if (FINAL && tid < kScaSlots) {
            xin = T.tin[t * kScaSlots + tid];
            xinb = T.tinb[t * kScaSlots + tid];
            S.slotcell[tid] = -1;
        }
        if (!FINAL && tid < kScaSlots) {  // every slot starts as "no exit"; the exit forest's accumulators empty
            const int64_t node = t * kScaSlots + tid;
            T.exit_of[node] = -1;
            T.yslot[node] = -1;
            T.tin[node] = 0;
            T.tinb[node] = 0;
        }
        if (tid == 0) S.next = 0;
        if constexpr (!FINAL) {
            static_assert(kThreads == 256, "load_codes_i8 strides by 256");
            if (p.d8.dtype == PARGO_I8) load_codes_i8(p, r0 - 2, c0 - 2, S.cd, tid);
            else
                for (int i = tid; i < kH * kH; i += kThreads) S.cd[i] = decode8(p, r0 - 2 + i / kH, c0 - 2 + i % kH);
            __syncthreads();
            // Inflow masks of the tile and its 1-cell ring: bit mask_bit(k) set
            // when the neighbour at window index k flows into the cell (its code
            // names the cell, and the cell does not name it back).
            for (int i = tid; i < kM * kM; i += kThreads) {
                const int ca = i / kM + 1, cb = i % kM + 1;  // codes position
                const int8_t own = S.cd[ca * kH + cb];
                unsigned m = 0;
    #pragma unroll
                for (int k = 0; k < 9; k++) {
                    if (k == 4) continue;
                    const int8_t q = S.cd[(ca + k / 3 - 1) * kH + (cb + k % 3 - 1)];
                    if (q == 8 - k && own != k) m |= 1u << mask_bit(k);
                }
                S.im[i] = (uint8_t)m;
            }
            __syncthreads();
            // The in-tile forest.  A thread owns column lc = tid % 64 of rows
            // tid / 64 + 4q; the raster's work region (rows and columns 1 ..
            // n - 2) in tile-local coordinates bounds every test.
            unsigned long long nvalid = 0, nring = 0;
            const int wr_lo = (int)max((int64_t)-2, 1 - r0), wr_hi = (int)min((int64_t)kT + 1, p.rows - 2 - r0);
            const int wc_lo = (int)max((int64_t)-2, 1 - c0), wc_hi = (int)min((int64_t)kT + 1, p.cols - 2 - c0);
            auto work = [&](int lr, int lc) { return lr >= wr_lo && lr <= wr_hi && lc >= wc_lo && lc <= wc_hi; };
            const int lc = tid & (kT - 1);
#pragma unroll 2
            for (int q = 0; q < kCells / kThreads; q++) {
                const int lr = (tid >> 6) + q * (kThreads / kT);
                const int i = lr * kT + lc;
                const int ca = lr + 2, cb = lc + 2;
                int16_t lp = -1;
                int deg = 0;
                uint8_t f = 0;
                const int8_t k = S.cd[ca * kH + cb];
                if (lr < th && lc < tw && work(lr, lc) && k != kNodata) {
                    f = 1;
                    nvalid++;
                    if (k >= 0) {
                        const int a = k / 3 - 1, b = k % 3 - 1;
                        const int tr = lr + a, tc = lc + b;
                        const int8_t tk = S.cd[(ca + a) * kH + (cb + b)];
                        if (work(tr, tc) && tk != kNodata && tk != 8 - k)
                            lp = (tr >= 0 && tc >= 0 && tr < th && tc < tw) ? (int16_t)(tr * kT + tc) : (int16_t)-2;
                    }
                    // children: in-tile ones count towards the walk; an inflow from
                    // the ring is never released; a non-source child that follows
                    // the cell in raster order is not pulled by the single sweep.
                    unsigned m = S.im[(lr + 1) * kM + lc + 1];
                    while (m) {
                        const int bit = __ffs(m) - 1;
                        m &= m - 1;
                        const int kk = bit < 4 ? bit : bit + 1;
                        const int a = kk / 3 - 1, b = kk % 3 - 1;
                        const int qr = lr + a, qc = lc + b;
                        if (!work(qr, qc)) {
                            nring++;
                            continue;
                        }
                        if (qr >= 0 && qc >= 0 && qr < th && qc < tw) deg++;
                        if (kk > 4 && S.im[(qr + 1) * kM + qc + 1] != 0) f |= 2;  // kk > 4: a later cell in raster order
                    }
                }
                S.lpar[i] = lp;
                reinterpret_cast<uint8_t*>(S.flagw)[i] = (uint8_t)(f | (f && deg == 0 ? 8 : 0));  // leaves fixed before any walk
                S.acc[i] = 0;  // counted below, once the paths' last cells are known
                if (lr < th && lc < tw) s.forest[(r0 + lr) * p.cols + (c0 + lc)] = pack_forest(f, deg, lp);
            }
            atomicAdd(&S.cnt[0], nvalid);
            if (nring) atomicAdd(&S.cnt[2], nring);
            __syncthreads();
        } else {
            // The forest the first pass built, one word per cell, every load
            // of a thread issued before the first is unpacked.
            constexpr int kPer = kCells / kThreads;  // 16
            uint32_t fw[kPer];
#pragma unroll
            for (int q = 0; q < kPer; q++) {
                const int i = tid + q * kThreads;
                const int lr = i / kT, lc = i % kT;
                fw[q] = pack_forest(0, 0, -1);  // outside the raster: no cell
                if (lr < th && lc < tw) fw[q] = s.forest[(r0 + lr) * p.cols + (c0 + lc)];
            }
            __syncthreads();  // every slot reset to -1 above before any is claimed below
            unsigned long long nvalid = 0;
#pragma unroll
            for (int q = 0; q < kPer; q++) {
                const int i = tid + q * kThreads;
                const unsigned f = fw[q] & 3u, deg = (fw[q] >> 4) & 0xFu;
                // parent + 2 straight from the word (bits 8-20), then valid, bad and leaf
                S.lpar[i] = (int16_t)(uint16_t)(((fw[q] >> 8) & 0x1FFFu) | ((f & 1u) << 13) | (((f >> 1) & 1u) << 14) |
                                                ((f && deg == 0 ? 1u : 0u) << 15));
                S.acc[i] = (typename Smem::Acc)deg * Smem::kOne;
                if (f & 1u) {
                    nvalid++;
                    const int sl = slot_of(i / kT, i % kT, th, tw);
                    if (sl >= 0) S.slotcell[sl] = (int16_t)i;
                }
            }
            atomicAdd(&S.cnt[0], nvalid);
            __syncthreads();
        }
        if (FINAL) {
            // the external inflow of each valid border cell, and its flag: an
            // inflow from another tile that was not pulled
            const int i = tid < kScaSlots ? S.slotcell[tid] : -1;
            if (i >= 0) {
                S.acc[i] += (typename Smem::Acc)xin;
                if (xinb & 1u)  // the bad bit of its packed parent word (lpar is 4-byte aligned)
                    atomicOr(reinterpret_cast<unsigned*>(S.lpar) + (i >> 1), (1u << 14) << (16 * (i & 1)));
            }
            __syncthreads();
        }
        // Final pass: the topological walk from the in-tile leaves.
        using Acc = typename Smem::Acc;
        unsigned long long ndone = 0;
        if constexpr (FINAL) {
            // Topological walk from the in-tile leaves: a walker holds the value
            // of its cell's word once every child has folded in (a leaf's word is
            // final from the start; anything else's is the last child's return
            // value plus its own add), so a step is one atomic on the parent.
            // Walkers take leaves from one shared cursor (a warp's lanes that
            // need one take consecutive cells with a single atomic), so a lane
            // that ends a chain starts the next leaf while long chains go on.
            {
                const int lane = tid & 31;
                int cur = -1;
                Acc v = 0;
                for (;;) {
                    const unsigned need = __ballot_sync(0xffffffffu, cur == -1);
                    if (need) {
                        int base = 0;
                        if (lane == __ffs(need) - 1) base = atomicAdd(&S.next, __popc(need));
                        base = __shfl_sync(0xffffffffu, base, __ffs(need) - 1);
                        if (cur == -1) {
                            const int i = base + __popc(need & ((1u << lane) - 1));
                            if (i < kCells && S.p_leaf(i)) {
                                cur = i;
                                v = S.acc[i];
                            } else if (i >= kCells) {
                                cur = -2;  // no leaves left for this lane
                            }
                        }
                    }
                    if (!__any_sync(0xffffffffu, cur >= 0) && !__any_sync(0xffffffffu, cur == -1)) break;
                    if (cur >= 0) {
                        const Acc tot = 1 + (v & Smem::kSum);
                        const bool bad = S.p_bad(cur) || ((v >> Smem::kBadShift) & 0xFu) != 0;
                        S.acc[cur] = Smem::kDone | (bad ? Smem::kBadOne : (Acc)0) | tot;  // nothing else writes it now
                        ndone++;
                        const int par = S.parent(cur);
                        if (par < 0) {
                            cur = -1;
                        } else {
                            const Acc delta = tot + (bad ? Smem::kBadOne : (Acc)0) - Smem::kOne;  // the count field is >= 1
                            const Acc old = atomicAdd(&S.acc[par], delta);
                            if (((old >> Smem::kDegShift) & 0xFu) != 1u) {
                                cur = -1;  // another child is still to come
                            } else {
                                v = old + delta;
                                cur = par;
                            }
                        }
                    }
                }
            }
        }
        atomicAdd(&S.cnt[1], ndone);
        __syncthreads();
        if (!FINAL) {
            // Parents become the path's last cell by pointer jumping (a
            // parent pointer is replaced by its parent's while that is a
            // cell): 12 rounds cover any acyclic path of a 64 x 64 tile, and
            // a pointer is an ancestor of its cell at every moment, so the
            // rounds need no read/write separation.  The last cell keeps its
            // own -1 or -2.  lpar is rebuilt by the final pass.
#pragma unroll 1
            for (int round = 0; round < 12; round++) {
                int moved = 0;
                for (int i = tid; i < kCells; i += kThreads) {
                    const int q = S.lpar[i];
                    if (q < 0) continue;
                    const int q2 = ((volatile int16_t*)S.lpar)[q];
                    if (q2 >= 0) {
                        S.lpar[i] = (int16_t)q2;
                        moved = 1;
                    }
                }
                if (!__syncthreads_or(moved)) break;  // every pointer is at its path's last cell
            }
            // The in-tile subtree of an exit is the set of cells whose path
            // ends at it: its size is their count and its bad flag the OR of
            // their own, taken with one atomic per group of a warp's lanes
            // that share the exit.  A cell whose path ends (its last cell has
            // no parent here) is done; a path still inside the tile after the
            // jumps runs into a cycle.
            for (int i = tid; i < kCells; i += kThreads) {
                const int q = S.lpar[i];
                const int last = q >= 0 ? q : i;
                const int lp = S.lpar[last];
                const unsigned f = S.flag(i);
                const bool valid = (f & 1u) != 0, ends = valid && lp < 0;
                if (ends) atomicOr(&S.acc[i], Smem::kDone);
                const bool to_exit = ends && lp == -2;
                const unsigned grp = __match_any_sync(0xffffffffu, to_exit ? last : -1);
                const unsigned lead = __ffs(grp) - 1;
                const bool bad_any = (__ballot_sync(0xffffffffu, to_exit && (f & 2u)) & grp) != 0;
                if (to_exit && (tid & 31) == (int)lead) {
                    atomicAdd(&S.acc[last], (Acc)__popc(grp));
                    if (bad_any) atomicOr(&S.acc[last], Smem::kBadOne);
                }
            }
            __syncthreads();
            // Border cells: the exit each in-tile path reaches; exits record
            // their in-tile totals and the entry they feed.
            for (int i = tid; i < kCells; i += kThreads) {
                const int lr = i / kT, lc = i % kT;
                if (lr >= th || lc >= tw) continue;
                const int sl = slot_of(lr, lc, th, tw);
                if (sl < 0) continue;
                const int64_t node = t * kScaSlots + sl;
                int32_t ex = -1, ys = -1;
                if (S.done(i)) {  // completed: its path is acyclic
                    const int cur = S.lpar[i] >= 0 ? S.lpar[i] : i;  // the path's last cell (pointers jumped above)
                    if (S.lpar[cur] == -2) {
                        const int er = cur / kT, ec = cur % kT;
                        ex = (int32_t)(t * kScaSlots + slot_of(er, ec, th, tw));
                    }
                    if (S.lpar[i] == -2) {  // this cell is an exit: where its flow enters
                        const int8_t k = S.cd[(lr + 2) * kH + (lc + 2)];
                        const int64_t yr = r0 + lr + k / 3 - 1, yc = c0 + lc + k % 3 - 1;
                        const int64_t yt = (yr / kT) * T.tiles_x + (yc / kT);
                        const int yth = (int)min((int64_t)kT, p.rows - (yr / kT) * kT);
                        const int ytw = (int)min((int64_t)kT, p.cols - (yc / kT) * kT);
                        ys = (int32_t)(yt * kScaSlots + slot_of((int)(yr % kT), (int)(yc % kT), yth, ytw));
                        T.tot[node] = xpack(S.total(i), S.sub_bad(i));
                    }
                }
                T.exit_of[node] = ex;
                T.yslot[node] = ys;
            }
            if (tid == 0 && S.cnt[2]) atomicAdd(&s.counters[6], S.cnt[2]);
        } else {
            // Converged contract: the output itself (a valid cell's count, 0
            // where a cycle left it uncompleted; nodata elsewhere), plus the
            // counts of the cells around the raster's last work cell for its
            // nodata quirk.  Shipped contract: counts and flags for the
            // output pass, which needs neighbours in other tiles.
            const int64_t lastr = p.rows - 2, lastc = p.cols - 2;
            for (int i = tid; i < kCells; i += kThreads) {
                const int lr = i / kT, lc = i % kT;
                if (lr >= th || lc >= tw) continue;
                const int64_t r = r0 + lr, c = c0 + lc;
                const int64_t g = r * p.cols + c;
                const bool valid = S.p_valid(i);
                const bool ok = valid && S.done(i);
                const unsigned long long tot = ok ? (unsigned long long)S.total(i) : 0ULL;
                if (p.shipped) {
                    s.conv[g] = tot;
                    s.ship[g] = ok ? (unsigned long long)S.sub_bad(i) : 0ULL;
                } else {
                    if (p.out.dtype == PARGO_F64)  // the count's double from its bits: no FP64 conversion
                        reinterpret_cast<double*>(p.out.base + r * p.out.pitch)[c] =
                            valid ? __longlong_as_double((long long)count_bits(tot)) : p.out.nodata;
                    else
                        put_value(p.out, r, c, valid ? (double)tot : p.out.nodata);
                    if (r >= lastr - 1 && r <= lastr + 1 && c >= lastc - 1 && c <= lastc + 1) s.conv[g] = tot;
                }
            }
            if (tid == 0) {
                atomicAdd(&s.counters[1], S.cnt[0]);
                atomicAdd(&s.counters[0], S.cnt[1]);
            }
        }
        __syncthreads();
    }
}

// Exit forest: parents and in-degrees.
__global__ void sca_exit_links_kernel(ScaScratch s, ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    unsigned long long nexit = 0;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x) {
        const int32_t y = T.yslot[x];
        int32_t px = -1;
        if (y >= 0) {
            nexit++;
            px = T.exit_of[y];
            if (px >= 0) atomicAdd(&T.tot[px], kXOne);
        }
        T.xpar[x] = px;
    }
    nexit = __reduce_add_sync(0xffffffffu, (unsigned)nexit);
    if ((threadIdx.x & 31) == 0 && nexit) atomicAdd(&s.counters[4], nexit);
}

// Exit forest: mark its leaves (exits that no other exit feeds: a zero count
// field once every link is in) in bit 1 of tinb, before any walk lowers a
// count to zero.
__global__ void sca_exit_leaves_kernel(ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    for (int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; x < n; x += (int64_t)gridDim.x * blockDim.x)
        if (T.yslot[x] >= 0 && (T.tot[x] >> kXCountShift) == 0) T.tinb[x] |= 2u;
}

// Exit forest: totals by a topological walk from its leaves; each exit
// feeds its total into the entry it flows into.  A step is one atomic add on
// the parent's packed word, whose return value tells the walker whether it
// was the last child and, if so, the parent's complete sum.  A thread takes
// the leaves of its grid-stride range one after another.
__global__ void sca_exit_walk_kernel(ScaScratch s, ScaTiles T) {
    const int64_t n = T.tiles_x * T.tiles_y * kScaSlots;
    const int64_t stride = (int64_t)gridDim.x * blockDim.x;
    unsigned long long ndone = 0;
    int64_t x = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    int64_t cur = -1;
    unsigned long long v = 0;
    for (;;) {
        if (cur < 0) {
            for (; x < n; x += stride)
                if (T.yslot[x] >= 0 && (T.tinb[x] & 2u)) break;
            if (x >= n) break;
            cur = x;
            v = T.tot[x];
            x += stride;
        }
        const unsigned long long tot = v & kXSum;
        const bool bad = ((v >> kXBadShift) & kXCountMask) != 0;
        const int32_t y = T.yslot[cur];
        atomicAdd(&T.tin[y], tot);
        if (bad) atomicOr(&T.tinb[y], 1u);  // bit 0: not pulled (bit 1 marks y's own leaf state)
        ndone++;
        const int32_t px = T.xpar[cur];
        if (px < 0) {
            cur = -1;
            continue;
        }
        const unsigned long long delta = tot + (bad ? kXBadOne : 0ULL) - kXOne;  // the count field is >= 1
        const unsigned long long old = atomicAdd(&T.tot[px], delta);
        if ((old >> kXCountShift) != 1ULL) {
            cur = -1;  // another exit still feeds it
            continue;
        }
        v = old + delta;
        cur = px;
    }
    ndone = __reduce_add_sync(0xffffffffu, (unsigned)ndone);
    if ((threadIdx.x & 31) == 0 && ndone) atomicAdd(&s.counters[5], ndone);
}

// Output: converged counts, or the shipped sweep's pulled sums.
// Converged contract, after the fused output: the raster's last work cell,
// when its code is nodata, holds nodata plus what flows into it (the
// reference accumulates into it before it notices the nodata).
__global__ void sca_last_cell_kernel(const ScaParams p, ScaScratch s) {
    if (p.rows < 3 || p.cols < 3) return;
    const int64_t r = p.rows - 2, c = p.cols - 2, i = r * p.cols + c;
    if (decode8(p, r, c) != kNodata) return;
    unsigned long long sum = 0;
    for (int a = -1; a <= 1; a++)
        for (int b = -1; b <= 1; b++) {
            if (!(a || b)) continue;
            const int k = (a + 1) * 3 + (b + 1);
            if (!in_work(p, r + a, c + b) || decode8(p, r + a, c + b) != 8 - k) continue;
            sum += s.conv[i + a * p.cols + b];
        }
    put_value(p.out, r, c, p.out.nodata + (double)sum);
}

__global__ void sca_output_kernel(const ScaParams p, ScaScratch s) {
    const int64_t n = p.rows * p.cols;
    const int64_t last = (p.rows - 2) * p.cols + (p.cols - 2);
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        const int64_t r = i / p.cols, c = i % p.cols;
        const bool work = in_work(p, r, c);
        const int8_t me = work ? decode8(p, r, c) : kNodata;
        const bool is_last = i == last && p.rows >= 3 && p.cols >= 3;
        double v = p.out.nodata;
        if (me != kNodata || is_last) {
            unsigned long long sum = 0;
            if (me != kNodata && !p.shipped) {
                sum = s.conv[i];
            } else {
                // children: neighbours whose code names this cell (and, for a
                // valid cell, that it does not name back)
                for (int a = -1; a <= 1; a++)
                    for (int b = -1; b <= 1; b++) {
                        if (!(a || b)) continue;
                        const int k = (a + 1) * 3 + (b + 1);
                        if (!in_work(p, r + a, c + b) || (me != kNodata && me == k)) continue;
                        if (decode8(p, r + a, c + b) != 8 - k) continue;
                        const int64_t q = i + a * p.cols + b;
                        const unsigned long long cq = s.conv[q];
                        const bool pulled = cq == 1 || (q < i && s.ship[q] == 0);
                        if (!p.shipped || pulled) sum += cq;
                    }
                if (me != kNodata) sum += 1;
            }
            v = me != kNodata ? (double)sum : p.out.nodata + (double)sum;
        }
        put_value(p.out, r, c, v);
    }
}

}  // namespace

size_t sca_tiles_bytes(int64_t rows, int64_t cols) {
    const int64_t nodes = ((rows + kT - 1) / kT) * ((cols + kT - 1) / kT) * kScaSlots;
    return (size_t)nodes * (3 * 4 + 2 * 8 + 4) + 256;
}

ScaTiles sca_tiles_layout(void* base, int64_t rows, int64_t cols) {
    ScaTiles T{};
    T.tiles_y = (rows + kT - 1) / kT;
    T.tiles_x = (cols + kT - 1) / kT;
    const int64_t nodes = T.tiles_x * T.tiles_y * kScaSlots;
    char* b = (char*)(((uintptr_t)base + 15) & ~(uintptr_t)15);
    T.tot = (unsigned long long*)b;
    b += nodes * 8;
    T.tin = (unsigned long long*)b;
    b += nodes * 8;
    T.exit_of = (int32_t*)b;
    b += nodes * 4;
    T.yslot = (int32_t*)b;
    b += nodes * 4;
    T.xpar = (int32_t*)b;
    b += nodes * 4;
    T.tinb = (uint32_t*)b;
    return T;
}

cudaError_t sca_run_tiled(const ScaParams& p, const ScaScratch& s, const ScaTiles& T, cudaStream_t st) {
    const int64_t n = p.rows * p.cols;
    if (n == 0) return cudaSuccess;
    cudaError_t e = cudaMemsetAsync(s.counters, 0, 8 * sizeof(unsigned long long), st);
    if (e != cudaSuccess) return e;
    const size_t smem0 = sizeof(TileSmem<false>), smem1 = sizeof(TileSmem<true>);
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<false>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem0)) !=
        cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<true>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem1)) !=
        cudaSuccess)
        return e;
    // all of the SM's unified memory as shared memory: 6 first-pass and 5
    // final-pass tiles in flight per SM
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<false>, cudaFuncAttributePreferredSharedMemoryCarveout, 100)) !=
        cudaSuccess)
        return e;
    if ((e = cudaFuncSetAttribute(sca_tile_kernel<true>, cudaFuncAttributePreferredSharedMemoryCarveout, 100)) !=
        cudaSuccess)
        return e;
    int dev = 0, sms = 0, per0 = 0, per1 = 0;
    if ((e = cudaGetDevice(&dev)) != cudaSuccess) return e;
    if ((e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev)) != cudaSuccess) return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per0, sca_tile_kernel<false>, kThreads, smem0)) !=
        cudaSuccess)
        return e;
    if ((e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per1, sca_tile_kernel<true>, kThreads, smem1)) !=
        cudaSuccess)
        return e;
    const int64_t ntiles = T.tiles_x * T.tiles_y;
    int64_t grid0 = (int64_t)sms * (per0 > 0 ? per0 : 1), grid1 = (int64_t)sms * (per1 > 0 ? per1 : 1);
    if (grid0 > ntiles) grid0 = ntiles;
    if (grid1 > ntiles) grid1 = ntiles;
    sca_tile_kernel<false><<<(unsigned)grid0, kThreads, smem0, st>>>(p, s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    const int64_t nodes = ntiles * kScaSlots;
    int64_t nb = (nodes + 255) / 256;
    if (nb > 8192) nb = 8192;
    sca_exit_links_kernel<<<(unsigned)nb, 256, 0, st>>>(s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_exit_leaves_kernel<<<(unsigned)nb, 256, 0, st>>>(T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_exit_walk_kernel<<<(unsigned)nb, 256, 0, st>>>(s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    sca_tile_kernel<true><<<(unsigned)grid1, kThreads, smem1, st>>>(p, s, T);
    if ((e = cudaGetLastError()) != cudaSuccess) return e;
    if (!p.shipped) {  // the final tile pass wrote the output
        sca_last_cell_kernel<<<1, 1, 0, st>>>(p, s);
        return cudaGetLastError();
    }
    int64_t blocks = (n + 255) / 256;
    if (blocks > 8192) blocks = 8192;
    sca_output_kernel<<<(unsigned)blocks, 256, 0, st>>>(p, s);
    return cudaGetLastError();
}

}  // namespace pargo
