// window.cu -- the sync-free solve (SYNCFREE_WINDOW) and the level analysis by ONE CTA that
// walks the rows from the bottom of U (row n-1) to the top in 32-row blocks.
//
// Why one CTA: a deep DAG (the 2M-row irregular system has 348,506 levels for 2M rows) is bound
// by the latency of every dependency hop, not by bandwidth.  A hop through L2 (one SM publishes,
// another polls) costs ~375 ns on this GPU; inside one SM a hop is a shared-memory store and
// load.  So one CTA solves the whole system, and every recent x lives in a ring of kWinRing rows
// in shared memory.  One SM still has ample FP64 and load throughput for the work between hops
// (the 2M system: 15M FMAs, 206 MB of entries).
//
// Blocks: block t holds rows [n - 32(t+1), n - 32t) (the last one may be short); lane l of the
// warp owning block t takes row n - 1 - 32t - l.  Warp w owns blocks w, w + W, w + 2W, ...
// Every lane walks its CSR row from the right (largest column = solved earliest).  At the block's
// start it consumes every entry that is already available; the rest go in warp lockstep rounds
// of straight-line code, one entry per lane per round (no lane spins alone in divergent code).
// x of a column c is read from the ring when c < top(t) + reach, else from global memory.
//
// Staging: a block's entries (when they fit kCap entries per buffer), its row pointers,
// reciprocal diagonal and right-hand side are copied into the warp's shared buffers by cp.async
// one block ahead (row pointers two blocks ahead, since they size the copy), so no global load of
// the matrix sits between a dependency arriving and the row finishing.  A block with more
// entries than the buffer reads them from global memory (L1-cached).
//
// Ring protocol (no slot is read while it holds another row's value):
//   * block t starts only when blocks t-W-1 ... t-2W+1 are done (done flags in shared memory);
//     by induction every block <= t-W-1 is then done;
//   * at its start, block t resets the ring slots of block t+W (its warp's next block) to the
//     pending value.  Their previous rows (block t+W - kWinRing/32) are read through the ring
//     only by blocks up to (t+W - kWinRing/32) + reach/32 <= t-W-1, all done, and every block
//     that reads block t+W's rows starts after block t has started;
//   * reach = kWinRing - 32 (2W + 1) makes both hold; columns at or above top(t) + reach belong
//     to blocks <= t-W-1 (done) and are read from global x.
// Forward progress: every wait (a start condition, a pending x) is on a higher block, so the
// waits form no cycle and all W warps of the one CTA are resident.  Every spin is bounded by
// the spin budget and the abort flag, as in every other kernel here.  Rounds do not sleep: each
// warp has its own SM sub-partition at W = 4, and a sleeping round only delays the next hop.
//
// Arithmetic: the solve accumulates the ready entries right to left; at the first entry it has
// to wait for, it switches to the scaled form p = (b_i - sum) / U_ii and folds each later term
// as p = fma(-U_ij / U_ii, x_j, p), so a dependency hop costs one FP64 FMA.  The levels
// (core.cpp:244-270) take the maximum over the row's columns: level_i = 1 + max_j level_j
// (1 for a diagonal-only row), with 0 as the pending value, bit-exact.
#include <cstdlib>
#include <cstring>
#include <type_traits>
#include "common.cuh"
#include "kernels.cuh"
namespace sptrsv { int window_backoff_ns(); int window_warps(); }
namespace sptrsv { int window_backoff_ns(); int window_warps(); }

namespace sptrsv {

constexpr int kWinRing = 4096;   // rows of x held in shared memory (power of two)
constexpr int kWinFlags = 64;    // done-flag slots (power of two, multiple of W, >= 2W)
constexpr int kWinSmemBudget = 200 * 1024;

template <typename T> struct WinVal;
template <> struct WinVal<double> {
    static __device__ __forceinline__ double pending() { return Pend<double>::value(); }
    static __device__ __forceinline__ bool is_pending(double v) { return Pend<double>::is(v); }
};
template <> struct WinVal<float> {
    static __device__ __forceinline__ float pending() { return Pend<float>::value(); }
    static __device__ __forceinline__ bool is_pending(float v) { return Pend<float>::is(v); }
};
template <> struct WinVal<int> {
    static __device__ __forceinline__ int pending() { return 0; }
    static __device__ __forceinline__ bool is_pending(int v) { return v == 0; }
};

// Shared-memory layout: the ring and the done flags, then per warp three row-pointer slots,
// two reciprocal-diagonal / right-hand-side slots and two entry buffers of kCap entries.
template <typename T, int W> struct WinLayout {
    static constexpr bool kLevels = std::is_same<T, int>::value;
    static constexpr int kRpSlot = 36;  // 33 row pointers, padded to 16 bytes
    static constexpr size_t kFixed = (size_t)kWinRing * sizeof(T) + kWinFlags * sizeof(int);
    static constexpr size_t kPerWarpFixed = 3 * kRpSlot * sizeof(int) + (kLevels ? 0 : 2 * 2 * 32 * sizeof(T));
    static constexpr size_t kPerEntry = 2 * (sizeof(int) + (kLevels ? 0 : sizeof(T)));
    // entries per buffer: what the budget leaves, a multiple of 32
    static constexpr int kCap = (int)(((kWinSmemBudget - kFixed) / W - kPerWarpFixed) / kPerEntry) / 32 * 32;
    static constexpr size_t kPerWarp = kPerWarpFixed + (size_t)kCap * kPerEntry;
    static constexpr size_t kBytes = kFixed + (size_t)W * kPerWarp;
    static_assert(kCap >= 64, "staging buffers too small");
};

__device__ __forceinline__ void cpa4(void* s, const void* g) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(s);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;\n" ::"r"(a), "l"(g) : "memory");
}
__device__ __forceinline__ void cpa8(void* s, const void* g) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(s);
    asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(a), "l"(g) : "memory");
}
template <typename T> __device__ __forceinline__ void cpa(T* s, const T* g) {
    if constexpr (sizeof(T) == 8) cpa8(s, g);
    else cpa4(s, g);
}
__device__ __forceinline__ void cpa_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void cpa_wait_all() { asm volatile("cp.async.wait_all;\n" ::: "memory"); }

// Rows [lo, top) of block t.
__device__ __forceinline__ int win_top(int n, int t) { return n - 32 * t; }
__device__ __forceinline__ int win_lo(int n, int t) { return max(0, n - 32 * t - 32); }

// One warp's staging buffers.
template <typename T, int W> struct WinStage {
    int* rp;   // [3][kRpSlot]
    T* inv;    // [2][32]
    T* bb;     // [2][32]
    int* col;  // [2][kCap]
    T* val;    // [2][kCap]
    __device__ WinStage(char* base) {
        using L = WinLayout<T, W>;
        rp = (int*)base;
        char* p = base + 3 * L::kRpSlot * sizeof(int);
        if constexpr (!L::kLevels) {
            inv = (T*)p;
            bb = inv + 64;
            p += 2 * 2 * 32 * sizeof(T);
        } else {
            inv = bb = nullptr;
        }
        col = (int*)p;
        p += 2 * (size_t)L::kCap * sizeof(int);
        val = L::kLevels ? nullptr : (T*)p;
    }
};

// Copy block t's row pointers (rows lo .. top, inclusive) into rp slot `rs`.
template <typename T, int W>
__device__ __forceinline__ void win_stage_rp(const WinStage<T, W>& S, int rs, const int* rp, int n, int t, int lane) {
    const int lo = win_lo(n, t), top = win_top(n, t);
    int* d = S.rp + rs * WinLayout<T, W>::kRpSlot;
    for (int q = lane; q <= top - lo; q += 32) cpa4(d + q, rp + lo + q);
}

// Copy block t's entries (when they fit), reciprocal diagonal and right-hand side into data slot
// `ds`; its row pointers are already in rp slot `rs`.
template <typename T, int W>
__device__ __forceinline__ void win_stage_data(const WinStage<T, W>& S, int rs, int ds, const int* col, const T* val,
                                               const T* invd, const T* b, int n, int t, int lane) {
    using L = WinLayout<T, W>;
    const int lo = win_lo(n, t), top = win_top(n, t);
    const int* r = S.rp + rs * L::kRpSlot;
    const int e0 = r[0], cnt = r[top - lo] - e0;
    if (cnt <= L::kCap) {
        int* dc = S.col + ds * L::kCap;
        for (int q = lane; q < cnt; q += 32) cpa4(dc + q, col + e0 + q);
        if constexpr (!L::kLevels) {
            T* dv = S.val + ds * L::kCap;
            for (int q = lane; q < cnt; q += 32) cpa(dv + q, val + e0 + q);
        }
    }
    if constexpr (!L::kLevels) {
        const int i = top - 1 - lane;
        if (i >= lo) {
            cpa(S.inv + ds * 32 + lane, invd + i);
            cpa(S.bb + ds * 32 + lane, b + i);
        }
    }
}

// x in global memory: rows of this CTA only, plain stores and loads, ordered by the done-flag
// protocol's CTA fences (a reader only loads x of rows in finished blocks, after the acquire fence
// that follows the flag).  GPU-scope relaxed accesses measured no different.
template <typename T>
__device__ __forceinline__ T win_ld(const T* p) { return *p; }
template <typename T>
__device__ __forceinline__ void win_st(T* p, T v) { *p = v; }
// Bounded wait for x of a row in a finished block (never expected to wait): the value, or the
// pending value on timeout or abort (the timeout recorded).
template <typename T>
__device__ __noinline__ T win_wait(const T* p, Ctl* ctl, int64_t budget) {
    const uint64_t t0 = gtimer();
    for (;;) {
        const T v = *(const volatile T*)p;
        if (!WinVal<T>::is_pending(v)) return v;
        if (aborted(ctl)) return v;
        if ((int64_t)(gtimer() - t0) > budget) {
            record_error(ctl, SPTRSV_ERR_TIMEOUT);
            return v;
        }
        __nanosleep(64);
    }
}

template <typename T, int W>
__global__ void __launch_bounds__(W * 32, 1)
k_window(int n, const int* __restrict__ rp, const int* __restrict__ col, const T* __restrict__ val,
         const T* __restrict__ invd, const T* __restrict__ b, T* x, Ctl* ctl, int64_t budget) {
    using L = WinLayout<T, W>;
    constexpr bool kLevels = L::kLevels;
    constexpr int RM = kWinRing - 1;
    constexpr int reach = kWinRing - 32 * (2 * W + 1);
    static_assert(reach >= 32 * (W + 1), "ring too small for W warps");
    static_assert(kWinFlags % W == 0 && kWinFlags >= 2 * W, "flag slots");
    if (*(volatile const int*)&ctl->done) return;  // an inner solve after the refinement converged
    extern __shared__ __align__(16) char win_smem[];
    T* ring = reinterpret_cast<T*>(win_smem);
    int* dflag = reinterpret_cast<int*>(win_smem + (size_t)kWinRing * sizeof(T));
    volatile T* vring = ring;
    volatile int* vflag = dflag;
    for (int q = threadIdx.x; q < kWinRing; q += blockDim.x) ring[q] = WinVal<T>::pending();
    for (int q = threadIdx.x; q < kWinFlags; q += blockDim.x) dflag[q] = -1;

    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nblk = (n + 31) >> 5;
    const WinStage<T, W> S(win_smem + L::kFixed + (size_t)warp * L::kPerWarp);
    // prologue: row pointers of the warp's first two blocks, then the first block's data
    if (warp < nblk) {
        win_stage_rp<T, W>(S, 0, rp, n, warp, lane);
        if (warp + W < nblk) win_stage_rp<T, W>(S, 1, rp, n, warp + W, lane);
        cpa_commit();
        cpa_wait_all();
        __syncwarp();
        win_stage_data<T, W>(S, 0, 0, col, val, invd, b, n, warp, lane);
        cpa_commit();
    }
    __syncthreads();

    int lmax = 0;  // levels: largest level of this lane's rows
    int j = 0;     // this warp's block count
    // The lane's state for the warp's next block, prepared at the end of the block before it (in
    // the prologue for the first): its staged row scaled to the weights w_ij = -U_ij / U_ii (a
    // dependency hop then costs one FMA and no round multiplies), and its far columns -- rows of
    // blocks finished long before, read from global x -- folded into the partial sum.  So a block
    // starts with its walk over the ring.
    int nk = 0;                   // the entry to consume next
    T np = T(0), nacc = T(0);     // partial sums: b_i / U_ii + far terms (solves); max (levels)
    bool nfail = false;           // a far value never arrived (not expected): the lane gives up
    auto prepare = [&](int u, int jj) {
        const int ds_u = jj & 1;
        const int top = win_top(n, u), lo = win_lo(n, u);
        const int* rS = S.rp + (jj % 3) * L::kRpSlot;
        const int e0 = rS[0];
        const bool staged = rS[top - lo] - e0 <= L::kCap;
        const int i = top - 1 - lane;
        const int far = top + reach;
        nk = e0;
        np = nacc = T(0);
        nfail = false;
        if (i < lo) return;
        const int s = rS[i - lo];
        int k = rS[i - lo + 1] - 1;
        const int* rcol = staged ? S.col + ds_u * L::kCap + (s - e0) : col + s;
        T* rval = nullptr;
        T di = T(0), p = T(0), p2 = T(0), acc = T(0);
        if constexpr (!kLevels) {
            rval = staged ? S.val + ds_u * L::kCap + (s - e0) : const_cast<T*>(val) + s;
            di = S.inv[ds_u * 32 + lane];
            p = S.bb[ds_u * 32 + lane] * di;
            if (staged)
                for (int q = s + 1; q <= k; ++q) rval[q - s] = -rval[q - s] * di;
        }
        auto weight = [&](int q) -> T {
            if constexpr (kLevels) return T(0);
            else return staged ? rval[q - s] : -rval[q - s] * di;
        };
        // far columns (blocks <= u-W-1, done before block u-W started), four loads in flight
        int c = k > s ? rcol[k - s] : 0;
        bool fail = false;
        while (k > s && c >= far) {
            int cq[4];
            T vq[4], xq[4];
            bool use[4];
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                const int kq = k - q;
                use[q] = (q == 0 || use[q - 1]) && kq > s;
                cq[q] = use[q] ? rcol[kq - s] : 0;
                use[q] = use[q] && cq[q] >= far;
                vq[q] = use[q] ? weight(kq) : T(0);
            }
#pragma unroll
            for (int q = 0; q < 4; ++q) xq[q] = use[q] ? win_ld<T>(x + cq[q]) : T(0);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                // not expected: those blocks are done.  Wait all the same, bounded like every wait.
                if (use[q] && !fail && WinVal<T>::is_pending(xq[q])) {
                    xq[q] = win_wait<T>(x + cq[q], ctl, budget);
                    fail = WinVal<T>::is_pending(xq[q]);
                }
            }
            if (fail) break;
            int used = 0;
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                if (use[q]) {
                    if constexpr (kLevels) acc = max(acc, xq[q]);
                    else if (q & 1) p2 = fma(vq[q], xq[q], p2);
                    else p = fma(vq[q], xq[q], p);
                    ++used;
                }
            }
            k -= used;
            if (k > s) c = rcol[k - s];
        }
        nk = k;
        np = p + p2;
        nacc = acc;
        nfail = fail;
    };
    if (warp < nblk) {
        cpa_wait_all();
        __syncwarp();
        prepare(warp, 0);
    }
    for (int t = warp; t < nblk; t += W, ++j) {
        // 1. start condition: blocks t-W-1 ... t-2W+1 done (lane q checks block t-W-1-q)
        {
            const int tt = t - W - 1 - lane;
            bool ready = lane >= W - 1 || tt < 0 || vflag[tt & (kWinFlags - 1)] >= tt;
            if (!__all_sync(0xffffffffu, ready)) {
                const uint64_t t0 = gtimer();
                unsigned it = 0;
                bool fail = false;
                while (!__all_sync(0xffffffffu, ready || fail)) {
                    __nanosleep(32);
                    if (!ready) ready = vflag[tt & (kWinFlags - 1)] >= tt;
                    if ((++it & 63u) == 0) {
                        if (aborted(ctl)) fail = true;
                        else if ((int64_t)(gtimer() - t0) > budget) {
                            record_error(ctl, SPTRSV_ERR_TIMEOUT);
                            fail = true;
                        }
                    }
                }
                if (__any_sync(0xffffffffu, fail)) {
            cpa_wait_all();  // the warp's own copies in flight end before it returns
            return;
        }
            }
            __threadfence_block();
        }
        // 2. this block's staged data (copied one block ago) is complete
        cpa_wait_all();
        __syncwarp();
        const int rs = j % 3, ds = j & 1;
        // 3. stage ahead: row pointers of block t+2W, data of block t+W; reset block t+W's ring slots
        if (t + 2 * W < nblk) win_stage_rp<T, W>(S, (j + 2) % 3, rp, n, t + 2 * W, lane);
        if (t + W < nblk) win_stage_data<T, W>(S, (j + 1) % 3, (j + 1) & 1, col, val, invd, b, n, t + W, lane);
        cpa_commit();
        const int top = win_top(n, t), lo = win_lo(n, t);
        if (t + W < nblk) {
            const int r2 = top - 32 * W - 1 - lane;
            if (r2 >= 0) vring[r2 & RM] = WinVal<T>::pending();
        }
        // 4. the rows of block t
        const int* rS = S.rp + rs * L::kRpSlot;
        const int e0 = rS[0];
        const bool staged = rS[top - lo] - e0 <= L::kCap;
        const int i = top - 1 - lane;
        const int far = top + reach;
        bool done = i < lo;
        int s = e0, k = e0, c = 0;  // a lane without a row (short last block) reads entry e0 harmlessly
        if (!done) {
            s = rS[i - lo];
            k = nk;  // prepared: the far columns are folded in already
        }
        // the lane's entries through one pointer: the staged copy in shared memory, else global
        const int* rcol = staged ? S.col + ds * L::kCap + (s - e0) : col + s;
        T* rval = nullptr;  // the lane's row values (staged: scaled in place below)
        if constexpr (!kLevels) rval = staged ? S.val + ds * L::kCap + (s - e0) : const_cast<T*>(val) + s;
        auto ecol = [&](int q) -> int { return rcol[q - s]; };
        // levels: acc; solves: p = b_i / U_ii + sum of w_ij x_j (the prepared part so far)
        T acc = nacc, di = T(0), p = np;
        bool fail = nfail;
        if (fail) done = true;  // the lane gives up: no rounds, no publication; the warp returns
        if constexpr (!kLevels) {
            if (!done) di = S.inv[ds * 32 + lane];
        }
        // xm is this lane's value once its row is finished.
        T xm = WinVal<T>::pending();
        // The block's rows, compiled twice: a staged block's weights are loads, a block read from
        // global memory has each weight scaled as it is loaded.
        auto block_rows = [&](auto staged_c) {
        constexpr bool kStaged = decltype(staged_c)::value;
        (void)kStaged;  // the level analysis has no weights
        auto weight = [&](int q) -> T {
            if constexpr (kLevels) return T(0);
            else if constexpr (kStaged) return rval[q - s];
            else return -rval[q - s] * di;
        };
        T v = T(0);  // the head's weight
        T p2 = T(0);  // a second accumulator for the setup's FMAs (two chains instead of one)
        (void)p2;
        if (!done) {
            if (k > s) {
                c = ecol(k);
                v = weight(k);
            }
        }
        // the rest: one walk over what is ready, then lockstep rounds over the remaining entries.
        // walk right to left consuming ready entries (into the two accumulators by the entry's
        // parity); stops at the first pending one
        auto walk = [&]() {
            while (k > s) {
                const T xv = c >= far ? win_ld<T>(x + c) : vring[c & RM];
                if (WinVal<T>::is_pending(xv)) break;
                if constexpr (kLevels) acc = max(acc, xv);
                else if (k & 1) p2 = fma(v, xv, p2);
                else p = fma(v, xv, p);
                if (--k > s) {
                    c = ecol(k);
                    v = weight(k);
                }
            }
            if constexpr (!kLevels) {
                p += p2;
                p2 = T(0);
            }
        };
        auto finish = [&]() {
            if constexpr (kLevels) {
                xm = T(1) + acc;
                lmax = max(lmax, xm);
            } else {
                xm = Pend<T>::fix(p);
            }
            vring[i & RM] = xm;  // global x is written once the whole block is done
            done = true;
        };
        if (!done) {
            walk();
            if (k <= s) finish();
        }
        // The remaining entries, one per round (the head, entry k, is pending).  A round is the same
        // straight-line code for every lane: the head's value from the ring (the pending pattern
        // until its row is finished, in this block or another), one FMA, and the move to the next
        // entry, whose column and weight were loaded a round ahead.  (Handing in-block values over
        // by warp shuffles instead -- two shuffles and a select a round -- measured slower on the
        // 2M-row system: 140.5 against 131.0 ms for the solve, 97.2 against 80.4 ms for the
        // levels, same GPU; so did two entries a round, and an L1 prefetch of the far columns.
        // Writing each finished row to global x at once, rather than the block's 32 rows in one
        // coalesced store at its end, cost 131.1 against 118.1 ms; forming each next weight by a
        // multiply in the round, rather than scaling the staged row once, 118.2 against 110.8 ms;
        // one round per loop pass instead of two (one vote, one timer countdown per pass), 110.8
        // against 107.0 ms and 79.9 against 76.2 ms for the levels; four per pass, 99.7 and
        // 73.4 ms.  With the setup specialised for staged blocks and two FMA chains in it, eight
        // warps take 77.1 and 44.7 ms; eight rounds per pass, 73.6 and 40.4 ms; each block
        // prepared (its row scaled, its far columns folded in) at the end of the warp's block
        // before it, 68.0 and 41.4 ms.)
        // Registers hold the head (entry k: column c, weight w) and the next entry (cn, wn: k-1, an
        // index past the row's start clamped to it and never consumed), loaded a round ahead.  The
        // loop is compiled twice: for a staged block its weights are loads, for a block read from
        // global memory each is scaled as it is loaded (see block_rows).
        T w = v, wn = T(0);
        (void)w;
        int cn = 0;
        if (!done) {
            const int k1 = max(k - 1, s);
            cn = ecol(k1);
            wn = weight(k1);
        }
        __syncwarp();  // the lanes' ring stores of rows finished above before the rounds' loads
        // the budget's timer starts at the block for short budgets, else at round 31 of the block
        uint64_t t0 = budget < 1000000 ? gtimer() : 0;
        auto rounds = [&]() {
            auto step = [&]() {
                // The head's value from the ring: rows of this block and of the blocks in flight
                // are stored there when they finish (the __syncwarp that ends a round orders this
                // warp's stores before the next round's loads).  A column beyond the ring's reach
                // is read from global x: rows need not be sorted, so such an entry can follow a
                // near one (rare; the far loop took the sorted case).  A finished lane's stale
                // column reads a slot whose value is discarded.
                T x0;
                if (__builtin_expect(c >= far, 0)) x0 = win_ld<T>(x + c);
                else x0 = vring[c & RM];
                const bool rdy = !done && !WinVal<T>::is_pending(x0);
                if constexpr (kLevels) acc = rdy ? max(acc, x0) : acc;
                else p = rdy ? fma(w, x0, p) : p;
                k -= (int)rdy;
                c = rdy ? cn : c;
                if constexpr (!kLevels) w = rdy ? wn : w;
                {
                    // the entry after the head, for the next round (a repeated load when nothing
                    // moved)
                    const int k1 = max(k - 1, s);
                    cn = ecol(k1);
                    wn = weight(k1);
                }
                {
                    // the row's completion without a branch: value, ring store, flag
                    const bool fin = rdy && k <= s;
                    T xf;
                    if constexpr (kLevels) xf = T(1) + acc;
                    else xf = Pend<T>::fix(p);
                    xm = fin ? xf : xm;
                    if constexpr (kLevels) lmax = fin ? max(lmax, xf) : lmax;
                    if (fin) vring[i & RM] = xf;
                    done = done || fin;
                }
                __syncwarp();
            };
            int cd = 31;  // rounds to the next timer check (eight per loop pass)
            for (;;) {
                if (__all_sync(0xffffffffu, done)) break;
                step();
                step();  // harmless when every lane finished in an earlier one
                step();
                step();
                step();
                step();
                step();
                step();
                if ((cd -= 8) <= 0) {
                    cd = 256;
                    if (aborted(ctl)) fail = true;
                    else if (t0 == 0) t0 = gtimer();
                    else if ((int64_t)(gtimer() - t0) > budget) {
                        record_error(ctl, SPTRSV_ERR_TIMEOUT);
                        fail = true;
                    }
                    if (__any_sync(0xffffffffu, fail)) {
                        fail = true;
                        break;
                    }
                }
            }
        };
        rounds();
        };
        if (staged) block_rows(std::true_type{});
        else block_rows(std::false_type{});
        if (__any_sync(0xffffffffu, fail)) {
            cpa_wait_all();  // the warp's own copies in flight end before it returns
            return;
        }
        // 5. block t done: its rows to global x in one coalesced store; those stores, the ring
        //    stores and the reset of block t+W's slots before the flag
        if (i >= lo) win_st<T>(x + i, xm);
        __threadfence_block();
        __syncwarp();
        if (lane == 0) vflag[t & (kWinFlags - 1)] = t;
        // 6. the warp's next block: its data (staged at this block's start) has landed
        if (t + W < nblk) {
            cpa_wait_all();
            __syncwarp();
            prepare(t + W, j + 1);
        }
    }
    cpa_wait_all();  // no copy left in flight when the warp exits
    if constexpr (kLevels) {
        for (int o = 16; o > 0; o >>= 1) lmax = max(lmax, __shfl_xor_sync(0xffffffffu, lmax, o));
        if (lane == 0 && lmax > 0) atomicMax(&ctl->max_level, lmax);
    }
}

// ---------------------------------------------------------------------------------------
template <typename T, int W>
static int window_launch(int n, const int* rp, const int* col, const T* val, const T* invd, const T* b, T* x,
                         Ctl* ctl, int64_t budget, cudaStream_t st, int64_t* launches) {
    using L = WinLayout<T, W>;
    static bool configured[64] = {};
    int dev = 0;
    CUDA_TRY(cudaGetDevice(&dev));
    if (dev < 0 || dev >= 64) return SPTRSV_ERR_INVALID_ARG;
    if (!configured[dev]) {
        CUDA_TRY(cudaFuncSetAttribute(k_window<T, W>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)L::kBytes));
        configured[dev] = true;
    }
    k_window<T, W><<<1, W * 32, L::kBytes, st>>>(n, rp, col, val, invd, b, x, ctl, budget);
    ++*launches;
    CUDA_TRY(cudaGetLastError());
    return 0;
}

// Warps of the window CTA: SPTRSV_WINDOW_WARPS = 2, 4, 8 or 16 forces one; otherwise 8 while a
// 32-row block's entries (at the matrix's mean row length) fill at most 90 % of the 8-warp staging
// buffer, else 4 (more warps hide more of each block's setup behind the other warps' rounds, but
// leave less staging space per warp).  Measured on the 2M-row system (8.6 entries per row, same
// GPU): the solve 124.7 / 77.1 / 92.7 ms and the levels 74.4 / 44.7 / 52.7 ms at 4 / 8 / 16 warps;
// on 200k-row random factors the solve at 8 warps 7.7 / 12.4 / 15.8 ms against 12.4 / 17.4 /
// 21.8 ms at 4 with 8.6 / 15.5 / 21.7 entries per row, and 51.2 against 25.9 ms with 27.4 (whose
// blocks no longer fit 8 warps' buffers).
template <typename T>
static int window_pick_warps(int n, long long nnz) {
    const int forced = window_warps();
    if (forced) return forced;
    if (n <= 0 || nnz <= 0) return 4;
    return 32.0 * (double)nnz / n <= 0.9 * WinLayout<T, 8>::kCap ? 8 : 4;
}

template <typename T>
static int window_dispatch(int n, long long nnz, const int* rp, const int* col, const T* val, const T* invd,
                           const T* b, T* x, Ctl* ctl, int64_t budget, cudaStream_t st, int64_t* launches) {
    switch (window_pick_warps<T>(n, nnz)) {
        case 2: return window_launch<T, 2>(n, rp, col, val, invd, b, x, ctl, budget, st, launches);
        case 16: return window_launch<T, 16>(n, rp, col, val, invd, b, x, ctl, budget, st, launches);
        case 8: return window_launch<T, 8>(n, rp, col, val, invd, b, x, ctl, budget, st, launches);
        default: return window_launch<T, 4>(n, rp, col, val, invd, b, x, ctl, budget, st, launches);
    }
}

// SPTRSV_WINDOW_WARPS (2, 4, 8 or 16), or 0 when unset.
int window_warps() {
    static int w = [] {
        const char* e = getenv("SPTRSV_WINDOW_WARPS");
        const int v = e ? atoi(e) : 0;
        return (v == 2 || v == 4 || v == 8 || v == 16) ? v : 0;
    }();
    return w;
}

int launch_window(bool f32, const SolveArgs& a) {
    if (a.rhs != 1) return SPTRSV_ERR_UNSUPPORTED;
    if (f32)
        return window_dispatch<float>(a.n, a.nnz, a.rp, a.col, (const float*)a.val, (const float*)a.invd,
                                      (const float*)a.b, (float*)a.x, a.ctl, a.budget, a.st, a.launches);
    return window_dispatch<double>(a.n, a.nnz, a.rp, a.col, (const double*)a.val, (const double*)a.invd,
                                   (const double*)a.b, (double*)a.x, a.ctl, a.budget, a.st, a.launches);
}

int launch_window_levels(int n, long long nnz, const int* rp, const int* col, int* level, Ctl* ctl, int64_t budget,
                         cudaStream_t st, int64_t* launches) {
    return window_dispatch<int>(n, nnz, rp, col, nullptr, nullptr, nullptr, level, ctl, budget, st, launches);
}

}  // namespace sptrsv
