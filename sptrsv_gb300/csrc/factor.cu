// factor.cu -- the upstream step: a multifrontal supernodal Cholesky A = U^T U of a symmetric
// positive definite matrix on the GPU, producing U in the solver's CSR layout (diagonal first in
// every row) and its supernode partition.  The reference takes its factors from an external
// sparse Cholesky; this builds them from A and an elimination tree of fronts.
//
// Symbolic step (host): front t pivots rows f0 .. f1-1 and hands its update matrix to its parent.
// Its row set is S_t = [f0, f1) followed, sorted, by every row >= f1 adjacent in A to one of its
// pivots or in one of its children's update sets.  U's pattern follows: row f0 + k holds S_t[k:].
// Numeric step (GPU, by tree level): a front's height is 0 for a leaf and one more than its
// highest child otherwise; the fronts of one height are independent, so each step below is one
// launch over every front of the level (a work list of fronts and a prefix of their CTA counts).
// The dense front F_t (|S_t| x |S_t|, column major, lower triangle) gets A's entries and its
// children's update matrices (extend-add, the children in order), then a blocked right-looking
// Cholesky over its first w = f1 - f0 columns in 64-column panels: the panel's diagonal tile
// factored by one CTA, the rows below it solved against that tile, the trailing lower triangle
// updated by a tiled FP64 rank-64 product.  Running the trailing updates over the whole front
// leaves the Schur complement -- the update matrix for the parent -- in F_t[w:, w:].  Column
// f0 + k of L = U^T is F_t[k:, k], copied into U's row f0 + k.  The fronts of a level share one
// region of a single arena, reused once the level's parents have taken their update matrices;
// every entry sees the same operations in the same order as a front-by-front run.
#include <algorithm>
#include <chrono>
#include <cstdlib>
#include <cstdint>
#include <cstring>
#include <type_traits>
#include <vector>
#include "common.cuh"
#include "sptrsv_gb300.h"
#include "tc.cuh"

namespace sptrsv {

constexpr int kFb = 64;       // panel width and update tile
constexpr int kTrsmRows = 16;  // rows per CTA of the panel solve

// Where the fronts live: front t is F = arena + foff[t], fm[t] x fm[t], pivots fstart[t] ..
// fstart[t+1]-1.
struct FrontTab {
    const int* fstart;
    const int* fm;
    const int64_t* foff;
};

// The work item of CTA b in a launch over nlist fronts with CTA prefix counts: the largest f with
// prefix[f] <= b (every listed front has at least one CTA).
__device__ __forceinline__ int fr_item(const int* __restrict__ prefix, int nlist, int b) {
    int lo = 0, hi = nlist - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (prefix[mid] <= b) lo = mid;
        else hi = mid - 1;
    }
    return lo;
}

// (i, j), j <= i, of the e-th entry of a lower triangle walked row by row.
__device__ __forceinline__ void fr_tri(int e, int& i, int& j) {
    i = (int)((sqrtf(8.0f * e + 1.0f) - 1.0f) * 0.5f);
    while ((i + 1) * (i + 2) / 2 <= e) ++i;
    while (i * (i + 1) / 2 > e) --i;
    j = e - i * (i + 1) / 2;
}

// A's entries of the listed fronts, one CTA per front: F_t[idx[q]] = v[q] for q in off[t] ..
// off[t+1]-1 (idx within the front).
__global__ void k_fr_scatter(double* __restrict__ arena, FrontTab ft, const int* __restrict__ list,
                             const int64_t* __restrict__ off, const int64_t* __restrict__ idx,
                             const double* __restrict__ v) {
    const int t = list[blockIdx.x];
    double* F = arena + ft.foff[t];
    for (int64_t q = off[t] + threadIdx.x; q < off[t + 1]; q += blockDim.x) F[idx[q]] = v[q];
}

// F_p[map[r] + map[s] m] += C[(wc + r) + (wc + s) mc] for s <= r < nu: child c = child[blockIdx.y]
// adds its update matrix (the lower triangle of its front past its pivots) into its parent p.
// One launch takes at most one child of each parent, so no two CTAs add into the same entry.
__global__ void k_fr_extend_add(double* __restrict__ arena, FrontTab ft, const int* __restrict__ child,
                                const int* __restrict__ parent, const int* __restrict__ maps,
                                const int64_t* __restrict__ map_start) {
    const int c = child[blockIdx.y], p = parent[c];
    const int wc = ft.fstart[c + 1] - ft.fstart[c], mc = ft.fm[c], nu = mc - wc, m = ft.fm[p];
    const double* C = arena + ft.foff[c];
    double* F = arena + ft.foff[p];
    const int* map = maps + map_start[c];
    const long long total = (long long)nu * nu;
    for (long long e = blockIdx.x * (long long)blockDim.x + threadIdx.x; e < total;
         e += (long long)gridDim.x * blockDim.x) {
        const int s = (int)(e / nu), r = (int)(e - (long long)s * nu);
        if (r < s) continue;
        F[(size_t)map[r] + (size_t)map[s] * m] += C[(size_t)(wc + r) + (size_t)(wc + s) * mc];
    }
}

// Cholesky of the kb x kb diagonal tile at (k0, k0) of front list[blockIdx.x], lower, in place
// (one CTA of 256 threads per front).  A pivot that is not positive (or not finite) sets *bad and
// the factor is not used.  Column j is scaled by the reciprocal square root of its pivot (its
// diagonal becomes d * rsqrt(d)), then the rest of the tile takes its rank-1 update.  The next
// pivot is final as soon as its own update is made, so warp 7 makes that one update and the next
// reciprocal root while warps 0-6 update the other entries of the rest's lower triangle (from a
// table of (row, column) pairs: no lane idles on the upper half): the square root is off the
// chain of columns, which is one scale and one update step per column.
__global__ void __launch_bounds__(256) k_fr_potrf(double* __restrict__ arena, FrontTab ft,
                                                  const int* __restrict__ list, int k0, int* bad) {
    __shared__ double T[kFb][kFb + 1];
    __shared__ int pairs[kFb * (kFb + 1) / 2];  // e = i (i + 1) / 2 + c  ->  i << 8 | c, c <= i
    __shared__ double rs;
    const int t = list[blockIdx.x];
    double* F = arena + ft.foff[t];
    const int m = ft.fm[t], kb = min(kFb, ft.fstart[t + 1] - ft.fstart[t] - k0);
    constexpr int kUpd = 224;  // threads of warps 0-6
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, c = e / kb;
        T[r][c] = r >= c ? F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] : 0.0;
    }
    for (int e = threadIdx.x; e < kFb * (kFb + 1) / 2; e += blockDim.x) {
        int i, c;
        fr_tri(e, i, c);
        pairs[e] = i << 8 | c;
    }
    __syncthreads();
    // the root of pivot j: its reciprocal to rs, the root itself in place
    auto root = [&](int j) {
        const double d = T[j][j];
        if (!(d > 0.0) || !isfinite(d)) atomicExch(bad, 1);
        const double dd = d > 0.0 ? d : 1.0, r = rsqrt(dd);
        T[j][j] = dd * r;
        rs = r;
    };
    if (threadIdx.x == kUpd) root(0);
    __syncthreads();
    for (int j = 0; j < kb; ++j) {
        const double r = rs;
        for (int i = j + 1 + threadIdx.x; i < kb; i += blockDim.x) T[i][j] *= r;
        __syncthreads();
        const int rest = kb - j - 1, np = rest * (rest + 1) / 2;
        if (threadIdx.x < kUpd) {
            for (int e = 1 + threadIdx.x; e < np; e += kUpd) {
                const int pr = pairs[e], i = j + 1 + (pr >> 8), c = j + 1 + (pr & 255);
                T[i][c] = fma(-T[i][j], T[c][j], T[i][c]);
            }
        } else if (threadIdx.x == kUpd && rest > 0) {
            T[j + 1][j + 1] = fma(-T[j + 1][j], T[j + 1][j], T[j + 1][j + 1]);
            root(j + 1);
        }
        __syncthreads();
    }
    for (int e = threadIdx.x; e < kb * kb; e += blockDim.x) {
        const int r = e % kb, c = e / kb;
        if (r >= c) F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] = T[r][c];
    }
}

// Rows r0 .. m-1 of the panel (columns k0 .. k0+kb-1, r0 = k0 + kb) of each listed front:
// X L^T = B with L the factored tile.  kTrsmRows rows per CTA, eight lanes per row (one warp
// holds four rows).  The columns go in blocks of eight: lane q first forms its column's sum over
// the blocks already solved (the row's solved values and L's rows come from shared memory, four
// partial sums), then the block's 8 x 8 triangle is solved across the eight lanes by shuffles.
// A row's 2,016 FMAs are spread over eight lanes, and the dependent chain is eight short blocks.
__global__ void __launch_bounds__(kTrsmRows * 8) k_fr_trsm(double* __restrict__ arena, FrontTab ft,
                                                           const int* __restrict__ list,
                                                           const int* __restrict__ prefix, int nlist, int k0) {
    __shared__ double L[kFb][kFb + 1];
    __shared__ double X[kTrsmRows][kFb + 1];
    __shared__ double dinv[kFb];
    const int f = fr_item(prefix, nlist, blockIdx.x), t = list[f];
    double* F = arena + ft.foff[t];
    const int m = ft.fm[t], kb = min(kFb, ft.fstart[t + 1] - ft.fstart[t] - k0);
    const int row0 = k0 + kb + (blockIdx.x - prefix[f]) * kTrsmRows;
    for (int e = threadIdx.x; e < kFb * kFb; e += blockDim.x) {
        const int r = e % kFb, c = e / kFb;
        L[r][c] = r < kb && c <= r ? F[(size_t)(k0 + r) + (size_t)(k0 + c) * m] : 0.0;
    }
    for (int e = threadIdx.x; e < kTrsmRows * kb; e += blockDim.x) {
        const int rr = e % kTrsmRows, c = e / kTrsmRows;
        X[rr][c] = row0 + rr < m ? F[(size_t)(row0 + rr) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    if (threadIdx.x < kFb) dinv[threadIdx.x] = threadIdx.x < kb ? 1.0 / L[threadIdx.x][threadIdx.x] : 0.0;
    __syncthreads();
    const int g = threadIdx.x >> 3, q = threadIdx.x & 7;
    const unsigned full = 0xffffffffu;
    for (int j0 = 0; j0 < kb; j0 += 8) {
        const int c = j0 + q;
        double s0 = c < kb ? X[g][c] : 0.0, s1 = 0.0, s2 = 0.0, s3 = 0.0;
        for (int p = 0; p < j0; p += 4) {
            s0 = fma(-X[g][p], L[c][p], s0);
            s1 = fma(-X[g][p + 1], L[c][p + 1], s1);
            s2 = fma(-X[g][p + 2], L[c][p + 2], s2);
            s3 = fma(-X[g][p + 3], L[c][p + 3], s3);
        }
        double s = (s0 + s1) + (s2 + s3), x = 0.0;
#pragma unroll
        for (int p = 0; p < 8; ++p) {
            const double xp = __shfl_sync(full, s * dinv[j0 + p], p, 8);
            if (q == p) x = xp;
            if (q > p) s = fma(-xp, L[c][j0 + p], s);
        }
        if (c < kb) X[g][c] = x;
        __syncwarp();
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kTrsmRows * kb; e += blockDim.x) {
        const int rr = e % kTrsmRows, c = e / kTrsmRows;
        if (row0 + rr < m) F[(size_t)(row0 + rr) + (size_t)(k0 + c) * m] = X[rr][c];
    }
}

// The trailing lower triangle F[r0:, r0:] -= P P^T with P = F[r0:, k0:k0+kb] of each listed
// front: one 64 x 64 output tile per CTA (the CTA's item is the tile's index in the lower
// triangle of tiles), 256 threads of 4 x 4 outputs each.
__global__ void __launch_bounds__(256) k_fr_syrk(double* __restrict__ arena, FrontTab ft, const int* __restrict__ list,
                                                 const int* __restrict__ prefix, int nlist, int k0) {
    const int f = fr_item(prefix, nlist, blockIdx.x), t = list[f];
    double* F = arena + ft.foff[t];
    const int m = ft.fm[t], kb = min(kFb, ft.fstart[t + 1] - ft.fstart[t] - k0), r0 = k0 + kb;
    int ti, tj;
    fr_tri(blockIdx.x - prefix[f], ti, tj);
    extern __shared__ double fr_sm[];
    double* A = fr_sm;                    // [kFb][kFb + 1]: rows of tile ti
    double* B = fr_sm + kFb * (kFb + 1);  // [kFb][kFb + 1]: rows of tile tj
    const int rA = r0 + ti * kFb, rB = r0 + tj * kFb;
    for (int e = threadIdx.x; e < kFb * kb; e += blockDim.x) {
        const int rr = e % kFb, c = e / kFb;
        A[rr * (kFb + 1) + c] = rA + rr < m ? F[(size_t)(rA + rr) + (size_t)(k0 + c) * m] : 0.0;
        B[rr * (kFb + 1) + c] = rB + rr < m ? F[(size_t)(rB + rr) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    const int tx = threadIdx.x & 15, ty = threadIdx.x >> 4;
    double acc[4][4] = {};
    for (int c = 0; c < kb; ++c) {
        double a[4], b[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
            a[u] = A[(ty * 4 + u) * (kFb + 1) + c];
            b[u] = B[(tx * 4 + u) * (kFb + 1) + c];
        }
#pragma unroll
        for (int u = 0; u < 4; ++u)
#pragma unroll
            for (int v = 0; v < 4; ++v) acc[u][v] = fma(a[u], b[v], acc[u][v]);
    }
    // the 16 outputs are read first, then written (no load waits behind a store)
    double cur[4][4];
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int row = rA + ty * 4 + u, colx = rB + tx * 4 + v;
            cur[u][v] = row < m && colx <= row ? F[(size_t)row + (size_t)colx * m] : 0.0;
        }
#pragma unroll
    for (int u = 0; u < 4; ++u)
#pragma unroll
        for (int v = 0; v < 4; ++v) {
            const int row = rA + ty * 4 + u, colx = rB + tx * 4 + v;
            if (row < m && colx <= row) F[(size_t)row + (size_t)colx * m] = cur[u][v] - acc[u][v];
        }
}

// ---- the trailing update on the tensor cores
// C -= P P^T with P the panel's rows below its diagonal tile (K = kb <= 64 columns), FP64-accurate
// from BF16 digit slices (the fixed-point split product of Ozaki, Ogita, Oishi and Rump, 2012, in
// tc.cuh): every row i of P is 2^e_i times eight signed 7-bit digit vectors d_1..d_8, so
// (P P^T)_ij = 2^(e_i + e_j) sum_{p,q} 2^(-7(p+q)) (d_p[i] . d_q[j]).  Pairs with p + q <= 9 are
// formed (the rest lie below FP64 rounding); the products of one digit diagonal k = p + q share a
// TMEM accumulator, at most eight 64-term sums of products below 2^14: integers below 2^23, exact
// in FP32.  The epilogue packs diagonals 2..5 and 6..9 into two integers below 2^44 (exact in
// int64, then exact as FP64, built by integer operations with the scale in the exponent) and
// subtracts them from C -- two FP64-pipe operations per output instead of the 64 FMAs of the FP64
// tile (k_fr_syrk).
constexpr int kTcBlk = 64;                                  // rows per digit block
constexpr int kTcSlice = kTcBlk * kFb * 2;                  // one digit slice of a block (K = 64), bytes
constexpr int kTcRec = tc::kDigits * kTcSlice + kTcBlk * 4;  // a block: eight slices, then row exponents
constexpr int kTcM = 128, kTcN = 32;                        // output tile: 128 rows x 32 columns
constexpr int kTcChunk = 4;                                 // tiles per CTA (128 columns), one A block
constexpr int kTcEpiWarps = 8;                              // epilogue warps; warp 8 loads and issues
constexpr unsigned kTcSlA = kTcM * kFb * 2, kTcSlB = kTcN * kFb * 2;  // one digit slice of A / of B
constexpr size_t kTcSmem = (size_t)tc::kDigits * (kTcSlA + 2 * kTcSlB) + (kTcM + kTcChunk * kTcN) * 4 + 128;
constexpr int kTcMinRest = 256;                             // fronts with fewer rows below use k_fr_syrk
// CTAs of one front's tensor-core update: row block I takes min(I + 1, chunks) chunks of tiles
__host__ __device__ __forceinline__ int tc_ctas_of_block(int I, int nchunks) { return I + 1 < nchunks ? I + 1 : nchunks; }

// Digit blocks of the listed fronts' panel rows below the diagonal tile: CTA b of front f makes
// block b (rows r0 + 64 b ..) in buf at (prefix[f] + b) * kTcRec; rows past the front are zero.
__global__ void __launch_bounds__(256) k_fr_split(const double* __restrict__ arena, FrontTab ft,
                                                  const int* __restrict__ list, const int* __restrict__ prefix,
                                                  int nlist, int k0, unsigned char* __restrict__ buf) {
    __shared__ double P[kTcBlk][kFb + 1];
    __shared__ int s_exp[kTcBlk];
    const int f = fr_item(prefix, nlist, blockIdx.x), t = list[f], b = blockIdx.x - prefix[f];
    const double* F = arena + ft.foff[t];
    const int m = ft.fm[t], kb = min(kFb, ft.fstart[t + 1] - ft.fstart[t] - k0);
    const int row0 = k0 + kb + b * kTcBlk;
    unsigned char* rec = buf + (size_t)blockIdx.x * kTcRec;
    if (threadIdx.x < kTcBlk) s_exp[threadIdx.x] = tc::kExpZero;
    for (int e = threadIdx.x; e < kTcBlk * kFb; e += blockDim.x) {
        const int rr = e % kTcBlk, c = e / kTcBlk;
        P[rr][c] = row0 + rr < m && c < kb ? F[(size_t)(row0 + rr) + (size_t)(k0 + c) * m] : 0.0;
    }
    __syncthreads();
    for (int e = threadIdx.x; e < kTcBlk * kFb; e += blockDim.x) {
        const int rr = e % kTcBlk, c = e / kTcBlk;
        if (P[rr][c] != 0.0) atomicMax(&s_exp[rr], tc::exp_bound(P[rr][c]));
    }
    __syncthreads();
    // element i of the tile layout: (k & 7) fastest, then (r & 7), (k >> 3), (r >> 3), so that a
    // warp writes 64 consecutive bytes of every slice
    for (int i = threadIdx.x; i < kTcBlk * kFb; i += blockDim.x) {
        const int k = (i & 7) | ((i >> 6) & 7) << 3, rr = ((i >> 3) & 7) | (i >> 9) << 3;
        float d[tc::kDigits];
        tc::digits(P[rr][k], s_exp[rr], d);
#pragma unroll
        for (int q = 0; q < tc::kDigits; ++q)
            reinterpret_cast<__nv_bfloat16*>(rec + q * kTcSlice)[i] = __float2bfloat16(d[q]);
    }
    if (threadIdx.x < kTcBlk) reinterpret_cast<int*>(rec + tc::kDigits * kTcSlice)[threadIdx.x] = s_exp[threadIdx.x];
}

// X 2^s as an FP64 value for an integer 0 < |X| < 2^53 -- exact, so built from X's bits with
// integer operations (sign, leading-bit position, the 52 bits below it, the exponent with s
// added) instead of a conversion and a multiply on the FP64 pipe; ldexp where the result would not
// be a normal number.
__device__ __forceinline__ double fr_exact(long long X, int s) {
    const unsigned long long a = (unsigned long long)(X < 0 ? -X : X);
    const int lz = __clzll((long long)a);
    const int ex = (63 - lz) + s + 1023;
    if (ex < 1 || ex > 2046) return ldexp((double)X, s);
    const unsigned long long mant = (a << (lz - 11)) & 0xFFFFFFFFFFFFFull;
    return __longlong_as_double((long long)((X < 0 ? 1ull << 63 : 0ull) | ((unsigned long long)ex << 52) | mant));
}

// Tiles 4c .. 4c+3 (32 columns each, those with a part on or below the diagonal) of row block I
// (128 rows) of each listed front's trailing lower triangle.  Warp 8 is the producer: bulk copies
// of the A digit blocks (2I, 2I+1, kept for the whole chunk) and, per tile, of the B digits (half
// a block) into one of two buffers, then 144 MMAs of 128 x 32 x 16 by one thread into one of two
// TMEM accumulator sets (eight digit diagonals x 32 columns each).  Warps 0-7 are the epilogue:
// warp w reads TMEM lanes 32 (w % 4) .. + 31 and columns 16 (w / 4) .. + 15 of the tile, so the
// MMAs of tile n + 1 run while tile n's outputs are formed and written.  Barriers: A (once), B
// and MMA per buffer (phase = use of the buffer), epilogue-done per TMEM set (256 arrivals).  All
// waits are bounded; a timeout records SPTRSV_ERR_TIMEOUT in ctl, which every waiter polls.
__global__ void __launch_bounds__(32 * (kTcEpiWarps + 1), 1)
    k_fr_syrk_tc(double* __restrict__ arena, FrontTab ft, const int* __restrict__ list,
                 const int* __restrict__ prefix, int nlist, const int* __restrict__ sprefix, int k0,
                 const unsigned char* __restrict__ buf, Ctl* ctl, int64_t budget) {
    extern __shared__ __align__(128) unsigned char fr_tc[];
    unsigned char* sA = fr_tc;                                      // 8 slices x 128 rows x 64
    unsigned char* sB = fr_tc + (size_t)tc::kDigits * kTcSlA;       // 2 buffers x 8 slices x 32 rows x 64
    int* sAe = reinterpret_cast<int*>(sB + 2 * (size_t)tc::kDigits * kTcSlB);
    int* sBe = sAe + kTcM;                                          // the chunk's columns
    __shared__ __align__(8) uint64_t barA, barB[2], barM[2], barE[2];
    __shared__ uint32_t s_tmem;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int f = fr_item(prefix, nlist, blockIdx.x), t = list[f];
    double* F = arena + ft.foff[t];
    const int m = ft.fm[t], kb = min(kFb, ft.fstart[t + 1] - ft.fstart[t] - k0), r0 = k0 + kb;
    const int nJ = (m - r0 + kTcN - 1) / kTcN, nC = (nJ + kTcChunk - 1) / kTcChunk;
    int e = blockIdx.x - prefix[f], I = 0;
    for (;;) {
        const int c = tc_ctas_of_block(I, nC);
        if (e < c) break;
        e -= c;
        ++I;
    }
    const int J0 = e * kTcChunk, nt = min(kTcChunk, min(4 * I + 4, nJ) - J0);  // tiles J0 .. J0+nt-1
    const unsigned char* blocks = buf + (size_t)sprefix[f] * kTcRec;
    if (warp == 0) tc::tmem_alloc(&s_tmem, 2 * tc::kDigits * kTcN);
    if (tid == 0) {
        tc::mbar_init(&barA, 1);
        for (int b = 0; b < 2; ++b) {
            tc::mbar_init(&barB[b], 1);
            tc::mbar_init(&barM[b], 1);
            tc::mbar_init(&barE[b], 32 * kTcEpiWarps);
        }
    }
    tc::fence_before();
    __syncthreads();
    tc::fence_after();
    const uint32_t tmem = s_tmem;
    if (warp == kTcEpiWarps) {
        if (lane == 0) {
            // A (two blocks) and the exponents of the chunk's B rows, then the first two B tiles
            tc::mbar_expect_tx(&barA, tc::kDigits * kTcSlA + kTcM * 4 + nt * kTcN * 4);
            for (int h = 0; h < 2; ++h) {
                const unsigned char* rec = blocks + (size_t)(2 * I + h) * kTcRec;
                for (int q = 0; q < tc::kDigits; ++q)
                    tc::bulk_g2s(sA + q * kTcSlA + h * kTcSlice, rec + q * kTcSlice, kTcSlice, &barA);
                tc::bulk_g2s(sAe + kTcBlk * h, rec + tc::kDigits * kTcSlice, kTcBlk * 4, &barA);
            }
            for (int n = 0; n < nt; ++n) {
                const int J = J0 + n;
                tc::bulk_g2s(sBe + n * kTcN, blocks + (size_t)(J >> 1) * kTcRec + tc::kDigits * kTcSlice + (J & 1) * kTcN * 4,
                             kTcN * 4, &barA);
            }
            int loads[2] = {0, 0}, commits[2] = {0, 0};  // uses of each buffer's barriers
            auto load_b = [&](int n) {  // B digits of tile n into buffer n & 1
                const int J = J0 + n, b = n & 1;
                ++loads[b];
                const unsigned char* rec = blocks + (size_t)(J >> 1) * kTcRec + (J & 1) * kTcSlB;
                tc::mbar_expect_tx(&barB[b], tc::kDigits * kTcSlB);
                for (int q = 0; q < tc::kDigits; ++q)
                    tc::bulk_g2s(sB + ((size_t)b * tc::kDigits + q) * kTcSlB, rec + q * kTcSlice, kTcSlB, &barB[b]);
            };
            load_b(0);
            if (nt > 1) load_b(1);
            bool ok = tc::mbar_wait(&barA, 0, ctl, budget);
            const uint32_t id = tc::idesc_bf16_f32(kTcM, kTcN), a0 = tc::smem(sA);
            for (int n = 0; n < nt && ok; ++n) {
                const int b = n & 1;
                const unsigned ph = (n >> 1) & 1;
                ok = tc::mbar_wait(&barB[b], ph, ctl, budget);
                if (ok && n >= 2) ok = tc::mbar_wait(&barE[b], ph ^ 1, ctl, budget);  // tile n-2 read out
                if (!ok) break;
                tc::fence_after();
                const uint32_t b0 = tc::smem(sB + (size_t)b * tc::kDigits * kTcSlB), d0 = tmem + (uint32_t)b * tc::kDigits * kTcN;
                for (int k = 2; k <= 9; ++k) {
                    uint32_t acc = 0;
                    for (int p = max(1, k - tc::kDigits); p <= min(tc::kDigits, k - 1); ++p) {
                        const int q = k - p;
                        for (int ks = 0; ks < kFb / 16; ++ks) {
                            const uint64_t da = tc::desc(a0 + (p - 1) * kTcSlA + ks * 256, 128, kFb * 16);
                            const uint64_t db = tc::desc(b0 + (q - 1) * kTcSlB + ks * 256, 128, kFb * 16);
                            tc::mma_bf16(d0 + (uint32_t)(k - 2) * kTcN, da, db, id, acc);
                            acc = 1;
                        }
                    }
                }
                tc::mma_commit(&barM[b]);
                ++commits[b];
                if (n + 2 < nt) {  // buffer b again for tile n + 2 once these MMAs have read it
                    ok = tc::mbar_wait(&barM[b], ph, ctl, budget);
                    if (ok) load_b(n + 2);
                }
            }
            // nothing of ours left in flight: the last phase of every barrier this thread armed
            // completes (a barrier's earlier phases completed before its later ones were armed)
            tc::mbar_drain(&barA, 0, budget);
            for (int b = 0; b < 2; ++b) {
                if (loads[b]) tc::mbar_drain(&barB[b], (loads[b] - 1) & 1, budget);
                if (commits[b]) tc::mbar_drain(&barM[b], (commits[b] - 1) & 1, budget);
            }
        }
    } else {
        // epilogue: row R of the tile, columns c0 .. c0+15 of each 32-column tile
        const int R = 32 * (warp & 3) + lane, c0 = 16 * (warp >> 2), row = r0 + I * kTcM + R;
        bool ok = tc::mbar_wait(&barA, 0, ctl, budget);
        const int ei = ok ? sAe[R] : tc::kExpZero;
        const bool live = row < m && ei != tc::kExpZero;
        const double* crow = F + (size_t)(live ? row : 0);
        for (int n = 0; n < nt; ++n) {
            const int b = n & 1, colb = r0 + (J0 + n) * kTcN + c0;
            double cv[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) cv[j] = live && colb + j <= row ? crow[(size_t)(colb + j) * m] : 0.0;
            if (ok) ok = tc::mbar_wait(&barM[b], (n >> 1) & 1, ctl, budget);
            tc::fence_after();
            long long th[16], tl[16];
#pragma unroll
            for (int j = 0; j < 16; ++j) th[j] = tl[j] = 0;
#pragma unroll
            for (int half = 0; half < 2; ++half) {
                uint32_t v[4][16];
#pragma unroll
                for (int u = 0; u < 4; ++u)
                    tc::tmem_ld16_async(tmem + ((uint32_t)(32 * (warp & 3)) << 16) + (uint32_t)b * tc::kDigits * kTcN +
                                            (uint32_t)(4 * half + u) * kTcN + c0,
                                        v[u]);
                tc::tmem_wait_ld();
#pragma unroll
                for (int u = 0; u < 4; ++u) tc::tmem_regs_after_wait(v[u]);
#pragma unroll
                for (int u = 0; u < 4; ++u)
#pragma unroll
                    for (int j = 0; j < 16; ++j) {
                        const long long a = (long long)__float2int_rn(__uint_as_float(v[u][j]));
                        if (half == 0) th[j] += a * (1ll << (7 * (3 - u)));  // diagonal k = 2 + u
                        else tl[j] += a * (1ll << (7 * (3 - u)));            // diagonal k = 6 + u
                    }
            }
            tc::fence_before();
            tc::mbar_arrive(&barE[b]);  // this thread is done with TMEM set b
            if (ok && live) {
#pragma unroll
                for (int j = 0; j < 16; ++j) {
                    const int col = colb + j, ej = sBe[n * kTcN + c0 + j];
                    if (col > row || ej == tc::kExpZero) continue;
                    // sum_k acc_k 2^(-7k) = th 2^-35 + tl 2^-63, each part exact in FP64
                    double v = cv[j];
                    if (tl[j]) v -= fr_exact(tl[j], ei + ej - 63);
                    if (th[j]) v -= fr_exact(th[j], ei + ej - 35);
                    F[(size_t)row + (size_t)col * m] = v;
                }
            }
        }
    }
    tc::fence_before();
    __syncthreads();
    if (warp == 0) tc::tmem_dealloc(tmem, 2 * tc::kDigits * kTcN);
}

// U's rows of the listed fronts: one CTA per pivot, row f0 + k (k < w) holds columns S_t[k:]
// (rows = the fronts' row sets, front t's at rows + soff[t]) with values F[k:, k].
__global__ void k_fr_copy_rows(const double* __restrict__ arena, FrontTab ft, const int* __restrict__ list,
                               const int* __restrict__ prefix, int nlist, const int* __restrict__ rows,
                               const int64_t* __restrict__ soff, const int64_t* __restrict__ rp,
                               int* __restrict__ ucol, double* __restrict__ uval) {
    const int f = fr_item(prefix, nlist, blockIdx.x), t = list[f], k = blockIdx.x - prefix[f];
    const double* F = arena + ft.foff[t];
    const int* S = rows + soff[t];
    const int m = ft.fm[t];
    const int64_t base = rp[ft.fstart[t] + k];
    for (int r = k + threadIdx.x; r < m; r += blockDim.x) {
        ucol[base + (r - k)] = S[r];
        uval[base + (r - k)] = F[(size_t)r + (size_t)k * m];
    }
}

// U lives on the device (the factor owns it); the host copies are made when first asked for.
struct Factor {
    int n = 0, device = 0;
    std::vector<int64_t> rp;
    std::vector<int> snodes;
    int* d_rp32 = nullptr;  // int32 row pointer, when nnz < 2^31 (what sptrsv_analyse_device takes)
    int* d_col = nullptr;
    double* d_val = nullptr;
    double symbolic_s = 0.0, numeric_s = 0.0;  // host wall time of the two steps
    ~Factor() {
        if (d_rp32 || d_col || d_val) {
            int cur = 0;
            cudaGetDevice(&cur);
            cudaSetDevice(device);
            cudaFree(d_rp32);
            cudaFree(d_col);
            cudaFree(d_val);
            cudaSetDevice(cur);
        }
    }
};

}  // namespace sptrsv

using namespace sptrsv;

extern "C" int sptrsv_factor_multifrontal(int device, int n, const int64_t* a_rp, const int* a_col,
                                          const double* a_val, int nf, const int* front_start,
                                          const int* front_parent, int max_width, void** out) {
    if (!out) return SPTRSV_ERR_INVALID_ARG;
    *out = nullptr;
    if (n <= 0 || nf <= 0 || !a_rp || !a_col || !a_val || !front_start || !front_parent || max_width <= 0)
        return SPTRSV_ERR_INVALID_ARG;
    if (front_start[0] != 0 || front_start[nf] != n) return SPTRSV_ERR_INVALID_ARG;
    for (int t = 0; t < nf; ++t) {
        if (front_start[t + 1] <= front_start[t]) return SPTRSV_ERR_INVALID_ARG;
        const int p = front_parent[t];
        if (p != -1 && (p <= t || p >= nf)) return SPTRSV_ERR_INVALID_ARG;  // a postorder: parents come later
    }
    if (a_rp[0] != 0) return SPTRSV_ERR_ROW_PTR;
    for (int i = 0; i < n; ++i)
        if (a_rp[i + 1] < a_rp[i]) return SPTRSV_ERR_ROW_PTR;
    const int64_t annz = a_rp[n];
    for (int64_t e = 0; e < annz; ++e)
        if (a_col[e] < 0 || a_col[e] >= n) return SPTRSV_ERR_COL_RANGE;
    // ---- symbolic: row sets, index maps, U's pattern, supernodes
    const auto t_begin = std::chrono::steady_clock::now();
    std::vector<std::vector<int>> children(nf), S(nf);
    for (int t = 0; t < nf; ++t)
        if (front_parent[t] >= 0) children[front_parent[t]].push_back(t);
    std::vector<int64_t> a_idx_off(nf + 1, 0), map_start(nf, 0);
    std::vector<int64_t> a_idx;
    std::vector<double> a_v;
    a_idx.reserve((size_t)(annz / 2 + n));
    a_v.reserve((size_t)(annz / 2 + n));
    std::vector<int> maps;
    std::vector<int> mark(n, -1), posmap(n, 0);  // posmap: a row's place in the current front
    std::vector<int> below, merged;
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], f1 = front_start[t + 1];
        // rows below the pivots: A's (few, sorted here), merged with each child's update rows
        // (already sorted), duplicates dropped
        below.clear();
        for (int p = f0; p < f1; ++p)
            for (int64_t e = a_rp[p]; e < a_rp[p + 1]; ++e) {
                const int q = a_col[e];
                if (q >= f1 && mark[q] != t) {
                    mark[q] = t;
                    below.push_back(q);
                }
            }
        std::sort(below.begin(), below.end());
        for (int c : children[t]) {
            const int wc = front_start[c + 1] - front_start[c];
            const int* u = S[c].data() + wc;
            const int* ue = S[c].data() + S[c].size();
            if (u < ue && *u < f0) return SPTRSV_ERR_INVALID_ARG;  // an update row no ancestor pivots
            while (u < ue && *u < f1) ++u;                          // the parent's own pivots
            merged.clear();
            size_t k = 0;
            while (k < below.size() || u < ue) {
                int q;
                if (u == ue || (k < below.size() && below[k] < *u)) q = below[k++];
                else if (k < below.size() && below[k] == *u) q = below[k++], ++u;
                else q = *u++;
                merged.push_back(q);
            }
            below.swap(merged);
        }
        std::vector<int>& St = S[t];
        St.reserve((size_t)(f1 - f0) + below.size());
        for (int p = f0; p < f1; ++p) St.push_back(p);
        St.insert(St.end(), below.begin(), below.end());
        const int m = (int)St.size();
        if (front_parent[t] < 0 && m != f1 - f0) return SPTRSV_ERR_INVALID_ARG;  // an update nobody takes
        for (size_t k = 0; k < below.size(); ++k) posmap[below[k]] = (f1 - f0) + (int)k;
        auto pos = [&](int q) -> int { return q < f1 ? q - f0 : posmap[q]; };
        // A's lower-triangle entries of the pivot columns
        for (int p = f0; p < f1; ++p)
            for (int64_t e = a_rp[p]; e < a_rp[p + 1]; ++e) {
                const int q = a_col[e];
                if (q < p) continue;
                a_idx.push_back((int64_t)pos(q) + (int64_t)(p - f0) * m);
                a_v.push_back(a_val[e]);
            }
        a_idx_off[t + 1] = (int64_t)a_idx.size();
        // the children's update rows within this front
        for (int c : children[t]) {
            const int wc = front_start[c + 1] - front_start[c];
            map_start[c] = (int64_t)maps.size();
            for (size_t k = wc; k < S[c].size(); ++k) maps.push_back(pos(S[c][k]));
        }
    }
    Factor* fct = new Factor;
    fct->n = n;
    fct->rp.assign(n + 1, 0);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], w = front_start[t + 1] - f0, m = (int)S[t].size();
        for (int k = 0; k < w; ++k) fct->rp[f0 + k + 1] = m - k;
    }
    for (int i = 0; i < n; ++i) fct->rp[i + 1] += fct->rp[i];
    fct->device = device;
    fct->snodes.push_back(0);
    for (int t = 0; t < nf; ++t) {
        const int f0 = front_start[t], f1 = front_start[t + 1], w = f1 - f0;
        const int pieces = (w + max_width - 1) / max_width, step = (w + pieces - 1) / pieces;
        for (int a = f0; a < f1; a += step) fct->snodes.push_back(std::min(f1, a + step));
    }
    // ---- schedule: levels by height, one arena region per level, the launches' work lists
    std::vector<int> height(nf, 0), fm(nf);
    for (int t = 0; t < nf; ++t) {
        fm[t] = (int)S[t].size();
        if (front_parent[t] >= 0) height[front_parent[t]] = std::max(height[front_parent[t]], height[t] + 1);
    }
    const int H = *std::max_element(height.begin(), height.end()) + 1;
    std::vector<std::vector<int>> level(H);
    for (int t = 0; t < nf; ++t) level[height[t]].push_back(t);
    // a level's region lives from its own step to its parents' extend-add; first fit over the
    // regions still live when the level starts
    struct Region {
        int64_t off, size;
        int last;
    };
    std::vector<Region> live;  // by offset
    std::vector<int64_t> foff(nf), lvl_off(H), lvl_size(H);
    int64_t arena_size = 0;
    for (int h = 0; h < H; ++h) {
        int64_t size = 0;
        int last = h;
        for (int t : level[h]) {
            foff[t] = size;
            size += ((int64_t)fm[t] * fm[t] + 31) / 32 * 32;  // 256-byte aligned fronts
            if (front_parent[t] >= 0) last = std::max(last, height[front_parent[t]]);
        }
        live.erase(std::remove_if(live.begin(), live.end(), [&](const Region& r) { return r.last < h; }), live.end());
        int64_t at = 0;
        size_t k = 0;
        for (; k < live.size() && live[k].off - at < size; ++k) at = live[k].off + live[k].size;
        live.insert(live.begin() + k, Region{at, size, last});
        lvl_off[h] = at;
        lvl_size[h] = size;
        arena_size = std::max(arena_size, at + size);
        for (int t : level[h]) foff[t] += at;
    }
    std::vector<int> rows;  // every front's row set, U's column indices
    std::vector<int64_t> soff(nf);
    for (int t = 0; t < nf; ++t) {
        soff[t] = (int64_t)rows.size();
        rows.insert(rows.end(), S[t].begin(), S[t].end());
    }
    enum { kScatter, kExtend, kPotrf, kTrsm, kSyrk, kSplit, kSyrkTc, kCopy };
    struct Launch {
        int kind, k0, nlist, total;  // total: CTAs (kExtend: CTAs per child)
        int64_t list;                // offset of the list in sched; the CTA prefix (nlist + 1) follows it
        int64_t aux;                 // kSyrkTc: offset of the matching kSplit launch's list
    };
    // the trailing updates of fronts with at least kTcMinRest rows below the panel go to the tensor
    // cores unless SPTRSV_FACTOR_UPDATE=fp64
    const char* upd_env = getenv("SPTRSV_FACTOR_UPDATE");
    const bool use_tc = !(upd_env && std::strcmp(upd_env, "fp64") == 0);
    int64_t tc_blocks_max = 0;
    std::vector<int> sched;
    std::vector<std::vector<Launch>> launches(H);
    auto add = [&](int h, int kind, int k0, const std::vector<int>& lst, const std::vector<int>& cnt, int total) {
        if (lst.empty()) return;
        Launch L{kind, k0, (int)lst.size(), total, (int64_t)sched.size(), 0};
        sched.insert(sched.end(), lst.begin(), lst.end());
        if (!cnt.empty()) {
            int acc = 0;
            for (int c : cnt) {
                sched.push_back(acc);
                acc += c;
            }
            sched.push_back(acc);
            L.total = acc;
        }
        launches[h].push_back(L);
    };
    for (int h = 0; h < H; ++h) {
        add(h, kScatter, 0, level[h], {}, (int)level[h].size());
        // extend-add: the r-th children of the level's fronts in one launch, r = 0, 1, ...
        for (size_t r = 0;; ++r) {
            std::vector<int> kids;
            long long most = 0;
            bool any = false;
            for (int t : level[h]) {
                if (r >= children[t].size()) continue;
                any = true;
                const int c = children[t][r], nu = fm[c] - (front_start[c + 1] - front_start[c]);
                if (nu <= 0) continue;
                kids.push_back(c);
                most = std::max(most, (long long)nu * nu);
            }
            if (!any) break;
            const int gx = (int)std::min<long long>(1024, (most + 255) / 256);
            for (size_t a = 0; a < kids.size(); a += 65535)
                add(h, kExtend, 0, std::vector<int>(kids.begin() + a, kids.begin() + std::min(kids.size(), a + 65535)),
                    {}, gx);
        }
        int panels = 0;
        for (int t : level[h]) panels = std::max(panels, (front_start[t + 1] - front_start[t] + kFb - 1) / kFb);
        for (int p = 0; p < panels; ++p) {
            const int k0 = p * kFb;
            std::vector<int> fac, upd, n_trsm, upd64, n_syrk, updtc, n_split, n_tc;
            for (int t : level[h]) {
                const int w = front_start[t + 1] - front_start[t];
                if (w <= k0) continue;
                fac.push_back(t);
                const int r0 = k0 + std::min(kFb, w - k0), rest = fm[t] - r0;
                if (rest <= 0) continue;
                upd.push_back(t);
                n_trsm.push_back((rest + kTrsmRows - 1) / kTrsmRows);
                if (use_tc && rest >= kTcMinRest) {
                    const int nI = (rest + kTcM - 1) / kTcM, nJ = (rest + kTcN - 1) / kTcN;
                    const int nC = (nJ + kTcChunk - 1) / kTcChunk;
                    int tiles = 0;  // CTAs
                    for (int i = 0; i < nI; ++i) tiles += tc_ctas_of_block(i, nC);
                    updtc.push_back(t);
                    n_split.push_back(2 * nI);
                    n_tc.push_back(tiles);
                } else {
                    const int tiles = (rest + kFb - 1) / kFb;
                    upd64.push_back(t);
                    n_syrk.push_back(tiles * (tiles + 1) / 2);
                }
            }
            add(h, kPotrf, k0, fac, {}, (int)fac.size());
            add(h, kTrsm, k0, upd, n_trsm, 0);
            if (!updtc.empty()) {
                add(h, kSplit, k0, updtc, n_split, 0);
                const int64_t split_list = launches[h].back().list;
                tc_blocks_max = std::max<int64_t>(tc_blocks_max, launches[h].back().total);
                add(h, kSyrkTc, k0, updtc, n_tc, 0);
                launches[h].back().aux = split_list;
            }
            add(h, kSyrk, k0, upd64, n_syrk, 0);
        }
        std::vector<int> widths;
        for (int t : level[h]) widths.push_back(front_start[t + 1] - front_start[t]);
        add(h, kCopy, 0, level[h], widths, 0);
    }
    const auto t_symbolic = std::chrono::steady_clock::now();
    fct->symbolic_s = std::chrono::duration<double>(t_symbolic - t_begin).count();
    // ---- numeric on the GPU: one stream, one arena
    int rc = 0;
    cudaStream_t st = nullptr;
    int *d_sched = nullptr, *d_fstart = nullptr, *d_fm = nullptr, *d_parent = nullptr, *d_maps = nullptr;
    int64_t *d_foff = nullptr, *d_mapstart = nullptr, *d_aidx = nullptr, *d_aoff = nullptr, *d_rp = nullptr,
            *d_soff = nullptr;
    int* d_rows = nullptr;
    double *d_av = nullptr, *d_arena = nullptr;
    const int64_t unnz = fct->rp[n];
    int* d_bad = nullptr;
    unsigned char* d_tcbuf = nullptr;
    Ctl* d_ctl = nullptr;
    auto fail = [&](cudaError_t e, const char* what) {
        if (!rc) rc = set_cuda_error(e, what);
    };
    auto ck = [&](cudaError_t e, const char* what) {
        if (e != cudaSuccess) fail(e, what);
        return rc == 0;
    };
    const size_t syrk_smem = sizeof(double) * 2 * kFb * (kFb + 1);
    do {
        if (!ck(cudaSetDevice(device), "cudaSetDevice")) break;
        if (!ck(cudaStreamCreateWithFlags(&st, cudaStreamNonBlocking), "stream")) break;
        if (!ck(cudaFuncSetAttribute(k_fr_syrk, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)syrk_smem), "attr") ||
            !ck(cudaFuncSetAttribute(k_fr_syrk_tc, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kTcSmem), "attr"))
            break;
        auto up = [&](auto** d, const auto* h, size_t count) {
            using E = std::remove_pointer_t<std::remove_pointer_t<decltype(d)>>;
            if (!ck(cudaMallocAsync((void**)d, sizeof(E) * std::max<size_t>(1, count), st), "alloc")) return false;
            return count == 0 || ck(cudaMemcpyAsync(*d, h, sizeof(E) * count, cudaMemcpyHostToDevice, st), "h2d");
        };
        if (!up(&d_sched, sched.data(), sched.size()) || !up(&d_fstart, front_start, (size_t)nf + 1) ||
            !up(&d_fm, fm.data(), (size_t)nf) || !up(&d_parent, front_parent, (size_t)nf) ||
            !up(&d_maps, maps.data(), maps.size()) || !up(&d_foff, foff.data(), (size_t)nf) ||
            !up(&d_mapstart, map_start.data(), (size_t)nf) || !up(&d_aidx, a_idx.data(), a_idx.size()) ||
            !up(&d_av, a_v.data(), a_v.size()) || !up(&d_aoff, a_idx_off.data(), (size_t)nf + 1) ||
            !up(&d_rp, fct->rp.data(), (size_t)n + 1) ||
            !up(&d_rows, rows.data(), rows.size()) || !up(&d_soff, soff.data(), (size_t)nf))
            break;
        // U's arrays outlive the call (plain cudaMalloc: the factor frees them, on any stream)
        if (!ck(cudaMalloc((void**)&fct->d_col, sizeof(int) * std::max<int64_t>(1, unnz)), "alloc U") ||
            !ck(cudaMalloc((void**)&fct->d_val, sizeof(double) * std::max<int64_t>(1, unnz)), "alloc U"))
            break;
        if (unnz < ((int64_t)1 << 31)) {
            std::vector<int> rp32(fct->rp.begin(), fct->rp.end());
            if (!ck(cudaMalloc((void**)&fct->d_rp32, sizeof(int) * (n + 1)), "alloc U") ||
                !ck(cudaMemcpyAsync(fct->d_rp32, rp32.data(), sizeof(int) * (n + 1), cudaMemcpyHostToDevice, st),
                    "h2d"))
                break;
        }
        if (!ck(cudaMallocAsync((void**)&d_arena, sizeof(double) * std::max<int64_t>(1, arena_size), st), "arena") ||
            !ck(cudaMallocAsync((void**)&d_bad, sizeof(int), st), "alloc") ||
            !ck(cudaMemsetAsync(d_bad, 0, sizeof(int), st), "memset") ||
            !ck(cudaMallocAsync((void**)&d_ctl, sizeof(Ctl), st), "alloc") ||
            !ck(cudaMemsetAsync(d_ctl, 0, sizeof(Ctl), st), "memset"))
            break;
        if (tc_blocks_max > 0 &&
            !ck(cudaMallocAsync((void**)&d_tcbuf, (size_t)tc_blocks_max * kTcRec, st), "digit blocks"))
            break;
        const FrontTab ft{d_fstart, d_fm, d_foff};
        for (int h = 0; h < H && !rc; ++h) {
            if (!ck(cudaMemsetAsync(d_arena + lvl_off[h], 0, sizeof(double) * lvl_size[h], st), "memset")) break;
            for (const Launch& L : launches[h]) {
                const int* lst = d_sched + L.list;
                const int* pre = lst + L.nlist;
                switch (L.kind) {
                    case kScatter:
                        k_fr_scatter<<<L.nlist, 256, 0, st>>>(d_arena, ft, lst, d_aoff, d_aidx, d_av);
                        break;
                    case kExtend:
                        k_fr_extend_add<<<dim3(L.total, L.nlist), 256, 0, st>>>(d_arena, ft, lst, d_parent, d_maps,
                                                                                 d_mapstart);
                        break;
                    case kPotrf: k_fr_potrf<<<L.nlist, 256, 0, st>>>(d_arena, ft, lst, L.k0, d_bad); break;
                    case kTrsm:
                        k_fr_trsm<<<L.total, kTrsmRows * 8, 0, st>>>(d_arena, ft, lst, pre, L.nlist, L.k0);
                        break;
                    case kSyrk:
                        k_fr_syrk<<<L.total, 256, syrk_smem, st>>>(d_arena, ft, lst, pre, L.nlist, L.k0);
                        break;
                    case kSplit:
                        k_fr_split<<<L.total, 256, 0, st>>>(d_arena, ft, lst, pre, L.nlist, L.k0, d_tcbuf);
                        break;
                    case kSyrkTc:
                        k_fr_syrk_tc<<<L.total, 32 * (kTcEpiWarps + 1), kTcSmem, st>>>(d_arena, ft, lst, pre, L.nlist,
                                                                     d_sched + L.aux + L.nlist, L.k0, d_tcbuf, d_ctl,
                                                                     kDefaultBudgetNs);
                        break;
                    default:
                        k_fr_copy_rows<<<L.total, 256, 0, st>>>(d_arena, ft, lst, pre, L.nlist, d_rows, d_soff, d_rp,
                                                                fct->d_col, fct->d_val);
                        break;
                }
            }
            ck(cudaGetLastError(), "front kernels");
        }
        if (rc) break;
        int bad = 0, status = 0;
        if (!ck(cudaMemcpyAsync(&bad, d_bad, sizeof(int), cudaMemcpyDeviceToHost, st), "d2h") ||
            !ck(cudaMemcpyAsync(&status, &d_ctl->status, sizeof(int), cudaMemcpyDeviceToHost, st), "d2h") ||
            !ck(cudaStreamSynchronize(st), "sync"))
            break;
        if (status) rc = status;              // a bounded wait of the tensor-core update gave up
        else if (bad) rc = SPTRSV_ERR_ZERO_PIVOT;  // not positive definite in this order
    } while (false);
    if (st) {
        for (void* p : {(void*)d_sched, (void*)d_fstart, (void*)d_fm, (void*)d_parent, (void*)d_maps, (void*)d_foff,
                        (void*)d_mapstart, (void*)d_aidx, (void*)d_av, (void*)d_aoff, (void*)d_rp, (void*)d_rows,
                        (void*)d_soff,
                        (void*)d_arena, (void*)d_bad, (void*)d_tcbuf, (void*)d_ctl})
            if (p) cudaFreeAsync(p, st);
        cudaStreamSynchronize(st);
        cudaStreamDestroy(st);
    }
    if (rc) {
        delete fct;
        return rc;
    }
    fct->numeric_s = std::chrono::duration<double>(std::chrono::steady_clock::now() - t_symbolic).count();
    *out = fct;
    return 0;
}

extern "C" int sptrsv_factor_info(void* f, int* n, int64_t* nnz, int* nsn) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (n) *n = F->n;
    if (nnz) *nnz = F->rp[F->n];
    if (nsn) *nsn = (int)F->snodes.size() - 1;
    return 0;
}

extern "C" int sptrsv_factor_copy(void* f, int64_t* row_ptr, int* col, double* val, int* supernodes) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (row_ptr) std::memcpy(row_ptr, F->rp.data(), sizeof(int64_t) * F->rp.size());
    if (supernodes) std::memcpy(supernodes, F->snodes.data(), sizeof(int) * F->snodes.size());
    const int64_t nnz = F->rp[F->n];
    if (!col && !val) return 0;
    int cur = 0;
    CUDA_TRY(cudaGetDevice(&cur));
    CUDA_TRY(cudaSetDevice(F->device));
    cudaError_t e = cudaSuccess;
    if (col) e = cudaMemcpy(col, F->d_col, sizeof(int) * nnz, cudaMemcpyDeviceToHost);
    if (val && e == cudaSuccess) e = cudaMemcpy(val, F->d_val, sizeof(double) * nnz, cudaMemcpyDeviceToHost);
    cudaSetDevice(cur);
    return e == cudaSuccess ? 0 : set_cuda_error(e, "factor copy");
}

extern "C" int sptrsv_factor_device(void* f, const int** d_row_ptr, const int** d_col, const double** d_val) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (!F->d_rp32) return SPTRSV_ERR_TOO_LARGE;  // 2^31 entries or more: no int32 row pointer
    if (d_row_ptr) *d_row_ptr = F->d_rp32;
    if (d_col) *d_col = F->d_col;
    if (d_val) *d_val = F->d_val;
    return 0;
}

extern "C" int sptrsv_factor_times(void* f, double* symbolic_s, double* numeric_s) {
    if (!f) return SPTRSV_ERR_INVALID_ARG;
    const Factor* F = static_cast<const Factor*>(f);
    if (symbolic_s) *symbolic_s = F->symbolic_s;
    if (numeric_s) *numeric_s = F->numeric_s;
    return 0;
}

extern "C" void sptrsv_factor_free(void* f) { delete static_cast<Factor*>(f); }
