// neighbor.cu -- FastNeighborList on the GPU.
//
// Reproduces core_create_space_partitioning + core_build_neighbor_lists
// (fortran/Core.f90:8130-8280, fortran/Geometry.f90:597-924) bit for bit,
// entry order included:
//
//  1. nb_assign: per atom, wrapped_coordinates and find_subcell_for_atom
//     (the same FP64 operations in the same order, no fused multiply-add).
//  2. A stable, atomics-free LSD radix sort of atoms by subcell id: the
//     subcell contents come out in ascending atom index, as the serial
//     insertion loop leaves them.
//  3. nb_scan<COUNT/FILL>: one warp per atom walks its 27 stencil subcells.
//     In the reference, atom a's list receives entries from the sweeps of
//     lower-index atoms b (ordered by b, then by b's stencil slot) followed by
//     the entries of a's own sweep (stencil order, subcell order; a periodic
//     self image adds (a, o) then (a, -o)).  Because a is found in b's slot s
//     exactly when b is in a's slot 26 - s with the opposite subcell offset,
//     and the separation seen from b is the exact negation of the one seen
//     from a, every entry can be produced from a's own stencil.  Entries of the
//     first kind carry the sort key (b, 26 - s); atoms that the reference puts
//     into an out-of-range subcell of a periodic axis are swept but never
//     found by others, and are handled by an explicit pass.
//  4. nb_sort_g0: per atom, the lower-index entries are placed by rank of key.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace pg {

namespace {

struct Split {
    int sp[3];
    int nx, ny, nz;
};

// wrapped_coordinates + find_subcell_for_atom (Geometry.f90:597-619, 884-924)
__global__ void nb_assign(int n, const double* __restrict__ pos, CellK C, Split S, int* __restrict__ cell_of,
                          int* __restrict__ key, int* __restrict__ val, int* __restrict__ wrap,
                          int* __restrict__ invisible, float4* __restrict__ posf) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    double p[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    posf[i] = make_float4((float)p[0], (float)p[1], (float)p[2], 0.0f);  // the stencil scan's FP32 screen
    double rel[3];
    for (int r = 0; r < 3; ++r)
        rel[r] = __dadd_rn(__dadd_rn(__dmul_rn(C.ic[r][0], p[0]), __dmul_rn(C.ic[r][1], p[1])),
                           __dmul_rn(C.ic[r][2], p[2]));
    int off[3];
    for (int a = 0; a < 3; ++a) {
        off[a] = 0;
        if (C.pbc[a]) {
            off[a] = -(int)floor(rel[a]);
            rel[a] = __dadd_rn(rel[a], (double)off[a]);
        }
    }
    double w[3];
    for (int r = 0; r < 3; ++r)
        w[r] = __dadd_rn(__dadd_rn(__dmul_rn(C.vc[r][0], rel[0]), __dmul_rn(C.vc[r][1], rel[1])),
                         __dmul_rn(C.vc[r][2], rel[2]));
    double f[3];
    for (int r = 0; r < 3; ++r)
        f[r] = __dadd_rn(__dadd_rn(__dmul_rn(C.ic[r][0], w[0]), __dmul_rn(C.ic[r][1], w[1])),
                         __dmul_rn(C.ic[r][2], w[2]));
    int idx[3];
    int inv = 0;
    for (int a = 0; a < 3; ++a) {
        double x = floor(__dmul_rn(f[a], (double)S.sp[a]));
        x = fmin(fmax(x, -1.0e9), 1.0e9);
        int k = (int)x;
        if (C.pbc[a]) {
            idx[a] = k % S.sp[a] + 1;  // Fortran mod: sign of the dividend
            if (idx[a] < 1 || idx[a] > S.sp[a]) inv = 1;
        } else {
            idx[a] = min(S.sp[a] + 1, max(0, k + 1));
        }
    }
    // index 0 of a periodic axis is possible only by rounding; lower values are not
    for (int a = 0; a < 3; ++a) idx[a] = max(idx[a], 0);
    int c = (idx[2] * S.ny + idx[1]) * S.nx + idx[0];
    cell_of[3 * i] = idx[0];
    cell_of[3 * i + 1] = idx[1];
    cell_of[3 * i + 2] = idx[2];
    key[i] = c;
    val[i] = i;
    wrap[3 * i] = off[0];
    wrap[3 * i + 1] = off[1];
    wrap[3 * i + 2] = off[2];
    invisible[i] = inv;
}

// ---- stable LSD radix sort (8-bit digits), atomics-free -------------------
constexpr int RS_THREADS = 256;
constexpr int RS_ROUNDS = 4;
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;

__global__ void radix_hist(int n, const int* __restrict__ keys, int shift, int nblocks, int* __restrict__ hist) {
    __shared__ int whist[RS_THREADS / 32][256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    for (int d = lane; d < 256; d += 32) whist[w][d] = 0;
    __syncwarp();
    const int tile0 = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        int e = tile0 + r * RS_THREADS + tid;
        int d = e < n ? (keys[e] >> shift) & 255 : -1;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        if (d >= 0 && lane == leader) whist[w][d] += __popc(peers);
        __syncwarp();
    }
    __syncthreads();
    int sum = 0;
    for (int ww = 0; ww < RS_THREADS / 32; ++ww) sum += whist[ww][tid];
    hist[tid * nblocks + blockIdx.x] = sum;
}

__global__ void radix_scatter(int n, const int* __restrict__ keys, const int* __restrict__ vals, int shift,
                              int nblocks, const int* __restrict__ offs, int* __restrict__ okeys,
                              int* __restrict__ ovals) {
    __shared__ int whist[RS_THREADS / 32][256];
    __shared__ int run[256];
    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    run[tid] = offs[tid * nblocks + blockIdx.x];
    const int tile0 = blockIdx.x * RS_TILE;
    for (int r = 0; r < RS_ROUNDS; ++r) {
        for (int ww = 0; ww < RS_THREADS / 32; ++ww) whist[ww][tid] = 0;
        __syncthreads();
        int e = tile0 + r * RS_THREADS + tid;
        int k = e < n ? keys[e] : 0;
        int d = e < n ? (k >> shift) & 255 : -1;
        unsigned peers = __match_any_sync(0xffffffffu, d);
        int leader = __ffs(peers) - 1;
        if (d >= 0 && lane == leader) whist[w][d] = __popc(peers);
        __syncthreads();
        if (d >= 0) {
            int rank = run[d] + __popc(peers & ((1u << lane) - 1u));
            for (int ww = 0; ww < w; ++ww) rank += whist[ww][d];
            okeys[rank] = k;
            ovals[rank] = vals[e];
        }
        __syncthreads();
        int add = 0;
        for (int ww = 0; ww < RS_THREADS / 32; ++ww) add += whist[ww][tid];
        run[tid] += add;
        __syncthreads();
    }
}

__global__ void cell_starts(int n, int ncell, const int* __restrict__ skeys, int* __restrict__ start) {
    int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p > n) return;
    int lo = p == 0 ? -1 : skeys[p - 1];
    int hi = p == n ? ncell : skeys[p];
    for (int c = lo + 1; c <= hi && c <= ncell; ++c) start[c] = p;
}

// Single-block exclusive scan (build-time sizes): out[0..n-1] the exclusive
// prefix sums of in (of its squares with square), out[n] and *total (may be
// null) the sum.  The block walks the input in tiles of 32 x blockDim.x
// elements: warp w takes 32 rows of 32 consecutive elements (coalesced loads
// and stores), scans each row with shuffles and carries its running sum, then
// the warps' sums are scanned and the tile's sum carried.  Integer sums: the
// result does not depend on the order.
template <typename T, typename U>
__global__ void __launch_bounds__(1024) scan_single_block(const T* __restrict__ in, U* __restrict__ out, int n,
                                                           U* __restrict__ total, int square) {
    constexpr int ROWS = 32;
    __shared__ U wsum[32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5, nw = blockDim.x >> 5;
    U carry = 0;
    for (long long base = 0; base < n; base += (long long)blockDim.x * ROWS) {
        const long long chunk = base + (long long)w * 32 * ROWS;
        U v[ROWS];
        U run = 0;
#pragma unroll
        for (int k = 0; k < ROWS; ++k) {
            const long long i = chunk + 32 * k + lane;
            U x = i < n ? (U)in[i] : (U)0;
            if (square) x *= x;
            U incl = x;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const U y = __shfl_up_sync(0xffffffffu, incl, o);
                if (lane >= o) incl += y;
            }
            v[k] = run + incl - x;
            run += __shfl_sync(0xffffffffu, incl, 31);
        }
        if (lane == 0) wsum[w] = run;
        __syncthreads();
        if (w == 0) {
            U x = lane < nw ? wsum[lane] : (U)0;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const U y = __shfl_up_sync(0xffffffffu, x, o);
                if (lane >= o) x += y;
            }
            if (lane < nw) wsum[lane] = x;  // inclusive over warps
        }
        __syncthreads();
        const U pre = carry + (w > 0 ? wsum[w - 1] : (U)0);
#pragma unroll
        for (int k = 0; k < ROWS; ++k) {
            const long long i = chunk + 32 * k + lane;
            if (i < n) out[i] = pre + v[k];
        }
        carry += wsum[nw - 1];
        __syncthreads();  // wsum is rewritten by the next tile
    }
    if (t == 0) {
        out[n] = carry;
        if (total) *total = carry;
    }
}

// The same exclusive scan (out[0..n-1], out[n] = total, *total) over many
// blocks in one pass (decoupled look-back): each block takes the next tile of
// LB_TILE values in order from a ticket, sums it, publishes the tile's sum
// (flag 1), then its first warp reads the records of the 32 tiles before it at
// once and adds their sums back to the nearest one that carries its inclusive
// prefix (flag 2), a window further back at a time; the block publishes its
// own inclusive prefix and writes its part.  A tile only waits on tiles with
// smaller tickets, whose blocks are already running, so every wait ends; each
// wait is also bounded, and a scan whose wait ran out writes -1 as its total
// (the host checks the totals it reads).  The last block to finish clears the
// records and counters (ctr: ticket, done, failed) for the next scan.  Thread
// t of a tile holds values 8t .. 8t + 7; the sums are of integers, so exact.
constexpr int LB_THREADS = 256, LB_PER = 8, LB_TILE = LB_THREADS * LB_PER;
constexpr unsigned long long LB_AGG = 1ull << 62, LB_INC = 2ull << 62, LB_VAL = (1ull << 32) - 1;
constexpr unsigned LB_POLLS = 1u << 22;

__global__ void __launch_bounds__(LB_THREADS) scan_lookback(const int* __restrict__ in, int* __restrict__ out, int n,
                                                            int* __restrict__ total, unsigned long long* rec,
                                                            unsigned* ctr, int ntiles) {
    __shared__ int s_tile, s_excl, s_last;
    __shared__ int s_wsum[LB_THREADS / 32];
    const int t = threadIdx.x, lane = t & 31, w = t >> 5;
    if (t == 0) s_tile = (int)atomicAdd(&ctr[0], 1u);
    __syncthreads();
    const int tile = s_tile;
    const long long base = (long long)tile * LB_TILE + (long long)t * LB_PER;
    int v[LB_PER];
    int run = 0;
#pragma unroll
    for (int k = 0; k < LB_PER; ++k) {
        const long long i = base + k;
        v[k] = run;
        run += i < n ? in[i] : 0;
    }
    // exclusive prefix of the thread sums over the tile
    int incl = run;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += y;
    }
    if (lane == 31) s_wsum[w] = incl;
    __syncthreads();
    int wpre = 0, agg = 0;
#pragma unroll
    for (int q = 0; q < LB_THREADS / 32; ++q) {
        if (q < w) wpre += s_wsum[q];
        agg += s_wsum[q];
    }
    if (w == 0) {
        int excl = 0;
        bool ok = true;
        if (tile == 0) {
            if (lane == 0) atomicExch(&rec[0], LB_INC | (unsigned)agg);
        } else {
            if (lane == 0) atomicExch(&rec[tile], LB_AGG | (unsigned)agg);
            for (int p = tile - 1;; p -= 32) {
                // lane l reads tile p - l (tiles before the first count as
                // inclusive prefixes of zero)
                const int q = p - lane;
                unsigned long long r = LB_INC;
                if (q >= 0) {
                    for (unsigned it = 0;; ++it) {
                        r = atomicAdd(&rec[q], 0ull);
                        if (r >> 62) break;
                        if (it >= LB_POLLS) break;
                        __nanosleep(64);
                    }
                }
                if (__any_sync(0xffffffffu, (r >> 62) == 0ull)) {
                    ok = false;
                    break;
                }
                const unsigned incs = __ballot_sync(0xffffffffu, (r >> 62) == 2ull);
                const int first = incs ? __ffs(incs) - 1 : 32;
                int c = lane <= first ? (int)(unsigned)(r & LB_VAL) : 0;
#pragma unroll
                for (int o = 16; o > 0; o >>= 1) c += __shfl_xor_sync(0xffffffffu, c, o);
                excl += c;
                if (incs) break;
            }
            if (lane == 0) {
                if (!ok) atomicExch(&ctr[2], 1u);
                atomicExch(&rec[tile], LB_INC | (unsigned)(excl + agg));
            }
        }
        if (lane == 0) s_excl = excl;
    }
    __syncthreads();
    const int excl = s_excl;
    const int pre = excl + wpre + incl - run;
#pragma unroll
    for (int k = 0; k < LB_PER; ++k) {
        const long long i = base + k;
        if (i < n) out[i] = pre + v[k];
    }
    if (tile == ntiles - 1 && t == 0) {
        out[n] = excl + agg;
        if (total) *total = excl + agg;
    }
    // the last block to finish marks a failed scan and clears the records
    __syncthreads();
    if (t == 0) {
        __threadfence();
        s_last = atomicAdd(&ctr[1], 1u) == (unsigned)(ntiles - 1) ? 1 : 0;
    }
    __syncthreads();
    if (s_last) {
        for (int q = t; q < ntiles; q += LB_THREADS) rec[q] = 0ull;
        if (t == 0) {
            __threadfence();
            if (atomicAdd(&ctr[2], 0u)) {
                out[n] = -1;
                if (total) *total = -1;
            }
            ctr[0] = 0u;
            ctr[1] = 0u;
            ctr[2] = 0u;
        }
    }
}

// subcell stencil of divide_cell (Geometry.f90:820-858)
__device__ __forceinline__ bool stencil(const int ci[3], int s, const int sp[3], const int pbc[3], int nb[3],
                                        int noff[3]) {
    const int d[3] = {s % 3 - 1, (s / 3) % 3 - 1, s / 9 - 1};
    bool inc = true;
    for (int a = 0; a < 3; ++a) {
        nb[a] = ci[a] + d[a];
        noff[a] = 0;
        if (pbc[a]) {
            while (nb[a] > sp[a]) {
                nb[a] -= sp[a];
                noff[a] += 1;
            }
            while (nb[a] < 1) {
                nb[a] += sp[a];
                noff[a] -= 1;
            }
        } else if (nb[a] < 0 || nb[a] > sp[a] + 1) {
            inc = false;
            nb[a] = 0;
        }
    }
    return inc;
}

// separation_vector + .o. (Geometry.f90:449-466, Quaternions.f90:475-484)
__device__ __forceinline__ double sep_d2(const CellK& C, const double* ra, const double* rb, const int o[3]) {
    double s[3];
    for (int c = 0; c < 3; ++c) s[c] = __dsub_rn(rb[c], ra[c]);
    // a zero offset adds +-0 to each component, which leaves the squared
    // distance exactly as it is: skipped
    for (int i = 0; i < 3; ++i)
        if (o[i] != 0)
            for (int c = 0; c < 3; ++c) s[c] = __dadd_rn(s[c], __dmul_rn((double)o[i], C.vc[c][i]));
    return __dadd_rn(__dadd_rn(__dmul_rn(s[0], s[0]), __dmul_rn(s[1], s[1])), __dmul_rn(s[2], s[2]));
}

// FP32 screen of the FP64 test sep_d2(...) < cut2, so that the FP64 pipe (a
// small fraction of the FP32 rate on this GPU) sees only the candidates near
// the cutoff: 1 when the FP64 test surely passes, 0 when it surely fails, -1
// when the FP32 value lies within its rounding band (the caller decides in
// FP64).  ra, rb: the positions rounded to FP32; vc: the cell rounded to FP32.
// Each component of the separation is a sum of terms of size at most m (the
// largest |coordinate|, |offset term| or |separation|), so its FP32 error is
// below 8 u m (u = 2^-24), and that of d2 below 28 u m sqrt(d2) + 3 u d2 + 200
// u^2 m^2; the band used is more than twice that (and covers the rounding of
// cut2 to FP32), so a certain verdict is the FP64 one.
__device__ __forceinline__ int screen_d2(const float ra[3], const float4 rb, const int o[3], const float (&vc)[3][3],
                                         float cut2) {
    float s[3] = {rb.x - ra[0], rb.y - ra[1], rb.z - ra[2]};
    float m = fmaxf(fmaxf(fabsf(ra[0]), fabsf(ra[1])), fabsf(ra[2]));
    m = fmaxf(m, fmaxf(fmaxf(fabsf(rb.x), fabsf(rb.y)), fabsf(rb.z)));
    if (o[0] | o[1] | o[2]) {
        const float of[3] = {(float)o[0], (float)o[1], (float)o[2]};
        for (int c = 0; c < 3; ++c) {
            const float t0 = of[0] * vc[c][0], t1 = of[1] * vc[c][1], t2 = of[2] * vc[c][2];
            m = fmaxf(m, fabsf(t0) + fabsf(t1) + fabsf(t2));
            s[c] += (t0 + t1) + t2;
        }
    }
    const float d2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
    const float D = fmaxf(d2, cut2);
    const float rD = sqrtf(D);
    m = fmaxf(m, rD);
    const float tol = 1.1920929e-7f * (32.0f * m * rD + 8.0f * D) + 2.3283064e-10f * m * m;
    if (d2 < cut2 - tol) return 1;
    if (d2 > cut2 + tol) return 0;
    return -1;
}

__device__ __forceinline__ bool lex_positive(const int o[3]) {
    if (o[0] != 0) return o[0] > 0;
    if (o[1] != 0) return o[1] > 0;
    return o[2] > 0;
}

struct ScanArgs {
    int n;
    const double* pos;
    const float4* posf;  // positions rounded to FP32 (screen)
    float vcf[3][3];     // cell rounded to FP32 (screen)
    const double* cut;
    const int* cell_of;
    const int* wrap;
    const int* cstart;
    const int* sorted;
    const int* invisible;
    const int* inv_list;
    const int* n_inv;  // device: atoms in out-of-range periodic subcells
    CellK C;
    Split S;
    // outputs
    int* g0count;
    int* g1count;
    const int* start;    // CSR start (FILL)
    const int* g0start;  // start of the atom's lower-index entries in the key buffer (FILL)
    long long* g0key;
    int4* g0val;
    int* idx;
    int* off;
};

constexpr int SCAN_THREADS = 256;

template <bool FILL>
__global__ void __launch_bounds__(SCAN_THREADS) nb_scan(ScanArgs A) {
    // per warp: the atom's 27 stencil subcells (first sorted slot, candidate
    // prefix, image offset), so that the candidates of all 27 are walked as
    // one stream with every lane busy -- the FP64 distance test dominates
    __shared__ int s_beg[SCAN_THREADS / 32][27], s_pre[SCAN_THREADS / 32][28], s_off[SCAN_THREADS / 32][27][3];
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
    const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= A.n) return;  // whole warps
    const double ra[3] = {A.pos[3 * a], A.pos[3 * a + 1], A.pos[3 * a + 2]};
    const double cut2 = __dmul_rn(A.cut[a], A.cut[a]);
    const float4 pa = A.posf[a];
    const float raf[3] = {pa.x, pa.y, pa.z};
    const float cut2f = (float)cut2;
    const int ci[3] = {A.cell_of[3 * a], A.cell_of[3 * a + 1], A.cell_of[3 * a + 2]};
    const int wa[3] = {A.wrap[3 * a], A.wrap[3 * a + 1], A.wrap[3 * a + 2]};
    const bool visible = A.invisible[a] == 0;
    const int lt = (1u << lane) - 1u;
    int n0 = 0, n1 = 0;
    int base1 = 0, base0 = 0;
    if (FILL) {
        base1 = A.start[a] + A.g0count[a];
        base0 = A.g0start[a];
    }
    int len = 0;
    if (lane < 27) {
        int nb[3], noff[3];
        int beg = 0;
        if (stencil(ci, lane, A.S.sp, A.C.pbc, nb, noff)) {
            const int c = (nb[2] * A.S.ny + nb[1]) * A.S.nx + nb[0];
            beg = A.cstart[c];
            len = A.cstart[c + 1] - beg;
        }
        s_beg[w][lane] = beg;
        for (int q = 0; q < 3; ++q) s_off[w][lane][q] = noff[q];
    }
    int incl = len;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int v = __shfl_up_sync(0xffffffffu, incl, o);
        if (lane >= o) incl += v;
    }
    if (lane == 0) s_pre[w][0] = 0;
    if (lane < 27) s_pre[w][lane + 1] = incl;
    const int total = __shfl_sync(0xffffffffu, incl, 26);
    __syncwarp();
    // candidates in stencil order, then sorted order within a subcell: the
    // order of the reference's loops (Core.f90:8190-8202)
    for (int u0 = 0; u0 < total; u0 += 32) {
        const int u = u0 + lane;
        int b = -1, mult = 0, grp = -1, s = 0;
        int o[3] = {0, 0, 0};
        if (u < total) {
            int lo = 0, hi = 26;  // the last subcell whose prefix is <= u
            while (lo < hi) {
                const int mid = (lo + hi + 1) >> 1;
                if (s_pre[w][mid] <= u) lo = mid;
                else hi = mid - 1;
            }
            s = lo;
            const int noff[3] = {s_off[w][s][0], s_off[w][s][1], s_off[w][s][2]};
            b = A.sorted[s_beg[w][s] + (u - s_pre[w][s])];
            if (b > a) {
                grp = 1;
                mult = 1;
            } else if (b == a) {
                if (lex_positive(noff)) {
                    grp = 1;
                    mult = 2;
                }
            } else if (visible) {
                grp = 0;
                mult = 1;
            }
            if (mult) {
                for (int q = 0; q < 3; ++q) o[q] = noff[q] - wa[q] + A.wrap[3 * b + q];
                const int v = screen_d2(raf, A.posf[b], o, A.vcf, cut2f);
                if (v == 0) {
                    mult = 0;
                } else if (v < 0) {
                    const double rb[3] = {A.pos[3 * b], A.pos[3 * b + 1], A.pos[3 * b + 2]};
                    if (!(sep_d2(A.C, ra, rb, o) < cut2)) mult = 0;
                }
            }
        }
        const unsigned m0 = __ballot_sync(0xffffffffu, mult && grp == 0);
        const unsigned m1 = __ballot_sync(0xffffffffu, mult && grp == 1);
        const unsigned m2 = __ballot_sync(0xffffffffu, mult == 2);
        if (FILL && mult) {
            if (grp == 0) {
                int p = base0 + n0 + __popc(m0 & lt);
                A.g0key[p] = ((long long)b << 5) | (long long)(26 - s);
                A.g0val[p] = make_int4(b, o[0], o[1], o[2]);
            } else {
                int p = base1 + n1 + __popc(m1 & lt) + __popc(m2 & lt);
                A.idx[p] = b;
                A.off[3 * p] = o[0];
                A.off[3 * p + 1] = o[1];
                A.off[3 * p + 2] = o[2];
                if (mult == 2) {
                    A.idx[p + 1] = b;
                    A.off[3 * p + 3] = -o[0];
                    A.off[3 * p + 4] = -o[1];
                    A.off[3 * p + 5] = -o[2];
                }
            }
        }
        n0 += __popc(m0);
        n1 += __popc(m1) + __popc(m2);
    }
    // lower-index atoms in out-of-range subcells of a periodic axis: their
    // sweep can reach a, but a's stencil never reaches them
    const int n_inv = *A.n_inv;
    if (visible && n_inv > 0) {
        for (int q0 = 0; q0 < n_inv; q0 += 32) {
            const int q = q0 + lane;
            int cnt = 0;
            int b = q < n_inv ? A.inv_list[q] : a;
            long long keys[27];
            int4 vals[27];
            if (b < a) {
                const int cb[3] = {A.cell_of[3 * b], A.cell_of[3 * b + 1], A.cell_of[3 * b + 2]};
                const int wb[3] = {A.wrap[3 * b], A.wrap[3 * b + 1], A.wrap[3 * b + 2]};
                const double rb[3] = {A.pos[3 * b], A.pos[3 * b + 1], A.pos[3 * b + 2]};
                for (int s = 0; s < 27; ++s) {
                    int nb[3], noff[3];
                    if (!stencil(cb, s, A.S.sp, A.C.pbc, nb, noff)) continue;
                    if (nb[0] != ci[0] || nb[1] != ci[1] || nb[2] != ci[2]) continue;
                    int o[3];
                    for (int k = 0; k < 3; ++k) o[k] = -noff[k] + wb[k] - wa[k];
                    if (sep_d2(A.C, ra, rb, o) < cut2) {
                        keys[cnt] = ((long long)b << 5) | (long long)s;
                        vals[cnt] = make_int4(b, o[0], o[1], o[2]);
                        ++cnt;
                    }
                }
            }
            // inclusive prefix of cnt over lanes
            int incl = cnt;
            for (int d = 1; d < 32; d <<= 1) {
                int v = __shfl_up_sync(0xffffffffu, incl, d);
                if (lane >= d) incl += v;
            }
            const int excl = incl - cnt;
            const int tot = __shfl_sync(0xffffffffu, incl, 31);
            if (FILL)
                for (int k = 0; k < cnt; ++k) {
                    A.g0key[base0 + n0 + excl + k] = keys[k];
                    A.g0val[base0 + n0 + excl + k] = vals[k];
                }
            n0 += tot;
        }
    }
    if (!FILL && lane == 0) {
        A.g0count[a] = n0;
        A.g1count[a] = n1;
    }
}

__global__ void add_counts(int n, const int* __restrict__ a, const int* __restrict__ b, int* __restrict__ c) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) c[i] = a[i] + b[i];
}

// place the lower-index entries of each atom by the rank of their key
__global__ void nb_sort_g0(int n, const int* __restrict__ g0count, const int* __restrict__ g0start,
                           const int* __restrict__ start, const long long* __restrict__ key,
                           const int4* __restrict__ val, int* __restrict__ idx, int* __restrict__ off) {
    const int lane = threadIdx.x & 31;
    const int a = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    if (a >= n) return;
    const int m = g0count[a], b0 = g0start[a], dst = start[a];
    for (int e = lane; e < m; e += 32) {
        const long long k = key[b0 + e];
        int rank = 0;
        for (int f = 0; f < m; ++f) rank += key[b0 + f] < k;
        const int4 v = val[b0 + e];
        idx[dst + rank] = v.x;
        off[3 * (dst + rank)] = v.y;
        off[3 * (dst + rank) + 1] = v.z;
        off[3 * (dst + rank) + 2] = v.w;
    }
}

__global__ void compact_flags(int n, const int* __restrict__ flag, const int* __restrict__ pos, int* __restrict__ out) {
    int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n && flag[i]) out[pos[i]] = i;
}

// ---- short list for bond-order terms -----------------------------------------
// lanes per atom of the reverse-entry search (short_reverse)
constexpr int ENTRY_LANES = 4;

__device__ __forceinline__ double entry_d2(const CellK& C, const double* __restrict__ pos, int a, int b, const int* o) {
    const double ra[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
    const double rb[3] = {pos[3 * b], pos[3 * b + 1], pos[3 * b + 2]};
    return sep_d2(C, ra, rb, o);
}

__global__ void short_count(int n, const double* __restrict__ pos, CellK C, const int* __restrict__ start,
                            const int* __restrict__ idx, const int* __restrict__ off, double r2,
                            int* __restrict__ cnt) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int c = 0;
    for (int e = start[a]; e < start[a + 1]; ++e)
        if (entry_d2(C, pos, a, idx[e], off + 3 * e) < r2) ++c;
    cnt[a] = c;
}

__global__ void short_fill(int n, const double* __restrict__ pos, CellK C, const int* __restrict__ start,
                           const int* __restrict__ idx, const int* __restrict__ off, double r2,
                           const int* __restrict__ sstart, int* __restrict__ sidx, int* __restrict__ soff) {
    int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    int p = sstart[a];
    for (int e = start[a]; e < start[a + 1]; ++e)
        if (entry_d2(C, pos, a, idx[e], off + 3 * e) < r2) {
            sidx[p] = idx[e];
            soff[3 * p] = off[3 * e];
            soff[3 * p + 1] = off[3 * e + 1];
            soff[3 * p + 2] = off[3 * e + 2];
            ++p;
        }
}

// separation_vector (Geometry.f90:449-466) of every short-list entry, rounded to FP32
__global__ void short_sep0(int n, const double* __restrict__ pos, CellK C, const int* __restrict__ start,
                           const int* __restrict__ idx, const int* __restrict__ off, F4* __restrict__ sep0) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    for (int e = start[a]; e < start[a + 1]; ++e) {
        const int b = idx[e];
        double s[3];
        for (int c = 0; c < 3; ++c) s[c] = __dsub_rn(pos[3 * b + c], pos[3 * a + c]);
        for (int i = 0; i < 3; ++i)
            for (int c = 0; c < 3; ++c) s[c] = __dadd_rn(s[c], __dmul_rn((double)off[3 * e + i], C.vc[c][i]));
        sep0[e] = F4{(float)s[0], (float)s[1], (float)s[2], 0.0f};
    }
}

// partner type of every short-list entry; the entry count is read on the
// device, so that the launch does not depend on it
__global__ void entry_types(const int* __restrict__ m_dev, const int* __restrict__ idx, const int* __restrict__ type,
                            int* __restrict__ out) {
    const int m = *m_dev;
    for (int e = blockIdx.x * blockDim.x + threadIdx.x; e < m; e += gridDim.x * blockDim.x) out[e] = type[idx[e]];
}

__global__ void short_reverse(int n, const int* __restrict__ start, const int* __restrict__ idx,
                              const int* __restrict__ off, int* __restrict__ rev, int* __restrict__ cnt) {
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    const int a = (int)(t / ENTRY_LANES), l = (int)(t % ENTRY_LANES);
    if (a >= n) return;
    if (l == 0) cnt[a] = start[a + 1] - start[a];
    for (int e = start[a] + l; e < start[a + 1]; e += ENTRY_LANES) {
        const int b = idx[e];
        int r = -1;
        for (int f = start[b]; f < start[b + 1]; ++f)
            if (idx[f] == a && off[3 * f] == -off[3 * e] && off[3 * f + 1] == -off[3 * e + 1] &&
                off[3 * f + 2] == -off[3 * e + 2]) {
                r = f;
                break;
            }
        rev[e] = r;
    }
}

// sort keys of the slot order: the atom's short-list count, the atom itself
__global__ void order_keys(int n, const int* __restrict__ cnt, int* __restrict__ keys, int* __restrict__ vals) {
    const int a = blockIdx.x * blockDim.x + threadIdx.x;
    if (a >= n) return;
    keys[a] = min(cnt[a], 65535);
    vals[a] = a;
}

// slot k: atom m = sorted[k], its first short-list entry and its count
__global__ void order_slots(int n, const int* __restrict__ sorted, const int* __restrict__ start,
                            const int* __restrict__ cnt, int* __restrict__ order, int4* __restrict__ slot) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const int m = sorted[k];
    order[k] = m;
    slot[k] = make_int4(m, start[m], cnt[m], 0);
}

__global__ void max_reduce(int n, const int* __restrict__ v, int* __restrict__ out) {
    __shared__ int sm[1024];
    int m = 0;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = max(m, v[i]);
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = max(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

__global__ void min_reduce(int n, const int* __restrict__ v, int* __restrict__ out) {
    __shared__ int sm[1024];
    int m = 0x7fffffff;
    for (int i = threadIdx.x; i < n; i += blockDim.x) m = min(m, v[i]);
    sm[threadIdx.x] = m;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = min(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) *out = sm[0];
}

// ---- all-pairs list for cells narrower than the cutoff --------------------
// The reference hands such systems to ASE's NeighborList (calculator.py:829-848,
// 905-915): both directions, no self pair, atoms i and j are neighbours when
// |r_j + n.cell - r_i| < c_i + c_j (cutoffs include the skin).  Order here:
// partner index, then image offsets in lexicographic order.
template <bool FILL>
__global__ void allpairs_scan(int n, const double* __restrict__ pos, const double* __restrict__ cut, CellK C,
                              int3 nimg, const int* __restrict__ start, int* __restrict__ cnt, int* __restrict__ idx,
                              int* __restrict__ off) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const double ri[3] = {pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]};
    int c = 0;
    const int base = FILL ? start[i] : 0;
    for (int j = 0; j < n; ++j) {
        const double rj[3] = {pos[3 * j], pos[3 * j + 1], pos[3 * j + 2]};
        const double rr = cut[i] + cut[j];
        const double rr2 = rr * rr;
        for (int a = -nimg.x; a <= nimg.x; ++a)
            for (int b = -nimg.y; b <= nimg.y; ++b)
                for (int d = -nimg.z; d <= nimg.z; ++d) {
                    if (j == i && a == 0 && b == 0 && d == 0) continue;
                    const int o[3] = {a, b, d};
                    if (sep_d2(C, ri, rj, o) < rr2) {
                        if (FILL) {
                            idx[base + c] = j;
                            off[3 * (base + c)] = a;
                            off[3 * (base + c) + 1] = b;
                            off[3 * (base + c) + 2] = d;
                        }
                        ++c;
                    }
                }
    }
    if (!FILL) cnt[i] = c;
}

inline int blocks(long long n, int t) { return (int)((n + t - 1) / t); }
// a grid-stride launch over about 8 entries per atom, at most 4 blocks per SM
inline int copy_grid(int n) { return std::max(1, std::min(blocks(8ll * n, 256), 4 * sm_count())); }

// The look-back scan's records for arrays of up to maxn values, sized and
// cleared on the host side of a build (never inside a capture).
void scan_prepare(pg_context* ctx, long long maxn) {
    const size_t ntiles = (size_t)std::max<long long>(1, (maxn + LB_TILE - 1) / LB_TILE);
    if (ctx->scan_ctr.n == 0) {
        ctx->scan_ctr.resize(3);
        PG_CUDA(cudaMemsetAsync(ctx->scan_ctr.p, 0, sizeof(unsigned) * ctx->scan_ctr.cap, ctx->stream));
    }
    if (ctx->scan_rec.n < ntiles) {
        ctx->scan_rec.resize(ntiles);
        PG_CUDA(cudaMemsetAsync(ctx->scan_rec.p, 0, sizeof(unsigned long long) * ctx->scan_rec.cap, ctx->stream));
    }
}

// Exclusive scan of n ints into out[0..n] (out[n] and *total, may be null: the
// sum): one block for short arrays, the multi-block look-back scan otherwise.
void scan_ints(pg_context* ctx, const int* in, int* out, int n, int* total, cudaStream_t st) {
    const int ntiles = (n + LB_TILE - 1) / LB_TILE;
    if (ntiles <= 2 || ctx->scan_rec.n < (size_t)ntiles || ctx->scan_ctr.n < 3)
        scan_single_block<int, int><<<1, 1024, 0, st>>>(in, out, n, total, 0);
    else
        scan_lookback<<<ntiles, LB_THREADS, 0, st>>>(in, out, n, total, ctx->scan_rec.p, ctx->scan_ctr.p, ntiles);
    PG_CHECK_LAUNCH();
}

}  // namespace

// get_optimal_splitting, Geometry.f90:679-707 (host, no fused multiply-add)
static void optimal_splitting(const Cell& C, double max_cut, int sp[3]) {
    for (int i = 0; i < 3; ++i) {
        int v1 = (i + 1) % 3, v2 = (i + 2) % 3;
        double a[3], b[3], nn[3], v[3];
        for (int r = 0; r < 3; ++r) {
            a[r] = C.vc[r][v1];
            b[r] = C.vc[r][v2];
            v[r] = C.vc[r][i];
        }
        nn[0] = a[1] * b[2] - a[2] * b[1];
        nn[1] = a[2] * b[0] - a[0] * b[2];
        nn[2] = a[0] * b[1] - a[1] * b[0];
        double len = std::fabs(v[0] * nn[0] + v[1] * nn[1] + v[2] * nn[2]) /
                     std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        if (max_cut < 0.1e-4)
            sp[i] = (int)std::floor(10.0 * len);
        else
            sp[i] = (int)std::floor(len / max_cut);
        if (sp[i] > 40) sp[i] = 40;
    }
}

void exclusive_scan_int(const int* in, int* out, int n, cudaStream_t s, DevBuf<int>& tmp, int* total_host) {
    tmp.resize(1);
    scan_single_block<int, int><<<1, 1024, 0, s>>>(in, out, n, tmp.p, 0);
    PG_CHECK_LAUNCH();
    if (total_host) {
        PG_CUDA(cudaMemcpyAsync(total_host, tmp.p, sizeof(int), cudaMemcpyDeviceToHost, s));
        PG_CUDA(cudaStreamSynchronize(s));
    }
}

// Run seq on the context's stream from its captured graph g when sig matches
// the values the graph was built from; otherwise capture seq anew (updating
// the executable graph in place when the topology allows) and launch it.
// Host work (buffer sizing) happens before, outside seq.
template <typename F>
static void run_segment(pg_context* ctx, SegGraph& g, unsigned long long sig, F&& seq) {
    if (!ctx->use_graphs) {
        seq();
        return;
    }
    if (g.exec && g.sig == sig) {
        PG_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
        return;
    }
    cudaGraph_t graph = nullptr;
    PG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
        seq();
    } catch (...) {
        cudaStreamEndCapture(ctx->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    PG_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
    bool updated = false;
    if (g.exec) {
        cudaGraphExecUpdateResultInfo info{};
        updated = cudaGraphExecUpdate(g.exec, graph, &info) == cudaSuccess;
        if (!updated) {
            (void)cudaGetLastError();  // a failed update leaves no sticky error
            cudaGraphExecDestroy(g.exec);
            g.exec = nullptr;
        }
    }
    if (!updated) {
        const cudaError_t e = cudaGraphInstantiate(&g.exec, graph, 0);
        if (e != cudaSuccess) g.exec = nullptr;
        cudaGraphDestroy(graph);
        PG_CUDA(e);
    } else {
        cudaGraphDestroy(graph);
    }
    g.sig = sig;
    PG_CUDA(cudaGraphLaunch(g.exec, ctx->stream));
}

static SigHash& add_cell(SigHash& h, const CellK& C) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) h.add(C.vc[r][c]).add(C.ic[r][c]);
    for (int a = 0; a < 3; ++a) h.add(C.pbc[a]);
    return h;
}

void build_neighbor_lists(pg_context* ctx, const double* h_cutoffs) {
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    double max_cut = 0.0;
    for (int i = 0; i < n; ++i)
        if (i == 0 || h_cutoffs[i] > max_cut) max_cut = h_cutoffs[i];
    // every atom's list holds all partners closer than its own cutoff
    ctx->list_min_cutoff = n > 0 ? *std::min_element(h_cutoffs, h_cutoffs + n) : 0.0;
    int sp[3];
    optimal_splitting(ctx->cell, max_cut, sp);
    for (int a = 0; a < 3; ++a)
        require(sp[a] >= 1, PG_ERR_SMALL_CELL,
                "cell narrower than the neighbour cutoff: the cell-list build does not apply");
    Split S;
    for (int a = 0; a < 3; ++a) S.sp[a] = sp[a];
    S.nx = sp[0] + 2;
    S.ny = sp[1] + 2;
    S.nz = sp[2] + 2;
    const int ncell = S.nx * S.ny * S.nz;
    CellK C = cell_kernel_view(ctx->cell);

    if (h_cutoffs != ctx->h_cutoffs.data()) ctx->cutoffs.upload(h_cutoffs, n, st);  // else: on the device already
    ctx->cell_of.resize(3 * (size_t)std::max(n, 1));
    ctx->wrap.resize(3 * (size_t)std::max(n, 1));
    ctx->keys_a.resize(std::max(n, 1));
    ctx->keys_b.resize(std::max(n, 1));
    ctx->vals_a.resize(std::max(n, 1));
    ctx->vals_b.resize(std::max(n, 1));
    ctx->invisible.resize(std::max(n, 1) + 1);
    ctx->cell_start.resize(ncell + 1);
    ctx->nb_posf.resize(std::max(n, 1));
    int bits = 1;
    while ((1 << bits) < ncell) ++bits;
    const int passes = (bits + 7) / 8;
    const int nblk = std::max(1, blocks(n, RS_TILE));
    ctx->radix_hist.resize((size_t)256 * nblk + 1);
    ctx->count_tmp.resize((size_t)256 * nblk + 1);
    scan_prepare(ctx, std::max<long long>(n, 256ll * nblk));
    ctx->sorted_atoms.resize(std::max(n, 1));
    ctx->scan_tmp.resize(std::max(n, 1) + 1);
    ctx->nb_totals.resize(4);  // [0] out-of-range atoms, [1] list entries, [2] lower-index entries
    ctx->nb_g0.resize(std::max(n, 1));
    ctx->nb_start.resize(n + 1);
    ctx->g0_start.resize(n + 1);
    int* ht = ctx->h_totals.get(4);
    DevBuf<int>& inv_list = ctx->keys_b;  // free after the sort

    ScanArgs A{};
    A.n = n;
    A.pos = ctx->pos.p;
    A.posf = ctx->nb_posf.p;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) A.vcf[r][c] = (float)C.vc[r][c];
    A.cut = ctx->cutoffs.p;
    A.cell_of = ctx->cell_of.p;
    A.wrap = ctx->wrap.p;
    A.cstart = ctx->cell_start.p;
    A.sorted = ctx->sorted_atoms.p;
    A.invisible = ctx->invisible.p;
    A.inv_list = inv_list.p;
    A.n_inv = ctx->nb_totals.p;
    A.C = C;
    A.S = S;
    A.g0count = ctx->nb_g0.p;
    A.g1count = ctx->vals_a.p;

    // stage 1: subcells, the sort by subcell, the counting scan and both
    // prefix sums, whose totals come back with one synchronisation
    auto stage1 = [&] {
        if (n > 0) {
            nb_assign<<<blocks(n, 256), 256, 0, st>>>(n, ctx->pos.p, C, S, ctx->cell_of.p, ctx->keys_a.p,
                                                      ctx->vals_a.p, ctx->wrap.p, ctx->invisible.p, ctx->nb_posf.p);
            PG_CHECK_LAUNCH();
        }
        // radix sort by subcell id
        int *k_in = ctx->keys_a.p, *v_in = ctx->vals_a.p, *k_out = ctx->keys_b.p, *v_out = ctx->vals_b.p;
        for (int p = 0; p < passes && n > 0; ++p) {
            radix_hist<<<nblk, RS_THREADS, 0, st>>>(n, k_in, 8 * p, nblk, ctx->radix_hist.p);
            PG_CHECK_LAUNCH();
            scan_ints(ctx, ctx->radix_hist.p, ctx->count_tmp.p, 256 * nblk, nullptr, st);
            radix_scatter<<<nblk, RS_THREADS, 0, st>>>(n, k_in, v_in, 8 * p, nblk, ctx->count_tmp.p, k_out, v_out);
            PG_CHECK_LAUNCH();
            std::swap(k_in, k_out);
            std::swap(v_in, v_out);
        }
        cell_starts<<<blocks(n + 1, 256), 256, 0, st>>>(n, ncell, k_in, ctx->cell_start.p);
        PG_CHECK_LAUNCH();
        if (n > 0)
            PG_CUDA(cudaMemcpyAsync(ctx->sorted_atoms.p, v_in, sizeof(int) * n, cudaMemcpyDeviceToDevice, st));
        // atoms in out-of-range periodic subcells: their count stays on the device
        scan_ints(ctx, ctx->invisible.p, ctx->scan_tmp.p, n, ctx->nb_totals.p, st);
        // inv_list may alias the sort's output buffer: the sorted atoms were copied first
        if (n > 0) {
            compact_flags<<<blocks(n, 256), 256, 0, st>>>(n, ctx->invisible.p, ctx->scan_tmp.p, inv_list.p);
            PG_CHECK_LAUNCH();
            nb_scan<false><<<blocks((long long)n * 32, SCAN_THREADS), SCAN_THREADS, 0, st>>>(A);
            PG_CHECK_LAUNCH();
            // CSR starts and lower-index key buffer starts
            add_counts<<<blocks(n, 256), 256, 0, st>>>(n, ctx->nb_g0.p, ctx->vals_a.p, ctx->keys_a.p);
            PG_CHECK_LAUNCH();
        }
        scan_ints(ctx, ctx->keys_a.p, ctx->nb_start.p, n, ctx->nb_totals.p + 1, st);
        scan_ints(ctx, ctx->nb_g0.p, ctx->g0_start.p, n, ctx->nb_totals.p + 2, st);
        PG_CUDA(cudaMemcpyAsync(ht, ctx->nb_totals.p, sizeof(int) * 4, cudaMemcpyDeviceToHost, st));
    };
    SigHash h1;
    h1.add(alloc_epoch()).add(n).add(ncell).add(passes).add(nblk).add(S).add(ht);
    add_cell(h1, C);
    run_segment(ctx, ctx->seg_g[0], h1.h, stage1);
    PG_CUDA(cudaStreamSynchronize(st));
    const int total = ht[1], total0 = ht[2];
    require(ht[0] >= 0 && total >= 0 && total0 >= 0, PG_ERR_CUDA, "neighbour-list prefix scan did not complete");
    ctx->nb_total = total;
    ctx->nb_idx.resize(std::max(total, 1));
    ctx->nb_off.resize(3 * (size_t)std::max(total, 1));
    ctx->g0_keys.resize(std::max(total0, 1));
    ctx->g0_vals.resize(std::max(total0, 1));
    A.start = ctx->nb_start.p;
    A.g0start = ctx->g0_start.p;
    A.g0key = ctx->g0_keys.p;
    A.g0val = ctx->g0_vals.p;
    A.idx = ctx->nb_idx.p;
    A.off = ctx->nb_off.p;
    // stage 2: the filling scan and the order of the lower-index entries
    auto stage2 = [&] {
        if (n > 0) {
            nb_scan<true><<<blocks((long long)n * 32, SCAN_THREADS), SCAN_THREADS, 0, st>>>(A);
            PG_CHECK_LAUNCH();
            nb_sort_g0<<<blocks((long long)n * 32, 256), 256, 0, st>>>(n, ctx->nb_g0.p, ctx->g0_start.p,
                                                                      ctx->nb_start.p, ctx->g0_keys.p, ctx->g0_vals.p,
                                                                      ctx->nb_idx.p, ctx->nb_off.p);
            PG_CHECK_LAUNCH();
        }
    };
    SigHash h2;
    h2.add(alloc_epoch()).add(n).add(S);
    add_cell(h2, C);
    run_segment(ctx, ctx->seg_g[1], h2.h, stage2);
    // the cutoffs (host copy) for rebuilds on the device coordinates
    if (h_cutoffs != ctx->h_cutoffs.data()) ctx->h_cutoffs.assign(h_cutoffs, h_cutoffs + n);
    ctx->list_kind = PG_LIST_CELLS;
    ctx->have_list = true;
    ctx->list_epoch++;
    ctx->state_epoch++;
    ctx->short_dirty = true;
}

void build_allpairs_lists(pg_context* ctx, const double* h_cutoffs) {
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    double mc = 0.0;
    for (int i = 0; i < n; ++i) mc = std::max(mc, h_cutoffs[i]);
    ctx->list_min_cutoff = n > 0 ? *std::min_element(h_cutoffs, h_cutoffs + n) : 0.0;
    const Cell& Cc = ctx->cell;
    int ni[3];
    for (int i = 0; i < 3; ++i) {
        ni[i] = 0;
        if (!Cc.pbc[i]) continue;
        int v1 = (i + 1) % 3, v2 = (i + 2) % 3;
        double a[3], b[3], nn[3], v[3];
        for (int r = 0; r < 3; ++r) {
            a[r] = Cc.vc[r][v1];
            b[r] = Cc.vc[r][v2];
            v[r] = Cc.vc[r][i];
        }
        nn[0] = a[1] * b[2] - a[2] * b[1];
        nn[1] = a[2] * b[0] - a[0] * b[2];
        nn[2] = a[0] * b[1] - a[1] * b[0];
        double len = std::fabs(v[0] * nn[0] + v[1] * nn[1] + v[2] * nn[2]) /
                     std::sqrt(nn[0] * nn[0] + nn[1] * nn[1] + nn[2] * nn[2]);
        require(len > 0.0, PG_ERR_INVALID, "degenerate periodic cell");
        ni[i] = (int)std::ceil(2.0 * mc / len);
        require(ni[i] <= 64, PG_ERR_INVALID, "cutoff spans too many periodic images");
    }
    CellK C = cell_kernel_view(Cc);
    if (h_cutoffs != ctx->h_cutoffs.data()) ctx->cutoffs.upload(h_cutoffs, n, st);
    ctx->nb_g0.resize(std::max(n, 1));
    ctx->nb_start.resize(n + 1);
    const int3 nimg = make_int3(ni[0], ni[1], ni[2]);
    if (n > 0) {
        allpairs_scan<false><<<blocks(n, 128), 128, 0, st>>>(n, ctx->pos.p, ctx->cutoffs.p, C, nimg, nullptr,
                                                             ctx->nb_g0.p, nullptr, nullptr);
        PG_CHECK_LAUNCH();
    }
    int total = 0;
    exclusive_scan_int(ctx->nb_g0.p, ctx->nb_start.p, n, st, ctx->count_tmp, &total);
    ctx->nb_total = total;
    ctx->nb_idx.resize(std::max(total, 1));
    ctx->nb_off.resize(3 * (size_t)std::max(total, 1));
    if (n > 0) {
        allpairs_scan<true><<<blocks(n, 128), 128, 0, st>>>(n, ctx->pos.p, ctx->cutoffs.p, C, nimg, ctx->nb_start.p,
                                                            nullptr, ctx->nb_idx.p, ctx->nb_off.p);
        PG_CHECK_LAUNCH();
    }
    if (h_cutoffs != ctx->h_cutoffs.data()) ctx->h_cutoffs.assign(h_cutoffs, h_cutoffs + n);
    ctx->list_kind = PG_LIST_ALL_PAIRS;
    ctx->have_list = true;
    ctx->list_epoch++;
    ctx->state_epoch++;
    ctx->short_dirty = true;
}

void install_neighbor_lists(pg_context* ctx, const int32_t* counts, const int32_t* idx, const int32_t* off) {
    const int n = ctx->n;
    ctx->list_min_cutoff = 0.0;  // unknown reach
    std::vector<int> start(n + 1, 0);
    for (int i = 0; i < n; ++i) {
        require(counts[i] >= 0, PG_ERR_INVALID, "negative neighbour count");
        start[i + 1] = start[i] + counts[i];
    }
    const int total = start[n];
    for (int e = 0; e < total; ++e) require(idx[e] >= 0 && idx[e] < n, PG_ERR_INVALID, "neighbour index out of range");
    ctx->nb_start.upload(start.data(), n + 1, ctx->stream);
    ctx->nb_idx.resize(std::max(total, 1));
    ctx->nb_off.resize(3 * (size_t)std::max(total, 1));
    if (total) {
        PG_CUDA(cudaMemcpyAsync(ctx->nb_idx.p, idx, sizeof(int) * total, cudaMemcpyHostToDevice, ctx->stream));
        PG_CUDA(cudaMemcpyAsync(ctx->nb_off.p, off, sizeof(int) * 3 * total, cudaMemcpyHostToDevice, ctx->stream));
    }
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->nb_total = total;
    ctx->list_kind = PG_LIST_INSTALLED;
    ctx->have_list = true;
    ctx->list_epoch++;
    ctx->state_epoch++;
    ctx->short_dirty = true;
}

// Start a list generation: remember the positions and take the full list's
// bond vectors there (used by the mixed-precision pair kernel).
void build_full_sep0(pg_context* ctx) {
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    CellK C = cell_kernel_view(ctx->cell);
    ctx->pos0.resize(3 * (size_t)std::max(n, 1));
    ctx->nb_sep0.resize((size_t)std::max<long long>(ctx->nb_total, 1));
    if (n > 0) {
        SigHash h;
        h.add(alloc_epoch()).add(n);
        add_cell(h, C);
        run_segment(ctx, ctx->seg_g[2], h.h, [&] {
            PG_CUDA(cudaMemcpyAsync(ctx->pos0.p, ctx->pos.p, sizeof(double) * 3 * n, cudaMemcpyDeviceToDevice, st));
            short_sep0<<<blocks(n, 128), 128, 0, st>>>(n, ctx->pos0.p, C, ctx->nb_start.p, ctx->nb_idx.p,
                                                      ctx->nb_off.p, ctx->nb_sep0.p);
            PG_CHECK_LAUNCH();
        });
    }
    ctx->sep0_epoch = ctx->list_epoch;
    ctx->short_dirty = true;
    ctx->state_epoch++;
}

void build_short_list(pg_context* ctx, bool same_positions) {
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    const double r = ctx->bo_radius + ctx->skin;
    CellK C = cell_kernel_view(ctx->cell);
    const double* p0 = ctx->pos0.p;  // positions of this list generation
    ctx->sh_count.resize(std::max(n, 1));
    ctx->sh_start.resize(n + 1);
    ctx->nb_totals.resize(4);
    scan_prepare(ctx, std::max<long long>(n, 256ll * std::max(1, blocks(n, RS_TILE))));
    int* ht = ctx->h_totals.get(4);
    // The short list is the full list itself when the cell-list build ran at
    // the generation's reference positions and no atom's list radius exceeds
    // r: every entry passed the same FP64 test (sep_d2) against a radius <= r,
    // so it passes against r (silicon: 3.0 + 0.5 A both).  Its entries and
    // bond vectors are then copied, and the count and its synchronisation
    // skipped.
    double max_cut = 0.0;
    for (double c : ctx->h_cutoffs) max_cut = std::max(max_cut, c);
    const bool copy_full = same_positions && ctx->list_kind == PG_LIST_CELLS && n > 0 &&
                           (int)ctx->h_cutoffs.size() == n && max_cut <= r && ctx->sep0_epoch == ctx->list_epoch;
    // stage 1: the short lists' lengths and starts; the total comes back
    auto stage1 = [&] {
        if (n > 0) {
            short_count<<<blocks(n, 128), 128, 0, st>>>(n, p0, C, ctx->nb_start.p, ctx->nb_idx.p, ctx->nb_off.p,
                                                       r * r, ctx->sh_count.p);
            PG_CHECK_LAUNCH();
        }
        scan_ints(ctx, ctx->sh_count.p, ctx->sh_start.p, n, ctx->nb_totals.p + 3, st);
        PG_CUDA(cudaMemcpyAsync(ht + 3, ctx->nb_totals.p + 3, sizeof(int), cudaMemcpyDeviceToHost, st));
    };
    int total = 0;
    if (copy_full) {
        total = (int)ctx->nb_total;
    } else {
        SigHash h1;
        h1.add(alloc_epoch()).add(n).add(r).add(ht);
        add_cell(h1, C);
        run_segment(ctx, ctx->seg_g[3], h1.h, stage1);
        PG_CUDA(cudaStreamSynchronize(st));
        total = ht[3];
        require(total >= 0, PG_ERR_CUDA, "short-list prefix scan did not complete");
    }
    ctx->sh_total = total;
    if (copy_full) {  // room for whole copies of the full list's buffers: sizes that do not move with the total
        ctx->sh_idx.resize(ctx->nb_idx.cap);
        ctx->sh_off.resize(ctx->nb_off.cap);
        ctx->sh_sep0.resize(ctx->nb_sep0.cap);
    } else {
        ctx->sh_idx.resize(std::max(total, 1));
        ctx->sh_off.resize(3 * (size_t)std::max(total, 1));
        ctx->sh_sep0.resize(std::max(total, 1));  // bond vectors of this list generation
    }
    ctx->sh_rev.resize(std::max(total, 1));
    ctx->sh_type.resize(std::max(total, 1));
    ctx->sh_order.resize(std::max(n, 1));
    ctx->sh_slot.resize(std::max(n, 1));
    const int nblk = std::max(1, blocks(n, RS_TILE));
    if (n > 0) {
        ctx->keys_a.resize(n);
        ctx->keys_b.resize(n);
        ctx->vals_a.resize(n);
        ctx->vals_b.resize(n);
        ctx->radix_hist.resize((size_t)256 * nblk + 1);
        ctx->count_tmp.resize((size_t)256 * nblk + 1);
    }
    // stage 2: fill, reverse entries, bond vectors, partner types, and the
    // atoms grouped by list length, stably (ties in index order), so that the
    // lane groups of one warp loop over the same number of bonds: a two-digit
    // radix sort of (count, atom) on the device (counts below 65536), then per
    // slot (atom, first entry, count).  No launch depends on the total.
    auto stage2 = [&] {
        if (n == 0) return;
        if (copy_full) {
            PG_CUDA(cudaMemcpyAsync(ctx->sh_start.p, ctx->nb_start.p, sizeof(int) * (n + 1), cudaMemcpyDeviceToDevice,
                                    st));
            PG_CUDA(cudaMemcpyAsync(ctx->sh_idx.p, ctx->nb_idx.p, sizeof(int) * ctx->nb_idx.cap,
                                    cudaMemcpyDeviceToDevice, st));
            PG_CUDA(cudaMemcpyAsync(ctx->sh_off.p, ctx->nb_off.p, sizeof(int) * ctx->nb_off.cap,
                                    cudaMemcpyDeviceToDevice, st));
            PG_CUDA(cudaMemcpyAsync(ctx->sh_sep0.p, ctx->nb_sep0.p, sizeof(F4) * ctx->nb_sep0.cap,
                                    cudaMemcpyDeviceToDevice, st));
            PG_CUDA(cudaMemcpyAsync(ctx->nb_totals.p + 3, ctx->nb_totals.p + 1, sizeof(int), cudaMemcpyDeviceToDevice,
                                    st));
        } else {
            short_fill<<<blocks(n, 128), 128, 0, st>>>(n, p0, C, ctx->nb_start.p, ctx->nb_idx.p, ctx->nb_off.p,
                                                      r * r, ctx->sh_start.p, ctx->sh_idx.p, ctx->sh_off.p);
            PG_CHECK_LAUNCH();
        }
        short_reverse<<<blocks((long long)n * ENTRY_LANES, 128), 128, 0, st>>>(n, ctx->sh_start.p, ctx->sh_idx.p, ctx->sh_off.p,
                                                     ctx->sh_rev.p, ctx->sh_count.p);
        PG_CHECK_LAUNCH();
        if (!copy_full) {
            short_sep0<<<blocks(n, 128), 128, 0, st>>>(n, p0, C, ctx->sh_start.p, ctx->sh_idx.p, ctx->sh_off.p,
                                                      ctx->sh_sep0.p);
            PG_CHECK_LAUNCH();
        }
        entry_types<<<copy_grid(n), 256, 0, st>>>(ctx->nb_totals.p + 3, ctx->sh_idx.p, ctx->type.p, ctx->sh_type.p);
        PG_CHECK_LAUNCH();
        order_keys<<<blocks(n, 256), 256, 0, st>>>(n, ctx->sh_count.p, ctx->keys_a.p, ctx->vals_a.p);
        PG_CHECK_LAUNCH();
        int *k_in = ctx->keys_a.p, *v_in = ctx->vals_a.p, *k_out = ctx->keys_b.p, *v_out = ctx->vals_b.p;
        for (int pass = 0; pass < 2; ++pass) {
            radix_hist<<<nblk, RS_THREADS, 0, st>>>(n, k_in, 8 * pass, nblk, ctx->radix_hist.p);
            PG_CHECK_LAUNCH();
            scan_ints(ctx, ctx->radix_hist.p, ctx->count_tmp.p, 256 * nblk, nullptr, st);
            radix_scatter<<<nblk, RS_THREADS, 0, st>>>(n, k_in, v_in, 8 * pass, nblk, ctx->count_tmp.p, k_out, v_out);
            PG_CHECK_LAUNCH();
            std::swap(k_in, k_out);
            std::swap(v_in, v_out);
        }
        order_slots<<<blocks(n, 256), 256, 0, st>>>(n, v_in, ctx->sh_start.p, ctx->sh_count.p, ctx->sh_order.p,
                                                    ctx->sh_slot.p);
        PG_CHECK_LAUNCH();
    };
    SigHash h2;
    h2.add(alloc_epoch()).add(n).add(r).add(nblk).add(copy_full);
    add_cell(h2, C);
    run_segment(ctx, ctx->seg_g[copy_full ? 5 : 4], h2.h, stage2);
    // Lists from the host may lack reverse entries: checked before use.  The
    // engine's own builds are symmetric by construction.
    if (ctx->list_kind == PG_LIST_INSTALLED) {
        DevBuf<int> mx;
        mx.resize(1);
        min_reduce<<<1, 1024, 0, st>>>(std::max(total, 1) * (total > 0), ctx->sh_rev.p, mx.p);
        PG_CHECK_LAUNCH();
        int hm = 0;
        PG_CUDA(cudaMemcpyAsync(&hm, mx.p, sizeof(int), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
        require(total == 0 || hm >= 0, PG_ERR_INVALID,
                "neighbour lists are not symmetric: a bond has no reverse entry (lists must be built both ways)");
    }
    ctx->short_dirty = false;
    ctx->state_epoch++;
}

}  // namespace pg
