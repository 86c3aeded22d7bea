// persist.cuh -- many independent systems evaluated by ONE persistent launch.
//
// No counterpart in the reference, which holds one system per process in its
// Fortran core (Core.f90:22-30).  The evaluation of every system of a batch is
// four phases -- displacements (and the cleared totals), pair terms, the
// Tersoff bond pass, the gather of the bond forces -- and a phase of one
// system may start when the phases it reads are complete for that system:
//   pair, bond    after the system's displacement tiles,
//   gather        after the system's bond and pair tiles (the gather adds the
//                 bond forces to the pair forces of the same atoms).
// The work list holds tiles (phase, system, first block, blocks) phase by
// phase -- every displacement tile, then every pair tile, every bond tile,
// every gather tile -- so that a tile's dependencies always sit earlier in the
// list.  A grid of resident blocks takes tiles in list order from one atomic
// ticket; before a pair, bond or gather tile its block waits for the
// per-system counters of the tiles it depends on.  Those tiles hold lower
// tickets, so they belong to blocks that are already running, and the oldest
// unfinished tile never waits: the loop cannot deadlock, whatever the number
// of resident blocks.  Every wait is bounded (a time limit and an iteration
// limit); a wait that runs out sets the status word, every block stops taking
// tiles, and the host reports PG_ERR_TIMEOUT instead of results.
//
// Tiles: "atoms per warp" is 32 / lanes per atom of the pair body (PG) and of
// the bond body (BG; PG_LANES_TRIPLET is the 4 x 4 triplet tile, 2 atoms per
// warp); "cells per block" is the number of consecutive atom blocks (cells of
// 128 threads) that one ticket hands to a block.  The batch's autotuner times
// the combinations on the batch itself.
#pragma once

#include <algorithm>
#include <map>
#include <type_traits>

#include "bond_body.cuh"
#include "pair_body.cuh"
#include "tri_body.cuh"

namespace pg {

// one work tile (32 bytes: two vector loads)
struct __align__(16) PTile {
    int phase;  // 0 displacements, 1 pair terms, 2 bond pass, 3 gather
    int sys;
    int blk0;   // first block of the phase in this system
    int nblk;   // consecutive blocks
    int need0;  // tiles it waits for: displacement tiles (pair, bond) or bond tiles (gather)
    int need1;  // pair tiles (gather)
    int pad0, pad1;
};

struct PersistArgs {
    const DispArgs* disp;  // per system
    const PairArgs* pair;  // per system (entries of systems without pair terms unused)
    const BondArgs* bond;  // per system (entries of systems without bond terms unused)
    const PTile* tiles;
    int ntiles;
    unsigned* ticket;      // next tile (zero before each launch)
    unsigned* done;        // per system x 4 phases: finished tiles (zero before each launch)
    int* status;           // 0; 1 when a wait gave up
    unsigned long long wait_ns;  // time limit of one wait
};

constexpr int PERSIST_THREADS = 128;
constexpr int PERSIST_MIN_BLOCKS = 7;  // resident blocks per SM the registers are capped for
constexpr unsigned PERSIST_MAX_POLLS = 1u << 24;  // iteration limit of one wait

__device__ __forceinline__ unsigned ld_acquire(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// counter increment with release semantics: after a __syncthreads(), the
// writes of every thread of the block are visible to a reader that acquires
// the new count
__device__ __forceinline__ void red_release(unsigned* p, unsigned v) {
    asm volatile("red.release.gpu.global.add.u32 [%0], %1;" ::"l"(p), "r"(v) : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// wait until *p >= need: false when the time or the iteration limit runs out,
// or when another block's wait has run out (status set)
__device__ __forceinline__ bool wait_count(const unsigned* p, unsigned need, unsigned long long limit_ns,
                                           const int* status) {
    if (ld_acquire(p) >= need) return true;
    const unsigned long long t0 = global_ns();
    for (unsigned it = 0; it < PERSIST_MAX_POLLS; ++it) {
        __nanosleep(128);
        if (ld_acquire(p) >= need) return true;
        if ((it & 31u) == 31u && (global_ns() - t0 > limit_ns || *(const volatile int*)status)) return false;
    }
    return false;
}

// thread 0: tile t (a ticket already taken, its record T) once its
// dependencies are complete, or -1 (list done, or a wait ran out here or
// elsewhere)
__device__ __forceinline__ int claim_tile(const PersistArgs& P, int t, const PTile& T) {
    if (t >= P.ntiles) return -1;
    if (*(volatile int*)P.status) return -1;
    const unsigned* d = P.done + 4 * (size_t)T.sys;
    bool ok = true;
    if (T.phase == 1 || T.phase == 2) {
        ok = wait_count(d, (unsigned)T.need0, P.wait_ns, P.status);
    } else if (T.phase == 3) {
        ok = wait_count(d + 2, (unsigned)T.need0, P.wait_ns, P.status) &&
             wait_count(d + 1, (unsigned)T.need1, P.wait_ns, P.status);
    }
    if (!ok) {
        atomicExch(P.status, 1);
        return -1;
    }
    return t;
}

// thread 0: start copying tile t's record into shared memory (asynchronous;
// copy_wait() before reading it)
__device__ __forceinline__ void copy_tile(const PersistArgs& P, int t, PTile* dst) {
    if (t >= P.ntiles) return;
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const PTile* src = P.tiles + t;
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d), "l"(src) : "memory");
    asm volatile("cp.async.ca.shared.global [%0], [%1], 16;" ::"r"(d + 16), "l"((const char*)src + 16) : "memory");
    asm volatile("cp.async.commit_group;" ::: "memory");
}
__device__ __forceinline__ void copy_wait() { asm volatile("cp.async.wait_all;" ::: "memory"); }

// Thread 0 takes the ticket of the block's next tile while the block works on
// the current one (the atomic's latency hidden behind the work).  A block then
// holds one tile it has not started; that tile is not older than any tile
// still waiting, so the oldest unfinished tile still never waits.
template <typename R, int PG, int BG, bool SPEC>
__global__ void __launch_bounds__(PERSIST_THREADS, PERSIST_MIN_BLOCKS)
    batch_persistent(const __grid_constant__ PersistArgs P) {
    constexpr bool TRI = BG == PG_LANES_TRIPLET;
    constexpr int GG = TRI ? 16 : BG;  // gather lanes (the triplet tile serves 8 atoms per block)
    __shared__ int s_tile;
    __shared__ PTile s_rec[2];  // the current tile's record and the next one's, in flight
    int next = 0;
    if (threadIdx.x == 0) {
        next = (int)atomicAdd(P.ticket, 1u);
        copy_tile(P, next, &s_rec[1]);
    }
    for (;;) {
        if (threadIdx.x == 0) {
            const int t = next;
            copy_wait();
            s_rec[0] = s_rec[1];
            if (t < P.ntiles) next = (int)atomicAdd(P.ticket, 1u);
            s_tile = claim_tile(P, t, s_rec[0]);
        }
        __syncthreads();
        const int t = s_tile;
        const PTile T = s_rec[0];
        __syncthreads();  // every thread has read s_tile, s_rec[0] before thread 0 writes them again
        if (t < 0) return;
        // the following tile's record, copied while the block works on this one
        if (threadIdx.x == 0) copy_tile(P, next, &s_rec[1]);
        if (T.phase == 0) {
            const DispArgs& A = P.disp[T.sys];
            for (int k = 0; k < T.nblk; ++k) disp_body(A, (T.blk0 + k) * PERSIST_THREADS + threadIdx.x);
        } else if (T.phase == 1) {
            const PairArgs& A = P.pair[T.sys];
            for (int k = 0; k < T.nblk; ++k) {
                pair_body<R, PG>(A, T.blk0 + k);
                __syncthreads();
            }
        } else if (T.phase == 2) {
            const BondArgs& A = P.bond[T.sys];
            if constexpr (TRI) {
                __shared__ TriStage<R> stage[TRI_ATOMS];
                __shared__ Fx128 wsum[TRI_THREADS / 32][7];
                __shared__ unsigned tdone;
                for (int k = 0; k < T.nblk; ++k) {
                    if (threadIdx.x == 0) tdone = 0u;
                    __syncthreads();
                    TriAcc<R> acc;
                    tri_atom<R, SPEC>(A, (T.blk0 + k) * TRI_ATOMS + (threadIdx.x >> 4), stage[threadIdx.x >> 4], acc);
                    if (A.acc) tri_publish(acc, wsum, &tdone, A.acc);
                    __syncthreads();
                }
            } else {
                for (int k = 0; k < T.nblk; ++k) {
                    bond_body<R, BG, SPEC>(A, T.blk0 + k, A.nblocks);
                    __syncthreads();
                }
            }
        } else {
            const BondArgs& A = P.bond[T.sys];
            for (int k = 0; k < T.nblk; ++k) gather_body<R, GG>(A, T.blk0 + k, A.nblocks);
        }
        // the tile's results visible device-wide before its counter moves
        __syncthreads();
        if (threadIdx.x == 0) red_release(P.done + 4 * (size_t)T.sys + T.phase, 1u);
    }
}

// The instantiations of one precision and one table mode (persist_*.cu, four
// translation units that compile in parallel): launch with the resident grid;
// returns the blocks per SM of the kernel.
template <typename R, bool SPEC>
int launch_persistent_impl(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st) {
    // resident blocks per SM of each instantiation, queried once (outside any capture)
    static std::map<const void*, int> occupancy;
    auto go = [&](auto kern) {
        int& per_sm = occupancy[(const void*)kern];
        if (per_sm == 0) {
            PG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, PERSIST_THREADS, 0));
            if (per_sm < 1) per_sm = 1;
        }
        const int grid = std::max(1, std::min(P.ntiles, per_sm * sms));
        kern<<<grid, PERSIST_THREADS, 0, st>>>(P);
        return per_sm;
    };
    auto by_bond = [&](auto pgt) -> int {
        constexpr int PGL = decltype(pgt)::value;
        switch (bg_lanes) {
            case 4: return go(batch_persistent<R, PGL, 4, SPEC>);
            case 8: return go(batch_persistent<R, PGL, 8, SPEC>);
            default: return go(batch_persistent<R, PGL, PG_LANES_TRIPLET, SPEC>);
        }
    };
    if (pg_lanes == 8) return by_bond(std::integral_constant<int, 8>{});
    return by_bond(std::integral_constant<int, 16>{});
}

// entry points of the four translation units
int launch_persistent_f32_spec(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st);
int launch_persistent_f32_table(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st);
int launch_persistent_f64_spec(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st);
int launch_persistent_f64_table(const PersistArgs& P, int pg_lanes, int bg_lanes, int sms, cudaStream_t st);

}  // namespace pg
