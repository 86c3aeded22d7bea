// tersoff_tri.cu -- the bond pass of the pair-bond-order (Tersoff) evaluation
// with one triplet per lane (the "triplet tile").
//
// Same physics, inputs and outputs as bond_pass (tersoff.cu: zeta_ij, B, the
// pair terms, the radial and three-body forces, the per-entry force records
// that gather_pass collects, the centre part per atom, energy and virial),
// following core_calculate_pair_bond_order_factor (Core.f90:2439-2637),
// core_post_process_pair_bond_order_factor (2763-2807) and
// core_add_pair_bond_order_forces (4952-5353).
//
// bond_pass gives each lane one bond i->j and loops over the other bonds i->k
// twice (zeta, then the gradient), so every lane carries a long chain of
// dependent arithmetic and the GPU, one wave deep at 32k atoms, waits on it.
// Here 16 lanes serve one atom as a 4 x 4 tile: lane (a, b) takes the triplet
// (bond e = 4 eb + a, neighbour k = 4 kb + b) of every block pair (eb, kb), so
// an atom with up to 4 bonds is one pass:
//   1. the geometry of the atom's bonds is staged in shared memory (unit
//      vector, 1/r, cutoff factor), one bond per lane;
//   2. each lane adds its triplet's zeta term; a row (the 4 lanes of one e)
//      sums them with shuffles, then computes B(zeta), dB/dzeta and the pair
//      terms of its bond;
//   3. each lane takes its triplet's gradient: the j parts are summed over the
//      row, the k parts over the column, and the centre part over all 16
//      lanes, all with shuffles in a fixed order (deterministic, no atomics);
//   4. the records (j part of entry e plus k parts landing on entry e) go to
//      the partner's own entry through the reverse index, as in bond_pass.
// A warp serves two atoms at a time (adjacent in the order of list length) and
// loops over atom pairs, keeping its energy and virial in registers until the
// end, so that the exact fixed-point totals are formed once per warp.
#include "args.cuh"
#include "bond.cuh"
#include "common.cuh"
#include "kernels.cuh"
#include "tri_body.cuh"

namespace pg {

namespace {

// One system: the warps loop over atom pairs (slots 2p, 2p + 1 in the order of
// list length), p = warp, warp + total warps, ...
template <typename R, bool SPEC>
__global__ void __launch_bounds__(TRI_THREADS) tri_pass(const __grid_constant__ BondArgs A) {
    __shared__ TriStage<R> stage[TRI_ATOMS];
    __shared__ Fx128 wsum[TRI_THREADS / 32][7];
    __shared__ unsigned done;
    if (threadIdx.x == 0) done = 0u;
    pdl_trigger();
    __syncthreads();
    pdl_wait();  // the displacements (mixed path) and the cleared totals come from the kernel before
    if (A.skip && *A.skip) return;  // uniform over the grid
    const int w = threadIdx.x >> 5, h = (threadIdx.x >> 4) & 1;
    TriStage<R>& S = stage[threadIdx.x >> 4];
    TriAcc<R> acc;
    const int pairs = (A.n + 1) >> 1;
    const int nw = gridDim.x * (TRI_THREADS / 32);
    for (int p = blockIdx.x * (TRI_THREADS / 32) + w; p < pairs; p += nw) tri_atom<R, SPEC>(A, 2 * p + h, S, acc);
    if (A.acc) tri_publish(acc, wsum, &done, A.acc);
}

// Many systems: tiles[t] = (system, block of that system); a block serves the
// 8 atoms (slots) blk * 8 .. blk * 8 + 7 of its system.
template <typename R, bool SPEC>
__global__ void __launch_bounds__(TRI_THREADS)
    tri_pass_batch(const BondArgs* __restrict__ sys, const int2* __restrict__ tiles, int ntiles) {
    __shared__ TriStage<R> stage[TRI_ATOMS];
    __shared__ Fx128 wsum[TRI_THREADS / 32][7];
    __shared__ unsigned done;
    pdl_trigger();
    pdl_wait();
    TriStage<R>& S = stage[threadIdx.x >> 4];
    for (int q = blockIdx.x; q < ntiles; q += gridDim.x) {
        const int2 tl = tiles[q];
        const BondArgs& A = sys[tl.x];
        if (threadIdx.x == 0) done = 0u;
        __syncthreads();
        TriAcc<R> acc;
        tri_atom<R, SPEC>(A, tl.y * TRI_ATOMS + (threadIdx.x >> 4), S, acc);
        if (A.acc) tri_publish(acc, wsum, &done, A.acc);
        __syncthreads();
    }
}

}  // namespace

// blocks of the single-system triplet tile: every SM filled (resident blocks),
// never more than the atom pairs need
int tri_blocks(int n) {
    static int per_sm[2][2] = {{0, 0}, {0, 0}};
    const int need = std::max(1, ((n + 1) / 2 + TRI_THREADS / 32 - 1) / (TRI_THREADS / 32));
    auto occ = [](auto kern) {
        int b = 0;
        if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&b, kern, TRI_THREADS, 0) != cudaSuccess || b < 1) b = 1;
        return b;
    };
    if (per_sm[0][0] == 0) {
        per_sm[0][0] = occ(tri_pass<float, false>);
        per_sm[0][1] = occ(tri_pass<float, true>);
        per_sm[1][0] = occ(tri_pass<double, false>);
        per_sm[1][1] = occ(tri_pass<double, true>);
    }
    const int resident = std::min(std::min(per_sm[0][0], per_sm[0][1]), std::min(per_sm[1][0], per_sm[1][1]));
    return std::min(need, resident * sm_count());
}

// blocks (tiles) of one system in the many-system triplet-tile launch
int tri_batch_blocks(int n) { return std::max(1, (n + TRI_ATOMS - 1) / TRI_ATOMS); }

void launch_tri_pass(const BondArgs& A, int n, int precision, cudaStream_t st) {
    const dim3 grid(tri_blocks(n)), block(TRI_THREADS);
    if (precision == PG_PREC_FP64) {
        if (A.spec) launch_pdl(tri_pass<double, true>, grid, block, st, A);
        else launch_pdl(tri_pass<double, false>, grid, block, st, A);
    } else {
        if (A.spec) launch_pdl(tri_pass<float, true>, grid, block, st, A);
        else launch_pdl(tri_pass<float, false>, grid, block, st, A);
    }
}

void launch_tri_batch(const BondArgs* sys, const int2* tiles, int ntiles, int grid, int precision, bool spec,
                      cudaStream_t st) {
    const dim3 g(grid), b(TRI_THREADS);
    if (precision == PG_PREC_FP64) {
        if (spec) launch_pdl(tri_pass_batch<double, true>, g, b, st, sys, tiles, ntiles);
        else launch_pdl(tri_pass_batch<double, false>, g, b, st, sys, tiles, ntiles);
    } else {
        if (spec) launch_pdl(tri_pass_batch<float, true>, g, b, st, sys, tiles, ntiles);
        else launch_pdl(tri_pass_batch<float, false>, g, b, st, sys, tiles, ntiles);
    }
}

}  // namespace pg
