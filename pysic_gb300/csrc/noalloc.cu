// noalloc.cu -- the bond-order evaluation with every per-call buffer in one
// static device array, for callers that must not allocate device memory while
// the call runs.
//
// The regular evaluation grows its scratch buffers (bond geometry, per-bond
// force parts, per-atom centre parts, displacements) with cudaMalloc on
// first use and whenever the lists grow.  This variant takes all of them from
// g_scratch, a file-scope __device__ array of PG_NOALLOC_SCRATCH_BYTES, and
// writes its results into device buffers the caller owns.
//
// Set-up: the first call on each context, with the context's device current,
// looks up the array's address with cudaGetSymbolAddress (which may load this
// library's device code) and keeps it in the context; make that first call
// before any stream capture.  The address belongs to the CUDA context that was
// current at the look-up: a context created after a device reset looks it up
// anew, while one created before the reset must not be used after it.
// Zeroing: only the 128-bit energy / virial totals must start at zero; they are
// cleared with cudaMemsetAsync at the start of every call.  Every other region
// is written before it is read within the call.  An empty system writes zero
// totals and launches nothing.
// Concurrency: the array is shared by every context on the device, so two calls
// that overlap in time (other threads, other streams) race on it; callers must
// order them.
#include "common.cuh"

namespace pg {

void launch_bond_order_scratch(pg_context* ctx, int precision, int G, void* bonds, void* fc, F4* disp, FxAcc* acc,
                               double* out_f);

namespace {

static __device__ __align__(256) unsigned char g_scratch[PG_NOALLOC_SCRATCH_BYTES];

// the array's device address in the CUDA context current on the context's
// device, looked up on the context's first call (the host-side symbol is not
// a device address)
void* scratch_address(pg_context* ctx) {
    if (ctx->noalloc_scratch == nullptr) {
        void* p = nullptr;
        PG_CUDA(cudaGetSymbolAddress(&p, g_scratch));
        ctx->noalloc_scratch = p;
    }
    return ctx->noalloc_scratch;
}

size_t align256(size_t b) { return (b + 255) & ~(size_t)255; }

// the rounded totals: energy, then the virial (xx, yy, zz, yz, xz, xy)
__global__ void totals_to_double(const FxAcc* __restrict__ acc, double* __restrict__ out) {
    const int c = threadIdx.x;
    if (c < 7) out[c] = fx_to_double(fx_from_limbs(acc[c]));
}

}  // namespace

void bond_order_noalloc(pg_context* ctx, int precision, double* d_forces, double* d_totals) {
    require(precision == PG_PREC_FP64 || precision == PG_PREC_MIXED, PG_ERR_INVALID, "unknown precision");
    require(d_forces != nullptr && d_totals != nullptr, PG_ERR_INVALID, "null output pointer");
    require(ctx->have_bond_terms, PG_ERR_NOT_READY, "no bond-order factors");
    require(!ctx->have_pair_kernel_terms && !ctx->ewald && !ctx->have_singles && !ctx->have_triplets &&
                !ctx->have_bond_charge_terms,
            PG_ERR_UNSUPPORTED,
            "the no-allocation call covers contexts whose every term runs in the bond-order kernels "
            "(no Ewald, single-atom, out-of-bond pair or charge-dependent terms)");
    // everything the regular path builds lazily must already exist
    require(ctx->have_list && !ctx->tables_dirty && ctx->sep0_epoch == ctx->list_epoch && !ctx->short_dirty,
            PG_ERR_NOT_READY,
            "tables or lists are not prepared: evaluate once with pg_calculate after the last change, "
            "then use the no-allocation call");
    unsigned char* base = (unsigned char*)scratch_address(ctx);
    if (ctx->n == 0) {  // no atoms: zero totals, nothing to launch
        PG_CUDA(cudaMemsetAsync(d_totals, 0, 7 * sizeof(double), ctx->stream));
        return;
    }
    int G = ctx->lanes != 0 ? ctx->lanes : ctx->tuned_lanes[precision];
    if (G == 0) G = 8;
    const size_t n = (size_t)ctx->n;
    const size_t ne = (size_t)std::max<long long>(ctx->sh_total, 1);
    const size_t rec = precision == PG_PREC_FP64 ? sizeof(D4) : sizeof(F4);
    const size_t b_acc = align256(8 * sizeof(FxAcc));
    // the displacement records exist only in the mixed path
    const size_t b_disp = precision == PG_PREC_MIXED ? align256(n * sizeof(F4)) : 0;
    const size_t b_fc = align256(3 * n * sizeof(double));
    const size_t b_bonds = align256(4 * ne * rec);
    const size_t need = b_acc + b_disp + b_fc + b_bonds;
    if (need > (size_t)PG_NOALLOC_SCRATCH_BYTES)
        throw Error(PG_ERR_INVALID, "the no-allocation bond-order call needs " + std::to_string(need) +
                                        " bytes of scratch for this system; its static limit is " +
                                        std::to_string((size_t)PG_NOALLOC_SCRATCH_BYTES) + " bytes");
    FxAcc* acc = (FxAcc*)base;
    F4* disp = (F4*)(base + b_acc);
    void* fc = base + b_acc + b_disp;
    void* bonds = base + b_acc + b_disp + b_fc;
    PG_CUDA(cudaMemsetAsync(acc, 0, sizeof(FxAcc) * 8, ctx->stream));
    launch_bond_order_scratch(ctx, precision, G, bonds, fc, disp, acc, d_forces);
    totals_to_double<<<1, 32, 0, ctx->stream>>>(acc, d_totals);
    PG_CHECK_LAUNCH();
}

}  // namespace pg
