// md.cu -- velocity Verlet molecular dynamics kept on the device.
//
// The reference runs MD through ASE: VelocityVerlet.step (ase/md/verlet.py)
// reads the momenta, calls get_forces on the calculator -- a Python call into
// the core with a full copy of the positions and forces -- and writes the new
// positions back, every step.  Here the whole step stays on the device, with
// ASE's order of operations and rounding (no fused multiply-adds):
//
//   md_kick_drift   p += (dt/2) F;  r += (dt p) / m;  flag a neighbour-list
//                   rebuild when an atom has moved more than skin/2 since the
//                   list was built (the FastNeighborList / ASE update policy)
//   evaluation      the force kernels of one evaluation (skipped on the flag)
//   md_kick         p += (dt/2) F; count the step; stop at the target
//
// captured once as a CUDA graph and replayed in chunks; the host reads the
// flags once per chunk.  A rebuild request ends the loop after the drift, with
// the step's forces pending: the caller rebuilds the lists from the device
// positions and calls again, and the step is finished first (forces, second
// kick).  Momenta and masses live on the device between calls.
#include <algorithm>
#include <cmath>
#include <cstring>

#include "common.cuh"

namespace pg {

void enqueue_evaluation(pg_context* ctx, int precision, int flags, int G, const int* skip);

namespace {

constexpr int MT = 256;

struct MdArgs {
    int n;
    double* pos;
    const double* pos0;  // positions at the last list build
    double* p;           // momenta
    const double* m;     // masses
    const double* f;     // forces of the last evaluation
    double dt, half, skin2;
    // [0] skip the evaluation and the second kick, [1] rebuild requested,
    // [2] steps done, [3] target, [5] loop finished (read by the next drift)
    int* flag;
};

__global__ void __launch_bounds__(MT) md_kick_drift(MdArgs A) {
    if (A.flag[5]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const double mi = A.m[i];
    double d2 = 0.0;
    for (int c = 0; c < 3; ++c) {
        const int k = 3 * i + c;
        const double p = __dadd_rn(A.p[k], __dmul_rn(A.half, A.f[k]));
        A.p[k] = p;
        const double r = __dadd_rn(A.pos[k], __ddiv_rn(__dmul_rn(A.dt, p), mi));
        A.pos[k] = r;
        const double d = r - A.pos0[k];
        d2 += d * d;
    }
    // every thread that sees it writes the same values
    if (!(d2 <= A.skin2)) {
        A.flag[1] = 1;
        A.flag[0] = 1;
    }
}

__global__ void __launch_bounds__(MT) md_kick(MdArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (A.flag[0]) {  // stopped (rebuild or target): the next drift must not run
        if (i == 0) A.flag[5] = 1;
        return;
    }
    if (i < A.n)
        for (int c = 0; c < 3; ++c) {
            const int k = 3 * i + c;
            A.p[k] = __dadd_rn(A.p[k], __dmul_rn(A.half, A.f[k]));
        }
    if (i == 0) {
        const int s = A.flag[2] + 1;
        A.flag[2] = s;
        if (s >= A.flag[3]) {
            A.flag[0] = 1;
            A.flag[5] = 1;
        }
    }
}

// the second kick of a step left pending by a rebuild request
__global__ void __launch_bounds__(MT) md_finish_step(MdArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    for (int c = 0; c < 3; ++c) {
        const int k = 3 * i + c;
        A.p[k] = __dadd_rn(A.p[k], __dmul_rn(A.half, A.f[k]));
    }
}

}  // namespace

void md_set_state(pg_context* ctx, const double* masses, const double* momenta) {
    require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
    const size_t n = (size_t)ctx->n;
    for (size_t i = 0; i < n; ++i)
        require(std::isfinite(masses[i]) && masses[i] > 0.0, PG_ERR_INVALID, "masses must be positive");
    ctx->md_m.upload(masses, std::max<size_t>(n, 1), ctx->stream);
    ctx->md_p.upload(momenta, std::max<size_t>(3 * n, 1), ctx->stream);
    ctx->md_pending = false;
    ctx->md_ready = true;
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

void md_get_state(pg_context* ctx, double* momenta, double* positions) {
    require(ctx->md_ready, PG_ERR_NOT_READY, "no dynamics state: call pg_md_set_state first");
    const size_t n = (size_t)ctx->n;
    if (momenta) ctx->md_p.download(momenta, 3 * n, ctx->stream);
    if (positions) ctx->pos.download(positions, 3 * n, ctx->stream);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
}

void md_run(pg_context* ctx, int precision, int n_steps, double dt, double skin, int* steps_done, int* rebuild) {
    require(ctx->md_ready, PG_ERR_NOT_READY, "no dynamics state: call pg_md_set_state first");
    require(std::isfinite(dt) && std::isfinite(skin) && skin >= 0.0, PG_ERR_INVALID, "invalid time step or skin");
    *steps_done = 0;
    *rebuild = 0;
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    const int flags = PG_WANT_FORCES;
    // one ordinary evaluation: the forces at the current positions (and the
    // lanes, buffers and tables every later launch uses)
    evaluate(ctx, precision, flags);
    if (n == 0 || n_steps <= 0) {
        PG_CUDA(cudaStreamSynchronize(st));
        return;
    }
    int G = ctx->lanes != 0 ? ctx->lanes : ctx->tuned_lanes[precision];
    if (G == 0) G = 8;
    ctx->md_flag.resize(8);
    PG_CUDA(cudaMemsetAsync(ctx->md_flag.p, 0, sizeof(int) * 8, st));
    MdArgs A{};
    A.n = n;
    A.pos = ctx->pos.p;
    A.pos0 = ctx->pos0.p;
    A.p = ctx->md_p.p;
    A.m = ctx->md_m.p;
    A.f = ctx->out_f.p;
    A.dt = dt;
    A.half = 0.5 * dt;
    A.skin2 = (0.5 * skin) * (0.5 * skin);
    A.flag = ctx->md_flag.p;
    const int nb = (n + MT - 1) / MT;
    int done = 0;
    // a step left pending by a rebuild: its forces were just evaluated
    if (ctx->md_pending) {
        md_finish_step<<<nb, MT, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        ctx->md_pending = false;
        done = 1;
    }
    const int target = n_steps - done;
    if (target > 0) {
        PG_CUDA(cudaMemcpyAsync(A.flag + 3, &target, sizeof(int), cudaMemcpyHostToDevice, st));
        auto one_step = [&] {
            md_kick_drift<<<nb, MT, 0, st>>>(A);
            enqueue_evaluation(ctx, precision, flags, G, A.flag);
            md_kick<<<nb, MT, 0, st>>>(A);
        };
        cudaGraphExec_t graph = nullptr;
        struct Drop {
            cudaGraphExec_t& x;
            ~Drop() {
                if (x) cudaGraphExecDestroy(x);
            }
        } drop{graph};
        if (ctx->use_graphs) {
            cudaGraph_t g = nullptr;
            PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                one_step();
            } catch (...) {
                cudaStreamEndCapture(st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            PG_CUDA(cudaStreamEndCapture(st, &g));
            const cudaError_t e = cudaGraphInstantiate(&graph, g, 0);
            cudaGraphDestroy(g);
            PG_CUDA(e);
        }
        int h[6] = {0, 0, 0, 0, 0, 0};
        int chunk = 4;
        for (int launched = 0; !h[5] && launched < target;) {
            const int k = std::min(chunk, target - launched);
            for (int s = 0; s < k; ++s) {
                if (graph) PG_CUDA(cudaGraphLaunch(graph, st));
                else one_step();
            }
            launched += k;
            PG_CHECK_LAUNCH();
            PG_CUDA(cudaMemcpyAsync(h, A.flag, sizeof(h), cudaMemcpyDeviceToHost, st));
            PG_CUDA(cudaStreamSynchronize(st));
            chunk = std::min(2 * chunk, 64);
        }
        done += h[2];
        if (h[1]) {
            *rebuild = 1;
            ctx->md_pending = true;
        }
    }
    PG_CUDA(cudaStreamSynchronize(st));
    *steps_done = done;
}

// The lists again from the device coordinates, with the cutoffs and the
// builder of the last build (the rebuild FastNeighborList makes when an atom
// has moved more than skin/2, calculator.py:29-189), then the list
// generation's reference positions and bond vectors and the short list.
static void rebuild_lists(pg_context* ctx) {
    require(ctx->list_kind == PG_LIST_CELLS || ctx->list_kind == PG_LIST_ALL_PAIRS, PG_ERR_NOT_READY,
            "the lists were installed from the host: rebuild them there (pg_md_verlet)");
    if (ctx->list_kind == PG_LIST_CELLS) build_neighbor_lists(ctx, ctx->h_cutoffs.data());
    else build_allpairs_lists(ctx, ctx->h_cutoffs.data());
    build_full_sep0(ctx);
    if (ctx->have_bond_terms) build_short_list(ctx, true);
}

// what the captured step's kernel arguments depend on beyond the context's
// fixed state: buffer addresses (any growth moves them), the pair kernel's lanes
// and the sections of the bond-pass scratch
static unsigned long long step_signature(const pg_context* ctx, int precision, int G) {
    unsigned long long h = alloc_epoch();
    h = h * 1000003ull + (unsigned long long)pair_lanes_for(ctx);
    h = h * 1000003ull + (unsigned long long)ctx->bo_stride;
    h = h * 1000003ull + (unsigned long long)(precision * 131 + G);
    return h;
}

void md_run_rebuilding(pg_context* ctx, int precision, int n_steps, double dt, double skin, int* steps_done,
                       int* rebuilds) {
    require(ctx->md_ready, PG_ERR_NOT_READY, "no dynamics state: call pg_md_set_state first");
    require(std::isfinite(dt) && std::isfinite(skin) && skin >= 0.0, PG_ERR_INVALID, "invalid time step or skin");
    require(ctx->list_kind == PG_LIST_CELLS || ctx->list_kind == PG_LIST_ALL_PAIRS, PG_ERR_NOT_READY,
            "the lists were installed from the host: run pg_md_verlet and rebuild them there");
    *steps_done = 0;
    *rebuilds = 0;
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    const int flags = PG_WANT_FORCES;
    int done = 0, nreb = 0;
    // a step left pending by pg_md_verlet: rebuild here and finish it
    if (ctx->md_pending) {
        rebuild_lists(ctx);
        ++nreb;
    }
    // the forces at the current positions (and the lanes, buffers and tables
    // every later launch uses)
    evaluate(ctx, precision, flags);
    if (n == 0 || n_steps <= 0) {
        PG_CUDA(cudaStreamSynchronize(st));
        *rebuilds = nreb;
        return;
    }
    int G = ctx->lanes != 0 ? ctx->lanes : ctx->tuned_lanes[precision];
    if (G == 0) G = 8;
    ctx->md_flag.resize(8);
    MdArgs A{};
    A.n = n;
    A.pos = ctx->pos.p;
    A.pos0 = ctx->pos0.p;
    A.p = ctx->md_p.p;
    A.m = ctx->md_m.p;
    A.f = ctx->out_f.p;
    A.dt = dt;
    A.half = 0.5 * dt;
    A.skin2 = (0.5 * skin) * (0.5 * skin);
    A.flag = ctx->md_flag.p;
    const int nb = (n + MT - 1) / MT;
    if (ctx->md_pending) {
        md_finish_step<<<nb, MT, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        ctx->md_pending = false;
        done = 1;
    }
    auto one_step = [&] {
        md_kick_drift<<<nb, MT, 0, st>>>(A);
        enqueue_evaluation(ctx, precision, flags, G, A.flag);
        md_kick<<<nb, MT, 0, st>>>(A);
    };
    // the step graph: kept by the context, refreshed (cudaGraphExecUpdate, or
    // instantiated anew) only when what its arguments come from has changed
    auto refresh_graph = [&] {
        if (!ctx->use_graphs) return;
        A.pos0 = ctx->pos0.p;
        A.f = ctx->out_f.p;
        unsigned long long bits[2];
        std::memcpy(&bits[0], &A.dt, sizeof(double));
        std::memcpy(&bits[1], &A.skin2, sizeof(double));
        const unsigned long long sig = (step_signature(ctx, precision, G) * 1000003ull + bits[0]) * 1000003ull + bits[1];
        if (ctx->md_exec && ctx->md_sig == sig) return;
        cudaGraph_t g = nullptr;
        PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
        try {
            one_step();
        } catch (...) {
            cudaStreamEndCapture(st, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        PG_CUDA(cudaStreamEndCapture(st, &g));
        bool updated = false;
        if (ctx->md_exec) {
            cudaGraphExecUpdateResultInfo info{};
            updated = cudaGraphExecUpdate(ctx->md_exec, g, &info) == cudaSuccess;
            if (!updated) {
                (void)cudaGetLastError();  // a failed update leaves no sticky error
                cudaGraphExecDestroy(ctx->md_exec);
                ctx->md_exec = nullptr;
            }
        }
        if (!updated) {
            const cudaError_t e = cudaGraphInstantiate(&ctx->md_exec, g, 0);
            if (e != cudaSuccess) ctx->md_exec = nullptr;
            cudaGraphDestroy(g);
            PG_CUDA(e);
        } else {
            cudaGraphDestroy(g);
        }
        ctx->md_sig = sig;
    };
    // flags: [0] skip, [1] rebuild requested, [2] steps done, [3] target, [5] finished
    int* hf = ctx->h_flag.get(8);
    std::fill(hf, hf + 8, 0);
    hf[2] = done;
    hf[3] = n_steps;
    PG_CUDA(cudaMemcpyAsync(A.flag, hf, sizeof(int) * 8, cudaMemcpyHostToDevice, st));
    refresh_graph();
    int chunk = 8, since = 0;
    while (done < n_steps) {
        const int k = std::max(1, std::min(chunk, n_steps - done));
        for (int s = 0; s < k; ++s) {
            if (ctx->md_exec) PG_CUDA(cudaGraphLaunch(ctx->md_exec, st));
            else one_step();
        }
        PG_CHECK_LAUNCH();
        PG_CUDA(cudaMemcpyAsync(hf, A.flag, sizeof(int) * 8, cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
        since += hf[2] - done;
        done = hf[2];
        if (!hf[5]) {  // the chunk ran through
            chunk = std::min(2 * chunk, 64);
            continue;
        }
        if (!hf[1]) break;  // the target reached
        // an atom moved more than skin/2: new lists at the drifted positions,
        // then the step's forces and second kick, then on
        rebuild_lists(ctx);
        ++nreb;
        enqueue_evaluation(ctx, precision, flags, G, nullptr);
        md_finish_step<<<nb, MT, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        ++done;
        chunk = std::max(2, std::min(since, 64));  // about one list generation per chunk
        since = 0;
        std::fill(hf, hf + 8, 0);
        hf[2] = done;
        hf[3] = n_steps;
        PG_CUDA(cudaMemcpyAsync(A.flag, hf, sizeof(int) * 8, cudaMemcpyHostToDevice, st));
        refresh_graph();
    }
    PG_CUDA(cudaStreamSynchronize(st));
    *steps_done = done;
    *rebuilds = nreb;
}

}  // namespace pg
