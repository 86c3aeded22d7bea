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

}  // namespace pg
