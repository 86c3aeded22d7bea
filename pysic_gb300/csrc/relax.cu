// relax.cu -- ChargeRelaxation 'dynamic' kept on the device.
//
// The reference loop (pysic/charges/relaxation.py:417-450) crosses into the
// Fortran core for every electronegativity evaluation and copies the arrays
// back each step.  Here one step is a fixed sequence of launches on the
// context's stream:
//
//   rx_update      q += q' dt + (F - gamma q') dt^2 / M ;  q' = (1 - gamma dt/2) q' + F dt / (2M)
//   electronegativity kernels (pair kernel + k-space Ewald) on the new q
//   rx_mean        mean(chi) over all atoms (deterministic FP64 sum)
//   rx_force       F = chi - mean ;  q' = (q' + F dt/(2M)) / (1 + gamma dt/2) ;  max F, max |dq|
//   rx_stop        error = max F (signed, relaxation.py:449); stop when error <= tol or steps reached
//
// Every kernel first reads a device flag and returns at once when the loop has
// stopped, so the host can enqueue a chunk of steps and read back only the
// flag and the statistics once per chunk.  Convergence statistics and charge
// sums are kept in FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"

namespace pg {

int pair_lanes_for(const pg_context* ctx);

namespace {

constexpr int RT = 256;

struct RxArgs {
    int n;
    double* q;
    double* rate;
    double* force;
    const double* chi;
    double dt, inv_m, friction, tol;
    int n_steps;
    int* flag;        // [0] stop flag, [1] steps taken
    double* stat;     // [0] error, [1] max |dq| of the last step, [2] mean chi
    double* part;     // per block: sum chi, max F, max |dq|
    int nblocks;
    F4* disp;         // mixed path: the FP32 charge copy in .w follows q (null: FP64 path)
};

__global__ void rx_update(RxArgs A) {
    __shared__ double sm[RT];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double dq = 0.0;
    if (i < A.n) {
        const double r = A.rate[i], f = A.force[i];
        dq = r * A.dt + (f - A.friction * r) * A.inv_m * A.dt * A.dt;
        const double q = A.q[i] + dq;
        A.q[i] = q;
        if (A.disp) A.disp[i].w = (float)q;
        A.rate[i] = (1.0 - 0.5 * A.friction * A.dt) * r + f * 0.5 * A.inv_m * A.dt;
    }
    sm[threadIdx.x] = fabs(dq);
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) A.part[3 * blockIdx.x + 2] = sm[0];
}

// mean of chi: per-block sums in rx_block_sums, then a single block adds them in order
__global__ void rx_block_sums(RxArgs A) {
    __shared__ double sm[RT];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    sm[threadIdx.x] = i < A.n ? A.chi[i] : 0.0;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] += sm[threadIdx.x + s];
        __syncthreads();
    }
    if (threadIdx.x == 0) A.part[3 * blockIdx.x] = sm[0];
}

__global__ void rx_mean(RxArgs A) {
    if (A.flag[0]) return;
    if (threadIdx.x == 0) {
        double s = 0.0, c = 0.0;
        for (int b = 0; b < A.nblocks; ++b) {
            const double y = A.part[3 * b] - c;
            const double t = s + y;
            c = (t - s) - y;
            s = t;
        }
        A.stat[2] = s / A.n;
    }
}

template <bool INIT>
__global__ void rx_force(RxArgs A) {
    __shared__ double sm[RT];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double f = -1e300;
    if (i < A.n) {
        f = A.chi[i] - A.stat[2];
        A.force[i] = f;
        // a non-finite force must not vanish in fmax (which drops NaN): it
        // becomes +inf, so the stop test sees it and the loop ends as diverged
        if (!isfinite(f)) f = __longlong_as_double(0x7ff0000000000000ll);
        if (!INIT) A.rate[i] = (A.rate[i] + f * 0.5 * A.inv_m * A.dt) / (1.0 + 0.5 * A.friction * A.dt);
    }
    sm[threadIdx.x] = f;
    __syncthreads();
    for (int s = blockDim.x / 2; s > 0; s >>= 1) {
        if (threadIdx.x < s) sm[threadIdx.x] = fmax(sm[threadIdx.x], sm[threadIdx.x + s]);
        __syncthreads();
    }
    if (threadIdx.x == 0) A.part[3 * blockIdx.x + 1] = sm[0];
}

__global__ void rx_stop(RxArgs A) {
    if (A.flag[0]) return;
    if (threadIdx.x == 0) {
        double e = -1e300, dq = 0.0;
        for (int b = 0; b < A.nblocks; ++b) {
            e = fmax(e, A.part[3 * b + 1]);
            dq = fmax(dq, A.part[3 * b + 2]);
        }
        const int steps = A.flag[1] + 1;
        A.flag[1] = steps;
        A.stat[0] = e;
        A.stat[1] = dq;
        // stop on convergence, on the step limit, or when the error is no
        // longer a finite number (diverging dynamics)
        if (e <= A.tol || steps >= A.n_steps || !isfinite(e)) A.flag[0] = 1;
    }
}

__global__ void rx_init_stat(RxArgs A) {
    if (threadIdx.x == 0) {
        double e = -1e300;
        for (int b = 0; b < A.nblocks; ++b) e = fmax(e, A.part[3 * b + 1]);
        A.stat[0] = e;
        A.stat[1] = 0.0;
    }
}

// The whole per-step bookkeeping in one block, for systems of up to
// FUSED_MAX atoms: mean of chi, forces and the second half of the rate update,
// the stop test and -- unless the loop stops -- the next step's charge update
// (so one step is the electronegativity kernels plus this one launch).  Same
// formulas and order of operations as rx_update ... rx_stop; sums in FP64 in a
// fixed order.  stat[3] carries the largest |dq| of the update to the next
// stop test.
constexpr int FUSED_THREADS = 1024;
constexpr int FUSED_MAX = 65536;

__device__ __forceinline__ double block_reduce(double v, bool is_max, double* sh) {
    const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
        const double u = __shfl_xor_sync(0xffffffffu, v, o);
        v = is_max ? fmax(v, u) : v + u;
    }
    __syncthreads();
    if (lane == 0) sh[w] = v;
    __syncthreads();
    if (w == 0) {
        v = lane < nw ? sh[lane] : (is_max ? -1e300 : 0.0);
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) {
            const double u = __shfl_xor_sync(0xffffffffu, v, o);
            v = is_max ? fmax(v, u) : v + u;
        }
        if (lane == 0) sh[0] = v;
    }
    __syncthreads();
    return sh[0];
}

template <bool INIT>
__global__ void __launch_bounds__(FUSED_THREADS) rx_fused(RxArgs A) {
    __shared__ double sh[32];
    __shared__ int s_stop;
    if (A.flag[0]) return;
    const int t = threadIdx.x, nt = blockDim.x;
    double s = 0.0;
    for (int i = t; i < A.n; i += nt) s += A.chi[i];
    const double mean = block_reduce(s, false, sh) / A.n;
    double e = -1e300;
    for (int i = t; i < A.n; i += nt) {
        double f = A.chi[i] - mean;
        A.force[i] = f;
        if (!INIT) A.rate[i] = (A.rate[i] + f * 0.5 * A.inv_m * A.dt) / (1.0 + 0.5 * A.friction * A.dt);
        if (!isfinite(f)) f = __longlong_as_double(0x7ff0000000000000ll);
        e = fmax(e, f);
    }
    e = block_reduce(e, true, sh);
    if (t == 0) {
        int stop;
        if (INIT) {
            A.stat[0] = e;
            A.stat[1] = 0.0;
            // the reference's loop starts from error = 2 tol and runs while error > tol
            stop = A.n_steps <= 0 || !(2.0 * A.tol > A.tol);
        } else {
            const int steps = A.flag[1] + 1;
            A.flag[1] = steps;
            A.stat[0] = e;
            A.stat[1] = A.stat[3];
            stop = e <= A.tol || steps >= A.n_steps || !isfinite(e);
        }
        if (stop) A.flag[0] = 1;
        s_stop = stop;
    }
    __syncthreads();
    if (s_stop) return;
    // the next step's update (rx_update)
    double dqm = 0.0;
    for (int i = t; i < A.n; i += nt) {
        const double r = A.rate[i], f = A.force[i];
        const double dq = r * A.dt + (f - A.friction * r) * A.inv_m * A.dt * A.dt;
        const double q = A.q[i] + dq;
        A.q[i] = q;
        if (A.disp) A.disp[i].w = (float)q;
        A.rate[i] = (1.0 - 0.5 * A.friction * A.dt) * r + f * 0.5 * A.inv_m * A.dt;
        dqm = fmax(dqm, fabs(dq));
    }
    dqm = block_reduce(dqm, true, sh);
    if (t == 0) A.stat[3] = dqm;
}

}  // namespace

// electronegativities of the current charges into ctx->out_chi, stopped by `skip`
static void enqueue_chi(pg_context* ctx, int precision, const int* skip) {
    const int G = pair_lanes_for(ctx);
    launch_pair_kernel_skip(ctx, precision, PG_WANT_ENEGS, true, true, G, nullptr, skip);
    if (ctx->ewald) launch_ewald_kspace_skip(ctx, precision, PG_WANT_ENEGS, true, false, nullptr, skip);
}

// results of a finished loop to the host; not converging is an error status
static void finish_relax(pg_context* ctx, const RxArgs& A, int n, double tolerance, double* rates, double* charges,
                         int* steps, double* error, double* max_dq) {
    cudaStream_t st = ctx->stream;
    int h_flag[2] = {0, 0};
    double h_stat[3] = {0.0, 0.0, 0.0};
    PG_CUDA(cudaMemcpyAsync(h_stat, A.stat, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(rates, A.rate, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(charges, A.q, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    *steps = h_flag[1];
    *error = h_stat[0];
    *max_dq = h_stat[1];
    if (!std::isfinite(h_stat[0]))
        throw Error(PG_ERR_NOT_CONVERGED, "charge relaxation diverged (non-finite electronegativity differences)");
    if (!(h_stat[0] <= tolerance))
        throw Error(PG_ERR_NOT_CONVERGED, "charge relaxation reached its step limit before the tolerance");
}

void relax_charges(pg_context* ctx, int precision, int n_steps, double dt, double inertia, double friction,
                   double tolerance, double* rates, double* charges, int* steps, double* error, double* max_dq) {
    require(ctx->have_list && ctx->have_atoms, PG_ERR_NOT_READY, "set atoms, potentials and lists first");
    prepare(ctx);
    const int n = ctx->n;
    cudaStream_t st = ctx->stream;
    const int nb = std::max(1, (n + RT - 1) / RT);
    ctx->out_chi.resize((size_t)std::max(n, 1));
    ctx->out_f.resize(3 * (size_t)std::max(n, 1));
    ctx->rq_rate.upload(rates, (size_t)n, st);
    ctx->rq_force.resize((size_t)std::max(n, 1));
    ctx->rq_stat.resize(4 + 3 * (size_t)nb);
    ctx->rq_flag.resize(2);
    PG_CUDA(cudaMemsetAsync(ctx->rq_flag.p, 0, sizeof(int) * 2, st));
    RxArgs A{};
    A.n = n;
    A.q = ctx->charge.p;
    A.rate = ctx->rq_rate.p;
    A.force = ctx->rq_force.p;
    A.chi = ctx->out_chi.p;
    A.dt = dt;
    A.inv_m = 1.0 / inertia;
    A.friction = friction;
    A.tol = tolerance;
    A.n_steps = n_steps;
    A.flag = ctx->rq_flag.p;
    A.stat = ctx->rq_stat.p;
    A.part = ctx->rq_stat.p + 4;
    A.nblocks = nb;
    ctx->launches = 0;
    // positions stay fixed during the relaxation: displacements (and the FP32
    // charges beside them) once; rx_update keeps the charges current
    if (precision == PG_PREC_MIXED) {
        launch_disp(ctx, nullptr);
        A.disp = ctx->disp32.p;
    }
    const bool fused = n <= FUSED_MAX;
    // initial differences (relaxation.py:433)
    enqueue_chi(ctx, precision, A.flag);
    if (fused) {
        rx_fused<true><<<1, FUSED_THREADS, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        // one step (electronegativity kernels + bookkeeping) as a CUDA graph,
        // replayed: every kernel of it checks the stop flag first.  The buffers
        // it uses were sized by the initial evaluation above.
        cudaGraphExec_t step = nullptr;
        if (ctx->use_graphs) {
            cudaGraph_t g = nullptr;
            PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                enqueue_chi(ctx, precision, A.flag);
                rx_fused<false><<<1, FUSED_THREADS, 0, st>>>(A);
            } catch (...) {
                cudaStreamEndCapture(st, &g);
                if (g) cudaGraphDestroy(g);
                throw;
            }
            PG_CUDA(cudaStreamEndCapture(st, &g));
            const cudaError_t e = cudaGraphInstantiate(&step, g, 0);
            cudaGraphDestroy(g);
            PG_CUDA(e);
        }
        struct Drop {
            cudaGraphExec_t& x;
            ~Drop() {
                if (x) cudaGraphExecDestroy(x);
            }
        } drop{step};
        int h_flag[2] = {0, 0};
        int chunk = 4;
        for (int c = 0; c < (1 << 20) && !h_flag[0]; ++c) {
            for (int k = 0; k < chunk; ++k) {
                if (step) {
                    PG_CUDA(cudaGraphLaunch(step, st));
                } else {
                    enqueue_chi(ctx, precision, A.flag);
                    rx_fused<false><<<1, FUSED_THREADS, 0, st>>>(A);
                }
            }
            PG_CHECK_LAUNCH();
            PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
            PG_CUDA(cudaStreamSynchronize(st));
            chunk = std::min(chunk * 2, 64);
        }
        finish_relax(ctx, A, n, tolerance, rates, charges, steps, error, max_dq);
        return;
    }
    rx_block_sums<<<nb, RT, 0, st>>>(A);
    rx_mean<<<1, 32, 0, st>>>(A);
    rx_force<true><<<nb, RT, 0, st>>>(A);
    rx_init_stat<<<1, 32, 0, st>>>(A);
    PG_CHECK_LAUNCH();
    int h_flag[2] = {0, 0};
    double h_stat[3] = {2.0 * tolerance, 0.0, 0.0};
    if (n_steps <= 0 || !(2.0 * tolerance > tolerance)) h_flag[0] = 1;
    // chunks of steps: all kernels test the stop flag, the host polls once per chunk
    int chunk = 4;
    const int max_launch_chunks = 1 << 20;
    for (int c = 0; c < max_launch_chunks && !h_flag[0]; ++c) {
        for (int s = 0; s < chunk; ++s) {
            rx_update<<<nb, RT, 0, st>>>(A);
            enqueue_chi(ctx, precision, A.flag);
            rx_block_sums<<<nb, RT, 0, st>>>(A);
            rx_mean<<<1, 32, 0, st>>>(A);
            rx_force<false><<<nb, RT, 0, st>>>(A);
            rx_stop<<<1, 32, 0, st>>>(A);
        }
        PG_CHECK_LAUNCH();
        PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
        chunk = std::min(chunk * 2, 64);
    }
    (void)h_stat;
    finish_relax(ctx, A, n, tolerance, rates, charges, steps, error, max_dq);
}

}  // namespace pg
