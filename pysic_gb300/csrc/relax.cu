// relax.cu -- ChargeRelaxation 'dynamic' kept on the device.
//
// The reference loop (pysic/charges/relaxation.py:417-450) crosses into the
// Fortran core for every electronegativity evaluation and copies the arrays
// back each step.  Here one step is a fixed sequence of launches on the
// context's stream, captured once as a CUDA graph and replayed:
//
//   electronegativity kernels (pair kernel + k-space Ewald) on the current q
//   rx_mean    block sums of chi; the last block to finish forms mean(chi)
//   rx_step    F = chi - mean;  q' = (q' + F dt/(2M)) / (1 + gamma dt/2);
//              save (q, q') as the result of this step, then already
//              q += q' dt + (F - gamma q') dt^2 / M;  q' = (1 - gamma dt/2) q' + F dt / (2M);
//              the last block takes error = max F (signed, relaxation.py:449)
//              and decides: stop when error <= tol, at the step limit, or when
//              the error is not finite (diverging dynamics)
//
// The initial pass (relaxation.py:433) is the electronegativities, rx_mean and
// rx_step<INIT>.  Every kernel first reads a device flag and returns at once
// when the loop has stopped, so the host enqueues chunks of steps and reads
// back only the flag once per chunk; the saved (q, q') of the stopping step
// are the result.  The "last block" of a kernel is found with an integer
// ticket (an atomic counter, no waiting); it combines the per-block partials
// in block order, so every statistic is deterministic.  Charges, rates and
// statistics are FP64.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"

namespace pg {

int pair_lanes_for(const pg_context* ctx);

namespace {

constexpr int RT = 256;

struct RxArgs {
    int n;
    double* q;
    double* rate;
    double* q_save;   // q and q' at the last stop test: the result when the loop stops
    double* rate_save;
    const double* chi;
    // the reference's coefficients, formed on the host in its order of
    // operations: dt^2, 1 - gamma dt / 2, 1 / (1 + gamma dt / 2), 1 / (2 M)
    double dt, dt2, inv_m, half_inv_m, friction, c_half, future, tol;
    double potential;  // potentiostat: the external potential that replaces mean(chi)
    int potentiostat;  // 1: fixed step count, no tolerance test (relaxation.py:453-481)
    int n_steps;
    int* flag;        // [0] stop flag, [1] steps taken, [2], [3] tickets of rx_mean, rx_step
    double* stat;     // [0] error, [1] max |dq| reported, [2] mean chi, [3] max |dq| of the last update
    double* part;     // per block: sum chi, max F, max |dq|
    int nblocks;
    F4* disp;         // mixed path: the FP32 charge copy in .w follows q (null: FP64 path)
};

__global__ void __launch_bounds__(RT) rx_mean(RxArgs A) {
    __shared__ double sh[RT / 32];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double s = block_reduce(i < A.n ? A.chi[i] : 0.0, false, sh);
    if (threadIdx.x == 0) A.part[3 * blockIdx.x] = s;
    if (last_block(A.flag + 2)) {
        const volatile double* p = A.part;
        double t = 0.0;
        for (int b = 0; b < A.nblocks; ++b) t += p[3 * b];
        A.stat[2] = t / A.n;
    }
}

// Forces, the second half of the rate update, the stop test and -- without
// waiting for the test -- the next update.  Before updating, each atom saves
// its charge and its completed rate: they are the loop's result if the last
// block decides to stop here, and the speculative update is then simply never
// used (every later kernel sees the flag and returns).
template <bool INIT>
__global__ void __launch_bounds__(RT) rx_step(RxArgs A) {
    __shared__ double sh[RT / 32];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double fm = -1e300, dq = 0.0;
    if (i < A.n) {
        // the reference's formulas, rounded after every operation as NumPy
        // does (no contraction into fused multiply-adds)
        const double f = __dsub_rn(A.chi[i], A.potentiostat ? A.potential : A.stat[2]);
        const double half = __dmul_rn(__dmul_rn(f, A.half_inv_m), A.dt);  // F / (2 M) dt
        double r = A.rate[i];
        if (!INIT) r = __dmul_rn(A.future, __dadd_rn(r, half));
        const double q0 = A.q[i];
        A.q_save[i] = q0;
        A.rate_save[i] = r;
        dq = __dadd_rn(__dmul_rn(r, A.dt),
                       __dmul_rn(__dmul_rn(__dsub_rn(f, __dmul_rn(A.friction, r)), A.inv_m), A.dt2));
        const double q = __dadd_rn(q0, dq);
        A.q[i] = q;
        if (A.disp) A.disp[i].w = (float)q;
        A.rate[i] = __dadd_rn(__dmul_rn(A.c_half, r), half);
        // a non-finite force must not vanish in fmax (which drops NaN): it
        // becomes +inf, so the stop test sees it and the loop ends as diverged
        fm = isfinite(f) ? f : __longlong_as_double(0x7ff0000000000000ll);
    }
    const double m = block_reduce(fm, true, sh);
    __syncthreads();
    const double d = block_reduce(fabs(dq), true, sh);
    if (threadIdx.x == 0) {
        A.part[3 * blockIdx.x + 1] = m;
        A.part[3 * blockIdx.x + 2] = d;
    }
    if (last_block(A.flag + 3)) {
        const volatile double* p = A.part;
        double e = -1e300, dmax = 0.0;
        for (int b = 0; b < A.nblocks; ++b) {
            e = fmax(e, p[3 * b + 1]);
            dmax = fmax(dmax, p[3 * b + 2]);
        }
        int stop;
        if (INIT) {
            A.stat[1] = 0.0;
            // the reference's loop starts from error = 2 tol and runs while error > tol
            stop = A.n_steps <= 0 || (!A.potentiostat && !(2.0 * A.tol > A.tol));
        } else {
            const int steps = A.flag[1] + 1;
            A.flag[1] = steps;
            A.stat[1] = A.stat[3];  // |dq| of the update that led to these charges
            stop = (!A.potentiostat && e <= A.tol) || steps >= A.n_steps || !isfinite(e);
        }
        A.stat[0] = e;
        A.stat[3] = dmax;
        if (stop) A.flag[0] = 1;
    }
}

}  // namespace

// electronegativities of the current charges into ctx->out_chi, stopped by `skip`
// (the real-space part from the loop's cached matrix when it has one)
static void enqueue_chi(pg_context* ctx, int precision, const int* skip, bool cached) {
    if (cached) {
        launch_chi_cache_apply(ctx, precision, skip);
    } else {
        const int G = pair_lanes_for(ctx);
        launch_pair_kernel_skip(ctx, precision, PG_WANT_ENEGS, true, true, G, nullptr, skip);
    }
    if (ctx->ewald) launch_ewald_kspace_skip(ctx, precision, PG_WANT_ENEGS, true, false, nullptr, skip);
    // Tersoff-scaled charge terms: B of every bond is fixed while the
    // positions are, kept from the loop's start
    if (ctx->have_bond_charge_terms) launch_bond_chi(ctx, precision, false, skip);
}

// results of a finished loop to the host; not converging is an error status
static void finish_relax(pg_context* ctx, const RxArgs& A, int n, double tolerance, double* rates, double* charges,
                         int* steps, double* error, double* max_dq) {
    cudaStream_t st = ctx->stream;
    int h_flag[2] = {0, 0};
    double h_stat[3] = {0.0, 0.0, 0.0};
    PG_CUDA(cudaMemcpyAsync(h_stat, A.stat, sizeof(double) * 3, cudaMemcpyDeviceToHost, st));
    // the state saved at the stopping test; the context keeps those charges
    PG_CUDA(cudaMemcpyAsync(A.q, A.q_save, sizeof(double) * n, cudaMemcpyDeviceToDevice, st));
    PG_CUDA(cudaMemcpyAsync(rates, A.rate_save, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(charges, A.q_save, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
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

void relax_charges(pg_context* ctx, int precision, int mode, int n_steps, double dt, double inertia, double friction,
                   double tolerance, double potential, double* rates, double* charges, int* steps, double* error,
                   double* max_dq) {
    require(ctx->have_list && ctx->have_atoms, PG_ERR_NOT_READY, "set atoms, potentials and lists first");
    prepare(ctx);
    const int n = ctx->n;
    if (n == 0) {  // nothing to relax
        *steps = 0;
        *error = 0.0;
        *max_dq = 0.0;
        return;
    }
    cudaStream_t st = ctx->stream;
    const int nb = std::max(1, (n + RT - 1) / RT);
    ctx->out_chi.resize((size_t)std::max(n, 1));
    ctx->out_f.resize(3 * (size_t)std::max(n, 1));
    ctx->rq_rate.upload(rates, (size_t)n, st);
    ctx->rq_save.resize(2 * (size_t)std::max(n, 1));
    ctx->rq_stat.resize(4 + 3 * (size_t)nb);
    ctx->rq_flag.resize(8);
    // stop flag, step count and the tickets start at zero
    PG_CUDA(cudaMemsetAsync(ctx->rq_flag.p, 0, sizeof(int) * 8, st));
    RxArgs A{};
    A.n = n;
    A.q = ctx->charge.p;
    A.rate = ctx->rq_rate.p;
    A.q_save = ctx->rq_save.p;
    A.rate_save = ctx->rq_save.p + std::max(n, 1);
    A.chi = ctx->out_chi.p;
    const bool pstat = mode == PG_RELAX_POTENTIOSTAT;
    A.dt = dt;
    A.dt2 = dt * dt;
    A.inv_m = 1.0 / inertia;
    A.half_inv_m = 0.5 * A.inv_m;  // F * 0.5 * (1/M) rounds like F * (0.5 / M): 0.5 scales exactly
    A.friction = pstat ? 0.0 : friction;
    A.c_half = 1.0 - 0.5 * A.friction * dt;
    A.future = 1.0 / (1.0 + 0.5 * A.friction * dt);
    A.tol = tolerance;
    A.potential = potential;
    A.potentiostat = pstat ? 1 : 0;
    A.n_steps = n_steps;
    A.flag = ctx->rq_flag.p;
    A.stat = ctx->rq_stat.p;
    A.part = ctx->rq_stat.p + 4;
    A.nblocks = nb;
    ctx->launches = 0;
    // positions stay fixed during the relaxation: displacements (and the FP32
    // charges beside them) once; rx_step keeps the charges current
    if (precision == PG_PREC_MIXED) {
        launch_disp(ctx, nullptr);
        A.disp = ctx->disp32.p;
    }
    const bool cached = chi_cache_prepare(ctx, precision);
    if (ctx->have_bond_charge_terms) {  // the bonds' B, fixed with the positions
        int G = ctx->lanes != 0 ? ctx->lanes : ctx->tuned_lanes[precision];
        launch_bond_b(ctx, precision, G == 0 ? 8 : G, nullptr);
    }
    // initial differences (relaxation.py:433) and the first update; the
    // potentiostat subtracts its fixed potential instead of the mean
    enqueue_chi(ctx, precision, A.flag, cached);
    if (!pstat) rx_mean<<<nb, RT, 0, st>>>(A);
    rx_step<true><<<nb, RT, 0, st>>>(A);
    PG_CHECK_LAUNCH();
    auto one_step = [&] {
        enqueue_chi(ctx, precision, A.flag, cached);
        if (!pstat) rx_mean<<<nb, RT, 0, st>>>(A);
        rx_step<false><<<nb, RT, 0, st>>>(A);
    };
    // one step as a CUDA graph, replayed; the buffers it uses were sized by the
    // initial pass above
    cudaGraphExec_t step = nullptr;
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
            if (step) PG_CUDA(cudaGraphLaunch(step, st));
            else one_step();
        }
        PG_CHECK_LAUNCH();
        PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
        chunk = std::min(chunk * 2, 64);
    }
    finish_relax(ctx, A, n, pstat ? INFINITY : tolerance, rates, charges, steps, error, max_dq);
}

}  // namespace pg
