// optimize.cu -- ChargeRelaxation 'optimize' on the device.
//
// The reference minimises the energy over the charges at fixed total charge
// with SciPy's SLSQP (pysic/charges/relaxation.py:483-488), one Python call
// into the core per energy and per gradient.  When the energy is quadratic in
// the charges -- Ewald Coulomb and charge_self terms eps q^n with n <= 2, the
// charge-dependent terms this engine evaluates -- the constrained minimum is
// the solution of a linear system, found here by projected conjugate gradients
// without leaving the device:
//
//   chi(q) = -dE/dq is affine: chi(q) = c0 - H q, c0 = chi(0), H p = c0 - chi(p)
//   residual r = chi(q) - mean(chi(q))        (the gradient projected on sum q = const)
//   p = r + beta p;  alpha = r.r / p.H p;  q += alpha p;  r -= alpha (H p - mean(H p))
//
// One iteration is one electronegativity evaluation (on the direction p, which
// stands in for the charges meanwhile) and three small kernels, replayed from
// a CUDA graph; every kernel reads a stop flag first, so the host polls once
// per chunk.  The loop stops when max |r| <= tolerance or after max_iter
// iterations; the true residual is then recomputed and the iteration restarted
// from the current charges if the recursive one had drifted.  Reductions run
// in a fixed order (reduce.cuh).  A direction of non-positive curvature stops
// the loop with an error: the energy has no minimum.
#include <algorithm>
#include <cmath>
#include <vector>

#include "common.cuh"
#include "reduce.cuh"

namespace pg {

int pair_lanes_for(const pg_context* ctx);

namespace {

constexpr int OT = 256;

struct CgArgs {
    int n, nblocks, max_iter;
    double tol;
    double* q;        // the iterate
    double* r;        // projected residual
    double* p;        // search direction
    double* hp;       // H p
    double* c0;       // chi(0)
    double* charge;   // the context's charges: the kernels before read them
    F4* disp;         // mixed path: FP32 charge copy in .w (null: FP64 path)
    const double* chi;
    double* part;     // per block: 2 partials
    double* stat;     // [0] r.r, [1] alpha, [2] beta, [3] mean H p, [4] max |r|, [5] mean chi, [6] p.H p
    int* flag;        // [0] stop, [1] iterations, [2] curvature failure, [3..5] tickets
};

__device__ __forceinline__ void set_charge(const CgArgs& A, int i, double v) {
    A.charge[i] = v;
    if (A.disp) A.disp[i].w = (float)v;
}

// q = charges; the charges become 0 (for chi(0))
__global__ void __launch_bounds__(OT) cg_begin(CgArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    A.q[i] = A.charge[i];
    set_charge(A, i, 0.0);
}

// c0 = chi(0); the charges back to q
__global__ void __launch_bounds__(OT) cg_c0(CgArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    A.c0[i] = A.chi[i];
    set_charge(A, i, A.q[i]);
}

// mean of chi (ticket 3)
__global__ void __launch_bounds__(OT) cg_mean(CgArgs A) {
    __shared__ double sh[OT / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double s = block_reduce(i < A.n ? A.chi[i] : 0.0, false, sh);
    if (threadIdx.x == 0) A.part[2 * blockIdx.x] = s;
    if (last_block(A.flag + 3)) {
        const volatile double* p = A.part;
        double t = 0.0;
        for (int b = 0; b < A.nblocks; ++b) t += p[2 * b];
        A.stat[5] = t / A.n;
    }
}

// r = chi(q) - mean, p = 0, beta = 0; r.r and max |r|; stop test (ticket 4).
// The iteration count carries over from earlier rounds.
__global__ void __launch_bounds__(OT) cg_start(CgArgs A) {
    __shared__ double sh[OT / 32];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double r = 0.0;
    if (i < A.n) {
        r = A.chi[i] - A.stat[5];
        A.r[i] = r;
        A.p[i] = 0.0;
    }
    const double rr = block_reduce(r * r, false, sh);
    __syncthreads();
    const double rm = block_reduce(isfinite(r) ? fabs(r) : INFINITY, true, sh);
    if (threadIdx.x == 0) {
        A.part[2 * blockIdx.x] = rr;
        A.part[2 * blockIdx.x + 1] = rm;
    }
    if (last_block(A.flag + 4)) {
        const volatile double* p = A.part;
        double t = 0.0, m = 0.0;
        for (int b = 0; b < A.nblocks; ++b) {
            t += p[2 * b];
            m = fmax(m, p[2 * b + 1]);
        }
        A.stat[0] = t;
        A.stat[2] = 0.0;
        A.stat[4] = m;
        A.flag[0] = (m <= A.tol || A.flag[1] >= A.max_iter || !isfinite(m)) ? 1 : 0;
    }
}

// p = r + beta p; the charges become p (for H p = c0 - chi(p))
__global__ void __launch_bounds__(OT) cg_dir(CgArgs A) {
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= A.n) return;
    const double p = A.r[i] + A.stat[2] * A.p[i];
    A.p[i] = p;
    set_charge(A, i, p);
}

// H p, p.H p and mean(H p); alpha (ticket 3)
__global__ void __launch_bounds__(OT) cg_curv(CgArgs A) {
    __shared__ double sh[OT / 32];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double php = 0.0, h = 0.0;
    if (i < A.n) {
        h = A.c0[i] - A.chi[i];
        A.hp[i] = h;
        php = A.p[i] * h;
    }
    const double a = block_reduce(php, false, sh);
    __syncthreads();
    const double b = block_reduce(h, false, sh);
    if (threadIdx.x == 0) {
        A.part[2 * blockIdx.x] = a;
        A.part[2 * blockIdx.x + 1] = b;
    }
    if (last_block(A.flag + 3)) {
        const volatile double* p = A.part;
        double t = 0.0, s = 0.0;
        for (int k = 0; k < A.nblocks; ++k) {
            t += p[2 * k];
            s += p[2 * k + 1];
        }
        A.stat[6] = t;
        A.stat[3] = s / A.n;
        if (!(t > 0.0)) {  // no positive curvature along p: the energy has no minimum
            A.flag[2] = 1;
            A.flag[0] = 1;
        } else {
            A.stat[1] = A.stat[0] / t;
        }
    }
}

// q += alpha p, r -= alpha (H p - mean), the new r.r, beta and the stop test
// (ticket 5); the charges are restored from q when the loop stops
__global__ void __launch_bounds__(OT) cg_step(CgArgs A) {
    __shared__ double sh[OT / 32];
    if (A.flag[0]) return;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const double alpha = A.stat[1], mh = A.stat[3];
    double r = 0.0;
    if (i < A.n) {
        A.q[i] += alpha * A.p[i];
        r = A.r[i] - alpha * (A.hp[i] - mh);
        A.r[i] = r;
    }
    const double rr = block_reduce(r * r, false, sh);
    __syncthreads();
    const double rm = block_reduce(isfinite(r) ? fabs(r) : INFINITY, true, sh);
    if (threadIdx.x == 0) {
        A.part[2 * blockIdx.x] = rr;
        A.part[2 * blockIdx.x + 1] = rm;
    }
    if (last_block(A.flag + 5)) {
        const volatile double* p = A.part;
        double t = 0.0, m = 0.0;
        for (int b = 0; b < A.nblocks; ++b) {
            t += p[2 * b];
            m = fmax(m, p[2 * b + 1]);
        }
        const int it = A.flag[1] + 1;
        A.flag[1] = it;
        A.stat[2] = t / A.stat[0];
        A.stat[0] = t;
        A.stat[4] = m;
        if (m <= A.tol || it >= A.max_iter || !isfinite(m)) A.flag[0] = 1;
    }
}

// the charges back to the iterate
__global__ void __launch_bounds__(OT) cg_restore(CgArgs A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < A.n) set_charge(A, i, A.q[i]);
}

}  // namespace

// electronegativities of the current charges; the real-space part from the
// cached matrix of the loop (charge_pair terms are excluded here)
static void enqueue_chi_skip(pg_context* ctx, int precision, const int* skip) {
    launch_chi_cache_apply(ctx, precision, skip);
    if (ctx->ewald) launch_ewald_kspace_skip(ctx, precision, PG_WANT_ENEGS, true, false, nullptr, skip);
}

static void enqueue_chi_on(pg_context* ctx, int precision) { enqueue_chi_skip(ctx, precision, nullptr); }

void optimize_charges(pg_context* ctx, int precision, int max_iter, double tolerance, double* charges, int* iterations,
                      double* error) {
    require(ctx->have_list && ctx->have_atoms, PG_ERR_NOT_READY, "set atoms, potentials and lists first");
    for (size_t r = 0; r < ctx->sr_kind.size(); ++r) {
        const int nq = (int)ctx->sr_params[4 * r + 1];
        require(ctx->sr_kind[r] != 0 || (nq >= 0 && nq <= 2), PG_ERR_UNSUPPORTED,
                "charge optimisation on the device needs an energy quadratic in the charges (charge_self n <= 2)");
    }
    prepare(ctx);
    require(!ctx->have_charge_pairs, PG_ERR_UNSUPPORTED,
            "charge optimisation on the device needs an energy quadratic in the charges (no charge_pair terms)");
    const int n = ctx->n;
    *iterations = 0;
    *error = 0.0;
    if (n == 0) return;
    cudaStream_t st = ctx->stream;
    const int nb = (n + OT - 1) / OT;
    ctx->out_chi.resize((size_t)n);
    ctx->out_f.resize(3 * (size_t)n);
    ctx->cg_buf.resize(5 * (size_t)n + 2 * (size_t)nb + 8);
    ctx->cg_flag.resize(8);
    PG_CUDA(cudaMemsetAsync(ctx->cg_flag.p, 0, sizeof(int) * 8, st));
    CgArgs A{};
    A.n = n;
    A.nblocks = nb;
    A.max_iter = max_iter;
    A.tol = tolerance;
    double* b = ctx->cg_buf.p;
    A.q = b;
    A.r = b + n;
    A.p = b + 2 * (size_t)n;
    A.hp = b + 3 * (size_t)n;
    A.c0 = b + 4 * (size_t)n;
    A.part = b + 5 * (size_t)n;
    A.stat = A.part + 2 * (size_t)nb;
    A.charge = ctx->charge.p;
    A.chi = ctx->out_chi.p;
    A.flag = ctx->cg_flag.p;
    ctx->launches = 0;
    // positions stay fixed: the displacements once; cg kernels keep .w current
    if (precision == PG_PREC_MIXED) {
        launch_disp(ctx, nullptr);
        A.disp = ctx->disp32.p;
    }
    require(chi_cache_prepare(ctx, precision), PG_ERR_UNSUPPORTED, "charge optimisation needs a linear chi");
    // c0 = chi(0)
    cg_begin<<<nb, OT, 0, st>>>(A);
    enqueue_chi_on(ctx, precision);
    cg_c0<<<nb, OT, 0, st>>>(A);
    PG_CHECK_LAUNCH();
    auto one_iter = [&] {
        cg_dir<<<nb, OT, 0, st>>>(A);
        enqueue_chi_skip(ctx, precision, A.flag);
        cg_curv<<<nb, OT, 0, st>>>(A);
        cg_step<<<nb, OT, 0, st>>>(A);
    };
    cudaGraphExec_t graph = nullptr;
    struct Drop {
        cudaGraphExec_t& x;
        ~Drop() {
            if (x) cudaGraphExecDestroy(x);
        }
    } drop{graph};
    int h_flag[3] = {0, 0, 0};
    // rounds: start from the true residual of the current charges
    for (int round = 0; round < 8; ++round) {
        enqueue_chi_on(ctx, precision);  // chi(q)
        cg_mean<<<nb, OT, 0, st>>>(A);
        cg_start<<<nb, OT, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
        PG_CUDA(cudaStreamSynchronize(st));
        if (h_flag[0]) break;  // converged (true residual) or out of iterations
        if (ctx->use_graphs && graph == nullptr) {
            cudaGraph_t g = nullptr;
            PG_CUDA(cudaStreamBeginCapture(st, cudaStreamCaptureModeThreadLocal));
            try {
                one_iter();
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
        int chunk = 4;
        while (!h_flag[0]) {
            for (int k = 0; k < chunk; ++k) {
                if (graph) PG_CUDA(cudaGraphLaunch(graph, st));
                else one_iter();
            }
            PG_CHECK_LAUNCH();
            PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
            PG_CUDA(cudaStreamSynchronize(st));
            chunk = std::min(2 * chunk, 64);
        }
        cg_restore<<<nb, OT, 0, st>>>(A);
        PG_CHECK_LAUNCH();
        if (h_flag[2]) break;  // curvature failure
        PG_CUDA(cudaMemsetAsync(A.flag, 0, sizeof(int), st));  // clear the stop flag, keep the count
    }
    // the final charges, the iterations and the residual of the last test
    double h_stat[5] = {0, 0, 0, 0, 0};
    PG_CUDA(cudaMemcpyAsync(h_stat, A.stat, sizeof(h_stat), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(charges, A.q, sizeof(double) * n, cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaMemcpyAsync(h_flag, A.flag, sizeof(h_flag), cudaMemcpyDeviceToHost, st));
    PG_CUDA(cudaStreamSynchronize(st));
    *iterations = h_flag[1];
    *error = h_stat[4];
    if (h_flag[2])
        throw Error(PG_ERR_NOT_CONVERGED, "charge optimisation: the energy is not convex in the charges");
    if (!std::isfinite(h_stat[4])) throw Error(PG_ERR_NOT_CONVERGED, "charge optimisation diverged");
    if (!(h_stat[4] <= tolerance))
        throw Error(PG_ERR_NOT_CONVERGED, "charge optimisation reached its iteration limit before the tolerance");
}

}  // namespace pg
