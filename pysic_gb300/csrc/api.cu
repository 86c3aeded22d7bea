// api.cu -- the C ABI of include/pysic_gb300.h: context life cycle, state
// setters, the evaluation pipeline and the lane-count autotuner.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstring>
#include <string>

#include "common.cuh"

namespace {
thread_local std::string g_last_error;

template <typename F>
int guarded(F&& f) {
    try {
        f();
        g_last_error.clear();
        return PG_OK;
    } catch (const pg::Error& e) {
        g_last_error = e.what();
        return e.status;
    } catch (const std::bad_alloc&) {
        g_last_error = "host out of memory";
        return PG_ERR_CUDA;
    } catch (const std::exception& e) {
        g_last_error = e.what();
        return PG_ERR_INVALID;
    }
}

void set_device(pg_context* ctx) { PG_CUDA(cudaSetDevice(ctx->device)); }

// the context's device, and any outstanding coordinate update finished
void use_device(pg_context* ctx) {
    set_device(ctx);
    pg::settle_coordinates(ctx);
}

void check_ctx(pg_context* ctx) { pg::require(ctx != nullptr, PG_ERR_INVALID, "null context"); }
}  // namespace

namespace pg {

// generate_supercell, Geometry.f90:177-195, with the transposes of
// pysic/calculator.py:1555-1565 (vectors = cell^T, inverse = inv(cell)^T).
void make_cell(const double* cell, const double* inv, const int32_t* pbc, Cell& C) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            C.vc[r][c] = cell[c * 3 + r];
            C.ic[r][c] = inv[c * 3 + r];
        }
    const double twopi = 2.0 * 3.14159265358979323846;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) C.rc[r][c] = twopi * C.ic[c][r];
    double a[3], b[3], d[3];
    for (int r = 0; r < 3; ++r) {
        a[r] = C.vc[r][0];
        b[r] = C.vc[r][1];
        d[r] = C.vc[r][2];
    }
    const double x0 = a[1] * b[2] - a[2] * b[1];
    const double x1 = a[2] * b[0] - a[0] * b[2];
    const double x2 = a[0] * b[1] - a[1] * b[0];
    C.volume = std::fabs(x0 * d[0] + x1 * d[1] + x2 * d[2]);
    for (int i = 0; i < 3; ++i) C.pbc[i] = pbc[i] != 0;
}

CellK cell_kernel_view(const Cell& C) {
    CellK k;
    std::memcpy(k.vc, C.vc, sizeof(k.vc));
    std::memcpy(k.ic, C.ic, sizeof(k.ic));
    for (int i = 0; i < 3; ++i) k.pbc[i] = C.pbc[i];
    return k;
}

// Lanes per atom of the full-list kernels: as few as keep the GPU busy.  Each
// group of lanes ends with its atom's reductions (force, energy, virial), so
// short lists on many atoms run best at 8 lanes (Sutton-Chen, 32k atoms, ~54
// neighbours: 8 lanes 1.7x faster than 32); small systems take more lanes per
// atom while there are fewer than 64k threads and at least 4 entries per lane.
int pair_lanes_for(const pg_context* ctx) {
    if (ctx->pair_lanes) return ctx->pair_lanes;
    const double avg = ctx->n > 0 ? (double)ctx->nb_total / ctx->n : 0.0;
    int G = 8;
    while (G < 32 && (long long)ctx->n * G < 65536 && avg >= 4.0 * G) G *= 2;
    return G;
}

void prepare(pg_context* ctx) {
    require(ctx->have_cell, PG_ERR_NOT_READY, "no cell: call pg_create_cell first");
    require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms: call pg_create_atoms first");
    require(ctx->have_list, PG_ERR_NOT_READY, "no neighbour lists: build or install them first");
    if (ctx->tables_dirty) fold_tables(ctx);
    if (ctx->sep0_epoch != ctx->list_epoch) build_full_sep0(ctx);
    if (ctx->have_bond_terms && ctx->short_dirty) build_short_list(ctx);
    if (ctx->ewald) ewald_prepare(ctx);
}

// one evaluation, enqueued on ctx->stream; G: lanes per atom of the bond kernels
// true when no value is an infinity or a NaN (one-time checks of new atoms)
static bool all_finite(const double* v, size_t n) {
    bool ok = true;
    for (size_t i = 0; i < n; ++i) ok &= std::isfinite(v[i]);
    return ok;
}

namespace {

// n doubles from src to dst (dst may be null: check only); any non-finite value
// sets *bad (every writer stores the same 1; bad may be null).  vec: both
// pointers 16-byte aligned, the loop moves double2 pairs.
__global__ void copy_check(const double* __restrict__ src, double* __restrict__ dst, long long n,
                           int* __restrict__ bad, int vec) {
    int b = 0;
    const long long stride = (long long)gridDim.x * blockDim.x;
    const long long t = blockIdx.x * (long long)blockDim.x + threadIdx.x;
    if (vec) {
        const long long n2 = n / 2;
        const double2* s2 = (const double2*)src;
        double2* d2 = (double2*)dst;
        for (long long i = t; i < n2; i += stride) {
            const double2 v = s2[i];
            b |= !isfinite(v.x) | !isfinite(v.y);
            if (dst) d2[i] = v;
        }
        if (t == 0 && (n & 1)) {
            const double v = src[n - 1];
            b |= !isfinite(v);
            if (dst) dst[n - 1] = v;
        }
    } else {
        for (long long i = t; i < n; i += stride) {
            const double v = src[i];
            b |= !isfinite(v);
            if (dst) dst[i] = v;
        }
    }
    if (bad != nullptr && __syncthreads_or(b) && threadIdx.x == 0) *bad = 1;
}

// the checked coordinates into place, unless the check failed
__global__ void coords_commit(const double* __restrict__ in, double* __restrict__ out, long long n,
                              const int* __restrict__ bad) {
    if (*bad) return;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = in[i];
}

// The totals of an evaluation as doubles and the verdict of the coordinate
// update it committed (bad may be null: none), written straight into
// page-locked host memory: one small store instead of two copy-engine
// transfers.
__global__ void publish_totals(pg::HostTotals* __restrict__ out, const pg::FxAcc* __restrict__ acc,
                               const int* __restrict__ bad) {
    const int c = threadIdx.x;
    if (c < 7) out->totals[c] = pg::fx_to_double(pg::fx_from_limbs(acc[c]));
    if (c == 7) out->bad = bad != nullptr ? *bad : 0;
    __threadfence_system();
}

int copy_blocks(long long n) {
    return (int)std::max<long long>(1, std::min<long long>((n + 255) / 256, 4ll * sm_count()));
}

}  // namespace

// n doubles from host to device (to_device) or device to host through the DMA
// engine (cudaMemcpyAsync); bad (may be null, host to device only): a check
// kernel over the staged copy sets it if any value is not finite.  (A copy
// kernel reading page-locked host memory through the host link measured no
// faster than the DMA engine for these sizes, about 7 us per 786 KB.)
static void host_copy(pg_context* ctx, const double* src, double* dst, long long n, bool to_device, int* bad) {
    if (n <= 0) return;
    cudaStream_t st = ctx->stream;
    PG_CUDA(cudaMemcpyAsync(dst, src, sizeof(double) * (size_t)n,
                            to_device ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToHost, st));
    if (to_device && bad != nullptr) {
        const int vec = (((uintptr_t)dst) & 15u) == 0 ? 1 : 0;
        copy_check<<<copy_blocks(vec ? n / 2 : n), 256, 0, st>>>(dst, nullptr, n, bad, vec);
        PG_CHECK_LAUNCH();
    }
}

// The commit of staged coordinates, checked for non-finite values when they
// were staged: moved into place only if all were finite, so that a rejected
// update leaves the old coordinates.  Enqueued in front of an evaluation (and
// captured with it into its graph) or on its own.
static void enqueue_coordinate_commit(pg_context* ctx) {
    const long long m = 3ll * ctx->n;
    ctx->commit_in_disp = false;
    const int vec = (((uintptr_t)ctx->pos_in.p) & 15u) == 0 ? 1 : 0;
    copy_check<<<copy_blocks(vec ? (m + 1) / 2 : m), 256, 0, ctx->stream>>>(ctx->pos_in.p, nullptr, m,
                                                                            ctx->pos_bad.p, vec);
    PG_CHECK_LAUNCH();
    coords_commit<<<copy_blocks(m), 256, 0, ctx->stream>>>(ctx->pos_in.p, ctx->pos.p, m, ctx->pos_bad.p);
    PG_CHECK_LAUNCH();
    ctx->launches += 2;
}

// A rejected update leaves the check flag set: clear it for the next one
// (enqueued after the verdict was read, so no kernel reads it meanwhile), and
// put the old coordinates back if the displacement pass had committed the
// update.
static void clear_check_flag(pg_context* ctx) {
    PG_CUDA(cudaMemsetAsync(ctx->pos_bad.p, 0, sizeof(int), ctx->stream));
    if (ctx->commit_in_disp)
        PG_CUDA(cudaMemcpyAsync(ctx->pos.p, ctx->pos_prev.p, sizeof(double) * 3 * (size_t)ctx->n,
                                cudaMemcpyDeviceToDevice, ctx->stream));
    ctx->commit_in_disp = false;
}

// Finish an outstanding coordinate update: commit it if no evaluation has done
// so, read the verdict of its check, fail if the check rejected the update.  Every entry point that reads the device coordinates outside an
// evaluation calls this first.
void settle_coordinates(pg_context* ctx) {
    if (ctx->upd_state == PG_UPD_NONE) return;
    if (ctx->upd_state == PG_UPD_STAGED) enqueue_coordinate_commit(ctx);
    int* bad = ctx->h_flag.get(1);
    PG_CUDA(cudaMemcpyAsync(bad, ctx->pos_bad.p, sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->upd_state = PG_UPD_NONE;
    if (*bad) clear_check_flag(ctx);
    require(*bad == 0, PG_ERR_INVALID, "non-finite atom position: the coordinate update was not applied");
}

// New coordinates for the context: copied to a staging buffer on the
// context's stream, without waiting.  The next evaluation checks them for
// non-finite values and commits them in front of its kernels (in its captured
// graph), and pg_calculate reads the verdict together with the results, so an
// update followed by an evaluation costs one copy in, one copy out and one
// synchronisation.  The copy is
// cudaMemcpyAsync: page-locked host memory is read asynchronously and must
// stay unchanged until the next call on the context that returns results;
// pageable memory is consumed on return.
static void update_coordinates(pg_context* ctx, const double* positions) {
    const long long m = 3ll * ctx->n;
    if (m == 0) return;
    if (ctx->upd_state != PG_UPD_NONE) settle_coordinates(ctx);  // one outstanding update at a time
    ctx->pos_in.resize((size_t)m);
    ctx->pos_prev.resize((size_t)m);
    if (ctx->pos_bad.n == 0) {  // the check flag stays clear between updates (clear_check_flag)
        ctx->pos_bad.resize(1);
        PG_CUDA(cudaMemsetAsync(ctx->pos_bad.p, 0, sizeof(int), ctx->stream));
    }
    host_copy(ctx, positions, ctx->pos_in.p, m, true, nullptr);  // staged; checked at the commit
    ctx->upd_state = PG_UPD_STAGED;
}

// The mixed path's displacement pass runs in front of the evaluation's other
// kernels (it also clears the totals).
static bool displacement_pass_runs(pg_context* ctx, int precision, int flags) {
    const bool wantF = flags & PG_WANT_FORCES, wantC = flags & PG_WANT_ENEGS, wantE = flags & PG_WANT_ENERGY;
    const bool run_pair = ctx->have_pair_kernel_terms || ctx->ewald || ctx->have_singles || ctx->n_agroups > 0;
    const bool run_bond = ctx->have_bond_terms && (wantE || wantF);
    const bool run_tri = ctx->have_triplets && (wantE || wantF);
    const bool run_bchi = ctx->have_bond_charge_terms && wantC;
    return precision == PG_PREC_MIXED && (run_pair || run_bond || run_tri || run_bchi);
}

// skip (may be null): a device flag every kernel reads first; nonzero makes the
// whole evaluation a no-op (loops replayed from a graph stop this way).
// commit: a staged coordinate update goes into place first -- inside the
// displacement pass when it runs, else by the check and commit kernels.
// pub (may be null): where the totals and the update verdict (pub_bad) go in
// page-locked memory; true when the evaluation's last kernel (the gather pass)
// has written them, false when the caller still has to.
static bool enqueue_evaluation_commit(pg_context* ctx, int precision, int flags, int G, const int* skip,
                                      bool commit, HostTotals* pub = nullptr, const int* pub_bad = nullptr) {
    const int n = ctx->n;
    const bool wantF = flags & PG_WANT_FORCES, wantC = flags & PG_WANT_ENEGS, wantE = flags & PG_WANT_ENERGY;
    ctx->out_f.resize(3 * (size_t)std::max(n, 1));
    ctx->out_chi.resize((size_t)std::max(n, 1));
    ctx->out_acc.resize(8);
    const bool run_pair = ctx->have_pair_kernel_terms || ctx->ewald || ctx->have_singles || ctx->n_agroups > 0;
    const bool run_bond = ctx->have_bond_terms && (wantE || wantF);
    const bool run_tri = ctx->have_triplets && (wantE || wantF);
    const bool run_bchi = ctx->have_bond_charge_terms && wantC;  // Tersoff-scaled charge terms' chi
    const int Gp = pair_lanes_for(ctx);
    FxAcc* acc = ctx->out_acc.p;
    bool first_f = true, first_chi = true;
    auto mark = [&](int k) {
        if (ctx->timing) PG_CUDA(cudaEventRecord(ctx->tev[k], ctx->stream));
    };
    mark(0);
    // the totals are integers that every kernel adds to: clear them first (the
    // mixed path's displacement pass does it on the way)
    if (displacement_pass_runs(ctx, precision, flags)) {
        launch_disp(ctx, skip, acc, commit);
    } else {
        if (commit) enqueue_coordinate_commit(ctx);
        PG_CUDA(cudaMemsetAsync(acc, 0, sizeof(FxAcc) * 8, ctx->stream));
    }
    // per-atom bond-order factors: B and dB/dsum before the terms they scale
    const bool run_af = ctx->n_agroups > 0 && (wantE || wantF);
    if (run_af) launch_atom_factors(ctx, precision, 0, false, nullptr, skip);
    if (run_pair) {
        launch_pair_kernel_skip(ctx, precision, flags, first_f, first_chi, Gp, acc, skip);
        if (wantF) first_f = false;
        if (wantC) first_chi = false;
    }
    if (run_af && wantF && !ctx->af_fused) {
        launch_atom_factors(ctx, precision, 1, first_f, acc, skip);
        first_f = false;
    }
    mark(1);
    // the gather pass is the last kernel to touch the totals: it publishes them
    const bool gather_last = pub != nullptr && run_bond && wantF && !run_tri && !ctx->ewald && !run_bchi;
    if (run_bond) {
        launch_bond_order_impl(ctx, precision, flags, first_f, G, acc, [&] { mark(2); }, skip,
                               gather_last ? pub : nullptr, pub_bad);
        if (wantF) first_f = false;
    } else {
        if (run_bchi) launch_bond_b(ctx, precision, G, skip);  // the bonds' B for bond_chi
        mark(2);
    }
    if (run_tri) {
        launch_triplets(ctx, precision, flags, first_f, acc, skip);
        if (wantF) first_f = false;
    }
    mark(3);
    if (ctx->ewald) {
        launch_ewald_kspace_skip(ctx, precision, flags, first_f, first_chi, acc, skip);
        if (wantF) first_f = false;
        if (wantC) first_chi = false;
    }
    if (run_bchi) {
        launch_bond_chi(ctx, precision, first_chi, skip);
        first_chi = false;
    }
    mark(4);
    if (wantF && first_f) PG_CUDA(cudaMemsetAsync(ctx->out_f.p, 0, sizeof(double) * 3 * n, ctx->stream));
    if (wantC && first_chi) PG_CUDA(cudaMemsetAsync(ctx->out_chi.p, 0, sizeof(double) * n, ctx->stream));
    mark(5);
    return gather_last;
}

void enqueue_evaluation(pg_context* ctx, int precision, int flags, int G, const int* skip) {
    enqueue_evaluation_commit(ctx, precision, flags, G, skip, false);
}

// Pick the lanes-per-atom tile of the bond-order kernels: each candidate is
// timed over several single evaluations (device events around each) and
// judged by its fastest one, so that host launch jitter does not decide.
static int autotune_lanes(pg_context* ctx, int precision, int flags) {
    const int options[5] = {4, 8, 16, 32, PG_LANES_TRIPLET};
    constexpr int REPS = 6;
    cudaEvent_t ev[REPS + 1];
    for (auto& e : ev) PG_CUDA(cudaEventCreate(&e));
    int best = 8;
    float best_ms = 1e30f;
    for (int o = 0; o < 5; ++o) {
        const int G = options[o];
        enqueue_evaluation(ctx, precision, flags, G, nullptr);  // warm-up
        for (int r = 0; r < REPS; ++r) {
            PG_CUDA(cudaEventRecord(ev[r], ctx->stream));
            enqueue_evaluation(ctx, precision, flags, G, nullptr);
        }
        PG_CUDA(cudaEventRecord(ev[REPS], ctx->stream));
        PG_CUDA(cudaEventSynchronize(ev[REPS]));
        float fastest = 1e30f;
        for (int r = 0; r < REPS; ++r) {
            float ms = 0;
            PG_CUDA(cudaEventElapsedTime(&ms, ev[r], ev[r + 1]));
            fastest = std::min(fastest, ms);
        }
        if (fastest < best_ms) {
            best_ms = fastest;
            best = G;
        }
    }
    for (auto& e : ev) cudaEventDestroy(e);
    return best;
}

// One evaluation enqueued on the context's stream, replayed from a captured
// graph when nothing it depends on has changed; a staged coordinate update is
// checked and committed in front of its kernels.  publish: a last kernel
// writes the totals and the update verdict into h_tot (pg_calculate).
static void evaluate_impl(pg_context* ctx, int precision, int flags, bool publish) {
    require(precision == PG_PREC_FP64 || precision == PG_PREC_MIXED, PG_ERR_INVALID, "unknown precision");
    // staged coordinates are committed in front of the evaluation's kernels,
    // unless set-up work that reads them comes first
    if (ctx->upd_state == PG_UPD_STAGED &&
        (ctx->tables_dirty || ctx->sep0_epoch != ctx->list_epoch || (ctx->have_bond_terms && ctx->short_dirty) ||
         (ctx->ewald && ctx->ew_tables_dirty) || !ctx->have_list))
        settle_coordinates(ctx);
    prepare(ctx);
    const bool commit = ctx->upd_state == PG_UPD_STAGED;
    if (ctx->n == 0) {  // no atoms: zero totals, nothing to launch
        ctx->out_acc.resize(8);
        PG_CUDA(cudaMemsetAsync(ctx->out_acc.p, 0, sizeof(FxAcc) * 8, ctx->stream));
        ctx->launches = 0;
        return;
    }
    int G = ctx->lanes;
    if (G == 0 && ctx->have_bond_terms) {
        if (ctx->tuned_lanes[precision] == 0) ctx->tuned_lanes[precision] = autotune_lanes(ctx, precision, flags);
        G = ctx->tuned_lanes[precision];
    }
    if (G == 0) G = 8;
    // the verdict published: that of an update committed now or by an
    // evaluation whose results were not read yet
    const bool verdict = ctx->upd_state != PG_UPD_NONE;
    pg::HostTotals* dtot = nullptr;
    if (publish) PG_CUDA(cudaHostGetDevicePointer((void**)&dtot, (void*)ctx->h_tot.get(1), 0));
    if (commit) ctx->commit_in_disp = displacement_pass_runs(ctx, precision, flags);
    auto sequence = [&] {
        const bool published = enqueue_evaluation_commit(ctx, precision, flags, G, nullptr, commit,
                                                         publish ? dtot : nullptr, verdict ? ctx->pos_bad.p : nullptr);
        if (publish && !published) {
            publish_totals<<<1, 32, 0, ctx->stream>>>(dtot, ctx->out_acc.p, verdict ? ctx->pos_bad.p : nullptr);
            PG_CHECK_LAUNCH();
            ctx->launches += 1;
        }
    };
    if (commit) ctx->upd_state = PG_UPD_CHECKED;  // the verdict is read with the results
    // events recorded inside a capture cannot be waited on: time with direct launches
    if (!ctx->use_graphs || ctx->timing) {
        ctx->launches = 0;
        sequence();
        return;
    }
    // replay a captured sequence if nothing it depends on has changed
    for (auto it = ctx->graphs.begin(); it != ctx->graphs.end(); ++it) {
        if (it->precision != precision || it->flags != flags || it->lanes != G || it->commit != commit ||
            it->pub != (publish && verdict) + publish * 2)
            continue;
        if (it->state == ctx->state_epoch && it->alloc == alloc_epoch()) {
            PG_CUDA(cudaGraphLaunch(it->exec, ctx->stream));
            ctx->launches = it->launches;
            return;
        }
        cudaGraphExecDestroy(it->exec);
        ctx->graphs.erase(it);
        break;
    }
    // run once directly (sizes every buffer), then capture the same sequence
    // (without running it: the direct run was this call's evaluation)
    ctx->launches = 0;
    sequence();
    const int launches = ctx->launches;
    const unsigned long long alloc_before = alloc_epoch();
    cudaGraph_t graph = nullptr;
    PG_CUDA(cudaStreamBeginCapture(ctx->stream, cudaStreamCaptureModeThreadLocal));
    try {
        sequence();
    } catch (...) {
        cudaStreamEndCapture(ctx->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        throw;
    }
    PG_CUDA(cudaStreamEndCapture(ctx->stream, &graph));
    if (alloc_epoch() != alloc_before) {  // a buffer grew during capture: do not keep the graph
        cudaGraphDestroy(graph);
        ctx->launches = launches;
        return;
    }
    cudaGraphExec_t exec = nullptr;
    cudaError_t e = cudaGraphInstantiate(&exec, graph, 0);
    cudaGraphDestroy(graph);
    PG_CUDA(e);
    ctx->graphs.push_back(pg_context::Graph{precision, flags, G, launches, commit, (publish && verdict) + publish * 2,
                                            ctx->state_epoch, alloc_epoch(), exec});
    ctx->launches = launches;
}

void evaluate(pg_context* ctx, int precision, int flags) { evaluate_impl(ctx, precision, flags, false); }

// The results of the last evaluation into host memory, and the verdict of a
// coordinate update that the evaluation committed: one synchronisation.
static void copy_results(pg_context* ctx, int flags, double* energy, double* forces, double* stress, double* enegs) {
    FxAcc* acc = ctx->h_acc.get(8);
    std::memset((void*)acc, 0, sizeof(FxAcc) * 8);
    double tot[8] = {0};
    cudaStream_t st = ctx->stream;
    const bool verdict = ctx->upd_state == PG_UPD_CHECKED;
    int* bad = ctx->h_flag.get(1);
    if (verdict) PG_CUDA(cudaMemcpyAsync(bad, ctx->pos_bad.p, sizeof(int), cudaMemcpyDeviceToHost, st));
    if (energy || stress) PG_CUDA(cudaMemcpyAsync(acc, ctx->out_acc.p, sizeof(FxAcc) * 8, cudaMemcpyDeviceToHost, st));
    if (forces && (flags & PG_WANT_FORCES)) host_copy(ctx, ctx->out_f.p, forces, 3ll * ctx->n, false, nullptr);
    if (enegs && (flags & PG_WANT_ENEGS)) host_copy(ctx, ctx->out_chi.p, enegs, (long long)ctx->n, false, nullptr);
    PG_CUDA(cudaStreamSynchronize(st));
    if (verdict) {
        ctx->upd_state = PG_UPD_NONE;
        if (*bad) clear_check_flag(ctx);
        require(*bad == 0, PG_ERR_INVALID,
                "non-finite atom position: the coordinate update was not applied (results are of the previous "
                "coordinates)");
    }
    for (int c = 0; c < 7; ++c) tot[c] = fx_to_double(fx_from_limbs(acc[c]));
    if (energy && (flags & PG_WANT_ENERGY)) *energy = tot[0];
    if (stress && (flags & PG_WANT_FORCES))
        for (int c = 0; c < 6; ++c) stress[c] = tot[1 + c];
}

// pg_calculate: the evaluation ends with a kernel that writes the totals and
// the update verdict into page-locked memory (h_tot), so that only the
// per-atom arrays travel by the copy engine; one synchronisation.
static void calculate(pg_context* ctx, int precision, int flags, double* energy, double* forces, double* stress,
                      double* enegs) {
    if (ctx->n == 0 || ctx->timing) {
        evaluate(ctx, precision, flags);
        copy_results(ctx, flags, energy, forces, stress, enegs);
        return;
    }
    const bool verdict = ctx->upd_state != PG_UPD_NONE;
    evaluate_impl(ctx, precision, flags, true);
    if (forces && (flags & PG_WANT_FORCES)) host_copy(ctx, ctx->out_f.p, forces, 3ll * ctx->n, false, nullptr);
    if (enegs && (flags & PG_WANT_ENEGS)) host_copy(ctx, ctx->out_chi.p, enegs, (long long)ctx->n, false, nullptr);
    PG_CUDA(cudaStreamSynchronize(ctx->stream));
    const HostTotals* t = ctx->h_tot.p;
    if (verdict) {
        ctx->upd_state = PG_UPD_NONE;
        if (t->bad) clear_check_flag(ctx);
        require(t->bad == 0, PG_ERR_INVALID,
                "non-finite atom position: the coordinate update was not applied (results are of the previous "
                "coordinates)");
    }
    if (energy && (flags & PG_WANT_ENERGY)) *energy = t->totals[0];
    if (stress && (flags & PG_WANT_FORCES))
        for (int c = 0; c < 6; ++c) stress[c] = t->totals[1 + c];
}

}  // namespace pg

extern "C" {

const char* pg_last_error(void) { return g_last_error.c_str(); }

const char* pg_version(void) { return "pysic_gb300 0.1 (sm_103a)"; }

int pg_create(pg_context** out) { return pg_create_on(out, -1); }

int pg_create_on(pg_context** out, int32_t device) {
    return guarded([&] {
        pg::require(out != nullptr, PG_ERR_INVALID, "null output pointer");
        *out = nullptr;
        int dev = 0;
        if (device >= 0) PG_CUDA(cudaSetDevice(device));
        PG_CUDA(cudaGetDevice(&dev));
        pg_context* ctx = new pg_context();
        ctx->device = dev;
        cudaError_t e = cudaStreamCreateWithFlags(&ctx->stream, cudaStreamNonBlocking);
        if (e != cudaSuccess) {
            delete ctx;
            throw pg::Error(PG_ERR_CUDA, std::string("cudaStreamCreate: ") + cudaGetErrorString(e));
        }
        *out = ctx;
    });
}

int pg_destroy(pg_context* ctx) {
    return guarded([&] {
        if (!ctx) return;
        cudaSetDevice(ctx->device);
        cudaStreamSynchronize(ctx->stream);
        cudaStreamDestroy(ctx->stream);
        delete ctx;
    });
}

int pg_create_cell(pg_context* ctx, const double* cell, const double* inv, const int32_t* pbc) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(cell && inv && pbc, PG_ERR_INVALID, "null cell argument");
        pg::make_cell(cell, inv, pbc, ctx->cell);
        std::memcpy(ctx->cell_rows, cell, sizeof(ctx->cell_rows));
        std::memcpy(ctx->inv_rows, inv, sizeof(ctx->inv_rows));
        ctx->have_cell = true;
        ctx->state_epoch++;
        ctx->have_list = false;
        ctx->ew_tables_dirty = true;
    });
}

int pg_create_atoms(pg_context* ctx, int32_t n, const double* positions, const double* charges,
                    const int32_t* types) {
    return guarded([&] {
        check_ctx(ctx);
        set_device(ctx);
        pg::require(n >= 0, PG_ERR_INVALID, "negative atom count");
        pg::require(n == 0 || (positions && charges && types), PG_ERR_INVALID, "null atom arrays");
        for (int i = 0; i < n; ++i) pg::require(types[i] >= 0 && types[i] < 64, PG_ERR_INVALID, "type out of range");
        pg::require(n == 0 || pg::all_finite(positions, 3 * (size_t)n), PG_ERR_INVALID, "non-finite atom position");
        ctx->n = n;
        ctx->pos.upload(positions, 3 * (size_t)n, ctx->stream);
        ctx->charge.upload(charges, (size_t)n, ctx->stream);
        ctx->type.upload(types, (size_t)n, ctx->stream);
        ctx->h_type.assign(types, types + n);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->upd_state = pg::PG_UPD_NONE;  // new atoms replace any outstanding update
        ctx->have_atoms = true;
        ctx->state_epoch++;
        ctx->have_list = false;
    });
}

int pg_update_atom_coordinates(pg_context* ctx, const double* positions) {
    return guarded([&] {
        check_ctx(ctx);
        set_device(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
        pg::require(ctx->n == 0 || positions != nullptr, PG_ERR_INVALID, "null positions");
        pg::update_coordinates(ctx, positions);
    });
}

int pg_update_atom_charges(pg_context* ctx, const double* charges) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
        ctx->charge.upload(charges, (size_t)ctx->n, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_get_atom_charges(pg_context* ctx, double* charges) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
        ctx->charge.download(charges, (size_t)ctx->n, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_set_pair_potentials(pg_context* ctx, int32_t n_types, int32_t n, const int32_t* kind, const double* params,
                           const double* cutoff, const double* soft, const uint64_t* mask1, const uint64_t* mask2,
                           const int32_t* group) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n_types >= 0 && n_types <= 64, PG_ERR_INVALID, "n_types must be within 0..64");
        pg::require(n >= 0, PG_ERR_INVALID, "negative record count");
        for (int r = 0; r < n; ++r)
            pg::require(kind[r] >= 0 && kind[r] <= 10, PG_ERR_UNSUPPORTED, "unknown pair potential kind");
        ctx->n_types = n_types;
        ctx->pr_kind.assign(kind, kind + n);
        ctx->pr_params.assign(params, params + 4 * (size_t)n);
        ctx->pr_cut.assign(cutoff, cutoff + n);
        ctx->pr_soft.assign(soft, soft + n);
        ctx->pr_m1.assign(mask1, mask1 + n);
        ctx->pr_m2.assign(mask2, mask2 + n);
        ctx->pr_group.assign(group, group + n);
        ctx->pr_nmul.clear();  // products are set after the records they extend
        ctx->pr_mul0.clear();
        ctx->tables_dirty = true;
    });
}

int pg_set_pair_products(pg_context* ctx, int32_t n_records, const int32_t* n_mul, const int32_t* mul0,
                         int32_t n_factors, const int32_t* kind, const double* params, const uint64_t* first) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n_records == (int)ctx->pr_kind.size(), PG_ERR_INVALID,
                    "one product entry per pair record set by pg_set_pair_potentials");
        pg::require(n_factors >= 0 && (n_factors == 0 || (kind && params && first)), PG_ERR_INVALID,
                    "invalid product factors");
        pg::require(n_records == 0 || (n_mul && mul0), PG_ERR_INVALID, "null product arrays");
        for (int r = 0; r < n_records; ++r) {
            pg::require(n_mul[r] >= 0 && n_mul[r] <= 8 && mul0[r] >= 0 && mul0[r] + n_mul[r] <= n_factors,
                        PG_ERR_INVALID, "product factors out of range (at most 8 factors besides the lead)");
        }
        for (int c = 0; c < n_factors; ++c)
            pg::require(kind[c] >= 0 && kind[c] <= 9, PG_ERR_UNSUPPORTED, "unknown pair potential kind in a product");
        ctx->pr_nmul.assign(n_mul, n_mul + n_records);
        ctx->pr_mul0.assign(mul0, mul0 + n_records);
        ctx->pm_kind.assign(kind, kind + n_factors);
        ctx->pm_params.assign(params, params + 4 * (size_t)n_factors);
        ctx->pm_first.assign(first, first + n_factors);
        ctx->tables_dirty = true;
    });
}

int pg_set_triplet_potentials(pg_context* ctx, int32_t n, const int32_t* kind, const double* params,
                              const double* cutoff, const double* soft, const uint64_t* mask1, const uint64_t* mask2,
                              const uint64_t* mask3, const uint64_t* center) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0 && n <= pg::PG_MAX_TRIPLET_RECORDS, PG_ERR_UNSUPPORTED,
                    "three-body records: at most 64 (distinct permutations of all target tuples)");
        pg::require(n == 0 || (kind && params && cutoff && soft && mask1 && mask2 && mask3 && center), PG_ERR_INVALID,
                    "null record arrays");
        for (int r = 0; r < n; ++r) pg::require(kind[r] == 0, PG_ERR_UNSUPPORTED, "unknown three-body kind");
        ctx->tr_kind.assign(kind, kind + n);
        ctx->tr_params.assign(params, params + 4 * (size_t)n);
        ctx->tr_cut.assign(cutoff, cutoff + n);
        ctx->tr_soft.assign(soft, soft + n);
        ctx->tr_m1.assign(mask1, mask1 + n);
        ctx->tr_m2.assign(mask2, mask2 + n);
        ctx->tr_m3.assign(mask3, mask3 + n);
        ctx->tr_center.assign(center, center + n);
        ctx->tables_dirty = true;
    });
}

int pg_set_quad_potentials(pg_context* ctx, int32_t n, const int32_t* kind, const double* params,
                           const double* cutoff, const double* soft, const uint64_t* masks,
                           const uint64_t* orig) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0 && n <= pg::PG_MAX_QUAD_RECORDS, PG_ERR_UNSUPPORTED,
                    "four-body records: at most 64 (distinct permutations of all target tuples)");
        pg::require(n == 0 || (kind && params && cutoff && soft && masks && orig), PG_ERR_INVALID,
                    "null record arrays");
        for (int r = 0; r < n; ++r) pg::require(kind[r] == 0, PG_ERR_UNSUPPORTED, "unknown four-body kind");
        ctx->qd_kind.assign(kind, kind + n);
        ctx->qd_params.assign(params, params + 4 * (size_t)n);
        ctx->qd_cut.assign(cutoff, cutoff + n);
        ctx->qd_soft.assign(soft, soft + n);
        ctx->qd_mask.assign(masks, masks + 4 * (size_t)n);
        ctx->qd_orig.assign(orig, orig + 4 * (size_t)n);
        ctx->tables_dirty = true;
    });
}

int pg_set_pair_first_targets(pg_context* ctx, int32_t n, const uint64_t* masks) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0 && (n == 0 || masks != nullptr), PG_ERR_INVALID, "invalid first-target masks");
        ctx->pr_first.assign(masks, masks + n);
        ctx->tables_dirty = true;
    });
}

int pg_set_pair_tables(pg_context* ctx, int64_t n_rows, const double* rows) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n_rows >= 0 && (n_rows == 0 || rows != nullptr), PG_ERR_INVALID, "invalid table rows");
        ctx->pr_table.assign(rows, rows + 2 * n_rows);
        ctx->tables_dirty = true;
    });
}

int pg_set_single_potentials(pg_context* ctx, int32_t n, const int32_t* kind, const double* params,
                             const uint64_t* mask) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0, PG_ERR_INVALID, "negative record count");
        for (int r = 0; r < n; ++r)
            pg::require(kind[r] >= 0 && kind[r] <= 2, PG_ERR_UNSUPPORTED, "unknown single-atom kind");
        ctx->sr_kind.assign(kind, kind + n);
        ctx->sr_params.assign(params, params + 4 * (size_t)n);
        ctx->sr_m.assign(mask, mask + n);
        ctx->sr_group.assign((size_t)n, -1);
        ctx->tables_dirty = true;
    });
}

int pg_set_single_groups(pg_context* ctx, int32_t n, const int32_t* group) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n == (int)ctx->sr_kind.size() && (n == 0 || group != nullptr), PG_ERR_INVALID,
                    "one group per single-atom record");
        ctx->sr_group.assign(group, group + n);
        ctx->tables_dirty = true;
    });
}

int pg_set_atom_factors(pg_context* ctx, int32_t n, const int32_t* kind, const double* params, const double* cutoff,
                        const double* soft, const uint64_t* mask1, const uint64_t* mask2, const int32_t* group) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0, PG_ERR_INVALID, "negative record count");
        pg::require(n == 0 || (kind && params && cutoff && soft && mask1 && mask2 && group), PG_ERR_INVALID,
                    "null record arrays");
        for (int r = 0; r < n; ++r) {
            pg::require(kind[r] >= 0 && kind[r] <= 5, PG_ERR_UNSUPPORTED, "unknown per-atom bond-order factor kind");
            pg::require(std::isfinite(cutoff[r]) && std::isfinite(soft[r]) && group[r] >= 0, PG_ERR_INVALID,
                        "invalid per-atom bond-order factor record");
        }
        ctx->af_kind.assign(kind, kind + n);
        ctx->af_params.assign(params, params + 5 * (size_t)n);
        ctx->af_cut.assign(cutoff, cutoff + n);
        ctx->af_soft.assign(soft, soft + n);
        ctx->af_m1.assign(mask1, mask1 + n);
        ctx->af_m2.assign(mask2, mask2 + n);
        ctx->af_group.assign(group, group + n);
        ctx->tables_dirty = true;
    });
}

int pg_set_bond_order_factors(pg_context* ctx, int32_t n, const double* params, const double* cutoff,
                              const double* soft, const uint64_t* mask1, const uint64_t* mask2,
                              const uint64_t* mask3, const int32_t* group) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(n >= 0, PG_ERR_INVALID, "negative record count");
        ctx->br_params.assign(params, params + 7 * (size_t)n);
        ctx->br_cut.assign(cutoff, cutoff + n);
        ctx->br_soft.assign(soft, soft + n);
        ctx->br_m1.assign(mask1, mask1 + n);
        ctx->br_m2.assign(mask2, mask2 + n);
        ctx->br_m3.assign(mask3, mask3 + n);
        ctx->br_group.assign(group, group + n);
        ctx->tables_dirty = true;
    });
}

int pg_set_ewald(pg_context* ctx, double real_cut, double k_radius, const int32_t* kmax, double sigma, double epsilon,
                 const double* scaler) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "set atoms before Ewald parameters");
        pg::require(sigma > 0 && epsilon > 0 && real_cut >= 0 && k_radius >= 0, PG_ERR_INVALID,
                    "invalid Ewald parameters");
        for (int a = 0; a < 3; ++a) pg::require(kmax[a] >= 0 && kmax[a] <= 512, PG_ERR_INVALID, "invalid k limit");
        ctx->ewald = true;
        ctx->ew_rc = real_cut;
        ctx->ew_kc = k_radius;
        ctx->ew_sigma = sigma;
        ctx->ew_eps = epsilon;
        for (int a = 0; a < 3; ++a) ctx->ew_kmax[a] = kmax[a];
        ctx->ew_scaler.upload(scaler, (size_t)ctx->n, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
        ctx->ew_tables_dirty = true;
        ctx->state_epoch++;
    });
}

int pg_clear_ewald(pg_context* ctx) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->ewald = false;
        ctx->state_epoch++;
    });
}

int pg_generate_neighbor_lists(pg_context* ctx, const double* cutoffs, double skin) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_cell && ctx->have_atoms, PG_ERR_NOT_READY, "set cell and atoms first");
        pg::require(skin >= 0, PG_ERR_INVALID, "negative skin");
        for (int i = 0; i < ctx->n; ++i)
            pg::require(std::isfinite(cutoffs[i]) && cutoffs[i] >= 0, PG_ERR_INVALID, "invalid cutoff");
        ctx->skin = skin;
        pg::build_neighbor_lists(ctx, cutoffs);
    });
}

int pg_generate_all_pairs_lists(pg_context* ctx, const double* cutoffs, double skin) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_cell && ctx->have_atoms, PG_ERR_NOT_READY, "set cell and atoms first");
        pg::require(skin >= 0, PG_ERR_INVALID, "negative skin");
        for (int i = 0; i < ctx->n; ++i)
            pg::require(std::isfinite(cutoffs[i]) && cutoffs[i] >= 0, PG_ERR_INVALID, "invalid cutoff");
        ctx->skin = skin;
        pg::build_allpairs_lists(ctx, cutoffs);
    });
}

int pg_get_neighbor_counts(pg_context* ctx, int32_t* counts) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_list, PG_ERR_NOT_READY, "no neighbour lists");
        std::vector<int> st(ctx->n + 1);
        ctx->nb_start.download(st.data(), ctx->n + 1, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
        for (int i = 0; i < ctx->n; ++i) counts[i] = st[i + 1] - st[i];
    });
}

int pg_get_neighbor_lists(pg_context* ctx, int32_t* neighbors, int32_t* offsets) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_list, PG_ERR_NOT_READY, "no neighbour lists");
        ctx->nb_idx.download(neighbors, (size_t)ctx->nb_total, ctx->stream);
        ctx->nb_off.download(offsets, 3 * (size_t)ctx->nb_total, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_create_neighbor_lists(pg_context* ctx, const int32_t* counts, const int32_t* neighbors, const int32_t* offsets,
                             double skin) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
        ctx->skin = skin;
        pg::install_neighbor_lists(ctx, counts, neighbors, offsets);
    });
}

int pg_calculate(pg_context* ctx, int32_t precision, int32_t flags, double* energy, double* forces, double* stress,
                 double* enegs) {
    return guarded([&] {
        check_ctx(ctx);
        set_device(ctx);
        pg::calculate(ctx, precision, flags, energy, forces, stress, enegs);
    });
}

int pg_get_atom_factors(pg_context* ctx, int32_t precision, int32_t group, double* factors) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(factors != nullptr, PG_ERR_INVALID, "null output");
        pg::evaluate(ctx, precision, PG_WANT_ENERGY);  // runs the factor pass of every group
        const int n = ctx->n;
        auto it = ctx->agroup_of.find(group);
        if (it == ctx->agroup_of.end() || n == 0) {  // no per-atom factors in the group: zeros, as the reference
            std::fill(factors, factors + n, 0.0);
            return;
        }
        const size_t o = (size_t)it->second * (size_t)n;
        if (precision == PG_PREC_FP64) {
            PG_CUDA(cudaMemcpyAsync(factors, ctx->af_B.p + o, sizeof(double) * n, cudaMemcpyDeviceToHost,
                                    ctx->stream));
        } else {
            std::vector<float> tmp((size_t)n);
            PG_CUDA(cudaMemcpyAsync(tmp.data(), (const float*)ctx->af_B.p + o, sizeof(float) * n,
                                    cudaMemcpyDeviceToHost, ctx->stream));
            PG_CUDA(cudaStreamSynchronize(ctx->stream));
            for (int i = 0; i < n; ++i) factors[i] = tmp[(size_t)i];
        }
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_get_atom_factor_gradients(pg_context* ctx, int32_t precision, int32_t group, int32_t atom, int32_t of_factor,
                                 double* gradients) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(gradients != nullptr, PG_ERR_INVALID, "null output");
        pg::require(atom >= 0 && atom < ctx->n, PG_ERR_INVALID, "atom index out of range");
        pg::evaluate(ctx, precision, PG_WANT_ENERGY);  // the sums and dB/dsum at the current positions
        pg::atom_factor_gradients(ctx, precision, group, atom, of_factor ? 1 : 0, gradients);
    });
}

int pg_calculate_energy(pg_context* ctx, int32_t precision, double* energy) {
    return pg_calculate(ctx, precision, PG_WANT_ENERGY, energy, nullptr, nullptr, nullptr);
}

int pg_calculate_forces(pg_context* ctx, int32_t precision, double* forces, double* stress) {
    return pg_calculate(ctx, precision, PG_WANT_FORCES, nullptr, forces, stress, nullptr);
}

int pg_calculate_electronegativities(pg_context* ctx, int32_t precision, double* enegs) {
    return pg_calculate(ctx, precision, PG_WANT_ENEGS, nullptr, nullptr, nullptr, enegs);
}

int pg_relax_charges(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double inertia,
                     double friction, double tolerance, double* rates, double* charges, int32_t* steps, double* error,
                     double* max_dq) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(inertia != 0.0, PG_ERR_INVALID, "zero charge inertia");
        pg::require(n_steps >= 0, PG_ERR_INVALID, "negative step count");
        pg::relax_charges(ctx, precision, pg::PG_RELAX_DYNAMIC, n_steps, timestep, inertia, friction, tolerance, 0.0,
                          rates, charges, steps, error, max_dq);
    });
}

int pg_optimize_charges(pg_context* ctx, int32_t precision, int32_t max_iterations, double tolerance,
                        double* charges, int32_t* iterations, double* error) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(max_iterations >= 0, PG_ERR_INVALID, "negative iteration count");
        pg::require(charges && iterations && error, PG_ERR_INVALID, "null output pointer");
        int it = 0;
        double err = 0.0;
        try {
            pg::optimize_charges(ctx, precision, max_iterations, tolerance, charges, &it, &err);
        } catch (...) {
            *iterations = it;
            *error = err;
            throw;
        }
        *iterations = it;
        *error = err;
    });
}

int pg_md_set_state(pg_context* ctx, const double* masses, const double* momenta) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->n == 0 || (masses && momenta), PG_ERR_INVALID, "null arrays");
        pg::md_set_state(ctx, masses, momenta);
    });
}

int pg_md_get_state(pg_context* ctx, double* momenta, double* positions) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::md_get_state(ctx, momenta, positions);
    });
}

int pg_md_verlet(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double skin,
                 int32_t* steps_done, int32_t* rebuild) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(steps_done && rebuild, PG_ERR_INVALID, "null output pointer");
        pg::require(n_steps >= 0, PG_ERR_INVALID, "negative step count");
        int s = 0, r = 0;
        pg::md_run(ctx, precision, n_steps, timestep, skin, &s, &r);
        *steps_done = s;
        *rebuild = r;
    });
}

int pg_md_run(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep, double skin, int32_t* steps_done,
              int32_t* rebuilds) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(steps_done && rebuilds, PG_ERR_INVALID, "null output pointer");
        pg::require(n_steps >= 0, PG_ERR_INVALID, "negative step count");
        int s = 0, r = 0;
        pg::md_run_rebuilding(ctx, precision, n_steps, timestep, skin, &s, &r);
        *steps_done = s;
        *rebuilds = r;
    });
}

int pg_get_list_positions(pg_context* ctx, double* positions) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(positions != nullptr, PG_ERR_INVALID, "null output pointer");
        pg::require(ctx->have_list && ctx->sep0_epoch == ctx->list_epoch, PG_ERR_NOT_READY,
                    "no list generation on the device yet (evaluate once after building the lists)");
        ctx->pos0.download(positions, 3 * (size_t)ctx->n, ctx->stream);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_relax_charges_potentiostat(pg_context* ctx, int32_t precision, int32_t n_steps, double timestep,
                                  double inertia, double potential, double* rates, double* charges, double* max_dchi) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(inertia != 0.0, PG_ERR_INVALID, "zero charge inertia");
        pg::require(n_steps >= 0, PG_ERR_INVALID, "negative step count");
        pg::require(std::isfinite(potential) && std::isfinite(timestep), PG_ERR_INVALID,
                    "non-finite potential or time step");
        int steps = 0;
        double err = 0.0, dq = 0.0;
        pg::relax_charges(ctx, precision, pg::PG_RELAX_POTENTIOSTAT, n_steps, timestep, inertia, 0.0, 0.0, potential,
                          rates, charges, &steps, &err, &dq);
        if (max_dchi) *max_dchi = err;
    });
}

int pg_get_bond_zeta(pg_context* ctx, double* zeta, int64_t capacity, int64_t* n_entries) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::prepare(ctx);
        pg::require(ctx->have_bond_terms, PG_ERR_NOT_READY, "no bond-order factors");
        *n_entries = ctx->sh_total;
        if (zeta && capacity >= ctx->sh_total) {
            pg::bond_zeta_diag(ctx);
            ctx->bo_zeta.download(zeta, (size_t)ctx->sh_total, ctx->stream);
            PG_CUDA(cudaStreamSynchronize(ctx->stream));
        }
    });
}

int pg_set_lanes_per_atom(pg_context* ctx, int32_t lanes) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(lanes == 0 || lanes == 4 || lanes == 8 || lanes == 16 || lanes == 32 || lanes == PG_LANES_TRIPLET,
                    PG_ERR_INVALID, "lanes per atom must be 0, 4, 8, 16, 32 or PG_LANES_TRIPLET (64)");
        ctx->lanes = lanes;
        ctx->state_epoch++;
    });
}

int pg_set_pair_lanes(pg_context* ctx, int32_t lanes) {
    return guarded([&] {
        check_ctx(ctx);
        pg::require(lanes == 0 || lanes == 8 || lanes == 16 || lanes == 32, PG_ERR_INVALID,
                    "pair lanes per atom must be 0, 8, 16 or 32");
        ctx->pair_lanes = lanes;
        ctx->state_epoch++;
    });
}

int pg_get_lanes_per_atom(pg_context* ctx, int32_t* lanes) {
    return guarded([&] {
        check_ctx(ctx);
        *lanes = ctx->lanes;
        if (*lanes == 0) *lanes = std::max(ctx->tuned_lanes[0], ctx->tuned_lanes[1]);
    });
}

int pg_device_evaluate(pg_context* ctx, int32_t precision, int32_t flags) {
    return guarded([&] {
        check_ctx(ctx);
        set_device(ctx);
        pg::evaluate(ctx, precision, flags);
    });
}

int pg_device_synchronize(pg_context* ctx) {
    return guarded([&] {
        check_ctx(ctx);
        PG_CUDA(cudaStreamSynchronize(ctx->stream));
    });
}

int pg_device_results(pg_context* ctx, double* energy, double* forces, double* stress, double* enegs) {
    return guarded([&] {
        check_ctx(ctx);
        set_device(ctx);
        pg::copy_results(ctx, PG_WANT_ENERGY | PG_WANT_FORCES | PG_WANT_ENEGS, energy, forces, stress, enegs);
    });
}

int pg_device_positions(pg_context* ctx, double** device_ptr) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->have_atoms, PG_ERR_NOT_READY, "no atoms");
        *device_ptr = ctx->pos.p;
    });
}

int pg_get_stream(pg_context* ctx, void** stream) {
    return guarded([&] {
        check_ctx(ctx);
        *stream = (void*)ctx->stream;
    });
}

int pg_bond_order_noalloc(pg_context* ctx, int32_t precision, double* d_forces, double* d_totals) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::bond_order_noalloc(ctx, precision, d_forces, d_totals);
    });
}

int pg_measure_fp32_peak(int32_t device, double* tflops, double* ms) {
    return guarded([&] { pg::measure_fp32_peak(device, tflops, ms); });
}

int pg_device_allocation_count(uint64_t* count) {
    return guarded([&] {
        pg::require(count != nullptr, PG_ERR_INVALID, "null output pointer");
        *count = pg::alloc_epoch();
    });
}

int pg_descriptors(pg_context* ctx, int32_t n_gauss, double r0, double r1, double width, double cutoff,
                   float* out) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(out != nullptr, PG_ERR_INVALID, "null output pointer");
        pg::descriptors(ctx, n_gauss, r0, r1, width, cutoff, out);
    });
}

static void check_mlp(pg_mlp* m) {
    pg::require(m != nullptr, PG_ERR_INVALID, "null network");
    PG_CUDA(cudaSetDevice(m->device));
}

int pg_mlp_create(pg_mlp** mlp, int32_t n_in, int32_t n_h1, int32_t n_h2, int32_t device) {
    return guarded([&] {
        pg::require(mlp != nullptr, PG_ERR_INVALID, "null output pointer");
        *mlp = nullptr;
        pg::mlp_create(mlp, n_in, n_h1, n_h2, device);
    });
}

int pg_mlp_destroy(pg_mlp* mlp) {
    return guarded([&] {
        if (mlp) {
            cudaSetDevice(mlp->device);
            delete mlp;
        }
    });
}

int pg_mlp_param_count(pg_mlp* mlp, int64_t* count) {
    return guarded([&] {
        check_mlp(mlp);
        *count = mlp->n_params;
    });
}

int pg_mlp_set_params(pg_mlp* mlp, const float* params, int64_t count) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_set_params(mlp, params, count);
    });
}

int pg_mlp_get_params(pg_mlp* mlp, float* params, int64_t count) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_get_params(mlp, params, count);
    });
}

int pg_mlp_add_samples(pg_mlp* mlp, const float* x, const float* y, int64_t n) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_add_samples(mlp, x, y, n);
    });
}

int pg_mlp_clear_samples(pg_mlp* mlp) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_clear_samples(mlp);
    });
}

int pg_mlp_train(pg_mlp* mlp, int32_t epochs, int32_t batch, float learning_rate, uint64_t seed,
                 float* epoch_loss) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_train(mlp, epochs, batch, learning_rate, seed, epoch_loss);
    });
}

int pg_mlp_gradients(pg_mlp* mlp, const float* x, const float* y, int64_t n, float* grad, double* loss) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_gradients(mlp, x, y, n, grad, loss);
    });
}

int pg_mlp_predict(pg_mlp* mlp, const float* x, int64_t n, float* y) {
    return guarded([&] {
        check_mlp(mlp);
        pg::mlp_predict(mlp, x, n, y);
    });
}

int pg_mlp_predict_charges(pg_mlp* mlp, pg_context* ctx, int32_t n_gauss, double r0, double r1, double width,
                           double cutoff, int32_t n_elements, const int32_t* type_element, const float* x_mean,
                           const float* x_scale, double y_mean, double y_scale, double total_charge,
                           double* charges) {
    return guarded([&] {
        check_mlp(mlp);
        check_ctx(ctx);
        use_device(ctx);
        pg::require(type_element && x_mean && x_scale, PG_ERR_INVALID, "null input arrays");
        pg::require(std::isfinite(y_mean) && std::isfinite(y_scale) && std::isfinite(total_charge), PG_ERR_INVALID,
                    "non-finite output scaling or total charge");
        pg::require(n_gauss >= 1 && width > 0 && cutoff > 0 && r1 >= r0, PG_ERR_INVALID,
                    "invalid descriptor parameters");
        pg::mlp_predict_charges(mlp, ctx, n_gauss, r0, r1, width, cutoff, n_elements, type_element, x_mean, x_scale,
                                y_mean, y_scale, total_charge, charges);
    });
}

static void check_batch(pg_batch* b) { pg::require(b != nullptr, PG_ERR_INVALID, "null batch"); }

int pg_batch_create(pg_batch** batch, int32_t device) {
    return guarded([&] {
        pg::require(batch != nullptr, PG_ERR_INVALID, "null output pointer");
        *batch = nullptr;
        pg::batch_create(batch, device);
    });
}

int pg_batch_destroy(pg_batch* batch) {
    return guarded([&] {
        if (batch) pg::batch_destroy(batch);
    });
}

int pg_batch_add(pg_batch* batch, pg_context* ctx) {
    return guarded([&] {
        check_batch(batch);
        check_ctx(ctx);
        pg::batch_add(batch, ctx);
    });
}

int pg_batch_set_lanes(pg_batch* batch, int32_t pair_lanes, int32_t bond_lanes) {
    return guarded([&] {
        check_batch(batch);
        pg::batch_set_lanes(batch, pair_lanes, bond_lanes);
    });
}

int pg_batch_get_lanes(pg_batch* batch, int32_t precision, int32_t* pair_lanes, int32_t* bond_lanes) {
    return guarded([&] {
        check_batch(batch);
        int p = 0, q = 0;
        pg::batch_get_lanes(batch, precision, &p, &q);
        *pair_lanes = p;
        *bond_lanes = q;
    });
}

int pg_batch_set_tile_blocks(pg_batch* batch, int32_t blocks) {
    return guarded([&] {
        check_batch(batch);
        pg::batch_set_tile_blocks(batch, blocks);
    });
}

int pg_batch_test_stall(pg_batch* batch, int32_t system, double wait_seconds) {
    return guarded([&] {
        check_batch(batch);
        pg::batch_test_stall(batch, system, wait_seconds);
    });
}

int pg_batch_get_tiles(pg_batch* batch, int32_t precision, int32_t mode, int32_t* pair_lanes, int32_t* bond_lanes,
                       int32_t* blocks) {
    return guarded([&] {
        check_batch(batch);
        pg::require(pair_lanes && bond_lanes && blocks, PG_ERR_INVALID, "null output");
        int p = 0, q = 0, c = 0;
        pg::batch_get_tiles(batch, precision, mode, &p, &q, &c);
        *pair_lanes = p;
        *bond_lanes = q;
        *blocks = c;
    });
}

int pg_batch_evaluate(pg_batch* batch, int32_t precision, int32_t flags, int32_t mode) {
    return guarded([&] {
        check_batch(batch);
        pg::batch_evaluate(batch, precision, flags, mode);
    });
}

int pg_batch_synchronize(pg_batch* batch) {
    return guarded([&] {
        check_batch(batch);
        pg::batch_synchronize(batch);
    });
}

int pg_batch_get_stream(pg_batch* batch, void** stream) {
    return guarded([&] {
        check_batch(batch);
        *stream = (void*)pg::batch_stream(batch);
    });
}

int pg_batch_last_launch_count(pg_batch* batch, int32_t* launches) {
    return guarded([&] {
        check_batch(batch);
        *launches = pg::batch_launches(batch);
    });
}

int pg_set_kernel_timing(pg_context* ctx, int32_t enable) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        if (enable && !ctx->tev[0])
            for (auto& e : ctx->tev) PG_CUDA(cudaEventCreate(&e));
        ctx->timing = enable != 0;
        ctx->state_epoch++;
    });
}

int pg_get_kernel_times(pg_context* ctx, float* ms) {
    return guarded([&] {
        check_ctx(ctx);
        use_device(ctx);
        pg::require(ctx->timing, PG_ERR_NOT_READY, "kernel timing is off");
        PG_CUDA(cudaEventSynchronize(ctx->tev[5]));
        for (int k = 0; k < 5; ++k) PG_CUDA(cudaEventElapsedTime(&ms[k], ctx->tev[k], ctx->tev[k + 1]));
    });
}

int pg_set_graphs(pg_context* ctx, int32_t enable) {
    return guarded([&] {
        check_ctx(ctx);
        ctx->use_graphs = enable != 0;
    });
}

int pg_last_launch_count(pg_context* ctx, int32_t* launches) {
    return guarded([&] {
        check_ctx(ctx);
        *launches = ctx->launches;
    });
}

}  // extern "C"
