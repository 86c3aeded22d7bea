// batch.cu -- many independent systems evaluated by one launch per kernel.
//
// No counterpart in the reference, which holds one system per process in its
// Fortran core (Core.f90:22-30).  A batch borrows contexts that are each fully
// set up (cell, atoms, interactions, neighbour lists).  One evaluation of the
// batch is a single launch of each kernel -- displacement / clearing, pair
// terms, bond-order pass, gather pass -- over a tile list in which tile t names
// (system, block of that system); the resident blocks walk the list, so small
// and large systems share the GPU without a launch per system.  The sequence is
// captured once in a CUDA graph and replayed.  Each system's results land in
// its own context (pg_device_results reads them).
//
// Tiles: lanes per atom of the pair kernel (atoms per warp 32/G, 128 threads
// per block) and of the bond-order kernels (one bond per lane, or the triplet
// tile) are chosen by timing the candidate pairs on the batch itself, unless
// set explicitly.
#include <algorithm>
#include <vector>

#include "args.cuh"
#include "common.cuh"

struct pg_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<pg_context*> sys;
    int pair_lanes = 0, bond_lanes = 0;  // 0: autotune
    int tuned[2][2] = {{0, 0}, {0, 0}};  // [precision][pair, bond]
    pg::DevBuf<pg::PairArgs> d_pair;
    pg::DevBuf<pg::BondArgs> d_bond;
    pg::DevBuf<pg::DispArgs> d_disp;
    pg::DevBuf<int2> t_pair, t_bond, t_disp;
    int n_pair = 0, n_bond = 0, n_disp = 0;
    bool spec = false, forces = false;
    struct Key {
        int precision, flags, pg, bg;
        unsigned long long state, alloc;
        bool operator==(const Key& o) const {
            return precision == o.precision && flags == o.flags && pg == o.pg && bg == o.bg && state == o.state &&
                   alloc == o.alloc;
        }
    };
    bool have_key = false;
    Key key{};
    cudaGraphExec_t graph = nullptr;
    int launches = 0;
    ~pg_batch() {
        if (graph) cudaGraphExecDestroy(graph);
        if (stream) cudaStreamDestroy(stream);
    }
};

namespace pg {

namespace {

constexpr int PAIR_THREADS = 128;
constexpr int DISP_THREADS = 256;

unsigned long long state_sum(const pg_batch* b) {
    unsigned long long s = 0;
    for (const pg_context* c : b->sys) s = s * 1000003ull + c->state_epoch;
    return s;
}

// size every per-system buffer the kernels touch (may allocate; never inside a capture)
void size_buffers(pg_batch* b, int precision) {
    for (pg_context* c : b->sys) {
        require(c->device == b->device, PG_ERR_INVALID, "every system of a batch must live on the batch's device");
        settle_coordinates(c);
        prepare(c);
        require(!c->ewald && !c->have_triplets && c->n_agroups == 0, PG_ERR_UNSUPPORTED,
                "the many-system launch covers pair and Tersoff bond-order terms; evaluate Ewald, three-body or "
                "per-atom bond-order systems one by one");
        const size_t n = (size_t)std::max(c->n, 1);
        c->out_f.resize(3 * n);
        c->out_chi.resize(n);
        c->out_acc.resize(8);
        if (precision == PG_PREC_MIXED) c->disp32.resize(n);
        if (c->have_bond_terms) prepare_bond_scratch(c, precision);
    }
}

// argument records and tile lists of all systems, uploaded to the device
void build(pg_batch* b, int precision, int flags, int pg_lanes, int bg_lanes) {
    const bool wantF = flags & PG_WANT_FORCES;
    std::vector<PairArgs> pa;
    std::vector<BondArgs> ba;
    std::vector<DispArgs> da;
    std::vector<int2> tp, tb, td;
    bool all_spec = true, any_bond = false;
    for (size_t s = 0; s < b->sys.size(); ++s) {
        pg_context* c = b->sys[s];
        FxAcc* acc = c->out_acc.p;
        da.push_back(make_disp_args(c, precision == PG_PREC_MIXED ? c->disp32.p : nullptr, nullptr, acc));
        const int nd = std::max(1, (c->n + DISP_THREADS - 1) / DISP_THREADS);
        for (int k = 0; k < nd; ++k) td.push_back(make_int2((int)s, k));
        const bool run_pair = c->have_pair_kernel_terms || c->have_singles;
        const bool run_bond = c->have_bond_terms;
        require(run_pair || run_bond, PG_ERR_NOT_READY, "a system of the batch has no interactions");
        if (run_pair) {
            const int slot = (int)pa.size();
            pa.push_back(make_pair_args(c, precision, flags, true, true, acc, nullptr));
            const int ap = PAIR_THREADS / pg_lanes;
            const int nbk = std::max(1, (c->n + ap - 1) / ap);
            for (int k = 0; k < nbk; ++k) tp.push_back(make_int2(slot, k));
        }
        if (run_bond) {
            any_bond = true;
            all_spec = all_spec && c->spec_ok;
            const int slot = (int)ba.size();
            BondArgs A = make_bond_args(c, precision, flags, !run_pair, acc);
            A.nblocks = bond_blocks(c->n, bg_lanes);
            ba.push_back(A);
            for (int k = 0; k < A.nblocks; ++k) tb.push_back(make_int2(slot, k));
        }
    }
    (void)wantF;
    b->spec = any_bond && all_spec;
    b->forces = wantF;
    b->n_pair = (int)tp.size();
    b->n_bond = (int)tb.size();
    b->n_disp = (int)td.size();
    if (!pa.empty()) b->d_pair.upload(pa.data(), pa.size(), b->stream);
    if (!ba.empty()) b->d_bond.upload(ba.data(), ba.size(), b->stream);
    b->d_disp.upload(da.data(), da.size(), b->stream);
    if (!tp.empty()) b->t_pair.upload(tp.data(), tp.size(), b->stream);
    if (!tb.empty()) b->t_bond.upload(tb.data(), tb.size(), b->stream);
    b->t_disp.upload(td.data(), td.size(), b->stream);
    PG_CUDA(cudaStreamSynchronize(b->stream));
}

void enqueue(pg_batch* b, int precision, int pg_lanes, int bg_lanes) {
    const int sms = sm_count();
    launch_disp_batch(b->d_disp.p, b->t_disp.p, b->n_disp, std::min(b->n_disp, sms * 8), b->stream);
    if (b->n_pair)
        launch_pair_batch(b->d_pair.p, b->t_pair.p, b->n_pair, std::min(b->n_pair, sms * 12), PAIR_THREADS,
                          precision, pg_lanes, b->stream);
    if (b->n_bond)
        launch_bond_batch(b->d_bond.p, b->t_bond.p, b->n_bond, std::min(b->n_bond, sms * 7), precision, bg_lanes,
                          b->spec, b->forces, b->stream);
    b->launches = 1 + (b->n_pair ? 1 : 0) + (b->n_bond ? (b->forces ? 2 : 1) : 0);
}

void run(pg_batch* b, int precision, int flags, int pgl, int bgl, bool use_graph) {
    size_buffers(b, precision);
    const pg_batch::Key k{precision, flags, pgl, bgl, state_sum(b), alloc_epoch()};
    if (!(b->have_key && b->key == k)) {
        build(b, precision, flags, pgl, bgl);
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        b->key = pg_batch::Key{precision, flags, pgl, bgl, state_sum(b), alloc_epoch()};
        b->have_key = true;
    }
    if (!use_graph) {
        enqueue(b, precision, pgl, bgl);
        return;
    }
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        PG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue(b, precision, pgl, bgl);
        } catch (...) {
            cudaStreamEndCapture(b->stream, &g);
            if (g) cudaGraphDestroy(g);
            throw;
        }
        PG_CUDA(cudaStreamEndCapture(b->stream, &g));
        cudaError_t e = cudaGraphInstantiate(&b->graph, g, 0);
        cudaGraphDestroy(g);
        PG_CUDA(e);
    }
    PG_CUDA(cudaGraphLaunch(b->graph, b->stream));
}

// the tile pair (pair-kernel lanes, bond-kernel lanes) with the fastest of
// several timed evaluations
void autotune(pg_batch* b, int precision, int flags, int& pgl, int& bgl) {
    const int pair_opts[3] = {8, 16, 32};
    const int bond_opts[3] = {4, 8, PG_LANES_TRIPLET};
    cudaEvent_t e0, e1;
    PG_CUDA(cudaEventCreate(&e0));
    PG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    for (int p : pair_opts)
        for (int q : bond_opts) {
            run(b, precision, flags, p, q, false);  // warm-up and sizing
            float fastest = 1e30f;
            for (int r = 0; r < 3; ++r) {
                PG_CUDA(cudaEventRecord(e0, b->stream));
                enqueue(b, precision, p, q);
                PG_CUDA(cudaEventRecord(e1, b->stream));
                PG_CUDA(cudaEventSynchronize(e1));
                float ms = 0;
                PG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
                fastest = std::min(fastest, ms);
            }
            if (fastest < best) {
                best = fastest;
                pgl = p;
                bgl = q;
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
}

}  // namespace

void batch_create(pg_batch** out, int device) {
    if (device >= 0) PG_CUDA(cudaSetDevice(device));
    int dev = 0;
    PG_CUDA(cudaGetDevice(&dev));
    pg_batch* b = new pg_batch();
    b->device = dev;
    cudaError_t e = cudaStreamCreateWithFlags(&b->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        delete b;
        PG_CUDA(e);
    }
    *out = b;
}

void batch_destroy(pg_batch* b) { delete b; }

void batch_add(pg_batch* b, pg_context* c) {
    require(c != nullptr, PG_ERR_INVALID, "null context");
    require(c->device == b->device, PG_ERR_INVALID, "the context lives on another device than the batch");
    b->sys.push_back(c);
    b->have_key = false;
}

void batch_set_lanes(pg_batch* b, int pair_lanes, int bond_lanes) {
    require(pair_lanes == 0 || pair_lanes == 8 || pair_lanes == 16 || pair_lanes == 32, PG_ERR_INVALID,
            "pair lanes per atom: 0 (autotune), 8, 16 or 32");
    require(bond_lanes == 0 || bond_lanes == 4 || bond_lanes == 8 || bond_lanes == 16 || bond_lanes == 32 ||
                bond_lanes == PG_LANES_TRIPLET,
            PG_ERR_INVALID, "bond-order lanes per atom: 0 (autotune), 4, 8, 16, 32 or PG_LANES_TRIPLET (64)");
    b->pair_lanes = pair_lanes;
    b->bond_lanes = bond_lanes;
}

void batch_get_lanes(pg_batch* b, int precision, int* pair_lanes, int* bond_lanes) {
    const int p = precision == PG_PREC_MIXED ? 1 : 0;
    *pair_lanes = b->pair_lanes ? b->pair_lanes : b->tuned[p][0];
    *bond_lanes = b->bond_lanes ? b->bond_lanes : b->tuned[p][1];
}

void batch_evaluate(pg_batch* b, int precision, int flags, int mode) {
    require(precision == PG_PREC_FP64 || precision == PG_PREC_MIXED, PG_ERR_INVALID, "unknown precision");
    require(!b->sys.empty(), PG_ERR_NOT_READY, "empty batch");
    require((flags & PG_WANT_ENEGS) == 0, PG_ERR_UNSUPPORTED, "the batch evaluates energies and forces");
    require(mode == 0 || mode == 1, PG_ERR_INVALID, "mode: 0 one launch for all systems, 1 one per system");
    if (mode == 1) {
        // the reference arrangement: every system evaluated on its own
        for (pg_context* c : b->sys) evaluate(c, precision, flags);
        b->launches = 0;
        for (pg_context* c : b->sys) b->launches += c->launches;
        return;
    }
    const int p = precision == PG_PREC_MIXED ? 1 : 0;
    int pgl = b->pair_lanes, bgl = b->bond_lanes;
    if (pgl == 0 || bgl == 0) {
        if (b->tuned[p][0] == 0) {
            size_buffers(b, precision);
            int tp = 16, tb = 4;
            autotune(b, precision, flags, tp, tb);
            b->tuned[p][0] = tp;
            b->tuned[p][1] = tb;
        }
        if (pgl == 0) pgl = b->tuned[p][0];
        if (bgl == 0) bgl = b->tuned[p][1];
    }
    run(b, precision, flags, pgl, bgl, true);
}

void batch_synchronize(pg_batch* b) {
    PG_CUDA(cudaStreamSynchronize(b->stream));
    for (pg_context* c : b->sys) PG_CUDA(cudaStreamSynchronize(c->stream));
}

int batch_launches(const pg_batch* b) { return b->launches; }
cudaStream_t batch_stream(const pg_batch* b) { return b->stream; }

}  // namespace pg
