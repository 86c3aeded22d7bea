// batch.cu -- many independent systems evaluated together.
//
// No counterpart in the reference, which holds one system per process in its
// Fortran core (Core.f90:22-30).  A batch borrows contexts that are each fully
// set up (cell, atoms, interactions, neighbour lists).  Three arrangements:
//   mode 0  ONE persistent launch (persist.cuh): resident blocks take
//           (phase, system, blocks) tiles from a work list in dependency order
//           -- displacements, pair terms, bond pass, gather -- with bounded
//           per-system waits; captured in a CUDA graph with the reset of its
//           counters and replayed;
//   mode 1  every system evaluated on its own (the reference's arrangement);
//   mode 2  one launch per phase over the tile list of all systems (four
//           launches in a CUDA graph).
// Each system's results land in its own context (pg_device_results reads them).
//
// Tiles: lanes per atom of the pair body (atoms per warp 32/G) and of the
// bond-order body (one bond per lane, or the triplet tile) and, for the
// persistent launch, the cells (blocks of 128 threads' atoms) one ticket hands
// out, are chosen by timing the candidates on the batch itself unless set
// explicitly.
#include <algorithm>
#include <vector>

#include "args.cuh"
#include "common.cuh"
#include "persist.cuh"

struct pg_batch {
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<pg_context*> sys;
    int pair_lanes = 0, bond_lanes = 0, tile_blocks = 0;  // 0: autotune
    int tuned[2][2] = {{0, 0}, {0, 0}};                   // phase launches: [precision][pair, bond]
    int tuned_p[2][3] = {{0, 0, 0}, {0, 0, 0}};           // persistent: [precision][pair, bond, cells]
    pg::DevBuf<pg::PairArgs> d_pair;
    pg::DevBuf<pg::BondArgs> d_bond;
    pg::DevBuf<pg::DispArgs> d_disp;
    pg::DevBuf<int2> t_pair, t_bond, t_disp;
    int n_pair = 0, n_bond = 0, n_disp = 0;
    // the persistent launch: per-system argument records, tiles, counters
    pg::DevBuf<pg::PairArgs> p_pair;
    pg::DevBuf<pg::BondArgs> p_bond;
    pg::DevBuf<pg::DispArgs> p_disp;
    pg::DevBuf<pg::PTile> p_tiles;
    pg::DevBuf<unsigned> p_sync;  // ticket, status, then 4 counters per system
    pg::PinnedBuf<int> h_status;
    int p_ntiles = 0;
    bool status_pending = false;
    int stall = -1;                            // test hook: system whose dependencies never complete
    unsigned long long wait_ns = 500000000ull;  // limit of one wait of the persistent launch
    bool spec = false, forces = false;
    struct Key {
        int precision, flags, pg, bg, cpb, mode, stall;
        unsigned long long state, alloc;
        bool operator==(const Key& o) const {
            return precision == o.precision && flags == o.flags && pg == o.pg && bg == o.bg && cpb == o.cpb &&
                   mode == o.mode && stall == o.stall && state == o.state && alloc == o.alloc;
        }
    };
    bool have_key = false;
    Key key{};
    // the systems' states (state_sum, alloc_epoch) when their own streams were
    // last waited for
    bool synced = false;
    unsigned long long synced_state = 0, synced_alloc = 0;
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
        require(!c->ewald && !c->have_triplets && c->n_agroups == 0 && !c->have_bond_charge_terms, PG_ERR_UNSUPPORTED,
                "the many-system launch covers pair and Tersoff bond-order terms; evaluate Ewald, three-body or "
                "per-atom bond-order systems one by one");
        const size_t n = (size_t)std::max(c->n, 1);
        c->out_f.resize(3 * n);
        c->out_chi.resize(n);
        c->out_acc.resize(8);
        if (precision == PG_PREC_MIXED) c->disp32.resize(n);
        if (c->have_bond_terms) prepare_bond_scratch(c, precision);
    }
    // The batch runs on its own stream and reads what the systems' streams
    // wrote: a list build or an upload may still be in flight there (the
    // short-list build returns without waiting).  Whenever a system's state
    // or any buffer changed, wait for every system's stream first.
    const unsigned long long st = state_sum(b), al = alloc_epoch();
    if (!b->synced || st != b->synced_state || al != b->synced_alloc) {
        for (pg_context* c : b->sys) PG_CUDA(cudaStreamSynchronize(c->stream));
        b->synced = true;
        b->synced_state = st;
        b->synced_alloc = al;
    }
}

// atoms per block of the pair body at G lanes (128 threads)
int pair_atoms_per_block(int G) { return PAIR_THREADS / G; }

// argument records and tile lists of all systems, uploaded to the device.
// mode 2: per-phase tile lists (int2 system slot, block); mode 0: the
// persistent work list (per-system records, tiles of cpb blocks in dependency
// order, the tile counts each phase waits for).
void build(pg_batch* b, int precision, int flags, int pg_lanes, int bg_lanes, int cpb, int mode) {
    const bool wantF = flags & PG_WANT_FORCES;
    const int ns = (int)b->sys.size();
    std::vector<PairArgs> pa;
    std::vector<BondArgs> ba;
    std::vector<DispArgs> da;
    std::vector<int2> tp, tb, td;
    std::vector<PTile> pt[4];
    std::vector<int4> need((size_t)ns, make_int4(0, 0, 0, 0));
    bool all_spec = true, any_bond = false;
    auto tiles_of = [&](int phase, int s, int nblocks) {
        int count = 0;
        for (int k = 0; k < nblocks; k += cpb, ++count)
            pt[phase].push_back(PTile{phase, s, k, std::min(cpb, nblocks - k), 0, 0, 0, 0});
        return count;
    };
    for (int s = 0; s < ns; ++s) {
        pg_context* c = b->sys[(size_t)s];
        FxAcc* acc = c->out_acc.p;
        const bool run_pair = c->have_pair_kernel_terms || c->have_singles;
        const bool run_bond = c->have_bond_terms;
        require(run_pair || run_bond, PG_ERR_NOT_READY, "a system of the batch has no interactions");
        const DispArgs D = make_disp_args(c, precision == PG_PREC_MIXED ? c->disp32.p : nullptr, nullptr, acc);
        PairArgs P{};
        BondArgs B{};
        if (run_pair) P = make_pair_args(c, precision, flags, true, true, acc, nullptr);
        if (run_bond) {
            any_bond = true;
            all_spec = all_spec && c->spec_ok;
            B = make_bond_args(c, precision, flags, !run_pair, acc);
            B.nblocks = bond_blocks(c->n, bg_lanes);
        }
        const int ap = pair_atoms_per_block(pg_lanes);
        const int n_pb = run_pair ? std::max(1, (c->n + ap - 1) / ap) : 0;
        if (mode == 0) {
            da.push_back(D);
            pa.push_back(P);
            ba.push_back(B);
            const int nd = std::max(1, (c->n + PERSIST_THREADS - 1) / PERSIST_THREADS);
            need[(size_t)s].x = tiles_of(0, s, nd);
            need[(size_t)s].y = run_pair ? tiles_of(1, s, n_pb) : 0;
            need[(size_t)s].z = run_bond ? tiles_of(2, s, B.nblocks) : 0;
            if (run_bond && wantF) tiles_of(3, s, B.nblocks);
            if (s == b->stall) need[(size_t)s].x += 1;  // a displacement tile that never comes
        } else {
            da.push_back(D);
            const int nd = std::max(1, (c->n + DISP_THREADS - 1) / DISP_THREADS);
            for (int k = 0; k < nd; ++k) td.push_back(make_int2(s, k));
            if (run_pair) {
                const int slot = (int)pa.size();
                pa.push_back(P);
                for (int k = 0; k < n_pb; ++k) tp.push_back(make_int2(slot, k));
            }
            if (run_bond) {
                const int slot = (int)ba.size();
                ba.push_back(B);
                for (int k = 0; k < B.nblocks; ++k) tb.push_back(make_int2(slot, k));
            }
        }
    }
    b->spec = any_bond && all_spec;
    b->forces = wantF;
    if (mode == 0) {
        // phase-major: every displacement tile, every pair tile, every bond
        // tile, every gather tile, each phase in system order.  Every dependency
        // sits earlier in the list, and the resident blocks mostly run the same
        // phase's code at a time (one body in the instruction caches); a block
        // moves on to the next phase's tiles without waiting for the others.
        std::vector<PTile> all;
        for (int ph = 0; ph < 4; ++ph) all.insert(all.end(), pt[ph].begin(), pt[ph].end());
        for (PTile& T : all) {  // the counts each tile waits for
            const int4 nd = need[(size_t)T.sys];
            if (T.phase == 1 || T.phase == 2) T.need0 = nd.x;
            if (T.phase == 3) {
                T.need0 = nd.z;
                T.need1 = nd.y;
            }
        }
        b->p_ntiles = (int)all.size();
        b->p_disp.upload(da.data(), da.size(), b->stream);
        b->p_pair.upload(pa.data(), pa.size(), b->stream);
        b->p_bond.upload(ba.data(), ba.size(), b->stream);
        b->p_tiles.upload(all.data(), all.size(), b->stream);
        b->p_sync.resize(2 + 4 * (size_t)ns);
        b->n_pair = b->n_bond = b->n_disp = 0;
    } else {
        b->n_pair = (int)tp.size();
        b->n_bond = (int)tb.size();
        b->n_disp = (int)td.size();
        if (!pa.empty()) b->d_pair.upload(pa.data(), pa.size(), b->stream);
        if (!ba.empty()) b->d_bond.upload(ba.data(), ba.size(), b->stream);
        b->d_disp.upload(da.data(), da.size(), b->stream);
        if (!tp.empty()) b->t_pair.upload(tp.data(), tp.size(), b->stream);
        if (!tb.empty()) b->t_bond.upload(tb.data(), tb.size(), b->stream);
        b->t_disp.upload(td.data(), td.size(), b->stream);
    }
    PG_CUDA(cudaStreamSynchronize(b->stream));
}

void enqueue(pg_batch* b, int precision, int pg_lanes, int bg_lanes, int mode) {
    const int sms = sm_count();
    if (mode == 0) {
        PersistArgs P{};
        P.disp = b->p_disp.p;
        P.pair = b->p_pair.p;
        P.bond = b->p_bond.p;
        P.tiles = b->p_tiles.p;
        P.ntiles = b->p_ntiles;
        P.ticket = b->p_sync.p;
        P.status = (int*)(b->p_sync.p + 1);
        P.done = b->p_sync.p + 2;
        P.wait_ns = b->wait_ns;
        PG_CUDA(cudaMemsetAsync(b->p_sync.p, 0, sizeof(unsigned) * b->p_sync.n, b->stream));
        const bool f32 = precision == PG_PREC_MIXED;
        if (f32 && b->spec) launch_persistent_f32_spec(P, pg_lanes, bg_lanes, sms, b->stream);
        else if (f32) launch_persistent_f32_table(P, pg_lanes, bg_lanes, sms, b->stream);
        else if (b->spec) launch_persistent_f64_spec(P, pg_lanes, bg_lanes, sms, b->stream);
        else launch_persistent_f64_table(P, pg_lanes, bg_lanes, sms, b->stream);
        PG_CHECK_LAUNCH();
        b->launches = 1;
        return;
    }
    launch_disp_batch(b->d_disp.p, b->t_disp.p, b->n_disp, std::min(b->n_disp, sms * 8), b->stream);
    if (b->n_pair)
        launch_pair_batch(b->d_pair.p, b->t_pair.p, b->n_pair, std::min(b->n_pair, sms * 12), PAIR_THREADS,
                          precision, pg_lanes, b->stream);
    if (b->n_bond)
        launch_bond_batch(b->d_bond.p, b->t_bond.p, b->n_bond, std::min(b->n_bond, sms * 7), precision, bg_lanes,
                          b->spec, b->forces, b->stream);
    b->launches = 1 + (b->n_pair ? 1 : 0) + (b->n_bond ? (b->forces ? 2 : 1) : 0);
}

// the persistent launch's status word to the host with the results
void fetch_status(pg_batch* b) {
    int* h = b->h_status.get(1);
    *h = 0;
    PG_CUDA(cudaMemcpyAsync(h, b->p_sync.p + 1, sizeof(int), cudaMemcpyDeviceToHost, b->stream));
    b->status_pending = true;
}

void run(pg_batch* b, int precision, int flags, int pgl, int bgl, int cpb, int mode, bool use_graph) {
    size_buffers(b, precision);
    const pg_batch::Key k{precision, flags, pgl, bgl, mode == 0 ? cpb : 0, mode, b->stall, state_sum(b),
                          alloc_epoch()};
    if (!(b->have_key && b->key == k)) {
        build(b, precision, flags, pgl, bgl, cpb, mode);
        if (b->graph) {
            cudaGraphExecDestroy(b->graph);
            b->graph = nullptr;
        }
        b->key = k;
        b->have_key = true;
    }
    if (!use_graph) {
        enqueue(b, precision, pgl, bgl, mode);
        if (mode == 0) fetch_status(b);
        return;
    }
    if (!b->graph) {
        cudaGraph_t g = nullptr;
        PG_CUDA(cudaStreamBeginCapture(b->stream, cudaStreamCaptureModeThreadLocal));
        try {
            enqueue(b, precision, pgl, bgl, mode);
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
    b->launches = mode == 0 ? 1 : b->launches;
    if (mode == 0) fetch_status(b);
}

// time one candidate tile: the fastest of three evaluations (device events)
float time_candidate(pg_batch* b, int precision, int flags, int p, int q, int c, int mode, cudaEvent_t e0,
                     cudaEvent_t e1) {
    run(b, precision, flags, p, q, c, mode, false);  // warm-up and sizing
    PG_CUDA(cudaStreamSynchronize(b->stream));
    require(mode != 0 || *b->h_status.p == 0, PG_ERR_TIMEOUT,
            "a wait of the persistent batch launch ran out (status word set)");
    b->status_pending = false;
    float fastest = 1e30f;
    for (int r = 0; r < 3; ++r) {
        PG_CUDA(cudaEventRecord(e0, b->stream));
        enqueue(b, precision, p, q, mode);
        PG_CUDA(cudaEventRecord(e1, b->stream));
        PG_CUDA(cudaEventSynchronize(e1));
        float ms = 0;
        PG_CUDA(cudaEventElapsedTime(&ms, e0, e1));
        fastest = std::min(fastest, ms);
    }
    return fastest;
}

// phase launches: the (pair lanes, bond lanes) pair with the fastest timed
// evaluation; persistent launch: (pair lanes, bond lanes, cells per ticket)
void autotune(pg_batch* b, int precision, int flags, int mode, int& pgl, int& bgl, int& cpb) {
    cudaEvent_t e0, e1;
    PG_CUDA(cudaEventCreate(&e0));
    PG_CUDA(cudaEventCreate(&e1));
    float best = 1e30f;
    const int bond_opts[3] = {4, 8, PG_LANES_TRIPLET};
    try {
        if (mode == 0) {
            const int pair_opts[2] = {8, 16};
            const int cell_opts[3] = {1, 2, 4};
            for (int p : pair_opts)
                for (int q : bond_opts)
                    for (int c : cell_opts) {
                        const float t = time_candidate(b, precision, flags, p, q, c, 0, e0, e1);
                        if (t < best) {
                            best = t;
                            pgl = p;
                            bgl = q;
                            cpb = c;
                        }
                    }
        } else {
            const int pair_opts[3] = {8, 16, 32};
            for (int p : pair_opts)
                for (int q : bond_opts) {
                    const float t = time_candidate(b, precision, flags, p, q, 1, 2, e0, e1);
                    if (t < best) {
                        best = t;
                        pgl = p;
                        bgl = q;
                    }
                }
        }
    } catch (...) {
        cudaEventDestroy(e0);
        cudaEventDestroy(e1);
        throw;
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

void batch_set_tile_blocks(pg_batch* b, int blocks) {
    require(blocks >= 0 && blocks <= 64, PG_ERR_INVALID, "cells per tile: 0 (autotune) to 64");
    b->tile_blocks = blocks;
}

void batch_test_stall(pg_batch* b, int system, double wait_seconds) {
    require(system >= -1 && system < (int)b->sys.size(), PG_ERR_INVALID, "no such system in the batch");
    require(wait_seconds > 0.0 && wait_seconds <= 1.0, PG_ERR_INVALID, "wait limit: (0, 1] s");
    b->stall = system;
    b->wait_ns = (unsigned long long)(wait_seconds * 1e9);
}

void batch_get_lanes(pg_batch* b, int precision, int* pair_lanes, int* bond_lanes) {
    const int p = precision == PG_PREC_MIXED ? 1 : 0;
    *pair_lanes = b->pair_lanes ? b->pair_lanes : b->tuned_p[p][0];
    *bond_lanes = b->bond_lanes ? b->bond_lanes : b->tuned_p[p][1];
}

void batch_get_tiles(pg_batch* b, int precision, int mode, int* pair_lanes, int* bond_lanes, int* blocks) {
    const int p = precision == PG_PREC_MIXED ? 1 : 0;
    if (mode == 2) {
        *pair_lanes = b->pair_lanes ? b->pair_lanes : b->tuned[p][0];
        *bond_lanes = b->bond_lanes ? b->bond_lanes : b->tuned[p][1];
        *blocks = 1;
        return;
    }
    *pair_lanes = b->pair_lanes ? b->pair_lanes : b->tuned_p[p][0];
    *bond_lanes = b->bond_lanes ? b->bond_lanes : b->tuned_p[p][1];
    *blocks = b->tile_blocks ? b->tile_blocks : b->tuned_p[p][2];
}

void batch_evaluate(pg_batch* b, int precision, int flags, int mode) {
    require(precision == PG_PREC_FP64 || precision == PG_PREC_MIXED, PG_ERR_INVALID, "unknown precision");
    require(!b->sys.empty(), PG_ERR_NOT_READY, "empty batch");
    require((flags & PG_WANT_ENEGS) == 0, PG_ERR_UNSUPPORTED, "the batch evaluates energies and forces");
    require(mode == 0 || mode == 1 || mode == 2, PG_ERR_INVALID,
            "mode: 0 one persistent launch, 1 one evaluation per system, 2 one launch per phase");
    if (mode == 1) {
        // the reference arrangement: every system evaluated on its own
        for (pg_context* c : b->sys) evaluate(c, precision, flags);
        b->launches = 0;
        for (pg_context* c : b->sys) b->launches += c->launches;
        return;
    }
    const int p = precision == PG_PREC_MIXED ? 1 : 0;
    int pgl = b->pair_lanes, bgl = b->bond_lanes, cpb = b->tile_blocks;
    if (mode == 0) {
        require(pgl == 0 || pgl == 8 || pgl == 16, PG_ERR_INVALID,
                "the persistent launch takes 8 or 16 pair lanes per atom");
        require(bgl == 0 || bgl == 4 || bgl == 8 || bgl == PG_LANES_TRIPLET, PG_ERR_INVALID,
                "the persistent launch takes 4 or 8 bond lanes per atom or the triplet tile");
        if (pgl == 0 || bgl == 0 || cpb == 0) {
            if (b->tuned_p[p][0] == 0) {
                size_buffers(b, precision);
                int tp = 8, tb = 4, tc = 1;
                autotune(b, precision, flags, 0, tp, tb, tc);
                b->tuned_p[p][0] = tp;
                b->tuned_p[p][1] = tb;
                b->tuned_p[p][2] = tc;
            }
            if (pgl == 0) pgl = b->tuned_p[p][0];
            if (bgl == 0) bgl = b->tuned_p[p][1];
            if (cpb == 0) cpb = b->tuned_p[p][2];
        }
    } else {
        if (pgl == 0 || bgl == 0) {
            if (b->tuned[p][0] == 0) {
                size_buffers(b, precision);
                int tp = 16, tb = 4, tc = 1;
                autotune(b, precision, flags, 2, tp, tb, tc);
                b->tuned[p][0] = tp;
                b->tuned[p][1] = tb;
            }
            if (pgl == 0) pgl = b->tuned[p][0];
            if (bgl == 0) bgl = b->tuned[p][1];
        }
        cpb = 1;
    }
    run(b, precision, flags, pgl, bgl, cpb, mode, true);
}

void batch_synchronize(pg_batch* b) {
    PG_CUDA(cudaStreamSynchronize(b->stream));
    for (pg_context* c : b->sys) PG_CUDA(cudaStreamSynchronize(c->stream));
    if (b->status_pending) {
        b->status_pending = false;
        require(*b->h_status.p == 0, PG_ERR_TIMEOUT,
                "a wait of the persistent batch launch ran out: the results of this evaluation are not valid");
    }
}

int batch_launches(const pg_batch* b) { return b->launches; }
cudaStream_t batch_stream(const pg_batch* b) { return b->stream; }

}  // namespace pg
