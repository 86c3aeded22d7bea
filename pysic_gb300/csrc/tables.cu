// tables.cu -- fold the interaction records into dense per-type tables.
//
// The reference walks, for every pair of atoms, the list of records that
// target the first atom and tests the second atom's element, tag or index
// (core_evaluate_local_doublet_*_B, Core.f90:4257-5606 with
// potential_affects_atom, Potentials.f90:1195-1259).  Here that test is done
// once per pair of atom types: table[ti][tj] lists the pair terms that apply,
// trip[ti][tj][tk] the Tersoff parameters of a triplet, post[ti][tj] the
// B(zeta) parameters of a centre type (core_post_process_pair_bond_order_factor,
// Core.f90:2763-2807: the first matching factor), maxbr[ti] the largest
// bond-order cutoff of the type (max_bond_radius, Core.f90:1030-1067).
#include <algorithm>
#include <map>
#include <set>
#include <vector>

#include "common.cuh"

namespace pg {

static inline bool has(uint64_t m, int t) { return (m >> t) & 1ull; }

void fold_tables(pg_context* ctx) {
    const int T = std::max(ctx->n_types, 1);
    cudaStream_t st = ctx->stream;
    for (int t : ctx->h_type)
        require(t < T, PG_ERR_INVALID, "atom type outside the interaction tables (set the potentials after the atoms)");
    const int nb = (int)ctx->br_cut.size();
    // Coordinator groups: groups of Tersoff factors (evaluated by the
    // bond-order kernels; each pair type takes the factors and post-processing
    // of the group its scaled terms name) and up to PG_MAX_AGROUPS groups of
    // per-atom factors (atomfactor.cu)
    std::set<int> tersoff_groups;
    for (int b = 0; b < nb; ++b) {
        require(ctx->br_group[b] >= 0, PG_ERR_INVALID, "a Tersoff factor without a group");
        tersoff_groups.insert(ctx->br_group[b]);
    }
    const int np0 = (int)ctx->pr_cut.size();
    // the Tersoff group of each (ti, tj) pair type: the one its scaled terms name
    std::vector<int> owner((size_t)T * T, -1);
    for (int r = 0; r < np0; ++r) {
        const int g = ctx->pr_group[r];
        if (!tersoff_groups.count(g)) continue;
        for (int ti = 0; ti < T; ++ti)
            for (int tj = 0; tj < T; ++tj) {
                if (!has(ctx->pr_m1[r], ti) || !has(ctx->pr_m2[r], tj)) continue;
                int& o = owner[(size_t)ti * T + tj];
                require(o < 0 || o == g, PG_ERR_UNSUPPORTED,
                        "one pair type scaled by two Coordinators of Tersoff factors is not evaluated by the GB300 "
                        "engine (one Tersoff group per element pair)");
                o = g;
            }
    }
    const int tersoff_gid = tersoff_groups.empty() ? -1 : *tersoff_groups.begin();
    std::map<int, int> gmap;  // coordinator group -> per-atom factor group
    for (size_t r = 0; r < ctx->af_kind.size(); ++r) {
        const int g = ctx->af_group[r];
        require(g >= 0 && !tersoff_groups.count(g), PG_ERR_UNSUPPORTED,
                "a Coordinator mixing per-atom and Tersoff factors is not evaluated by the GB300 engine");
        if (!gmap.count(g)) {
            require((int)gmap.size() < PG_MAX_AGROUPS, PG_ERR_UNSUPPORTED,
                    "more than 4 Coordinators of per-atom bond-order factors");
            const int k = (int)gmap.size();
            gmap[g] = k;
        }
    }
    ctx->n_agroups = (int)gmap.size();
    ctx->agroup_of = gmap;

    // bond-order tables
    std::vector<TripT<double>> trip((size_t)T * T * T);
    for (auto& t : trip) t = TripT<double>{};
    // per (ti, tj): the post-processing of the first factor of the pair type's
    // group centred on ti (core_post_process_pair_bond_order_factor, Core.f90:
    // 2763-2807); pair types no scaled term names take the first group's
    std::vector<PostT<double>> post((size_t)T * T, PostT<double>{0, 0, 0});
    std::vector<double> maxbr(T, 0.0);
    double bo_radius = 0.0;
    auto group_of_pair = [&](int ti, int tj) {
        const int o = owner[(size_t)ti * T + tj];
        return o >= 0 ? o : tersoff_gid;
    };
    for (int b = 0; b < nb; ++b) {
        const double* p = &ctx->br_params[7 * (size_t)b];
        bo_radius = std::max(bo_radius, ctx->br_cut[b]);
        for (int ti = 0; ti < T; ++ti) {
            if (!has(ctx->br_m1[b], ti)) continue;
            if (ctx->br_cut[b] > maxbr[ti]) maxbr[ti] = ctx->br_cut[b];
            for (int tj = 0; tj < T; ++tj) {
                if (ctx->br_group[b] != group_of_pair(ti, tj)) continue;
                PostT<double>& pp = post[(size_t)ti * T + tj];
                if (!pp.valid) pp = PostT<double>{p[0], p[1], 1};
                if (!has(ctx->br_m2[b], tj)) continue;
                for (int tk = 0; tk < T; ++tk) {
                    if (!has(ctx->br_m3[b], tk)) continue;
                    TripT<double>& tt = trip[((size_t)ti * T + tj) * T + tk];
                    require(!tt.valid, PG_ERR_UNSUPPORTED,
                            "two Tersoff factors act on the same (i, j, k) element triple");
                    tt.a = p[2];
                    tt.c2 = p[3] * p[3];
                    tt.d2 = p[4] * p[4];
                    tt.c2d2 = tt.c2 / tt.d2;
                    tt.h = p[5];
                    tt.mu = p[6];
                    tt.rc = ctx->br_cut[b];
                    tt.rs = ctx->br_soft[b];
                    tt.valid = 1;
                }
            }
        }
    }
    // cutoff of bond ik per (ti, tk): one pair (rc, rs) shared by all tj, or not uniform
    std::vector<double2> bcut((size_t)T * T, make_double2(0.0, 0.0));
    bool uniform = true;
    for (int ti = 0; ti < T; ++ti)
        for (int tk = 0; tk < T; ++tk) {
            bool seen = false;
            for (int tj = 0; tj < T; ++tj) {
                const TripT<double>& tt = trip[((size_t)ti * T + tj) * T + tk];
                if (!tt.valid) continue;
                double2& c = bcut[(size_t)ti * T + tk];
                if (!seen) {
                    c = make_double2(tt.rc, tt.rs);
                    seen = true;
                } else if (c.x != tt.rc || c.y != tt.rs) {
                    uniform = false;
                }
            }
        }
    ctx->bcut_uniform = uniform;
    std::vector<float2> bcut32(bcut.size());
    for (size_t q = 0; q < bcut.size(); ++q) bcut32[q] = make_float2((float)bcut[q].x, (float)bcut[q].y);
    ctx->d_bcut.upload(bcut.data(), bcut.size(), st);
    ctx->d_bcut32.upload(bcut32.data(), bcut32.size(), st);

    // pair terms: bond-order scaled terms define the bond-order kernel's reach
    const int np = (int)ctx->pr_cut.size();
    for (int r = 0; r < np; ++r)
        if (ctx->pr_group[r] >= 0) {
            require(tersoff_groups.count(ctx->pr_group[r]) || gmap.count(ctx->pr_group[r]), PG_ERR_INVALID,
                    "a potential has a coordinator without bond-order factors");
            if (tersoff_groups.count(ctx->pr_group[r])) bo_radius = std::max(bo_radius, ctx->pr_cut[r]);
        }
    const bool bond = nb > 0;
    ctx->have_bond_terms = bond;
    ctx->bo_radius = bo_radius;

    std::vector<PairT<double>> terms;
    std::vector<PairT<double>> factors;  // product factors, appended after every type pair's records
    std::vector<int2> index((size_t)T * T, make_int2(0, 0));
    bool pair_kernel_terms = false, charge_pairs = false, bond_charge_terms = false;
    // one pair term from a kind and 4 parameters (table rows checked here: the
    // kernels index rows t0 .. t0 + tn - 1 only)
    auto fill_params = [&](PairT<double>& t, const double* p4) {
        t.p0 = p4[0];
        t.p1 = p4[1];
        t.p2 = p4[2];
        t.p3 = p4[3];
        if (t.kind == 8 || t.kind == 9) {  // charge_exp / charge_abs: parameters as rows of the table array
            t.t0 = (int)t.p0;
            t.tn = t.kind == 8 ? 8 : 4;
            require(t.t0 >= 0 && (size_t)t.t0 + (size_t)t.tn <= ctx->pr_table.size() / 2, PG_ERR_INVALID,
                    "charge_exp / charge_abs: parameter rows out of bounds");
        }
        if (t.kind == 6) {  // tabulated: params first row, rows, range, scale
            t.t0 = (int)t.p0;
            t.tn = (int)t.p1;
            require(t.t0 >= 0 && t.tn >= 2 && (size_t)t.t0 + (size_t)t.tn <= ctx->pr_table.size() / 2 && t.p2 > 0.0,
                    PG_ERR_INVALID, "tabulated potential: table rows or range out of bounds");
            t.p0 = t.p2;  // range
            t.p1 = t.p3;  // scale
        }
        t.ni = t.kind == 4 ? integral_exponent(t.p2) : t.kind == 5 ? integral_exponent(t.p3) : PG_NOT_INT;
    };
    const bool have_products = (int)ctx->pr_nmul.size() == np;
    for (int ti = 0; ti < T; ++ti)
        for (int tj = 0; tj < T; ++tj) {
            int2& ix = index[(size_t)ti * T + tj];
            ix.x = (int)terms.size();
            for (int r = 0; r < np; ++r) {
                if (!has(ctx->pr_m1[r], ti) || !has(ctx->pr_m2[r], tj)) continue;
                PairT<double> t{};
                t.kind = ctx->pr_kind[r];
                const int g = ctx->pr_group[r];
                t.group = g >= 0 && tersoff_groups.count(g) ? 0 : -1;
                t.agroup = g >= 0 && !tersoff_groups.count(g) ? gmap.at(g) : -1;
                require(!(t.kind == 10 && (g >= 0 || (have_products && ctx->pr_nmul[r] > 0))), PG_ERR_UNSUPPORTED,
                        "step: bond-order scaling and products are not evaluated by the GB300 engine (its force is "
                        "not radial)");
                require(!(t.agroup >= 0 && t.kind >= 7), PG_ERR_UNSUPPORTED,
                        "per-atom bond-order scaling of charge-dependent terms is not evaluated by the GB300 engine");
                require(!(t.agroup >= 0 && have_products && ctx->pr_nmul[r] > 0), PG_ERR_UNSUPPORTED,
                        "per-atom bond-order scaling of products is not evaluated by the GB300 engine");
                fill_params(t, &ctx->pr_params[4 * (size_t)r]);
                t.first = r < (int)ctx->pr_first.size() ? ctx->pr_first[r] : 0ull;
                t.rc = ctx->pr_cut[r];
                // a product: its factors, in the record's own order
                t.nmul = have_products ? ctx->pr_nmul[r] : 0;
                t.mul0 = (int)factors.size();
                for (int c = 0; c < t.nmul; ++c) {
                    const int f = ctx->pr_mul0[r] + c;
                    PairT<double> u{};
                    u.kind = ctx->pm_kind[f];
                    require(u.kind != 10, PG_ERR_UNSUPPORTED,
                            "step: products are not evaluated by the GB300 engine (its force is not radial)");
                    u.group = u.agroup = -1;
                    fill_params(u, &ctx->pm_params[4 * (size_t)f]);
                    u.first = ctx->pm_first[f];
                    u.rc = u.rs = ctx->pr_cut[r];  // a spring factor is shifted at the product's cutoff
                    if (u.kind >= 7 && u.kind <= 9) charge_pairs = true;
                    factors.push_back(u);
                }
                const double soft = ctx->pr_soft[r];
                if (soft > 0.0 && soft < t.rc) {
                    t.smooth = 1;
                    t.rs = soft;
                } else {
                    t.smooth = 0;
                    t.rs = t.rc;
                }
                // unscaled charge-dependent and product terms stay in the pair kernel;
                // Tersoff-scaled ones go to the bond-order kernels, which then also
                // give their electronegativities (bond_chi)
                // (step, kind 10, has a force that is not radial: it stays in the pair kernel)
                const bool charge = t.kind >= 7 && t.kind <= 9;
                const bool qterm = charge || t.nmul > 0;
                t.in_bond_kernel = bond && t.agroup < 0 && t.kind != 10 &&
                                   (qterm ? t.group >= 0 : (t.group >= 0 || t.rc <= bo_radius));
                if (t.in_bond_kernel && qterm) bond_charge_terms = true;
                if (charge) charge_pairs = true;
                if (!t.in_bond_kernel) pair_kernel_terms = true;
                terms.push_back(t);
            }
            ix.y = (int)terms.size() - ix.x;
        }
    // the factors after all records; the records' factor indices point there
    {
        const int base = (int)terms.size();
        for (auto& t : terms)
            if (t.nmul > 0) t.mul0 += base;
        terms.insert(terms.end(), factors.begin(), factors.end());
    }
    // single-atom terms
    std::vector<SingleTerm> sterms;
    std::vector<int2> sindex(T, make_int2(0, 0));
    const int ns = (int)ctx->sr_kind.size();
    for (int t = 0; t < T; ++t) {
        sindex[t].x = (int)sterms.size();
        for (int r = 0; r < ns; ++r)
            if (has(ctx->sr_m[r], t)) {
                SingleTerm s{};
                s.kind = ctx->sr_kind[r];
                const int g = r < (int)ctx->sr_group.size() ? ctx->sr_group[r] : -1;
                s.agroup = -1;
                if (g >= 0) {
                    require(gmap.count(g) > 0, PG_ERR_UNSUPPORTED,
                            "single-atom terms are scaled by per-atom bond-order factors only");
                    require(s.kind != 0, PG_ERR_UNSUPPORTED,
                            "bond-order scaling of charge_self is not evaluated by the GB300 engine");
                    s.agroup = gmap.at(g);
                }
                for (int c = 0; c < 3; ++c) s.p[c] = ctx->sr_params[4 * (size_t)r + c];
                s.n = s.kind == 0 ? (int)s.p[1] : 0;  // charge_self: the reference's integer n = int(param2)
                sterms.push_back(s);
            }
        sindex[t].y = (int)sterms.size() - sindex[t].x;
    }
    ctx->have_singles = !sterms.empty();
    {
        bool scaled_pairs = false;
        for (const auto& t : terms) scaled_pairs = scaled_pairs || t.agroup >= 0;
        ctx->af_fused = ctx->n_agroups > 0 && !scaled_pairs;
    }
    ctx->have_pair_kernel_terms = pair_kernel_terms;
    ctx->have_charge_pairs = charge_pairs;
    ctx->have_bond_charge_terms = bond_charge_terms;

    // Single-species Tersoff (one type, one triplet, exponential pair terms that
    // all share the bond-order cutoff): the bond-order kernels take every
    // parameter as a kernel argument instead of looking tables up per triplet.
    ctx->spec_ok = false;
    if (T == 1 && trip[0].valid && post[0].valid && maxbr[0] == trip[0].rc) {
        const TripT<double>& t0 = trip[0];
        // the pair terms that run in the bond-order kernels (terms with a longer
        // reach, e.g. an added Lennard-Jones, stay in the pair kernel)
        std::vector<const PairT<double>*> bt;
        for (int q = 0; q < index[0].y; ++q) {
            const PairT<double>& pt = terms[(size_t)index[0].x + q];
            if (pt.in_bond_kernel) bt.push_back(&pt);
        }
        bool ok = !bt.empty() && (int)bt.size() <= PG_SPEC_MAX_TERMS;
        int mask = 0;
        for (size_t q = 0; ok && q < bt.size(); ++q) {
            const PairT<double>& pt = *bt[q];
            ok = pt.kind == 1 && pt.smooth && pt.rc == t0.rc && pt.rs == t0.rs;
            if (pt.group >= 0) mask |= 1 << q;
        }
        if (ok && mask != 0) {
            double* v = ctx->spec;
            v[SP_RC] = t0.rc;
            v[SP_RS] = t0.rs;
            v[SP_BETA] = post[0].beta;
            v[SP_ETA] = post[0].eta;
            v[SP_A] = t0.a;
            v[SP_C2] = t0.c2;
            v[SP_D2] = t0.d2;
            v[SP_C2D2] = t0.c2d2;
            v[SP_H] = t0.h;
            v[SP_MU] = t0.mu;
            for (size_t q = 0; q < bt.size(); ++q) {
                v[SP_TERMS + 2 * q] = bt[q]->p0;
                v[SP_TERMS + 2 * q + 1] = bt[q]->p1;
            }
            ctx->spec_nterm = (int)bt.size();
            ctx->spec_bomask = mask;
            ctx->spec_ok = true;
        }
    }

    if (terms.empty()) terms.push_back(PairT<double>{});
    if (sterms.empty()) sterms.push_back(SingleTerm{});
    std::vector<PairT<float>> terms32(terms.size());
    for (size_t q = 0; q < terms.size(); ++q) terms32[q] = cast_pair<float>(terms[q]);
    std::vector<TripT<float>> trip32(trip.size());
    for (size_t q = 0; q < trip.size(); ++q) trip32[q] = cast_trip<float>(trip[q]);
    std::vector<PostT<float>> post32(post.size());
    for (size_t q = 0; q < post.size(); ++q) post32[q] = cast_post<float>(post[q]);
    std::vector<float> maxbr32(maxbr.begin(), maxbr.end());
    ctx->n_pair_terms = (int)terms.size();
    ctx->d_pair_terms.upload(terms.data(), terms.size(), st);
    ctx->d_pair_terms32.upload(terms32.data(), terms32.size(), st);
    ctx->d_pair_index.upload(index.data(), index.size(), st);
    ctx->d_trip.upload(trip.data(), trip.size(), st);
    ctx->d_trip32.upload(trip32.data(), trip32.size(), st);
    ctx->d_post.upload(post.data(), post.size(), st);
    ctx->d_post32.upload(post32.data(), post32.size(), st);
    ctx->d_maxbr.upload(maxbr.data(), maxbr.size(), st);
    ctx->d_maxbr32.upload(maxbr32.data(), maxbr32.size(), st);
    ctx->d_single_terms.upload(sterms.data(), sterms.size(), st);
    ctx->d_single_index.upload(sindex.data(), sindex.size(), st);
    fold_atom_factors(ctx, gmap);
    // three-body records: the derived cos(theta_0)^n (calculate_derived_parameters_
    // bond_bending, Potentials.f90:3183-3194) and the integer exponents n, m
    {
        const int nt3 = (int)ctx->tr_kind.size();
        std::vector<TriT<double>> tri((size_t)std::max(nt3, 1));
        std::vector<TriT<float>> tri32((size_t)std::max(nt3, 1));
        for (int r = 0; r < nt3; ++r) {
            const double* p = ctx->tr_params.data() + 4 * (size_t)r;
            TriT<double> t{};
            t.kind = ctx->tr_kind[r];
            t.eps = p[0];
            t.c0 = std::pow(std::cos(p[1]), p[2]);
            t.n = (int)p[2];
            t.m = (int)p[3];
            t.rc = ctx->tr_cut[r];
            const double soft = ctx->tr_soft[r];
            t.smooth = soft > 0.0 && soft < t.rc;
            t.rs = t.smooth ? soft : t.rc;
            t.m2 = ctx->tr_m2[r];
            t.m3 = ctx->tr_m3[r];
            t.many = ctx->tr_m1[r] | ctx->tr_m2[r] | ctx->tr_m3[r];
            t.center = ctx->tr_center[r];
            tri[(size_t)r] = t;
            tri32[(size_t)r] = TriT<float>{(float)t.eps, (float)t.c0, (float)t.rc, (float)t.rs, t.n, t.m, t.smooth,
                                           t.kind, t.m2, t.m3, t.many, t.center};
        }
        ctx->n_tri = nt3;
        ctx->d_tri.upload(tri.data(), tri.size(), st);
        ctx->d_tri32.upload(tri32.data(), tri32.size(), st);
    }
    // four-body records: cos(phi_0) once per record (the evaluator's cos(params(2)),
    // Potentials.f90:3407)
    {
        const int nq = (int)ctx->qd_kind.size();
        std::vector<QuadT<double>> quad((size_t)std::max(nq, 1));
        std::vector<QuadT<float>> quad32((size_t)std::max(nq, 1));
        for (int r = 0; r < nq; ++r) {
            const double* p = ctx->qd_params.data() + 4 * (size_t)r;
            const uint64_t* mk = ctx->qd_mask.data() + 4 * (size_t)r;
            QuadT<double> q{};
            q.kind = ctx->qd_kind[r];
            q.k = p[0];
            q.cos0 = std::cos(p[1]);
            q.rc = ctx->qd_cut[r];
            const double soft = ctx->qd_soft[r];
            q.smooth = soft > 0.0 && soft < q.rc;
            q.rs = q.smooth ? soft : q.rc;
            q.m2 = mk[1];
            q.m3 = mk[2];
            q.m4 = mk[3];
            q.many = mk[0] | mk[1] | mk[2] | mk[3];
            for (int t = 0; t < 4; ++t) q.orig[t] = ctx->qd_orig[4 * (size_t)r + t];
            quad[(size_t)r] = q;
            QuadT<float> q32{(float)q.k, (float)q.cos0, (float)q.rc, (float)q.rs, q.smooth, q.kind,
                             q.m2, q.m3, q.m4, q.many, {q.orig[0], q.orig[1], q.orig[2], q.orig[3]}};
            quad32[(size_t)r] = q32;
        }
        ctx->n_quad = nq;
        ctx->d_quad.upload(quad.data(), quad.size(), st);
        ctx->d_quad32.upload(quad32.data(), quad32.size(), st);
    }
    ctx->have_triplets = ctx->n_tri > 0 || ctx->n_quad > 0;
    {
        std::vector<double> t64 = ctx->pr_table;
        if (t64.empty()) t64.assign(2, 0.0);
        std::vector<float> t32(t64.begin(), t64.end());
        ctx->d_tab64.upload(t64.data(), t64.size(), st);
        ctx->d_tab32.upload(t32.data(), t32.size(), st);
    }
    PG_CUDA(cudaStreamSynchronize(st));
    ctx->tables_dirty = false;
    ctx->state_epoch++;
    ctx->short_dirty = true;
}

}  // namespace pg
