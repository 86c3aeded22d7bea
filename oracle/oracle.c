/*
 * oracle.c -- FP64 CPU restatement of the Pysic Fortran core.
 *
 * TEST INFRASTRUCTURE: this file is the parity oracle.  Only tests/,
 * __graft_entry__.smoke() and bench.py's cpu_baseline / reference leg load it,
 * and only to check or time the reference algorithm; the product library
 * never links it.
 *
 * Each function follows the reference routine named in its comment, keeping
 * the reference's loop order and the left-to-right order of its floating-point
 * expressions, so that for one thread the results reproduce the reference's
 * arithmetic on a compiler that does not fuse multiply-adds (the recipe in
 * oracle/Makefile builds with -ffp-contract=off).  Paths are relative to the
 * Pysic project root.
 */
#include "oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* Utility.f90:11 */
static const double PI = 3.14159265358979323846;

/* ------------------------------------------------------------------ */
/* Geometry (fortran/Geometry.f90)                                      */
/* ------------------------------------------------------------------ */

typedef struct {
    double vc[3][3];  /* cell%vectors(r,c): component r of cell vector c      */
    double ic[3][3];  /* cell%inverse_cell(r,c)                               */
    double rc[3][3];  /* cell%reciprocal_cell(r,c) = 2 pi inverse(c,r)        */
    double volume;
    int pbc[3];
} fcell;

/* generate_supercell, Geometry.f90:177-195 (with the Python-side transposes of
 * pysic/calculator.py:1555-1565: vectors = cell^T, inverse = inv(cell)^T). */
static void make_cell(const orc_system* s, fcell* C) {
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) {
            C->vc[r][c] = s->cell[c * 3 + r];
            C->ic[r][c] = s->inv[c * 3 + r];
        }
    const double twopi = 2.0 * PI;
    for (int r = 0; r < 3; ++r)
        for (int c = 0; c < 3; ++c) C->rc[r][c] = twopi * C->ic[c][r];
    /* volume = |(v1 x v2) . v3|, Geometry.f90:192 with Quaternions.f90:475-500 */
    double a[3], b[3], d[3];
    for (int r = 0; r < 3; ++r) {
        a[r] = C->vc[r][0];
        b[r] = C->vc[r][1];
        d[r] = C->vc[r][2];
    }
    double x0 = a[1] * b[2] - a[2] * b[1];
    double x1 = a[2] * b[0] - a[0] * b[2];
    double x2 = a[0] * b[1] - a[1] * b[0];
    C->volume = fabs(x0 * d[0] + x1 * d[1] + x2 * d[2]);
    for (int i = 0; i < 3; ++i) C->pbc[i] = s->pbc[i] != 0;
}

/* relative_coordinates, Geometry.f90:510-519 (matmul, summed over c in order) */
static void rel_coords(const fcell* C, const double p[3], double rel[3]) {
    for (int r = 0; r < 3; ++r) rel[r] = C->ic[r][0] * p[0] + C->ic[r][1] * p[1] + C->ic[r][2] * p[2];
}

/* absolute_coordinates, Geometry.f90:531-540 */
static void abs_coords(const fcell* C, const double rel[3], double p[3]) {
    for (int r = 0; r < 3; ++r) p[r] = C->vc[r][0] * rel[0] + C->vc[r][1] * rel[1] + C->vc[r][2] * rel[2];
}

/* wrapped_coordinates, Geometry.f90:597-619 */
static void wrapped_coords(const fcell* C, const double p[3], double w[3], int off[3]) {
    double rel[3];
    rel_coords(C, p, rel);
    for (int i = 0; i < 3; ++i) {
        off[i] = 0;
        if (C->pbc[i]) {
            off[i] = -(int)floor(rel[i]);
            rel[i] = rel[i] + (double)off[i];
        }
    }
    abs_coords(C, rel, w);
}

/* separation_vector, Geometry.f90:449-466 */
static void separation(const fcell* C, const double* r1, const double* r2, const int off[3], double s[3]) {
    for (int c = 0; c < 3; ++c) s[c] = r2[c] - r1[c];
    for (int i = 0; i < 3; ++i)
        for (int c = 0; c < 3; ++c) s[c] = s[c] + (double)off[i] * C->vc[c][i];
}

/* .o. dot product, Quaternions.f90:475-484 */
static inline double dot3(const double a[3], const double b[3]) { return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]; }

/* pick, Geometry.f90:648-676 */
static int pick(int i1, int i2, const int off[3]) {
    if (i2 > i1) return 1;
    if (i2 == i1 && off[0] >= 0) {
        if (off[0] > 0) return 1;
        if (off[1] > 0) return 1;
        if (off[1] == 0 && off[2] > 0) return 1;
    }
    return 0;
}

/* get_optimal_splitting, Geometry.f90:679-707 */
static void optimal_splitting(const fcell* C, double max_cut, int splits[3]) {
    for (int i = 0; i < 3; ++i) {
        int v1 = (i + 1) % 3, v2 = (i + 2) % 3;
        double a[3], b[3], n[3], v[3];
        for (int r = 0; r < 3; ++r) {
            a[r] = C->vc[r][v1];
            b[r] = C->vc[r][v2];
            v[r] = C->vc[r][i];
        }
        n[0] = a[1] * b[2] - a[2] * b[1];
        n[1] = a[2] * b[0] - a[0] * b[2];
        n[2] = a[0] * b[1] - a[1] * b[0];
        double length = fabs(dot3(v, n)) / sqrt(dot3(n, n));
        if (max_cut < 0.1e-4)
            splits[i] = (int)floor(10.0 * length);
        else
            splits[i] = (int)floor(length / max_cut);
        if (splits[i] > 40) splits[i] = 40;
    }
}

typedef struct {
    int* atoms;
    int n, cap;
} ivec;

static void ivec_push(ivec* v, int x) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 16;
        v->atoms = (int*)realloc(v->atoms, sizeof(int) * (size_t)v->cap);
    }
    v->atoms[v->n++] = x;
}

typedef struct {
    int* data; /* 4 ints per entry: neighbour, offset x3 */
    int n, cap;
} nbvec;

static void nbvec_push(nbvec* v, int j, const int o[3]) {
    if (v->n == v->cap) {
        v->cap = v->cap ? 2 * v->cap : 32;
        v->data = (int*)realloc(v->data, sizeof(int) * 4 * (size_t)v->cap);
    }
    int* d = v->data + 4 * (size_t)v->n;
    d[0] = j;
    d[1] = o[0];
    d[2] = o[1];
    d[3] = o[2];
    v->n++;
}

/* generate_neighbor_lists (PyInterface.f90:1062-1072) ->
 * core_create_space_partitioning (Core.f90:8130-8141): get_optimal_splitting,
 * divide_cell (Geometry.f90:751-865), find_subcell_for_atom (Geometry.f90:884-924) ->
 * core_build_neighbor_lists (Core.f90:8148-8280). */
int64_t orc_build_neighbors(const orc_system* s, const double* cutoffs, int32_t* counts, int32_t* out_idx,
                            int32_t* out_off, int64_t cap) {
    const int n = s->n;
    if (n < 0) return -1;
    fcell C;
    make_cell(s, &C);
    double max_cut = 0.0;
    for (int i = 0; i < n; ++i)
        if (i == 0 || cutoffs[i] > max_cut) max_cut = cutoffs[i];
    int sp[3];
    optimal_splitting(&C, max_cut, sp);
    for (int a = 0; a < 3; ++a)
        if (sp[a] < 1) return -1; /* the Python layer never builds the fast list then */
    const int nx = sp[0] + 2, ny = sp[1] + 2, nz = sp[2] + 2;
    const size_t ncell = (size_t)nx * ny * nz;
    ivec* cells = (ivec*)calloc(ncell, sizeof(ivec));
    int* cell_of = (int*)malloc(sizeof(int) * 3 * (size_t)(n > 0 ? n : 1));
    int* wrap = (int*)malloc(sizeof(int) * 3 * (size_t)(n > 0 ? n : 1));
    /* find_subcell_for_atom for atoms 1..n in order */
    for (int i = 0; i < n; ++i) {
        double w[3], f[3];
        int off[3];
        wrapped_coords(&C, s->pos + 3 * (size_t)i, w, off);
        for (int a = 0; a < 3; ++a) wrap[3 * i + a] = off[a];
        rel_coords(&C, w, f);
        for (int a = 0; a < 3; ++a) {
            int k = (int)floor(f[a] * (double)sp[a]);
            int idx;
            if (C.pbc[a]) {
                idx = k % sp[a] + 1; /* Fortran mod: sign of the dividend */
            } else {
                idx = k + 1;
                if (idx < 0) idx = 0;
                if (idx > sp[a] + 1) idx = sp[a] + 1;
            }
            cell_of[3 * i + a] = idx;
        }
        ivec_push(&cells[((size_t)cell_of[3 * i + 2] * ny + cell_of[3 * i + 1]) * nx + cell_of[3 * i]], i);
    }
    nbvec* lists = (nbvec*)calloc((size_t)(n > 0 ? n : 1), sizeof(nbvec));
    for (int i1 = 0; i1 < n; ++i1) {
        const int* ci = cell_of + 3 * i1;
        const int* w1 = wrap + 3 * i1;
        for (int kn = -1; kn <= 1; ++kn)
            for (int jn = -1; jn <= 1; ++jn)
                for (int in = -1; in <= 1; ++in) {
                    /* divide_cell neighbour map, Geometry.f90:820-858 */
                    int nb[3] = {ci[0] + in, ci[1] + jn, ci[2] + kn};
                    int noff[3] = {0, 0, 0};
                    int include = 1;
                    for (int a = 0; a < 3; ++a) {
                        if (C.pbc[a]) {
                            while (nb[a] > sp[a]) {
                                nb[a] -= sp[a];
                                noff[a] += 1;
                            }
                            while (nb[a] < 1) {
                                nb[a] += sp[a];
                                noff[a] -= 1;
                            }
                        } else if (nb[a] < 0 || nb[a] > sp[a] + 1) {
                            include = 0;
                            nb[a] = 0;
                        }
                    }
                    if (!include) continue;
                    const ivec* cl = &cells[((size_t)nb[2] * ny + nb[1]) * nx + nb[0]];
                    for (int t = 0; t < cl->n; ++t) {
                        const int i2 = cl->atoms[t];
                        const int* w2 = wrap + 3 * i2;
                        if (!pick(i1, i2, noff)) continue;
                        int o[3], mo[3];
                        for (int a = 0; a < 3; ++a) {
                            o[a] = noff[a] - w1[a] + w2[a];
                            mo[a] = -noff[a] + w1[a] - w2[a];
                        }
                        double sep[3];
                        separation(&C, s->pos + 3 * (size_t)i1, s->pos + 3 * (size_t)i2, o, sep);
                        double d2 = dot3(sep, sep);
                        if (d2 < cutoffs[i1] * cutoffs[i1]) nbvec_push(&lists[i1], i2, o);
                        if (d2 < cutoffs[i2] * cutoffs[i2]) nbvec_push(&lists[i2], i1, mo);
                    }
                }
    }
    int64_t total = 0;
    for (int i = 0; i < n; ++i) {
        counts[i] = lists[i].n;
        total += lists[i].n;
    }
    if (out_idx && out_off && cap >= total) {
        int64_t p = 0;
        for (int i = 0; i < n; ++i)
            for (int e = 0; e < lists[i].n; ++e, ++p) {
                const int* d = lists[i].data + 4 * (size_t)e;
                out_idx[p] = d[0];
                out_off[3 * p] = d[1];
                out_off[3 * p + 1] = d[2];
                out_off[3 * p + 2] = d[3];
            }
    }
    for (size_t c = 0; c < ncell; ++c) free(cells[c].atoms);
    for (int i = 0; i < n; ++i) free(lists[i].data);
    free(cells);
    free(lists);
    free(cell_of);
    free(wrap);
    return total;
}

/* ------------------------------------------------------------------ */
/* Evaluators (fortran/Potentials.f90)                                  */
/* ------------------------------------------------------------------ */

/* smoothening_factor, Potentials.f90:442-457 */
static double smooth_factor(double r, double hard, double soft) {
    if (r > hard) return 0.0;
    if (r < soft) return 1.0;
    return 0.5 * (1.0 + cos(PI * (r - soft) / (hard - soft)));
}

/* smoothening_derivative, Potentials.f90:483-498 */
static double smooth_deriv(double r, double hard, double soft) {
    if (r > hard) return 0.0;
    if (r < soft) return 0.0;
    return -(0.5 * PI / (hard - soft) * sin(PI * (r - soft) / (hard - soft)));
}

/* evaluate_energy_LJ (2990-3005), _exp (3665-3680), _buckingham (4030-4045),
 * _spring (3069-3085), _power (4141-4152), _shift (4827-4842); cut is the
 * potential's hard cutoff (the spring is shifted by its value there) */
static double pair_energy(int kind, const double* p, double cut, double r1, const double* table) {
    if (kind == 0) {
        double ratio = p[1] / r1;
        double r6 = ratio * ratio * ratio * ratio * ratio * ratio;
        return p[0] * (r6 * r6 - r6);
    } else if (kind == 1) {
        return p[0] * exp(-(p[1] * r1));
    } else if (kind == 2) {
        double ratio = r1 / p[2];
        double r6 = 1.0 / (ratio * ratio * ratio * ratio * ratio * ratio);
        return p[0] * exp(-ratio) - p[1] * r6;
    } else if (kind == 3) {
        double r2 = r1 - p[1], r6 = cut - p[1];
        return r2 * r2 < r6 * r6 ? p[0] * 0.5 * (r2 * r2 - r6 * r6) : 0.0;
    } else if (kind == 4) {
        double ratio = p[1] / r1;
        return p[0] * pow(ratio, p[2]);
    } else if (kind == 5) {
        return p[0] * pow((p[1] - r1) / (p[1] - p[2]), p[3]);
    } else if (kind == 10) { /* evaluate_energy_step (4946-4967): e1, e2, r1, r2 */
        if (r1 < p[2]) return p[0];
        if (r1 > p[3]) return p[1];
        return (p[0] + p[1]) * 0.5 * (1.0 + 0.5 * cos(PI * (r1 - p[2]) / (p[3] - p[2])));
    } else { /* evaluate_energy_table (4267-4298): rows (V, d) from p[0], p[1] rows, range p[2], scale p[3] */
        const double* T = table + 2 * (int64_t)p[0];
        const int n_values = (int)p[1];
        const double max_r = p[2];
        const double dr = max_r / (n_values - 1);
        if (r1 >= max_r) return T[2 * (n_values - 1)];
        const int l = (int)floor(r1 / dr); /* lower_index - 1 */
        const double t = r1 / dr - l, t2 = t * t, t3 = t2 * t;
        return p[3] * (T[2 * l] * (2 * t3 - 3 * t2 + 1) + T[2 * l + 1] * dr / max_r * (t3 - 2 * t2 + t) +
                       T[2 * l + 2] * (3 * t2 - 2 * t3) + T[2 * l + 3] * dr / max_r * (t3 - t2));
    }
}

/* evaluate_force_LJ (2971-2983), _exp (3643-3655), _buckingham (4009-4022),
 * _spring (3042-3060), _power (4119-4132), _shift (4803-4818): force on atom 1 */
static void pair_force(int kind, const double* p, double cut, const double sep[3], double r1, double f[3],
                       const double* table) {
    if (kind == 0) {
        double ratio = p[1] / r1;
        double r6 = ratio * ratio * ratio * ratio * ratio * ratio;
        double pre = p[0] * (6.0 * r6 - 12.0 * r6 * r6);
        for (int c = 0; c < 3; ++c) f[c] = pre * sep[c] / (r1 * r1);
    } else if (kind == 1) {
        double pre = p[1] * p[0] * exp(-(p[1] * r1));
        for (int c = 0; c < 3; ++c) f[c] = -(pre * sep[c] / r1);
    } else if (kind == 2) {
        double ratio = r1 / p[2];
        double r6 = 1.0 / (ratio * ratio * ratio * ratio * ratio * ratio);
        double pre = -p[0] * ratio * exp(-ratio) + p[1] * 6.0 * r6;
        for (int c = 0; c < 3; ++c) f[c] = pre * sep[c] / (r1 * r1);
    } else if (kind == 3) {
        double r2 = r1 - p[1], r6 = cut - p[1];
        for (int c = 0; c < 3; ++c) f[c] = r2 * r2 < r6 * r6 ? p[0] * r2 * sep[c] / r1 : 0.0;
    } else if (kind == 4) {
        double n = p[2], ratio = p[1] / r1;
        for (int c = 0; c < 3; ++c) f[c] = p[0] * (-n * pow(ratio, n)) * sep[c] / (r1 * r1);
    } else if (kind == 5) {
        double a = p[1], b = p[2], n = p[3];
        for (int c = 0; c < 3; ++c) f[c] = -p[0] * n / (a - b) * pow((a - r1) / (a - b), n - 1.0) * sep[c] / r1;
    } else if (kind == 10) { /* evaluate_force_step (4917-4937): the same value on all three
                                components, not along the bond, as the reference has it */
        const double v = (r1 < p[2] || r1 > p[3])
                             ? 0.0
                             : (p[0] + p[1]) * 0.25 * PI / (p[3] - p[2]) * sin(PI * (r1 - p[2]) / (p[3] - p[2]));
        for (int c = 0; c < 3; ++c) f[c] = v;
    } else { /* evaluate_force_table (4227-4258) */
        const double* T = table + 2 * (int64_t)p[0];
        const int n_values = (int)p[1];
        const double max_r = p[2];
        const double dr = max_r / (n_values - 1);
        for (int c = 0; c < 3; ++c) f[c] = 0.0;
        if (r1 >= max_r) return;
        const int l = (int)floor(r1 / dr);
        const double t = r1 / dr - l, t2 = t * t;
        const double pre = p[3] * (T[2 * l] / dr * 6 * (t2 - t) + T[2 * l + 1] / max_r * (3 * t2 - 4 * t + 1) +
                                   T[2 * l + 2] / dr * 6 * (t - t2) + T[2 * l + 3] / max_r * (3 * t2 - 2 * t));
        for (int c = 0; c < 3; ++c) f[c] = pre / r1 * sep[c];
    }
}

static inline int has(uint64_t mask, int t) { return (int)((mask >> t) & 1u); }

/* One factor of a product potential for the pair (atom1, atom2) as the loop
 * picks it: its energy, its force on atom 1 and its electronegativities of
 * atoms 1 and 2, without any cut factor (evaluate_energy_component,
 * evaluate_force_component, evaluate_electronegativity_component,
 * Potentials.f90:2512-2890).  Charge terms have no force routine; other terms
 * no electronegativity. */
static void product_component(const orc_model* m, int kind, const double* p, uint64_t first, double rc, int t1,
                              double q1, double q2, const double sep[3], double d, double* e, double f[3],
                              double en[2]) {
    for (int c = 0; c < 3; ++c) f[c] = 0.0;
    en[0] = en[1] = 0.0;
    if (kind < 7) {
        *e = pair_energy(kind, p, rc, d, m->pair_table);
        pair_force(kind, p, rc, sep, d, f, m->pair_table);
        return;
    }
    const int direct = has(first, t1);
    if (kind == 7) {
        const int n1 = direct ? (int)p[1] : (int)p[2], n2 = direct ? (int)p[2] : (int)p[1];
        *e = p[0] * (__builtin_powi(q1, n1) * __builtin_powi(q2, n2));
        en[0] = n1 > 0 ? -p[0] * (n1 * __builtin_powi(q1, n1 - 1) * __builtin_powi(q2, n2)) : 0.0;
        en[1] = n2 > 0 ? -p[0] * (n2 * __builtin_powi(q1, n1) * __builtin_powi(q2, n2 - 1)) : 0.0;
    } else if (kind == 8) {
        const double* c = m->pair_table + 2 * (int64_t)p[0];
        const double r2 = c[direct ? 1 : 5], r3 = c[direct ? 5 : 1];
        const double r4 = c[direct ? 3 : 7], r5 = c[direct ? 7 : 3];
        const double r6 = c[direct ? 11 : 12], r7 = c[direct ? 12 : 11];
        const double r8 = c[direct ? 13 : 14], r9 = c[direct ? 14 : 13];
        const double d3 = c[direct ? 9 : 10], d4 = c[direct ? 10 : 9];
        const double d5 = r8 * (r4 - q1), d6 = r9 * (r5 - q2);
        const double d1 = r2 + pow(fabs(d5), r6), d2 = r3 + pow(fabs(d6), r7);
        const double v = c[0] * exp(0.5 * (d3 * d1 + d4 * d2));
        *e = v;
        en[0] = v * d3 * 0.5 * r6 * pow(fabs(d5), r6 - 1.0) * copysign(1.0, d5) * r8;
        en[1] = v * d4 * 0.5 * r7 * pow(fabs(d6), r7 - 1.0) * copysign(1.0, d6) * r9;
    } else {
        const double* c = m->pair_table + 2 * (int64_t)p[0];
        const double* s1 = c + (direct ? 0 : 4);
        const double* s2 = c + (direct ? 4 : 0);
        double f1 = s1[0] + s1[1] * pow(fabs(q1 - s1[2]), s1[3]);
        double f2 = s2[0] + s2[1] * pow(fabs(q2 - s2[2]), s2[3]);
        if (f1 < 0.0) f1 = 0.0;
        if (f2 < 0.0) f2 = 0.0;
        *e = sqrt(f1 * f2);
        const double abs1 = fabs(q1 - s1[2]), abs2 = fabs(q2 - s2[2]);
        const double pow1 = pow(abs1, s1[3] - 1), pow2 = pow(abs2, s2[3] - 1);
        double g1 = s1[0] + s1[1] * abs1 * pow1, g2 = s2[0] + s2[1] * abs2 * pow2;
        const double dd1 = -s1[3] * pow1 * copysign(1.0, q1 - s1[2]) * s1[1];
        const double dd2 = -s2[3] * pow2 * copysign(1.0, q2 - s2[2]) * s2[1];
        double inv_sqrt = 0.5 / sqrt(g1 * g2);
        if (g1 < 0.0) {
            g1 = 0.0;
            inv_sqrt = 0.0;
        }
        if (g2 < 0.0) {
            g2 = 0.0;
            inv_sqrt = 0.0;
        }
        en[0] = inv_sqrt * dd1 * g2;
        en[1] = inv_sqrt * dd2 * g1;
    }
}

/* A product of n factors (the record itself, then its components): energy,
 * force on atom 1 and electronegativities combined as evaluate_energy /
 * evaluate_forces / evaluate_electronegativity do for n_product > 1
 * (Potentials.f90:2512-2700): each factor's force and electronegativity
 * weighted by E / E_k, or by the product of the others where E_k = 0. */
static void product_term(const orc_model* m, int r, int t1, double q1, double q2, const double sep[3], double d,
                         double* e, double f[3], double en[2]) {
    const int n = 1 + m->pair_nmul[r];
    double ek[16], fk[16][3], nk[16][2];
    for (int k = 0; k < n && k < 16; ++k) {
        const int c = m->pair_mul0[r] + k - 1;
        const int kind = k == 0 ? m->pair_kind[r] : m->mul_kind[c];
        const double* p = k == 0 ? m->pair_params + 4 * (size_t)r : m->mul_params + 4 * (size_t)c;
        const uint64_t first = k == 0 ? m->pair_first[r] : m->mul_first[c];
        product_component(m, kind, p, first, m->pair_cutoff[r], t1, q1, q2, sep, d, &ek[k], fk[k], nk[k]);
    }
    double energy = 1.0;
    for (int k = 0; k < n; ++k) energy *= ek[k];
    *e = energy;
    for (int c = 0; c < 3; ++c) f[c] = 0.0;
    en[0] = en[1] = 0.0;
    for (int k = 0; k < n; ++k) {
        double w;
        if (ek[k] != 0.0) {
            w = energy / ek[k];
        } else {
            w = 1.0;
            for (int q = 0; q < n; ++q)
                if (q != k) w *= ek[q];
        }
        for (int c = 0; c < 3; ++c) f[c] += w * fk[k][c];
        en[0] += w * nk[k][0];
        en[1] += w * nk[k][1];
    }
}

/* evaluate_pair_bond_order_factor_tersoff, Potentials.f90:5744-5795.
 * sep1 = separations(:,1), sep2 = separations(:,2) */
static double tersoff_factor(const double* bp, double cut, double soft, const double sep1[3], const double sep2[3],
                             double r1, double r2) {
    double t1[3] = {-sep1[0], -sep1[1], -sep1[2]};
    double cosine = dot3(t1, sep2) / (r1 * r2);
    double mu = bp[6], a1 = bp[2], cc1 = bp[3] * bp[3], dd1 = bp[4] * bp[4], h1 = bp[5];
    double decay1 = smooth_factor(r2, cut, soft);
    double xi1 = decay1 * exp(pow(a1 * (r1 - r2), mu));
    double gee1 = 1.0 + cc1 / dd1 - cc1 / (dd1 + (h1 - cosine) * (h1 - cosine));
    return xi1 * gee1;
}

/* evaluate_pair_bond_order_gradient_tersoff, Potentials.f90:5806-5902.
 * g[a][c]: component c of the gradient with respect to atom a (a = 0: atoms(1),
 * 1: atoms(2) the centre, 2: atoms(3)). */
static void tersoff_gradient(const double* bp, double cut, double soft, const double sep1[3], const double sep2[3],
                             double r1, double r2, double g[3][3]) {
    double t1[3], t2[3], u1[3], u2[3];
    for (int c = 0; c < 3; ++c) {
        t1[c] = -sep1[c];
        t2[c] = sep2[c];
        u1[c] = t1[c] / r1;
        u2[c] = t2[c] / r2;
    }
    double dot = dot3(t1, t2);
    double ratio = 1.0 / (r1 * r2);
    double cosine = dot * ratio;
    double nr1[3][3] = {{0}}, nr2[3][3] = {{0}}, nc[3][3], tm2[3][3] = {{0}};
    double t3[3], t4[3];
    for (int c = 0; c < 3; ++c) {
        nr1[1][c] = -u1[c];
        nr1[0][c] = u1[c];
        nr2[1][c] = -u2[c];
        nr2[2][c] = u2[c];
        t3[c] = t2[c] - dot / (r1 * r1) * t1[c];
        t4[c] = t1[c] - dot / (r2 * r2) * t2[c];
    }
    for (int c = 0; c < 3; ++c) {
        nc[0][c] = t3[c] * ratio;
        nc[1][c] = -(t3[c] + t4[c]) * ratio;
        nc[2][c] = t4[c] * ratio;
    }
    double mu = bp[6], a1 = bp[2], cc1 = bp[3] * bp[3], dd1 = bp[4] * bp[4], h1 = bp[5];
    double decay1 = smooth_factor(r2, cut, soft);
    double dfac = smooth_deriv(r2, cut, soft);
    double t6[3] = {u2[0] * dfac, u2[1] * dfac, u2[2] * dfac};
    for (int c = 0; c < 3; ++c) {
        tm2[1][c] = -t6[c];
        tm2[2][c] = t6[c];
    }
    double e1a = pow(a1 * (r1 - r2), mu - 1.0);
    double e1b = a1 * (r1 - r2) * e1a;
    double xi1 = exp(e1b);
    double hc = h1 - cosine;
    double gee1 = 1.0 + cc1 / dd1 - cc1 / (dd1 + hc * hc);
    double sc = decay1 * (exp(e1b) * a1 * mu * e1a);
    double nxi[3][3], ng[3][3];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) nxi[a][c] = tm2[a][c] * xi1 + sc * (nr1[a][c] - nr2[a][c]);
    xi1 = xi1 * decay1;
    double X = dd1 + hc * hc;
    double pre = -(cc1 / (X * X) * 2.0 * hc);
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) ng[a][c] = pre * nc[a][c];
    for (int a = 0; a < 3; ++a)
        for (int c = 0; c < 3; ++c) g[a][c] = nxi[a][c] * gee1 + xi1 * ng[a][c];
}

/* post_process_bond_order_factor_tersoff, Potentials.f90:5910-5921 */
static double tersoff_post(const double* bp, double raw) {
    double beta = bp[0], eta = bp[1];
    return pow(1.0 + pow(beta * raw, eta), -1.0 / (2.0 * eta));
}

/* post_process_bond_order_gradient_tersoff, Potentials.f90:5929-5961 (scalar
 * part: the routine multiplies its raw_gradient argument by this value). */
static double tersoff_post_grad_scale(const double* bp, double raw, double g) {
    double beta = bp[0], eta = bp[1];
    if (eta == 0.0) return 0.0;
    if (raw == 0.0 && eta <= 1.0) return 0.0;
    double inv_eta = -1.0 / (2.0 * eta);
    return inv_eta * pow(1.0 + pow(beta * raw, eta), inv_eta - 1.0) * eta * pow(beta * raw, eta - 1.0) * beta * g;
}

/* ------------------------------------------------------------------ */
/* Core loop (fortran/Core.f90)                                         */
/* ------------------------------------------------------------------ */

typedef struct {
    const orc_system* s;
    const orc_model* m;
    const orc_nblist* nb;
    fcell C;
    double* maxbr; /* per atom: max_bond_radius, Core.f90:1030-1067 */
    double* smooth_soft;
    int* smoothened;
    int n_groups;      /* groups with per-atom factors: 0 .. n_groups-1 */
    double* af_raw;    /* n_groups x n: per-atom bond-order sums */
    double* af_fac;    /* n_groups x n: post-processed per-atom factors (saved_bond_order_factors) */
} ctx_t;


/* first post-processing factor of the atom's element in the group:
 * core_post_process_pair_bond_order_factor, Core.f90:2763-2807 */
static int post_index(const ctx_t* X, int t, int group) {
    const orc_model* m = X->m;
    for (int b = 0; b < m->n_bond; ++b)
        if (has(m->bond_mask1[b], t) && m->bond_group[b] == group) return b;
    return -1;
}

/* core_calculate_pair_bond_order_factor, Core.f90:2439-2637 */
static void pair_bo_sums(const ctx_t* X, int i, int j, const double sep[3], double d, int group, double sums[2]) {
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const orc_nblist* nb = X->nb;
    sums[0] = sums[1] = 0.0;
    double s1[3] = {-sep[0], -sep[1], -sep[2]};
    for (int pass = 0; pass < 2; ++pass) {
        const int c = pass == 0 ? i : j;     /* centre */
        const int o = pass == 0 ? j : i;     /* other end of the bond */
        if (pass == 1)
            for (int q = 0; q < 3; ++q) s1[q] = sep[q];
        const int tc = s->type[c], to = s->type[o];
        for (int e = nb->start[c]; e < nb->start[c + 1]; ++e) {
            const int k = nb->idx[e];
            double s2[3];
            separation(&X->C, s->pos + 3 * (size_t)c, s->pos + 3 * (size_t)k, nb->off + 3 * (size_t)e, s2);
            double d2 = sqrt(dot3(s2, s2));
            if (!(s1[0] + s2[0] != 0.0 || s1[1] + s2[1] != 0.0 || s1[2] + s2[2] != 0.0)) continue;
            if (!(d2 < X->maxbr[c])) continue;
            const int tk = s->type[k];
            for (int b = 0; b < m->n_bond; ++b) {
                if (!has(m->bond_mask1[b], tc) || m->bond_group[b] != group) continue;
                if (!has(m->bond_mask2[b], to)) continue;
                if (!has(m->bond_mask3[b], tk)) continue;
                sums[pass] += tersoff_factor(m->bond_params + 7 * (size_t)b, m->bond_cutoff[b], m->bond_soft[b], s1,
                                             s2, d, d2);
            }
        }
    }
}

/* core_add_pair_bond_order_forces, Core.f90:4952-5353 */
static void pair_bo_forces(const ctx_t* X, int i, int j, double prefactor, const double sep[3], double d, int group,
                           const double sums[2], double* F, double* stress) {
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const orc_nblist* nb = X->nb;
    double virial[2][6] = {{0}};
    int pp[2];
    double pf[2] = {0, 0};
    pp[0] = post_index(X, s->type[i], group);
    pp[1] = post_index(X, s->type[j], group);
    for (int q = 0; q < 2; ++q)
        if (pp[q] >= 0) pf[q] = tersoff_post_grad_scale(m->bond_params + 7 * (size_t)pp[q], sums[q], 1.0);
    double s1[3] = {-sep[0], -sep[1], -sep[2]};
    for (int pass = 0; pass < 2; ++pass) {
        const int c = pass == 0 ? i : j;
        const int o = pass == 0 ? j : i;
        if (pass == 1)
            for (int q = 0; q < 3; ++q) s1[q] = sep[q];
        const int tc = s->type[c], to = s->type[o];
        for (int e = nb->start[c]; e < nb->start[c + 1]; ++e) {
            const int k = nb->idx[e];
            double s2[3];
            separation(&X->C, s->pos + 3 * (size_t)c, s->pos + 3 * (size_t)k, nb->off + 3 * (size_t)e, s2);
            double d2 = sqrt(dot3(s2, s2));
            if (!(s1[0] + s2[0] != 0.0 || s1[1] + s2[1] != 0.0 || s1[2] + s2[2] != 0.0)) continue;
            if (!(d2 < X->maxbr[c])) continue;
            const int tk = s->type[k];
            for (int b = 0; b < m->n_bond; ++b) {
                if (!has(m->bond_mask1[b], tc) || m->bond_group[b] != group) continue;
                if (!has(m->bond_mask2[b], to)) continue;
                if (!has(m->bond_mask3[b], tk)) continue;
                double g[3][3], ng[3][3];
                tersoff_gradient(m->bond_params + 7 * (size_t)b, m->bond_cutoff[b], m->bond_soft[b], s1, s2, d, d2, g);
                for (int a = 0; a < 3; ++a)
                    for (int q = 0; q < 3; ++q)
                        ng[a][q] = pp[pass] >= 0 ? -(pf[pass] * prefactor * g[a][q]) : -(prefactor * g[a][q]);
                for (int q = 0; q < 3; ++q) {
                    F[3 * (size_t)o + q] += ng[0][q];
                    F[3 * (size_t)c + q] += ng[1][q];
                    F[3 * (size_t)k + q] += ng[2][q];
                }
                double* v = virial[pass];
                v[0] = v[0] - s1[0] * g[0][0] + s2[0] * g[2][0];
                v[1] = v[1] - s1[1] * g[0][1] + s2[1] * g[2][1];
                v[2] = v[2] - s1[2] * g[0][2] + s2[2] * g[2][2];
                v[3] = v[3] - s1[1] * g[0][2] + s2[1] * g[2][2];
                v[4] = v[4] - s1[0] * g[0][2] + s2[0] * g[2][2];
                v[5] = v[5] - s1[0] * g[0][1] + s2[0] * g[2][1];
            }
        }
    }
    double tv[2][6];
    for (int q = 0; q < 2; ++q)
        for (int c = 0; c < 6; ++c)
            tv[q][c] = pp[q] >= 0 ? tersoff_post_grad_scale(m->bond_params + 7 * (size_t)pp[q], sums[q], virial[q][c])
                                  : virial[q][c];
    for (int c = 0; c < 6; ++c) stress[c] = stress[c] - prefactor * (tv[0][c] + tv[1][c]);
}

static double post_process(const ctx_t* X, int t, int group, double raw) {
    int b = post_index(X, t, group);
    if (b < 0) return raw;
    return tersoff_post(X->m->bond_params + 7 * (size_t)b, raw);
}

/* ---- per-atom (level-1) bond-order factors ---- */

/* kinds 0 neighbors, 1 power_bond, 4 table_bond act on pairs; 2 c_scale,
 * 3 sqrt_scale, 5 table_scale post-process an atom's sum */
static int afac_two_target(int kind) { return kind == 0 || kind == 1 || kind == 4; }

/* The cubic Hermite form of the tabulated factors (Potentials.f90:6496-6576,
 * 6663-6765): rows (V, d) from p[0], p[1] rows, range p[2], scale p[3]; value
 * and derivative at x < range. */
static void afac_hermite(const double* table, const double* p, double x, double* v, double* dv) {
    const double* T = table + 2 * (int64_t)p[0];
    const int n_values = (int)p[1];
    const double max_r = p[2];
    const double dr = max_r / (n_values - 1);
    const int l = (int)floor(x / dr); /* lower_index - 1 */
    const double t = x / dr - l, t2 = t * t, t3 = t2 * t;
    *v = p[3] * (T[2 * l] * (2 * t3 - 3 * t2 + 1) + T[2 * l + 1] * dr / max_r * (t3 - 2 * t2 + t) +
                 T[2 * l + 2] * (3 * t2 - 2 * t3) + T[2 * l + 3] * dr / max_r * (t3 - t2));
    *dv = p[3] * (T[2 * l] / dr * 6 * (t2 - t) + T[2 * l + 1] / max_r * (3 * t2 - 4 * t + 1) +
                  T[2 * l + 2] / dr * 6 * (t - t2) + T[2 * l + 3] / max_r * (3 * t2 - 2 * t));
}

static double afac_table_last(const double* table, const double* p) {
    return table[2 * ((int64_t)p[0] + (int64_t)p[1] - 1)];
}

/* evaluate_bond_order_factor_coordination (Potentials.f90:5631-5645), _power
 * (6293-6306) and _table (6663-6700; beyond the range the last value, neither
 * scaled nor smoothed): the symmetric two-target factor c(r) */
static double afac_value(const orc_model* m, int r, double d) {
    const double* p = m->afac_params + 5 * (size_t)r;
    const double f = smooth_factor(d, m->afac_cutoff[r], m->afac_soft[r]);
    if (m->afac_kind[r] == 0) return f;
    if (m->afac_kind[r] == 4) {
        if (d >= p[2]) return afac_table_last(m->pair_table, p);
        double v, dv;
        afac_hermite(m->pair_table, p, d, &v, &dv);
        return v * f;
    }
    return f * pow(p[0] / d, p[1]);
}

/* evaluate_bond_order_gradient_coordination (5656-5673) and _power (6317-6347):
 * g11 = gradient of atom 1's term with respect to atom 1, g12 with respect to atom 2 */
static void afac_gradient(const orc_model* m, int r, const double sep[3], double d, double g11[3], double g12[3]) {
    const double* p = m->afac_params + 5 * (size_t)r;
    const double inv = 1.0 / d;
    const double dv = smooth_deriv(d, m->afac_cutoff[r], m->afac_soft[r]);
    double t[3];
    for (int c = 0; c < 3; ++c) t[c] = sep[c] * inv * dv;
    if (m->afac_kind[r] == 0) {
        for (int c = 0; c < 3; ++c) {
            g11[c] = -t[c];
            g12[c] = t[c];
        }
        return;
    }
    if (m->afac_kind[r] == 4) {
        /* evaluate_bond_order_gradient_table (6711-6765): zero beyond the range;
           the cut factor's gradient enters inside the smoothing band only.
           The reference leaves t3 unassigned in this routine; t^3 is used. */
        for (int c = 0; c < 3; ++c) g11[c] = g12[c] = 0.0;
        if (d >= p[2]) return;
        double v, dvv;
        afac_hermite(m->pair_table, p, d, &v, &dvv);
        const double decay = smooth_factor(d, m->afac_cutoff[r], m->afac_soft[r]);
        const double factor = (decay > 0.0 && decay < 1.0) ? v : 0.0;
        for (int c = 0; c < 3; ++c) {
            g11[c] = -t[c] * factor - decay * dvv * inv * sep[c];
            g12[c] = -g11[c];
        }
        return;
    }
    const double n = p[1], ratio_n = pow(p[0] * inv, n);
    const double decay = smooth_factor(d, m->afac_cutoff[r], m->afac_soft[r]);
    for (int c = 0; c < 3; ++c) {
        g11[c] = -t[c] * ratio_n + n * decay * ratio_n * inv * inv * sep[c];
        g12[c] = -g11[c];
    }
}

/* first post-processing per-atom factor of the atom's element in the group
 * (core_post_process_bond_order_factors, Core.f90:2697-2712) */
static int afac_post_index(const orc_model* m, int t, int group) {
    for (int r = 0; r < m->n_afac; ++r)
        if (!afac_two_target(m->afac_kind[r]) && has(m->afac_mask1[r], t) && m->afac_group[r] == group) return r;
    return -1;
}

/* post_process_bond_order_factor_scaler_1 (Potentials.f90:6021-6035), _sqrt
 * (6402-6414) and _table (6496-6532: 0 for sums <= 0, the last value, unscaled,
 * beyond the range) */
static double afac_post(const orc_model* m, int r, double raw) {
    const double* p = m->afac_params + 5 * (size_t)r;
    if (m->afac_kind[r] == 3) return raw <= 0.0 ? 0.0 : p[0] * sqrt(raw);
    if (m->afac_kind[r] == 5) {
        if (raw <= 0.0) return 0.0;
        if (raw >= p[2]) return afac_table_last(m->pair_table, p);
        double v, dv;
        afac_hermite(m->pair_table, p, raw, &v, &dv);
        return v;
    }
    const double dN = (raw - p[1]) * p[2];
    return dN > p[4] ? p[0] * dN / (1.0 + exp(p[3] * dN)) : 0.0;
}

/* post_process_bond_order_gradient_scaler_1 (6044-6063) and _sqrt (6423-6436), one component */
static double afac_post_grad(const orc_model* m, int r, double raw, double g) {
    const double* p = m->afac_params + 5 * (size_t)r;
    if (m->afac_kind[r] == 3) return raw <= 0.0 ? 0.0 : p[0] / (2.0 * sqrt(raw)) * g;
    if (m->afac_kind[r] == 5) { /* 6541-6576 */
        if (raw <= 0.0 || raw >= p[2]) return 0.0;
        double v, dv;
        afac_hermite(m->pair_table, p, raw, &v, &dv);
        return dv * g;
    }
    const double dN = (raw - p[1]) * p[2];
    if (!(dN > p[4])) return 0.0;
    const double expo = exp(p[3] * dN), inv_exp = 1.0 / (1.0 + expo);
    return p[0] * p[2] * (inv_exp - dN * inv_exp * inv_exp * p[3] * expo) * g;
}

/* core_calculate_bond_order_factors (Core.f90:2015-2404), two-target level-1
 * part: every picked pair adds the factor of each record of atom1's element
 * (position 1) whose position 2 matches atom2 to both atoms' sums; then
 * core_post_process_bond_order_factors (2671-2735) */
static void afac_sums(ctx_t* X) {
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const orc_nblist* nb = X->nb;
    const int n = s->n;
    X->af_raw = (double*)calloc((size_t)X->n_groups * (size_t)(n ? n : 1), sizeof(double));
    X->af_fac = (double*)calloc((size_t)X->n_groups * (size_t)(n ? n : 1), sizeof(double));
    for (int g = 0; g < X->n_groups; ++g) {
        double* raw = X->af_raw + (size_t)g * n;
        for (int i = 0; i < n; ++i) {
            const int ti = s->type[i];
            for (int e = nb->start[i]; e < nb->start[i + 1]; ++e) {
                const int j = nb->idx[e];
                const int* o = nb->off + 3 * (size_t)e;
                if (!pick(i, j, o)) continue;
                double sep[3];
                separation(&X->C, s->pos + 3 * (size_t)i, s->pos + 3 * (size_t)j, o, sep);
                const double d = sqrt(dot3(sep, sep));
                if (!(d < X->maxbr[i])) continue;
                const int tj = s->type[j];
                for (int r = 0; r < m->n_afac; ++r) {
                    if (!afac_two_target(m->afac_kind[r]) || !has(m->afac_mask1[r], ti)) continue;
                    if (m->afac_group[r] != g || !(m->afac_cutoff[r] > d)) continue;
                    if (!has(m->afac_mask2[r], tj)) continue;
                    const double c = afac_value(m, r, d);
                    raw[i] += c;
                    raw[j] += c;
                }
            }
        }
        for (int i = 0; i < n; ++i) {
            const int r = afac_post_index(m, s->type[i], g);
            X->af_fac[(size_t)g * n + i] = r >= 0 ? afac_post(m, r, raw[i]) : raw[i];
        }
    }
}

static double saved_factor(const ctx_t* X, int group, int i) {
    return group < X->n_groups ? X->af_fac[(size_t)group * X->s->n + i] : 0.0;
}

/* core_add_bond_order_forces, Core.f90:4745-4933: -prefactor times the gradient
 * of atom a's per-atom factor, over all of a's neighbours (no pick) */
static void afac_forces(const ctx_t* X, int group, int a, double prefactor, double* F, double* stress) {
    if (group >= X->n_groups) return;
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const orc_nblist* nb = X->nb;
    const int ta = s->type[a];
    const double raw = X->af_raw[(size_t)group * s->n + a];
    const int post = afac_post_index(m, ta, group);
    double virial[6] = {0, 0, 0, 0, 0, 0};
    for (int e = nb->start[a]; e < nb->start[a + 1]; ++e) {
        const int j = nb->idx[e];
        double sep[3];
        separation(&X->C, s->pos + 3 * (size_t)a, s->pos + 3 * (size_t)j, nb->off + 3 * (size_t)e, sep);
        const double d = sqrt(dot3(sep, sep));
        if (!(d < X->maxbr[a])) continue;
        const int tj = s->type[j];
        for (int r = 0; r < m->n_afac; ++r) {
            if (!has(m->afac_mask1[r], ta) || m->afac_group[r] != group || !(m->afac_cutoff[r] > d)) continue;
            if (!has(m->afac_mask2[r], tj) || !afac_two_target(m->afac_kind[r])) continue;
            double g11[3], g12[3], n1[3], n2[3];
            afac_gradient(m, r, sep, d, g11, g12);
            for (int c = 0; c < 3; ++c) {
                if (post >= 0) {
                    n1[c] = -(prefactor * afac_post_grad(m, post, raw, g11[c]));
                    n2[c] = -(prefactor * afac_post_grad(m, post, raw, g12[c]));
                } else {
                    n1[c] = -(prefactor * g11[c]);
                    n2[c] = -(prefactor * g12[c]);
                }
                F[3 * (size_t)a + c] += n1[c];
                F[3 * (size_t)j + c] += n2[c];
            }
            virial[0] += sep[0] * g12[0];
            virial[1] += sep[1] * g12[1];
            virial[2] += sep[2] * g12[2];
            virial[3] += sep[1] * g12[2];
            virial[4] += sep[0] * g12[2];
            virial[5] += sep[0] * g12[1];
        }
    }
    for (int c = 0; c < 6; ++c) {
        const double tv = post >= 0 ? afac_post_grad(m, post, raw, virial[c]) : virial[c];
        stress[c] = stress[c] - prefactor * tv;
    }
}

typedef struct {
    const ctx_t* X;
    int what, a0, a1;
    double energy;
    double stress[6];
    double* F;     /* per-thread n x 3 */
    double* chi;   /* per-thread n */
} loop_job;

/* One bond_bend term of the triplet x - c - y, s1 = x -> c, s2 = c -> y:
 * evaluate_energy_bond_bending / evaluate_force_bond_bending (Potentials.f90:
 * 3206-3314; the derived cos(theta_0)^n of 3183-3194) with the cut factors and
 * the virial of core_evaluate_local_triplet_B (Core.f90:6760-6991). */
static int ipow_i(double x, int k, double* out) {
    double v = 1.0;
    for (int q = 0; q < (k < 0 ? -k : k); ++q) v *= x;
    *out = k < 0 ? 1.0 / v : v;
    return 0;
}

static void quad_chain(const orc_model* m, const orc_system* s, uint64_t qm, loop_job* J, const int x[4],
                       const int tp[3], const double s1[3], double d1, const double s2[3], double d2,
                       const double s3[3], double d3);

static void tri_term(const orc_model* m, int r, loop_job* J, int x, int c, int y, const double s1[3], double d1,
                     const double s2[3], double d2) {
    const double* p = m->tri_params + 4 * (size_t)r;
    const int n = (int)p[2], mm = (int)p[3];
    const double derived = pow(cos(p[1]), p[2]);
    const double rc = m->tri_cutoff[r], soft = m->tri_soft[r];
    const int smoothened = soft > 0.0 && soft < rc;
    double f1 = 1.0, f2 = 1.0, g1[3] = {0, 0, 0}, g2[3] = {0, 0, 0};
    if (smoothened) {
        f1 = smooth_factor(d1, rc, soft);
        f2 = smooth_factor(d2, rc, soft);
        const double q1 = smooth_deriv(d1, rc, soft), q2 = smooth_deriv(d2, rc, soft);
        for (int k = 0; k < 3; ++k) {
            g1[k] = s1[k] / d1 * q1; /* smoothening_gradient: f'(d) times the direction */
            g2[k] = s2[k] / d2 * q2;
        }
    }
    /* energy: r3 = (-sep1) . sep2, (r3 / (r1 r2))^n - derived, eps r6^m */
    double t1[3] = {-s1[0], -s1[1], -s1[2]};
    const double r3 = dot3(t1, s2);
    double cn, e6;
    ipow_i(r3 / (d1 * d2), n, &cn);
    ipow_i(cn - derived, mm, &e6);
    const double v = p[0] * e6;
    if (J->what == 0) {
        J->energy += v * f1 * f2;
        return;
    }
    if (J->what != 1) return;
    /* forces of evaluate_force_bond_bending */
    double tmp3[3], tmp4[3];
    for (int k = 0; k < 3; ++k) {
        tmp3[k] = s2[k] - r3 / (d1 * d1) * t1[k];
        tmp4[k] = t1[k] - r3 / (d2 * d2) * s2[k];
    }
    const double ratio = 1.0 / (d1 * d2);
    const double cosplain = r3 * ratio;
    double cospower, dm;
    ipow_i(cosplain, n - 1, &cospower);
    ipow_i(cospower * cosplain - derived, mm - 1, &dm);
    const double r6 = p[0] * (mm * n) * dm * cospower;
    double fx[3], fc[3], fy[3];
    for (int k = 0; k < 3; ++k) {
        const double a = -tmp3[k] * ratio * r6, b = (tmp3[k] + tmp4[k]) * ratio * r6, w = -tmp4[k] * ratio * r6;
        const double e = smoothened ? v : 0.0;
        fx[k] = a * f1 * f2 + g1[k] * f2 * e;
        fc[k] = b * f1 * f2 + (-g1[k] * f2 + g2[k] * f1) * e;
        fy[k] = w * f1 * f2 - g2[k] * f1 * e;
    }
    for (int k = 0; k < 3; ++k) {
        J->F[3 * (size_t)x + k] += fx[k];
        J->F[3 * (size_t)c + k] += fc[k];
        J->F[3 * (size_t)y + k] += fy[k];
    }
    double* st = J->stress;
    st[0] += s1[0] * fc[0] + (s1[0] + s2[0]) * fy[0];
    st[1] += s1[1] * fc[1] + (s1[1] + s2[1]) * fy[1];
    st[2] += s1[2] * fc[2] + (s1[2] + s2[2]) * fy[2];
    st[3] += s1[1] * fc[2] + (s1[1] + s2[1]) * fy[2];
    st[4] += s1[0] * fc[2] + (s1[0] + s2[0]) * fy[2];
    st[5] += s1[0] * fc[1] + (s1[0] + s2[0]) * fy[1];
}

/* A pair record (r) of the picked pair (i = atom1, j = atom2) that depends on
 * the charges or is a product, with the record's group of bond-order factors:
 * V (v), the force on i from V (fp, without the cut factor) and the
 * electronegativities of i and j (en); the energy v f (b_i + b_j + B_ij +
 * B_ji) / 2 with the per-atom factors b and the pair factors B of the group
 * (core_evaluate_local_doublet_energy_B, Core.f90:4257-4385), its forces with
 * the factors' gradients (_forces_B, 5371-5606) and the electronegativities
 * en f times the same mean factor (_electronegativities_B, 5622-5775). */
static void scaled_charge_term(const ctx_t* X, loop_job* J, int r, int i, int j, double v, const double fp[3],
                               const double en[2], const double sep[3], double d, const double dir[3]) {
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const int grp = m->pair_group[r];
    const int sm = X->smoothened[r];
    const double rc = m->pair_cutoff[r], rs = X->smooth_soft[r];
    const double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
    double sums[2];
    pair_bo_sums(X, i, j, sep, d, grp, sums);
    const double B1 = post_process(X, s->type[i], grp, sums[0]);
    const double B2 = post_process(X, s->type[j], grp, sums[1]);
    const double bsum = (saved_factor(X, grp, i) + saved_factor(X, grp, j) + B1 + B2) * 0.5;
    if (J->what == 0) {
        J->energy += v * cut * bsum;
        return;
    }
    if (J->what == 2) {
        J->chi[i] += en[0] * cut * bsum;
        J->chi[j] += en[1] * cut * bsum;
        return;
    }
    double* F = J->F;
    double* st = J->stress;
    afac_forces(X, grp, i, 0.5 * v * cut, F, st);
    afac_forces(X, grp, j, 0.5 * v * cut, F, st);
    pair_bo_forces(X, i, j, 0.5 * v * cut, sep, d, grp, sums, F, st);
    double cg[3] = {0, 0, 0};
    if (sm) {
        const double dv = smooth_deriv(d, rc, rs);
        for (int c = 0; c < 3; ++c) cg[c] = dir[c] * dv;
    }
    double p2[3];
    for (int c = 0; c < 3; ++c) {
        const double p1 = (fp[c] * cut + v * cg[c]) * bsum;
        p2[c] = -p1;
        F[3 * (size_t)i + c] += p1;
        F[3 * (size_t)j + c] += p2[c];
    }
    st[0] += sep[0] * p2[0];
    st[1] += sep[1] * p2[1];
    st[2] += sep[2] * p2[2];
    st[3] += sep[1] * p2[2];
    st[4] += sep[0] * p2[2];
    st[5] += sep[0] * p2[1];
}

/* The per-atom body of core_loop_over_local_interactions, Core.f90:3249-3946,
 * for atoms [a0, a1). Singlets: core_evaluate_local_singlet (4095-4239);
 * inline Ewald real space (3416-3460); doublets: core_evaluate_local_doublet_
 * energy_B (4257-4385) and _forces_B (5371-5606). */
static void* loop_range(void* arg) {
    loop_job* J = (loop_job*)arg;
    const ctx_t* X = J->X;
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const orc_nblist* nb = X->nb;
    const double eps = m->ewald_eps, sig = m->ewald_sigma;
    const double inv_eps_4pi = 1.0 / (4.0 * PI * eps);
    const double inv_sigma_sqrt_2 = 1.0 / (sqrt(2.0) * sig);
    const double inv_sigma_sqrt_2pi = 1.0 / (sqrt(2.0 * PI) * sig);
    const double inv_sigma_sq_2 = inv_sigma_sqrt_2 * inv_sigma_sqrt_2;
    const double inv_sigma_sqrt_2perpi = 2.0 * inv_sigma_sqrt_2pi;
    double* F = J->F;
    double* chi = J->chi;
    double* st = J->stress;
    for (int i = J->a0; i < J->a1; ++i) {
        const int ti = s->type[i];
        const double qi = s->charge[i];
        for (int r = 0; r < m->n_single; ++r) {
            if (!has(m->single_mask[r], ti)) continue;
            const double* p = m->single_params + 4 * (size_t)r;
            const int kind = m->single_kind[r];
            const int grp = m->single_group ? m->single_group[r] : -1;
            /* the singlet's energy V and electronegativity; with a coordinator,
               core_evaluate_local_singlet (Core.f90:4095-4239) scales them by the
               atom's factor and replaces the singlet's own force by -V grad(B_i) */
            double V = 0.0, E = 0.0, Fs[3] = {0, 0, 0};
            if (kind == 0) { /* charge_self, Potentials.f90:4341-4375 */
                int n = (int)p[1];
                V = p[0] * __builtin_powi(qi, n);
                E = -(p[0] * n * __builtin_powi(qi, n - 1));
            } else if (kind == 1) { /* constant potential, 3942-3966 */
                V = p[0];
            } else { /* constant force, 3122-3147: F on the atom, energy -F . position */
                const double* x = s->pos + 3 * (size_t)i;
                V = -(p[0] * x[0] + p[1] * x[1] + p[2] * x[2]);
                for (int c = 0; c < 3; ++c) Fs[c] = p[c];
            }
            if (grp >= 0) {
                const double B = saved_factor(X, grp, i);
                if (J->what == 0) J->energy += V * B;
                else if (J->what == 1) afac_forces(X, grp, i, V, F, st);
                else chi[i] += E * B;
            } else {
                if (J->what == 0) J->energy += V;
                else if (J->what == 1)
                    for (int c = 0; c < 3; ++c) F[3 * (size_t)i + c] += Fs[c];
                else if (kind == 0) chi[i] += E;
            }
        }
        for (int e = nb->start[i]; e < nb->start[i + 1]; ++e) {
            const int j = nb->idx[e];
            const int* o = nb->off + 3 * (size_t)e;
            if (!pick(i, j, o)) continue;
            const int tj = s->type[j];
            double sep[3];
            separation(&X->C, s->pos + 3 * (size_t)i, s->pos + 3 * (size_t)j, o, sep);
            double d = sqrt(dot3(sep, sep));
            double dir[3] = {0, 0, 0};
            if (d != 0.0)
                for (int c = 0; c < 3; ++c) dir[c] = sep[c] / d;
            if (m->ewald && d < m->ewald_rc) {
                const double q1 = qi, q2 = s->charge[j];
                if (J->what == 0) {
                    J->energy += q1 * q2 * (1.0 - erf(d * inv_sigma_sqrt_2)) / d * inv_eps_4pi;
                } else if (J->what == 1) {
                    double inv_dist = 1.0 / d;
                    double pre = -(inv_eps_4pi * q1 * q2 *
                                   ((1.0 - erf(d * inv_sigma_sqrt_2)) * inv_dist * inv_dist +
                                    inv_sigma_sqrt_2perpi * exp(-(d * d * inv_sigma_sq_2)) * inv_dist));
                    double tf[3];
                    for (int c = 0; c < 3; ++c) tf[c] = pre * sep[c] * inv_dist;
                    for (int c = 0; c < 3; ++c) {
                        F[3 * (size_t)i + c] += tf[c];
                        F[3 * (size_t)j + c] -= tf[c];
                    }
                    st[0] -= sep[0] * tf[0];
                    st[1] -= sep[1] * tf[1];
                    st[2] -= sep[2] * tf[2];
                    st[3] -= sep[1] * tf[2];
                    st[4] -= sep[0] * tf[2];
                    st[5] -= sep[0] * tf[1];
                } else {
                    double tmp = -(inv_eps_4pi / d * (1.0 - erf(d * inv_sigma_sqrt_2)));
                    chi[i] += q2 * tmp;
                    chi[j] += q1 * tmp;
                }
            }
            for (int r = 0; r < m->n_pair; ++r) {
                if (!has(m->pair_mask1[r], ti)) continue;
                if (!(m->pair_cutoff[r] > d)) continue;
                if (!has(m->pair_mask2[r], tj)) continue;
                const int kind = m->pair_kind[r];
                if (m->pair_group[r] >= 0 && ((m->pair_nmul && m->pair_nmul[r] > 0) || kind >= 7)) {
                    /* a charge-dependent term or product scaled by bond-order factors
                       (the doublet routines with bo_factors and pair_bo_factors,
                       Core.f90:4257-4385, 5371-5606, 5622-5775) */
                    double v, fp[3], en[2];
                    product_term(m, r, ti, qi, s->charge[j], sep, d, &v, fp, en);
                    scaled_charge_term(X, J, r, i, j, v, fp, en, sep, d, dir);
                    continue;
                }
                if (m->pair_nmul && m->pair_nmul[r] > 0) {
                    /* a product of potentials (n_product > 1): the product's energy, force and
                       electronegativities times the record's smooth cut (Core.f90:4257-4385,
                       5371-5606, 5622-5775); products carry no bond-order factor */
                    const int smp = X->smoothened[r];
                    const double rcp = m->pair_cutoff[r], rsp = X->smooth_soft[r];
                    double v, fp[3], en[2];
                    product_term(m, r, ti, qi, s->charge[j], sep, d, &v, fp, en);
                    const double cut = smp ? smooth_factor(d, rcp, rsp) : 1.0;
                    if (J->what == 0) {
                        J->energy += v * cut;
                    } else if (J->what == 1) {
                        double cg[3] = {0, 0, 0}, p2[3];
                        if (smp) {
                            const double dv = smooth_deriv(d, rcp, rsp);
                            for (int c = 0; c < 3; ++c) cg[c] = dir[c] * dv;
                        }
                        for (int c = 0; c < 3; ++c) {
                            const double p1 = fp[c] * cut + v * cg[c];
                            p2[c] = -fp[c] * cut - v * cg[c];
                            F[3 * (size_t)i + c] += p1;
                            F[3 * (size_t)j + c] += p2[c];
                        }
                        st[0] += sep[0] * p2[0];
                        st[1] += sep[1] * p2[1];
                        st[2] += sep[2] * p2[2];
                        st[3] += sep[1] * p2[2];
                        st[4] += sep[0] * p2[2];
                        st[5] += sep[0] * p2[1];
                    } else {
                        chi[i] += en[0] * cut;
                        chi[j] += en[1] * cut;
                    }
                    continue;
                }
                /* non-charge pair potentials have zero electronegativity */
                if (J->what == 2 && (kind < 7 || kind == 10)) continue;
                const double* p = m->pair_params + 4 * (size_t)r;
                const int grp = m->pair_group[r];
                const int sm = X->smoothened[r];
                const double rc = m->pair_cutoff[r], rs = X->smooth_soft[r];
                if (kind == 9) {
                    /* charge_abs, Potentials.f90:4525-4728: sqrt(f1(q1) f2(q2)), f(q) = a + b |q - Q|^n
                       (negative f taken as 0), parameters (a, b, Q, n) of the unpermuted first
                       target on atom1 when its type is that target's; rows from p[0] hold
                       a1, b1, Q1, n1, a2, b2, Q2, n2; only the cut factor's gradient acts */
                    const double* c = m->pair_table + 2 * (int64_t)p[0];
                    const int direct = has(m->pair_first[r], ti);
                    const double* s1 = c + (direct ? 0 : 4);
                    const double* s2 = c + (direct ? 4 : 0);
                    const double qq1 = s->charge[i], qq2 = s->charge[j];
                    double v;
                    if (J->what == 2) {
                        const double abs1 = fabs(qq1 - s1[2]), abs2 = fabs(qq2 - s2[2]);
                        const double pow1 = pow(abs1, s1[3] - 1), pow2 = pow(abs2, s2[3] - 1);
                        double f1 = s1[0] + s1[1] * abs1 * pow1, f2 = s2[0] + s2[1] * abs2 * pow2;
                        const double d1 = -s1[3] * pow1 * copysign(1.0, qq1 - s1[2]) * s1[1];
                        const double d2 = -s2[3] * pow2 * copysign(1.0, qq2 - s2[2]) * s2[1];
                        double inv_sqrt = 0.5 / sqrt(f1 * f2);
                        if (f1 < 0.0) {
                            f1 = 0.0;
                            inv_sqrt = 0.0;
                        }
                        if (f2 < 0.0) {
                            f2 = 0.0;
                            inv_sqrt = 0.0;
                        }
                        const double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
                        chi[i] += inv_sqrt * d1 * f2 * cut;
                        chi[j] += inv_sqrt * d2 * f1 * cut;
                        continue;
                    }
                    {
                        double f1 = s1[0] + s1[1] * pow(fabs(qq1 - s1[2]), s1[3]);
                        double f2 = s2[0] + s2[1] * pow(fabs(qq2 - s2[2]), s2[3]);
                        if (f1 < 0.0) f1 = 0.0;
                        if (f2 < 0.0) f2 = 0.0;
                        v = sqrt(f1 * f2);
                    }
                    const double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
                    if (J->what == 0) {
                        J->energy += v * cut;
                    } else if (sm) {
                        const double dv = smooth_deriv(d, rc, rs);
                        double p2[3];
                        for (int c3 = 0; c3 < 3; ++c3) {
                            const double g = dir[c3] * dv;
                            F[3 * (size_t)i + c3] += v * g;
                            p2[c3] = -v * g;
                            F[3 * (size_t)j + c3] += p2[c3];
                        }
                        st[0] += sep[0] * p2[0];
                        st[1] += sep[1] * p2[1];
                        st[2] += sep[2] * p2[2];
                        st[3] += sep[1] * p2[2];
                        st[4] += sep[0] * p2[2];
                        st[5] += sep[0] * p2[1];
                    }
                    continue;
                }
                if (kind == 8) {
                    /* charge_exp, Potentials.f90:3691-3903: epsilon exp((xi_1 D_1 + xi_2 D_2)/2),
                       D(q) = Rmax + |beta (Qmax - q)|^eta, parameters swapped unless atom1
                       is the unpermuted first target; rows from p[0] hold eps, Rmax1, Rmin1,
                       Qmax1, Qmin1, Rmax2, Rmin2, Qmax2, Qmin2, xi1, xi2, eta1, eta2, beta1,
                       beta2; no force routine, so only the cut factor's gradient acts */
                    const double* c = m->pair_table + 2 * (int64_t)p[0];
                    const double q1 = s->charge[i], q2 = s->charge[j];
                    const int direct = has(m->pair_first[r], ti);
                    const double r2 = c[direct ? 1 : 5], r3 = c[direct ? 5 : 1];
                    const double r4 = c[direct ? 3 : 7], r5 = c[direct ? 7 : 3];
                    const double r6 = c[direct ? 11 : 12], r7 = c[direct ? 12 : 11];
                    const double r8 = c[direct ? 13 : 14], r9 = c[direct ? 14 : 13];
                    const double d3 = c[direct ? 9 : 10], d4 = c[direct ? 10 : 9];
                    const double d5 = r8 * (r4 - q1), d6 = r9 * (r5 - q2);
                    const double d1 = r2 + pow(fabs(d5), r6), d2 = r3 + pow(fabs(d6), r7);
                    const double v = c[0] * exp(0.5 * (d3 * d1 + d4 * d2));
                    const double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
                    if (J->what == 0) {
                        J->energy += v * cut;
                    } else if (J->what == 1) {
                        if (sm) {
                            const double dv = smooth_deriv(d, rc, rs);
                            double p2[3];
                            for (int c3 = 0; c3 < 3; ++c3) {
                                const double g = dir[c3] * dv;
                                F[3 * (size_t)i + c3] += v * g;
                                p2[c3] = -v * g;
                                F[3 * (size_t)j + c3] += p2[c3];
                            }
                            st[0] += sep[0] * p2[0];
                            st[1] += sep[1] * p2[1];
                            st[2] += sep[2] * p2[2];
                            st[3] += sep[1] * p2[2];
                            st[4] += sep[0] * p2[2];
                            st[5] += sep[0] * p2[1];
                        }
                    } else {
                        const double e2 = v * d4 * 0.5 * r7 * pow(fabs(d6), r7 - 1.0) * copysign(1.0, d6) * r9;
                        const double e1 = v * d3 * 0.5 * r6 * pow(fabs(d5), r6 - 1.0) * copysign(1.0, d5) * r8;
                        chi[i] += e1 * cut;
                        chi[j] += e2 * cut;
                    }
                    continue;
                }
                if (kind == 7) {
                    /* charge_pair, Potentials.f90:4415-4513: epsilon q1^n1 q2^n2, the
                       exponents swapped unless atom1 is the unpermuted first target;
                       no force routine, so only the cut factor's gradient acts */
                    const double q1 = s->charge[i], q2 = s->charge[j];
                    const int direct = has(m->pair_first[r], ti);
                    const int n1 = direct ? (int)p[1] : (int)p[2], n2 = direct ? (int)p[2] : (int)p[1];
                    const double v = p[0] * (__builtin_powi(q1, n1) * __builtin_powi(q2, n2));
                    const double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
                    if (J->what == 0) {
                        J->energy += v * cut;
                    } else if (J->what == 1) {
                        if (sm) {
                            const double dv = smooth_deriv(d, rc, rs);
                            double p2[3];
                            for (int c = 0; c < 3; ++c) {
                                const double g = dir[c] * dv;
                                F[3 * (size_t)i + c] += v * g;
                                p2[c] = -v * g;
                                F[3 * (size_t)j + c] += p2[c];
                            }
                            st[0] += sep[0] * p2[0];
                            st[1] += sep[1] * p2[1];
                            st[2] += sep[2] * p2[2];
                            st[3] += sep[1] * p2[2];
                            st[4] += sep[0] * p2[2];
                            st[5] += sep[0] * p2[1];
                        }
                    } else {
                        const double e1 = n1 > 0 ? -p[0] * (n1 * __builtin_powi(q1, n1 - 1) * __builtin_powi(q2, n2)) : 0.0;
                        const double e2 = n2 > 0 ? -p[0] * (n2 * __builtin_powi(q1, n1) * __builtin_powi(q2, n2 - 1)) : 0.0;
                        chi[i] += e1 * cut;
                        chi[j] += e2 * cut;
                    }
                    continue;
                }
                if (J->what == 0) {
                    double B1 = 0, B2 = 0;
                    if (grp >= 0) {
                        double sums[2];
                        pair_bo_sums(X, i, j, sep, d, grp, sums);
                        B1 = post_process(X, ti, grp, sums[0]);
                        B2 = post_process(X, tj, grp, sums[1]);
                    }
                    double cut = sm ? smooth_factor(d, rc, rs) : 1.0;
                    double v = pair_energy(kind, p, rc, d, m->pair_table);
                    if (grp >= 0)
                        J->energy += v * cut * (saved_factor(X, grp, i) + saved_factor(X, grp, j) + B1 + B2) * 0.5;
                    else J->energy += v * cut;
                } else {
                    double v = (grp >= 0 || sm) ? pair_energy(kind, p, rc, d, m->pair_table) : 0.0;
                    double cut = 1.0, cg[3] = {0, 0, 0};
                    if (sm) {
                        cut = smooth_factor(d, rc, rs);
                        double dv = smooth_deriv(d, rc, rs);
                        for (int c = 0; c < 3; ++c) cg[c] = dir[c] * dv;
                    }
                    double B1 = 0, B2 = 0;
                    if (grp >= 0) {
                        double sums[2];
                        pair_bo_sums(X, i, j, sep, d, grp, sums);
                        B1 = post_process(X, ti, grp, sums[0]);
                        B2 = post_process(X, tj, grp, sums[1]);
                        afac_forces(X, grp, i, 0.5 * v * cut, F, st);
                        afac_forces(X, grp, j, 0.5 * v * cut, F, st);
                        pair_bo_forces(X, i, j, 0.5 * v * cut, sep, d, grp, sums, F, st);
                    }
                    double f1[3], p1[3], p2[3];
                    pair_force(kind, p, rc, sep, d, f1, m->pair_table);
                    for (int c = 0; c < 3; ++c) {
                        if (grp >= 0) {
                            double bsum = (saved_factor(X, grp, i) + saved_factor(X, grp, j) + B1 + B2) * 0.5;
                            p1[c] = (f1[c] * cut + v * cg[c]) * bsum;
                            p2[c] = (-f1[c] * cut - v * cg[c]) * bsum;
                        } else {
                            p1[c] = f1[c] * cut + v * cg[c];
                            p2[c] = -f1[c] * cut - v * cg[c];
                        }
                    }
                    for (int c = 0; c < 3; ++c) {
                        F[3 * (size_t)i + c] += p1[c];
                        F[3 * (size_t)j + c] += p2[c];
                    }
                    st[0] += sep[0] * p2[0];
                    st[1] += sep[1] * p2[1];
                    st[2] += sep[2] * p2[2];
                    st[3] += sep[1] * p2[2];
                    st[4] += sep[0] * p2[2];
                    st[5] += sep[0] * p2[1];
                }
            }
            /* three-body records (Core.f90:3540-3943): the doublet routines flag
               the many-body potentials of this pair, then the two triplet loops */
            if ((m->n_tri > 0 || m->n_quad > 0) && d != 0.0) {
                uint64_t rm = 0, qm = 0;
                for (int r = 0; r < m->n_tri; ++r) {
                    const uint64_t many = m->tri_mask1[r] | m->tri_mask2[r] | m->tri_mask3[r];
                    if (m->tri_cutoff[r] > d && has(many, ti) && has(m->tri_mask2[r], tj)) rm |= 1ull << r;
                }
                for (int r = 0; r < m->n_quad; ++r) {
                    const uint64_t* mk = m->quad_mask + 4 * (size_t)r;
                    if (m->quad_cutoff[r] > d && has(mk[0] | mk[1] | mk[2] | mk[3], ti) && has(mk[1], tj))
                        qm |= 1ull << r;
                }
                if (rm || qm) {
                    const double s21[3] = {-sep[0], -sep[1], -sep[2]};
                    /* atom2 - atom1 - atom3, atom3 among atom1's neighbours */
                    for (int l = nb->start[i]; l < nb->start[i + 1]; ++l) {
                        const int k = nb->idx[l];
                        const int* ol = nb->off + 3 * (size_t)l;
                        const int o23[3] = {ol[0] - o[0], ol[1] - o[1], ol[2] - o[2]};
                        if (!pick(j, k, o23)) continue;
                        double s13[3];
                        separation(&X->C, s->pos + 3 * (size_t)i, s->pos + 3 * (size_t)k, ol, s13);
                        const double d13 = sqrt(dot3(s13, s13));
                        if (d13 == 0.0) continue;
                        const int tk = s->type[k];
                        for (int r = 0; r < m->n_tri; ++r)
                            if (((rm >> r) & 1) && has(m->tri_mask3[r], tk) && has(m->tri_center[r], ti) &&
                                m->tri_cutoff[r] > d13)
                                tri_term(m, r, J, j, i, k, s21, d, s13, d13);
                        if (!qm) continue;
                        /* atom4 - atom2 - atom1 - atom3, atom4 among atom2's neighbours (Core.f90:3614-3690) */
                        for (int q = nb->start[j]; q < nb->start[j + 1]; ++q) {
                            const int w = nb->idx[q];
                            const int* oq = nb->off + 3 * (size_t)q;
                            const int o34[3] = {oq[0] - o23[0], oq[1] - o23[1], oq[2] - o23[2]};
                            if (!pick(k, w, o34) || w == i) continue;
                            const int mo[3] = {-oq[0], -oq[1], -oq[2]};
                            double s42[3];
                            separation(&X->C, s->pos + 3 * (size_t)w, s->pos + 3 * (size_t)j, mo, s42);
                            const int x[4] = {w, j, i, k}, tp[3] = {0, 1, 3};
                            quad_chain(m, s, qm, J, x, tp, s42, sqrt(dot3(s42, s42)), s21, d, s13, d13);
                        }
                        /* atom2 - atom1 - atom3 - atom4, atom4 among atom3's neighbours (3695-3750) */
                        for (int q = nb->start[k]; q < nb->start[k + 1]; ++q) {
                            const int w = nb->idx[q];
                            const int* oq = nb->off + 3 * (size_t)q;
                            const int o24[3] = {oq[0] + o23[0], oq[1] + o23[1], oq[2] + o23[2]};
                            if (!pick(j, w, o24) || w == i) continue;
                            double s34[3];
                            separation(&X->C, s->pos + 3 * (size_t)k, s->pos + 3 * (size_t)w, oq, s34);
                            const int x[4] = {j, i, k, w}, tp[3] = {0, 2, 3};
                            quad_chain(m, s, qm, J, x, tp, s21, d, s13, d13, s34, sqrt(dot3(s34, s34)));
                        }
                    }
                    /* atom1 - atom2 - atom3, atom3 among atom2's neighbours */
                    for (int l = nb->start[j]; l < nb->start[j + 1]; ++l) {
                        const int k = nb->idx[l];
                        const int* ol = nb->off + 3 * (size_t)l;
                        const int o13[3] = {ol[0] + o[0], ol[1] + o[1], ol[2] + o[2]};
                        if (!pick(i, k, o13)) continue;
                        double s23[3];
                        separation(&X->C, s->pos + 3 * (size_t)j, s->pos + 3 * (size_t)k, ol, s23);
                        const double d23 = sqrt(dot3(s23, s23));
                        if (d23 == 0.0) continue;
                        const int tk = s->type[k];
                        for (int r = 0; r < m->n_tri; ++r)
                            if (((rm >> r) & 1) && has(m->tri_mask3[r], tk) && has(m->tri_center[r], tj) &&
                                m->tri_cutoff[r] > d23)
                                tri_term(m, r, J, i, j, k, sep, d, s23, d23);
                        if (!qm) continue;
                        /* atom4 - atom1 - atom2 - atom3, atom4 among atom1's neighbours (3807-3880) */
                        for (int q = nb->start[i]; q < nb->start[i + 1]; ++q) {
                            const int w = nb->idx[q];
                            const int* oq = nb->off + 3 * (size_t)q;
                            const int o34[3] = {oq[0] - o13[0], oq[1] - o13[1], oq[2] - o13[2]};
                            if (!pick(k, w, o34) || w == j) continue;
                            const int mo[3] = {-oq[0], -oq[1], -oq[2]};
                            double s41[3];
                            separation(&X->C, s->pos + 3 * (size_t)w, s->pos + 3 * (size_t)i, mo, s41);
                            const int x[4] = {w, i, j, k}, tp[3] = {0, 2, 3};
                            quad_chain(m, s, qm, J, x, tp, s41, sqrt(dot3(s41, s41)), sep, d, s23, d23);
                        }
                        /* atom1 - atom2 - atom3 - atom4, atom4 among atom3's neighbours (3885-3940) */
                        for (int q = nb->start[k]; q < nb->start[k + 1]; ++q) {
                            const int w = nb->idx[q];
                            const int* oq = nb->off + 3 * (size_t)q;
                            const int o14[3] = {oq[0] + o13[0], oq[1] + o13[1], oq[2] + o13[2]};
                            if (!pick(i, w, o14) || w == j) continue;
                            double s34[3];
                            separation(&X->C, s->pos + 3 * (size_t)k, s->pos + 3 * (size_t)w, oq, s34);
                            const int x[4] = {i, j, k, w}, tp[3] = {1, 2, 3};
                            quad_chain(m, s, qm, J, x, tp, sep, d, s23, d23, s34, sqrt(dot3(s34, s34)));
                        }
                    }
                }
            }
        }
    }
    return NULL;
}

/* evaluate_energy_dihedral / evaluate_force_dihedral, Potentials.f90:3380-3611:
 * V = k/2 (cos phi - cos phi_0)^2 of the chain 1-2-3-4 (v12, v23, v34 its
 * separations), cos phi from the projections of v12 and v34 perpendicular to
 * v23; zero unless the atoms' types match the unpermuted targets forwards or
 * backwards.  f[a] is the force on chain atom a. */
static int dihedral(const orc_model* m, int r, const int t[4], const double v12[3], const double v23[3],
                    const double v34[3], double* e, double f[4][3]) {
    const uint64_t* o = m->quad_orig + 4 * (size_t)r;
    const int ok = (has(o[0], t[0]) && has(o[1], t[1]) && has(o[2], t[2]) && has(o[3], t[3])) ||
                   (has(o[0], t[3]) && has(o[1], t[2]) && has(o[2], t[1]) && has(o[3], t[0]));
    *e = 0.0;
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c) f[a][c] = 0.0;
    if (!ok) return 0;
    const double k = m->quad_params[4 * (size_t)r], cos0 = cos(m->quad_params[4 * (size_t)r + 1]);
    const double r2 = sqrt(dot3(v23, v23));
    const double inv_r2 = 1.0 / (r2 * r2);
    const double a12 = dot3(v12, v23), a34 = dot3(v34, v23);
    double p1[3], p2[3];
    for (int c = 0; c < 3; ++c) {
        p1[c] = -(v12[c] - a12 * inv_r2 * v23[c]);
        p2[c] = v34[c] - a34 * inv_r2 * v23[c];
    }
    const double dot = dot3(p1, p2);
    const double inv_p1 = 1.0 / sqrt(dot3(p1, p1)), inv_p2 = 1.0 / sqrt(dot3(p2, p2));
    const double ratio = inv_p1 * inv_p2;
    const double off = dot * ratio - cos0;
    *e = 0.5 * k * off * off;
    double dd[4][3], dq1[4][3], dq2[4][3];
    for (int c = 0; c < 3; ++c) {
        dd[0][c] = -(v34[c] - a34 * inv_r2 * v23[c]);
        dd[1][c] = v34[c] - a34 * inv_r2 * (v23[c] - v12[c]) + a12 * inv_r2 * v34[c] -
                   2.0 * a12 * a34 * inv_r2 * inv_r2 * v23[c];
        dd[2][c] = -(v12[c] + a34 * inv_r2 * v12[c] + a12 * inv_r2 * (v34[c] - v23[c]) -
                     2.0 * a12 * a34 * inv_r2 * inv_r2 * v23[c]);
        dd[3][c] = v12[c] - a12 * inv_r2 * v23[c];
        dq2[0][c] = 0.0;
        dq2[1][c] = a34 * inv_r2 * v34[c] - a34 * a34 * inv_r2 * inv_r2 * v23[c];
        dq2[2][c] = -v34[c] + a34 * inv_r2 * (v23[c] - v34[c]) + a34 * a34 * inv_r2 * inv_r2 * v23[c];
        dq2[3][c] = v34[c] - a34 * inv_r2 * v23[c];
        dq1[0][c] = -v12[c] + a12 * inv_r2 * v23[c];
        dq1[1][c] = v12[c] - a12 * inv_r2 * (v23[c] - v12[c]) - a12 * a12 * inv_r2 * inv_r2 * v23[c];
        dq1[2][c] = -a12 * inv_r2 * v12[c] + a12 * a12 * inv_r2 * inv_r2 * v23[c];
        dq1[3][c] = 0.0;
    }
    const double pre = k * off * ratio;
    for (int a = 0; a < 4; ++a)
        for (int c = 0; c < 3; ++c)
            f[a][c] = pre * (dd[a][c] + dq1[a][c] * dot * inv_p1 * inv_p1 + dq2[a][c] * dot * inv_p2 * inv_p2);
    return 1;
}

/* core_evaluate_local_quadruplet_B (Core.f90:7450-7883) for the chain x[0..3]
 * with separations s1, s2, s3 and distances d1..d3: the records the doublet
 * flagged (qm), the types of chain positions tp[0..2] tested as target
 * positions 2, 3, 4, every bond within the record's cutoff; energy times the
 * three cut factors, forces with the cut gradients, and the virial
 * s1 (x) F2 + (s1 + s2) (x) F3 + (s1 + s2 + s3) (x) F4. */
static void quad_chain(const orc_model* m, const orc_system* s, uint64_t qm, loop_job* J, const int x[4],
                       const int tp[3], const double s1[3], double d1, const double s2[3], double d2,
                       const double s3[3], double d3) {
    const int t[4] = {s->type[x[0]], s->type[x[1]], s->type[x[2]], s->type[x[3]]};
    for (int r = 0; r < m->n_quad; ++r) {
        if (!((qm >> r) & 1)) continue;
        const uint64_t* mk = m->quad_mask + 4 * (size_t)r;
        const double rc = m->quad_cutoff[r], soft = m->quad_soft[r];
        if (!(has(mk[1], t[tp[0]]) && rc > d1 && has(mk[2], t[tp[1]]) && has(mk[3], t[tp[2]]) && rc > d2 &&
              rc > d3))
            continue;
        if (d1 == 0.0 || d2 == 0.0 || d3 == 0.0) continue;
        double e, fq[4][3];
        dihedral(m, r, t, s1, s2, s3, &e, fq);
        const int sm = soft > 0.0 && soft < rc;
        const double c1 = sm ? smooth_factor(d1, rc, soft) : 1.0, c2 = sm ? smooth_factor(d2, rc, soft) : 1.0,
                     c3 = sm ? smooth_factor(d3, rc, soft) : 1.0;
        if (J->what == 0) {
            J->energy += e * c1 * c2 * c3;
            continue;
        }
        if (J->what != 1) continue;  /* no electronegativity */
        double g1[3] = {0, 0, 0}, g2[3] = {0, 0, 0}, g3[3] = {0, 0, 0};
        if (sm) {
            const double q1 = smooth_deriv(d1, rc, soft), q2 = smooth_deriv(d2, rc, soft),
                         q3 = smooth_deriv(d3, rc, soft);
            for (int c = 0; c < 3; ++c) {
                g1[c] = q1 * s1[c] / d1;
                g2[c] = q2 * s2[c] / d2;
                g3[c] = q3 * s3[c] / d3;
            }
        } else {
            e = 0.0;  /* the energy enters the forces only through the cut gradients */
        }
        double qf[4][3];
        for (int c = 0; c < 3; ++c) {
            qf[0][c] = fq[0][c] * c1 * c2 * c3 + g1[c] * c2 * c3 * e;
            qf[1][c] = fq[1][c] * c1 * c2 * c3 + (-g1[c] * c2 * c3 + g2[c] * c1 * c3) * e;
            qf[2][c] = fq[2][c] * c1 * c2 * c3 + (g3[c] * c1 * c2 - g2[c] * c1 * c3) * e;
            qf[3][c] = fq[3][c] * c1 * c2 * c3 - g3[c] * c1 * c2 * e;
        }
        double* F = J->F;
        for (int a = 0; a < 4; ++a)
            for (int c = 0; c < 3; ++c) F[3 * (size_t)x[a] + c] += qf[a][c];
        double s12[3], s123[3];
        for (int c = 0; c < 3; ++c) {
            s12[c] = s1[c] + s2[c];
            s123[c] = s12[c] + s3[c];
        }
        double* st = J->stress;
        st[0] += s1[0] * qf[1][0] + s12[0] * qf[2][0] + s123[0] * qf[3][0];
        st[1] += s1[1] * qf[1][1] + s12[1] * qf[2][1] + s123[1] * qf[3][1];
        st[2] += s1[2] * qf[1][2] + s12[2] * qf[2][2] + s123[2] * qf[3][2];
        st[3] += s1[1] * qf[1][2] + s12[1] * qf[2][2] + s123[1] * qf[3][2];
        st[4] += s1[0] * qf[1][2] + s12[0] * qf[2][2] + s123[0] * qf[3][2];
        st[5] += s1[0] * qf[1][1] + s12[0] * qf[2][1] + s123[0] * qf[3][1];
    }
}

/* k-space Ewald: calculate_ewald_energy (Potentials.f90:1428-1653),
 * calculate_ewald_forces (1675-1971), calculate_ewald_electronegativities
 * (1992-2249), all with include_realspace = .false. and no dipole correction
 * (Core.f90:3983-4060). */
typedef struct {
    const ctx_t* X;
    int what, a0, a1, nk;
    const double* kv;   /* 4 per listed k: kx, ky, kz, weight flag (k3 == 0 ? 1 : 2) */
    double* S;          /* 2 per k (per-thread partial) */
    double e2, e4;
} sk_job;

static void* sk_range(void* arg) {
    sk_job* J = (sk_job*)arg;
    const orc_system* s = J->X->s;
    const orc_model* m = J->X->m;
    for (int i = J->a0; i < J->a1; ++i) {
        const double q1 = s->charge[i] * m->ewald_scaler[i];
        if (J->what != 2 && q1 == 0.0) continue;
        const double* r = s->pos + 3 * (size_t)i;
        for (int k = 0; k < J->nk; ++k) {
            const double* kv = J->kv + 4 * (size_t)k;
            double dot = kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2];
            if (J->what == 0) {
                double sine = q1 * sin(dot), cosine = q1 * cos(dot);
                J->S[2 * k] += cosine;
                J->S[2 * k + 1] += sine;
            } else {
                double sn = sin(dot), cs = cos(dot);
                J->S[2 * k] += q1 * cs;
                J->S[2 * k + 1] += -(q1 * sn);
            }
        }
        J->e2 += q1 * q1;
        J->e4 += q1;
    }
    return NULL;
}

typedef struct {
    const ctx_t* X;
    int what, a0, a1, nk;
    const double* kv;
    const double* S;
    double* F;
    double* chi;
    double stress[6];
    double qsum;
} kf_job;

static void* kf_range(void* arg) {
    kf_job* J = (kf_job*)arg;
    const orc_system* s = J->X->s;
    const orc_model* m = J->X->m;
    const double sig = m->ewald_sigma, eps = m->ewald_eps;
    const double inv_eps_2v = 1.0 / (2.0 * J->X->C.volume * eps);
    const double inv_eps_4pi = 1.0 / (4.0 * PI * eps);
    const double inv_sigma_sqrt_2pi = 1.0 / (sqrt(2.0 * PI) * sig);
    for (int i = J->a0; i < J->a1; ++i) {
        const double q1 = s->charge[i] * m->ewald_scaler[i];
        const double* r = s->pos + 3 * (size_t)i;
        if (J->what == 1) {
            double f[3] = {0, 0, 0};
            for (int k = 0; k < J->nk; ++k) {
                const double* kv = J->kv + 4 * (size_t)k;
                double dist = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
                double dot = kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2];
                double sn = sin(dot), cs = cos(dot);
                double kq[3] = {q1 * kv[0], q1 * kv[1], q1 * kv[2]};
                double w = kv[3] == 1.0 ? 2.0 : 4.0;
                double pre = inv_eps_2v * exp(-(sig * sig * dist * 0.5)) / dist * w;
                for (int c = 0; c < 3; ++c) {
                    double nf1 = -sn * kq[c], nf2 = cs * kq[c];
                    f[c] = f[c] - pre * (J->S[2 * k] * nf1 - J->S[2 * k + 1] * nf2);
                }
            }
            for (int c = 0; c < 3; ++c) J->F[3 * (size_t)i + c] = f[c];
            J->stress[0] += r[0] * (f[0] + 0.0);
            J->stress[1] += r[1] * (f[1] + 0.0);
            J->stress[2] += r[2] * (f[2] + 0.0);
            J->stress[3] += r[1] * (f[2] + 0.0);
            J->stress[4] += r[0] * (f[2] + 0.0);
            J->stress[5] += r[0] * (f[1] + 0.0);
        } else {
            double x = J->chi[i] - m->ewald_scaler[i] * inv_eps_2v * (-(sig * sig * J->qsum));
            for (int k = 0; k < J->nk; ++k) {
                const double* kv = J->kv + 4 * (size_t)k;
                double dist = kv[0] * kv[0] + kv[1] * kv[1] + kv[2] * kv[2];
                double dot = kv[0] * r[0] + kv[1] * r[1] + kv[2] * r[2];
                double sn = sin(dot), cs = cos(dot);
                double w = kv[3] == 1.0 ? 2.0 : 4.0;
                x = x - inv_eps_2v * exp(-(sig * sig * dist * 0.5)) / dist * w * (J->S[2 * k] * cs - J->S[2 * k + 1] * sn);
            }
            J->chi[i] = x;
        }
        (void)inv_eps_4pi;
        (void)inv_sigma_sqrt_2pi;
    }
    return NULL;
}

static void run_jobs(void* (*fn)(void*), void* jobs, size_t stride, int threads) {
    if (threads <= 1) {
        fn(jobs);
        return;
    }
    pthread_t* th = (pthread_t*)malloc(sizeof(pthread_t) * (size_t)threads);
    for (int t = 0; t < threads; ++t) pthread_create(&th[t], NULL, fn, (char*)jobs + stride * (size_t)t);
    for (int t = 0; t < threads; ++t) pthread_join(th[t], NULL);
    free(th);
}

/* The listed k vectors in the reference loop order (k1, k2 outer, k3 >= 0 inner). */
static int list_kvectors(const ctx_t* X, double** out) {
    const orc_model* m = X->m;
    const int K1 = m->ewald_kmax[0], K2 = m->ewald_kmax[1], K3 = m->ewald_kmax[2];
    const double kcsq = m->ewald_kc * m->ewald_kc;
    size_t cap = (size_t)(2 * K1 + 1) * (2 * K2 + 1) * (K3 + 1);
    double* kv = (double*)malloc(sizeof(double) * 4 * (cap ? cap : 1));
    int nk = 0;
    for (int k1 = -K1; k1 <= K1; ++k1)
        for (int k2 = -K2; k2 <= K2; ++k2)
            for (int k3 = 0; k3 <= K3; ++k3) {
                if (!(k1 != 0 || k2 != 0 || k3 != 0)) continue;
                double v[3];
                for (int c = 0; c < 3; ++c)
                    v[c] = (double)k1 * X->C.rc[c][0] + (double)k2 * X->C.rc[c][1] + (double)k3 * X->C.rc[c][2];
                if (dot3(v, v) < kcsq) {
                    double* d = kv + 4 * (size_t)nk++;
                    d[0] = v[0];
                    d[1] = v[1];
                    d[2] = v[2];
                    d[3] = k3 == 0 ? 1.0 : 2.0;
                }
            }
    *out = kv;
    return nk;
}

static void ewald_kspace(const ctx_t* X, int what, int threads, double* energy, double* F, double* stress,
                         double* chi) {
    const orc_system* s = X->s;
    const orc_model* m = X->m;
    const int n = s->n;
    double* kv;
    const int nk = list_kvectors(X, &kv);
    sk_job* sj = (sk_job*)calloc((size_t)threads, sizeof(sk_job));
    for (int t = 0; t < threads; ++t) {
        sj[t].X = X;
        sj[t].what = what;
        sj[t].a0 = (int)((int64_t)n * t / threads);
        sj[t].a1 = (int)((int64_t)n * (t + 1) / threads);
        sj[t].nk = nk;
        sj[t].kv = kv;
        sj[t].S = (double*)calloc(2 * (size_t)(nk ? nk : 1), sizeof(double));
    }
    run_jobs(sk_range, sj, sizeof(sk_job), threads);
    double* S = sj[0].S;
    double e2 = sj[0].e2, e4 = sj[0].e4;
    for (int t = 1; t < threads; ++t) {
        for (int k = 0; k < 2 * nk; ++k) S[k] += sj[t].S[k];
        e2 += sj[t].e2;
        e4 += sj[t].e4;
    }
    const double sig = m->ewald_sigma, eps = m->ewald_eps;
    const double inv_eps_4pi = 1.0 / (4.0 * PI * eps);
    const double inv_eps_2v = 1.0 / (2.0 * X->C.volume * eps);
    const double inv_sigma_sqrt_2pi = 1.0 / (sqrt(2.0 * PI) * sig);
    if (what == 0) {
        double e3 = 0.0;
        for (int k = 0; k < nk; ++k) {
            const double* d = kv + 4 * (size_t)k;
            double dist = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
            double ex = exp(-(sig * sig * dist * 0.5)) / dist;
            double s2 = S[2 * k] * S[2 * k] + S[2 * k + 1] * S[2 * k + 1];
            if (d[3] == 1.0) e3 = e3 + ex * s2;
            else e3 = e3 + 2.0 * ex * s2;
        }
        double en[7];
        en[0] = 0.0 * inv_eps_4pi;
        en[1] = -(e2 * inv_eps_4pi * inv_sigma_sqrt_2pi);
        en[2] = e3 * inv_eps_2v;
        en[3] = -(e4 * e4 * 0.5 * inv_eps_2v * sig * sig);
        en[4] = 0.0;
        en[5] = 0.0;
        en[6] = 0.0;
        double tot = 0.0;
        for (int c = 0; c < 7; ++c) tot += en[c];
        *energy = tot;
    } else {
        kf_job* kj = (kf_job*)calloc((size_t)threads, sizeof(kf_job));
        double* self = NULL;
        if (what == 2) {
            /* self term and charge sum: Potentials.f90:2121-2125 */
            self = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
            for (int i = 0; i < n; ++i) {
                double q1 = s->charge[i] * m->ewald_scaler[i];
                self[i] = 0.0 + 2.0 * q1 * inv_eps_4pi * inv_sigma_sqrt_2pi;
            }
        }
        for (int t = 0; t < threads; ++t) {
            kj[t].X = X;
            kj[t].what = what;
            kj[t].a0 = sj[t].a0;
            kj[t].a1 = sj[t].a1;
            kj[t].nk = nk;
            kj[t].kv = kv;
            kj[t].S = S;
            kj[t].F = F;
            kj[t].chi = self;
            kj[t].qsum = e4;
        }
        run_jobs(kf_range, kj, sizeof(kf_job), threads);
        if (what == 1) {
            for (int c = 0; c < 6; ++c) {
                double v = 0.0;
                for (int t = 0; t < threads; ++t) v += kj[t].stress[c];
                stress[c] = v;
            }
        } else {
            for (int i = 0; i < n; ++i) chi[i] = self[i];
            free(self);
        }
        free(kj);
    }
    for (int t = 0; t < threads; ++t) free(sj[t].S);
    free(sj);
    free(kv);
}

static void setup_ctx(ctx_t* X, const orc_system* s, const orc_model* m, const orc_nblist* nb) {
    X->s = s;
    X->m = m;
    X->nb = nb;
    make_cell(s, &X->C);
    const int n = s->n;
    X->maxbr = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
    for (int i = 0; i < n; ++i) {
        double mc = 0.0;
        for (int b = 0; b < m->n_bond; ++b)
            if (has(m->bond_mask1[b], s->type[i]) && m->bond_cutoff[b] > mc) mc = m->bond_cutoff[b];
        for (int r = 0; r < m->n_afac; ++r)
            if (has(m->afac_mask1[r], s->type[i]) && m->afac_cutoff[r] > mc) mc = m->afac_cutoff[r];
        X->maxbr[i] = mc;
    }
    /* create_potential, Potentials.f90:2382-2388 */
    X->smooth_soft = (double*)calloc((size_t)(m->n_pair ? m->n_pair : 1), sizeof(double));
    X->smoothened = (int*)calloc((size_t)(m->n_pair ? m->n_pair : 1), sizeof(int));
    for (int r = 0; r < m->n_pair; ++r) {
        if (m->pair_soft[r] > 0.0 && m->pair_soft[r] < m->pair_cutoff[r]) {
            X->smooth_soft[r] = m->pair_soft[r];
            X->smoothened[r] = 1;
        } else {
            X->smooth_soft[r] = m->pair_cutoff[r];
            X->smoothened[r] = 0;
        }
    }
    /* core_fill_bond_order_storage (Core.f90:553-571): the per-atom factors of
       every group, once per evaluation */
    X->n_groups = 0;
    for (int r = 0; r < m->n_afac; ++r)
        if (m->afac_group[r] + 1 > X->n_groups) X->n_groups = m->afac_group[r] + 1;
    X->af_raw = NULL;
    X->af_fac = NULL;
    if (X->n_groups > 0) afac_sums(X);
}

static void free_ctx(ctx_t* X) {
    free(X->maxbr);
    free(X->smooth_soft);
    free(X->smoothened);
    free(X->af_raw);
    free(X->af_fac);
}

/* core_calculate_energy / forces / electronegativities, Core.f90:7910-7979,
 * driving core_loop_over_local_interactions, Core.f90:3249-4082. */
int orc_evaluate(const orc_system* s, const orc_model* m, const orc_nblist* nb, int what, int threads, double* energy,
                 double* forces, double* stress, double* enegs) {
    if (what < 0 || what > 2) return -1;
    if (threads < 1) threads = 1;
    if (threads > s->n && s->n > 0) threads = s->n;
    ctx_t X;
    setup_ctx(&X, s, m, nb);
    const int n = s->n;
    loop_job* jobs = (loop_job*)calloc((size_t)threads, sizeof(loop_job));
    for (int t = 0; t < threads; ++t) {
        jobs[t].X = &X;
        jobs[t].what = what;
        jobs[t].a0 = (int)((int64_t)n * t / threads);
        jobs[t].a1 = (int)((int64_t)n * (t + 1) / threads);
        if (what == 1) jobs[t].F = (double*)calloc(3 * (size_t)(n ? n : 1), sizeof(double));
        if (what == 2) jobs[t].chi = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
    }
    run_jobs(loop_range, jobs, sizeof(loop_job), threads);
    if (what == 0) {
        double e = 0.0;
        for (int t = 0; t < threads; ++t) e += jobs[t].energy;
        if (m->ewald) {
            double ek;
            ewald_kspace(&X, 0, threads, &ek, NULL, NULL, NULL);
            e = e + ek;
        }
        *energy = e;
    } else if (what == 1) {
        for (size_t c = 0; c < 3 * (size_t)n; ++c) {
            double v = 0.0;
            for (int t = 0; t < threads; ++t) v += jobs[t].F[c];
            forces[c] = v;
        }
        for (int c = 0; c < 6; ++c) {
            double v = 0.0;
            for (int t = 0; t < threads; ++t) v += jobs[t].stress[c];
            stress[c] = v;
        }
        if (m->ewald) {
            double* fk = (double*)calloc(3 * (size_t)(n ? n : 1), sizeof(double));
            double sk[6];
            ewald_kspace(&X, 1, threads, NULL, fk, sk, NULL);
            for (size_t c = 0; c < 3 * (size_t)n; ++c) forces[c] = forces[c] + fk[c];
            for (int c = 0; c < 6; ++c) stress[c] = stress[c] + sk[c];
            free(fk);
        }
    } else {
        for (int i = 0; i < n; ++i) {
            double v = 0.0;
            for (int t = 0; t < threads; ++t) v += jobs[t].chi[i];
            enegs[i] = v;
        }
        if (m->ewald) {
            double* ck = (double*)calloc((size_t)(n ? n : 1), sizeof(double));
            ewald_kspace(&X, 2, threads, NULL, NULL, NULL, ck);
            for (int i = 0; i < n; ++i) enegs[i] = enegs[i] + ck[i];
            free(ck);
        }
    }
    for (int t = 0; t < threads; ++t) {
        free(jobs[t].F);
        free(jobs[t].chi);
    }
    free(jobs);
    free_ctx(&X);
    return 0;
}

int orc_bond_zeta(const orc_system* s, const orc_model* m, const orc_nblist* nb, int group, double* zeta) {
    ctx_t X;
    setup_ctx(&X, s, m, nb);
    for (int i = 0; i < s->n; ++i)
        for (int e = nb->start[i]; e < nb->start[i + 1]; ++e) {
            const int j = nb->idx[e];
            double sep[3];
            separation(&X.C, s->pos + 3 * (size_t)i, s->pos + 3 * (size_t)j, nb->off + 3 * (size_t)e, sep);
            double d = sqrt(dot3(sep, sep));
            double sums[2];
            pair_bo_sums(&X, i, j, sep, d, group, sums);
            zeta[e] = sums[0];
        }
    free_ctx(&X);
    return 0;
}

int orc_atom_factors(const orc_system* s, const orc_model* m, const orc_nblist* nb, int group, double* raw,
                     double* factor) {
    ctx_t X;
    setup_ctx(&X, s, m, nb);
    for (int i = 0; i < s->n; ++i) {
        raw[i] = group < X.n_groups ? X.af_raw[(size_t)group * s->n + i] : 0.0;
        factor[i] = saved_factor(&X, group, i);
    }
    free_ctx(&X);
    return 0;
}

/* core_calculate_bond_order_gradients (Core.f90:1157-1644, two-target level-1
 * part) with core_post_process_bond_order_gradients (2842-2934): the gradient of
 * every atom's factor with respect to moving atom a (of_factor = 0), or, as
 * core_calculate_bond_order_gradients_of_factor (1979-1989) with
 * core_post_process_bond_order_gradients_of_factor (2972-3080), the gradient of
 * atom a's factor with respect to moving every atom (of_factor = 1).  Records of
 * a's element at position 1, over all of a's neighbours; out is n x 3. */
int orc_atom_factor_gradients(const orc_system* s, const orc_model* m, const orc_nblist* nb, int group, int a,
                              int of_factor, double* out) {
    if (a < 0 || a >= s->n) return -1;
    ctx_t X;
    setup_ctx(&X, s, m, nb);
    const int n = s->n;
    double* temp = (double*)calloc(3 * (size_t)(n ? n : 1), sizeof(double));
    const int ta = s->type[a];
    for (int e = nb->start[a]; e < nb->start[a + 1]; ++e) {
        const int j = nb->idx[e];
        double sep[3];
        separation(&X.C, s->pos + 3 * (size_t)a, s->pos + 3 * (size_t)j, nb->off + 3 * (size_t)e, sep);
        const double d = sqrt(dot3(sep, sep));
        if (!(d < X.maxbr[a])) continue;
        const int tj = s->type[j];
        for (int r = 0; r < m->n_afac; ++r) {
            if (!has(m->afac_mask1[r], ta) || m->afac_group[r] != group || !(m->afac_cutoff[r] > d)) continue;
            if (!has(m->afac_mask2[r], tj) || !afac_two_target(m->afac_kind[r])) continue;
            double g11[3], g12[3];
            afac_gradient(m, r, sep, d, g11, g12);
            for (int c = 0; c < 3; ++c) {
                temp[3 * (size_t)a + c] += g11[c];
                /* the factor is symmetric: the gradient of atom 2's term with
                   respect to atom 1 is g11, with respect to atom 2 it is g12 */
                temp[3 * (size_t)j + c] += of_factor ? g12[c] : g11[c];
            }
        }
    }
    for (int i = 0; i < n; ++i) {
        const int owner = of_factor ? a : i;
        const int post = afac_post_index(m, s->type[owner], group);
        const double raw = group < X.n_groups ? X.af_raw[(size_t)group * n + owner] : 0.0;
        for (int c = 0; c < 3; ++c)
            out[3 * (size_t)i + c] = post >= 0 ? afac_post_grad(m, post, raw, temp[3 * (size_t)i + c])
                                               : temp[3 * (size_t)i + c];
    }
    free(temp);
    free_ctx(&X);
    return 0;
}
