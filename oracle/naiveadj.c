/*
 * naiveadj.c -- CPU oracle (test infrastructure only) for the differentiable
 * form of the hot path: the FP64 kick-drift-kick trajectory of
 * src/Simulator.jl:154-256 (intended physics: truncated LJ + cutoff Coulomb of
 * src/Forces.jl, boundary_reflect! walls of src/Simulator.jl:81-111), a
 * Gaussian-smoothed pair-distance histogram of the final positions, and the
 * squared deviation of that histogram from a target.
 *
 * The reference has no derivative code; its differentiation story is
 * ForwardDiff over the Julia CPU path, which is not available here.  This file
 * is its stand-in: the same discrete program evaluated once in plain FP64 and
 * once in forward-mode dual numbers (value + 3 tangents: d/dsigma, d/depsilon
 * and a directional derivative along a given (dx0, dv0)), the way ForwardDiff
 * would propagate Dual numbers through it.  Branches (the cutoff test, the
 * wall clamps) are taken on values; a clamped coordinate has zero tangent and
 * a flipped velocity a negated tangent -- the derivative of the piecewise map.
 *
 * Histogram:  h_b = (1/N) sum_{i<j, r_ij < r_max} s(r_ij) exp(-(r_ij - c_b)^2 / (2 w^2))
 *   c_b = (b + 1/2) r_max / bins, w = smoothing width, s(r) = 1 below r_switch
 *   and 1 - t^3 (10 - 15 t + 6 t^2), t = (r - r_switch)/(r_max - r_switch),
 *   above it (a C2 switch to 0 at r_max, so the histogram is differentiable
 *   where pairs cross r_max).
 * Loss:       L = sum_b (h_b - target_b)^2.
 *
 * Events (for finite-difference checks): an order-free 128-bit sum of hashes
 * of every (step, i, j) pair inside the force cutoff and every (step, i, axis)
 * wall clamp.  Two runs with equal event sums took the same branches, so
 * their losses are one smooth function of the parameters between them.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "naiveref.h"

/* ------------------------------------------------------------ dual numbers */

#define NT 3
typedef struct {
    double v;
    double d[NT];
} dual;

static inline dual dc(double v) {
    dual r;
    r.v = v;
    for (int k = 0; k < NT; ++k) r.d[k] = 0.0;
    return r;
}
static inline dual dadd(dual a, dual b) {
    dual r;
    r.v = a.v + b.v;
    for (int k = 0; k < NT; ++k) r.d[k] = a.d[k] + b.d[k];
    return r;
}
static inline dual dsub(dual a, dual b) {
    dual r;
    r.v = a.v - b.v;
    for (int k = 0; k < NT; ++k) r.d[k] = a.d[k] - b.d[k];
    return r;
}
static inline dual dmul(dual a, dual b) {
    dual r;
    r.v = a.v * b.v;
    for (int k = 0; k < NT; ++k) r.d[k] = a.d[k] * b.v + a.v * b.d[k];
    return r;
}
static inline dual dscale(dual a, double s) {
    dual r;
    r.v = a.v * s;
    for (int k = 0; k < NT; ++k) r.d[k] = a.d[k] * s;
    return r;
}
static inline dual drecip(dual a) {
    dual r;
    r.v = 1.0 / a.v;
    const double g = -r.v * r.v;
    for (int k = 0; k < NT; ++k) r.d[k] = g * a.d[k];
    return r;
}
static inline dual dsqrt(dual a) {
    dual r;
    r.v = sqrt(a.v);
    const double g = 0.5 / r.v;
    for (int k = 0; k < NT; ++k) r.d[k] = g * a.d[k];
    return r;
}
static inline dual dexp(dual a) {
    dual r;
    r.v = exp(a.v);
    for (int k = 0; k < NT; ++k) r.d[k] = r.v * a.d[k];
    return r;
}

/* --------------------------------------------------------------- cell list */

typedef struct {
    int nc[3];
    double lo[3], cs[3];
    int32_t *head, *next, *cell;
} cells;

static int cells_build(cells* c, const double* xv, int32_t n, double rc) {
    for (int d = 0; d < 3; ++d) { c->lo[d] = INFINITY; }
    double hi[3] = {-INFINITY, -INFINITY, -INFINITY};
    for (int32_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) {
            if (xv[3 * i + d] < c->lo[d]) c->lo[d] = xv[3 * i + d];
            if (xv[3 * i + d] > hi[d]) hi[d] = xv[3 * i + d];
        }
    int64_t ncell = 1;
    for (int d = 0; d < 3; ++d) {
        double ext = hi[d] - c->lo[d];
        int k = (int)floor(ext / rc);
        if (k < 1) k = 1;
        if (k > 512) k = 512;
        c->nc[d] = k;
        c->cs[d] = ext > 0 ? ext / k : 1.0;
        ncell *= k;
    }
    c->head = (int32_t*)malloc(sizeof(int32_t) * (size_t)ncell);
    c->next = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    c->cell = (int32_t*)malloc(sizeof(int32_t) * (size_t)n);
    if (!c->head || !c->next || !c->cell) return -1;
    for (int64_t k = 0; k < ncell; ++k) c->head[k] = -1;
    for (int32_t i = n - 1; i >= 0; --i) {
        int ci[3];
        for (int d = 0; d < 3; ++d) {
            int k = (int)floor((xv[3 * i + d] - c->lo[d]) / c->cs[d]);
            if (k < 0) k = 0;
            if (k >= c->nc[d]) k = c->nc[d] - 1;
            ci[d] = k;
        }
        const int32_t id = (ci[2] * c->nc[1] + ci[1]) * c->nc[0] + ci[0];
        c->cell[i] = id;
        c->next[i] = c->head[id];
        c->head[id] = i;
    }
    return 0;
}

static void cells_free(cells* c) {
    free(c->head);
    free(c->next);
    free(c->cell);
}

/* Runs the body once for every unordered pair I < J in neighbouring cells. */
#define CELLS_FOR_PAIRS(c, n, I, J, ...)                                                    \
    for (int32_t I = 0; I < (n); ++I) {                                                     \
        const int32_t id_ = (c).cell[I];                                                    \
        const int cx_ = id_ % (c).nc[0], cy_ = (id_ / (c).nc[0]) % (c).nc[1],               \
                  cz_ = id_ / ((c).nc[0] * (c).nc[1]);                                      \
        for (int oz_ = -1; oz_ <= 1; ++oz_)                                                 \
            for (int oy_ = -1; oy_ <= 1; ++oy_)                                             \
                for (int ox_ = -1; ox_ <= 1; ++ox_) {                                       \
                    const int X_ = cx_ + ox_, Y_ = cy_ + oy_, Z_ = cz_ + oz_;               \
                    if (X_ < 0 || Y_ < 0 || Z_ < 0 || X_ >= (c).nc[0] || Y_ >= (c).nc[1] || \
                        Z_ >= (c).nc[2])                                                    \
                        continue;                                                           \
                    for (int32_t J = (c).head[(Z_ * (c).nc[1] + Y_) * (c).nc[0] + X_];      \
                         J >= 0; J = (c).next[J]) {                                         \
                        if (J <= I) continue;                                               \
                        __VA_ARGS__                                                         \
                    }                                                                       \
                }                                                                           \
    }

static inline uint64_t amix(uint64_t z) {
    z += 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

static inline void event(uint64_t ev[2], uint64_t a, uint64_t b) {
    const uint64_t x = amix(a * 0x9E3779B97F4A7C15ull ^ amix(b));
    ev[0] += x;
    ev[1] += amix(x ^ 0x5851F42D4C957F2Dull);
}

/* ----------------------------------------------------- the dual program */

typedef struct {
    const ref_md_params* p;
    const ref_adj_spec* s;
    int32_t n;
    dual sigma, eps;
} prog;

/* Forces (dual) over every pair inside the cutoff. */
static int forces_dual(const prog* P, const dual* x, const double* q, dual* f, int64_t step,
                       uint64_t ev[2]) {
    const int32_t n = P->n;
    double* xv = (double*)calloc(3 * (size_t)n, sizeof(double));
    if (!xv) return -1;
    for (int32_t k = 0; k < 3 * n; ++k) xv[k] = x[k].v;
    cells c = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, NULL, NULL, NULL};
    if (cells_build(&c, xv, n, P->p->cutoff)) { free(xv); cells_free(&c); return -1; }
    for (int32_t k = 0; k < 3 * n; ++k) f[k] = dc(0.0);
    const double rc2 = P->p->cutoff * P->p->cutoff;
    const dual sig2 = dmul(P->sigma, P->sigma);
    CELLS_FOR_PAIRS(c, n, i, j, {
        const double ex = xv[3 * i] - xv[3 * j], ey = xv[3 * i + 1] - xv[3 * j + 1],
                     ez = xv[3 * i + 2] - xv[3 * j + 2];
        if (!(ex * ex + ey * ey + ez * ez < rc2)) continue;
        if (ev) event(ev, (uint64_t)step, ((uint64_t)i << 32) | (uint64_t)j);
        const dual dx = dsub(x[3 * i], x[3 * j]);
        const dual dy = dsub(x[3 * i + 1], x[3 * j + 1]);
        const dual dz = dsub(x[3 * i + 2], x[3 * j + 2]);
        const dual r2 = dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz));
        const dual inv_r2 = drecip(r2);
        const dual s2 = dmul(sig2, inv_r2);
        const dual s6 = dmul(dmul(s2, s2), s2);
        dual fmag = dmul(dscale(P->eps, 24.0),
                         dmul(inv_r2, dsub(dscale(dmul(s6, s6), 2.0), s6)));
        if (P->p->coulomb_k != 0.0 && q) {
            const dual inv_r = drecip(dsqrt(r2));
            fmag = dadd(fmag, dscale(dmul(inv_r, inv_r2), P->p->coulomb_k * q[i] * q[j]));
        }
        const dual fx = dmul(fmag, dx), fy = dmul(fmag, dy), fz = dmul(fmag, dz);
        f[3 * i] = dadd(f[3 * i], fx);
        f[3 * i + 1] = dadd(f[3 * i + 1], fy);
        f[3 * i + 2] = dadd(f[3 * i + 2], fz);
        f[3 * j] = dsub(f[3 * j], fx);
        f[3 * j + 1] = dsub(f[3 * j + 1], fy);
        f[3 * j + 2] = dsub(f[3 * j + 2], fz);
    });
    cells_free(&c);
    free(xv);
    return 0;
}

/* Smoothed histogram (dual) of the pair distances of x. */
static int hist_dual(const prog* P, const dual* x, dual* h) {
    const int32_t n = P->n;
    const ref_adj_spec* s = P->s;
    double* xv = (double*)calloc(3 * (size_t)n, sizeof(double));
    if (!xv) return -1;
    for (int32_t k = 0; k < 3 * n; ++k) xv[k] = x[k].v;
    cells c = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, NULL, NULL, NULL};
    if (cells_build(&c, xv, n, s->r_max)) { free(xv); cells_free(&c); return -1; }
    for (int b = 0; b < s->bins; ++b) h[b] = dc(0.0);
    const double rm2 = s->r_max * s->r_max;
    const double bw = s->r_max / s->bins;
    const double inv2w2 = 1.0 / (2.0 * s->width * s->width);
    const double rs = s->r_switch, span = s->r_max - s->r_switch;
    CELLS_FOR_PAIRS(c, n, i, j, {
        const double ex = xv[3 * i] - xv[3 * j], ey = xv[3 * i + 1] - xv[3 * j + 1],
                     ez = xv[3 * i + 2] - xv[3 * j + 2];
        if (!(ex * ex + ey * ey + ez * ez < rm2)) continue;
        const dual dx = dsub(x[3 * i], x[3 * j]);
        const dual dy = dsub(x[3 * i + 1], x[3 * j + 1]);
        const dual dz = dsub(x[3 * i + 2], x[3 * j + 2]);
        const dual r = dsqrt(dadd(dadd(dmul(dx, dx), dmul(dy, dy)), dmul(dz, dz)));
        dual sw = dc(1.0);
        if (r.v > rs) {
            const dual t = dscale(dsub(r, dc(rs)), 1.0 / span);
            const dual t3 = dmul(dmul(t, t), t);
            const dual poly = dadd(dsub(dc(10.0), dscale(t, 15.0)), dscale(dmul(t, t), 6.0));
            sw = dsub(dc(1.0), dmul(t3, poly));
        }
        for (int b = 0; b < s->bins; ++b) {
            const dual u = dsub(r, dc((b + 0.5) * bw));
            h[b] = dadd(h[b], dmul(sw, dexp(dscale(dmul(u, u), -inv2w2))));
        }
    });
    for (int b = 0; b < s->bins; ++b) h[b] = dscale(h[b], 1.0 / n);
    cells_free(&c);
    free(xv);
    return 0;
}

/*
 * The whole program in dual numbers.  Returns REF_OK or a negative status.
 */
int ref_adj_dual(const ref_md_params* p, const ref_adj_spec* s, int32_t n, const double* x0,
                 const double* v0, const double* q, const double* m, const double* dx0,
                 const double* dv0, const double* target, double* hist, double* loss,
                 double dloss[3], double* x_out, double* v_out, uint64_t events[2]) {
    if (!p || !s || n <= 1 || !x0 || !v0 || s->bins <= 0 || !(s->width > 0) ||
        !(s->r_max > 0) || !(s->r_switch <= s->r_max))
        return REF_ERR_ARG;
    prog P = {p, s, n, dc(p->sigma), dc(p->epsilon)};
    P.sigma.d[0] = 1.0;
    P.eps.d[1] = 1.0;
    dual* x = (dual*)malloc(sizeof(dual) * 3 * (size_t)n);
    dual* v = (dual*)malloc(sizeof(dual) * 3 * (size_t)n);
    dual* f = (dual*)malloc(sizeof(dual) * 3 * (size_t)n);
    dual* h = (dual*)malloc(sizeof(dual) * (size_t)s->bins);
    if (!x || !v || !f || !h) { free(x); free(v); free(f); free(h); return REF_ERR_NOMEM; }
    for (int32_t k = 0; k < 3 * n; ++k) {
        x[k] = dc(x0[k]);
        v[k] = dc(v0[k]);
        x[k].d[2] = dx0 ? dx0[k] : 0.0;
        v[k].d[2] = dv0 ? dv0[k] : 0.0;
    }
    uint64_t ev[2] = {0, 0};
    int rc = REF_OK;
    const double hdt = 0.5 * p->dt;
    if (forces_dual(&P, x, q, f, 0, ev)) rc = REF_ERR_NOMEM;
    for (int64_t st = 0; st < s->steps && rc == REF_OK; ++st) {
        for (int32_t i = 0; i < n; ++i) {
            const double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) {
                const int32_t k = 3 * i + d;
                v[k] = dadd(v[k], dscale(f[k], hdt * im));
                x[k] = dadd(x[k], dscale(v[k], p->dt));
                /* boundary_reflect! (Simulator.jl:81-111) */
                if (p->box_lo[d] > x[k].v) {
                    v[k] = dscale(v[k], -1.0);
                    x[k] = dc(p->box_lo[d]);
                    event(ev, (uint64_t)st | (1ull << 62), (uint64_t)k);
                }
                if (p->box_hi[d] < x[k].v) {
                    v[k] = dscale(v[k], -1.0);
                    x[k] = dc(p->box_hi[d]);
                    event(ev, (uint64_t)st | (1ull << 62), (uint64_t)k);
                }
            }
        }
        if (forces_dual(&P, x, q, f, st + 1, ev)) { rc = REF_ERR_NOMEM; break; }
        for (int32_t i = 0; i < n; ++i) {
            const double im = m ? 1.0 / m[i] : 1.0;
            for (int d = 0; d < 3; ++d) v[3 * i + d] = dadd(v[3 * i + d], dscale(f[3 * i + d], hdt * im));
        }
    }
    if (rc == REF_OK && hist_dual(&P, x, h)) rc = REF_ERR_NOMEM;
    if (rc == REF_OK) {
        dual L = dc(0.0);
        for (int b = 0; b < s->bins; ++b) {
            if (hist) hist[b] = h[b].v;
            const dual e = dsub(h[b], dc(target ? target[b] : 0.0));
            L = dadd(L, dmul(e, e));
        }
        if (loss) *loss = L.v;
        if (dloss)
            for (int k = 0; k < NT; ++k) dloss[k] = L.d[k];
        for (int32_t k = 0; k < 3 * n; ++k) {
            if (x_out) x_out[k] = x[k].v;
            if (v_out) v_out[k] = v[k].v;
        }
        if (events) { events[0] = ev[0]; events[1] = ev[1]; }
    }
    free(x); free(v); free(f); free(h);
    return rc;
}
