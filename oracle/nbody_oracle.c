/*
 * nbody_oracle.c -- CPU oracle for the GB300 FMM step.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product links this file: it is
 * loaded by tests/, by __graft_entry__.smoke() as the checker, and by
 * bench.py for the timed CPU baseline.  It is plain, serial (or simply
 * threaded) C written for clarity, not speed.
 *
 * Contents
 *   1. Morton keys on a 21-bit-per-axis grid of the root box, stable sort.
 *   2. Bucket octree (capacity C, depth cap 21), breadth-first node order,
 *      non-empty children only.  This restates the semantics the reference
 *      relies on from its external octree: node_t (min corner + extent,
 *      contiguous leaf ranges per subtree, include/nbody/device/types.h:116-141)
 *      and the capacity/depth rule (src/open_cl_simulation.cpp:41-47,280-283).
 *      Conventions that the reference leaves to the absent octree library are
 *      fixed here: child k = octant bits with x = bit 0, upper child when the
 *      coordinate is >= the split plane, depth cap 21.
 *   3. Dual-tree interaction finding.  Restates src/interaction.cl:10-100
 *      (split both cells, MAC 3/4 (wA+wB)^2 / d^2 < theta^2 on geometric
 *      centres, A != B for approximation, empty children dropped) and the host
 *      classification of src/open_cl_simulation.cpp:247-266
 *      (reducible -> refine, !approx -> leaf pair, approx -> node pair).
 *      Lists are produced per target cell (both orientations of every pair).
 *   4. Cartesian order-p FMM in FP64 about geometric cell centres with the
 *      Plummer-softened kernel 1/sqrt(r^2+eps^2).  Order 1 is the reference's
 *      own expansion: monopole source (src/moment.cl:43, src/field.cl:34-47)
 *      and a constant local field copied to every particle of the target
 *      subtree (src/field.cl:203-210).
 *   5. The reference order-0 FMM restated in FP32 arithmetic following
 *      src/field.cl:17-47 (pair and node fields), src/force.cl:21-81
 *      (F = q * sum of fields) and src/open_cl_simulation.cpp:600-607
 *      (explicit Euler: v += F/m dt, x += v_old dt), with four bugs of the
 *      reference's host code fixed (M2M runs, interaction slots are distinct,
 *      the leaf partition covers every leaf, every batch is integrated).
 *   6. FP64 softened direct sum (forces and potential) and its adjoint.
 *   7. A port of src/naive_simulation.cpp:7-46 (the reference CPU path), with
 *      its delta[1]=delta[2]=x bug reproduced by default (switchable), used
 *      as the timed CPU baseline.
 */
#include <math.h>
#include <pthread.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define ORC_LEVELS 21          /* bits per axis; deepest level index */
#define ORC_PMAX 10
#define ORC_TMAX ((ORC_PMAX + 1) * (ORC_PMAX + 2) * (ORC_PMAX + 3) / 6)

/* ------------------------------------------------------------------ */
/* multi-index tables (total-degree order, nx descending, ny descending) */
/* ------------------------------------------------------------------ */
static int mi_nx[ORC_TMAX], mi_ny[ORC_TMAX], mi_nz[ORC_TMAX];
static double fact[32];
static int mi_ready = 0;

static int nterms(int p) { return (p + 1) * (p + 2) * (p + 3) / 6; }

static int mi_idx(int nx, int ny, int nz) {
    int d = nx + ny + nz;
    int s = ny + nz;
    return d * (d + 1) * (d + 2) / 6 + s * (s + 1) / 2 + nz;
}

static void mi_init(void) {
    if (mi_ready) return;
    for (int d = 0; d <= ORC_PMAX; ++d)
        for (int nx = d; nx >= 0; --nx)
            for (int ny = d - nx; ny >= 0; --ny) {
                int nz = d - nx - ny;
                int k = mi_idx(nx, ny, nz);
                mi_nx[k] = nx; mi_ny[k] = ny; mi_nz[k] = nz;
            }
    fact[0] = 1.0;
    for (int i = 1; i < 32; ++i) fact[i] = fact[i - 1] * i;
    mi_ready = 1;
}

int orc_term_index(int nx, int ny, int nz) { return mi_idx(nx, ny, nz); }
int orc_nterms(int p) { return nterms(p); }

/* monomials y^n / n! for |n| <= p */
static void monomials(int p, const double y[3], double* out) {
    int T = nterms(p);
    out[0] = 1.0;
    for (int k = 1; k < T; ++k) {
        int nx = mi_nx[k], ny = mi_ny[k], nz = mi_nz[k];
        if (nx > 0) out[k] = out[mi_idx(nx - 1, ny, nz)] * y[0] / nx;
        else if (ny > 0) out[k] = out[mi_idx(nx, ny - 1, nz)] * y[1] / ny;
        else out[k] = out[mi_idx(nx, ny, nz - 1)] * y[2] / nz;
    }
}

/* D_n(r) = d^n/dr^n (|r|^2+eps^2)^(-1/2) for |n| <= p (Hermite recursion) */
static void derivs(int p, const double r[3], double eps2, double* D) {
    static __thread double R[ORC_PMAX + 1][ORC_TMAX];
    double s = r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + eps2;
    double inv = 1.0 / sqrt(s), inv2 = 1.0 / s;
    double F = inv;
    for (int m = 0; m <= p; ++m) {
        R[m][0] = F;
        F *= -(2.0 * m + 1.0) * inv2;
    }
    for (int m = p - 1; m >= 0; --m) {
        int T = nterms(p - m);
        for (int k = 1; k < T; ++k) {
            int nx = mi_nx[k], ny = mi_ny[k], nz = mi_nz[k];
            double v;
            if (nx > 0) {
                v = r[0] * R[m + 1][mi_idx(nx - 1, ny, nz)];
                if (nx > 1) v += (nx - 1) * R[m + 1][mi_idx(nx - 2, ny, nz)];
            } else if (ny > 0) {
                v = r[1] * R[m + 1][mi_idx(nx, ny - 1, nz)];
                if (ny > 1) v += (ny - 1) * R[m + 1][mi_idx(nx, ny - 2, nz)];
            } else {
                v = r[2] * R[m + 1][mi_idx(nx, ny, nz - 1)];
                if (nz > 1) v += (nz - 1) * R[m + 1][mi_idx(nx, ny, nz - 2)];
            }
            R[m][k] = v;
        }
    }
    memcpy(D, R[0], sizeof(double) * nterms(p));
}

void orc_derivs(int p, const double* r, double eps2, double* D) { mi_init(); derivs(p, r, eps2, D); }

/* ------------------------------------------------------------------ */
/* Morton keys                                                          */
/* ------------------------------------------------------------------ */
static uint32_t quantize(double x, double origin, double scale) {
    double q = (x - origin) * scale;       /* scale = 2^21 / side */
    if (!(q >= 0.0)) return 0;
    if (q >= 2097151.0) return 2097151u;
    return (uint32_t)q;
}

static uint64_t interleave(uint32_t ix, uint32_t iy, uint32_t iz) {
    uint64_t k = 0;
    for (int b = 0; b < ORC_LEVELS; ++b) {
        k |= (uint64_t)((ix >> b) & 1u) << (3 * b);
        k |= (uint64_t)((iy >> b) & 1u) << (3 * b + 1);
        k |= (uint64_t)((iz >> b) & 1u) << (3 * b + 2);
    }
    return k;
}

void orc_morton_keys(int64_t n, const double* pos, const double* box, uint64_t* keys) {
    double scale = 2097152.0 / box[3];
    for (int64_t i = 0; i < n; ++i)
        keys[i] = interleave(quantize(pos[3 * i], box[0], scale),
                             quantize(pos[3 * i + 1], box[1], scale),
                             quantize(pos[3 * i + 2], box[2], scale));
}

/* stable sort of keys: returns perm with keys[perm] non-decreasing, ties by index */
static const uint64_t* g_sort_keys;
static int cmp_perm(const void* a, const void* b) {
    uint32_t i = *(const uint32_t*)a, j = *(const uint32_t*)b;
    uint64_t ki = g_sort_keys[i], kj = g_sort_keys[j];
    if (ki < kj) return -1;
    if (ki > kj) return 1;
    return (i > j) - (i < j);
}
void orc_sort_keys(int64_t n, const uint64_t* keys, uint32_t* perm) {
    for (int64_t i = 0; i < n; ++i) perm[i] = (uint32_t)i;
    g_sort_keys = keys;
    qsort(perm, (size_t)n, sizeof(uint32_t), cmp_perm);
}

/* ------------------------------------------------------------------ */
/* context: sorted particles + octree + lists + expansions              */
/* ------------------------------------------------------------------ */
typedef struct {
    int32_t* a; int64_t n, cap;
} ivec;
static void iv_push(ivec* v, int32_t x) {
    if (v->n == v->cap) { v->cap = v->cap ? 2 * v->cap : 16; v->a = (int32_t*)realloc(v->a, sizeof(int32_t) * v->cap); }
    v->a[v->n++] = x;
}

typedef struct orc_ctx {
    int64_t n;
    double box[4];
    int cap, maxlevel;
    uint32_t* perm;      /* sorted position -> input index */
    uint64_t* keys;      /* sorted keys */
    double* pos;         /* sorted positions (3n) */
    double* q;           /* sorted charges */
    double* m;           /* sorted masses */
    /* nodes, breadth-first */
    int64_t nnodes, nnodes_cap;
    int32_t *level, *ix, *iy, *iz, *begin, *count, *parent, *child_begin, *nchild;
    int depth;
    int64_t level_start[ORC_LEVELS + 2];
    /* per-target lists */
    ivec *m2l, *p2p, *pend;
    int lists_ready;
} orc_ctx;

static void node_grow(orc_ctx* c) {
    if (c->nnodes < c->nnodes_cap) return;
    c->nnodes_cap = c->nnodes_cap ? 2 * c->nnodes_cap : 1024;
    size_t b = sizeof(int32_t) * c->nnodes_cap;
    c->level = realloc(c->level, b); c->ix = realloc(c->ix, b); c->iy = realloc(c->iy, b);
    c->iz = realloc(c->iz, b); c->begin = realloc(c->begin, b); c->count = realloc(c->count, b);
    c->parent = realloc(c->parent, b); c->child_begin = realloc(c->child_begin, b);
    c->nchild = realloc(c->nchild, b);
}

static int64_t add_node(orc_ctx* c, int lev, int x, int y, int z, int b, int cnt, int par) {
    node_grow(c);
    int64_t k = c->nnodes++;
    c->level[k] = lev; c->ix[k] = x; c->iy[k] = y; c->iz[k] = z;
    c->begin[k] = b; c->count[k] = cnt; c->parent[k] = par;
    c->child_begin[k] = -1; c->nchild[k] = 0;
    return k;
}

static int is_leaf(const orc_ctx* c, int64_t k) { return c->nchild[k] == 0; }

/* box = {origin x, y, z, side} */
orc_ctx* orc_create(int64_t n, const double* pos, const double* q, const double* m,
                    const double* box, int cap, int maxlevel) {
    mi_init();
    orc_ctx* c = (orc_ctx*)calloc(1, sizeof(orc_ctx));
    c->n = n; memcpy(c->box, box, sizeof(double) * 4);
    c->cap = cap; c->maxlevel = maxlevel > ORC_LEVELS ? ORC_LEVELS : maxlevel;
    uint64_t* k0 = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    orc_morton_keys(n, pos, box, k0);
    c->perm = (uint32_t*)malloc(sizeof(uint32_t) * (n ? n : 1));
    orc_sort_keys(n, k0, c->perm);
    c->keys = (uint64_t*)malloc(sizeof(uint64_t) * (n ? n : 1));
    c->pos = (double*)malloc(sizeof(double) * 3 * (n ? n : 1));
    c->q = (double*)malloc(sizeof(double) * (n ? n : 1));
    c->m = (double*)malloc(sizeof(double) * (n ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        uint32_t j = c->perm[i];
        c->keys[i] = k0[j];
        memcpy(c->pos + 3 * i, pos + 3 * (int64_t)j, sizeof(double) * 3);
        c->q[i] = q ? q[j] : 1.0;
        c->m[i] = m ? m[j] : 1.0;
    }
    free(k0);
    /* breadth-first build */
    add_node(c, 0, 0, 0, 0, 0, (int)n, -1);
    c->level_start[0] = 0;
    int lev = 0;
    int64_t lo = 0, hi = 1;
    c->depth = 0;
    while (lo < hi) {
        c->level_start[lev] = lo;
        c->depth = lev;
        for (int64_t k = lo; k < hi; ++k) {
            if (c->count[k] > cap && lev < c->maxlevel) {
                int shift = 3 * (ORC_LEVELS - 1 - lev);
                int b = c->begin[k], e = b + c->count[k];
                int first = 1;
                int i = b;
                for (int d = 0; d < 8; ++d) {
                    int j = i;
                    while (j < e && (int)((c->keys[j] >> shift) & 7u) == d) ++j;
                    if (j > i) {
                        int64_t ch = add_node(c, lev + 1, 2 * c->ix[k] + (d & 1), 2 * c->iy[k] + ((d >> 1) & 1),
                                              2 * c->iz[k] + (d >> 2), i, j - i, (int)k);
                        if (first) { c->child_begin[k] = (int32_t)ch; first = 0; }
                        c->nchild[k]++;
                    }
                    i = j;
                }
            }
        }
        lo = hi; hi = c->nnodes; ++lev;
    }
    for (int l = c->depth + 1; l < ORC_LEVELS + 2; ++l) c->level_start[l] = c->nnodes;
    return c;
}

void orc_destroy(orc_ctx* c) {
    if (!c) return;
    free(c->perm); free(c->keys); free(c->pos); free(c->q); free(c->m);
    free(c->level); free(c->ix); free(c->iy); free(c->iz); free(c->begin); free(c->count);
    free(c->parent); free(c->child_begin); free(c->nchild);
    if (c->m2l) {
        for (int64_t k = 0; k < c->nnodes; ++k) { free(c->m2l[k].a); free(c->p2p[k].a); free(c->pend[k].a); }
        free(c->m2l); free(c->p2p); free(c->pend);
    }
    free(c);
}

/* Replaces the particles' positions, charges and masses (input order; NULL
   keeps the current values) while the tree and the interaction lists stay as
   built: evaluations after this are the FMM with a frozen tree, whose
   finite differences give the derivative the adjoint computes. */
void orc_set_particles(orc_ctx* c, const double* pos, const double* q, const double* m) {
    for (int64_t i = 0; i < c->n; ++i) {
        uint32_t j = c->perm[i];
        if (pos) memcpy(c->pos + 3 * i, pos + 3 * (int64_t)j, sizeof(double) * 3);
        if (q) c->q[i] = q[j];
        if (m) c->m[i] = m[j];
    }
}

int64_t orc_nnodes(const orc_ctx* c) { return c->nnodes; }
int orc_depth(const orc_ctx* c) { return c->depth; }

void orc_get_order(const orc_ctx* c, uint32_t* perm, uint64_t* keys) {
    if (perm) memcpy(perm, c->perm, sizeof(uint32_t) * c->n);
    if (keys) memcpy(keys, c->keys, sizeof(uint64_t) * c->n);
}

/* nodes as int32 rows: level, ix, iy, iz, begin, count, parent, child_begin, nchild */
void orc_get_nodes(const orc_ctx* c, int32_t* out) {
    for (int64_t k = 0; k < c->nnodes; ++k) {
        int32_t* r = out + 9 * k;
        r[0] = c->level[k]; r[1] = c->ix[k]; r[2] = c->iy[k]; r[3] = c->iz[k];
        r[4] = c->begin[k]; r[5] = c->count[k]; r[6] = c->parent[k];
        r[7] = c->child_begin[k]; r[8] = c->nchild[k];
    }
}

/* geometry in fine units (side / 2^22) */
static void centre_fine(const orc_ctx* c, int64_t k, int64_t out[3]) {
    int sh = ORC_LEVELS - c->level[k];
    out[0] = ((int64_t)2 * c->ix[k] + 1) << sh;
    out[1] = ((int64_t)2 * c->iy[k] + 1) << sh;
    out[2] = ((int64_t)2 * c->iz[k] + 1) << sh;
}
static int64_t width_fine(const orc_ctx* c, int64_t k) { return (int64_t)1 << (ORC_LEVELS + 1 - c->level[k]); }

static void centre(const orc_ctx* c, int64_t k, double out[3]) {
    double w = c->box[3] / (double)(1 << c->level[k]);
    out[0] = c->box[0] + (c->ix[k] + 0.5) * w;
    out[1] = c->box[1] + (c->iy[k] + 0.5) * w;
    out[2] = c->box[2] + (c->iz[k] + 0.5) * w;
}
/* exact displacement c_a - c_b in FP64 (dyadic, computed from integer coordinates) */
static void displacement(const orc_ctx* c, int64_t a, int64_t b, double out[3]) {
    int64_t ca[3], cb[3];
    centre_fine(c, a, ca); centre_fine(c, b, cb);
    double u = c->box[3] / 4194304.0;
    for (int d = 0; d < 3; ++d) out[d] = (double)(ca[d] - cb[d]) * u;
}

/* src/interaction.cl:64-79 in its own FP32 operation order: approx iff A != B
   and extent^2 / distance^2 < theta^2 with distance^2 = ((x*x + y*y) + z*z) + 0
   and extent^2 = (0.75 * (wA+wB)) * (wA+wB), all single precision.  Lengths are
   in fine units (side / 2^22), a power-of-two rescaling of the reference's box
   units, which leaves every rounding unchanged.  Compiled without FMA
   contraction (oracle/Makefile). */
static int mac_accept(const orc_ctx* c, int64_t t, int64_t s, double theta2) {
    if (t == s) return 0;
    int64_t ct[3], cs[3];
    centre_fine(c, t, ct); centre_fine(c, s, cs);
    float dx = (float)(cs[0] - ct[0]), dy = (float)(cs[1] - ct[1]), dz = (float)(cs[2] - ct[2]);
    float d2 = ((dx * dx + dy * dy) + dz * dz) + 0.0f;
    float es = (float)(width_fine(c, t) + width_fine(c, s));
    float e2 = (0.75f * es) * es;
    return e2 / d2 < (float)theta2;
}

/* theta2 is passed as (double)((float)theta * (float)theta), the value the
   reference computes in FP32 (src/interaction.cl:78). */
int orc_traverse(orc_ctx* c, double theta2) {
    int64_t nn = c->nnodes;
    if (c->m2l) {
        for (int64_t k = 0; k < nn; ++k) { free(c->m2l[k].a); free(c->p2p[k].a); free(c->pend[k].a); }
        free(c->m2l); free(c->p2p); free(c->pend);
    }
    c->m2l = (ivec*)calloc(nn, sizeof(ivec));
    c->p2p = (ivec*)calloc(nn, sizeof(ivec));
    c->pend = (ivec*)calloc(nn, sizeof(ivec));
    if (c->n == 0) { c->lists_ready = 1; return 0; }
    if (is_leaf(c, 0)) iv_push(&c->p2p[0], 0);
    else iv_push(&c->pend[0], 0);
    ivec queue = {0, 0, 0};
    for (int64_t t = 1; t < nn; ++t) {
        int64_t par = c->parent[t];
        queue.n = 0;
        for (int64_t i = 0; i < c->pend[par].n; ++i) {
            int32_t s = c->pend[par].a[i];
            if (is_leaf(c, s)) iv_push(&queue, s);
            else for (int j = 0; j < c->nchild[s]; ++j) iv_push(&queue, c->child_begin[s] + j);
        }
        for (int64_t h = 0; h < queue.n; ++h) {
            int32_t s = queue.a[h];
            if (mac_accept(c, t, s, theta2)) iv_push(&c->m2l[t], s);
            else if (is_leaf(c, t) && is_leaf(c, s)) iv_push(&c->p2p[t], s);
            else if (!is_leaf(c, t)) iv_push(&c->pend[t], s);
            else for (int j = 0; j < c->nchild[s]; ++j) iv_push(&queue, c->child_begin[s] + j);
        }
    }
    free(queue.a);
    c->lists_ready = 1;
    return 0;
}

/* which: 0 = M2L, 1 = P2P, 2 = pending (refinement) */
int64_t orc_list_size(const orc_ctx* c, int which) {
    const ivec* v = which == 0 ? c->m2l : which == 1 ? c->p2p : c->pend;
    int64_t s = 0;
    for (int64_t k = 0; k < c->nnodes; ++k) s += v[k].n;
    return s;
}
void orc_get_list(const orc_ctx* c, int which, int32_t* pairs) {
    const ivec* v = which == 0 ? c->m2l : which == 1 ? c->p2p : c->pend;
    int64_t o = 0;
    for (int64_t k = 0; k < c->nnodes; ++k)
        for (int64_t i = 0; i < v[k].n; ++i) { pairs[2 * o] = (int32_t)k; pairs[2 * o + 1] = v[k].a[i]; ++o; }
}

/* ------------------------------------------------------------------ */
/* order-p FMM in FP64                                                  */
/* ------------------------------------------------------------------ */
/* acc (3n) and pot (n) are written in INPUT order.  acc = (q_i/m_i) G E(x_i),
   pot = -G psi(x_i) (potential per unit charge, self term excluded).
   Expansions (nnodes x T) are returned if M_out/L_out are non-null. */
int orc_fmm(orc_ctx* c, int p, double eps, double G, double* acc, double* pot, double* M_out, double* L_out) {
    if (!c->lists_ready || p < 1 || p > ORC_PMAX) return -1;
    int64_t nn = c->nnodes;
    int T = nterms(p);
    double eps2 = eps * eps;
    double* M = (double*)calloc((size_t)nn * T, sizeof(double));
    double* L = (double*)calloc((size_t)nn * T, sizeof(double));
    double mono[ORC_TMAX], D[ORC_TMAX];
    /* P2M at leaves */
    for (int64_t k = 0; k < nn; ++k) {
        if (!is_leaf(c, k)) continue;
        double ck[3]; centre(c, k, ck);
        for (int i = c->begin[k]; i < c->begin[k] + c->count[k]; ++i) {
            double y[3] = {c->pos[3 * i] - ck[0], c->pos[3 * i + 1] - ck[1], c->pos[3 * i + 2] - ck[2]};
            monomials(p, y, mono);
            for (int a = 0; a < T; ++a) M[k * T + a] += c->q[i] * mono[a];
        }
    }
    /* M2M, deepest level first */
    for (int64_t k = nn - 1; k >= 0; --k) {
        if (is_leaf(c, k)) continue;
        for (int j = 0; j < c->nchild[k]; ++j) {
            int64_t ch = c->child_begin[k] + j;
            double d[3]; displacement(c, ch, k, d);
            monomials(p, d, mono);
            for (int a = 0; a < T; ++a) {
                double s = 0;
                for (int b = 0; b <= a; ++b) {
                    int ex = mi_nx[a] - mi_nx[b], ey = mi_ny[a] - mi_ny[b], ez = mi_nz[a] - mi_nz[b];
                    if (ex < 0 || ey < 0 || ez < 0) continue;
                    s += M[ch * T + b] * mono[mi_idx(ex, ey, ez)];
                }
                M[k * T + a] += s;
            }
        }
    }
    /* M2L */
    for (int64_t t = 0; t < nn; ++t) {
        for (int64_t i = 0; i < c->m2l[t].n; ++i) {
            int64_t s = c->m2l[t].a[i];
            double r[3]; displacement(c, t, s, r);
            derivs(p, r, eps2, D);
            for (int a = 0; a < T; ++a) {
                double acc_ = 0;
                int da = mi_nx[a] + mi_ny[a] + mi_nz[a];
                for (int b = 0; b < nterms(p - da); ++b) {
                    int db = mi_nx[b] + mi_ny[b] + mi_nz[b];
                    double sg = (db & 1) ? -1.0 : 1.0;
                    acc_ += sg * M[s * T + b] * D[mi_idx(mi_nx[a] + mi_nx[b], mi_ny[a] + mi_ny[b], mi_nz[a] + mi_nz[b])];
                }
                L[t * T + a] += acc_;
            }
        }
    }
    /* L2L, root first */
    for (int64_t k = 1; k < nn; ++k) {
        int64_t par = c->parent[k];
        double d[3]; displacement(c, k, par, d);
        monomials(p, d, mono);
        for (int a = 0; a < T; ++a) {
            int da = mi_nx[a] + mi_ny[a] + mi_nz[a];
            double s = 0;
            for (int b = 0; b < nterms(p - da); ++b)
                s += L[par * T + mi_idx(mi_nx[a] + mi_nx[b], mi_ny[a] + mi_ny[b], mi_nz[a] + mi_nz[b])] * mono[b];
            L[k * T + a] += s;
        }
    }
    /* L2P + P2P */
    for (int64_t t = 0; t < nn; ++t) {
        if (!is_leaf(c, t)) continue;
        double ct[3]; centre(c, t, ct);
        for (int i = c->begin[t]; i < c->begin[t] + c->count[t]; ++i) {
            double xi = c->pos[3 * i], yi = c->pos[3 * i + 1], zi = c->pos[3 * i + 2];
            double y[3] = {xi - ct[0], yi - ct[1], zi - ct[2]};
            monomials(p - 1 >= 0 ? p : 0, y, mono);
            double E[3] = {0, 0, 0}, psi = 0;
            for (int a = 0; a < T; ++a) psi += L[t * T + a] * mono[a];
            for (int a = 0; a < nterms(p - 1); ++a) {
                E[0] += L[t * T + mi_idx(mi_nx[a] + 1, mi_ny[a], mi_nz[a])] * mono[a];
                E[1] += L[t * T + mi_idx(mi_nx[a], mi_ny[a] + 1, mi_nz[a])] * mono[a];
                E[2] += L[t * T + mi_idx(mi_nx[a], mi_ny[a], mi_nz[a] + 1)] * mono[a];
            }
            for (int64_t li = 0; li < c->p2p[t].n; ++li) {
                int64_t s = c->p2p[t].a[li];
                for (int j = c->begin[s]; j < c->begin[s] + c->count[s]; ++j) {
                    if (j == i) continue;
                    double dx = c->pos[3 * j] - xi, dy = c->pos[3 * j + 1] - yi, dz = c->pos[3 * j + 2] - zi;
                    double s2 = dx * dx + dy * dy + dz * dz + eps2;
                    if (s2 == 0.0) continue;
                    double inv = 1.0 / sqrt(s2);
                    double inv3 = inv * inv * inv;
                    E[0] += c->q[j] * dx * inv3; E[1] += c->q[j] * dy * inv3; E[2] += c->q[j] * dz * inv3;
                    psi += c->q[j] * inv;
                }
            }
            uint32_t o = c->perm[i];
            double f = G * c->q[i] / c->m[i];
            if (acc) { acc[3 * o] = f * E[0]; acc[3 * o + 1] = f * E[1]; acc[3 * o + 2] = f * E[2]; }
            if (pot) pot[o] = -G * psi;
        }
    }
    if (M_out) memcpy(M_out, M, sizeof(double) * nn * T);
    if (L_out) memcpy(L_out, L, sizeof(double) * nn * T);
    free(M); free(L);
    return 0;
}

/* ------------------------------------------------------------------ */
/* reference order-0 FMM restated in FP32                               */
/* ------------------------------------------------------------------ */
/* Per particle (INPUT order) returns the two force sums the reference keeps
   apart: leaf (P2P) force and node (M2L) force, F = q * sum(field) with
   field from src/field.cl:17-47 and FORCE_CONSTANT = -1, PARTICLE_RADIUS = eps.
   Node moments: monopole about the geometric centre (src/moment.cl:27,43),
   summed up the tree (the intended M2M of src/moment.cl:129-150). */
static void f_centre(const orc_ctx* c, int64_t k, float out[3]) {
    /* position + dimensions / 2 in FP32 (src/field.cl:190-191) */
    double w = c->box[3] / (double)(1 << c->level[k]);
    float px = (float)(c->box[0] + c->ix[k] * w), py = (float)(c->box[1] + c->iy[k] * w),
          pz = (float)(c->box[2] + c->iz[k] * w);
    float fw = (float)w;
    out[0] = px + fw / 2.0f; out[1] = py + fw / 2.0f; out[2] = pz + fw / 2.0f;
}

int orc_ref_forces_f32(orc_ctx* c, float eps, float* f_leaf, float* f_node) {
    if (!c->lists_ready) return -1;
    int64_t nn = c->nnodes, n = c->n;
    float* qn = (float*)calloc(nn, sizeof(float));
    float* pf = (float*)malloc(sizeof(float) * 4 * (n ? n : 1));
    for (int64_t i = 0; i < n; ++i) {
        pf[4 * i] = (float)c->pos[3 * i]; pf[4 * i + 1] = (float)c->pos[3 * i + 1];
        pf[4 * i + 2] = (float)c->pos[3 * i + 2]; pf[4 * i + 3] = 0.0f;
    }
    for (int64_t k = nn - 1; k >= 0; --k) {
        if (is_leaf(c, k)) {
            float s = 0.0f;
            for (int i = c->begin[k]; i < c->begin[k] + c->count[k]; ++i) s += (float)c->q[i];
            qn[k] = s;
        } else {
            float s = 0.0f;
            for (int j = 0; j < c->nchild[k]; ++j) s += qn[c->child_begin[k] + j];
            qn[k] = s;
        }
    }
    const float fc = -1.0f, e2 = eps * eps;
    /* one node field per (target node, source node) interaction, src/field.cl:34-47 */
    int64_t* nf_off = (int64_t*)calloc((size_t)nn + 1, sizeof(int64_t));
    for (int64_t t = 0; t < nn; ++t) nf_off[t + 1] = nf_off[t] + c->m2l[t].n;
    float* En = (float*)calloc((size_t)3 * (nf_off[nn] ? nf_off[nn] : 1), sizeof(float));
    for (int64_t t = 0; t < nn; ++t) {
        float ct[3]; f_centre(c, t, ct);
        for (int64_t i = 0; i < c->m2l[t].n; ++i) {
            int64_t s = c->m2l[t].a[i];
            float cs[3]; f_centre(c, s, cs);
            float r[3] = {ct[0] - cs[0], ct[1] - cs[1], ct[2] - cs[2]};
            float rm = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + 0.0f * 0.0f + e2);
            float r3 = rm * rm * rm;
            for (int d = 0; d < 3; ++d) En[3 * (nf_off[t] + i) + d] = qn[s] * (fc * r[d] / r3);
        }
    }
    for (int64_t i = 0; i < n; ++i) for (int d = 0; d < 3; ++d) { f_leaf[3 * c->perm[i] + d] = 0; f_node[3 * c->perm[i] + d] = 0; }
    for (int64_t t = 0; t < nn; ++t) {
        if (!is_leaf(c, t)) continue;
        for (int i = c->begin[t]; i < c->begin[t] + c->count[t]; ++i) {
            /* node slots of the leaf: its own and its ancestors' node interactions
               (src/open_cl_simulation.cpp:436-473), each converted F = q * field
               (src/force.cl:224-231) and summed */
            float Et[3] = {0, 0, 0};
            float qi_ = (float)c->q[i];
            for (int64_t a = t; a >= 0; a = c->parent[a])
                for (int64_t f = nf_off[a]; f < nf_off[a + 1]; ++f)
                    for (int d = 0; d < 3; ++d) Et[d] += qi_ * En[3 * f + d];
            float qi = (float)c->q[i];
            float F[3] = {0, 0, 0};
            for (int64_t li = 0; li < c->p2p[t].n; ++li) {
                int64_t s = c->p2p[t].a[li];
                for (int j = c->begin[s]; j < c->begin[s] + c->count[s]; ++j) {
                    if (j == i) continue;
                    float r[3] = {pf[4 * j] - pf[4 * i], pf[4 * j + 1] - pf[4 * i + 1], pf[4 * j + 2] - pf[4 * i + 2]};
                    float rm = sqrtf(r[0] * r[0] + r[1] * r[1] + r[2] * r[2] + 0.0f * 0.0f + e2);
                    float r3 = rm * rm * rm;
                    for (int d = 0; d < 3; ++d) F[d] += qi * (-(float)c->q[j] * (fc * r[d] / r3));
                }
            }
            uint32_t o = c->perm[i];
            for (int d = 0; d < 3; ++d) { f_leaf[3 * o + d] = F[d]; f_node[3 * o + d] = Et[d]; }
        }
    }
    free(qn); free(pf); free(En); free(nf_off);
    return 0;
}

/* ------------------------------------------------------------------ */
/* FP64 direct sum (threaded over targets)                              */
/* ------------------------------------------------------------------ */
typedef struct {
    int64_t n; const double *pos, *q, *m; double eps2, G;
    int64_t nt; const int64_t* tgt; double *acc, *pot;
    int64_t lo, hi;
} direct_job;

static void* direct_worker(void* arg) {
    direct_job* J = (direct_job*)arg;
    for (int64_t ti = J->lo; ti < J->hi; ++ti) {
        int64_t i = J->tgt ? J->tgt[ti] : ti;
        double xi = J->pos[3 * i], yi = J->pos[3 * i + 1], zi = J->pos[3 * i + 2];
        double E[3] = {0, 0, 0}, psi = 0;
        for (int64_t j = 0; j < J->n; ++j) {
            if (j == i) continue;
            double dx = J->pos[3 * j] - xi, dy = J->pos[3 * j + 1] - yi, dz = J->pos[3 * j + 2] - zi;
            double s2 = dx * dx + dy * dy + dz * dz + J->eps2;
            if (s2 == 0.0) continue;
            double inv = 1.0 / sqrt(s2), inv3 = inv * inv * inv;
            double qj = J->q ? J->q[j] : 1.0;
            E[0] += qj * dx * inv3; E[1] += qj * dy * inv3; E[2] += qj * dz * inv3;
            psi += qj * inv;
        }
        double qi = J->q ? J->q[i] : 1.0, mi = J->m ? J->m[i] : 1.0;
        double f = J->G * qi / mi;
        if (J->acc) { J->acc[3 * ti] = f * E[0]; J->acc[3 * ti + 1] = f * E[1]; J->acc[3 * ti + 2] = f * E[2]; }
        if (J->pot) J->pot[ti] = -J->G * psi;
    }
    return NULL;
}

/* acc/pot rows follow the target list (or all particles if tgt == NULL) */
void orc_direct(int64_t n, const double* pos, const double* q, const double* m, double eps, double G,
                int64_t nt, const int64_t* tgt, double* acc, double* pot, int nthreads) {
    if (!tgt) nt = n;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    pthread_t th[64];
    direct_job J[64];
    for (int t = 0; t < nthreads; ++t) {
        J[t] = (direct_job){n, pos, q, m, eps * eps, G, nt, tgt, acc, pot, nt * t / nthreads, nt * (t + 1) / nthreads};
        pthread_create(&th[t], NULL, direct_worker, &J[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------ */
/* FP64 direct-sum force adjoint (vector-Jacobian product)              */
/* ------------------------------------------------------------------ */
/* With a_i = G q_i/m_i sum_{j != i} q_j K(x_j - x_i), K(r) = r / s^(3/2),
   s = |r|^2 + eps^2, returns for S = sum_i mu_i . a_i:
     gx_k = dS/dx_k = sum_{l != k} T(x_l - x_k) (q_k nu_l - q_l nu_k),
            T(r) = I / s^(3/2) - 3 r r^T / s^(5/2),  nu_i = G q_i/m_i mu_i
     gq_k = dS/dq_k = sum_{l != k} nu_l . K(x_k - x_l) + G/m_k mu_k . E_k
     gm_k = dS/dm_k = -G q_k/m_k^2 mu_k . E_k                             */
typedef struct {
    int64_t n; const double *pos, *q, *m, *nu, *mu; double eps2, G;
    double *gx, *gq, *gm; int64_t lo, hi;
} vjp_job;

static void* vjp_worker(void* arg) {
    vjp_job* J = (vjp_job*)arg;
    for (int64_t k = J->lo; k < J->hi; ++k) {
        const double xk = J->pos[3 * k], yk = J->pos[3 * k + 1], zk = J->pos[3 * k + 2];
        const double qk = J->q[k];
        const double* nk = J->nu + 3 * k;
        double g[3] = {0, 0, 0}, gq = 0, E[3] = {0, 0, 0};
        for (int64_t l = 0; l < J->n; ++l) {
            if (l == k) continue;
            const double rx = J->pos[3 * l] - xk, ry = J->pos[3 * l + 1] - yk, rz = J->pos[3 * l + 2] - zk;
            const double s = rx * rx + ry * ry + rz * rz + J->eps2;
            if (s == 0.0) continue;
            const double inv = 1.0 / sqrt(s), inv3 = inv * inv * inv, inv5 = inv3 * inv * inv;
            const double* nl = J->nu + 3 * l;
            const double ql = J->q[l];
            const double w[3] = {qk * nl[0] - ql * nk[0], qk * nl[1] - ql * nk[1], qk * nl[2] - ql * nk[2]};
            const double rw = rx * w[0] + ry * w[1] + rz * w[2];
            g[0] += w[0] * inv3 - 3.0 * rx * rw * inv5;
            g[1] += w[1] * inv3 - 3.0 * ry * rw * inv5;
            g[2] += w[2] * inv3 - 3.0 * rz * rw * inv5;
            gq -= (nl[0] * rx + nl[1] * ry + nl[2] * rz) * inv3;
            E[0] += ql * rx * inv3; E[1] += ql * ry * inv3; E[2] += ql * rz * inv3;
        }
        const double* mk = J->mu + 3 * k;
        const double muE = mk[0] * E[0] + mk[1] * E[1] + mk[2] * E[2];
        J->gx[3 * k] = g[0]; J->gx[3 * k + 1] = g[1]; J->gx[3 * k + 2] = g[2];
        J->gq[k] = gq + J->G / J->m[k] * muE;
        J->gm[k] = -J->G * qk / (J->m[k] * J->m[k]) * muE;
    }
    return NULL;
}

void orc_direct_vjp(int64_t n, const double* pos, const double* q, const double* m, double eps, double G,
                    const double* mu, double* gx, double* gq, double* gm, int nthreads) {
    double* nu = (double*)malloc(sizeof(double) * 3 * (n ? n : 1));
    for (int64_t i = 0; i < n; ++i)
        for (int d = 0; d < 3; ++d) nu[3 * i + d] = G * q[i] / m[i] * mu[3 * i + d];
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 64) nthreads = 64;
    pthread_t th[64];
    vjp_job J[64];
    for (int t = 0; t < nthreads; ++t) {
        J[t] = (vjp_job){n, pos, q, m, nu, mu, eps * eps, G, gx, gq, gm, n * t / nthreads, n * (t + 1) / nthreads};
        pthread_create(&th[t], NULL, vjp_worker, &J[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    free(nu);
}

/* Adjoint of `steps` kick-drift-kick steps with direct-sum forces: given
   gxT = dL/dx_N and gvT = dL/dv_N, returns dL/dx_0, dL/dv_0, dL/dq, dL/dm.
   Reverse sweep: lv_{N-1/2} = lv_N, lx_N += dt/2 J_N^T lv_N; then for
   n = N-1..0: lv_{n+1/2} += dt lx_{n+1} (drift), lx_n += c J_n^T lv_{n+1/2}
   with c = dt (n >= 1) or dt/2 (n = 0) (kicks), parameters likewise. */
void orc_leapfrog_adjoint(int64_t n, const double* pos0, const double* vel0, const double* q, const double* m,
                          double eps, double G, double dt, int steps, const double* gxT, const double* gvT,
                          double* gx0, double* gv0, double* gq, double* gm, int nthreads) {
    size_t sz = 3 * (size_t)n;
    double* xs = (double*)malloc(sizeof(double) * sz * (steps + 1));
    double* v = (double*)malloc(sizeof(double) * sz);
    double* acc = (double*)malloc(sizeof(double) * sz);
    memcpy(xs, pos0, sizeof(double) * sz);
    memcpy(v, vel0, sizeof(double) * sz);
    orc_direct(n, xs, q, m, eps, G, 0, NULL, acc, NULL, nthreads);
    for (int s = 0; s < steps; ++s) {
        double* x0 = xs + sz * s;
        double* x1 = xs + sz * (s + 1);
        for (size_t i = 0; i < sz; ++i) { v[i] += 0.5 * dt * acc[i]; x1[i] = x0[i] + dt * v[i]; }
        orc_direct(n, x1, q, m, eps, G, 0, NULL, acc, NULL, nthreads);
        for (size_t i = 0; i < sz; ++i) v[i] += 0.5 * dt * acc[i];
    }
    double* lx = gx0;
    double* lv = gv0;
    memcpy(lx, gxT, sizeof(double) * sz);
    memcpy(lv, gvT, sizeof(double) * sz);
    for (int64_t i = 0; i < n; ++i) { gq[i] = 0; gm[i] = 0; }
    double* mu = (double*)malloc(sizeof(double) * sz);
    double* gx = (double*)malloc(sizeof(double) * sz);
    double* tq = (double*)malloc(sizeof(double) * (n ? n : 1));
    double* tm = (double*)malloc(sizeof(double) * (n ? n : 1));
    for (int pt = steps; pt >= 0; --pt) {
        if (pt < steps)
            for (size_t i = 0; i < sz; ++i) lv[i] += dt * lx[i];      /* drift of step pt */
        const double c = (pt == steps || pt == 0) ? 0.5 * dt : dt;
        for (size_t i = 0; i < sz; ++i) mu[i] = c * lv[i];
        orc_direct_vjp(n, xs + sz * pt, q, m, eps, G, mu, gx, tq, tm, nthreads);
        for (size_t i = 0; i < sz; ++i) lx[i] += gx[i];
        for (int64_t i = 0; i < n; ++i) { gq[i] += tq[i]; gm[i] += tm[i]; }
    }
    free(xs); free(v); free(acc); free(mu); free(gx); free(tq); free(tm);
}

/* ------------------------------------------------------------------ */
/* FP64 direct-sum KDK leapfrog (trajectory oracle)                     */
/* ------------------------------------------------------------------ */
/* state is advanced in place; acc holds a(x) at entry (computed if first_call) */
void orc_leapfrog(int64_t n, double* pos, double* vel, const double* q, const double* m, double eps, double G,
                  double dt, int steps, double* acc, int have_acc, int nthreads) {
    if (!have_acc) orc_direct(n, pos, q, m, eps, G, 0, NULL, acc, NULL, nthreads);
    for (int s = 0; s < steps; ++s) {
        for (int64_t i = 0; i < 3 * n; ++i) { vel[i] += 0.5 * dt * acc[i]; pos[i] += dt * vel[i]; }
        orc_direct(n, pos, q, m, eps, G, 0, NULL, acc, NULL, nthreads);
        for (int64_t i = 0; i < 3 * n; ++i) vel[i] += 0.5 * dt * acc[i];
    }
}

/* ------------------------------------------------------------------ */
/* port of the reference CPU path, src/naive_simulation.cpp:7-46        */
/* ------------------------------------------------------------------ */
/* pos/vel are 4 floats per particle (x, y, z, w) as the reference's
   vector_t; fix_delta = 0 reproduces delta = (dx, dx, dx)
   (src/naive_simulation.cpp:10-14). */
float orc_naive_steps(int n, float* pos, float* vel, const float* mass, const float* charge, float G, float dt,
                      int steps, int fix_delta) {
    float time = 0.0f;
    for (int s = 0; s < steps; ++s) {
        for (unsigned i = 1; i < (unsigned)n; ++i) {
            for (unsigned j = 0; j < i; ++j) {
                float d0 = pos[4 * j] - pos[4 * i];
                float d1 = fix_delta ? pos[4 * j + 1] - pos[4 * i + 1] : pos[4 * j] - pos[4 * i];
                float d2 = fix_delta ? pos[4 * j + 2] - pos[4 * i + 2] : pos[4 * j] - pos[4 * i];
                float r = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
                float cf = charge[i] * charge[j];
                float ma = mass[i], mb = mass[j];
                float f0 = G * cf * d0 / (r * r * r);
                float f1 = G * cf * d1 / (r * r * r);
                float f2 = G * cf * d2 / (r * r * r);
                vel[4 * i] += f0 / ma * dt; vel[4 * i + 1] += f1 / ma * dt; vel[4 * i + 2] += f2 / ma * dt;
                vel[4 * j] -= f0 / mb * dt; vel[4 * j + 1] -= f1 / mb * dt; vel[4 * j + 2] -= f2 / mb * dt;
            }
        }
        for (unsigned i = 0; i < (unsigned)n; ++i) {
            pos[4 * i] += vel[4 * i] * dt; pos[4 * i + 1] += vel[4 * i + 1] * dt; pos[4 * i + 2] += vel[4 * i + 2] * dt;
        }
        time += dt;
    }
    return time;
}

/* The same serial loop restricted to rows i in [i0, i1) of the triangle
   (every j < i), i.e. a bounded sample of one step of
   src/naive_simulation.cpp:8-34 with identical per-pair arithmetic and
   update order.  Positions are not drifted.  Returns the pairs evaluated. */
int64_t orc_naive_rows(int n, const float* pos, float* vel, const float* mass, const float* charge, float G, float dt,
                       int i0, int i1, int fix_delta) {
    int64_t pairs = 0;
    for (unsigned i = (unsigned)(i0 < 1 ? 1 : i0); i < (unsigned)i1 && i < (unsigned)n; ++i) {
        for (unsigned j = 0; j < i; ++j) {
            float d0 = pos[4 * j] - pos[4 * i];
            float d1 = fix_delta ? pos[4 * j + 1] - pos[4 * i + 1] : pos[4 * j] - pos[4 * i];
            float d2 = fix_delta ? pos[4 * j + 2] - pos[4 * i + 2] : pos[4 * j] - pos[4 * i];
            float r = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
            float cf = charge[i] * charge[j];
            float ma = mass[i], mb = mass[j];
            float f0 = G * cf * d0 / (r * r * r);
            float f1 = G * cf * d1 / (r * r * r);
            float f2 = G * cf * d2 / (r * r * r);
            vel[4 * i] += f0 / ma * dt; vel[4 * i + 1] += f1 / ma * dt; vel[4 * i + 2] += f2 / ma * dt;
            vel[4 * j] -= f0 / mb * dt; vel[4 * j + 1] -= f1 / mb * dt; vel[4 * j + 2] -= f2 / mb * dt;
        }
        pairs += i;
    }
    return pairs;
}

/* Threaded form of the same per-pair arithmetic for timing on many cores:
   each thread owns a block of targets i and sums over every j != i (so each
   unordered pair is evaluated twice instead of once with Newton's third
   law).  Only velocities of the targets [t0, t1) are updated (a bounded
   sample); positions are not drifted.  Returns the number of pair
   evaluations done. */
typedef struct {
    int n; const float *pos, *mass, *charge; float* vel; float G, dt; int fix; int lo, hi;
} naive_job;
static void* naive_worker(void* arg) {
    naive_job* J = (naive_job*)arg;
    for (int i = J->lo; i < J->hi; ++i) {
        float dv0 = 0, dv1 = 0, dv2 = 0;
        for (int j = 0; j < J->n; ++j) {
            if (j == i) continue;
            float d0 = J->pos[4 * j] - J->pos[4 * i];
            float d1 = J->fix ? J->pos[4 * j + 1] - J->pos[4 * i + 1] : d0;
            float d2 = J->fix ? J->pos[4 * j + 2] - J->pos[4 * i + 2] : d0;
            float r = sqrtf(d0 * d0 + d1 * d1 + d2 * d2);
            float cf = J->charge[i] * J->charge[j];
            float ma = J->mass[i];
            float r3 = r * r * r;
            dv0 += J->G * cf * d0 / r3 / ma * J->dt;
            dv1 += J->G * cf * d1 / r3 / ma * J->dt;
            dv2 += J->G * cf * d2 / r3 / ma * J->dt;
        }
        J->vel[4 * i] += dv0; J->vel[4 * i + 1] += dv1; J->vel[4 * i + 2] += dv2;
    }
    return NULL;
}
int64_t orc_naive_kick_mt(int n, const float* pos, float* vel, const float* mass, const float* charge, float G,
                          float dt, int t0, int t1, int fix_delta, int nthreads) {
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    naive_job J[256];
    int cnt = t1 - t0;
    for (int t = 0; t < nthreads; ++t) {
        J[t] = (naive_job){n, pos, mass, charge, vel, G, dt, fix_delta,
                           t0 + (int)((int64_t)cnt * t / nthreads), t0 + (int)((int64_t)cnt * (t + 1) / nthreads)};
        pthread_create(&th[t], NULL, naive_worker, &J[t]);
    }
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    return (int64_t)cnt * (n - 1);
}
