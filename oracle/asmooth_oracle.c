/*
 * asmooth_oracle.c -- CPU oracle (TEST INFRASTRUCTURE ONLY; see asmooth_oracle.h).
 *
 * Build with -O2 -ffp-contract=off (no FMA contraction) so that every float
 * expression rounds exactly like the reference compiled the same way, on x86_64
 * and on aarch64 alike.  Citations are file:line in junkoda/asmooth.
 */
#include "asmooth_oracle.h"

#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define QUOTA 16 /* KDTree::allocate(np, 16) at clumping_tree_main.cpp:199 */

/* ------------------------------------------------------------------------- */
/* float helpers: the reference's expression order                           */
/* ------------------------------------------------------------------------- */

/* norm2 (nbr_search.cpp:20-25, fof.cpp:15-20): ((dx*dx + dy*dy) + dz*dz) */
static inline float norm2f(const float* a, const float* b)
{
    const float dx = a[0] - b[0];
    const float dy = a[1] - b[1];
    const float dz = a[2] - b[2];
    return dx * dx + dy * dy + dz * dz;
}

/* ker (nbr_search.cpp:27-37): tensor-product tent weight, left to right */
static inline float kerf(const float* a, const float* b, float hinv)
{
    return hinv * hinv * hinv * (1.0f - fabsf(a[0] - b[0]) * hinv)
                              * (1.0f - fabsf(a[1] - b[1]) * hinv)
                              * (1.0f - fabsf(a[2] - b[2]) * hinv);
}

/* f, ker_integ (coarse_mesh.cpp:10-22): exact cell integral of the unit tent */
static inline float tent_f(float x) { return x >= 1.0f ? 0.5f : x - 0.5f * x * x; }
static inline float ker_integ(float x1, float x2)
{
    const float fac1 = (float)(-1 + 2 * (x1 > 0.0f));
    const float fac2 = (float)(-1 + 2 * (x2 > 0.0f));
    return fac2 * tent_f(fac2 * x2) - fac1 * tent_f(fac1 * x1);
}
/* The library's cell weight (asg_common.cuh tent_integral_rn): the tent's
 * integral over [a, b] in cancellation-free forms, every operation rounded
 * as written (-ffp-contract=off), and the cell edge's offset from the particle
 * in units of h, fma(i, dx, -x) * hinv. */
static inline float tent_pos(float t) { return t >= 1.0f ? 0.5f : t * (1.0f - 0.5f * t); }
static inline float tent_integral(float a, float b)
{
    if (a >= 1.0f || b <= -1.0f) return 0.0f;
    if (a >= 0.0f) {
        if (b >= 1.0f) { const float u = 1.0f - a; return 0.5f * u * u; }
        return (b - a) * (1.0f - 0.5f * (a + b));
    }
    if (b <= 0.0f) {
        if (a <= -1.0f) { const float u = 1.0f + b; return 0.5f * u * u; }
        return (b - a) * (1.0f + 0.5f * (a + b));
    }
    return tent_pos(b) + tent_pos(-a);
}
static inline float edge_off(int i, float dx, float x, float hinv) { return fmaf((float)i, dx, -x) * hinv; }
static inline float lib_weight(int i, float dx, float x, float hinv)
{
    return tent_integral(edge_off(i, dx, x, hinv), edge_off(i + 1, dx, x, hinv));
}
static inline double tent_f64(double x) { return x >= 1.0 ? 0.5 : x - 0.5 * x * x; }
static inline double ker_integ64(double x1, double x2)
{
    const double fac1 = (double)(-1 + 2 * (x1 > 0.0));
    const double fac2 = (double)(-1 + 2 * (x2 > 0.0));
    return fac2 * tent_f64(fac2 * x2) - fac1 * tent_f64(fac1 * x1);
}

/* ------------------------------------------------------------------------- */
/* KDTreeSimple (kdtree_balanced.cpp:212-296)                                 */
/* ------------------------------------------------------------------------- */
typedef struct {
    int direction;
    float left, right;
    int content[2];
} onode; /* struct Node (kdtree_balanced.h:6-10) */

typedef struct {
    onode* nodes;
    int nn, cap;
    float* px;  /* positions in tree order (3 per particle) */
    int* perm;  /* perm[k] = input index of the particle at tree position k */
    float* bb;  /* per-node AABB (6 floats) for the exact searches, or NULL */
    int n;
} otree;

static int tree_node_alloc(otree* t, int inode)
{
    if (inode >= t->cap) {
        int cap = t->cap * 2;
        while (cap <= inode) cap *= 2;
        onode* nn = (onode*)realloc(t->nodes, sizeof(onode) * (size_t)cap);
        if (!nn) return -1;
        t->nodes = nn;
        t->cap = cap;
    }
    if (inode + 1 > t->nn) t->nn = inode + 1;
    return 0;
}

static inline void swap_particle(otree* t, int a, int b)
{
    float tx = t->px[3 * a], ty = t->px[3 * a + 1], tz = t->px[3 * a + 2];
    t->px[3 * a] = t->px[3 * b]; t->px[3 * a + 1] = t->px[3 * b + 1]; t->px[3 * a + 2] = t->px[3 * b + 2];
    t->px[3 * b] = tx; t->px[3 * b + 1] = ty; t->px[3 * b + 2] = tz;
    int ti = t->perm[a]; t->perm[a] = t->perm[b]; t->perm[b] = ti;
}

static int build_tree(const float* x, int n, otree* t)
{
    memset(t, 0, sizeof(*t));
    t->n = n;
    t->cap = 1024;
    t->nodes = (onode*)malloc(sizeof(onode) * (size_t)t->cap);
    t->px = (float*)malloc(sizeof(float) * 3 * (size_t)(n > 0 ? n : 1));
    t->perm = (int*)malloc(sizeof(int) * (size_t)(n > 0 ? n : 1));
    if (!t->nodes || !t->px || !t->perm) return -2;
    memcpy(t->px, x, sizeof(float) * 3 * (size_t)n);
    for (int k = 0; k < n; ++k) t->perm[k] = k;
    if (n <= 0) return -1;
    return 0;
}

static void free_tree(otree* t)
{
    free(t->nodes);
    free(t->px);
    free(t->perm);
    free(t->bb);
    memset(t, 0, sizeof(*t));
}

/* construct_tree_recursive (kdtree_balanced.cpp:230-296) in iterative form:
 * bisect the node's box at the midpoint of the next axis with a Hoare
 * partition; same node numbering (pre-order, left subtree first) and the same
 * particle permutation; the parent's content[] is patched by index. */
typedef struct { int inode, begin, end, dir, parent, side; float l3[3], r3[3]; } bframe;

static int construct(otree* t, float left, float right)
{
    int cap = 256, sp = 0, err = 0;
    bframe* st = (bframe*)malloc(sizeof(bframe) * (size_t)cap);
    if (!st) return -2;
    bframe f0 = {0, 0, t->n, 0, -1, 0, {left, left, left}, {right, right, right}};
    st[sp++] = f0;
    int next_inode = 0; /* last node index used so far */
    while (sp > 0) {
        bframe f = st[--sp];
        /* pre-order numbering: a node gets the next index when it is visited */
        int inode = (f.parent < 0) ? 0 : ++next_inode;
        if (tree_node_alloc(t, inode)) { err = -2; break; }
        if (f.parent >= 0) t->nodes[f.parent].content[f.side] = inode;
        onode* nd = &t->nodes[inode];
        nd->direction = f.dir;
        nd->left = f.l3[f.dir];
        nd->right = f.r3[f.dir];
        if (f.end - f.begin < QUOTA) {
            nd->content[0] = -f.begin - 1;
            nd->content[1] = -f.end;
            continue;
        }
        nd->content[0] = nd->content[1] = 0;
        const int i = (f.dir + 1) % 3;
        const float mid = f.l3[i] + 0.5f * (f.r3[i] - f.l3[i]);
        int j1 = f.begin, j2 = f.end - 1;
        for (;;) {
            while (j1 < f.end && t->px[3 * j1 + i] < mid) ++j1;
            while (j2 >= f.begin && t->px[3 * j2 + i] >= mid) --j2;
            if (j1 < j2) {
                swap_particle(t, j1, j2);
                ++j1; --j2;
            } else
                break;
        }
        if (!(j1 >= f.begin && j1 <= f.end && j1 - j2 == 1)) { err = -3; break; }
        const int pmid = j1;
        if (sp + 2 > cap) {
            cap *= 2;
            bframe* ns = (bframe*)realloc(st, sizeof(bframe) * (size_t)cap);
            if (!ns) { err = -2; break; }
            st = ns;
        }
        /* push right first so that the left subtree is numbered first */
        if (pmid < f.end) {
            bframe r = f;
            r.inode = -1; r.begin = pmid; r.end = f.end; r.dir = i; r.parent = inode; r.side = 1;
            r.l3[i] = mid;
            st[sp++] = r;
        }
        if (pmid != f.begin) {
            bframe l = f;
            l.inode = -1; l.begin = f.begin; l.end = pmid; l.dir = i; l.parent = inode; l.side = 0;
            l.r3[i] = mid;
            st[sp++] = l;
        }
    }
    free(st);
    return err;
}

static int make_tree(const float* x, int n, float left, float right, otree* t)
{
    int e = build_tree(x, n, t);
    if (e) { free_tree(t); return e; }
    e = construct(t, left, right);
    if (e) { free_tree(t); return e; }
    return 0;
}

/* per-node AABB of the particles below it (for conservative exact pruning) */
static void node_bbox(otree* t)
{
    t->bb = (float*)malloc(sizeof(float) * 6 * (size_t)t->nn);
    /* children have larger indices than parents (pre-order): sweep backwards */
    for (int k = t->nn - 1; k >= 0; --k) {
        float* b = t->bb + 6 * k;
        const onode* nd = &t->nodes[k];
        b[0] = b[1] = b[2] = FLT_MAX;
        b[3] = b[4] = b[5] = -FLT_MAX;
        if (nd->content[0] < 0) {
            for (int i = -nd->content[0] - 1; i < -nd->content[1]; ++i)
                for (int d = 0; d < 3; ++d) {
                    float v = t->px[3 * i + d];
                    if (v < b[d]) b[d] = v;
                    if (v > b[3 + d]) b[3 + d] = v;
                }
        } else {
            for (int s = 0; s < 2; ++s) {
                int c = nd->content[s];
                if (c <= 0) continue;
                const float* cb = t->bb + 6 * c;
                for (int d = 0; d < 3; ++d) {
                    if (cb[d] < b[d]) b[d] = cb[d];
                    if (cb[3 + d] > b[3 + d]) b[3 + d] = cb[3 + d];
                }
            }
        }
    }
}

static inline double bbox_dist2(const float* b, const float* q)
{
    double s = 0.0;
    for (int d = 0; d < 3; ++d) {
        double lo = (double)b[d] - (double)q[d], hi = (double)q[d] - (double)b[3 + d];
        double e = lo > 0.0 ? lo : (hi > 0.0 ? hi : 0.0);
        s += e * e;
    }
    return s;
}

/* ------------------------------------------------------------------------- */
/* faithful kNN: KNeighbors (k_neighbors.h:9-51) + find_nbr_recursive         */
/* ------------------------------------------------------------------------- */
typedef struct { float x[ORC_K + 1]; int s[ORC_K + 1]; } knbrs_t;

static inline void kn_clear(knbrs_t* k)
{
    for (int i = 0; i < ORC_K; ++i) { k->x[i] = FLT_MAX; k->s[i] = -1; }
    k->x[ORC_K] = -FLT_MAX;
}

/* KNeighbors::push (k_neighbors.h:25-35): x[] descending, x[0] = current k-th */
static inline void kn_push(knbrs_t* k, float val, int p)
{
    if (val < k->x[0]) {
        int i;
        for (i = 0; val < k->x[i + 1]; ++i) {
            k->x[i] = k->x[i + 1];
            k->s[i] = k->s[i + 1];
        }
        k->x[i] = val;
        k->s[i] = p;
    }
}

/* find_nbr_recursive (nbr_search.cpp:91-127) */
static void find_nbr(const otree* t, int node, const float* x, knbrs_t* kn)
{
    const onode* n = &t->nodes[node];
    const float r = sqrtf(kn->x[0]);
    const float y = x[n->direction];
    if (y + r < n->left || y - r > n->right) return;
    if (n->content[0] < 0) {
        for (int i = -n->content[0] - 1; i < -n->content[1]; ++i) {
            float d2 = norm2f(x, t->px + 3 * i);
            if (d2 < r * r) kn_push(kn, d2, i);
        }
        return;
    }
    const int cases = (n->content[0] > 0) + 2 * (n->content[1] > 0);
    switch (cases) {
    case 1: find_nbr(t, n->content[0], x, kn); break;
    case 2: find_nbr(t, n->content[1], x, kn); break;
    case 3: {
        const onode* nx = &t->nodes[n->content[0]];
        const int near = x[nx->direction] >= nx->right;
        find_nbr(t, n->content[near], x, kn);
        find_nbr(t, n->content[!near], x, kn);
        break;
    }
    default: break;
    }
}

int orc_neighbor_search(const float* x, int n, float left, float right, int nthreads,
                        float* rk, float* dens, int* nbr, float* nbr_d2)
{
    if (!x || n < ORC_K || !rk || !dens) return -1;
    otree t;
    int e = make_tree(x, n, left, right, &t);
    if (e) return e;
    float* dt = (float*)malloc(sizeof(float) * (size_t)n); /* dens in tree order */
    float* rt = (float*)malloc(sizeof(float) * (size_t)n);
    if (!dt || !rt) { free(dt); free(rt); free_tree(&t); return -2; }
    for (int k = 0; k < n; ++k) dt[k] = dens[t.perm[k]];
    int bad = 0;

    if (nthreads <= 1) {
        knbrs_t kn;
        for (int i = 0; i < n; ++i) { /* clumping_tree_main.cpp:428-430 */
            const float* xq = t.px + 3 * i;
            kn_clear(&kn);
            find_nbr(&t, 0, xq, &kn);
            if (!(kn.x[0] > 0.0f)) { bad = 1; break; }
            rt[i] = sqrtf(kn.x[0]);
            const float hinv = 1.0f / rt[i];
            for (int s = 1; s < ORC_K; ++s) { /* nbr_search.cpp:78-84 */
                const int q = kn.s[s];
                dt[q] += kerf(xq, t.px + 3 * q, hinv);
            }
            if (nbr) {
                for (int s = 0; s < ORC_K; ++s) {
                    nbr[(size_t)t.perm[i] * ORC_K + s] = t.perm[kn.s[s]];
                    if (nbr_d2) nbr_d2[(size_t)t.perm[i] * ORC_K + s] = kn.x[s];
                }
            }
        }
    } else {
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads) reduction(| : bad)
#endif
        for (int i = 0; i < n; ++i) {
            knbrs_t kn;
            const float* xq = t.px + 3 * i;
            kn_clear(&kn);
            find_nbr(&t, 0, xq, &kn);
            if (!(kn.x[0] > 0.0f)) { bad = 1; continue; }
            rt[i] = sqrtf(kn.x[0]);
            const float hinv = 1.0f / rt[i];
            for (int s = 1; s < ORC_K; ++s) {
                const int q = kn.s[s];
                const float w = kerf(xq, t.px + 3 * q, hinv);
#ifdef _OPENMP
#pragma omp atomic
#endif
                dt[q] += w;
            }
            if (nbr) {
                for (int s = 0; s < ORC_K; ++s) {
                    nbr[(size_t)t.perm[i] * ORC_K + s] = t.perm[kn.s[s]];
                    if (nbr_d2) nbr_d2[(size_t)t.perm[i] * ORC_K + s] = kn.x[s];
                }
            }
        }
    }
    if (!bad)
        for (int k = 0; k < n; ++k) {
            rk[t.perm[k]] = rt[k];
            dens[t.perm[k]] = dt[k];
        }
    free(dt);
    free(rt);
    free_tree(&t);
    return bad ? -4 : 0;
}

/* ------------------------------------------------------------------------- */
/* exact kNN by key (d2, index)                                              */
/* ------------------------------------------------------------------------- */
typedef struct { float d2[ORC_K]; int id[ORC_K]; int m; } topk_t; /* ascending */

static inline int key_less(float da, int ia, float db, int ib)
{
    return da < db || (da == db && ia < ib);
}

static inline void topk_push(topk_t* k, float d2, int id)
{
    if (k->m == ORC_K && !key_less(d2, id, k->d2[ORC_K - 1], k->id[ORC_K - 1])) return;
    int i = (k->m < ORC_K) ? k->m++ : ORC_K - 1;
    while (i > 0 && key_less(d2, id, k->d2[i - 1], k->id[i - 1])) {
        k->d2[i] = k->d2[i - 1];
        k->id[i] = k->id[i - 1];
        --i;
    }
    k->d2[i] = d2;
    k->id[i] = id;
}

static void find_exact(const otree* t, int node, const float* q, topk_t* k)
{
    if (k->m == ORC_K) {
        /* fl(d2) >= true d2 * (1 - 4 eps): a 1e-5 relative margin is conservative */
        double lim = (double)k->d2[ORC_K - 1] * (1.0 + 1e-5) + 1e-30;
        if (bbox_dist2(t->bb + 6 * node, q) > lim) return;
    }
    const onode* n = &t->nodes[node];
    if (n->content[0] < 0) {
        for (int i = -n->content[0] - 1; i < -n->content[1]; ++i)
            topk_push(k, norm2f(q, t->px + 3 * i), t->perm[i]);
        return;
    }
    int c0 = n->content[0], c1 = n->content[1];
    if (c0 > 0 && c1 > 0) {
        if (bbox_dist2(t->bb + 6 * c1, q) < bbox_dist2(t->bb + 6 * c0, q)) { int s = c0; c0 = c1; c1 = s; }
        find_exact(t, c0, q, k);
        find_exact(t, c1, q, k);
    } else if (c0 > 0)
        find_exact(t, c0, q, k);
    else if (c1 > 0)
        find_exact(t, c1, q, k);
}

int orc_knn_exact(const float* x, int n, float left, float right, int nthreads,
                  float* t33, int* idx33, int* nbr)
{
    if (!x || n < ORC_K || !t33 || !idx33) return -1;
    otree t;
    int e = make_tree(x, n, left, right, &t);
    if (e) return e;
    node_bbox(&t);
    if (nthreads < 1) nthreads = 1;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(nthreads)
#endif
    for (int i = 0; i < n; ++i) {
        topk_t k;
        k.m = 0;
        find_exact(&t, 0, x + 3 * (size_t)i, &k);
        t33[i] = k.d2[ORC_K - 1];
        idx33[i] = k.id[ORC_K - 1];
        if (nbr)
            for (int s = 0; s < ORC_K; ++s) nbr[(size_t)i * ORC_K + s] = k.id[s];
    }
    free_tree(&t);
    return 0;
}

int orc_dens_from_lists(const float* x, int n, const int* nbr, const float* t33,
                        float* rk_out, float* dens32, double* dens64)
{
    if (!x || !nbr || !t33 || n < ORC_K) return -1;
    for (int p = 0; p < n; ++p) {
        const float rk = sqrtf(t33[p]);
        if (!(rk > 0.0f)) return -4;
        if (rk_out) rk_out[p] = rk;
        const float hinv = 1.0f / rk;
        const double hinv64 = 1.0 / (double)rk;
        const float* xp = x + 3 * (size_t)p;
        for (int s = 0; s < ORC_K - 1; ++s) { /* the 32 nearest: all but the 33rd */
            const int q = nbr[(size_t)p * ORC_K + s];
            const float* xq = x + 3 * (size_t)q;
            if (dens32) dens32[q] += kerf(xp, xq, hinv);
            if (dens64) {
                double w = hinv64 * hinv64 * hinv64;
                for (int d = 0; d < 3; ++d) w *= (1.0 - fabs((double)xp[d] - (double)xq[d]) * hinv64);
                dens64[q] += w;
            }
        }
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* mesh deposit                                                               */
/* ------------------------------------------------------------------------- */

/* One particle's deposit position and cell range: the plain form's clipped
 * range (coarse_mesh.cpp:72-75) or the periodic form's shifted, unclipped one
 * (global_mesh.cpp:52-69).  Returns 0 when the periodic form skips the
 * particle (outside [0, boxsize)). */
static int dep_range(const float* y, float h, float boxsize, int nc, int periodic,
                     const float off[3], float xp[3], int lo[3], int hi[3])
{
    if (periodic) {
        if (y[0] < 0.0f || y[0] >= boxsize || y[1] < 0.0f || y[1] >= boxsize ||
            y[2] < 0.0f || y[2] >= boxsize)
            return 0;
        for (int i = 0; i < 3; ++i) xp[i] = y[i] + off[i];
    } else {
        for (int i = 0; i < 3; ++i) xp[i] = y[i];
    }
    for (int i = 0; i < 3; ++i) {
        if (periodic) {
            lo[i] = (int)floorf((xp[i] - h) / boxsize * nc);
            hi[i] = 1 + (int)ceilf((xp[i] + h) / boxsize * nc);
        } else {
            int a = (int)((xp[i] - h) / boxsize * nc);
            int b = 1 + (int)((xp[i] + h) / boxsize * nc);
            lo[i] = a > 0 ? a : 0;
            hi[i] = b < nc ? b : nc;
        }
    }
    return 1;
}

/* The float and FP64 deposit of every particle, in parallel over the mesh's
 * z-planes: each plane takes its particles in index order, so every cell sums
 * its contributions in the serial loop's order and the float mesh is the
 * serial one bit for bit.  The FP64 totals are summed per plane, then over
 * the planes in order.  mesh64 holds the FP64 restatement (weights computed in
 * double), or with fw the FP64 sums of the library's cell weights: the
 * products k0*k1*k2 of its float 1-D weights (lib_weight) taken in double,
 * times 1, dens or v.  The totals are always the FP64 sums of those weights (n
 * and halo), the quantity the library's FP64 totals reproduce.
 * Returns -4 if some rk is not positive. */
static int dep_by_planes(const float* x, const float* v, const float* dens, const float* rk,
                         const int* igrp, int n, float boxsize, int nc, int sign, int periodic,
                         const float off[3], int nthreads, float* mesh, double* mesh64,
                         double* totals, int fw)
{
    const size_t nmesh = (size_t)nc * nc * nc;
    const float dx = boxsize / nc;
    const int nc2 = nc * nc;
    const int lw = fw || totals;  /* the library's float weights are needed */
    size_t* start = (size_t*)calloc((size_t)nc + 1, sizeof(size_t));
    double* pt = (double*)calloc(2 * (size_t)nc, sizeof(double));
    if (!start || !pt) { free(start); free(pt); return -2; }
    int bad = 0;
    /* entries (particle, z) per wrapped plane, particles in index order */
    for (int j = 0; j < n; ++j) {
        float xp[3]; int lo[3], hi[3];
        const float h = rk[j];
        if (!(h > 0.0f)) { bad = 1; continue; }
        if (!dep_range(x + 3 * (size_t)j, h, boxsize, nc, periodic, off, xp, lo, hi)) continue;
        for (int iz = lo[2]; iz < hi[2]; ++iz) start[((iz % nc) + nc) % nc + 1]++;
    }
    for (int p = 0; p < nc; ++p) start[p + 1] += start[p];
    int* ej = (int*)malloc(start[nc] * sizeof(int) + 1);
    int* ez = (int*)malloc(start[nc] * sizeof(int) + 1);
    size_t* fill = (size_t*)malloc((size_t)nc * sizeof(size_t));
    if (!ej || !ez || !fill) { free(ej); free(ez); free(fill); free(start); free(pt); return -2; }
    memcpy(fill, start, (size_t)nc * sizeof(size_t));
    for (int j = 0; j < n; ++j) {
        float xp[3]; int lo[3], hi[3];
        const float h = rk[j];
        if (!(h > 0.0f)) continue;
        if (!dep_range(x + 3 * (size_t)j, h, boxsize, nc, periodic, off, xp, lo, hi)) continue;
        for (int iz = lo[2]; iz < hi[2]; ++iz) {
            const size_t e = fill[((iz % nc) + nc) % nc]++;
            ej[e] = j;
            ez[e] = iz;
        }
    }
    float* const mn = mesh;
    float* const mh = mn + nmesh;
    float* const mc = mh + nmesh;
    float* const mv = mc + nmesh;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 1) num_threads(nthreads)
#endif
    for (int p = 0; p < nc; ++p) {
        double tn = 0.0, th = 0.0;
        for (size_t e = start[p]; e < start[p + 1]; ++e) {
            const int j = ej[e], iz = ez[e];
            float xp[3]; int lo[3], hi[3];
            const float h = rk[j];
            dep_range(x + 3 * (size_t)j, h, boxsize, nc, periodic, off, xp, lo, hi);
            const float hinv = 1.0f / h;
            const float ds = dx * hinv;
            const double hinv64 = 1.0 / (double)h;
            const double ds64 = (double)dx * hinv64;
            const int to_halo = sign * igrp[j] > 0;
            float s1 = (iz * dx - xp[2]) * hinv;
            const float k2 = ker_integ(s1, s1 + ds);
            const float l2 = lw ? lib_weight(iz, dx, xp[2], hinv) : 0.0f;
            double t64 = ((double)iz * (double)dx - (double)xp[2]) * hinv64;
            const double k2d = ker_integ64(t64, t64 + ds64);
            for (int iy = lo[1]; iy < hi[1]; ++iy) {
                s1 = (iy * dx - xp[1]) * hinv;
                const float k1 = ker_integ(s1, s1 + ds);
                const float l1 = lw ? lib_weight(iy, dx, xp[1], hinv) : 0.0f;
                t64 = ((double)iy * (double)dx - (double)xp[1]) * hinv64;
                const double k1d = ker_integ64(t64, t64 + ds64);
                for (int ix = lo[0]; ix < hi[0]; ++ix) {
                    s1 = (ix * dx - xp[0]) * hinv;
                    const float k0 = ker_integ(s1, s1 + ds);
                    const size_t idx = (size_t)p * nc2 + (size_t)((iy % nc + nc) % nc) * nc +
                                       (size_t)((ix % nc + nc) % nc);
                    const float ker3 = k0 * k1 * k2;
                    const double lw3 = lw ? (double)lib_weight(ix, dx, xp[0], hinv) * (double)l1 *
                                                (double)l2 : 0.0;
                    if (!to_halo) {
                        mn[idx] += ker3;
                        mc[idx] += ker3 * dens[j];
                        mv[3 * idx] += ker3 * v[3 * (size_t)j];
                        mv[3 * idx + 1] += ker3 * v[3 * (size_t)j + 1];
                        mv[3 * idx + 2] += ker3 * v[3 * (size_t)j + 2];
                        tn += lw3;
                    } else {
                        mh[idx] += ker3;
                        th += lw3;
                    }
                    if (mesh64) {
                        t64 = ((double)ix * (double)dx - (double)xp[0]) * hinv64;
                        const double w = fw ? lw3 : ker_integ64(t64, t64 + ds64) * k1d * k2d;
                        if (!to_halo) {
                            mesh64[idx] += w;
                            mesh64[2 * nmesh + idx] += w * (double)dens[j];
                            mesh64[3 * nmesh + 3 * idx] += w * (double)v[3 * (size_t)j];
                            mesh64[3 * nmesh + 3 * idx + 1] += w * (double)v[3 * (size_t)j + 1];
                            mesh64[3 * nmesh + 3 * idx + 2] += w * (double)v[3 * (size_t)j + 2];
                        } else {
                            mesh64[nmesh + idx] += w;
                        }
                    }
                }
            }
        }
        pt[2 * p] = tn;
        pt[2 * p + 1] = th;
    }
    if (totals) {
        totals[0] = totals[1] = 0.0;
        for (int p = 0; p < nc; ++p) { totals[0] += pt[2 * p]; totals[1] += pt[2 * p + 1]; }
    }
    free(ej); free(ez); free(fill); free(start); free(pt);
    return bad ? -4 : 0;
}

int orc_assign_on_mesh(const float* x, const float* v, const float* dens, const float* rk,
                       const int* igrp, int n, float boxsize, int nc, int sign,
                       int periodic, const float* offset, int nthreads,
                       float* mesh, double* mesh64, double* totals)
{
    if (!x || !v || !dens || !rk || !igrp || !mesh || nc <= 0 || n < 0) return -1;
    const size_t nmesh = (size_t)nc * nc * nc;
    float* const mn = mesh;
    float* const mh = mn + nmesh;
    float* const mc = mh + nmesh;
    float* const mv = mc + nmesh;
    const float dx = boxsize / nc;
    const int nc2 = nc * nc;
    const float off[3] = {periodic && offset ? offset[0] : 0.0f,
                          periodic && offset ? offset[1] : 0.0f,
                          periodic && offset ? offset[2] : 0.0f};
    int bad = 0;
    if (nthreads < 1) nthreads = 1;
    const int par = nthreads > 1 && !mesh64 && !totals;
    /* the FP64 sums (in parallel, deterministically; the float mesh is the
     * serial loop's); without them the loop below runs serially or with the
     * atomics of the reference's OpenMP build */
    if (mesh64 || totals)
        return dep_by_planes(x, v, dens, rk, igrp, n, boxsize, nc, sign, periodic, off, nthreads,
                             mesh, mesh64, totals, 0);

#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(par ? nthreads : 1) reduction(| : bad)
#endif
    for (int j = 0; j < n; ++j) {
        const float* y = x + 3 * (size_t)j;
        float xp[3];
        if (periodic) { /* global_mesh.cpp:52-61 */
            if (y[0] < 0.0f || y[0] >= boxsize || y[1] < 0.0f || y[1] >= boxsize ||
                y[2] < 0.0f || y[2] >= boxsize)
                continue;
            xp[0] = y[0] + off[0];
            xp[1] = y[1] + off[1];
            xp[2] = y[2] + off[2];
        } else {
            xp[0] = y[0]; xp[1] = y[1]; xp[2] = y[2];
        }
        const float h = rk[j];
        if (!(h > 0.0f)) { bad = 1; continue; }
        const float hinv = 1.0f / h;
        int lo[3], hi[3];
        for (int i = 0; i < 3; ++i) {
            if (periodic) { /* global_mesh.cpp:66-69 */
                lo[i] = (int)floorf((xp[i] - h) / boxsize * nc);
                hi[i] = 1 + (int)ceilf((xp[i] + h) / boxsize * nc);
            } else { /* coarse_mesh.cpp:72-75 */
                int a = (int)((xp[i] - h) / boxsize * nc);
                int b = 1 + (int)((xp[i] + h) / boxsize * nc);
                lo[i] = a > 0 ? a : 0;
                hi[i] = b < nc ? b : nc;
            }
        }
        const float ds = dx * hinv;
        const double hinv64 = 1.0 / (double)h;
        const double ds64 = (double)dx * hinv64;
        const int to_halo = sign * igrp[j] > 0;
        for (int iz = lo[2]; iz < hi[2]; ++iz) {
            float s1 = (iz * dx - xp[2]) * hinv;
            const float k2 = ker_integ(s1, s1 + ds);
            double t64 = ((double)iz * (double)dx - (double)xp[2]) * hinv64;
            const double k2d = ker_integ64(t64, t64 + ds64);
            for (int iy = lo[1]; iy < hi[1]; ++iy) {
                s1 = (iy * dx - xp[1]) * hinv;
                const float k1 = ker_integ(s1, s1 + ds);
                t64 = ((double)iy * (double)dx - (double)xp[1]) * hinv64;
                const double k1d = ker_integ64(t64, t64 + ds64);
                for (int ix = lo[0]; ix < hi[0]; ++ix) {
                    s1 = (ix * dx - xp[0]) * hinv;
                    const float k0 = ker_integ(s1, s1 + ds);
                    size_t idx;
                    if (periodic)
                        idx = (size_t)((iz + nc) % nc) * nc2 + (size_t)((iy + nc) % nc) * nc + (size_t)((ix + nc) % nc);
                    else
                        idx = (size_t)iz * nc2 + (size_t)iy * nc + (size_t)ix;
                    const float ker3 = k0 * k1 * k2;
                    if (!to_halo) {
                        if (par) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mn[idx] += ker3;
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mc[idx] += ker3 * dens[j];
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mv[3 * idx] += ker3 * v[3 * (size_t)j];
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mv[3 * idx + 1] += ker3 * v[3 * (size_t)j + 1];
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mv[3 * idx + 2] += ker3 * v[3 * (size_t)j + 2];
                        } else {
                            mn[idx] += ker3;
                            mc[idx] += ker3 * dens[j];
                            mv[3 * idx] += ker3 * v[3 * (size_t)j];
                            mv[3 * idx + 1] += ker3 * v[3 * (size_t)j + 1];
                            mv[3 * idx + 2] += ker3 * v[3 * (size_t)j + 2];
                        }
                    } else {
                        if (par) {
#ifdef _OPENMP
#pragma omp atomic
#endif
                            mh[idx] += ker3;
                        } else {
                            mh[idx] += ker3;
                        }
                    }
                    if (mesh64) {
                        t64 = ((double)ix * (double)dx - (double)xp[0]) * hinv64;
                        const double k0d = ker_integ64(t64, t64 + ds64);
                        const double w = k0d * k1d * k2d;
                        double* m64 = mesh64;
                        if (!to_halo) {
                            m64[idx] += w;
                            m64[2 * nmesh + idx] += w * (double)dens[j];
                            m64[3 * nmesh + 3 * idx] += w * (double)v[3 * (size_t)j];
                            m64[3 * nmesh + 3 * idx + 1] += w * (double)v[3 * (size_t)j + 1];
                            m64[3 * nmesh + 3 * idx + 2] += w * (double)v[3 * (size_t)j + 2];
                        } else {
                            m64[nmesh + idx] += w;
                        }
                    }
                }
            }
        }
    }
    return bad ? -4 : 0;
}

/* As orc_assign_on_mesh (float mesh the same bit for bit), with mesh64 and the
 * totals the FP64 sums of the library's cell weights (the products of its
 * float 1-D weights, lib_weight) instead of the FP64 restatement: what a
 * deposit that forms and sums those weights without rounding error gives. */
int orc_assign_on_mesh_fw(const float* x, const float* v, const float* dens, const float* rk,
                          const int* igrp, int n, float boxsize, int nc, int sign, int periodic,
                          const float* offset, int nthreads, float* mesh, double* mesh64,
                          double* totals)
{
    if (!x || !v || !dens || !rk || !igrp || !mesh || !mesh64 || nc <= 0 || n < 0) return -1;
    const float off[3] = {periodic && offset ? offset[0] : 0.0f,
                          periodic && offset ? offset[1] : 0.0f,
                          periodic && offset ? offset[2] : 0.0f};
    return dep_by_planes(x, v, dens, rk, igrp, n, boxsize, nc, sign, periodic, off,
                         nthreads < 1 ? 1 : nthreads, mesh, mesh64, totals, 1);
}

int orc_assign_on_density_mesh(const float* x, const float* rk, const int* igrp, int n,
                               float boxsize, int nc, int sign, float* mesh)
{
    if (!x || !rk || !igrp || !mesh || nc <= 0) return -1;
    const float dx = boxsize / nc;
    const int nc2 = nc * nc;
    for (int j = 0; j < n; ++j) {
        const float* xp = x + 3 * (size_t)j;
        const float h = rk[j];
        if (!(h > 0.0f)) return -4;
        const float hinv = 1.0f / h;
        int lo[3], hi[3];
        for (int i = 0; i < 3; ++i) {
            int a = (int)((xp[i] - h) / boxsize * nc);
            int b = 1 + (int)((xp[i] + h) / boxsize * nc);
            lo[i] = a > 0 ? a : 0;
            hi[i] = b < nc ? b : nc;
        }
        const float ds = dx * hinv;
        for (int iz = lo[2]; iz < hi[2]; ++iz) {
            float s1 = (iz * dx - xp[2]) * hinv;
            const float k2 = ker_integ(s1, s1 + ds);
            for (int iy = lo[1]; iy < hi[1]; ++iy) {
                s1 = (iy * dx - xp[1]) * hinv;
                const float k1 = ker_integ(s1, s1 + ds);
                for (int ix = lo[0]; ix < hi[0]; ++ix) {
                    s1 = (ix * dx - xp[0]) * hinv;
                    const float k0 = ker_integ(s1, s1 + ds);
                    const float ker3 = k0 * k1 * k2;
                    if (sign * igrp[j] <= 0) mesh[(size_t)iz * nc2 + (size_t)iy * nc + ix] += ker3;
                }
            }
        }
    }
    return 0;
}

double orc_mesh_total(const float* mesh, int nc)
{
    const size_t nmesh = (size_t)nc * nc * nc;
    double m = 0.0;
    for (size_t j = 0; j < nmesh; ++j) m += mesh[j];
    return m;
}

int orc_normalise_mesh(float* mesh, int nc, float boxsize)
{
    if (!mesh || nc <= 0) return -1;
    const size_t nmesh = (size_t)nc * nc * nc;
    const float vol = powf(boxsize / nc, 3.0f);
    float* n = mesh;
    float* halo = mesh + nmesh;
    float* c = halo + nmesh;
    float* v = c + nmesh;
    for (size_t j = 0; j < nmesh; ++j) {
        if (n[j] > 0.0f) {
            c[j] *= vol / (n[j] * n[j]);
            v[3 * j] /= n[j];
            v[3 * j + 1] /= n[j];
            v[3 * j + 2] /= n[j];
        } else {
            c[j] = v[3 * j] = v[3 * j + 1] = v[3 * j + 2] = 0.0f;
        }
        n[j] *= 8.0f;
        halo[j] *= 8.0f;
    }
    return 0;
}

/* ------------------------------------------------------------------------- */
/* FOF (fof.cpp:34-166)                                                        */
/* ------------------------------------------------------------------------- */
typedef struct { int* q; int head, tail, cap; } iqueue;

static int iq_push(iqueue* qu, int v)
{
    if (qu->tail == qu->cap) {
        if (qu->head > 0) {
            memmove(qu->q, qu->q + qu->head, sizeof(int) * (size_t)(qu->tail - qu->head));
            qu->tail -= qu->head;
            qu->head = 0;
        } else {
            int cap = qu->cap * 2;
            int* nq = (int*)realloc(qu->q, sizeof(int) * (size_t)cap);
            if (!nq) return -1;
            qu->q = nq;
            qu->cap = cap;
        }
    }
    qu->q[qu->tail++] = v;
    return 0;
}

/* link_friends_recursive1 (fof.cpp:73-102) */
static void link_friends(const otree* t, int node, const float* x, float ll, int exact,
                         iqueue* fr, int grp, int* gt, int* err)
{
    const onode* n = &t->nodes[node];
    if (exact) {
        const double lim = (double)(ll * ll) * (1.0 + 1e-5) + 1e-30;
        if (bbox_dist2(t->bb + 6 * node, x) > lim) return;
    } else {
        const float y = x[n->direction];
        if (y + ll < n->left || y - ll > n->right) return;
    }
    if (n->content[0] < 0) {
        for (int i = -n->content[0] - 1; i < -n->content[1]; ++i) {
            if (gt[i] < grp) {
                const float d2 = norm2f(x, t->px + 3 * i);
                if (d2 <= ll * ll) {
                    if (gt[i] != 0) *err = -5;
                    if (iq_push(fr, i)) *err = -2;
                    gt[i] = grp;
                }
            }
        }
        return;
    }
    if (n->content[0]) link_friends(t, n->content[0], x, ll, exact, fr, grp, gt, err);
    if (n->content[1]) link_friends(t, n->content[1], x, ll, exact, fr, grp, gt, err);
}

int orc_group_fof(const float* x, int n, float left, float right, float ll, int exact,
                  int* igrp, int* ngroup)
{
    if (!x || !igrp || !ngroup || n <= 0) return -1;
    otree t;
    int e = make_tree(x, n, left, right, &t);
    if (e) return e;
    if (exact) node_bbox(&t);
    int* gt = (int*)malloc(sizeof(int) * (size_t)n);
    iqueue fr = {(int*)malloc(sizeof(int) * 1024), 0, 0, 1024};
    if (!gt || !fr.q) { free(gt); free(fr.q); free_tree(&t); return -2; }
    for (int k = 0; k < n; ++k) gt[k] = igrp[t.perm[k]];
    int ng = 0, err = 0;
    for (int i = 0; i < n && !err; ++i) { /* group_fof (fof.cpp:54-68) */
        if (gt[i] > 0) continue;
        ng++;
        gt[i] = ng;
        fr.head = fr.tail = 0;
        iq_push(&fr, i);
        while (fr.head < fr.tail && !err) {
            const int f = fr.q[fr.head++];
            link_friends(&t, 0, t.px + 3 * f, ll, exact, &fr, ng, gt, &err);
        }
    }
    for (int k = 0; k < n; ++k) igrp[t.perm[k]] = gt[k];
    *ngroup = ng;
    free(gt);
    free(fr.q);
    free_tree(&t);
    return err;
}

int orc_remove_small_groups(int* igrp, int n, int ngrp, int* nhalo)
{
    if (!igrp || !nhalo || ngrp < 0 || ngrp > n) return -1;
    const int threshold = 20; /* fof.cpp:107 */
    int* nf = (int*)calloc((size_t)ngrp + 1, sizeof(int));
    if (!nf) return -2;
    for (int j = 0; j < n; ++j) {
        if (igrp[j] < 0 || igrp[j] > ngrp) { free(nf); return -1; }
        nf[igrp[j]]++;
    }
    int nh = 0;
    for (int j = 1; j <= ngrp; ++j) nf[j] = nf[j] >= threshold ? ++nh : 0;
    nf[0] = 0;
    for (int j = 0; j < n; ++j) igrp[j] = nf[igrp[j]];
    *nhalo = nh;
    free(nf);
    return 0;
}

/* Zipped particle decode (read_pm_file_zip, file_reader2.cpp:187-252): fine
 * cells in (k, j, i) order, x fastest, each with counts8[cell] particles or,
 * for 255, the next value of counts32; particle p at
 *   x = mesh_scale*((off[3p] + 0.5f)/256.0f + i - 1.0f) - shift[0]   (i 1-based)
 *   v = vel[3p] / v_r2i
 * Returns 0 when exactly np_local particles are decoded, -1 otherwise. */
int orc_decode_zip(const unsigned char* off, const short* vel, const unsigned char* counts8,
                   const int* counts32, int n32, int np_local, int nc, int mesh_scale, float v_r2i,
                   const float* shift, float* x, float* v)
{
    int np = 0, j3 = 0;
    size_t cell = 0;
    for (int k = 1; k <= nc; ++k)
        for (int j = 1; j <= nc; ++j)
            for (int i = 1; i <= nc; ++i, ++cell) {
                int rr = counts8[cell];
                if (rr == 255) {
                    if (j3 >= n32) return -1;
                    rr = counts32[j3++];
                }
                for (int l = 1; l <= rr; ++l, ++np) {
                    if (np >= np_local) return -1;
                    const int c[3] = {i, j, k};
                    for (int d = 0; d < 3; ++d) {
                        x[3 * (size_t)np + d] =
                            mesh_scale * ((off[3 * (size_t)np + d] + 0.5f) / 256.0f + c[d] - 1.0f) -
                            shift[d];
                        v[3 * (size_t)np + d] = vel[3 * (size_t)np + d] / v_r2i;
                    }
                }
            }
    return np == np_local ? 0 : -1;
}

/* FOF halo catalogue (write_fof_halos, fof.cpp:169-219): per label 1..nhalo
 * the float sums of x and v in array order (fof.cpp:183-193), divided by the
 * member count (:199-202); halos whose centre is strictly inside (0, boxsize)^3
 * are kept in label order (:203-207).  out holds nhalo records of 7 words
 * {x[3], v[3], (int) nfof}.  The reference never clears v[2] (:179 clears x[2]
 * twice); here it starts at 0, which is what the reference gives on a zeroed
 * buffer. */
int orc_fof_halos(const float* x, const float* v, const int* igrp, int n, int nhalo,
                  float boxsize, float* out, int* nlocal)
{
    if (!x || !v || !igrp || !out || !nlocal || n < 0 || nhalo < 0) return -1;
    float* h = (float*)calloc((size_t)nhalo + 1, 7 * sizeof(float));
    int* nf = (int*)calloc((size_t)nhalo + 1, sizeof(int));
    if (!h || !nf) { free(h); free(nf); return -2; }
    for (int j = 0; j < n; ++j) {
        const int i = igrp[j] - 1;
        if (i < 0 || i >= nhalo) continue;
        nf[i]++;
        for (int k = 0; k < 3; ++k) {
            h[7 * i + k] += x[3 * j + k];
            h[7 * i + 3 + k] += v[3 * j + k];
        }
    }
    int nl = 0;
    for (int j = 0; j < nhalo; ++j) {
        float r[7];
        for (int k = 0; k < 6; ++k) r[k] = h[7 * j + k] / (float)nf[j];
        memcpy(&r[6], &nf[j], 4);
        if (0.0f < r[0] && r[0] < boxsize && 0.0f < r[1] && r[1] < boxsize && 0.0f < r[2] &&
            r[2] < boxsize)
            memcpy(out + 7 * (size_t)nl++, r, sizeof r);
    }
    *nlocal = nl;
    free(h);
    free(nf);
    return 0;
}

/* ------------------------------------------------------------------------- */
/* SO-halo marking (nbr_search.cpp:140-165, clumping_tree_main.cpp:474-485)    */
/* ------------------------------------------------------------------------- */
static int mark_rec(const otree* t, int node, const float* x, float r, int exact, int* gt)
{
    int np_halo = 0;
    const onode* n = &t->nodes[node];
    if (exact) {
        const double lim = (double)(r * r) * (1.0 + 1e-5) + 1e-30;
        if (bbox_dist2(t->bb + 6 * node, x) > lim) return 0;
    } else {
        const float y = x[n->direction];
        if (y + r < n->left || y - r > n->right) return 0;
    }
    if (n->content[0] < 0) {
        for (int i = -n->content[0] - 1; i < -n->content[1]; ++i) {
            const float d2 = norm2f(x, t->px + 3 * i);
            if (d2 < r * r) {
                gt[i] = -1;
                np_halo++;
            }
        }
        return np_halo;
    }
    if (n->content[0]) np_halo += mark_rec(t, n->content[0], x, r, exact, gt);
    if (n->content[1]) np_halo += mark_rec(t, n->content[1], x, r, exact, gt);
    return np_halo;
}

int orc_mark_halo_particles(const float* x, int n, float left, float right,
                            const float* halos, int nh, int exact,
                            int* igrp, long* np_halo, double* m_halo)
{
    if (!x || !igrp || n <= 0 || nh < 0 || (nh > 0 && !halos)) return -1;
    otree t;
    int e = make_tree(x, n, left, right, &t);
    if (e) return e;
    if (exact) node_bbox(&t);
    int* gt = (int*)malloc(sizeof(int) * (size_t)n);
    if (!gt) { free_tree(&t); return -2; }
    for (int k = 0; k < n; ++k) gt[k] = igrp[t.perm[k]];
    long np = 0;
    double mh = 0.0;
    for (int i = 0; i < nh; ++i) {
        const float* h = halos + 5 * (size_t)i;
        if (left < h[0] && h[0] < right && left < h[1] && h[1] < right && left < h[2] && h[2] < right) {
            np += mark_rec(&t, 0, h, h[3], exact, gt);
            mh += h[4] / 8.0f;
        }
    }
    for (int k = 0; k < n; ++k) igrp[t.perm[k]] = gt[k];
    if (np_halo) *np_halo = np;
    if (m_halo) *m_halo = mh;
    free(gt);
    free_tree(&t);
    return 0;
}
