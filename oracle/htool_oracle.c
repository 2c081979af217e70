/*
 * htool_oracle.c -- CPU restatement of htool's H-matrix hot path.
 *
 * TEST INFRASTRUCTURE.  This file is the checker for the htool_gb300 GPU
 * library: the pytest suite, __graft_entry__.smoke() and the cpu_baseline /
 * reference arm of bench.py load it (as oracle/liboracle.so) to produce the
 * expected cluster trees, block trees, partialACA factors and H-matrix
 * products on the same seeded inputs.  Nothing in htool_gb300 links, loads or
 * calls it.
 *
 * It restates, in plain C, the algorithms of upstream htool 0.8.1:
 *   - PCA cluster tree with geometric splitting
 *       include/htool/clustering/cluster.hpp:57-92, pca.hpp:15-128,
 *       splitting.hpp:11-120, misc/evp.hpp:43-130
 *   - block tree and Rjasanow-Steinbach admissibility
 *       include/htool/blocks/blocks.hpp:37-139, 237-278,
 *       admissibility_conditions.hpp:16-19
 *   - partialACA
 *       include/htool/lrmat/partialACA.hpp:39-171
 *   - HMatrix assembly with false-positive recursion
 *       include/htool/types/hmatrix.hpp:286-341, 423-607, 701-735
 *   - H-matrix product
 *       include/htool/types/hmatrix.hpp:844-911, 1074-1182,
 *       lrmat/lrmat.hpp:89-100, types/matrix.hpp:320-383
 * Floating-point operation order follows the upstream code wherever it is
 * observable (cluster centres, radii, covariance, eigenvector, ACA pivots and
 * stopping estimate); BLAS axpy / 3x3 gemm are taken as fused multiply-adds,
 * as OpenBLAS computes them.  Build with -ffp-contract=off.
 *
 * Parity pins: the fixtures under tests/golden were produced by the upstream
 * headers compiled by oracle/refbuild; tests/test_oracle_golden.py checks this file against
 * them bit-for-bit (trees, tasks, ranks) and to 1e-13 (products).
 */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* ------------------------------------------------------------------ */
/* kernels                                                             */
/* ------------------------------------------------------------------ */
/* Kernel ids (shared with the GPU library and the reference driver):
 *   0: 1/(1e-5 + r)
 *   1: 1/(4 pi r), 0 where r == 0
 *   2: exp(i k r)/(4 pi r), 0 where r == 0 (complex; see orc_kernel_z) */
static double orc_dist3(const double *a, const double *b) {
    double s = 0;
    for (int p = 0; p < 3; p++) {
        double d = a[p] - b[p];
        s += d * d;
    }
    return sqrt(s);
}

static double orc_kernel_d(int id, const double *a, const double *b) {
    double r = orc_dist3(a, b);
    if (id == 0)
        return 1. / (1e-5 + r);
    if (r == 0.)
        return 0.;
    return 1. / (4 * M_PI * r);
}

/* column-major M x N block, VirtualGenerator::copy_submatrix contract
 * (include/htool/types/virtual_generator.hpp:22) */
static void orc_copy_submatrix(int id, const double *xt, const double *xs, int M, int N, const int *rows, const int *cols, double *ptr) {
    for (int j = 0; j < N; j++)
        for (int i = 0; i < M; i++)
            ptr[i + (size_t)M * j] = orc_kernel_d(id, xt + 3 * (size_t)rows[i], xs + 3 * (size_t)cols[j]);
}

/* ------------------------------------------------------------------ */
/* cluster tree                                                        */
/* ------------------------------------------------------------------ */
typedef struct {
    int depth, rank, offset, size, counter, nb_sons, first_son;
    double rad, ctr[3];
} orc_node;

typedef struct {
    int n, minclustersize;
    int *perm;
    orc_node *nodes;
    int nnodes, cap;
    int min_depth, max_depth;
} orc_tree;

static int orc_new_node(orc_tree *T) {
    if (T->nnodes == T->cap) {
        T->cap   = T->cap ? 2 * T->cap : 64;
        T->nodes = (orc_node *)realloc(T->nodes, sizeof(orc_node) * T->cap);
    }
    memset(&T->nodes[T->nnodes], 0, sizeof(orc_node));
    return T->nnodes++;
}

/* solve_EVP_3 (misc/evp.hpp:43-130): eigenvector of the largest eigenvalue
 * of a symmetric 3x3 covariance matrix c (column-major). */
static void orc_evp3(const double *c, double *dir) {
#define C(i, j) c[(i) + 3 * (j)]
    dir[0] = dir[1] = dir[2] = 0;
    double p1 = C(0, 1) * C(0, 1) + C(0, 2) * C(0, 2) + C(1, 2) * C(1, 2);
    double eig[3];
    if (p1 < 1e-16) {
        eig[0] = C(0, 0);
        eig[1] = C(1, 1);
        eig[2] = C(2, 2);
        dir[0] = 1;
        dir[1] = 0;
        dir[2] = 0;
        if (eig[0] < eig[1]) {
            double t = eig[0];
            eig[0]   = eig[1];
            eig[1]   = t;
            dir[0]   = 0;
            dir[1]   = 1;
            dir[2]   = 0;
        }
        if (eig[0] < eig[2]) {
            double t = eig[0];
            eig[0]   = eig[2];
            eig[2]   = t;
            dir[0]   = 0;
            dir[1]   = 0;
            dir[2]   = 1;
        }
        return;
    }
    double q  = (C(0, 0) + C(1, 1) + C(2, 2)) / 3.;
    double p2 = (C(0, 0) - q) * (C(0, 0) - q) + (C(1, 1) - q) * (C(1, 1) - q) + (C(2, 2) - q) * (C(2, 2) - q) + 2. * p1;
    double p  = sqrt(p2 / 6.);
    double B[9];
    double ip = 1. / p;
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++)
            B[i + 3 * j] = ip * (C(i, j) - (i == j ? q : q * 0.));
#define Bm(i, j) B[(i) + 3 * (j)]
    double detB = Bm(0, 0) * (Bm(1, 1) * Bm(2, 2) - Bm(1, 2) * Bm(2, 1)) - Bm(0, 1) * (Bm(1, 0) * Bm(2, 2) - Bm(1, 2) * Bm(2, 0)) + Bm(0, 2) * (Bm(1, 0) * Bm(2, 1) - Bm(1, 1) * Bm(2, 0));
#undef Bm
    double r = detB / 2.;
    double phi;
    if (r <= -1)
        phi = 3.14159265358979323846 / 3.;
    else if (r >= 1)
        phi = 0;
    else
        phi = acos(r) / 3.;
    eig[0] = q + 2. * p * cos(phi);
    eig[2] = q + 2. * p * cos(phi + (2. * 3.14159265358979323846 / 3.));
    eig[1] = 3. * q - eig[0] - eig[2];
    if (fabs(eig[1]) < 1.e-12)
        eig[1] = 0.;
    if (fabs(eig[2]) < 1.e-12)
        eig[2] = 0.;
    if (fabs(eig[0]) < 1.e-16) {
        dir[0] = dir[1] = dir[2] = 0. * dir[0];
        return;
    }
    /* prod = (cov - e1 I)(cov - e2 I); the 3x3 product goes through BLAS
     * gemm upstream (types/matrix.hpp:283-289), i.e. a fused multiply-add
     * chain over k = 0, 1, 2 */
    double A1[9], A2[9], P[9];
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            A1[i + 3 * j] = C(i, j) - (i == j ? eig[1] : eig[1] * 0.);
            A2[i + 3 * j] = C(i, j) - (i == j ? eig[2] : eig[2] * 0.);
        }
    for (int j = 0; j < 3; j++)
        for (int i = 0; i < 3; i++) {
            double s = A1[i] * A2[3 * j];
            s        = fma(A1[i + 3], A2[1 + 3 * j], s);
            s        = fma(A1[i + 6], A2[2 + 3 * j], s);
            P[i + 3 * j] = s;
        }
    int ind = 0;
    double dn;
    do {
        dir[0] = P[0 + 3 * ind];
        dir[1] = P[1 + 3 * ind];
        dir[2] = P[2 + 3 * ind];
        dn     = sqrt(dir[0] * dir[0] + dir[1] * dir[1] + dir[2] * dir[2]);
        ind++;
    } while (dn < 1.e-15 && ind < 3);
    if (dn < 1.e-15) {
        dir[0] = 1;
        dir[1] = 0;
        dir[2] = 0;
    } else {
        dir[0] /= dn;
        dir[1] /= dn;
        dir[2] /= dn;
    }
#undef C
}

static double orc_dot3(const double *a, const double *b) { return ((0. + a[0] * b[0]) + a[1] * b[1]) + a[2] * b[2]; }

/* splitting.hpp:63-120 (geometric).  Writes the son of every point of num
 * into son[], returns 0 on success, 1 if a son would be empty (the caller
 * then needs regular splitting, never the case for nb_sons <= 2). */
static int orc_geometric_split(const double *x, const int *num, int n, const double *ctr, const double *dir, int nb_sons, int *son) {
    if (nb_sons == 2) {
        for (int j = 0; j < n; j++) {
            double dx[3];
            for (int p = 0; p < 3; p++)
                dx[p] = x[3 * (size_t)num[j] + p] - ctr[p];
            son[j] = orc_dot3(dir, dx) > 0 ? 0 : 1;
        }
        return 0;
    }
    if (n <= 1) {
        for (int j = 0; j < n; j++)
            son[j] = 0;
        return n == 0 && nb_sons > 0;
    }
    /* std::minmax_element: first smallest, last largest projection */
    int imin = 0, imax = 0;
    double pmin = orc_dot3(x + 3 * (size_t)num[0], dir), pmax = pmin;
    for (int j = 1; j < n; j++) {
        double pj = orc_dot3(x + 3 * (size_t)num[j], dir);
        if (pj < pmin) {
            pmin = pj;
            imin = j;
        }
        if (!(pj < pmax)) {
            pmax = pj;
            imax = j;
        }
    }
    const double *mn = x + 3 * (size_t)num[imin], *mx = x + 3 * (size_t)num[imax];
    double d[3];
    for (int p = 0; p < 3; p++)
        d[p] = mx[p] - mn[p];
    double length = orc_dot3(d, dir) / (double)nb_sons;
    int *cnt      = (int *)calloc(nb_sons, sizeof(int));
    for (int j = 0; j < n; j++) {
        double dx[3];
        for (int p = 0; p < 3; p++)
            dx[p] = x[3 * (size_t)num[j] + p] - mn[p];
        int idx = (int)(orc_dot3(dx, dir) / length);
        idx     = idx == nb_sons ? idx - 1 : idx;
        son[j]  = idx;
        cnt[idx]++;
    }
    int empty = 0;
    for (int p = 0; p < nb_sons; p++)
        empty |= cnt[p] == 0;
    free(cnt);
    return empty;
}

typedef struct {
    int node;
    int *num;
} orc_item;

/* Cluster::build (cluster.hpp:57-92) + PCA::recursive_build (pca.hpp:15-128)
 * in a run of size_world MPI ranks: the root has size_world sons at depth 1
 * (pca.hpp:28), son p holding the points of rank p (pca.hpp:93-99); one rank
 * gives the root a single son. */
void *orc_cluster_build_world(int n, const double *x, int minclustersize, int nb_sons, int size_world) {
    if (nb_sons == -1)
        nb_sons = 2;
    orc_tree *T       = (orc_tree *)calloc(1, sizeof(orc_tree));
    T->n              = n;
    T->minclustersize = minclustersize;
    T->perm           = (int *)malloc(sizeof(int) * (n ? n : 1));
    T->min_depth      = -1;
    T->max_depth      = 0;
    int root          = orc_new_node(T);
    T->nodes[root].rank = -1;
    T->nodes[root].size = n;
    int stack_cap = 64, top = 0;
    orc_item *st  = (orc_item *)malloc(sizeof(orc_item) * stack_cap);
    st[top].node  = root;
    st[top].num   = (int *)malloc(sizeof(int) * (n ? n : 1));
    for (int i = 0; i < n; i++)
        st[top].num[i] = i;
    top++;
    while (top > 0) {
        orc_item it = st[--top];
        orc_node *c = &T->nodes[it.node];
        int np      = c->size;
        int nsons   = c->depth == 0 ? size_world : nb_sons;
        /* centre: sum of g*x with g = 1, times 1/G (pca.hpp:30-46) */
        double G = 0;
        for (int j = 0; j < np; j++)
            G += 1.;
        double xc[3] = {0, 0, 0};
        for (int j = 0; j < np; j++)
            for (int p = 0; p < 3; p++)
                xc[p] += 1. * x[3 * (size_t)it.num[j] + p];
        double iG = 1. / G;
        for (int p = 0; p < 3; p++)
            xc[p] = xc[p] * iG;
        memcpy(c->ctr, xc, sizeof(xc));
        /* radius and covariance (pca.hpp:49-64) */
        double cov[9] = {0};
        double rad    = 0;
        for (int j = 0; j < np; j++) {
            double u[3];
            for (int p = 0; p < 3; p++)
                u[p] = x[3 * (size_t)it.num[j] + p] - xc[p];
            double nr = sqrt(fabs(orc_dot3(u, u))) + 0.;
            rad       = rad > nr ? rad : nr;
            for (int p = 0; p < 3; p++)
                for (int q = 0; q < 3; q++)
                    cov[p + 3 * q] += 1. * u[p] * u[q];
        }
        c->rad = rad;
        double dir[3];
        orc_evp3(cov, dir);
        /* sons */
        int first = T->nnodes;
        for (int p = 0; p < nsons; p++) {
            int s                = orc_new_node(T);
            c                    = &T->nodes[it.node];
            T->nodes[s].counter  = c->counter * nsons + p;
            T->nodes[s].depth    = c->depth + 1;
        }
        c->first_son = first;
        c->nb_sons   = nsons;
        int *son     = (int *)malloc(sizeof(int) * (np ? np : 1));
        if (orc_geometric_split(x, it.num, np, c->ctr, dir, nsons, son)) {
            fprintf(stderr, "orc_cluster_build: regular splitting fallback is not restated\n");
            abort();
        }
        int *cnt = (int *)calloc(nsons, sizeof(int));
        for (int j = 0; j < np; j++)
            cnt[son[j]]++;
        int **numb = (int **)malloc(sizeof(int *) * nsons);
        int *fill  = (int *)calloc(nsons, sizeof(int));
        for (int p = 0; p < nsons; p++)
            numb[p] = (int *)malloc(sizeof(int) * (cnt[p] ? cnt[p] : 1));
        for (int j = 0; j < np; j++)
            numb[son[j]][fill[son[j]]++] = it.num[j];
        int count = 0;
        for (int p = 0; p < nsons; p++) {
            orc_node *s = &T->nodes[first + p];
            s->offset   = c->offset + count;
            s->size     = cnt[p];
            count += cnt[p];
            s->rank = c->depth == 0 ? s->counter : c->rank;
        }
        int ok = 1;
        for (int p = 0; p < nsons; p++)
            ok = ok && (cnt[p] >= minclustersize);
        if (ok || c->rank == -1) {
            for (int p = 0; p < nsons; p++) {
                if (top == stack_cap) {
                    stack_cap *= 2;
                    st = (orc_item *)realloc(st, sizeof(orc_item) * stack_cap);
                }
                st[top].node = first + p;
                st[top].num  = numb[p];
                top++;
            }
        } else {
            if (c->depth > T->max_depth)
                T->max_depth = c->depth;
            if (T->min_depth < 0 || c->depth < T->min_depth)
                T->min_depth = c->depth;
            /* clear_sons: the sons are the last nodes created */
            T->nnodes    = first;
            c->nb_sons   = 0;
            c->first_son = 0;
            memcpy(T->perm + c->offset, it.num, sizeof(int) * np);
            for (int p = 0; p < nsons; p++)
                free(numb[p]);
        }
        free(numb);
        free(fill);
        free(cnt);
        free(son);
        free(it.num);
    }
    free(st);
    return T;
}

void *orc_cluster_build(int n, const double *x, int minclustersize, int nb_sons) { return orc_cluster_build_world(n, x, minclustersize, nb_sons, 1); }

/* MasterOffset (cluster.hpp:42, pca.hpp:98): (offset, size) of the depth-1
 * cluster of every rank; returns the number of ranks */
int orc_cluster_masteroffset(void *p, int *out) {
    orc_tree *T = (orc_tree *)p;
    orc_node *r = &T->nodes[0];
    if (out)
        for (int q = 0; q < r->nb_sons; q++) {
            out[2 * q]     = T->nodes[r->first_son + q].offset;
            out[2 * q + 1] = T->nodes[r->first_son + q].size;
        }
    return r->nb_sons;
}

void orc_cluster_free(void *p) {
    orc_tree *T = (orc_tree *)p;
    free(T->perm);
    free(T->nodes);
    free(T);
}

int orc_cluster_nnodes(void *p) { return ((orc_tree *)p)->nnodes; }

static void orc_export_rec(orc_tree *T, int v, int *k, int *node_i, double *node_d) {
    orc_node *c         = &T->nodes[v];
    node_i[6 * *k + 0]  = c->depth;
    node_i[6 * *k + 1]  = c->rank;
    node_i[6 * *k + 2]  = c->offset;
    node_i[6 * *k + 3]  = c->size;
    node_i[6 * *k + 4]  = c->nb_sons;
    node_i[6 * *k + 5]  = c->counter;
    node_d[4 * *k + 0]  = c->rad;
    for (int q = 0; q < 3; q++)
        node_d[4 * *k + 1 + q] = c->ctr[q];
    (*k)++;
    for (int s = 0; s < c->nb_sons; s++)
        orc_export_rec(T, c->first_son + s, k, node_i, node_d);
}

/* same layout as the reference driver: pre-order, sons in order */
void orc_cluster_export(void *p, int *perm, int *node_i, double *node_d) {
    orc_tree *T = (orc_tree *)p;
    memcpy(perm, T->perm, sizeof(int) * T->n);
    int k = 0;
    orc_export_rec(T, 0, &k, node_i, node_d);
}

void orc_cluster_depths(void *p, int *mn, int *mx) {
    *mn = ((orc_tree *)p)->min_depth;
    *mx = ((orc_tree *)p)->max_depth;
}

/* ------------------------------------------------------------------ */
/* block tree                                                          */
/* ------------------------------------------------------------------ */
typedef struct {
    int t, s, adm;
} orc_task;

typedef struct {
    orc_task *v;
    int n, cap;
} orc_tasks;

static void orc_push_task(orc_tasks *L, int t, int s, int adm) {
    if (L->n == L->cap) {
        L->cap = L->cap ? 2 * L->cap : 256;
        L->v   = (orc_task *)realloc(L->v, sizeof(orc_task) * L->cap);
    }
    L->v[L->n].t   = t;
    L->v[L->n].s   = s;
    L->v[L->n].adm = adm;
    L->n++;
}

/* RjasanowSteinbach::ComputeAdmissibility (admissibility_conditions.hpp:16-19) */
static int orc_admissible(const orc_node *t, const orc_node *s, double eta) {
    double d[3];
    for (int p = 0; p < 3; p++)
        d[p] = t->ctr[p] - s->ctr[p];
    double dist = sqrt(fabs(orc_dot3(d, d)));
    double mn   = t->rad < s->rad ? t->rad : s->rad;
    double sep  = dist - t->rad - s->rad;
    sep         = sep > 0. ? sep : 0.;
    return 2 * mn < eta * sep;
}

typedef struct {
    orc_tree *T, *S;
    double eta;
    size_t maxblocksize;
    int mintargetdepth, minsourcedepth;
    orc_tasks tasks;
} orc_bt;

/* Block::build_block_tree (blocks.hpp:37-139); returns 1 = "not pushed" */
static int orc_bt_rec(orc_bt *B, int t, int s, int adm) {
    orc_node *tn = &B->T->nodes[t], *sn = &B->S->nodes[s];
    size_t bsize = (size_t)tn->size * (size_t)sn->size;
    int deep     = tn->rank >= 0 && tn->depth >= B->mintargetdepth && sn->depth >= B->minsourcedepth;
    if (adm && deep) {
        orc_push_task(&B->tasks, t, s, 1);
        return 0;
    }
    int split_t;
    if (sn->nb_sons == 0) {
        if (tn->nb_sons == 0)
            return 1;
        split_t = 1;
    } else if (tn->nb_sons == 0) {
        split_t = 0;
    } else {
        split_t = tn->size > sn->size;
    }
    int ns    = split_t ? tn->nb_sons : sn->nb_sons;
    int first = split_t ? tn->first_son : sn->first_son;
    int *np   = (int *)malloc(sizeof(int) * ns);
    int *kid  = (int *)malloc(sizeof(int) * ns);
    int *kadm = (int *)malloc(sizeof(int) * ns);
    int all   = 1;
    for (int p = 0; p < ns; p++) {
        int tt  = split_t ? first + p : t;
        int ss  = split_t ? s : first + p;
        kid[p]  = split_t ? tt : ss;
        kadm[p] = orc_admissible(&B->T->nodes[tt], &B->S->nodes[ss], B->eta);
        np[p]   = orc_bt_rec(B, tt, ss, kadm[p]);
        all     = all && np[p];
    }
    int ret;
    if (bsize <= B->maxblocksize && all && deep) {
        ret = 1;
    } else {
        for (int p = 0; p < ns; p++)
            if (np[p])
                orc_push_task(&B->tasks, split_t ? kid[p] : t, split_t ? s : kid[p], kadm[p]);
        ret = 0;
    }
    free(np);
    free(kid);
    free(kadm);
    return ret;
}

static orc_tree *orc_cmp_T, *orc_cmp_S;
static int orc_task_cmp(const void *a, const void *b) {
    const orc_task *x = (const orc_task *)a, *y = (const orc_task *)b;
    int xt = orc_cmp_T->nodes[x->t].offset, yt = orc_cmp_T->nodes[y->t].offset;
    if (xt != yt)
        return xt < yt ? -1 : 1;
    int xs = orc_cmp_S->nodes[x->s].offset, ys = orc_cmp_S->nodes[y->s].offset;
    return xs < ys ? -1 : (xs > ys);
}

/* Block::build with UPLO 'N' (blocks.hpp:237-278): tasks, then the local
 * filter (every task whose target cluster belongs to `rank`) and the
 * (t.offset, s.offset) sort. */
static orc_tasks orc_block_build(orc_tree *T, orc_tree *S, double eta, int rank) {
    orc_bt B;
    memset(&B, 0, sizeof(B));
    B.T            = T;
    B.S            = S;
    B.eta          = eta;
    B.maxblocksize = 1000000;
    int adm        = orc_admissible(&T->nodes[0], &S->nodes[0], eta);
    if (orc_bt_rec(&B, 0, 0, adm))
        orc_push_task(&B.tasks, 0, 0, adm);
    /* local cluster = the depth-1 son of `rank` */
    orc_tasks L;
    memset(&L, 0, sizeof(L));
    for (int b = 0; b < B.tasks.n; b++)
        if (T->nodes[B.tasks.v[b].t].rank == rank)
            orc_push_task(&L, B.tasks.v[b].t, B.tasks.v[b].s, B.tasks.v[b].adm);
    free(B.tasks.v);
    orc_cmp_T = T;
    orc_cmp_S = S;
    qsort(L.v, L.n, sizeof(orc_task), orc_task_cmp);
    return L;
}

int orc_block_tasks_rank(void *ct, void *cs, double eta, int rank, int *out) {
    orc_tree *T = (orc_tree *)ct, *S = (orc_tree *)cs;
    orc_tasks L = orc_block_build(T, S, eta, rank);
    if (out)
        for (int b = 0; b < L.n; b++) {
            out[5 * b + 0] = T->nodes[L.v[b].t].offset;
            out[5 * b + 1] = T->nodes[L.v[b].t].size;
            out[5 * b + 2] = S->nodes[L.v[b].s].offset;
            out[5 * b + 3] = S->nodes[L.v[b].s].size;
            out[5 * b + 4] = L.v[b].adm;
        }
    int n = L.n;
    free(L.v);
    return n;
}

int orc_block_tasks(void *ct, void *cs, double eta, int *out) { return orc_block_tasks_rank(ct, cs, eta, 0, out); }

/* ------------------------------------------------------------------ */
/* partialACA                                                          */
/* ------------------------------------------------------------------ */
/* partialACA<double>::copy_low_rank_approximation (partialACA.hpp:39-171).
 * reqrank < 0: adaptive to eps.  Returns the rank (-1 = rejected as not
 * profitable or first row zero); on success *U (M x rank, col-major) and
 * *V (rank x N, col-major) are malloc'd. */
int orc_partial_aca(int kernel, const double *xt, const double *xs, double eps, int reqrank, int M, int N, const int *rows, const int *cols, const double *tctr, double **U, double **V) {
    double dist = 1e30;
    int I       = 0;
    for (int i = 0; i < M; i++) {
        const double *a = xt + 3 * (size_t)rows[i];
        double s        = 0;
        for (int p = 0; p < 3; p++)
            s = s + (a[p] - tctr[p]) * (a[p] - tctr[p]);
        double ad = sqrt(s);
        if (dist > ad) {
            dist = ad;
            I    = i;
        }
    }
    int J = 0, q = 0;
    int cap = 16;
    double **uu = (double **)malloc(sizeof(double *) * cap), **vv = (double **)malloc(sizeof(double *) * cap);
    int nuv = 0;
    char *vrow = (char *)calloc(M, 1), *vcol = (char *)calloc(N, 1);
    double frob = 0, aux = 0;
    /* q*(M+N) > M*N with the reference's 32-bit int products */
    int32_t MN = (int32_t)((uint32_t)M * (uint32_t)N);
    while ((reqrank > 0 && q < (reqrank < (M < N ? M : N) ? reqrank : (M < N ? M : N))) || (reqrank < 0 && (q == 0 || sqrt(aux / frob) > eps))) {
        q += 1;
        if ((int32_t)((uint32_t)q * (uint32_t)(M + N)) > MN) {
            q = -1;
            break;
        }
        double *r = (double *)malloc(sizeof(double) * N);
        orc_copy_submatrix(kernel, xt, xs, 1, N, &rows[I], cols, r);
        for (int j = 0; j < nuv; j++) {
            double coef = -uu[j][I];
            for (int k = 0; k < N; k++)
                r[k] = fma(coef, vv[j][k], r[k]);
        }
        double pivot = 0., tmp;
        for (int k = 0; k < N; k++) {
            if (vcol[k])
                continue;
            tmp = fabs(r[k]);
            if (tmp < pivot)
                continue;
            pivot = tmp;
            J     = k;
        }
        vrow[I]      = 1;
        double gamma = 1. / r[J];
        if (fabs(r[J]) > 1e-15) {
            double *c = (double *)malloc(sizeof(double) * M);
            orc_copy_submatrix(kernel, xt, xs, M, 1, rows, &cols[J], c);
            for (int k = 0; k < nuv; k++) {
                double coef = -vv[k][J];
                for (int i = 0; i < M; i++)
                    c[i] = fma(coef, uu[k][i], c[i]);
            }
            for (int i = 0; i < M; i++)
                c[i] = c[i] * gamma;
            pivot = 0.;
            for (int k = 0; k < M; k++) {
                if (vrow[k])
                    continue;
                tmp = fabs(c[k]);
                if (tmp < pivot)
                    continue;
                pivot = tmp;
                I     = k;
            }
            vcol[J] = 1;
            if (reqrank < 0) {
                double cc = 0, rr = 0, fa = 0;
                for (int i = 0; i < M; i++)
                    cc += c[i] * c[i];
                for (int k = 0; k < N; k++)
                    rr += r[k] * r[k];
                aux = fabs(cc) * fabs(rr);
                for (int j = 0; j < nuv; j++) {
                    double d1 = 0, d2 = 0;
                    for (int k = 0; k < N; k++)
                        d1 += vv[j][k] * r[k];
                    for (int i = 0; i < M; i++)
                        d2 += uu[j][i] * c[i];
                    fa += d1 * d2;
                }
                frob += aux + 2 * fa;
            }
            if (nuv == cap) {
                cap *= 2;
                uu = (double **)realloc(uu, sizeof(double *) * cap);
                vv = (double **)realloc(vv, sizeof(double *) * cap);
            }
            uu[nuv] = c;
            vv[nuv] = r;
            nuv++;
        } else {
            free(r);
            q -= 1;
            if (q == 0)
                q = -1;
            break;
        }
    }
    int rank = q;
    *U       = NULL;
    *V       = NULL;
    if (rank > 0) {
        *U = (double *)malloc(sizeof(double) * (size_t)M * rank);
        *V = (double *)malloc(sizeof(double) * (size_t)rank * N);
        for (int k = 0; k < rank; k++) {
            memcpy(*U + (size_t)k * M, uu[k], sizeof(double) * M);
            for (int j = 0; j < N; j++)
                (*V)[(size_t)rank * j + k] = vv[k][j];
        }
    }
    for (int j = 0; j < nuv; j++) {
        free(uu[j]);
        free(vv[j]);
    }
    free(uu);
    free(vv);
    free(vrow);
    free(vcol);
    return rank;
}

/* ------------------------------------------------------------------ */
/* H-matrix assembly                                                   */
/* ------------------------------------------------------------------ */
typedef struct {
    int oi, oj, m, n, rank;
    double *U, *V; /* U m x rank col-major, V rank x n col-major (ld = rank) */
} orc_lr;
typedef struct {
    int oi, oj, m, n;
    double *D; /* m x n col-major */
} orc_dense;

typedef struct {
    orc_lr *lr;
    int nlr, caplr;
    orc_dense *dn;
    int ndn, capdn;
    int false_positive;
} orc_leafset;

typedef struct {
    orc_tree *T, *S;
    int nr, nc, kernel;
    int rank, loff, lsize; /* local target rows of `rank` (local_offset, local_size) */
    double eps, eta;
    const double *xt, *xs;
    orc_leafset L;
    double build_seconds;
} orc_hmat;

static void orc_add_lr(orc_leafset *L, orc_lr v) {
    if (L->nlr == L->caplr) {
        L->caplr = L->caplr ? 2 * L->caplr : 64;
        L->lr    = (orc_lr *)realloc(L->lr, sizeof(orc_lr) * L->caplr);
    }
    L->lr[L->nlr++] = v;
}

/* HMatrix::AddNearFieldMat (hmatrix.hpp:701-716) */
static void orc_add_dense(orc_hmat *H, orc_leafset *L, int t, int s) {
    orc_node *tn = &H->T->nodes[t], *sn = &H->S->nodes[s];
    orc_dense d;
    d.oi = tn->offset;
    d.oj = sn->offset;
    d.m  = tn->size;
    d.n  = sn->size;
    d.D  = (double *)malloc(sizeof(double) * (size_t)d.m * d.n + 8);
    orc_copy_submatrix(H->kernel, H->xt, H->xs, d.m, d.n, H->T->perm + d.oi, H->S->perm + d.oj, d.D);
    if (L->ndn == L->capdn) {
        L->capdn = L->capdn ? 2 * L->capdn : 64;
        L->dn    = (orc_dense *)realloc(L->dn, sizeof(orc_dense) * L->capdn);
    }
    L->dn[L->ndn++] = d;
}

/* HMatrix::ComputeAdmissibleBlock (hmatrix.hpp:504-607); returns 1 = not pushed */
static int orc_compute_adm(orc_hmat *H, orc_leafset *L, int t, int s, int adm) {
    orc_node *tn = &H->T->nodes[t], *sn = &H->S->nodes[s];
    if (adm) {
        double *U, *V;
        int rank = orc_partial_aca(H->kernel, H->xt, H->xs, H->eps, -1, tn->size, sn->size, H->T->perm + tn->offset, H->S->perm + sn->offset, tn->ctr, &U, &V);
        if (rank != -1) {
            orc_lr v = {tn->offset, sn->offset, tn->size, sn->size, rank, U, V};
            orc_add_lr(L, v);
            return 0;
        }
        L->false_positive++;
    }
    size_t bsize = (size_t)tn->size * (size_t)sn->size;
    int split_t;
    if (sn->nb_sons == 0) {
        if (tn->nb_sons == 0)
            return 1;
        split_t = 1;
    } else if (tn->nb_sons == 0) {
        split_t = 0;
    } else {
        split_t = tn->size > sn->size;
    }
    int ns    = split_t ? tn->nb_sons : sn->nb_sons;
    int first = split_t ? tn->first_son : sn->first_son;
    int *np   = (int *)malloc(sizeof(int) * ns);
    int all   = 1;
    for (int p = 0; p < ns; p++) {
        int tt = split_t ? first + p : t, ss = split_t ? s : first + p;
        np[p]  = orc_compute_adm(H, L, tt, ss, orc_admissible(&H->T->nodes[tt], &H->S->nodes[ss], H->eta));
        all    = all && np[p];
    }
    int ret;
    if (bsize <= 1000000 && all) {
        ret = 1;
    } else {
        for (int p = 0; p < ns; p++)
            if (np[p])
                orc_add_dense(H, L, split_t ? first + p : t, split_t ? s : first + p);
        ret = 0;
    }
    free(np);
    return ret;
}

static int orc_lr_cmp(const void *a, const void *b) {
    const orc_lr *x = (const orc_lr *)a, *y = (const orc_lr *)b;
    if (x->oi != y->oi)
        return x->oi < y->oi ? -1 : 1;
    return x->oj < y->oj ? -1 : (x->oj > y->oj);
}
static int orc_dn_cmp(const void *a, const void *b) {
    const orc_dense *x = (const orc_dense *)a, *y = (const orc_dense *)b;
    if (x->oi != y->oi)
        return x->oi < y->oi ? -1 : 1;
    return x->oj < y->oj ? -1 : (x->oj > y->oj);
}

static double orc_now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* HMatrix(t, s, eps, eta, 'N', 'N') with partialACA, then build(gen, xt, xs)
 * (hmatrix.hpp:115, 286-341, 423-501) as rank `rank` of the run the cluster
 * trees were built for: the leaves of its local tasks only, local rows
 * (local_offset, local_size) = its depth-1 target cluster
 * (hmatrix.hpp:320-321).  OpenMP over local tasks as upstream. */
void *orc_hmatrix_build_rank(void *ct, void *cs, int nr, const double *xt, int nc, const double *xs, int kernel, double eps, double eta, int rank) {
    orc_hmat *H = (orc_hmat *)calloc(1, sizeof(orc_hmat));
    H->T        = (orc_tree *)ct;
    H->S        = (orc_tree *)cs;
    {
        orc_node *root = &H->T->nodes[0];
        orc_node *loc  = &H->T->nodes[root->first_son + rank];
        H->rank        = rank;
        H->loff        = loc->offset;
        H->lsize       = loc->size;
    }
    H->nr       = nr;
    H->nc       = nc;
    H->kernel   = kernel;
    H->eps      = eps;
    H->eta      = eta;
    H->xt       = xt;
    H->xs       = xs;
    double t0   = orc_now();
    orc_tasks tasks = orc_block_build(H->T, H->S, eta, rank);
    int ntask       = tasks.n;
    orc_leafset *per = (orc_leafset *)calloc(ntask ? ntask : 1, sizeof(orc_leafset));
#pragma omp parallel for schedule(guided)
    for (int p = 0; p < ntask; p++) {
        orc_task tk = tasks.v[p];
        if (!tk.adm) {
            orc_add_dense(H, &per[p], tk.t, tk.s);
        } else if (orc_compute_adm(H, &per[p], tk.t, tk.s, 1)) {
            orc_add_dense(H, &per[p], tk.t, tk.s);
        }
    }
    for (int p = 0; p < ntask; p++) {
        for (int b = 0; b < per[p].nlr; b++)
            orc_add_lr(&H->L, per[p].lr[b]);
        for (int b = 0; b < per[p].ndn; b++) {
            if (H->L.ndn == H->L.capdn) {
                H->L.capdn = H->L.capdn ? 2 * H->L.capdn : 64;
                H->L.dn    = (orc_dense *)realloc(H->L.dn, sizeof(orc_dense) * H->L.capdn);
            }
            H->L.dn[H->L.ndn++] = per[p].dn[b];
        }
        H->L.false_positive += per[p].false_positive;
        free(per[p].lr);
        free(per[p].dn);
    }
    free(per);
    free(tasks.v);
    qsort(H->L.lr, H->L.nlr, sizeof(orc_lr), orc_lr_cmp);
    qsort(H->L.dn, H->L.ndn, sizeof(orc_dense), orc_dn_cmp);
    H->build_seconds = orc_now() - t0;
    return H;
}

void *orc_hmatrix_build(void *ct, void *cs, int nr, const double *xt, int nc, const double *xs, int kernel, double eps, double eta) {
    return orc_hmatrix_build_rank(ct, cs, nr, xt, nc, xs, kernel, eps, eta, 0);
}

void orc_hmatrix_local(void *p, int *offset, int *size) {
    orc_hmat *H = (orc_hmat *)p;
    *offset     = H->loff;
    *size       = H->lsize;
}

void orc_hmatrix_free(void *p) {
    orc_hmat *H = (orc_hmat *)p;
    for (int b = 0; b < H->L.nlr; b++) {
        free(H->L.lr[b].U);
        free(H->L.lr[b].V);
    }
    for (int b = 0; b < H->L.ndn; b++)
        free(H->L.dn[b].D);
    free(H->L.lr);
    free(H->L.dn);
    free(H);
}

double orc_hmatrix_build_seconds(void *p) { return ((orc_hmat *)p)->build_seconds; }

void orc_hmatrix_counts(void *p, int *nlr, int *nd, int *false_positive) {
    orc_hmat *H = (orc_hmat *)p;
    *nlr        = H->L.nlr;
    *nd         = H->L.ndn;
    if (false_positive)
        *false_positive = H->L.false_positive;
}

/* same layouts as the reference driver */
void orc_hmatrix_leaves(void *p, int *lr, int *dn) {
    orc_hmat *H = (orc_hmat *)p;
    for (int b = 0; b < H->L.nlr; b++) {
        orc_lr *v     = &H->L.lr[b];
        lr[5 * b + 0] = v->oi;
        lr[5 * b + 1] = v->oj;
        lr[5 * b + 2] = v->m;
        lr[5 * b + 3] = v->n;
        lr[5 * b + 4] = v->rank;
    }
    for (int b = 0; b < H->L.ndn; b++) {
        orc_dense *v  = &H->L.dn[b];
        dn[4 * b + 0] = v->oi;
        dn[4 * b + 1] = v->oj;
        dn[4 * b + 2] = v->m;
        dn[4 * b + 3] = v->n;
    }
}

void orc_hmatrix_factors(void *p, double *uv, double *dense) {
    orc_hmat *H = (orc_hmat *)p;
    size_t o    = 0;
    if (uv)
        for (int b = 0; b < H->L.nlr; b++) {
            orc_lr *v = &H->L.lr[b];
            memcpy(uv + o, v->U, sizeof(double) * (size_t)v->m * v->rank);
            o += (size_t)v->m * v->rank;
            memcpy(uv + o, v->V, sizeof(double) * (size_t)v->n * v->rank);
            o += (size_t)v->n * v->rank;
        }
    o = 0;
    if (dense)
        for (int b = 0; b < H->L.ndn; b++) {
            orc_dense *v = &H->L.dn[b];
            memcpy(dense + o, v->D, sizeof(double) * (size_t)v->m * v->n);
            o += (size_t)v->m * v->n;
        }
}

/* ------------------------------------------------------------------ */
/* H-matrix product                                                    */
/* ------------------------------------------------------------------ */
/* mvprod_global_to_global (hmatrix.hpp:1074-1182) for one rank: gather x
 * through the source permutation, accumulate every leaf into a per-thread
 * buffer (hmatrix.hpp:844-911; LowRankMatrix::add_mvprod_row_major =
 * V-gemv then U-gemv, lrmat.hpp:89-100), reduce, scatter through the target
 * permutation.  x and y hold mu column-major right-hand sides. */
/* the leaf loop of mymvprod_global_to_local (hmatrix.hpp:844-911): xp is
 * the input in cluster numbering (nc per right-hand side), yp receives rows
 * row0 .. row0 + nrows (nrows per right-hand side, zeroed here) */
static void orc_apply_leaves(orc_hmat *H, const double *xp, double *yp, int mu, int row0, int nrows) {
    int nc = H->nc;
    memset(yp, 0, sizeof(double) * (size_t)nrows * mu);
    int nlr = H->L.nlr, ndn = H->L.ndn;
#pragma omp parallel
    {
        double *tmp = (double *)calloc((size_t)nrows * mu + 1, sizeof(double));
        double a[4096];
#pragma omp for schedule(guided) nowait
        for (int b = 0; b < nlr + ndn; b++) {
            for (int c = 0; c < mu; c++) {
                const double *xs = xp + (size_t)c * nc;
                double *ys       = tmp + (size_t)c * nrows;
                if (b < nlr) {
                    orc_lr *v = &H->L.lr[b];
                    int r     = v->rank;
                    double *ap = r <= 4096 ? a : (double *)malloc(sizeof(double) * r);
                    for (int k = 0; k < r; k++)
                        ap[k] = 0;
                    for (int j = 0; j < v->n; j++) {
                        double xj       = xs[v->oj + j];
                        const double *col = v->V + (size_t)r * j;
                        for (int k = 0; k < r; k++)
                            ap[k] += col[k] * xj;
                    }
                    for (int k = 0; k < r; k++) {
                        const double *col = v->U + (size_t)v->m * k;
                        double ak         = ap[k];
                        for (int i = 0; i < v->m; i++)
                            ys[v->oi - row0 + i] += col[i] * ak;
                    }
                    if (ap != a)
                        free(ap);
                } else {
                    orc_dense *v = &H->L.dn[b - nlr];
                    for (int j = 0; j < v->n; j++) {
                        double xj         = xs[v->oj + j];
                        const double *col = v->D + (size_t)v->m * j;
                        for (int i = 0; i < v->m; i++)
                            ys[v->oi - row0 + i] += col[i] * xj;
                    }
                }
            }
        }
#pragma omp critical
        {
            for (size_t i = 0; i < (size_t)nrows * mu; i++)
                yp[i] += tmp[i];
        }
        free(tmp);
    }
}

/* mvprod_global_to_global (hmatrix.hpp:1074-1182) for one rank: gather x
 * through the source permutation, accumulate every leaf into a per-thread
 * buffer (hmatrix.hpp:844-911; LowRankMatrix::add_mvprod_row_major =
 * V-gemv then U-gemv, lrmat.hpp:89-100), reduce, scatter through the target
 * permutation.  x and y hold mu column-major right-hand sides. */
void orc_hmatrix_mvprod(void *p, const double *x, double *y, int mu) {
    orc_hmat *H = (orc_hmat *)p;
    int nr = H->nr, nc = H->nc;
    double *xp = (double *)malloc(sizeof(double) * (size_t)nc * mu);
    double *yp = (double *)malloc(sizeof(double) * (size_t)nr * mu + 8);
    for (int c = 0; c < mu; c++)
        for (int i = 0; i < nc; i++)
            xp[(size_t)c * nc + i] = x[(size_t)c * nc + H->S->perm[i]];
    orc_apply_leaves(H, xp, yp, mu, 0, nr);
    for (int c = 0; c < mu; c++)
        for (int i = 0; i < nr; i++)
            y[(size_t)c * nr + H->T->perm[i]] = yp[(size_t)c * nr + i];
    free(xp);
    free(yp);
}

/* mymvprod_global_to_local (hmatrix.hpp:844-911): x is the whole input in
 * cluster numbering (what local_to_global_source all-gathers,
 * hmatrix.hpp:963-977), y the rank's local target rows local_offset ..
 * local_offset + local_size; both column-major per right-hand side */
void orc_hmatrix_mvprod_global_to_local(void *p, const double *x, double *y, int mu) {
    orc_hmat *H = (orc_hmat *)p;
    orc_apply_leaves(H, x, y, mu, H->loff, H->lsize);
}

/* median wall time of reps products after one warm-up */
double orc_hmatrix_time_mvprod(void *p, const double *x, double *y, int mu, int reps) {
    orc_hmatrix_mvprod(p, x, y, mu);
    double *t = (double *)malloc(sizeof(double) * reps);
    for (int i = 0; i < reps; i++) {
        double t0 = orc_now();
        orc_hmatrix_mvprod(p, x, y, mu);
        t[i] = orc_now() - t0;
    }
    for (int i = 1; i < reps; i++)
        for (int j = i; j > 0 && t[j] < t[j - 1]; j--) {
            double s = t[j];
            t[j]     = t[j - 1];
            t[j - 1] = s;
        }
    double m = t[reps / 2];
    free(t);
    return m;
}

/* dense rows of the kernel matrix (user numbering) times x: sampled oracle */
void orc_dense_rows_mvprod(int kernel, int nc, const double *xt, const double *xs, int nrows, const int *rows, const double *x, double *out) {
#pragma omp parallel for schedule(static)
    for (int a = 0; a < nrows; a++) {
        double s = 0;
        for (int j = 0; j < nc; j++)
            s += orc_kernel_d(kernel, xt + 3 * (size_t)rows[a], xs + 3 * (size_t)j) * x[j];
        out[a] = s;
    }
}

int orc_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void orc_set_num_threads(int n) {
#ifdef _OPENMP
    omp_set_num_threads(n);
#else
    (void)n;
#endif
}
