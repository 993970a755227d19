/*
 * gh_oracle.c -- CPU oracle for the GravHopper force path.  TEST INFRASTRUCTURE ONLY.
 *
 * This file restates, in plain C, the arithmetic of the reference extension
 * gravhopper/_jbgrav.c so that the CUDA engine can be checked against it on
 * identical inputs.  It is used only by tests/, by __graft_entry__.smoke() and by the
 * CPU-baseline leg of bench.py.  The product path never links or calls it.
 *
 * Differences from the reference that do not change results:
 *   - O(N) memory: the reference materialises N*N*3 + N*N doubles of temporaries
 *     (_jbgrav.c:148-149, 307-308); here each target walks the sources directly, in
 *     the same ascending-j order and with the same operation order, so every
 *     output bit is the same.
 *   - Targets are split over P pthreads.  Each target is computed by one thread
 *     in the reference's order, so the result does not depend on P.
 *   - The octree lives in flat arrays instead of malloc'd nodes; the insertion
 *     order, the centre recurrence, the moment accumulation order and the walk's
 *     summation order are those of _jbgrav.c:360-541, 737-806.
 *   - Pathological inputs that make the reference recurse without bound
 *     (duplicate positions, _jbgrav.c:401-413) return GHOR_ERR_DEPTH instead.
 *
 * Build with -ffp-contract=off: the reference's own build (setup.py, no extra
 * flags) on x86-64 has no FMA instructions, and contracting a*b+c on aarch64 would
 * change the last bit.
 */
#include <math.h>
#include <pthread.h>
#include <time.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#define GHOR_OK 0
#define GHOR_ERR_ARG 1
#define GHOR_ERR_OOM 2
#define GHOR_ERR_DEPTH 3

/* ------------------------------------------------------------------------- */
/* Direct summation                                                           */
/* ------------------------------------------------------------------------- */

/*
 * One target against all sources.
 * self_index >= 0: the target is source self_index; that source is skipped and no
 *   zero guard is applied (directsummation_workhorse, _jbgrav.c:155-185).
 * self_index <  0: all sources are summed; r^2+eps^2 == 0 gives a zero term
 *   (directsummation_position_workhorse, _jbgrav.c:314-345).
 * Per pair: d = x_j - x_i (the reference stores -(x_i - x_j), which is the same
 * IEEE value), r2 = ((dx*dx + dy*dy) + dz*dz), s = r2 + eps^2,
 * inv = 1/s/sqrt(s), acc_k += (m_j*d_k)*inv, j ascending.
 */
static void direct_one(const double *pos, const double *mass, int64_t np,
                       const double *t, int64_t self_index, double eps2,
                       double *out)
{
    double ax = 0.0, ay = 0.0, az = 0.0;
    const double tx = t[0], ty = t[1], tz = t[2];
    for (int64_t j = 0; j < np; j++) {
        if (j == self_index) continue;
        double dx = pos[3 * j + 0] - tx;
        double dy = pos[3 * j + 1] - ty;
        double dz = pos[3 * j + 2] - tz;
        double r2 = dx * dx;
        r2 = r2 + dy * dy;
        r2 = r2 + dz * dz;
        double s = r2 + eps2;
        double inv;
        if (self_index < 0 && s == 0.0)
            inv = 0.0;
        else
            inv = 1.0 / s / sqrt(s);
        double m = mass[j];
        ax = ax + (m * dx) * inv;
        ay = ay + (m * dy) * inv;
        az = az + (m * dz) * inv;
    }
    out[0] = ax;
    out[1] = ay;
    out[2] = az;
}

/* ------------------------------------------------------------------------- */
/* Octree                                                                     */
/* ------------------------------------------------------------------------- */

typedef struct {
    double center[3];
    double size, halfsize;
    double mass;
    double firstmoment[3];
    double com[3];
    int32_t branches[8];
    int64_t leaf;   /* particle index if this node holds exactly one particle, else -1 */
    int32_t empty;
} ornode;

typedef struct {
    ornode *nodes;
    int64_t count, cap;
    const double *pos, *mass;
} ortree;

static int64_t ortree_new_node(ortree *t, const double *center, double size)
{
    if (t->count == t->cap) {
        int64_t ncap = t->cap ? 2 * t->cap : 1024;
        ornode *nn = (ornode *)realloc(t->nodes, sizeof(ornode) * (size_t)ncap);
        if (!nn) return -1;
        t->nodes = nn;
        t->cap = ncap;
    }
    ornode *n = &t->nodes[t->count];
    /* gravoct_init, _jbgrav.c:360-384 */
    n->size = size;
    n->halfsize = 0.5 * size;
    for (int i = 0; i < 3; i++) {
        n->center[i] = center[i];
        n->firstmoment[i] = 0.0;
        n->com[i] = 0.0;
    }
    for (int i = 0; i < 8; i++) n->branches[i] = -1;
    n->mass = 0.0;
    n->empty = 1;
    n->leaf = -1;
    return t->count++;
}

/* gravoct_calc_subnode + gravoct_calc_branchnum, _jbgrav.c:441-462: ties go low. */
static int branch_of(const ornode *n, const double *p, double *subcenter)
{
    int b = 0;
    for (int i = 0; i < 3; i++) {
        double sgn;
        if (p[i] > n->center[i]) {
            b += (1 << i);
            sgn = 1.0;
        } else {
            sgn = -1.0;
        }
        /* subcenter = center + subnode*0.5*halfsize, _jbgrav.c:406 and :426 */
        subcenter[i] = n->center[i] + sgn * 0.5 * n->halfsize;
    }
    return b;
}

static void make_leaf(ortree *t, int64_t node, int64_t p)
{
    ornode *n = &t->nodes[node];
    const double m = t->mass[p];
    n->empty = 0;
    n->leaf = p;
    n->mass = m;
    for (int i = 0; i < 3; i++) n->firstmoment[i] = m * t->pos[3 * p + i];
}

/*
 * gravoct_add_particle, _jbgrav.c:387-437, as a loop.  The reference updates an
 * internal node's moments after recursing into the child; each node still sees
 * its particles in insertion order, which is all that matters for the sums.
 */
static int ortree_insert(ortree *t, int64_t p, int maxdepth)
{
    int64_t node = 0;
    int depth = 0;
    const double *pp = &t->pos[3 * p];
    for (;;) {
        if (t->nodes[node].empty) {
            make_leaf(t, node, p);
            return GHOR_OK;
        }
        if (t->nodes[node].leaf >= 0) {
            /* push the resident particle one level down, then re-add p here */
            int64_t q = t->nodes[node].leaf;
            double sc[3];
            int b = branch_of(&t->nodes[node], &t->pos[3 * q], sc);
            int64_t c = ortree_new_node(t, sc, t->nodes[node].halfsize);
            if (c < 0) return GHOR_ERR_OOM;
            t->nodes[node].branches[b] = (int32_t)c;
            make_leaf(t, c, q);
            t->nodes[node].leaf = -1;
            continue;
        }
        double sc[3];
        int b = branch_of(&t->nodes[node], pp, sc);
        ornode *n = &t->nodes[node];
        n->mass += t->mass[p];
        for (int i = 0; i < 3; i++) n->firstmoment[i] += t->mass[p] * pp[i];
        int64_t c = n->branches[b];
        if (c < 0) {
            c = ortree_new_node(t, sc, n->halfsize);
            if (c < 0) return GHOR_ERR_OOM;
            t->nodes[node].branches[b] = (int32_t)c;
        }
        node = c;
        if (++depth > maxdepth) return GHOR_ERR_DEPTH;
    }
}

/* gravoct_finalize, _jbgrav.c:467-483 */
static void ortree_finalize(ortree *t)
{
    for (int64_t k = 0; k < t->count; k++) {
        ornode *n = &t->nodes[k];
        if (n->leaf >= 0) {
            for (int i = 0; i < 3; i++) n->com[i] = t->pos[3 * n->leaf + i];
        } else {
            for (int i = 0; i < 3; i++) n->com[i] = n->firstmoment[i] / n->mass;
        }
    }
}

/* gravoct_calc_accel, _jbgrav.c:487-541 (recursive, children summed in branch order) */
static void ortree_accel(const ortree *t, int64_t node, const double *p, double eps2,
                         double theta, double *force)
{
    const ornode *n = &t->nodes[node];
    double node_dist = 0.0;
    for (int i = 0; i < 3; i++)
        node_dist += (n->center[i] - p[i]) * (n->center[i] - p[i]);
    node_dist = sqrt(node_dist);
    if (n->leaf >= 0 || (n->size / node_dist) < theta) {
        double d[3], r2 = 0.0;
        for (int i = 0; i < 3; i++) {
            d[i] = n->com[i] - p[i];
            r2 += d[i] * d[i];
        }
        double s = r2 + eps2;
        double inv = (s == 0.0) ? 0.0 : 1.0 / s / sqrt(s);
        for (int i = 0; i < 3; i++) force[i] = d[i] * n->mass * inv;
    } else {
        double bf[3];
        force[0] = force[1] = force[2] = 0.0;
        for (int j = 0; j < 8; j++) {
            if (n->branches[j] >= 0) {
                ortree_accel(t, n->branches[j], p, eps2, theta, bf);
                for (int i = 0; i < 3; i++) force[i] += bf[i];
            }
        }
    }
}

/* treeforce_workhorse bounding box and root cell, _jbgrav.c:746-775 */
static void root_cell(const double *pos, int64_t np, double eps, double *center,
                      double *boxsize)
{
    double mn[3], mx[3];
    for (int i = 0; i < 3; i++) mn[i] = mx[i] = pos[i];
    for (int64_t k = 1; k < np; k++) {
        for (int j = 0; j < 3; j++) {
            double q = pos[3 * k + j];
            if (q < mn[j]) mn[j] = q;
            if (q > mx[j]) mx[j] = q;
        }
    }
    double bs = mx[0] - mn[0] + eps;
    for (int i = 1; i < 3; i++)
        if ((mx[i] - mn[i]) > bs) bs = mx[i] - mn[i] + eps;
    for (int i = 0; i < 3; i++) center[i] = 0.5 * (mn[i] + mx[i]);
    *boxsize = bs;
}

/* ------------------------------------------------------------------------- */
/* Threading over targets                                                     */
/* ------------------------------------------------------------------------- */

typedef struct {
    int kind; /* 0 direct, 1 tree */
    const double *pos, *mass, *tpos;
    int64_t np, nt;
    int self_mode;
    double eps, theta;
    const ortree *tree;
    double *out;
    int64_t t0, t1;
} job;

static void *run_job(void *arg)
{
    job *jb = (job *)arg;
    const double eps2 = jb->eps * jb->eps;
    for (int64_t i = jb->t0; i < jb->t1; i++) {
        if (jb->kind == 0) {
            direct_one(jb->pos, jb->mass, jb->np, &jb->tpos[3 * i],
                       jb->self_mode ? i : -1, eps2, &jb->out[3 * i]);
        } else {
            ortree_accel(jb->tree, 0, &jb->tpos[3 * i], eps2, jb->theta, &jb->out[3 * i]);
        }
    }
    return NULL;
}

static void run_threads(job *proto, int nthreads)
{
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if (proto->nt < nthreads) nthreads = proto->nt > 0 ? (int)proto->nt : 1;
    job jobs[256];
    pthread_t th[256];
    int64_t per = (proto->nt + nthreads - 1) / nthreads;
    for (int k = 0; k < nthreads; k++) {
        jobs[k] = *proto;
        jobs[k].t0 = k * per < proto->nt ? k * per : proto->nt;
        jobs[k].t1 = (k + 1) * per < proto->nt ? (k + 1) * per : proto->nt;
    }
    for (int k = 1; k < nthreads; k++) pthread_create(&th[k], NULL, run_job, &jobs[k]);
    run_job(&jobs[0]);
    for (int k = 1; k < nthreads; k++) pthread_join(th[k], NULL);
}

/* ------------------------------------------------------------------------- */
/* Public oracle entry points                                                 */
/* ------------------------------------------------------------------------- */

/*
 * Direct summation.  self_mode=1 follows _jbgrav.direct_summation (targets are the
 * sources, j == i skipped); self_mode=0 follows direct_summation_position.
 * Sources are read from `pos`; targets from `tpos` (ignored when self_mode=1).
 */
int ghor_direct(const double *pos, const double *mass, int64_t np, const double *tpos,
                int64_t nt, double eps, int self_mode, double *out, int nthreads)
{
    if (np < 0 || nt < 0) return GHOR_ERR_ARG;
    job j;
    memset(&j, 0, sizeof(j));
    j.kind = 0;
    j.pos = pos;
    j.mass = mass;
    j.np = np;
    j.self_mode = self_mode;
    j.tpos = self_mode ? pos : tpos;
    j.nt = self_mode ? np : nt;
    j.eps = eps;
    j.out = out;
    run_threads(&j, nthreads);
    return GHOR_OK;
}

/*
 * Barnes-Hut tree force (treeforce_workhorse, _jbgrav.c:737-806).  tpos may equal
 * pos (tree_force) or hold separate points (tree_force_position).  np == 0 gives
 * zeros (the reference reads pos[0] out of bounds there).
 */
static double now_s(void)
{
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* times_out (optional, 2 doubles): seconds spent building the tree and walking it. */
int ghor_tree(const double *pos, const double *mass, int64_t np, const double *tpos,
              int64_t nt, double eps, double theta, double *out, int nthreads,
              int maxdepth, int64_t *nnodes_out, double *times_out)
{
    double t0 = now_s();
    if (np < 0 || nt < 0) return GHOR_ERR_ARG;
    if (np == 0) {
        memset(out, 0, sizeof(double) * 3 * (size_t)nt);
        if (nnodes_out) *nnodes_out = 0;
        return GHOR_OK;
    }
    ortree t;
    memset(&t, 0, sizeof(t));
    t.pos = pos;
    t.mass = mass;
    double c[3], bs;
    root_cell(pos, np, eps, c, &bs);
    if (ortree_new_node(&t, c, bs) < 0) return GHOR_ERR_OOM;
    for (int64_t p = 0; p < np; p++) {
        int rc = ortree_insert(&t, p, maxdepth);
        if (rc != GHOR_OK) {
            free(t.nodes);
            return rc;
        }
    }
    ortree_finalize(&t);
    double t1 = now_s();
    if (nnodes_out) *nnodes_out = t.count;
    job j;
    memset(&j, 0, sizeof(j));
    j.kind = 1;
    j.tree = &t;
    j.tpos = tpos;
    j.nt = nt;
    j.eps = eps;
    j.theta = theta;
    j.out = out;
    run_threads(&j, nthreads);
    if (times_out) {
        times_out[0] = t1 - t0;
        times_out[1] = now_s() - t1;
    }
    free(t.nodes);
    return GHOR_OK;
}

/*
 * Softened potential energy  sum_{i<j} -m_i m_j / sqrt(r^2+eps^2)  in code units
 * (G=1), accumulated per i in ascending j and then over i in ascending order.
 * The reference has no energy routine; this is the diagnostic the engine reports.
 */
int ghor_potential(const double *pos, const double *mass, int64_t np, double eps,
                   double *phi_out)
{
    const double eps2 = eps * eps;
    double tot = 0.0;
    for (int64_t i = 0; i < np; i++) {
        double acc = 0.0;
        for (int64_t j = i + 1; j < np; j++) {
            double dx = pos[3 * j] - pos[3 * i];
            double dy = pos[3 * j + 1] - pos[3 * i + 1];
            double dz = pos[3 * j + 2] - pos[3 * i + 2];
            double s = dx * dx + dy * dy + dz * dz + eps2;
            if (s > 0.0) acc += mass[j] / sqrt(s);
        }
        tot += mass[i] * acc;
    }
    *phi_out = -tot;
    return GHOR_OK;
}
