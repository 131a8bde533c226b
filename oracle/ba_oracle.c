/*
 * CPU restatement of zeroslam's factor-graph bundle adjustment (the oracle).
 * TEST INFRASTRUCTURE ONLY: see ba_oracle.h. Every function names the
 * reference lines it follows.
 */
#include "ba_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ---------------------------------------------------------------- threads
 * The restatement may spread its loops over host threads. Every floating-point
 * value is still computed by the same operations in the same order as with one
 * thread (threads own disjoint outputs; sums keep their serial order), so the
 * results are bit-for-bit those of the serial restatement for any thread count. */

static int g_threads = 1;

void zso_set_threads(int n) { g_threads = n < 1 ? 1 : (n > 256 ? 256 : n); }
int zso_get_threads(void) { return g_threads; }

typedef void (*range_fn)(void* ctx, long long lo, long long hi);

typedef struct range_job {
    range_fn fn;
    void* ctx;
    long long lo, hi;
} range_job;

static void* range_run(void* a) {
    range_job* j = (range_job*)a;
    j->fn(j->ctx, j->lo, j->hi);
    return NULL;
}

/* fn over [bounds[t], bounds[t+1]) for t < parts, one thread each (the caller
 * runs part 0). */
static void run_parts(range_fn fn, void* ctx, const long long* bounds, int parts) {
    range_job jobs[256];
    pthread_t tid[256];
    int started[256];
    for (int t = 0; t < parts; ++t) {
        jobs[t].fn = fn; jobs[t].ctx = ctx; jobs[t].lo = bounds[t]; jobs[t].hi = bounds[t + 1];
        started[t] = 0;
    }
    for (int t = 1; t < parts; ++t) started[t] = pthread_create(&tid[t], NULL, range_run, &jobs[t]) == 0;
    range_run(&jobs[0]);
    for (int t = 1; t < parts; ++t) {
        if (started[t]) pthread_join(tid[t], NULL);
        else range_run(&jobs[t]); /* no thread to be had: run the part here */
    }
}

/* fn over [0, n) in g_threads equal contiguous parts (serial below min_n). */
static void parallel_for(long long n, long long min_n, range_fn fn, void* ctx) {
    int parts = g_threads;
    if (n < min_n || parts <= 1) parts = 1;
    if (parts > n) parts = (int)(n > 0 ? n : 1);
    long long bounds[257];
    for (int t = 0; t <= parts; ++t) bounds[t] = n * t / parts;
    run_parts(fn, ctx, bounds, parts);
}

#define PENALTY 0.3 /* source/factor_graph.hpp:981 */

/* ---------------------------------------------------------------- lie / camera */

/* Quaternion product (w, x, y, z), term order of source/lie.hpp:337-344. */
static void qmul(const double a[4], const double b[4], double o[4]) {
    o[0] = a[0] * b[0] - a[1] * b[1] - a[2] * b[2] - a[3] * b[3];
    o[1] = a[0] * b[1] + a[1] * b[0] + a[2] * b[3] - a[3] * b[2];
    o[2] = a[0] * b[2] - a[1] * b[3] + a[2] * b[0] + a[3] * b[1];
    o[3] = a[0] * b[3] + a[1] * b[2] - a[2] * b[1] + a[3] * b[0];
}

/* Rotate a point by q (w, x, y, z) as q (0, p) q*, source/lie.hpp:347-362;
 * the quaternion is not normalised. */
static void qrotate(const double q[4], const double p[3], double o[3]) {
    const double pq[4] = {0.0, p[0], p[1], p[2]};
    const double qc[4] = {q[0], -q[1], -q[2], -q[3]};
    double t[4], r[4];
    qmul(q, pq, t);
    qmul(t, qc, r);
    o[0] = r[1];
    o[1] = r[2];
    o[2] = r[3];
}

/* Rotation matrix of q, source/lie.hpp:188-204 (assumes a unit quaternion). */
static void qmatrix(const double q[4], double R[9]) {
    const double tx = 2.0 * q[1], ty = 2.0 * q[2], tz = 2.0 * q[3];
    const double txx = tx * q[1], txy = tx * q[2], txz = tx * q[3], txw = tx * q[0];
    const double tyy = ty * q[2], tyz = ty * q[3], tyw = ty * q[0];
    const double tzz = tz * q[3], tzw = tz * q[0];
    R[0] = 1.0 - (tyy + tzz); R[1] = txy - tzw;         R[2] = txz + tyw;
    R[3] = txy + tzw;         R[4] = 1.0 - (txx + tzz); R[5] = tyz - txw;
    R[6] = txz - tyw;         R[7] = tyz + txw;         R[8] = 1.0 - (txx + tyy);
}

/* so3::exp, source/lie.hpp:247-264. */
static void so3_exp(const double w[3], double q[4]) {
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    double re, sc;
    if (th2 < 1e-6 * 1e-6) {
        const double th4 = th2 * th2;
        re = 1.0 - (1.0 / 8.0) * th2 + (1.0 / 384.0) * th4;
        sc = 0.5 - (1.0 / 48.0) * th2 + (1.0 / 3840.0) * th4;
    } else {
        const double th = sqrt(th2);
        const double h = 0.5 * th;
        re = cos(h);
        sc = sin(h) / th;
    }
    q[0] = re;
    q[1] = w[0] * sc;
    q[2] = w[1] * sc;
    q[3] = w[2] * sc;
}

/* so3::left_jacobian, source/lie.hpp:284-294. */
static void so3_left_jacobian(const double w[3], double J[9]) {
    const double th2 = w[0] * w[0] + w[1] * w[1] + w[2] * w[2];
    const double H[9] = {0.0, -w[2], w[1], w[2], 0.0, -w[0], -w[1], w[0], 0.0};
    double H2[9];
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) {
            double s = 0.0;
            for (int k = 0; k < 3; ++k) s += H[i * 3 + k] * H[k * 3 + j];
            H2[i * 3 + j] = s;
        }
    double a, b;
    if (th2 < 1e-6 * 1e-6) {
        a = 0.5;
        b = 1.0 / 6.0;
    } else {
        const double th = sqrt(th2);
        a = (1.0 - cos(th)) / th2;
        b = (th - sin(th)) / (th2 * th);
    }
    for (int i = 0; i < 9; ++i) J[i] = ((i % 4 == 0) ? 1.0 : 0.0) + a * H[i] + b * H2[i];
}

void zso_pose_plus(double p[7], const double d[6]) {
    /* vertex_pose::plus, source/factor_graph.hpp:947-960: T <- exp(d) T with
     * se3::exp (source/lie.hpp:446-450) and se3 * se3 (source/lie.hpp:521-526). */
    const double q[4] = {p[6], p[3], p[4], p[5]};
    const double t[3] = {p[0], p[1], p[2]};
    double dq[4], J[9], dt[3], nq[4], rt[3];
    so3_exp(d, dq);
    so3_left_jacobian(d, J);
    for (int i = 0; i < 3; ++i) dt[i] = J[i * 3 + 0] * d[3] + J[i * 3 + 1] * d[4] + J[i * 3 + 2] * d[5];
    qmul(dq, q, nq);
    qrotate(dq, t, rt);
    p[0] = rt[0] + dt[0];
    p[1] = rt[1] + dt[1];
    p[2] = rt[2] + dt[2];
    p[3] = nq[1];
    p[4] = nq[2];
    p[5] = nq[3];
    p[6] = nq[0];
}

int zso_edge(const double pose[7], const double X[3], const double uv[2], const double intr[4],
             double r[2], double Jp[12], double Jl[6]) {
    /* edge_reprojection::compute_residual / compute_jacobians,
     * source/factor_graph.hpp:990-1048, and pinhole::project, source/camera.hpp:91-126. */
    const double q[4] = {pose[6], pose[3], pose[4], pose[5]};
    double Xc[3];
    qrotate(q, X, Xc);
    Xc[0] += pose[0];
    Xc[1] += pose[1];
    Xc[2] += pose[2];
    double Jc[6];
    int front = !(Xc[2] < 1.0e-12);
    if (front) {
        const double iz = 1.0 / Xc[2];
        const double u = intr[0] * (Xc[0] * iz) + intr[2];
        const double v = intr[1] * (Xc[1] * iz) + intr[3];
        r[0] = uv[0] - u;
        r[1] = uv[1] - v;
        const double iz2 = iz * iz;
        Jc[0] = intr[0] * iz; Jc[1] = 0.0; Jc[2] = -intr[0] * Xc[0] * iz2;
        Jc[3] = 0.0; Jc[4] = intr[1] * iz; Jc[5] = -intr[1] * Xc[1] * iz2;
    } else {
        const double pen = -PENALTY * Xc[2];
        r[0] = pen;
        r[1] = pen;
        Jc[0] = 0.0; Jc[1] = 0.0; Jc[2] = PENALTY;
        Jc[3] = 0.0; Jc[4] = 0.0; Jc[5] = PENALTY;
    }
    if (Jp) {
        const double Xv = Xc[0], Yv = Xc[1], Zv = Xc[2];
        const double P[18] = {0.0, Zv, -Yv, 1.0, 0.0, 0.0,
                              -Zv, 0.0, Xv, 0.0, 1.0, 0.0,
                              Yv, -Xv, 0.0, 0.0, 0.0, 1.0};
        for (int i = 0; i < 2; ++i)
            for (int c = 0; c < 6; ++c) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += Jc[i * 3 + k] * P[k * 6 + c];
                Jp[i * 6 + c] = -s;
            }
    }
    if (Jl) {
        double R[9];
        qmatrix(q, R);
        for (int i = 0; i < 2; ++i)
            for (int c = 0; c < 3; ++c) {
                double s = 0.0;
                for (int k = 0; k < 3; ++k) s += Jc[i * 3 + k] * R[k * 3 + c];
                Jl[i * 3 + c] = -s;
            }
    }
    return front;
}

void zso_loss(int kind, double delta, double e2, double rho[3]) {
    /* source/factor_graph.hpp:851-934 */
    const double d2 = delta * delta;
    if (kind == 1) {
        if (e2 <= d2) {
            rho[0] = e2; rho[1] = 1.0; rho[2] = 0.0;
        } else {
            const double e = sqrt(e2);
            rho[0] = 2.0 * e * delta - d2;
            rho[1] = delta / e;
            rho[2] = -0.5 * rho[1] / e2;
        }
    } else if (kind == 2) {
        const double inv = 1.0 / d2;
        const double aux = inv * e2 + 1.0;
        rho[0] = d2 * log(aux);
        rho[1] = 1.0 / aux;
        rho[2] = -inv * (rho[1] * rho[1]);
    } else if (kind == 3) {
        if (e2 <= d2) {
            const double aux = e2 / d2;
            const double om = 1.0 - aux;
            const double om2 = om * om;
            const double om3 = om2 * om;
            rho[0] = d2 * (1.0 - om3) / 3.0;
            rho[1] = om2;
            rho[2] = -2.0 * om / d2;
        } else {
            rho[0] = d2 / 3.0; rho[1] = 0.0; rho[2] = 0.0;
        }
    } else {
        rho[0] = e2; rho[1] = 1.0; rho[2] = 0.0;
    }
}

static const double IDENT2[4] = {1.0, 0.0, 0.0, 1.0};

static double edge_chi2(const double r[2], const double* om) {
    /* r^T Omega r, source/factor_graph.hpp:217-219 */
    const double a = r[0] * om[0] + r[1] * om[2];
    const double b = r[0] * om[1] + r[1] * om[3];
    return a * r[0] + b * r[1];
}

static void chi2_terms(void* ctx, long long lo, long long hi) {
    const zso_problem* p = ((const zso_problem**)ctx)[0];
    double* term = ((double**)ctx)[1];
    for (long long o = lo; o < hi; ++o) {
        const double* pose = p->poses + 7LL * p->obs_pose[o];
        const double* X = p->landmarks + 3LL * p->obs_landmark[o];
        double r[2];
        zso_edge(pose, X, p->obs_uv + 2 * o, p->intrinsics, r, NULL, NULL);
        const double* om = p->obs_info ? p->obs_info + 4 * o : IDENT2;
        const double e2 = edge_chi2(r, om);
        double rho[3];
        zso_loss(p->loss_kind, p->loss_delta, e2, rho);
        term[o] = p->loss_kind ? rho[0] : e2;
    }
}

double zso_chi2(const zso_problem* p) {
    /* get_current_chi, source/factor_graph.hpp:618-629: the edges' robust
     * terms (in parallel), then their sum in edge order */
    double* term = malloc(((size_t)p->num_obs + 1) * sizeof(double));
    if (!term) return NAN;
    void* ctx[2] = {(void*)p, term};
    parallel_for(p->num_obs, 4096, chi2_terms, ctx);
    double total = 0.0;
    for (long long o = 0; o < p->num_obs; ++o) total += term[o];
    free(term);
    return total;
}

int zso_invert3(const double a[9], double o[9]) {
    /* matrix::invert<3>, source/matrix.hpp:749-774 */
    const double det = +a[0] * (a[4] * a[8] - a[7] * a[5]) - a[1] * (a[3] * a[8] - a[5] * a[6]) +
                       a[2] * (a[3] * a[7] - a[4] * a[6]);
    double scale = 0.0;
    for (int i = 0; i < 9; ++i) scale = fmax(scale, fabs(a[i]));
    if (!(fabs(det) > scale * scale * scale * 1e-12)) {
        memset(o, 0, 9 * sizeof(double));
        return 0;
    }
    const double id = 1.0 / det;
    o[0] = (a[4] * a[8] - a[7] * a[5]) * id;
    o[1] = (a[2] * a[7] - a[1] * a[8]) * id;
    o[2] = (a[1] * a[5] - a[2] * a[4]) * id;
    o[3] = (a[5] * a[6] - a[3] * a[8]) * id;
    o[4] = (a[0] * a[8] - a[2] * a[6]) * id;
    o[5] = (a[3] * a[2] - a[0] * a[5]) * id;
    o[6] = (a[3] * a[7] - a[6] * a[4]) * id;
    o[7] = (a[6] * a[1] - a[0] * a[7]) * id;
    o[8] = (a[0] * a[4] - a[3] * a[1]) * id;
    return 1;
}

typedef struct chol_ctx {
    const double* A;
    double* L;
    int n, i0;
} chol_ctx;

/* Rows i0 + [lo, hi) of the factor, columns k < i0 (rows < i0 are final):
 * the reference's formula for each entry, k outer so that each earlier row is
 * read once per part. */
static void chol_rows(void* c, long long lo, long long hi) {
    const chol_ctx* x = (const chol_ctx*)c;
    const int n = x->n;
    for (int k = 0; k < x->i0; ++k) {
        const double* Lk = x->L + (size_t)k * n;
        for (long long r = lo; r < hi; ++r) {
            const size_t i = (size_t)(x->i0 + r);
            double* Li = x->L + i * n;
            double v = x->A[i * n + k];
            for (int j = 0; j < k; ++j) v -= Li[j] * Lk[j];
            Li[k] = v / Lk[k];
        }
    }
}

int zso_cholesky(const double* A, int n, double* L) {
    /* decompose_cholesky, source/matrix_decomposition_cholesky.hpp:26-59: row
     * by row, L_ik = (A_ik - sum_{j<k} L_ij L_kj) / L_kk, then the pivot
     * A_ii - sum_{j<i} L_ij^2 must exceed 1e-14 max|A_ii|. Rows go in blocks of
     * 64: the columns left of a block depend only on earlier rows and are
     * formed for all its rows in parallel; the rest of the block follows row by
     * row. Each entry is the same sequence of operations as in the serial
     * loop; after a failed pivot the rows below it are zero, as there. */
    memset(L, 0, (size_t)n * n * sizeof(double));
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = fmax(scale, fabs(A[(size_t)i * n + i]));
    const double eps = scale * 1e-14;
    const int B = 64;
    for (int i0 = 0; i0 < n; i0 += B) {
        const int i1 = i0 + B < n ? i0 + B : n;
        if (i0 > 0) {
            chol_ctx c = {A, L, n, i0};
            parallel_for(i1 - i0, (long long)(n >= 512 ? 1 : B + 1), chol_rows, &c);
        }
        for (int i = i0; i < i1; ++i) {
            double* Li = L + (size_t)i * n;
            for (int k = i0; k < i; ++k) {
                const double* Lk = L + (size_t)k * n;
                double v = A[(size_t)i * n + k];
                for (int j = 0; j < k; ++j) v -= Li[j] * Lk[j];
                Li[k] = v / Lk[k];
            }
            double v = A[(size_t)i * n + i];
            for (int j = 0; j < i; ++j) v -= Li[j] * Li[j];
            if (!(v > eps)) {
                if (i + 1 < n) memset(L + (size_t)(i + 1) * n, 0, (size_t)(n - i - 1) * n * sizeof(double));
                return 0;
            }
            Li[i] = sqrt(v);
        }
    }
    return 1;
}

int zso_cholesky_solve(const double* L, const double* b, int n, double* x) {
    /* solve_cholesky, source/matrix_decomposition_cholesky.hpp:61-95 */
    double scale = 0.0;
    for (int i = 0; i < n; ++i) scale = fmax(scale, fabs(L[(size_t)i * n + i]));
    const double eps = scale * 1e-7;
    for (int i = 0; i < n; ++i) {
        x[i] = b[i];
        for (int j = 0; j < i; ++j) x[i] -= L[(size_t)i * n + j] * x[j];
        if (!(fabs(L[(size_t)i * n + i]) > eps)) return 0;
        x[i] /= L[(size_t)i * n + i];
    }
    for (int i = n; i-- > 0;) {
        for (int j = i + 1; j < n; ++j) x[i] -= L[(size_t)j * n + i] * x[j];
        if (!(fabs(L[(size_t)i * n + i]) > eps)) return 0;
        x[i] /= L[(size_t)i * n + i];
    }
    return 1;
}

/* ---------------------------------------------------------------- linearisation */

typedef struct lin {
    int K, L;
    double* hpp;   /* K*36 */
    double* hll;   /* L*9 */
    double* b;     /* 6K + 3L */
    /* H_pl blocks grouped by landmark, one per distinct non-fixed pose: */
    int* lm_ptr;   /* L+1 */
    int* blk_pose; /* nblk */
    double* hpl;   /* nblk*18 */
    int nblk;
} lin;

static void lin_free(lin* s) {
    free(s->hpp); free(s->hll); free(s->b); free(s->lm_ptr); free(s->blk_pose); free(s->hpl);
}

/* Per edge: r (2), J_p (12), J_l (6), the robust weight W (4), rho' and
 * Omega r (2). */
#define EDGE_TERMS 27

static void edge_terms(void* ctx, long long lo, long long hi) {
    const zso_problem* p = (const zso_problem*)((void**)ctx)[0];
    double* et = (double*)((void**)ctx)[1];
    for (long long o = lo; o < hi; ++o) {
        double* e = et + EDGE_TERMS * o;
        double* r = e;
        double* W = e + 20;
        const int pi = p->obs_pose[o], li = p->obs_landmark[o];
        zso_edge(p->poses + 7LL * pi, p->landmarks + 3LL * li, p->obs_uv + 2 * o, p->intrinsics, r, e + 2, e + 14);
        const double* om = p->obs_info ? p->obs_info + 4 * o : IDENT2;
        /* edge_base::robust_info, source/factor_graph.hpp:254-269 */
        for (int i = 0; i < 4; ++i) W[i] = om[i];
        double drho = 1.0;
        if (p->loss_kind) {
            const double e2 = edge_chi2(r, om);
            double rho[3];
            zso_loss(p->loss_kind, p->loss_delta, e2, rho);
            drho = rho[1];
            for (int i = 0; i < 4; ++i) W[i] = rho[1] * om[i];
            if ((rho[1] + 2.0 * rho[2] * e2) > 0.0) {
                const double we0 = om[0] * r[0] + om[1] * r[1];
                const double we1 = om[2] * r[0] + om[3] * r[1];
                W[0] += 2.0 * rho[2] * we0 * we0;
                W[1] += 2.0 * rho[2] * we0 * we1;
                W[2] += 2.0 * rho[2] * we1 * we0;
                W[3] += 2.0 * rho[2] * we1 * we1;
            }
        }
        e[24] = drho;
        /* Omega r for the gradient (the non-robust information scaled by drho). */
        e[25] = om[0] * r[0] + om[1] * r[1];
        e[26] = om[2] * r[0] + om[3] * r[1];
    }
}

typedef struct lin_ctx {
    const zso_problem* p;
    lin* s;
    const double* et;
    double* hpl_obs;
} lin_ctx;

/* H_pp, b_p and the per-edge H_pl blocks of the poses in [k0, k1): each
 * pose's sums over its edges in edge order. */
static void lin_pose_sums(void* ctx, long long k0, long long k1) {
    const lin_ctx* x = (const lin_ctx*)ctx;
    const zso_problem* p = x->p;
    for (long long o = 0; o < p->num_obs; ++o) {
        const int pi = p->obs_pose[o], li = p->obs_landmark[o];
        if (pi < k0 || pi >= k1 || p->pose_fixed[pi]) continue;
        const double* e = x->et + EDGE_TERMS * o;
        const double *Jp = e + 2, *Jl = e + 14, *W = e + 20, *orr = e + 25;
        const double drho = e[24];
        double JtW[12]; /* 6x2 */
        for (int a = 0; a < 6; ++a) {
            JtW[a * 2 + 0] = Jp[0 * 6 + a] * W[0] + Jp[1 * 6 + a] * W[2];
            JtW[a * 2 + 1] = Jp[0 * 6 + a] * W[1] + Jp[1 * 6 + a] * W[3];
        }
        double* H = x->s->hpp + 36LL * pi;
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c) H[a * 6 + c] += JtW[a * 2] * Jp[c] + JtW[a * 2 + 1] * Jp[6 + c];
        if (!p->landmark_fixed[li]) {
            double* B = x->hpl_obs + 18 * o;
            for (int a = 0; a < 6; ++a)
                for (int c = 0; c < 3; ++c) B[a * 3 + c] = JtW[a * 2] * Jl[c] + JtW[a * 2 + 1] * Jl[3 + c];
        }
        for (int a = 0; a < 6; ++a) x->s->b[6 * pi + a] -= drho * (Jp[a] * orr[0] + Jp[6 + a] * orr[1]);
    }
}

/* H_ll and b_l of the landmarks in [l0, l1), each summed in edge order. */
static void lin_landmark_sums(void* ctx, long long l0, long long l1) {
    const lin_ctx* x = (const lin_ctx*)ctx;
    const zso_problem* p = x->p;
    const int n = 6 * p->num_poses;
    for (long long o = 0; o < p->num_obs; ++o) {
        const int li = p->obs_landmark[o];
        if (li < l0 || li >= l1 || p->landmark_fixed[li]) continue;
        const double* e = x->et + EDGE_TERMS * o;
        const double *Jl = e + 14, *W = e + 20, *orr = e + 25;
        const double drho = e[24];
        double JtW[6]; /* 3x2 */
        for (int a = 0; a < 3; ++a) {
            JtW[a * 2 + 0] = Jl[0 * 3 + a] * W[0] + Jl[1 * 3 + a] * W[2];
            JtW[a * 2 + 1] = Jl[0 * 3 + a] * W[1] + Jl[1 * 3 + a] * W[3];
        }
        double* H = x->s->hll + 9LL * li;
        for (int a = 0; a < 3; ++a)
            for (int c = 0; c < 3; ++c) H[a * 3 + c] += JtW[a * 2] * Jl[c] + JtW[a * 2 + 1] * Jl[3 + c];
        for (int a = 0; a < 3; ++a) x->s->b[n + 3 * li + a] -= drho * (Jl[a] * orr[0] + Jl[3 + a] * orr[1]);
    }
}

/* make_hessian, source/factor_graph.hpp:648-732: per-edge terms (in
 * parallel), then every pose's and landmark's sums in edge order. */
static int linearise(const zso_problem* p, lin* s) {
    const int K = p->num_poses, L = p->num_landmarks;
    const long long M = p->num_obs;
    const int n = 6 * K;
    memset(s, 0, sizeof(*s));
    s->K = K; s->L = L;
    s->hpp = calloc((size_t)K * 36, sizeof(double));
    s->hll = calloc((size_t)L * 9 + 1, sizeof(double));
    s->b = calloc((size_t)n + 3 * (size_t)L + 1, sizeof(double));
    s->lm_ptr = calloc((size_t)L + 1, sizeof(int));
    double* hpl_obs = calloc((size_t)M * 18 + 1, sizeof(double));
    if (!s->hpp || !s->hll || !s->b || !s->lm_ptr || !hpl_obs) { free(hpl_obs); lin_free(s); return 0; }
    /* per-edge terms (in parallel), then the sums in edge order */
    double* et = malloc(((size_t)M + 1) * EDGE_TERMS * sizeof(double));
    if (!et) { free(hpl_obs); lin_free(s); return 0; }
    void* ectx[2] = {(void*)p, et};
    parallel_for(M, 4096, edge_terms, ectx);
    lin_ctx c = {p, s, et, hpl_obs};
    parallel_for(K, 64, lin_pose_sums, &c);
    parallel_for(L, 1024, lin_landmark_sums, &c);
    free(et);
    /* Group the pose-landmark blocks by landmark, one block per distinct pose
     * (duplicate observations of a pair add up, as the hash map does). */
    int* cnt = calloc((size_t)L + 1, sizeof(int));
    long long* order = malloc(((size_t)M + 1) * sizeof(long long));
    for (long long o = 0; o < M; ++o) cnt[p->obs_landmark[o] + 1]++;
    for (int l = 0; l < L; ++l) cnt[l + 1] += cnt[l];
    int* fill = calloc((size_t)L + 1, sizeof(int));
    for (long long o = 0; o < M; ++o) {
        const int l = p->obs_landmark[o];
        order[cnt[l] + fill[l]++] = o;
    }
    s->blk_pose = malloc(((size_t)M + 1) * sizeof(int));
    s->hpl = calloc((size_t)M * 18 + 1, sizeof(double));
    int nb = 0;
    for (int l = 0; l < L; ++l) {
        s->lm_ptr[l] = nb;
        long long* seg = order + cnt[l];
        const int d = cnt[l + 1] - cnt[l];
        /* insertion sort by pose, stable */
        for (int i = 1; i < d; ++i) {
            long long v = seg[i];
            int j = i - 1;
            while (j >= 0 && p->obs_pose[seg[j]] > p->obs_pose[v]) { seg[j + 1] = seg[j]; --j; }
            seg[j + 1] = v;
        }
        if (p->landmark_fixed[l]) continue;
        for (int i = 0; i < d; ++i) {
            const long long o = seg[i];
            const int pi = p->obs_pose[o];
            if (p->pose_fixed[pi]) continue;
            if (nb > s->lm_ptr[l] && s->blk_pose[nb - 1] == pi) {
                for (int k = 0; k < 18; ++k) s->hpl[18LL * (nb - 1) + k] += hpl_obs[18 * o + k];
            } else {
                s->blk_pose[nb] = pi;
                memcpy(s->hpl + 18LL * nb, hpl_obs + 18 * o, 18 * sizeof(double));
                ++nb;
            }
        }
    }
    s->lm_ptr[L] = nb;
    s->nblk = nb;
    free(cnt); free(order); free(fill); free(hpl_obs);
    return 1;
}

typedef struct schur_ctx {
    const struct lin* s;
    const double* Wb;
    double* S;
} schur_ctx;

/* The Schur products W_a H_b^T of every landmark whose row pose a lies in
 * [p0, p1), added to S in landmark order. */
static void schur_rows(void* c, long long p0, long long p1) {
    const schur_ctx* x = (const schur_ctx*)c;
    const struct lin* s = x->s;
    const int n = 6 * s->K;
    for (int l = 0; l < s->L; ++l)
        for (int ka = s->lm_ptr[l]; ka < s->lm_ptr[l + 1]; ++ka) {
            const int ia = s->blk_pose[ka];
            if (ia < p0 || ia >= p1) continue;
            const double* W = x->Wb + 18LL * ka;
            for (int kb = s->lm_ptr[l]; kb < s->lm_ptr[l + 1]; ++kb) {
                const double* H = s->hpl + 18LL * kb;
                const int ib = s->blk_pose[kb];
                for (int a = 0; a < 6; ++a) {
                    double* row = x->S + (size_t)(6 * ia + a) * n + 6 * ib;
                    for (int c = 0; c < 6; ++c)
                        row[c] += W[a * 3] * H[c * 3] + W[a * 3 + 1] * H[c * 3 + 1] + W[a * 3 + 2] * H[c * 3 + 2];
                }
            }
        }
}

/* Pose ranges of about equal Schur work (blocks x landmark degree) per thread. */
static int schur_parts(const struct lin* s, long long* bounds) {
    int parts = g_threads;
    if (parts > s->K) parts = s->K > 0 ? s->K : 1;
    if ((long long)s->nblk < 20000) parts = 1;
    bounds[0] = 0;
    if (parts == 1) {
        bounds[1] = s->K;
        return 1;
    }
    double* w = calloc((size_t)s->K + 1, sizeof(double));
    double total = 0.0;
    for (int l = 0; l < s->L; ++l) {
        const int d = s->lm_ptr[l + 1] - s->lm_ptr[l];
        for (int k = s->lm_ptr[l]; k < s->lm_ptr[l + 1]; ++k) w[s->blk_pose[k]] += d;
        total += (double)d * d;
    }
    int t = 1;
    double acc = 0.0;
    for (int k = 0; k < s->K && t < parts; ++k) {
        acc += w[k];
        if (acc >= total * t / parts) bounds[t++] = k + 1;
    }
    while (t <= parts) bounds[t++] = s->K;
    free(w);
    return parts;
}

/* solve_linear_system, source/factor_graph.hpp:736-806. */
static int solve_system(const zso_problem* p, const lin* s, double lambda, double* S_out, double* bs_out,
                        double* delta) {
    const int K = s->K, L = s->L, n = 6 * K;
    double* S = calloc((size_t)n * n + 1, sizeof(double));
    double* Lf = malloc(((size_t)n * n + 1) * sizeof(double));
    double* bs = malloc(((size_t)n + 1) * sizeof(double));
    double* hinv = calloc((size_t)L * 9 + 1, sizeof(double));
    double* Wb = malloc(((size_t)s->nblk * 18 + 1) * sizeof(double));
    int ok = 0;
    if (!S || !Lf || !bs || !hinv || !Wb) goto done;
    /* damped H_ll inverses; fixed landmarks keep a zero block, a singular
     * block is left zero as the ignored invert() result does. */
    for (int l = 0; l < L; ++l) {
        if (p->landmark_fixed[l]) continue;
        double A[9];
        memcpy(A, s->hll + 9LL * l, sizeof(A));
        A[0] += lambda; A[4] += lambda; A[8] += lambda;
        zso_invert3(A, hinv + 9LL * l);
    }
    /* W = H_pl H_ll^-1 per block */
    for (int l = 0; l < L; ++l)
        for (int k = s->lm_ptr[l]; k < s->lm_ptr[l + 1]; ++k) {
            const double* H = s->hpl + 18LL * k;
            const double* I = hinv + 9LL * l;
            double* W = Wb + 18LL * k;
            for (int a = 0; a < 6; ++a)
                for (int c = 0; c < 3; ++c)
                    W[a * 3 + c] = H[a * 3 + 0] * I[0 * 3 + c] + H[a * 3 + 1] * I[1 * 3 + c] + H[a * 3 + 2] * I[2 * 3 + c];
        }
    /* b_s = b_p - W b_l */
    memcpy(bs, s->b, (size_t)n * sizeof(double));
    for (int l = 0; l < L; ++l)
        for (int k = s->lm_ptr[l]; k < s->lm_ptr[l + 1]; ++k) {
            const double* W = Wb + 18LL * k;
            const double* bl = s->b + n + 3LL * l;
            double* t = bs + 6LL * s->blk_pose[k];
            for (int a = 0; a < 6; ++a) t[a] -= W[a * 3] * bl[0] + W[a * 3 + 1] * bl[1] + W[a * 3 + 2] * bl[2];
        }
    /* C = sum_l W_l H_l^T accumulated into S, then S = (H_pp + lambda I) - C;
     * threads own pose rows of C (each entry's sum keeps landmark order) */
    {
        schur_ctx c = {s, Wb, S};
        long long bounds[257];
        const int parts = schur_parts(s, bounds);
        run_parts(schur_rows, &c, bounds, parts);
    }
    for (size_t i = 0; i < (size_t)n * n; ++i) S[i] = -S[i];
    for (int k = 0; k < K; ++k)
        for (int a = 0; a < 6; ++a)
            for (int c = 0; c < 6; ++c) {
                double h = s->hpp[36LL * k + a * 6 + c];
                if (a == c) h += lambda;
                S[(size_t)(6 * k + a) * n + 6 * k + c] += h;
            }
    if (S_out) memcpy(S_out, S, (size_t)n * n * sizeof(double));
    if (bs_out) memcpy(bs_out, bs, (size_t)n * sizeof(double));
    memset(delta, 0, ((size_t)n + 3 * (size_t)L) * sizeof(double));
    if (!zso_cholesky(S, n, Lf) || !zso_cholesky_solve(Lf, bs, n, delta)) goto done;
    /* delta_l = H_ll^-1 (b_l - H_lp delta_p) */
    for (int l = 0; l < L; ++l) {
        double v[3] = {s->b[n + 3 * l], s->b[n + 3 * l + 1], s->b[n + 3 * l + 2]};
        for (int k = s->lm_ptr[l]; k < s->lm_ptr[l + 1]; ++k) {
            const double* H = s->hpl + 18LL * k;
            const double* dp = delta + 6LL * s->blk_pose[k];
            for (int c = 0; c < 3; ++c) {
                double acc = 0.0;
                for (int a = 0; a < 6; ++a) acc += H[a * 3 + c] * dp[a];
                v[c] -= acc;
            }
        }
        const double* I = hinv + 9LL * l;
        for (int c = 0; c < 3; ++c) delta[n + 3 * l + c] = I[c * 3] * v[0] + I[c * 3 + 1] * v[1] + I[c * 3 + 2] * v[2];
    }
    ok = 1;
done:
    free(S); free(Lf); free(bs); free(hinv); free(Wb);
    return ok;
}

static double max_diag(const lin* s) {
    /* source/factor_graph.hpp:513-520 */
    double m = 0.0;
    for (int k = 0; k < s->K; ++k)
        for (int a = 0; a < 6; ++a) m = fmax(fabs(s->hpp[36LL * k + 7 * a]), m);
    for (int l = 0; l < s->L; ++l)
        for (int a = 0; a < 3; ++a) m = fmax(fabs(s->hll[9LL * l + 4 * a]), m);
    return fmin(5e10, m);
}

double zso_initial_lambda(const zso_problem* p) {
    lin s;
    if (!linearise(p, &s)) return NAN;
    const double v = 1e-5 * max_diag(&s);
    lin_free(&s);
    return v;
}

int zso_linear_step(const zso_problem* p, double lambda, double* S, double* bs, double* delta, double* b,
                    double* hpp, double* hll) {
    lin s;
    if (!linearise(p, &s)) return 0;
    const size_t nall = 6 * (size_t)p->num_poses + 3 * (size_t)p->num_landmarks;
    double* d = delta ? delta : malloc((nall + 1) * sizeof(double));
    const int ok = solve_system(p, &s, lambda, S, bs, d);
    if (b) memcpy(b, s.b, nall * sizeof(double));
    if (hpp) memcpy(hpp, s.hpp, (size_t)p->num_poses * 36 * sizeof(double));
    if (hll) memcpy(hll, s.hll, (size_t)p->num_landmarks * 9 * sizeof(double));
    if (!delta) free(d);
    lin_free(&s);
    return ok;
}

/* factor_graph::solve, source/factor_graph.hpp:489-615, as a state machine:
 * zso_lm_begin (:494-536), zso_lm_iteration (one pass of the outer loop,
 * :538-611) and zso_lm_end; zso_solve runs them in sequence. */
struct zso_lm {
    zso_problem* p;
    lin s;
    int use_relative, it, success, stopped, have_lin;
    double nu, chi2, lambda, legacy;
    double *delta, *bk_pose, *bk_lm;
    zso_report rr;
};

zso_lm* zso_lm_begin(zso_problem* p, int use_relative) {
    zso_lm* m = calloc(1, sizeof(zso_lm));
    if (!m) return NULL;
    m->p = p;
    m->use_relative = use_relative;
    const int K = p->num_poses, L = p->num_landmarks, n = 6 * K;
    const size_t nall = (size_t)n + 3 * (size_t)L;
    if (p->num_obs == 0 || (K == 0 && L == 0)) {
        m->stopped = 1;
        return m;
    }
    if (!linearise(p, &m->s)) {
        m->stopped = 1;
        return m;
    }
    m->have_lin = 1;
    m->nu = 2.0;
    m->chi2 = zso_chi2(p);
    m->rr.chi2_initial = m->chi2;
    m->lambda = 1e-5 * max_diag(&m->s);
    m->legacy = 1e-10 * m->chi2;
    m->delta = calloc(nall + 1, sizeof(double));
    m->bk_pose = malloc(((size_t)K * 7 + 1) * sizeof(double));
    m->bk_lm = malloc(((size_t)L * 3 + 1) * sizeof(double));
    return m;
}

int zso_lm_iteration(zso_lm* m) {
    if (!m || m->stopped) return 0;
    zso_problem* p = m->p;
    const int K = p->num_poses, L = p->num_landmarks, n = 6 * K;
    const size_t nall = (size_t)n + 3 * (size_t)L;
    const int max_failures = 10;
    m->rr.iterations = m->it + 1;
    const double last = m->chi2;
    int failures = 0;
    while (failures < max_failures) {
        m->rr.attempts++;
        if (!solve_system(p, &m->s, m->lambda, NULL, NULL, m->delta)) {
            m->rr.chol_failures++;
            memset(m->delta, 0, nall * sizeof(double));
            m->lambda *= m->nu;
            m->nu *= 2.0;
            ++failures;
            if (!isfinite(m->lambda)) break;
            continue;
        }
        /* update_states, source/factor_graph.hpp:809-830 */
        memcpy(m->bk_pose, p->poses, (size_t)K * 7 * sizeof(double));
        memcpy(m->bk_lm, p->landmarks, (size_t)L * 3 * sizeof(double));
        for (int k = 0; k < K; ++k)
            if (!p->pose_fixed[k]) zso_pose_plus(p->poses + 7LL * k, m->delta + 6LL * k);
        for (int l = 0; l < L; ++l)
            if (!p->landmark_fixed[l])
                for (int c = 0; c < 3; ++c) p->landmarks[3LL * l + c] += m->delta[n + 3 * l + c];
        double scale = 0.0;
        for (size_t i = 0; i < nall; ++i) scale += m->delta[i] * (m->lambda * m->delta[i] + m->s.b[i]);
        scale += 1e-3;
        const double chi_new = zso_chi2(p);
        const double rho = (m->chi2 - chi_new) / scale;
        int good = 0;
        if (rho > 0 && isfinite(chi_new)) {
            double alpha = 1.0 - pow(2.0 * rho - 1.0, 3.0);
            alpha = fmin(alpha, 2.0 / 3.0);
            m->lambda *= fmax(1.0 / 3.0, alpha);
            m->nu = 2.0;
            m->chi2 = chi_new;
            good = 1;
            ++m->success;
        } else {
            m->lambda *= m->nu;
            m->nu *= 2.0;
        }
        if (!isfinite(m->lambda)) break;
        if (good) {
            lin_free(&m->s);
            m->have_lin = 0;
            if (!linearise(p, &m->s)) {
                m->success = -1;
                m->stopped = 1;
                return 0;
            }
            m->have_lin = 1;
            break;
        }
        /* rollback_states, source/factor_graph.hpp:833-846 */
        memcpy(p->poses, m->bk_pose, (size_t)K * 7 * sizeof(double));
        memcpy(p->landmarks, m->bk_lm, (size_t)L * 3 * sizeof(double));
        ++failures;
    }
    ++m->it;
    const double thr = m->use_relative ? 1e-6 * fmax(last, 1e-12) : m->legacy;
    if (failures >= max_failures || (last - m->chi2) < thr || !isfinite(m->lambda)) m->stopped = 1;
    return !m->stopped;
}

void zso_lm_report(const zso_lm* m, zso_report* rep) {
    if (!m || !rep) return;
    *rep = m->rr;
    rep->accepted = m->success;
    rep->chi2_final = m->chi2;
    rep->lambda_final = m->lambda;
}

int zso_lm_end(zso_lm* m, zso_report* rep) {
    if (!m) return 0;
    m->rr.accepted = m->success;
    m->rr.chi2_final = m->chi2;
    m->rr.lambda_final = m->lambda;
    if (rep) *rep = m->rr;
    const int success = m->success;
    if (m->have_lin) lin_free(&m->s);
    free(m->delta); free(m->bk_pose); free(m->bk_lm);
    free(m);
    return success;
}

int zso_solve(zso_problem* p, int iterations, int use_relative, zso_report* rep) {
    zso_lm* m = zso_lm_begin(p, use_relative);
    if (!m) return 0;
    for (int it = 0; it < iterations; ++it)
        if (!zso_lm_iteration(m)) break;
    return zso_lm_end(m, rep);
}

/* ---------------------------------------------------------------- map culling */

/* The reference's cull constants, source/map.hpp:272,281-282,304,316. */
#define CULL_AGE 500
#define CULL_FEW_OBS 4
#define CULL_RECENT 7
#define CULL_ERROR 5.991f

void zso_pose_rt(const double pose[7], double Rt[12]) {
    const double q[4] = {pose[6], pose[3], pose[4], pose[5]};
    qmatrix(q, Rt);
    Rt[9] = pose[0];
    Rt[10] = pose[1];
    Rt[11] = pose[2];
}

/* One observation's error term of source/map.hpp:290-308: the frame maps the
 * landmark (R X + t, the summation order of source/matrix.hpp:494-509),
 * camera::pinhole::project (source/camera.hpp:91-111) and the Euclidean
 * pixel distance (source/matrix.hpp:177-183) rounded to float; 5.991 when the
 * point does not project. */
static float cull_error(const double Rt[12], const double intr[4], const double X[3], const float kp[2]) {
    double m[3];
    for (int i = 0; i < 3; ++i) {
        double s = 0.0;
        for (int k = 0; k < 3; ++k) s += Rt[3 * i + k] * X[k];
        m[i] = s + Rt[9 + i];
    }
    if (m[2] < 1.0e-12) return CULL_ERROR;
    const double iz = 1.0 / m[2];
    const double ux = m[0] * iz, uy = m[1] * iz;
    const double px = intr[0] * ux + intr[2];
    const double py = intr[1] * uy + intr[3];
    const double dx = (double)kp[0] - px, dy = (double)kp[1] - py;
    double ls = 0.0;
    ls += dx * dx;
    ls += dy * dy;
    return (float)sqrt(ls);
}

/* map::cull, source/map.hpp:269-323, one landmark at a time. */
long long zso_map_cull(const zso_cull_map* m, unsigned char* erase, float* mean_error) {
    long long erased = 0;
    for (int l = 0; l < m->num_landmarks; ++l) {
        int e = 0;
        float mean = -1.0f;
        if (m->landmark_id[l] + CULL_AGE >= m->landmark_id_generator) {
            const long long o0 = m->landmark_obs[l], o1 = m->landmark_obs[l + 1];
            if (o1 <= o0) {
                e = 1; /* no observations, map.hpp:277-280 and 281-287 */
            } else if (o1 - o0 <= CULL_FEW_OBS && m->obs_frame_id[o1 - 1] + CULL_RECENT < m->frame_id_generator) {
                e = 1;
            } else {
                float err = 0.0f;
                long long processed = 0;
                for (long long o = o0; o < o1; ++o) {
                    const int f = m->obs_frame[o];
                    if (f < 0) continue;
                    err += cull_error(m->frame_pose + 12 * (long long)f, m->frame_intrinsics + 4 * (long long)f,
                                      m->landmarks + 3 * (long long)l, m->obs_keypoint + 2 * o);
                    ++processed;
                }
                if (processed == 0) {
                    e = 1;
                } else {
                    mean = err / (float)processed;
                    e = mean >= CULL_ERROR;
                }
            }
        }
        if (erase) erase[l] = (unsigned char)e;
        if (mean_error) mean_error[l] = mean;
        erased += e;
    }
    return erased;
}

/* so3 from a rotation matrix, source/lie.hpp:159-180 (the branch on the trace
 * and, below it, on the largest diagonal entry, as written there). */
void zso_rt_pose(const double Rt[12], double pose[7]) {
    const double* R = Rt;
    double q[4];
    const double tr = R[0] + R[4] + R[8];
    if (tr > 0) {
        const double s = sqrt(tr + 1);
        const double inv = 0.5 / s;
        q[0] = 0.5 * s;
        q[1] = (R[7] - R[5]) * inv;
        q[2] = (R[2] - R[6]) * inv;
        q[3] = (R[3] - R[1]) * inv;
    } else {
        const int i = (R[0] < R[4]) ? (1 + (R[4] < R[8])) : (2 * (R[0] < R[8]));
        const int j = (i + 1) % 3, k = (j + 1) % 3;
        const double s = sqrt(R[3 * i + i] - R[3 * j + j] - R[3 * k + k] + 1.0);
        const double inv = 0.5 / s;
        q[0] = (R[3 * j + k] - R[3 * k + j]) * inv;
        q[1 + i] = 0.5 * s;
        q[1 + j] = (R[3 * i + j] + R[3 * j + i]) * inv;
        q[1 + k] = (R[3 * i + k] + R[3 * k + i]) * inv;
    }
    pose[0] = Rt[9];
    pose[1] = Rt[10];
    pose[2] = Rt[11];
    pose[3] = q[1];
    pose[4] = q[2];
    pose[5] = q[3];
    pose[6] = q[0];
}

/* ---------------------------------------------------------------- matching */

/* distance<256>, source/feature.hpp:1139-1187: the popcount of the XOR of
 * the two 32-byte descriptors, counted per byte from a table of the 256
 * byte values' bit counts. */
static unsigned int hamming256(const unsigned char* a, const unsigned char* b) {
    static unsigned char bits[256];
    static int ready = 0;
    if (!ready) {
        for (int v = 0; v < 256; ++v) {
            int c = 0;
            for (int x = v; x; x >>= 1) c += x & 1;
            bits[v] = (unsigned char)c;
        }
        ready = 1;
    }
    unsigned int d = 0;
    for (int i = 0; i < 32; ++i) d += bits[a[i] ^ b[i]];
    return d;
}

/* feature::find_matches, source/feature.hpp:1190-1235. */
long long zso_find_matches(const unsigned char* lhs, long long n_lhs, const unsigned char* rhs, long long n_rhs,
                           float threshold, long long k, zso_match* matches, long long size) {
    if (k <= 0 || size <= 0) return 0;
    long long count = 0;
    for (long long i = 0; i < n_lhs; ++i) {
        if (count + k > size) break;
        for (long long m = 0; m < k; ++m) {
            matches[count + m].lhs_index = (unsigned long long)i;
            matches[count + m].rhs_index = 0;
            matches[count + m].score = threshold;
        }
        for (long long j = 0; j < n_rhs; ++j) {
            const float score = (float)hamming256(lhs + 32 * i, rhs + 32 * j);
            for (long long m = 0; m < k; ++m) {
                if (score < matches[count + m].score) {
                    for (long long s = k - 1; s > m; --s) matches[count + s] = matches[count + s - 1];
                    matches[count + m].score = score;
                    matches[count + m].rhs_index = (unsigned long long)j;
                    matches[count + m].lhs_index = (unsigned long long)i;
                    break;
                }
            }
        }
        const long long save = count;
        for (long long m = 0; m < k; ++m)
            if (matches[save + m].score < threshold) ++count;
    }
    return count;
}
