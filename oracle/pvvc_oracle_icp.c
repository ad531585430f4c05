/*
 * pvvc_oracle_icp.c -- CPU restatement of point-to-point ICP as the reference
 * calls it through pcl::IterativeClosestPoint (src/registration/icp.cc:21-102)
 * and of ICPBase::CloudMSE (src/registration/registration_base.cc:114-158).
 *
 * TEST INFRASTRUCTURE ONLY.  PCL (>= 1.10, not vendored, not installed here)
 * holds the algorithm; this is written from its documented semantics, not
 * from its source:
 *   - correspondences: exact nearest target point of each transformed source
 *     point, kept if its squared distance <= max_corr_dist^2;
 *   - fewer than 3 correspondences: not converged, stop;
 *   - rigid estimate per iteration: centroids, cross-covariance, SVD
 *     (Kabsch / Umeyama without scale), reflection fixed; composed as
 *     T = T_inc * T;
 *   - convergence after each iteration, in order: iteration cap (counts as
 *     converged); |R_inc| close to I (cos angle >= 1 - transform_eps) and
 *     |t_inc|^2 <= transform_eps; |mse - mse_prev| < mse_abs_eps (absolute, PCL
 *     default 1e-12); relative
 *     |mse - mse_prev| / mse_prev < fitness_eps; mse = mean squared distance
 *     of the iteration's correspondences, mse_prev starts at DBL_MAX;
 *   - fitness score: mean squared NN distance of the finally transformed
 *     source (getFitnessScore with max_range = DBL_MAX).
 * ICP parity is therefore unpinned against PCL itself.  Computed in double
 * precision with an exact grid nearest-neighbour search.
 */
#include <float.h>
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "pvvc_oracle.h"

/* ---- exact nearest neighbour on a uniform grid ---- */
typedef struct {
    double lo[3], h;
    int dim[3];
    int* start; /* cell -> first point (+ sentinel) */
    float* pts; /* points sorted by cell */
    int* orig;  /* input index of each sorted point */
    size_t n;
} grid_t;

static int grid_build(grid_t* g, const float* p, size_t n) {
    double lo[3] = {DBL_MAX, DBL_MAX, DBL_MAX}, hi[3] = {-DBL_MAX, -DBL_MAX, -DBL_MAX};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            if (p[3 * i + a] < lo[a]) lo[a] = p[3 * i + a];
            if (p[3 * i + a] > hi[a]) hi[a] = p[3 * i + a];
        }
    double ext = 0;
    for (int a = 0; a < 3; ++a) ext = fmax(ext, hi[a] - lo[a]);
    g->h = fmax(ext / 24.0, 1.0);
    for (int a = 0; a < 3; ++a) {
        g->lo[a] = lo[a];
        g->dim[a] = (int)floor((hi[a] - lo[a]) / g->h) + 1;
    }
    size_t nc = (size_t)g->dim[0] * g->dim[1] * g->dim[2];
    g->start = (int*)calloc(nc + 1, sizeof(int));
    g->pts = (float*)malloc(3 * n * sizeof(float) + 4);
    g->orig = (int*)malloc(n * sizeof(int) + 4);
    int* cell = (int*)malloc(n * sizeof(int) + 4);
    if (!g->start || !g->pts || !g->orig || !cell) { free(cell); return PVO_ERR_NOMEM; }
    for (size_t i = 0; i < n; ++i) {
        int c[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = (int)floor((p[3 * i + a] - g->lo[a]) / g->h);
            if (c[a] >= g->dim[a]) c[a] = g->dim[a] - 1;
        }
        cell[i] = (c[2] * g->dim[1] + c[1]) * g->dim[0] + c[0];
        g->start[cell[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
    int* fill = (int*)malloc((nc + 1) * sizeof(int));
    memcpy(fill, g->start, (nc + 1) * sizeof(int));
    for (size_t i = 0; i < n; ++i) {
        g->orig[fill[cell[i]]] = (int)i;
        memcpy(g->pts + 3 * fill[cell[i]]++, p + 3 * i, 3 * sizeof(float));
    }
    free(fill);
    free(cell);
    g->n = n;
    return PVO_OK;
}

static void grid_free(grid_t* g) {
    free(g->start);
    free(g->pts);
    free(g->orig);
}

/* squared distance to the nearest point, exact: rings of cells in growing
 * Chebyshev radius until the ring cannot hold anything closer.  Among points
 * at the same distance the one first in the input wins, so the answer does
 * not depend on the grid. */
static double grid_nn(const grid_t* g, const double q[3], int* idx) {
    /* rings of cells around the query's cell clamped into the grid; a point in
     * ring r lies at least (r-1)*h from the query (also for queries outside) */
    int c[3];
    for (int a = 0; a < 3; ++a) {
        double t = floor((q[a] - g->lo[a]) / g->h);
        if (t < 0) t = 0;
        if (t > g->dim[a] - 1) t = g->dim[a] - 1;
        c[a] = (int)t;
    }
    double best = DBL_MAX;
    int bi = -1;
    int maxr = g->dim[0];
    if (g->dim[1] > maxr) maxr = g->dim[1];
    if (g->dim[2] > maxr) maxr = g->dim[2];
    for (int r = 0; r <= maxr; ++r) {
        if (r > 0 && bi >= 0) {
            double lb = (r - 1) * g->h;
            if (lb * lb * 0.999 > best) break;
        }
        for (int z = c[2] - r; z <= c[2] + r; ++z) {
            if (z < 0 || z >= g->dim[2]) continue;
            for (int y = c[1] - r; y <= c[1] + r; ++y) {
                if (y < 0 || y >= g->dim[1]) continue;
                for (int x = c[0] - r; x <= c[0] + r; ++x) {
                    if (x < 0 || x >= g->dim[0]) continue;
                    if (abs(x - c[0]) != r && abs(y - c[1]) != r && abs(z - c[2]) != r) continue;
                    int cc = (z * g->dim[1] + y) * g->dim[0] + x;
                    for (int k = g->start[cc]; k < g->start[cc + 1]; ++k) {
                        double dx = g->pts[3 * k] - q[0], dy = g->pts[3 * k + 1] - q[1], dz = g->pts[3 * k + 2] - q[2];
                        double d = dx * dx + dy * dy + dz * dz;
                        if (d < best || (bi >= 0 && d == best && g->orig[k] < g->orig[bi])) { best = d; bi = k; }
                    }
                }
            }
        }
    }
    if (idx) *idx = bi;
    return best;
}

/* ---- 3x3 SVD by one-sided Jacobi (double) ----
 * A pair of columns is rotated while |c| > 1e-15 sqrt(a b) (Demmel-Veselic
 * relative test); the sweeps end when a whole sweep rotates nothing. */
static void svd3(const double A[9], double U[9], double S[3], double V[9]) {
    double B[9];
    memcpy(B, A, sizeof(B));
    for (int i = 0; i < 9; ++i) V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    for (int sweep = 0; sweep < 60; ++sweep) {
        int rotated = 0;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double a = 0, b = 0, c = 0;
                for (int i = 0; i < 3; ++i) {
                    a += B[3 * i + p] * B[3 * i + p];
                    b += B[3 * i + q] * B[3 * i + q];
                    c += B[3 * i + p] * B[3 * i + q];
                }
                if (!(fabs(c) > 1e-15 * sqrt(a * b))) continue;
                rotated = 1;
                double zeta = (b - a) / (2 * c);
                double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
                double cs = 1 / sqrt(1 + t * t), sn = cs * t;
                for (int i = 0; i < 3; ++i) {
                    double bp = B[3 * i + p], bq = B[3 * i + q];
                    B[3 * i + p] = cs * bp - sn * bq;
                    B[3 * i + q] = sn * bp + cs * bq;
                    double vp = V[3 * i + p], vq = V[3 * i + q];
                    V[3 * i + p] = cs * vp - sn * vq;
                    V[3 * i + q] = sn * vp + cs * vq;
                }
            }
        if (!rotated) break;
    }
    for (int j = 0; j < 3; ++j) {
        double s = sqrt(B[j] * B[j] + B[3 + j] * B[3 + j] + B[6 + j] * B[6 + j]);
        S[j] = s;
        for (int i = 0; i < 3; ++i) U[3 * i + j] = s > 1e-300 ? B[3 * i + j] / s : (i == j ? 1.0 : 0.0);
    }
}

static double det3(const double M[9]) {
    return M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) + M[2] * (M[3] * M[7] - M[4] * M[6]);
}

/* rigid transform (R,t) minimising sum |R p + t - q|^2 from the sums */
static void kabsch(double n, const double sp[3], const double sq[3], const double spq[9], double R[9], double t[3]) {
    double cp[3], cq[3], H[9];
    for (int a = 0; a < 3; ++a) { cp[a] = sp[a] / n; cq[a] = sq[a] / n; }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[3 * i + j] = spq[3 * i + j] - n * cp[i] * cq[j];
    double U[9], S[3], V[9];
    svd3(H, U, S, V);
    /* R = V U^T */
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) R[3 * i + j] = V[3 * i] * U[3 * j] + V[3 * i + 1] * U[3 * j + 1] + V[3 * i + 2] * U[3 * j + 2];
    if (det3(R) < 0) {
        /* flip the axis of the smallest singular value */
        int k = 0;
        for (int j = 1; j < 3; ++j) if (S[j] < S[k]) k = j;
        for (int i = 0; i < 3; ++i) V[3 * i + k] = -V[3 * i + k];
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[3 * i + j] = V[3 * i] * U[3 * j] + V[3 * i + 1] * U[3 * j + 1] + V[3 * i + 2] * U[3 * j + 2];
    }
    for (int i = 0; i < 3; ++i) t[i] = cq[i] - (R[3 * i] * cp[0] + R[3 * i + 1] * cp[1] + R[3 * i + 2] * cp[2]);
}

int pvo_icp_align(const float* src, size_t ns, const float* tgt, size_t nt, const float* init, const pvo_icp_params* p,
                  float* T_out, float* fitness, int* iters, int* converged) {
    if (!src || !tgt || !ns || !nt || !p || !T_out) return PVO_ERR_ARG;
    grid_t g;
    if (grid_build(&g, tgt, nt)) return PVO_ERR_NOMEM;
    double T[16];
    for (int i = 0; i < 16; ++i) T[i] = init ? init[i] : ((i % 5 == 0) ? 1.0 : 0.0);
    const double corr2 = (double)p->max_corr_dist * (double)p->max_corr_dist;
    double prev_mse = DBL_MAX;
    int it = 0, conv = 0;
    for (;;) {
        double sp[3] = {0, 0, 0}, sq[3] = {0, 0, 0}, spq[9] = {0}, sd = 0, cnt = 0;
        for (size_t i = 0; i < ns; ++i) {
            double x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2], q[3];
            for (int r = 0; r < 3; ++r) q[r] = T[4 * r] * x + T[4 * r + 1] * y + T[4 * r + 2] * z + T[4 * r + 3];
            int k;
            double d = grid_nn(&g, q, &k);
            if (k < 0 || d > corr2) continue;
            const float* m = g.pts + 3 * k;
            for (int a = 0; a < 3; ++a) { sp[a] += q[a]; sq[a] += m[a]; }
            for (int a = 0; a < 3; ++a)
                for (int b = 0; b < 3; ++b) spq[3 * a + b] += q[a] * m[b];
            sd += d;
            cnt += 1;
        }
        if (cnt < 3) { conv = 0; break; }
        double R[9], t[3];
        kabsch(cnt, sp, sq, spq, R, t);
        double Tn[16];
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 4; ++j) Tn[4 * i + j] = R[3 * i] * T[j] + R[3 * i + 1] * T[4 + j] + R[3 * i + 2] * T[8 + j] + (j == 3 ? t[i] : 0.0);
        }
        for (int j = 0; j < 4; ++j) Tn[12 + j] = T[12 + j];
        memcpy(T, Tn, sizeof(T));
        ++it;
        /* convergence (DefaultConvergenceCriteria semantics) */
        if (it >= p->max_iter) { conv = 1; break; }
        double cosang = 0.5 * (R[0] + R[4] + R[8] - 1.0);
        double tr2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
        if (cosang >= 1.0 - (double)p->transform_eps && tr2 <= (double)p->transform_eps) { conv = 1; break; }
        double mse = sd / cnt;
        if (fabs(mse - prev_mse) < (double)p->mse_abs_eps) { conv = 1; break; }
        if (fabs(mse - prev_mse) / prev_mse < (double)p->fitness_eps) { conv = 1; break; }
        prev_mse = mse;
    }
    /* fitness score of the final transform */
    double fs = 0;
    for (size_t i = 0; i < ns; ++i) {
        double x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2], q[3];
        for (int r = 0; r < 3; ++r) q[r] = T[4 * r] * x + T[4 * r + 1] * y + T[4 * r + 2] * z + T[4 * r + 3];
        fs += grid_nn(&g, q, NULL);
    }
    grid_free(&g);
    for (int i = 0; i < 16; ++i) T_out[i] = (float)T[i];
    if (fitness) *fitness = (float)(fs / (double)ns);
    if (iters) *iters = it;
    if (converged) *converged = conv;
    return PVO_OK;
}

/* ICPBase::CloudMSE (registration_base.cc:114-158) */
float pvo_cloud_mse(const float* a, size_t na, const float* b, size_t nb) {
    if (!a || !b || !na || !nb) return -1.0f;
    grid_t ga, gb;
    if (grid_build(&gb, b, nb)) return -1.0f;
    if (grid_build(&ga, a, na)) { grid_free(&gb); return -1.0f; }
    double m1 = 0, m2 = 0;
    for (size_t i = 0; i < na; ++i) {
        double q[3] = {a[3 * i], a[3 * i + 1], a[3 * i + 2]};
        m1 += grid_nn(&gb, q, NULL);
    }
    for (size_t i = 0; i < nb; ++i) {
        double q[3] = {b[3 * i], b[3 * i + 1], b[3 * i + 2]};
        m2 += grid_nn(&ga, q, NULL);
    }
    grid_free(&ga);
    grid_free(&gb);
    m1 /= (double)na;
    m2 /= (double)nb;
    return (float)(m1 > m2 ? m1 : m2);
}

/* ---- many pairs on a thread pool (PatchesRegistration::Task's queue,
 * src/registration/patches_registration.cc:42-126) ---- */
#include <pthread.h>

typedef struct {
    int npairs;
    const float* src;
    const uint32_t* soff;
    const float* tgt;
    const uint32_t* toff;
    const pvo_icp_params* p;
    float* T;
    float* fit;
    int* iters;
    int* conv;
    pthread_mutex_t mu;
    int next;
} icp_job_t;

static void* icp_worker(void* arg) {
    icp_job_t* j = (icp_job_t*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int i = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (i >= j->npairs) break;
        const uint32_t a = j->soff[i], b = j->soff[i + 1], c = j->toff[i], d = j->toff[i + 1];
        pvo_icp_align(j->src + 3ull * a, b - a, j->tgt + 3ull * c, d - c, NULL, j->p, j->T + 16 * i, j->fit + i,
                      j->iters + i, j->conv + i);
    }
    return NULL;
}

int pvo_icp_batch(int npairs, const float* src, const uint32_t* soff, const float* tgt, const uint32_t* toff,
                  const pvo_icp_params* p, float* T, float* fit, int* iters, int* conv, int nthreads) {
    icp_job_t j = {npairs, src, soff, tgt, toff, p, T, fit, iters, conv};
    pthread_mutex_init(&j.mu, NULL);
    j.next = 0;
    if (nthreads < 1) nthreads = 1;
    pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
    int started = 0;
    for (int i = 0; i < nthreads; ++i)
        if (pthread_create(&th[i], NULL, icp_worker, &j) == 0) started++;
        else break;
    if (!started) icp_worker(&j);
    for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
    free(th);
    pthread_mutex_destroy(&j.mu);
    return PVO_OK;
}

/* ---- colour interpolation (GoPEncoding::Interpolation + the k-NN loop of
 * GoPEncoding::Encode, src/patch/GoP_encoding.cc:73-95,131-150) ----
 * PCL's KdTree (FLANN, exact) returns the k nearest points with squared
 * distances accumulated in float, x then y then z, sorted ascending; ties
 * here go to the lower source index.  The arithmetic below follows the
 * reference's statement order in float. */
#define KNN_MAX 64
typedef struct {
    float d[KNN_MAX];
    int i[KNN_MAX];
    int n, k;
} knn_t;

static int knn_less(float da, int ia, float db, int ib) { return da < db || (da == db && ia < ib); }

static void knn_offer(knn_t* s, float d, int idx) {
    if (s->n == s->k && !knn_less(d, idx, s->d[s->n - 1], s->i[s->n - 1])) return;
    int j = s->n < s->k ? s->n++ : s->n - 1;
    while (j > 0 && knn_less(d, idx, s->d[j - 1], s->i[j - 1])) {
        s->d[j] = s->d[j - 1];
        s->i[j] = s->i[j - 1];
        --j;
    }
    s->d[j] = d;
    s->i[j] = idx;
}

static float sqdist(const float* p, float qx, float qy, float qz) {
    float dx = p[0] - qx, dy = p[1] - qy, dz = p[2] - qz;
    float a = dx * dx;
    a = a + dy * dy;
    a = a + dz * dz;
    return a;
}

/* the reference's Interpolation on the found neighbours, then ColorYUV(r,g,b,false) */
static void knn_interp(const knn_t* s, const uint8_t* rgb, float* out) {
    float w[KNN_MAX];
    for (int j = 0; j < s->n; ++j) {
        float d = s->d[j];
        if (d <= 1e-6f) d = 1e-6f;
        w[j] = 1.0f / d;
    }
    float sum = 0.0f;
    for (int j = 0; j < s->n; ++j) sum = sum + w[j];
    for (int j = 0; j < s->n; ++j) w[j] = w[j] / sum;
    float r = 0.0f, g = 0.0f, b = 0.0f;
    for (int j = 0; j < s->n; ++j) {
        const uint8_t* c = rgb + 3 * (size_t)s->i[j];
        r = r + w[j] * (float)c[0];
        g = g + w[j] * (float)c[1];
        b = b + w[j] * (float)c[2];
    }
    out[0] = r * 0.299f + g * 0.587f + b * 0.114f;
    out[1] = r * -0.168736f - g * 0.331264f + b * 0.5f + 128;
    out[2] = r * 0.5f - g * 0.418688f - b * 0.081312f + 128;
}

/* uniform float grid over the source: about two points per cell, cells of
 * at least one voxel; ring search pruned by the k-th distance */
typedef struct {
    float lo[3], h;
    int dim[3];
    int* start;
    int* idx; /* source indices sorted by cell */
} fgrid_t;

static int fgrid_build(fgrid_t* g, const float* p, size_t n) {
    float lo[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, hi[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            if (p[3 * i + a] < lo[a]) lo[a] = p[3 * i + a];
            if (p[3 * i + a] > hi[a]) hi[a] = p[3 * i + a];
        }
    double vol = 1;
    for (int a = 0; a < 3; ++a) vol *= fmax(hi[a] - lo[a], 1.0);
    double h = cbrt(vol / (2.0 * (double)n));
    if (h < 1.0) h = 1.0;
    for (;;) {
        double cells = 1;
        for (int a = 0; a < 3; ++a) cells *= floor((hi[a] - lo[a]) / h) + 1;
        if (cells <= 4.0 * (double)n + 64) break;
        h *= 1.25;
    }
    g->h = (float)h;
    size_t nc = 1;
    for (int a = 0; a < 3; ++a) {
        g->lo[a] = lo[a];
        g->dim[a] = (int)floor((hi[a] - lo[a]) / h) + 1;
        nc *= (size_t)g->dim[a];
    }
    g->start = (int*)calloc(nc + 1, sizeof(int));
    g->idx = (int*)malloc(n * sizeof(int) + 4);
    int* cell = (int*)malloc(n * sizeof(int) + 4);
    if (!g->start || !g->idx || !cell) {
        free(cell);
        return PVO_ERR_NOMEM;
    }
    for (size_t i = 0; i < n; ++i) {
        int c[3];
        for (int a = 0; a < 3; ++a) {
            c[a] = (int)floor(((double)p[3 * i + a] - g->lo[a]) / g->h);
            if (c[a] < 0) c[a] = 0;
            if (c[a] >= g->dim[a]) c[a] = g->dim[a] - 1;
        }
        cell[i] = (c[2] * g->dim[1] + c[1]) * g->dim[0] + c[0];
        g->start[cell[i] + 1]++;
    }
    for (size_t c = 0; c < nc; ++c) g->start[c + 1] += g->start[c];
    int* fill = (int*)malloc((nc + 1) * sizeof(int));
    memcpy(fill, g->start, (nc + 1) * sizeof(int));
    for (size_t i = 0; i < n; ++i) g->idx[fill[cell[i]]++] = (int)i;
    free(fill);
    free(cell);
    return PVO_OK;
}

static void fgrid_free(fgrid_t* g) {
    free(g->start);
    free(g->idx);
}

static void fgrid_knn(const fgrid_t* g, const float* src, float qx, float qy, float qz, knn_t* s) {
    const double q[3] = {qx, qy, qz};
    int c[3];
    for (int a = 0; a < 3; ++a) {
        double t = floor((q[a] - g->lo[a]) / g->h);
        if (t < 0) t = 0;
        if (t > g->dim[a] - 1) t = g->dim[a] - 1;
        c[a] = (int)t;
    }
    int maxr = g->dim[0];
    if (g->dim[1] > maxr) maxr = g->dim[1];
    if (g->dim[2] > maxr) maxr = g->dim[2];
    for (int r = 0; r <= maxr; ++r) {
        if (r > 0 && s->n == s->k) {
            /* a point in ring r lies at least (r-1)*h away (margin for rounding) */
            double lb = (r - 1) * (double)g->h;
            if (lb * lb * 0.999 > s->d[s->n - 1]) break;
        }
        for (int z = c[2] - r; z <= c[2] + r; ++z) {
            if (z < 0 || z >= g->dim[2]) continue;
            for (int y = c[1] - r; y <= c[1] + r; ++y) {
                if (y < 0 || y >= g->dim[1]) continue;
                for (int x = c[0] - r; x <= c[0] + r; ++x) {
                    if (x < 0 || x >= g->dim[0]) continue;
                    if (abs(x - c[0]) != r && abs(y - c[1]) != r && abs(z - c[2]) != r) continue;
                    const int cc = (z * g->dim[1] + y) * g->dim[0] + x;
                    for (int m = g->start[cc]; m < g->start[cc + 1]; ++m) {
                        const int i = g->idx[m];
                        knn_offer(s, sqdist(src + 3 * (size_t)i, qx, qy, qz), i);
                    }
                }
            }
        }
    }
}

/* ColorYUV(const pcl::PointXYZRGB&) (include/common/common.h:94-98) */
static void yuv_of_rgb(const uint8_t* c, float* o) {
    const float r = c[0], g = c[1], b = c[2];
    o[0] = r * 0.299f + g * 0.587f + b * 0.114f;
    o[1] = r * -0.168736f - g * 0.331264f + b * 0.5f + 128;
    o[2] = r * 0.5f - g * 0.418688f - b * 0.081312f + 128;
}

/* common::MSE::Compute (src/registration/registration_base.cc:168-223):
 * every point of p against its nearest neighbour in q, then q against p,
 * accumulated as the reference does -- the geometric error in float, each
 * colour term as a double square added into a float sum -- and divided by
 * the cloud sizes.  out = {geo p->q, geo q->p, Y.., Y.., U.., U.., V.., V..}.
 * An empty cloud sets its side to -1 and the call returns early (:170-177).
 * Neighbour ties go to the lower index (PCL's k-d tree leaves it open). */
int pvo_cloud_quality(const float* p, const uint8_t* prgb, size_t np, const float* q, const uint8_t* qrgb, size_t nq,
                      int brute, double* out) {
    float m[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    if (!np) m[0] = m[2] = m[4] = m[6] = -1.0f;
    if (!nq) m[1] = m[3] = m[5] = m[7] = -1.0f;
    if (np && nq) {
        for (int dir = 0; dir < 2; ++dir) {
            const float* a = dir ? q : p;
            const uint8_t* ac = dir ? qrgb : prgb;
            const size_t na = dir ? nq : np;
            const float* b = dir ? p : q;
            const uint8_t* bc = dir ? prgb : qrgb;
            const size_t nb = dir ? np : nq;
            fgrid_t g;
            memset(&g, 0, sizeof(g));
            if (!brute && fgrid_build(&g, b, nb)) return PVO_ERR_NOMEM;
            float geo = 0, ey = 0, eu = 0, ev = 0;
            for (size_t i = 0; i < na; ++i) {
                knn_t s;
                s.n = 0;
                s.k = 1;
                const float* x = a + 3 * i;
                if (brute)
                    for (size_t j = 0; j < nb; ++j) knn_offer(&s, sqdist(b + 3 * j, x[0], x[1], x[2]), (int)j);
                else
                    fgrid_knn(&g, b, x[0], x[1], x[2], &s);
                geo += s.d[0];
                float ya[3], yb[3];
                yuv_of_rgb(ac + 3 * i, ya);
                yuv_of_rgb(bc + 3 * (size_t)s.i[0], yb);
                /* pp is the point of p, qq its neighbour in q (and the other way round) */
                const float dy = dir ? yb[0] - ya[0] : ya[0] - yb[0];
                const float du = dir ? yb[1] - ya[1] : ya[1] - yb[1];
                const float dv = dir ? yb[2] - ya[2] : ya[2] - yb[2];
                ey = (float)((double)ey + pow((double)dy, 2));
                eu = (float)((double)eu + pow((double)du, 2));
                ev = (float)((double)ev + pow((double)dv, 2));
            }
            if (!brute) fgrid_free(&g);
            m[dir] = geo / (float)na;
            m[2 + dir] = ey / (float)na;
            m[4 + dir] = eu / (float)na;
            m[6 + dir] = ev / (float)na;
        }
    }
    for (int k = 0; k < 8; ++k) out[k] = m[k];
    return PVO_OK;
}

int pvo_knn_colors(const float* q, size_t nq, const float* src, const uint8_t* rgb, size_t ns, int k, int brute,
                   float* yuv_out) {
    if (!src || !rgb || !ns || k < 1 || k > KNN_MAX || (nq && (!q || !yuv_out))) return PVO_ERR_ARG;
    fgrid_t g;
    memset(&g, 0, sizeof(g));
    if (!brute && fgrid_build(&g, src, ns)) return PVO_ERR_NOMEM;
    for (size_t t = 0; t < nq; ++t) {
        knn_t s;
        s.n = 0;
        s.k = k < (int)ns ? k : (int)ns;
        const float qx = q[3 * t], qy = q[3 * t + 1], qz = q[3 * t + 2];
        if (brute) {
            for (size_t i = 0; i < ns; ++i) knn_offer(&s, sqdist(src + 3 * i, qx, qy, qz), (int)i);
        } else {
            fgrid_knn(&g, src, qx, qy, qz, &s);
        }
        knn_interp(&s, rgb, yuv_out + 3 * t);
    }
    if (!brute) fgrid_free(&g);
    return PVO_OK;
}

typedef struct {
    int npairs, k;
    const float* q;
    const uint64_t* qoff;
    const uint32_t* qn;
    const float* src;
    const uint8_t* rgb;
    const uint32_t* soff;
    float* yuv;
    const uint64_t* out_off;
    pthread_mutex_t mu;
    int next, rc;
} knn_job_t;

static void* knn_worker(void* arg) {
    knn_job_t* j = (knn_job_t*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        int p = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (p >= j->npairs) break;
        const uint32_t a = j->soff[p], b = j->soff[p + 1];
        int rc = pvo_knn_colors(j->q + 3 * j->qoff[p], j->qn[p], j->src + 3ull * a, j->rgb + 3ull * a, b - a, j->k, 0,
                                j->yuv + 3 * j->out_off[p]);
        if (rc) {
            pthread_mutex_lock(&j->mu);
            j->rc = rc;
            pthread_mutex_unlock(&j->mu);
        }
    }
    return NULL;
}

int pvo_knn_colors_batch(int npairs, const float* q, const uint64_t* qoff, const uint32_t* qn, const float* src,
                         const uint8_t* rgb, const uint32_t* soff, int k, float* yuv, const uint64_t* out_off,
                         int nthreads) {
    knn_job_t j = {npairs, k, q, qoff, qn, src, rgb, soff, yuv, out_off};
    pthread_mutex_init(&j.mu, NULL);
    j.next = 0;
    j.rc = 0;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    pthread_t th[256];
    for (int t = 0; t < nthreads; ++t) pthread_create(&th[t], NULL, knn_worker, &j);
    for (int t = 0; t < nthreads; ++t) pthread_join(th[t], NULL);
    pthread_mutex_destroy(&j.mu);
    return j.rc;
}
