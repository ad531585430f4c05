/* pvvc_oracle_fit.c -- TEST INFRASTRUCTURE: a CPU restatement of the
 * reference encoder's fitting cloud, PatchFitting::Compute with the direct
 * clustering every reference config selects (src/patch/patch_fitting.cc:
 * 92-136 Compute, :138-236 Clustering, :238-381 Split; octree_base.cc:
 * 102-162 SubSpaceCenter / CheckSubSpace / CheckSpaceEmpty).  Used only by
 * the tests to check the GPU version; pinned to the reference's own
 * PatchFitting compiled here (oracle/_ref).
 *
 * The reference draws its k-means seeds and its empty-cluster replacements
 * from the process-wide rand(); one call here draws from a private glibc
 * generator seeded like srand(seed), so it equals the reference's Compute
 * after srand(seed).  Nearest centroids: exact, float squared distance
 * accumulated x, y, z, the lower index among equal distances (PCL's k-d tree
 * leaves that order open). */
#define _DEFAULT_SOURCE
#include <float.h>
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#include "pvvc_oracle.h"

typedef struct {
    float x, y, z;
} p3_t;

typedef struct {
    const float* const* pts;
    const uint32_t* n;
    int np;
    float err_ths;
    int max_iter;
    int max_height;
    struct random_data rd;
    char state[128];
    float* out;
    size_t cap, nout;
    int status;
    long cells, iters, empties;
} fit_t;

static int32_t fit_rand(fit_t* f) {
    int32_t r = 0;
    random_r(&f->rd, &r);
    return r;
}

/* lists[patch] = point indices of that patch in this cell, in order */
typedef struct {
    int** idx;
    int* cnt;
} cell_t;

static void clustering(fit_t* f, const cell_t* c) {
    size_t total = 0;
    for (int i = 0; i < f->np; ++i) total += (size_t)c->cnt[i];
    const int k = (int)roundf((float)total / (float)f->np);
    ++f->cells;
    p3_t* pts = (p3_t*)malloc((total ? total : 1) * sizeof(p3_t));
    p3_t* ctr = (p3_t*)malloc((k ? k : 1) * sizeof(p3_t));
    p3_t* nxt = (p3_t*)malloc((k ? k : 1) * sizeof(p3_t));
    int* cnt = (int*)malloc((k ? k : 1) * sizeof(int));
    if (!pts || !ctr || !nxt || !cnt) {
        f->status = PVO_ERR_NOMEM;
        goto done;
    }
    size_t m = 0;
    for (int i = 0; i < f->np; ++i)
        for (int j = 0; j < c->cnt[i]; ++j) {
            const float* p = f->pts[i] + 3 * (size_t)c->idx[i][j];
            pts[m].x = p[0];
            pts[m].y = p[1];
            pts[m].z = p[2];
            ++m;
        }
    /* seeds: a partial Fisher-Yates shuffle from the back (the reference's
     * loop runs one step further, into rand() % 0, when k equals the point
     * count; that needs a single patch or half a point per patch) */
    int nc = 0;
    for (long i = (long)total - 1; i >= (long)total - k && i >= 0; --i) {
        const long j = fit_rand(f) % (i + 1);
        const p3_t t = pts[i];
        pts[i] = pts[j];
        pts[j] = t;
        ctr[nc++] = pts[i];
    }
    int iter = 1;
    for (; iter <= f->max_iter; ++iter) {
        for (int q = 0; q < k; ++q) {
            nxt[q].x = nxt[q].y = nxt[q].z = 0.0f;
            cnt[q] = 0;
        }
        for (size_t j = 0; j < total; ++j) {
            float best = FLT_MAX;
            int bi = 0;
            for (int q = 0; q < k; ++q) {
                const float dx = ctr[q].x - pts[j].x, dy = ctr[q].y - pts[j].y, dz = ctr[q].z - pts[j].z;
                float d = dx * dx;
                d = d + dy * dy;
                d = d + dz * dz;
                if (d < best) {
                    best = d;
                    bi = q;
                }
            }
            if (k) {
                nxt[bi].x += pts[j].x;
                nxt[bi].y += pts[j].y;
                nxt[bi].z += pts[j].z;
                cnt[bi]++;
            }
        }
        float error = 0.0f;
        for (int q = 0; q < k; ++q) {
            if (cnt[q] == 0) {
                ++f->empties;
                nxt[q] = pts[fit_rand(f) % total];
            } else {
                nxt[q].x /= (float)cnt[q];
                nxt[q].y /= (float)cnt[q];
                nxt[q].z /= (float)cnt[q];
            }
            error = (float)((double)error + sqrt(pow((double)(nxt[q].x - ctr[q].x), 2) + pow((double)(nxt[q].y - ctr[q].y), 2) +
                                                 pow((double)(nxt[q].z - ctr[q].z), 2)));
        }
        error /= (float)k;
        p3_t* t = ctr;
        ctr = nxt;
        nxt = t;
        if (error < f->err_ths) break;
    }
    f->iters += iter;
    if (f->nout + (size_t)k > f->cap) {
        f->status = PVO_ERR_SIZE;
    } else {
        for (int q = 0; q < k; ++q) {
            f->out[3 * f->nout] = ctr[q].x;
            f->out[3 * f->nout + 1] = ctr[q].y;
            f->out[3 * f->nout + 2] = ctr[q].z;
            ++f->nout;
        }
    }
done:
    free(pts);
    free(ctr);
    free(nxt);
    free(cnt);
}

static void split(fit_t* f, const cell_t* c, p3_t ctr, p3_t rng, int h) {
    if (f->status) return;
    int empty = 1;
    for (int i = 0; i < f->np; ++i) empty &= c->cnt[i] == 0;
    if (empty) return;
    if (h >= f->max_height) {
        clustering(f, c);
        return;
    }
    /* eight subspaces: bit 2 x <= cx, bit 1 y <= cy, bit 0 z <= cz */
    cell_t sub[8];
    for (int s = 0; s < 8; ++s) {
        sub[s].idx = (int**)malloc(f->np * sizeof(int*));
        sub[s].cnt = (int*)calloc(f->np, sizeof(int));
        for (int i = 0; i < f->np; ++i) sub[s].idx[i] = (int*)malloc(((size_t)c->cnt[i] + 1) * sizeof(int));
    }
    for (int i = 0; i < f->np; ++i)
        for (int j = 0; j < c->cnt[i]; ++j) {
            const float* p = f->pts[i] + 3 * (size_t)c->idx[i][j];
            int pos = 0;
            pos |= p[0] > ctr.x ? 0 : 1;
            pos <<= 1;
            pos |= p[1] > ctr.y ? 0 : 1;
            pos <<= 1;
            pos |= p[2] > ctr.z ? 0 : 1;
            sub[pos].idx[i][sub[pos].cnt[i]++] = c->idx[i][j];
        }
    int ok = 1;  /* CheckSubSpace: in every subspace all patches or none */
    for (int s = 0; s < 8 && ok; ++s) {
        int nonempty = 0;
        for (int i = 0; i < f->np; ++i) nonempty += sub[s].cnt[i] ? 1 : 0;
        if (nonempty != 0 && nonempty != f->np) ok = 0;
    }
    if (!ok) {
        clustering(f, c);
    } else {
        const p3_t sr = {rng.x / 2.0f, rng.y / 2.0f, rng.z / 2.0f};
        for (int s = 0; s < 8; ++s) {
            /* SubSpaceCenter (octree_base.cc:102-120) */
            p3_t sc;
            sc.x = (s & 4) ? ctr.x - sr.x / 2.0f : ctr.x + sr.x / 2.0f;
            sc.y = (s & 2) ? ctr.y - sr.y / 2.0f : ctr.y + sr.y / 2.0f;
            sc.z = (s & 1) ? ctr.z - sr.z / 2.0f : ctr.z + sr.z / 2.0f;
            split(f, &sub[s], sc, sr, h + 1);
        }
    }
    for (int s = 0; s < 8; ++s) {
        for (int i = 0; i < f->np; ++i) free(sub[s].idx[i]);
        free(sub[s].idx);
        free(sub[s].cnt);
    }
}

long pvo_fitting_cloud(int npatches, const float* const* xyz, const uint32_t* n, float clustering_ths,
                       float clustering_err_ths, int max_iter, unsigned seed, float* out, size_t cap, long* stats) {
    if (npatches < 1 || !xyz || !n || !out) return -PVO_ERR_ARG;
    fit_t f;
    memset(&f, 0, sizeof(f));
    f.pts = xyz;
    f.n = n;
    f.np = npatches;
    f.err_ths = clustering_err_ths;
    f.max_iter = max_iter;
    f.out = out;
    f.cap = cap;
    if (initstate_r(seed, f.state, sizeof(f.state), &f.rd) != 0) return -PVO_ERR_ARG;
    /* Compute (patch_fitting.cc:92-136): the maxima start at FLT_TRUE_MIN as in the reference */
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_TRUE_MIN, FLT_TRUE_MIN, FLT_TRUE_MIN};
    for (int i = 0; i < npatches; ++i)
        for (uint32_t j = 0; j < n[i]; ++j)
            for (int a = 0; a < 3; ++a) {
                const float v = xyz[i][3 * (size_t)j + a];
                mn[a] = v < mn[a] ? v : mn[a];
                mx[a] = v > mx[a] ? v : mx[a];
            }
    const p3_t ctr = {(mx[0] + mn[0]) / 2.0f, (mx[1] + mn[1]) / 2.0f, (mx[2] + mn[2]) / 2.0f};
    const p3_t rng = {mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
    const float big = fmaxf(rng.x, fmaxf(rng.y, rng.z));
    const int range_height = (int)ceilf(log2f(big));
    const int ths_height = (int)ceilf(log2f(clustering_ths));
    f.max_height = range_height - ths_height;
    cell_t root;
    root.idx = (int**)malloc(npatches * sizeof(int*));
    root.cnt = (int*)malloc(npatches * sizeof(int));
    for (int i = 0; i < npatches; ++i) {
        root.cnt[i] = (int)n[i];
        root.idx[i] = (int*)malloc(((size_t)n[i] + 1) * sizeof(int));
        for (uint32_t j = 0; j < n[i]; ++j) root.idx[i][j] = (int)j;
    }
    split(&f, &root, ctr, rng, 0);
    for (int i = 0; i < npatches; ++i) free(root.idx[i]);
    free(root.idx);
    free(root.cnt);
    if (stats) {
        stats[0] = f.cells;
        stats[1] = f.iters;
        stats[2] = f.empties;
    }
    return f.status ? -f.status : (long)f.nout;
}
