/*
 * pvvc_oracle.c -- CPU restatement of the patchVVC per-patch codec path.
 *
 * TEST INFRASTRUCTURE ONLY: the parity oracle.  The shipped library never
 * links or calls this file.  Every function names the reference file:line it
 * restates; paths are relative to the patchVVC-plus project root.
 *
 * Compile with -ffp-contract=off: the reference's arithmetic is evaluated as
 * separately rounded float operations, left to right.
 */
#include "pvvc_oracle.h"

#include <float.h>
#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

/* ------------------------------------------------------------------------ */
/* RLGR constants (include/common/entropy_codec.h:38-48)                     */
/* ------------------------------------------------------------------------ */
#define RL_L 4
#define RL_D1 1
#define RL_D0 1
#define RL_U1 2
#define RL_U0 3
#define FIX_BITS 64
#define HALF_FIX_BITS 32
#define MASK64(k) ((k) >= 64 ? ~0ULL : ((1ULL << (k)) - 1ULL))

/* zig-zag maps (entropy_codec.h:55-81) */
static uint64_t sign2unsign(int64_t x) {
    if (x < 0) return (((uint64_t)(-x)) << 1) - 1;
    return ((uint64_t)x) << 1;
}
static int64_t unsign2sign(uint64_t x) {
    int64_t a = (int64_t)(x >> 1);
    return (x & 1) ? -a - 1 : a;
}

/* ---- encoder bit writer (entropy_codec.cc:22-63) ---- */
typedef struct {
    uint64_t buf;
    int cnt;
    uint8_t* out;
    size_t len, cap;
    int overflow;
} bw_t;

static void bw_flush(bw_t* w) { /* entropy_codec.cc:22-29 */
    while (w->cnt >= 8) {
        w->cnt -= 8;
        uint8_t b = (uint8_t)((w->buf >> w->cnt) & 0xff);
        if (w->len < w->cap) w->out[w->len] = b; else w->overflow = 1;
        w->len++;
    }
}
static void bw_bit(bw_t* w, unsigned x) { /* :31-36 */
    w->buf = (w->buf << 1) | (x & 1u);
    w->cnt++;
    bw_flush(w);
}
static void bw_bits(bw_t* w, uint64_t x, int bits) { /* :38-47 */
    if (bits > FIX_BITS - 8) {
        bw_bits(w, x >> HALF_FIX_BITS, bits - HALF_FIX_BITS);
        bw_bits(w, x & MASK64(HALF_FIX_BITS), HALF_FIX_BITS);
        return;
    }
    w->buf = (bits == 64 ? 0 : (w->buf << bits)) + x; /* '+' as the reference */
    w->cnt += bits;
    bw_flush(w);
}
static void bw_gr(bw_t* w, uint64_t x, int bits) { /* :49-63 */
    uint64_t p = x >> bits;
    if (p < (uint64_t)HALF_FIX_BITS) {
        bw_bits(w, MASK64(p + 1) - 1, (int)p + 1); /* p ones then a zero */
        bw_bits(w, x & MASK64(bits), bits);
    } else {
        bw_bits(w, MASK64(HALF_FIX_BITS), HALF_FIX_BITS);
        bw_bits(w, x, HALF_FIX_BITS);
    }
}

/* RLGREncoder::Encode + GetResult (entropy_codec.cc:65-159) */
size_t pvo_rlgr_encode(const int64_t* sym, size_t n, uint8_t* out, size_t cap) {
    bw_t w = {0, 0, out, 0, cap, 0};
    uint64_t u = 0, k_P = 0, k_RP = 2 * RL_L, m = 0, k = 0, k_R, p;
    for (size_t i = 0; i < n; ++i) {
        u = sign2unsign(sym[i]);
        k = k_P / RL_L;
        k_R = k_RP / RL_L;
        if (k) {
            if (u) {
                --u;
                bw_bit(&w, 0);
                bw_bits(&w, m, (int)k);
                bw_gr(&w, u, (int)k_R);
                p = u >> k_R;
                if (p) {
                    k_RP += p - 1;
                    if (k_RP > (uint64_t)(HALF_FIX_BITS * RL_L)) k_RP = HALF_FIX_BITS * RL_L;
                } else {
                    k_RP = k_RP < 2 ? 0 : k_RP - 2;
                }
                k_P = k_P < RL_D1 ? 0 : k_P - RL_D1;
                m = 0;
            } else {
                ++m;
                if (m == ((uint64_t)1 << k)) {
                    bw_bit(&w, 1);
                    k_P += RL_U1;
                    m = 0;
                }
            }
        } else {
            bw_gr(&w, u, (int)k_R);
            p = u >> k_R;
            if (p) {
                k_RP = k_RP + p - 1;
                if (k_RP > (uint64_t)(HALF_FIX_BITS * RL_L)) k_RP = HALF_FIX_BITS * RL_L;
            } else {
                k_RP = k_RP < 2 ? 0 : k_RP - 2;
            }
            if (u) k_P = k_P < RL_D0 ? 0 : k_P - RL_D0;
            else k_P += RL_U0;
            m = 0;
        }
    }
    /* trailing run (:144-147); the reference reads k/u_data of the last
     * iteration, which are zero-initialised here for an empty input */
    if (n > 0 && k && !u) {
        bw_bit(&w, 0);
        bw_bits(&w, m, (int)(k_P / RL_L));
    }
    /* GetResult (:150-159): pad to a byte boundary with zeros */
    int r = w.cnt % 8;
    if (r) bw_bits(&w, 0, 8 - r);
    else bw_flush(&w);
    return w.overflow ? 0 : w.len;
}

/* ---- decoder bit reader (entropy_codec.cc:163-205) ---- */
typedef struct {
    uint64_t buf;
    int cnt;
    const uint8_t *now, *end;
    int err;
} br_t;

static void br_fill(br_t* r) { /* :163-176 */
    while (r->cnt <= FIX_BITS - 8) {
        if (r->now != r->end) {
            r->buf = (r->buf << 8) + *r->now++;
            r->cnt += 8;
        } else {
            return;
        }
    }
}
static unsigned br_bit(br_t* r) { /* :178-184 */
    if (r->cnt == 0) br_fill(r);
    if (r->cnt == 0) { r->err = 1; return 0; }
    --r->cnt;
    return (unsigned)((r->buf >> r->cnt) & 1u);
}
static uint64_t br_bits(br_t* r, int bits) { /* :186-194 */
    if (bits > FIX_BITS - 8) {
        uint64_t hi = br_bits(r, bits - HALF_FIX_BITS) << HALF_FIX_BITS;
        return hi + br_bits(r, HALF_FIX_BITS);
    }
    br_fill(r);
    if (bits == 0) return 0; /* masked by MASK(0) whatever the shift gives */
    if (r->cnt < bits) { r->err = 1; r->cnt = 0; return 0; }
    r->cnt -= bits;
    return (r->buf >> r->cnt) & MASK64(bits);
}
static uint64_t br_gr(br_t* r, int bits) { /* :196-205 */
    uint64_t p = 0;
    while (br_bit(r)) {
        if (r->err) return 0;
        p++;
        if (p >= (uint64_t)HALF_FIX_BITS) return br_bits(r, HALF_FIX_BITS);
    }
    return (p << bits) + br_bits(r, bits);
}

/* RLGRDecoder::Decode (entropy_codec.cc:207-283) */
int pvo_rlgr_decode(const uint8_t* in, size_t nbytes, size_t nsym, int64_t* out) {
    br_t r = {0, 0, in, in + nbytes, 0};
    uint64_t u, k_P = 0, k_RP = 2 * RL_L, m, k, k_R, p;
    size_t n = 0;
    while (n < nsym) {
        k = k_P / RL_L;
        k_R = k_RP / RL_L;
        if (k) {
            m = 0;
            while (br_bit(&r)) {
                m += (uint64_t)1 << k;
                k_P += RL_U1;
                k = k_P / RL_L;
            }
            if (r.err) return PVO_ERR_OVERRUN;
            m += br_bits(&r, (int)k);
            if (r.err) return PVO_ERR_OVERRUN;
            while (m--) {
                if (n < nsym) out[n] = 0;
                ++n;
            }
            if (n >= nsym) break;
            u = br_gr(&r, (int)k_R);
            if (r.err) return PVO_ERR_OVERRUN;
            out[n++] = unsign2sign(u + 1);
            p = u >> k_R;
            if (p) {
                k_RP += p - 1;
                if (k_RP > (uint64_t)(HALF_FIX_BITS * RL_L)) k_RP = HALF_FIX_BITS * RL_L;
            } else {
                k_RP = k_RP < 2 ? 0 : k_RP - 2;
            }
            k_P = k_P < RL_D1 ? 0 : k_P - RL_D1;
        } else {
            u = br_gr(&r, (int)k_R);
            if (r.err) return PVO_ERR_OVERRUN;
            out[n++] = unsign2sign(u);
            p = u >> k_R;
            if (p) {
                k_RP = k_RP + p - 1;
                if (k_RP > (uint64_t)(HALF_FIX_BITS * RL_L)) k_RP = HALF_FIX_BITS * RL_L;
            } else {
                k_RP = k_RP < 2 ? 0 : k_RP - 2;
            }
            if (u) k_P = k_P < RL_D0 ? 0 : k_P - RL_D0;
            else k_P += RL_U0;
        }
    }
    return PVO_OK;
}

/* ------------------------------------------------------------------------ */
/* Octree tables (include/octree/octree.h:76,79)                             */
/* ------------------------------------------------------------------------ */
static const uint8_t kNodeValue[8] = {0x80, 0x40, 0x20, 0x10, 0x08, 0x04, 0x02, 0x01};
static const int kNodeWeight[8][2] = {{0, 0}, {2, 3}, {4, 6}, {5, 7}, {8, 12}, {9, 13}, {10, 14}, {11, 15}};

typedef struct { float y, u, v; } yuv_t;

static yuv_t yuv_scale(yuv_t a, float s) { yuv_t r = {a.y * s, a.u * s, a.v * s}; return r; }
static yuv_t yuv_add(yuv_t a, yuv_t b) { yuv_t r = {a.y + b.y, a.u + b.u, a.v + b.v}; return r; }

/* HaarTransform (src/octree/octree_base.cc:164-184) */
static void haar(int w0, int w1, yuv_t g0, yuv_t g1, yuv_t* G, yuv_t* H) {
    yuv_t z = {0, 0, 0};
    if (w0 == 0 && w1 == 0) { *G = z; *H = z; return; }
    float base = sqrtf((float)(w0 + w1));
    float t00 = sqrtf((float)w0) / base, t01 = sqrtf((float)w1) / base;
    float t10 = -sqrtf((float)w1) / base, t11 = sqrtf((float)w0) / base;
    *G = yuv_add(yuv_scale(g0, t00), yuv_scale(g1, t01));
    *H = yuv_add(yuv_scale(g0, t10), yuv_scale(g1, t11));
}
/* InvertHaarTransform (octree_base.cc:186-206) */
static void ihaar(int w0, int w1, yuv_t g0, yuv_t g1, yuv_t* G, yuv_t* H) {
    yuv_t z = {0, 0, 0};
    if (w0 == 0 && w1 == 0) { *G = z; *H = z; return; }
    float base = sqrtf((float)(w0 + w1));
    float t00 = sqrtf((float)w0) / base, t01 = -sqrtf((float)w1) / base;
    float t10 = sqrtf((float)w1) / base, t11 = sqrtf((float)w0) / base;
    *G = yuv_add(yuv_scale(g0, t00), yuv_scale(g1, t01));
    *H = yuv_add(yuv_scale(g0, t10), yuv_scale(g1, t11));
}

typedef struct {
    uint8_t value;
    int32_t index[8];   /* child index in the next level, -1 if empty */
    int32_t weight[16];
    yuv_t raht[16];
    int32_t pt_first, pt_count; /* leaves: range into the encoder's point permutation */
} node_t;

typedef struct {
    node_t* v;
    size_t n, cap;
} level_t;

static int level_push(level_t* l, const node_t* nd) {
    if (l->n == l->cap) {
        size_t nc = l->cap ? l->cap * 2 : 64;
        node_t* p = (node_t*)realloc(l->v, nc * sizeof(node_t));
        if (!p) return -1;
        l->v = p;
        l->cap = nc;
    }
    l->v[l->n++] = *nd;
    return 0;
}

/* SubSpaceCenter (octree_base.cc:102-120): child of _center at _pos with the
 * child's range _range ("subrange"); bit set means the minus side. */
static void subspace_center(const float c[3], const float r[3], int pos, float out[3]) {
    out[0] = (pos & 4) ? c[0] - r[0] / 2.0f : c[0] + r[0] / 2.0f;
    out[1] = (pos & 2) ? c[1] - r[1] / 2.0f : c[1] + r[1] / 2.0f;
    out[2] = (pos & 1) ? c[2] - r[2] / 2.0f : c[2] + r[2] / 2.0f;
}

/* ------------------------------------------------------------------------ */
/* Encoder octree (src/octree/raht_octree.cc)                               */
/* ------------------------------------------------------------------------ */
struct pvo_encoder {
    int height;
    float center[3], range[3];
    level_t* levels;
    const float* xyz;  /* borrowed during construction only */
    int32_t* perm;     /* point indices grouped by leaf, leaf order */
    size_t nperm, npts;
    int32_t* scratch;
    int err;
};

/* RAHTOctree::AddNode (raht_octree.cc:115-187); pts is a stable-ordered list. */
static int32_t enc_add_node(pvo_encoder* e, int32_t* pts, size_t cnt, int h, const float c[3], const float r[3]) {
    if (cnt == 0 || e->err) return -1;
    node_t nd;
    memset(&nd, 0, sizeof(nd));
    if (h == e->height - 1) {
        nd.value = 0xff;
        nd.pt_first = (int32_t)e->nperm;
        nd.pt_count = (int32_t)cnt;
        memcpy(e->perm + e->nperm, pts, cnt * sizeof(int32_t));
        e->nperm += cnt;
        nd.weight[1] = 1;
        for (int i = 0; i < 8; ++i) nd.index[i] = -1;
        if (level_push(&e->levels[h], &nd)) { e->err = PVO_ERR_NOMEM; return -1; }
        return (int32_t)(e->levels[h].n - 1);
    }
    for (int i = 0; i < 8; ++i) nd.index[i] = -1;
    float sub[3] = {r[0] / 2.0f, r[1] / 2.0f, r[2] / 2.0f};
    /* stable 8-way partition (raht_octree.cc:141-149) */
    size_t counts[8] = {0};
    int32_t* tmp = e->scratch; /* reused: partition is finished before recursing */
    for (size_t i = 0; i < cnt; ++i) {
        const float* p = e->xyz + 3 * (size_t)pts[i];
        int pos = 0;
        pos |= p[0] > c[0] ? 0 : 1;
        pos <<= 1;
        pos |= p[1] > c[1] ? 0 : 1;
        pos <<= 1;
        pos |= p[2] > c[2] ? 0 : 1;
        counts[pos]++;
    }
    size_t start[8], s = 0;
    for (int i = 0; i < 8; ++i) { start[i] = s; s += counts[i]; }
    size_t fill[8];
    memcpy(fill, start, sizeof(fill));
    for (size_t i = 0; i < cnt; ++i) {
        const float* p = e->xyz + 3 * (size_t)pts[i];
        int pos = 0;
        pos |= p[0] > c[0] ? 0 : 1;
        pos <<= 1;
        pos |= p[1] > c[1] ? 0 : 1;
        pos <<= 1;
        pos |= p[2] > c[2] ? 0 : 1;
        tmp[fill[pos]++] = pts[i];
    }
    memcpy(pts, tmp, cnt * sizeof(int32_t));
    for (int i = 0; i < 8; ++i) {
        if (counts[i] == 0) continue;
        nd.value |= kNodeValue[i];
        float sc[3];
        subspace_center(c, sub, i, sc);
        nd.index[i] = enc_add_node(e, pts + start[i], counts[i], h + 1, sc, sub);
        if (e->err) return -1;
    }
    for (int i = 0; i < 8; ++i)
        if (nd.index[i] != -1) nd.weight[i + 8] = e->levels[h + 1].v[nd.index[i]].weight[1];
    for (int i = 7; i > 0; --i) nd.weight[i] = nd.weight[kNodeWeight[i][0]] + nd.weight[kNodeWeight[i][1]];
    if (level_push(&e->levels[h], &nd)) { e->err = PVO_ERR_NOMEM; return -1; }
    return (int32_t)(e->levels[h].n - 1);
}

/* RAHTOctree::MakeTree (raht_octree.cc:62-113) */
pvo_encoder* pvo_encoder_new(const float* xyz, size_t n, float resolution, int* status) {
    if (status) *status = PVO_ERR_ARG;
    if (!xyz || n == 0 || resolution < 0.0f) return NULL;
    float min_x = FLT_MAX, min_y = FLT_MAX, min_z = FLT_MAX;
    float max_x = FLT_TRUE_MIN, max_y = FLT_TRUE_MIN, max_z = FLT_TRUE_MIN;
    for (size_t i = 0; i < n; ++i) {
        const float* p = xyz + 3 * i;
        min_x = fminf(min_x, p[0]); min_y = fminf(min_y, p[1]); min_z = fminf(min_z, p[2]);
        max_x = fmaxf(max_x, p[0]); max_y = fmaxf(max_y, p[1]); max_z = fmaxf(max_z, p[2]);
    }
    pvo_encoder* e = (pvo_encoder*)calloc(1, sizeof(*e));
    if (!e) return NULL;
    e->center[0] = max_x / 2.0f + min_x / 2.0f;
    e->center[1] = max_y / 2.0f + min_y / 2.0f;
    e->center[2] = max_z / 2.0f + min_z / 2.0f;
    float dx = max_x - min_x, dy = max_y - min_y, dz = max_z - min_z;
    float max_range = fmaxf(dx, fmaxf(dy, dz));
    if (max_range <= 0.0f) max_range = 1.0f;
    int max_height = (int)ceilf(log2f(max_range));
    int ths_height = (int)ceilf(log2f(resolution));
    e->height = max_height - ths_height + 1;
    if (e->height <= 0) { free(e); return NULL; }
    max_range = powf(2.0f, (float)max_height);
    e->range[0] = e->range[1] = e->range[2] = max_range;
    e->levels = (level_t*)calloc((size_t)e->height, sizeof(level_t));
    e->perm = (int32_t*)malloc(n * sizeof(int32_t));
    e->scratch = (int32_t*)malloc(n * sizeof(int32_t));
    int32_t* pts = (int32_t*)malloc(n * sizeof(int32_t));
    if (!e->levels || !e->perm || !e->scratch || !pts) { free(pts); pvo_encoder_free(e); if (status) *status = PVO_ERR_NOMEM; return NULL; }
    for (size_t i = 0; i < n; ++i) pts[i] = (int32_t)i;
    e->xyz = xyz;
    e->npts = n;
    enc_add_node(e, pts, n, 0, e->center, e->range);
    free(pts);
    e->xyz = NULL;
    if (e->err) { int s = e->err; pvo_encoder_free(e); if (status) *status = s; return NULL; }
    if (status) *status = PVO_OK;
    return e;
}

void pvo_encoder_free(pvo_encoder* e) {
    if (!e) return;
    if (e->levels) for (int i = 0; i < e->height; ++i) free(e->levels[i].v);
    free(e->levels);
    free(e->perm);
    free(e->scratch);
    free(e);
}

size_t pvo_encoder_leaf_count(const pvo_encoder* e) { return e->levels[e->height - 1].n; }
int pvo_encoder_height(const pvo_encoder* e) { return e->height; }

/* SaveTreeCore (octree_base.cc:20-31) */
static void save_tree_core(const float c[3], const float r[3], int h, uint8_t* out) {
    float d[6] = {c[0], c[1], c[2], r[0], r[1], r[2]};
    for (int i = 0; i < 6; ++i) {
        uint32_t t;
        memcpy(&t, &d[i], 4);
        out[4 * i + 0] = (uint8_t)(t >> 24);
        out[4 * i + 1] = (uint8_t)(t >> 16);
        out[4 * i + 2] = (uint8_t)(t >> 8);
        out[4 * i + 3] = (uint8_t)(t >> 0);
    }
    out[24] = (uint8_t)h;
}

/* GetOctree (raht_octree.cc:47-56) */
size_t pvo_encoder_geometry(const pvo_encoder* e, uint8_t* out, size_t cap) {
    size_t need = 25;
    for (int i = 0; i < e->height - 1; ++i) need += e->levels[i].n;
    if (cap < need) return 0;
    save_tree_core(e->center, e->range, e->height, out);
    size_t o = 25;
    for (int i = 0; i < e->height - 1; ++i)
        for (size_t j = 0; j < e->levels[i].n; ++j) out[o++] = e->levels[i].v[j].value;
    return o;
}

/* HierarchicalTransform (octree_base.cc:65-82) */
static void node_forward(node_t* nd) {
    yuv_t H[8];
    memset(H, 0, sizeof(H));
    for (int i = 7; i > 0; --i) {
        yuv_t G, Hh;
        haar(nd->weight[kNodeWeight[i][0]], nd->weight[kNodeWeight[i][1]], nd->raht[kNodeWeight[i][0]], nd->raht[kNodeWeight[i][1]], &G, &Hh);
        nd->raht[i] = G;
        H[i] = Hh;
    }
    nd->raht[0] = nd->raht[1];
    for (int i = 1; i <= 7; ++i) nd->raht[i] = H[i];
}

/* RAHTOctree::RAHT (raht_octree.cc:189-247) */
int pvo_encoder_raht(pvo_encoder* e, const float* yuv, float* coef_out) {
    level_t* leaf = &e->levels[e->height - 1];
    for (size_t j = 0; j < leaf->n; ++j) {
        node_t* nd = &leaf->v[j];
        yuv_t t = {0, 0, 0};
        for (int32_t q = 0; q < nd->pt_count; ++q) {
            const float* c = yuv + 3 * (size_t)e->perm[nd->pt_first + q];
            t.y += c[0]; t.u += c[1]; t.v += c[2];
        }
        float cntf = (float)nd->pt_count; /* ColorYUV::operator/=(int) */
        t.y /= cntf; t.u /= cntf; t.v /= cntf;
        nd->raht[0] = t;
    }
    for (int i = e->height - 2; i >= 0; --i) {
        level_t* L = &e->levels[i];
        for (size_t j = 0; j < L->n; ++j) {
            node_t* nd = &L->v[j];
            for (int c = 0; c < 8; ++c)
                if (nd->index[c] != -1) nd->raht[c + 8] = e->levels[i + 1].v[nd->index[c]].raht[0];
            node_forward(nd);
        }
    }
    /* collect DC then ACs level by level, then reverse (:227-241) */
    size_t nl = leaf->n, o = 0;
    float* tmp = (float*)malloc(nl * 3 * sizeof(float));
    if (!tmp) return PVO_ERR_NOMEM;
    yuv_t dc = e->levels[0].v[0].raht[0];
    tmp[0] = dc.y; tmp[1] = dc.u; tmp[2] = dc.v;
    o = 1;
    for (int i = 0; i < e->height - 1; ++i) {
        level_t* L = &e->levels[i];
        for (size_t j = 0; j < L->n; ++j) {
            node_t* nd = &L->v[j];
            for (int idx = 1; idx < 8; ++idx) {
                if (nd->weight[kNodeWeight[idx][0]] != 0 && nd->weight[kNodeWeight[idx][1]] != 0) {
                    if (o >= nl) { free(tmp); return PVO_ERR_SIZE; }
                    tmp[3 * o + 0] = nd->raht[idx].y;
                    tmp[3 * o + 1] = nd->raht[idx].u;
                    tmp[3 * o + 2] = nd->raht[idx].v;
                    o++;
                }
            }
        }
    }
    if (o != nl) { free(tmp); return PVO_ERR_SIZE; }
    for (size_t i = 0; i < nl; ++i) memcpy(coef_out + 3 * i, tmp + 3 * (nl - 1 - i), 3 * sizeof(float));
    free(tmp);
    return PVO_OK;
}

/* quantise (GoP_encoding.cc:184-189) + RLGR (GoP_encoding.cc:190-193) */
size_t pvo_encode_colors(const float* coef, size_t nleaf, uint8_t qp, uint8_t* out, size_t cap) {
    int64_t* q = (int64_t*)malloc(3 * nleaf * sizeof(int64_t) + 8);
    if (!q) return 0;
    float QP = (float)qp;
    for (size_t j = 0; j < nleaf; ++j) {
        q[j] = (int64_t)roundf(coef[3 * j + 0] / QP);
        q[j + nleaf] = (int64_t)roundf(coef[3 * j + 1] / QP);
        q[j + 2 * nleaf] = (int64_t)roundf(coef[3 * j + 2] / QP);
    }
    size_t r = pvo_rlgr_encode(q, 3 * nleaf, out, cap);
    free(q);
    return r;
}

/* ------------------------------------------------------------------------ */
/* Decoder (src/octree/invert_raht_octree.cc)                               */
/* ------------------------------------------------------------------------ */
struct pvo_decoder {
    int valid;          /* an intra slice has been decoded */
    uint8_t type;
    int height;
    float center[3], range[3];
    level_t* levels;
    size_t n;           /* leaf count */
    float* xyz;         /* leaf centres, leaf order */
    yuv_t* ref;         /* reference colours (intra result) */
    yuv_t* out;         /* current colours */
    int fp64;           /* also run the FP64 restatement of the inverse RAHT */
    double* ref64;      /* its reference colours, 3 per leaf */
    double* out64;      /* its current colours, 3 per leaf */
};

pvo_decoder* pvo_decoder_new(void) { return (pvo_decoder*)calloc(1, sizeof(pvo_decoder)); }

static void dec_clear(pvo_decoder* d) {
    if (d->levels) for (int i = 0; i < d->height; ++i) free(d->levels[i].v);
    free(d->levels);
    free(d->xyz);
    free(d->ref);
    free(d->out);
    free(d->ref64);
    free(d->out64);
    d->levels = NULL; d->xyz = NULL; d->ref = NULL; d->out = NULL; d->ref64 = NULL; d->out64 = NULL;
    d->height = 0; d->n = 0; d->valid = 0;
}

void pvo_decoder_free(pvo_decoder* d) {
    if (!d) return;
    dec_clear(d);
    free(d);
}

size_t pvo_decoder_size(const pvo_decoder* d) { return d->n; }

/* LoadTreeCore (octree_base.cc:33-48) */
static void load_tree_core(const uint8_t* p, float c[3], float r[3], int* h) {
    float d[6];
    for (int i = 0; i < 6; ++i) {
        uint32_t t = ((uint32_t)p[4 * i] << 24) | ((uint32_t)p[4 * i + 1] << 16) | ((uint32_t)p[4 * i + 2] << 8) | (uint32_t)p[4 * i + 3];
        memcpy(&d[i], &t, 4);
    }
    c[0] = d[0]; c[1] = d[1]; c[2] = d[2];
    r[0] = d[3]; r[1] = d[4]; r[2] = d[5];
    *h = p[24];
}

/* AddPoints (invert_raht_octree.cc:203-254), written as an explicit DFS */
static int dec_add_points(pvo_decoder* d, int h, int32_t idx, const float c[3], const float r[3], size_t* npts) {
    if (h >= d->height || (size_t)idx >= d->levels[h].n) return PVO_ERR_GEOMETRY;
    node_t* nd = &d->levels[h].v[idx];
    if (h == d->height - 1) {
        nd->value = 0xff;
        nd->weight[1] = 1;
        if (*npts >= d->n) return PVO_ERR_SIZE;
        memcpy(d->xyz + 3 * (*npts), c, 3 * sizeof(float));
        (*npts)++;
        return PVO_OK;
    }
    float sub[3] = {r[0] / 2.0f, r[1] / 2.0f, r[2] / 2.0f};
    for (int i = 0; i < 8; ++i) {
        if (nd->index[i] != -1) {
            float sc[3];
            subspace_center(c, sub, i, sc);
            int s = dec_add_points(d, h + 1, nd->index[i], sc, sub, npts);
            if (s) return s;
            nd = &d->levels[h].v[idx];
        }
    }
    for (int i = 0; i < 8; ++i)
        if (nd->index[i] != -1) nd->weight[i + 8] = d->levels[h + 1].v[nd->index[i]].weight[1];
    for (int i = 7; i > 0; --i) nd->weight[i] = nd->weight[kNodeWeight[i][0]] + nd->weight[kNodeWeight[i][1]];
    return PVO_OK;
}

/* MakeTree (invert_raht_octree.cc:122-201) */
static int dec_make_tree(pvo_decoder* d, const uint8_t* geo, size_t gsz, uint32_t size) {
    if (!geo || gsz < 25) return PVO_ERR_GEOMETRY;
    load_tree_core(geo, d->center, d->range, &d->height);
    if (d->height <= 0) return PVO_ERR_GEOMETRY;
    d->levels = (level_t*)calloc((size_t)d->height, sizeof(level_t));
    if (!d->levels) return PVO_ERR_NOMEM;
    size_t it = 25, curr = 1;
    for (int lv = 0; lv < d->height - 1; ++lv) {
        size_t next = 0;
        level_t* L = &d->levels[lv];
        L->v = (node_t*)calloc(curr ? curr : 1, sizeof(node_t));
        if (!L->v) return PVO_ERR_NOMEM;
        L->n = L->cap = curr;
        for (size_t c = 0; c < curr; ++c) {
            /* the reference stops assigning when the stream ends (:168); the
             * nodes left over keep value 0 and no children */
            if (it < gsz) {
                node_t* nd = &L->v[c];
                nd->value = geo[it];
                for (int i = 0; i < 8; ++i) {
                    if ((geo[it] & kNodeValue[i]) == 0) nd->index[i] = -1;
                    else nd->index[i] = (int32_t)next++;
                }
                it++;
            } else {
                return PVO_ERR_GEOMETRY; /* reference: indexes never assigned (UB) */
            }
        }
        curr = next;
    }
    if (curr != size) return PVO_ERR_SIZE;
    level_t* leaf = &d->levels[d->height - 1];
    leaf->v = (node_t*)calloc(curr ? curr : 1, sizeof(node_t));
    if (!leaf->v) return PVO_ERR_NOMEM;
    leaf->n = leaf->cap = curr;
    for (size_t j = 0; j < curr; ++j)
        for (int i = 0; i < 8; ++i) leaf->v[j].index[i] = -1;
    d->n = curr;
    d->xyz = (float*)malloc(3 * (curr ? curr : 1) * sizeof(float));
    d->ref = (yuv_t*)calloc(curr ? curr : 1, sizeof(yuv_t));
    d->out = (yuv_t*)calloc(curr ? curr : 1, sizeof(yuv_t));
    if (!d->xyz || !d->ref || !d->out) return PVO_ERR_NOMEM;
    size_t npts = 0;
    int s = dec_add_points(d, 0, 0, d->center, d->range, &npts);
    if (s) return s;
    return npts == curr ? PVO_OK : PVO_ERR_SIZE;
}

/* InvertHierarchicalTransform (octree_base.cc:84-100) */
static void node_inverse(node_t* nd) {
    yuv_t H[8];
    for (int i = 0; i < 8; ++i) H[i] = nd->raht[i];
    nd->raht[1] = H[0];
    for (int i = 1; i < 8; ++i) {
        yuv_t G, Hh;
        ihaar(nd->weight[kNodeWeight[i][0]], nd->weight[kNodeWeight[i][1]], nd->raht[i], H[i], &G, &Hh);
        nd->raht[kNodeWeight[i][0]] = G;
        nd->raht[kNodeWeight[i][1]] = Hh;
    }
}

/* InvertRAHT (invert_raht_octree.cc:256-317); coef is in stream order
 * (Y,U,V interleaved per coefficient) and is consumed reversed. */
static int dec_inverse_raht(pvo_decoder* d, const yuv_t* coef, int predict) {
    size_t n = d->n, it = 0;
    if (n == 0) return PVO_ERR_SIZE;
#define COEF(k) coef[n - 1 - (k)]
    d->levels[0].v[0].raht[0] = COEF(it);
    ++it;
    for (int i = 0; i < d->height - 1; ++i) {
        level_t* L = &d->levels[i];
        for (size_t j = 0; j < L->n; ++j) {
            node_t* nd = &L->v[j];
            for (int idx = 1; idx < 8; ++idx) {
                if (nd->weight[kNodeWeight[idx][0]] != 0 && nd->weight[kNodeWeight[idx][1]] != 0) {
                    if (it >= n) return PVO_ERR_SIZE;
                    nd->raht[idx] = COEF(it);
                    ++it;
                }
            }
            node_inverse(nd);
            for (int c = 0; c < 8; ++c)
                if (nd->index[c] != -1) d->levels[i + 1].v[nd->index[c]].raht[0] = nd->raht[c + 8];
        }
    }
#undef COEF
    level_t* leaf = &d->levels[d->height - 1];
    for (size_t j = 0; j < n; ++j) d->out[j] = leaf->v[j].raht[0];
    if (predict) {
        for (size_t j = 0; j < n; ++j) {
            d->out[j].y += d->ref[j].y;
            d->out[j].u += d->ref[j].u;
            d->out[j].v += d->ref[j].v;
        }
    } else {
        memcpy(d->ref, d->out, n * sizeof(yuv_t));
    }
    return PVO_OK;
}

/* The inverse RAHT of dec_inverse_raht in FP64: the same tree, weights,
 * coefficient order and butterfly order (InvertHaarTransform,
 * octree_base.cc:186-206, with sqrt and the divisions in double), the
 * dequantised coefficients exact as doubles, the reference colours of a
 * predictive slice the FP64 intra result.  It measures the error of the FP32
 * arithmetic the reference decoder (and the product, bit for bit) uses. */
static int dec_inverse_raht_fp64(pvo_decoder* d, const int64_t* sym, uint8_t qp, int predict) {
    const size_t n = d->n;
    if (!d->out64) d->out64 = (double*)calloc(3 * (n ? n : 1), sizeof(double));
    if (!d->ref64) d->ref64 = (double*)calloc(3 * (n ? n : 1), sizeof(double));
    if (!d->out64 || !d->ref64) return PVO_ERR_NOMEM;
    /* coefficient k of the stream order, reversed per plane (invert_raht_octree.cc:63-69) */
#define C64(k, p) ((double)(sym[(size_t)(p) * n + (n - 1 - (k))] * (int64_t)qp))
    size_t widest = 1;
    for (int i = 0; i < d->height; ++i) widest = d->levels[i].n > widest ? d->levels[i].n : widest;
    double* cur = (double*)malloc(3 * widest * sizeof(double));
    double* nxt = (double*)malloc(3 * widest * sizeof(double));
    if (!cur || !nxt) { free(cur); free(nxt); return PVO_ERR_NOMEM; }
    size_t it = 0;
    for (int p = 0; p < 3; ++p) cur[p] = C64(0, p);
    ++it;
    for (int i = 0; i < d->height - 1; ++i) {
        const level_t* L = &d->levels[i];
        for (size_t j = 0; j < L->n; ++j) {
            const node_t* nd = &L->v[j];
            double g[16][3], h[8][3];
            for (int p = 0; p < 3; ++p) g[1][p] = cur[3 * j + p];
            for (int idx = 1; idx < 8; ++idx) {
                const int coded = nd->weight[kNodeWeight[idx][0]] != 0 && nd->weight[kNodeWeight[idx][1]] != 0;
                if (coded && it >= n) { free(cur); free(nxt); return PVO_ERR_SIZE; }
                for (int p = 0; p < 3; ++p) h[idx][p] = coded ? C64(it, p) : 0.0;
                if (coded) ++it;
            }
            for (int idx = 1; idx < 8; ++idx) {
                const int w0 = nd->weight[kNodeWeight[idx][0]], w1 = nd->weight[kNodeWeight[idx][1]];
                double a = 0, b = 0;
                if (w0 || w1) {
                    const double base = sqrt((double)(w0 + w1));
                    a = sqrt((double)w0) / base;
                    b = sqrt((double)w1) / base;
                }
                for (int p = 0; p < 3; ++p) {
                    const double x = g[idx][p], y = h[idx][p];
                    g[kNodeWeight[idx][0]][p] = a * x - b * y;
                    g[kNodeWeight[idx][1]][p] = b * x + a * y;
                }
            }
            for (int c = 0; c < 8; ++c)
                if (nd->index[c] != -1)
                    for (int p = 0; p < 3; ++p) nxt[3 * (size_t)nd->index[c] + p] = g[c + 8][p];
        }
        double* t = cur; cur = nxt; nxt = t;
    }
#undef C64
    for (size_t j = 0; j < n; ++j)
        for (int p = 0; p < 3; ++p) {
            const double v = cur[3 * j + p];
            if (predict) d->out64[3 * j + p] = v + d->ref64[3 * j + p];
            else d->out64[3 * j + p] = d->ref64[3 * j + p] = v;
        }
    free(cur);
    free(nxt);
    return PVO_OK;
}

void pvo_decoder_enable_fp64(pvo_decoder* d, int on) { d->fp64 = on; }

int pvo_decoder_get_yuv_fp64(const pvo_decoder* d, double* yuv) {
    if (!d->valid || !d->fp64 || !d->out64) return PVO_ERR_NO_REFERENCE;
    memcpy(yuv, d->out64, 3 * d->n * sizeof(double));
    return PVO_OK;
}

/* SetSlice (invert_raht_octree.cc:22-85) */
int pvo_decoder_set_slice(pvo_decoder* d, uint8_t type, uint32_t size, uint8_t qp,
                          const uint8_t* geo, size_t gsz, const uint8_t* col, size_t csz) {
    if (!(type & PVO_TYPE_VALID)) return PVO_ERR_BAD_SLICE;
    if (!geo && !col) return PVO_ERR_BAD_SLICE;
    int predict = (type & PVO_TYPE_PREDICT) != 0;
    if (!d->valid && predict) return PVO_ERR_NO_REFERENCE;
    if (predict && size != d->n) return PVO_ERR_SIZE;
    int64_t* sym = (int64_t*)malloc(3 * (size_t)size * sizeof(int64_t) + 8);
    yuv_t* coef = (yuv_t*)malloc((size_t)size * sizeof(yuv_t) + 8);
    if (!sym || !coef) { free(sym); free(coef); return PVO_ERR_NOMEM; }
    int s = pvo_rlgr_decode(col, csz, 3 * (size_t)size, sym);
    if (s) { free(sym); free(coef); return s; }
    /* dequantise (:63-69): float(int64 * qp) */
    for (uint32_t i = 0; i < size; ++i) {
        coef[i].y = (float)(sym[i] * (int64_t)qp);
        coef[i].u = (float)(sym[i + size] * (int64_t)qp);
        coef[i].v = (float)(sym[i + 2 * (size_t)size] * (int64_t)qp);
    }
    if (!predict) {
        const int fp64 = d->fp64;
        dec_clear(d);
        d->fp64 = fp64;
        s = dec_make_tree(d, geo, gsz, size);
        if (s) { dec_clear(d); free(coef); free(sym); return s; }
    }
    s = dec_inverse_raht(d, coef, predict);
    free(coef);
    if (!s && d->fp64) s = dec_inverse_raht_fp64(d, sym, qp, predict);
    free(sym);
    if (s) return s;
    d->valid = 1;
    d->type = type;
    return PVO_OK;
}

/* ColorYUV::ConvertRGB (include/common/common.h:154-158) */
void pvo_yuv_to_rgb(const float* c, uint8_t* rgb, float* rgb_f) {
    float r = c[0] + 1.4020f * (c[2] - 128.0f);
    float g = c[0] - 0.3441f * (c[1] - 128.0f) - 0.7141f * (c[2] - 128.0f);
    float b = c[0] + 1.7720f * (c[1] - 128.0f);
    float v[3] = {roundf(r), roundf(g), roundf(b)};
    for (int i = 0; i < 3; ++i) {
        if (rgb_f) rgb_f[i] = v[i];
        float x = v[i] < 0.0f ? 0.0f : (v[i] > 255.0f ? 255.0f : v[i]);
        if (rgb) rgb[i] = (uint8_t)x;
    }
}

/* GetPatch (invert_raht_octree.cc:87-120) */
int pvo_decoder_get_patch(const pvo_decoder* d, float* xyz, float* yuv, uint8_t* rgb) {
    if (!d->valid || d->n == 0) return PVO_ERR_NO_REFERENCE;
    if (xyz) memcpy(xyz, d->xyz, 3 * d->n * sizeof(float));
    for (size_t i = 0; i < d->n; ++i) {
        const float c[3] = {d->out[i].y, d->out[i].u, d->out[i].v};
        if (yuv) memcpy(yuv + 3 * i, c, sizeof(c));
        if (rgb) pvo_yuv_to_rgb(c, rgb + 3 * i, NULL);
    }
    return PVO_OK;
}

/* pvvc_decompression.cc:141-150 */
void pvo_transform(const float* m, const float* in, size_t n, float* out) {
    for (size_t i = 0; i < n; ++i) {
        float x = in[3 * i], y = in[3 * i + 1], z = in[3 * i + 2];
        out[3 * i + 0] = x * m[0] + y * m[1] + z * m[2] + m[3];
        out[3 * i + 1] = x * m[4] + y * m[5] + z * m[6] + m[7];
        out[3 * i + 2] = x * m[8] + y * m[9] + z * m[10] + m[11];
    }
}

/* ------------------------------------------------------------------------ */
/* Frame decode with a task queue over slices (pvvc_decompression.cc:86-150) */
/* ------------------------------------------------------------------------ */
typedef struct {
    pvo_decoder** dec;
    int ndec;
    const pvo_frame* f;
    float* xyz;
    uint8_t* rgb;
    int32_t* status;
    pthread_mutex_t mu;
    uint32_t next;
} frame_job_t;

static void decode_one(frame_job_t* j, uint32_t s) {
    const pvo_frame* f = j->f;
    int32_t pi = f->index[s];
    if (pi < 0 || pi >= j->ndec || !j->dec[pi]) { j->status[s] = PVO_ERR_ARG; return; }
    pvo_decoder* d = j->dec[pi];
    int st = pvo_decoder_set_slice(d, f->type[s], f->size[s], f->qp[s], f->geo[s], f->gsz[s], f->col[s], f->csz[s]);
    if (st == PVO_OK) {
        size_t n = d->n;
        float* xyz = j->xyz + 3 * f->out_off[s];
        uint8_t* rgb = j->rgb + 3 * f->out_off[s];
        pvo_decoder_get_patch(d, xyz, NULL, rgb);
        pvo_transform(f->mv + 16 * (size_t)s, xyz, n, xyz);
    }
    j->status[s] = st;
}

static void* frame_worker(void* arg) {
    frame_job_t* j = (frame_job_t*)arg;
    for (;;) {
        pthread_mutex_lock(&j->mu);
        uint32_t s = j->next++;
        pthread_mutex_unlock(&j->mu);
        if (s >= j->f->n) break;
        decode_one(j, s);
    }
    return NULL;
}

int pvo_decode_frame(pvo_decoder** decoders, int ndecoders, const pvo_frame* f,
                     float* xyz_out, uint8_t* rgb_out, int32_t* status, int nthreads) {
    frame_job_t j;
    j.dec = decoders; j.ndec = ndecoders; j.f = f; j.xyz = xyz_out; j.rgb = rgb_out; j.status = status;
    j.next = 0;
    pthread_mutex_init(&j.mu, NULL);
    if (nthreads <= 1) {
        frame_worker(&j);
    } else {
        pthread_t* th = (pthread_t*)malloc((size_t)nthreads * sizeof(pthread_t));
        int started = 0;
        for (int i = 0; i < nthreads; ++i)
            if (pthread_create(&th[i], NULL, frame_worker, &j) == 0) started++;
            else break;
        if (started == 0) frame_worker(&j);
        for (int i = 0; i < started; ++i) pthread_join(th[i], NULL);
        free(th);
    }
    pthread_mutex_destroy(&j.mu);
    int bad = 0;
    for (uint32_t s = 0; s < f->n; ++s) bad |= status[s] != 0;
    return bad ? PVO_ERR_ARG : PVO_OK;
}
