// encoder.cc -- CPU GoP encoder back end (see encoder.h).
#include "encoder.h"

#include <algorithm>
#include <cfloat>
#include <cmath>
#include <cstring>
#include <numeric>

#include "pvvc_gb300.h"

namespace pvvc {
namespace {

constexpr int kL = 4, kU0 = 3, kD0 = 1, kU1 = 2, kD1 = 1;
// child slot pairs of the 7 butterflies, include/octree/octree.h:79
constexpr int kPair[8][2] = {{0, 0}, {2, 3}, {4, 6}, {5, 7}, {8, 12}, {9, 13}, {10, 14}, {11, 15}};

inline uint64_t zigzag(int64_t x) { return x < 0 ? ((uint64_t)(-x) << 1) - 1 : (uint64_t)x << 1; }
inline int64_t unzigzag(uint64_t x) { return (x & 1) ? -(int64_t)(x >> 1) - 1 : (int64_t)(x >> 1); }
inline uint64_t mask(int k) { return k >= 64 ? ~0ull : ((1ull << k) - 1); }

// MSB-first bit writer; same bytes as RLGREncoder's Write/Flush
// (entropy_codec.cc:22-47), including its '+' when a value exceeds its width.
struct BitWriter {
    std::vector<uint8_t> out;
    uint64_t acc = 0;  // pending bits, right-aligned
    int n = 0;         // pending bit count (< 8 between calls)
    void put(uint64_t v, int bits) {
        if (bits > 56) {
            put(v >> 32, bits - 32);
            put(v & mask(32), 32);
            return;
        }
        acc = (acc << bits) + v;
        n += bits;
        while (n >= 8) {
            n -= 8;
            out.push_back((uint8_t)(acc >> n));
        }
    }
    void gr(uint64_t x, int k) {  // GRWrite, entropy_codec.cc:49-63
        uint64_t p = x >> k;
        if (p < 32) {
            put(mask((int)p + 1) - 1, (int)p + 1);
            put(x & mask(k), k);
        } else {
            put(mask(32), 32);
            put(x, 32);
        }
    }
};

}  // namespace

std::vector<uint8_t> rlgr_encode(const int64_t* sym, size_t n) {
    BitWriter w;
    w.out.reserve(n / 2 + 16);
    uint64_t u = 0, kP = 0, kRP = 2 * kL, m = 0, k = 0;
    for (size_t i = 0; i < n; ++i) {
        u = zigzag(sym[i]);
        k = kP / kL;
        const uint64_t kR = kRP / kL;
        if (k) {
            if (u) {
                --u;
                w.put(0, 1);
                w.put(m, (int)k);
                w.gr(u, (int)kR);
                const uint64_t p = u >> kR;
                if (p) kRP = std::min<uint64_t>(kRP + p - 1, 32 * kL);
                else kRP = kRP < 2 ? 0 : kRP - 2;
                kP = kP < (uint64_t)kD1 ? 0 : kP - kD1;
                m = 0;
            } else if (++m == (1ull << k)) {
                w.put(1, 1);
                kP += kU1;
                m = 0;
            }
        } else {
            w.gr(u, (int)kR);
            const uint64_t p = u >> kR;
            if (p) kRP = std::min<uint64_t>(kRP + p - 1, 32 * kL);
            else kRP = kRP < 2 ? 0 : kRP - 2;
            if (u) kP = kP < (uint64_t)kD0 ? 0 : kP - kD0;
            else kP += kU0;
            m = 0;
        }
    }
    if (n > 0 && k && !u) {  // trailing run, entropy_codec.cc:144-147
        w.put(0, 1);
        w.put(m, (int)(kP / kL));
    }
    if (w.n) w.put(0, 8 - w.n);  // byte padding, :150-159
    return std::move(w.out);
}

int rlgr_decode(const uint8_t* in, size_t nbytes, size_t nsym, int64_t* out) {
    const uint8_t* p = in;
    const uint8_t* end = in + nbytes;
    uint64_t win = 0;  // next bits, MSB-aligned
    int avail = 0;     // valid bits in win
    uint64_t consumed_ok = 0;
    auto refill = [&]() {
        while (avail <= 56) {
            uint64_t b = p < end ? *p++ : 0;
            win |= b << (56 - avail);
            avail += 8;
        }
    };
    const uint64_t total_bits = (uint64_t)nbytes * 8;
    uint64_t used = 0;
    auto take = [&](int bits) -> uint64_t {  // bits <= 32
        refill();
        uint64_t v = bits ? win >> (64 - bits) : 0;
        win = bits == 64 ? 0 : win << bits;
        avail -= bits;
        used += bits;
        return v;
    };
    auto ones = [&]() -> int {  // count leading ones (<= 32), not consumed
        refill();
        uint64_t inv = ~win;
        int c = inv ? __builtin_clzll(inv) : 64;
        return c > 32 ? 32 : c;
    };
    auto gr = [&](int k) -> uint64_t {
        int q = ones();
        if (q >= 32) {
            take(32);
            return take(32);
        }
        take(q + 1);
        return ((uint64_t)q << k) + take(k);
    };
    uint64_t kP = 0, kRP = 2 * kL;
    size_t i = 0;
    (void)consumed_ok;
    while (i < nsym) {
        uint64_t k = kP / kL;
        const int kR = (int)(kRP / kL);
        uint64_t u;
        if (k) {
            uint64_t m = 0;
            for (;;) {
                int q = ones();
                int t = q < 32 ? q : 31;
                for (int j = 0; j < t; ++j) {
                    m += 1ull << k;
                    kP += kU1;
                    k = kP / kL;
                }
                take(t);
                if (q < 32) break;
                if (used > total_bits) return PVVC_ERR_OVERRUN;
            }
            take(1);
            m += take((int)k);
            if (used > total_bits) return PVVC_ERR_OVERRUN;
            for (; m && i < nsym; --m) out[i++] = 0;
            if (i >= nsym) break;
            u = gr(kR);
            if (used > total_bits) return PVVC_ERR_OVERRUN;
            out[i++] = unzigzag(u + 1);
            const uint64_t pq = u >> kR;
            if (pq) kRP = std::min<uint64_t>(kRP + pq - 1, 32 * kL);
            else kRP = kRP < 2 ? 0 : kRP - 2;
            kP = kP < (uint64_t)kD1 ? 0 : kP - kD1;
        } else {
            u = gr(kR);
            if (used > total_bits) return PVVC_ERR_OVERRUN;
            out[i++] = unzigzag(u);
            const uint64_t pq = u >> kR;
            if (pq) kRP = std::min<uint64_t>(kRP + pq - 1, 32 * kL);
            else kRP = kRP < 2 ? 0 : kRP - 2;
            if (u) kP = kP < (uint64_t)kD0 ? 0 : kP - kD0;
            else kP += kU0;
        }
    }
    return PVVC_OK;
}

// ---- octree ---------------------------------------------------------------

int PatchTree::build(const float* xyz, size_t n, float resolution) {
    if (!xyz || n == 0 || resolution < 0.0f) return PVVC_ERR_ARG;
    // bounding box and tree size exactly as raht_octree.cc:77-103
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_TRUE_MIN, FLT_TRUE_MIN, FLT_TRUE_MIN};
    for (size_t i = 0; i < n; ++i)
        for (int a = 0; a < 3; ++a) {
            mn[a] = std::min(mn[a], xyz[3 * i + a]);
            mx[a] = std::max(mx[a], xyz[3 * i + a]);
        }
    for (int a = 0; a < 3; ++a) center_[a] = mx[a] / 2.0f + mn[a] / 2.0f;
    float maxr = std::max(mx[0] - mn[0], std::max(mx[1] - mn[1], mx[2] - mn[2]));
    if (maxr <= 0.0f) maxr = 1.0f;
    const int max_h = (int)std::ceil(std::log2(maxr));
    const int ths_h = (int)std::ceil(std::log2(resolution));
    height_ = max_h - ths_h + 1;
    if (height_ <= 0) return PVVC_ERR_ARG;
    if (height_ > 22) return PVVC_ERR_TREE;  // 3 bits per level in a 64-bit path code
    range_ = std::pow(2.0f, (float)max_h);
    npts_ = n;

    // Path code of every point: the child position at each internal level,
    // computed with the same float centre updates as AddNode's recursion
    // (raht_octree.cc:138-164, SubSpaceCenter octree_base.cc:102-120).
    const int H = height_;
    std::vector<uint64_t> code(n);
    for (size_t i = 0; i < n; ++i) {
        float c[3] = {center_[0], center_[1], center_[2]};
        float r = range_;
        uint64_t k = 0;
        for (int l = 0; l < H - 1; ++l) {
            const float sub = r / 2.0f, half = sub / 2.0f;
            int pos = 0;
            for (int a = 0; a < 3; ++a) {
                const bool minus = !(xyz[3 * i + a] > c[a]);
                pos = (pos << 1) | (minus ? 1 : 0);
                c[a] = minus ? c[a] - half : c[a] + half;
            }
            k = (k << 3) | (uint64_t)pos;
            r = sub;
        }
        code[i] = k;
    }
    order_.resize(n);
    std::iota(order_.begin(), order_.end(), 0u);
    std::stable_sort(order_.begin(), order_.end(), [&](uint32_t a, uint32_t b) { return code[a] < code[b]; });

    // leaves: runs of equal codes (a leaf averages the points in its voxel)
    leaf_first_.clear();
    point_leaf_.assign(n, 0);
    std::vector<uint64_t> level_code;  // codes of the current level's nodes
    for (size_t i = 0; i < n; ++i) {
        if (i == 0 || code[order_[i]] != code[order_[i - 1]]) {
            leaf_first_.push_back((uint32_t)i);
            level_code.push_back(code[order_[i]]);
        }
        point_leaf_[order_[i]] = (uint32_t)(leaf_first_.size() - 1);
    }
    leaf_count_ = leaf_first_.size();
    leaf_first_.push_back((uint32_t)n);

    // internal levels, bottom-up: parent code = child code >> 3
    occ_.assign(H > 1 ? H - 1 : 0, {});
    first_child_.assign(H > 1 ? H - 1 : 0, {});
    for (int l = H - 2; l >= 0; --l) {
        std::vector<uint64_t> parent;
        auto& occ = occ_[l];
        auto& fc = first_child_[l];
        for (size_t j = 0; j < level_code.size(); ++j) {
            const uint64_t pc = level_code[j] >> 3;
            const int pos = (int)(level_code[j] & 7);
            if (parent.empty() || parent.back() != pc) {
                parent.push_back(pc);
                occ.push_back(0);
                fc.push_back((uint32_t)j);
            }
            occ.back() |= (uint8_t)(0x80u >> pos);
        }
        level_code.swap(parent);
    }
    return PVVC_OK;
}

std::vector<uint8_t> PatchTree::geometry() const {
    std::vector<uint8_t> g;
    const float d[6] = {center_[0], center_[1], center_[2], range_, range_, range_};
    for (float f : d) {  // SaveTreeCore, octree_base.cc:20-31 (big-endian bit patterns)
        uint32_t t;
        std::memcpy(&t, &f, 4);
        g.push_back((uint8_t)(t >> 24));
        g.push_back((uint8_t)(t >> 16));
        g.push_back((uint8_t)(t >> 8));
        g.push_back((uint8_t)t);
    }
    g.push_back((uint8_t)height_);
    for (const auto& lv : occ_) g.insert(g.end(), lv.begin(), lv.end());
    return g;
}

namespace {
struct YUV {
    float y, u, v;
};
static_assert(sizeof(YUV) == 12, "YUV rows alias float[3]");
inline YUV axpby(YUV a, float s, YUV b, float t) {  // a*s + b*t, per channel
    return {a.y * s + b.y * t, a.u * s + b.u * t, a.v * s + b.v * t};
}
}  // namespace

void PatchTree::leaf_yuv(const float* yuv, float* out) const {
    for (size_t j = 0; j < leaf_count_; ++j) {
        YUV t{0, 0, 0};
        for (uint32_t q = leaf_first_[j]; q < leaf_first_[j + 1]; ++q) {
            const float* c = yuv + 3ull * order_[q];
            t.y += c[0];
            t.u += c[1];
            t.v += c[2];
        }
        const float cnt = (float)(leaf_first_[j + 1] - leaf_first_[j]);
        out[3 * j] = t.y / cnt;
        out[3 * j + 1] = t.u / cnt;
        out[3 * j + 2] = t.v / cnt;
    }
}

void PatchTree::raht(const float* yuv, std::vector<float>* coef_out) const {
    const int H = height_;
    // leaf signal: mean colour of the voxel's points (raht_octree.cc:204-211)
    std::vector<YUV> g(leaf_count_), gn;
    std::vector<int32_t> w(leaf_count_, 1), wn;
    leaf_yuv(yuv, reinterpret_cast<float*>(g.data()));
    // bottom-up HierarchicalTransform (octree_base.cc:65-82); the AC
    // coefficients of each level are kept to be emitted top-down later.
    std::vector<std::vector<YUV>> ac(H > 1 ? H - 1 : 0);
    for (int l = H - 2; l >= 0; --l) {
        const auto& occ = occ_[l];
        const auto& fc = first_child_[l];
        const size_t nn = occ.size();
        gn.assign(nn, {0, 0, 0});
        wn.assign(nn, 0);
        auto& acl = ac[l];
        acl.clear();
        for (size_t j = 0; j < nn; ++j) {
            YUV s[16];
            int32_t ww[16];
            std::memset(s, 0, sizeof(s));
            std::memset(ww, 0, sizeof(ww));
            uint32_t ch = fc[j];
            for (int c = 0; c < 8; ++c)
                if (occ[j] & (0x80u >> c)) {
                    s[8 + c] = g[ch];
                    ww[8 + c] = w[ch];
                    ++ch;
                }
            for (int i = 7; i > 0; --i) ww[i] = ww[kPair[i][0]] + ww[kPair[i][1]];
            YUV hh[8];
            std::memset(hh, 0, sizeof(hh));
            for (int i = 7; i > 0; --i) {  // HaarTransform, octree_base.cc:164-184
                const int w0 = ww[kPair[i][0]], w1 = ww[kPair[i][1]];
                if (w0 == 0 && w1 == 0) {
                    s[i] = {0, 0, 0};
                    hh[i] = {0, 0, 0};
                    continue;
                }
                const float base = std::sqrt((float)(w0 + w1));
                const float a = std::sqrt((float)w0) / base, b = std::sqrt((float)w1) / base;
                const YUV g0 = s[kPair[i][0]], g1 = s[kPair[i][1]];
                s[i] = axpby(g0, a, g1, b);
                hh[i] = axpby(g0, -b, g1, a);
            }
            gn[j] = s[1];
            wn[j] = ww[1];
            for (int i = 1; i < 8; ++i)
                if (ww[kPair[i][0]] != 0 && ww[kPair[i][1]] != 0) acl.push_back(hh[i]);
        }
        g.swap(gn);
        w.swap(wn);
    }
    // stream: DC, then each level's ACs in BFS order; reversed (:227-241)
    std::vector<YUV> stream;
    stream.reserve(leaf_count_);
    stream.push_back(g[0]);
    for (int l = 0; l < H - 1; ++l) stream.insert(stream.end(), ac[l].begin(), ac[l].end());
    coef_out->resize(3 * stream.size());
    const size_t m = stream.size();
    for (size_t i = 0; i < m; ++i) {
        const YUV& c = stream[m - 1 - i];
        (*coef_out)[3 * i] = c.y;
        (*coef_out)[3 * i + 1] = c.u;
        (*coef_out)[3 * i + 2] = c.v;
    }
}

std::vector<uint8_t> encode_colors(const float* coef, size_t nleaf, uint8_t qp) {
    std::vector<int64_t> q(3 * nleaf);
    const float QP = (float)qp;
    for (size_t j = 0; j < nleaf; ++j)
        for (int c = 0; c < 3; ++c) q[j + c * nleaf] = (int64_t)std::round(coef[3 * j + c] / QP);
    return rlgr_encode(q.data(), q.size());
}

}  // namespace pvvc

// ---- C ABI -----------------------------------------------------------------
extern "C" int64_t pvvc_rlgr_encode(const int64_t* sym, uint64_t n, uint8_t* out, uint64_t cap) {
    if ((!sym && n) || (!out && cap)) return -PVVC_ERR_ARG;
    auto r = pvvc::rlgr_encode(sym, n);
    if (r.size() > cap) return -PVVC_ERR_CAPACITY;
    if (!r.empty()) std::memcpy(out, r.data(), r.size());
    return (int64_t)r.size();
}

extern "C" int pvvc_rlgr_decode_host(const uint8_t* in, uint64_t nbytes, uint64_t nsym, int64_t* out) {
    if ((!in && nbytes) || (!out && nsym)) return PVVC_ERR_ARG;
    return pvvc::rlgr_decode(in, nbytes, nsym, out);
}

extern "C" int pvvc_encode_patch_gop(const float* xyz, uint32_t n, const float* yuv, int32_t nframes, const uint8_t* qp,
                                     uint8_t* geo_out, uint64_t geo_cap, uint64_t* geo_len, uint8_t* col_out,
                                     uint64_t col_cap_per_frame, uint64_t* col_len, uint32_t* leaf_count) {
    if (!xyz || !n || !yuv || nframes <= 0 || !qp || !geo_out || !geo_len || !col_out || !col_len || !leaf_count)
        return PVVC_ERR_ARG;
    for (int f = 0; f < nframes; ++f)
        if (qp[f] == 0) return PVVC_ERR_ARG;  // GoP_encoding.cc:106-108
    pvvc::PatchTree t;
    int s = t.build(xyz, n);
    if (s) return s;
    auto g = t.geometry();
    if (g.size() > geo_cap) return PVVC_ERR_CAPACITY;
    std::memcpy(geo_out, g.data(), g.size());
    *geo_len = g.size();
    *leaf_count = (uint32_t)t.leaf_count();
    std::vector<float> coef;
    for (int f = 0; f < nframes; ++f) {
        t.raht(yuv + 3ull * n * f, &coef);
        auto c = pvvc::encode_colors(coef.data(), t.leaf_count(), qp[f]);
        if (c.size() > col_cap_per_frame) return PVVC_ERR_CAPACITY;
        std::memcpy(col_out + col_cap_per_frame * f, c.data(), c.size());
        col_len[f] = c.size();
    }
    return PVVC_OK;
}

extern "C" int pvvc_patch_leaf_yuv(const float* xyz, uint32_t n, const float* yuv, int32_t nframes, uint8_t* geo_out,
                                   uint64_t geo_cap, uint64_t* geo_len, float* leaf_out, uint64_t leaf_cap,
                                   uint32_t* leaf_count) {
    if (!xyz || !n || !yuv || nframes <= 0 || !geo_out || !geo_len || !leaf_out || !leaf_count) return PVVC_ERR_ARG;
    pvvc::PatchTree t;
    int s = t.build(xyz, n);
    if (s) return s;
    auto g = t.geometry();
    if (g.size() > geo_cap || t.leaf_count() > leaf_cap) return PVVC_ERR_CAPACITY;
    std::memcpy(geo_out, g.data(), g.size());
    *geo_len = g.size();
    *leaf_count = (uint32_t)t.leaf_count();
    for (int f = 0; f < nframes; ++f) t.leaf_yuv(yuv + 3ull * n * f, leaf_out + 3ull * leaf_cap * f);
    return PVVC_OK;
}
