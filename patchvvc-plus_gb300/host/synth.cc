// synth.cc -- synthetic sequences and their bitstreams (see synth.h).
#include "synth.h"

#include <algorithm>
#include <atomic>
#include <cmath>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "bitstream.h"
#include "encoder.h"
#include "pvvc_gb300.h"

namespace {

// ---- deterministic hashing / random numbers --------------------------------
inline uint64_t mix64(uint64_t x) {  // splitmix64 finaliser
    x += 0x9E3779B97F4A7C15ull;
    x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
    x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
    return x ^ (x >> 31);
}
inline uint64_t hash4(uint64_t a, uint64_t b, uint64_t c, uint64_t d) {
    return mix64(mix64(mix64(mix64(a) ^ b) ^ c) ^ d);
}
inline double u01(uint64_t h) { return (double)(h >> 11) * (1.0 / 9007199254740992.0); }
inline double normal(uint64_t h) {  // Box-Muller from one 64-bit hash
    double u1 = ((double)(h >> 40) + 0.5) / 16777216.0;
    double u2 = (double)((h >> 16) & 0xFFFFFF) / 16777216.0;
    return std::sqrt(-2.0 * std::log(u1)) * std::cos(6.283185307179586 * u2);
}

struct Rng {
    uint64_t s;
    explicit Rng(uint64_t seed) : s(seed) {}
    uint64_t next() { return s = mix64(s); }
    double uniform(double a, double b) { return a + (b - a) * u01(next()); }
    double gauss() { return normal(next()); }
};

struct Mat3 {
    double m[9];
};
Mat3 mul(const Mat3& a, const Mat3& b) {
    Mat3 r;
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) r.m[3 * i + j] = a.m[3 * i] * b.m[j] + a.m[3 * i + 1] * b.m[3 + j] + a.m[3 * i + 2] * b.m[6 + j];
    return r;
}
Mat3 axis_angle(const double a[3], double th) {
    const double c = std::cos(th), s = std::sin(th), t = 1 - c, x = a[0], y = a[1], z = a[2];
    return {{t * x * x + c, t * x * y - s * z, t * x * z + s * y, t * x * y + s * z, t * y * y + c, t * y * z - s * x,
             t * x * z - s * y, t * y * z + s * x, t * z * z + c}};
}
void rand_axis(Rng& r, double a[3]) {
    double n = 0;
    do {
        for (int i = 0; i < 3; ++i) a[i] = r.gauss();
        n = std::sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
    } while (n < 1e-6);
    for (int i = 0; i < 3; ++i) a[i] /= n;
}

struct Prim {
    int kind;           // 0 ellipsoid, 1 capsule
    double ax[3];       // ellipsoid semi-axes; capsule: half-length, radius, -
    Mat3 R0;
    double axis[3], omega;  // rotation axis and angle per frame
    double C0[3], A[3], phase[3];
    double cphase;
    uint64_t tex;
};

constexpr double kTransOmega = 0.05;  // rad / frame of the oscillating translation

void prim_pose(const Prim& p, int t, Mat3* R, double C[3]) {
    *R = mul(axis_angle(p.axis, p.omega * t), p.R0);
    for (int i = 0; i < 3; ++i) C[i] = p.C0[i] + p.A[i] * std::sin(kTransOmega * t + p.phase[i]);
}

// canonical surface voxels (local frame, integer lattice)
std::vector<int16_t> surface(const Prim& p) {
    std::vector<int16_t> out;
    auto inside = [&](double x, double y, double z) {
        if (p.kind == 0) {
            const double u = x / p.ax[0], v = y / p.ax[1], w = z / p.ax[2];
            return u * u + v * v + w * w <= 1.0;
        }
        const double h = p.ax[0], r = p.ax[1];
        const double zc = std::max(-h, std::min(h, z));
        return x * x + y * y + (z - zc) * (z - zc) <= r * r;
    };
    int ext[3];
    if (p.kind == 0) {
        for (int i = 0; i < 3; ++i) ext[i] = (int)std::ceil(p.ax[i]) + 1;
    } else {
        ext[0] = ext[1] = (int)std::ceil(p.ax[1]) + 1;
        ext[2] = (int)std::ceil(p.ax[0] + p.ax[1]) + 1;
    }
    for (int x = -ext[0]; x <= ext[0]; ++x)
        for (int y = -ext[1]; y <= ext[1]; ++y)
            for (int z = -ext[2]; z <= ext[2]; ++z) {
                if (!inside(x, y, z)) continue;
                if (inside(x + 1, y, z) && inside(x - 1, y, z) && inside(x, y + 1, z) && inside(x, y - 1, z) &&
                    inside(x, y, z + 1) && inside(x, y, z - 1))
                    continue;
                out.push_back((int16_t)x);
                out.push_back((int16_t)y);
                out.push_back((int16_t)z);
            }
    return out;
}

// 3-D value noise, lattice 32 voxels, smoothstep interpolation, in [0,1)
double value_noise(double x, double y, double z, uint64_t seed) {
    const double L = 32.0;
    x /= L;
    y /= L;
    z /= L;
    const double fx = std::floor(x), fy = std::floor(y), fz = std::floor(z);
    const double tx = x - fx, ty = y - fy, tz = z - fz;
    auto sm = [](double t) { return t * t * (3 - 2 * t); };
    const double sx = sm(tx), sy = sm(ty), sz = sm(tz);
    auto lat = [&](int64_t i, int64_t j, int64_t k) { return u01(hash4(seed, (uint64_t)i, (uint64_t)j, (uint64_t)k)); };
    const int64_t ix = (int64_t)fx, iy = (int64_t)fy, iz = (int64_t)fz;
    double c[2][2][2];
    for (int a = 0; a < 2; ++a)
        for (int b = 0; b < 2; ++b)
            for (int d = 0; d < 2; ++d) c[a][b][d] = lat(ix + a, iy + b, iz + d);
    auto lerp = [](double a, double b, double t) { return a + (b - a) * t; };
    const double x00 = lerp(c[0][0][0], c[1][0][0], sx), x10 = lerp(c[0][1][0], c[1][1][0], sx);
    const double x01 = lerp(c[0][0][1], c[1][0][1], sx), x11 = lerp(c[0][1][1], c[1][1][1], sx);
    return lerp(lerp(x00, x10, sy), lerp(x01, x11, sy), sz);
}

// ColorYUV(const pcl::PointXYZRGB&), include/common/common.h:95-99
inline void rgb_to_yuv(uint8_t r8, uint8_t g8, uint8_t b8, float* o) {
    const float r = r8, g = g8, b = b8;
    o[0] = r * 0.299f + g * 0.587f + b * 0.114f;
    o[1] = r * -0.168736f - g * 0.331264f + b * 0.5f + 128;
    o[2] = r * 0.5f - g * 0.418688f - b * 0.081312f + 128;
}

struct GofData {
    int t0 = 0, nframes = 0;
    std::vector<int32_t> vox;     // n x 3 integer voxel coordinates (world, frame t0)
    std::vector<float> mat;       // n x 3 material coordinates
    std::vector<int32_t> prim;    // primitive id per point
    std::vector<uint32_t> patch_first;  // patch ranges (+ sentinel), points sorted by patch
    std::vector<int32_t> patch_prim;    // owning primitive of each patch
};

template <class F>
void parallel_for(int n, int nthreads, F f) {
    nthreads = std::max(1, std::min(nthreads, n));
    std::atomic<int> next{0};
    auto work = [&] {
        for (int i; (i = next.fetch_add(1)) < n;) f(i);
    };
    std::vector<std::thread> th;
    for (int i = 1; i < nthreads; ++i) th.emplace_back(work);
    work();
    for (auto& t : th) t.join();
}

}  // namespace

struct pvvc_synth {
    pvvc_synth_config cfg;
    std::vector<Prim> prims;
    std::vector<std::vector<int16_t>> surf;
    std::vector<GofData> gofs;
    std::vector<std::vector<uint8_t>> frames;
    std::vector<uint64_t> frame_points;

    void colour(const GofData& g, uint32_t i, int t, uint8_t rgb[3]) const {
        const int k = g.prim[i];
        const Prim& p = prims[k];
        const float* m = &g.mat[3 * (size_t)i];
        const double illum = 1.0 + 0.05 * std::sin(6.283185307179586 * t / 90.0 + p.cphase);
        for (int c = 0; c < 3; ++c) {
            double v = 255.0 * value_noise(m[0] + 1000.0 * c, m[1], m[2], p.tex) * illum;
            v += cfg.color_noise * normal(hash4(cfg.seed ^ 0xC0102ull, (uint64_t)t, ((uint64_t)g.t0 << 32) | i, (uint64_t)c));
            v = std::round(v);
            rgb[c] = (uint8_t)std::max(0.0, std::min(255.0, v));
        }
    }

    void motion(const GofData& g, int patch, int t, float mv[16]) const {
        const Prim& p = prims[g.patch_prim[patch]];
        Mat3 R1, R0m;
        double C1[3], C0[3];
        prim_pose(p, t, &R1, C1);
        prim_pose(p, g.t0, &R0m, C0);
        // Q = R(t) R(t0)^T ; x_t = Q (x_t0 - C(t0)) + C(t)
        Mat3 R0t;
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R0t.m[3 * i + j] = R0m.m[3 * j + i];
        const Mat3 Q = mul(R1, R0t);
        double tr[3];
        for (int i = 0; i < 3; ++i) tr[i] = C1[i] - (Q.m[3 * i] * C0[0] + Q.m[3 * i + 1] * C0[1] + Q.m[3 * i + 2] * C0[2]);
        for (int i = 0; i < 3; ++i) {
            for (int j = 0; j < 3; ++j) mv[4 * i + j] = (float)Q.m[3 * i + j];
            mv[4 * i + 3] = (float)tr[i];
        }
        mv[12] = mv[13] = mv[14] = 0.f;
        mv[15] = 1.f;
        if (t == g.t0) {  // the intra slice carries the identity
            for (int i = 0; i < 16; ++i) mv[i] = (i % 5 == 0) ? 1.f : 0.f;
        }
    }
};

extern "C" int pvvc_synth_create(const pvvc_synth_config* cfgp, pvvc_synth** out) {
    if (!cfgp || !out || cfgp->grid_bits < 4 || cfgp->grid_bits > 16 || cfgp->nprims <= 0 || cfgp->nframes <= 0 ||
        cfgp->gof <= 0 || cfgp->qp_i == 0 || cfgp->qp_p == 0)
        return PVVC_ERR_ARG;
    auto s = std::make_unique<pvvc_synth>();
    s->cfg = *cfgp;
    const auto& c = s->cfg;
    const double G = (double)(1 << c.grid_bits);
    Rng rng(c.seed * 0x9E3779B97F4A7C15ull + 17);
    // primitives at scale 1, then rescale to hit the point target
    for (int k = 0; k < c.nprims; ++k) {
        Prim p{};
        p.kind = (k % 3 == 2) ? 1 : 0;
        for (int i = 0; i < 3; ++i) p.ax[i] = rng.uniform(c.axis_min, c.axis_max) / 2.0;
        if (p.kind == 1) {
            p.ax[0] = rng.uniform(c.axis_min, c.axis_max) / 2.0;        // half length
            p.ax[1] = rng.uniform(c.axis_min, c.axis_max) / 4.0;        // radius
        }
        double a0[3];
        rand_axis(rng, a0);
        p.R0 = axis_angle(a0, rng.uniform(0, 6.283185307179586));
        rand_axis(rng, p.axis);
        p.omega = rng.uniform(-c.rot_deg, c.rot_deg) * 3.141592653589793 / 180.0;
        for (int i = 0; i < 3; ++i) {
            p.A[i] = rng.uniform(0, c.trans_vox / kTransOmega);
            p.phase[i] = rng.uniform(0, 6.283185307179586);
        }
        p.cphase = rng.uniform(0, 6.283185307179586);
        p.tex = rng.next();
        s->prims.push_back(p);
    }
    auto build_surfaces = [&]() {
        s->surf.assign(c.nprims, {});
        parallel_for(c.nprims, c.nthreads, [&](int k) { s->surf[k] = surface(s->prims[k]); });
        size_t tot = 0;
        for (auto& v : s->surf) tot += v.size() / 3;
        return tot;
    };
    size_t tot = build_surfaces();
    if (c.target_points > 0 && tot > 0) {
        const double sc = std::sqrt((double)c.target_points / (double)tot);
        for (auto& p : s->prims)
            for (int i = 0; i < 3; ++i) p.ax[i] *= sc;
        build_surfaces();
    }
    // centres: keep the moving primitive inside the grid
    for (auto& p : s->prims) {
        double ext = std::max(p.ax[0], std::max(p.ax[1], p.ax[2]));
        if (p.kind == 1) ext = p.ax[0] + p.ax[1];
        for (int i = 0; i < 3; ++i) {
            const double margin = std::min(G / 2 - 1, ext + p.A[i] + 2);
            p.C0[i] = rng.uniform(margin, G - margin);
        }
    }
    // GoPs
    const int ngof = (c.nframes + c.gof - 1) / c.gof;
    s->gofs.resize(ngof);
    s->frame_points.assign(c.nframes, 0);
    parallel_for(ngof, c.nthreads, [&](int gi) {
        GofData& g = s->gofs[gi];
        g.t0 = gi * c.gof;
        g.nframes = std::min(c.gof, c.nframes - g.t0);
        Rng jr(hash4(c.seed, 0x71773ull, (uint64_t)gi, 0));
        // voxelise all primitive surfaces at frame t0
        std::vector<uint64_t> key;
        std::vector<int32_t> vx, pr;
        std::vector<float> mt;
        for (int k = 0; k < c.nprims; ++k) {
            Mat3 R;
            double C[3];
            prim_pose(s->prims[k], g.t0, &R, C);
            const auto& sv = s->surf[k];
            for (size_t q = 0; q < sv.size() / 3; ++q) {
                const double m[3] = {(double)sv[3 * q], (double)sv[3 * q + 1], (double)sv[3 * q + 2]};
                int32_t v[3];
                bool ok = true;
                for (int i = 0; i < 3; ++i) {
                    double w = R.m[3 * i] * m[0] + R.m[3 * i + 1] * m[1] + R.m[3 * i + 2] * m[2] + C[i];
                    w += c.jitter * jr.gauss();
                    v[i] = (int32_t)std::lround(w);
                    ok &= v[i] >= 0 && v[i] < (int32_t)G;
                }
                if (!ok) continue;
                // Morton key (x,y,z interleaved) for patching and de-duplication
                uint64_t mk = 0;
                for (int b = c.grid_bits - 1; b >= 0; --b)
                    mk = (mk << 3) | (uint64_t)(((v[0] >> b) & 1) << 2 | ((v[1] >> b) & 1) << 1 | ((v[2] >> b) & 1));
                key.push_back((mk << 20) | (uint64_t)(vx.size() / 3 & 0xFFFFF));
                vx.insert(vx.end(), v, v + 3);
                mt.push_back((float)m[0]);
                mt.push_back((float)m[1]);
                mt.push_back((float)m[2]);
                pr.push_back(k);
            }
        }
        // sort by Morton code, keep the first point of each voxel
        std::vector<uint32_t> ord(pr.size());
        for (uint32_t i = 0; i < ord.size(); ++i) ord[i] = i;
        std::vector<uint64_t> mk(pr.size());
        for (size_t i = 0; i < pr.size(); ++i) {
            uint64_t m = 0;
            for (int b = c.grid_bits - 1; b >= 0; --b)
                m = (m << 3) | (uint64_t)(((vx[3 * i] >> b) & 1) << 2 | ((vx[3 * i + 1] >> b) & 1) << 1 | ((vx[3 * i + 2] >> b) & 1));
            mk[i] = m;
        }
        std::stable_sort(ord.begin(), ord.end(), [&](uint32_t a, uint32_t b) { return mk[a] < mk[b]; });
        for (size_t q = 0; q < ord.size(); ++q) {
            const uint32_t i = ord[q];
            if (q > 0 && mk[i] == mk[ord[q - 1]]) continue;
            g.vox.insert(g.vox.end(), &vx[3 * i], &vx[3 * i] + 3);
            g.mat.insert(g.mat.end(), &mt[3 * i], &mt[3 * i] + 3);
            g.prim.push_back(pr[i]);
        }
        // patches: consecutive Morton runs of sampled sizes
        const uint32_t n = (uint32_t)g.prim.size();
        Rng pr_rng(hash4(c.seed, 0x9A7C4ull, (uint64_t)gi, 1));
        uint32_t pos = 0;
        while (pos < n) {
            double sz;
            if (c.size_mode == 0) sz = pr_rng.uniform(c.size_a, c.size_b);
            else sz = std::max((double)c.size_min, std::min((double)c.size_max, c.size_a * std::exp(c.size_b * pr_rng.gauss())));
            uint32_t len = (uint32_t)std::max(1.0, std::round(sz));
            const uint32_t minsz = (uint32_t)std::max(1.0f, c.size_mode == 0 ? c.size_a : c.size_min);
            if (n - pos < len + minsz) len = n - pos;  // fold a short tail into the last patch
            g.patch_first.push_back(pos);
            // owning primitive: the most frequent in the run
            std::vector<int> cnt(c.nprims, 0);
            for (uint32_t i = pos; i < pos + len; ++i) cnt[g.prim[i]]++;
            g.patch_prim.push_back((int32_t)(std::max_element(cnt.begin(), cnt.end()) - cnt.begin()));
            pos += len;
        }
        g.patch_first.push_back(n);
    });
    *out = s.release();
    return PVVC_OK;
}

extern "C" void pvvc_synth_destroy(pvvc_synth* s) { delete s; }
extern "C" int32_t pvvc_synth_gof_count(const pvvc_synth* s) { return s ? (int32_t)s->gofs.size() : 0; }
extern "C" int32_t pvvc_synth_patch_count(const pvvc_synth* s, int32_t gof) {
    if (!s || gof < 0 || gof >= (int32_t)s->gofs.size()) return 0;
    return (int32_t)s->gofs[gof].patch_first.size() - 1;
}

namespace {
// Colours the encoder sees for one patch: frame 0 absolute YUV, later frames
// the residual against frame 0 (GoP_encoding.cc:145-149).
void patch_colours(const pvvc_synth* s, const GofData& g, int patch, float* yuv) {
    const uint32_t a = g.patch_first[patch], b = g.patch_first[patch + 1], n = b - a;
    for (int f = 0; f < g.nframes; ++f) {
        float* out = yuv + 3ull * n * f;
        for (uint32_t i = 0; i < n; ++i) {
            uint8_t rgb[3];
            s->colour(g, a + i, g.t0 + f, rgb);
            rgb_to_yuv(rgb[0], rgb[1], rgb[2], out + 3 * i);
            if (f > 0)
                for (int c = 0; c < 3; ++c) out[3 * i + c] -= yuv[3 * i + c];
        }
    }
}
}  // namespace

extern "C" int pvvc_synth_patch(const pvvc_synth* s, int32_t gof, int32_t patch, float* xyz, float* yuv,
                                float* mv_rowmajor, uint32_t* n, int32_t* nframes) {
    if (!s || gof < 0 || gof >= (int32_t)s->gofs.size()) return PVVC_ERR_ARG;
    const GofData& g = s->gofs[gof];
    if (patch < 0 || patch + 1 >= (int32_t)g.patch_first.size()) return PVVC_ERR_ARG;
    const uint32_t a = g.patch_first[patch], b = g.patch_first[patch + 1];
    if (n) *n = b - a;
    if (nframes) *nframes = g.nframes;
    if (xyz)
        for (uint32_t i = a; i < b; ++i)
            for (int c = 0; c < 3; ++c) xyz[3ull * (i - a) + c] = (float)g.vox[3ull * i + c];
    if (yuv) patch_colours(s, g, patch, yuv);
    if (mv_rowmajor)
        for (int f = 0; f < g.nframes; ++f) s->motion(g, patch, g.t0 + f, mv_rowmajor + 16 * f);
    return PVVC_OK;
}

extern "C" int pvvc_synth_encode(pvvc_synth* s) {
    if (!s) return PVVC_ERR_ARG;
    const auto& c = s->cfg;
    s->frames.assign(c.nframes, {});
    for (auto& g : s->gofs) {
        const int np = (int)g.patch_first.size() - 1;
        std::vector<std::vector<pvvc::Slice>> per_patch(np);
        std::atomic<int> err{0};
        parallel_for(np, c.nthreads, [&](int p) {
            const uint32_t a = g.patch_first[p], n = g.patch_first[p + 1] - a;
            std::vector<float> xyz(3ull * n), yuv(3ull * n * g.nframes), mv(16ull * g.nframes);
            pvvc_synth_patch(s, (int32_t)(&g - &s->gofs[0]), p, xyz.data(), yuv.data(), mv.data(), nullptr, nullptr);
            pvvc::PatchTree tree;
            if (tree.build(xyz.data(), n)) {
                err = PVVC_ERR_TREE;
                return;
            }
            auto geo = tree.geometry();
            // the reference encoder's optional zstd stage: keep the compressed
            // payload only when it is smaller (GoP_encoding.cc:158-200)
            auto maybe_zstd = [&](std::vector<uint8_t>* payload, uint8_t bit, uint8_t* type) {
                if (!c.zstd_level || payload->empty()) return;
                std::vector<uint8_t> z;
                if (pvvc::zstd_compress(payload->data(), payload->size(), c.zstd_level, &z) == PVVC_OK &&
                    z.size() < payload->size()) {
                    payload->swap(z);
                    *type |= bit;
                }
            };
            std::vector<float> coef;
            auto& out = per_patch[p];
            for (int f = 0; f < g.nframes; ++f) {
                tree.raht(yuv.data() + 3ull * n * f, &coef);
                pvvc::Slice sl;
                const bool intra = f == 0;
                sl.type = intra ? pvvc::kTypeDefaultIntra : pvvc::kTypeDefaultPredict;
                sl.timestamp = g.t0 + f;
                sl.index = p;
                sl.size = tree.leaf_count();
                sl.qp = intra ? c.qp_i : c.qp_p;
                // Slice.mv is column-major (Eigen); mv[] here is row-major
                for (int r = 0; r < 4; ++r)
                    for (int cc = 0; cc < 4; ++cc) sl.mv[cc * 4 + r] = mv[16 * f + r * 4 + cc];
                if (intra) {
                    sl.geometry = geo;
                    maybe_zstd(&sl.geometry, pvvc::kTypeGeoZstd, &sl.type);
                }
                sl.color = pvvc::encode_colors(coef.data(), tree.leaf_count(), sl.qp);
                maybe_zstd(&sl.color, pvvc::kTypeColorZstd, &sl.type);
                out.push_back(std::move(sl));
            }
        });
        if (err) return err;
        for (int f = 0; f < g.nframes; ++f) {
            std::vector<pvvc::Slice> sl;
            sl.reserve(np);
            uint64_t pts = 0;
            for (int p = 0; p < np; ++p) {
                pts += per_patch[p][f].size;
                sl.push_back(std::move(per_patch[p][f]));
            }
            s->frames[g.t0 + f] = pvvc::write_frame(pvvc::frame_from_slices(std::move(sl)));
            s->frame_points[g.t0 + f] = pts;
        }
    }
    return PVVC_OK;
}

extern "C" int pvvc_synth_frame(const pvvc_synth* s, int32_t frame, const uint8_t** bytes, uint64_t* len) {
    if (!s || frame < 0 || frame >= (int32_t)s->frames.size() || !bytes || !len) return PVVC_ERR_ARG;
    *bytes = s->frames[frame].data();
    *len = s->frames[frame].size();
    return s->frames[frame].empty() ? PVVC_ERR_ARG : PVVC_OK;
}

extern "C" uint64_t pvvc_synth_frame_points(const pvvc_synth* s, int32_t frame) {
    if (!s || frame < 0 || frame >= (int32_t)s->frame_points.size()) return 0;
    return s->frame_points[frame];
}
