// bitstream.cc -- .slice / .frame byte layouts and host-side zstd compression.
#include "bitstream.h"

#include <dlfcn.h>

#include <algorithm>
#include <cstring>
#include <mutex>

#include "pvvc_gb300.h"

namespace pvvc {
namespace {

struct Writer {
    std::vector<uint8_t> b;
    template <class T>
    void put(const T& v) {
        const uint8_t* p = reinterpret_cast<const uint8_t*>(&v);
        b.insert(b.end(), p, p + sizeof(T));
    }
    void bytes(const uint8_t* p, size_t n) {
        if (n) b.insert(b.end(), p, p + n);
    }
};

struct Reader {
    const uint8_t* p;
    size_t len, pos = 0;
    bool ok = true;
    template <class T>
    T get() {
        T v{};
        if (pos + sizeof(T) > len) {
            ok = false;
            return v;
        }
        std::memcpy(&v, p + pos, sizeof(T));
        pos += sizeof(T);
        return v;
    }
    bool take(size_t n, std::vector<uint8_t>* out) {
        if (n > len - pos || pos > len) {
            ok = false;
            return false;
        }
        out->assign(p + pos, p + pos + n);
        pos += n;
        return true;
    }
};

}  // namespace

// SaveSlice (src/io/slice_io.cc:20-118)
std::vector<uint8_t> write_slice(const Slice& s) {
    Writer w;
    w.put(s.type);
    w.put(s.timestamp);
    w.put(s.index);
    w.put(s.size);
    w.put(s.qp);
    for (int i = 0; i < 16; ++i) w.put(s.mv[i]);
    if (!(s.type & kTypePredict)) {
        w.put(static_cast<uint64_t>(s.geometry.size()));
        w.bytes(s.geometry.data(), s.geometry.size());
    }
    if (!(s.type & kTypeSkip)) {
        w.put(static_cast<uint64_t>(s.color.size()));
        w.bytes(s.color.data(), s.color.size());
    }
    return std::move(w.b);
}

// LoadSlice (src/io/slice_io.cc:120-206)
int parse_slice(const uint8_t* p, size_t len, Slice* s) {
    Reader r{p, len};
    s->type = r.get<uint8_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    if (!(s->type & kTypeValid)) return PVVC_ERR_BAD_SLICE;
    s->timestamp = r.get<int32_t>();
    s->index = r.get<int32_t>();
    s->size = r.get<uint64_t>();
    s->qp = r.get<uint8_t>();
    for (int i = 0; i < 16; ++i) s->mv[i] = r.get<float>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    s->geometry.clear();
    s->color.clear();
    if (!(s->type & kTypePredict)) {
        uint64_t g = r.get<uint64_t>();
        if (!r.ok || g == 0) return PVVC_ERR_FORMAT;
        if (!r.take(g, &s->geometry)) return PVVC_ERR_FORMAT;
    }
    if (!(s->type & kTypeSkip)) {
        uint64_t c = r.get<uint64_t>();
        if (!r.ok || c == 0) return PVVC_ERR_FORMAT;
        if (!r.take(c, &s->color)) return PVVC_ERR_FORMAT;
    }
    return PVVC_OK;
}

// ChangeSliceToFrame body (src/io/slice_io.cc:258-316)
std::vector<uint8_t> write_frame(const Frame& f) {
    Writer w;
    const uint32_t n = static_cast<uint32_t>(f.count());
    w.put(f.timestamp);
    w.put(n);
    w.bytes(reinterpret_cast<const uint8_t*>(f.index.data()), 4ull * n);
    w.bytes(f.type.data(), n);
    w.bytes(reinterpret_cast<const uint8_t*>(f.size.data()), 4ull * n);
    w.bytes(f.qp.data(), n);
    w.bytes(reinterpret_cast<const uint8_t*>(f.mv.data()), 64ull * n);
    for (uint32_t i = 0; i < n; ++i) w.put(static_cast<uint32_t>(f.geometry[i].size()));
    for (uint32_t i = 0; i < n; ++i) w.bytes(f.geometry[i].data(), f.geometry[i].size());
    for (uint32_t i = 0; i < n; ++i) w.put(static_cast<uint32_t>(f.color[i].size()));
    for (uint32_t i = 0; i < n; ++i) w.bytes(f.color[i].data(), f.color[i].size());
    return std::move(w.b);
}

// io::LoadFrame (src/cuda/common/slice_io.cu:143-275), without the zstd step
int parse_frame(const uint8_t* p, size_t len, Frame* f) {
    Reader r{p, len};
    f->timestamp = r.get<int32_t>();
    uint32_t n = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    // each slice needs at least 4+1+4+1+64+4+4 bytes: reject absurd counts early
    if (static_cast<uint64_t>(n) * 82ull > len) return PVVC_ERR_FORMAT;
    f->index.resize(n);
    f->type.resize(n);
    f->size.resize(n);
    f->qp.resize(n);
    f->mv.resize(16ull * n);
    f->geometry.assign(n, {});
    f->color.assign(n, {});
    for (uint32_t i = 0; i < n; ++i) f->index[i] = r.get<int32_t>();
    for (uint32_t i = 0; i < n; ++i) f->type[i] = r.get<uint8_t>();
    for (uint32_t i = 0; i < n; ++i) f->size[i] = r.get<uint32_t>();
    for (uint32_t i = 0; i < n; ++i) f->qp[i] = r.get<uint8_t>();
    for (uint64_t i = 0; i < 16ull * n; ++i) f->mv[i] = r.get<float>();
    std::vector<uint32_t> gsz(n), csz(n);
    for (uint32_t i = 0; i < n; ++i) gsz[i] = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i)
        if (gsz[i] && !r.take(gsz[i], &f->geometry[i])) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i) csz[i] = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i)
        if (csz[i] && !r.take(csz[i], &f->color[i])) return PVVC_ERR_FORMAT;
    return PVVC_OK;
}

Frame frame_from_slices(std::vector<Slice> slices) {
    std::stable_sort(slices.begin(), slices.end(), [](const Slice& a, const Slice& b) { return a.index < b.index; });
    Frame f;
    f.timestamp = slices.empty() ? -1 : slices.front().timestamp;
    for (auto& s : slices) {
        f.index.push_back(s.index);
        f.type.push_back(s.type);
        f.size.push_back(static_cast<uint32_t>(s.size));
        f.qp.push_back(s.qp);
        // column-major (Eigen) -> row-major, as ChangeSliceToFrame writes i(row, col)
        for (int r = 0; r < 4; ++r)
            for (int c = 0; c < 4; ++c) f.mv.push_back(s.mv[c * 4 + r]);
        f.geometry.push_back(std::move(s.geometry));
        f.color.push_back(std::move(s.color));
    }
    return f;
}

// ---- zstd via dlopen ------------------------------------------------------
namespace {
struct Zstd {
    void* h = nullptr;
    size_t (*compressBound)(size_t) = nullptr;
    size_t (*compress)(void*, size_t, const void*, size_t, int) = nullptr;
    unsigned (*isError)(size_t) = nullptr;
    int (*maxLevel)(void) = nullptr;
    int (*minLevel)(void) = nullptr;
};
Zstd* zstd() {
    static Zstd z;
    static std::once_flag once;
    std::call_once(once, [] {
        const char* names[] = {"libzstd.so.1", "libzstd.so"};
        for (const char* n : names) {
            z.h = dlopen(n, RTLD_NOW | RTLD_LOCAL);
            if (z.h) break;
        }
        if (!z.h) return;
        z.compressBound = reinterpret_cast<size_t (*)(size_t)>(dlsym(z.h, "ZSTD_compressBound"));
        z.compress = reinterpret_cast<size_t (*)(void*, size_t, const void*, size_t, int)>(dlsym(z.h, "ZSTD_compress"));
        z.isError = reinterpret_cast<unsigned (*)(size_t)>(dlsym(z.h, "ZSTD_isError"));
        z.maxLevel = reinterpret_cast<int (*)(void)>(dlsym(z.h, "ZSTD_maxCLevel"));
        z.minLevel = reinterpret_cast<int (*)(void)>(dlsym(z.h, "ZSTD_minCLevel"));
        if (!z.compressBound || !z.compress || !z.isError || !z.maxLevel || !z.minLevel) {
            dlclose(z.h);
            z.h = nullptr;
        }
    });
    return z.h ? &z : nullptr;
}
}  // namespace

bool zstd_available() { return zstd() != nullptr; }

// ZstdEncoder::Encode (src/common/entropy_codec.cc:304-324)
int zstd_compress(const uint8_t* src, size_t n, int level, std::vector<uint8_t>* out) {
    Zstd* z = zstd();
    if (!z) return PVVC_ERR_ZSTD;
    level = std::min(level, z->maxLevel());
    level = std::max(level, z->minLevel());
    out->resize(z->compressBound(n));
    size_t r = z->compress(out->data(), out->size(), src, n, level);
    if (z->isError(r)) return PVVC_ERR_ZSTD;
    out->resize(r);
    return PVVC_OK;
}

int parse_frame_view(const uint8_t* p, size_t len, FrameView* f) {
    Reader r{p, len};
    f->timestamp = r.get<int32_t>();
    uint32_t n = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    if (static_cast<uint64_t>(n) * 82ull > len) return PVVC_ERR_FORMAT;
    f->index.resize(n);
    f->type.resize(n);
    f->size.resize(n);
    f->qp.resize(n);
    f->mv.resize(16ull * n);
    f->geo.assign(n, nullptr);
    f->col.assign(n, nullptr);
    f->gsz.assign(n, 0);
    f->csz.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) f->index[i] = r.get<int32_t>();
    for (uint32_t i = 0; i < n; ++i) f->type[i] = r.get<uint8_t>();
    for (uint32_t i = 0; i < n; ++i) f->size[i] = r.get<uint32_t>();
    for (uint32_t i = 0; i < n; ++i) f->qp[i] = r.get<uint8_t>();
    for (uint64_t i = 0; i < 16ull * n; ++i) f->mv[i] = r.get<float>();
    auto span = [&](uint32_t sz, const uint8_t** at) {
        if (sz > len - r.pos || r.pos > len) return false;
        *at = p + r.pos;
        r.pos += sz;
        return true;
    };
    for (uint32_t i = 0; i < n; ++i) f->gsz[i] = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i)
        if (f->gsz[i] && !span(f->gsz[i], &f->geo[i])) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i) f->csz[i] = r.get<uint32_t>();
    if (!r.ok) return PVVC_ERR_FORMAT;
    for (uint32_t i = 0; i < n; ++i)
        if (f->csz[i] && !span(f->csz[i], &f->col[i])) return PVVC_ERR_FORMAT;
    return PVVC_OK;
}


}  // namespace pvvc
