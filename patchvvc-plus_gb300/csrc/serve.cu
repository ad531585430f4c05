// serve.cu -- playback server: continuous batching of .frame requests from
// many concurrent streams onto one GPU (contract in include/pvvc_gb300.h).
//
// Threads:
//   caller threads  submit: parse the .frame header (zero-copy: payload
//                   pointers index the caller's bytes), queue per stream
//   worker          forms a batch from everything queued (round-robin over
//                   streams), packs payloads into pinned staging, plans,
//                   uploads on the copy stream, enqueues the decode on the
//                   compute stream behind the upload's event
//   completion      waits for each batch's event in order, stamps its frames
//                   and publishes them to pollers
// Up to `inflight` batches are queued on the GPU: while batch k decodes, the
// worker packs and uploads batch k+1, so the GPU goes from one decode to the
// next without a host round trip.  Batches run in order on one compute
// stream, so a stream's predictive frames always see the state its earlier
// intra frames left.
#include <cuda_runtime.h>

#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <vector>

#include "../host/bitstream.h"
#include "decode_internal.h"
#include "zstd_core.h"

namespace pvvc {
namespace {

// One queued frame: header arrays copied out of the .frame bytes, payloads
// referenced in place (zstd payloads compressed, for the GPU to inflate).
struct Request {
    uint64_t tag = 0;
    int32_t stream = -1;
    double submit_us = 0;
    uint32_t n = 0;
    std::vector<int32_t> index;
    std::vector<uint8_t> type, qp;
    std::vector<uint32_t> size, gsz, csz;
    std::vector<float> mv;
    std::vector<const uint8_t*> gp, cp;
    std::vector<uint32_t> gzl, czl;  // compressed length of a zstd payload (0: raw); gsz/csz are then its raw size
    uint64_t points = 0, bytes = 0;  // bytes: 4-aligned packed payload size
    uint64_t zbytes = 0;             // compressed bytes of the zstd payloads
    int32_t nz = 0;
    bool has_intra = false;
    // batch bookkeeping
    uint64_t handle = 0, ring_off = 0;
    int32_t first_slice = 0, slot_base = 0;
};

inline uint32_t rd32(const uint8_t* p) {
    uint32_t v;
    std::memcpy(&v, p, 4);
    return v;
}

// Zero-copy .frame header parse (layout of src/io/slice_io.cc:258-316).
int parse_request(const uint8_t* b, uint64_t len, Request* r) {
    if (!b || len < 8) return PVVC_ERR_FORMAT;
    const uint32_t n = rd32(b + 4);
    if ((uint64_t)n * 82 > len) return PVVC_ERR_FORMAT;
    r->n = n;
    r->index.resize(n);
    r->type.resize(n);
    r->size.resize(n);
    r->qp.resize(n);
    r->mv.resize(16ull * n);
    r->gsz.resize(n);
    r->csz.resize(n);
    r->gp.resize(n);
    r->cp.resize(n);
    uint64_t o = 8;
    std::memcpy(r->index.data(), b + o, 4ull * n);
    o += 4ull * n;
    std::memcpy(r->type.data(), b + o, n);
    o += n;
    std::memcpy(r->size.data(), b + o, 4ull * n);
    o += 4ull * n;
    std::memcpy(r->qp.data(), b + o, n);
    o += n;
    std::memcpy(r->mv.data(), b + o, 64ull * n);
    o += 64ull * n;
    if (o + 4ull * n > len) return PVVC_ERR_FORMAT;
    std::memcpy(r->gsz.data(), b + o, 4ull * n);
    o += 4ull * n;
    for (uint32_t i = 0; i < n; ++i) {
        if (o + r->gsz[i] > len) return PVVC_ERR_FORMAT;
        r->gp[i] = b + o;
        o += r->gsz[i];
    }
    if (o + 4ull * n > len) return PVVC_ERR_FORMAT;
    std::memcpy(r->csz.data(), b + o, 4ull * n);
    o += 4ull * n;
    for (uint32_t i = 0; i < n; ++i) {
        if (o + r->csz[i] > len) return PVVC_ERR_FORMAT;
        r->cp[i] = b + o;
        o += r->csz[i];
    }
    // zstd payloads stay compressed: the batch inflates them on the GPU in
    // place of the reference loader's host zstd stage (slice_io.cu:233-265).
    // The raw size is the first frame's declared content size, which the
    // reference's ZstdDecoder requires (entropy_codec.cc:343-347).
    r->gzl.assign(n, 0);
    r->czl.assign(n, 0);
    for (uint32_t i = 0; i < n; ++i) {
        for (int which = 0; which < 2; ++which) {
            const uint8_t bit = which ? PVVC_TYPE_COLOR_ZSTD : PVVC_TYPE_GEO_ZSTD;
            uint32_t& sz = which ? r->csz[i] : r->gsz[i];
            const uint8_t* ptr = which ? r->cp[i] : r->gp[i];
            if (!(r->type[i] & bit) || sz == 0) continue;
            uint64_t raw = 0;
            if (!pvvc_zstd::content_size(ptr, sz, &raw) || raw == 0 || raw == pvvc_zstd::kUnknown || raw > 0xFFFFFFFFull)
                return PVVC_ERR_ZSTD;
            (which ? r->czl : r->gzl)[i] = sz;
            r->zbytes += sz;
            r->nz++;
            sz = (uint32_t)raw;
        }
        r->type[i] &= (uint8_t)~(PVVC_TYPE_GEO_ZSTD | PVVC_TYPE_COLOR_ZSTD);
    }
    for (uint32_t i = 0; i < n; ++i) {
        r->points += r->size[i];
        r->bytes = align_up(align_up(r->bytes + r->gsz[i], 4) + r->csz[i], 4);
        if (!(r->type[i] & PVVC_TYPE_PREDICT)) r->has_intra = true;
    }
    return PVVC_OK;
}

struct Stream {
    bool open = false;
    int32_t slot_base = 0, nslots = 0;
    std::deque<Request*> pending;
    uint64_t outstanding = 0;     // submitted, not yet completed
    std::vector<uint8_t> seen;    // batch formation scratch (per slot)
};

// Decoded-frame ring in units of points: allocations in FIFO order, released
// in any order, reclaimed from the oldest.
struct Ring {
    struct Entry {
        uint64_t off, n;
        bool released;
    };
    uint64_t cap = 0;
    uint64_t first_handle = 1;  // handle of entries.front()
    std::deque<Entry> entries;
    // offset of a new allocation of n points, or ~0 if it does not fit now
    uint64_t alloc(uint64_t n, uint64_t* handle) {
        if (n > cap) return ~0ull;
        uint64_t off;
        if (entries.empty()) {
            off = 0;
        } else {
            const uint64_t tail = entries.front().off;
            const uint64_t head = entries.back().off + entries.back().n;
            if (head >= tail) {  // not wrapped: free space is [head, cap) and [0, tail)
                if (cap - head >= n) off = head;
                else if (n < tail) off = 0;
                else return ~0ull;
            } else {  // wrapped: free space is [head, tail)
                if (tail - head > n) off = head;
                else return ~0ull;
            }
        }
        // a zero-point frame takes no space but still gets a handle
        entries.push_back({off, n, false});
        *handle = first_handle + entries.size() - 1;
        return off;
    }
    Entry* find(uint64_t h) {
        if (h < first_handle || h >= first_handle + entries.size()) return nullptr;
        return &entries[h - first_handle];
    }
    bool release(uint64_t h) {
        Entry* e = find(h);
        if (!e || e->released) return false;
        e->released = true;
        while (!entries.empty() && entries.front().released) {
            entries.pop_front();
            ++first_handle;
        }
        return true;
    }
};

struct Batch {
    pvvc_plan plan;
    HostBuf h_payload, h_status;
    DevBuf d_payload, d_status, ws;
    cudaEvent_t e_h2d = nullptr, e_start = nullptr, e_done = nullptr;
    std::vector<Request*> reqs;
    int32_t id = 0, nslices = 0;
    double launch_us = 0;
    int rc = PVVC_OK;
    bool busy = false;
    // host arrays of the batch description
    std::vector<int32_t> slot;
    std::vector<uint8_t> type, qp;
    std::vector<uint32_t> size, gsz, csz;
    std::vector<float> mv;
    std::vector<uint64_t> goff, coff, oo;
};

}  // namespace
}  // namespace pvvc

using namespace pvvc;

struct pvvc_server {
    pvvc_server_config cfg{};
    int device = 0;
    std::chrono::steady_clock::time_point t0;
    pvvc_state* state = nullptr;
    std::vector<int32_t> slot_owner;  // -1 free, else stream id
    DevBuf ring_xyz, ring_rgb;
    Ring ring;
    std::vector<std::unique_ptr<Batch>> batches;
    std::deque<int> inflight;  // batch indices in launch order
    cudaStream_t compute = nullptr, copy = nullptr;
    std::vector<Stream> streams;
    int rr = 0;
    std::deque<pvvc_completion> done;
    std::mutex mu;
    std::condition_variable cv_work, cv_done, cv_poll;
    bool stop = false, worker_done = false;
    std::thread worker, completer;
    pvvc_server_stats st{};
    int32_t next_batch = 0;
    uint64_t reserved = 0;

    double now() const {
        return std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count();
    }
    bool any_pending() const {
        for (const auto& s : streams)
            if (!s.pending.empty()) return true;
        return false;
    }
    int free_batch() const {
        for (size_t i = 0; i < batches.size(); ++i)
            if (!batches[i]->busy) return (int)i;
        return -1;
    }
    void worker_loop();
    void completion_loop();
    int launch(Batch& b);
};

// Batch formation + launch.  Holds `mu` only while taking requests.
void pvvc_server::worker_loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_work.wait(lk, [&] { return stop || (any_pending() && free_batch() >= 0); });
        if (stop) break;
        const int bi = free_batch();
        Batch& b = *batches[bi];
        // take every queued frame that fits, round-robin over streams
        b.reqs.clear();
        uint64_t pts = 0;
        bool full = false, ring_full = false;
        const int ns = (int)streams.size();
        for (int k = 0; k < ns && !full; ++k) {
            Stream& s = streams[(rr + k) % ns];
            if (s.pending.empty()) continue;
            std::fill(s.seen.begin(), s.seen.end(), 0);
            while (!s.pending.empty()) {
                Request* r = s.pending.front();
                // an intra slice rebuilds its slot: it may not share a batch
                // with an earlier slice of that slot
                bool clash = false;
                for (uint32_t i = 0; i < r->n && !clash; ++i)
                    clash = !(r->type[i] & PVVC_TYPE_PREDICT) && s.seen[r->index[i]];
                if (clash) break;
                if (!b.reqs.empty() && (pts + r->points > cfg.max_batch_points ||
                                        (int32_t)b.reqs.size() >= cfg.max_batch_frames)) {
                    full = true;
                    break;
                }
                uint64_t h = 0;
                const uint64_t off = ring.alloc(r->points, &h);
                if (off == ~0ull) {
                    full = ring_full = true;
                    break;
                }
                r->handle = h;
                r->ring_off = off;
                r->slot_base = s.slot_base;
                for (uint32_t i = 0; i < r->n; ++i) s.seen[r->index[i]] = 1;
                s.pending.pop_front();
                b.reqs.push_back(r);
                pts += r->points;
            }
        }
        rr = (rr + 1) % std::max(ns, 1);
        if (b.reqs.empty()) {
            // only the output ring can block a non-empty queue: wait for a release
            if (ring_full) cv_work.wait_for(lk, std::chrono::milliseconds(1));
            continue;
        }
        b.busy = true;
        b.id = next_batch++;
        lk.unlock();
        b.rc = launch(b);
        b.launch_us = now();
        lk.lock();
        inflight.push_back(bi);
        cv_done.notify_all();
    }
    worker_done = true;
    cv_done.notify_all();
}

// Pack, plan, upload and enqueue one batch (no lock held).
int pvvc_server::launch(Batch& b) {
    uint64_t bytes = 0, zbytes = 0;
    int32_t nsl = 0, nz = 0;
    for (Request* r : b.reqs) {
        r->first_slice = nsl;
        nsl += (int32_t)r->n;
        bytes += r->bytes;
        zbytes += r->zbytes;
        nz += r->nz;
    }
    b.nslices = nsl;
    // payload buffer: the raw payloads the plan indexes; then the zstd
    // payloads, compressed, and their job arrays (source offset, raw offset,
    // source length, raw size, slice, status), one host-to-device copy for all
    const uint64_t zstart = align_up(bytes + 16, 16), a_src = align_up(zstart + zbytes, 16), a_dst = a_src + 8ull * nz,
                   a_len = a_dst + 8ull * nz, a_cap = a_len + 4ull * nz, a_slice = a_cap + 4ull * nz,
                   a_stat = a_slice + 4ull * nz, total = nz ? a_stat + 4ull * nz : bytes;
    if (b.h_payload.ensure(total + 16) != cudaSuccess || b.d_payload.ensure(total + 16) != cudaSuccess ||
        b.h_status.ensure(4ull * std::max(nsl, 1)) != cudaSuccess || b.d_status.ensure(4ull * std::max(nsl, 1)) != cudaSuccess)
        return PVVC_ERR_NOMEM;
    b.slot.resize(nsl);
    b.type.resize(nsl);
    b.qp.resize(nsl);
    b.size.resize(nsl);
    b.gsz.resize(nsl);
    b.csz.resize(nsl);
    b.mv.resize(16ull * nsl);
    b.goff.resize(nsl);
    b.coff.resize(nsl);
    b.oo.resize(nsl);
    uint8_t* hp = static_cast<uint8_t*>(b.h_payload.p);
    uint64_t* zsrc = reinterpret_cast<uint64_t*>(hp + a_src);
    uint64_t* zdst = reinterpret_cast<uint64_t*>(hp + a_dst);
    uint32_t* zlen = reinterpret_cast<uint32_t*>(hp + a_len);
    uint32_t* zcap = reinterpret_cast<uint32_t*>(hp + a_cap);
    int32_t* zsl = reinterpret_cast<int32_t*>(hp + a_slice);
    uint64_t off = 0, zo = zstart;
    int32_t k = 0, q = 0;
    auto put = [&](const uint8_t* p, uint32_t raw, uint32_t zl) {  // one payload at `off`
        if (!raw) return;
        if (!zl) {
            std::memcpy(hp + off, p, raw);
            return;
        }
        std::memcpy(hp + zo, p, zl);
        zsrc[q] = zo;
        zdst[q] = off;
        zlen[q] = zl;
        zcap[q] = raw;
        zsl[q] = k;
        zo += zl;
        ++q;
    };
    for (Request* r : b.reqs) {
        uint64_t po = r->ring_off;
        for (uint32_t i = 0; i < r->n; ++i, ++k) {
            b.slot[k] = r->slot_base + r->index[i];
            b.type[k] = r->type[i];
            b.qp[k] = r->qp[i];
            b.size[k] = r->size[i];
            std::memcpy(&b.mv[16ull * k], &r->mv[16ull * i], 64);
            b.goff[k] = off;
            b.gsz[k] = r->gsz[i];
            put(r->gp[i], r->gsz[i], r->gzl[i]);
            off = align_up(off + r->gsz[i], 4);
            b.coff[k] = off;
            b.csz[k] = r->csz[i];
            put(r->cp[i], r->csz[i], r->czl[i]);
            off = align_up(off + r->csz[i], 4);
            b.oo[k] = po;
            po += r->size[i];
        }
    }
    std::memset(hp + off, 0, 16);
    pvvc_batch_desc d{nsl, b.slot.data(), b.type.data(), b.size.data(), b.qp.data(), b.mv.data(), b.goff.data(),
                      b.gsz.data(), b.coff.data(), b.csz.data(), b.oo.data()};
    int rc = build_plan(&d, &b.plan, &cfg.tune, copy);
    if (rc) return rc;
    if (b.ws.ensure(b.plan.ws_bytes) != cudaSuccess) return PVVC_ERR_NOMEM;
    if (cudaMemcpyAsync(b.d_payload.p, hp, (nz ? total : off) + 16, cudaMemcpyHostToDevice, copy) != cudaSuccess ||
        cudaEventRecord(b.e_h2d, copy) != cudaSuccess || cudaStreamWaitEvent(compute, b.e_h2d, 0) != cudaSuccess ||
        cudaEventRecord(b.e_start, compute) != cudaSuccess)
        return PVVC_ERR_CUDA;
    uint8_t* dp = static_cast<uint8_t*>(b.d_payload.p);
    rc = pvvc_zstd_launch(nz, dp, reinterpret_cast<const uint64_t*>(dp + a_src), reinterpret_cast<const uint32_t*>(dp + a_len),
                          dp, reinterpret_cast<const uint64_t*>(dp + a_dst), reinterpret_cast<const uint32_t*>(dp + a_cap),
                          nullptr, reinterpret_cast<int32_t*>(dp + a_stat), compute);
    if (rc) return rc;
    rc = run_decode(&b.plan, state, static_cast<const uint8_t*>(b.d_payload.p), static_cast<float*>(ring_xyz.p),
                    static_cast<uint8_t*>(ring_rgb.p), nullptr, static_cast<int32_t*>(b.d_status.p), b.ws.p, b.ws.cap, compute,
                    nullptr);
    if (rc) return rc;
    rc = pvvc_zstd_merge_status(nz, reinterpret_cast<const int32_t*>(dp + a_stat), reinterpret_cast<const int32_t*>(dp + a_slice),
                                static_cast<int32_t*>(b.d_status.p), compute);
    if (rc) return rc;
    if (cudaMemcpyAsync(b.h_status.p, b.d_status.p, 4ull * nsl, cudaMemcpyDeviceToHost, compute) != cudaSuccess ||
        cudaEventRecord(b.e_done, compute) != cudaSuccess)
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}

void pvvc_server::completion_loop() {
    cudaSetDevice(device);
    std::unique_lock<std::mutex> lk(mu);
    for (;;) {
        cv_done.wait(lk, [&] { return !inflight.empty() || worker_done; });
        if (inflight.empty()) break;
        const int bi = inflight.front();
        Batch& b = *batches[bi];
        lk.unlock();
        // e_done follows the batch's status read-back on the compute stream
        bool ok = b.rc == PVVC_OK && cudaEventSynchronize(b.e_done) == cudaSuccess;
        const double t = now();
        float ms = 0.f;
        if (ok) cudaEventElapsedTime(&ms, b.e_start, b.e_done);
        const int32_t* hs = static_cast<const int32_t*>(b.h_status.p);
        lk.lock();
        st.batches++;
        st.gpu_busy_us += ms * 1e3;
        for (Request* r : b.reqs) {
            pvvc_completion c{};
            c.tag = r->tag;
            c.handle = r->handle;
            c.stream_id = r->stream;
            c.status = ok ? PVVC_OK : (b.rc ? b.rc : PVVC_ERR_CUDA);
            if (ok)
                for (uint32_t i = 0; i < r->n; ++i)
                    if (hs[r->first_slice + i]) {
                        c.status = hs[r->first_slice + i];
                        break;
                    }
            c.npoints = r->points;
            c.xyz = static_cast<const float*>(ring_xyz.p) + 3 * r->ring_off;
            c.rgb = static_cast<const uint8_t*>(ring_rgb.p) + 3 * r->ring_off;
            c.submit_us = r->submit_us;
            c.launch_us = b.launch_us;
            c.done_us = t;
            c.batch_id = b.id;
            c.batch_frames = (int32_t)b.reqs.size();
            done.push_back(c);
            st.frames++;
            st.points += r->points;
            st.slices += r->n;
            streams[r->stream].outstanding--;
            delete r;
        }
        b.reqs.clear();
        b.busy = false;
        inflight.pop_front();
        cv_work.notify_all();
        cv_poll.notify_all();
    }
}

namespace {
uint64_t slot_bytes(int32_t max_leaves, int32_t max_nodes) {
    const uint64_t Nn = (uint64_t)max_nodes, Nl = (uint64_t)max_leaves;
    return sizeof(SlotInfo) + Nn * (1 + 1 + 4 + 4 + sizeof(float2) * 7 + 4 + 12) + Nl * 24;
}
}  // namespace

extern "C" int pvvc_server_create(const pvvc_server_config* cfg_in, pvvc_server** out) {
    if (!cfg_in || !out) return PVVC_ERR_ARG;
    *out = nullptr;
    auto s = std::make_unique<pvvc_server>();
    pvvc_server_config c = *cfg_in;
    if (!c.max_leaves) c.max_leaves = 8192;
    if (!c.max_nodes) c.max_nodes = 2 * c.max_leaves;
    if (!c.max_batch_points) c.max_batch_points = 32ull << 20;
    if (!c.ring_points) c.ring_points = 256ull << 20;
    if (!c.inflight) c.inflight = 2;
    if (!c.max_batch_frames) c.max_batch_frames = 4096;
    if (c.inflight < 1 || c.inflight > 4 || c.max_leaves < 0 || c.max_nodes < 0 || c.max_batch_frames < 1 ||
        c.ring_points < c.max_batch_points)
        return PVVC_ERR_ARG;
    if (resolve_tune(&c.tune, &c.tune)) return PVVC_ERR_ARG;
    s->cfg = c;
    s->t0 = std::chrono::steady_clock::now();
    if (cudaGetDevice(&s->device) != cudaSuccess || prepare_kernels() != cudaSuccess) return PVVC_ERR_CUDA;
    // fixed reservations: output ring, per-batch staging and workspace
    const uint64_t ring_bytes = 15ull * c.ring_points;
    const uint64_t grp_scratch = 2ull * c.max_leaves * 96 * 4 * (uint64_t)(c.tune.group_ctas_per_sm * sm_count());
    const uint64_t ws_guess = 96ull * c.max_batch_points + grp_scratch + (1ull << 20);
    const uint64_t pay_guess = 4ull * c.max_batch_points + 4096;
    const uint64_t fixed = ring_bytes + (uint64_t)c.inflight * (ws_guess + pay_guess + (4ull << 20));
    const uint64_t sb = slot_bytes(c.max_leaves, c.max_nodes);
    if (c.hbm_budget_bytes <= fixed + sb) return PVVC_ERR_CAPACITY;
    const uint64_t nslots = std::min<uint64_t>((c.hbm_budget_bytes - fixed) / sb, 1ull << 30);
    if (pvvc_state_create((int32_t)std::min<uint64_t>(nslots, INT32_MAX), c.max_leaves, c.max_nodes, &s->state) != PVVC_OK)
        return PVVC_ERR_NOMEM;
    s->slot_owner.assign(nslots, -1);
    if (s->ring_xyz.ensure(12ull * c.ring_points) != cudaSuccess || s->ring_rgb.ensure(3ull * c.ring_points) != cudaSuccess) {
        pvvc_state_destroy(s->state);
        return PVVC_ERR_NOMEM;
    }
    s->ring.cap = c.ring_points;
    bool ok = cudaStreamCreateWithFlags(&s->compute, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamCreateWithFlags(&s->copy, cudaStreamNonBlocking) == cudaSuccess;
    for (int i = 0; ok && i < c.inflight; ++i) {
        auto b = std::make_unique<Batch>();
        ok = cudaEventCreateWithFlags(&b->e_h2d, cudaEventDisableTiming) == cudaSuccess &&
             cudaEventCreate(&b->e_start) == cudaSuccess && cudaEventCreate(&b->e_done) == cudaSuccess &&
             b->ws.ensure(ws_guess) == cudaSuccess && b->d_payload.ensure(pay_guess) == cudaSuccess &&
             b->h_payload.ensure(pay_guess) == cudaSuccess;
        s->batches.push_back(std::move(b));
    }
    if (!ok) {
        pvvc_server_destroy(s.release());
        return PVVC_ERR_NOMEM;
    }
    s->reserved = ring_bytes + nslots * sb;
    for (auto& b : s->batches) s->reserved += b->ws.cap + b->d_payload.cap;
    s->st.slots_total = nslots;
    s->st.slots_free = nslots;
    pvvc_server* raw = s.get();
    s->worker = std::thread([raw] { raw->worker_loop(); });
    s->completer = std::thread([raw] { raw->completion_loop(); });
    *out = s.release();
    return PVVC_OK;
}

extern "C" int pvvc_server_destroy(pvvc_server* s) {
    if (!s) return PVVC_ERR_ARG;
    {
        std::lock_guard<std::mutex> g(s->mu);
        s->stop = true;
    }
    s->cv_work.notify_all();
    if (s->worker.joinable()) s->worker.join();
    if (s->completer.joinable()) s->completer.join();
    if (s->compute) cudaStreamSynchronize(s->compute);
    if (s->copy) cudaStreamSynchronize(s->copy);
    for (auto& b : s->batches) {
        if (b->e_h2d) cudaEventDestroy(b->e_h2d);
        if (b->e_start) cudaEventDestroy(b->e_start);
        if (b->e_done) cudaEventDestroy(b->e_done);
    }
    for (auto& st : s->streams)
        for (Request* r : st.pending) delete r;
    if (s->compute) cudaStreamDestroy(s->compute);
    if (s->copy) cudaStreamDestroy(s->copy);
    if (s->state) pvvc_state_destroy(s->state);
    delete s;
    return PVVC_OK;
}

extern "C" int pvvc_server_open_stream(pvvc_server* s, int32_t nslots, int32_t* stream_id) {
    if (!s || !stream_id || nslots <= 0) return PVVC_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    // first fit over the slot pool
    const int64_t total = (int64_t)s->slot_owner.size();
    int64_t base = -1, run = 0;
    for (int64_t i = 0; i < total; ++i) {
        run = s->slot_owner[i] < 0 ? run + 1 : 0;
        if (run == nslots) {
            base = i - nslots + 1;
            break;
        }
    }
    if (base < 0) return PVVC_ERR_CAPACITY;
    int32_t id = -1;
    for (size_t i = 0; i < s->streams.size(); ++i)
        if (!s->streams[i].open && s->streams[i].outstanding == 0) {
            id = (int32_t)i;
            break;
        }
    if (id < 0) {
        id = (int32_t)s->streams.size();
        s->streams.emplace_back();
    }
    Stream& st = s->streams[id];
    st.open = true;
    st.slot_base = (int32_t)base;
    st.nslots = nslots;
    st.pending.clear();
    st.outstanding = 0;
    st.seen.assign(nslots, 0);
    for (int64_t i = base; i < base + nslots; ++i) s->slot_owner[i] = id;
    // forget whatever earlier streams left in these slots (stream-ordered
    // before any of this stream's batches)
    if (cudaMemsetAsync(s->state->v.info + base, 0, sizeof(SlotInfo) * nslots, s->compute) != cudaSuccess)
        return PVVC_ERR_CUDA;
    s->st.slots_free -= nslots;
    s->st.streams_open++;
    *stream_id = id;
    return PVVC_OK;
}

extern "C" int pvvc_server_close_stream(pvvc_server* s, int32_t id) {
    if (!s) return PVVC_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (id < 0 || id >= (int32_t)s->streams.size() || !s->streams[id].open) return PVVC_ERR_ARG;
    Stream& st = s->streams[id];
    st.open = false;  // no new submissions
    s->cv_poll.wait(lk, [&] { return st.outstanding == 0; });
    for (int64_t i = st.slot_base; i < st.slot_base + st.nslots; ++i) s->slot_owner[i] = -1;
    s->st.slots_free += st.nslots;
    s->st.streams_open--;
    return PVVC_OK;
}

extern "C" int pvvc_server_submit(pvvc_server* s, int32_t id, const uint8_t* bytes, uint64_t len, uint64_t tag) {
    if (!s) return PVVC_ERR_ARG;
    auto r = std::make_unique<Request>();
    const int rc = parse_request(bytes, len, r.get());
    if (rc) return rc;
    r->tag = tag;
    r->stream = id;
    std::lock_guard<std::mutex> g(s->mu);
    if (id < 0 || id >= (int32_t)s->streams.size() || !s->streams[id].open) return PVVC_ERR_ARG;
    Stream& st = s->streams[id];
    for (uint32_t i = 0; i < r->n; ++i)
        if (r->index[i] < 0 || r->index[i] >= st.nslots) return PVVC_ERR_ARG;
    if (r->points > s->cfg.max_batch_points) return PVVC_ERR_CAPACITY;
    r->submit_us = s->now();
    st.pending.push_back(r.release());
    st.outstanding++;
    s->cv_work.notify_one();
    return PVVC_OK;
}

extern "C" int pvvc_server_poll(pvvc_server* s, pvvc_completion* out, int32_t cap, int32_t* n, int32_t wait_us) {
    if (!s || !n || cap < 0 || (cap && !out)) return PVVC_ERR_ARG;
    std::unique_lock<std::mutex> lk(s->mu);
    if (s->done.empty() && wait_us > 0)
        s->cv_poll.wait_for(lk, std::chrono::microseconds(wait_us), [&] { return !s->done.empty(); });
    int32_t k = 0;
    while (k < cap && !s->done.empty()) {
        out[k++] = s->done.front();
        s->done.pop_front();
    }
    *n = k;
    return PVVC_OK;
}

extern "C" int pvvc_server_read(pvvc_server* s, uint64_t handle, float* xyz_host, uint8_t* rgb_host) {
    if (!s) return PVVC_ERR_ARG;
    uint64_t off, n;
    {
        std::lock_guard<std::mutex> g(s->mu);
        Ring::Entry* e = s->ring.find(handle);
        if (!e || e->released) return PVVC_ERR_ARG;
        off = e->off;
        n = e->n;
    }
    if (!n) return PVVC_OK;
    if (xyz_host && cudaMemcpy(xyz_host, static_cast<const float*>(s->ring_xyz.p) + 3 * off, 12 * n, cudaMemcpyDeviceToHost) !=
                        cudaSuccess)
        return PVVC_ERR_CUDA;
    if (rgb_host && cudaMemcpy(rgb_host, static_cast<const uint8_t*>(s->ring_rgb.p) + 3 * off, 3 * n, cudaMemcpyDeviceToHost) !=
                        cudaSuccess)
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}

extern "C" int pvvc_server_release(pvvc_server* s, uint64_t handle) {
    if (!s) return PVVC_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    if (!s->ring.release(handle)) return PVVC_ERR_ARG;
    s->cv_work.notify_all();
    return PVVC_OK;
}

extern "C" int pvvc_server_stats_get(pvvc_server* s, pvvc_server_stats* out) {
    if (!s || !out) return PVVC_ERR_ARG;
    std::lock_guard<std::mutex> g(s->mu);
    *out = s->st;
    out->reserved_bytes = s->reserved;
    return PVVC_OK;
}
