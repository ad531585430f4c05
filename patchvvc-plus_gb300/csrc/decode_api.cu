// decode_api.cu -- host side of the decode path: state pools, work-queue
// plans, the stream-ordered decode call, the end-to-end host call and the
// reference-signature shim.  See include/pvvc_gb300.h for the contract.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <deque>
#include <memory>
#include <mutex>
#include <numeric>
#include <thread>
#include <vector>

#include "../host/bitstream.h"
#include "decode_internal.h"
#include "zstd_core.h"

namespace pvvc {

// zero fields -> defaults; out-of-range fields -> PVVC_ERR_ARG
int resolve_tune(const pvvc_tune* in, pvvc_tune* out) {
    pvvc_tune t{kGroupCtasPerSm, kMinGroup, kRlgrBlock, kRlgrLongCtas, kRlgrMidPct, kRlgrLongLanes};
    if (in) {
        if (in->group_ctas_per_sm) t.group_ctas_per_sm = in->group_ctas_per_sm;
        if (in->min_group) t.min_group = in->min_group;
        if (in->rlgr_block) t.rlgr_block = in->rlgr_block;
        if (in->rlgr_long_ctas) t.rlgr_long_ctas = in->rlgr_long_ctas;
        if (in->rlgr_mid_pct) t.rlgr_mid_pct = in->rlgr_mid_pct;
        if (in->rlgr_long_lanes) t.rlgr_long_lanes = in->rlgr_long_lanes;
    }
    if (t.rlgr_long_lanes != 8 && t.rlgr_long_lanes != 16 && t.rlgr_long_lanes != 32) return PVVC_ERR_ARG;
    if (t.rlgr_mid_pct < -1 || t.rlgr_mid_pct > 90) return PVVC_ERR_ARG;
    if (t.group_ctas_per_sm < 1 || t.group_ctas_per_sm > 4 || t.min_group < 1 || t.min_group > 32) return PVVC_ERR_ARG;
    if (t.rlgr_long_ctas < -1 || t.rlgr_long_ctas > 152) return PVVC_ERR_ARG;
    if (t.rlgr_block != 32 && t.rlgr_block != 64 && t.rlgr_block != 128 && t.rlgr_block != 256) return PVVC_ERR_ARG;
    *out = t;
    return PVVC_OK;
}

namespace {

// A process-wide pool of host worker threads for the host call's and the
// planner's parallel loops (creating threads per loop cost milliseconds per
// call: a host call runs a few dozen such loops).  Several threads may run
// loops at once (the planners, the packer, the main thread): a loop is a
// job on a queue, the caller works on its own job too, and waits until
// every item is done and no worker still holds the job.
class HostPool {
  public:
    // Workers: the host threads but four, which the host call's own threads
    // (the caller, the packer and two planners) use: with one worker per
    // core, a worker preempted in the middle of a loop held up the loop's
    // caller for a scheduler time slice.
    static HostPool& get() {
        static HostPool p(std::max(1, (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency())) - 4));
        return p;
    }
    template <class F>
    void run(int n, int helpers, F&& fn) {
        Job job;
        job.n = n;
        job.fn = [&fn](int i) { fn(i); };
        {
            std::lock_guard<std::mutex> g(mu_);
            for (int k = 0; k < helpers; ++k) queue_.push_back(&job);
        }
        cv_.notify_all();
        work(job);
        std::unique_lock<std::mutex> g(mu_);
        // entries of this job no worker has taken yet
        for (auto it = queue_.begin(); it != queue_.end();) it = *it == &job ? queue_.erase(it) : it + 1;
        done_cv_.wait(g, [&] { return job.active == 0; });
    }
    ~HostPool() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stop_ = true;
        }
        cv_.notify_all();
        for (auto& t : workers_) t.join();
    }

  private:
    struct Job {
        std::function<void(int)> fn;
        int n = 0;
        std::atomic<int> next{0};
        int active = 0;  // workers inside work() (guarded by mu_)
    };
    explicit HostPool(int nthreads) {
        for (int t = 0; t < nthreads; ++t) workers_.emplace_back([this] { loop(); });
    }
    static void work(Job& job) {
        for (int i; (i = job.next.fetch_add(1)) < job.n;) job.fn(i);
    }
    void loop() {
        std::unique_lock<std::mutex> g(mu_);
        for (;;) {
            cv_.wait(g, [&] { return stop_ || !queue_.empty(); });
            if (stop_) return;
            Job* job = queue_.front();
            queue_.pop_front();
            ++job->active;
            g.unlock();
            work(*job);
            g.lock();
            if (--job->active == 0) done_cv_.notify_all();
        }
    }
    std::mutex mu_;
    std::condition_variable cv_, done_cv_;
    std::deque<Job*> queue_;
    std::vector<std::thread> workers_;
    bool stop_ = false;
};

// Runs fn(i) for i in [0, n) on up to `threads` host threads (the calling
// thread and pool workers).
template <class F>
void parallel_for(int n, int threads, F fn) {
    threads = std::max(1, std::min(threads, n));
    if (threads == 1) {
        for (int i = 0; i < n; ++i) fn(i);
        return;
    }
    HostPool::get().run(n, threads - 1, fn);
}

// Host threads for the planner's and the host call's parallel loops.
int host_threads() { return (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency())); }
// The planner's share of them on this thread (several plans built at once
// split the threads between them); 0: all.
thread_local int g_plan_threads = 0;
int plan_threads() { return g_plan_threads > 0 ? g_plan_threads : host_threads(); }

// Stable sort of slice indices by (size descending, slot ascending): an LSD
// radix sort over four 16-bit digits of ((~size) << 32 | slot), skipping the
// digits every key shares.  Ties keep their input order, as std::stable_sort
// with that comparator would.
void sort_by_size_slot(const uint32_t* size, const int32_t* slot, std::vector<int32_t>& ids) {
    const size_t n = ids.size();
    if (n < 2) return;
    std::vector<uint64_t> key(n), key2(n);
    std::vector<int32_t> ids2(n);
    for (size_t i = 0; i < n; ++i) key[i] = ((uint64_t)(~size[ids[i]]) << 32) | (uint32_t)slot[ids[i]];
    std::vector<uint32_t> cnt(65537);
    for (int d = 0; d < 4; ++d) {
        const int sh = 16 * d;
        std::fill(cnt.begin(), cnt.end(), 0u);
        for (size_t i = 0; i < n; ++i) ++cnt[((key[i] >> sh) & 0xFFFFu) + 1];
        if (cnt[((key[0] >> sh) & 0xFFFFu) + 1] == n) continue;  // one bucket: nothing to reorder
        for (int b = 0; b < 65536; ++b) cnt[b + 1] += cnt[b];
        for (size_t i = 0; i < n; ++i) {
            const uint32_t b = (uint32_t)((key[i] >> sh) & 0xFFFFu);
            const uint32_t at = cnt[b]++;
            key2[at] = key[i];
            ids2[at] = ids[i];
        }
        key.swap(key2);
        ids.swap(ids2);
    }
}
}  // namespace

// The queue to the device: synchronously (upload == nullptr), or from
// pinned mirrors on `upload`, or (defer, whatever `upload` is) left for
// upload_plan on the stream the caller gives it.  (Deferred copies must not
// fall back to synchronous ones for the default stream: a planner thread's
// cudaMemcpy waited for the decode already queued there, 3 ms a part.)
int copy_plan(pvvc_plan* p, cudaStream_t upload, bool defer) {
    const size_t n = (size_t)p->nslices;
    if (n == 0) return PVVC_OK;
    const size_t wb = sizeof(SliceWork) * n, ob = 4ull * n;
    const size_t gb = sizeof(GroupDesc) * p->groups.size(), ib = 4ull * p->idx.size();
    if (p->d_work.ensure(wb) != cudaSuccess || p->d_order.ensure(ob) != cudaSuccess ||
        p->d_groups.ensure(std::max<size_t>(gb, 16)) != cudaSuccess || p->d_idx.ensure(std::max<size_t>(ib, 16)) != cudaSuccess)
        return PVVC_ERR_NOMEM;
    auto put = [&](DevBuf& d, HostBuf& h, const void* src, size_t bytes) -> bool {
        if (!bytes) return true;
        if (!upload && !defer) return cudaMemcpy(d.p, src, bytes, cudaMemcpyHostToDevice) == cudaSuccess;
        if (src != h.p) {
            if (h.ensure(bytes) != cudaSuccess) return false;
            std::memcpy(h.p, src, bytes);
        }
        return defer || cudaMemcpyAsync(d.p, h.p, bytes, cudaMemcpyHostToDevice, upload) == cudaSuccess;
    };
    p->device_records = false;
    if (!put(p->d_work, p->h_work, p->h_work.p, wb) || !put(p->d_order, p->h_order, p->order.data(), ob) ||
        !put(p->d_groups, p->h_groups, p->groups.data(), gb) || !put(p->d_idx, p->h_idx, p->idx.data(), ib))
        return PVVC_ERR_CUDA;
    p->upload_pending = defer;  // the copies are queued later by upload_plan
    p->device_records = !defer;
    return PVVC_OK;
}

int upload_plan(pvvc_plan* p, cudaStream_t s) {
    if (p->refresh_pending) {
        // the call's per-slice fields up, then gathered into the records
        p->refresh_pending = false;
        const pvvc_batch_desc& d = p->refresh_src;
        const size_t n = (size_t)d.nslices;
        const size_t a8 = align_up(8 * n, 256), a4 = align_up(4 * n, 256), a1 = align_up(n, 256);
        const size_t total = 3 * a8 + 2 * a4 + a1 + 64 * n;
        if (p->d_call.ensure(total) != cudaSuccess) return PVVC_ERR_NOMEM;
        uint8_t* b = static_cast<uint8_t*>(p->d_call.p);
        uint8_t* at[7] = {b, b + a8, b + 2 * a8, b + 3 * a8, b + 3 * a8 + a4, b + 3 * a8 + 2 * a4, b + 3 * a8 + 2 * a4 + a1};
        const void* src[7] = {d.col_off, d.geo_off, d.out_off, d.col_size, d.geo_size, d.qp, d.mv};
        const size_t bytes[7] = {8 * n, 8 * n, 8 * n, 4 * n, 4 * n, n, 64 * n};
        for (int k = 0; k < 7; ++k)
            if (cudaMemcpyAsync(at[k], src[k], bytes[k], cudaMemcpyHostToDevice, s) != cudaSuccess) return PVVC_ERR_CUDA;
        const CallFields f{reinterpret_cast<const uint64_t*>(at[0]), reinterpret_cast<const uint64_t*>(at[1]),
                           reinterpret_cast<const uint64_t*>(at[2]), reinterpret_cast<const uint32_t*>(at[3]),
                           reinterpret_cast<const uint32_t*>(at[4]), at[5], reinterpret_cast<const float*>(at[6])};
        if (launch_refresh(static_cast<SliceWork*>(p->d_work.p), (int)n, f, s) != cudaSuccess) return PVVC_ERR_CUDA;
        return PVVC_OK;
    }
    if (!p->upload_pending) return PVVC_OK;
    p->upload_pending = false;
    const size_t n = (size_t)p->nslices;
    const size_t wb = sizeof(SliceWork) * n, ob = 4ull * n;
    const size_t gb = sizeof(GroupDesc) * p->groups.size(), ib = 4ull * p->idx.size();
    auto put = [&](DevBuf& d, HostBuf& h, size_t bytes) {
        return !bytes || cudaMemcpyAsync(d.p, h.p, bytes, cudaMemcpyHostToDevice, s) == cudaSuccess;
    };
    if (!put(p->d_work, p->h_work, wb) || !put(p->d_order, p->h_order, ob) || !put(p->d_groups, p->h_groups, gb) ||
        !put(p->d_idx, p->h_idx, ib))
        return PVVC_ERR_CUDA;
    p->device_records = true;
    return PVVC_OK;
}

int build_plan(const pvvc_batch_desc* d, pvvc_plan* p, const pvvc_tune* tune, cudaStream_t upload, bool defer) {
    if (!d || d->nslices < 0) return PVVC_ERR_ARG;
    if (resolve_tune(tune, &p->tune)) return PVVC_ERR_ARG;
    auto t_last = std::chrono::steady_clock::now();
    auto lap = [&](int k) {  // host milliseconds of the plan's stages (pvvc_plan_host_times)
        const auto now = std::chrono::steady_clock::now();
        p->host_ms[k] = std::chrono::duration<double, std::milli>(now - t_last).count();
        t_last = now;
    };
    const int n = d->nslices;
    if (n > 0 && (!d->slot || !d->type || !d->size || !d->qp || !d->mv || !d->geo_off || !d->geo_size || !d->col_off ||
                  !d->col_size || !d->out_off))
        return PVVC_ERR_ARG;
    p->refresh_pending = false;
    // The queue's structure -- order, tiers, groups, coefficient regions,
    // workspace -- depends on the slices' slots, types and sizes (and the
    // launch shapes) only.  When those equal the last build's (the same
    // layout decoded again: the next loop of a sequence, the same parts of a
    // host call), only the per-call fields of the records are refreshed.
    if (p->cache_valid && n > 0 && n == p->nslices && std::memcmp(&p->key_tune, &p->tune, sizeof(pvvc_tune)) == 0 &&
        std::memcmp(p->key_slot.data(), d->slot, 4ull * n) == 0 && std::memcmp(p->key_type.data(), d->type, n) == 0 &&
        std::memcmp(p->key_size.data(), d->size, 4ull * n) == 0) {
        if (defer && p->device_records) {
            // a host call's plan whose records are on the device: their
            // per-call fields are gathered there by k_refresh (upload_plan),
            // from the call's description arrays in their own order
            uint64_t m = 0;
            for (int i = 0; i < n; ++i) m = std::max<uint64_t>(m, d->out_off[i] + d->size[i]);
            p->total_points = m;
            p->refresh_src = *d;
            p->refresh_pending = true;
            lap(0);
            for (int k = 1; k < 5; ++k) p->host_ms[k] = 0;
            return PVVC_OK;
        }
        SliceWork* const W = static_cast<SliceWork*>(p->h_work.p);
        constexpr int kChunk = 4096;
        const int nch = (n + kChunk - 1) / kChunk;
        std::vector<uint64_t> ch_pts(nch, 0);
        parallel_for(nch, plan_threads(), [&](int c) {
            uint64_t m = 0;
            for (int q = c * kChunk, e = std::min(n, q + kChunk); q < e; ++q) {
                SliceWork& w = W[q];
                const int i = w.orig;
                w.col_off = d->col_off[i];
                w.geo_off = d->geo_off[i];
                w.out_off = d->out_off[i];
                w.csz = d->col_size[i];
                w.gsz = d->geo_size[i];
                w.qp = d->qp[i];
                for (int k = 0; k < 12; ++k) w.mv[k] = d->mv[16ull * i + k];
                m = std::max<uint64_t>(m, w.out_off + w.n);
            }
            ch_pts[c] = m;
        });
        p->total_points = 0;
        for (uint64_t m : ch_pts) p->total_points = std::max(p->total_points, m);
        lap(0);
        for (int k = 1; k < 4; ++k) p->host_ms[k] = 0;
        t_last = std::chrono::steady_clock::now();
        const int rc = copy_plan(p, upload, defer);
        lap(4);
        return rc;
    }
    p->cache_valid = false;
    // (after the reuse path: that one makes no CUDA call, so a planner thread
    // of the host call -- a new thread each call -- pays no first-call setup
    // of the CUDA runtime, which took milliseconds)
    if (prepare_kernels() != cudaSuccess) return PVVC_ERR_CUDA;
    std::vector<int32_t> intra, pred;
    int32_t max_slot = -1;
    for (int i = 0; i < n; ++i) {
        if (d->slot[i] < 0) return PVVC_ERR_ARG;
        max_slot = std::max(max_slot, d->slot[i]);
        ((d->type[i] & PVVC_TYPE_PREDICT) ? pred : intra).push_back(i);
    }
    // at most one intra slice per slot in a batch (it rebuilds the slot)
    {
        std::vector<int32_t> s;
        for (int i : intra) s.push_back(d->slot[i]);
        std::sort(s.begin(), s.end());
        if (std::adjacent_find(s.begin(), s.end()) != s.end()) return PVVC_ERR_ARG;
    }
    // largest first; equal sizes grouped by slot, so that the frames of one
    // patch run next to each other and share its tree tables in L2
    sort_by_size_slot(d->size, d->slot, intra);
    sort_by_size_slot(d->size, d->slot, pred);
    p->nslices = n;
    p->nintra = (int32_t)intra.size();
    p->max_slot = max_slot;
    // the queue's records are built in the page-locked mirror they are
    // uploaded from (every field of every record is written below)
    if (p->h_work.ensure(std::max<size_t>(sizeof(SliceWork) * n, 16)) != cudaSuccess) return PVVC_ERR_NOMEM;
    SliceWork* const W = static_cast<SliceWork*>(p->h_work.p);
    uint64_t coef = 0, fb = 0, pts = 0;
    // the queue: intra slices, then predictive ones.  The records are filled
    // in parallel (the descriptor is gathered in sorted order, so most reads
    // miss the cache); the coefficient regions are laid out further down.
    auto fill = [&](int q) {
        const int i = q < (int)intra.size() ? intra[q] : pred[q - intra.size()];
        SliceWork& w = W[q];
        std::memset(&w, 0, sizeof(w));
        w.col_off = d->col_off[i];
        w.geo_off = d->geo_off[i];
        w.out_off = d->out_off[i];
        w.csz = d->col_size[i];
        w.gsz = d->geo_size[i];
        w.n = d->size[i];
        w.slot = d->slot[i];
        w.orig = i;
        w.type = d->type[i];
        w.qp = d->qp[i];
        for (int k = 0; k < 12; ++k) w.mv[k] = d->mv[16ull * i + k];
    };
    // Chunks of the queue in parallel; each also sums its slices' fallback
    // buffers (6 floats per point of a slice above kRahtWcap leaves) and
    // its output extent, and the offsets follow from a prefix over chunks.
    constexpr int kFillChunk = 4096;
    const int nch = (n + kFillChunk - 1) / kFillChunk;
    std::vector<uint64_t> ch_fb(nch + 1, 0), ch_pts(nch, 0);
    auto fill_chunk = [&](int c) {
        uint64_t f = 0, m = 0;
        for (int q = c * kFillChunk, e = std::min(n, q + kFillChunk); q < e; ++q) {
            fill(q);
            const SliceWork& w = W[q];
            if (w.n > (uint32_t)kRahtWcap) f += 6ull * w.n;
            m = std::max<uint64_t>(m, w.out_off + w.n);
        }
        ch_fb[c + 1] = f;
        ch_pts[c] = m;
    };
    if (nch < 2)
        for (int c = 0; c < nch; ++c) fill_chunk(c);
    else
        parallel_for(nch, plan_threads(), fill_chunk);
    for (int c = 0; c < nch; ++c) {
        ch_fb[c + 1] += ch_fb[c];
        pts = std::max(pts, ch_pts[c]);
    }
    fb = ch_fb[nch];
    auto fb_chunk = [&](int c) {  // fallback-buffer offsets, in queue order from the chunk's base
        uint64_t f = ch_fb[c];
        for (int q = c * kFillChunk, e = std::min(n, q + kFillChunk); q < e; ++q) {
            SliceWork& w = W[q];
            if (w.n > (uint32_t)kRahtWcap) {
                w.fb_off = f;
                f += 6ull * w.n;
            } else {
                w.fb_off = ~0ull;
            }
        }
    };
    if (nch < 2)
        for (int c = 0; c < nch; ++c) fb_chunk(c);
    else
        parallel_for(nch, plan_threads(), fb_chunk);
    p->total_points = pts;
    lap(0);  // split, sort, queue records
    // RLGR order: all slices by size, so that a warp decodes similar lengths.
    // The queue holds the intra slices, then the predictive ones, each run
    // already sorted by (size descending, slot): merging the two runs (ties
    // from the first) is the stable sort of the whole queue by that key.
    p->order.resize(n);
    {
        const int ni = p->nintra;
        std::vector<int32_t> qa(ni), qb(n - ni);
        std::iota(qa.begin(), qa.end(), 0);
        std::iota(qb.begin(), qb.end(), ni);
        std::merge(qa.begin(), qa.end(), qb.begin(), qb.end(), p->order.begin(), [&](int32_t a, int32_t b) {
            if (W[a].n != W[b].n) return W[a].n > W[b].n;
            return W[a].slot < W[b].slot;
        });
    }
    // the head of that order goes to the long-slice launch (at most a quarter
    // of the slices, so that small batches still spread over many SMs)
    p->nlong = 0;
    p->nmid = 0;
    if (p->tune.rlgr_long_ctas > 0 && n >= 8) {
        p->nlong = std::min<int32_t>(kRlgrLongBlock * p->tune.rlgr_long_ctas, n / 4);
        if (p->side.ensure(true) != cudaSuccess) return PVVC_ERR_CUDA;
        // the larger part of the rest forms the medium tier
        if (p->tune.rlgr_mid_pct > 0) {
            p->nmid = (int32_t)((int64_t)(n - p->nlong) * p->tune.rlgr_mid_pct / 100);
            if (p->nmid > 0 && p->side2.ensure() != cudaSuccess) return PVVC_ERR_CUDA;
        }
    }
    if (!intra.empty() && p->tree.ensure() != cudaSuccess) return PVVC_ERR_CUDA;
    lap(1);  // RLGR order and tiers
    // inverse-RAHT schedule: slices grouped by slot (largest slots first)
    {
        // queue indices bucketed by slot (slots in order of first appearance,
        // each bucket in queue order): a counting sort into one array
        std::vector<int32_t> where(max_slot + 1, -1), slot_of, cnt_of;
        std::vector<int32_t> bucket_of(n);
        for (int q2 = 0; q2 < n; ++q2) {
            const int32_t sl = W[q2].slot;
            if (where[sl] < 0) {
                where[sl] = (int32_t)slot_of.size();
                slot_of.push_back(sl);
                cnt_of.push_back(0);
            }
            bucket_of[q2] = where[sl];
            ++cnt_of[where[sl]];
        }
        const int nb = (int)slot_of.size();
        std::vector<int32_t> bstart(nb + 1, 0), flat(n);
        for (int b = 0; b < nb; ++b) bstart[b + 1] = bstart[b] + cnt_of[b];
        {
            std::vector<int32_t> at(bstart.begin(), bstart.end() - 1);
            for (int q2 = 0; q2 < n; ++q2) flat[at[bucket_of[q2]]++] = q2;
        }
        std::vector<int32_t> ord(nb);
        std::iota(ord.begin(), ord.end(), 0);
        std::stable_sort(ord.begin(), ord.end(),
                         [&](int32_t a, int32_t b) { return W[flat[bstart[a]]].n > W[flat[bstart[b]]].n; });
        std::vector<GroupDesc> ga, gb;
        std::vector<int32_t> items, la, lb;
        items.reserve(n);
        for (int32_t si : ord) {
            const int32_t* L = flat.data() + bstart[si];  // the slot's queue indices
            const size_t Ln = (size_t)(bstart[si + 1] - bstart[si]);
            const bool has_intra = !(W[L[0]].type & PVVC_TYPE_PREDICT);
            for (size_t c0 = 0; c0 < Ln; c0 += 32) {
                const int cnt = (int)std::min<size_t>(32, Ln - c0);
                const bool first = c0 == 0;
                const bool phase_b = has_intra && !first;
                if ((first && has_intra) || cnt >= p->tune.min_group) {
                    GroupDesc g{slot_of[si], (int32_t)items.size(), cnt, (int16_t)((first && has_intra) ? 1 : 0)};
                    items.insert(items.end(), L + c0, L + c0 + cnt);
                    (phase_b ? gb : ga).push_back(g);
                } else {
                    auto& dst = phase_b ? lb : la;
                    dst.insert(dst.end(), L + c0, L + c0 + cnt);
                }
            }
        }
        // Window groups: phase-A groups of at least kWinGroupMin slices, all
        // of one size, in size tiers of whole groups (ga is already largest
        // first), so a tier's inverse RAHT waits for its own RLGR only.  The
        // long tier's slices -- the critical path -- are decoded by the
        // per-slice long launch, whose iterations are the cheapest, into
        // planes cleared first; the medium and short tiers by the windowed
        // RLGR, a warp per group, whose planes need no clear.  The slices of
        // no window group get one per-slice RLGR launch.
        p->nwin = 0;
        p->nwin_slices = 0;
        {
            std::vector<GroupDesc> gw, gr;
            for (const GroupDesc& g : ga) {
                bool ok = g.count >= kWinGroupMin;
                for (int l = 1; ok && l < g.count; ++l) ok = W[items[g.first + l]].n == W[items[g.first]].n;
                (ok ? gw : gr).push_back(g);
            }
            if (!gw.empty()) {
                const int nw = (int)gw.size();
                p->nwin = nw;
                p->ngroups_a_long = (p->tune.rlgr_long_ctas > 0 && nw >= 8)
                                        ? std::min(kWinGroupsPerLongCta * p->tune.rlgr_long_ctas, nw / 4)
                                        : 0;
                p->ngroups_a_mid = p->tune.rlgr_mid_pct > 0
                                       ? (int32_t)((int64_t)(nw - p->ngroups_a_long) * p->tune.rlgr_mid_pct / 100)
                                       : 0;
                p->ngroups_a_mid2 = kMidSplit > 1 && p->ngroups_a_mid >= kMidSplitMin ? p->ngroups_a_mid / 2 : 0;
                p->ngroups_a_mid -= p->ngroups_a_mid2;
                if (p->ngroups_a_long > 0 && p->side.ensure(true) != cudaSuccess) return PVVC_ERR_CUDA;
                if (p->ngroups_a_mid > 0 && p->side2.ensure() != cudaSuccess) return PVVC_ERR_CUDA;
                if (p->ngroups_a_mid2 > 0 && p->side3.ensure() != cudaSuccess) return PVVC_ERR_CUDA;
                ga = gw;
                ga.insert(ga.end(), gr.begin(), gr.end());
                // RLGR order: the window groups' slices in group order (sizes
                // descending; the long tier's slices first, their count in
                // nlong), then the other slices, largest first
                std::vector<uint8_t> inw(n, 0);
                std::vector<int32_t> ord2;
                ord2.reserve(n);
                p->nlong = 0;
                p->nmid = 0;
                for (int gi = 0; gi < nw; ++gi) {
                    const GroupDesc& g = gw[gi];
                    for (int l = 0; l < g.count; ++l) {
                        inw[items[g.first + l]] = 1;
                        ord2.push_back(items[g.first + l]);
                    }
                    if (gi < p->ngroups_a_long) p->nlong += g.count;
                }
                p->nwin_slices = (int32_t)ord2.size();
                for (int32_t q : p->order)
                    if (!inw[q]) ord2.push_back(q);
                p->order.swap(ord2);
            }
        }
        if (p->nwin == 0) {
            // phase-A groups that hold a slice of the long-slice RLGR launch first:
            // the others can be inverse-transformed as soon as the short launch ends
            // (tier 2), then those with a medium-tier slice (tier 1), then the rest
            {
                std::vector<uint8_t> tier(n, 0);
                for (int i = 0; i < p->nlong + p->nmid; ++i) tier[p->order[i]] = i < p->nlong ? 2 : 1;
                std::vector<GroupDesc> gl, gm, gs;
                for (const GroupDesc& g : ga) {
                    int t = 0;
                    for (int l = 0; l < g.count; ++l) t = std::max<int>(t, tier[items[g.first + l]]);
                    (t == 2 ? gl : t == 1 ? gm : gs).push_back(g);
                }
                p->ngroups_a_long = (int32_t)gl.size();
                p->ngroups_a_mid = (int32_t)gm.size();
                p->ngroups_a_mid2 = 0;
                ga = gl;
                ga.insert(ga.end(), gm.begin(), gm.end());
                ga.insert(ga.end(), gs.begin(), gs.end());
            }
        }
        p->groups = ga;
        p->groups.insert(p->groups.end(), gb.begin(), gb.end());
        p->long_split_off = (int32_t)p->groups.size();
        p->nlong_split = 0;
        if (p->nwin > 0 && kLongSplit > 1)
            for (int gi = 0; gi < p->ngroups_a_long; ++gi)
                for (int h = 0; h < kLongSplit; ++h) {
                    GroupDesc g = ga[gi];
                    g.part = (uint8_t)h;
                    g.parts = (uint8_t)kLongSplit;
                    p->groups.push_back(g);
                    ++p->nlong_split;
                }
        p->ngroups_a = (int32_t)ga.size();
        p->ngroups_b = (int32_t)gb.size();
        p->idx = items;
        p->list_a_off = (int32_t)p->idx.size();
        p->idx.insert(p->idx.end(), la.begin(), la.end());
        p->list_b_off = (int32_t)p->idx.size();
        p->idx.insert(p->idx.end(), lb.begin(), lb.end());
        p->nlist_a = (int32_t)la.size();
        p->nlist_b = (int32_t)lb.size();
        // coefficient regions: a group shares one frame-interleaved region
        // (stride 32), every other slice owns contiguous planes
        // (window groups first; a region holds the largest slice of its group)
        uint64_t c = 0;
        p->coef_win_floats = 0;
        for (int32_t gi = 0; gi < p->ngroups_a + p->ngroups_b; ++gi) {  // (not the long groups' split copies)
            const GroupDesc& g = p->groups[gi];
            uint32_t gn = 0;
            for (int l = 0; l < g.count; ++l) {
                SliceWork& w = W[p->idx[g.first + l]];
                w.coef_off = c;
                w.coef_stride = 32;
                w.coef_lane = (uint32_t)l;
                gn = std::max(gn, w.n);
            }
            c += 3ull * gn * 32;
            if ((int32_t)gi + 1 == p->nwin) p->coef_win_floats = c;
        }
        for (int li = p->list_a_off; li < (int)p->idx.size(); ++li) {
            SliceWork& w = W[p->idx[li]];
            w.coef_off = c;
            w.coef_stride = 1;
            w.coef_lane = 0;
            c += 3ull * w.n;
        }
        coef = c;
        p->coef_floats = coef;
        // the prefix of the planes that the long-slice RLGR launch writes
        // (its groups come first; a long slice outside a group extends it)
        p->coef_long_floats = 0;
        p->coef_mid_floats = 0;
        for (int i = 0; i < p->nlong + p->nmid; ++i) {
            const SliceWork& w = W[p->order[i]];
            const uint64_t e = w.coef_off + 3ull * w.n * w.coef_stride;
            if (i < p->nlong) p->coef_long_floats = std::max(p->coef_long_floats, e);
            p->coef_mid_floats = std::max(p->coef_mid_floats, e);
        }
    }
    lap(2);  // groups and coefficient regions
    // workspace layout
    uint64_t off = 0;
    p->ws_coef = off;
    off = align_up(off + coef * 4, 256);
    p->ws_fb = off;
    off = align_up(off + fb * 4, 256);
    p->ws_tstatus = off;
    off = align_up(off + 4ull * n, 256);
    p->ws_rstatus = off;
    off = align_up(off + 4ull * n, 256);
    p->ws_fstatus = off;
    off = align_up(off + 4ull * n, 256);
    // group kernel: per persistent CTA two level buffers of [width][32 lanes][3]
    // floats; an internal level of a valid tree is never wider than its leaves
    {
        uint32_t maxn = 0;
        for (const auto& g : p->groups) maxn = std::max(maxn, W[p->idx[g.first]].n);
        p->grp_ctas = std::min<int32_t>(p->ngroups_a + p->ngroups_b, p->tune.group_ctas_per_sm * sm_count());
        p->grp_floats = 2ull * std::max<uint32_t>(maxn, 1) * 96;
        p->ws_grp = off;
        off = align_up(off + 4ull * p->grp_floats * std::max(p->grp_ctas, 1), 256);
        // the long-slice groups run beside the others, with level buffers of their own
        const int32_t nlg = p->nlong_split > 0 ? p->nlong_split : p->ngroups_a_long;  // the long groups' launch
        p->grp_ctas_long = nlg > 0 ? std::min<int32_t>(nlg, p->grp_ctas) : 0;
        p->ws_grp_long = off;
        off = align_up(off + 4ull * p->grp_floats * p->grp_ctas_long, 256);
        p->grp_ctas_mid = p->ngroups_a_mid > 0 ? std::min<int32_t>(p->ngroups_a_mid, p->grp_ctas) : 0;
        p->ws_grp_mid = off;
        off = align_up(off + 4ull * p->grp_floats * p->grp_ctas_mid, 256);
        p->grp_ctas_mid2 = p->ngroups_a_mid2 > 0 ? std::min<int32_t>(p->ngroups_a_mid2, p->grp_ctas) : 0;
        p->ws_grp_mid2 = off;
        off = align_up(off + 4ull * p->grp_floats * p->grp_ctas_mid2, 256);
        p->ws_counter = off;
        off = align_up(off + 32, 256);
    }
    p->ws_bytes = std::max<uint64_t>(off, 256);
    lap(3);  // workspace layout
    // upload: synchronous from the plan's vectors, or (upload != nullptr)
    // stream-ordered from pinned mirrors that stay untouched until the plan is
    // rebuilt (the caller orders that after the copies)
    const int rc = copy_plan(p, upload, defer);
    lap(4);  // upload
    if (rc == PVVC_OK && n > 0) {  // the layout this structure was built for
        p->key_slot.assign(d->slot, d->slot + n);
        p->key_type.assign(d->type, d->type + n);
        p->key_size.assign(d->size, d->size + n);
        p->key_tune = p->tune;
        p->cache_valid = true;
    }
    return rc;
}

int run_decode(const pvvc_plan* p, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb, float* p24,
               int32_t* status, void* ws, uint64_t ws_bytes, cudaStream_t s, void* const* events) {
    if (!p || !st) return PVVC_ERR_ARG;
    if (p->nslices == 0) return PVVC_OK;
    if (!payload || (reinterpret_cast<uintptr_t>(payload) & 15u)) return PVVC_ERR_ARG;
    if (!ws || ws_bytes < p->ws_bytes || (reinterpret_cast<uintptr_t>(ws) & 255u)) return PVVC_ERR_CAPACITY;
    if (p->max_slot >= st->v.nslots) return PVVC_ERR_ARG;
    uint8_t* w = static_cast<uint8_t*>(ws);
    float* coef = reinterpret_cast<float*>(w + p->ws_coef);
    float* fb = reinterpret_cast<float*>(w + p->ws_fb);
    int32_t* ts = reinterpret_cast<int32_t*>(w + p->ws_tstatus);
    int32_t* rs = reinterpret_cast<int32_t*>(w + p->ws_rstatus);
    int32_t* fs = reinterpret_cast<int32_t*>(w + p->ws_fstatus);
    const SliceWork* dw = static_cast<const SliceWork*>(p->d_work.p);
    const int32_t* ord = static_cast<const int32_t*>(p->d_order.p);
    auto mark = [&](int i) {
        return !events || cudaEventRecord(static_cast<cudaEvent_t>(events[i]), s) == cudaSuccess;
    };
    if (!mark(0)) return PVVC_ERR_CUDA;
    // The tree expansion reads only geometry payloads and writes only slot
    // tables, the coefficient clear and RLGR only colour payloads and
    // coefficient planes: without stage markers the tree runs beside them on
    // a stream of their own, joined (event `mid`) before the inverse RAHT.
    const bool tree_aside = !events && p->nintra > 0;
    if (tree_aside) {
        const SideStream& tr = p->tree;
        if (cudaEventRecord(tr.fork, s) != cudaSuccess || cudaStreamWaitEvent(tr.s, tr.fork, 0) != cudaSuccess ||
            launch_tree(dw, p->nintra, payload, st->v, ts, tr.s) != cudaSuccess || cudaEventRecord(tr.mid, tr.s) != cudaSuccess)
            return PVVC_ERR_CUDA;
    } else if (launch_tree(dw, p->nintra, payload, st->v, ts, s) != cudaSuccess || !mark(1)) {
        return PVVC_ERR_CUDA;
    }
    float* gsc = reinterpret_cast<float*>(w + p->ws_grp);
    int* cnt = reinterpret_cast<int*>(w + p->ws_counter);  // queue counters: A long, B, A short, A medium, A medium 2
    const GroupDesc* dg = static_cast<const GroupDesc*>(p->d_groups.p);
    const int32_t* di = static_cast<const int32_t*>(p->d_idx.p);
    auto raht_groups = [&](int first, int count, int* counter, float* scratch, int ctas, cudaStream_t on) {
        return count <= 0 || launch_raht_group(dw, dg + first, count, di, st->v, coef, ts, rs, fs, xyz, rgb, p24, status,
                                               scratch, p->grp_floats, ctas, counter, on) == cudaSuccess;
    };
    auto clear = [&](uint64_t from, uint64_t to) {
        return to <= from || cudaMemsetAsync(coef + from, 0, 4ull * (to - from), s) == cudaSuccess;
    };
    auto fork = [&](const SideStream& sd) {
        return cudaEventRecord(sd.fork, s) == cudaSuccess && cudaStreamWaitEvent(sd.s, sd.fork, 0) == cudaSuccess;
    };
    if (p->nwin > 0) {
        // RLGR in size tiers of whole window groups: the long tier (the
        // per-slice long launch, its planes cleared first) on SMs of its own
        // (stream `side`), the medium tier windowed (stream `side2`), the
        // short tier windowed and then the per-slice launch of the other
        // slices (this stream; only their planes are cleared).  Each tier's
        // groups are inverse-transformed on its stream once that tier is
        // decoded and the trees are built.
        const SideStream& L = p->side;
        const SideStream& M = p->side2;
        const SideStream& M2 = p->side3;
        const int nl = p->ngroups_a_long, nm = p->ngroups_a_mid, nm2 = p->ngroups_a_mid2, nw = p->nwin;
        const int nrest = p->nslices - p->nwin_slices;
        const int wwarps = std::max(1, p->tune.rlgr_block / 32);
        if (nl > 0 && (!clear(0, p->coef_long_floats) || !fork(L) ||
                       launch_rlgr_long(dw, ord, p->nlong, payload, coef, rs, p->tune.rlgr_long_lanes, kRlgrLongSmem, L.s) !=
                           cudaSuccess))
            return PVVC_ERR_CUDA;
        if (nm > 0 &&
            (!fork(M) || launch_rlgr_win(dw, dg + nl, nm, di, payload, coef, rs, wwarps, M.s) != cudaSuccess))
            return PVVC_ERR_CUDA;
        if (nm2 > 0 &&
            (!fork(M2) || launch_rlgr_win(dw, dg + nl + nm, nm2, di, payload, coef, rs, wwarps, M2.s) != cudaSuccess))
            return PVVC_ERR_CUDA;
        const int ns0 = nl + nm + nm2;  // the short tier's first group
        if (launch_rlgr_win(dw, dg + ns0, nw - ns0, di, payload, coef, rs, wwarps, s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (nrest > 0 && (!clear(p->coef_win_floats, p->coef_floats) ||
                          launch_rlgr(dw, ord + p->nwin_slices, nrest, payload, coef, rs, p->tune.rlgr_block, kRlgrShortSmem,
                                      s) != cudaSuccess))
            return PVVC_ERR_CUDA;
        if (events) {
            // stage markers: every tier decoded, then every group
            if ((nl > 0 && (cudaEventRecord(L.join, L.s) != cudaSuccess || cudaStreamWaitEvent(s, L.join, 0) != cudaSuccess)) ||
                (nm > 0 && (cudaEventRecord(M.join, M.s) != cudaSuccess || cudaStreamWaitEvent(s, M.join, 0) != cudaSuccess)) ||
                (nm2 > 0 && (cudaEventRecord(M2.join, M2.s) != cudaSuccess || cudaStreamWaitEvent(s, M2.join, 0) != cudaSuccess)) ||
                !mark(2) || !raht_groups(0, p->ngroups_a, cnt, gsc, p->grp_ctas, s))
                return PVVC_ERR_CUDA;
        } else {
            // the long groups, each split over several CTAs (their copies after the phase-B groups)
            const int lf = p->nlong_split > 0 ? p->long_split_off : 0, ln = p->nlong_split > 0 ? p->nlong_split : nl;
            if (nl > 0 && ((tree_aside && cudaStreamWaitEvent(L.s, p->tree.mid, 0) != cudaSuccess) ||
                           !raht_groups(lf, ln, cnt, reinterpret_cast<float*>(w + p->ws_grp_long), p->grp_ctas_long, L.s) ||
                           cudaEventRecord(L.join, L.s) != cudaSuccess))
                return PVVC_ERR_CUDA;
            if (nm > 0 && ((tree_aside && cudaStreamWaitEvent(M.s, p->tree.mid, 0) != cudaSuccess) ||
                           !raht_groups(nl, nm, cnt + 3, reinterpret_cast<float*>(w + p->ws_grp_mid), p->grp_ctas_mid,
                                        M.s) ||
                           cudaEventRecord(M.join, M.s) != cudaSuccess))
                return PVVC_ERR_CUDA;
            if (nm2 > 0 && ((tree_aside && cudaStreamWaitEvent(M2.s, p->tree.mid, 0) != cudaSuccess) ||
                            !raht_groups(nl + nm, nm2, cnt + 4, reinterpret_cast<float*>(w + p->ws_grp_mid2),
                                         p->grp_ctas_mid2, M2.s) ||
                            cudaEventRecord(M2.join, M2.s) != cudaSuccess))
                return PVVC_ERR_CUDA;
            if ((tree_aside && cudaStreamWaitEvent(s, p->tree.mid, 0) != cudaSuccess) ||
                !raht_groups(ns0, p->ngroups_a - ns0, cnt + 2, gsc, p->grp_ctas, s) ||
                (nl > 0 && cudaStreamWaitEvent(s, L.join, 0) != cudaSuccess) ||
                (nm > 0 && cudaStreamWaitEvent(s, M.join, 0) != cudaSuccess) ||
                (nm2 > 0 && cudaStreamWaitEvent(s, M2.join, 0) != cudaSuccess))
                return PVVC_ERR_CUDA;
        }
    } else if (p->nlong == 0) {
        // zero symbols are not written by the decoder: clear the planes first
        if (!clear(0, p->coef_floats) ||
            launch_rlgr(dw, ord, p->nslices, payload, coef, rs, p->tune.rlgr_block, 0, s) != cudaSuccess || !mark(2))
            return PVVC_ERR_CUDA;
        if (tree_aside && cudaStreamWaitEvent(s, p->tree.mid, 0) != cudaSuccess) return PVVC_ERR_CUDA;
        if (!raht_groups(0, p->ngroups_a, cnt, gsc, p->grp_ctas, s)) return PVVC_ERR_CUDA;
    } else {
        // Size tiers, largest first in `order`: the long slices on SMs of their
        // own (stream `side`), the medium ones (stream `side2`), the rest (this
        // stream).  Each tier's planes are cleared just before it forks.
        const SideStream& L = p->side;
        const SideStream& M = p->side2;
        const int nl = p->nlong, nm = p->nmid, ns = p->nslices - nl - nm;
        const uint64_t cl = p->coef_long_floats, cm = std::max(p->coef_mid_floats, cl);
        if (!clear(0, cl) || !fork(L) ||
            launch_rlgr_long(dw, ord, nl, payload, coef, rs, p->tune.rlgr_long_lanes, kRlgrLongSmem, L.s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (nm > 0 && (!clear(cl, cm) || !fork(M) ||
                       launch_rlgr(dw, ord + nl, nm, payload, coef, rs, p->tune.rlgr_block, kRlgrShortSmem, M.s) !=
                           cudaSuccess ||
                       cudaEventRecord(M.mid, M.s) != cudaSuccess))
            return PVVC_ERR_CUDA;
        if (!clear(nm > 0 ? cm : cl, p->coef_floats) ||
            launch_rlgr(dw, ord + nl + nm, ns, payload, coef, rs, p->tune.rlgr_block, kRlgrShortSmem, s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        const int na_l = p->ngroups_a_long, na_m = p->ngroups_a_mid, na_s = p->ngroups_a - na_l - na_m;
        if (events) {
            // stage markers: every tier decoded, then every group
            if (cudaEventRecord(L.join, L.s) != cudaSuccess || cudaStreamWaitEvent(s, L.join, 0) != cudaSuccess ||
                (nm > 0 && cudaStreamWaitEvent(s, M.mid, 0) != cudaSuccess) || !mark(2) ||
                !raht_groups(0, p->ngroups_a, cnt, gsc, p->grp_ctas, s))
                return PVVC_ERR_CUDA;
        } else {
            // Each tier's groups follow its decode on its stream.  A group can
            // straddle a size cut, so a tier's groups also wait for the
            // smaller tiers' decode (which ends sooner); all wait for the trees.
            if (tree_aside && cudaStreamWaitEvent(s, p->tree.mid, 0) != cudaSuccess) return PVVC_ERR_CUDA;
            if (cudaEventRecord(L.mid, s) != cudaSuccess) return PVVC_ERR_CUDA;  // the small tier decoded, trees built
            if (nm > 0 && (cudaStreamWaitEvent(M.s, L.mid, 0) != cudaSuccess ||
                           !raht_groups(na_l, na_m, cnt + 3, reinterpret_cast<float*>(w + p->ws_grp_mid), p->grp_ctas_mid,
                                        M.s) ||
                           cudaEventRecord(M.join, M.s) != cudaSuccess))
                return PVVC_ERR_CUDA;
            if (cudaStreamWaitEvent(L.s, L.mid, 0) != cudaSuccess ||
                (nm > 0 && cudaStreamWaitEvent(L.s, M.mid, 0) != cudaSuccess) ||
                !raht_groups(0, na_l, cnt, reinterpret_cast<float*>(w + p->ws_grp_long), p->grp_ctas_long, L.s) ||
                cudaEventRecord(L.join, L.s) != cudaSuccess)
                return PVVC_ERR_CUDA;
            if (!raht_groups(na_l + na_m, na_s, cnt + 2, gsc, p->grp_ctas, s) ||
                cudaStreamWaitEvent(s, L.join, 0) != cudaSuccess || (nm > 0 && cudaStreamWaitEvent(s, M.join, 0) != cudaSuccess))
                return PVVC_ERR_CUDA;
        }
    }
    // phase A: the slices of slots without a group here, inverse-transformed by a CTA each
    if (launch_raht_slice(dw, di + p->list_a_off, p->nlist_a, st->v, coef, fb, ts, rs, fs, xyz, rgb, p24, status, kRahtWcap,
                          s) != cudaSuccess ||
        !mark(3))
        return PVVC_ERR_CUDA;
    // phase B: predictive slices whose intra colours phase A produced
    if (launch_raht_group(dw, dg + p->ngroups_a, p->ngroups_b, di, st->v, coef, ts, rs, fs, xyz, rgb, p24, status, gsc,
                          p->grp_floats, p->grp_ctas, cnt + 1, s) != cudaSuccess ||
        launch_raht_slice(dw, di + p->list_b_off, p->nlist_b, st->v, coef, fb, ts, rs, fs, xyz, rgb, p24, status, kRahtWcap, s) !=
            cudaSuccess ||
        !mark(4))
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}

}  // namespace pvvc

using namespace pvvc;

extern "C" const char* pvvc_status_string(int s) {
    switch (s) {
        case PVVC_OK: return "ok";
        case PVVC_ERR_ARG: return "invalid argument";
        case PVVC_ERR_OVERRUN: return "colour bitstream ended before all symbols were decoded";
        case PVVC_ERR_GEOMETRY: return "occupancy stream short or malformed";
        case PVVC_ERR_SIZE: return "leaf count does not match the slice size";
        case PVVC_ERR_NO_REFERENCE: return "predictive slice without an intra slice";
        case PVVC_ERR_BAD_SLICE: return "invalid slice type";
        case PVVC_ERR_NOMEM: return "out of memory";
        case PVVC_ERR_CUDA: return "CUDA runtime error";
        case PVVC_ERR_ZSTD: return "zstd payload cannot be decoded";
        case PVVC_ERR_FORMAT: return "malformed .frame / .slice bytes";
        case PVVC_ERR_CAPACITY: return "output or workspace too small";
        case PVVC_ERR_TREE: return "octree exceeds the state slot capacity";
        default: return "unknown status";
    }
}

extern "C" int pvvc_state_create(int32_t nslots, int32_t max_leaves, int32_t max_nodes, pvvc_state** out) {
    if (!out || nslots <= 0 || max_leaves <= 0 || max_nodes <= 0) return PVVC_ERR_ARG;
    *out = nullptr;
    auto st = std::make_unique<pvvc_state>();
    StateView& v = st->v;
    v.nslots = nslots;
    v.max_leaves = max_leaves;
    v.max_nodes = max_nodes;
    const size_t S = (size_t)nslots, Nn = (size_t)max_nodes, Nl = (size_t)max_leaves;
    bool ok = true;
    auto alloc = [&](void** p, size_t bytes) {
        if (!ok) return;
        if (cudaMalloc(p, bytes) != cudaSuccess) ok = false;
    };
    alloc((void**)&v.info, sizeof(SlotInfo) * S);
    alloc((void**)&v.occ, S * Nn);
    alloc((void**)&v.mask, S * Nn);
    alloc((void**)&v.cbase, 4 * S * Nn);
    alloc((void**)&v.coff, 4 * S * Nn);
    alloc((void**)&v.ab, sizeof(float2) * 7 * S * Nn);
    alloc((void**)&v.wsum, 4 * S * Nn);
    alloc((void**)&v.ctr, 12 * S * Nn);
    alloc((void**)&v.xyz, 12 * S * Nl);
    alloc((void**)&v.ref, 12 * S * Nl);
    if (!ok || cudaMemset(v.info, 0, sizeof(SlotInfo) * S) != cudaSuccess) {
        pvvc_state_destroy(st.release());
        return PVVC_ERR_NOMEM;
    }
    *out = st.release();
    return PVVC_OK;
}

extern "C" int pvvc_state_destroy(pvvc_state* st) {
    if (!st) return PVVC_ERR_ARG;
    StateView& v = st->v;
    void* ptrs[] = {v.info, v.occ, v.mask, v.cbase, v.coff, v.ab, v.wsum, v.ctr, v.xyz, v.ref};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    for (cudaEvent_t e : st->part_done)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : st->zdone)
        if (e) cudaEventDestroy(e);
    for (cudaEvent_t e : st->up_done)
        if (e) cudaEventDestroy(e);
    for (int h = 0; h < pvvc_state::kParts; ++h)
        for (cudaEvent_t e : {st->t_up[h], st->t_dec[h], st->t_cp[h]})
            if (e) cudaEventDestroy(e);
    if (st->t_start) cudaEventDestroy(st->t_start);
    if (st->copy) cudaStreamDestroy(st->copy);
    if (st->zside) cudaStreamDestroy(st->zside);
    if (st->up) cudaStreamDestroy(st->up);
    delete st;
    return PVVC_OK;
}

extern "C" int pvvc_state_reset(pvvc_state* st, void* stream) {
    if (!st) return PVVC_ERR_ARG;
    return cudaMemsetAsync(st->v.info, 0, sizeof(SlotInfo) * st->v.nslots, (cudaStream_t)stream) == cudaSuccess ? PVVC_OK
                                                                                                                : PVVC_ERR_CUDA;
}

extern "C" int pvvc_plan_create_tuned(const pvvc_batch_desc* desc, const pvvc_tune* tune, pvvc_plan** out) {
    if (!out) return PVVC_ERR_ARG;
    *out = nullptr;
    auto p = std::make_unique<pvvc_plan>();
    int s = build_plan(desc, p.get(), tune, nullptr);
    if (s) return s;
    *out = p.release();
    return PVVC_OK;
}

extern "C" int pvvc_plan_create(const pvvc_batch_desc* desc, pvvc_plan** out) {
    return pvvc_plan_create_tuned(desc, nullptr, out);
}

extern "C" int pvvc_plan_info_get(const pvvc_plan* p, pvvc_plan_info* info) {
    if (!p || !info) return PVVC_ERR_ARG;
    std::memset(info, 0, sizeof(*info));
    info->nslices = p->nslices;
    info->nintra = p->nintra;
    info->groups_a = p->ngroups_a;
    info->groups_b = p->ngroups_b;
    info->singles_a = p->nlist_a;
    info->singles_b = p->nlist_b;
    info->group_ctas = p->grp_ctas;
    info->tune = p->tune;
    info->clear_bytes =
        p->nwin > 0
            ? 4ull * p->coef_long_floats + (p->nslices > p->nwin_slices ? 4ull * (p->coef_floats - p->coef_win_floats) : 0ull)
            : 4ull * p->coef_floats;
    if (p->nslices > 0 && p->nwin > 0)
        info->kernels = (p->nintra > 0) + (p->ngroups_a_long > 0) + (p->ngroups_a_mid > 0) + (p->ngroups_a_mid2 > 0) +
                        (p->nwin > p->ngroups_a_long + p->ngroups_a_mid + p->ngroups_a_mid2) +
                        (p->nslices > p->nwin_slices) + (p->ngroups_a_long > 0) + (p->ngroups_a_mid > 0) +
                        (p->ngroups_a_mid2 > 0) +
                        (p->ngroups_a > p->ngroups_a_long + p->ngroups_a_mid + p->ngroups_a_mid2) + (p->nlist_a > 0) +
                        (p->ngroups_b > 0) +
                        (p->nlist_b > 0);
    else if (p->nslices > 0)
        info->kernels = (p->nintra > 0) + 1 + (p->nlong > 0) + (p->nmid > 0) +
                        (p->nlong > 0 ? (p->ngroups_a_long > 0) + (p->ngroups_a_mid > 0) +
                                            (p->ngroups_a > p->ngroups_a_long + p->ngroups_a_mid)
                                      : (p->ngroups_a > 0)) +
                        (p->nlist_a > 0) + (p->ngroups_b > 0) + (p->nlist_b > 0);
    return PVVC_OK;
}

namespace {
// device time of `reps` decodes of `p` (ms each), or a negative value on error
// Mean device time of one decode of plan p, as the decode is meant to run:
// captured once into a CUDA graph and replayed on s (stream launches time
// differently where a plan runs kernels side by side).
float time_plan(pvvc_plan* p, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb, int32_t* status,
                DevBuf& ws, int reps, cudaStream_t s) {
    // the median of `reps` timed replays of the plan's graph (one untimed
    // replay first): robust to the odd slow replay, so that the search does
    // not chase noise
    if (ws.ensure(p->ws_bytes) != cudaSuccess) return -1.f;
    reps = std::max(1, std::min(reps, 64));
    cudaStream_t cs = nullptr;
    cudaGraph_t g = nullptr;
    cudaGraphExec_t ge = nullptr;
    std::vector<cudaEvent_t> ev(reps + 1, nullptr);
    float ms = -1.f;
    bool ok = cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) == cudaSuccess &&
              cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) == cudaSuccess;
    if (ok) {
        const int rc = run_decode(p, st, payload, xyz, rgb, nullptr, status, ws.p, ws.cap, cs, nullptr);
        ok = cudaStreamEndCapture(cs, &g) == cudaSuccess && rc == PVVC_OK && g;
    }
    ok = ok && cudaGraphInstantiate(&ge, g, 0) == cudaSuccess;
    for (auto& e : ev) ok = ok && cudaEventCreate(&e) == cudaSuccess;
    ok = ok && cudaGraphLaunch(ge, s) == cudaSuccess;  // untimed: first touch of the workspace, L2 state
    ok = ok && cudaEventRecord(ev[0], s) == cudaSuccess;
    for (int r = 0; ok && r < reps; ++r)
        ok = cudaGraphLaunch(ge, s) == cudaSuccess && cudaEventRecord(ev[r + 1], s) == cudaSuccess;
    if (ok && cudaEventSynchronize(ev[reps]) == cudaSuccess) {
        std::vector<float> t(reps);
        for (int r = 0; ok && r < reps; ++r) ok = cudaEventElapsedTime(&t[r], ev[r], ev[r + 1]) == cudaSuccess;
        if (ok) {
            std::sort(t.begin(), t.end());
            ms = (reps & 1) ? t[reps / 2] : 0.5f * (t[reps / 2 - 1] + t[reps / 2]);
        }
    }
    for (auto& e : ev)
        if (e) cudaEventDestroy(e);
    if (ge) cudaGraphExecDestroy(ge);
    if (g) cudaGraphDestroy(g);
    if (cs) cudaStreamDestroy(cs);
    return ms;
}
}  // namespace

extern "C" int pvvc_plan_autotune(const pvvc_batch_desc* desc, pvvc_state* st, const uint8_t* payload, int32_t reps,
                                  void* stream, pvvc_tune* best, float* best_ms) {
    if (!desc || !st || !best || reps <= 0) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    pvvc_plan probe;
    int rc = build_plan(desc, &probe, nullptr, nullptr);
    if (rc) return rc;
    DevBuf xyz, rgb, status, ws;
    if (xyz.ensure(std::max<uint64_t>(12 * probe.total_points, 4)) != cudaSuccess ||
        rgb.ensure(std::max<uint64_t>(3 * probe.total_points, 4)) != cudaSuccess ||
        status.ensure(std::max<uint64_t>(4ull * probe.nslices, 4)) != cudaSuccess)
        return PVVC_ERR_NOMEM;
    float* dx = static_cast<float*>(xyz.p);
    uint8_t* dr = static_cast<uint8_t*>(rgb.p);
    int32_t* ds = static_cast<int32_t*>(status.p);
    pvvc_tune cur = probe.tune;
    float cur_ms = time_plan(&probe, st, payload, dx, dr, ds, ws, reps, s);
    if (cur_ms < 0) return PVVC_ERR_CUDA;
    // coordinate search: each field in turn over its candidates, twice
    const int32_t ctas[] = {1, 2, 3, 4};
    const int32_t groups[] = {2, 4, 8, 16};
    const int32_t blocks[] = {32, 64, 128, 256};
    const int32_t longs[] = {-1, 16, 32, 48, 64, 96};
    const int32_t mids[] = {-1, 15, 30, 50, 70};
    const int32_t lanes[] = {8, 16, 32};
    for (int pass = 0; pass < 2; ++pass) {
        bool moved = false;
        for (int field = 0; field < 6; ++field) {
            const int32_t* cand = field == 0 ? ctas
                                : field == 1 ? groups
                                : field == 2 ? blocks
                                : field == 3 ? longs
                                : field == 4 ? mids
                                             : lanes;
            const int nc = field == 3 ? 6 : field == 4 ? 5 : field == 5 ? 3 : 4;
            for (int c = 0; c < nc; ++c) {
                pvvc_tune t = cur;
                int32_t* f = field == 0 ? &t.group_ctas_per_sm
                           : field == 1 ? &t.min_group
                           : field == 2 ? &t.rlgr_block
                           : field == 3 ? &t.rlgr_long_ctas
                           : field == 4 ? &t.rlgr_mid_pct
                                        : &t.rlgr_long_lanes;
                if (*f == cand[c]) continue;
                *f = cand[c];
                pvvc_plan pl;
                if ((rc = build_plan(desc, &pl, &t, nullptr))) return rc;
                const float ms = time_plan(&pl, st, payload, dx, dr, ds, ws, reps, s);
                if (ms < 0) return PVVC_ERR_CUDA;
                if (ms < cur_ms * 0.99f) {
                    cur = t;
                    cur_ms = ms;
                    moved = true;
                }
            }
        }
        if (!moved) break;
    }
    *best = cur;
    if (best_ms) *best_ms = cur_ms;
    return PVVC_OK;
}

struct pvvc_graph {
    cudaGraph_t graph = nullptr;
    cudaGraphExec_t exec = nullptr;
};

extern "C" int pvvc_graph_create(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                                 float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, pvvc_graph** out) {
    if (!out || !plan || !st) return PVVC_ERR_ARG;
    *out = nullptr;
    if (prepare_kernels() != cudaSuccess) return PVVC_ERR_CUDA;
    cudaStream_t cs;
    if (cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking) != cudaSuccess) return PVVC_ERR_CUDA;
    auto g = std::make_unique<pvvc_graph>();
    int rc = PVVC_OK;
    if (cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal) != cudaSuccess) {
        rc = PVVC_ERR_CUDA;
    } else {
        rc = run_decode(plan, st, payload, xyz, rgb, points24, status, workspace, workspace_bytes, cs, nullptr);
        cudaGraph_t gr = nullptr;
        const cudaError_t e = cudaStreamEndCapture(cs, &gr);  // ends the capture on every path
        g->graph = gr;
        if (rc == PVVC_OK && (e != cudaSuccess || !gr)) rc = PVVC_ERR_CUDA;
    }
    if (rc == PVVC_OK && cudaGraphInstantiate(&g->exec, g->graph, 0) != cudaSuccess) rc = PVVC_ERR_CUDA;
    cudaStreamDestroy(cs);
    if (rc) {
        pvvc_graph_destroy(g.release());
        return rc;
    }
    *out = g.release();
    return PVVC_OK;
}

extern "C" int pvvc_graph_launch(pvvc_graph* g, void* stream) {
    if (!g || !g->exec) return PVVC_ERR_ARG;
    return cudaGraphLaunch(g->exec, (cudaStream_t)stream) == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_graph_destroy(pvvc_graph* g) {
    if (!g) return PVVC_ERR_ARG;
    if (g->exec) cudaGraphExecDestroy(g->exec);
    if (g->graph) cudaGraphDestroy(g->graph);
    delete g;
    return PVVC_OK;
}

extern "C" int pvvc_plan_destroy(pvvc_plan* p) {
    if (!p) return PVVC_ERR_ARG;
    delete p;
    return PVVC_OK;
}

extern "C" int pvvc_plan_host_times(const pvvc_plan* p, double* out, int32_t n) {
    if (!p || !out || n < 0) return PVVC_ERR_ARG;
    for (int k = 0; k < n && k < 5; ++k) out[k] = p->host_ms[k];
    return PVVC_OK;
}

extern "C" int pvvc_plan_query(const pvvc_plan* p, uint64_t* total_points, uint64_t* workspace_bytes) {
    if (!p) return PVVC_ERR_ARG;
    if (total_points) *total_points = p->total_points;
    if (workspace_bytes) *workspace_bytes = p->ws_bytes;
    return PVVC_OK;
}

extern "C" int pvvc_decode(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                           float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, void* stream) {
    return run_decode(plan, st, payload, xyz, rgb, points24, status, workspace, workspace_bytes, (cudaStream_t)stream,
                      nullptr);
}

extern "C" int pvvc_decode_profiled(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                                    float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, void* stream,
                                    void* const* events) {
    if (!events) return PVVC_ERR_ARG;
    return run_decode(plan, st, payload, xyz, rgb, points24, status, workspace, workspace_bytes, (cudaStream_t)stream, events);
}


namespace {
constexpr int kStages = 22;
thread_local double g_stage_ms[kStages] = {};  // see pvvc_host_stage_times

// A zstd payload of a parsed frame, left compressed for the GPU.
struct ZJob {
    int32_t slice;       // within its frame
    int32_t which;       // 0 geometry, 1 colour
    const uint8_t* src;  // the compressed bytes (in the caller's frame)
    uint32_t len;
    uint64_t zoff;       // staging offset in the packed payload
};

// Replaces each zstd payload of `f` by a job: its size becomes the first
// frame's declared content size, which the reference's ZstdDecoder sizes its
// output by and requires to be known and non-zero (entropy_codec.cc:343-347),
// its bytes are dropped from the view, and the type's zstd bits cleared.
int frame_view_zstd_jobs(FrameView* f, std::vector<ZJob>* jobs) {
    for (size_t i = 0; i < f->count(); ++i) {
        for (int which = 0; which < 2; ++which) {
            const uint8_t bit = which ? (uint8_t)PVVC_TYPE_COLOR_ZSTD : (uint8_t)PVVC_TYPE_GEO_ZSTD;
            const uint8_t*& at = which ? f->col[i] : f->geo[i];
            uint32_t& sz = which ? f->csz[i] : f->gsz[i];
            if (!(f->type[i] & bit) || !sz) continue;
            uint64_t raw = 0;
            if (!pvvc_zstd::content_size(at, sz, &raw) || raw == 0 || raw == pvvc_zstd::kUnknown || raw > 0xFFFFFFFFull)
                return PVVC_ERR_ZSTD;
            jobs->push_back(ZJob{(int32_t)i, which, at, sz, 0});
            at = nullptr;
            sz = (uint32_t)raw;
        }
        f->type[i] &= (uint8_t)~(PVVC_TYPE_GEO_ZSTD | PVVC_TYPE_COLOR_ZSTD);
    }
    return PVVC_OK;
}
struct StageClock {
    std::chrono::steady_clock::time_point t = std::chrono::steady_clock::now();
    double lap() {  // ms since the previous lap
        const auto now = std::chrono::steady_clock::now();
        const double ms = std::chrono::duration<double, std::milli>(now - t).count();
        t = now;
        return ms;
    }
};
}  // namespace

extern "C" int pvvc_host_stage_times(double* out, int32_t n) {
    if (!out || n < 0) return PVVC_ERR_ARG;
    for (int i = 0; i < n && i < kStages; ++i) out[i] = g_stage_ms[i];
    return PVVC_OK;
}

extern "C" int pvvc_decode_frames_host(pvvc_state* st, int32_t nframes, const uint8_t* const* frame_bytes,
                                       const uint64_t* frame_len, float* xyz_host, uint8_t* rgb_host, uint64_t cap_points,
                                       uint64_t* npoints_out, int32_t* status_host, int32_t status_cap, void* stream) {
    if (!st || nframes < 0 || (nframes && (!frame_bytes || !frame_len))) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    const int threads = host_threads();
    StageClock clk;
    for (double& v : g_stage_ms) v = 0;
    // device timeline of the parts (pvvc_host_stage_times out[13..21])
    if (!st->t_start) {
        bool ok = cudaEventCreate(&st->t_start) == cudaSuccess;
        for (int h = 0; ok && h < pvvc_state::kParts; ++h)
            ok = cudaEventCreate(&st->t_up[h]) == cudaSuccess && cudaEventCreate(&st->t_dec[h]) == cudaSuccess &&
                 cudaEventCreate(&st->t_cp[h]) == cudaSuccess;
        if (!ok) return PVVC_ERR_CUDA;
    }
    if (cudaEventRecord(st->t_start, s) != cudaSuccess) return PVVC_ERR_CUDA;
    // parse (io::LoadFrame), frames in parallel; the payloads stay in the
    // caller's bytes until they are packed, and zstd payloads stay compressed:
    // the GPU inflates them in place of the loader's host zstd stage
    // (slice_io.cu:233-265)
    std::vector<FrameView> frames(nframes);
    std::vector<std::vector<ZJob>> fz(nframes);
    std::vector<int> prc(nframes, PVVC_OK);
    parallel_for(nframes, threads, [&](int f) {
        prc[f] = parse_frame_view(frame_bytes[f], frame_len[f], &frames[f]);
        if (!prc[f]) prc[f] = frame_view_zstd_jobs(&frames[f], &fz[f]);
    });
    for (int r : prc)
        if (r) return r;
    g_stage_ms[0] = clk.lap();
    // payload layout (4-byte aligned) and the batch description, in frame order
    uint64_t bytes = 0, pts = 0;
    int32_t nsl = 0;
    std::vector<int32_t> ffirst(nframes + 1, 0);
    for (int f = 0; f < nframes; ++f) {
        ffirst[f] = nsl;
        nsl += (int32_t)frames[f].count();
    }
    ffirst[nframes] = nsl;
    // the call's description arrays, carved from one grow-only page-locked
    // buffer that the state keeps (a fresh allocation of this size would come
    // from new pages each call, and their first-touch faults cost
    // milliseconds; page-locked, a reused plan's per-call fields go to the
    // device straight from here)
    int32_t *slot, *index;
    uint8_t *type, *qp;
    uint32_t *size, *gsz, *csz;
    float* mv;
    uint64_t *goff, *coff, *oo;
    {
        const size_t n = (size_t)std::max(nsl, 1);
        uint64_t at[11], o = 0;
        const size_t bytes[11] = {4 * n, 4 * n, n, n, 4 * n, 4 * n, 4 * n, 64 * n, 8 * n, 8 * n, 8 * n};
        for (int i = 0; i < 11; ++i) {
            at[i] = o;
            o = align_up(o + bytes[i], 64);
        }
        if (st->host_desc.ensure(o) != cudaSuccess) return PVVC_ERR_NOMEM;
        unsigned char* b = static_cast<unsigned char*>(st->host_desc.p);
        slot = reinterpret_cast<int32_t*>(b + at[0]);
        index = reinterpret_cast<int32_t*>(b + at[1]);
        type = b + at[2];
        qp = b + at[3];
        size = reinterpret_cast<uint32_t*>(b + at[4]);
        gsz = reinterpret_cast<uint32_t*>(b + at[5]);
        csz = reinterpret_cast<uint32_t*>(b + at[6]);
        mv = reinterpret_cast<float*>(b + at[7]);
        goff = reinterpret_cast<uint64_t*>(b + at[8]);
        coff = reinterpret_cast<uint64_t*>(b + at[9]);
        oo = reinterpret_cast<uint64_t*>(b + at[10]);
    }
    // The description in two passes: the patch indices and types (all that
    // splitting the call into runs and parts needs) and each frame's payload
    // bytes and points first, for every frame; the rest -- sizes, steps,
    // motions and payload offsets -- per frame range, so that a call decoded
    // in parts describes part 0 first and starts on it while the other parts
    // are described and planned on other threads.
    std::vector<uint64_t> fbytes(nframes + 1, 0);  // payload bytes before each frame
    std::vector<uint64_t> fpts(nframes + 1, 0);    // points before each frame
    parallel_for(nframes, threads, [&](int f) {
        const FrameView& fr = frames[f];
        uint64_t b = 0, q = 0;
        for (size_t i = 0; i < fr.count(); ++i) {
            const int32_t k = ffirst[f] + (int32_t)i;
            index[k] = fr.index[i];
            type[k] = fr.type[i];
            b += align_up(fr.gsz[i], 4) + align_up(fr.csz[i], 4);
            q += fr.size[i];
        }
        fbytes[f + 1] = b;
        fpts[f + 1] = q;
    });
    for (int f = 0; f < nframes; ++f) {
        fbytes[f + 1] += fbytes[f];
        fpts[f + 1] += fpts[f];
    }
    bytes = fbytes[nframes];
    pts = fpts[nframes];
    auto describe = [&](int f0, int f1, int nthreads) {  // frames [f0, f1)
        parallel_for(f1 - f0, nthreads, [&](int q0) {
            const int f = f0 + q0;
            const FrameView& fr = frames[f];
            uint64_t b = fbytes[f], q = fpts[f];
            for (size_t i = 0; i < fr.count(); ++i) {
                const int32_t k = ffirst[f] + (int32_t)i;
                qp[k] = fr.qp[i];
                size[k] = fr.size[i];
                std::memcpy(&mv[16ull * k], &fr.mv[16 * i], 64);
                gsz[k] = fr.gsz[i];
                csz[k] = fr.csz[i];
                goff[k] = b;
                b = align_up(b + gsz[k], 4);
                coff[k] = b;
                b = align_up(b + csz[k], 4);
                oo[k] = q;
                q += size[k];
            }
        });
    };
    if (npoints_out) *npoints_out = pts;
    if (pts > cap_points || (status_host && status_cap < nsl)) return PVVC_ERR_CAPACITY;
    // zstd staging after the raw region: the compressed payloads, then the
    // job arrays (source offset, raw offset, source length, raw size, slice)
    // and a status per job, all carried by the one host-to-device copy
    int32_t nz = 0;
    uint64_t zend = align_up(bytes + 16, 16);
    for (int f = 0; f < nframes; ++f)
        for (ZJob& j : fz[f]) {
            j.zoff = zend;
            zend += j.len;
            ++nz;
        }
    const uint64_t a_src_off = align_up(zend, 16), a_dst_off = a_src_off + 8ull * nz, a_src_len = a_dst_off + 8ull * nz,
                   a_cap = a_src_len + 4ull * nz, a_slice = a_cap + 4ull * nz, a_status = a_slice + 4ull * nz;
    const uint64_t total = nz ? a_status + 4ull * nz : bytes;
    if (st->h_payload.ensure(total + 16) != cudaSuccess) return PVVC_ERR_NOMEM;
    uint8_t* hp = static_cast<uint8_t*>(st->h_payload.p);
    std::memset(hp + bytes, 0, 16);  // the decoder reads whole 16-byte blocks
    bool described = false;  // every frame's full description written
    if (nz) {
        describe(0, nframes, threads);
        described = true;
        uint64_t* zs = reinterpret_cast<uint64_t*>(hp + a_src_off);
        uint64_t* zd = reinterpret_cast<uint64_t*>(hp + a_dst_off);
        uint32_t* zl = reinterpret_cast<uint32_t*>(hp + a_src_len);
        uint32_t* zc = reinterpret_cast<uint32_t*>(hp + a_cap);
        int32_t* zk = reinterpret_cast<int32_t*>(hp + a_slice);
        int32_t q = 0;
        for (int f = 0; f < nframes; ++f)
            for (const ZJob& j : fz[f]) {
                const int32_t k = ffirst[f] + j.slice;
                zs[q] = j.zoff;
                zl[q] = j.len;
                zd[q] = j.which ? coff[k] : goff[k];
                zc[q] = j.which ? csz[k] : gsz[k];
                zk[q] = k;
                ++q;
            }
    }
    if (st->payload.ensure(total + 16) != cudaSuccess) return PVVC_ERR_NOMEM;
    if (st->xyz.ensure(std::max<uint64_t>(12 * pts, 4)) != cudaSuccess) return PVVC_ERR_NOMEM;
    if (st->rgb.ensure(std::max<uint64_t>(3 * pts, 4)) != cudaSuccess) return PVVC_ERR_NOMEM;
    if (st->status.ensure(std::max<uint64_t>(4ull * nsl, 4)) != cudaSuccess) return PVVC_ERR_NOMEM;
    // Intra slices of different frames of one call may hit the same patch
    // index (a new GoP).  Split the call into runs of frames without a
    // repeated intra index.
    const int32_t nslots = st->v.nslots;
    std::vector<int32_t> bounds{0};  // first slice of each run
    {
        std::vector<uint8_t> seen(std::max(nslots, 1), 0);
        for (int f = 0; f < nframes; ++f) {
            bool clash = false;
            for (int32_t k = ffirst[f]; k < ffirst[f + 1]; ++k)
                if (!(type[k] & PVVC_TYPE_PREDICT) && index[k] >= 0 && index[k] < nslots && seen[index[k]]) clash = true;
            if (clash) {
                bounds.push_back(ffirst[f]);
                std::fill(seen.begin(), seen.end(), 0);
            }
            for (int32_t k = ffirst[f]; k < ffirst[f + 1]; ++k)
                if (index[k] >= 0 && index[k] < nslots) seen[index[k]] = 1;
        }
        bounds.push_back(nsl);
    }
    const int nruns = (int)bounds.size() - 1;
    // All runs in one decode: each intra slice but an index's last one in
    // the call writes a slot region of its own (run r of R -> region R-1-r
    // of `stride` slots), predictive slices read the region of their index's
    // latest intra slice, and every index ends in its own slot (region 0), as
    // run-by-run decoding leaves it.  This needs every predictive slice's
    // intra slice inside the call and R regions of slots in the state.
    int32_t stride = 0;
    for (int32_t k = 0; k < nsl; ++k) stride = std::max(stride, index[k] + 1);
    bool merge = nruns > 1 && stride > 0 && (int64_t)nruns * stride <= nslots;
    if (merge) {
        std::vector<int32_t> region(stride, -1);  // region of each index's latest intra slice
        std::vector<int32_t> last_run(stride, -1);
        for (int r = 0; r < nruns; ++r)
            for (int32_t k = bounds[r]; k < bounds[r + 1]; ++k)
                if (index[k] >= 0 && !(type[k] & PVVC_TYPE_PREDICT)) last_run[index[k]] = r;
        for (int r = 0; r < nruns && merge; ++r)
            for (int32_t k = bounds[r]; k < bounds[r + 1]; ++k) {
                const int32_t i = index[k];
                if (i < 0) {
                    slot[k] = i;  // rejected by the plan as before
                    continue;
                }
                if (!(type[k] & PVVC_TYPE_PREDICT)) region[i] = last_run[i] == r ? 0 : nruns - 1 - r;
                if (region[i] < 0) {  // predictive before any intra of its index in this call
                    merge = false;
                    break;
                }
                slot[k] = region[i] * stride + i;
            }
    }
    if (!merge)
        for (int32_t k = 0; k < nsl; ++k) slot[k] = index[k];
    // A merged call of several GoPs is decoded in parts, split at run (GoP)
    // boundaries near equal slice counts: each part has its own plan, and a
    // part's xyz/rgb go back to the host on a second stream while the host
    // plans and the GPU decodes the next part.  The device-to-host copy runs
    // at the host link's rate and is the longest stage, so starting it early
    // shortens the call.
    std::vector<int32_t> cuts{0};
    if (merge && nruns >= 2 && (xyz_host || rgb_host)) {
        const int parts = std::min(nruns, (int)pvvc_state::kParts);
        for (int q = 1; q < parts; ++q) {  // the run boundary nearest the q-th cut fraction of the slices
            const double at = parts == pvvc_state::kParts ? pvvc_state::kCutAt[q - 1] : (double)q / parts;
            int32_t best = -1;
            for (int r = 1; r < nruns; ++r)
                if (bounds[r] > cuts.back() && (best < 0 || std::fabs(bounds[r] - at * nsl) < std::fabs(best - at * nsl)))
                    best = bounds[r];
            if (best > cuts.back() && best < nsl) cuts.push_back(best);
        }
        cuts.push_back(nsl);
        if (!st->copy && cudaStreamCreateWithFlags(&st->copy, cudaStreamNonBlocking) != cudaSuccess) return PVVC_ERR_CUDA;
        for (cudaEvent_t& e : st->part_done)
            if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return PVVC_ERR_CUDA;
    }
    const int nparts = (int)cuts.size() - 1;  // 0: not split
    // zstd jobs of each part: jobs are in slice order, so a part's jobs are
    // the contiguous range of those whose slice lies in it
    std::vector<int32_t> zcut(std::max(nparts, 1) + 1, 0);
    if (nparts > 0 && nz) {
        const int32_t* zk = reinterpret_cast<const int32_t*>(hp + a_slice);
        for (int h = 1; h < nparts; ++h)
            zcut[h] = (int32_t)(std::lower_bound(zk, zk + nz, cuts[h]) - zk);
        zcut[nparts] = nz;
        if (!st->zside && cudaStreamCreateWithFlags(&st->zside, cudaStreamNonBlocking) != cudaSuccess) return PVVC_ERR_CUDA;
        for (cudaEvent_t& e : st->zdone)
            if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return PVVC_ERR_CUDA;
    }
    // The payload bytes go into pinned memory on helper threads while this
    // thread splits the call into runs and plans.  As soon as they are
    // packed, the packer thread queues their copy to the device and the zstd
    // inflation on `s`, so both run on the GPU during planning; the decode
    // is queued after the packer has finished.
    bool sent_ok = true;
    // Raw payloads of a call decoded in parts go up part by part: the packer
    // packs a part's frames into pinned memory and counts it in `packed`;
    // the main thread queues the part's copy on the upload stream right
    // before the part's decode, so part 0's decode starts while the later
    // parts are still being packed.
    const bool by_part = nz == 0 && nparts >= 2 && bytes > 0;
    std::vector<int> fcut;
    std::mutex pk_mu;
    std::condition_variable pk_cv;
    int packed = 0;  // parts whose copy (and event) is queued
    std::vector<char> part_described(std::max(nparts, 1), 0);  // by part: each part's frames described
    if (!by_part && !described) {
        describe(0, nframes, threads);
        described = true;
    }
    if (by_part) {
        if (!st->up && cudaStreamCreateWithFlags(&st->up, cudaStreamNonBlocking) != cudaSuccess) return PVVC_ERR_CUDA;
        for (cudaEvent_t& e : st->up_done)
            if (!e && cudaEventCreateWithFlags(&e, cudaEventDisableTiming) != cudaSuccess) return PVVC_ERR_CUDA;
        for (int h = 0; h <= nparts; ++h)  // every cut is the first slice of a frame
            fcut.push_back((int)(std::lower_bound(ffirst.begin(), ffirst.end(), cuts[h]) - ffirst.begin()));
        // part 0 is on the critical path: described here with every thread,
        // before the packer and the other parts' planners start
        describe(fcut[0], fcut[1], threads);
        part_described[0] = 1;
    }
    std::thread packer([&] {
        if (by_part) {
            for (int h = 0; h < nparts; ++h) {
                const int f0 = fcut[h], f1 = fcut[h + 1];
                {  // the part's payload offsets are written by its planner
                    std::unique_lock<std::mutex> g(pk_mu);
                    pk_cv.wait(g, [&] { return part_described[h] != 0; });
                }
                parallel_for(f1 - f0, threads, [&](int q) {
                    const int f = f0 + q;
                    FrameView& fr = frames[f];
                    for (size_t i = 0; i < fr.count(); ++i) {
                        const int32_t k = ffirst[f] + (int32_t)i;
                        if (gsz[k] && fr.geo[i]) std::memcpy(hp + goff[k], fr.geo[i], gsz[k]);
                        if (csz[k] && fr.col[i]) std::memcpy(hp + coff[k], fr.col[i], csz[k]);
                    }
                });
                std::lock_guard<std::mutex> g(pk_mu);
                packed = h + 1;
                pk_cv.notify_all();
            }
            return;
        }
        parallel_for(nframes, std::max(1, threads / 2), [&](int f) {
            FrameView& fr = frames[f];
            for (size_t i = 0; i < fr.count(); ++i) {
                const int32_t k = ffirst[f] + (int32_t)i;
                if (gsz[k] && fr.geo[i]) std::memcpy(hp + goff[k], fr.geo[i], gsz[k]);
                if (csz[k] && fr.col[i]) std::memcpy(hp + coff[k], fr.col[i], csz[k]);
            }
            for (const ZJob& j : fz[f]) std::memcpy(hp + j.zoff, j.src, j.len);
        });
        if (bytes && cudaMemcpyAsync(st->payload.p, hp, total + 16, cudaMemcpyHostToDevice, s) != cudaSuccess) {
            sent_ok = false;
            return;
        }
        if (!nz) return;
        uint8_t* dp = static_cast<uint8_t*>(st->payload.p);
        auto inflate = [&](int32_t j0, int32_t j1, cudaStream_t on) {  // jobs [j0, j1)
            return pvvc_zstd_launch(j1 - j0, dp, reinterpret_cast<const uint64_t*>(dp + a_src_off) + j0,
                                    reinterpret_cast<const uint32_t*>(dp + a_src_len) + j0, dp,
                                    reinterpret_cast<const uint64_t*>(dp + a_dst_off) + j0,
                                    reinterpret_cast<const uint32_t*>(dp + a_cap) + j0, nullptr,
                                    reinterpret_cast<int32_t*>(dp + a_status) + j0, on) == PVVC_OK;
        };
        if (nparts < 2) {
            sent_ok = inflate(0, nz, s);
            return;
        }
        // the first part's payloads on `s`, before its decode; the others on
        // a side stream, each part's decode waiting for its own event
        sent_ok = inflate(zcut[0], zcut[1], s) && cudaEventRecord(st->zdone[0], s) == cudaSuccess &&
                  cudaStreamWaitEvent(st->zside, st->zdone[0], 0) == cudaSuccess;
        for (int h = 1; h < nparts && sent_ok; ++h)
            sent_ok = inflate(zcut[h], zcut[h + 1], st->zside) && cudaEventRecord(st->zdone[h], st->zside) == cudaSuccess;
    });
    struct JoinOnExit {
        std::thread& t;
        ~JoinOnExit() {
            if (t.joinable()) t.join();
        }
    } join_packer{packer};
    auto payload_queued = [&]() -> bool {  // the copy (and inflation) queued before the first decode
        if (packer.joinable()) packer.join();
        return sent_ok;
    };
    g_stage_ms[1] = clk.lap();
    // the decode writes device buffers; each part's points go back to the host
    // with a copy as soon as the part is decoded.  (Decode kernels writing
    // page-locked host memory straight over the link were measured slower:
    // their stores reach the host as partial lines.)
    float* out_xyz = static_cast<float*>(st->xyz.p);
    uint8_t* out_rgb = static_cast<uint8_t*>(st->rgb.p);
    // The parts' plans are built at once: part 0 on this thread, the others
    // on worker threads (each with its share of the host threads), and each
    // part's decode is queued as soon as its plan is ready.
    std::vector<int> plan_rc(std::max(nparts, 1), PVVC_OK);
    auto plan_part = [&](int h, int nthreads) {
        if (by_part && h > 0) {  // describe the part's frames first (the packer waits for them)
            describe(fcut[h], fcut[h + 1], nthreads);
            std::lock_guard<std::mutex> g(pk_mu);
            part_described[h] = 1;
            pk_cv.notify_all();
        }
        g_plan_threads = nthreads;
        const int32_t first = cuts[h], cnt = cuts[h + 1] - first;
        pvvc_plan* pl = h ? &st->part_plan[h - 1] : &st->plan;
        pvvc_batch_desc d{cnt,          slot + first, type + first, size + first, qp + first, mv + 16ull * first,
                          goff + first, gsz + first, coff + first, csz + first, oo + first};
        plan_rc[h] = build_plan(&d, pl, nullptr, s, true);  // copies queued by this thread below
        g_plan_threads = 0;
    };
    std::vector<std::thread> planners;
    struct JoinAll {
        std::vector<std::thread>& v;
        ~JoinAll() {
            for (auto& t : v)
                if (t.joinable()) t.join();
        }
    } join_planners{planners};
    const int share = std::max(1, threads / std::max(nparts, 1));
    for (int h = 1; h < nparts; ++h) planners.emplace_back(plan_part, h, share);
    if (nparts > 0) plan_part(0, share);
    int rc = PVVC_OK;
    for (int h = 0; h < nparts && rc == PVVC_OK; ++h) {
        const int32_t first = cuts[h], cnt = cuts[h + 1] - first;
        pvvc_plan* pl = h ? &st->part_plan[h - 1] : &st->plan;
        if (h > 0) planners[h - 1].join();
        rc = plan_rc[h];
        if (rc) break;
        for (int k = 0; k < 5; ++k) g_stage_ms[8 + k] += pl->host_ms[k];
        g_stage_ms[2] += clk.lap();
        if (st->ws.ensure(pl->ws_bytes) != cudaSuccess) return PVVC_ERR_NOMEM;
        if (upload_plan(pl, s) != PVVC_OK) return PVVC_ERR_CUDA;
        g_stage_ms[5] += clk.lap();
        if (by_part) {
            {
                std::unique_lock<std::mutex> g(pk_mu);
                pk_cv.wait(g, [&] { return packed > h; });
            }
            // this thread queues the part's upload (one thread makes every CUDA call of the call)
            const int f0 = fcut[h], f1 = fcut[h + 1];
            const uint64_t a = fbytes[f0], e = h + 1 == nparts ? bytes + 16 : fbytes[f1];
            if (e > a && (cudaMemcpyAsync(static_cast<uint8_t*>(st->payload.p) + a, hp + a, e - a, cudaMemcpyHostToDevice,
                                          st->up) != cudaSuccess ||
                          cudaEventRecord(st->up_done[h], st->up) != cudaSuccess ||
                          cudaEventRecord(st->t_up[h], st->up) != cudaSuccess ||
                          cudaStreamWaitEvent(s, st->up_done[h], 0) != cudaSuccess))
                return PVVC_ERR_CUDA;
        } else if (!payload_queued()) {
            return PVVC_ERR_CUDA;
        }
        if (h > 0 && nz && cudaStreamWaitEvent(s, st->zdone[h], 0) != cudaSuccess) return PVVC_ERR_CUDA;
        g_stage_ms[4] += clk.lap();
        rc = run_decode(pl, st, static_cast<const uint8_t*>(st->payload.p), out_xyz, out_rgb, nullptr,
                        static_cast<int32_t*>(st->status.p) + first, st->ws.p, st->ws.cap, s, nullptr);
        if (rc) break;
        g_stage_ms[6] += clk.lap();
        // this part's points: [oo[first], end of its last slice), contiguous in frame order
        const uint64_t p0 = oo[first], p1 = oo[first + cnt - 1] + size[first + cnt - 1];
        if (cudaEventRecord(st->part_done[h], s) != cudaSuccess || cudaEventRecord(st->t_dec[h], s) != cudaSuccess ||
            cudaStreamWaitEvent(st->copy, st->part_done[h], 0) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (xyz_host && p1 > p0 &&
            cudaMemcpyAsync(xyz_host + 3 * p0, static_cast<float*>(st->xyz.p) + 3 * p0, 12 * (p1 - p0), cudaMemcpyDeviceToHost,
                            st->copy) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (rgb_host && p1 > p0 &&
            cudaMemcpyAsync(rgb_host + 3 * p0, static_cast<uint8_t*>(st->rgb.p) + 3 * p0, 3 * (p1 - p0), cudaMemcpyDeviceToHost,
                            st->copy) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (cudaEventRecord(st->t_cp[h], st->copy) != cudaSuccess) return PVVC_ERR_CUDA;
        g_stage_ms[7] += clk.lap();
    }
    if (rc) return rc;
    const int32_t split = nparts > 0 ? 1 : 0;
    const std::vector<int32_t> one_run{0, nsl};
    const std::vector<int32_t> no_runs{0};
    const std::vector<int32_t>& runs = split > 0 ? no_runs : merge ? one_run : bounds;
    for (size_t b = 0; b + 1 < runs.size() && rc == PVVC_OK; ++b) {
        const int32_t first = runs[b], cnt = runs[b + 1] - first;
        if (cnt <= 0) continue;
        pvvc_batch_desc d{cnt,          slot + first, type + first, size + first, qp + first, mv + 16ull * first,
                          goff + first, gsz + first, coff + first, csz + first, oo + first};
        // the plan's arrays go up on `s` from pinned mirrors that stay as
        // they are until the next plan, which follows a synchronisation
        rc = build_plan(&d, &st->plan, nullptr, s);
        if (rc) break;
        if (st->ws.ensure(st->plan.ws_bytes) != cudaSuccess) return PVVC_ERR_NOMEM;
        if (!payload_queued()) return PVVC_ERR_CUDA;
        g_stage_ms[2] += clk.lap();
        rc = run_decode(&st->plan, st, static_cast<const uint8_t*>(st->payload.p), out_xyz, out_rgb, nullptr,
                        static_cast<int32_t*>(st->status.p) + first, st->ws.p, st->ws.cap, s, nullptr);
        // the plan's host arrays are rebuilt by the next run: finish this one first
        if (rc == PVVC_OK && runs.size() > 2 && cudaStreamSynchronize(s) != cudaSuccess) rc = PVVC_ERR_CUDA;
        g_stage_ms[3] += clk.lap();
    }
    if (rc) return rc;
    // a payload that did not inflate marks its slice (the call fails below)
    if (nz && pvvc_zstd_merge_status(nz, reinterpret_cast<const int32_t*>(static_cast<uint8_t*>(st->payload.p) + a_status),
                                     reinterpret_cast<const int32_t*>(static_cast<uint8_t*>(st->payload.p) + a_slice),
                                     static_cast<int32_t*>(st->status.p), s) != PVVC_OK)
        return PVVC_ERR_CUDA;
    if (split <= 0) {
        if (xyz_host && pts && cudaMemcpyAsync(xyz_host, st->xyz.p, 12 * pts, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        if (rgb_host && pts && cudaMemcpyAsync(rgb_host, st->rgb.p, 3 * pts, cudaMemcpyDeviceToHost, s) != cudaSuccess)
            return PVVC_ERR_CUDA;
    }
    if (status_host && nsl && cudaMemcpyAsync(status_host, st->status.p, 4ull * nsl, cudaMemcpyDeviceToHost, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    std::vector<int32_t> zst(nz);
    if (nz && cudaMemcpyAsync(zst.data(), static_cast<uint8_t*>(st->payload.p) + a_status, 4ull * nz, cudaMemcpyDeviceToHost,
                              s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PVVC_ERR_CUDA;
    if (split > 0 && cudaStreamSynchronize(st->copy) != cudaSuccess) return PVVC_ERR_CUDA;
    g_stage_ms[3] += clk.lap();
    for (int h = 0; h < nparts && h < pvvc_state::kParts; ++h) {  // the parts' device timeline
        float ms = 0.f;
        if (by_part && cudaEventElapsedTime(&ms, st->t_start, st->t_up[h]) == cudaSuccess) g_stage_ms[13 + 3 * h] = ms;
        if (cudaEventElapsedTime(&ms, st->t_start, st->t_dec[h]) == cudaSuccess) g_stage_ms[14 + 3 * h] = ms;
        if (cudaEventElapsedTime(&ms, st->t_start, st->t_cp[h]) == cudaSuccess) g_stage_ms[15 + 3 * h] = ms;
    }
    cudaGetLastError();  // a part without a timing event leaves no error behind
    for (int32_t z : zst)  // the reference throws on a payload libzstd cannot inflate
        if (z != PVVC_OK) return PVVC_ERR_ZSTD;
    return PVVC_OK;
}

extern "C" int pvvc_launch_cudaProcess(int grid, int block, float* out_points24, int timestamp, int* inner_offset, int* index,
                                       uint8_t* type, float** mv, uint32_t* size, uint8_t* qp, uint8_t** geometry,
                                       uint32_t* geometry_size, uint8_t** color, uint32_t* color_size, pvvc_state* decoders,
                                       int patch_size, void* stream) {
    (void)grid;
    (void)block;
    (void)timestamp;
    if (!decoders || patch_size < 0 || !out_points24) return PVVC_ERR_ARG;
    if (patch_size == 0) return PVVC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    const int n = patch_size;
    std::vector<int> h_off(n), h_idx(n);
    std::vector<uint8_t> h_type(n), h_qp(n);
    std::vector<uint32_t> h_size(n), h_gsz(n), h_csz(n);
    std::vector<float*> h_mv(n);
    std::vector<uint8_t*> h_geo(n), h_col(n);
    auto d2h = [&](void* dst, const void* src, size_t b) {
        return cudaMemcpyAsync(dst, src, b, cudaMemcpyDeviceToHost, s) == cudaSuccess;
    };
    if (!d2h(h_off.data(), inner_offset, 4ull * n) || !d2h(h_idx.data(), index, 4ull * n) || !d2h(h_type.data(), type, n) ||
        !d2h(h_qp.data(), qp, n) || !d2h(h_size.data(), size, 4ull * n) || !d2h(h_gsz.data(), geometry_size, 4ull * n) ||
        !d2h(h_csz.data(), color_size, 4ull * n) || !d2h(h_mv.data(), mv, sizeof(float*) * n) ||
        !d2h(h_geo.data(), geometry, sizeof(uint8_t*) * n) || !d2h(h_col.data(), color, sizeof(uint8_t*) * n))
        return PVVC_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PVVC_ERR_CUDA;
    std::vector<float> h_m(16ull * n);
    for (int i = 0; i < n; ++i)
        if (!d2h(&h_m[16ull * i], h_mv[i], 64)) return PVVC_ERR_CUDA;
    if (cudaStreamSynchronize(s) != cudaSuccess) return PVVC_ERR_CUDA;
    // payload base: the lowest payload pointer; offsets are address differences
    uintptr_t base = UINTPTR_MAX;
    for (int i = 0; i < n; ++i) {
        if (h_gsz[i] && h_geo[i]) base = std::min(base, reinterpret_cast<uintptr_t>(h_geo[i]));
        if (h_csz[i] && h_col[i]) base = std::min(base, reinterpret_cast<uintptr_t>(h_col[i]));
    }
    if (base == UINTPTR_MAX) return PVVC_ERR_ARG;
    base &= ~uintptr_t(15);
    std::vector<int32_t> slot(n);
    std::vector<uint64_t> goff(n), coff(n), oo(n);
    for (int i = 0; i < n; ++i) {
        slot[i] = h_idx[i];
        goff[i] = h_gsz[i] ? reinterpret_cast<uintptr_t>(h_geo[i]) - base : 0;
        coff[i] = h_csz[i] ? reinterpret_cast<uintptr_t>(h_col[i]) - base : 0;
        oo[i] = (uint64_t)h_off[i];
    }
    pvvc_batch_desc d{n, slot.data(), h_type.data(), h_size.data(), h_qp.data(), h_m.data(), goff.data(), h_gsz.data(),
                      coff.data(), h_csz.data(), oo.data()};
    int rc = build_plan(&d, &decoders->plan, nullptr, nullptr);
    if (rc) return rc;
    if (decoders->ws.ensure(decoders->plan.ws_bytes) != cudaSuccess) return PVVC_ERR_NOMEM;
    rc = run_decode(&decoders->plan, decoders, reinterpret_cast<const uint8_t*>(base), nullptr, nullptr, out_points24, nullptr,
                    decoders->ws.p, decoders->ws.cap, s, nullptr);
    if (rc) return rc;
    return cudaStreamSynchronize(s) == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}
