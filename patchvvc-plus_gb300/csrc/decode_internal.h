// decode_internal.h -- host-side internals of the decode path shared by the
// C ABI (decode_api.cu) and the serving runtime (serve.cu): plan and state
// objects, grow-only buffers, the planner and the stream-ordered decode.
#pragma once

#include <cuda_runtime.h>

#include <cstdint>
#include <memory>
#include <new>
#include <vector>

#include "decode_types.h"
#include "pvvc_gb300.h"

// zstd_kernels.cu: pvvc_zstd_inflate_batch without the argument checks
int pvvc_zstd_launch(int32_t njobs, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len, uint8_t* dst,
                     const uint64_t* dst_off, const uint32_t* dst_cap, uint32_t* out_len, int32_t* status, cudaStream_t s);
// status[zslice[j]] = PVVC_ERR_ZSTD for every job j whose zstatus is not PVVC_OK
int pvvc_zstd_merge_status(int32_t njobs, const int32_t* zstatus, const int32_t* zslice, int32_t* status, cudaStream_t s);

namespace pvvc {
cudaError_t launch_tree(const SliceWork* work, int nintra, const uint8_t* payload, const StateView& st, int32_t* tstatus,
                        cudaStream_t s);
cudaError_t launch_rlgr(const SliceWork* work, const int32_t* order, int nslices, const uint8_t* payload, float* coef,
                        int32_t* rstatus, int block, int smem, cudaStream_t s);
cudaError_t launch_rlgr_long(const SliceWork* work, const int32_t* order, int nslices, const uint8_t* payload, float* coef,
                             int32_t* rstatus, int lanes, int smem, cudaStream_t s);
cudaError_t launch_rlgr_win(const SliceWork* work, const GroupDesc* groups, int ngroups, const int32_t* items,
                            const uint8_t* payload, float* coef, int32_t* rstatus, int warps, cudaStream_t s);
cudaError_t prepare_kernels();
cudaError_t launch_refresh(SliceWork* work, int n, const CallFields& f, cudaStream_t s);
cudaError_t launch_raht_slice(const SliceWork* work, const int32_t* list, int count, const StateView& st, const float* coef,
                              float* fallback, const int32_t* tstatus, const int32_t* rstatus, int32_t* fstatus, float* xyz,
                              uint8_t* rgb, float* p24, int32_t* status, int wcap, cudaStream_t s);
cudaError_t launch_raht_group(const SliceWork* work, const GroupDesc* groups, int ngroups, const int32_t* items,
                              const StateView& st, const float* coef, const int32_t* tstatus, const int32_t* rstatus,
                              int32_t* fstatus, float* xyz, uint8_t* rgb, float* p24, int32_t* status, float* scratch,
                              uint64_t scratch_floats, int nctas, int* counter, cudaStream_t s);

// default launch shapes: persistent CTAs of the group kernel per SM (its
// registers allow four), the group threshold, the RLGR block, and
// the CTAs that decode the longest slices on SMs of their own
constexpr int kGroupCtasPerSm = 3;
constexpr int kMinGroup = 4;
constexpr int kRlgrBlock = 64;
constexpr int kRlgrLongCtas = 16;
constexpr int kRlgrMidPct = 50;
constexpr int kRlgrLongLanes = 32;
// window mode: the medium tier splits in kMidSplit sub-tiers (1 or 2) when it
// has at least kMidSplitMin groups
constexpr int kMidSplit = 2;
constexpr int kMidSplitMin = 64;
// window mode: the long tier's groups (the largest, the last to finish)
// are inverse-transformed by kLongSplit CTAs each
constexpr int kLongSplit = 2;

// the SM count (queried once)
inline int sm_count() {
    static int n = 0;
    if (!n) {
        int dev = 0;
        cudaGetDevice(&dev);
        if (cudaDeviceGetAttribute(&n, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || n <= 0) n = 132;
    }
    return n;
}

// level-signal capacity (nodes) of the shared-memory path of k_raht
constexpr int kRahtWcap = 1024;

inline uint64_t align_up(uint64_t v, uint64_t a) { return (v + a - 1) / a * a; }

// grow-only device buffer
struct DevBuf {
    void* p = nullptr;
    size_t cap = 0;
    ~DevBuf() {
        if (p) cudaFree(p);
    }
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFree(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMalloc(&p, n);
        if (e == cudaSuccess) cap = n;
        return e;
    }
};
// a second stream and fork/join events, so that a decode can run two kernels
// side by side (also under stream capture, where they become graph branches)
struct SideStream {
    cudaStream_t s = nullptr;
    cudaEvent_t fork = nullptr, join = nullptr, mid = nullptr;  // mid: a point of the main stream the side one waits for
    SideStream() = default;
    SideStream(const SideStream&) = delete;
    SideStream& operator=(const SideStream&) = delete;
    ~SideStream() {
        if (fork) cudaEventDestroy(fork);
        if (join) cudaEventDestroy(join);
        if (mid) cudaEventDestroy(mid);
        if (s) cudaStreamDestroy(s);
    }
    // urgent: the stream gets the device's greatest priority, so that its
    // CTAs are dispatched ahead of the other streams' (the decode's longest
    // chain of dependent work runs on it)
    cudaError_t ensure(bool urgent = false) {
        cudaError_t e = cudaSuccess;
        if (!s) {
            int least = 0, greatest = 0;
            if (urgent && cudaDeviceGetStreamPriorityRange(&least, &greatest) == cudaSuccess)
                e = cudaStreamCreateWithPriority(&s, cudaStreamNonBlocking, greatest);
            else
                e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
        }
        if (e == cudaSuccess && !fork) e = cudaEventCreateWithFlags(&fork, cudaEventDisableTiming);
        if (e == cudaSuccess && !join) e = cudaEventCreateWithFlags(&join, cudaEventDisableTiming);
        if (e == cudaSuccess && !mid) e = cudaEventCreateWithFlags(&mid, cudaEventDisableTiming);
        return e;
    }
};
struct HostBuf {  // pinned, grow-only
    void* p = nullptr;
    size_t cap = 0;
    ~HostBuf() {
        if (p) cudaFreeHost(p);
    }
    cudaError_t ensure(size_t n) {
        if (n <= cap) return cudaSuccess;
        if (p) cudaFreeHost(p);
        p = nullptr;
        cap = 0;
        cudaError_t e = cudaMallocHost(&p, n);
        if (e == cudaSuccess) cap = n;
        return e;
    }
};
}  // namespace pvvc

struct pvvc_plan {
    pvvc_tune tune{};  // resolved launch shapes
    double host_ms[5] = {};  // host time of the last build's stages (pvvc_plan_host_times)
    int32_t nslices = 0, nintra = 0, max_slot = -1;
    uint64_t total_points = 0;
    uint64_t ws_coef = 0, ws_fb = 0, ws_tstatus = 0, ws_rstatus = 0, ws_fstatus = 0, ws_bytes = 0;
    uint64_t ws_grp = 0, ws_counter = 0, grp_floats = 0;  // group-kernel level buffers, queue counters
    int32_t grp_ctas = 0, grp_ctas_long = 0, grp_ctas_mid = 0;
    uint64_t ws_grp_long = 0, ws_grp_mid = 0;  // level buffers of the long and medium groups' launches
    int32_t grp_ctas_mid2 = 0;
    uint64_t ws_grp_mid2 = 0;
    // window mode: the long tier's groups again, each split over
    // kLongSplit CTAs for their inverse transform (after the phase-B groups)
    int32_t long_split_off = 0, nlong_split = 0;
    uint64_t coef_floats = 0;
    uint64_t coef_long_floats = 0;  // planes prefix the long-slice RLGR launch writes
    uint64_t coef_mid_floats = 0;   // ... and the medium tier
    std::vector<int32_t> order;
    // inverse-RAHT schedule: phase A needs only this batch's trees; phase B
    // also needs phase A's intra colours.  Groups go to the warp kernel,
    // lists to the per-slice kernel.
    std::vector<pvvc::GroupDesc> groups;  // [A groups | B groups]
    int32_t ngroups_a = 0, ngroups_b = 0;
    int32_t ngroups_a_long = 0;           // leading phase-A groups that hold a long-launch slice
    int32_t ngroups_a_mid = 0;            // the next phase-A groups: a medium-tier slice, no long one
    // window mode: the medium tier's groups split in two sub-tiers (the
    // larger first) on streams of their own, so that the second's inverse
    // transform starts as soon as its shorter RLGR ends; the second's count
    int32_t ngroups_a_mid2 = 0;
    // leading phase-A groups decoded by the windowed RLGR (then ngroups_a_long
    // and ngroups_a_mid count its long and medium tiers), their slices (the
    // head of `order`) and their coefficient planes (never cleared)
    int32_t nwin = 0, nwin_slices = 0;
    uint64_t coef_win_floats = 0;
    std::vector<int32_t> idx;             // [group items | slice list A | slice list B]
    int32_t nlist_a = 0, nlist_b = 0, list_a_off = 0, list_b_off = 0;
    pvvc::DevBuf d_work, d_order, d_groups, d_idx;
    pvvc::HostBuf h_work;  // the queue's records, built here (page-locked) and uploaded from here
    pvvc::HostBuf h_order, h_groups, h_idx;  // pinned mirrors of stream-ordered uploads
    int32_t nlong = 0;       // the first nlong slices of `order` go to the long-slice RLGR launch
    int32_t nmid = 0;        // the next nmid slices to the medium tier
    pvvc::SideStream side;   // the long tier's stream
    pvvc::SideStream side2;  // the medium tier's stream
    pvvc::SideStream side3;  // window mode: the medium tier's second half
    pvvc::SideStream tree;   // the tree expansion's stream (beside the coefficient clear and RLGR)
    bool upload_pending = false;  // built with deferred copies, not yet queued
    // d_work holds this plan's records (their upload is queued): a rebuild of
    // the same layout for a host call may refresh them on the device instead
    bool device_records = false;
    // a pending device refresh: the host call's description arrays (page-
    // locked, alive until the call ends) to upload, then k_refresh
    bool refresh_pending = false;
    pvvc_batch_desc refresh_src{};
    pvvc::DevBuf d_call;  // their device copies
    // the layout of the last full build (slots, types, sizes, shapes): a
    // build of the same layout refreshes the records only
    bool cache_valid = false;
    std::vector<int32_t> key_slot;
    std::vector<uint8_t> key_type;
    std::vector<uint32_t> key_size;
    pvvc_tune key_tune{};
};

struct pvvc_state {
    pvvc::StateView v{};
    // buffers of the end-to-end host call, kept across calls
    pvvc::DevBuf payload, xyz, rgb, ws, status;
    pvvc::HostBuf h_payload;
    pvvc::HostBuf host_desc;  // the host call's description arrays (page-locked)
    pvvc_plan plan;
    static constexpr int kParts = 3;        // a multi-GoP call is decoded in up to this many parts
    // part boundaries, as fractions of the slices: a small first part starts
    // the device work (and its outputs' trip to the host) early, while the
    // other parts are still being planned
    static constexpr double kCutAt[kParts - 1] = {0.15, 0.4};
    pvvc_plan part_plan[kParts - 1];        // the plans of parts 1.. (part 0 uses `plan`)
    cudaStream_t copy = nullptr;            // device-to-host copies that overlap the next part's decode
    cudaEvent_t part_done[kParts] = {};
    cudaStream_t zside = nullptr;           // zstd inflation of the parts after the first
    cudaStream_t up = nullptr;              // host-to-device copies of the parts' raw payloads
    cudaEvent_t up_done[kParts] = {};
    // timing events of the call's device timeline: its start, and per part
    // the end of its upload, of its decode and of its copy back
    cudaEvent_t t_start = nullptr, t_up[kParts] = {}, t_dec[kParts] = {}, t_cp[kParts] = {};
    cudaEvent_t zdone[kParts] = {};
};

namespace pvvc {
// zero tune fields -> defaults; out-of-range fields -> PVVC_ERR_ARG
int resolve_tune(const pvvc_tune* in, pvvc_tune* out);
// Sort a batch into the work queue and upload it: synchronously, or with
// `upload` set, stream-ordered on that stream from pinned mirrors; with
// `defer` as well, the copies are left for upload_plan (so that one thread
// queues every CUDA call of a host call while others plan).
int build_plan(const pvvc_batch_desc* d, pvvc_plan* p, const pvvc_tune* tune, cudaStream_t upload, bool defer = false);
int upload_plan(pvvc_plan* p, cudaStream_t s);
int copy_plan(pvvc_plan* p, cudaStream_t upload, bool defer);
// Enqueue one planned decode on `s` (events: optional stage markers).
int run_decode(const pvvc_plan* p, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb, float* p24,
               int32_t* status, void* ws, uint64_t ws_bytes, cudaStream_t s, void* const* events);
}  // namespace pvvc
