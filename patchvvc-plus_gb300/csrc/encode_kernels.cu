// encode_kernels.cu -- GB300 (sm_103a) encoder back end of the colour path:
// forward RAHT, quantisation and RLGR coding of a batch of slices.
//
//   k_tree     (decode_kernels.cu) expands each intra slice's geometry
//              payload into its slot's tables, exactly as for decoding
//   k_fwd_raht one persistent CTA per group of slices that share a slot (the
//              frames of one patch as the 32 lanes of every warp): bottom-up
//              HierarchicalTransform (src/octree/octree_base.cc:65-82,
//              164-184) level by level, the coded high-pass coefficients
//              quantised (src/patch/GoP_encoding.cc:184-189) into the
//              slice's symbol planes in stream (reversed) order
//   k_rlgr_enc one thread per slice: RLGREncoder::Encode/GetResult
//              (src/common/entropy_codec.cc:65-159) into the caller's buffer
//
// Bit-exactness with the CPU encoder: the butterfly pairs come from k_tree
// (the decoder's own a = sqrt(w0)/base, b = sqrt(w1)/base); every FP32
// operation is an explicitly rounded intrinsic in the reference's order.
#include <cuda_runtime.h>

#include <algorithm>
#include <cstring>
#include <memory>
#include <new>
#include <vector>

#include "decode_internal.h"

namespace pvvc {
namespace {

constexpr int kEncWarps = 8;

__device__ __forceinline__ constexpr int epair0(int i) {
    return i == 1 ? 2 : i == 2 ? 4 : i == 3 ? 5 : i == 4 ? 8 : i == 5 ? 9 : i == 6 ? 10 : 11;
}
__device__ __forceinline__ constexpr int epair1(int i) {
    return i == 1 ? 3 : i == 2 ? 6 : i == 3 ? 7 : i == 4 ? 12 : i == 5 ? 13 : i == 6 ? 14 : 15;
}

// static_cast<FIX_DATA_INT>(std::round(c / QP)) (GoP_encoding.cc:186-188)
__device__ __forceinline__ int32_t quantise(float c, float qp) { return (int32_t)roundf(__fdiv_rn(c, qp)); }

// k_fwd_raht: lanes = the group's slices.  The level signal (children's DC)
// lives in the CTA's scratch as [node][yuv][lane]; levels run bottom-up with
// a CTA barrier each.  Symbol planes use the plan's frame-interleaved group
// regions: symbol j of plane p at coef_off + (p*N + j)*32 + lane.
__global__ void __launch_bounds__(32 * kEncWarps) k_fwd_raht(const SliceWork* __restrict__ work,
                                                             const GroupDesc* __restrict__ groups, int ngroups,
                                                             const int32_t* __restrict__ items, StateView st,
                                                             const float* __restrict__ leaf_yuv, int32_t* __restrict__ sym,
                                                             const int32_t* __restrict__ tstatus, int32_t* __restrict__ fstatus,
                                                             float* __restrict__ scratch, uint64_t scratch_floats,
                                                             int* __restrict__ counter) {
    __shared__ int s_g, s_H, s_ls[kMaxLevels + 1];
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    float* const bufA = scratch + (uint64_t)blockIdx.x * scratch_floats;
    float* const bufB = bufA + scratch_floats / 2;
    for (;;) {
        if (tid == 0) s_g = atomicAdd(counter, 1);
        __syncthreads();
        const int gi = s_g;
        if (gi >= ngroups) break;
        const GroupDesc G = groups[gi];
        const bool have = lane < G.count;
        const int item = have ? items[G.first + lane] : 0;
        const SliceWork& w = work[item];
        int err = PVVC_OK;
        if (have) {
            if (!(w.type & PVVC_TYPE_VALID)) err = PVVC_ERR_BAD_SLICE;
            else if (!(w.type & PVVC_TYPE_PREDICT)) err = tstatus[item];
            if (!err) {
                const SlotInfo* si = st.info + w.slot;
                if (!si->valid) err = PVVC_ERR_NO_REFERENCE;
                else if ((uint32_t)si->leaves != w.n) err = PVVC_ERR_SIZE;
            }
            if (wid == 0) fstatus[item] = err;
        }
        const bool act = have && !err;
        const bool any = __any_sync(0xffffffffu, act);
        if (tid == 0) {
            const SlotInfo* si = st.info + G.slot;
            s_H = si->height;
            for (int l = 0; l < kMaxLevels + 1; ++l) s_ls[l] = si->level_start[l];
        }
        __syncthreads();
        if (any) {
            const int H = s_H;
            const size_t nb = (size_t)G.slot * st.max_nodes;
            const uint32_t N = act ? w.n : 0;
            const float qp = act ? (float)w.qp : 1.f;
            const float* leaf = leaf_yuv + (act ? 3 * w.out_off : 0);
            int32_t* sy = sym + (act ? w.coef_off + lane : 0);
            // coefficient k (0 = DC, un-reversed order) -> symbol N-1-k of each plane
            auto put = [&](uint32_t k, float y, float u, float v) {
                if (!act) return;
                const size_t j = (size_t)(N - 1 - k);
                sy[j * 32] = quantise(y, qp);
                sy[((size_t)N + j) * 32] = quantise(u, qp);
                sy[((size_t)2 * N + j) * 32] = quantise(v, qp);
            };
            if (H == 1) {
                if (wid == 0 && act) put(0, leaf[0], leaf[1], leaf[2]);
            } else {
                float* gIn = bufA;   // children's DC of the level being transformed
                float* gOut = bufB;  // its nodes' DC
                for (int l = H - 2; l >= 0; --l) {
                    const int a = s_ls[l], b = s_ls[l + 1];
                    const bool last = l == H - 2;  // children are leaves
                    for (int j = wid; j < b - a; j += kEncWarps) {
                        const size_t node = nb + a + j;
                        const uint32_t byte = __ldg(st.occ + node), cb = __ldg(st.cbase + node);
                        const uint32_t m = __ldg(st.mask + node);
                        const uint32_t ci = __ldg(st.coff + node);
                        const float2* ab = st.ab + node * 7;
                        float sy8[16], su8[16], sv8[16];
#pragma unroll
                        for (int c = 0; c < 16; ++c) sy8[c] = su8[c] = sv8[c] = 0.f;
                        uint32_t r = 0;
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            if (!(byte & (0x80u >> c))) continue;
                            if (act) {
                                if (last) {
                                    const float* p = leaf + 3ull * (cb + r);
                                    sy8[8 + c] = p[0];
                                    su8[8 + c] = p[1];
                                    sv8[8 + c] = p[2];
                                } else {
                                    const float* p = gIn + (size_t)(cb + r) * 96 + lane;
                                    sy8[8 + c] = p[0];
                                    su8[8 + c] = p[32];
                                    sv8[8 + c] = p[64];
                                }
                            }
                            ++r;
                        }
                        // HaarTransform for i = 7..1: G = g0 a + g1 b, H = g0 (-b) + g1 a
                        float hy[8], hu[8], hv[8];
#pragma unroll
                        for (int i = 7; i > 0; --i) {
                            const float2 t = __ldg(ab + (i - 1));
                            const float nb2 = -t.y;
                            const float g0y = sy8[epair0(i)], g1y = sy8[epair1(i)];
                            const float g0u = su8[epair0(i)], g1u = su8[epair1(i)];
                            const float g0v = sv8[epair0(i)], g1v = sv8[epair1(i)];
                            sy8[i] = __fadd_rn(__fmul_rn(g0y, t.x), __fmul_rn(g1y, t.y));
                            su8[i] = __fadd_rn(__fmul_rn(g0u, t.x), __fmul_rn(g1u, t.y));
                            sv8[i] = __fadd_rn(__fmul_rn(g0v, t.x), __fmul_rn(g1v, t.y));
                            hy[i] = __fadd_rn(__fmul_rn(g0y, nb2), __fmul_rn(g1y, t.x));
                            hu[i] = __fadd_rn(__fmul_rn(g0u, nb2), __fmul_rn(g1u, t.x));
                            hv[i] = __fadd_rn(__fmul_rn(g0v, nb2), __fmul_rn(g1v, t.x));
                        }
                        // the node's DC to its parent (or the stream's coefficient 0)
                        if (l == 0) {
                            put(0, sy8[1], su8[1], sv8[1]);
                        } else {
                            float* q = gOut + (size_t)j * 96 + lane;
                            q[0] = sy8[1];
                            q[32] = su8[1];
                            q[64] = sv8[1];
                        }
                        // coded high-pass coefficients (both weights > 0) at the node's offsets
#pragma unroll
                        for (int i = 1; i < 8; ++i)
                            if (m & (1u << i)) put(ci + __popc(m & ((1u << i) - 2u)), hy[i], hu[i], hv[i]);
                    }
                    __syncthreads();
                    float* t = gIn;
                    gIn = gOut;
                    gOut = t;
                }
            }
        }
        __syncthreads();
    }
}

// RLGREncoder: MSB-first bit writer over a 64-bit accumulator with the
// reference's '+' (a value wider than its field would carry into the pending
// bits before it; every caller here passes v < 2^bits, since the symbols are
// int32), emitted as big-endian 32-bit words in order.
struct BitSink {
    uint32_t* out;       // 4-byte aligned region
    uint32_t cap;        // bytes
    uint32_t nwords = 0; // whole 32-bit words emitted
    uint32_t nbytes = 0; // set by finish()
    uint64_t acc = 0;    // pending bits in the low n bits
    int n = 0;           // < 32 between calls
    bool overflow = false;
    __device__ __forceinline__ void emit(uint32_t w) {
        if (++nwords * 4u <= cap) out[nwords - 1] = __byte_perm(w, 0, 0x0123);
        else overflow = true;
    }
    __device__ __forceinline__ void put(uint64_t v, int bits) {
        if (bits > 32) {
            put(v >> 32, bits - 32);
            put(v & 0xFFFFFFFFull, 32);
            return;
        }
        acc = (acc << bits) + v;
        n += bits;
        if (n >= 32) {
            n -= 32;
            emit((uint32_t)(acc >> n));
        }
    }
    __device__ __forceinline__ void gr(uint64_t x, int k) {  // GRWrite
        const uint64_t p = x >> k;
        if (p < 32) {
            put((1ull << (p + 1)) - 2, (int)p + 1);  // p ones and a zero
            put(x & ((1ull << k) - 1), k);
        } else {
            put(0xFFFFFFFFull, 32);
            put(x, 32);
        }
    }
    __device__ __forceinline__ void finish() {  // zero bits up to the byte boundary
        nbytes = nwords * 4u + (uint32_t)((n + 7) >> 3);
        if (n) {
            const uint32_t w = (uint32_t)(acc << (32 - n));
            if (nbytes <= cap) out[nwords] = __byte_perm(w, 0, 0x0123);
            else overflow = true;
        }
    }
};

constexpr uint64_t kL = 4, kU0 = 3, kD0 = 1, kU1 = 2, kD1 = 1;

constexpr int kEncRlgrBlock = 128;
constexpr int kEncPf = 16;  // symbols per prefetch batch
// The largest slices (first in `order`) are encoded kEncLongLanes to a warp
// by the first CTAs of the launch, the rest kEncRestLanes to a warp: the
// encoder's branches diverge between lanes, and a warp of 32 long slices
// would take their divergent paths one after another.
constexpr int kEncLongLanes = 2;
constexpr int kEncLongCtas = 304;
constexpr int kEncLongSlices = kEncLongCtas * (kEncRlgrBlock / 32) * kEncLongLanes;
constexpr int kEncRestLanes = 32;

__global__ void __launch_bounds__(kEncRlgrBlock) k_rlgr_enc(const SliceWork* __restrict__ work,
                                                           const int32_t* __restrict__ order, int nslices, int nlong,
                                                           int long_ctas,
                           const int32_t* __restrict__ sym, uint8_t* __restrict__ out, const uint64_t* __restrict__ out_off,
                           const uint32_t* __restrict__ out_cap, uint32_t* __restrict__ out_len,
                           int32_t* __restrict__ fstatus) {
    __shared__ int32_t s_sym[kEncPf][kEncRlgrBlock];  // column threadIdx.x: this thread's batch
    const int lane = threadIdx.x & 31;
    int t;
    if ((int)blockIdx.x < long_ctas) {
        t = ((int)blockIdx.x * (kEncRlgrBlock / 32) + (int)(threadIdx.x >> 5)) * kEncLongLanes + lane;
        if (lane >= kEncLongLanes || t >= nlong) return;
    } else {
        t = nlong + (((int)blockIdx.x - long_ctas) * (kEncRlgrBlock / 32) + (int)(threadIdx.x >> 5)) * kEncRestLanes + lane;
        if (lane >= kEncRestLanes || t >= nslices) return;
    }
    const int item = order[t];
    const SliceWork& w = work[item];
    if (fstatus[item] != PVVC_OK) {
        out_len[w.orig] = 0;
        return;
    }
    const uint32_t N = w.n;
    const int32_t* s = sym + w.coef_off + w.coef_lane;
    const size_t cs = w.coef_stride;
    BitSink bw{reinterpret_cast<uint32_t*>(out + out_off[w.orig]), out_cap[w.orig]};
    uint64_t u = 0, kP = 0, kRP = 2 * kL, m = 0, k = 0;
    const uint64_t total = 3ull * N;
    auto encode = [&](int64_t x) {
        u = x < 0 ? ((uint64_t)(-x) << 1) - 1 : (uint64_t)x << 1;  // Sign2Unsign
        k = kP / kL;
        const uint64_t kR = kRP / kL;
        if (k) {
            if (u) {
                --u;
                bw.put(0, 1);
                bw.put(m, (int)k);
                bw.gr(u, (int)kR);
                const uint64_t p = u >> kR;
                kRP = p ? min(kRP + p - 1, 32 * kL) : (kRP < 2 ? 0 : kRP - 2);
                kP = kP < kD1 ? 0 : kP - kD1;
                m = 0;
            } else if (++m == (1ull << k)) {
                bw.put(1, 1);
                kP += kU1;
                m = 0;
            }
        } else {
            bw.gr(u, (int)kR);
            const uint64_t p = u >> kR;
            kRP = p ? min(kRP + p - 1, 32 * kL) : (kRP < 2 ? 0 : kRP - 2);
            kP = u ? (kP < kD0 ? 0 : kP - kD0) : kP + kU0;
            m = 0;
        }
    };
    // The symbols of a slice sit coef_stride apart (frame-interleaved planes),
    // one sector each: they are loaded kEncPf at a time into registers, the
    // next batch in flight while this one is encoded from the thread's own
    // shared-memory column, so the chain does not wait on every load.
    int32_t nxt[kEncPf];
#pragma unroll
    for (int j = 0; j < kEncPf; ++j) nxt[j] = (uint64_t)j < total ? s[(uint64_t)j * cs] : 0;
    for (uint64_t b0 = 0; b0 < total && !bw.overflow; b0 += kEncPf) {
        uint32_t nz = 0;  // bit j: symbol b0 + j is nonzero
#pragma unroll
        for (int j = 0; j < kEncPf; ++j) {
            s_sym[j][threadIdx.x] = nxt[j];
            nz |= (uint32_t)(nxt[j] != 0) << j;
        }
        if (b0 + kEncPf < total) {
#pragma unroll
            for (int j = 0; j < kEncPf; ++j) nxt[j] = b0 + kEncPf + j < total ? s[(b0 + kEncPf + j) * cs] : 0;
        }
        const int cnt = total - b0 < (uint64_t)kEncPf ? (int)(total - b0) : kEncPf;
        int j = 0;
        while (j < cnt) {
            const int32_t x = s_sym[j][threadIdx.x];
            if (x != 0 || kP < kL) {
                encode(x);
                ++j;
                continue;
            }
            // Zeros in run mode, taken together: each symbol would add one to
            // m and, when m reaches 2^k, write a 1 and raise kP by kU1 (k only
            // grows, so the run stays in run mode).  `k` ends as the value the
            // last zero saw, as the trailing-run test after the loop expects.
            const uint32_t rest = nz >> j;
            int z = rest ? __ffs(rest) - 1 : cnt - j;
            if (z > cnt - j) z = cnt - j;
            j += z;
            uint64_t left = (uint64_t)z;
            while (left) {
                k = kP / kL;
                const uint64_t need = (1ull << k) - m;
                if (left >= need) {
                    left -= need;
                    bw.put(1, 1);
                    kP += kU1;
                    m = 0;
                } else {
                    m += left;
                    left = 0;
                }
            }
            u = 0;
        }
    }
    if (total > 0 && k && !u) {  // trailing run (entropy_codec.cc:144-147)
        bw.put(0, 1);
        bw.put(m, (int)(kP / kL));
    }
    bw.finish();
    out_len[w.orig] = bw.overflow ? 0 : bw.nbytes;
    if (bw.overflow) fstatus[item] = PVVC_ERR_CAPACITY;
}

__global__ void k_status_out(const SliceWork* __restrict__ work, int n, const int32_t* __restrict__ fstatus,
                             int32_t* __restrict__ status) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t < n) status[work[t].orig] = fstatus[t];
}

}  // namespace
}  // namespace pvvc

using namespace pvvc;

struct pvvc_encoder {
    pvvc_plan plan;
    DevBuf ws, off, cap;
    HostBuf h_off, h_cap;
};

extern "C" int pvvc_encoder_create(pvvc_encoder** out) {
    if (!out) return PVVC_ERR_ARG;
    *out = new (std::nothrow) pvvc_encoder();
    return *out ? PVVC_OK : PVVC_ERR_NOMEM;
}

extern "C" int pvvc_encoder_destroy(pvvc_encoder* e) {
    if (!e) return PVVC_ERR_ARG;
    delete e;
    return PVVC_OK;
}

extern "C" int pvvc_encode_colors(pvvc_encoder* enc, const pvvc_batch_desc* desc, pvvc_state* st, const uint8_t* payload,
                                  const float* leaf_yuv, uint8_t* out, const uint64_t* out_byte_off, const uint32_t* out_cap,
                                  uint32_t* out_len, int32_t* status, void* stream) {
    if (!enc || !desc || !st || desc->nslices < 0) return PVVC_ERR_ARG;
    const int n = desc->nslices;
    if (n == 0) return PVVC_OK;
    if (!payload || !leaf_yuv || !out || !out_byte_off || !out_cap || !out_len || !status) return PVVC_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(payload) & 15u) || (reinterpret_cast<uintptr_t>(out) & 3u)) return PVVC_ERR_ARG;
    for (int i = 0; i < n; ++i)
        if ((out_byte_off[i] & 3u) || (out_cap[i] & 3u)) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // every slot's slices in groups of up to 32 (no per-slice path), no RLGR split
    const pvvc_tune t{1, 1, 128, -1, -1, 32};
    pvvc_plan& p = enc->plan;
    int rc = build_plan(desc, &p, &t, nullptr);
    if (rc) return rc;
    if (p.max_slot >= st->v.nslots) return PVVC_ERR_ARG;
    if (p.nlist_a || p.nlist_b) return PVVC_ERR_ARG;  // min_group 1 groups every slice
    const uint64_t sym_bytes = 4ull * p.coef_floats;  // int32 symbols in the planes' layout
    const uint64_t scratch_bytes = 4ull * p.grp_floats * std::max(p.grp_ctas, 1);
    const uint64_t o_sym = 0, o_scr = align_up(sym_bytes, 256), o_ts = align_up(o_scr + scratch_bytes, 256),
                   o_fs = align_up(o_ts + 4ull * n, 256), o_cnt = align_up(o_fs + 4ull * n, 256), total = o_cnt + 256;
    if (enc->ws.ensure(total) != cudaSuccess || enc->off.ensure(8ull * n) != cudaSuccess ||
        enc->cap.ensure(4ull * n) != cudaSuccess || enc->h_off.ensure(8ull * n) != cudaSuccess ||
        enc->h_cap.ensure(4ull * n) != cudaSuccess)
        return PVVC_ERR_NOMEM;
    std::memcpy(enc->h_off.p, out_byte_off, 8ull * n);
    std::memcpy(enc->h_cap.p, out_cap, 4ull * n);
    uint8_t* w = static_cast<uint8_t*>(enc->ws.p);
    int32_t* sym = reinterpret_cast<int32_t*>(w + o_sym);
    float* scr = reinterpret_cast<float*>(w + o_scr);
    int32_t* ts = reinterpret_cast<int32_t*>(w + o_ts);
    int32_t* fs = reinterpret_cast<int32_t*>(w + o_fs);
    int* cnt = reinterpret_cast<int*>(w + o_cnt);
    const SliceWork* dw = static_cast<const SliceWork*>(p.d_work.p);
    if (cudaMemcpyAsync(enc->off.p, enc->h_off.p, 8ull * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(enc->cap.p, enc->h_cap.p, 4ull * n, cudaMemcpyHostToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(cnt, 0, sizeof(int), s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    if (launch_tree(dw, p.nintra, payload, st->v, ts, s) != cudaSuccess) return PVVC_ERR_CUDA;
    const int ng = p.ngroups_a + p.ngroups_b;
    const int grid = std::min(ng, std::max(p.grp_ctas, 1));
    k_fwd_raht<<<grid, 32 * kEncWarps, 0, s>>>(dw, static_cast<const GroupDesc*>(p.d_groups.p), ng,
                                               static_cast<const int32_t*>(p.d_idx.p), st->v, leaf_yuv, sym, ts, fs, scr,
                                               p.grp_floats, cnt);
    const int nlong = n < kEncLongSlices ? n : kEncLongSlices;
    const int per_long_cta = (kEncRlgrBlock / 32) * kEncLongLanes;
    const int long_ctas = (nlong + per_long_cta - 1) / per_long_cta;
    const int per_rest_cta = (kEncRlgrBlock / 32) * kEncRestLanes;
    k_rlgr_enc<<<long_ctas + (n - nlong + per_rest_cta - 1) / per_rest_cta, kEncRlgrBlock, 0, s>>>(
        dw, static_cast<const int32_t*>(p.d_order.p), n, nlong, long_ctas, sym, out,
                                                static_cast<const uint64_t*>(enc->off.p),
                                                static_cast<const uint32_t*>(enc->cap.p), out_len, fs);
    k_status_out<<<(n + 255) / 256, 256, 0, s>>>(dw, n, fs, status);
    if (cudaGetLastError() != cudaSuccess) return PVVC_ERR_CUDA;
    // the host arrays above are reused by the next call: finish this one
    return cudaStreamSynchronize(s) == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}
