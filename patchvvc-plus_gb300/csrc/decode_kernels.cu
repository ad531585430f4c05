// decode_kernels.cu -- GB300 (sm_103a) kernels of the patchVVC decode path.
//
//   k_tree  one CTA per intra slice: occupancy bytes -> BFS octree tables
//           (child bases by block scans of popcounts), subtree weights,
//           butterfly coefficients, coefficient offsets, node and leaf
//           centres.  Restates InvertRAHTOctree::MakeTree/AddPoints
//           (src/octree/invert_raht_octree.cc:122-254) level-parallel.
//   k_rlgr  one thread per slice: adaptive run-length / Golomb-Rice decode
//           of 3N symbols with a 64-bit window and count-leading-ones,
//           fused dequantisation, written un-reversed as Y|U|V planes.
//           Restates RLGRDecoder::Decode (src/common/entropy_codec.cc:163-283)
//           and the dequantisation of invert_raht_octree.cc:63-69.
//   k_raht  one CTA per slice: level-synchronous inverse RAHT (7 butterflies
//           per internal node, octree_base.cc:84-100,186-206) with the level
//           signal in shared memory, fused with the reference-colour add
//           (invert_raht_octree.cc:304-311), YUV->RGB (common.h:154-158) and
//           the rigid transform (pvvc_decompression.cc:141-150).
//
// Bit-exactness with the CPU decoder: every float operation is an explicitly
// rounded intrinsic (__fadd_rn/__fmul_rn/__fdiv_rn/__fsqrt_rn), evaluated in
// the reference's order, so nothing is contracted into an FMA.
#include <cuda_runtime.h>

#include <cstdint>

#include "decode_types.h"
#include "pvvc_gb300.h"

namespace pvvc {

// child slots of butterfly i (include/octree/octree.h:79); constexpr so that
// unrolled loops index the per-thread slot arrays with constants (registers)
__device__ __forceinline__ constexpr int pair0(int i) {
    return i == 1 ? 2 : i == 2 ? 4 : i == 3 ? 5 : i == 4 ? 8 : i == 5 ? 9 : i == 6 ? 10 : 11;
}
__device__ __forceinline__ constexpr int pair1(int i) {
    return i == 1 ? 3 : i == 2 ? 6 : i == 3 ? 7 : i == 4 ? 12 : i == 5 ? 13 : i == 6 ? 14 : 15;
}

// ---------------------------------------------------------------------------
// block-wide exclusive scan (T threads, T multiple of 32)
template <int T>
__device__ __forceinline__ uint32_t block_excl_scan(uint32_t v, uint32_t* total, uint32_t* s_warp) {
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < T / 32 ? s_warp[lane] : 0;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            uint32_t y = __shfl_up_sync(0xffffffffu, t, o);
            if (lane >= o) t += y;
        }
        if (lane < T / 32) s_warp[lane] = t;  // inclusive warp totals
    }
    __syncthreads();
    const uint32_t warp_base = wid ? s_warp[wid - 1] : 0;
    *total = s_warp[T / 32 - 1];
    __syncthreads();  // s_warp reused by the next call
    return warp_base + x - v;
}

__device__ __forceinline__ float load_be_float(const uint8_t* p) {
    const uint32_t t = ((uint32_t)p[0] << 24) | ((uint32_t)p[1] << 16) | ((uint32_t)p[2] << 8) | (uint32_t)p[3];
    return __uint_as_float(t);
}

// ---------------------------------------------------------------------------
// k_tree
template <int T>
__global__ void __launch_bounds__(T) k_tree(const SliceWork* __restrict__ work, const uint8_t* __restrict__ payload,
                                            StateView st, int32_t* __restrict__ tstatus) {
    __shared__ uint32_t s_warp[T / 32];
    __shared__ int s_err, s_H, s_lstart[kMaxLevels + 1];
    __shared__ float s_c[3], s_r[kMaxLevels + 1][3];
    const int item = blockIdx.x;
    const SliceWork& w = work[item];
    const int tid = threadIdx.x;
    SlotInfo* info = st.info + w.slot;
    const size_t nb = (size_t)w.slot * st.max_nodes;
    const size_t lb = (size_t)w.slot * st.max_leaves;
    const uint8_t* g = payload + w.geo_off;

    if (!(w.type & PVVC_TYPE_VALID)) {  // SetSlice rejects it before touching state (:25-27)
        if (tid == 0) tstatus[item] = PVVC_ERR_BAD_SLICE;
        return;
    }
    if (tid == 0) {
        int err = PVVC_OK, H = 0;
        info->valid = 0;
        if (w.gsz < 25) {
            err = PVVC_ERR_GEOMETRY;
        } else {
            for (int a = 0; a < 3; ++a) {
                s_c[a] = load_be_float(g + 4 * a);
                s_r[0][a] = load_be_float(g + 12 + 4 * a);
            }
            H = g[24];
            if (H < 1) err = PVVC_ERR_GEOMETRY;
            else if (H > kMaxLevels) err = PVVC_ERR_TREE;
            for (int l = 1; l <= H && l <= kMaxLevels; ++l)
                for (int a = 0; a < 3; ++a) s_r[l][a] = __fdiv_rn(s_r[l - 1][a], 2.0f);
        }
        s_err = err;
        s_H = H;
    }
    __syncthreads();
    if (s_err) {
        if (tid == 0) tstatus[item] = s_err;
        return;
    }
    const int H = s_H;

    // ---- level expansion (MakeTree, invert_raht_octree.cc:158-192) ----
    uint32_t pos = 25, count = 1, nbase = 0, max_w = 0;
    for (int l = 0; l < H - 1; ++l) {
        if (pos + count > w.gsz) { if (tid == 0) s_err = PVVC_ERR_GEOMETRY; }
        else if (nbase + count > (uint32_t)st.max_nodes) { if (tid == 0) s_err = PVVC_ERR_TREE; }
        __syncthreads();
        if (s_err) break;
        if (tid == 0) s_lstart[l] = (int)nbase;
        max_w = max(max_w, count);
        uint32_t running = 0;
        for (uint32_t c0 = 0; c0 < count; c0 += T) {
            const uint32_t j = c0 + tid;
            const uint32_t byte = j < count ? g[pos + j] : 0u;
            uint32_t tot;
            const uint32_t ex = block_excl_scan<T>(__popc(byte), &tot, s_warp);
            if (j < count) {
                st.occ[nb + nbase + j] = (uint8_t)byte;
                st.cbase[nb + nbase + j] = running + ex;
            }
            running += tot;
        }
        pos += count;
        nbase += count;
        count = running;
    }
    if (tid == 0 && !s_err) {
        s_lstart[H - 1] = (int)nbase;
        if (count != w.n) s_err = PVVC_ERR_SIZE;
        else if (count > (uint32_t)st.max_leaves) s_err = PVVC_ERR_TREE;
    }
    __syncthreads();
    if (s_err) {
        if (tid == 0) tstatus[item] = s_err;
        return;
    }
    __threadfence_block();

    // ---- subtree weights, bottom-up (AddPoints, :236-247) ----
    for (int l = H - 2; l >= 0; --l) {
        const int a = s_lstart[l], b = s_lstart[l + 1];
        for (int j = a + tid; j < b; j += T) {
            const uint32_t byte = st.occ[nb + j], cb = st.cbase[nb + j], k = __popc(byte);
            uint32_t tot = k;
            if (l < H - 2) {
                tot = 0;
                for (uint32_t c = 0; c < k; ++c) tot += st.wsum[nb + b + cb + c];
            }
            st.wsum[nb + j] = tot;
        }
        __syncthreads();
    }

    // ---- butterflies and coefficient counts per node ----
    // coefficient offsets need a BFS-order scan over all internal nodes
    uint32_t running = 1;  // coefficient 0 is the DC
    for (int l = 0; l < H - 1; ++l) {
        const int a = s_lstart[l], b = s_lstart[l + 1];
        for (int c0 = a; c0 < b; c0 += T) {
            const int j = c0 + tid;
            uint32_t cnt = 0;
            if (j < b) {
                const uint32_t byte = st.occ[nb + j], cb = st.cbase[nb + j];
                int wt[16];
#pragma unroll
                for (int i = 0; i < 16; ++i) wt[i] = 0;
                uint32_t r = 0;
#pragma unroll
                for (int c = 0; c < 8; ++c)
                    if (byte & (0x80u >> c)) {
                        wt[8 + c] = (l == H - 2) ? 1 : (int)st.wsum[nb + b + cb + r];
                        ++r;
                    }
#pragma unroll
                for (int i = 7; i > 0; --i) wt[i] = wt[pair0(i)] + wt[pair1(i)];
                uint32_t m = 0;
#pragma unroll
                for (int i = 1; i < 8; ++i) {
                    const int w0 = wt[pair0(i)], w1 = wt[pair1(i)];
                    float av = 0.f, bv = 0.f;
                    if (w0 != 0 || w1 != 0) {
                        const float base = __fsqrt_rn(__int2float_rn(w0 + w1));
                        av = __fdiv_rn(__fsqrt_rn(__int2float_rn(w0)), base);
                        bv = __fdiv_rn(__fsqrt_rn(__int2float_rn(w1)), base);
                    }
                    if (w0 != 0 && w1 != 0) m |= 1u << i;
                    st.ab[(nb + j) * 7 + (i - 1)] = make_float2(av, bv);
                }
                st.mask[nb + j] = (uint8_t)m;
                cnt = __popc(m);
            }
            uint32_t tot;
            const uint32_t ex = block_excl_scan<T>(cnt, &tot, s_warp);
            if (j < b) st.coff[nb + j] = running + ex;
            running += tot;
        }
    }
    // a well-formed tree codes exactly one coefficient per leaf; an empty
    // occupancy byte breaks that and would send reads past the planes
    if (running != count) {
        if (tid == 0) tstatus[item] = PVVC_ERR_GEOMETRY;
        return;
    }

    // ---- centres, top-down (SubSpaceCenter, octree_base.cc:102-120) ----
    if (tid == 0) {
        st.ctr[nb * 3 + 0] = s_c[0];
        st.ctr[nb * 3 + 1] = s_c[1];
        st.ctr[nb * 3 + 2] = s_c[2];
        if (H == 1) {
            st.xyz[lb * 3 + 0] = s_c[0];
            st.xyz[lb * 3 + 1] = s_c[1];
            st.xyz[lb * 3 + 2] = s_c[2];
        }
    }
    __syncthreads();
    for (int l = 0; l < H - 1; ++l) {
        const int a = s_lstart[l], b = s_lstart[l + 1];
        // child offset = (range_l / 2) / 2, per axis
        const float ox = __fdiv_rn(s_r[l + 1][0], 2.0f), oy = __fdiv_rn(s_r[l + 1][1], 2.0f), oz = __fdiv_rn(s_r[l + 1][2], 2.0f);
        for (int j = a + tid; j < b; j += T) {
            const uint32_t byte = st.occ[nb + j], cb = st.cbase[nb + j];
            const float cx = st.ctr[(nb + j) * 3 + 0], cy = st.ctr[(nb + j) * 3 + 1], cz = st.ctr[(nb + j) * 3 + 2];
            uint32_t r = 0;
            for (int c = 0; c < 8; ++c) {
                if (!(byte & (0x80u >> c))) continue;
                const float x = (c & 4) ? __fsub_rn(cx, ox) : __fadd_rn(cx, ox);
                const float y = (c & 2) ? __fsub_rn(cy, oy) : __fadd_rn(cy, oy);
                const float z = (c & 1) ? __fsub_rn(cz, oz) : __fadd_rn(cz, oz);
                float* dst = (l < H - 2) ? st.ctr + (nb + b + cb + r) * 3 : st.xyz + (lb + cb + r) * 3;
                dst[0] = x;
                dst[1] = y;
                dst[2] = z;
                ++r;
            }
        }
        __syncthreads();
    }

    if (tid == 0) {
        info->height = H;
        info->nodes = (int)nbase;
        info->leaves = (int)count;
        info->max_width = (int)max_w;
        for (int l = 0; l < H; ++l) info->level_start[l] = s_lstart[l];
        __threadfence();
        info->valid = 1;
        tstatus[item] = PVVC_OK;
    }
}

// ---------------------------------------------------------------------------
// k_rlgr: bit reader over 32-bit big-endian words
struct BitReader {
    const uint32_t* wp;   // next word
    const uint32_t* wend; // one past the last word holding payload bytes
    uint64_t win;         // next bits, MSB-aligned; bits past `nb` are zero
    int nb;               // valid bits in win
    uint32_t used_hi;     // consumed bits beyond the payload (overrun detector)
    int64_t left;         // payload bits not yet consumed

    __device__ __forceinline__ void refill() {
        while (nb <= 32) {
            const uint32_t v = wp < wend ? __byte_perm(__ldg(wp), 0, 0x0123) : 0u;
            ++wp;
            win |= (uint64_t)v << (32 - nb);
            nb += 32;
        }
    }
    __device__ __forceinline__ void consume(int k) {
        win = k >= 64 ? 0ull : (win << k);
        nb -= k;
        left -= k;
    }
    __device__ __forceinline__ uint32_t peek(int k) const { return k ? (uint32_t)(win >> (64 - k)) : 0u; }
    __device__ __forceinline__ int ones() const { return __clzll(~win); }
};

constexpr int kRlL = 4, kRlU0 = 3, kRlD0 = 1, kRlU1 = 2, kRlD1 = 1;

// GRRead (entropy_codec.cc:196-205): q ones then a zero then k bits; 32 ones
// escape to a raw 32-bit value.
__device__ __forceinline__ uint64_t gr_read(BitReader& br, int k) {
    br.refill();
    const int q = br.ones();
    if (q >= 32) {
        br.consume(32);
        br.refill();
        const uint64_t v = br.peek(32);
        br.consume(32);
        return v;
    }
    br.consume(q + 1);
    br.refill();
    const uint64_t r = br.peek(k);
    br.consume(k);
    return ((uint64_t)q << k) + r;
}

__global__ void __launch_bounds__(128) k_rlgr(const SliceWork* __restrict__ work, const int32_t* __restrict__ order,
                                              int nslices, const uint8_t* __restrict__ payload, float* __restrict__ coef,
                                              int32_t* __restrict__ rstatus) {
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= nslices) return;
    const int item = order[t];
    const SliceWork& w = work[item];
    const uint32_t N = w.n;
    const uint64_t total = 3ull * N;
    const long long qp = w.qp;

    BitReader br;
    const uint64_t start = w.col_off;
    const uint32_t* base = reinterpret_cast<const uint32_t*>(payload + (start & ~3ull));
    br.wp = base;
    br.wend = reinterpret_cast<const uint32_t*>(payload + ((start + w.csz + 3) & ~3ull));
    br.win = 0;
    br.nb = 0;
    br.left = 8ll * w.csz;
    br.refill();
    const int skip = (int)(start & 3) * 8;
    br.win <<= skip;
    br.nb -= skip;
    br.refill();

    float* plane = coef + w.coef_off;  // Y, then U, then V (N floats each)
    uint32_t j = 0;                    // position within the current plane
    uint64_t n = 0;
    int err = 0;
    // symbol `n` goes to coefficient N-1-j of the current plane (the stream is reversed)
    auto emit = [&](float v) {
        plane[N - 1 - j] = v;
        if (++j == N) {
            j = 0;
            plane += N;
        }
        ++n;
    };

    uint32_t kP = 0, kRP = 2 * kRlL;
    while (n < total) {
        uint32_t k = kP / kRlL;
        const int kR = (int)(kRP / kRlL);
        uint64_t u;
        if (k) {
            // run mode: each leading '1' is a full run of 2^k zeros (k grows as it goes)
            uint64_t m = 0;
            for (;;) {
                br.refill();
                const int q = min(br.ones(), br.nb);
                for (int i = 0; i < q; ++i) {
                    m += 1ull << k;
                    kP += kRlU1;
                    k = kP / kRlL;
                }
                br.consume(q);
                if (q < 32 || br.left < -64) break;
            }
            br.consume(1);
            br.refill();
            if (k > 32) { err = PVVC_ERR_OVERRUN; break; }
            m += br.peek((int)k);
            br.consume((int)k);
            if (br.left < 0) { err = PVVC_ERR_OVERRUN; break; }
            const uint64_t z = m < total - n ? m : total - n;
            for (uint64_t i = 0; i < z; ++i) emit(0.0f);
            if (n >= total) break;
            u = gr_read(br, kR);
            if (br.left < 0) { err = PVVC_ERR_OVERRUN; break; }
            const uint64_t uu = u + 1;  // Unsign2Sign(u_data + 1)
            const long long s = (uu & 1) ? -(long long)(uu >> 1) - 1 : (long long)(uu >> 1);
            emit(__ll2float_rn(s * qp));
            const uint64_t p = u >> kR;
            if (p) kRP = (uint32_t)(kRP + p - 1 > 32ull * kRlL ? 32ull * kRlL : kRP + p - 1);
            else kRP = kRP < 2 ? 0 : kRP - 2;
            kP = kP < (uint32_t)kRlD1 ? 0 : kP - kRlD1;
        } else {
            u = gr_read(br, kR);
            if (br.left < 0) { err = PVVC_ERR_OVERRUN; break; }
            const long long s = (u & 1) ? -(long long)(u >> 1) - 1 : (long long)(u >> 1);
            emit(__ll2float_rn(s * qp));
            const uint64_t p = u >> kR;
            if (p) kRP = (uint32_t)(kRP + p - 1 > 32ull * kRlL ? 32ull * kRlL : kRP + p - 1);
            else kRP = kRP < 2 ? 0 : kRP - 2;
            if (u) kP = kP < (uint32_t)kRlD0 ? 0 : kP - kRlD0;
            else kP += kRlU0;
        }
    }
    rstatus[item] = err;
}

// ---------------------------------------------------------------------------
// k_raht
struct OutPtrs {
    float* xyz;
    uint8_t* rgb;
    float* p24;
    int32_t* status;  // caller's status, indexed by SliceWork::orig (may be null)
};

__device__ __forceinline__ uint8_t to_u8(float v) {
    const float r = roundf(v);  // std::round: half away from zero
    return (uint8_t)fminf(fmaxf(r, 0.0f), 255.0f);
}

// one leaf: reference add / store, YUV->RGB, transform, output
__device__ __forceinline__ void emit_leaf(const SliceWork& w, const StateView& st, size_t lb, uint32_t leaf, float y,
                                          float u, float v, bool predict, const OutPtrs& o) {
    float* ref = st.ref + (lb + leaf) * 3;
    if (predict) {
        y = __fadd_rn(y, ref[0]);
        u = __fadd_rn(u, ref[1]);
        v = __fadd_rn(v, ref[2]);
    } else {
        ref[0] = y;
        ref[1] = u;
        ref[2] = v;
    }
    const float* p = st.xyz + (lb + leaf) * 3;
    const float x0 = p[0], y0 = p[1], z0 = p[2];
    const float* m = w.mv;
    const float X = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[0]), __fmul_rn(y0, m[1])), __fmul_rn(z0, m[2])), m[3]);
    const float Y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[4]), __fmul_rn(y0, m[5])), __fmul_rn(z0, m[6])), m[7]);
    const float Z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[8]), __fmul_rn(y0, m[9])), __fmul_rn(z0, m[10])), m[11]);
    const float du = __fsub_rn(u, 128.0f), dv = __fsub_rn(v, 128.0f);
    const float R = __fadd_rn(y, __fmul_rn(1.4020f, dv));
    const float G = __fsub_rn(__fsub_rn(y, __fmul_rn(0.3441f, du)), __fmul_rn(0.7141f, dv));
    const float B = __fadd_rn(y, __fmul_rn(1.7720f, du));
    const uint64_t oi = w.out_off + leaf;
    if (o.xyz) {
        o.xyz[oi * 3 + 0] = X;
        o.xyz[oi * 3 + 1] = Y;
        o.xyz[oi * 3 + 2] = Z;
    }
    if (o.rgb) {
        o.rgb[oi * 3 + 0] = to_u8(R);
        o.rgb[oi * 3 + 1] = to_u8(G);
        o.rgb[oi * 3 + 2] = to_u8(B);
    }
    if (o.p24) {  // CUDA2OpenGL.cu:44-58: unrounded /255, patches under 10 points white
        float* q = o.p24 + oi * 6;
        const bool white = w.n < 10;
        q[0] = X;
        q[1] = Y;
        q[2] = Z;
        q[3] = white ? 1.0f : __fdiv_rn(R, 255.0f);
        q[4] = white ? 1.0f : __fdiv_rn(G, 255.0f);
        q[5] = white ? 1.0f : __fdiv_rn(B, 255.0f);
    }
}

template <int T>
__global__ void __launch_bounds__(T) k_raht(const SliceWork* __restrict__ work, int first_item, StateView st,
                                            const float* __restrict__ coef, float* __restrict__ fallback,
                                            const int32_t* __restrict__ tstatus, const int32_t* __restrict__ rstatus,
                                            int32_t* __restrict__ fstatus, OutPtrs o, int wcap) {
    extern __shared__ float s_g[];  // [2][wcap][3]
    __shared__ SlotInfo s_info;
    __shared__ int s_err;
    const int item = first_item + blockIdx.x;
    const SliceWork& w = work[item];
    const int tid = threadIdx.x;
    const bool predict = (w.type & PVVC_TYPE_PREDICT) != 0;

    if (tid == 0) {
        // status priority: slice type, then the tree (intra) or the reference
        // (predictive), then the colour stream
        int err = PVVC_OK;
        if (!(w.type & PVVC_TYPE_VALID)) err = PVVC_ERR_BAD_SLICE;
        else if (!predict) err = tstatus[item];
        if (!err) {
            s_info = st.info[w.slot];
            if (!s_info.valid) err = PVVC_ERR_NO_REFERENCE;
            else if ((uint32_t)s_info.leaves != w.n) err = PVVC_ERR_SIZE;
            else if (s_info.max_width > wcap && (w.fb_off == ~0ull || s_info.max_width > (int)w.n)) err = PVVC_ERR_TREE;
        }
        if (!err) err = rstatus[item];
        // an intra slice that fails leaves its slot without a reference
        if (err && !predict && (w.type & PVVC_TYPE_VALID)) st.info[w.slot].valid = 0;
        s_err = err;
        fstatus[item] = err;
        if (o.status) o.status[w.orig] = err;
    }
    __syncthreads();
    if (s_err) return;

    const int H = s_info.height;
    const size_t nb = (size_t)w.slot * st.max_nodes;
    const size_t lb = (size_t)w.slot * st.max_leaves;
    const uint32_t N = w.n;
    const float* cy = coef + w.coef_off;
    const float* cu = cy + N;
    const float* cv = cu + N;

    if (H == 1) {
        if (tid == 0) emit_leaf(w, st, lb, 0, cy[0], cu[0], cv[0], predict, o);
        return;
    }
    float *gA, *gB;
    int cap;
    if (s_info.max_width <= wcap) {
        gA = s_g;
        gB = s_g + 3 * wcap;
        cap = wcap;
    } else {
        gA = fallback + w.fb_off;
        gB = gA + 3ull * N;
        cap = (int)N;
    }
    (void)cap;
    if (tid == 0) {
        gA[0] = cy[0];
        gA[1] = cu[0];
        gA[2] = cv[0];
    }
    __syncthreads();

    for (int l = 0; l < H - 1; ++l) {
        const int a = s_info.level_start[l], b = s_info.level_start[l + 1];
        const bool last = (l == H - 2);
        for (int j = tid; j < b - a; j += T) {
            const size_t node = nb + a + j;
            const uint32_t byte = st.occ[node], m = st.mask[node], cb = st.cbase[node];
            uint32_t ci = st.coff[node];
            float sy[16], su[16], sv[16];
            sy[1] = gA[3 * j];
            su[1] = gA[3 * j + 1];
            sv[1] = gA[3 * j + 2];
#pragma unroll
            for (int i = 1; i < 8; ++i) {
                const float2 t = st.ab[node * 7 + (i - 1)];
                float hy = 0.f, hu = 0.f, hv = 0.f;
                if (m & (1u << i)) {
                    hy = cy[ci];
                    hu = cu[ci];
                    hv = cv[ci];
                    ++ci;
                }
                const float gy = sy[i], gu = su[i], gv = sv[i];
                const float nbv = -t.y;
                // [G;H] = [[a,-b],[b,a]] [g;h]   (InvertHaarTransform)
                sy[pair0(i)] = __fadd_rn(__fmul_rn(gy, t.x), __fmul_rn(hy, nbv));
                su[pair0(i)] = __fadd_rn(__fmul_rn(gu, t.x), __fmul_rn(hu, nbv));
                sv[pair0(i)] = __fadd_rn(__fmul_rn(gv, t.x), __fmul_rn(hv, nbv));
                sy[pair1(i)] = __fadd_rn(__fmul_rn(gy, t.y), __fmul_rn(hy, t.x));
                su[pair1(i)] = __fadd_rn(__fmul_rn(gu, t.y), __fmul_rn(hu, t.x));
                sv[pair1(i)] = __fadd_rn(__fmul_rn(gv, t.y), __fmul_rn(hv, t.x));
            }
            uint32_t r = 0;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (!(byte & (0x80u >> c))) continue;
                const uint32_t child = cb + r;
                ++r;
                if (!last) {
                    gB[3 * child] = sy[8 + c];
                    gB[3 * child + 1] = su[8 + c];
                    gB[3 * child + 2] = sv[8 + c];
                } else {
                    emit_leaf(w, st, lb, child, sy[8 + c], su[8 + c], sv[8 + c], predict, o);
                }
            }
        }
        __syncthreads();
        float* t = gA;
        gA = gB;
        gB = t;
    }
}

// ---------------------------------------------------------------------------
// launchers (host)
constexpr int kTreeThreads = 256;
constexpr int kRahtThreads = 128;

cudaError_t launch_tree(const SliceWork* work, int nintra, const uint8_t* payload, const StateView& st, int32_t* tstatus,
                        cudaStream_t s) {
    if (nintra <= 0) return cudaSuccess;
    k_tree<kTreeThreads><<<nintra, kTreeThreads, 0, s>>>(work, payload, st, tstatus);
    return cudaGetLastError();
}

cudaError_t launch_rlgr(const SliceWork* work, const int32_t* order, int nslices, const uint8_t* payload, float* coef,
                        int32_t* rstatus, cudaStream_t s) {
    if (nslices <= 0) return cudaSuccess;
    k_rlgr<<<(nslices + 127) / 128, 128, 0, s>>>(work, order, nslices, payload, coef, rstatus);
    return cudaGetLastError();
}

cudaError_t launch_raht(const SliceWork* work, int first, int count, const StateView& st, const float* coef, float* fallback,
                        const int32_t* tstatus, const int32_t* rstatus, int32_t* fstatus, float* xyz, uint8_t* rgb, float* p24,
                        int32_t* status, int wcap, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    const size_t smem = 2ull * wcap * 3 * sizeof(float);
    static bool attr_set = false;
    if (!attr_set) {
        cudaFuncSetAttribute(k_raht<kRahtThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
        attr_set = true;
    }
    OutPtrs o{xyz, rgb, p24, status};
    k_raht<kRahtThreads><<<count, kRahtThreads, smem, s>>>(work, first, st, coef, fallback, tstatus, rstatus, fstatus, o, wcap);
    return cudaGetLastError();
}

}  // namespace pvvc
