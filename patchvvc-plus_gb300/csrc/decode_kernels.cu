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

#include <mutex>

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
// k_rlgr
//
// Bit window: 64 bits `hi:lo` of the stream with the next bit at bit `o`
// (0..31, counted from the MSB) of `hi`: peek() returns the next 32 bits with
// one funnel shift, advance(n <= 32) consumes n of them and takes the next
// word into the window when `o` passes 32.  Words come from 16-byte payload
// blocks staged in shared memory: each thread owns a ring of kRing block
// slots (slot j of thread t at s_ring[j * blockDim + t], so a warp's 16-byte
// reads are conflict-free), filled by cp.async kRing - 1 blocks -- about 75
// loop iterations -- ahead of their use, so the serial chain does not wait
// on global memory.  `cur` holds the words of the current block not yet
// taken (the next one in cur.x).  Blocks past the payload are zero-filled.
constexpr int kRing = 4;

__device__ __forceinline__ void ring_fetch(uint4* slot, const uint4* src, bool valid) {
    const uint32_t d = (uint32_t)__cvta_generic_to_shared(slot);
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(d), "l"(src), "r"(valid ? 16 : 0) : "memory");
    asm volatile("cp.async.commit_group;\n" ::: "memory");
}
// every block but the kRing - 2 most recently requested has landed
__device__ __forceinline__ void ring_wait() { asm volatile("cp.async.wait_group %0;\n" ::"n"(kRing - 2) : "memory"); }

struct BitReader {
    const uint4* p;      // next block to request
    const uint4* end;    // one past the last block holding payload bytes
    const uint4* first;  // the slice's first block
    uint4* ring;         // this thread's slot 0
    uint32_t stride;     // between slots (uint4 units)
    uint32_t rb;         // blocks read from the ring
    uint4 cur;
    uint32_t ci;         // words left in cur
    uint32_t hi, lo;
    uint32_t o;

    __device__ __forceinline__ static uint32_t be(uint32_t w) { return __byte_perm(w, 0, 0x0123); }
    __device__ __forceinline__ void request() {  // block p into the slot of the block read last
        const bool valid = p < end;
        ring_fetch(ring + ((rb + kRing - 1) & (kRing - 1)) * stride, valid ? p : first, valid);
        ++p;
    }
    __device__ __forceinline__ uint4 next_block() {
        ring_wait();
        const uint4 v = ring[(rb & (kRing - 1)) * stride];
        request();
        ++rb;
        return v;
    }
    __device__ __forceinline__ void init(const uint8_t* payload, uint64_t off, uint32_t nbytes, uint4* ring0, uint32_t str) {
        first = p = reinterpret_cast<const uint4*>(payload + (off & ~15ull));
        end = reinterpret_cast<const uint4*>(payload + ((off + nbytes + 15) & ~15ull));
        ring = ring0;
        stride = str;
        rb = 0;
        for (int j = 0; j < kRing - 1; ++j) {  // blocks 0 .. kRing-2 into slots 0 .. kRing-2
            const bool valid = p < end;
            ring_fetch(ring + j * stride, valid ? p : first, valid);
            ++p;
        }
        const uint4 b0 = next_block();
        hi = be(b0.x);
        lo = be(b0.y);
        cur = make_uint4(b0.z, b0.w, 0u, 0u);
        ci = 2;
        o = 0;
        uint32_t skip = (uint32_t)(off & 15) * 8;  // payload bytes before the slice's first byte
        while (skip >= 32) {
            advance(32);
            skip -= 32;
        }
        advance(skip);
    }
    // the next 32 bits of the stream
    __device__ __forceinline__ uint32_t peek() const { return __funnelshift_l(lo, hi, o); }
    // consume n <= 32 bits; branch-free apart from the block refill (a lane
    // needs one about every 25 iterations)
    __device__ __forceinline__ void advance(uint32_t n) {
        o += n;
        const bool take = o >= 32;
        o &= 31u;
        hi = take ? lo : hi;
        lo = take ? be(cur.x) : lo;
        cur.x = take ? cur.y : cur.x;
        cur.y = take ? cur.z : cur.y;
        cur.z = take ? cur.w : cur.z;
        ci -= take ? 1u : 0u;
        if (ci == 0) {
            cur = next_block();
            ci = 4;
        }
    }
    // payload bits consumed: the words that entered the window before hi,
    // plus o, minus the bytes before the slice in its first block
    __device__ __forceinline__ int64_t consumed(uint64_t off) const {
        const int64_t words = (int64_t)rb * 4 - (int64_t)ci;  // entered the window
        return (words - 2) * 32 + (int64_t)o - (int64_t)(off & 15) * 8;
    }
    // no copy of this thread's left in flight (before its shared memory is reused)
    __device__ __forceinline__ void drain() const { asm volatile("cp.async.wait_all;\n" ::: "memory"); }
};

constexpr uint32_t kRlU0 = 3, kRlU1 = 2, kRlD0 = 1, kRlD1 = 1, kRlMaxRP = 32 * 4;

// Zero-run length of `c` leading ones read in run mode from state kP
// (entropy_codec.cc:228-233): the i-th one stands for 2^((kP + 2i) >> 2)
// zeros, kP growing by U1 = 2 per one, so the exponents go in pairs.  With
// S(n) = sum_{i<n} 2^(i>>1) = 2 (2^(n>>1) - 1) + (n & 1) 2^(n>>1):
//   kP & 3 in {0,1}:  sum = 2^(kP>>2) S(c)
//   kP & 3 in {2,3}:  sum = 2^(kP>>2) (S(c+1) - 1)
// Every term is below 2^k with k = (kP + 2c) >> 2, so when the whole run code
// (c ones, a zero, k bits) fits 32 bits the length fits 32 bits too.
__device__ __forceinline__ uint32_t run_ones_length(uint32_t kP, uint32_t c) {
    const uint32_t hi = (kP >> 1) & 1u;  // exponent pairs start one late
    const uint32_t n = c + hi;
    const uint32_t h = 1u << (n >> 1);
    const uint32_t S = 2 * (h - 1) + (n & 1u) * h - hi;
    return S << (kP >> 2);
}

// bits [at, at + k) of w (k <= 32; k = 0 gives 0, and so does at >= 32)
__device__ __forceinline__ uint32_t field(uint32_t w, uint32_t at, uint32_t k) {
    return __funnelshift_rc(__funnelshift_lc(0u, w, at), 0u, 32u - k);
}

// k_rlgr: one thread per slice.  The coefficient planes are zeroed before the
// launch, so a run of zeros only moves the output position; symbol j of a
// plane goes to coefficient N-1-j (the stream is reversed).  The loop keeps
// 32-bit state only: `dst` walks down the current plane, `rem` counts the
// plane's symbols still to come, `left` all symbols still to come.
//
// One iteration = an optional zero run (run mode, kP >= 4) followed by one
// Golomb-Rice symbol.  The common case -- run code and symbol code together
// within the next 32 bits, a symbol below 2^23, the run inside the current
// plane -- is one branch-free line that every lane of a warp executes in
// step, whatever mode its slice is in (a lane outside run mode computes an
// empty run): the run's leading ones are counted with one clz and summed in
// closed form (run_ones_length), the symbol's ones with a second clz on the
// same 32 bits, and one advance consumes both.  Its dependent chain is about
// fifteen integer operations.  All other iterations (longer codes, the
// 32-ones escape, wide symbols, runs across a plane or to the end of the
// slice) take the general path, which reads the codes piece by piece as the
// reference does; at q = 8 about one lane-iteration in 4,000 goes there.
//
// LANES < 32: only the first LANES lanes of each warp decode (the rest exit at
// once), so a warp executes the union of fewer lanes' paths per iteration --
// for the longest slices, whose serial chains set the kernel's length.
template <int T, int LANES = 32>
__global__ void __launch_bounds__(T) k_rlgr(const SliceWork* __restrict__ work, const int32_t* __restrict__ order,
                                              int nslices, const uint8_t* __restrict__ payload, float* __restrict__ coef,
                                              int32_t* __restrict__ rstatus) {
    const int g = blockIdx.x * blockDim.x + threadIdx.x;
    if ((g & 31) >= LANES) return;
    const int t = (g >> 5) * LANES + (g & 31);
    if (t >= nslices) return;
    const int item = order[t];
    const SliceWork& wk = work[item];
    const uint32_t N = wk.n;
    const int32_t qp = wk.qp;
    if (N == 0) {
        rstatus[item] = PVVC_OK;
        return;
    }
    const uint64_t off = wk.col_off;
    const uint32_t csz = wk.csz;
    extern __shared__ uint4 s_ring[];  // kRing * blockDim payload blocks
    BitReader br;
    br.init(payload, off, csz, s_ring + threadIdx.x, blockDim.x);
    const uint32_t csh = wk.coef_stride == 32 ? 5u : 0u;   // coefficient stride 32 (group region) or 1
    const int64_t cs = (int64_t)1 << csh;
    const int64_t wrap = (int64_t)(2 * N - 1) << csh;       // last coefficient of a plane -> top of the next
    float* dst = coef + wk.coef_off + ((uint64_t)(N - 1) << csh) + wk.coef_lane;  // coefficient of the next symbol
    uint32_t rem = N;                         // symbols left in the current plane
    uint32_t left = 3u * N;                   // symbols left in the slice
    uint32_t kP = 0, kRP = 8;
    int err = PVVC_OK;
    for (;;) {
        // ---- common case: the whole iteration within the next 32 bits ----
        const uint32_t v = br.peek();
        const bool run = kP >= 4;
        const uint32_t c = run ? __clz(~v) : 0u;   // leading ones of the run code
        const uint32_t kP2 = kP + 2 * c;           // kP after the ones
        const uint32_t k = run ? (kP2 >> 2) : 0u;  // remainder bits of the run code
        const uint32_t r = run ? c + 1 + k : 0u;   // bits of the run code
        const uint32_t v2 = __funnelshift_lc(0u, v, r);  // the symbol's code, left-aligned
        const uint32_t q = __clz(~v2);             // its leading ones
        const uint32_t kR = kRP >> 2;
        const uint32_t nb = r + q + 1 + kR;        // bits of the whole iteration
        const uint32_t u = (q << kR) | field(v2, q + 1, kR);
        const uint32_t m = run ? run_ones_length(kP, c) + field(v, c + 1, k) : 0u;  // zeros of the run
        if (nb <= 32 && u < (1u << 23) && m < rem) {
            br.advance(nb);
            dst -= (int64_t)m << csh;
            const uint32_t zz = u + (uint32_t)run;  // Unsign2Sign(u + after_run) * qp, stored unless zero
            const int32_t sym = (int32_t)(zz >> 1) ^ -(int32_t)(zz & 1);
            if (sym) *dst = __int2float_rn(sym * qp);
            // adaptation (entropy_codec.cc:245-281); here p = u >> kR = q
            kRP = q ? min(kRP + q - 1, kRlMaxRP) : (kRP < 2 ? 0u : kRP - 2);
            kP = (run || u) ? (kP2 ? kP2 - kRlD1 : 0u) : kP2 + kRlU0;  // D0 = D1 = 1
            left -= m + 1;
            rem -= m + 1;
            const bool end_of_plane = rem == 0;
            dst += end_of_plane ? wrap : -cs;
            rem = end_of_plane ? N : rem;
            if (left == 0) break;
            continue;
        }
        // ---- general path: the codes read piece by piece ----
        uint32_t mm = 0;   // zeros in the run
        uint32_t kPr = kP;  // kP after the run's ones
        if (run) {
            // zero run (entropy_codec.cc:226-233): ones, a zero, k remainder bits
            uint64_t m64 = 0;
            uint32_t kk = kP >> 2;
            uint32_t cc;
            int guard = 0;
            do {
                cc = __clz(~br.peek());
                for (uint32_t i = 0; i < cc; ++i) {
                    m64 += 1ull << (kk & 31);
                    kPr += kRlU1;
                    kk = kPr >> 2;
                }
                br.advance(cc);
            } while (cc == 32 && ++guard < 64);
            br.advance(1);
            if (kk > 31) {
                err = PVVC_ERR_OVERRUN;
                break;
            }
            m64 += br.peek() >> (32 - kk);
            br.advance(kk);
            mm = m64 > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)m64;
        }
        // skip mm zeros (they may cross plane boundaries)
        {
            uint32_t z = mm < left ? mm : left;
            left -= z;
            while (z >= rem && rem) {
                z -= rem;
                dst += (int64_t)(2 * N - rem) << csh;  // to the top of the next plane
                rem = N;
            }
            dst -= (int64_t)z << csh;
            rem -= z;
        }
        if (left == 0) break;
        // Golomb-Rice symbol (GRRead, entropy_codec.cc:196-205)
        const uint32_t w = br.peek();
        const uint32_t qq = __clz(~w);
        uint64_t uw;
        uint32_t pq;
        if (qq < 32) {
            br.advance(qq + 1);
            uint32_t rr = 0;
            if (kR) {
                rr = kR >= 32 ? br.peek() : (br.peek() >> (32 - kR));
                br.advance(kR >= 32 ? 32u : kR);
            }
            uw = ((uint64_t)qq << kR) | rr;
            pq = qq;
        } else {  // 32 ones: a raw 32-bit value follows
            br.advance(32);
            const uint32_t raw = br.peek();
            br.advance(32);
            uw = raw;
            // p may be far above the kRP cap; any p > kRlMaxRP saturates
            // kRP + p - 1 at the cap (kRP >= 0), so clamp p to kRlMaxRP + 1,
            // not kRlMaxRP (that would leave kRP one short when kRP = 0)
            const uint32_t t2 = kR >= 32 ? 0u : (raw >> kR);
            pq = t2 > kRlMaxRP ? kRlMaxRP + 1 : t2;
        }
        kRP = pq ? min(kRP + pq - 1, kRlMaxRP) : (kRP < 2 ? 0u : kRP - 2);
        kP = (run || uw) ? (kPr ? kPr - kRlD1 : 0u) : kPr + kRlU0;
        {
            const uint64_t zz = uw + (uint64_t)run;
            const long long sym = (long long)(zz >> 1) ^ -(long long)(zz & 1);
            if (sym) *dst = __ll2float_rn(sym * (long long)qp);
        }
        --left;
        const bool end_of_plane = --rem == 0;
        dst += end_of_plane ? wrap : -cs;
        rem = end_of_plane ? N : rem;
        if (left == 0) break;
    }
    // bits consumed vs the payload (the reference reads past it, which is undefined)
    if (!err) {
        if (br.consumed(off) > 8ll * csz) err = PVVC_ERR_OVERRUN;
    }
    br.drain();
    rstatus[item] = err;
}

// ---------------------------------------------------------------------------
// k_rlgr_win: RLGR of the slices of one group (the frames of one patch, all
// of the same size N), one warp per group, lane l decoding the group's slice
// l.  The group's coefficients live in its frame-interleaved region: stream
// position s of every lane's slice (plane s / N, coefficient N-1 - s % N)
// is one 128-byte line, lane l's word at offset l.
//
// Instead of scattered 4-byte stores into planes cleared beforehand, each
// lane stages its nonzero symbols in a shared-memory window of WROWS rows
// (row r = stream position r: the 32 lanes' words of that line, their eight
// 16-byte chunks XOR-swizzled by r & 7).  Every kWinCheck iterations the
// warp takes the smallest position any lane can still write
// (__reduce_min_sync); rows below it are final for every lane.  Each full
// unit of 32 final rows is written out with lane l taking row unit + l:
// eight 16-byte loads of its row (conflict-free thanks to the swizzle), eight
// 16-byte stores of the whole line, zeros included, and the row cleared.  A
// lane whose next symbol lands beyond the window keeps it pending and pauses
// until the window reaches it.  So the planes need no clear, every line is
// written once, in full, and no partially written line ever leaves L2.
//
// The decode loop is k_rlgr's with linear stream positions: the common path
// also takes runs that cross a plane boundary.  Every round of the loop
// either consumes a symbol in some lane or moves the window forward (a
// paused lane's position is at least WROWS rows ahead of the window, so the
// minimum has passed a whole unit), so the loop ends after at most 3N rounds
// per lane plus one flush per unit of rows.
constexpr uint32_t kWinCheck = 4;        // iterations between window checks (a multiple of 2)
constexpr uint32_t kWinUnit = 32;        // rows written out together (one per lane)
constexpr int kWinRows = 64;             // window rows (8 KB per warp)

// shared memory of a windowed CTA: rings and windows, at least 16 KB (with
// the 1 KB the SM keeps per CTA, more than the 15 KB a long per-slice CTA's
// SM has left)
constexpr int kWinMinSmem = 16 * 1024;
__host__ __device__ constexpr int win_smem(int warps, int rows) {
    return warps * (32 * kRing * 16 + rows * 32 * 4) > kWinMinSmem ? warps * (32 * kRing * 16 + rows * 32 * 4)
                                                                   : kWinMinSmem;
}

template <int WARPS, int WROWS>
__global__ void __launch_bounds__(32 * WARPS) k_rlgr_win(const SliceWork* __restrict__ work,
                                                         const GroupDesc* __restrict__ groups, int ngroups,
                                                         const int32_t* __restrict__ items,
                                                         const uint8_t* __restrict__ payload, float* __restrict__ coef,
                                                         int32_t* __restrict__ rstatus) {
    static_assert((WROWS & (WROWS - 1)) == 0 && WROWS >= 2 * (int)kWinUnit, "window rows: a power of two");
    extern __shared__ uint4 s_dyn[];  // [kRing][blockDim] payload blocks, then [WARPS][WROWS][32] floats
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int gi = blockIdx.x * WARPS + wid;
    if (gi >= ngroups) return;  // the whole warp
    float* const win = reinterpret_cast<float*>(s_dyn + kRing * blockDim.x) + (size_t)wid * WROWS * 32;
    // word of (row r, lane) in the window: chunk (lane / 4) ^ (r & 7), word lane % 4
    auto slot = [&](uint32_t r) { return ((r & (WROWS - 1)) << 5) + ((((uint32_t)lane >> 2) ^ (r & 7u)) << 2) + (lane & 3); };
    const GroupDesc G = groups[gi];
    const int item0 = items[G.first];
    const uint32_t N = work[item0].n;
    const uint32_t total = 3u * N;
    const uint64_t region = work[item0].coef_off;
    const int item = lane < G.count ? items[G.first + lane] : -1;
    for (int i = lane; i < WROWS * 8; i += 32) reinterpret_cast<float4*>(win)[i] = make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();  // rows are cleared by all lanes, then written by their owners
    BitReader br;
    bool done = true, pend = false;
    int err = PVVC_OK;
    int32_t qp = 0;
    uint64_t off = 0;
    uint32_t csz = 0;
    if (item >= 0) {
        const SliceWork& wk = work[item];
        if (wk.n != N) {
            rstatus[item] = PVVC_ERR_SIZE;  // the planner keeps such slices out of window groups
        } else if (N == 0) {
            rstatus[item] = PVVC_OK;
        } else {
            qp = wk.qp;
            off = wk.col_off;
            csz = wk.csz;
            br.init(payload, off, csz, s_dyn + threadIdx.x, blockDim.x);
            done = false;
        }
    }
    uint32_t s = 0;                 // stream position of this lane's next symbol
    uint32_t kP = 0, kRP = 8;
    uint32_t pend_q = 0;            // a pending symbol's position and value
    float pend_v = 0.f;
    uint32_t base = 0;              // rows below `base` are written out (warp-uniform)
    uint32_t bp = 0, bc = N - 1;    // plane and coefficient index of row `base`
    for (uint32_t it = 1;; ++it) {
        if (!done && !pend) {
            uint32_t q = 0xFFFFFFFFu;  // position of a nonzero symbol decoded in this iteration
            float val = 0.f;
            // ---- common case: the whole iteration within the next 32 bits ----
            const uint32_t v = br.peek();
            const bool run = kP >= 4;
            const uint32_t c = run ? __clz(~v) : 0u;
            const uint32_t kP2 = kP + 2 * c;
            const uint32_t k = run ? (kP2 >> 2) : 0u;
            const uint32_t r = run ? c + 1 + k : 0u;
            const uint32_t v2 = __funnelshift_lc(0u, v, r);
            const uint32_t qq = __clz(~v2);
            const uint32_t kR = kRP >> 2;
            const uint32_t nb = r + qq + 1 + kR;
            const uint32_t u = (qq << kR) | field(v2, qq + 1, kR);
            const uint32_t m = run ? run_ones_length(kP, c) + field(v, c + 1, k) : 0u;
            if (nb <= 32 && u < (1u << 23) && m < total - s) {
                br.advance(nb);
                const uint32_t zz = u + (uint32_t)run;
                const int32_t sym = (int32_t)(zz >> 1) ^ -(int32_t)(zz & 1);
                if (sym) {
                    q = s + m;
                    val = __int2float_rn(sym * qp);
                }
                kRP = qq ? min(kRP + qq - 1, kRlMaxRP) : (kRP < 2 ? 0u : kRP - 2);
                kP = (run || u) ? (kP2 ? kP2 - kRlD1 : 0u) : kP2 + kRlU0;
                s += m + 1;
            } else {
                // ---- general path: the codes read piece by piece ----
                uint32_t mm = 0, kPr = kP;
                if (run) {
                    uint64_t m64 = 0;
                    uint32_t kk = kP >> 2;
                    uint32_t cc;
                    int guard = 0;
                    do {
                        cc = __clz(~br.peek());
                        for (uint32_t i = 0; i < cc; ++i) {
                            m64 += 1ull << (kk & 31);
                            kPr += kRlU1;
                            kk = kPr >> 2;
                        }
                        br.advance(cc);
                    } while (cc == 32 && ++guard < 64);
                    br.advance(1);
                    if (kk > 31) {
                        err = PVVC_ERR_OVERRUN;
                    } else {
                        m64 += br.peek() >> (32 - kk);
                        br.advance(kk);
                        mm = m64 > 0xFFFFFFFFull ? 0xFFFFFFFFu : (uint32_t)m64;
                    }
                }
                if (!err) {
                    s += min(mm, total - s);  // zeros, possibly across planes
                    if (s < total) {
                        const uint32_t w = br.peek();
                        const uint32_t qw = __clz(~w);
                        uint64_t uw;
                        uint32_t pw;
                        if (qw < 32) {
                            br.advance(qw + 1);
                            uint32_t rr = 0;
                            if (kR) {
                                rr = kR >= 32 ? br.peek() : (br.peek() >> (32 - kR));
                                br.advance(kR >= 32 ? 32u : kR);
                            }
                            uw = ((uint64_t)qw << kR) | rr;
                            pw = qw;
                        } else {  // 32 ones: a raw 32-bit value follows (see k_rlgr on the clamp)
                            br.advance(32);
                            const uint32_t raw = br.peek();
                            br.advance(32);
                            uw = raw;
                            const uint32_t t2 = kR >= 32 ? 0u : (raw >> kR);
                            pw = t2 > kRlMaxRP ? kRlMaxRP + 1 : t2;
                        }
                        kRP = pw ? min(kRP + pw - 1, kRlMaxRP) : (kRP < 2 ? 0u : kRP - 2);
                        kP = (run || uw) ? (kPr ? kPr - kRlD1 : 0u) : kPr + kRlU0;
                        const uint64_t zz = uw + (uint64_t)run;
                        const long long sym = (long long)(zz >> 1) ^ -(long long)(zz & 1);
                        if (sym) {
                            q = s;
                            val = __ll2float_rn(sym * (long long)qp);
                        }
                        ++s;
                    }
                }
            }
            if (q != 0xFFFFFFFFu) {
                if (q - base < (uint32_t)WROWS) {
                    win[slot(q)] = val;
                } else {
                    pend = true;
                    pend_q = q;
                    pend_v = val;
                }
            }
            if (err || s >= total) {
                done = true;
                // bits consumed vs the payload (the reference reads past it, which is undefined)
                if (!err && br.consumed(off) > 8ll * csz) err = PVVC_ERR_OVERRUN;
                br.drain();
                rstatus[item] = err;
            }
        }
        if (it % kWinCheck) continue;
        // ---- the window (warp-uniform) ----
        const uint32_t lb = pend ? pend_q : (done ? total : s);  // this lane writes no row below lb
        const uint32_t mn = __reduce_min_sync(0xffffffffu, lb);
        if (mn - base < kWinUnit && mn < total) continue;
        // write out whole units of final rows (and at the end the last,
        // partial one); rows from base + WROWS on were never staged: zeros
        const uint32_t lim = base + WROWS;
        const uint32_t stop = mn == total ? total : base + (mn - base) / kWinUnit * kWinUnit;
        __syncwarp();  // every lane's staged words are visible to the row's owner
        while (base < stop) {
            const uint32_t r = base + (uint32_t)lane;  // this lane's row
            if (r < stop) {
                // its plane and coefficient, from row base's: lane rows down
                uint32_t p = bp, c = bc;
                uint32_t d = (uint32_t)lane;
                while (d > c) {  // past the plane's coefficient 0: to the top of the next
                    d -= c + 1;
                    c = N - 1;
                    ++p;
                }
                c -= d;
                float4* dst = reinterpret_cast<float4*>(coef + region + (((uint64_t)p * N + c) << 5));
                if (r < lim) {
                    float4* row = reinterpret_cast<float4*>(win + ((r & (WROWS - 1)) << 5));
#pragma unroll
                    for (uint32_t j = 0; j < 8; ++j) {
                        const uint32_t pj = j ^ (r & 7u);
                        dst[j] = row[pj];
                        row[pj] = make_float4(0.f, 0.f, 0.f, 0.f);
                    }
                } else {
#pragma unroll
                    for (uint32_t j = 0; j < 8; ++j) dst[j] = make_float4(0.f, 0.f, 0.f, 0.f);
                }
            }
            // row base += one unit (warp-uniform)
            uint32_t d = kWinUnit;
            while (d > bc) {
                d -= bc + 1;
                bc = N - 1;
                ++bp;
            }
            bc -= d;
            base += kWinUnit;
        }
        base = stop;
        __syncwarp();  // cleared rows before their owners' next writes
        if (pend && pend_q - base < (uint32_t)WROWS) {
            win[slot(pend_q)] = pend_v;
            pend = false;
        }
        if (mn == total) break;
    }
}

// ---------------------------------------------------------------------------
// k_raht
struct OutPtrs {
    float* xyz;
    uint8_t* rgb;
    float* p24;
    int32_t* status;  // caller's status, indexed by SliceWork::orig (may be null)
};

// std::round (half away from zero), clamped to [0, 255].  Clamping first
// commutes with the rounding (it is monotone and 0 and 255 are integers);
// for a clamped c >= 0, round(c) = floor(c + 0.5), and the sum rounded
// toward -inf keeps that floor exact, since every integer is a float.  NaN
// clamps to 0, as fmaxf(roundf(NaN), 0) does.
__device__ __forceinline__ uint8_t to_u8(float v) {
    const float c = fminf(fmaxf(v, 0.0f), 255.0f);
    return (uint8_t)__float2uint_rd(__fadd_rd(c, 0.5f));
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

// Inverse hierarchical transform of one internal node (octree_base.cc:84-100):
// the node's DC `g` and its coded coefficients -> the 8 child slots (absent
// children's slots hold values nobody reads).
__device__ __forceinline__ void inverse_node(const StateView& st, size_t node, const float* __restrict__ cy,
                                             const float* __restrict__ cu, const float* __restrict__ cv, float gy, float gu,
                                             float gv, float (&oy)[8], float (&ou)[8], float (&ov)[8]) {
    const uint32_t m = st.mask[node];
    uint32_t ci = st.coff[node];
    const float2* ab = st.ab + node * 7;
    float sy[8], su[8], sv[8];  // slots 1..7 (index 0 unused)
    sy[1] = gy;
    su[1] = gu;
    sv[1] = gv;
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        const float2 t = ab[i - 1];
        float hy = 0.f, hu = 0.f, hv = 0.f;
        if (m & (1u << i)) {
            hy = cy[ci];
            hu = cu[ci];
            hv = cv[ci];
            ++ci;
        }
        const float ay = sy[i], au = su[i], av = sv[i];
        const float nbv = -t.y;
        // [G;H] = [[a,-b],[b,a]] [g;h]   (InvertHaarTransform, octree_base.cc:186-206)
        const float Gy = __fadd_rn(__fmul_rn(ay, t.x), __fmul_rn(hy, nbv));
        const float Gu = __fadd_rn(__fmul_rn(au, t.x), __fmul_rn(hu, nbv));
        const float Gv = __fadd_rn(__fmul_rn(av, t.x), __fmul_rn(hv, nbv));
        const float Hy = __fadd_rn(__fmul_rn(ay, t.y), __fmul_rn(hy, t.x));
        const float Hu = __fadd_rn(__fmul_rn(au, t.y), __fmul_rn(hu, t.x));
        const float Hv = __fadd_rn(__fmul_rn(av, t.y), __fmul_rn(hv, t.x));
        if (pair0(i) < 8) {
            sy[pair0(i)] = Gy; su[pair0(i)] = Gu; sv[pair0(i)] = Gv;
            sy[pair1(i)] = Hy; su[pair1(i)] = Hu; sv[pair1(i)] = Hv;
        } else {
            oy[pair0(i) - 8] = Gy; ou[pair0(i) - 8] = Gu; ov[pair0(i) - 8] = Gv;
            oy[pair1(i) - 8] = Hy; ou[pair1(i) - 8] = Hu; ov[pair1(i) - 8] = Hv;
        }
    }
}

// Status of one slice before its inverse RAHT.  Priority: slice type, then
// the tree (intra) or the reference (predictive), then the colour stream.
__device__ __forceinline__ int slice_status(const SliceWork& w, int item, const StateView& st, const int32_t* tstatus,
                                            const int32_t* rstatus) {
    const bool predict = (w.type & PVVC_TYPE_PREDICT) != 0;
    int err = PVVC_OK;
    if (!(w.type & PVVC_TYPE_VALID)) err = PVVC_ERR_BAD_SLICE;
    else if (!predict) err = tstatus[item];
    if (!err) {
        const SlotInfo* si = st.info + w.slot;
        if (!si->valid) err = PVVC_ERR_NO_REFERENCE;
        else if ((uint32_t)si->leaves != w.n) err = PVVC_ERR_SIZE;
    }
    if (!err) err = rstatus[item];
    return err;
}

// k_raht_slice: one CTA per slice, level-synchronous over all internal levels
// with the level signal in shared memory (global fallback for wide levels).
// Used for slices that share their tree with few others in the batch.
template <int T>
__global__ void __launch_bounds__(T) k_raht_slice(const SliceWork* __restrict__ work, const int32_t* __restrict__ list,
                                                  StateView st, const float* __restrict__ coef, float* __restrict__ fallback,
                                                  const int32_t* __restrict__ tstatus, const int32_t* __restrict__ rstatus,
                                                  int32_t* __restrict__ fstatus, OutPtrs o, int wcap) {
    extern __shared__ float s_g[];  // [2][wcap][3]
    __shared__ SlotInfo s_info;
    __shared__ int s_err;
    const int item = list[blockIdx.x];
    const SliceWork& w = work[item];
    const int tid = threadIdx.x;
    const bool predict = (w.type & PVVC_TYPE_PREDICT) != 0;
    if (tid == 0) {
        int err = slice_status(w, item, st, tstatus, rstatus);
        if (!err) {
            s_info = st.info[w.slot];
            if (s_info.max_width > wcap && (w.fb_off == ~0ull || s_info.max_width > (int)w.n)) err = PVVC_ERR_TREE;
        }
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
    if (s_info.max_width <= wcap) {
        gA = s_g;
        gB = s_g + 3 * wcap;
    } else {
        gA = fallback + w.fb_off;
        gB = gA + 3ull * N;
    }
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
            const uint32_t byte = st.occ[node], cb = st.cbase[node];
            float oy[8], ou[8], ov[8];
            inverse_node(st, node, cy, cu, cv, gA[3 * j], gA[3 * j + 1], gA[3 * j + 2], oy, ou, ov);
            uint32_t r = 0;
#pragma unroll
            for (int c = 0; c < 8; ++c) {
                if (!(byte & (0x80u >> c))) continue;
                const uint32_t child = cb + r;
                ++r;
                if (!last) {
                    gB[3 * child] = oy[c];
                    gB[3 * child + 1] = ou[c];
                    gB[3 * child + 2] = ov[c];
                } else {
                    emit_leaf(w, st, lb, child, oy[c], ou[c], ov[c], predict, o);
                }
            }
        }
        __syncthreads();
        float* t = gA;
        gA = gB;
        gB = t;
    }
}

// inverse_node for a lane that may be inactive (no coefficient loads then),
// given the node's coded-slot mask `m`, first coefficient `ci` and butterfly
// pairs ab[i * AS] (AS = 1: the state's node record; 32: a warp's staged
// rows).  Coded slot i reads coefficient ci + (coded slots below i), so the
// node's coefficient loads are independent and issue together.
//
// `m` is the same in every lane (the lanes share the tree), so each slot's
// branch is uniform.  An uncoded butterfly has a zero weight on one side
// and h = 0: with (a, b) = (1, 0), G = g*1 + 0*(-0) = g exactly and H feeds
// only the empty side; with (0, 1), H = g*1 + 0*0 = g + 0 (+0 for g = -0)
// and G feeds only the empty side; with both weights zero neither is read.
// So G = g, H = g + 0 reproduce every value a child can see.
template <int S, int AS>  // coefficient stride (32 in frame-interleaved group regions), ab stride
__device__ __forceinline__ void lane_node_md(uint32_t m, uint32_t ci, const float2* ab, bool act, const float* cy,
                                             const float* cu, const float* cv, float gy, float gu, float gv,
                                             float (&oy)[8], float (&ou)[8], float (&ov)[8]) {
    float hy[8], hu[8], hv[8];
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        const bool coded = act && (m & (1u << i));
        const size_t k = (size_t)(ci + __popc(m & ((1u << i) - 2u))) * S;
        hy[i] = coded ? __ldg(cy + k) : 0.f;
        hu[i] = coded ? __ldg(cu + k) : 0.f;
        hv[i] = coded ? __ldg(cv + k) : 0.f;
    }
    float sy[8], su[8], sv[8];
    sy[1] = gy;
    su[1] = gu;
    sv[1] = gv;
#pragma unroll
    for (int i = 1; i < 8; ++i) {
        const float ay = sy[i], au = su[i], av = sv[i];
        float Gy, Gu, Gv, Hy, Hu, Hv;
        if (m & (1u << i)) {
            const float2 t = ab[(i - 1) * AS];
            const float nbv = -t.y;
            // [G;H] = [[a,-b],[b,a]] [g;h]   (InvertHaarTransform, octree_base.cc:186-206)
            Gy = __fadd_rn(__fmul_rn(ay, t.x), __fmul_rn(hy[i], nbv));
            Gu = __fadd_rn(__fmul_rn(au, t.x), __fmul_rn(hu[i], nbv));
            Gv = __fadd_rn(__fmul_rn(av, t.x), __fmul_rn(hv[i], nbv));
            Hy = __fadd_rn(__fmul_rn(ay, t.y), __fmul_rn(hy[i], t.x));
            Hu = __fadd_rn(__fmul_rn(au, t.y), __fmul_rn(hu[i], t.x));
            Hv = __fadd_rn(__fmul_rn(av, t.y), __fmul_rn(hv[i], t.x));
        } else {
            Gy = ay;
            Gu = au;
            Gv = av;
            Hy = __fadd_rn(ay, 0.0f);
            Hu = __fadd_rn(au, 0.0f);
            Hv = __fadd_rn(av, 0.0f);
        }
        if (pair0(i) < 8) {
            sy[pair0(i)] = Gy; su[pair0(i)] = Gu; sv[pair0(i)] = Gv;
            sy[pair1(i)] = Hy; su[pair1(i)] = Hu; sv[pair1(i)] = Hv;
        } else {
            oy[pair0(i) - 8] = Gy; ou[pair0(i) - 8] = Gu; ov[pair0(i) - 8] = Gv;
            oy[pair1(i) - 8] = Hy; ou[pair1(i) - 8] = Hu; ov[pair1(i) - 8] = Hv;
        }
    }
}

template <int S>
__device__ __forceinline__ void lane_node(const StateView& st, size_t node, bool act, const float* cy, const float* cu,
                                          const float* cv, float gy, float gu, float gv, float (&oy)[8], float (&ou)[8],
                                          float (&ov)[8]) {
    lane_node_md<S, 1>(__ldg(st.mask + node), __ldg(st.coff + node), st.ab + node * 7, act, cy, cu, cv, gy, gu, gv, oy, ou,
                       ov);
}

// A warp's staged node records: kRowNodes consecutive nodes of one level.
constexpr int kRowNodes = 32;
struct NodeRows {
    uint32_t occ[kRowNodes], cb[kRowNodes], mask[kRowNodes], coff[kRowNodes];
    float2 ab[7][kRowNodes];
};

// k_raht_group: persistent CTAs; each takes the next group of slices that
// share a slot (the frames of one patch) from a queue.  Lane f of every warp
// owns frame f (same control flow in all lanes, node records are broadcast
// loads).  The intra slice, when the group has one, is lane 0 and hands its
// leaf colours to the predictive lanes by shuffle.
//
// Levels above the last two internal ones: the 8 warps split each level's
// nodes and the CTA synchronises per level.  The level signal lives in the
// CTA's own scratch region as [node][yuv][lane], so each warp access is one
// 128-byte line.
//
// The last two internal levels (most of the nodes) go without a barrier or
// a level buffer: warp w takes a contiguous range of last-level nodes, whose
// leaves are contiguous too, and walks their parents alongside -- each
// parent's children DCs go to the warp's shared-memory rows [yuv][child]
// [lane] (a lane reads back only its own column), the first parent found by
// a 32-way search of the parents' child offsets.  A parent whose children
// straddle two warps' ranges is transformed by both.  The warp stages its
// finished points in its own rows [frame][leaf]; when the next node's leaves
// would not fit, it writes the staged leaves of every frame as contiguous
// runs and goes on.  Against a level buffer in global memory for the last
// internal level too, this cut the kernel's DRAM bytes by a quarter.  The
// kernel needs 80 registers without spills: 3 CTAs of 8 warps per SM.
constexpr int kGrpWarps = 8;
constexpr int kWarpLeaves = 16;              // staged leaves per warp (a node adds <= 8)
constexpr int kStageRow = kWarpLeaves + 1;   // odd row length: the 32 lanes' column stores hit 32 banks
static_assert(kWarpLeaves == 16, "the flush maps a frame's staged leaves onto a half-warp");

// A warp stages colours only: leaf centres are the same in every frame of
// the group, and the flush transforms them with each frame's matrix.
template <bool P24>
struct WarpStage {
    uint32_t rgb[32][kStageRow];
};
template <>
struct WarpStage<true> {
    uint32_t rgb[32][kStageRow];
    float fr[32][kStageRow], fg[32][kStageRow], fb[32][kStageRow];  // points24 colours
};
template <bool P24>
struct GroupStage {
    WarpStage<P24> w[kGrpWarps];
};

template <bool P24>
__global__ void __launch_bounds__(32 * kGrpWarps, 3) k_raht_group(const SliceWork* __restrict__ work,
                                                               const GroupDesc* __restrict__ groups, int ngroups,
                                                               const int32_t* __restrict__ items, StateView st,
                                                               const float* __restrict__ coef,
                                                               const int32_t* __restrict__ tstatus,
                                                               const int32_t* __restrict__ rstatus,
                                                               int32_t* __restrict__ fstatus, OutPtrs o,
                                                               float* __restrict__ scratch, uint64_t scratch_floats,
                                                               int* __restrict__ counter) {
    extern __shared__ __align__(16) unsigned char s_raw[];
    GroupStage<P24>& sg = *reinterpret_cast<GroupStage<P24>*>(s_raw);
    __shared__ int s_g, s_H, s_ls[kMaxLevels + 1];
    __shared__ uint64_t s_out[32];
    __shared__ int s_act[32], s_white[32];
    __shared__ float s_mv[32][13];  // each frame's transform rows (odd stride: the lanes' row fills hit 32 banks)
    __shared__ NodeRows s_nodes[kGrpWarps];
    __shared__ float s_dc[kGrpWarps][3][8][32];  // each warp's current parent: its children's DCs [yuv][child][lane]
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    WarpStage<P24>& ws = sg.w[wid];
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
        const bool intra_lane = have && G.intra && lane == 0;
        int err = have ? slice_status(w, item, st, tstatus, rstatus) : PVVC_OK;
        const int ierr = G.intra ? __shfl_sync(0xffffffffu, err, 0) : PVVC_OK;
        if (ierr && !intra_lane && have && !err) err = PVVC_ERR_NO_REFERENCE;
        const bool act = have && !err;
        if (wid == 0) {
            if (ierr && lane == 0) st.info[G.slot].valid = 0;  // a failed intra slice empties the slot
            if (have) {
                fstatus[item] = err;
                if (o.status) o.status[w.orig] = err;
            }
            s_act[lane] = act;
            s_out[lane] = act ? w.out_off : 0;
            s_white[lane] = act && w.n < 10;
#pragma unroll
            for (int i = 0; i < 12; ++i) s_mv[lane][i] = act ? w.mv[i] : 0.f;
        }
        const bool any = __any_sync(0xffffffffu, act);  // the same in every warp
        const bool ref_lane0 = G.intra && !ierr;
        if (tid == 0) {
            const SlotInfo* si = st.info + G.slot;
            s_H = si->height;
            for (int l = 0; l < kMaxLevels + 1; ++l) s_ls[l] = si->level_start[l];
        }
        __syncthreads();
        if (any) {
            const int H = s_H;
            const size_t nb = (size_t)G.slot * st.max_nodes;
            const size_t lb = (size_t)G.slot * st.max_leaves;
            const uint32_t N = act ? w.n : 0;
            // frame-interleaved region: coefficient i of plane p at (p*N + i)*32 + lane
            const float* cy = coef + (act ? w.coef_off + lane : 0);
            const float* cu = cy + (size_t)N * 32;
            const float* cv = cu + (size_t)N * 32;
            // one finished leaf of this lane's frame into the warp's stage
            auto finish = [&](uint32_t leaf, uint32_t slot_local, float y, float u, float v) {
                float ry, ru, rv;
                if (ref_lane0) {
                    ry = __shfl_sync(0xffffffffu, y, 0);
                    ru = __shfl_sync(0xffffffffu, u, 0);
                    rv = __shfl_sync(0xffffffffu, v, 0);
                } else {
                    const float* r = st.ref + (lb + leaf) * 3;
                    ry = __ldg(r);
                    ru = __ldg(r + 1);
                    rv = __ldg(r + 2);
                }
                if (!act) return;
                if (intra_lane) {
                    float* r = st.ref + (lb + leaf) * 3;
                    r[0] = y;
                    r[1] = u;
                    r[2] = v;
                } else {
                    y = __fadd_rn(y, ry);
                    u = __fadd_rn(u, ru);
                    v = __fadd_rn(v, rv);
                }
                const float du = __fsub_rn(u, 128.0f), dv = __fsub_rn(v, 128.0f);
                const float R = __fadd_rn(y, __fmul_rn(1.4020f, dv));
                const float Gc = __fsub_rn(__fsub_rn(y, __fmul_rn(0.3441f, du)), __fmul_rn(0.7141f, dv));
                const float B = __fadd_rn(y, __fmul_rn(1.7720f, du));
                ws.rgb[lane][slot_local] = (uint32_t)to_u8(R) | ((uint32_t)to_u8(Gc) << 8) | ((uint32_t)to_u8(B) << 16);
                if constexpr (P24) {
                    ws.fr[lane][slot_local] = __fdiv_rn(R, 255.0f);
                    ws.fg[lane][slot_local] = __fdiv_rn(Gc, 255.0f);
                    ws.fb[lane][slot_local] = __fdiv_rn(B, 255.0f);
                }
            };
            // the warp writes its staged leaves [base, base + cnt) of every active
            // frame, two frames per pass: half-warp h writes frame f0 + h, its
            // lanes consecutive points of that frame.  The leaf centre (read
            // once) goes through the frame's transform here.
            auto flush = [&](uint32_t base, uint32_t cnt) {
                __syncwarp();
                const uint32_t i = lane & 15, h = lane >> 4;
                float x0 = 0.f, y0 = 0.f, z0 = 0.f;
                if (i < cnt) {
                    const float* p = st.xyz + (lb + base + i) * 3;
                    x0 = __ldg(p);
                    y0 = __ldg(p + 1);
                    z0 = __ldg(p + 2);
                }
                for (uint32_t f0 = 0; f0 < 32; f0 += 2) {
                    const uint32_t f = f0 + h;
                    if (i >= cnt || !s_act[f]) continue;
                    const uint64_t oi = s_out[f] + base + i;
                    const float* m = s_mv[f];
                    const float X = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[0]), __fmul_rn(y0, m[1])), __fmul_rn(z0, m[2])), m[3]);
                    const float Y = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[4]), __fmul_rn(y0, m[5])), __fmul_rn(z0, m[6])), m[7]);
                    const float Z = __fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(x0, m[8]), __fmul_rn(y0, m[9])), __fmul_rn(z0, m[10])), m[11]);
                    if (o.xyz) {
                        o.xyz[oi * 3 + 0] = X;
                        o.xyz[oi * 3 + 1] = Y;
                        o.xyz[oi * 3 + 2] = Z;
                    }
                    const uint32_t c = ws.rgb[f][i];
                    if (o.rgb) {
                        o.rgb[oi * 3 + 0] = (uint8_t)c;
                        o.rgb[oi * 3 + 1] = (uint8_t)(c >> 8);
                        o.rgb[oi * 3 + 2] = (uint8_t)(c >> 16);
                    }
                    if constexpr (P24) {
                        float* q = o.p24 + oi * 6;
                        const bool white = s_white[f];
                        q[0] = X;
                        q[1] = Y;
                        q[2] = Z;
                        q[3] = white ? 1.0f : ws.fr[f][i];
                        q[4] = white ? 1.0f : ws.fg[f][i];
                        q[5] = white ? 1.0f : ws.fb[f][i];
                    }
                }
                __syncwarp();
            };
            if (H == 1) {
                if (wid == 0 && G.part == 0) {
                    const float gy = act ? cy[0] : 0.f, gu = act ? cu[0] : 0.f, gv = act ? cv[0] : 0.f;
                    finish(0, 0, gy, gu, gv);
                    flush(0, 1);
                }
            } else {
                float* gA = bufA;
                float* gB = bufB;
                if (wid == 0) {
                    gA[lane] = act ? cy[0] : 0.f;
                    gA[32 + lane] = act ? cu[0] : 0.f;
                    gA[64 + lane] = act ? cv[0] : 0.f;
                }
                __syncthreads();
                for (int l = 0; l < H - 3; ++l) {  // internal levels above the last two
                    const int a = s_ls[l], b = s_ls[l + 1];
                    for (int j = wid; j < b - a; j += kGrpWarps) {
                        const size_t node = nb + a + j;
                        const uint32_t byte = __ldg(st.occ + node), cb = __ldg(st.cbase + node);
                        const float* g3 = gA + (size_t)j * 96 + lane;
                        float oy[8], ou[8], ov[8];
                        lane_node<32>(st, node, act, cy, cu, cv, g3[0], g3[32], g3[64], oy, ou, ov);
                        uint32_t r = 0;
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            if (!(byte & (0x80u >> c))) continue;
                            float* go = gB + (size_t)(cb + r) * 96 + lane;
                            ++r;
                            go[0] = oy[c];
                            go[32] = ou[c];
                            go[64] = ov[c];
                        }
                    }
                    __syncthreads();
                    float* t = gA;
                    gA = gB;
                    gB = t;
                }
                // gA: the DCs of level H - 3 (the parents), or for H = 2 the root's
                const int a = s_ls[H - 2], cnt = s_ls[H - 1] - a;                       // last internal level
                const int pa = H >= 3 ? s_ls[H - 3] : 0, pcnt = H >= 3 ? s_ls[H - 2] - pa : 1;  // its parents
                float(&dc)[3][8][32] = s_dc[wid];
                uint32_t pc0 = 0, pc1 = 0;  // the current parent's children [pc0, pc1) of the last level
                // parent pj: its children's DCs into dc, compacted (child pc0 + r at row r)
                auto parent = [&](int pj) {
                    if (H == 2) {  // the root is the only last-level node: its DC as the one child
                        dc[0][0][lane] = gA[lane];
                        dc[1][0][lane] = gA[32 + lane];
                        dc[2][0][lane] = gA[64 + lane];
                        pc0 = 0;
                        pc1 = 1;
                        return;
                    }
                    const size_t node = nb + pa + pj;
                    const uint32_t byte = __ldg(st.occ + node), cb = __ldg(st.cbase + node);
                    const float* g3 = gA + (size_t)pj * 96 + lane;
                    float oy[8], ou[8], ov[8];
                    lane_node<32>(st, node, act, cy, cu, cv, g3[0], g3[32], g3[64], oy, ou, ov);
                    uint32_t r = 0;
#pragma unroll
                    for (int c = 0; c < 8; ++c) {
                        if (!(byte & (0x80u >> c))) continue;
                        dc[0][r][lane] = oy[c];
                        dc[1][r][lane] = ou[c];
                        dc[2][r][lane] = ov[c];
                        ++r;
                    }
                    pc0 = cb;
                    pc1 = cb + r;
                };
                // the group's region (every lane's frame shares it) and plane
                // stride, from lane 0, which always holds a slice
                const uint64_t g_off = __shfl_sync(0xffffffffu, have ? w.coef_off : 0ull, 0);
                const uint32_t g_n = __shfl_sync(0xffffffffu, have ? w.n : 0u, 0);
                const float* const g_coef = coef + g_off;
                // Node t+1's coefficient lines into L1 while node t is
                // transformed: lane l < 21 takes line (plane l / 7, coded slot
                // l % 7).
                auto prefetch_node = [&](const NodeRows& r, int t) {
                    const uint32_t nc = __popc(r.mask[t] & 0xFEu);
                    if (lane < 21) {
                        const uint32_t k = (uint32_t)lane % 7u, pl = (uint32_t)lane / 7u;
                        if (k < nc) {
                            const float* line = g_coef + ((size_t)pl * g_n + r.coff[t] + k) * 32;
                            asm volatile("prefetch.global.L1 [%0];" ::"l"(line));
                        }
                    }
                };
                // this warp's share of the last-level nodes: of all the
                // warps of the CTAs the group is split over
                const int parts = G.parts > 1 ? G.parts : 1, vw = G.part * kGrpWarps + wid;
                const int per = (cnt + kGrpWarps * parts - 1) / (kGrpWarps * parts);
                const int j0 = min(cnt, vw * per), j1 = min(cnt, j0 + per);
                uint32_t base = 0, staged = 0;
                int pj = 0;
                if (j0 < j1) {
                    base = __ldg(st.cbase + nb + a + j0);
                    if (H >= 3) {
                        // the parent of node j0: the last parent whose first
                        // child is at or below j0 (child offsets ascend)
                        int lo = 0, hi = pcnt;
                        while (hi - lo > 1) {
                            const int step = (hi - lo + 31) >> 5;
                            const int idx = lo + lane * step;
                            const bool le = idx < hi && (int)__ldg(st.cbase + nb + pa + idx) <= j0;
                            const uint32_t bal = __ballot_sync(0xffffffffu, le);  // lanes 0.. k hold; lane 0 always
                            lo += (bal ? 31 - __clz(bal) : 0) * step;
                            hi = min(hi, lo + step);
                        }
                        pj = lo;
                    }
                    parent(pj);
                }
                NodeRows& nr = s_nodes[wid];
                for (int jb = j0; jb < j1; jb += kRowNodes) {
                    // the next node records, one node per lane, all loads in flight at once
                    const int nn = min(kRowNodes, j1 - jb);
                    __syncwarp();
                    if (lane < nn) {
                        const size_t node = nb + a + jb + lane;
                        nr.occ[lane] = __ldg(st.occ + node);
                        nr.cb[lane] = __ldg(st.cbase + node);
                        nr.mask[lane] = __ldg(st.mask + node);
                        nr.coff[lane] = __ldg(st.coff + node);
                        const float2* ab = st.ab + node * 7;
#pragma unroll
                        for (int i = 0; i < 7; ++i) nr.ab[i][lane] = __ldg(ab + i);
                    }
                    __syncwarp();
                    if (nn > 0) prefetch_node(nr, 0);
                    for (int t = 0; t < nn; ++t) {
                        if (t + 1 < nn) prefetch_node(nr, t + 1);
                        const uint32_t jc = (uint32_t)(jb + t);
                        while (jc >= pc1 && pj + 1 < pcnt) parent(++pj);  // the next parent with children
                        const uint32_t byte = nr.occ[t], cb = nr.cb[t];
                        const uint32_t k = __popc(byte);
                        if (staged + k > (uint32_t)kWarpLeaves) {
                            flush(base, staged);
                            base += staged;
                            staged = 0;
                        }
                        const uint32_t rc = jc - pc0 < 8u ? jc - pc0 : 0u;  // its row (in range for a well-formed tree)
                        float oy[8], ou[8], ov[8];
                        lane_node_md<32, kRowNodes>(nr.mask[t], nr.coff[t], &nr.ab[0][t], act, cy, cu, cv, dc[0][rc][lane],
                                                    dc[1][rc][lane], dc[2][rc][lane], oy, ou, ov);
                        uint32_t r = 0;
#pragma unroll
                        for (int c = 0; c < 8; ++c) {
                            if (!(byte & (0x80u >> c))) continue;
                            finish(cb + r, cb + r - base, oy[c], ou[c], ov[c]);
                            ++r;
                        }
                        staged = cb + k - base;
                    }
                }
                if (staged) flush(base, staged);
            }
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------------------
// k_refresh: the per-call fields of a reused plan's records, gathered from
// the call's description arrays by each record's caller index.
__global__ void k_refresh(SliceWork* __restrict__ work, int n, CallFields f) {
    const int q = blockIdx.x * blockDim.x + threadIdx.x;
    if (q >= n) return;
    SliceWork& w = work[q];
    const int i = w.orig;
    w.col_off = f.col_off[i];
    w.geo_off = f.geo_off[i];
    w.out_off = f.out_off[i];
    w.csz = f.csz[i];
    w.gsz = f.gsz[i];
    w.qp = f.qp[i];
#pragma unroll
    for (int k = 0; k < 12; ++k) w.mv[k] = f.mv[16ull * i + k];
}

// ---------------------------------------------------------------------------
// launchers (host)
constexpr int kTreeThreads = 256;
constexpr int kRahtThreads = 128;

// Dynamic shared-memory limits of the inverse-RAHT kernels, set once per
// device before any launch (and so before any stream capture: the launchers
// themselves make only capturable calls).
cudaError_t prepare_kernels() {
    static std::mutex mu;
    static bool done[64] = {};
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return e;
    std::lock_guard<std::mutex> g(mu);
    if (dev >= 0 && dev < 64 && done[dev]) return cudaSuccess;
    e = cudaFuncSetAttribute(k_raht_slice<kRahtThreads>, cudaFuncAttributeMaxDynamicSharedMemorySize, 200 * 1024);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_raht_group<false>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(GroupStage<false>));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_raht_group<true>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                 (int)sizeof(GroupStage<true>));
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rlgr<32>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rlgr<64>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rlgr<128>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess) e = cudaFuncSetAttribute(k_rlgr<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr<256, 16>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr<512, 8>, cudaFuncAttributeMaxDynamicSharedMemorySize, kRlgrLongSmem);
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr_win<1, kWinRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, win_smem(1, kWinRows));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr_win<2, kWinRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, win_smem(2, kWinRows));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr_win<4, kWinRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, win_smem(4, kWinRows));
    if (e == cudaSuccess)
        e = cudaFuncSetAttribute(k_rlgr_win<8, kWinRows>, cudaFuncAttributeMaxDynamicSharedMemorySize, win_smem(8, kWinRows));
    if (e == cudaSuccess && dev >= 0 && dev < 64) done[dev] = true;
    return e;
}

cudaError_t launch_tree(const SliceWork* work, int nintra, const uint8_t* payload, const StateView& st, int32_t* tstatus,
                        cudaStream_t s) {
    if (nintra <= 0) return cudaSuccess;
    k_tree<kTreeThreads><<<nintra, kTreeThreads, 0, s>>>(work, payload, st, tstatus);
    return cudaGetLastError();
}

// smem: dynamic shared memory reserved per CTA (unused by the kernel; it
// limits which CTAs share an SM, see kRlgrLongSmem)
cudaError_t launch_refresh(SliceWork* work, int n, const CallFields& f, cudaStream_t s) {
    if (n <= 0) return cudaSuccess;
    k_refresh<<<(n + 255) / 256, 256, 0, s>>>(work, n, f);
    return cudaGetLastError();
}

cudaError_t launch_rlgr(const SliceWork* work, const int32_t* order, int nslices, const uint8_t* payload, float* coef,
                        int32_t* rstatus, int block, int smem, cudaStream_t s) {
    if (nslices <= 0) return cudaSuccess;
    const int grid = (nslices + block - 1) / block;
    smem = smem > block * kRing * 16 ? smem : block * kRing * 16;  // at least the payload rings
    switch (block) {
        case 32: k_rlgr<32><<<grid, 32, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        case 64: k_rlgr<64><<<grid, 64, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        case 128: k_rlgr<128><<<grid, 128, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        case 256: k_rlgr<256><<<grid, 256, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// The long-slice launch: kRlgrLongBlock slices per CTA, `lanes` (8, 16, 32)
// of them per warp.
cudaError_t launch_rlgr_long(const SliceWork* work, const int32_t* order, int nslices, const uint8_t* payload, float* coef,
                             int32_t* rstatus, int lanes, int smem, cudaStream_t s) {
    if (nslices <= 0) return cudaSuccess;
    static_assert(kRlgrLongBlock == 128, "a long CTA holds 128 slices");
    static_assert(kRlgrLongSmem >= 512 * kRing * 16, "the long launch's reservation holds its payload rings");
    const int grid = (nslices + kRlgrLongBlock - 1) / kRlgrLongBlock;
    switch (lanes) {
        case 8: k_rlgr<512, 8><<<grid, 512, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        case 16: k_rlgr<256, 16><<<grid, 256, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        case 32: k_rlgr<128><<<grid, 128, smem, s>>>(work, order, nslices, payload, coef, rstatus); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

// Windowed RLGR of `ngroups` groups, one warp each, `warps` per CTA; a
// warp's rings and window take 10 KB, a CTA at least kWinMinSmem, more than
// the SM of a long per-slice CTA has left.
cudaError_t launch_rlgr_win(const SliceWork* work, const GroupDesc* groups, int ngroups, const int32_t* items,
                            const uint8_t* payload, float* coef, int32_t* rstatus, int warps, cudaStream_t s) {
    if (ngroups <= 0) return cudaSuccess;
    static_assert(win_smem(1, kWinRows) + 1024 > 228 * 1024 - (kRlgrLongSmem + 1024),
                  "a windowed CTA must not fit beside a long CTA");
    const int grid = (ngroups + warps - 1) / warps;
    switch (warps) {
        case 1: k_rlgr_win<1, kWinRows><<<grid, 32, win_smem(1, kWinRows), s>>>(work, groups, ngroups, items, payload, coef, rstatus); break;
        case 2: k_rlgr_win<2, kWinRows><<<grid, 64, win_smem(2, kWinRows), s>>>(work, groups, ngroups, items, payload, coef, rstatus); break;
        case 4: k_rlgr_win<4, kWinRows><<<grid, 128, win_smem(4, kWinRows), s>>>(work, groups, ngroups, items, payload, coef, rstatus); break;
        case 8: k_rlgr_win<8, kWinRows><<<grid, 256, win_smem(8, kWinRows), s>>>(work, groups, ngroups, items, payload, coef, rstatus); break;
        default: return cudaErrorInvalidValue;
    }
    return cudaGetLastError();
}

cudaError_t launch_raht_slice(const SliceWork* work, const int32_t* list, int count, const StateView& st, const float* coef,
                              float* fallback, const int32_t* tstatus, const int32_t* rstatus, int32_t* fstatus, float* xyz,
                              uint8_t* rgb, float* p24, int32_t* status, int wcap, cudaStream_t s) {
    if (count <= 0) return cudaSuccess;
    const size_t smem = 2ull * wcap * 3 * sizeof(float);
    OutPtrs o{xyz, rgb, p24, status};
    k_raht_slice<kRahtThreads><<<count, kRahtThreads, smem, s>>>(work, list, st, coef, fallback, tstatus, rstatus, fstatus, o,
                                                                 wcap);
    return cudaGetLastError();
}

cudaError_t launch_raht_group(const SliceWork* work, const GroupDesc* groups, int ngroups, const int32_t* items,
                              const StateView& st, const float* coef, const int32_t* tstatus, const int32_t* rstatus,
                              int32_t* fstatus, float* xyz, uint8_t* rgb, float* p24, int32_t* status, float* scratch,
                              uint64_t scratch_floats, int nctas, int* counter, cudaStream_t s) {
    if (ngroups <= 0) return cudaSuccess;
    if (cudaMemsetAsync(counter, 0, sizeof(int), s) != cudaSuccess) return cudaGetLastError();
    OutPtrs o{xyz, rgb, p24, status};
    const int grid = ngroups < nctas ? ngroups : nctas;
    if (p24)
        k_raht_group<true><<<grid, 32 * kGrpWarps, sizeof(GroupStage<true>), s>>>(
            work, groups, ngroups, items, st, coef, tstatus, rstatus, fstatus, o, scratch, scratch_floats, counter);
    else
        k_raht_group<false><<<grid, 32 * kGrpWarps, sizeof(GroupStage<false>), s>>>(
            work, groups, ngroups, items, st, coef, tstatus, rstatus, fstatus, o, scratch, scratch_floats, counter);
    return cudaGetLastError();
}

}  // namespace pvvc
