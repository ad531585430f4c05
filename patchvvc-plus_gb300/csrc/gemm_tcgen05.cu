// gemm_tcgen05.cu -- BF16 GEMM on the 5th-generation tensor cores (sm_103a)
// for the point-cloud registration network's training and inference.
//
//   C[M,N] = epilogue( A[M,K] . B[N,K]^T )     A, B bf16, K contiguous
//
// Persistent CTAs (one per SM for BN = 256) walk the 128 x BN tiles of C
// (BN = 64, 128 or 256; split-K over a third tile index).  Six warps:
//   warp 0, lane 0   TMA producer: 128x64 A and BNx64 B tiles (128-byte
//                    swizzle) into a 3- to 7-stage shared-memory ring that runs on
//                    across tiles, completion counted on the stage's `full`
//                    mbarrier
//   warp 1, lane 0   MMA issuer: tcgen05.mma kind::f16 (M=128, N=BN, K=16)
//                    four per stage into one of two FP32 accumulators in
//                    tensor memory (2*BN columns); tcgen05.commit frees the
//                    stage (`empty`) and, after a tile's last stage, marks
//                    its accumulator full
//   warps 2-9        epilogue: two warps per 32-lane TMEM quarter, each with
//                    half the columns: tcgen05.ld (one C row per thread),
//                    bias / ReLU / mask, store; then the accumulator is
//                    released to the MMA issuer
// so a tile's loads and MMAs overlap the previous tile's stores.
// Every mbarrier wait is bounded; a wait that gives up sets the device error
// word (read by pvvc_device_error_take) and the CTA skips the rest of its
// work instead of hanging.
#include <cuda.h>
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <algorithm>
#include <cstdint>
#include <mutex>

#include "pvvc_gb300.h"

namespace pvvc {
namespace {

constexpr int kBM = 128, kBK = 64, kStages = 8;  // kStages: the most ring stages of any tile width
constexpr uint32_t kSpinLimit = 1u << 26;  // ~seconds of try_wait polling

__device__ int g_tc_error;  // nonzero: a bounded wait gave up (first code wins)

__device__ __forceinline__ uint32_t smem_u32(const void* p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t* bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void mbar_expect_tx(uint64_t* bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

// Bounded wait for the phase of parity `parity` to complete.  false: gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int code) {
    const uint32_t a = smem_u32(bar);
    for (uint32_t i = 0; i < kSpinLimit; ++i) {
        uint32_t ok;
        asm volatile(
            "{\n\t.reg .pred p;\n\t"
            "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
            "selp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(ok)
            : "r"(a), "r"(parity)
            : "memory");
        if (ok) return true;
        if (*(volatile int*)&g_tc_error) return false;  // another CTA already failed
    }
    atomicCAS(&g_tc_error, 0, code);
    return false;
}

__device__ __forceinline__ void tma_load_2d(void* dst, const CUtensorMap* map, uint64_t* bar, int x, int y) {
    asm volatile(
        "cp.async.bulk.tensor.2d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
            smem_u32(dst)),
        "l"(reinterpret_cast<uint64_t>(map)), "r"(x), "r"(y), "r"(smem_u32(bar))
        : "memory");
}

// Shared-memory matrix descriptor: K-major operand tile with 128-byte
// swizzle (rows of 64 bf16, 8-row swizzle atoms 1024 bytes apart).
__device__ __forceinline__ uint64_t smem_desc_sw128(uint32_t addr) {
    uint64_t d = 0;
    d |= (uint64_t)((addr & 0x3FFFFu) >> 4);  // start address
    d |= (uint64_t)1 << 16;                   // leading byte offset (unused by swizzled K-major)
    d |= (uint64_t)(1024 >> 4) << 32;         // stride byte offset: next 8-row group
    d |= (uint64_t)1 << 46;                   // descriptor version (tcgen05)
    d |= (uint64_t)2 << 61;                   // layout: 128-byte swizzle
    return d;
}

// Instruction descriptor of kind::f16: D f32, A and B bf16, both K-major.
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem_d, uint64_t a, uint64_t b, uint32_t idesc, uint32_t accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(tmem_d),
        "l"(a), "l"(b), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void mbar_arrive(uint64_t* bar) {
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mma_commit(uint64_t* bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

// 32 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32]) {
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}

struct EpiArgs {
    void* C;
    int64_t ldc;
    const float* bias;
    const __nv_bfloat16* aux;
    int64_t ldaux;
};

constexpr int kTileA = kBM * kBK * 2;  // 16 KB

// Epilogue of one 128 x BN tile: this thread's accumulator row (TMEM lane
// `tl`'s columns) through bias / ReLU / mask into C row `row`.  A warp
// instruction (tcgen05.ld): every lane of the warp calls it.
template <int BN, int EPI>
__device__ __forceinline__ void epilogue_row(uint32_t tl, int row, int M, int n0, int cbeg, int cend, const EpiArgs& ep) {
#pragma unroll 1
    for (int c0 = cbeg; c0 < cend; c0 += 32) {
        float v[32];
        tmem_ld32(tl + c0, v);
        if (row >= M) continue;
        const int col = n0 + c0;
        if (EPI == PVVC_GEMM_BIAS_RELU_BF16 || EPI == PVVC_GEMM_MASK_BF16) {
            __nv_bfloat16* out = static_cast<__nv_bfloat16*>(ep.C) + (int64_t)row * ep.ldc + col;
            if (EPI == PVVC_GEMM_BIAS_RELU_BF16) {
#pragma unroll
                for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + (ep.bias ? ep.bias[col + j] : 0.f), 0.f);
            } else {
                const uint4* ax = reinterpret_cast<const uint4*>(ep.aux + (int64_t)row * ep.ldaux + col);
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    const uint4 w = ax[q];
                    const __nv_bfloat16* h = reinterpret_cast<const __nv_bfloat16*>(&w);
#pragma unroll
                    for (int j = 0; j < 8; ++j)
                        if (!(__bfloat162float(h[j]) > 0.f)) v[q * 8 + j] = 0.f;
                }
            }
            uint4* o4 = reinterpret_cast<uint4*>(out);
#pragma unroll
            for (int q = 0; q < 4; ++q) {
                __nv_bfloat162 p[4];
#pragma unroll
                for (int j = 0; j < 4; ++j) p[j] = __floats2bfloat162_rn(v[q * 8 + 2 * j], v[q * 8 + 2 * j + 1]);
                o4[q] = *reinterpret_cast<uint4*>(p);
            }
        } else {
            float* out = static_cast<float*>(ep.C) + (int64_t)row * ep.ldc + col;
            if (EPI == PVVC_GEMM_F32) {
#pragma unroll
                for (int q = 0; q < 8; ++q) {
                    float4 f;
                    f.x = v[4 * q] + (ep.bias ? ep.bias[col + 4 * q] : 0.f);
                    f.y = v[4 * q + 1] + (ep.bias ? ep.bias[col + 4 * q + 1] : 0.f);
                    f.z = v[4 * q + 2] + (ep.bias ? ep.bias[col + 4 * q + 2] : 0.f);
                    f.w = v[4 * q + 3] + (ep.bias ? ep.bias[col + 4 * q + 3] : 0.f);
                    reinterpret_cast<float4*>(out)[q] = f;
                }
            } else {  // PVVC_GEMM_F32_ACCUM
#pragma unroll
                for (int j = 0; j < 32; ++j) atomicAdd(out + j, v[j]);
            }
        }
    }
}

// Epilogue of one warp's 32 rows (row0 + lane) of a bf16 tile: 64 columns at
// a time go through the warp's shared-memory buffer (32 rows x 8 chunks of
// 16 bytes, chunk j of row r at j ^ (r & 7), so that neither the row-wise
// writes nor the column-wise reads conflict), then out as full 128-byte row
// segments, four rows per store instruction.  Other epilogues store by row.
template <int BN, int EPI>
__device__ __forceinline__ void epilogue_warp(uint32_t tl, int row0, int M, int n0, int cbeg, int cend, const EpiArgs& ep,
                                              uint4* stage) {
    const int lane = threadIdx.x & 31, row = row0 + lane;
    if constexpr (EPI == PVVC_GEMM_BIAS_RELU_BF16 || EPI == PVVC_GEMM_MASK_BF16) {
#pragma unroll 1
        for (int c0 = cbeg; c0 < cend; c0 += 64) {
#pragma unroll
            for (int h = 0; h < 2; ++h) {
                float v[32];
                tmem_ld32(tl + c0 + 32 * h, v);
                const int col = n0 + c0 + 32 * h;
                if (EPI == PVVC_GEMM_BIAS_RELU_BF16) {
#pragma unroll
                    for (int j = 0; j < 32; ++j) v[j] = fmaxf(v[j] + (ep.bias ? ep.bias[col + j] : 0.f), 0.f);
                } else if (row < M) {
                    const uint4* ax = reinterpret_cast<const uint4*>(ep.aux + (int64_t)row * ep.ldaux + col);
#pragma unroll
                    for (int q = 0; q < 4; ++q) {
                        const uint4 w = ax[q];
                        const __nv_bfloat16* hb = reinterpret_cast<const __nv_bfloat16*>(&w);
#pragma unroll
                        for (int j = 0; j < 8; ++j)
                            if (!(__bfloat162float(hb[j]) > 0.f)) v[q * 8 + j] = 0.f;
                    }
                }
#pragma unroll
                for (int q = 0; q < 4; ++q) {
                    __nv_bfloat162 pk[4];
#pragma unroll
                    for (int j = 0; j < 4; ++j) pk[j] = __floats2bfloat162_rn(v[q * 8 + 2 * j], v[q * 8 + 2 * j + 1]);
                    stage[lane * 8 + ((4 * h + q) ^ (lane & 7))] = *reinterpret_cast<uint4*>(pk);
                }
            }
            __syncwarp();
#pragma unroll
            for (int i = 0; i < 8; ++i) {
                const int r = i * 4 + (lane >> 3), ch = lane & 7;
                const uint4 val = stage[r * 8 + (ch ^ (r & 7))];
                if (row0 + r < M)
                    *reinterpret_cast<uint4*>(static_cast<__nv_bfloat16*>(ep.C) + (int64_t)(row0 + r) * ep.ldc + n0 + c0 +
                                              ch * 8) = val;
            }
            __syncwarp();
        }
    } else {
        epilogue_row<BN, EPI>(tl, row, M, n0, cbeg, cend, ep);
    }
}

// ---------------------------------------------------------------------------
// The persistent kernel (roles in the file header).  CTA c takes tiles c,
// c + gridDim.x, ... (m-tile fastest, then n-tile, then the K split); its
// accumulator u & 1 holds its u-th tile.
// ring depth: as many stages as fit beside the eight staging buffers, so
// that narrow tiles (whose GEMMs are long K loops) keep more bytes in flight
template <int BN>
__host__ __device__ constexpr int persist_stages() {
    return BN == 256 ? 3 : (BN == 128 ? 5 : 7);
}
template <int BN>
struct PersistBars {
    uint64_t full[kStages], empty[kStages], acc_full[2], acc_empty[2];
    uint32_t tmem_base;
};
constexpr int kStageChunks = 32 * 8;  // one epilogue warp's staging buffer, 16-byte chunks
constexpr int kEpiWarps = 8;          // two per TMEM lane quarter, each draining half the columns
template <int BN>
__host__ __device__ constexpr size_t persist_bars_bytes() {
    return (sizeof(PersistBars<BN>) + 15) / 16 * 16;
}
template <int BN>
__host__ __device__ constexpr size_t persist_smem_bytes() {
    return 1024 + (size_t)persist_stages<BN>() * (kTileA + BN * kBK * 2) + persist_bars_bytes<BN>() +
           kEpiWarps * kStageChunks * 16;
}
constexpr int kPersistThreads = 64 + 32 * kEpiWarps;

template <int BN, int EPI>
__global__ void __launch_bounds__(kPersistThreads, 1)
    k_gemm_bf16_tn_persist(const __grid_constant__ CUtensorMap map_a, const __grid_constant__ CUtensorMap map_b, int M,
                           int K, int mtiles, int ntiles, int splits, int kb_per_split, EpiArgs ep) {
    extern __shared__ uint8_t smem_raw[];
    uint8_t* const base = reinterpret_cast<uint8_t*>((reinterpret_cast<uintptr_t>(smem_raw) + 1023) & ~uintptr_t(1023));
    constexpr int S = persist_stages<BN>();
    PersistBars<BN>& sm = *reinterpret_cast<PersistBars<BN>*>(base + (size_t)S * (kTileA + BN * kBK * 2));
    uint4* const stage = reinterpret_cast<uint4*>(reinterpret_cast<uint8_t*>(&sm) + persist_bars_bytes<BN>());
    auto tile_a = [&](uint32_t st) { return base + (size_t)st * kTileA; };
    auto tile_b = [&](uint32_t st) { return base + (size_t)S * kTileA + (size_t)st * BN * kBK * 2; };
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int nkb = K / kBK;
    const int ntiles_all = mtiles * ntiles * splits;
    auto tile_of = [&](int t, int& m0, int& n0, int& kb0, int& kb1) {
        const int mt = t % mtiles, r = t / mtiles;
        m0 = mt * kBM;
        n0 = (r % ntiles) * BN;
        kb0 = (r / ntiles) * kb_per_split;
        kb1 = min(nkb, kb0 + kb_per_split);
    };
    if (threadIdx.x == 0) {
        for (int st = 0; st < S; ++st) {
            mbar_init(&sm.full[st], 1);
            mbar_init(&sm.empty[st], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&sm.acc_full[b], 1);
            mbar_init(&sm.acc_empty[b], kEpiWarps);  // one arrive per epilogue warp
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncwarp();
    if (warp == 1) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(&sm.tmem_base)),
                     "r"(2 * BN));
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
    const uint32_t tmem = sm.tmem_base;
    int m0, n0, kb0, kb1;
    if (warp == 0) {
        if (lane == 0) {  // producer
            bool ok = true;
            uint32_t it = 0;
            for (int t = blockIdx.x; t < ntiles_all && ok; t += gridDim.x) {
                tile_of(t, m0, n0, kb0, kb1);
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const uint32_t st = it % S, ph = (it / S) & 1;
                    if (!(ok = mbar_wait(&sm.empty[st], ph ^ 1, 1))) break;
                    mbar_expect_tx(&sm.full[st], (kBM + BN) * kBK * 2);
                    tma_load_2d(tile_a(st), &map_a, &sm.full[st], kb * kBK, m0);
                    tma_load_2d(tile_b(st), &map_b, &sm.full[st], kb * kBK, n0);
                }
            }
        }
    } else if (warp == 1) {
        if (lane == 0) {  // MMA issuer
            constexpr uint32_t idesc = idesc_bf16(kBM, BN);
            bool ok = true;
            uint32_t it = 0, u = 0;
            for (int t = blockIdx.x; t < ntiles_all && ok; t += gridDim.x, ++u) {
                tile_of(t, m0, n0, kb0, kb1);
                const uint32_t b = u & 1, use = u >> 1;
                if (!(ok = mbar_wait(&sm.acc_empty[b], (use & 1) ^ 1, 4))) break;
                asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                const uint32_t acc = tmem + b * BN;
                for (int kb = kb0; kb < kb1; ++kb, ++it) {
                    const uint32_t st = it % S, ph = (it / S) & 1;
                    if (!(ok = mbar_wait(&sm.full[st], ph, 2))) break;
                    asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
                    const uint64_t da = smem_desc_sw128(smem_u32(tile_a(st)));
                    const uint64_t db = smem_desc_sw128(smem_u32(tile_b(st)));
#pragma unroll
                    for (int k = 0; k < kBK / 16; ++k)  // +32 bytes per K=16 step inside the swizzle row
                        mma_bf16(acc, da + 2 * k, db + 2 * k, idesc, (kb > kb0 || k > 0) ? 1u : 0u);
                    mma_commit(&sm.empty[st]);
                }
                if (ok) mma_commit(&sm.acc_full[b]);  // fires when the tile's MMAs have completed
            }
        }
    } else {  // epilogue warps 2..9
        const int q = warp & 3;  // the TMEM lane quarter this warp may read
        const int half = (warp - 2) >> 2;
        // its half of the columns (BN = 64: the first warp of each quarter takes all)
        const int cbeg = BN >= 128 ? half * (BN / 2) : 0, cend = BN >= 128 ? cbeg + BN / 2 : (half ? 0 : BN);
        uint32_t u = 0;
        for (int t = blockIdx.x; t < ntiles_all; t += gridDim.x, ++u) {
            tile_of(t, m0, n0, kb0, kb1);
            const uint32_t b = u & 1, use = u >> 1;
            // warp-uniform: tcgen05.ld in the epilogue is a .sync.aligned warp instruction
            if (!__all_sync(0xffffffffu, mbar_wait(&sm.acc_full[b], use & 1, 3))) break;
            asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory");
            epilogue_warp<BN, EPI>(tmem + b * BN + ((uint32_t)(q * 32) << 16), m0 + q * 32, M, n0, cbeg, cend, ep,
                                   stage + (warp - 2) * kStageChunks);
            asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
            __syncwarp();
            if (lane == 0) mbar_arrive(&sm.acc_empty[b]);
        }
    }
    asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory");
    __syncthreads();
    if (warp == 1) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(2 * BN));
}

// ---- host ----------------------------------------------------------------
using EncodeTiled = CUresult (*)(CUtensorMap*, CUtensorMapDataType, cuuint32_t, void*, const cuuint64_t*, const cuuint64_t*,
                                 const cuuint32_t*, const cuuint32_t*, CUtensorMapInterleave, CUtensorMapSwizzle,
                                 CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

EncodeTiled encode_fn() {
    static EncodeTiled fn = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<EncodeTiled>(p);
    });
    return fn;
}

// rows x K bf16 matrix (row stride ld elements) as a TMA map of box_rows x 64 tiles
bool make_map(CUtensorMap* m, const void* base, int64_t rows, int64_t K, int64_t ld, int box_rows) {
    EncodeTiled enc = encode_fn();
    if (!enc) return false;
    const cuuint64_t dims[2] = {(cuuint64_t)K, (cuuint64_t)rows};
    const cuuint64_t strides[1] = {(cuuint64_t)ld * 2};
    const cuuint32_t box[2] = {(cuuint32_t)kBK, (cuuint32_t)box_rows};
    const cuuint32_t estr[2] = {1, 1};
    return enc(m, CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2, const_cast<void*>(base), dims, strides, box, estr,
               CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_128B, CU_TENSOR_MAP_L2_PROMOTION_L2_256B,
               CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) == CUDA_SUCCESS;
}

template <int BN, int EPI>
cudaError_t launch_bn(const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, int splits, const EpiArgs& ep,
                      cudaStream_t s) {
    // once per instantiation: the shared-memory opt-in and how many CTAs fit
    // on an SM (two accumulators of BN columns each must fit the 512 TMEM
    // columns of all resident CTAs)
    static std::once_flag once;
    static cudaError_t attr = cudaSuccess;
    static int per_sm = 1;
    std::call_once(once, [&] {
        attr = cudaFuncSetAttribute(k_gemm_bf16_tn_persist<BN, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    (int)persist_smem_bytes<BN>());
        int occ = 0;
        if (attr == cudaSuccess)
            attr = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_gemm_bf16_tn_persist<BN, EPI>, kPersistThreads,
                                                                 persist_smem_bytes<BN>());
        per_sm = std::max(1, std::min(occ, 512 / (2 * BN)));
    });
    if (attr != cudaSuccess) return attr;
    int dev = 0, sms = 0;
    cudaError_t e = cudaGetDevice(&dev);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (e != cudaSuccess) return e;
    const int nkb = K / kBK;
    const int per = (nkb + splits - 1) / splits;
    const int z = (nkb + per - 1) / per;
    const int mtiles = (M + kBM - 1) / kBM, ntiles = N / BN;
    const long long tiles = (long long)mtiles * ntiles * z;
    const int grid = (int)std::min<long long>(tiles, (long long)sms * per_sm);
    k_gemm_bf16_tn_persist<BN, EPI><<<grid, kPersistThreads, persist_smem_bytes<BN>(), s>>>(ma, mb, M, K, mtiles, ntiles, z,
                                                                                            per, ep);
    return cudaGetLastError();
}

template <int BN>
cudaError_t launch_epi(int epi, const CUtensorMap& ma, const CUtensorMap& mb, int M, int N, int K, int splits,
                       const EpiArgs& ep, cudaStream_t s) {
    switch (epi) {
        case PVVC_GEMM_BIAS_RELU_BF16: return launch_bn<BN, PVVC_GEMM_BIAS_RELU_BF16>(ma, mb, M, N, K, splits, ep, s);
        case PVVC_GEMM_F32: return launch_bn<BN, PVVC_GEMM_F32>(ma, mb, M, N, K, splits, ep, s);
        case PVVC_GEMM_F32_ACCUM: return launch_bn<BN, PVVC_GEMM_F32_ACCUM>(ma, mb, M, N, K, splits, ep, s);
        case PVVC_GEMM_MASK_BF16: return launch_bn<BN, PVVC_GEMM_MASK_BF16>(ma, mb, M, N, K, splits, ep, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace

// Internal entry (also behind the C ABI): see pvvc_gemm_bf16.
int gemm_bf16(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb, void* C,
              int64_t ldc, const float* bias, const void* aux, int64_t ldaux, int32_t epi, int32_t splits,
              cudaStream_t s) {
    if (M < 0 || N <= 0 || K <= 0 || K % kBK || N % 64 || !A || !B || !C || splits < 1) return PVVC_ERR_ARG;
    if (lda % 8 || ldb % 8 || lda < K || ldb < K) return PVVC_ERR_ARG;
    if ((reinterpret_cast<uintptr_t>(A) | reinterpret_cast<uintptr_t>(B) | reinterpret_cast<uintptr_t>(C)) & 15)
        return PVVC_ERR_ARG;
    const bool bf16_out = epi == PVVC_GEMM_BIAS_RELU_BF16 || epi == PVVC_GEMM_MASK_BF16;
    if (ldc < N || (bf16_out ? ldc % 8 : ldc % 4)) return PVVC_ERR_ARG;
    if (epi == PVVC_GEMM_MASK_BF16 && (!aux || ldaux < N || ldaux % 8 || (reinterpret_cast<uintptr_t>(aux) & 15)))
        return PVVC_ERR_ARG;
    if (epi != PVVC_GEMM_F32_ACCUM && splits != 1) return PVVC_ERR_ARG;  // only accumulation combines partials
    if (M == 0) return PVVC_OK;
    const int BN = N % 256 == 0 ? 256 : N % 128 == 0 ? 128 : 64;
    CUtensorMap ma, mb;
    if (!make_map(&ma, A, M, K, lda, kBM) || !make_map(&mb, B, N, K, ldb, BN)) return PVVC_ERR_CUDA;
    EpiArgs ep{C, ldc, bias, static_cast<const __nv_bfloat16*>(aux), ldaux};
    cudaError_t e = BN == 256 ? launch_epi<256>(epi, ma, mb, M, N, K, splits, ep, s)
                  : BN == 128 ? launch_epi<128>(epi, ma, mb, M, N, K, splits, ep, s)
                              : launch_epi<64>(epi, ma, mb, M, N, K, splits, ep, s);
    return e == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

int device_error_take(int* code) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_tc_error, sizeof(int)) != cudaSuccess) return PVVC_ERR_CUDA;
    if (v) {
        const int z = 0;
        if (cudaMemcpyToSymbol(g_tc_error, &z, sizeof(int)) != cudaSuccess) return PVVC_ERR_CUDA;
    }
    *code = v;
    return PVVC_OK;
}

}  // namespace pvvc

extern "C" int pvvc_gemm_bf16(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb,
                              void* C, int64_t ldc, const float* bias, const void* aux, int64_t ldaux, int32_t epilogue,
                              int32_t splits, void* stream) {
    return pvvc::gemm_bf16(M, N, K, A, lda, B, ldb, C, ldc, bias, aux, ldaux, epilogue, splits, (cudaStream_t)stream);
}

namespace pvvc {
int icp_error_take(int* code);  // icp_kernels.cu
}

extern "C" int pvvc_device_error_take(int32_t* code) {
    if (!code) return PVVC_ERR_ARG;
    int v = 0, w = 0;
    int rc = pvvc::device_error_take(&v);
    const int rc2 = pvvc::icp_error_take(&w);
    if (rc == PVVC_OK) rc = rc2;
    *code = v ? v : w;
    return rc;
}
