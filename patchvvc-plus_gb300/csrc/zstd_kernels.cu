// zstd_kernels.cu -- batched zstd inflation on the GPU (one warp per payload)
// and the same decoder run on the host.
//
// Replaces the host zstd stage of the reference loader (ZstdDecoder::Decode,
// src/common/entropy_codec.cc:341-360, called by io::LoadFrame,
// src/cuda/common/slice_io.cu:233-265) for payloads already on the device.
// The decoder itself is zstd_core.h.
#include <cuda_runtime.h>

#include <memory>
#include <mutex>

#include "pvvc_gb300.h"
#include "zstd_core.h"

namespace {

constexpr int kZWarps = 1;  // payloads per CTA (one warp each; faster than four per CTA)
constexpr size_t kZSmem = kZWarps * sizeof(pvvc_zstd::Shared);

// Warp w of CTA b inflates job b * kZWarps + w: src[src_off, +src_len) into
// dst[dst_off, +dst_cap).
__global__ void __launch_bounds__(32 * kZWarps)
    k_zstd(int32_t njobs, const uint8_t* src, const uint64_t* __restrict__ src_off, const uint32_t* __restrict__ src_len,
           uint8_t* dst, const uint64_t* __restrict__ dst_off, const uint32_t* __restrict__ dst_cap,
           uint32_t* __restrict__ out_len, int32_t* __restrict__ status) {
    extern __shared__ __align__(16) unsigned char zsmem[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int job = blockIdx.x * kZWarps + warp;
    if (job >= njobs) return;  // the whole warp
    pvvc_zstd::Shared& sh = reinterpret_cast<pvvc_zstd::Shared*>(zsmem)[warp];
    const int64_t r = pvvc_zstd::decompress(sh, src + src_off[job], src_len[job], dst + dst_off[job], dst_cap[job], lane, 32);
    if (lane == 0) {
        if (out_len) out_len[job] = r < 0 ? 0u : (uint32_t)r;
        status[job] = r < 0 ? PVVC_ERR_ZSTD : PVVC_OK;
    }
}

// A failed job marks its slice: status[slice[j]] = PVVC_ERR_ZSTD.
__global__ void k_zstd_merge(int32_t njobs, const int32_t* __restrict__ zstatus, const int32_t* __restrict__ zslice,
                             int32_t* __restrict__ status) {
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j < njobs && zstatus[j] != PVVC_OK) status[zslice[j]] = PVVC_ERR_ZSTD;
}

std::mutex g_zattr_mu;
bool g_zattr[128] = {};

bool zstd_attr_ready() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 128) return false;
    std::lock_guard<std::mutex> lk(g_zattr_mu);
    if (!g_zattr[dev]) {
        if (cudaFuncSetAttribute(k_zstd, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)kZSmem) != cudaSuccess)
            return false;
        g_zattr[dev] = true;
    }
    return true;
}

}  // namespace

int pvvc_zstd_launch(int32_t njobs, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len, uint8_t* dst,
                     const uint64_t* dst_off, const uint32_t* dst_cap, uint32_t* out_len, int32_t* status,
                     cudaStream_t s) {
    if (njobs == 0) return PVVC_OK;
    if (!zstd_attr_ready()) return PVVC_ERR_CUDA;
    const int grid = (njobs + kZWarps - 1) / kZWarps;
    k_zstd<<<grid, 32 * kZWarps, kZSmem, s>>>(njobs, src, src_off, src_len, dst, dst_off, dst_cap, out_len, status);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

int pvvc_zstd_merge_status(int32_t njobs, const int32_t* zstatus, const int32_t* zslice, int32_t* status, cudaStream_t s) {
    if (njobs == 0) return PVVC_OK;
    k_zstd_merge<<<(njobs + 255) / 256, 256, 0, s>>>(njobs, zstatus, zslice, status);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_zstd_inflate_batch(int32_t njobs, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len,
                                       uint8_t* dst, const uint64_t* dst_off, const uint32_t* dst_cap, uint32_t* out_len,
                                       int32_t* status, void* stream) {
    if (njobs < 0) return PVVC_ERR_ARG;
    if (njobs && (!src || !src_off || !src_len || !dst || !dst_off || !dst_cap || !status)) return PVVC_ERR_ARG;
    return pvvc_zstd_launch(njobs, src, src_off, src_len, dst, dst_off, dst_cap, out_len, status, (cudaStream_t)stream);
}

extern "C" int pvvc_zstd_content_size(const uint8_t* src, uint64_t n, uint64_t* size) {
    if (!src || !size) return PVVC_ERR_ARG;
    return pvvc_zstd::content_size(src, n, size) ? PVVC_OK : PVVC_ERR_ZSTD;
}

extern "C" int pvvc_zstd_inflate_host(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len) {
    if ((!src && n) || (!dst && cap)) return PVVC_ERR_ARG;
    std::unique_ptr<pvvc_zstd::Shared> sh(new (std::nothrow) pvvc_zstd::Shared);
    if (!sh) return PVVC_ERR_NOMEM;
    const int64_t r = pvvc_zstd::decompress(*sh, src, n, dst, cap, 0, 1);
    if (out_len) *out_len = r < 0 ? 0 : (uint64_t)r;
    return r < 0 ? PVVC_ERR_ZSTD : PVVC_OK;
}
