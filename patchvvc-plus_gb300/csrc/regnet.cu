// regnet.cu -- the patch-registration proposal network: a PointNet-style
// model that maps a (source, target) patch pair to an initial rigid
// transform for ICP, trained and run on the GPU by this file's kernels and
// the tcgen05 GEMM (gemm_tcgen05.cu).  No reference counterpart: the
// reference starts every registration from the identity
// (src/registration/icp.cc:21-102).
//
// Model (per pair; P = 256 points sampled from each cloud):
//   x0  = (p - centroid(cloud)) / s,   s = RMS radius of the source sample
//   X1  = relu(W1 x0 + b1)      3 -> 64     CUDA cores (fused with sampling)
//   X2  = relu(X1 W2^T + b2)   64 -> 128    tcgen05 GEMM, bf16 out
//   Y3  = relu(X2 W3^T + b3)  128 -> 256    tcgen05 GEMM, bf16 out
//   G   = max over the P rows of each cloud (argmax kept); H0 = [G_src, G_tgt]
//   H1  = relu(H0 W4^T + b4)  512 -> 256    tcgen05 GEMM
//   H2  = relu(H1 W5^T + b5)  256 -> 128    tcgen05 GEMM
//   out = W6 H2 + b6          128 -> 6      CUDA cores: omega (axis-angle), delta
//   T   = [R(omega) | c_t - R c_s + s * delta]
// Loss: mean over pairs of lambda_w |omega - omega*|^2 + |delta - delta*|^2,
// with (omega*, delta*) from the converged ICP transform.
// Backward: GEMMs for the dense layers (weights transposed for dX, the
// activations transposed for dW with split-K accumulation); the max-pool
// backward is exact and sparse: only a cloud's argmax rows receive gradient,
// so dW3 and dX2 are gathers/scatters over those rows instead of dense GEMMs.
// Parameters: one fp32 master vector (AdamW state beside it) plus bf16
// copies of W2..W5 in both layouts.
#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include <cmath>
#include <cstdint>
#include <cstring>
#include <memory>
#include <vector>

#include "decode_internal.h"
#include "pvvc_gb300.h"

namespace pvvc {
int gemm_bf16(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb, void* C,
              int64_t ldc, const float* bias, const void* aux, int64_t ldaux, int32_t epi, int32_t splits,
              cudaStream_t s);

namespace {

constexpr int kP = 256;  // points sampled per cloud
constexpr int kD1 = 64, kD2 = 128, kD3 = 256, kH0 = 512, kH1 = 256, kH2 = 128, kOut = 6;

// flat parameter layout (fp32 master)
struct Layout {
    int64_t w1, b1, w2, b2, w3, b3, w4, b4, w5, b5, w6, b6, total;
    Layout() {
        int64_t o = 0;
        auto take = [&](int64_t n) {
            const int64_t r = o;
            o += n;
            return r;
        };
        w1 = take(kD1 * 3);
        b1 = take(kD1);
        w2 = take(kD2 * kD1);
        b2 = take(kD2);
        w3 = take(kD3 * kD2);
        b3 = take(kD3);
        w4 = take(kH1 * kH0);
        b4 = take(kH1);
        w5 = take(kH2 * kH1);
        b5 = take(kH2);
        w6 = take(kOut * kH2);
        b6 = take(kOut);
        total = o;
    }
};
const Layout kL;

__device__ __forceinline__ uint32_t mix32(uint64_t x) {
    x ^= x >> 33;
    x *= 0xff51afd7ed558ccdull;
    x ^= x >> 33;
    x *= 0xc4ceb9fe1a85ec53ull;
    x ^= x >> 33;
    return (uint32_t)x;
}

// sum of v over a block of 256 threads (red: 8 floats of shared memory)
__device__ __forceinline__ float block_sum256(float v, float* red) {
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = v;
    __syncthreads();
    float t = 0.f;
    for (int w = 0; w < 8; ++w) t += red[w];
    return t;
}

// X1 row = relu(W1 x0 + b1) as 64 bf16 (128 bytes)
__device__ __forceinline__ void layer1_row(const float* w1, const float* b1, float x, float y, float z,
                                           __nv_bfloat16* out) {
    uint4* o4 = reinterpret_cast<uint4*>(out);
#pragma unroll
    for (int q = 0; q < kD1 / 8; ++q) {
        __nv_bfloat162 h[4];
#pragma unroll
        for (int j = 0; j < 4; ++j) {
            const int a = q * 8 + 2 * j, b = a + 1;
            const float va = fmaxf(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w1[3 * a], x), __fmul_rn(w1[3 * a + 1], y)),
                                                     __fmul_rn(w1[3 * a + 2], z)),
                                           b1[a]),
                                   0.f);
            const float vb = fmaxf(__fadd_rn(__fadd_rn(__fadd_rn(__fmul_rn(w1[3 * b], x), __fmul_rn(w1[3 * b + 1], y)),
                                                     __fmul_rn(w1[3 * b + 2], z)),
                                           b1[b]),
                                   0.f);
            h[j] = __floats2bfloat162_rn(va, vb);
        }
        o4[q] = *reinterpret_cast<uint4*>(h);
    }
}

// One pair per block (256 threads, one sampled point per thread and side):
// sample with replacement (hash of seed, pair, side, j), centre each cloud on
// its sample mean, scale both by the source sample's RMS radius, write x0
// (fp32) and X1 (bf16), the pair's frame (c_s, c_t, s) and, when labels are
// given, the regression target (omega*, delta*).
__global__ void __launch_bounds__(256) k_sample_l1(int npairs, const int32_t* __restrict__ ids, const float* __restrict__ src,
                                                   const uint32_t* __restrict__ soff, const float* __restrict__ tgt,
                                                   const uint32_t* __restrict__ toff, uint64_t seed,
                                                   const float* __restrict__ w1, const float* __restrict__ b1,
                                                   float* __restrict__ x0, __nv_bfloat16* __restrict__ x1,
                                                   float* __restrict__ frame, const float* __restrict__ T_label,
                                                   const float* __restrict__ omega_label, float* __restrict__ y) {
    __shared__ float red[8];
    const int b = blockIdx.x, j = threadIdx.x;
    if (b >= npairs) return;
    const int pid = ids ? ids[b] : b;
    float p[2][3];
    for (int side = 0; side < 2; ++side) {
        const uint32_t* off = side ? toff : soff;
        const float* pts = side ? tgt : src;
        const uint32_t lo = off[pid], n = off[pid + 1] - lo;
        const uint32_t k = n ? mix32(seed * 0x9E3779B97F4A7C15ull ^ ((uint64_t)pid << 20) ^ ((uint64_t)side << 19) ^ j) % n : 0;
        for (int d = 0; d < 3; ++d) p[side][d] = n ? pts[3ull * (lo + k) + d] : 0.f;
    }
    float c[2][3];
    for (int side = 0; side < 2; ++side)
        for (int d = 0; d < 3; ++d) c[side][d] = block_sum256(p[side][d], red) / kP;
    const float dx = p[0][0] - c[0][0], dy = p[0][1] - c[0][1], dz = p[0][2] - c[0][2];
    const float s = sqrtf(block_sum256(dx * dx + dy * dy + dz * dz, red) / kP) + 1e-3f;
    const float inv = 1.f / s;
    for (int side = 0; side < 2; ++side) {
        const int64_t row = ((int64_t)b * 2 + side) * kP + j;
        const float x = (p[side][0] - c[side][0]) * inv, yy = (p[side][1] - c[side][1]) * inv,
                    z = (p[side][2] - c[side][2]) * inv;
        x0[3 * row] = x;
        x0[3 * row + 1] = yy;
        x0[3 * row + 2] = z;
        layer1_row(w1, b1, x, yy, z, x1 + row * kD1);
    }
    if (j == 0) {
        float* f = frame + 7 * b;
        for (int d = 0; d < 3; ++d) {
            f[d] = c[0][d];
            f[3 + d] = c[1][d];
        }
        f[6] = s;
        if (T_label) {  // delta* = (t* - (c_t - R* c_s)) / s
            const float* T = T_label + 16 * pid;
            for (int d = 0; d < 3; ++d) {
                const float rc = T[4 * d] * c[0][0] + T[4 * d + 1] * c[0][1] + T[4 * d + 2] * c[0][2];
                y[6 * b + 3 + d] = (T[4 * d + 3] - (c[1][d] - rc)) * inv;
                y[6 * b + d] = omega_label[3 * pid + d];
            }
        }
    }
}

// X1 from given x0 rows (the gradient-check entry)
__global__ void k_l1(int64_t rows, const float* __restrict__ x0, const float* __restrict__ w1, const float* __restrict__ b1,
                     __nv_bfloat16* __restrict__ x1) {
    const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (r >= rows) return;
    layer1_row(w1, b1, x0[3 * r], x0[3 * r + 1], x0[3 * r + 2], x1 + r * kD1);
}

// max over each cloud's P rows of Y3 (first maximum), into H0 = [G_src | G_tgt]
__global__ void __launch_bounds__(256) k_pool(const __nv_bfloat16* __restrict__ y3, __nv_bfloat16* __restrict__ h0,
                                              int32_t* __restrict__ amax) {
    const int c = blockIdx.x, ch = threadIdx.x;
    const __nv_bfloat16* base = y3 + (int64_t)c * kP * kD3 + ch;
    float best = __bfloat162float(base[0]);
    int arg = 0;
    for (int r = 1; r < kP; ++r) {
        const float v = __bfloat162float(base[(int64_t)r * kD3]);
        if (v > best) {
            best = v;
            arg = r;
        }
    }
    h0[(int64_t)(c >> 1) * kH0 + (c & 1) * kD3 + ch] = __float2bfloat16_rn(best);
    amax[c * kD3 + ch] = arg;
}

// Output layer, loss and its gradient.  One pair per block of 128 threads.
// out = W6 H2 + b6; loss += sum_j w_j (out_j - y_j)^2 / B; dOut = 2 w (out - y) / B;
// dW6 += dOut H2^T, db6 += dOut; dH2 = (W6^T dOut) masked by H2 > 0 (bf16).
__global__ void __launch_bounds__(128) k_head(int npairs, const __nv_bfloat16* __restrict__ h2, const float* __restrict__ w6,
                                              const float* __restrict__ b6, const float* __restrict__ y, float lambda_w,
                                              float* __restrict__ out, float* __restrict__ loss, float* __restrict__ gw6,
                                              float* __restrict__ gb6, __nv_bfloat16* __restrict__ dh2) {
    __shared__ float part[4][kOut];
    __shared__ float dout[kOut];
    const int b = blockIdx.x, k = threadIdx.x;
    const float h = __bfloat162float(h2[(int64_t)b * kH2 + k]);
    for (int j = 0; j < kOut; ++j) {
        float v = w6[j * kH2 + k] * h;
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((k & 31) == 0) part[k >> 5][j] = v;
    }
    __syncthreads();
    if (k < kOut) {
        const float o = part[0][k] + part[1][k] + part[2][k] + part[3][k] + b6[k];
        out[kOut * b + k] = o;
        if (y) {
            const float w = k < 3 ? lambda_w : 1.f;
            const float e = o - y[kOut * b + k];
            atomicAdd(loss, w * e * e / npairs);
            dout[k] = 2.f * w * e / npairs;
            atomicAdd(gb6 + k, dout[k]);
        }
    }
    if (!y) return;
    __syncthreads();
    float g = 0.f;
    for (int j = 0; j < kOut; ++j) {
        atomicAdd(gw6 + j * kH2 + k, dout[j] * h);
        g += w6[j * kH2 + k] * dout[j];
    }
    dh2[(int64_t)b * kH2 + k] = __float2bfloat16_rn(h > 0.f ? g : 0.f);
}

// out[C,R] = in[R,C]^T (bf16), 32x32 tiles
__global__ void k_transpose(const __nv_bfloat16* __restrict__ in, int64_t R, int64_t C, __nv_bfloat16* __restrict__ out) {
    __shared__ __nv_bfloat16 t[32][34];
    const int64_t r0 = blockIdx.y * 32ll, c0 = blockIdx.x * 32ll;
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int64_t r = r0 + i, c = c0 + threadIdx.x;
        t[i][threadIdx.x] = (r < R && c < C) ? in[r * C + c] : __float2bfloat16_rn(0.f);
    }
    __syncthreads();
    for (int i = threadIdx.y; i < 32; i += 8) {
        const int64_t c = c0 + i, r = r0 + threadIdx.x;
        if (c < C && r < R) out[c * R + r] = t[threadIdx.x][i];
    }
}

// out[C,R] = in[R,C]^T for even R and C: 64x64 tiles, each thread moving
// bf16 pairs, so that a warp reads and writes 128 contiguous bytes per row.
// part (optional): the tile's column sums, part[blockIdx.y * C + c], for
// k_colsum_parts.
__global__ void __launch_bounds__(256) k_transpose_pairs(const __nv_bfloat16* __restrict__ in, int64_t R, int64_t C,
                                                         __nv_bfloat16* __restrict__ out, float* __restrict__ part) {
    __shared__ __nv_bfloat16 t[64][66];  // odd word stride: column reads spread over the banks
    __shared__ float red[8][64];
    const int64_t r0 = blockIdx.y * 64ll, c0 = blockIdx.x * 64ll;
    const int tx = threadIdx.x, ty = threadIdx.y;
    float s0 = 0.f, s1 = 0.f;
    for (int i = ty; i < 64; i += 8) {
        const int64_t r = r0 + i, c = c0 + 2 * tx;
        __nv_bfloat162 v = __floats2bfloat162_rn(0.f, 0.f);
        if (r < R && c < C) v = *reinterpret_cast<const __nv_bfloat162*>(in + r * C + c);
        t[i][2 * tx] = v.x;
        t[i][2 * tx + 1] = v.y;
        s0 += __bfloat162float(v.x);
        s1 += __bfloat162float(v.y);
    }
    if (part) {
        red[ty][2 * tx] = s0;
        red[ty][2 * tx + 1] = s1;
    }
    __syncthreads();
    if (part && ty == 0) {
        for (int h = 0; h < 2; ++h) {
            const int64_t c = c0 + 2 * tx + h;
            float a = 0.f;
            for (int y = 0; y < 8; ++y) a += red[y][2 * tx + h];
            if (c < C) part[blockIdx.y * C + c] = a;
        }
    }
    for (int i = ty; i < 64; i += 8) {
        const int64_t c = c0 + i, r = r0 + 2 * tx;
        if (c < C && r < R) {
            __nv_bfloat162 v;
            v.x = t[2 * tx][i];
            v.y = t[2 * tx + 1][i];
            *reinterpret_cast<__nv_bfloat162*>(out + c * R + r) = v;
        }
    }
}

// g[c] += sum over r of part[r * C + c]: 32 columns x 8 row phases per
// block, `rows_per_block` rows per block, one atomic per column per block
__global__ void __launch_bounds__(256) k_colsum_parts(const float* __restrict__ part, int64_t nrows, int C,
                                                      int64_t rows_per_block, float* __restrict__ g) {
    __shared__ float red[8][32];
    const int c = blockIdx.x * 32 + threadIdx.x;
    const int64_t r0 = blockIdx.y * rows_per_block, r1 = min(nrows, r0 + rows_per_block);
    float a = 0.f;
    if (c < C)
        for (int64_t r = r0 + threadIdx.y; r < r1; r += 8) a += part[r * C + c];
    red[threadIdx.y][threadIdx.x] = a;
    __syncthreads();
    if (threadIdx.y == 0 && c < C) {
        float t = 0.f;
        for (int y = 0; y < 8; ++y) t += red[y][threadIdx.x];
        atomicAdd(g + c, t);
    }
}

// g[c] += sum over rows of in[r, c] (bf16 in, fp32 partial sums per block)
__global__ void k_colsum(const __nv_bfloat16* __restrict__ in, int64_t R, int C, int64_t rows_per_block,
                         float* __restrict__ g) {
    const int64_t r0 = blockIdx.x * rows_per_block;
    const int64_t r1 = min(R, r0 + rows_per_block);
    for (int c = threadIdx.x; c < C; c += blockDim.x) {
        float s = 0.f;
        for (int64_t r = r0; r < r1; ++r) s += __bfloat162float(in[r * C + c]);
        atomicAdd(g + c, s);
    }
}

// gradient flowing into a pooled channel (zero where the pooled value is 0:
// every row of that channel was cut by the ReLU)
__device__ __forceinline__ float pooled_grad(const float* dh0, const __nv_bfloat16* h0, int c, int ch) {
    const int64_t i = (int64_t)(c >> 1) * kH0 + (c & 1) * kD3 + ch;
    return __bfloat162float(h0[i]) > 0.f ? dh0[i] : 0.f;
}

// dW3[n, :] = sum over clouds of g(c, n) X2[argmax(c, n), :];  db3[n] = sum g.
// One channel and one of kPoolParts cloud ranges per block, one input
// feature per thread; the ranges' sums are combined by atomics.  Clouds go
// in chunks: the chunk's gradients and argmax rows are staged in shared
// memory by independent loads, then the X2 rows are gathered kGather at a
// time, so the loads overlap.
constexpr int kPoolChunk = 1024;
constexpr int kPoolParts = 4;  // cloud ranges per channel (k_pool_bwd_w3's grid.y)
constexpr int kGather = 8;
__global__ void __launch_bounds__(kD2) k_pool_bwd_w3(int nclouds, const float* __restrict__ dh0,
                                                    const __nv_bfloat16* __restrict__ h0, const int32_t* __restrict__ amax,
                                                    const __nv_bfloat16* __restrict__ x2, float* __restrict__ gw3,
                                                    float* __restrict__ gb3) {
    __shared__ float s_g[kPoolChunk];
    __shared__ int32_t s_row[kPoolChunk];  // argmax row within the cloud
    const int n = blockIdx.x, k = threadIdx.x;
    // this block's share of the clouds: gridDim.y parts, combined by atomics
    const int per = (nclouds + gridDim.y - 1) / gridDim.y;
    const int cbeg = blockIdx.y * per, cend = min(nclouds, cbeg + per);
    float acc = 0.f, accb = 0.f;
    for (int c0 = cbeg; c0 < cend; c0 += kPoolChunk) {
        const int cn = min(kPoolChunk, cend - c0);
        __syncthreads();
        for (int i = k; i < cn; i += kD2) {
            s_g[i] = pooled_grad(dh0, h0, c0 + i, n);
            s_row[i] = amax[(c0 + i) * kD3 + n];
        }
        __syncthreads();
        for (int i0 = 0; i0 < cn; i0 += kGather) {
            float xv[kGather];
#pragma unroll
            for (int j = 0; j < kGather; ++j) {
                const int i = min(i0 + j, cn - 1);
                xv[j] = __bfloat162float(x2[((int64_t)(c0 + i) * kP + s_row[i]) * kD2 + k]);
            }
#pragma unroll
            for (int j = 0; j < kGather; ++j) {
                const int i = i0 + j;
                if (i < cn) {
                    const float g = s_g[i];
                    if (g != 0.f) {
                        acc += g * xv[j];
                        accb += g;
                    }
                }
            }
        }
    }
    atomicAdd(gw3 + n * kD2 + k, acc);
    if (k == 0) atomicAdd(gb3 + n, accb);
}

// dY2 = (sum over channels n of g(c, n) W3[n, :] scattered to row argmax(c, n))
//       masked by X2 > 0, as dense bf16 rows.  One cloud per block.  The
// channels with a gradient are bucketed by their argmax row (a stable
// counting sort: channel order kept within a row); then each row's 128
// outputs are summed over its bucket in channel order and written at once,
// zero rows included, as column pairs (four rows per pass).
__global__ void __launch_bounds__(256) k_pool_bwd_x2(const float* __restrict__ dh0, const __nv_bfloat16* __restrict__ h0,
                                                    const int32_t* __restrict__ amax, const __nv_bfloat16* __restrict__ w3,
                                                    const __nv_bfloat16* __restrict__ x2, __nv_bfloat16* __restrict__ dy2) {
    static_assert(kD3 == 256 && kP == 256 && kD2 == 128, "one thread per channel and per row; 64 column pairs x 4 rows per pass");
    __shared__ float s_g[kD3];
    __shared__ int32_t s_row[kD3];
    __shared__ int32_t s_start[kP + 1];  // bucket of row r: s_list[s_start[r] .. s_start[r + 1])
    __shared__ int32_t s_list[kD3];
    const int c = blockIdx.x, t = threadIdx.x;
    const float g = pooled_grad(dh0, h0, c, t);
    const int r = amax[c * kD3 + t];
    s_g[t] = g;
    s_row[t] = g != 0.f ? r : -1;
    __syncthreads();
    // count of row t (thread t), then an exclusive scan over the 256 rows
    int cnt = 0;
    for (int n = 0; n < kD3; ++n) cnt += s_row[n] == t;
    int x = cnt;
    const int lane = t & 31, wid = t >> 5;
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __shared__ int32_t s_warp[8];
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    int before = 0;
    for (int w = 0; w < wid; ++w) before += s_warp[w];
    s_start[t] = before + x - cnt;
    if (t == kP - 1) s_start[kP] = before + x;
    __syncthreads();
    // channel t goes after the channels below it with the same row
    if (s_row[t] >= 0) {
        int rank = 0;
        for (int n = 0; n < t; ++n) rank += s_row[n] == s_row[t];
        s_list[s_start[s_row[t]] + rank] = t;
    }
    __syncthreads();
    // column pair kp of rows r0 + quarter: a warp moves 128 contiguous bytes
    const int kp = t & (kD2 / 2 - 1), quarter = t >> 6;
    const int64_t base = (int64_t)c * kP;
    for (int r0 = 0; r0 < kP; r0 += 4) {
        const int row = r0 + quarter;
        float a0 = 0.f, a1 = 0.f;
        for (int j = s_start[row]; j < s_start[row + 1]; ++j) {
            const int n = s_list[j];
            const __nv_bfloat162 w = *reinterpret_cast<const __nv_bfloat162*>(w3 + n * kD2 + 2 * kp);
            a0 += s_g[n] * __bfloat162float(w.x);
            a1 += s_g[n] * __bfloat162float(w.y);
        }
        const int64_t idx = (base + row) * kD2 + 2 * kp;
        const __nv_bfloat162 xv = *reinterpret_cast<const __nv_bfloat162*>(x2 + idx);
        *reinterpret_cast<__nv_bfloat162*>(dy2 + idx) = __floats2bfloat162_rn(__bfloat162float(xv.x) > 0.f ? a0 : 0.f,
                                                                               __bfloat162float(xv.y) > 0.f ? a1 : 0.f);
    }
}

// dW1 += dY1^T x0, db1 += colsum(dY1): 64 outputs x 4 row phases per block
__global__ void __launch_bounds__(256) k_bwd_w1(const __nv_bfloat16* __restrict__ dy1, const float* __restrict__ x0, int64_t R,
                                               int64_t rows_per_block, float* __restrict__ gw1, float* __restrict__ gb1) {
    __shared__ float red[4][kD1][4];
    const int o = threadIdx.x & 63, ph = threadIdx.x >> 6;
    const int64_t r0 = blockIdx.x * rows_per_block, r1 = min(R, r0 + rows_per_block);
    float a0 = 0.f, a1 = 0.f, a2 = 0.f, ab = 0.f;
#pragma unroll 4
    for (int64_t r = r0 + ph; r < r1; r += 4) {
        const float d = __bfloat162float(dy1[r * kD1 + o]);
        a0 += d * x0[3 * r];
        a1 += d * x0[3 * r + 1];
        a2 += d * x0[3 * r + 2];
        ab += d;
    }
    red[ph][o][0] = a0;
    red[ph][o][1] = a1;
    red[ph][o][2] = a2;
    red[ph][o][3] = ab;
    __syncthreads();
    if (ph == 0) {
        for (int q = 1; q < 4; ++q) {
            a0 += red[q][o][0];
            a1 += red[q][o][1];
            a2 += red[q][o][2];
            ab += red[q][o][3];
        }
        atomicAdd(gw1 + 3 * o, a0);
        atomicAdd(gw1 + 3 * o + 1, a1);
        atomicAdd(gw1 + 3 * o + 2, a2);
        atomicAdd(gb1 + o, ab);
    }
}

// AdamW on the flat fp32 vector (decoupled weight decay on weight matrices only)
__global__ void k_adamw(int64_t n, float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m,
                        float* __restrict__ v, const uint8_t* __restrict__ decay, float lr, float b1, float b2, float eps,
                        float wd, float bc1, float bc2) {
    const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    const float upd = (mi / bc1) / (sqrtf(vi / bc2) + eps);
    p[i] = p[i] - lr * (upd + (decay[i] ? wd * p[i] : 0.f));
}

// bf16 copies of an [R, C] fp32 weight: W (R x C) and W^T (C x R)
__global__ void k_cast_weight(const float* __restrict__ w, int R, int C, __nv_bfloat16* __restrict__ wb,
                              __nv_bfloat16* __restrict__ wt) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= R * C) return;
    const int r = i / C, c = i % C;
    const __nv_bfloat16 h = __float2bfloat16_rn(w[i]);
    wb[i] = h;
    wt[(int64_t)c * R + r] = h;
}

// T = [R(omega) | c_t - R c_s + s delta] (row-major 4x4) from the network output
__global__ void k_finalize(int npairs, const float* __restrict__ out, const float* __restrict__ frame, float* __restrict__ T) {
    const int b = blockIdx.x * blockDim.x + threadIdx.x;
    if (b >= npairs) return;
    const float* o = out + kOut * b;
    const float* f = frame + 7 * b;
    const double wx = o[0], wy = o[1], wz = o[2];
    const double th = sqrt(wx * wx + wy * wy + wz * wz);
    double R[9] = {1, 0, 0, 0, 1, 0, 0, 0, 1};
    if (th > 1e-12) {  // Rodrigues
        const double kx = wx / th, ky = wy / th, kz = wz / th, s = sin(th), c1 = 1.0 - cos(th);
        R[0] = 1 - c1 * (ky * ky + kz * kz);
        R[1] = -s * kz + c1 * kx * ky;
        R[2] = s * ky + c1 * kx * kz;
        R[3] = s * kz + c1 * kx * ky;
        R[4] = 1 - c1 * (kx * kx + kz * kz);
        R[5] = -s * kx + c1 * ky * kz;
        R[6] = -s * ky + c1 * kx * kz;
        R[7] = s * kx + c1 * ky * kz;
        R[8] = 1 - c1 * (kx * kx + ky * ky);
    }
    float* t = T + 16 * b;
    for (int r = 0; r < 3; ++r) {
        const double rc = R[3 * r] * f[0] + R[3 * r + 1] * f[1] + R[3 * r + 2] * f[2];
        t[4 * r] = (float)R[3 * r];
        t[4 * r + 1] = (float)R[3 * r + 1];
        t[4 * r + 2] = (float)R[3 * r + 2];
        t[4 * r + 3] = (float)(f[3 + r] - rc + f[6] * o[3 + r]);
    }
    t[12] = t[13] = t[14] = 0.f;
    t[15] = 1.f;
}

}  // namespace
}  // namespace pvvc

using namespace pvvc;

struct pvvc_regnet {
    int64_t nparam = 0;
    DevBuf p, g, m, v, decay;                          // fp32 master, grad, Adam moments, decay mask
    DevBuf w2b, w2t, w3b, w3t, w4b, w4t, w5b, w5t;     // bf16 copies (W, W^T)
    int64_t step = 0;
    // activations and scratch for up to `cap` pairs
    int64_t cap = 0;
    DevBuf x0, x1, x2, y3, h0, amax, h1, h2, out, frame, y, dh2, dh1, dh0, dy2, dy1, ta, tb, loss, ids;
    DevBuf part;  // column sums of dY2 per 64-row tile (the db2 reduction)
};

namespace {
uint64_t splitmix(uint64_t& s) {
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

int ensure_cap(pvvc_regnet* n, int64_t B) {
    if (B <= n->cap) return PVVC_OK;
    const int64_t M = 2 * B * kP;
    bool ok = n->x0.ensure(12 * M) == cudaSuccess && n->x1.ensure(2 * M * kD1) == cudaSuccess &&
              n->x2.ensure(2 * M * kD2) == cudaSuccess && n->y3.ensure(2 * M * kD3) == cudaSuccess &&
              n->h0.ensure(2 * B * kH0) == cudaSuccess && n->amax.ensure(4 * 2 * B * kD3) == cudaSuccess &&
              n->h1.ensure(2 * B * kH1) == cudaSuccess && n->h2.ensure(2 * B * kH2) == cudaSuccess &&
              n->out.ensure(4 * B * kOut) == cudaSuccess && n->frame.ensure(4 * B * 7) == cudaSuccess &&
              n->y.ensure(4 * B * kOut) == cudaSuccess && n->dh2.ensure(2 * B * kH2) == cudaSuccess &&
              n->dh1.ensure(2 * B * kH1) == cudaSuccess && n->dh0.ensure(4 * B * kH0) == cudaSuccess &&
              n->dy2.ensure(2 * M * kD2) == cudaSuccess && n->dy1.ensure(2 * M * kD1) == cudaSuccess &&
              n->ta.ensure(2 * M * kD2) == cudaSuccess && n->tb.ensure(2 * M * kD1 + 2 * B * kH0) == cudaSuccess &&
              n->loss.ensure(16) == cudaSuccess && n->ids.ensure(4 * B) == cudaSuccess &&
              n->part.ensure(4 * ((M + 63) / 64) * kD2) == cudaSuccess;
    if (!ok) return PVVC_ERR_NOMEM;
    n->cap = B;
    return PVVC_OK;
}

int refresh_bf16(pvvc_regnet* n, cudaStream_t s) {
    const float* p = static_cast<const float*>(n->p.p);
    struct {
        int64_t off;
        int R, C;
        DevBuf *wb, *wt;
    } ws[] = {{kL.w2, kD2, kD1, &n->w2b, &n->w2t},
              {kL.w3, kD3, kD2, &n->w3b, &n->w3t},
              {kL.w4, kH1, kH0, &n->w4b, &n->w4t},
              {kL.w5, kH2, kH1, &n->w5b, &n->w5t}};
    for (auto& w : ws) {
        const int cnt = w.R * w.C;
        k_cast_weight<<<(cnt + 255) / 256, 256, 0, s>>>(p + w.off, w.R, w.C, static_cast<__nv_bfloat16*>(w.wb->p),
                                                        static_cast<__nv_bfloat16*>(w.wt->p));
    }
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

#define BF(x) static_cast<__nv_bfloat16*>(n->x.p)
#define F32(x) static_cast<float*>(n->x.p)

// Forward from X1 (already written) through the head.  y == nullptr: no loss.
int forward_from_x1(pvvc_regnet* n, int64_t B, const float* y, float lambda_w, bool grads, cudaStream_t s) {
    const int64_t M = 2 * B * kP;
    const float* p = F32(p);
    int rc;
    if ((rc = gemm_bf16((int32_t)M, kD2, kD1, BF(x1), kD1, BF(w2b), kD1, BF(x2), kD2, p + kL.b2, nullptr, 0,
                        PVVC_GEMM_BIAS_RELU_BF16, 1, s)))
        return rc;
    if ((rc = gemm_bf16((int32_t)M, kD3, kD2, BF(x2), kD2, BF(w3b), kD2, BF(y3), kD3, p + kL.b3, nullptr, 0,
                        PVVC_GEMM_BIAS_RELU_BF16, 1, s)))
        return rc;
    k_pool<<<(unsigned)(2 * B), kD3, 0, s>>>(BF(y3), BF(h0), static_cast<int32_t*>(n->amax.p));
    if ((rc = gemm_bf16((int32_t)B, kH1, kH0, BF(h0), kH0, BF(w4b), kH0, BF(h1), kH1, p + kL.b4, nullptr, 0,
                        PVVC_GEMM_BIAS_RELU_BF16, 1, s)))
        return rc;
    if ((rc = gemm_bf16((int32_t)B, kH2, kH1, BF(h1), kH1, BF(w5b), kH1, BF(h2), kH2, p + kL.b5, nullptr, 0,
                        PVVC_GEMM_BIAS_RELU_BF16, 1, s)))
        return rc;
    float* g = F32(g);
    k_head<<<(unsigned)B, kH2, 0, s>>>((int)B, BF(h2), p + kL.w6, p + kL.b6, grads ? y : nullptr, lambda_w, F32(out),
                                       F32(loss), g + kL.w6, g + kL.b6, BF(dh2));
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

// dW += dY^T X over `rows` rows: transposes into scratch, then a split-K GEMM.
// With gb and part (scratch of ceil(rows/64) * dout floats) and even sizes,
// the transpose of dY also yields db += column sums of dY.
int weight_grad(int64_t rows, int dout, int din, const __nv_bfloat16* dy, const __nv_bfloat16* x, __nv_bfloat16* dyT,
                __nv_bfloat16* xT, float* gw, cudaStream_t s, float* gb = nullptr, float* part = nullptr) {
    const bool pairs = rows % 2 == 0 && dout % 2 == 0 && din % 2 == 0;
    auto transpose = [&](const __nv_bfloat16* in, int cols, __nv_bfloat16* out, float* prt) {
        dim3 blk(32, 8);
        if (pairs)
            k_transpose_pairs<<<dim3((cols + 63) / 64, (unsigned)((rows + 63) / 64)), blk, 0, s>>>(in, rows, cols, out, prt);
        else
            k_transpose<<<dim3((cols + 31) / 32, (unsigned)((rows + 31) / 32)), blk, 0, s>>>(in, rows, cols, out);
    };
    const bool fused_db = gb && part && pairs;
    transpose(dy, dout, dyT, fused_db ? part : nullptr);
    if (fused_db) {
        const int64_t nparts = (rows + 63) / 64, per = 128;
        k_colsum_parts<<<dim3((dout + 31) / 32, (unsigned)((nparts + per - 1) / per)), dim3(32, 8), 0, s>>>(part, nparts, dout,
                                                                                                         per, gb);
    } else if (gb) {
        k_colsum<<<(unsigned)((rows + 1023) / 1024), 128, 0, s>>>(dy, rows, dout, 1024, gb);
    }
    transpose(x, din, xT, nullptr);
    const int nkb = (int)(rows / 64);
    const int splits = std::max(1, std::min(nkb, 2 * sm_count() / std::max(1, (dout + 127) / 128)));
    return gemm_bf16(dout, din, (int32_t)rows, dyT, rows, xT, rows, gw, din, nullptr, nullptr, 0, PVVC_GEMM_F32_ACCUM,
                     splits, s);
}

// Backward after forward_from_x1 (k_head wrote dH2, dW6, db6).  x0 rows for dW1.
int backward(pvvc_regnet* n, int64_t B, cudaStream_t s) {
    const int64_t M = 2 * B * kP;
    float* g = F32(g);
    int rc;
    // head layers: dW5, db5, dH1
    if ((rc = weight_grad(B, kH2, kH1, BF(dh2), BF(h1), BF(ta), BF(tb), g + kL.w5, s))) return rc;
    k_colsum<<<(unsigned)((B + 63) / 64), 128, 0, s>>>(BF(dh2), B, kH2, 64, g + kL.b5);
    if ((rc = gemm_bf16((int32_t)B, kH1, kH2, BF(dh2), kH2, BF(w5t), kH2, BF(dh1), kH1, nullptr, BF(h1), kH1,
                        PVVC_GEMM_MASK_BF16, 1, s)))
        return rc;
    // dW4, db4, dH0 (fp32)
    if ((rc = weight_grad(B, kH1, kH0, BF(dh1), BF(h0), BF(ta), BF(tb), g + kL.w4, s))) return rc;
    k_colsum<<<(unsigned)((B + 63) / 64), 256, 0, s>>>(BF(dh1), B, kH1, 64, g + kL.b4);
    if ((rc = gemm_bf16((int32_t)B, kH0, kH1, BF(dh1), kH1, BF(w4t), kH1, F32(dh0), kH0, nullptr, nullptr, 0, PVVC_GEMM_F32,
                        1, s)))
        return rc;
    // max-pool + layer 3 (sparse): dW3, db3, dY2
    k_pool_bwd_w3<<<dim3(kD3, kPoolParts), kD2, 0, s>>>((int)(2 * B), F32(dh0), BF(h0), static_cast<int32_t*>(n->amax.p), BF(x2), g + kL.w3,
                                      g + kL.b3);
    k_pool_bwd_x2<<<(unsigned)(2 * B), 256, 0, s>>>(F32(dh0), BF(h0), static_cast<int32_t*>(n->amax.p),
                                                                            BF(w3b), BF(x2), BF(dy2));
    // layer 2: dW2, db2, dY1
    if ((rc = weight_grad(M, kD2, kD1, BF(dy2), BF(x1), BF(ta), BF(tb), g + kL.w2, s, g + kL.b2, F32(part))))
        return rc;
    if ((rc = gemm_bf16((int32_t)M, kD1, kD2, BF(dy2), kD2, BF(w2t), kD2, BF(dy1), kD1, nullptr, BF(x1), kD1,
                        PVVC_GEMM_MASK_BF16, 1, s)))
        return rc;
    // layer 1
    k_bwd_w1<<<(unsigned)((M + 511) / 512), 256, 0, s>>>(BF(dy1), F32(x0), M, 512, g + kL.w1, g + kL.b1);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

}  // namespace

extern "C" int pvvc_regnet_param_count(void) { return (int)kL.total; }

extern "C" int pvvc_regnet_create(uint64_t seed, pvvc_regnet** out) {
    if (!out) return PVVC_ERR_ARG;
    *out = nullptr;
    auto n = std::make_unique<pvvc_regnet>();
    n->nparam = kL.total;
    const size_t bytes = 4ull * kL.total;
    if (n->p.ensure(bytes) || n->g.ensure(bytes) || n->m.ensure(bytes) || n->v.ensure(bytes) || n->decay.ensure(kL.total) ||
        n->w2b.ensure(2 * kD2 * kD1) || n->w2t.ensure(2 * kD2 * kD1) || n->w3b.ensure(2 * kD3 * kD2) ||
        n->w3t.ensure(2 * kD3 * kD2) || n->w4b.ensure(2 * kH1 * kH0) || n->w4t.ensure(2 * kH1 * kH0) ||
        n->w5b.ensure(2 * kH2 * kH1) || n->w5t.ensure(2 * kH2 * kH1))
        return PVVC_ERR_NOMEM;
    // He-uniform weights (fan-in), zero biases, from a seeded splitmix64
    std::vector<float> h(kL.total, 0.f);
    std::vector<uint8_t> dec(kL.total, 0);
    uint64_t st = seed;
    auto init = [&](int64_t off, int rows, int fan_in) {
        const double a = std::sqrt(6.0 / fan_in);
        for (int64_t i = 0; i < (int64_t)rows * fan_in; ++i) {
            const double u = (splitmix(st) >> 11) * (1.0 / 9007199254740992.0);
            h[off + i] = (float)((2 * u - 1) * a);
            dec[off + i] = 1;
        }
    };
    init(kL.w1, kD1, 3);
    init(kL.w2, kD2, kD1);
    init(kL.w3, kD3, kD2);
    init(kL.w4, kH1, kH0);
    init(kL.w5, kH2, kH1);
    init(kL.w6, kOut, kH2);
    for (int64_t i = kL.w6; i < kL.w6 + kOut * kH2; ++i) h[i] *= 0.1f;  // small initial output
    if (cudaMemcpy(n->p.p, h.data(), bytes, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemcpy(n->decay.p, dec.data(), kL.total, cudaMemcpyHostToDevice) != cudaSuccess ||
        cudaMemset(n->m.p, 0, bytes) != cudaSuccess || cudaMemset(n->v.p, 0, bytes) != cudaSuccess)
        return PVVC_ERR_CUDA;
    if (refresh_bf16(n.get(), nullptr) || cudaDeviceSynchronize() != cudaSuccess) return PVVC_ERR_CUDA;
    *out = n.release();
    return PVVC_OK;
}

extern "C" int pvvc_regnet_destroy(pvvc_regnet* n) {
    if (!n) return PVVC_ERR_ARG;
    delete n;
    return PVVC_OK;
}

extern "C" int pvvc_regnet_get_params(pvvc_regnet* n, float* host, int64_t count) {
    if (!n || !host || count != n->nparam) return PVVC_ERR_ARG;
    return cudaMemcpy(host, n->p.p, 4ull * count, cudaMemcpyDeviceToHost) == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_regnet_set_params(pvvc_regnet* n, const float* host, int64_t count) {
    if (!n || !host || count != n->nparam) return PVVC_ERR_ARG;
    if (cudaMemcpy(n->p.p, host, 4ull * count, cudaMemcpyHostToDevice) != cudaSuccess) return PVVC_ERR_CUDA;
    const size_t bytes = 4ull * count;
    if (cudaMemset(n->m.p, 0, bytes) != cudaSuccess || cudaMemset(n->v.p, 0, bytes) != cudaSuccess) return PVVC_ERR_CUDA;
    n->step = 0;
    if (refresh_bf16(n, nullptr)) return PVVC_ERR_CUDA;
    return cudaDeviceSynchronize() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_regnet_grad(pvvc_regnet* n, int32_t npairs, const float* x0, const float* y, float lambda_w,
                                float* grad_out, float* loss_out, void* stream) {
    if (!n || npairs <= 0 || !x0 || !y) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = ensure_cap(n, npairs);
    if (rc) return rc;
    const int64_t B = npairs, M = 2 * B * kP;
    if (cudaMemcpyAsync(n->x0.p, x0, 12 * M, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemcpyAsync(n->y.p, y, 4 * B * kOut, cudaMemcpyDeviceToDevice, s) != cudaSuccess ||
        cudaMemsetAsync(n->g.p, 0, 4ull * n->nparam, s) != cudaSuccess || cudaMemsetAsync(n->loss.p, 0, 4, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    const float* p = F32(p);
    k_l1<<<(unsigned)((M + 255) / 256), 256, 0, s>>>(M, F32(x0), p + kL.w1, p + kL.b1, BF(x1));
    if ((rc = forward_from_x1(n, B, F32(y), lambda_w, true, s))) return rc;
    if ((rc = backward(n, B, s))) return rc;
    if (grad_out && cudaMemcpyAsync(grad_out, n->g.p, 4ull * n->nparam, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    if (loss_out && cudaMemcpyAsync(loss_out, n->loss.p, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}

extern "C" int pvvc_regnet_train_step(pvvc_regnet* n, int32_t npairs, const int32_t* pair_ids, const float* src,
                                      const uint32_t* src_off, const float* tgt, const uint32_t* tgt_off, const float* T_label,
                                      const float* omega_label, uint64_t seed, const pvvc_adamw* opt, float* loss_out,
                                      void* stream) {
    if (!n || npairs <= 0 || !pair_ids || !src || !src_off || !tgt || !tgt_off || !T_label || !omega_label || !opt)
        return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = ensure_cap(n, npairs);
    if (rc) return rc;
    const int64_t B = npairs;
    if (cudaMemsetAsync(n->g.p, 0, 4ull * n->nparam, s) != cudaSuccess || cudaMemsetAsync(n->loss.p, 0, 4, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    const float* p = F32(p);
    k_sample_l1<<<(unsigned)B, kP, 0, s>>>((int)B, pair_ids, src, src_off, tgt, tgt_off, seed, p + kL.w1, p + kL.b1, F32(x0),
                                           BF(x1), F32(frame), T_label, omega_label, F32(y));
    if ((rc = forward_from_x1(n, B, F32(y), opt->lambda_w, true, s))) return rc;
    if ((rc = backward(n, B, s))) return rc;
    n->step++;
    const float bc1 = 1.f - (float)std::pow((double)opt->beta1, (double)n->step);
    const float bc2 = 1.f - (float)std::pow((double)opt->beta2, (double)n->step);
    k_adamw<<<(unsigned)((n->nparam + 255) / 256), 256, 0, s>>>(n->nparam, F32(p), F32(g), F32(m), F32(v),
                                                                static_cast<const uint8_t*>(n->decay.p), opt->lr, opt->beta1,
                                                                opt->beta2, opt->eps, opt->weight_decay, bc1, bc2);
    if ((rc = refresh_bf16(n, s))) return rc;
    if (loss_out && cudaMemcpyAsync(loss_out, n->loss.p, 4, cudaMemcpyDeviceToDevice, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}

extern "C" int pvvc_propose(pvvc_regnet* n, int32_t npairs, const float* src, const uint32_t* src_off, const float* tgt,
                            const uint32_t* tgt_off, uint64_t seed, float* T_out, void* stream) {
    if (!n || npairs < 0 || (npairs && (!src || !src_off || !tgt || !tgt_off || !T_out))) return PVVC_ERR_ARG;
    if (npairs == 0) return PVVC_OK;
    cudaStream_t s = (cudaStream_t)stream;
    int rc = ensure_cap(n, npairs);
    if (rc) return rc;
    const int64_t B = npairs;
    const float* p = F32(p);
    k_sample_l1<<<(unsigned)B, kP, 0, s>>>((int)B, nullptr, src, src_off, tgt, tgt_off, seed, p + kL.w1, p + kL.b1, F32(x0),
                                           BF(x1), F32(frame), nullptr, nullptr, nullptr);
    if ((rc = forward_from_x1(n, B, nullptr, 1.f, false, s))) return rc;
    k_finalize<<<(unsigned)((B + 127) / 128), 128, 0, s>>>((int)B, F32(out), F32(frame), T_out);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_regnet_outputs(pvvc_regnet* n, int32_t npairs, float* out6, void* stream) {
    if (!n || !out6 || npairs <= 0 || npairs > n->cap) return PVVC_ERR_ARG;
    return cudaMemcpyAsync(out6, n->out.p, 4ull * kOut * npairs, cudaMemcpyDeviceToDevice, (cudaStream_t)stream) == cudaSuccess
               ? PVVC_OK
               : PVVC_ERR_CUDA;
}
