// quality_kernels.cu -- the codec's quality measure on the GPU: the symmetric
// nearest-neighbour geometry and Y/U/V errors of two coloured clouds,
// restating common::MSE::Compute (src/registration/registration_base.cc:
// 168-223), from which the decoder reports PSNR (pvvc_decompression.cc:
// 151-171).
//
//   k_q_bbox / k_q_header   bounding box of a cloud and a uniform grid over
//                           it (cell edge h, at most `cap` cells)
//   k_q_count / k_q_scatter counting sort of the cloud's points by cell
//                           (float4 x, y, z, input index)
//   k_scan_*                exclusive prefix sum of the cell counts
//   k_q_query               per query point: the exact nearest neighbour in
//                           the other cloud's grid, searched ring by ring of
//                           cells until no closer point can remain; FP32
//                           squared distance accumulated x, y, z; among
//                           equal distances the lower input index (the
//                           reference's k-d tree leaves that order open);
//                           the squared Y/U/V differences of the two
//                           points' BT.601 colours (common.h:94-98); per-block
//                           sums in double
//   k_q_final               the per-block sums added in block order
//                           (deterministic), divided by the query count
#include <cuda_runtime.h>

#include <algorithm>
#include <cfloat>
#include <cstdint>

#include "pvvc_gb300.h"

namespace pvvc {
namespace {

constexpr int kQThreads = 256;
constexpr int kScanBlock = 1024;  // elements per scan block (4 per thread)
constexpr uint32_t kQMaxCells = 1u << 24;

struct QGrid {
    float lo[3];
    float h;
    int dim[3];
    int ncells;
};

__device__ __forceinline__ int f2ord(float f) {  // order-preserving float -> int
    const int i = __float_as_int(f);
    return i >= 0 ? i : i ^ 0x7FFFFFFF;
}
__device__ __forceinline__ float ord2f(int i) { return __int_as_float(i >= 0 ? i : i ^ 0x7FFFFFFF); }

__global__ void k_q_init(int* mm) {
    if (threadIdx.x < 3) mm[threadIdx.x] = f2ord(FLT_MAX);
    else if (threadIdx.x < 6) mm[threadIdx.x] = f2ord(-FLT_MAX);
}

__global__ void __launch_bounds__(kQThreads) k_q_bbox(const float* __restrict__ xyz, uint32_t n, int* __restrict__ mm) {
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        for (int k = 0; k < 3; ++k) {
            const float v = xyz[3ull * i + k];
            mn[k] = fminf(mn[k], v);
            mx[k] = fmaxf(mx[k], v);
        }
    for (int o = 16; o; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    if ((threadIdx.x & 31) == 0)
        for (int k = 0; k < 3; ++k) {
            atomicMin(mm + k, f2ord(mn[k]));
            atomicMax(mm + 3 + k, f2ord(mx[k]));
        }
}

// A grid over the box with about `cap` cells: cell edge h >= 0.5 spread over
// the box's own shape, grown until the cell count fits.
__global__ void k_q_header(const int* __restrict__ mm, uint32_t n, uint32_t cap, QGrid* __restrict__ g) {
    if (threadIdx.x != 0) return;
    QGrid q;
    float e[3], ext = 0.f;
    for (int k = 0; k < 3; ++k) {
        q.lo[k] = n ? ord2f(mm[k]) : 0.f;
        e[k] = n ? ord2f(mm[3 + k]) - q.lo[k] : 0.f;
        if (!(e[k] >= 0.f) || !(e[k] < 1e30f)) e[k] = 0.f;  // non-finite coordinates: one cell along that axis
        ext = fmaxf(ext, e[k]);
    }
    const float fl = fmaxf(ext / 1024.f, 1e-3f);
    const float vol = fmaxf(e[0], fl) * fmaxf(e[1], fl) * fmaxf(e[2], fl);
    float h = fmaxf(cbrtf(vol / (float)cap), 0.5f);
    long long cells = 0;
    for (int guard = 0; guard < 400; ++guard) {
        cells = 1;
        for (int k = 0; k < 3; ++k) cells *= (long long)floorf(e[k] / h) + 1;
        if (cells <= (long long)cap) break;
        h *= 1.05f;
    }
    q.h = h;
    for (int k = 0; k < 3; ++k) q.dim[k] = (int)floorf(e[k] / h) + 1;
    if (cells > (long long)cap || cells < 1) {  // absurd extents: one cell
        q.h = FLT_MAX;
        q.dim[0] = q.dim[1] = q.dim[2] = 1;
        cells = 1;
    }
    q.ncells = (int)cells;
    *g = q;
}

__device__ __forceinline__ int qcell(const QGrid& g, float v, int k) {
    const int c = (int)floorf(__fdiv_rn(v - g.lo[k], g.h));
    return min(max(c, 0), g.dim[k] - 1);
}

__global__ void __launch_bounds__(kQThreads) k_q_count(const float* __restrict__ xyz, uint32_t n, const QGrid* __restrict__ gp,
                                                     uint32_t* __restrict__ cnt) {
    const QGrid g = *gp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const int cx = qcell(g, xyz[3ull * i], 0), cy = qcell(g, xyz[3ull * i + 1], 1), cz = qcell(g, xyz[3ull * i + 2], 2);
        atomicAdd(cnt + ((size_t)cz * g.dim[1] + cy) * g.dim[0] + cx, 1u);
    }
}

// exclusive scan: each block scans kScanBlock elements and writes its total
__global__ void __launch_bounds__(256) k_scan_blocks(uint32_t* __restrict__ v, uint32_t n, uint32_t* __restrict__ totals) {
    __shared__ uint32_t s_w[8];
    const uint32_t base = blockIdx.x * kScanBlock + threadIdx.x * 4;
    uint32_t a[4], sum = 0;
    for (int k = 0; k < 4; ++k) {
        a[k] = base + k < n ? v[base + k] : 0u;
        sum += a[k];
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = sum;
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_w[wid] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t r = 0;
        for (int w = 0; w < 8; ++w) {
            const uint32_t t = s_w[w];
            s_w[w] = r;
            r += t;
        }
        totals[blockIdx.x] = r;
    }
    __syncthreads();
    uint32_t run = s_w[wid] + x - sum;
    for (int k = 0; k < 4; ++k) {
        if (base + k < n) v[base + k] = run;
        run += a[k];
    }
}
// one block: exclusive scan of the block totals (serial chunks per thread)
__global__ void __launch_bounds__(1024) k_scan_totals(uint32_t* __restrict__ t, uint32_t n) {
    __shared__ uint32_t s[1024];
    const uint32_t per = (n + 1023) / 1024, b = threadIdx.x * per;
    uint32_t sum = 0;
    for (uint32_t k = 0; k < per; ++k)
        if (b + k < n) sum += t[b + k];
    s[threadIdx.x] = sum;
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t r = 0;
        for (int i = 0; i < 1024; ++i) {
            const uint32_t x = s[i];
            s[i] = r;
            r += x;
        }
    }
    __syncthreads();
    uint32_t run = s[threadIdx.x];
    for (uint32_t k = 0; k < per; ++k)
        if (b + k < n) {
            const uint32_t x = t[b + k];
            t[b + k] = run;
            run += x;
        }
}
__global__ void __launch_bounds__(256) k_scan_add(uint32_t* __restrict__ v, uint32_t n, const uint32_t* __restrict__ totals) {
    const uint32_t base = blockIdx.x * kScanBlock;
    const uint32_t add = totals[blockIdx.x];
    for (uint32_t k = threadIdx.x; k < kScanBlock; k += blockDim.x)
        if (base + k < n) v[base + k] += add;
}

__global__ void __launch_bounds__(kQThreads) k_q_scatter(const float* __restrict__ xyz, uint32_t n, const QGrid* __restrict__ gp,
                                                       const uint32_t* __restrict__ start, uint32_t* __restrict__ cursor,
                                                       float4* __restrict__ sorted) {
    const QGrid g = *gp;
    for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float x = xyz[3ull * i], y = xyz[3ull * i + 1], z = xyz[3ull * i + 2];
        const size_t c = ((size_t)qcell(g, z, 2) * g.dim[1] + qcell(g, y, 1)) * g.dim[0] + qcell(g, x, 0);
        const uint32_t at = start[c] + atomicAdd(cursor + c, 1u);
        sorted[at] = make_float4(x, y, z, __int_as_float((int)i));
    }
}

// BT.601 YUV of an RGB point (ColorYUV(const pcl::PointXYZRGB&), common.h:94-98)
__device__ __forceinline__ void yuv601(const uint8_t* c, float* o) {
    const float r = c[0], g = c[1], b = c[2];
    o[0] = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.299f), __fmul_rn(g, 0.587f)), __fmul_rn(b, 0.114f));
    o[1] = __fadd_rn(__fadd_rn(__fsub_rn(__fmul_rn(r, -0.168736f), __fmul_rn(g, 0.331264f)), __fmul_rn(b, 0.5f)), 128.0f);
    o[2] = __fadd_rn(__fsub_rn(__fsub_rn(__fmul_rn(r, 0.5f), __fmul_rn(g, 0.418688f)), __fmul_rn(b, 0.081312f)), 128.0f);
}

// One thread per query point; per-block sums of (d, dY^2, dU^2, dV^2).
__global__ void __launch_bounds__(kQThreads) k_q_query(const float* __restrict__ q, const uint8_t* __restrict__ qrgb, uint32_t nq,
                                                     const QGrid* __restrict__ gp, const uint32_t* __restrict__ start,
                                                     uint32_t nt, const float4* __restrict__ sorted,
                                                     const uint8_t* __restrict__ trgb, double* __restrict__ partial) {
    __shared__ double s_sum[kQThreads / 32][4];
    const QGrid g = *gp;
    double acc[4] = {0, 0, 0, 0};
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < nq && nt > 0) {
        const float x = q[3ull * i], y = q[3ull * i + 1], z = q[3ull * i + 2];
        const int cx = qcell(g, x, 0), cy = qcell(g, y, 1), cz = qcell(g, z, 2);
        float best = FLT_MAX;
        int bi = 0x7FFFFFFF;
        const int rmax = max(g.dim[0], max(g.dim[1], g.dim[2]));
        for (int r = 0; r < rmax; ++r) {
            for (int dz = -r; dz <= r; ++dz) {
                const int zz = cz + dz;
                if (zz < 0 || zz >= g.dim[2]) continue;
                for (int dy = -r; dy <= r; ++dy) {
                    const int yy = cy + dy;
                    if (yy < 0 || yy >= g.dim[1]) continue;
                    // cells of the shell: all of a z or y face, else the two x faces
                    const int step = (abs(dz) == r || abs(dy) == r) ? 1 : 2 * r;
                    for (int dx = -r; dx <= r; dx += step) {
                        const int xx = cx + dx;
                        if (xx < 0 || xx >= g.dim[0]) continue;
                        const size_t c = ((size_t)zz * g.dim[1] + yy) * g.dim[0] + xx;
                        const uint32_t a = start[c], b = start[c + 1];
                        for (uint32_t k = a; k < b; ++k) {
                            const float4 p = sorted[k];
                            const float ex = __fsub_rn(x, p.x), ey = __fsub_rn(y, p.y), ez = __fsub_rn(z, p.z);
                            const float d = __fadd_rn(__fadd_rn(__fmul_rn(ex, ex), __fmul_rn(ey, ey)), __fmul_rn(ez, ez));
                            const int pi = __float_as_int(p.w);
                            if (d < best || (d == best && pi < bi)) {
                                best = d;
                                bi = pi;
                            }
                        }
                    }
                }
            }
            // every point of a ring beyond r lies at least r*h away (with a
            // margin for the rounding of the cell assignment)
            const float bound = (float)r * g.h * 0.99999f;
            if (best < bound * bound) break;
        }
        float qc[3], tc[3];
        yuv601(qrgb + 3ull * i, qc);
        yuv601(trgb + 3ull * bi, tc);
        acc[0] = (double)best;
        for (int k = 0; k < 3; ++k) {
            const double e = (double)__fsub_rn(qc[k], tc[k]);
            acc[1 + k] = e * e;
        }
    }
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    for (int k = 0; k < 4; ++k) {
        double v = acc[k];
        for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0) s_sum[wid][k] = v;
    }
    __syncthreads();
    if (threadIdx.x < 4) {
        double v = 0;
        for (int w = 0; w < kQThreads / 32; ++w) v += s_sum[w][threadIdx.x];
        partial[4ull * blockIdx.x + threadIdx.x] = v;
    }
}

// out[2k + dir] = sums of block partials in block order / query count
__global__ void k_q_final(const double* __restrict__ partial, uint32_t nblocks, uint32_t nq, int dir,
                          double* __restrict__ out) {
    if (threadIdx.x >= 4) return;
    double v = 0;
    for (uint32_t b = 0; b < nblocks; ++b) v += partial[4ull * b + threadIdx.x];
    out[2 * threadIdx.x + dir] = nq ? v / (double)nq : -1.0;
}

// an empty cloud: MSE::Compute sets that side's errors to -1 and returns
// without computing the other (registration_base.cc:168-177)
__global__ void k_q_empty(double* __restrict__ out, int a_empty, int b_empty) {
    if (threadIdx.x < 4) {
        out[2 * threadIdx.x] = a_empty ? -1.0 : 0.0;
        out[2 * threadIdx.x + 1] = b_empty ? -1.0 : 0.0;
    }
}

uint32_t qcap(uint64_t n) {
    const uint64_t c = 4 * n;
    return (uint32_t)(c < 64 ? 64 : (c > kQMaxCells ? kQMaxCells : c));
}
uint64_t al(uint64_t v) { return (v + 255) / 256 * 256; }

// workspace of one grid over n points
struct QLayout {
    uint64_t hdr, mm, cnt, cur, tot, sorted, bytes;
};
QLayout qlayout(uint64_t n, uint64_t at) {
    QLayout l;
    const uint64_t cap = qcap(n);
    l.hdr = at;
    l.mm = al(l.hdr + sizeof(QGrid));
    l.cnt = al(l.mm + 6 * sizeof(int));
    l.cur = al(l.cnt + 4 * (cap + 1));
    l.tot = al(l.cur + 4 * (cap + 1));
    l.sorted = al(l.tot + 4 * ((cap + 1 + kScanBlock - 1) / kScanBlock));
    l.bytes = al(l.sorted + 16 * (n ? n : 1)) - at;
    return l;
}

cudaError_t build_grid(const float* xyz, uint32_t n, uint8_t* ws, const QLayout& l, cudaStream_t s) {
    const uint32_t cap = qcap(n);
    QGrid* g = reinterpret_cast<QGrid*>(ws + l.hdr);
    int* mm = reinterpret_cast<int*>(ws + l.mm);
    uint32_t* cnt = reinterpret_cast<uint32_t*>(ws + l.cnt);
    uint32_t* cur = reinterpret_cast<uint32_t*>(ws + l.cur);
    uint32_t* tot = reinterpret_cast<uint32_t*>(ws + l.tot);
    float4* sorted = reinterpret_cast<float4*>(ws + l.sorted);
    const int blocks = (int)std::min<uint64_t>((n + kQThreads - 1) / kQThreads, 4096);
    k_q_init<<<1, 32, 0, s>>>(mm);
    if (n) k_q_bbox<<<blocks, kQThreads, 0, s>>>(xyz, n, mm);
    k_q_header<<<1, 32, 0, s>>>(mm, n, cap, g);
    if (cudaMemsetAsync(cnt, 0, 4ull * (cap + 1), s) != cudaSuccess || cudaMemsetAsync(cur, 0, 4ull * (cap + 1), s) != cudaSuccess)
        return cudaErrorUnknown;
    if (n) k_q_count<<<blocks, kQThreads, 0, s>>>(xyz, n, g, cnt);
    const uint32_t m = cap + 1, nb = (m + kScanBlock - 1) / kScanBlock;
    k_scan_blocks<<<nb, 256, 0, s>>>(cnt, m, tot);
    k_scan_totals<<<1, 1024, 0, s>>>(tot, nb);
    k_scan_add<<<nb, 256, 0, s>>>(cnt, m, tot);
    if (n) k_q_scatter<<<blocks, kQThreads, 0, s>>>(xyz, n, g, cnt, cur, sorted);
    return cudaGetLastError();
}

}  // namespace
}  // namespace pvvc

using namespace pvvc;

extern "C" int pvvc_cloud_quality_workspace_size(uint64_t npoints_a, uint64_t npoints_b, uint64_t* bytes) {
    if (!bytes) return PVVC_ERR_ARG;
    const QLayout la = qlayout(npoints_a, 0), lb = qlayout(npoints_b, 0);
    const uint64_t nblk = std::max<uint64_t>((npoints_a + kQThreads - 1) / kQThreads, (npoints_b + kQThreads - 1) / kQThreads);
    *bytes = la.bytes + lb.bytes + al(32ull * std::max<uint64_t>(nblk, 1));
    return PVVC_OK;
}

extern "C" int pvvc_cloud_quality(uint64_t npoints_a, const float* xyz_a, const uint8_t* rgb_a, uint64_t npoints_b,
                                  const float* xyz_b, const uint8_t* rgb_b, double* mse_out, void* workspace,
                                  uint64_t workspace_bytes, void* stream) {
    if (!mse_out || !workspace || (npoints_a && (!xyz_a || !rgb_a)) || (npoints_b && (!xyz_b || !rgb_b))) return PVVC_ERR_ARG;
    if (npoints_a > 0x7FFFFFFFull || npoints_b > 0x7FFFFFFFull) return PVVC_ERR_ARG;
    if (reinterpret_cast<uintptr_t>(workspace) & 255u) return PVVC_ERR_ARG;
    uint64_t need = 0;
    pvvc_cloud_quality_workspace_size(npoints_a, npoints_b, &need);
    if (workspace_bytes < need) return PVVC_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (npoints_a == 0 || npoints_b == 0) {
        k_q_empty<<<1, 32, 0, s>>>(mse_out, npoints_a == 0, npoints_b == 0);
        return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
    }
    uint8_t* ws = static_cast<uint8_t*>(workspace);
    const QLayout la = qlayout(npoints_a, 0), lb = qlayout(npoints_b, la.bytes);
    double* partial = reinterpret_cast<double*>(ws + la.bytes + lb.bytes);
    const uint32_t na = (uint32_t)npoints_a, nb = (uint32_t)npoints_b;
    if (build_grid(xyz_a, na, ws, la, s) != cudaSuccess || build_grid(xyz_b, nb, ws, lb, s) != cudaSuccess) return PVVC_ERR_CUDA;
    // direction 0: every point of A against B's grid (MSE's .first); 1: B against A
    for (int dir = 0; dir < 2; ++dir) {
        const uint32_t nq = dir ? nb : na, nt = dir ? na : nb;
        const float* q = dir ? xyz_b : xyz_a;
        const uint8_t* qc = dir ? rgb_b : rgb_a;
        const uint8_t* tc = dir ? rgb_a : rgb_b;
        const QLayout& lt = dir ? la : lb;
        const uint32_t blocks = std::max<uint32_t>((nq + kQThreads - 1) / kQThreads, 1);
        k_q_query<<<blocks, kQThreads, 0, s>>>(q, qc, nq, reinterpret_cast<const QGrid*>(ws + lt.hdr),
                                             reinterpret_cast<const uint32_t*>(ws + lt.cnt), nt,
                                             reinterpret_cast<const float4*>(ws + lt.sorted), tc, partial);
        k_q_final<<<1, 32, 0, s>>>(partial, blocks, nq, dir, mse_out);
    }
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}
