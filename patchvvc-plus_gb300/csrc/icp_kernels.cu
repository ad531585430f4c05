// icp_kernels.cu -- batched point-to-point ICP for the encoder (sm_103a).
//
// Replaces registration::ICP::Align (src/registration/icp.cc:21-102, which
// wraps pcl::IterativeClosestPoint) for many patch pairs at once, and
// ICPBase::CloudMSE (src/registration/registration_base.cc:114-158).
//
//   k_grid   one CTA per pair: a uniform grid over the target points
//            (cubic cells of at least one voxel, spread over the box's
//            shape, about kmul cells per point and at most 16384):
//            bounding box by block reduction,
//            counting sort of the points into cells (shared-memory
//            histogram + block scan), written to the workspace as float4
//            (x, y, z, index of the point in its pair).
//   k_icp    one CTA per pair, all iterations: each thread transforms its
//            source points, finds the exact nearest target point by rings of
//            grid cells (FP32), and accumulates the correspondence sums with
//            Kahan-compensated FP32 additions; the block reduces them in FP64
//            and one thread solves the 3x3 Kabsch problem by a Jacobi SVD in
//            FP64 and applies the convergence tests of the PCL criteria.
//   k_nn_mean  mean squared NN distance of (transformed) query points to a
//            gridded cloud, per pair.
//   k_knn_color  colour interpolation of the GoP encoder (k nearest source
//            points per query point, inverse-distance weights, BT.601 YUV);
//            k_knn_sub turns later frames into residuals against frame 0.
#include <cuda_runtime.h>

#include <cfloat>
#include <cstdint>
#include <mutex>

#include "pvvc_gb300.h"

namespace pvvc {

// Cell budget of a grid over n points: kmul * n cells, at least 64 and at
// most kMaxCells.  A pair's cell-start array (budget + 1 ints) begins at
// kmul * (first point of the pair) + 65 * pair, so the regions of all pairs
// follow from the point offsets alone and never overlap.
constexpr int kMaxCells = 16384;
constexpr int kGridSmem = 4 * (kMaxCells + 1);
constexpr int kIcpCellMul = 2;      // cells per target point, pvvc_icp_batch / pvvc_cloud_mse_batch
constexpr int kNoAllocCellMul = 2;  // cells per target point, pvvc_icp_batch_noalloc
__host__ __device__ __forceinline__ int cell_budget(int kmul, uint32_t n) {
    const long long c = (long long)kmul * n;
    return (int)(c < 64 ? 64 : (c > kMaxCells ? kMaxCells : c));
}
__host__ __device__ __forceinline__ uint64_t cell_base(int kmul, uint32_t first, int pair) {
    return (uint64_t)kmul * first + 65ull * (uint64_t)pair;
}
__host__ __device__ constexpr uint64_t cell_ints(int kmul, uint64_t npoints, int32_t npairs) {
    return (uint64_t)kmul * npoints + 65ull * (uint64_t)npairs;
}

// Error word of the fixed-scratch entry point: set (to PVVC_ERR_CAPACITY) by
// a k_grid CTA whose pair lies beyond the scratch's point capacity; read and
// cleared by icp_error_take (pvvc_device_error_take).
__device__ int g_icp_error = 0;

struct GridHdr {  // per pair
    float lo[3];
    float h;
    int dim[3];
    int pad;
};

// ---------------------------------------------------------------------------
template <int T>
__global__ void __launch_bounds__(T) k_grid(const float* __restrict__ pts, const uint32_t* __restrict__ off,
                                            const float* __restrict__ xform, GridHdr* __restrict__ hdr,
                                            int* __restrict__ cstart, float4* __restrict__ sorted, int kmul,
                                            uint32_t cap = 0xFFFFFFFFu) {
    extern __shared__ int s_cnt[];  // kGridSmem bytes: budget + 1 counters
    __shared__ float s_red[T / 32][6];
    __shared__ float s_box[6];
    __shared__ int s_warp[T / 32];
    const int pair = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t a = off[pair], b = off[pair + 1], n = b - a;
    // cap: the point capacity of a fixed scratch (pvvc_icp_batch_noalloc).
    // A pair whose offsets run past it, or backwards, writes nothing.
    if (b > cap || a > b) {
        if (tid == 0) atomicExch(&g_icp_error, PVVC_ERR_CAPACITY);
        return;
    }
    const int C = cell_budget(kmul, n);
    float M[12];
    const bool tr = xform != nullptr;
    if (tr)
        for (int i = 0; i < 12; ++i) M[i] = xform[pair * 16 + i];
    auto load = [&](uint32_t i, float* p) {
        const float x = pts[3ull * i], y = pts[3ull * i + 1], z = pts[3ull * i + 2];
        if (!tr) {
            p[0] = x; p[1] = y; p[2] = z;
        } else {
            for (int r = 0; r < 3; ++r) p[r] = M[4 * r] * x + M[4 * r + 1] * y + M[4 * r + 2] * z + M[4 * r + 3];
        }
    };
    // bounding box
    float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {-FLT_MAX, -FLT_MAX, -FLT_MAX};
    for (uint32_t i = a + tid; i < b; i += T) {
        float p[3];
        load(i, p);
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], p[k]);
            mx[k] = fmaxf(mx[k], p[k]);
        }
    }
    for (int o = 16; o; o >>= 1)
        for (int k = 0; k < 3; ++k) {
            mn[k] = fminf(mn[k], __shfl_xor_sync(0xffffffffu, mn[k], o));
            mx[k] = fmaxf(mx[k], __shfl_xor_sync(0xffffffffu, mx[k], o));
        }
    if (lane == 0)
        for (int k = 0; k < 3; ++k) {
            s_red[wid][k] = mn[k];
            s_red[wid][3 + k] = mx[k];
        }
    for (int c = tid; c <= C; c += T) s_cnt[c] = 0;
    __syncthreads();
    if (tid == 0) {
        for (int w = 1; w < T / 32; ++w)
            for (int k = 0; k < 3; ++k) {
                s_red[0][k] = fminf(s_red[0][k], s_red[w][k]);
                s_red[0][3 + k] = fmaxf(s_red[0][3 + k], s_red[w][3 + k]);
            }
        // Cells spread over the box's own shape: edge h with about C
        // cells in the box (an elongated patch gets more cells along its long
        // axis), grown until the cell count fits; at least one voxel.
        float e[3], ext = 0.f;
        for (int k = 0; k < 3; ++k) {
            e[k] = n ? s_red[0][3 + k] - s_red[0][k] : 0.f;
            ext = fmaxf(ext, e[k]);
        }
        GridHdr g;
        {
            const float fl = fmaxf(ext / 1024.f, 1e-3f);  // floor for flat axes
            const float vol = fmaxf(e[0], fl) * fmaxf(e[1], fl) * fmaxf(e[2], fl);
            float h = fmaxf(cbrtf(vol / (float)C), 1.0f);
            for (int guard = 0; guard < 200; ++guard) {
                long long cells = 1;
                for (int k = 0; k < 3; ++k) cells *= min((long long)floorf(e[k] / h) + 1, 1023ll);
                if (cells <= C) break;
                h *= 1.05f;
            }
            g.h = h;
        }
        long long cells = 1;
        for (int k = 0; k < 3; ++k) {
            g.lo[k] = n ? s_red[0][k] : 0.f;
            g.dim[k] = n ? min((int)floorf(e[k] / g.h) + 1, 1023) : 1;
            cells *= g.dim[k];
            s_box[k] = g.lo[k];
        }
        // non-finite or absurd extents: one cell holding every point
        if (!(g.h < FLT_MAX) || g.dim[0] < 1 || g.dim[1] < 1 || g.dim[2] < 1 || cells > C) {
            g.h = FLT_MAX;
            g.dim[0] = g.dim[1] = g.dim[2] = 1;
        }
        s_box[3] = g.h;
        s_box[4] = __int_as_float(g.dim[0]);
        s_box[5] = __int_as_float(g.dim[1] * 1024 + g.dim[2]);
        g.pad = 0;
        hdr[pair] = g;
    }
    __syncthreads();
    const float lo0 = s_box[0], lo1 = s_box[1], lo2 = s_box[2], h = s_box[3];
    const int d0 = __float_as_int(s_box[4]), d12 = __float_as_int(s_box[5]), d1 = d12 / 1024, d2 = d12 % 1024;
    auto cell_of = [&](const float* p) {
        int cx = min(max((int)floorf((p[0] - lo0) / h), 0), d0 - 1);
        int cy = min(max((int)floorf((p[1] - lo1) / h), 0), d1 - 1);
        int cz = min(max((int)floorf((p[2] - lo2) / h), 0), d2 - 1);
        return (cz * d1 + cy) * d0 + cx;
    };
    for (uint32_t i = a + tid; i < b; i += T) {
        float p[3];
        load(i, p);
        atomicAdd(&s_cnt[cell_of(p) + 1], 1);
    }
    __syncthreads();
    // exclusive scan of C+1 counters (serial per warp chunk, then warp offsets)
    const int per = (C + 1 + T - 1) / T;
    int loc = 0;
    for (int k = 0; k < per; ++k) {
        const int c = tid * per + k;
        if (c <= C) loc += s_cnt[c];
    }
    int x = loc;
    for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) s_warp[wid] = x;
    __syncthreads();
    if (tid == 0)
        for (int w = 1; w < T / 32; ++w) s_warp[w] += s_warp[w - 1];
    __syncthreads();
    int run = (wid ? s_warp[wid - 1] : 0) + x - loc;
    for (int k = 0; k < per; ++k) {
        const int c = tid * per + k;
        if (c <= C) {
            run += s_cnt[c];
            s_cnt[c] = run;  // inclusive prefix of counts[0..c] == start of cell c (counts shifted by one)
        }
    }
    __syncthreads();
    int* cs = cstart + cell_base(kmul, a, pair);
    for (int c = tid; c <= C; c += T) cs[c] = s_cnt[c];
    __syncthreads();
    for (uint32_t i = a + tid; i < b; i += T) {
        float p[3];
        load(i, p);
        const int slot = atomicAdd(&s_cnt[cell_of(p)], 1);
        sorted[a + slot] = make_float4(p[0], p[1], p[2], __int_as_float((int)(i - a)));
    }
}

// exact nearest neighbour: squared distance (and the point) of the closest
// gridded point to q, searching rings of cells around q's cell clamped into
// the grid; a point in ring r lies at least (r-1)*h from q.  Among points at
// the same distance the one first in the input wins, so the answer does not
// depend on the grid's cell size or on the order the cells are visited in.
__device__ __forceinline__ float grid_nn(const GridHdr& g, const int* __restrict__ cs, const float4* __restrict__ sp, uint32_t base,
                                         float qx, float qy, float qz, float* nx, float* ny, float* nz) {
    const int cx = min(max((int)floorf((qx - g.lo[0]) / g.h), 0), g.dim[0] - 1);
    const int cy = min(max((int)floorf((qy - g.lo[1]) / g.h), 0), g.dim[1] - 1);
    const int cz = min(max((int)floorf((qz - g.lo[2]) / g.h), 0), g.dim[2] - 1);
    float best = FLT_MAX;
    float bx = 0.f, by = 0.f, bz = 0.f;
    int bi = 0x7fffffff;
    const int maxr = max(g.dim[0], max(g.dim[1], g.dim[2]));
    for (int r = 0; r <= maxr; ++r) {
        if (r > 0 && best < FLT_MAX) {
            const float lb = (float)(r - 1) * g.h;
            if (lb * lb * 0.999f > best) break;
        }
        for (int z = max(cz - r, 0); z <= min(cz + r, g.dim[2] - 1); ++z) {
            const bool zr = (z == cz - r) || (z == cz + r);
            // squared distance from q to the cell's box along an axis
            auto gap2 = [&](int c, float q, float lo) {
                const float a = lo + (float)c * g.h, b = a + g.h;
                const float d = q < a ? a - q : (q > b ? q - b : 0.f);
                return d * d;
            };
            const float dz2 = gap2(z, qz, g.lo[2]);
            if (dz2 * 0.999f > best) continue;
            for (int y = max(cy - r, 0); y <= min(cy + r, g.dim[1] - 1); ++y) {
                const float dyz2 = dz2 + gap2(y, qy, g.lo[1]);
                if (dyz2 * 0.999f > best) continue;
                const bool yr = zr || (y == cy - r) || (y == cy + r);
                // on interior rows only the two x faces belong to the ring
                int x = max(cx - r, 0);
                const int xe = min(cx + r, g.dim[0] - 1);
                const int step = yr ? 1 : max(2 * r, 1);
                if (!yr && x != cx - r) x = (cx + r <= xe) ? cx + r : xe + 1;
                for (; x <= xe; x += step) {
                    // a cell farther than the best so far cannot hold a strictly
                    // closer point (0.999: margin for the rounding of the bound)
                    if ((dyz2 + gap2(x, qx, g.lo[0])) * 0.999f > best) continue;
                    const int c = (z * g.dim[1] + y) * g.dim[0] + x;
                    const int e = __ldg(cs + c + 1);
                    for (int k = __ldg(cs + c); k < e; ++k) {
                        const float4 p = __ldg(sp + base + k);
                        const float dx = p.x - qx, dy = p.y - qy, dz = p.z - qz;
                        const float d = dx * dx + dy * dy + dz * dz;
                        const int pi = __float_as_int(p.w);
                        if (d < best || (d == best && pi < bi)) {
                            best = d;
                            bi = pi;
                            bx = p.x;
                            by = p.y;
                            bz = p.z;
                        }
                    }
                }
            }
        }
    }
    *nx = bx;
    *ny = by;
    *nz = bz;
    return best;
}

// ---- FP64 3x3 Kabsch (one-sided Jacobi SVD) ---------------------------------
// A pair of columns is rotated only while |c| > 1e-15 sqrt(a b) (their cosine
// above about 4.5 FP64 ulps, the Demmel-Veselic test); the sweeps end when a
// whole sweep rotates nothing.  The test is relative, so it ends after a few
// sweeps whatever the scale of A (the correspondence sums reach 1e7 and
// more); the rounding of c is below 3.5 ulps of sqrt(a b), so it always ends.
__device__ void svd3(const double* A, double* U, double* S, double* V) {
    double B[9];
    for (int i = 0; i < 9; ++i) {
        B[i] = A[i];
        V[i] = (i % 4 == 0) ? 1.0 : 0.0;
    }
    for (int sweep = 0; sweep < 40; ++sweep) {
        bool rotated = false;
        for (int p = 0; p < 2; ++p)
            for (int q = p + 1; q < 3; ++q) {
                double a = 0, b = 0, c = 0;
                for (int i = 0; i < 3; ++i) {
                    a += B[3 * i + p] * B[3 * i + p];
                    b += B[3 * i + q] * B[3 * i + q];
                    c += B[3 * i + p] * B[3 * i + q];
                }
                if (!(fabs(c) > 1e-15 * sqrt(a * b))) continue;
                rotated = true;
                const double zeta = (b - a) / (2 * c);
                const double t = (zeta >= 0 ? 1.0 : -1.0) / (fabs(zeta) + sqrt(1 + zeta * zeta));
                const double cs = 1 / sqrt(1 + t * t), sn = cs * t;
                for (int i = 0; i < 3; ++i) {
                    const double bp = B[3 * i + p], bq = B[3 * i + q];
                    B[3 * i + p] = cs * bp - sn * bq;
                    B[3 * i + q] = sn * bp + cs * bq;
                    const double vp = V[3 * i + p], vq = V[3 * i + q];
                    V[3 * i + p] = cs * vp - sn * vq;
                    V[3 * i + q] = sn * vp + cs * vq;
                }
            }
        if (!rotated) break;
    }
    for (int j = 0; j < 3; ++j) {
        const double s = sqrt(B[j] * B[j] + B[3 + j] * B[3 + j] + B[6 + j] * B[6 + j]);
        S[j] = s;
        for (int i = 0; i < 3; ++i) U[3 * i + j] = s > 1e-300 ? B[3 * i + j] / s : (i == j ? 1.0 : 0.0);
    }
}

__device__ void kabsch(double n, const double* sp, const double* sq, const double* spq, double* R, double* t) {
    double cp[3], cq[3], H[9], U[9], S[3], V[9];
    for (int a = 0; a < 3; ++a) {
        cp[a] = sp[a] / n;
        cq[a] = sq[a] / n;
    }
    for (int i = 0; i < 3; ++i)
        for (int j = 0; j < 3; ++j) H[3 * i + j] = spq[3 * i + j] - n * cp[i] * cq[j];
    svd3(H, U, S, V);
    auto vut = [&]() {
        for (int i = 0; i < 3; ++i)
            for (int j = 0; j < 3; ++j) R[3 * i + j] = V[3 * i] * U[3 * j] + V[3 * i + 1] * U[3 * j + 1] + V[3 * i + 2] * U[3 * j + 2];
    };
    vut();
    const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) + R[2] * (R[3] * R[7] - R[4] * R[6]);
    if (det < 0) {
        int k = 0;
        for (int j = 1; j < 3; ++j)
            if (S[j] < S[k]) k = j;
        for (int i = 0; i < 3; ++i) V[3 * i + k] = -V[3 * i + k];
        vut();
    }
    for (int i = 0; i < 3; ++i) t[i] = cq[i] - (R[3 * i] * cp[0] + R[3 * i + 1] * cp[1] + R[3 * i + 2] * cp[2]);
}

// Kahan-compensated FP32 accumulator
struct KSum {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x) {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
    __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

constexpr int kIcpThreads = 256;
constexpr int kNSum = 17;  // count, sum p (3), sum q (3), sum p q^T (9), sum d^2

__global__ void __launch_bounds__(kIcpThreads) k_icp(const float* __restrict__ src, const uint32_t* __restrict__ soff,
                                                     const uint32_t* __restrict__ toff, const GridHdr* __restrict__ hdr,
                                                     const int* __restrict__ cstart, const float4* __restrict__ tsorted,
                                                     int kmul, const float* __restrict__ init, pvvc_icp_params prm,
                                                     float* __restrict__ T_out, float* __restrict__ mse_out,
                                                     int32_t* __restrict__ iters_out, uint8_t* __restrict__ conv_out,
                                                     uint32_t cap = 0xFFFFFFFFu) {
    __shared__ double s_part[kIcpThreads / 32][kNSum];
    __shared__ double s_T[16];
    __shared__ float s_Tf[12];
    __shared__ int s_done;
    __shared__ double s_prev;
    const int pair = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t a = soff[pair], b = soff[pair + 1];
    const uint32_t tb = toff[pair];
    if (toff[pair + 1] > cap || tb > toff[pair + 1]) {  // k_grid built no grid for this pair
        if (tid < 16) T_out[pair * 16 + tid] = __int_as_float(0x7fc00000);
        if (tid == 0) {
            if (mse_out) mse_out[pair] = __int_as_float(0x7fc00000);
            if (iters_out) iters_out[pair] = 0;
            if (conv_out) conv_out[pair] = 0;
        }
        return;
    }
    const GridHdr g = hdr[pair];
    const int* cs = cstart + cell_base(kmul, tb, pair);
    const bool empty_t = toff[pair + 1] == tb;
    if (tid == 0) {
        for (int i = 0; i < 16; ++i) s_T[i] = init ? (double)init[pair * 16 + i] : ((i % 5 == 0) ? 1.0 : 0.0);
        s_done = 0;
        s_prev = DBL_MAX;
    }
    __syncthreads();
    const double corr2 = (double)prm.max_corr_dist * (double)prm.max_corr_dist;
    int it = 0, conv = 0;
    while (true) {
        if (tid < 12) s_Tf[tid] = (float)s_T[tid];
        __syncthreads();
        KSum acc[kNSum];
        for (uint32_t i = a + tid; i < b && !empty_t; i += kIcpThreads) {
            const float x = __ldg(src + 3ull * i), y = __ldg(src + 3ull * i + 1), z = __ldg(src + 3ull * i + 2);
            const float qx = s_Tf[0] * x + s_Tf[1] * y + s_Tf[2] * z + s_Tf[3];
            const float qy = s_Tf[4] * x + s_Tf[5] * y + s_Tf[6] * z + s_Tf[7];
            const float qz = s_Tf[8] * x + s_Tf[9] * y + s_Tf[10] * z + s_Tf[11];
            float mx, my, mz;
            const float d = grid_nn(g, cs, tsorted, tb, qx, qy, qz, &mx, &my, &mz);
            if ((double)d > corr2) continue;
            acc[0].add(1.f);
            acc[1].add(qx);
            acc[2].add(qy);
            acc[3].add(qz);
            acc[4].add(mx);
            acc[5].add(my);
            acc[6].add(mz);
            acc[7].add(qx * mx);
            acc[8].add(qx * my);
            acc[9].add(qx * mz);
            acc[10].add(qy * mx);
            acc[11].add(qy * my);
            acc[12].add(qy * mz);
            acc[13].add(qz * mx);
            acc[14].add(qz * my);
            acc[15].add(qz * mz);
            acc[16].add(d);
        }
        // block reduction in FP64
#pragma unroll
        for (int k = 0; k < kNSum; ++k) {
            double v = acc[k].value();
            for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
            if (lane == 0) s_part[wid][k] = v;
        }
        __syncthreads();
        // lane k of warp 0 totals sum k over the warps
        if (wid == 0 && lane < kNSum) {
            double v = 0;
            for (int w = 0; w < kIcpThreads / 32; ++w) v += s_part[w][lane];
            s_part[0][lane] = v;
        }
        __syncwarp();
        if (tid == 0) {
            double sum[kNSum];
            for (int k = 0; k < kNSum; ++k) sum[k] = s_part[0][k];
            const double cnt = sum[0];
            if (cnt < 3) {
                s_done = 2;  // too few correspondences: not converged
            } else {
                double R[9], t[3];
                kabsch(cnt, sum + 1, sum + 4, sum + 7, R, t);
                double Tn[16];
                for (int i = 0; i < 3; ++i)
                    for (int j = 0; j < 4; ++j)
                        Tn[4 * i + j] = R[3 * i] * s_T[j] + R[3 * i + 1] * s_T[4 + j] + R[3 * i + 2] * s_T[8 + j] + (j == 3 ? t[i] : 0.0);
                for (int j = 0; j < 4; ++j) Tn[12 + j] = s_T[12 + j];
                for (int i = 0; i < 16; ++i) s_T[i] = Tn[i];
                ++it;
                const double cosang = 0.5 * (R[0] + R[4] + R[8] - 1.0);
                const double tr2 = t[0] * t[0] + t[1] * t[1] + t[2] * t[2];
                const double mse = sum[16] / cnt;
                if (it >= prm.max_iter) s_done = 1;
                else if (cosang >= 1.0 - (double)prm.transform_eps && tr2 <= (double)prm.transform_eps) s_done = 1;
                else if (fabs(mse - s_prev) < (double)prm.mse_abs_eps) s_done = 1;
                else if (fabs(mse - s_prev) / s_prev < (double)prm.fitness_eps) s_done = 1;
                s_prev = mse;
            }
        }
        __syncthreads();
        const int done = s_done;
        if (done) {
            conv = done == 1;
            break;
        }
        __syncthreads();
    }
    // fitness score of the final transform (getFitnessScore)
    if (tid < 12) s_Tf[tid] = (float)s_T[tid];
    __syncthreads();
    KSum fs;
    for (uint32_t i = a + tid; i < b && !empty_t; i += kIcpThreads) {
        const float x = __ldg(src + 3ull * i), y = __ldg(src + 3ull * i + 1), z = __ldg(src + 3ull * i + 2);
        const float qx = s_Tf[0] * x + s_Tf[1] * y + s_Tf[2] * z + s_Tf[3];
        const float qy = s_Tf[4] * x + s_Tf[5] * y + s_Tf[6] * z + s_Tf[7];
        const float qz = s_Tf[8] * x + s_Tf[9] * y + s_Tf[10] * z + s_Tf[11];
        float mx, my, mz;
        fs.add(grid_nn(g, cs, tsorted, tb, qx, qy, qz, &mx, &my, &mz));
    }
    double v = fs.value();
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_part[wid][0] = v;
    __syncthreads();
    if (tid == 0) {
        double tot = 0;
        for (int w = 0; w < kIcpThreads / 32; ++w) tot += s_part[w][0];
        for (int i = 0; i < 16; ++i) T_out[pair * 16 + i] = (float)s_T[i];
        if (mse_out) mse_out[pair] = (b > a && !empty_t) ? (float)(tot / (double)(b - a)) : -1.0f;
        if (iters_out) iters_out[pair] = it;
        if (conv_out) conv_out[pair] = (uint8_t)(conv && !empty_t);
    }
}

// mean squared NN distance of each pair's (transformed) queries to its grid
__global__ void __launch_bounds__(kIcpThreads) k_nn_mean(const float* __restrict__ q, const uint32_t* __restrict__ qoff,
                                                         const float* __restrict__ xform, const uint32_t* __restrict__ goff,
                                                         const GridHdr* __restrict__ hdr, const int* __restrict__ cstart,
                                                         const float4* __restrict__ sorted, int kmul, float* __restrict__ out) {
    __shared__ double s_part[kIcpThreads / 32];
    const int pair = blockIdx.x, tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t a = qoff[pair], b = qoff[pair + 1];
    const GridHdr g = hdr[pair];
    const uint32_t gb = goff[pair];
    const int* cs = cstart + cell_base(kmul, gb, pair);
    const bool empty = goff[pair + 1] == gb;
    float M[12];
    for (int i = 0; i < 12; ++i) M[i] = xform ? xform[pair * 16 + i] : ((i % 5 == 0) ? 1.f : 0.f);
    KSum acc;
    for (uint32_t i = a + tid; i < b && !empty; i += kIcpThreads) {
        const float x = q[3ull * i], y = q[3ull * i + 1], z = q[3ull * i + 2];
        const float qx = M[0] * x + M[1] * y + M[2] * z + M[3];
        const float qy = M[4] * x + M[5] * y + M[6] * z + M[7];
        const float qz = M[8] * x + M[9] * y + M[10] * z + M[11];
        float mx, my, mz;
        acc.add(grid_nn(g, cs, sorted, gb, qx, qy, qz, &mx, &my, &mz));
    }
    double v = acc.value();
    for (int o = 16; o; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) s_part[wid] = v;
    __syncthreads();
    if (tid == 0) {
        double tot = 0;
        for (int w = 0; w < kIcpThreads / 32; ++w) tot += s_part[w];
        out[pair] = (b > a && !empty) ? (float)(tot / (double)(b - a)) : -1.0f;
    }
}

// ---------------------------------------------------------------------------
// Colour interpolation of the GoP encoder (GoPEncoding::Interpolation and the
// k-NN loop of GoPEncoding::Encode, src/patch/GoP_encoding.cc:73-95,131-150):
// for every point of a query cloud (the GoP's fitting cloud), the k nearest
// points of a source patch by FP32 squared distance, accumulated x, y, z as
// PCL's exact k-d tree does; among equal distances the lower source index
// first.  Weights 1/max(d, 1e-6) normalised by their sum, weighted RGB, then
// BT.601 to YUV (common.h:83-92), each operation rounded in the reference's
// order.  The source patch is gridded by k_grid (points carry their index).
constexpr int kKnnMax = 16;
constexpr int kKnnThreads = 256;

__device__ __forceinline__ bool knn_less(float da, int ia, float db, int ib) { return da < db || (da == db && ia < ib); }

// The min(k, n) nearest gridded points to q, ascending in the thread's
// shared-memory columns ld[0..k-1][tid], li[...]; returns how many.  The
// k-th entry stays in registers: most candidates lose against it, and an
// insertion shifts the column (rare once the k-th distance is tight).
__device__ __forceinline__ int grid_knn(const GridHdr& g, const int* __restrict__ cs, const float4* __restrict__ sp,
                                        uint32_t base, float qx, float qy, float qz, int k, float (*ld)[kKnnThreads],
                                        int (*li)[kKnnThreads]) {
    const int tid = threadIdx.x;
    int cnt = 0;
    float kd = INFINITY;  // the k-th entry (distance, index) once k are held
    int ki = 0x7fffffff;
    const int cx = min(max((int)floorf((qx - g.lo[0]) / g.h), 0), g.dim[0] - 1);
    const int cy = min(max((int)floorf((qy - g.lo[1]) / g.h), 0), g.dim[1] - 1);
    const int cz = min(max((int)floorf((qz - g.lo[2]) / g.h), 0), g.dim[2] - 1);
    auto gap2 = [&](int c, float q, float lo) {
        const float a = lo + (float)c * g.h, b = a + g.h;
        const float d = q < a ? a - q : (q > b ? q - b : 0.f);
        return d * d;
    };
    const int maxr = max(g.dim[0], max(g.dim[1], g.dim[2]));
    for (int r = 0; r <= maxr; ++r) {
        if (r > 0 && cnt == k) {
            const float lb = (float)(r - 1) * g.h;
            if (lb * lb * 0.999f > kd) break;
        }
        for (int z = max(cz - r, 0); z <= min(cz + r, g.dim[2] - 1); ++z) {
            const bool zr = (z == cz - r) || (z == cz + r);
            const float dz2 = gap2(z, qz, g.lo[2]);
            if (dz2 * 0.999f > kd) continue;
            for (int y = max(cy - r, 0); y <= min(cy + r, g.dim[1] - 1); ++y) {
                const float dyz2 = dz2 + gap2(y, qy, g.lo[1]);
                if (dyz2 * 0.999f > kd) continue;
                const bool yr = zr || (y == cy - r) || (y == cy + r);
                int x = max(cx - r, 0);
                const int xe = min(cx + r, g.dim[0] - 1);
                const int step = yr ? 1 : max(2 * r, 1);
                if (!yr && x != cx - r) x = (cx + r <= xe) ? cx + r : xe + 1;
                for (; x <= xe; x += step) {
                    // a cell whose box is farther than the k-th cannot hold a
                    // point that ranks before it (0.999: rounding margin)
                    if ((dyz2 + gap2(x, qx, g.lo[0])) * 0.999f > kd) continue;
                    const int c = (z * g.dim[1] + y) * g.dim[0] + x;
                    const int e = __ldg(cs + c + 1);
                    for (int m = __ldg(cs + c); m < e; ++m) {
                        const float4 p = __ldg(sp + base + m);
                        const float dx = __fsub_rn(p.x, qx), dy = __fsub_rn(p.y, qy), dz = __fsub_rn(p.z, qz);
                        const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                        const int pi = __float_as_int(p.w);
                        if (!knn_less(d, pi, kd, ki)) continue;
                        int j = cnt < k ? cnt++ : k - 1;  // the slot freed (or the k-th, dropped)
                        while (j > 0 && knn_less(d, pi, ld[j - 1][tid], li[j - 1][tid])) {
                            ld[j][tid] = ld[j - 1][tid];
                            li[j][tid] = li[j - 1][tid];
                            --j;
                        }
                        ld[j][tid] = d;
                        li[j][tid] = pi;
                        if (cnt == k) {
                            kd = ld[k - 1][tid];
                            ki = li[k - 1][tid];
                        }
                    }
                }
            }
        }
    }
    return cnt;
}

__global__ void __launch_bounds__(kKnnThreads) k_knn_color(const float* __restrict__ q, const uint64_t* __restrict__ qoff,
                                                           const uint32_t* __restrict__ qn, const uint32_t* __restrict__ soff,
                                                           const GridHdr* __restrict__ hdr, const int* __restrict__ cstart,
                                                           const float4* __restrict__ sorted, int kmul,
                                                           const uint8_t* __restrict__ rgb, int k, float* __restrict__ yuv,
                                                           const uint64_t* __restrict__ out_off, int32_t* __restrict__ status) {
    __shared__ float s_d[kKnnMax][kKnnThreads];
    __shared__ int s_i[kKnnMax][kKnnThreads];
    const int pair = blockIdx.x, tid = threadIdx.x;
    const uint32_t sb = soff[pair], ns = soff[pair + 1] - sb, n = qn[pair];
    const float* qp = q + 3 * qoff[pair];
    float* op = yuv + 3 * out_off[pair];
    if (ns == 0) {  // the reference's k-d tree rejects an empty cloud
        for (uint32_t i = tid; i < 3 * n; i += kKnnThreads) op[i] = 0.f;
        if (tid == 0 && status) status[pair] = PVVC_ERR_ARG;
        return;
    }
    const GridHdr g = hdr[pair];
    const int* cs = cstart + cell_base(kmul, sb, pair);
    const int kk = min(k, (int)ns);
    for (uint32_t t = tid; t < n; t += kKnnThreads) {
        const int cnt = grid_knn(g, cs, sorted, sb, qp[3 * t], qp[3 * t + 1], qp[3 * t + 2], kk, s_d, s_i);
        // GoPEncoding::Interpolation: weights 1/max(d, 1e-6), their sum in
        // order, then the normalised weights times the colours in order
        float sum = 0.f;
        for (int j = 0; j < cnt; ++j) {
            const float d = s_d[j][tid];
            sum = __fadd_rn(sum, __fdiv_rn(1.0f, d <= 1e-6f ? 1e-6f : d));
        }
        float r = 0.f, gc = 0.f, b = 0.f;
        for (int j = 0; j < cnt; ++j) {
            const float d = s_d[j][tid];
            const float wj = __fdiv_rn(__fdiv_rn(1.0f, d <= 1e-6f ? 1e-6f : d), sum);
            const uint8_t* c = rgb + 3 * (size_t)(sb + (uint32_t)s_i[j][tid]);
            r = __fadd_rn(r, __fmul_rn(wj, (float)c[0]));
            gc = __fadd_rn(gc, __fmul_rn(wj, (float)c[1]));
            b = __fadd_rn(b, __fmul_rn(wj, (float)c[2]));
        }
        op[3 * t] = __fadd_rn(__fadd_rn(__fmul_rn(r, 0.299f), __fmul_rn(gc, 0.587f)), __fmul_rn(b, 0.114f));
        op[3 * t + 1] =
            __fadd_rn(__fadd_rn(__fsub_rn(__fmul_rn(r, -0.168736f), __fmul_rn(gc, 0.331264f)), __fmul_rn(b, 0.5f)), 128.0f);
        op[3 * t + 2] =
            __fadd_rn(__fsub_rn(__fsub_rn(__fmul_rn(r, 0.5f), __fmul_rn(gc, 0.418688f)), __fmul_rn(b, 0.081312f)), 128.0f);
    }
    if (tid == 0 && status) status[pair] = PVVC_OK;
}

// residuals of the later frames (GoP_encoding.cc:144-148): pair p with
// base[p] >= 0 subtracts that pair's colours, point by point; the base must
// have no base of its own and as many query points
__global__ void k_knn_sub(int npairs, const uint32_t* __restrict__ qn, const int32_t* __restrict__ base,
                          float* __restrict__ yuv, const uint64_t* __restrict__ out_off, int32_t* __restrict__ status) {
    const int pair = blockIdx.x;
    const int b = base[pair];
    if (b < 0) return;
    if (b >= npairs || base[b] >= 0 || qn[b] != qn[pair]) {
        if (threadIdx.x == 0 && status) status[pair] = PVVC_ERR_ARG;
        return;
    }
    float* o = yuv + 3 * out_off[pair];
    const float* f0 = yuv + 3 * out_off[b];
    for (uint32_t i = threadIdx.x; i < 3 * qn[pair]; i += blockDim.x) o[i] = __fsub_rn(o[i], f0[i]);
}

// ---------------------------------------------------------------------------
// pvvc_icp_batch_noalloc: the same two kernels as pvvc_icp_batch, with the
// target grid kept in a fixed file-scope device array instead of a
// caller-provided workspace, so that the call allocates nothing.
namespace {
constexpr int32_t kNoAllocMaxPairs = 512;
constexpr uint64_t kNoAllocMaxTgtPoints = 1ull << 20;  // 1,048,576 target points
constexpr uint64_t kNoAllocHdrOff = 0;
constexpr uint64_t kNoAllocCellOff = (sizeof(GridHdr) * kNoAllocMaxPairs + 255) / 256 * 256;
constexpr uint64_t kNoAllocSortedOff =
    kNoAllocCellOff + (4ull * cell_ints(kNoAllocCellMul, kNoAllocMaxTgtPoints, kNoAllocMaxPairs) + 255) / 256 * 256;
constexpr uint64_t kNoAllocBytes = kNoAllocSortedOff + (16ull * kNoAllocMaxTgtPoints + 255) / 256 * 256;  // ~25 MB
}  // namespace
}  // namespace pvvc

// Every GPU that loads this library holds this array (~25 MB) until the
// process exits.  All calls share it and it keeps the last call's contents;
// the grid build overwrites every byte a call reads, so nothing needs
// clearing between calls.  Host code must not use the name as a pointer:
// the device address comes from cudaGetSymbolAddress below.
static __device__ __align__(256) unsigned char g_icp_noalloc_scratch[pvvc::kNoAllocBytes];

namespace pvvc {
namespace {
std::mutex g_noalloc_mu;
// Per device ordinal, the CUDA context the cached values belong to: the
// array's device address and k_grid's shared-memory opt-in live only as long
// as that context, so a device reset (a new primary context) makes the next
// call look them up again.
struct CtxCache {
    unsigned long long ctx = 0;  // cuCtxGetId of the context; 0 = nothing cached
    void* addr = nullptr;        // device address of the fixed array
    bool grid_attr = false;      // k_grid's opt-in done
};
CtxCache g_ctx_cache[128];

typedef int (*CtxGetCurrentFn)(void**);
typedef int (*CtxGetIdFn)(void*, unsigned long long*);

// Unique id of the calling thread's current context (0 if it cannot be read).
unsigned long long current_ctx_id() {
    static CtxGetCurrentFn get_cur = nullptr;
    static CtxGetIdFn get_id = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        void* p = nullptr;
        cudaDriverEntryPointQueryResult q;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetCurrent", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_cur = reinterpret_cast<CtxGetCurrentFn>(p);
        p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuCtxGetId", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            get_id = reinterpret_cast<CtxGetIdFn>(p);
    });
    void* ctx = nullptr;
    unsigned long long id = 0;
    if (!get_cur || !get_id || get_cur(&ctx) != 0 || !ctx || get_id(ctx, &id) != 0) return 0;
    return id;
}

// The cache entry of the current device, reset when its context changed.
// Called with g_noalloc_mu held; the runtime has made the context current.
CtxCache* ctx_cache(int dev) {
    if (dev < 0 || dev >= 128) return nullptr;
    unsigned long long id = current_ctx_id();
    if (id == 0 && cudaFree(nullptr) == cudaSuccess) id = current_ctx_id();  // no context yet: create it
    CtxCache& c = g_ctx_cache[dev];
    if (id == 0 || c.ctx != id) c = CtxCache{id, nullptr, false};
    return &c;
}
}  // namespace

// k_grid's histogram takes kGridSmem (64 KB) of dynamic shared memory, above
// the 48 KB default: opt in once per device context (the caller's current
// device).
bool grid_attr_ready() {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return false;
    std::lock_guard<std::mutex> lk(g_noalloc_mu);
    CtxCache* c = ctx_cache(dev);
    if (!c) return false;
    if (!c->grid_attr) {
        if (cudaFuncSetAttribute(k_grid<256>, cudaFuncAttributeMaxDynamicSharedMemorySize, kGridSmem) != cudaSuccess)
            return false;
        c->grid_attr = c->ctx != 0;  // without a context id, opt in on every call
    }
    return true;
}

// Reads and clears the ICP error word (PVVC_ERR_CAPACITY from a pair that lay
// beyond the fixed scratch of pvvc_icp_batch_noalloc).
int icp_error_take(int* code) {
    int v = 0;
    if (cudaMemcpyFromSymbol(&v, g_icp_error, sizeof(int)) != cudaSuccess) return PVVC_ERR_CUDA;
    if (v) {
        const int z = 0;
        if (cudaMemcpyToSymbol(g_icp_error, &z, sizeof(int)) != cudaSuccess) return PVVC_ERR_CUDA;
    }
    *code = v;
    return PVVC_OK;
}

__global__ void k_max2(const float* __restrict__ a, int n, float* __restrict__ o) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) o[i] = fmaxf(a[i], a[i + n]);
}

}  // namespace pvvc

using namespace pvvc;

namespace {
inline uint64_t al(uint64_t v) { return (v + 255) / 256 * 256; }
struct IcpWs {
    GridHdr* hdr;
    int* cstart;
    float4* sorted;
    GridHdr* hdr2;
    int* cstart2;
    float4* sorted2;
    float* tmp;
};
uint64_t ws_bytes(int32_t npairs, uint64_t nsrc, uint64_t ntgt, IcpWs* w, void* base) {
    uint64_t o = 0;
    auto take = [&](uint64_t b) {
        uint64_t r = o;
        o = al(o + b);
        return r;
    };
    const uint64_t h = take(sizeof(GridHdr) * npairs), c = take(4ull * cell_ints(kIcpCellMul, ntgt, npairs)),
                   s = take(16ull * ntgt);
    const uint64_t h2 = take(sizeof(GridHdr) * npairs), c2 = take(4ull * cell_ints(kIcpCellMul, nsrc, npairs)),
                   s2 = take(16ull * nsrc);
    const uint64_t t = take(8ull * npairs);
    if (w && base) {
        uint8_t* p = static_cast<uint8_t*>(base);
        w->hdr = reinterpret_cast<GridHdr*>(p + h);
        w->cstart = reinterpret_cast<int*>(p + c);
        w->sorted = reinterpret_cast<float4*>(p + s);
        w->hdr2 = reinterpret_cast<GridHdr*>(p + h2);
        w->cstart2 = reinterpret_cast<int*>(p + c2);
        w->sorted2 = reinterpret_cast<float4*>(p + s2);
        w->tmp = reinterpret_cast<float*>(p + t);
    }
    return o;
}
}  // namespace

extern "C" int pvvc_icp_workspace_size(int32_t npairs, uint64_t total_src_points, uint64_t total_tgt_points, uint64_t* bytes) {
    if (npairs < 0 || !bytes) return PVVC_ERR_ARG;
    *bytes = ws_bytes(npairs, total_src_points, total_tgt_points, nullptr, nullptr);
    return PVVC_OK;
}

extern "C" int pvvc_icp_batch(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                              const uint32_t* tgt_off, const float* init, const pvvc_icp_params* params, float* T_out,
                              float* mse_out, int32_t* iters_out, uint8_t* converged_out, void* workspace,
                              uint64_t workspace_bytes, uint64_t total_src_points, uint64_t total_tgt_points, void* stream) {
    if (npairs < 0 || !params || params->max_iter < 1) return PVVC_ERR_ARG;
    if (npairs == 0) return PVVC_OK;
    if (!src_xyz || !src_off || !tgt_xyz || !tgt_off || !T_out || !workspace) return PVVC_ERR_ARG;
    IcpWs w;
    if (ws_bytes(npairs, total_src_points, total_tgt_points, &w, workspace) > workspace_bytes) return PVVC_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (!grid_attr_ready()) return PVVC_ERR_CUDA;
    k_grid<256><<<npairs, 256, kGridSmem, s>>>(tgt_xyz, tgt_off, nullptr, w.hdr, w.cstart, w.sorted, kIcpCellMul);
    k_icp<<<npairs, kIcpThreads, 0, s>>>(src_xyz, src_off, tgt_off, w.hdr, w.cstart, w.sorted, kIcpCellMul, init, *params,
                                         T_out, mse_out,
                                         iters_out, converged_out);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_cloud_mse_batch(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                                    const uint32_t* tgt_off, const float* T, float* mse_out, void* workspace,
                                    uint64_t workspace_bytes, uint64_t total_src_points, uint64_t total_tgt_points,
                                    void* stream) {
    if (npairs < 0) return PVVC_ERR_ARG;
    if (npairs == 0) return PVVC_OK;
    if (!src_xyz || !src_off || !tgt_xyz || !tgt_off || !mse_out || !workspace) return PVVC_ERR_ARG;
    IcpWs w;
    if (ws_bytes(npairs, total_src_points, total_tgt_points, &w, workspace) > workspace_bytes) return PVVC_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    // transformed source -> target, and target -> transformed source; max of both
    if (!grid_attr_ready()) return PVVC_ERR_CUDA;
    k_grid<256><<<npairs, 256, kGridSmem, s>>>(tgt_xyz, tgt_off, nullptr, w.hdr, w.cstart, w.sorted, kIcpCellMul);
    k_grid<256><<<npairs, 256, kGridSmem, s>>>(src_xyz, src_off, T, w.hdr2, w.cstart2, w.sorted2, kIcpCellMul);
    k_nn_mean<<<npairs, kIcpThreads, 0, s>>>(src_xyz, src_off, T, tgt_off, w.hdr, w.cstart, w.sorted, kIcpCellMul, w.tmp);
    k_nn_mean<<<npairs, kIcpThreads, 0, s>>>(tgt_xyz, tgt_off, nullptr, src_off, w.hdr2, w.cstart2, w.sorted2, kIcpCellMul,
                                             w.tmp + npairs);
    k_max2<<<(npairs + 255) / 256, 256, 0, s>>>(w.tmp, npairs, mse_out);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

namespace {
uint64_t knn_ws_bytes(int32_t npairs, uint64_t nsrc, GridHdr** hdr, int** cstart, float4** sorted, void* base) {
    uint64_t o = 0;
    auto take = [&](uint64_t b) {
        const uint64_t r = o;
        o = al(o + b);
        return r;
    };
    const uint64_t h = take(sizeof(GridHdr) * npairs), c = take(4ull * cell_ints(kIcpCellMul, nsrc, npairs)),
                   s = take(16ull * nsrc);
    if (base) {
        uint8_t* p = static_cast<uint8_t*>(base);
        *hdr = reinterpret_cast<GridHdr*>(p + h);
        *cstart = reinterpret_cast<int*>(p + c);
        *sorted = reinterpret_cast<float4*>(p + s);
    }
    return o;
}
}  // namespace

extern "C" int pvvc_knn_colors_workspace_size(int32_t npairs, uint64_t total_src_points, uint64_t* bytes) {
    if (npairs < 0 || !bytes) return PVVC_ERR_ARG;
    *bytes = knn_ws_bytes(npairs, total_src_points, nullptr, nullptr, nullptr, nullptr);
    return PVVC_OK;
}

extern "C" int pvvc_knn_colors_batch(int32_t npairs, const float* query_xyz, const uint64_t* query_off,
                                     const uint32_t* query_n, const float* src_xyz, const uint8_t* src_rgb,
                                     const uint32_t* src_off, int32_t k, const int32_t* base_pair, float* yuv_out,
                                     const uint64_t* out_off, int32_t* status, void* workspace, uint64_t workspace_bytes,
                                     uint64_t total_src_points, void* stream) {
    if (npairs < 0 || k < 1 || k > kKnnMax) return PVVC_ERR_ARG;
    if (npairs == 0) return PVVC_OK;
    if (!query_xyz || !query_off || !query_n || !src_xyz || !src_rgb || !src_off || !yuv_out || !out_off || !workspace)
        return PVVC_ERR_ARG;
    GridHdr* hdr = nullptr;
    int* cstart = nullptr;
    float4* sorted = nullptr;
    if (knn_ws_bytes(npairs, total_src_points, &hdr, &cstart, &sorted, workspace) > workspace_bytes) return PVVC_ERR_CAPACITY;
    cudaStream_t s = (cudaStream_t)stream;
    if (!grid_attr_ready()) return PVVC_ERR_CUDA;
    k_grid<256><<<npairs, 256, kGridSmem, s>>>(src_xyz, src_off, nullptr, hdr, cstart, sorted, kIcpCellMul);
    k_knn_color<<<npairs, kKnnThreads, 0, s>>>(query_xyz, query_off, query_n, src_off, hdr, cstart, sorted, kIcpCellMul, src_rgb, k,
                                       yuv_out, out_off, status);
    if (base_pair) k_knn_sub<<<npairs, 256, 0, s>>>(npairs, query_n, base_pair, yuv_out, out_off, status);
    return cudaGetLastError() == cudaSuccess ? PVVC_OK : PVVC_ERR_CUDA;
}

extern "C" int pvvc_icp_batch_noalloc(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                                      const uint32_t* tgt_off, const float* init, const pvvc_icp_params* params, float* T_out,
                                      float* mse_out, int32_t* iters_out, uint8_t* converged_out, uint64_t total_tgt_points,
                                      void* stream) {
    if (npairs < 0 || !params || params->max_iter < 1) return PVVC_ERR_ARG;
    if (npairs > kNoAllocMaxPairs || total_tgt_points > kNoAllocMaxTgtPoints) return PVVC_ERR_CAPACITY;
    if (npairs == 0) return PVVC_OK;
    if (!src_xyz || !src_off || !tgt_xyz || !tgt_off || !T_out) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // the array's device address, looked up with the caller's device current
    // on the first call in each context; that lookup is not allowed while the
    // stream is being captured
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess) return PVVC_ERR_CUDA;
    void* base = nullptr;
    {
        std::lock_guard<std::mutex> lk(g_noalloc_mu);
        CtxCache* c = ctx_cache(dev);
        if (!c) return PVVC_ERR_ARG;
        if (!c->addr) {
            cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
            if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) return PVVC_ERR_CUDA;
            if (cs != cudaStreamCaptureStatusNone) return PVVC_ERR_ARG;
            void* p = nullptr;
            if (cudaGetSymbolAddress(&p, g_icp_noalloc_scratch) != cudaSuccess || !p) return PVVC_ERR_CUDA;
            c->addr = c->ctx ? p : nullptr;  // without a context id, look it up on every call
            base = p;
        } else {
            base = c->addr;
        }
    }
    uint8_t* b = static_cast<uint8_t*>(base);
    GridHdr* hdr = reinterpret_cast<GridHdr*>(b + kNoAllocHdrOff);
    int* cstart = reinterpret_cast<int*>(b + kNoAllocCellOff);
    float4* sorted = reinterpret_cast<float4*>(b + kNoAllocSortedOff);
    if (!grid_attr_ready()) return PVVC_ERR_CUDA;
    // The kernels bound every pair by the array's point capacity themselves
    // (a pair past it gets NaN results and PVVC_ERR_CAPACITY in
    // pvvc_device_error_take), whatever total_tgt_points says.  Launched
    // through cudaLaunchKernel so that the return code is these launches'
    // own, not an error left by earlier unrelated work.
    const float* nul = nullptr;
    int kmul = kNoAllocCellMul;
    uint32_t cap = (uint32_t)kNoAllocMaxTgtPoints;
    void* ga[] = {(void*)&tgt_xyz, (void*)&tgt_off, (void*)&nul, (void*)&hdr, (void*)&cstart, (void*)&sorted, (void*)&kmul,
                  (void*)&cap};
    if (cudaLaunchKernel((const void*)k_grid<256>, dim3(npairs), dim3(256), ga, kGridSmem, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    const int* ccs = cstart;
    const float4* csorted = sorted;
    const GridHdr* chdr = hdr;
    pvvc_icp_params prm = *params;
    void* ia[] = {(void*)&src_xyz, (void*)&src_off, (void*)&tgt_off, (void*)&chdr, (void*)&ccs, (void*)&csorted,
                  (void*)&kmul, (void*)&init, (void*)&prm, (void*)&T_out, (void*)&mse_out, (void*)&iters_out,
                  (void*)&converged_out, (void*)&cap};
    if (cudaLaunchKernel((const void*)k_icp, dim3(npairs), dim3(kIcpThreads), ia, 0, s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    return PVVC_OK;
}
