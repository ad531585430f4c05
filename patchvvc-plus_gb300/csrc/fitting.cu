// fitting.cu -- the encoder's fitting cloud on the GPU: PatchFitting::Compute
// with the direct clustering every reference config selects
// (src/patch/patch_fitting.cc:92-136 Compute, :138-236 Clustering, :238-381
// Split; octree_base.cc:102-162).
//
// Host: the octree descent over the GoP's registered patches (Split), which
// ends in clustering cells -- a cell where some octant would hold points of
// only some patches, or one at the threshold height.  A cell's points are
// its patches' points, patch by patch, in input order; its k is the mean
// point count per patch, rounded.
//
// Device: k_kmeans, one CTA per cell: the reference's seeding (a partial
// Fisher-Yates shuffle from the back, drawing rand() % (i + 1)), then up to
// max_iter rounds of exact nearest-centroid assignment (FP32 squared
// distance accumulated x, y, z; the lower centroid index among equal
// distances, as the exact k-d tree the reference is pinned with), centroid
// sums in point order in FP32, an empty cluster replaced by a random point,
// and the mean centroid shift (square roots in double, summed into a float)
// against clustering_err_ths.
//
// Random numbers.  The reference draws from the process-wide rand(); a call
// here gives every GoP its own generator -- glibc's rand() algorithm seeded
// like srand(seed), through random_r -- so a GoP's fitting cloud equals the
// reference's Compute after srand(seed).  A cell's draws are the next ones
// of its GoP's sequence after the cells before it, which consumed k draws
// each plus one per empty cluster.  Empty clusters are rare, so every cell is
// first run with its draws placed as if none occurred; a cell whose position
// in the sequence turns out different (a cell before it had empty clusters),
// or that used up its window, runs again with the right draws.
#include <cuda_runtime.h>

#include <algorithm>
#include <atomic>
#include <cfloat>
#include <cmath>
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <thread>
#include <vector>

#include "decode_internal.h"
#include "pvvc_gb300.h"

namespace pvvc {
namespace {

struct FitCell {
    uint32_t first;   // first point (into the cells' point array)
    uint32_t n;       // points
    uint32_t k;       // centroids
    uint32_t out;     // first centroid of the GoP's fitting clouds (output index)
    uint64_t draw;    // this cell's window in the draw array
    uint32_t window;  // draws in the window
    int32_t pad;
};

constexpr int kFitThreads = 256;
constexpr uint32_t kFitSlack = 8;  // extra draws per window for empty clusters

// k_kmeans: one CTA per cell of `todo`.  used[c] = draws consumed, or
// window + 1 when the window ran out (the cell must run again).
__global__ void __launch_bounds__(kFitThreads) k_kmeans(const float* __restrict__ pts, const FitCell* __restrict__ cells,
                                                        const int32_t* __restrict__ todo, const uint32_t* __restrict__ draws,
                                                        float* __restrict__ work, float* __restrict__ cbuf,
                                                        float* __restrict__ nbuf, uint32_t* __restrict__ cnt,
                                                        int32_t* __restrict__ asg, float err_ths, int max_iter,
                                                        float* __restrict__ out, uint32_t* __restrict__ used,
                                                        int32_t* __restrict__ iters) {
    __shared__ int s_done;
    __shared__ uint32_t s_used;
    const int ci = todo[blockIdx.x];
    const FitCell c = cells[ci];
    const uint32_t n = c.n, k = c.k;
    float* w = work + 3ull * c.first;
    float* ctr = cbuf + 3ull * c.first;
    float* nxt = nbuf + 3ull * c.first;
    uint32_t* cc = cnt + c.first;
    int32_t* as = asg + c.first;
    const uint32_t* dr = draws + c.draw;
    for (uint32_t i = threadIdx.x; i < 3 * n; i += blockDim.x) w[i] = pts[3ull * c.first + i];
    __syncthreads();
    if (threadIdx.x == 0) {  // seeds (patch_fitting.cc:160-165)
        uint32_t d = 0;
        int nc = 0;
        for (long i = (long)n - 1; i >= (long)n - (long)k && i >= 0; --i) {
            const uint32_t r = d < c.window ? dr[d] : 0u;
            ++d;
            const long j = (long)(r % (uint32_t)(i + 1));
            for (int a = 0; a < 3; ++a) {
                const float t = w[3 * i + a];
                w[3 * i + a] = w[3 * j + a];
                w[3 * j + a] = t;
            }
            for (int a = 0; a < 3; ++a) ctr[3 * nc + a] = w[3 * i + a];
            ++nc;
        }
        s_used = d;
        s_done = 0;
    }
    __syncthreads();
    int iter = 1;
    for (; iter <= max_iter; ++iter) {
        // nearest centroid of every point (:179-189)
        for (uint32_t j = threadIdx.x; j < n; j += blockDim.x) {
            const float px = w[3 * j], py = w[3 * j + 1], pz = w[3 * j + 2];
            float best = FLT_MAX;
            int bi = 0;
            for (uint32_t q = 0; q < k; ++q) {
                const float dx = __fsub_rn(ctr[3 * q], px), dy = __fsub_rn(ctr[3 * q + 1], py),
                            dz = __fsub_rn(ctr[3 * q + 2], pz);
                const float d = __fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz));
                if (d < best) {
                    best = d;
                    bi = (int)q;
                }
            }
            as[j] = bi;
        }
        for (uint32_t q = threadIdx.x; q < k; q += blockDim.x) {
            nxt[3 * q] = nxt[3 * q + 1] = nxt[3 * q + 2] = 0.f;
            cc[q] = 0;
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            // sums in point order, FP32 (:184-188)
            if (k)
                for (uint32_t j = 0; j < n; ++j) {
                    const int q = as[j];
                    nxt[3 * q] = __fadd_rn(nxt[3 * q], w[3 * j]);
                    nxt[3 * q + 1] = __fadd_rn(nxt[3 * q + 1], w[3 * j + 1]);
                    nxt[3 * q + 2] = __fadd_rn(nxt[3 * q + 2], w[3 * j + 2]);
                    cc[q] += 1;
                }
            // new centroids, empty ones drawn at random, and the mean shift (:191-214)
            uint32_t d = s_used;
            float error = 0.f;
            for (uint32_t q = 0; q < k; ++q) {
                if (cc[q] == 0) {
                    const uint32_t r = d < c.window ? dr[d] : 0u;
                    ++d;
                    const uint32_t j = r % n;
                    for (int a = 0; a < 3; ++a) nxt[3 * q + a] = w[3 * j + a];
                } else {
                    const float m = (float)cc[q];
                    for (int a = 0; a < 3; ++a) nxt[3 * q + a] = __fdiv_rn(nxt[3 * q + a], m);
                }
                const double ex = (double)__fsub_rn(nxt[3 * q], ctr[3 * q]);
                const double ey = (double)__fsub_rn(nxt[3 * q + 1], ctr[3 * q + 1]);
                const double ez = (double)__fsub_rn(nxt[3 * q + 2], ctr[3 * q + 2]);
                error = (float)__dadd_rn((double)error,
                                         __dsqrt_rn(__dadd_rn(__dadd_rn(__dmul_rn(ex, ex), __dmul_rn(ey, ey)), __dmul_rn(ez, ez))));
            }
            error = __fdiv_rn(error, (float)k);
            s_used = d;
            s_done = error < err_ths;
        }
        __syncthreads();
        // the new centroids become current (:215-217)
        for (uint32_t i = threadIdx.x; i < 3 * k; i += blockDim.x) ctr[i] = nxt[i];
        __syncthreads();
        if (s_done) break;
    }
    for (uint32_t i = threadIdx.x; i < 3 * k; i += blockDim.x) out[3ull * c.out + i] = ctr[i];
    if (threadIdx.x == 0) {
        used[ci] = s_used > c.window ? c.window + 1 : s_used;
        iters[ci] = iter > max_iter ? max_iter : iter;
    }
}

struct Vec3 {
    float x, y, z;
};

// The octree descent of one GoP (Split, patch_fitting.cc:238-381, with direct
// clustering): cells appended to `cells`, their points to `cpts`.
struct Splitter {
    const float* xyz;              // all points of the call
    const uint32_t* poff;          // patch point ranges (global indices)
    int p0, np;                    // the GoP's patches
    int max_height;
    std::vector<uint32_t> idx;     // point indices, patch by patch, partitioned in place
    std::vector<uint32_t> tmp;
    std::vector<uint8_t> oct;
    std::vector<float>* cpts;
    std::vector<FitCell>* cells;
    uint32_t out_base;             // the GoP's first output centroid
    uint32_t nout = 0;

    void emit(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b) {
        uint64_t total = 0;
        for (int i = 0; i < np; ++i) total += b[i] - a[i];
        FitCell c{};
        c.first = (uint32_t)(cpts->size() / 3);
        c.n = (uint32_t)total;
        c.k = (uint32_t)std::max(0.0f, std::round((float)total / (float)np));
        c.out = out_base + nout;
        nout += c.k;
        for (int i = 0; i < np; ++i)
            for (uint32_t t = a[i]; t < b[i]; ++t) {
                const float* p = xyz + 3ull * idx[t];
                cpts->insert(cpts->end(), p, p + 3);
            }
        cells->push_back(c);
    }
    void split(const std::vector<uint32_t>& a, const std::vector<uint32_t>& b, Vec3 ctr, Vec3 rng, int h) {
        bool empty = true;
        for (int i = 0; i < np; ++i) empty &= a[i] == b[i];
        if (empty) return;
        if (h >= max_height) {
            emit(a, b);
            return;
        }
        // octant of every point: bit 2 x <= cx, bit 1 y <= cy, bit 0 z <= cz
        std::vector<uint32_t> cnt(8 * (size_t)np, 0);
        for (int i = 0; i < np; ++i)
            for (uint32_t t = a[i]; t < b[i]; ++t) {
                const float* p = xyz + 3ull * idx[t];
                const uint8_t o = (uint8_t)(((p[0] > ctr.x ? 0 : 1) << 2) | ((p[1] > ctr.y ? 0 : 1) << 1) | (p[2] > ctr.z ? 0 : 1));
                oct[t] = o;
                ++cnt[8 * (size_t)i + o];
            }
        // CheckSubSpace: every octant holds points of all patches or of none
        for (int s = 0; s < 8; ++s) {
            int nonempty = 0;
            for (int i = 0; i < np; ++i) nonempty += cnt[8 * (size_t)i + s] ? 1 : 0;
            if (nonempty != 0 && nonempty != np) {
                emit(a, b);
                return;
            }
        }
        // stable partition of each patch's range by octant
        std::vector<uint32_t> ca(8 * (size_t)np), cb(8 * (size_t)np);
        for (int i = 0; i < np; ++i) {
            uint32_t at = a[i];
            uint32_t pos[8];
            for (int s = 0; s < 8; ++s) {
                ca[(size_t)s * np + i] = at;
                pos[s] = at;
                at += cnt[8 * (size_t)i + s];
                cb[(size_t)s * np + i] = at;
            }
            for (uint32_t t = a[i]; t < b[i]; ++t) tmp[pos[oct[t]]++] = idx[t];
            std::copy(tmp.begin() + a[i], tmp.begin() + b[i], idx.begin() + a[i]);
        }
        const Vec3 sr{rng.x / 2.0f, rng.y / 2.0f, rng.z / 2.0f};
        for (int s = 0; s < 8; ++s) {
            // SubSpaceCenter (octree_base.cc:102-120)
            const Vec3 sc{(s & 4) ? ctr.x - sr.x / 2.0f : ctr.x + sr.x / 2.0f, (s & 2) ? ctr.y - sr.y / 2.0f : ctr.y + sr.y / 2.0f,
                          (s & 1) ? ctr.z - sr.z / 2.0f : ctr.z + sr.z / 2.0f};
            std::vector<uint32_t> sa(ca.begin() + (size_t)s * np, ca.begin() + (size_t)(s + 1) * np);
            std::vector<uint32_t> sb(cb.begin() + (size_t)s * np, cb.begin() + (size_t)(s + 1) * np);
            split(sa, sb, sc, sr, h + 1);
        }
    }
    // Compute (patch_fitting.cc:92-136)
    void run(float clustering_ths) {
        float mn[3] = {FLT_MAX, FLT_MAX, FLT_MAX}, mx[3] = {FLT_TRUE_MIN, FLT_TRUE_MIN, FLT_TRUE_MIN};
        std::vector<uint32_t> a(np), b(np);
        uint32_t at = 0;
        for (int i = 0; i < np; ++i) {
            a[i] = at;
            for (uint32_t j = poff[p0 + i]; j < poff[p0 + i + 1]; ++j) {
                idx[at++] = j;
                for (int d = 0; d < 3; ++d) {
                    const float v = xyz[3ull * j + d];
                    mn[d] = v < mn[d] ? v : mn[d];
                    mx[d] = v > mx[d] ? v : mx[d];
                }
            }
            b[i] = at;
        }
        const Vec3 ctr{(mx[0] + mn[0]) / 2.0f, (mx[1] + mn[1]) / 2.0f, (mx[2] + mn[2]) / 2.0f};
        const Vec3 rng{mx[0] - mn[0], mx[1] - mn[1], mx[2] - mn[2]};
        const int range_height = (int)std::ceil(std::log2(std::max(rng.x, std::max(rng.y, rng.z))));
        const int ths_height = (int)std::ceil(std::log2(clustering_ths));
        max_height = range_height - ths_height;
        split(a, b, ctr, rng, 0);
    }
};

}  // namespace
}  // namespace pvvc

struct pvvc_fitter {
    pvvc::DevBuf pts, cells, todo, draws, work, cbuf, nbuf, cnt, asg, out, used, iters;
};

using namespace pvvc;

extern "C" int pvvc_fitter_create(pvvc_fitter** out) {
    if (!out) return PVVC_ERR_ARG;
    *out = new (std::nothrow) pvvc_fitter();
    return *out ? PVVC_OK : PVVC_ERR_NOMEM;
}

extern "C" int pvvc_fitter_destroy(pvvc_fitter* f) {
    if (!f) return PVVC_ERR_ARG;
    delete f;
    return PVVC_OK;
}

extern "C" int pvvc_fitting_clouds(pvvc_fitter* f, int32_t ngops, const int32_t* gop_patch, const uint32_t* patch_off,
                                   const float* xyz, const uint32_t* seeds, float clustering_ths, float clustering_err_ths,
                                   int32_t max_iter, float* out_xyz, uint64_t out_cap, uint64_t* out_off, int32_t* stats,
                                   void* stream) {
    if (!f || ngops < 0 || (ngops && (!gop_patch || !patch_off || !xyz || !seeds || !out_off))) return PVVC_ERR_ARG;
    if (!(clustering_ths > 0.f) || max_iter < 1) return PVVC_ERR_ARG;
    cudaStream_t s = (cudaStream_t)stream;
    // ---- the octree descent of every GoP (host threads, one GoP each) ----
    for (int g = 0; g < ngops; ++g)
        if (gop_patch[g + 1] - gop_patch[g] < 1 || gop_patch[g] < 0) return PVVC_ERR_ARG;
    std::vector<std::vector<float>> gpts(ngops);
    std::vector<std::vector<FitCell>> gcells(ngops);
    std::vector<uint32_t> gout(ngops, 0);
    {
        std::atomic<int> next{0};
        auto work = [&] {
            for (int g; (g = next.fetch_add(1)) < ngops;) {
                Splitter sp;
                sp.xyz = xyz;
                sp.poff = patch_off;
                sp.p0 = gop_patch[g];
                sp.np = gop_patch[g + 1] - gop_patch[g];
                const uint32_t npts = patch_off[sp.p0 + sp.np] - patch_off[sp.p0];
                sp.idx.assign(npts, 0);
                sp.tmp.assign(npts, 0);
                sp.oct.assign(npts, 0);
                sp.cpts = &gpts[g];
                sp.cells = &gcells[g];
                sp.out_base = 0;
                sp.run(clustering_ths);
                gout[g] = sp.nout;
            }
        };
        const int nt = (int)std::min<unsigned>(16, std::max(1u, std::thread::hardware_concurrency()));
        std::vector<std::thread> pool;
        for (int t = 1; t < std::min(nt, ngops); ++t) pool.emplace_back(work);
        work();
        for (auto& t : pool) t.join();
    }
    // the GoPs' cells one after another: points, output ranges and cell lists
    std::vector<float> cpts;
    std::vector<FitCell> cells;
    std::vector<uint32_t> gop_first_cell(ngops + 1, 0);
    out_off[0] = 0;
    for (int g = 0; g < ngops; ++g) {
        const uint32_t pbase = (uint32_t)(cpts.size() / 3);
        for (FitCell c : gcells[g]) {
            c.first += pbase;
            c.out += (uint32_t)out_off[g];
            cells.push_back(c);
        }
        cpts.insert(cpts.end(), gpts[g].begin(), gpts[g].end());
        std::vector<float>().swap(gpts[g]);
        out_off[g + 1] = out_off[g] + gout[g];
        gop_first_cell[g + 1] = (uint32_t)cells.size();
    }
    const uint64_t total_out = out_off[ngops];
    if (stats) {
        stats[0] = (int32_t)cells.size();
        stats[1] = stats[2] = stats[3] = 0;
    }
    if (total_out > out_cap) return PVVC_ERR_CAPACITY;
    if (cells.empty()) return PVVC_OK;
    if (!out_xyz) return PVVC_ERR_ARG;
    const uint64_t N = cpts.size() / 3;
    if (N > 0xFFFFFFFFull) return PVVC_ERR_CAPACITY;
    // ---- device buffers ----
    if (f->pts.ensure(12 * N) || f->cells.ensure(sizeof(FitCell) * cells.size()) || f->todo.ensure(4 * cells.size()) ||
        f->work.ensure(12 * N) || f->cbuf.ensure(12 * N) || f->nbuf.ensure(12 * N) || f->cnt.ensure(4 * N) ||
        f->asg.ensure(4 * N) || f->out.ensure(12 * std::max<uint64_t>(total_out, 1)) || f->used.ensure(4 * cells.size()) ||
        f->iters.ensure(4 * cells.size()))
        return PVVC_ERR_NOMEM;
    if (cudaMemcpyAsync(f->pts.p, cpts.data(), 12 * N, cudaMemcpyHostToDevice, s) != cudaSuccess) return PVVC_ERR_CUDA;
    // ---- draws: every GoP's generator, cells placed by the draws before them ----
    std::vector<uint32_t> extra(cells.size(), 0), window(cells.size(), kFitSlack), used(cells.size(), 0);
    std::vector<int32_t> iters(cells.size(), 0);
    std::vector<uint64_t> placed(cells.size(), ~0ull);  // sequence position each cell last ran with
    std::vector<uint8_t> done(cells.size(), 0);
    int rounds = 0;
    for (;;) {
        // positions in each GoP's sequence, from the extra draws known so far
        std::vector<uint64_t> pos(cells.size());
        std::vector<int32_t> todo;
        uint64_t ndraws = 0;
        std::vector<uint64_t> seq_need(ngops, 0);
        for (int g = 0; g < ngops; ++g) {
            uint64_t at = 0;
            for (uint32_t c = gop_first_cell[g]; c < gop_first_cell[g + 1]; ++c) {
                pos[c] = at;
                at += cells[c].k + extra[c];
                if (!done[c] || placed[c] != pos[c]) todo.push_back((int32_t)c);
                seq_need[g] = std::max<uint64_t>(seq_need[g], pos[c] + cells[c].k + window[c]);
            }
        }
        if (todo.empty()) break;
        if (++rounds > 64) return PVVC_ERR_CUDA;  // cannot happen: each round settles the first unsettled cell of a GoP
        // the draw windows of the cells to run
        std::vector<uint64_t> seq_base(ngops + 1, 0);
        for (int g = 0; g < ngops; ++g) seq_base[g + 1] = seq_base[g] + seq_need[g];
        std::vector<uint32_t> draws(std::max<uint64_t>(seq_base[ngops], 1));
        for (int g = 0; g < ngops; ++g) {
            struct random_data rd;
            char state[128];
            std::memset(&rd, 0, sizeof(rd));
            if (initstate_r(seeds[g], state, sizeof(state), &rd) != 0) return PVVC_ERR_ARG;
            for (uint64_t t = 0; t < seq_need[g]; ++t) {
                int32_t r = 0;
                random_r(&rd, &r);
                draws[seq_base[g] + t] = (uint32_t)r;
            }
        }
        for (int g = 0; g < ngops; ++g)
            for (uint32_t c = gop_first_cell[g]; c < gop_first_cell[g + 1]; ++c) {
                cells[c].draw = seq_base[g] + pos[c];
                cells[c].window = cells[c].k + window[c];
            }
        ndraws = draws.size();
        if (f->draws.ensure(4 * ndraws) != cudaSuccess ||
            cudaMemcpyAsync(f->draws.p, draws.data(), 4 * ndraws, cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(f->cells.p, cells.data(), sizeof(FitCell) * cells.size(), cudaMemcpyHostToDevice, s) != cudaSuccess ||
            cudaMemcpyAsync(f->todo.p, todo.data(), 4 * todo.size(), cudaMemcpyHostToDevice, s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        k_kmeans<<<(unsigned)todo.size(), kFitThreads, 0, s>>>(
            static_cast<const float*>(f->pts.p), static_cast<const FitCell*>(f->cells.p), static_cast<const int32_t*>(f->todo.p),
            static_cast<const uint32_t*>(f->draws.p), static_cast<float*>(f->work.p), static_cast<float*>(f->cbuf.p),
            static_cast<float*>(f->nbuf.p), static_cast<uint32_t*>(f->cnt.p), static_cast<int32_t*>(f->asg.p),
            clustering_err_ths, max_iter, static_cast<float*>(f->out.p), static_cast<uint32_t*>(f->used.p),
            static_cast<int32_t*>(f->iters.p));
        if (cudaGetLastError() != cudaSuccess ||
            cudaMemcpyAsync(used.data(), f->used.p, 4 * cells.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaMemcpyAsync(iters.data(), f->iters.p, 4 * cells.size(), cudaMemcpyDeviceToHost, s) != cudaSuccess ||
            cudaStreamSynchronize(s) != cudaSuccess)
            return PVVC_ERR_CUDA;
        for (int32_t c : todo) {
            placed[c] = pos[c];
            if (used[c] > cells[c].window) {  // the window ran out: widen it and run again
                window[c] *= 4;
                done[c] = 0;
                placed[c] = ~0ull;
            } else {
                extra[c] = used[c] - std::min(used[c], cells[c].k);
                done[c] = 1;
            }
        }
    }
    if (cudaMemcpyAsync(out_xyz, f->out.p, 12 * total_out, cudaMemcpyDeviceToHost, s) != cudaSuccess ||
        cudaStreamSynchronize(s) != cudaSuccess)
        return PVVC_ERR_CUDA;
    if (stats) {
        int64_t it = 0, ex = 0;
        for (size_t c = 0; c < cells.size(); ++c) {
            it += iters[c];
            ex += extra[c];
        }
        stats[1] = (int32_t)std::min<int64_t>(it, INT32_MAX);
        stats[2] = (int32_t)ex;
        stats[3] = rounds;
    }
    return PVVC_OK;
}
