/*
 * pvvc_oracle.h -- CPU restatement of the patchVVC per-patch decode path.
 *
 * TEST INFRASTRUCTURE ONLY.  This is the parity oracle: plain C, written from
 * the reference's algorithm (each function cites the reference file:line it
 * restates).  Only the tests, the smoke check and the CPU-baseline leg of the
 * benchmark may load it, and only as the checker.  The shipped library never
 * links or calls it.
 *
 * Parity is pinned: the restatement is checked against the reference's own
 * sources compiled here against shim headers (oracle/Makefile, target "ref")
 * and against the golden fixtures those produced (tests/golden/).
 *
 * Build flags matter: -ffp-contract=off so that a*b+c is never fused, which is
 * what the reference's x86 build (no FMA) computes.
 */
#ifndef PVVC_ORACLE_H_
#define PVVC_ORACLE_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* status codes (shared meaning with the product library's per-slice status) */
enum {
    PVO_OK = 0,
    PVO_ERR_ARG = 1,         /* bad argument                                  */
    PVO_ERR_OVERRUN = 2,     /* bitstream ended before all symbols decoded    */
    PVO_ERR_GEOMETRY = 3,    /* occupancy stream short / malformed            */
    PVO_ERR_SIZE = 4,        /* leaf count != slice size                      */
    PVO_ERR_NO_REFERENCE = 5,/* predictive slice without an intra slice       */
    PVO_ERR_BAD_SLICE = 6,   /* slice type has no VALID bit                   */
    PVO_ERR_NOMEM = 7,
};

/* slice type bits (include/common/common.h:31-56) */
#define PVO_TYPE_VALID 0x01u
#define PVO_TYPE_PREDICT 0x02u
#define PVO_TYPE_SKIP 0x04u
#define PVO_TYPE_GEO_ZSTD 0x08u
#define PVO_TYPE_COLOR_ZSTD 0x10u

/* ---- RLGR (src/common/entropy_codec.cc) ---- */
/* Encode n signed symbols; returns bytes written (<= cap) or 0 on overflow. */
size_t pvo_rlgr_encode(const int64_t* sym, size_t n, uint8_t* out, size_t cap);
/* Decode nsym symbols from nbytes of payload into out. Returns PVO_OK or PVO_ERR_OVERRUN. */
int pvo_rlgr_decode(const uint8_t* in, size_t nbytes, size_t nsym, int64_t* out);

/* ---- encoder octree + forward RAHT (src/octree/raht_octree.cc) ---- */
typedef struct pvo_encoder pvo_encoder;
/* MakeTree over n points (xyz interleaved); resolution as octree.resolution. */
pvo_encoder* pvo_encoder_new(const float* xyz, size_t n, float resolution, int* status);
void pvo_encoder_free(pvo_encoder* e);
size_t pvo_encoder_leaf_count(const pvo_encoder* e);
int pvo_encoder_height(const pvo_encoder* e);
/* GetOctree: 25-byte core + BFS occupancy bytes; returns size (0 if cap too small). */
size_t pvo_encoder_geometry(const pvo_encoder* e, uint8_t* out, size_t cap);
/* RAHT of per-input-point YUV (n x 3) -> leaf_count x 3 coefficients, already
 * in stream (reversed) order.  Returns PVO_OK. */
int pvo_encoder_raht(pvo_encoder* e, const float* yuv, float* coef_out);
/* Quantise (GoP_encoding.cc:184-189) and RLGR-encode (entropy_codec.cc:65-159)
 * the coefficients as Y-plane || U-plane || V-plane.  Returns bytes or 0. */
size_t pvo_encode_colors(const float* coef, size_t nleaf, uint8_t qp, uint8_t* out, size_t cap);

/* ---- decoder (src/octree/invert_raht_octree.cc) ---- */
typedef struct pvo_decoder pvo_decoder;
pvo_decoder* pvo_decoder_new(void);
void pvo_decoder_free(pvo_decoder* d);
/* SetSlice: geometry is used only by intra slices; payloads are raw (already
 * zstd-decompressed). */
int pvo_decoder_set_slice(pvo_decoder* d, uint8_t type, uint32_t size, uint8_t qp,
                          const uint8_t* geo, size_t gsz, const uint8_t* col, size_t csz);
size_t pvo_decoder_size(const pvo_decoder* d);
/* GetPatch: leaf centres (pre-transform), leaf YUV, and RGB as the reference
 * rounds it (common.h:154-158), clamped to [0,255] where the reference's cast
 * is undefined.  Any output pointer may be NULL. */
int pvo_decoder_get_patch(const pvo_decoder* d, float* xyz, float* yuv, uint8_t* rgb);
/* FP64 restatement of the inverse RAHT, run beside the FP32 one on every
 * slice once enabled (before the slot's intra slice); the leaf YUV in double. */
void pvo_decoder_enable_fp64(pvo_decoder* d, int on);
int pvo_decoder_get_yuv_fp64(const pvo_decoder* d, double* yuv);

/* per-point rigid transform, mv row-major (pvvc_decompression.cc:141-150) */
void pvo_transform(const float* mv_rowmajor, const float* xyz_in, size_t n, float* xyz_out);
/* YUV -> RGB (common.h:154-158) for one point; rgb_f receives the pre-cast floats */
void pvo_yuv_to_rgb(const float* yuv, uint8_t* rgb, float* rgb_f);

/* ---- whole-frame decode with a thread pool (pvvc_decompression.cc:86-150) ----
 * Slices of one frame (SoA as in the .frame format).  decoders[] is indexed by
 * patch index and persists across frames.  Output: per slice at out_off[i],
 * transformed xyz (float x3) and rgb (u8 x3).  status[i] per slice. */
typedef struct {
    uint32_t n;              /* slice count */
    const int32_t* index;    /* patch index per slice */
    const uint8_t* type;
    const uint32_t* size;
    const uint8_t* qp;
    const float* mv;         /* n x 16, row-major */
    const uint8_t* const* geo;
    const uint32_t* gsz;
    const uint8_t* const* col;
    const uint32_t* csz;
    const uint64_t* out_off; /* point offset of each slice in the output */
} pvo_frame;

int pvo_decode_frame(pvo_decoder** decoders, int ndecoders, const pvo_frame* f,
                     float* xyz_out, uint8_t* rgb_out, int32_t* status, int nthreads);

/* ---- point-to-point ICP restatement (PCL IterativeClosestPoint semantics,
 * src/registration/icp.cc:21-102) and CloudMSE (registration_base.cc:114-158) ---- */
typedef struct {
    float max_corr_dist;     /* icp.correspondence_ths */
    int max_iter;            /* icp.iteration_ths */
    float fitness_eps;       /* icp.mse_ths (Euclidean fitness epsilon) */
    float transform_eps;     /* icp.transformation_ths */
    float mse_abs_eps;       /* absolute MSE change threshold (PCL default 1e-12) */
} pvo_icp_params;

/* Align src onto tgt starting from init (row-major 4x4, may be NULL = identity).
 * Writes the final transform (row-major), fitness score, iterations used and
 * whether it converged. */
int pvo_icp_align(const float* src, size_t ns, const float* tgt, size_t nt,
                  const float* init, const pvo_icp_params* p,
                  float* T_out, float* fitness, int* iters, int* converged);
/* pvo_icp_align over many pairs (point ranges soff/toff) with nthreads threads. */
int pvo_icp_batch(int npairs, const float* src, const uint32_t* soff, const float* tgt, const uint32_t* toff,
                  const pvo_icp_params* p, float* T, float* fit, int* iters, int* conv, int nthreads);
/* Symmetric mean squared NN distance, max of both directions. */
float pvo_cloud_mse(const float* a, size_t na, const float* b, size_t nb);
/* common::MSE::Compute: geometric and Y/U/V errors of p against q and q
 * against p (out[8]: geo p->q, geo q->p, Y, Y, U, U, V, V); brute: exact
 * search over all points instead of the grid. */
int pvo_cloud_quality(const float* p, const uint8_t* prgb, size_t np, const float* q, const uint8_t* qrgb, size_t nq,
                      int brute, double* out);

/* Colour interpolation of the GoP encoder (GoPEncoding::Interpolation and its
 * k-NN loop, src/patch/GoP_encoding.cc:73-95,131-150): for each query point,
 * the k nearest source points by FP32 squared distance (ties: lower source
 * index first; fewer when the source is smaller), weights 1/max(d, 1e-6)
 * normalised by their sum, the weighted RGB, then BT.601 to YUV (common.h:
 * 83-92).  yuv_out: nq x 3 floats.  brute = 1 tests every source point (the
 * definition); brute = 0 searches a uniform grid and returns the same
 * neighbours.  Returns 0 or PVO_ERR_ARG (empty source, k < 1 or k > 64). */
int pvo_knn_colors(const float* q, size_t nq, const float* src, const uint8_t* rgb, size_t ns, int k, int brute,
                   float* yuv_out);
/* pvo_knn_colors over many pairs (query ranges qoff/qn, source ranges soff,
 * outputs at out_off) with the grid search on nthreads threads. */
int pvo_knn_colors_batch(int npairs, const float* q, const uint64_t* qoff, const uint32_t* qn, const float* src,
                         const uint8_t* rgb, const uint32_t* soff, int k, float* yuv, const uint64_t* out_off,
                         int nthreads);

/* libzstd's ZSTD_decompress over a batch of payloads on nthreads host
 * threads (the reference's zstd stage); status 0 or 9 per payload.  Returns
 * -1 when libzstd cannot be loaded. */
int pvo_libzstd_inflate_batch(int n, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len, uint8_t* dst,
                              const uint64_t* dst_off, const uint32_t* dst_cap, int32_t* status, int nthreads);


/* PatchFitting::Compute with direct clustering (patch_fitting.cc:92-381): the
 * GoP's registered patches -> the fitting cloud (k-means centroids, xyz into
 * out[3 * cap]).  The rand() draws come from a private glibc generator seeded
 * like srand(seed).  Returns the point count or -status; stats (optional):
 * {clustering cells, k-means iterations, empty-cluster redraws}. */
long pvo_fitting_cloud(int npatches, const float* const* xyz, const uint32_t* n, float clustering_ths,
                       float clustering_err_ths, int max_iter, unsigned seed, float* out, size_t cap, long* stats);

#ifdef __cplusplus
}
#endif
#endif
