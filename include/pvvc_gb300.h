/*
 * pvvc_gb300.h -- C ABI of the GB300-native patchVVC per-patch codec path.
 *
 * Every entry point is extern "C" with plain pointers and sizes.  Device
 * pointers are CUDA device memory owned by the caller; `stream` is a
 * cudaStream_t passed as void* (NULL = the legacy default stream).  Calls that
 * take a stream are stream-ordered and do not synchronise unless stated.
 * Errors are returned as PVVC_* status codes; per-slice decode failures are
 * reported in a caller-provided status array and never abort the batch.
 *
 * Each declaration names the reference interface it replaces (paths are
 * relative to the patchVVC-plus project root).
 */
#ifndef PVVC_GB300_H_
#define PVVC_GB300_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* ---- status codes ---------------------------------------------------- */
#define PVVC_OK 0
#define PVVC_ERR_ARG 1          /* invalid argument                               */
#define PVVC_ERR_OVERRUN 2      /* colour bitstream ended before 3*size symbols    */
#define PVVC_ERR_GEOMETRY 3     /* occupancy stream short or malformed            */
#define PVVC_ERR_SIZE 4         /* leaf count != slice size, or size > capacity   */
#define PVVC_ERR_NO_REFERENCE 5 /* predictive slice before any intra slice        */
#define PVVC_ERR_BAD_SLICE 6    /* slice type lacks the VALID bit                 */
#define PVVC_ERR_NOMEM 7        /* allocation failed                              */
#define PVVC_ERR_CUDA 8         /* a CUDA runtime call failed                     */
#define PVVC_ERR_ZSTD 9         /* zstd payload without libzstd, or corrupt       */
#define PVVC_ERR_FORMAT 10      /* .frame / .slice bytes malformed                */
#define PVVC_ERR_CAPACITY 11    /* output / workspace too small                   */
#define PVVC_ERR_TREE 12        /* tree deeper or wider than the state slot holds */

/* slice type bits, include/common/common.h:31-56 */
#define PVVC_TYPE_VALID 0x01
#define PVVC_TYPE_PREDICT 0x02
#define PVVC_TYPE_SKIP 0x04
#define PVVC_TYPE_GEO_ZSTD 0x08
#define PVVC_TYPE_COLOR_ZSTD 0x10

const char* pvvc_status_string(int status);

/* ---- per-patch decoder state ---------------------------------------------
 * Replaces the caller-allocated device array of persistent
 * vvc::client::octree::InvertRAHTOctree objects (include/cuda/octree.cuh,
 * src/cuda/common/manager.cc:235-238) and the CPU decoder's per-index
 * handlers (src/codec/pvvc_decompression.cc:119-122).  A state holds `nslots`
 * slots; slot i keeps the tree, leaf centres and reference colours of the
 * last intra slice decoded into it (at most max_leaves leaves and max_nodes
 * internal octree nodes).  Device memory, allocated here. */
typedef struct pvvc_state pvvc_state;
int pvvc_state_create(int32_t nslots, int32_t max_leaves, int32_t max_nodes, pvvc_state** out);
int pvvc_state_destroy(pvvc_state* st);
/* Mark every slot empty (a predictive slice then reports NO_REFERENCE). */
int pvvc_state_reset(pvvc_state* st, void* stream);

/* ---- decode plan ---------------------------------------------------------
 * HOST-side slice metadata of one batch (any mix of intra and predictive
 * slices of any frames, at most one intra slice per slot).  It replaces the
 * host staging of src/cuda/common/manager.cc:41-72 and
 * test/test_decode_only.cc:97-123: the per-slice index/type/size/qp/mv and
 * payload pointers become offsets into one device payload buffer, and
 * inner_offset becomes out_off. */
typedef struct {
    int32_t nslices;
    const int32_t* slot;      /* state slot per slice (the patch index)           */
    const uint8_t* type;      /* slice type bits                                   */
    const uint32_t* size;     /* decoded point count                               */
    const uint8_t* qp;        /* quantisation step                                 */
    const float* mv;          /* nslices x 16 floats, row-major (.frame layout)    */
    const uint64_t* geo_off;  /* byte offset of the raw geometry payload (intra)   */
    const uint32_t* geo_size; /* 0 for predictive slices                           */
    const uint64_t* col_off;  /* byte offset of the raw colour (RLGR) payload      */
    const uint32_t* col_size;
    const uint64_t* out_off;  /* first output point of the slice                   */
} pvvc_batch_desc;

typedef struct pvvc_plan pvvc_plan;
/* Sorts the batch into the work queue (intra first, then by size) and uploads
 * it (synchronous).  The plan is reusable for any payload with the same
 * layout, and pvvc_decode on it is CUDA-graph capturable. */
int pvvc_plan_create(const pvvc_batch_desc* desc, pvvc_plan** out);
int pvvc_plan_destroy(pvvc_plan* plan);
/* total output points, device workspace bytes pvvc_decode needs */
int pvvc_plan_query(const pvvc_plan* plan, uint64_t* total_points, uint64_t* workspace_bytes);

/* Launch shapes of a plan.  A zero field takes the built-in default.  No
 * reference counterpart: the reference launches one thread per slice
 * (src/cuda/render/render.cc:269-301, block = 1).
 *
 * RLGR runs in one of two forms.  Groups of at least 16 slices of one slot,
 * all of one size (the frames of a patch in a GoP), form size tiers of whole
 * groups: the long tier is decoded one thread per slice into planes cleared
 * beforehand, the medium and short tiers one warp per group, each warp
 * staging its coefficients in a shared-memory window and writing them as
 * whole lines (no plane clear).  Every other slice is decoded one thread per
 * slice into planes cleared beforehand; when no group qualifies, those
 * slices are split into the size tiers below. */
typedef struct {
    int32_t group_ctas_per_sm; /* persistent CTAs of the grouped inverse-RAHT kernel per SM: 1..4 (default 3)   */
    int32_t min_group;         /* a slot's predictive slices share one warp when at least this many: 1..32 (4) */
    int32_t rlgr_block;        /* threads per CTA of the RLGR kernels: 32, 64, 128 or 256 (default 64); the
                                  windowed form runs rlgr_block / 32 groups per CTA                               */
    int32_t rlgr_long_ctas;    /* CTAs of 128 threads that decode the longest slices (with window groups: the
                                  slices of the 4 x rlgr_long_ctas largest groups) alone on an SM each, side by
                                  side with the rest: 0..152 (default 16); -1 turns the split off                */
    int32_t rlgr_mid_pct;      /* with the split on: percent of the other slices or groups (the larger ones)
                                  decoded, and their groups inverse-transformed, on a third stream: 0..90
                                  (default 50); -1 off                                                            */
    int32_t rlgr_long_lanes;   /* slices per warp in the per-slice long launch: 8, 16 or 32 (default 32)        */
} pvvc_tune;
int pvvc_plan_create_tuned(const pvvc_batch_desc* desc, const pvvc_tune* tune, pvvc_plan** out);

/* What a plan launches: counts of its work items and of the kernels one
 * pvvc_decode of it runs (every kernel with an empty grid is skipped). */
typedef struct {
    int32_t nslices, nintra;
    int32_t groups_a, groups_b;   /* warp groups of the two inverse-RAHT phases    */
    int32_t singles_a, singles_b; /* slices inverse-transformed by a CTA of their own */
    int32_t kernels;              /* kernel launches per decode                    */
    int32_t group_ctas;           /* grid of the grouped inverse-RAHT kernel        */
    pvvc_tune tune;               /* the shapes in force (defaults resolved)         */
    uint64_t clear_bytes;         /* coefficient bytes zeroed by memset nodes per decode */
} pvvc_plan_info;
int pvvc_plan_info_get(const pvvc_plan* plan, pvvc_plan_info* info);
/* Host milliseconds of the last build of `plan` (no reference counterpart):
 * out[0] the split into intra and predictive slices, their size sorts and the
 * queue records, out[1] the RLGR order and size tiers, out[2] the
 * inverse-RAHT groups and coefficient regions, out[3] the workspace layout,
 * out[4] the upload of the queue.  Fills min(n, 5) values. */
int pvvc_plan_host_times(const pvvc_plan* plan, double* out, int32_t n);

/* Autotuner: plans `desc` under a set of candidate launch shapes (a
 * coordinate search over the six pvvc_tune fields, starting at the
 * defaults), captures one decode of the batch under each into a CUDA graph,
 * replays it `reps` times on `stream` timed with CUDA events, and returns the
 * fastest shapes and their median device time per decode.  The
 * decodes run for real: afterwards `st` holds what one pvvc_decode of the
 * batch leaves.  It allocates its own workspace and outputs, and
 * synchronises `stream`.  `payload` as for pvvc_decode. */
int pvvc_plan_autotune(const pvvc_batch_desc* desc, pvvc_state* st, const uint8_t* payload, int32_t reps, void* stream,
                       pvvc_tune* best, float* best_ms);

/* Decode one planned batch: RLGR -> dequantise -> (intra: occupancy tree
 * expansion) -> inverse RAHT -> (+ reference colours) -> YUV->RGB -> rigid
 * transform.  Replaces launch_cudaProcess / processCUDA
 * (src/cuda/render/CUDA2OpenGL.cu:37-74, include/cuda/render.cuh:42-57) and
 * the CPU path InvertRAHTOctree::SetSlice/GetPatch + the transform loop
 * (src/octree/invert_raht_octree.cc:22-120, pvvc_decompression.cc:141-150).
 *   payload      device bytes the plan's offsets index (raw, not zstd); the
 *                base must be 16-byte aligned and the buffer readable up to the
 *                16-byte boundary after its last payload byte (the colour
 *                stream is read in 16-byte blocks)
 *   xyz          device float[3*points] transformed coordinates (or NULL)
 *   rgb          device uint8[3*points] colours rounded as the CPU decoder
 *                rounds them, clamped to [0,255] (or NULL)
 *   points24     device float[6*points] in the reference GPU layout
 *                {x,y,z,r/255,g/255,b/255} (CUDA2OpenGL.cu:12-16,44-58) (or NULL)
 *   status       device int32[nslices]: per-slice PVVC_* status (or NULL)
 *   workspace    device scratch of pvvc_plan_query's size */
int pvvc_decode(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, void* stream);

/* pvvc_decode with a CUDA event recorded on `stream` before the first kernel
 * and after each of its four stages (tree expansion; RLGR; inverse RAHT of
 * the slices that need only this batch's trees, including every intra slice;
 * inverse RAHT of the predictive slices that need phase-three colours):
 * events[0..4] must be created by the caller.  No reference counterpart: the reference only
 * prints wall-clock frame times (test/test_decode_only.cc:129-150). */
int pvvc_decode_profiled(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                         float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, void* stream,
                         void* const* events);

/* One planned decode captured in a CUDA graph: the arguments of pvvc_decode
 * are bound at creation, and each pvvc_graph_launch replays the whole decode
 * (its memsets and kernels) as one graph launch on `stream`.  The plan, the
 * state and every buffer must outlive the graph; the payload buffer's
 * CONTENTS may change between launches as long as its layout is the plan's
 * (e.g. the next GoP of a stream with identical slice sizes).  Creation
 * captures on a private stream and does not touch the caller's streams. */
typedef struct pvvc_graph pvvc_graph;
int pvvc_graph_create(const pvvc_plan* plan, pvvc_state* st, const uint8_t* payload, float* xyz, uint8_t* rgb,
                      float* points24, int32_t* status, void* workspace, uint64_t workspace_bytes, pvvc_graph** out);
int pvvc_graph_launch(pvvc_graph* graph, void* stream);
int pvvc_graph_destroy(pvvc_graph* graph);

/* ---- end-to-end host call ------------------------------------------------
 * Decode whole .frame files held in HOST memory (the bytes of one or more
 * consecutive frames of one sequence, in decode order) into HOST arrays.
 * Mirrors io::LoadFrame + the H2D staging + launch_cudaProcess + the D2H
 * read-back (src/cuda/common/slice_io.cu:143-275, manager.cc:41-72,230-270):
 * payloads are copied to the device (zstd payloads compressed, then
 * inflated there by the kernel of pvvc_zstd_inflate_batch instead of the
 * loader's host zstd stage), decoded, and xyz/rgb are copied back.  A call
 * of several GoPs is decoded in parts whose plans are built concurrently on
 * host threads; each part's points are copied back as soon as it is decoded,
 * while the next part decodes.  The state keeps the parts' plans: a call
 * with the previous call's layout (slices' slots, types and sizes) reuses
 * them, their per-call fields gathered on the device.  Any stream works,
 * the default one included (the plans' copies are queued on `stream` after
 * planning, never synchronously).  Page-locked output arrays (cudaHostAlloc /
 * cudaHostRegister) let those copies run at the link's full rate.  Slot =
 * patch index.  Synchronises `stream` before returning.  status_host
 * receives one entry per slice, in file order; a zstd payload that does not
 * inflate marks its slice PVVC_ERR_ZSTD and the call returns PVVC_ERR_ZSTD. */
int pvvc_decode_frames_host(pvvc_state* st, int32_t nframes, const uint8_t* const* frame_bytes, const uint64_t* frame_len,
                            float* xyz_host, uint8_t* rgb_host, uint64_t cap_points, uint64_t* npoints_out,
                            int32_t* status_host, int32_t status_cap, void* stream);
/* Wall-clock milliseconds of the stages of the calling thread's last
 * pvvc_decode_frames_host (no counterpart in the reference):
 * out[0] parse (with the zstd frame headers), out[1] the batch description and the split into
 * runs (for a call decoded in parts, only the indices and types: each part's
 * sizes, motions and offsets are described by its planner, so they count in
 * out[2]), out[2] planning (host) and plan upload, out[3] the wait for the
 * last device-to-host copies (and, for a call decoded in one piece, its
 * decode), out[4] the wait for the payload packed into pinned memory beside
 * the planning, out[5] workspace growth, out[6] queuing the decode kernels,
 * out[7] queuing the device-to-host copies of each part, out[8..12] the
 * parts' planning stages summed (pvvc_plan_host_times), and for a call
 * decoded in parts the device timeline, in milliseconds after the call's
 * start on `stream`: out[13 + 3h] part h's payload uploaded, out[14 + 3h]
 * part h decoded, out[15 + 3h] part h's points copied back (h = 0..2).
 * Fills min(n, 22) values; zeros before any call. */
int pvvc_host_stage_times(double* out, int32_t n);

/* ---- zstd payloads on the GPU ----------------------------------------------
 * Batched ZSTD_decompress for payloads that carry a zstd type bit.  Replaces
 * the host zstd stage of the reference loader (ZstdDecoder::Decode,
 * src/common/entropy_codec.cc:341-360, called from io::LoadFrame,
 * src/cuda/common/slice_io.cu:233-265, and io::LoadSlice/LoadFrame,
 * src/io/slice_io.cc).  Job j inflates src[src_off[j], +src_len[j]) into
 * dst[dst_off[j], +dst_cap[j]) with ZSTD_decompress's contract: every zstd
 * frame of the input is decoded and appended, skippable frames are skipped,
 * and the job fails (status PVVC_ERR_ZSTD, out_len 0) on a malformed frame, a
 * frame whose decoded size differs from its declared content size, a content
 * checksum mismatch, output beyond dst_cap, a dictionary id, a legacy
 * (pre-1.0) frame, or trailing bytes.  On well-formed frames the output is
 * byte-identical to libzstd's.  On corrupt ones the decoder never accepts what
 * libzstd rejects; it is stricter in one place (a Huffman literal stream must
 * end exactly on its first bit, which libzstd's fast 4-stream path does not
 * check).  Arrays are device memory; out_len may be NULL.  One warp per job;
 * stream-ordered.  The reference sizes dst by the first frame's declared
 * content size: pvvc_zstd_content_size reads it on the host. */
int pvvc_zstd_inflate_batch(int32_t njobs, const uint8_t* src, const uint64_t* src_off, const uint32_t* src_len,
                            uint8_t* dst, const uint64_t* dst_off, const uint32_t* dst_cap, uint32_t* out_len,
                            int32_t* status, void* stream);
/* ZSTD_getFrameContentSize of the first frame of a host buffer: *size gets the
 * declared size, 0 for a skippable frame, UINT64_MAX when the frame does not
 * declare it; PVVC_ERR_ZSTD when the header is malformed or truncated. */
int pvvc_zstd_content_size(const uint8_t* src, uint64_t n, uint64_t* size);
/* The same decoder as pvvc_zstd_inflate_batch, run on host buffers by one
 * thread.  No reference counterpart; it lets a host without a GPU check the
 * decoder against libzstd. */
int pvvc_zstd_inflate_host(const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t* out_len);

/* ---- reference-signature shim --------------------------------------------
 * Same arguments as launch_cudaProcess (include/cuda/render.cuh:42-57) with
 * the decoder array replaced by a pvvc_state (slot = index[i]).  All arrays
 * are device memory as in the reference; out receives the 24-byte Points
 * layout.  Unlike the reference, it runs on `stream`, returns a status, and
 * copies the small metadata arrays to the host to plan (it synchronises). */
int pvvc_launch_cudaProcess(int grid, int block, float* out_points24, int timestamp, int* inner_offset, int* index,
                            uint8_t* type, float** mv, uint32_t* size, uint8_t* qp, uint8_t** geometry,
                            uint32_t* geometry_size, uint8_t** color, uint32_t* color_size, pvvc_state* decoders,
                            int patch_size, void* stream);

/* ---- encoder (CPU) -------------------------------------------------------
 * GoP encoding of one patch: the octree of the shared geometry
 * (RAHTOctree::MakeTree/GetOctree, src/octree/raht_octree.cc:47-187), one
 * RAHT + quantisation + RLGR payload per frame (raht_octree.cc:189-247,
 * src/patch/GoP_encoding.cc:172-205, src/common/entropy_codec.cc:65-159).
 * xyz: n x 3 points; yuv: nframes x n x 3 colours per input point, frame 0
 * absolute and frames >0 residuals; qp per frame.  Outputs are host buffers;
 * *geo_len / col_len[f] receive sizes; leaf_count receives the slice size. */
int pvvc_encode_patch_gop(const float* xyz, uint32_t n, const float* yuv, int32_t nframes, const uint8_t* qp,
                          uint8_t* geo_out, uint64_t geo_cap, uint64_t* geo_len, uint8_t* col_out, uint64_t col_cap_per_frame,
                          uint64_t* col_len, uint32_t* leaf_count);

/* Octree geometry payload of one patch and, per frame, its leaf signal: each
 * leaf's mean YUV in decode (BFS) leaf order (RAHTOctree::MakeTree/GetOctree
 * and the voxel averaging of RAHTOctree::RAHT, src/octree/raht_octree.cc:47-
 * 211).  yuv: nframes x n x 3; leaf_out: nframes x leaf_cap x 3.  The input
 * of pvvc_encode_colors. */
int pvvc_patch_leaf_yuv(const float* xyz, uint32_t n, const float* yuv, int32_t nframes, uint8_t* geo_out,
                        uint64_t geo_cap, uint64_t* geo_len, float* leaf_out, uint64_t leaf_cap, uint32_t* leaf_count);

/* ---- GPU encoder back end -------------------------------------------------
 * Colour payloads of a batch of slices on the GPU: forward RAHT
 * (RAHTOctree::RAHT, src/octree/raht_octree.cc:189-247, HaarTransform
 * octree_base.cc:164-184), quantisation (GoP_encoding.cc:184-189) and RLGR
 * (RLGREncoder, src/common/entropy_codec.cc:65-159), byte-identical to the
 * CPU encoder.  The batch is described as for pvvc_decode: slot, type (an
 * intra slice's geometry payload at geo_off in `payload`, device, 16-byte
 * aligned), size, qp; col_off/col_size are ignored.  leaf_yuv (device):
 * slice k's leaf signal (pvvc_patch_leaf_yuv; frame 0 of a GoP absolute,
 * later frames residuals) at float offset 3 * out_off[k].  out (device): slice
 * k's payload at byte offset out_byte_off[k] (host array, multiple of 4), at
 * most out_cap[k] bytes (host array, multiple of 4); out_len (device) gets
 * its length, status (device) a PVVC status per slice (PVVC_ERR_CAPACITY when
 * the payload does not fit).  Intra slices rebuild their slot's tree in `st`
 * as decoding does.  Synchronises `stream`. */
typedef struct pvvc_encoder pvvc_encoder;
int pvvc_encoder_create(pvvc_encoder** out);
int pvvc_encoder_destroy(pvvc_encoder* enc);
int pvvc_encode_colors(pvvc_encoder* enc, const pvvc_batch_desc* desc, pvvc_state* st, const uint8_t* payload,
                       const float* leaf_yuv, uint8_t* out, const uint64_t* out_byte_off, const uint32_t* out_cap,
                       uint32_t* out_len, int32_t* status, void* stream);

/* RLGR codec on host buffers (entropy_codec.cc:65-283) */
int64_t pvvc_rlgr_encode(const int64_t* sym, uint64_t n, uint8_t* out, uint64_t cap);
int pvvc_rlgr_decode_host(const uint8_t* in, uint64_t nbytes, uint64_t nsym, int64_t* out);

/* ---- batched GPU ICP (encoder) -------------------------------------------
 * Point-to-point ICP of many (source, target) patch pairs in one launch.
 * Replaces the per-pair registration::ICP::Align (src/registration/icp.cc:21-102,
 * pcl::IterativeClosestPoint) as called by PatchFitting::AddPatch
 * (src/patch/patch_fitting.cc:58-79) and PatchesRegistration::Task
 * (src/registration/patches_registration.cc:80-90).  Device arrays:
 *   src_xyz/tgt_xyz  float[3*total] points of all pairs, concatenated
 *   src_off/tgt_off  uint32[npairs+1] point ranges
 *   init             float[npairs*16] row-major initial transforms (or NULL = I)
 *   T_out            float[npairs*16] row-major final transforms
 *   mse_out          float[npairs] final mean squared NN distance (fitness)
 *   iters_out        int32[npairs], converged_out uint8[npairs] (may be NULL)
 * Semantics of the PCL criteria the reference configures (icp.cc:56-96):
 * correspondences beyond max_corr_dist are dropped; fewer than 3 stop the
 * pair unconverged; the loop ends at max_iter (converged), when the update's
 * rotation cosine >= 1 - transform_eps and its squared translation <=
 * transform_eps, or when the correspondence MSE changes by less than
 * mse_abs_eps absolute or fitness_eps relative.  mse_out is the fitness score of the
 * final transform (mean squared NN distance of all source points). */
typedef struct {
    float max_corr_dist;  /* icp.correspondence_ths */
    int32_t max_iter;     /* icp.iteration_ths */
    float fitness_eps;    /* stop when |delta MSE| < fitness_eps (icp.mse_ths) */
    float transform_eps;  /* stop when the update is below this (icp.transformation_ths) */
    float mse_abs_eps;    /* stop when |delta MSE| < this (PCL's absolute MSE threshold, 1e-12 by default) */
} pvvc_icp_params;
/* device workspace bytes of pvvc_icp_batch / pvvc_cloud_mse_batch */
int pvvc_icp_workspace_size(int32_t npairs, uint64_t total_src_points, uint64_t total_tgt_points, uint64_t* bytes);
int pvvc_icp_batch(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                   const uint32_t* tgt_off, const float* init, const pvvc_icp_params* params, float* T_out,
                   float* mse_out, int32_t* iters_out, uint8_t* converged_out, void* workspace,
                   uint64_t workspace_bytes, uint64_t total_src_points, uint64_t total_tgt_points, void* stream);
/* pvvc_icp_batch without a workspace argument and without any allocation.
 * No counterpart in the reference.  It exists for callers that cannot
 * allocate device memory at the point where they register patches: an
 * encoder embedded in a host application that has already reserved the
 * GPU's memory for its own pool, or a per-frame callback where cudaMalloc's
 * implicit device-wide synchronisation would stall work in flight.  The
 * grid scratch lives in one fixed device array of about 25 MB that every GPU
 * loading the library holds until exit.  Limits: npairs <= 512 and
 * total_tgt_points (which must equal tgt_off[npairs]) <= 1,048,576;
 * larger batches return PVVC_ERR_CAPACITY.  The kernels also check every
 * pair's tgt_off against that capacity on the device: a pair that runs past
 * it (a caller that understated total_tgt_points) gets NaN results, nothing
 * is written outside the array, and pvvc_device_error_take reports
 * PVVC_ERR_CAPACITY.  The first call in each CUDA context of a device looks
 * up the array's address (cudaGetSymbolAddress) with that device current;
 * that first call returns PVVC_ERR_ARG on a stream under capture, so make
 * it before any stream capture.  The address is cached per context: after a
 * device reset the next call looks it up again.  All calls share the array:
 * calls that overlap on the GPU (different streams, or different host
 * threads on the same device) race and must be serialised by the caller.
 * Results are those of pvvc_icp_batch. */
int pvvc_icp_batch_noalloc(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                           const uint32_t* tgt_off, const float* init, const pvvc_icp_params* params, float* T_out,
                           float* mse_out, int32_t* iters_out, uint8_t* converged_out, uint64_t total_tgt_points,
                           void* stream);
/* Symmetric NN mean squared distance of each pair after applying T
 * (ICPBase::CloudMSE, src/registration/registration_base.cc:114-158). */
int pvvc_cloud_mse_batch(int32_t npairs, const float* src_xyz, const uint32_t* src_off, const float* tgt_xyz,
                         const uint32_t* tgt_off, const float* T, float* mse_out, void* workspace,
                         uint64_t workspace_bytes, uint64_t total_src_points, uint64_t total_tgt_points, void* stream);

/* ---- fitting cloud of the GoP encoder ------------------------------------
 * Replaces PatchFitting::Compute with the direct clustering that every
 * reference config selects (src/patch/patch_fitting.cc:92-381): the
 * registered patches of a GoP (one per frame, in frame order) -> the fitting
 * cloud, the centroids of k-means runs over the clustering cells of an
 * octree descent.  The descent runs on the host; every cell's k-means on the
 * GPU (exact nearest centroids, FP32 sums in point order, the reference's
 * seeding and empty-cluster redraws).  The reference draws from the
 * process-wide rand(); here GoP g draws from its own generator -- glibc's
 * rand() algorithm seeded like srand(seeds[g]) -- so a GoP's fitting cloud
 * equals the reference's Compute after srand(seeds[g]).
 *   gop_patch   int32[ngops+1]: GoP g = patches [gop_patch[g], gop_patch[g+1])
 *   patch_off   uint32[npatches+1]: patch p = points [patch_off[p], patch_off[p+1])
 *   xyz         HOST float[3*points], the registered patches' points
 *   out_xyz     HOST float[3*out_cap]; out_off HOST uint64[ngops+1] receives
 *               each GoP's range of the fitting clouds
 *   stats       optional int32[4]: clustering cells, k-means iterations,
 *               empty-cluster redraws, device rounds
 * Parameters as in PVVCParam_t::patch (the configs: 1.0, 0.1, 100).  A cell
 * whose k would be zero (fewer points than half the patches) gives no
 * centroid, and one whose k equals its point count takes every point; the
 * reference reads past its containers in both.  Synchronises `stream`. */
typedef struct pvvc_fitter pvvc_fitter;
int pvvc_fitter_create(pvvc_fitter** out);
int pvvc_fitter_destroy(pvvc_fitter* fitter);
int pvvc_fitting_clouds(pvvc_fitter* fitter, int32_t ngops, const int32_t* gop_patch, const uint32_t* patch_off,
                        const float* xyz, const uint32_t* seeds, float clustering_ths, float clustering_err_ths,
                        int32_t max_iter, float* out_xyz, uint64_t out_cap, uint64_t* out_off, int32_t* stats,
                        void* stream);

/* ---- reconstruction quality --------------------------------------------
 * Replaces common::MSE::SetClouds + Compute + GetGeoMSEs/GetYMSEs/GetUMSEs/
 * GetVMSEs (src/registration/registration_base.cc:160-240), the measure the
 * decoder turns into PSNR (src/codec/pvvc_decompression.cc:151-171:
 * PSNR_geo = 10 log10(1024^2 / max(geo)), PSNR_Y = 10 log10(256^2 / max(Y))).
 * Two coloured clouds A (the reference's p_, e.g. the source frame) and B
 * (q_, e.g. the decoded frame), device memory: xyz float[3n], rgb uint8[3n].
 * For every point of A its exact nearest neighbour in B (FP32 squared
 * distance, x, y, z accumulated in order; the lower index of B among equal
 * distances), and the squared differences of their BT.601 Y, U, V
 * (ColorYUV(const PointXYZRGB&), include/common/common.h:94-98); then the
 * same for B against A.  mse_out: device double[8] = {geo A->B, geo B->A,
 * Y A->B, Y B->A, U A->B, U B->A, V A->B, V B->A}, each the mean over the
 * query cloud (summed in double; the reference sums in float).  An empty
 * cloud gives -1 on its side and 0 on the other, as the reference returns
 * early.  Stream-ordered; workspace of pvvc_cloud_quality_workspace_size
 * bytes, 256-byte aligned. */
int pvvc_cloud_quality_workspace_size(uint64_t npoints_a, uint64_t npoints_b, uint64_t* bytes);
int pvvc_cloud_quality(uint64_t npoints_a, const float* xyz_a, const uint8_t* rgb_a, uint64_t npoints_b,
                       const float* xyz_b, const uint8_t* rgb_b, double* mse_out, void* workspace,
                       uint64_t workspace_bytes, void* stream);

/* ---- colour interpolation of the GoP encoder -------------------------------
 * Replaces GoPEncoding::Interpolation and the k-NN loop of GoPEncoding::Encode
 * (src/patch/GoP_encoding.cc:73-95,131-150) for many (query cloud, source
 * patch) pairs: the query cloud is a GoP's fitting cloud, the source one
 * frame's patch with its RGB colours.  Per query point: the k nearest source
 * points by FP32 squared distance (x, y, z accumulated in order, as PCL's
 * exact k-d tree), the lower source index first among equal distances, and
 * fewer when the patch is smaller; weights 1/max(d, 1e-6) normalised by
 * their sum; the weighted RGB converted to YUV by BT.601 (common.h:83-92),
 * every operation rounded in the reference's order.  base_pair (optional):
 * pair p with base_pair[p] >= 0 then becomes the residual against that pair
 * (GoP_encoding.cc:144-148; the base needs no base of its own and the same
 * query count).  All arrays are device memory:
 *   query_xyz + 3*query_off[p], query_n[p] points   (pairs may share a cloud)
 *   src_xyz, src_rgb: source p = points [src_off[p], src_off[p+1])
 *   yuv_out + 3*out_off[p]: query_n[p] YUV triples
 *   status (optional): per pair 0, or PVVC_ERR_ARG for an empty patch (its
 *   output zeroed) or a bad base.
 * k: 1..16 (the reference's patch.interpolation_num defaults to 10).
 * Stream-ordered; workspace of pvvc_knn_colors_workspace_size bytes. */
int pvvc_knn_colors_workspace_size(int32_t npairs, uint64_t total_src_points, uint64_t* bytes);
int pvvc_knn_colors_batch(int32_t npairs, const float* query_xyz, const uint64_t* query_off, const uint32_t* query_n,
                          const float* src_xyz, const uint8_t* src_rgb, const uint32_t* src_off, int32_t k,
                          const int32_t* base_pair, float* yuv_out, const uint64_t* out_off, int32_t* status,
                          void* workspace, uint64_t workspace_bytes, uint64_t total_src_points, void* stream);

/* ---- BF16 tensor-core GEMM ------------------------------------------------
 * The building block of the registration network's training and inference
 * kernels (no reference counterpart: the reference registers with PCL ICP
 * from the identity).  C[M,N] = epilogue(A[M,K] . B[N,K]^T): A and B bf16
 * row-major with K contiguous (lda, ldb in elements, multiples of 8; K a
 * multiple of 64; N a multiple of 64; pointers 16-byte aligned), FP32
 * accumulation in tensor memory (tcgen05.mma).  Epilogues:
 *   PVVC_GEMM_BIAS_RELU_BF16  C bf16 = max(acc + bias, 0)   (bias may be NULL)
 *   PVVC_GEMM_F32             C f32  = acc + bias            (bias may be NULL)
 *   PVVC_GEMM_F32_ACCUM       C f32 += acc, K split `splits` ways (partials
 *                             added atomically; the only epilogue with splits > 1)
 *   PVVC_GEMM_MASK_BF16       C bf16 = acc where aux[M,N] (bf16) > 0, else 0
 * Stream-ordered.  A kernel whose bounded internal wait gave up sets a device
 * error code that pvvc_device_error_take returns (and clears); 0 = none.
 * The same call also returns (and clears) PVVC_ERR_CAPACITY when an ICP
 * kernel found a pair beyond its fixed scratch (pvvc_icp_batch_noalloc). */
#define PVVC_GEMM_BIAS_RELU_BF16 0
#define PVVC_GEMM_F32 1
#define PVVC_GEMM_F32_ACCUM 2
#define PVVC_GEMM_MASK_BF16 3
int pvvc_gemm_bf16(int32_t M, int32_t N, int32_t K, const void* A, int64_t lda, const void* B, int64_t ldb, void* C,
                   int64_t ldc, const float* bias, const void* aux, int64_t ldaux, int32_t epilogue, int32_t splits,
                   void* stream);
int pvvc_device_error_take(int32_t* code);

/* ---- learned ICP initialisation -------------------------------------------
 * A PointNet-style network proposes each pair's initial transform for
 * pvvc_icp_batch (`init`).  No reference counterpart: the reference starts
 * every registration from the identity (src/registration/icp.cc:21-102).
 * Inputs: 256 points sampled (with replacement, seeded) from each cloud,
 * centred on their sample mean and scaled by the source sample's RMS radius;
 * shared MLP 3-64-128-256 per point, max-pool per cloud, MLP 512-256-128-6 ->
 * (omega, delta): R = exp(omega), t = c_t - R c_s + s * delta.  BF16 weights
 * and activations, FP32 accumulation (tcgen05).  Training targets come from
 * converged ICP: omega* = log R*, delta* from t*.  Parameters are one fp32
 * vector of pvvc_regnet_param_count() floats (get/set for checkpoints). */
typedef struct pvvc_regnet pvvc_regnet;
typedef struct {
    float lr, beta1, beta2, eps, weight_decay; /* AdamW (decoupled decay on weight matrices) */
    float lambda_w;                            /* loss weight of the rotation part           */
} pvvc_adamw;
int pvvc_regnet_param_count(void);
int pvvc_regnet_create(uint64_t seed, pvvc_regnet** out);
int pvvc_regnet_destroy(pvvc_regnet* net);
int pvvc_regnet_get_params(pvvc_regnet* net, float* host, int64_t count);
/* also resets the AdamW moments and step */
int pvvc_regnet_set_params(pvvc_regnet* net, const float* host, int64_t count);
/* One training step on the pairs pair_ids[0..npairs) of a device dataset
 * (clouds as for pvvc_icp_batch; T_label [*,16] row-major converged ICP
 * transforms, omega_label [*,3] their axis-angle): sample, forward, loss,
 * backward, AdamW.  loss_out: device float (or NULL).  Stream-ordered. */
int pvvc_regnet_train_step(pvvc_regnet* net, int32_t npairs, const int32_t* pair_ids, const float* src,
                           const uint32_t* src_off, const float* tgt, const uint32_t* tgt_off, const float* T_label,
                           const float* omega_label, uint64_t seed, const pvvc_adamw* opt, float* loss_out, void* stream);
/* Gradient of the loss for given normalised inputs x0 [npairs*2*256*3] (pair
 * b's source rows then target rows) and targets y [npairs*6]: grad_out
 * [param_count] (device), loss_out (device float).  No update. */
int pvvc_regnet_grad(pvvc_regnet* net, int32_t npairs, const float* x0, const float* y, float lambda_w, float* grad_out,
                     float* loss_out, void* stream);
/* Proposed transforms T_out [npairs*16] (row-major) for every pair. */
int pvvc_propose(pvvc_regnet* net, int32_t npairs, const float* src, const uint32_t* src_off, const float* tgt,
                 const uint32_t* tgt_off, uint64_t seed, float* T_out, void* stream);
/* The last forward's raw outputs (omega, delta) [npairs*6] (device). */
int pvvc_regnet_outputs(pvvc_regnet* net, int32_t npairs, float* out6, void* stream);

/* ---- playback server -----------------------------------------------------
 * Decodes .frame requests of many concurrent playback streams with
 * continuous batching.  It replaces the reference client's single decode
 * thread (src/cuda/common/manager.cc:230-270: one stream, one frame per
 * launch_cudaProcess, synchronised after each).  A worker thread takes every
 * request that has arrived, across streams, packs it into one batch (frames
 * of one stream in submission order; a stream's next intra frame waits for
 * the next batch), uploads it on a copy stream while the previous batch
 * decodes, and enqueues one planned decode per batch on a compute stream;
 * a completion thread stamps each frame when its batch's event fires.
 * Per-patch state (trees, reference colours) and decoded frames stay in HBM.
 *
 * Memory: at creation the server reserves, within hbm_budget_bytes, the
 * output ring, `inflight` batch workspaces, and a pool of patch-state slots
 * with the rest.  A stream is admitted (pvvc_server_open_stream) only when a
 * contiguous range of `nslots` free slots exists: PVVC_ERR_CAPACITY
 * otherwise, and closing a stream frees its range.  Timestamps are
 * microseconds on the server's steady clock. */
typedef struct {
    uint64_t hbm_budget_bytes;   /* device memory the server may reserve in total                 */
    int32_t max_leaves;          /* points per patch slot (default 8192)                          */
    int32_t max_nodes;           /* internal octree nodes per slot (default 2 * max_leaves)         */
    uint64_t max_batch_points;   /* points of one batch (default 32M)                             */
    uint64_t ring_points;        /* decoded points held until released (default 256M)             */
    int32_t inflight;            /* batches queued on the GPU at once: 1..4 (default 2)           */
    int32_t max_batch_frames;    /* frames of one batch (default 4096)                            */
    pvvc_tune tune;              /* launch shapes of every batch                                  */
} pvvc_server_config;

typedef struct {
    uint64_t tag;          /* the caller's tag of the request                          */
    uint64_t handle;       /* pass to pvvc_server_release / pvvc_server_read           */
    int32_t stream_id;
    int32_t status;        /* PVVC_OK or the status of the frame's first failed slice  */
    uint64_t npoints;
    const float* xyz;      /* device float[3*npoints]: valid until released           */
    const uint8_t* rgb;    /* device uint8[3*npoints]                                   */
    double submit_us;      /* request accepted                                          */
    double launch_us;      /* its batch enqueued on the GPU                             */
    double done_us;        /* its batch finished on the GPU                             */
    int32_t batch_id;
    int32_t batch_frames;  /* frames in that batch                                      */
} pvvc_completion;

typedef struct {
    uint64_t batches, frames, points, slices;
    uint64_t slots_total, slots_free, streams_open;
    uint64_t reserved_bytes;    /* device memory the server holds                       */
    double gpu_busy_us;         /* sum of batch device times (CUDA events)              */
} pvvc_server_stats;

typedef struct pvvc_server pvvc_server;
int pvvc_server_create(const pvvc_server_config* cfg, pvvc_server** out);
/* Waits for the batches already on the GPU, drops frames still queued, frees everything. */
int pvvc_server_destroy(pvvc_server* s);
int pvvc_server_open_stream(pvvc_server* s, int32_t nslots, int32_t* stream_id);
/* Frees the stream's slots once its submitted frames have completed. */
int pvvc_server_close_stream(pvvc_server* s, int32_t stream_id);
/* Queue one .frame of a stream (host bytes that the caller keeps unchanged
 * until the frame's completion is polled).  The frame header is parsed here;
 * a malformed frame or a patch index >= the stream's nslots is refused with
 * PVVC_ERR_FORMAT / PVVC_ERR_ARG and not queued. */
int pvvc_server_submit(pvvc_server* s, int32_t stream_id, const uint8_t* frame_bytes, uint64_t len, uint64_t tag);
/* Up to `cap` completions in completion order, waiting up to wait_us for the first. */
int pvvc_server_poll(pvvc_server* s, pvvc_completion* out, int32_t cap, int32_t* n, int32_t wait_us);
/* Copy a completed frame to host memory (synchronous). */
int pvvc_server_read(pvvc_server* s, uint64_t handle, float* xyz_host, uint8_t* rgb_host);
/* Return a completed frame's output space to the ring. */
int pvvc_server_release(pvvc_server* s, uint64_t handle);
int pvvc_server_stats_get(pvvc_server* s, pvvc_server_stats* out);

#ifdef __cplusplus
}
#endif
#endif
