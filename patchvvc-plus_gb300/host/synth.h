// synth.h -- seeded synthetic volumetric-video sequences and their patchVVC
// bitstreams.  They stand in for the 8i voxelised full-body sequences the
// reference configs point at: a union of ellipsoid / capsule surfaces
// voxelised on a 2^grid_bits grid, smooth value-noise colour plus N(0,4)
// noise, per-primitive rigid motion, patches of a prescribed size
// distribution, GoP structure of one intra frame plus rigid-motion predicted
// frames.  Not part of the drop-in boundary (the reference has no
// counterpart); exported for the tests and the benchmark.
#pragma once

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct {
    int32_t grid_bits;       /* 9 -> 512^3, 10 -> 1024^3                       */
    int32_t nprims;          /* ellipsoids / capsules                           */
    float axis_min, axis_max;/* full axis lengths (voxels) before rescaling     */
    int32_t target_points;   /* primitives are rescaled to about this many pts  */
    int32_t nframes, gof;    /* sequence length and GoP length                  */
    int32_t size_mode;       /* 0: uniform[size_a,size_b]; 1: lognormal(median
                                size_a, sigma size_b) clipped to [size_min,size_max] */
    float size_a, size_b, size_min, size_max;
    uint8_t qp_i, qp_p;      /* quantisation steps of intra / predictive slices */
    float rot_deg, trans_vox;/* per-frame motion bounds                         */
    float jitter;            /* surface jitter (voxels) at re-voxelisation      */
    float color_noise;       /* per-frame colour noise sigma                    */
    uint64_t seed;
    int32_t nthreads;
    int32_t zstd_level;      /* 0: raw payloads; else each payload is zstd-compressed
                                at this level and kept when smaller, with the slice
                                type's zstd bit set (GoP_encoding.cc:158-200)     */
} pvvc_synth_config;

typedef struct pvvc_synth pvvc_synth;

/* Generates the sequence (geometry, patches, colours, motion). */
int pvvc_synth_create(const pvvc_synth_config* cfg, pvvc_synth** out);
void pvvc_synth_destroy(pvvc_synth* s);
int32_t pvvc_synth_gof_count(const pvvc_synth* s);
int32_t pvvc_synth_patch_count(const pvvc_synth* s, int32_t gof);
/* Points of one patch (its shared GoP geometry), the per-frame colours the
 * encoder sees (frame 0 absolute YUV, later frames residual YUV, per input
 * point) and the per-frame row-major mv.  Pass NULL buffers to query n and
 * the frame count. */
int pvvc_synth_patch(const pvvc_synth* s, int32_t gof, int32_t patch, float* xyz, float* yuv, float* mv_rowmajor,
                     uint32_t* n, int32_t* nframes);
/* Encodes every GoP (CPU, nthreads) into .frame byte blobs. */
int pvvc_synth_encode(pvvc_synth* s);
/* Bytes of encoded frame `frame` (valid until destroy). */
int pvvc_synth_frame(const pvvc_synth* s, int32_t frame, const uint8_t** bytes, uint64_t* len);
/* Total decoded points of a frame. */
uint64_t pvvc_synth_frame_points(const pvvc_synth* s, int32_t frame);

#ifdef __cplusplus
}
#endif
