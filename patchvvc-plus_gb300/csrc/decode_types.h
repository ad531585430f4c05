// decode_types.h -- device-side layouts shared by the decode kernels and
// their host launchers.
#pragma once

#include <cstdint>

namespace pvvc {

constexpr int kMaxLevels = 32;  // octree height limit (the header stores a u8)

// One slice in the work queue (queue order = intra first, then by size).
// RLGR launches split by slice length: a CTA of the long-slice launch (128
// threads, one warp per scheduler) reserves this much dynamic shared memory,
// which no RLGR code uses, so that no other CTA fits on its SM -- neither one
// of the other RLGR launch (kRlgrShortSmem each) nor one of the grouped
// inverse RAHT (~20 KB) that runs beside it.  The serial bit chains of the
// longest slices then run without sharing issue slots, while the rest of the
// decode fills the remaining SMs.
constexpr int kRlgrLongSmem = 212 * 1024;
constexpr int kRlgrShortSmem = 32 * 1024;
constexpr int kRlgrLongBlock = 128;
// Window groups (decoded by the windowed RLGR, one warp per group, unless
// they are in the long tier): at least this many slices, all of one size;
// the long tier takes kWinGroupsPerLongCta of them per long CTA.
constexpr int kWinGroupMin = 16;
constexpr int kWinGroupsPerLongCta = 4;

struct SliceWork {
    uint64_t col_off;   // colour payload byte offset
    uint64_t geo_off;   // geometry payload byte offset (intra)
    uint64_t out_off;   // first output point
    uint64_t coef_off;  // float offset of the slice's 3 coefficient planes in workspace
    uint64_t fb_off;    // float offset of the level-buffer fallback region (~0: none)
    uint32_t csz, gsz;
    uint32_t n;         // slice size (points)
    int32_t slot;       // state slot
    int32_t orig;       // index in the caller's arrays (status)
    uint8_t type, qp, pad0, pad1;
    // coefficient (plane p, index i) lives at coef_off + (p*n + i)*coef_stride + coef_lane:
    // slices decoded by one warp share a frame-interleaved region (stride 32,
    // lane = position in the group), the others own contiguous planes
    uint32_t coef_stride, coef_lane;
    float mv[12];       // first three rows of the row-major 4x4
};

// The per-call fields of the records, in the caller's slice order (device
// copies of a host call's description arrays): a plan reused for the same
// layout takes them from here on the device (k_refresh).
struct CallFields {
    const uint64_t* col_off;
    const uint64_t* geo_off;
    const uint64_t* out_off;
    const uint32_t* csz;
    const uint32_t* gsz;
    const uint8_t* qp;
    const float* mv;  // 16 per slice (row-major 4x4)
};

// Per-slot header of a decoded tree (device).
struct SlotInfo {
    int32_t valid;          // an intra slice populated the slot
    int32_t height;         // octree height H (levels 0..H-1, leaves at H-1)
    int32_t nodes;          // internal nodes (levels 0..H-2)
    int32_t leaves;         // leaf count (= slice size)
    int32_t max_width;      // widest internal level
    int32_t level_start[kMaxLevels + 1];  // first internal node of each level
};

// Device pointers of a state pool (slot-major arrays).
struct StateView {
    SlotInfo* info;          // [nslots]
    uint8_t* occ;            // [nslots * max_nodes] occupancy byte
    uint8_t* mask;           // [nslots * max_nodes] coded-coefficient bits (1..7)
    uint32_t* cbase;         // [nslots * max_nodes] first child (index within next level)
    uint32_t* coff;          // [nslots * max_nodes] first coefficient index
    float2* ab;              // [nslots * max_nodes * 7] butterfly (a,b) per i = 1..7
    uint32_t* wsum;          // [nslots * max_nodes] subtree leaf count (build scratch)
    float* ctr;              // [nslots * max_nodes * 3] node centres (build scratch)
    float* xyz;              // [nslots * max_leaves * 3] leaf centres
    float* ref;              // [nslots * max_leaves * 3] reference YUV (intra result)
    int32_t nslots, max_leaves, max_nodes;
};

// A group of slices of one slot inverse-transformed by one warp (one lane
// per slice).  When the group holds the slot's intra slice it is lane 0.
struct GroupDesc {
    int32_t slot;
    int32_t first;  // into the group item list
    int32_t count;  // <= 32
    int16_t intra;
    // the inverse transform of a group may be split over `parts` CTAs (0
    // means 1), each repeating the levels above the last two and taking
    // part `part` of the last-level nodes
    uint8_t part, parts;
};
static_assert(sizeof(GroupDesc) == 16, "GroupDesc: four words");

}  // namespace pvvc
