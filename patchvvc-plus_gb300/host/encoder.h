// encoder.h -- CPU GoP encoder back end: octree geometry, forward RAHT,
// quantisation and RLGR coding.  Produces bitstreams byte-identical to the
// reference encoder (src/patch/GoP_encoding.cc:97-211 with
// src/octree/raht_octree.cc and src/common/entropy_codec.cc).
#pragma once

#include <cstdint>
#include <vector>

namespace pvvc {

// Adaptive run-length / Golomb-Rice coder (H. S. Malvar, DCC 2006) with the
// reference's constants L=4, U0=3, D0=1, U1=2, D1=1 and its byte padding.
std::vector<uint8_t> rlgr_encode(const int64_t* sym, size_t n);
// Host decoder, table-free 64-bit window (same semantics as the reference's
// RLGRDecoder::Decode).  Returns 0 or PVVC_ERR_OVERRUN.
int rlgr_decode(const uint8_t* in, size_t nbytes, size_t nsym, int64_t* out);

// Octree of one patch's (shared, GoP-wide) geometry.
class PatchTree {
  public:
    // RAHTOctree::MakeTree semantics (raht_octree.cc:62-113) with octree
    // resolution `resolution`.  Returns 0 or a PVVC status.
    int build(const float* xyz, size_t n, float resolution = 1.0f);
    size_t leaf_count() const { return leaf_count_; }
    int height() const { return height_; }
    // 25-byte core + BFS occupancy bytes (raht_octree.cc:47-56)
    std::vector<uint8_t> geometry() const;
    // Forward RAHT of per-input-point YUV (n x 3): leaf_count x 3
    // coefficients in stream (reversed) order (raht_octree.cc:189-247).
    void raht(const float* yuv, std::vector<float>* coef) const;
    // Leaf signal of per-input-point YUV (n x 3): each leaf's mean colour in
    // decode (BFS) leaf order, leaf_count x 3 (raht_octree.cc:204-211)
    void leaf_yuv(const float* yuv, float* out) const;
    // leaf (decode-order) index of each input point
    const std::vector<uint32_t>& point_leaf() const { return point_leaf_; }

  private:
    int height_ = 0;
    float center_[3] = {0, 0, 0}, range_ = 0;
    size_t npts_ = 0, leaf_count_ = 0;
    std::vector<uint32_t> order_;          // input points sorted by leaf (stable)
    std::vector<uint32_t> leaf_first_;     // leaf -> first entry in order_ (+ sentinel)
    std::vector<uint32_t> point_leaf_;
    // per internal level: occupancy byte and index of the first child
    std::vector<std::vector<uint8_t>> occ_;
    std::vector<std::vector<uint32_t>> first_child_;
};

// Quantise (GoP_encoding.cc:184-189) and RLGR-encode coefficients
// (leaf_count x 3, stream order) as Y || U || V.
std::vector<uint8_t> encode_colors(const float* coef, size_t nleaf, uint8_t qp);

}  // namespace pvvc
