// bitstream.h -- patchVVC slice / frame containers and their byte layouts.
//
// Byte-compatible with the reference's writers and readers:
//   .slice  src/io/slice_io.cc:20-206  (u8 type, i32 ts, i32 index, u64 size,
//           u8 qp, f32[16] mv column-major, [intra: u64 gsz, bytes],
//           [!skip: u64 csz, bytes])
//   .frame  src/io/slice_io.cc:258-316 and src/cuda/common/slice_io.cu:143-275
//           (i32 ts, u32 n, i32 index[n], u8 type[n], u32 size[n], u8 qp[n],
//            f32 mv[n][16] row-major, u32 gsz[n], geometry bytes,
//            u32 csz[n], colour bytes)
// Slice type bits: include/common/common.h:31-56.
#pragma once

#include <cstdint>
#include <string>
#include <vector>

namespace pvvc {

enum : uint8_t {
    kTypeValid = 0x01,
    kTypePredict = 0x02,
    kTypeSkip = 0x04,
    kTypeGeoZstd = 0x08,
    kTypeColorZstd = 0x10,
    kTypeDefaultIntra = 0x01,
    kTypeDefaultPredict = 0x03,
};

struct Slice {
    uint8_t type = 0;
    int32_t timestamp = -1;
    int32_t index = -1;
    uint64_t size = 0;
    uint8_t qp = 1;
    float mv[16] = {1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1};  // column-major (Eigen)
    std::vector<uint8_t> geometry;
    std::vector<uint8_t> color;
};

// One timestamp's slices in structure-of-arrays form (common::Frame,
// include/common/common.h:362-413).  mv is row-major, 16 floats per slice.
struct Frame {
    int32_t timestamp = -1;
    std::vector<int32_t> index;
    std::vector<uint8_t> type;
    std::vector<uint32_t> size;
    std::vector<uint8_t> qp;
    std::vector<float> mv;
    std::vector<std::vector<uint8_t>> geometry;
    std::vector<std::vector<uint8_t>> color;
    size_t count() const { return index.size(); }
};

// A parsed .frame whose slice payloads point into the parsed bytes (no
// copies).  Valid while those bytes live.
struct FrameView {
    int32_t timestamp = -1;
    std::vector<int32_t> index;
    std::vector<uint8_t> type;
    std::vector<uint32_t> size;
    std::vector<uint8_t> qp;
    std::vector<float> mv;
    std::vector<const uint8_t*> geo, col;
    std::vector<uint32_t> gsz, csz;
    size_t count() const { return index.size(); }
};

// Serialise / parse.  Parsers return 0 or a PVVC_ERR_* status and never read
// past `len`.
std::vector<uint8_t> write_slice(const Slice& s);
int parse_slice(const uint8_t* p, size_t len, Slice* out);
std::vector<uint8_t> write_frame(const Frame& f);
int parse_frame(const uint8_t* p, size_t len, Frame* out);
// parse_frame's checks, the payloads left in place
int parse_frame_view(const uint8_t* p, size_t len, FrameView* out);

// Frame from slices sorted by patch index (ChangeSliceToFrame, slice_io.cc:208-322).
Frame frame_from_slices(std::vector<Slice> slices);

// zstd compression on the host (ZstdEncoder::Encode), for the synthetic
// generator's zstd stage.  libzstd is loaded at run time; zstd_available()
// is false when it is not present.  Payloads are inflated on the GPU
// (zstd_core.h), never here.
bool zstd_available();
int zstd_compress(const uint8_t* src, size_t n, int level, std::vector<uint8_t>* out);


}  // namespace pvvc
