// zstd_core.h -- zstd frame decoder (RFC 8878) shared by the GPU kernel (one
// warp per payload) and its host build.
//
// The reference inflates every payload whose slice type carries a zstd bit
// with libzstd on the host: ZstdDecoder::Decode (src/common/entropy_codec.cc:
// 341-360) sizes the output by ZSTD_getFrameContentSize of the first frame and
// calls ZSTD_decompress (io::LoadFrame, src/cuda/common/slice_io.cu:233-265;
// src/io/slice_io.cc).  decompress() below has ZSTD_decompress's contract:
// every frame of the input is decoded into dst (skippable frames are
// skipped), and the call fails where libzstd 1.5 fails on the same bytes:
// reserved bits set, a dictionary id, a frame whose decoded size differs from
// its declared content size, a bad content checksum, output beyond `cap`,
// trailing bytes, and the entropy-stream checks listed at each function.
// Legacy (pre-1.0) frames are not decoded.
//
// The decoder is written once for both targets.  All lanes of a warp run the
// same control flow and parse the same header bytes (uniform loads); lane 0
// alone builds tables and decodes the sequence stream, lanes 0-3 decode the
// four Huffman literal streams, and every lane copies bytes.  Values that
// lane 0 computes reach the other lanes through `Shared` after a warp sync.
// On the host there is one lane and the syncs are no-ops.
#pragma once
#include <stdint.h>

#if defined(__CUDACC__)
#define ZFN __host__ __device__ __forceinline__
#else
#define ZFN inline
#endif

namespace pvvc_zstd {

#if defined(__CUDA_ARCH__)
ZFN void wsync() { __syncwarp(); }
ZFN bool any_lane(bool v) { return __any_sync(0xffffffffu, v); }
ZFN uint32_t from_lane0(uint32_t v) { return __shfl_sync(0xffffffffu, v, 0); }
ZFN int highbit(uint32_t v) { return 31 - __clz((int)v); }  // v > 0
ZFN uint32_t same_value_lanes(uint32_t v) { return __match_any_sync(0xffffffffu, v); }
ZFN int popc(uint32_t v) { return __popc(v); }
#else
ZFN void wsync() {}
ZFN bool any_lane(bool v) { return v; }
ZFN uint32_t from_lane0(uint32_t v) { return v; }
ZFN int highbit(uint32_t v) { return 31 - __builtin_clz(v); }
ZFN uint32_t same_value_lanes(uint32_t) { return 1u; }
ZFN int popc(uint32_t v) { return __builtin_popcount(v); }
#endif

constexpr int kHufLogMax = 12;  // HUF_TABLELOG_MAX: the largest code the decoder accepts
constexpr int kLLLog = 9, kMLLog = 9, kOFLog = 8;
constexpr int kMaxLL = 35, kMaxML = 52, kMaxOF = 31;
constexpr uint32_t kBlockMax = 128u * 1024u;
constexpr int kSeqBatch = 32;  // sequences decoded by lane 0 ahead of the warp's copies

struct Cell {  // one FSE decoding-table entry
    uint16_t base;  // next-state baseline
    uint8_t sym;
    uint8_t nb;  // state bits to read
};

// Everything a decoder keeps between lanes and between blocks of a frame.
struct Shared {
    uint16_t huf[1 << kHufLogMax];  // Huffman table: (symbol << 4) | code length
    Cell ll[1 << kLLLog], ml[1 << kMLLog], of[1 << kOFLog];
    Cell wt[64];                    // Huffman weight table (accuracy log <= 6)
    int16_t norm[256];              // normalised counts of the table being built
    uint8_t w[256];                 // Huffman weights
    uint16_t cnt[256];              // scratch of the FSE table builder
    uint32_t seq_ll[kSeqBatch], seq_ml[kSeqBatch], seq_off[kSeqBatch];
    int32_t wcount[16];             // Huffman fill: symbols per weight, then the next rank per weight
    int32_t wpos[16];               //   first table entry of each weight
    int32_t hlog;                   // Huffman table log (0: none yet in this frame)
    int32_t llog, mlog, olog;       // accuracy logs of the sequence tables (-1: undefined)
    int32_t val[8];                 // lane-0 results for the warp
};

// ---- byte helpers ----------------------------------------------------------
ZFN uint32_t le16(const uint8_t* p) { return (uint32_t)p[0] | ((uint32_t)p[1] << 8); }
ZFN uint32_t le24(const uint8_t* p) { return le16(p) | ((uint32_t)p[2] << 16); }
ZFN uint32_t le32(const uint8_t* p) { return le24(p) | ((uint32_t)p[3] << 24); }
ZFN uint64_t le64(const uint8_t* p) { return (uint64_t)le32(p) | ((uint64_t)le32(p + 4) << 32); }

// ---- backward bit stream (FSE and Huffman streams) -------------------------
// Bit i of the stream is bit (i & 7) of byte i >> 3.  The last byte's highest
// set bit marks the end; reading starts just below it and goes down.  A read
// of n bits returns the next n bits, the highest stream bit as the MSB.  Bits
// below the first byte read as zero; `pos` (the stream bits not yet consumed)
// going negative is libzstd's overflow state.  The next bits sit
// left-aligned in a 64-bit container: a read is one shift out of its top,
// and 32 more bits are taken from the stream whenever fewer than a read
// needs remain.
struct BackBits {
    const uint8_t* p;
    int32_t n;
    int32_t pos;    // stream bits [0, pos) not yet consumed
    int32_t valid;  // container bits (from the top) that hold stream bits pos-1, pos-2, ...
    uint64_t c;

    // stream bits [b0, b0 + 32), bit b0 + 31 as the MSB; bits outside the stream are zero
    ZFN uint32_t bits32(int32_t b0) const {
        const int32_t k0 = b0 >> 3;  // floor
        uint64_t v = 0;
        if (k0 >= 0 && k0 + 5 <= n) {
            v = (uint64_t)le32(p + k0) | ((uint64_t)p[k0 + 4] << 32);
        } else {
            for (int i = 4; i >= 0; --i) {
                const int32_t k = k0 + i;
                v = (v << 8) | ((k >= 0 && k < n) ? p[k] : 0u);
            }
        }
        return (uint32_t)(v >> (b0 & 7));
    }
    ZFN void fill() {  // valid < 32 on entry
        const int32_t lo = pos - valid;  // the highest stream bit not in the container is lo - 1
        if (lo <= 0) {                   // only zeros below: the container's low bits are zero already
            valid = 64;
            return;
        }
        c |= (uint64_t)bits32(lo - 32) << (32 - valid);
        valid += 32;
    }
    // false: empty stream or a zero last byte (BIT_initDStream's errors)
    ZFN bool init(const uint8_t* s, int64_t len) {
        p = s;
        n = (int32_t)len;
        if (len <= 0 || s[len - 1] == 0) return false;
        pos = 8 * (int32_t)(len - 1) + highbit(s[len - 1]);
        c = 0;
        valid = 0;
        fill();
        fill();
        return true;
    }
    ZFN uint32_t peek(int nb) {  // nb <= 32
        if (valid < nb) fill();
        return nb ? (uint32_t)(c >> (64 - nb)) : 0u;
    }
    ZFN void skip(int nb) {  // after a peek of at least nb bits
        c <<= nb;
        pos -= nb;
        valid -= nb;
    }
    ZFN uint32_t read(int nb) {
        const uint32_t v = peek(nb);
        skip(nb);
        return v;
    }
};

// ---- FSE ----------------------------------------------------------------
// Forward bits of a table description: bit i is bit (i & 7) of byte i >> 3,
// bytes at or past n read as zero.  nb <= 24.
ZFN uint32_t fwd_bits(const uint8_t* p, int64_t n, int64_t bit, int nb) {
    const int64_t b = bit >> 3;
    uint32_t v = 0;
    for (int i = 0; i < 4; ++i)
        if (b + i < n) v |= (uint32_t)p[b + i] << (8 * i);
    return (v >> (bit & 7)) & ((1u << nb) - 1u);
}

// FSE table description (RFC 8878 4.1.1; libzstd FSE_readNCount).  Fills
// norm[0..*nsym) and *log; returns the bytes used, or -1 when the description
// is corrupt: accuracy log above maxlog, more than maxsym + 1 symbols, counts
// that do not sum to 1 << log, or more bytes than n.
ZFN int read_ncount(const uint8_t* p, int64_t n, int16_t* norm, int* nsym, int* log, int maxlog, int maxsym) {
    if (n < 1) return -1;
    const int al = (int)fwd_bits(p, n, 0, 4) + 5;
    if (al > maxlog) return -1;
    int64_t bit = 4;
    int remaining = (1 << al) + 1, threshold = 1 << al, nb = al + 1;
    int s = 0;
    bool prev0 = false;
    while (remaining > 1) {
        if (prev0) {  // 2-bit repeat flags: 3 means three more zeros and another flag
            int z = s;
            for (;;) {
                const uint32_t f = fwd_bits(p, n, bit, 2);
                bit += 2;
                z += (int)f;
                if (f != 3) break;
                if (z > maxsym + 1) return -1;
            }
            if (z >= maxsym + 1) return -1;
            while (s < z) norm[s++] = 0;
        }
        const int mx = (2 * threshold - 1) - remaining;
        const uint32_t v = fwd_bits(p, n, bit, nb);
        int count;
        if ((int)(v & (uint32_t)(threshold - 1)) < mx) {
            count = (int)(v & (uint32_t)(threshold - 1));
            bit += nb - 1;
        } else {
            count = (int)(v & (uint32_t)(2 * threshold - 1));
            if (count >= threshold) count -= mx;
            bit += nb;
        }
        --count;  // -1: a "less than one" probability, worth one cell
        remaining -= count < 0 ? -count : count;
        norm[s++] = (int16_t)count;
        prev0 = count == 0;
        if (remaining < 1) return -1;
        while (remaining < threshold) {
            --nb;
            threshold >>= 1;
        }
        if (remaining > 1 && s >= maxsym + 1) return -1;
    }
    const int64_t bytes = (bit + 7) >> 3;
    if (bytes > n) return -1;
    *nsym = s;
    *log = al;
    return (int)bytes;
}

// Decoding table from normalised counts (RFC 8878 4.1.1 "FSE table from
// distribution"; libzstd ZSTD_buildFSETable / FSE_buildDTable): "less than
// one" symbols take the top cells, the others are spread with step
// (size >> 1) + (size >> 3) + 3 over the remaining cells, then each cell gets
// its state bits and baseline from its symbol's running count.  Lane 0 only.
// `cnt` is scratch of nsym entries.  false: the spread does not close.
ZFN bool build_fse(Cell* t, const int16_t* norm, int nsym, int log, uint16_t* cnt) {
    const int size = 1 << log;
    int high = size - 1;
    for (int s = 0; s < nsym; ++s) {
        if (norm[s] == -1) {
            t[high--].sym = (uint8_t)s;
            cnt[s] = 1;
        } else {
            cnt[s] = (uint16_t)norm[s];
        }
    }
    const int step = (size >> 1) + (size >> 3) + 3, mask = size - 1;
    int pos = 0;
    for (int s = 0; s < nsym; ++s)
        for (int i = 0; i < norm[s]; ++i) {
            t[pos].sym = (uint8_t)s;
            do {
                pos = (pos + step) & mask;
            } while (pos > high);
        }
    if (pos != 0) return false;
    for (int u = 0; u < size; ++u) {
        const uint32_t next = cnt[t[u].sym]++;
        const int nbits = log - highbit(next);
        t[u].nb = (uint8_t)nbits;
        t[u].base = (uint16_t)((next << nbits) - (uint32_t)size);
    }
    return true;
}

// ---- sequence code tables (RFC 8878 3.1.1.3.2.1.1, 3.1.1.3.2.2) ----------
// Literal-length and match-length codes: value = base + that many extra bits
// (the tables of the RFC, as closed forms; each base is the previous base
// plus 2^bits of the previous code).
ZFN int ll_bits(int c) {
    return c < 16 ? 0 : c < 20 ? 1 : c < 22 ? 2 : c < 24 ? 3 : c == 24 ? 4 : c == 25 ? 6 : c - 19;
}
ZFN uint32_t ll_base(int c) {
    return c < 16 ? (uint32_t)c
         : c < 20 ? 16u + 2u * (c - 16)
         : c < 22 ? 24u + 4u * (c - 20)
         : c < 24 ? 32u + 8u * (c - 22)
         : c == 24 ? 48u : 1u << (c - 19);
}
ZFN int ml_bits(int c) {
    return c < 32 ? 0 : c < 36 ? 1 : c < 38 ? 2 : c < 40 ? 3 : c < 42 ? 4 : c == 42 ? 5 : c - 36;
}
ZFN uint32_t ml_base(int c) {
    return c < 32 ? (uint32_t)c + 3u
         : c < 36 ? 35u + 2u * (c - 32)
         : c < 38 ? 43u + 4u * (c - 36)
         : c < 40 ? 51u + 8u * (c - 38)
         : c < 42 ? 67u + 16u * (c - 40)
         : c == 42 ? 99u : (1u << (c - 36)) + 3u;
}

// Predefined distributions (RFC 8878 3.1.1.3.2.2.1-3): literal lengths and
// match lengths at accuracy log 6, offsets at log 5.  Each string holds the
// counts + 1 (so "less than one" is 0).
ZFN int predefined(int kind, int16_t* norm) {  // kind 0 LL, 1 OF, 2 ML; returns the symbol count
    const char* ll = "\5\4\3\3\3\3\3\3\3\3\3\3\3\2\2\2\3\3\3\3\3\3\3\3\3\4\3\2\2\2\2\2\0\0\0\0";
    const char* ml = "\2\5\4\3\3\3\3\3\3\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2"
                     "\2\2\2\2\2\2\2\2\2\2\0\0\0\0\0\0\0";
    const char* of = "\2\2\2\2\2\2\3\3\3\2\2\2\2\2\2\2\2\2\2\2\2\2\2\2\0\0\0\0\0";
    const char* d = kind == 0 ? ll : kind == 1 ? of : ml;
    const int n = kind == 0 ? 36 : kind == 1 ? 29 : 53;
    for (int i = 0; i < n; ++i) norm[i] = (int16_t)(d[i] - 1);
    return n;
}

// ---- Huffman ----------------------------------------------------------------
// Huffman tree description (RFC 8878 4.2.1; libzstd HUF_readStats): weights
// of symbols 0..n-2 either as 4-bit fields or FSE-compressed with two
// interleaved states, the last weight implied by the total.  Lane 0 only:
// writes sh.w[0..*nsym), returns the bytes used or -1, *log = the table log.
ZFN int read_huf_weights(Shared& sh, const uint8_t* p, int64_t n, int* nsym, int* log) {
    if (n < 1) return -1;
    const int hb = p[0];
    int nw = 0, used;
    if (hb >= 128) {
        nw = hb - 127;
        const int bytes = (nw + 1) / 2;
        if (bytes + 1 > n) return -1;
        for (int i = 0; i < nw; ++i) sh.w[i] = (uint8_t)((i & 1) ? (p[1 + i / 2] & 15) : (p[1 + i / 2] >> 4));
        used = bytes + 1;
    } else {
        if (hb + 1 > n) return -1;
        const uint8_t* q = p + 1;
        int ns, al;
        const int h = read_ncount(q, hb, sh.norm, &ns, &al, 6, 255);
        if (h < 0) return -1;
        if (!build_fse(sh.wt, sh.norm, ns, al, sh.cnt)) return -1;
        BackBits br;
        if (!br.init(q + h, hb - h)) return -1;
        uint32_t s1 = br.read(al), s2 = br.read(al);
        // libzstd FSE_decompress_usingDTable_generic: symbols alternate between
        // the two states; once a state update runs past the stream start the
        // other state's symbol is the last one.  At most 255 weights.
        for (;;) {
            if (nw > 253) return -1;
            sh.w[nw++] = sh.wt[s1].sym;
            s1 = sh.wt[s1].base + br.read(sh.wt[s1].nb);
            if (br.pos < 0) {
                sh.w[nw++] = sh.wt[s2].sym;
                break;
            }
            if (nw > 253) return -1;
            sh.w[nw++] = sh.wt[s2].sym;
            s2 = sh.wt[s2].base + br.read(sh.wt[s2].nb);
            if (br.pos < 0) {
                sh.w[nw++] = sh.wt[s1].sym;
                break;
            }
        }
        used = hb + 1;
    }
    uint32_t total = 0;
    int rank1 = 0;
    for (int i = 0; i < nw; ++i) {
        if (sh.w[i] > kHufLogMax) return -1;
        total += (1u << sh.w[i]) >> 1;
        rank1 += sh.w[i] == 1;
    }
    if (total == 0) return -1;
    const int tlog = highbit(total) + 1;
    if (tlog > kHufLogMax) return -1;
    const uint32_t rest = (1u << tlog) - total;
    if (rest != (1u << highbit(rest))) return -1;  // the implied weight must close the tree
    const int last = highbit(rest) + 1;
    sh.w[nw] = (uint8_t)last;
    rank1 += last == 1;
    if (rank1 < 2 || (rank1 & 1)) return -1;
    *nsym = nw + 1;
    *log = tlog;
    return used;
}

// Decoding table of 1 << log entries from sh.w (libzstd HUF_readDTableX1):
// symbols ordered by weight, then by value, each taking 2^(w-1) consecutive
// entries from index 0; an entry holds the symbol and its code length
// log + 1 - w.  The lanes count the symbols of each weight, then rank each
// symbol among the lower symbols of its weight (rounds of nl symbols, lanes
// of equal weight matched in a round) and write its own entries.
ZFN void fill_huf(Shared& sh, int nsym, int log, int lane, int nl) {
    if (lane < 16) sh.wcount[lane] = 0;
    if (nl == 1)
        for (int w = 1; w < 16; ++w) sh.wcount[w] = 0;
    wsync();
    for (int base = 0; base < nsym; base += nl) {  // symbols per weight
        const int s = base + lane;
        const uint32_t w = s < nsym ? sh.w[s] : 0u;
        const uint32_t peers = same_value_lanes(w);
        if (s < nsym && w && (peers & ((1u << lane) - 1u)) == 0)  // the lowest lane of each weight counts it
            sh.wcount[w] += popc(peers);
        wsync();
    }
    if (lane == 0) {  // first table entry of each weight; the counts become the next rank
        int pos = 0;
        for (int w = 1; w <= log; ++w) {
            sh.wpos[w] = pos;
            pos += sh.wcount[w] << (w - 1);
            sh.wcount[w] = 0;
        }
    }
    wsync();
    for (int base = 0; base < nsym; base += nl) {
        const int s = base + lane;
        const uint32_t w = s < nsym ? sh.w[s] : 0u;
        const uint32_t peers = same_value_lanes(w);
        if (s < nsym && w) {
            const int r = sh.wcount[w] + popc(peers & ((1u << lane) - 1u));
            const int at = sh.wpos[w] + (r << (w - 1)), len = 1 << (w - 1);
            const uint16_t v = (uint16_t)((s << 4) | (log + 1 - (int)w));
            for (int i = 0; i < len; ++i) sh.huf[at + i] = v;
        }
        wsync();
        if (s < nsym && w && (peers & ((1u << lane) - 1u)) == 0) sh.wcount[w] += popc(peers);
        wsync();
    }
}

// One Huffman stream of `count` symbols into out[0..count) (libzstd
// HUF_decompress1X1_usingDTable): each step looks up the next `log` bits and
// consumes the entry's code length.  The stream must end exactly at its first
// bit.  false: bad stream.
ZFN bool huf_stream(const Shared& sh, int log, const uint8_t* s, int64_t len, uint8_t* out, uint32_t count) {
    BackBits br;
    if (!br.init(s, len)) return false;
    for (uint32_t i = 0; i < count; ++i) {
        const uint16_t e = sh.huf[br.peek(log)];
        br.skip(e & 15);
        out[i] = (uint8_t)(e >> 4);
    }
    return br.pos == 0;
}

// ---- XXH64 (content checksum; the xxHash specification, seed 0) ------------
ZFN uint64_t rotl64(uint64_t x, int r) { return (x << r) | (x >> (64 - r)); }
ZFN uint64_t xxh64(const uint8_t* p, uint64_t len) {
    const uint64_t P1 = 0x9E3779B185EBCA87ull, P2 = 0xC2B2AE3D27D4EB4Full, P3 = 0x165667B19E3779F9ull,
                   P4 = 0x85EBCA77C2B2AE63ull, P5 = 0x27D4EB2F165667C5ull;
    uint64_t i = 0, h;
    if (len >= 32) {
        uint64_t v[4] = {P1 + P2, P2, 0, 0 - P1};
        for (; i + 32 <= len; i += 32)
            for (int k = 0; k < 4; ++k) v[k] = rotl64(v[k] + le64(p + i + 8 * k) * P2, 31) * P1;
        h = rotl64(v[0], 1) + rotl64(v[1], 7) + rotl64(v[2], 12) + rotl64(v[3], 18);
        for (int k = 0; k < 4; ++k) h = (h ^ (rotl64(v[k] * P2, 31) * P1)) * P1 + P4;
    } else {
        h = P5;
    }
    h += len;
    for (; i + 8 <= len; i += 8) h = rotl64(h ^ (rotl64(le64(p + i) * P2, 31) * P1), 27) * P1 + P4;
    if (i + 4 <= len) {
        h = rotl64(h ^ ((uint64_t)le32(p + i) * P1), 23) * P2 + P3;
        i += 4;
    }
    for (; i < len; ++i) h = rotl64(h ^ (p[i] * P5), 11) * P1;
    h ^= h >> 33;
    h *= P2;
    h ^= h >> 29;
    h *= P3;
    h ^= h >> 32;
    return h;
}

// ---- blocks ------------------------------------------------------------------
struct FrameState {
    int hlog;              // Huffman table log, 0 = no table yet (treeless literals need one)
    int llog, olog, mlog;  // sequence table logs, -1 = undefined (repeat mode needs one)
    uint32_t rep[3];       // repeat offsets (lane 0)
};

// Copy n literal bytes to dst + o.  kind 0: from `from` (the block, never
// overlapping dst), 1: the byte `rle`, 2: from `from` inside dst at or after
// dst + o (each chunk is read before it is written).
ZFN void put_lits(uint8_t* dst, uint64_t o, const uint8_t* from, uint8_t rle, int kind, uint32_t n, int lane, int nl) {
    if (kind == 2) {
        for (uint32_t b = 0; b < n; b += (uint32_t)nl) {
            const uint32_t i = b + (uint32_t)lane;
            uint8_t v = 0;
            if (i < n) v = from[i];
            wsync();
            if (i < n) dst[o + i] = v;
        }
    } else {
        for (uint32_t i = (uint32_t)lane; i < n; i += (uint32_t)nl) dst[o + i] = kind ? rle : from[i];
    }
    wsync();
}

// Match of length n at offset off (1 <= off <= o): dst[o + i] = dst[o + i - off].
ZFN void put_match(uint8_t* dst, uint64_t o, uint32_t off, uint32_t n, int lane, int nl) {
    if (off >= (uint32_t)nl) {  // chunks of nl bytes never read their own writes
        for (uint32_t b = 0; b < n; b += (uint32_t)nl) {
            const uint32_t i = b + (uint32_t)lane;
            if (i < n) dst[o + i] = dst[o + i - off];
            wsync();
        }
    } else {  // short offsets repeat the last `off` bytes: byte i copies o - off + (i mod off)
        const uint32_t step = (uint32_t)nl % off;
        uint32_t r = (uint32_t)lane % off;
        for (uint32_t i = (uint32_t)lane; i < n; i += (uint32_t)nl) {
            dst[o + i] = dst[o - off + r];
            r += step;
            if (r >= off) r -= off;
        }
        wsync();
    }
}

// One sequence-table description (libzstd ZSTD_buildSeqTable).  kind 0 LL,
// 1 OF, 2 ML; mode 0 predefined, 1 RLE, 2 FSE-compressed, 3 repeat (`lg`,
// the current log, must be defined).  Lane 0 only.  Returns the bytes used or
// -1; *lg receives the table's accuracy log.
ZFN int seq_table(Shared& sh, int kind, int mode, const uint8_t* q, int64_t qn, int* lg) {
    Cell* t = kind == 0 ? sh.ll : kind == 1 ? sh.of : sh.ml;
    const int maxsym = kind == 0 ? kMaxLL : kind == 1 ? kMaxOF : kMaxML;
    const int maxlog = kind == 0 ? kLLLog : kind == 1 ? kOFLog : kMLLog;
    if (mode == 0) {
        const int ns = predefined(kind, sh.norm);
        const int al = kind == 1 ? 5 : 6;
        if (!build_fse(t, sh.norm, ns, al, sh.cnt)) return -1;
        *lg = al;
        return 0;
    }
    if (mode == 1) {
        if (qn < 1 || q[0] > maxsym) return -1;
        t[0].sym = q[0];
        t[0].nb = 0;
        t[0].base = 0;
        *lg = 0;
        return 1;
    }
    if (mode == 2) {
        int ns, al;
        const int used = read_ncount(q, qn, sh.norm, &ns, &al, maxlog, maxsym);
        if (used < 0 || !build_fse(t, sh.norm, ns, al, sh.cnt)) return -1;
        *lg = al;
        return used;
    }
    return *lg < 0 ? -1 : 0;
}

// One compressed block (RFC 8878 3.1.1.3; libzstd ZSTD_decompressBlock_internal)
// of bsz bytes at b, decoded to dst + op.  Literals that sequences will copy
// are first decoded into the top of dst ([cap - nlit, cap)): the output
// pointer stays below the unread literals as long as the declared sizes hold,
// and a sequence that would overwrite unread literals would also make the
// frame's output exceed `cap`, so it is rejected.  false: corrupt block.
ZFN bool compressed_block(Shared& sh, FrameState& fs, const uint8_t* b, uint32_t bsz, uint8_t* dst, uint64_t cap,
                          uint64_t& op, uint64_t fstart, int lane, int nl) {
    if (bsz < 2) return false;
    // ---- literals section header (ZSTD_decodeLiteralsBlock) ----
    const int ltype = b[0] & 3, lfmt = (b[0] >> 2) & 3;
    const uint64_t room = cap - op < kBlockMax ? cap - op : kBlockMax;
    uint32_t lhs, nlit, lcs = 0, used;
    int nstreams = 0;
    if (ltype <= 1) {  // raw or RLE
        if (lfmt == 1) {
            lhs = 2;
            if (ltype == 1 && bsz < 3) return false;
            nlit = le16(b) >> 4;
        } else if (lfmt == 3) {
            lhs = 3;
            if (bsz < (ltype == 0 ? 3u : 4u)) return false;
            nlit = le24(b) >> 4;
        } else {
            lhs = 1;
            nlit = b[0] >> 3;
        }
        if (nlit > room) return false;
        if (ltype == 0 && (uint64_t)lhs + nlit > bsz) return false;
        used = ltype == 0 ? lhs + nlit : lhs + 1;
    } else {  // Huffman-coded, with a new table (2) or the previous one (3)
        if (bsz < 5) return false;
        const uint32_t h = le32(b);
        if (lfmt <= 1) {
            lhs = 3;
            nlit = (h >> 4) & 0x3FF;
            lcs = (h >> 14) & 0x3FF;
            nstreams = lfmt == 0 ? 1 : 4;
        } else if (lfmt == 2) {
            lhs = 4;
            nlit = (h >> 4) & 0x3FFF;
            lcs = h >> 18;
            nstreams = 4;
        } else {
            lhs = 5;
            nlit = (h >> 4) & 0x3FFFF;
            lcs = (h >> 22) + ((uint32_t)b[4] << 10);
            nstreams = 4;
        }
        if (nlit > kBlockMax) return false;
        if (nstreams == 4 && nlit < 6) return false;
        if ((uint64_t)lcs + lhs > bsz) return false;
        if (nlit > room) return false;
        if (ltype == 3 && fs.hlog == 0) return false;
        used = lhs + lcs;
    }
    // ---- sequences section header (ZSTD_decodeSeqHeaders) ----
    const uint8_t* q = b + used;
    int64_t qn = (int64_t)bsz - used;
    if (qn < 1) return false;
    uint32_t nseq = q[0];
    int sh_len = 1;
    if (nseq == 255) {
        if (qn < 3) return false;
        nseq = le16(q + 1) + 0x7F00;
        sh_len = 3;
    } else if (nseq >= 128) {
        if (qn < 2) return false;
        nseq = ((nseq - 128) << 8) + q[1];
        sh_len = 2;
    }
    if (nseq == 0 && qn != sh_len) return false;  // extraneous bytes after an empty sequences section
    // ---- literals ----
    int lkind = ltype == 0 ? 0 : ltype == 1 ? 1 : 2;
    const uint8_t* lsrc = b + lhs;
    const uint8_t rle = ltype == 1 ? b[lhs] : 0;
    const uint64_t lpos = nseq ? cap - nlit : op;  // where Huffman literals are decoded
    if (nstreams) {
        const uint8_t* hp = b + lhs;
        int64_t hn = lcs;
        if (ltype == 2) {
            int hu = 0, ns = 0, lg = 0;
            if (lane == 0) hu = read_huf_weights(sh, hp, hn, &ns, &lg);
            hu = (int)from_lane0((uint32_t)hu);
            ns = (int)from_lane0((uint32_t)ns);
            lg = (int)from_lane0((uint32_t)lg);
            if (hu < 0 || hu >= hn) return false;
            fill_huf(sh, ns, lg, lane, nl);
            fs.hlog = lg;
            hp += hu;
            hn -= hu;
        }
        bool bad = false;
        if (nstreams == 1) {
            if (lane == 0) bad = !huf_stream(sh, fs.hlog, hp, hn, dst + lpos, nlit);
        } else {
            if (hn < 10) return false;
            const int64_t l1 = le16(hp), l2 = le16(hp + 2), l3 = le16(hp + 4);
            const int64_t l4 = hn - 6 - l1 - l2 - l3;
            if (l4 < 0) return false;
            const uint32_t seg = (nlit + 3) / 4;
            for (int k = lane; k < 4; k += nl) {
                const int64_t at = 6 + (k > 0 ? l1 : 0) + (k > 1 ? l2 : 0) + (k > 2 ? l3 : 0);
                const int64_t len = k == 0 ? l1 : k == 1 ? l2 : k == 2 ? l3 : l4;
                const uint32_t cnt = k < 3 ? seg : nlit - 3 * seg;
                bad |= !huf_stream(sh, fs.hlog, hp + at, len, dst + lpos + (uint64_t)k * seg, cnt);
            }
        }
        if (any_lane(bad)) return false;
        wsync();
        lsrc = dst + lpos;
    }
    if (nseq == 0) {  // the literals are the block
        if (lkind != 2) put_lits(dst, op, lsrc, rle, lkind, nlit, lane, nl);
        op += nlit;
        return true;
    }
    // ---- sequences (ZSTD_decompressSequences): lane 0 decodes, the warp copies ----
    q += sh_len;
    qn -= sh_len;
    if (qn < 1 || (q[0] & 3)) return false;
    const int modes = q[0];
    ++q;
    --qn;
    int tu = 0;
    for (int kind = 0; kind < 3; ++kind) {  // LL, OF, ML
        const int mode = kind == 0 ? modes >> 6 : kind == 1 ? (modes >> 4) & 3 : (modes >> 2) & 3;
        if (lane == 0) {
            int lg = kind == 0 ? fs.llog : kind == 1 ? fs.olog : fs.mlog;
            tu = seq_table(sh, kind, mode, q, qn, &lg);
            if (kind == 0) fs.llog = lg;
            else if (kind == 1) fs.olog = lg;
            else fs.mlog = lg;
        }
        tu = (int)from_lane0((uint32_t)tu);
        if (tu < 0) return false;
        q += tu;
        qn -= tu;
    }
    BackBits br;
    uint32_t sll = 0, sof = 0, sml = 0;
    bool bad = false;
    if (lane == 0) {
        if (!br.init(q, qn)) {
            bad = true;
        } else {
            sll = br.read(fs.llog);
            sof = br.read(fs.olog);
            sml = br.read(fs.mlog);
        }
    }
    if (any_lane(bad)) return false;
    uint64_t out = op;  // lane 0's output position while it decodes
    uint32_t li = 0;    // literals lane 0 has assigned
    uint32_t lu = 0;    // literals the warp has copied
    for (uint32_t s0 = 0; s0 < nseq; s0 += kSeqBatch) {
        const uint32_t cnt = nseq - s0 < (uint32_t)kSeqBatch ? nseq - s0 : (uint32_t)kSeqBatch;
        if (lane == 0) {
            for (uint32_t j = 0; j < cnt && !bad; ++j) {
                const Cell cl = sh.ll[sll], co = sh.of[sof], cm = sh.ml[sml];
                const uint32_t ob = br.read(co.sym);  // offset bits, then match length, then literal length
                const uint32_t ml = ml_base(cm.sym) + br.read(ml_bits(cm.sym));
                const uint32_t ll = ll_base(cl.sym) + br.read(ll_bits(cl.sym));
                const uint64_t ov = (1ull << co.sym) + ob;
                uint32_t off;
                if (ov > 3) {
                    off = (uint32_t)(ov - 3);
                    fs.rep[2] = fs.rep[1];
                    fs.rep[1] = fs.rep[0];
                    fs.rep[0] = off;
                } else {
                    const uint32_t idx = (uint32_t)ov - 1 + (ll == 0);
                    if (idx == 0) {
                        off = fs.rep[0];
                    } else if (idx == 1) {
                        off = fs.rep[1];
                        fs.rep[1] = fs.rep[0];
                        fs.rep[0] = off;
                    } else if (idx == 2) {
                        off = fs.rep[2];
                        fs.rep[2] = fs.rep[1];
                        fs.rep[1] = fs.rep[0];
                        fs.rep[0] = off;
                    } else {
                        off = fs.rep[0] - 1;
                        fs.rep[2] = fs.rep[1];
                        fs.rep[1] = fs.rep[0];
                        fs.rep[0] = off;
                    }
                }
                if (s0 + j + 1 < nseq) {  // state updates: LL, ML, OF
                    sll = cl.base + br.read(cl.nb);
                    sml = cm.base + br.read(cm.nb);
                    sof = co.base + br.read(co.nb);
                }
                // ZSTD_execSequence's checks, plus the unread-literal guard
                if (ll > nlit - li || (uint64_t)ll + ml > cap - out || off == 0 || off > out + ll - fstart ||
                    (lkind == 2 && out + ml > lpos + li))
                    bad = true;
                sh.seq_ll[j] = ll;
                sh.seq_ml[j] = ml;
                sh.seq_off[j] = off;
                li += ll;
                out += (uint64_t)ll + ml;
            }
            if (!bad && s0 + cnt == nseq && br.pos != 0) bad = true;  // the stream must end exactly
        }
        if (any_lane(bad)) return false;
        wsync();
        for (uint32_t j = 0; j < cnt; ++j) {
            const uint32_t ll = sh.seq_ll[j], ml = sh.seq_ml[j], off = sh.seq_off[j];
            put_lits(dst, op, lsrc + lu, rle, lkind, ll, lane, nl);
            op += ll;
            lu += ll;
            put_match(dst, op, off, ml, lane, nl);
            op += ml;
        }
        wsync();  // lane 0 rewrites the batch next
    }
    if (nlit - lu > cap - op) return false;  // the last literals must fit (ZSTD_decompressSequences)
    put_lits(dst, op, lsrc + lu, rle, lkind, nlit - lu, lane, nl);  // the last literals
    op += nlit - lu;
    return true;
}

// ---- frames ------------------------------------------------------------------
constexpr uint32_t kMagic = 0xFD2FB528u;
constexpr uint64_t kUnknown = ~0ull;

struct FrameHeader {
    uint32_t hsize;     // header bytes
    uint64_t content;   // declared content size, kUnknown if absent
    int checksum;
};

// Frame header (RFC 8878 3.1.1.1; libzstd ZSTD_getFrameHeader).  n >= 5 and
// the magic number checked by the caller.  false: reserved bit set, window
// log above 31, a dictionary id, or a header longer than n.
ZFN bool frame_header(const uint8_t* s, uint64_t n, FrameHeader* h) {
    const uint32_t fhd = s[4];
    const int did = fhd & 3, single = (fhd >> 5) & 1, fcsid = fhd >> 6;
    const int did_len = did == 3 ? 4 : did;
    const int fcs_len = fcsid == 0 ? single : fcsid == 1 ? 2 : fcsid == 2 ? 4 : 8;
    const uint32_t hs = 5 + !single + did_len + fcs_len;
    if (n < hs) return false;
    if (fhd & 8) return false;
    uint32_t pos = 5;
    if (!single && (s[pos++] >> 3) + 10 > 31) return false;
    uint32_t dict = 0;
    for (int i = 0; i < did_len; ++i) dict |= (uint32_t)s[pos + i] << (8 * i);
    pos += did_len;
    if (dict) return false;  // no dictionary is loaded (ZSTD_decompress)
    uint64_t c = kUnknown;
    if (fcs_len == 1) c = s[pos];
    else if (fcs_len == 2) c = le16(s + pos) + 256;
    else if (fcs_len == 4) c = le32(s + pos);
    else if (fcs_len == 8) c = le64(s + pos);
    h->hsize = hs;
    h->content = c;
    h->checksum = (fhd >> 2) & 1;
    return true;
}

// One frame at s (n bytes available, magic checked) into dst + op; advances
// op and returns the input bytes used, or -1 (libzstd ZSTD_decompressFrame).
ZFN int64_t frame(Shared& sh, const uint8_t* s, uint64_t n, uint8_t* dst, uint64_t cap, uint64_t& op, int lane, int nl) {
    if (n < 6 + 3) return -1;
    FrameHeader fh;
    if (!frame_header(s, n, &fh) || n < (uint64_t)fh.hsize + 3) return -1;
    FrameState fs;
    fs.hlog = 0;
    fs.llog = fs.olog = fs.mlog = -1;
    fs.rep[0] = 1;
    fs.rep[1] = 4;
    fs.rep[2] = 8;
    const uint64_t start = op;
    uint64_t ip = fh.hsize;
    for (;;) {
        if (n - ip < 3) return -1;
        const uint32_t bh = le24(s + ip);
        ip += 3;
        const int last = bh & 1, bt = (bh >> 1) & 3;
        const uint32_t bs = bh >> 3;
        if (bt == 3) return -1;
        const uint64_t csz = bt == 1 ? 1 : bs;
        if (csz > n - ip) return -1;
        if (bt == 0) {  // raw
            if (bs > cap - op) return -1;
            put_lits(dst, op, s + ip, 0, 0, bs, lane, nl);
            op += bs;
        } else if (bt == 1) {  // RLE
            if (bs > cap - op) return -1;
            put_lits(dst, op, nullptr, s[ip], 1, bs, lane, nl);
            op += bs;
        } else {
            if (bs >= kBlockMax) return -1;
            if (!compressed_block(sh, fs, s + ip, bs, dst, cap, op, start, lane, nl)) return -1;
        }
        ip += csz;
        if (last) break;
    }
    if (fh.content != kUnknown && op - start != fh.content) return -1;
    if (fh.checksum) {
        if (n - ip < 4) return -1;
        uint32_t h = 0;
        if (lane == 0) h = (uint32_t)xxh64(dst + start, op - start);
        h = from_lane0(h);
        if (h != le32(s + ip)) return -1;
        ip += 4;
    }
    return (int64_t)ip;
}

// ZSTD_decompress(dst, cap, src, n): every frame in src, skippable frames
// skipped.  Returns the bytes written, or -1.  `sh` is the caller's (one per
// warp on the GPU); lane / nl: this thread's lane and the lanes taking part.
ZFN int64_t decompress(Shared& sh, const uint8_t* src, uint64_t n, uint8_t* dst, uint64_t cap, int lane, int nl) {
    uint64_t ip = 0, op = 0;
    while (n - ip >= 5) {
        const uint32_t magic = le32(src + ip);
        if ((magic & 0xFFFFFFF0u) == 0x184D2A50u) {
            if (n - ip < 8) return -1;
            const uint64_t sz = le32(src + ip + 4);
            if (sz > 0xFFFFFFFFull - 8 || 8 + sz > n - ip) return -1;
            ip += 8 + sz;
            continue;
        }
        if (magic != kMagic) return -1;
        const int64_t r = frame(sh, src + ip, n - ip, dst, cap, op, lane, nl);
        if (r < 0) return -1;
        ip += (uint64_t)r;
    }
    if (ip != n) return -1;
    return (int64_t)op;
}

// ZSTD_getFrameContentSize of the first frame: the declared size, 0 for a
// skippable frame, kUnknown when absent; false when the header is malformed.
ZFN bool content_size(const uint8_t* src, uint64_t n, uint64_t* size) {
    if (n < 5) return false;
    const uint32_t magic = le32(src);
    if ((magic & 0xFFFFFFF0u) == 0x184D2A50u) {
        if (n < 8) return false;
        *size = 0;
        return true;
    }
    if (magic != kMagic) return false;
    const uint32_t fhd = src[4];
    if (fhd & 8) return false;
    // ZSTD_getFrameContentSize does not reject a dictionary id; read past it
    const int did = fhd & 3, single = (fhd >> 5) & 1, fcsid = fhd >> 6;
    const int did_len = did == 3 ? 4 : did;
    const int fcs_len = fcsid == 0 ? single : fcsid == 1 ? 2 : fcsid == 2 ? 4 : 8;
    const uint32_t hs = 5 + !single + did_len + fcs_len;
    if (n < hs) return false;
    if (!single && (src[5] >> 3) + 10 > 31) return false;
    const uint32_t pos = 5 + !single + did_len;
    uint64_t c = kUnknown;
    if (fcs_len == 1) c = src[pos];
    else if (fcs_len == 2) c = le16(src + pos) + 256;
    else if (fcs_len == 4) c = le32(src + pos);
    else if (fcs_len == 8) c = le64(src + pos);
    *size = c;
    return true;
}

}  // namespace pvvc_zstd
