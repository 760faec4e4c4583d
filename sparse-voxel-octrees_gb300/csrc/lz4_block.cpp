// lz4_block.cpp — LZ4 block format codec for the .oct container.
//
// Written from the published LZ4 block format description: a block is a
// sequence of (token, literals, match) records.  The token's high nibble is
// the literal count and its low nibble the match length minus 4; a nibble of
// 15 continues in following bytes (each 255 adds 255 and the first byte
// below 255 ends it).  A match is a 16-bit little-endian offset back into
// already-decoded output.  The last record carries literals only; the last
// 5 bytes are always literals and the last match starts at least 12 bytes
// before the block end.
//
// The reference writes its .oct payload in 64 MiB blocks with a streaming
// compressor (VoxelOctree.cpp:92-123) whose blocks may reference the previous
// block's bytes; its loader (VoxelOctree.cpp:57-90) decodes into one
// contiguous buffer.  The compressor here emits independent blocks (valid
// input for that loader); the decoder accepts references into earlier blocks
// so it reads the reference's own files.
#include <cstring>

#include "svo_internal.h"

namespace svo {
namespace {
constexpr int kMinMatch = 4;
constexpr size_t kLastLiterals = 5;
constexpr size_t kMatchSafeZone = 12;
constexpr int kHashBits = 16;
constexpr size_t kMaxOffset = 65535;

inline uint32_t read32(const uint8_t *p) {
    uint32_t v;
    std::memcpy(&v, p, 4);
    return v;
}
inline uint32_t hash4(uint32_t v) { return (v * 2654435761u) >> (32 - kHashBits); }

inline uint8_t *put_length(uint8_t *op, size_t len) {
    while (len >= 255) {
        *op++ = 255;
        len -= 255;
    }
    *op++ = (uint8_t)len;
    return op;
}
}  // namespace

size_t lz4_compress_bound(size_t n) { return n + n / 255 + 16; }

size_t lz4_compress_block(const uint8_t *src, size_t n, uint8_t *dst, size_t cap) {
    if (cap < lz4_compress_bound(n)) return 0;
    std::vector<uint32_t> table((size_t)1 << kHashBits, 0xFFFFFFFFu);
    uint8_t *op = dst;
    size_t anchor = 0, ip = 0;
    if (n > kMatchSafeZone + 1) {
        const size_t match_limit = n - kMatchSafeZone;  // a match must start before this
        const size_t extend_limit = n - kLastLiterals;  // and end before this
        while (ip < match_limit) {
            uint32_t seq = read32(src + ip);
            uint32_t h = hash4(seq);
            uint32_t ref = table[h];
            table[h] = (uint32_t)ip;
            if (ref == 0xFFFFFFFFu || ip - ref > kMaxOffset || read32(src + ref) != seq) {
                ++ip;
                continue;
            }
            size_t len = kMinMatch;
            while (ip + len < extend_limit && src[ref + len] == src[ip + len]) ++len;
            size_t lit = ip - anchor;
            size_t ml = len - kMinMatch;
            uint8_t *token = op++;
            *token = (uint8_t)(((lit >= 15 ? 15 : lit) << 4) | (ml >= 15 ? 15 : ml));
            if (lit >= 15) op = put_length(op, lit - 15);
            std::memcpy(op, src + anchor, lit);
            op += lit;
            size_t off = ip - ref;
            *op++ = (uint8_t)(off & 0xFF);
            *op++ = (uint8_t)(off >> 8);
            if (ml >= 15) op = put_length(op, ml - 15);
            ip += len;
            anchor = ip;
        }
    }
    size_t lit = n - anchor;
    uint8_t *token = op++;
    *token = (uint8_t)((lit >= 15 ? 15 : lit) << 4);
    if (lit >= 15) op = put_length(op, lit - 15);
    std::memcpy(op, src + anchor, lit);
    op += lit;
    return (size_t)(op - dst);
}

static inline void copy8(uint8_t *d, const uint8_t *s) {
    uint64_t v;
    std::memcpy(&v, s, 8);
    std::memcpy(d, &v, 8);
}

int lz4_decompress_block(const uint8_t *src, size_t src_len, uint8_t *out, size_t pos0, size_t out_len) {
    size_t ip = 0, op = pos0;
    const size_t end = pos0 + out_len;
    while (op < end) {
        if (ip >= src_len) return -1;
        uint8_t token = src[ip++];
        size_t lit = token >> 4;
        if (lit == 15) {
            uint8_t b;
            do {
                if (ip >= src_len) return -1;
                b = src[ip++];
                lit += b;
            } while (b == 255);
        }
        if (lit > src_len - ip || lit > end - op) return -1;
        if (lit <= 16 && end - op >= 16 && src_len - ip >= 16) {  // short run with slack on both sides
            copy8(out + op, src + ip);
            copy8(out + op + 8, src + ip + 8);
        } else {
            std::memcpy(out + op, src + ip, lit);
        }
        ip += lit;
        op += lit;
        if (op == end) break;
        if (src_len - ip < 2) return -1;
        size_t off = (size_t)src[ip] | ((size_t)src[ip + 1] << 8);
        ip += 2;
        if (off == 0 || off > op) return -1;
        size_t ml = token & 15;
        if (ml == 15) {
            uint8_t b;
            do {
                if (ip >= src_len) return -1;
                b = src[ip++];
                ml += b;
            } while (b == 255);
        }
        ml += kMinMatch;
        if (ml > end - op) return -1;
        uint8_t *dst = out + op;
        const uint8_t *from = dst - off;
        if (off >= 8 && end - op >= ml + 8) {
            // 8-byte steps: every source chunk lies before its destination
            for (size_t k = 0; k < ml; k += 8) copy8(dst + k, from + k);
        } else if (off >= ml) {
            std::memcpy(dst, from, ml);
        } else {
            for (size_t k = 0; k < ml; ++k) dst[k] = from[k];
        }
        op += ml;
    }
    return 0;
}

}  // namespace svo
