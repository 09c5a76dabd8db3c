// state_format.h -- binary layout of saved solver states and frame records.
//
// The reference has no state output besides the GL vertex buffer it renders
// (ParticleData::Map/Unmap, SPH2S_FINAL_SINGLE_SCALE/ParticleData.cpp:47-66)
// and the rendered pixels VideoWriter writes to a video file
// (SPH2S_FINAL_SINGLE_SCALE/VideoWriter/VideoWriter.cpp:41-49).  The headless
// replacement has two little-endian formats:
//
//   state  "SPHSTAT1" | u32 version | u32 kind | u64 step | kind-specific body
//          | u64 checksum (word-wise FNV-1a over every preceding byte)
//   frame  "SPHFRM01" | u32 kind | u32 fields | u64 step | kind-specific arrays
//
// A state holds everything the next step depends on, in the order the next
// step starts from, so a solver created from it continues bit for bit like
// the solver it was saved from.  Frames are appended records for offline
// inspection; they cannot be resumed from.
#pragma once
#include <cstddef>
#include <cstdint>
#include <cstring>

namespace sph_io {

constexpr char kStateMagic[8] = {'S', 'P', 'H', 'S', 'T', 'A', 'T', '1'};
constexpr char kFrameMagic[8] = {'S', 'P', 'H', 'F', 'R', 'M', '0', '1'};
constexpr uint32_t kStateVersion = 1;
constexpr uint32_t kKindSingleScale = 1;
constexpr uint32_t kKindTwoScale = 2;

struct StatePrefix {
    char magic[8];
    uint32_t version;
    uint32_t kind;
    uint64_t step;
};
static_assert(sizeof(StatePrefix) == 24, "state prefix layout");

struct FramePrefix {
    char magic[8];
    uint32_t kind;
    uint32_t fields;
    uint64_t step;
};
static_assert(sizeof(FramePrefix) == 24, "frame prefix layout");

// FNV-1a with 64-bit words as the unit (the tail is zero-padded to a word);
// it detects truncation and corruption, it is not a cryptographic digest.
inline uint64_t checksum(const void* data, size_t bytes) {
    const unsigned char* p = static_cast<const unsigned char*>(data);
    uint64_t h = 0xcbf29ce484222325ull;
    size_t k = 0;
    for (; k + 8 <= bytes; k += 8) {
        uint64_t w;
        std::memcpy(&w, p + k, 8);
        h = (h ^ w) * 0x100000001b3ull;
    }
    if (k < bytes) {
        uint64_t w = 0;
        std::memcpy(&w, p + k, bytes - k);
        h = (h ^ w) * 0x100000001b3ull;
    }
    return h;
}

// Sequential writer / bounds-checked reader over a caller's buffer.
struct Writer {
    unsigned char* base;
    size_t off = 0;
    unsigned char* take(size_t n) {
        unsigned char* p = base + off;
        off += n;
        return p;
    }
    void put(const void* src, size_t n) { std::memcpy(take(n), src, n); }
};

struct Reader {
    const unsigned char* base;
    size_t size;
    size_t off = 0;
    bool get(void* dst, size_t n) {
        if (n > size - off) return false;
        std::memcpy(dst, base + off, n);
        off += n;
        return true;
    }
    const unsigned char* view(size_t n) {
        if (n > size - off) return nullptr;
        const unsigned char* p = base + off;
        off += n;
        return p;
    }
};

// Validates magic, version, kind and the trailing checksum of a state buffer.
inline bool check_state(const void* src, size_t bytes, uint32_t kind, StatePrefix* prefix) {
    if (!src || bytes < sizeof(StatePrefix) + 8) return false;
    std::memcpy(prefix, src, sizeof(StatePrefix));
    if (std::memcmp(prefix->magic, kStateMagic, 8) != 0) return false;
    if (prefix->version != kStateVersion || prefix->kind != kind) return false;
    uint64_t stored;
    std::memcpy(&stored, static_cast<const unsigned char*>(src) + bytes - 8, 8);
    return stored == checksum(src, bytes - 8);
}

}  // namespace sph_io
