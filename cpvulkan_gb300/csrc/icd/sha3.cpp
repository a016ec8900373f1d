// sha3.cpp — SHA3-256 (FIPS 202, Keccak-f[1600], rate 1088 bits, domain
// suffix 0x06), used for the pipeline-cache key as the reference does
// (CPVulkan/Pipeline.cpp:570-597, CPVulkan/sha3.c). Written from the FIPS 202
// specification.
#include <cstring>

#include "icd.h"

namespace cpv::icd {

namespace {

constexpr uint64_t kRoundConstants[24] = {
    0x0000000000000001ull, 0x0000000000008082ull, 0x800000000000808Aull, 0x8000000080008000ull,
    0x000000000000808Bull, 0x0000000080000001ull, 0x8000000080008081ull, 0x8000000000008009ull,
    0x000000000000008Aull, 0x0000000000000088ull, 0x0000000080008009ull, 0x000000008000000Aull,
    0x000000008000808Bull, 0x800000000000008Bull, 0x8000000000008089ull, 0x8000000000008003ull,
    0x8000000000008002ull, 0x8000000000000080ull, 0x000000000000800Aull, 0x800000008000000Aull,
    0x8000000080008081ull, 0x8000000000008080ull, 0x0000000080000001ull, 0x8000000080008008ull,
};

// Rotation offsets r[x + 5y].
constexpr int kRho[25] = {0, 1, 62, 28, 27, 36, 44, 6, 55, 20, 3, 10, 43, 25, 39, 41, 45, 15, 21, 8, 18, 2, 61, 56, 14};

inline uint64_t rotl(uint64_t v, int n) { return n == 0 ? v : (v << n) | (v >> (64 - n)); }

void keccak_f(uint64_t a[25]) {
    for (int round = 0; round < 24; round++) {
        uint64_t c[5], d[5], b[25];
        for (int x = 0; x < 5; x++) c[x] = a[x] ^ a[x + 5] ^ a[x + 10] ^ a[x + 15] ^ a[x + 20];
        for (int x = 0; x < 5; x++) d[x] = c[(x + 4) % 5] ^ rotl(c[(x + 1) % 5], 1);
        for (int i = 0; i < 25; i++) a[i] ^= d[i % 5];
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) b[y + 5 * ((2 * x + 3 * y) % 5)] = rotl(a[x + 5 * y], kRho[x + 5 * y]);
        for (int x = 0; x < 5; x++)
            for (int y = 0; y < 5; y++) a[x + 5 * y] = b[x + 5 * y] ^ (~b[(x + 1) % 5 + 5 * y] & b[(x + 2) % 5 + 5 * y]);
        a[0] ^= kRoundConstants[round];
    }
}

void absorb_block(uint64_t state[25], const uint8_t* block, size_t rate) {
    for (size_t i = 0; i < rate / 8; i++) {
        uint64_t lane = 0;
        for (int b = 0; b < 8; b++) lane |= static_cast<uint64_t>(block[8 * i + b]) << (8 * b);
        state[i] ^= lane;
    }
    keccak_f(state);
}

}  // namespace

std::array<uint8_t, 32> sha3_256(const void* data, size_t size) {
    constexpr size_t rate = 136;
    uint64_t state[25] = {};
    const uint8_t* p = static_cast<const uint8_t*>(data);
    while (size >= rate) {
        absorb_block(state, p, rate);
        p += rate;
        size -= rate;
    }
    uint8_t last[rate] = {};
    std::memcpy(last, p, size);
    last[size] ^= 0x06;
    last[rate - 1] ^= 0x80;
    absorb_block(state, last, rate);
    std::array<uint8_t, 32> out{};
    for (int i = 0; i < 32; i++) out[i] = static_cast<uint8_t>(state[i / 8] >> (8 * (i % 8)));
    return out;
}

}  // namespace cpv::icd
