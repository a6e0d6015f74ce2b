// Restated StdRng (see stdrng.h).
#include "stdrng.h"

#include <stdlib.h>
#include <string.h>

#include <random>

namespace kbwg {

static inline uint32_t rotl32(uint32_t x, int r) { return (x << r) | (x >> (32 - r)); }

#define KBWG_QR(a, b, c, d)        \
    a += b, d ^= a, d = rotl32(d, 16); \
    c += d, b ^= c, b = rotl32(b, 12); \
    a += b, d ^= a, d = rotl32(d, 8);  \
    c += d, b ^= c, b = rotl32(b, 7)

void chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds, uint32_t out[16]) {
    uint32_t in[16] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};  // "expand 32-byte k"
    for (int i = 0; i < 8; i++) in[4 + i] = key[i];
    in[12] = (uint32_t)counter;
    in[13] = (uint32_t)(counter >> 32);
    in[14] = (uint32_t)stream;
    in[15] = (uint32_t)(stream >> 32);
    uint32_t x[16];
    memcpy(x, in, sizeof x);
    for (int r = 0; r < rounds; r += 2) {
        KBWG_QR(x[0], x[4], x[8], x[12]);  // columns
        KBWG_QR(x[1], x[5], x[9], x[13]);
        KBWG_QR(x[2], x[6], x[10], x[14]);
        KBWG_QR(x[3], x[7], x[11], x[15]);
        KBWG_QR(x[0], x[5], x[10], x[15]);  // diagonals
        KBWG_QR(x[1], x[6], x[11], x[12]);
        KBWG_QR(x[2], x[7], x[8], x[13]);
        KBWG_QR(x[3], x[4], x[9], x[14]);
    }
    for (int i = 0; i < 16; i++) out[i] = x[i] + in[i];
}
#undef KBWG_QR

StdRng StdRng::seed_from_u64(uint64_t state) {
    StdRng r;
    for (int i = 0; i < 8; i++) {  // PCG32 (XSH RR), one word per 4-byte chunk
        state = state * 6364136223846793005ull + 11634580027462260723ull;
        const uint32_t xorshifted = (uint32_t)(((state >> 18) ^ state) >> 27);
        const int rot = (int)(state >> 59);
        const uint32_t x = rot ? ((xorshifted >> rot) | (xorshifted << (32 - rot))) : xorshifted;
        r.key[i] = x;  // the seed bytes are x little-endian; the key words read them little-endian
    }
    return r;
}

uint32_t StdRng::next_u32() {
    if (idx >= 16) {
        chacha_block(key, counter, 0, 12, buf);
        counter++;
        idx = 0;
    }
    return buf[idx++];
}

uint64_t StdRng::next_u64() {
    const uint64_t lo = next_u32();
    const uint64_t hi = next_u32();
    return (hi << 32) | lo;
}

double StdRng::uniform01() {
    const uint64_t bits = (next_u64() >> 12) | 0x3FF0000000000000ull;
    double v;
    memcpy(&v, &bits, 8);
    return v - 1.0;
}

uint64_t kbw_seed_from_env() {
    const char *t = getenv("KBW_SEED");
    bool ok = t != nullptr && *t != '\0';
    uint64_t v = 0;
    if (ok) {
        const char *p = t;
        if (*p == '+') p++;
        ok = *p != '\0';
        for (; ok && *p; p++) {
            if (*p < '0' || *p > '9') {
                ok = false;
                break;
            }
            const uint64_t d = (uint64_t)(*p - '0');
            if (v > (UINT64_MAX - d) / 10) {
                ok = false;
                break;
            }
            v = v * 10 + d;
        }
    }
    if (ok) return v;
    std::random_device rd;  // the reference falls back to rand::random()
    return ((uint64_t)rd() << 32) ^ (uint64_t)rd();
}

}  // namespace kbwg
