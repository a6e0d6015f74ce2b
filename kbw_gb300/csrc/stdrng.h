// The draw generator of a register: rand's StdRng as the reference's
// QubitManager creates it (kbw src/quantum_execution.rs:181-191:
// StdRng::seed_from_u64(KBW_SEED)), restated from the published algorithms.
//
//  * StdRng is ChaCha with 12 rounds (ChaCha12Rng): 256-bit key = the seed,
//    64-bit block counter from 0 in state words 12-13, stream 0 in words
//    14-15; the output is the keystream's 32-bit words in order, and
//    next_u64 joins two consecutive words, the first as the low half.
//  * seed_from_u64 expands the u64 to the 32-byte seed with PCG32 (XSH RR):
//    per 4-byte chunk, state = state * 6364136223846793005 +
//    11634580027462260723, x = rotr32((u32)(((state >> 18) ^ state) >> 27),
//    state >> 59), stored little-endian.
//  * WeightedIndex::sample draws one UniformFloat<f64> sample per call:
//    the 52 high bits of next_u64 as the mantissa of a double in [1, 2),
//    minus 1 (src/convert.rs:60-64, src/quantum_execution.rs:279-282).
//
// The ChaCha core is pinned by the RFC 7539 known answers (20 rounds); the
// composition (seed expansion, round count, word order) follows the crates'
// published sources, which are not available here: parity with the
// reference's actual stream is unpinned.
#pragma once

#include <stdint.h>

namespace kbwg {

// One ChaCha block: key (8 words), 64-bit counter (words 12-13) and stream
// (words 14-15), `rounds` rounds (even), output 16 words.
void chacha_block(const uint32_t key[8], uint64_t counter, uint64_t stream, int rounds, uint32_t out[16]);

struct StdRng {
    uint32_t key[8] = {0};
    uint64_t counter = 0;
    uint32_t buf[16] = {0};
    int idx = 16;  // next unread word of buf (16: generate)

    static StdRng seed_from_u64(uint64_t seed);
    uint32_t next_u32();
    uint64_t next_u64();
    // UniformFloat<f64> draw in [0, 1) from one next_u64
    double uniform01();
};

// The reference's seed: KBW_SEED when it parses as a u64 (Rust's u64
// FromStr: an optional '+', then decimal digits, no overflow), else a
// random one.
uint64_t kbw_seed_from_env();

}  // namespace kbwg
