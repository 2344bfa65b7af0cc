// host_common.h -- host-side helpers shared by the text readers, generators and the engine:
// the thread-local error message, the counter-based PRNG and a parallel radix sort.
#pragma once
#include <cstdint>
#include <cstring>
#include <string>
#include <vector>

namespace dsssp {

void set_error(const char* fmt, ...);
int fail(int code, const char* fmt, ...);

// ---- counter-based PRNG: value i of stream s of a seed is mix(key(seed, s) + i*golden) ----
// (SplitMix64's finaliser; no state, so parallel draws are reproducible on any host).
constexpr uint64_t kGolden = 0x9E3779B97F4A7C15ull;

inline uint64_t mix64(uint64_t z) {
    z += kGolden;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

struct Stream {
    uint64_t key;
    Stream(uint64_t seed, uint64_t stream) : key(mix64(mix64(seed) ^ mix64(stream * 0xD1B54A32D192ED03ull))) {}
    uint64_t at(uint64_t i) const { return mix64(key + i * kGolden); }
    // uniform integer in [lo, hi] (Lemire's multiply-shift)
    int64_t range(uint64_t i, int64_t lo, int64_t hi) const {
        unsigned __int128 p = (unsigned __int128)at(i) * (uint64_t)(hi - lo + 1);
        return lo + (int64_t)(uint64_t)(p >> 64);
    }
    double unit(uint64_t i) const { return (double)(at(i) >> 11) * (1.0 / 9007199254740992.0); }
};

inline uint64_t pair_key(uint32_t a, uint32_t b) {
    return a < b ? ((uint64_t)a << 32) | b : ((uint64_t)b << 32) | a;
}

// Sorts 64-bit keys in place (LSD radix, 8-bit digits, parallel histogram + scatter).
void radix_sort_u64(std::vector<uint64_t>& keys);

int num_host_threads();

}  // namespace dsssp
