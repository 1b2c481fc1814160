// host_rng.hpp — seeded random numbers for measure, sample and random Clifford
// circuits.
//
// The reference draws from rand 0.8 StdRng, i.e. rand_chacha 0.3 ChaCha12Rng
// (crates/necstar/src/state/stabilizer_decomposed_state/measurement.rs:12-15,
// sampling.rs:22-25, crates/stabilizer-ch-form-rust/src/circuit/
// random_clifford.rs:193-196).  The stream here is that generator, restated
// from the published ChaCha algorithm (D. J. Bernstein, "ChaCha, a variant of
// Salsa20", 2008) in the layout StdRng::from_seed uses:
//  * state words 0-3: the constants "expand 32-byte k"; 4-11: the 32 seed
//    bytes as little-endian words; 12-13: a 64-bit block counter from 0;
//    14-15: the stream id 0;
//  * 12 rounds (6 double rounds), then the input added word by word;
//  * outputs: the keystream's 32-bit words in order, block after block; a
//    64-bit draw is two words, the first as the low half;
//  * a uniform double in [0, 1) is the top 53 bits of a 64-bit draw × 2^-53
//    (rand's Standard f64); a fair bit is the top bit of a 32-bit draw (a
//    widening multiply by the range 2, which never rejects).
// So measure() and random_clifford() draw what the reference draws for the
// same 32-byte seed.  Binomial variates (sampling) are exact in law but not
// rand_distr 0.4's algorithm: direct Bernoulli trials for n ≤ 64, otherwise
// Devroye's beta-splitting recursion (Non-Uniform Random Variate Generation,
// 1986, ch. X) with Marsaglia–Tsang gamma variates (ACM TOMS 26(3), 2000) and
// Marsaglia's polar normal method.  A NULL seed takes 32 bytes from
// std::random_device (the reference: from_entropy).
#pragma once

#include <cmath>
#include <cstdint>
#include <cstring>
#include <random>

namespace nsg {

struct ChaChaCore {
    static constexpr uint32_t kSigma[4] = {0x61707865u, 0x3320646eu, 0x79622d32u, 0x6b206574u};
    static uint32_t rotl32(uint32_t x, int k) { return (x << k) | (x >> (32 - k)); }
    static void quarter(uint32_t* x, int a, int b, int c, int d) {
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 16);
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 12);
        x[a] += x[b]; x[d] = rotl32(x[d] ^ x[a], 8);
        x[c] += x[d]; x[b] = rotl32(x[b] ^ x[c], 7);
    }
    // One block: `rounds` rounds (an even number) over the 16-word input.
    static void block(const uint32_t in[16], int rounds, uint32_t out[16]) {
        uint32_t x[16];
        std::memcpy(x, in, sizeof(x));
        for (int r = 0; r < rounds; r += 2) {
            quarter(x, 0, 4, 8, 12);
            quarter(x, 1, 5, 9, 13);
            quarter(x, 2, 6, 10, 14);
            quarter(x, 3, 7, 11, 15);
            quarter(x, 0, 5, 10, 15);
            quarter(x, 1, 6, 11, 12);
            quarter(x, 2, 7, 8, 13);
            quarter(x, 3, 4, 9, 14);
        }
        for (int i = 0; i < 16; i++) out[i] = x[i] + in[i];
    }
};

struct HostRng {
    uint32_t in[16];
    uint32_t buf[16];
    int pos = 16;  // next unread word of buf

    explicit HostRng(const uint8_t* seed32) {
        uint8_t key[32];
        if (seed32) {
            std::memcpy(key, seed32, 32);
        } else {
            std::random_device rd;
            for (int i = 0; i < 32; i += 4) {
                const uint32_t w = rd();
                std::memcpy(key + i, &w, 4);  // byte order is irrelevant for entropy
            }
        }
        for (int i = 0; i < 4; i++) in[i] = ChaChaCore::kSigma[i];
        for (int i = 0; i < 8; i++)
            in[4 + i] = (uint32_t)key[4 * i] | ((uint32_t)key[4 * i + 1] << 8) | ((uint32_t)key[4 * i + 2] << 16) |
                        ((uint32_t)key[4 * i + 3] << 24);
        in[12] = in[13] = in[14] = in[15] = 0;
    }
    uint32_t next_u32() {
        if (pos == 16) {
            ChaChaCore::block(in, 12, buf);
            if (++in[12] == 0) ++in[13];  // 64-bit block counter
            pos = 0;
        }
        return buf[pos++];
    }
    uint64_t next() {
        const uint64_t lo = next_u32();
        return lo | ((uint64_t)next_u32() << 32);
    }
    int bit() { return (int)(next_u32() >> 31); }
    double uniform() { return (double)(next() >> 11) * (1.0 / 9007199254740992.0); }
    double uniform_open() {  // (0, 1)
        double u;
        do u = uniform();
        while (u == 0.0);
        return u;
    }
    double normal() {  // Marsaglia polar method
        double u, v, q;
        do {
            u = 2.0 * uniform() - 1.0;
            v = 2.0 * uniform() - 1.0;
            q = u * u + v * v;
        } while (q >= 1.0 || q == 0.0);
        return u * std::sqrt(-2.0 * std::log(q) / q);
    }
    double gamma(double a) {  // Marsaglia–Tsang, a > 0
        if (a < 1.0) {
            double u = uniform_open();
            return gamma(a + 1.0) * std::pow(u, 1.0 / a);
        }
        double d = a - 1.0 / 3.0, c = 1.0 / std::sqrt(9.0 * d);
        for (;;) {
            double x, v;
            do {
                x = normal();
                v = 1.0 + c * x;
            } while (v <= 0.0);
            v = v * v * v;
            double u = uniform_open();
            if (u < 1.0 - 0.0331 * (x * x) * (x * x)) return d * v;
            if (std::log(u) < 0.5 * x * x + d * (1.0 - v + std::log(v))) return d * v;
        }
    }
    double beta(double a, double b) {
        double x = gamma(a), y = gamma(b);
        return x / (x + y);
    }
    uint64_t binomial(uint64_t n, double p) {
        if (!(p > 0.0) || n == 0) return 0;
        if (p >= 1.0) return n;
        uint64_t acc = 0;
        while (n > 64) {
            // Devroye: the a-th order statistic of n uniforms is Beta(a, n+1-a).
            uint64_t a = 1 + n / 2, b = n + 1 - a;
            double x = beta((double)a, (double)b);
            if (x >= p) {
                n = a - 1;
                p = p / x;
            } else {
                acc += a;
                n = b - 1;
                p = (p - x) / (1.0 - x);
            }
            if (!(p > 0.0) || n == 0) return acc;
            if (p >= 1.0) return acc + n;
        }
        for (uint64_t i = 0; i < n; i++) acc += (uniform() < p) ? 1 : 0;
        return acc;
    }
};

}  // namespace nsg
