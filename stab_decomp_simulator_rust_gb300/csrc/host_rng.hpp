// host_rng.hpp — seeded random numbers for measure/sample.
//
// The reference draws from rand 0.8 StdRng (ChaCha12) and rand_distr 0.4
// Binomial (crates/necstar/src/state/stabilizer_decomposed_state/
// sampling.rs:22-25,156-158; measurement.rs:12-15,75).  Those third-party
// streams are not reproduced; outcomes follow the same distributions:
//  * xoshiro256** (Blackman & Vigna) seeded from the 32 seed bytes through
//    SplitMix64; a NULL seed uses the clock;
//  * uniform doubles from the top 53 bits;
//  * Binomial(n, p) exactly in law: direct Bernoulli trials for n ≤ 64,
//    otherwise Devroye's beta-splitting recursion (Non-Uniform Random
//    Variate Generation, 1986, ch. X) with Marsaglia–Tsang gamma variates
//    (ACM TOMS 26(3), 2000) and Marsaglia's polar normal method.
#pragma once

#include <chrono>
#include <cmath>
#include <cstdint>
#include <cstring>

namespace nsg {

struct HostRng {
    uint64_t s[4];

    static uint64_t splitmix(uint64_t& x) {
        uint64_t z = (x += 0x9E3779B97F4A7C15ULL);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
        return z ^ (z >> 31);
    }
    explicit HostRng(const uint8_t* seed32) {
        uint64_t w[4] = {0, 0, 0, 0};
        if (seed32) {
            for (int i = 0; i < 4; i++) std::memcpy(&w[i], seed32 + 8 * i, 8);
        } else {
            w[0] = (uint64_t)std::chrono::high_resolution_clock::now().time_since_epoch().count();
            w[1] = (uint64_t)(uintptr_t)this;
        }
        uint64_t x = 0x243F6A8885A308D3ULL;  // every seed word enters the chain once
        for (int i = 0; i < 4; i++) {
            x ^= w[i];
            s[i] = splitmix(x);
        }
    }
    static uint64_t rotl(uint64_t x, int k) { return (x << k) | (x >> (64 - k)); }
    uint64_t next() {
        uint64_t r = rotl(s[1] * 5, 7) * 9;
        uint64_t t = s[1] << 17;
        s[2] ^= s[0];
        s[3] ^= s[1];
        s[1] ^= s[2];
        s[0] ^= s[3];
        s[2] ^= t;
        s[3] = rotl(s[3], 45);
        return r;
    }
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
