/*
 * cnncrf_xavier.h -- the seeded Xavier-uniform weight generator used for the
 * synthetic-weight workloads (the reference ships trained weights only).
 * Shared by the library and the CPU oracle so both build identical nets.
 *
 * Array i (a filter of npz shape (co, ci, kh, kw)) is filled in npz order with
 *   w[j] = (float)((2*u_j - 1) * a),  a = sqrt(6 / (fan_in + fan_out)),
 *   fan_in = ci*kh*kw, fan_out = co*kh*kw,
 * u_j = (splitmix64() >> 40) * 2^-24 from a SplitMix64 stream (Steele, Lea &
 * Flood, OOPSLA 2014) started at seed ^ (0x9E3779B97F4A7C15 * (i + 1)).
 * Bias arrays are zero.
 */
#ifndef CNNCRF_XAVIER_H
#define CNNCRF_XAVIER_H

#include <math.h>
#include <stdint.h>

static inline uint64_t cnncrf_splitmix64(uint64_t *state)
{
    uint64_t z = (*state += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}

/* Fill a filter array of npz shape (co, ci, kh, kw) for parameter slot `index`. */
static inline void cnncrf_xavier_fill(float *w, int co, int ci, int kh, int kw, uint64_t seed,
                                      int index)
{
    uint64_t st = seed ^ (0x9E3779B97F4A7C15ull * (uint64_t)(index + 1));
    double fan_in = (double)ci * kh * kw, fan_out = (double)co * kh * kw;
    double a = sqrt(6.0 / (fan_in + fan_out));
    long n = (long)co * ci * kh * kw;
    for (long j = 0; j < n; ++j) {
        double u = (double)(cnncrf_splitmix64(&st) >> 40) * (1.0 / 16777216.0);
        w[j] = (float)((2.0 * u - 1.0) * a);
    }
}

#endif /* CNNCRF_XAVIER_H */
