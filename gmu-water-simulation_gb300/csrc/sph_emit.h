// sph_emit.h -- the disc emitter's particle generator, shared by the host generator
// (sph_scene_fountain_emit) and the device emitter (sph_emit_fountain) so that both produce
// the same bits. It generalises the reference's FOUNTAIN source
// (src/CBaseParticleSimulator.cpp:187-210: a fixed pattern of 7 particles per step at
// v_y = 3.2 box) to a seeded disc of n particles per step with Gaussian velocity spread.
//
// Only integer operations and correctly rounded double +, -, *, / and sqrt are used: on the
// device through the explicitly rounded intrinsics, on the host compiled without
// floating-point contraction. No math-library function is called, so no library's rounding
// enters the result:
//   - each particle draws from its own splitmix64 stream keyed by (seed, step, index);
//   - the disc position is sampled by rejection from the enclosing square;
//   - the three normals come from two draws of Marsaglia's polar method
//     (Marsaglia & Bray 1964), whose logarithm is computed here from the series
//     ln m = 2 atanh((m - 1)/(m + 1)) after splitting off the binary exponent.
// Rejection loops are bounded (64 tries); an exhausted loop takes the centre (position)
// or a zero normal pair, identically on host and device.
#ifndef SPH_EMIT_H
#define SPH_EMIT_H

#include <stdint.h>
#include <string.h>

#ifdef __CUDACC__
#define SPH_HD __host__ __device__ __forceinline__
#else
#define SPH_HD inline
#include <cmath>
#endif

namespace sph {
namespace emit {

SPH_HD double dadd(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dadd_rn(a, b);
#else
    return a + b;
#endif
}
SPH_HD double dsub(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dsub_rn(a, b);
#else
    return a - b;
#endif
}
SPH_HD double dmul(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __dmul_rn(a, b);
#else
    return a * b;
#endif
}
SPH_HD double ddiv(double a, double b)
{
#ifdef __CUDA_ARCH__
    return __ddiv_rn(a, b);
#else
    return a / b;
#endif
}
SPH_HD double dsqrt(double a)
{
#ifdef __CUDA_ARCH__
    return __dsqrt_rn(a);
#else
    return std::sqrt(a);
#endif
}
SPH_HD float to_float(double a)
{
#ifdef __CUDA_ARCH__
    return __double2float_rn(a);
#else
    return (float) a;
#endif
}
SPH_HD uint64_t bits_of(double a)
{
#ifdef __CUDA_ARCH__
    return (uint64_t) __double_as_longlong(a);
#else
    uint64_t u;
    memcpy(&u, &a, sizeof u);
    return u;
#endif
}
SPH_HD double from_bits(uint64_t u)
{
#ifdef __CUDA_ARCH__
    return __longlong_as_double((long long) u);
#else
    double a;
    memcpy(&a, &u, sizeof a);
    return a;
#endif
}

// splitmix64 (Steele, Lea, Flood 2014)
SPH_HD uint64_t next(uint64_t &s)
{
    uint64_t z = (s += 0x9E3779B97F4A7C15ull);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return z ^ (z >> 31);
}
// uniform in [-1, 1) on a 2^-52 grid (exact in double)
SPH_HD double sym(uint64_t &s) { return dsub(dmul((double) (next(s) >> 11), 0x1.0p-52), 1.0); }

// natural logarithm of a positive normal double
SPH_HD double ln_pos(double x)
{
    const uint64_t b = bits_of(x);
    int e = (int) ((b >> 52) & 0x7FF) - 1023;
    double m = from_bits((b & 0x000FFFFFFFFFFFFFull) | 0x3FF0000000000000ull);  // [1, 2)
    if (m > 1.4142135623730951) {  // move m into [sqrt(1/2), sqrt(2))
        m = dmul(m, 0.5);
        e += 1;
    }
    const double y = ddiv(dsub(m, 1.0), dadd(m, 1.0)), y2 = dmul(y, y);  // |y| <= 0.1716
    double term = y, sum = y;
    for (int k = 1; k <= 13; k++) {  // next term below 2^-60 of the sum
        term = dmul(term, y2);
        sum = dadd(sum, ddiv(term, (double) (2 * k + 1)));
    }
    return dadd(dmul((double) e, 0.6931471805599453), dmul(2.0, sum));
}

// two independent standard normals
SPH_HD void polar_pair(uint64_t &s, double &g0, double &g1)
{
    for (int t = 0; t < 64; t++) {
        const double u = sym(s), v = sym(s);
        const double q = dadd(dmul(u, u), dmul(v, v));
        if (q > 0.0 && q < 1.0) {
            const double f = dsqrt(ddiv(dmul(-2.0, ln_pos(q)), q));
            g0 = dmul(u, f);
            g1 = dmul(v, f);
            return;
        }
    }
    g0 = 0.0;
    g1 = 0.0;
}

// particle k of emission step `step`: position on the disc of `radius` around `center` in the
// plane y = center.y, velocity (0, speed, 0) + sigma * N(0, I)
SPH_HD void particle(uint64_t seed, uint32_t step, uint32_t k, const float center[3], float radius, float speed,
                     float sigma, float xyz[3], float vel[3])
{
    uint64_t s = seed ^ (0xD1B54A32D192ED03ull * ((uint64_t) step + 1)) ^ (0x8CB92BA72F3D8DD7ull * ((uint64_t) k + 1));
    next(s);
    double dx = 0.0, dz = 0.0;
    for (int t = 0; t < 64; t++) {
        const double a = sym(s), b = sym(s);
        if (dadd(dmul(a, a), dmul(b, b)) <= 1.0) {
            dx = a;
            dz = b;
            break;
        }
    }
    xyz[0] = to_float(dadd((double) center[0], dmul((double) radius, dx)));
    xyz[1] = center[1];
    xyz[2] = to_float(dadd((double) center[2], dmul((double) radius, dz)));
    double g0, g1, g2, g3;
    polar_pair(s, g0, g1);
    polar_pair(s, g2, g3);
    (void) g3;
    vel[0] = to_float(dmul((double) sigma, g0));
    vel[1] = to_float(dadd((double) speed, dmul((double) sigma, g1)));
    vel[2] = to_float(dmul((double) sigma, g2));
}

}  // namespace emit
}  // namespace sph

#endif  // SPH_EMIT_H
