// sph_scenes.cpp -- seeded scene generators (host only). The reference's own dam break
// (src/CBaseParticleSimulator.cpp:38-58) plus the synthetic workloads: a jittered
// lattice, a batch plan of dam breaks, and a disc emitter. All arithmetic that decides a
// coordinate is float, in a fixed order, so that other implementations (the tests' numpy
// restatement) reproduce the coordinates bit for bit; compile without FMA contraction.
#include <cmath>
#include <cstdint>

#include "../../include/sph_cuda.h"
#include "sph_emit.h"

namespace {

// splitmix64 (Steele, Lea, Flood 2014): state += golden gamma, then two xor-shift-multiply
// rounds and a final xor-shift.
struct SplitMix64 {
    uint64_t s;
    uint64_t next()
    {
        uint64_t z = (s += 0x9E3779B97F4A7C15ull);
        z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
        z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
        return z ^ (z >> 31);
    }
    // uniform in [0, 1) with 24 bits, exact in float
    float u24() { return (float) (next() >> 40) * 0x1.0p-24f; }
    // uniform in [0, 1) with 53 bits
    double u53() { return (double) (next() >> 11) * 0x1.0p-53; }
};

constexpr float kH = 0.0457f;  // include/CParticle.h:80

}  // namespace

extern "C" {

int64_t sph_scene_reference_dam_break(float box, float *xyz, uint64_t cap)
{
    const double halfParticle = kH / 2.0f;
    const float off = -box / 2.0f;
    int64_t n = 0;
    for (float y = 0; y < box; y += halfParticle)
        for (float x = 0; x < box / 4.0; x += halfParticle)
            for (float z = 0; z < box; z += halfParticle) {
                if (xyz && (uint64_t) n < cap) {
                    xyz[3 * n + 0] = x + off;
                    xyz[3 * n + 1] = y + off;
                    xyz[3 * n + 2] = z + off;
                }
                n++;
            }
    return n;
}

int sph_scene_lattice(const uint32_t dims[3], const float box[3], float spacing, float jitter, uint64_t seed,
                      float *xyz)
{
    if (!dims || !box || !xyz || !(spacing > 0) || !(jitter >= 0)) return SPH_ERR_ARG;
    SplitMix64 rng{seed};
    const float amp = jitter * spacing;
    const float ox = -box[0] / 2.0f, oy = -box[1] / 2.0f, oz = -box[2] / 2.0f;
    uint64_t n = 0;
    for (uint32_t iy = 0; iy < dims[1]; iy++)
        for (uint32_t ix = 0; ix < dims[0]; ix++)
            for (uint32_t iz = 0; iz < dims[2]; iz++) {
                const float jx = (rng.u24() * 2.0f - 1.0f) * amp;
                const float jy = (rng.u24() * 2.0f - 1.0f) * amp;
                const float jz = (rng.u24() * 2.0f - 1.0f) * amp;
                xyz[3 * n + 0] = (ox + (float) ix * spacing) + jx;
                xyz[3 * n + 1] = (oy + (float) iy * spacing) + jy;
                xyz[3 * n + 2] = (oz + (float) iz * spacing) + jz;
                n++;
            }
    return SPH_OK;
}

int sph_scene_batch_plan(uint32_t n_scenes, uint64_t seed, uint32_t nmin, uint32_t nmax, float amin, float amax,
                         uint32_t *dims, float *boxes)
{
    if (!dims || !boxes || nmin == 0 || nmax < nmin || !(amin > 0) || amax < amin) return SPH_ERR_ARG;
    SplitMix64 rng{seed};
    // the 20^3 lattice of the 1.0 x 1.0 x 0.5 m scene: box per lattice row
    const double per[3] = {1.0 / 20.0, 1.0 / 20.0, 0.5 / 20.0};
    const double lmin = std::log((double) nmin), lmax = std::log((double) nmax);
    for (uint32_t s = 0; s < n_scenes; s++) {
        const double nt = std::exp(lmin + rng.u53() * (lmax - lmin));
        double a[3];
        for (int k = 0; k < 3; k++) a[k] = (double) amin + rng.u53() * ((double) amax - (double) amin);
        const double base = std::cbrt(nt / (a[0] * a[1] * a[2]));
        for (int k = 0; k < 3; k++) {
            double d = std::floor(base * a[k] + 0.5);
            if (d < 1) d = 1;
            dims[3 * s + k] = (uint32_t) d;
            boxes[3 * s + k] = (float) (d * per[k]);
        }
    }
    return SPH_OK;
}

int sph_scene_fountain_emit(uint64_t seed, uint32_t step, uint32_t n, const float center[3], float radius, float speed,
                            float sigma, float *xyz, float *vel)
{
    if (!center || !xyz || !vel) return SPH_ERR_ARG;
    for (uint32_t k = 0; k < n; k++) sph::emit::particle(seed, step, k, center, radius, speed, sigma, xyz + 3 * (size_t) k,
                                                         vel + 3 * (size_t) k);
    return SPH_OK;
}

}  // extern "C"
