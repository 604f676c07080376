// sph_emit.cu -- the disc emitter on the device: particle k of an emission step is generated
// by thread k with the generator shared with the host (sph_emit.h), into the staging arrays
// that the append path ingests. No host buffer and no host-to-device copy is involved.
#include "sph_emit.h"
#include "sph_internal.h"

namespace sph {

__global__ void k_emit_fountain(uint64_t seed, uint32_t step, uint32_t n, float cx, float cy, float cz, float radius,
                                float speed, float sigma, float *__restrict__ xyz, float *__restrict__ vel)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    const float c[3] = {cx, cy, cz};
    float p[3], v[3];
    emit::particle(seed, step, k, c, radius, speed, sigma, p, v);
    for (int a = 0; a < 3; a++) {
        xyz[3 * (size_t) k + a] = p[a];
        vel[3 * (size_t) k + a] = v[a];
    }
}

cudaError_t launch_emit_fountain(uint64_t seed, uint32_t step, uint32_t n, const float center[3], float radius,
                                 float speed, float sigma, float *xyz, float *vel, cudaStream_t st)
{
    if (n == 0) return cudaSuccess;
    k_emit_fountain<<<(n + 127) / 128, 128, 0, st>>>(seed, step, n, center[0], center[1], center[2], radius, speed,
                                                    sigma, xyz, vel);
    return cudaGetLastError();
}

}  // namespace sph
