// sph_handoff.cu -- id-ordered positions (and velocities) of every particle as float3, for a
// front end: into the context's handoff buffers (copied to the host on a second stream) or
// straight into a caller's device array. Plain FP32 and FP64 states; the mixed form uses its
// own egress.
#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {

template <class R>
__global__ void __launch_bounds__(256) k_handoff(const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                                 const uint32_t *__restrict__ scene_off, uint32_t n,
                                                 float *__restrict__ xyz, float *__restrict__ v)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pp = ldc4(pos + i), vv = ldc4(vel + i);
    const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
    xyz[3 * (size_t) o] = (float) pp.x;
    xyz[3 * (size_t) o + 1] = (float) pp.y;
    xyz[3 * (size_t) o + 2] = (float) pp.z;
    if (v) {
        v[3 * (size_t) o] = (float) vv.x;
        v[3 * (size_t) o + 1] = (float) vv.y;
        v[3 * (size_t) o + 2] = (float) vv.z;
    }
}

template <class R>
cudaError_t launch_handoff(const DevBufs &b, uint32_t n, int layout_sorted, float *xyz, float *v, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const Vec4<R> *pos = (const Vec4<R> *) (layout_sorted ? b.pos_s : b.pos_u);
    const Vec4<R> *vel = (const Vec4<R> *) (layout_sorted ? b.vel_s : b.vel_u);
    k_handoff<R><<<(n + 255) / 256, 256, 0, st>>>(pos, vel, b.scene_off, n, xyz, v);
    return cudaGetLastError();
}

template cudaError_t launch_handoff<float>(const DevBufs &, uint32_t, int, float *, float *, cudaStream_t);
template cudaError_t launch_handoff<double>(const DevBufs &, uint32_t, int, float *, float *, cudaStream_t);

}  // namespace sph
