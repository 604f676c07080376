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

// Orthographic point splat of one scene along axis `a` onto a width x height image over the
// box face: pixel (u, v) of a particle = floor((p + box/2) * (pixels / box)) per image axis in
// explicitly rounded float, clamped to the image. Per pixel: the particle count and the
// smallest coordinate along the axis (the particle nearest to a viewer on the -a side), as an
// order-preserving integer so that atomicMin gives the same bits in any order.
__device__ __forceinline__ uint32_t order_key(float f)
{
    const uint32_t b = __float_as_uint(f);
    return (b & 0x80000000u) ? ~b : (b | 0x80000000u);
}

template <class R>
__global__ void __launch_bounds__(256) k_splat(const Vec4<R> *__restrict__ pos, uint32_t n, uint32_t scene, int a,
                                               float half_u, float half_v, float scale_u, float scale_v,
                                               uint32_t width, uint32_t height, uint32_t *__restrict__ count,
                                               uint32_t *__restrict__ depth_key)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> p = ldc4(pos + i);
    if (wbits(p.w) != scene) return;
    const float c[3] = {(float) p.x, (float) p.y, (float) p.z};
    const int au = a == 0 ? 1 : 0, av = a == 2 ? 1 : 2;
    const float fu = floorf(__fmul_rn(__fadd_rn(c[au], half_u), scale_u));
    const float fv = floorf(__fmul_rn(__fadd_rn(c[av], half_v), scale_v));
    // NaN and values below the image go to pixel 0, values beyond it to the last pixel
    const uint32_t u = fu >= (float) width ? width - 1 : (fu >= 0.0f ? (uint32_t) fu : 0u);
    const uint32_t v = fv >= (float) height ? height - 1 : (fv >= 0.0f ? (uint32_t) fv : 0u);
    const size_t pix = (size_t) v * width + u;
    if (count) atomicAdd(count + pix, 1u);
    if (depth_key) atomicMin(depth_key + pix, order_key(c[a]));
}

__global__ void k_splat_depth(uint32_t *__restrict__ key, size_t npix)
{
    const size_t k = (size_t) blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= npix) return;
    const uint32_t b = key[k];
    // back from the order-preserving key; an untouched pixel (all ones) becomes +inf
    key[k] = b == 0xFFFFFFFFu ? 0x7F800000u : ((b & 0x80000000u) ? (b & 0x7FFFFFFFu) : ~b);
}

template <class R>
cudaError_t launch_splat(const DevBufs &b, uint32_t n, int layout_sorted, uint32_t scene, int axis, float half_u,
                         float half_v, float scale_u, float scale_v, uint32_t width, uint32_t height,
                         uint32_t *count, float *depth, cudaStream_t st)
{
    const size_t npix = (size_t) width * height;
    cudaError_t e = cudaSuccess;
    if (count) e = cudaMemsetAsync(count, 0, 4 * npix, st);
    if (e == cudaSuccess && depth) e = cudaMemsetAsync(depth, 0xFF, 4 * npix, st);
    if (e != cudaSuccess) return e;
    const Vec4<R> *pos = (const Vec4<R> *) (layout_sorted ? b.pos_s : b.pos_u);
    if (n)
        k_splat<R><<<(n + 255) / 256, 256, 0, st>>>(pos, n, scene, axis, half_u, half_v, scale_u, scale_v, width,
                                                   height, count, (uint32_t *) depth);
    if (depth) k_splat_depth<<<(unsigned) ((npix + 255) / 256), 256, 0, st>>>((uint32_t *) depth, npix);
    return cudaGetLastError();
}

// Download straight into the caller's pinned host arrays: the id-ordered index of every
// particle first (a scatter within device memory), then one gather that writes the float3
// arrays in id order, so that the writes over the host link are contiguous.
template <class R>
__global__ void __launch_bounds__(256) k_id_index(const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                                  const uint32_t *__restrict__ scene_off, uint32_t n,
                                                  uint32_t *__restrict__ inv)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = __ldg(scene_off + wbits(ldc4(pos + i).w)) + wbits(ldc4(vel + i).w);
    if (o < n) inv[o] = i;
    else sph_check(false, CHK_EGRESS);
}

// 256 particles per block: the block's 3 x 256 floats of each array are assembled in shared
// memory and written out as 16-byte stores (the arrays are 16-byte aligned: the caller checks),
// so that the host link sees whole contiguous lines
template <class R>
__global__ void __launch_bounds__(256) k_gather_host(const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                                     const uint32_t *__restrict__ inv, uint32_t n,
                                                     float *__restrict__ xyz, float *__restrict__ v)
{
    __shared__ __align__(16) float buf[2][3 * 256];
    const uint32_t o0 = blockIdx.x * 256, o = o0 + threadIdx.x;
    const uint32_t cnt = min(256u, n - o0);  // particles of this block
    if (o < n) {
        const uint32_t i = __ldg(inv + o);
        if (xyz) {
            const Vec4<R> pp = ldc4(pos + i);
            buf[0][3 * threadIdx.x] = (float) pp.x;
            buf[0][3 * threadIdx.x + 1] = (float) pp.y;
            buf[0][3 * threadIdx.x + 2] = (float) pp.z;
        }
        if (v) {
            const Vec4<R> vv = ldc4(vel + i);
            buf[1][3 * threadIdx.x] = (float) vv.x;
            buf[1][3 * threadIdx.x + 1] = (float) vv.y;
            buf[1][3 * threadIdx.x + 2] = (float) vv.z;
        }
    }
    __syncthreads();
    const uint32_t nf = 3 * cnt;  // floats of this block per array
    for (int a = 0; a < 2; a++) {
        float *dst = a == 0 ? xyz : v;
        if (!dst) continue;
        float *out = dst + 3 * (size_t) o0;  // 16-byte aligned: o0 is a multiple of 256
        for (uint32_t k = threadIdx.x; 4 * k < nf; k += 256) {
            if (4 * k + 4 <= nf)
                *reinterpret_cast<float4 *>(out + 4 * k) = *reinterpret_cast<const float4 *>(&buf[a][4 * k]);
            else
                for (uint32_t e = 4 * k; e < nf; e++) out[e] = buf[a][e];
        }
    }
}

template <class R>
cudaError_t launch_gather_host(const DevBufs &b, uint32_t n, int layout_sorted, float *xyz, float *v, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const Vec4<R> *pos = (const Vec4<R> *) (layout_sorted ? b.pos_s : b.pos_u);
    const Vec4<R> *vel = (const Vec4<R> *) (layout_sorted ? b.vel_s : b.vel_u);
    k_id_index<R><<<(n + 255) / 256, 256, 0, st>>>(pos, vel, b.scene_off, n, b.inv);
    k_gather_host<R><<<(n + 255) / 256, 256, 0, st>>>(pos, vel, b.inv, n, xyz, v);
    return cudaGetLastError();
}

template cudaError_t launch_gather_host<float>(const DevBufs &, uint32_t, int, float *, float *, cudaStream_t);
template cudaError_t launch_handoff<float>(const DevBufs &, uint32_t, int, float *, float *, cudaStream_t);
template cudaError_t launch_handoff<double>(const DevBufs &, uint32_t, int, float *, float *, cudaStream_t);
template cudaError_t launch_splat<float>(const DevBufs &, uint32_t, int, uint32_t, int, float, float, float, float,
                                         uint32_t, uint32_t, uint32_t *, float *, cudaStream_t);
template cudaError_t launch_splat<double>(const DevBufs &, uint32_t, int, uint32_t, int, float, float, float, float,
                                          uint32_t, uint32_t, uint32_t *, float *, cudaStream_t);

SPH_CHECK_ACCESSOR(check_flags_handoff)

}  // namespace sph
