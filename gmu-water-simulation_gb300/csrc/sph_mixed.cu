// sph_mixed.cu -- the mixed-precision form of the step (SPH_MIXED).
//
// Same method and pass structure as the plain form (sph_kernels.cu), with these changes:
//  - neighbour positions are gathered as 16-bit codes per axis (8 bytes per particle instead
//    of 16): code = (c mod 8) << 13 | q, where c = floor((p + box/2) / h) is the particle's
//    unclamped cell along that axis and q its offset inside that cell in units of h / 8192.
//    The 16-bit two's-complement difference of two codes is the displacement in those units,
//    exactly, when the particles are less than 4 h apart along the axis; from 4 h to 7 h apart
//    it wraps to a magnitude above h, so the neighbour test still rejects the pair (every
//    neighbour candidate is within 7 h unless a particle has been pushed more than ~5 h
//    outside the box);
//  - neighbour velocities are gathered in FP16 (8 bytes instead of 16);
//  - density sums are compensated FP32 sums: each 32-candidate chunk is summed, and the chunk
//    sums are added with Kahan compensation;
//  - each particle's position is a hi/lo FP32 pair through the integration (TwoSum), and the
//    velocity update is the increment over dt, so no cancellation of x' - x occurs.
// The master state (hi, lo, FP32 velocity) is still read and written once per pass.
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {

constexpr float QUNITS = 8192.0f;        // code units per h
constexpr float QH2 = 67108864.0f;       // h^2 in code units^2 (2^26)

// ---- encoding ------------------------------------------------------------------------
// code of one axis from the hi/lo coordinate: unclamped cell c and offset q inside it
__device__ __forceinline__ uint32_t axis_code(float p, float lo, float half, float h, float inv_h, float to_units)
{
    const float t = (p + half) + lo;            // distance from the box's min wall
    const float c = floorf(t * inv_h);
    int q = __float2int_rd(fmaf(-c, h, t) * to_units);
    q = q < 0 ? 0 : (q > 8191 ? 8191 : q);      // rounding at a cell face
    return ((uint32_t) ((int) c & 7) << 13) | (uint32_t) q;
}

// displacement i - j in code units from the packed codes (x | y << 16, z)
__device__ __forceinline__ void code_delta(uint2 gi, uint2 gj, float &dx, float &dy, float &dz)
{
    const uint32_t dxy = __vsub2(gi.x, gj.x);
    dx = (float) (int16_t) (dxy & 0xffffu);
    dy = (float) ((int32_t) dxy >> 16);
    dz = (float) (int16_t) ((gi.y - gj.y) & 0xffffu);
}

__device__ __forceinline__ uint2 pack_half3(float x, float y, float z)
{
    const __half2 a = __floats2half2_rn(x, y);
    const __half2 b = __floats2half2_rn(z, 0.0f);
    return make_uint2(*reinterpret_cast<const uint32_t *>(&a), *reinterpret_cast<const uint32_t *>(&b));
}

__device__ __forceinline__ void unpack_half3(uint2 v, float &x, float &y, float &z)
{
    const float2 a = __half22float2(*reinterpret_cast<const __half2 *>(&v.x));
    const float2 b = __half22float2(*reinterpret_cast<const __half2 *>(&v.y));
    x = a.x;
    y = a.y;
    z = b.x;
}

// ---- grid: canonical rank + permute, writing the master state and the gather records ----
__global__ void __launch_bounds__(256) k_rank_permute_mixed(
    const uint2 *__restrict__ cid_u, uint32_t n, const uint32_t *__restrict__ start, const uint32_t *__restrict__ tmp,
    const Vec4<float> *__restrict__ pos_u, const Vec4<float> *__restrict__ lo_u, const Vec4<float> *__restrict__ vel_u,
    const SceneDev *__restrict__ scenes, Consts<float> c, MixConsts mc, Vec4<float> *__restrict__ pos_s,
    Vec4<float> *__restrict__ lo_s, Vec4<float> *__restrict__ vel_s, uint2 *__restrict__ gpos, uint2 *__restrict__ gvel)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 cd = cid_u[i];
    const uint32_t b = start[cd.x], e = start[cd.x + 1];
    if (!sph_check(b <= e && e <= n, CHK_SORT)) return;
    uint32_t r = 0;
    for (uint32_t k = b; k < e; k++) r += tmp[k] < cd.y ? 1u : 0u;
    const uint32_t dst = b + r;
    if (!sph_check(dst < e, CHK_SORT)) return;
    const Vec4<float> p = ld4(pos_u + i), lo = ld4(lo_u + i), v = ld4(vel_u + i);
    st4(pos_s + dst, p);
    st4(lo_s + dst, lo);
    st4(vel_s + dst, v);
    const SceneDev sc = load_scene(scenes, wbits(p.w));
    const uint32_t qx = axis_code(p.x, lo.x, sc.half[0], c.h, c.inv_h_f, mc.to_units);
    const uint32_t qy = axis_code(p.y, lo.y, sc.half[1], c.h, c.inv_h_f, mc.to_units);
    const uint32_t qz = axis_code(p.z, lo.z, sc.half[2], c.h, c.inv_h_f, mc.to_units);
    gpos[dst] = make_uint2(qx | (qy << 16), qz);
    gvel[dst] = pack_half3(v.x, v.y, v.z);
}

// Kahan step with explicitly rounded operations (no reassociation, no fused multiply-add)
__device__ __forceinline__ void kahan_add(float &sum, float &comp, float term)
{
    const float y = __fsub_rn(term, comp);
    const float t = __fadd_rn(sum, y);
    comp = __fsub_rn(__fsub_rn(t, sum), y);
    sum = t;
}

// ---- density: neighbour masks (as the plain mask kernel), compensated sums ---------------
__global__ void __launch_bounds__(128) k_density_mixed(const Vec4<float> *__restrict__ pos,
                                                       const uint2 *__restrict__ gpos, Vec4<float> *__restrict__ aux,
                                                       const uint32_t *__restrict__ start,
                                                       const SceneDev *__restrict__ scenes, uint32_t n,
                                                       Consts<float> c, MixConsts mc, uint32_t *__restrict__ masks)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<float> pi = ld4(pos + i);
    const uint2 gi = __ldg(gpos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<float>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    float sum = 0.0f, comp = 0.0f;
    int r = 0;
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx > 0 ? cx - 1 : 0, xh = cx + 1 < X ? cx + 1 : X - 1;
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++, r++) {
            const int z = cz + dz, y = cy + dy;
            if (z < 0 || z >= Z || y < 0 || y >= Y) continue;
            const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
            const uint32_t jb = __ldg(start + row + xl), je = __ldg(start + row + xh + 1);
            if (!sph_check(jb <= je && je <= n, CHK_ROW)) continue;
            int w = 0;
            for (uint32_t cb = jb; cb < je; cb += 32, w++) {
                // bit k of the chunk's word = candidate cb + k (bits enter at the top)
                const uint32_t ce = min(je, cb + 32u);
                uint32_t m = 0;
                float csum = 0.0f;  // the chunk's terms (at most 32), then one compensated add
#pragma unroll 4
                for (uint32_t j = cb; j < ce; j++) {
                    float x, yy, zz;
                    code_delta(gi, __ldg(gpos + j), x, yy, zz);
                    const float t = h2_minus_r2<float>(x, yy, zz, QH2);
                    m = (m >> 1) | (t > 0.0f ? 0x80000000u : 0u);
                    csum = poly6_acc<float>(csum, t);
                }
                kahan_add(sum, comp, csum);
                m >>= 32 - (ce - cb);
                if (w < MASK_WORDS) masks[(size_t) (r * MASK_WORDS + w) * n + i] = m;
            }
        }
    }
    const float rho = __fmul_rn(__fmul_rn(sum, mc.poly6_q), c.mass);
    const float p = __fmul_rn(c.k, __fsub_rn(rho, c.rho0));
    st4(aux + i, Vec4<float>{rho, p, __fdiv_rn(p, __fmul_rn(rho, rho)), __fdiv_rn(1.0f, rho)});
}

// ---- forces: mask-driven, code-unit displacements, FP16 neighbour velocities, hi/lo update ----
__global__ void __launch_bounds__(128, 8) k_forces_mixed(
    const Vec4<float> *__restrict__ pos, const Vec4<float> *__restrict__ lo_s, const Vec4<float> *__restrict__ vel,
    const Vec4<float> *__restrict__ aux, const uint2 *__restrict__ gpos, const uint2 *__restrict__ gvel,
    const uint32_t *__restrict__ start, const SceneDev *__restrict__ scenes, const ObstacleDev *__restrict__ obstacles,
    uint32_t n, Consts<float> c, MixConsts mc, const uint32_t *__restrict__ masks, Vec4<float> *__restrict__ pos_out,
    Vec4<float> *__restrict__ lo_out, Vec4<float> *__restrict__ vel_out, Vec4<float> *__restrict__ acc_out,
    uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<float> pi = ld4(pos + i);
    const Vec4<float> vi = ld4(vel + i);
    const Vec4<float> ai = ld4(aux + i);
    const uint2 gi = __ldg(gpos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<float>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const float qi = ai.z;
    float fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx > 0 ? cx - 1 : 0, xh = cx + 1 < X ? cx + 1 : X - 1;
    int r = 0;
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++, r++) {
            const int z = cz + dz, y = cy + dy;
            if (z < 0 || z >= Z || y < 0 || y >= Y) continue;
            const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
            const uint32_t jb = __ldg(start + row + xl), je = __ldg(start + row + xh + 1);
            if (!sph_check(jb <= je && je <= n, CHK_ROW)) continue;
            const uint32_t nw = (je - jb + 31) / 32;
            for (uint32_t w = 0; w < nw; w++) {
                const uint32_t cb = jb + 32 * w;
                uint32_t m = 0;
                if (w < (uint32_t) MASK_WORDS) {
                    m = __ldg(masks + (size_t) (r * MASK_WORDS + w) * n + i);
                } else {  // beyond the recorded chunks: test the candidates here
                    const uint32_t ce = min(je, cb + 32u);
                    for (uint32_t j = ce; j-- > cb;) {
                        float x, yy, zz;
                        code_delta(gi, __ldg(gpos + j), x, yy, zz);
                        m = (m << 1) | (h2_minus_r2<float>(x, yy, zz, QH2) > 0.0f ? 1u : 0u);
                    }
                }
                while (m) {
                    const uint32_t j = cb + (uint32_t) (__ffs(m) - 1);
                    m &= m - 1;
                    if (j == i || !sph_check(j < je, CHK_NEIGHBOUR)) continue;
                    float dx, dy_, dz_, vjx, vjy, vjz;
                    code_delta(gi, __ldg(gpos + j), dx, dy_, dz_);
                    unpack_half3(__ldg(gvel + j), vjx, vjy, vjz);
                    const float2 qa = __ldg(reinterpret_cast<const float2 *>(aux + j) + 1);
                    // at least one unit apart: two particles sharing a code (closer than the
                    // 5.6 um resolution) get no pressure direction rather than a 0/0
                    const float r2 = fmaxf(dx * dx + dy_ * dy_ + dz_ * dz_, 1.0f);
                    const float rinv = rsqrtf(r2);
                    const float hr = QUNITS - r2 * rinv;
                    const float wgt = (qi + qa.x) * (mc.spiky_q * hr * hr * rinv);
                    fpx += wgt * dx;
                    fpy += wgt * dy_;
                    fpz += wgt * dz_;
                    const float l = mc.visc_q * hr * qa.y;
                    fvx += (vjx - vi.x) * l;
                    fvy += (vjy - vi.y) * l;
                    fvz += (vjz - vi.z) * l;
                }
            }
        }
    }
    float ax, ay, az;
    accel_of<float>(pi, vi, ai.x, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, ax, ay, az);
    // x' = x + (v dt + (a dt) dt) with x = hi + lo carried by TwoSum; v' = increment / dt
    const Vec4<float> li = ld4(lo_s + i);
    const float dt = c.dt;
    const float ix = __fadd_rn(__fmul_rn(vi.x, dt), __fmul_rn(__fmul_rn(ax, dt), dt));
    const float iy = __fadd_rn(__fmul_rn(vi.y, dt), __fmul_rn(__fmul_rn(ay, dt), dt));
    const float iz = __fadd_rn(__fmul_rn(vi.z, dt), __fmul_rn(__fmul_rn(az, dt), dt));
    float hx, lx, hy, ly, hz, lz;
    two_sum(pi.x, __fadd_rn(li.x, ix), hx, lx);
    two_sum(pi.y, __fadd_rn(li.y, iy), hy, ly);
    two_sum(pi.z, __fadd_rn(li.z, iz), hz, lz);
    st4(pos_out + i, Vec4<float>{hx, hy, hz, pi.w});
    st4(lo_out + i, Vec4<float>{lx, ly, lz, 0.0f});
    st4(vel_out + i, Vec4<float>{__fdiv_rn(ix, dt), __fdiv_rn(iy, dt), __fdiv_rn(iz, dt), vi.w});
    if (acc_out) st4(acc_out + i, Vec4<float>{ax, ay, az, 0.0f});
    int qx, qy, qz;
    const uint32_t cell = hash_cell<float>(sc, hx, hy, hz, c, qx, qy, qz);
    atomicAdd(count + cell, 1u);
    cid_out[i] = make_uint2(cell, wbits(vi.w));
}

// ---- egress: id-ordered hi + lo positions (float or double), velocities, rho, p ---------
template <class T>
__global__ void __launch_bounds__(256) k_egress_mixed(const Vec4<float> *__restrict__ posL,
                                                      const Vec4<float> *__restrict__ loL,
                                                      const Vec4<float> *__restrict__ velL,
                                                      const Vec4<float> *__restrict__ posA,
                                                      const Vec4<float> *__restrict__ velA,
                                                      const Vec4<float> *__restrict__ aux,
                                                      const Vec4<float> *__restrict__ pos_u,
                                                      const Vec4<float> *__restrict__ vel_u,
                                                      const Vec4<float> *__restrict__ acc,
                                                      const uint32_t *__restrict__ scene_off, uint32_t n_state,
                                                      uint32_t n_aux, uint32_t n_acc, T *xyz, T *v, T *rho, T *p,
                                                      T *a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_state) {
        const Vec4<float> pp = ldc4(posL + i), ll = ldc4(loL + i), vv = ldc4(velL + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        xyz[3 * o] = (T) pp.x + (T) ll.x;
        xyz[3 * o + 1] = (T) pp.y + (T) ll.y;
        xyz[3 * o + 2] = (T) pp.z + (T) ll.z;
        v[3 * o] = vv.x; v[3 * o + 1] = vv.y; v[3 * o + 2] = vv.z;
    }
    if (i < n_aux) {
        const Vec4<float> pp = ldc4(posA + i), vv = ldc4(velA + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        const Vec4<float> ax = ldc4(aux + i);
        rho[o] = ax.x;
        p[o] = ax.y;
    }
    if (acc && i < n_acc) {
        const Vec4<float> pp = ldc4(pos_u + i), vv = ldc4(vel_u + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        const Vec4<float> aa = ldc4(acc + i);
        a[3 * o] = aa.x; a[3 * o + 1] = aa.y; a[3 * o + 2] = aa.z;
    }
}

// ---- launchers ----------------------------------------------------------------------------
static inline unsigned nblk(uint32_t n, unsigned t) { return (unsigned) ((n + t - 1) / t); }

cudaError_t mixed_permute(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    k_rank_permute_mixed<<<nblk(n, 256), 256, 0, st>>>(b.cid_u, n, b.start, b.tmp, (const Vec4<float> *) b.pos_u,
                                                       (const Vec4<float> *) b.lo_u, (const Vec4<float> *) b.vel_u,
                                                       b.scenes, c, mc, (Vec4<float> *) b.pos_s,
                                                       (Vec4<float> *) b.lo_s, (Vec4<float> *) b.vel_s, b.gpos, b.gvel);
    return cudaGetLastError();
}

cudaError_t mixed_density(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    // blocks of 128: the SMs finish the dense and sparse regions more evenly than with 256
    k_density_mixed<<<nblk(n, 128), 128, 0, st>>>((const Vec4<float> *) b.pos_s, b.gpos, (Vec4<float> *) b.aux,
                                                  b.start, b.scenes, n, c, mc, b.masks);
    return cudaGetLastError();
}

cudaError_t mixed_forces(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, bool record_acc,
                         cudaStream_t st)
{
    if (!n) return cudaSuccess;
    k_forces_mixed<<<nblk(n, 128), 128, 0, st>>>(
        (const Vec4<float> *) b.pos_s, (const Vec4<float> *) b.lo_s, (const Vec4<float> *) b.vel_s,
        (const Vec4<float> *) b.aux, b.gpos, b.gvel, b.start, b.scenes, b.obstacles, n, c, mc, b.masks,
        (Vec4<float> *) b.pos_u, (Vec4<float> *) b.lo_u, (Vec4<float> *) b.vel_u,
        record_acc ? (Vec4<float> *) b.acc : nullptr, b.cid_u, b.count);
    return cudaGetLastError();
}

cudaError_t mixed_egress(const DevBufs &b, uint32_t n_state, uint32_t n_aux, uint32_t n_acc, int layout_sorted,
                         int aux_sorted, bool f64, cudaStream_t st)
{
    if (!n_state) return cudaSuccess;
    const Vec4<float> *posL = (const Vec4<float> *) (layout_sorted ? b.pos_s : b.pos_u);
    const Vec4<float> *loL = (const Vec4<float> *) (layout_sorted ? b.lo_s : b.lo_u);
    const Vec4<float> *velL = (const Vec4<float> *) (layout_sorted ? b.vel_s : b.vel_u);
    const Vec4<float> *posA = (const Vec4<float> *) (aux_sorted ? b.pos_s : b.pos_u);
    const Vec4<float> *velA = (const Vec4<float> *) (aux_sorted ? b.vel_s : b.vel_u);
    const Vec4<float> *acc = (const Vec4<float> *) b.acc;
    if (f64)
        k_egress_mixed<double><<<nblk(n_state, 256), 256, 0, st>>>(
            posL, loL, velL, posA, velA, (const Vec4<float> *) b.aux, (const Vec4<float> *) b.pos_u,
            (const Vec4<float> *) b.vel_u, b.st_acc64 ? acc : nullptr, b.scene_off, n_state, n_aux, n_acc, b.st_xyz64,
            b.st_vel64, b.st_rho64, b.st_p64, b.st_acc64);
    else
        k_egress_mixed<float><<<nblk(n_state, 256), 256, 0, st>>>(
            posL, loL, velL, posA, velA, (const Vec4<float> *) b.aux, (const Vec4<float> *) b.pos_u,
            (const Vec4<float> *) b.vel_u, b.st_acc ? acc : nullptr, b.scene_off, n_state, n_aux, n_acc, b.st_xyz,
            b.st_vel, b.st_rho, b.st_p, b.st_acc);
    return cudaGetLastError();
}

SPH_CHECK_ACCESSOR(check_flags_mixed)

}  // namespace sph
