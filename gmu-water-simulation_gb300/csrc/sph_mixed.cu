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
//  - the force pass reads each neighbour from one packed 16-byte record that the density pass
//    writes: the three 16-bit position codes, the FP16 velocity, and the neighbour's two force
//    factors p/rho^2 and 1/rho in FP16, scaled by 2^10 and 2^14 into FP16's normal range
//    (relative rounding error at most 2^-11 each; the particle's own factors stay FP32);
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

__device__ __forceinline__ uint32_t pack_half2(float lo, float hi)
{
    const __half2 a = __floats2half2_rn(lo, hi);
    return *reinterpret_cast<const uint32_t *>(&a);
}

__device__ __forceinline__ float2 unpack_half2(uint32_t v)
{
    return __half22float2(*reinterpret_cast<const __half2 *>(&v));
}

// Scales of the FP16 force factors in the neighbour record: p/rho^2 lies in [-0.03, 0.001] and
// 1/rho in (0, 1/328] (a density always includes the particle's own term, m poly6(0) = 328.3), so
// these bring both into FP16's normal range with room on either side.
constexpr float Q_SCALE = 1024.0f;       // p / rho^2 * 2^10
constexpr float INV_SCALE = 16384.0f;    // 1 / rho * 2^14

// The force pass's view of a neighbour, one 16-byte record:
//   x: codes x | y << 16; y: code z | FP16 vx << 16; z: FP16 vy | FP16 vz << 16;
//   w: FP16 (p/rho^2 * 2^10) | FP16 (1/rho * 2^14) << 16
__device__ __forceinline__ uint4 make_record(uint2 g, float vx, float vy, float vz, float q, float inv)
{
    return make_uint4(g.x, (g.y & 0xffffu) | (pack_half2(vx, 0.0f) << 16), pack_half2(vy, vz),
                      pack_half2(q * Q_SCALE, inv * INV_SCALE));
}

// ---- grid: canonical rank + permute, writing the master state and the gather records ----
// (the state loads issued before the rank is counted, as in the plain form's k_rank_permute)
__global__ void __launch_bounds__(256) k_rank_permute_mixed(
    const uint2 *__restrict__ cid_u, uint32_t n, const uint32_t *__restrict__ start, const uint32_t *__restrict__ tmp,
    const Vec4<float> *__restrict__ pos_u, const Vec4<float> *__restrict__ lo_u, const Vec4<float> *__restrict__ vel_u,
    const SceneDev *__restrict__ scenes, Consts<float> c, MixConsts mc, Vec4<float> *__restrict__ pos_s,
    Vec4<float> *__restrict__ lo_s, Vec4<float> *__restrict__ vel_s, uint2 *__restrict__ gpos,
    uint32_t *__restrict__ big)
{
    chain_wait();
    if (blockIdx.x == 0 && threadIdx.x == 0) big[0] = 0;  // the crowded-cell list is used: empty for the next scan
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 cd = cid_u[i];
    const Vec4<float> p = ld4(pos_u + i), lo = ld4(lo_u + i), v = ld4(vel_u + i);
    const uint32_t b = start[cd.x], e = start[cd.x + 1];
    if (!sph_check(b <= e && e <= n, CHK_SORT)) return;
    const uint32_t dst = b + rank_in_cell(tmp, b, e, cd.y);
    if (!sph_check(dst < e, CHK_SORT)) return;
    st4(pos_s + dst, p);
    st4(lo_s + dst, lo);
    st4(vel_s + dst, v);
    const SceneDev sc = load_scene(scenes, wbits(p.w));
    const uint32_t qx = axis_code(p.x, lo.x, sc.half[0], c.h, c.inv_h_f, mc.to_units);
    const uint32_t qy = axis_code(p.y, lo.y, sc.half[1], c.h, c.inv_h_f, mc.to_units);
    const uint32_t qz = axis_code(p.z, lo.z, sc.half[2], c.h, c.inv_h_f, mc.to_units);
    gpos[dst] = make_uint2(qx | (qy << 16), qz);
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
template <int RAD>
__global__ void __launch_bounds__(128) k_density_mixed(const Vec4<float> *__restrict__ pos,
                                                       const uint2 *__restrict__ gpos, Vec4<float> *__restrict__ aux,
                                                       const uint32_t *__restrict__ start,
                                                       const SceneDev *__restrict__ scenes, uint32_t n,
                                                       Consts<float> c, MixConsts mc, uint32_t *__restrict__ masks,
                                                       const Vec4<float> *__restrict__ vel, uint4 *__restrict__ rec)
{
    using St = Stencil<RAD>;
    chain_wait();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<float> pi = ld4(pos + i);
    const uint2 gi = __ldg(gpos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<float>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    float sum = 0.0f, comp = 0.0f;
    const uint64_t keep = l2_keep_policy();  // masks and records: read by the force pass next
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx - RAD > 0 ? cx - RAD : 0, xh = cx + RAD < X ? cx + RAD : X - 1;
#pragma unroll 1
    for (int dz = -RAD; dz <= RAD; dz++) {
#pragma unroll 1
        for (int dy = -RAD; dy <= RAD; dy++) {
            const int r = (dz + RAD) * (2 * RAD + 1) + (dy + RAD);
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
                if (w < St::WORDS) st_keep(masks + (size_t) (r * St::WORDS + w) * n + i, m, keep);
            }
        }
    }
    const float rho = __fmul_rn(__fmul_rn(sum, mc.poly6_q), c.mass);
    const float p = __fmul_rn(c.k, __fsub_rn(rho, c.rho0));
    const float q = __fdiv_rn(p, __fmul_rn(rho, rho)), inv = __fdiv_rn(1.0f, rho);
    st4(aux + i, Vec4<float>{rho, p, q, inv});
    const Vec4<float> vi = ld4(vel + i);
    st_keep(rec + i, make_record(gi, vi.x, vi.y, vi.z, q, inv), keep);
}

// ---- forces: mask-driven, code-unit displacements, one 16-byte record per neighbour ----------
// Pressure and viscosity terms of one neighbour from its record (the plain form's pair terms in
// code units; src/CCPUParticleSimulator.cpp:177-183). qs = own p/rho^2 * 2^10.
__device__ __forceinline__ void mixed_pair(uint2 gi, const Vec4<float> &vi, float qs, uint4 r, const MixConsts &mc,
                                           float &fpx, float &fpy, float &fpz, float &fvx, float &fvy, float &fvz)
{
    float dx, dy, dz;
    code_delta(gi, make_uint2(r.x, r.y), dx, dy, dz);
    const float vjx = unpack_half2(r.y >> 16).x;
    const float2 vyz = unpack_half2(r.z);
    const float2 qv = unpack_half2(r.w);
    // at least one unit apart: two particles sharing a code (closer than the 5.6 um resolution)
    // get no pressure direction rather than a 0/0
    const float r2 = fmaxf(dx * dx + dy * dy + dz * dz, 1.0f);
    const float rinv = rsqrtf(r2);
    const float hr = QUNITS - r2 * rinv;
    const float wgt = (qs + qv.x) * (mc.spiky_q * (1.0f / Q_SCALE) * hr * hr * rinv);
    fpx += wgt * dx;
    fpy += wgt * dy;
    fpz += wgt * dz;
    const float l = mc.visc_q * (1.0f / INV_SCALE) * hr * qv.y;
    fvx += (vjx - vi.x) * l;
    fvy += (vyz.x - vi.y) * l;
    fvz += (vyz.y - vi.z) * l;
}

// Two accepted neighbours per iteration: both records are loaded before either's terms are
// added (two gathers in flight), the terms still added in candidate order. MINB and BLOCK set
// the register budget and block size (the launch variants of the mixed form).
template <int MINB, int BLOCK, int RAD>
__global__ void __launch_bounds__(BLOCK, MINB) k_forces_mixed(
    const Vec4<float> *__restrict__ pos, const Vec4<float> *__restrict__ lo_s, const Vec4<float> *__restrict__ vel,
    const Vec4<float> *__restrict__ aux, const uint2 *__restrict__ gpos, const uint4 *__restrict__ rec,
    const uint32_t *__restrict__ start, const SceneDev *__restrict__ scenes, const ObstacleDev *__restrict__ obstacles,
    uint32_t n, Consts<float> c, MixConsts mc, const uint32_t *__restrict__ masks, Vec4<float> *__restrict__ pos_out,
    Vec4<float> *__restrict__ lo_out, Vec4<float> *__restrict__ vel_out, Vec4<float> *__restrict__ acc_out,
    uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    chain_wait();
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const Vec4<float> pi = ld4(pos + i);
    const Vec4<float> vi = ld4(vel + i);
    const Vec4<float> ai = ld4(aux + i);
    const uint2 gi = __ldg(gpos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<float>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const float qs = ai.z * Q_SCALE;
    float fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    using St = Stencil<RAD>;
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx - RAD > 0 ? cx - RAD : 0, xh = cx + RAD < X ? cx + RAD : X - 1;
#pragma unroll 1
    for (int dz = -RAD; dz <= RAD; dz++) {
#pragma unroll 1
        for (int dy = -RAD; dy <= RAD; dy++) {
            const int r = (dz + RAD) * (2 * RAD + 1) + (dy + RAD);
            if (r + 1 < St::ROWS) prefetch_l1(masks + (size_t) ((r + 1) * St::WORDS) * n + i);
            const int z = cz + dz, y = cy + dy;
            if (z < 0 || z >= Z || y < 0 || y >= Y) continue;
            const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
            const uint32_t jb = __ldg(start + row + xl), je = __ldg(start + row + xh + 1);
            if (!sph_check(jb <= je && je <= n, CHK_ROW)) continue;
            const uint32_t nw = (je - jb + 31) / 32;
            // the row's recorded words loaded together at the start of the row
            const uint32_t *mr = masks + (size_t) (r * St::WORDS) * n + i;
            uint32_t wr[St::WORDS];
#pragma unroll
            for (int k = 0; k < St::WORDS; k++) wr[k] = nw > (uint32_t) k ? __ldg(mr + k * (size_t) n) : 0u;
            for (uint32_t w = 0; w < nw; w++) {
                const uint32_t cb = jb + 32 * w;
                uint32_t m = 0;
                if (w < (uint32_t) St::WORDS) {
                    m = wr[0];
#pragma unroll
                    for (int k = 1; k < St::WORDS; k++) m = w == (uint32_t) k ? wr[k] : m;
                } else {  // beyond the recorded chunks: test the candidates here
                    const uint32_t ce = min(je, cb + 32u);
                    for (uint32_t j = ce; j-- > cb;) {
                        float x, yy, zz;
                        code_delta(gi, __ldg(gpos + j), x, yy, zz);
                        m = (m << 1) | (h2_minus_r2<float>(x, yy, zz, QH2) > 0.0f ? 1u : 0u);
                    }
                }
                if (i - cb < 32u) m &= ~(1u << (i - cb));  // the particle itself
                while (m) {
                    const uint32_t j0 = cb + (uint32_t) (__ffs(m) - 1);
                    m &= m - 1;
                    const bool two = m != 0;
                    const uint32_t j1 = two ? cb + (uint32_t) (__ffs(m) - 1) : j0;
                    m &= m - 1;
                    if (!sph_check(j0 < je && j1 < je, CHK_NEIGHBOUR)) continue;
                    const uint4 r0 = __ldg(rec + j0), r1 = __ldg(rec + j1);
                    mixed_pair(gi, vi, qs, r0, mc, fpx, fpy, fpz, fvx, fvy, fvz);
                    if (two) mixed_pair(gi, vi, qs, r1, mc, fpx, fpy, fpz, fvx, fvy, fvz);
                }
            }
        }
    }
    // the scene record again rather than kept live across the pair loop (fewer registers)
    const SceneDev sc2 = load_scene(scenes, wbits(pi.w));
    float ax, ay, az;
    accel_of<float>(pi, vi, ai.x, sc2, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, ax, ay, az);
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
    const uint32_t cell = hash_cell<float>(sc2, hx, hy, hz, c, qx, qy, qz);
    count_add(count, c.gsum, cell);
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
    return launch_chained(k_rank_permute_mixed, nblk(n, 256), 256, st, b.cid_u, n, b.start, b.tmp,
                          (const Vec4<float> *) b.pos_u, (const Vec4<float> *) b.lo_u, (const Vec4<float> *) b.vel_u,
                          b.scenes, c, mc, (Vec4<float> *) b.pos_s, (Vec4<float> *) b.lo_s, (Vec4<float> *) b.vel_s,
                          b.gpos, b.big);
}

cudaError_t mixed_density(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, int cell_mult,
                          cudaStream_t st)
{
    if (!n) return cudaSuccess;
    // blocks of 128: the SMs finish the dense and sparse regions more evenly than with 256
    return launch_chained(cell_mult == 2 ? k_density_mixed<2> : k_density_mixed<1>, nblk(n, 128), 128, st,
                          (const Vec4<float> *) b.pos_s, b.gpos, (Vec4<float> *) b.aux, b.start, b.scenes, n, c, mc,
                          b.masks, (const Vec4<float> *) b.vel_s, (uint4 *) b.frec);
}

template <int MINB, int BLOCK, int RAD>
static cudaError_t launch_forces_mixed(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, bool record_acc,
                                       cudaStream_t st)
{
    return launch_chained(
        k_forces_mixed<MINB, BLOCK, RAD>, nblk(n, BLOCK), BLOCK, st, (const Vec4<float> *) b.pos_s,
        (const Vec4<float> *) b.lo_s, (const Vec4<float> *) b.vel_s, (const Vec4<float> *) b.aux, b.gpos,
        (const uint4 *) b.frec, b.start, b.scenes, b.obstacles, n, c, mc, b.masks, (Vec4<float> *) b.pos_u,
        (Vec4<float> *) b.lo_u, (Vec4<float> *) b.vel_u, record_acc ? (Vec4<float> *) b.acc : nullptr, b.cid_u,
        b.count);
}

template <int RAD>
static cudaError_t mixed_forces_rad(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, bool record_acc,
                                    int variant, cudaStream_t st)
{
    // variants: blocks of 128 threads at most 64 (0) or 48 (1) registers, blocks of 256 threads
    // with no cap (2) or at 48 registers (3); every variant computes the same bits
    switch (variant) {
    case 1: return launch_forces_mixed<10, 128, RAD>(b, n, c, mc, record_acc, st);
    case 2: return launch_forces_mixed<1, 256, RAD>(b, n, c, mc, record_acc, st);
    case 3: return launch_forces_mixed<5, 256, RAD>(b, n, c, mc, record_acc, st);
    default: return launch_forces_mixed<8, 128, RAD>(b, n, c, mc, record_acc, st);
    }
}

cudaError_t mixed_forces(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, bool record_acc, int variant,
                         int cell_mult, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    return cell_mult == 2 ? mixed_forces_rad<2>(b, n, c, mc, record_acc, variant, st)
                          : mixed_forces_rad<1>(b, n, c, mc, record_acc, variant, st);
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
