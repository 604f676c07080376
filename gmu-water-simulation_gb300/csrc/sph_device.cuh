// sph_device.cuh -- device helpers shared by the plain/FP64 kernels (sph_kernels.cu) and
// the mixed-precision kernels (sph_mixed.cu).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_internal.h"

namespace sph {

// ---- checked builds (SPH_CHECKED): a failed index check sets a bit of this translation
// unit's flag word and the access is skipped; sph_debug_check collects the words and verifies
// the pool's canaries. Other builds compile the checks away.
enum CheckBit : unsigned {
    CHK_SORT = 1u,       // a counting-sort scatter target or cell range outside the particles
    CHK_ROW = 2u,        // a neighbour row range outside the particles
    CHK_NEIGHBOUR = 4u,  // a neighbour index from the masks outside its row
    CHK_EGRESS = 8u,     // an id-ordered target outside the particles
};
#ifdef SPH_CHECKED
static __device__ unsigned g_check_flags;
__device__ __forceinline__ bool sph_check(bool ok, unsigned bit)
{
    if (!ok) atomicOr(&g_check_flags, bit);
    return ok;
}
#define SPH_CHECK_ACCESSOR(name)                                                            \
    cudaError_t name(uint32_t *out)                                                         \
    {                                                                                       \
        unsigned v = 0, z = 0;                                                              \
        cudaError_t e = cudaMemcpyFromSymbol(&v, g_check_flags, sizeof v);                  \
        if (e == cudaSuccess) e = cudaMemcpyToSymbol(g_check_flags, &z, sizeof z);          \
        *out |= v;                                                                          \
        return e;                                                                           \
    }
#else
__device__ __forceinline__ bool sph_check(bool, unsigned) { return true; }
#define SPH_CHECK_ACCESSOR(name) \
    cudaError_t name(uint32_t *) { return cudaSuccess; }
#endif

// ---- chained launches (programmatic dependent launch) between the step's kernels: a kernel
// launched by launch_chained may be scheduled while its predecessor in the stream is still
// draining. Such a kernel must call chain_wait() before anything else: it returns once the
// predecessor has completed and its writes are visible (griddepcontrol.wait), then lets the
// next chained kernel be scheduled. Since every chained kernel waits first, each completes only
// after its predecessor, and the stream's order holds transitively. A kernel launched the
// ordinary way passes through chain_wait() at once.
__device__ __forceinline__ void chain_wait()
{
    asm volatile("griddepcontrol.wait;" ::: "memory");
    asm volatile("griddepcontrol.launch_dependents;" ::: "memory");
}

template <typename... K, typename... A>
inline cudaError_t launch_chained(void (*kernel)(K...), unsigned grid, unsigned block, cudaStream_t st, A... args)
{
    cudaLaunchAttribute at[1];
    at[0].id = cudaLaunchAttributeProgrammaticStreamSerialization;
    at[0].val.programmaticStreamSerializationAllowed = 1;
    cudaLaunchConfig_t cfg = {};
    cfg.gridDim = dim3(grid);
    cfg.blockDim = dim3(block);
    cfg.dynamicSmemBytes = 0;
    cfg.stream = st;
    cfg.attrs = at;
    cfg.numAttrs = 1;
    return cudaLaunchKernelEx(&cfg, kernel, ((K) args)...);
}

template <class R>
struct alignas(4 * sizeof(R)) Vec4 {
    R x, y, z, w;
};

__device__ __forceinline__ Vec4<float> ld4(const Vec4<float> *p)
{
    const float4 v = __ldg(reinterpret_cast<const float4 *>(p));
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Vec4<double> ld4(const Vec4<double> *p)
{
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = __ldg(q), b = __ldg(q + 1);
    return {a.x, a.y, b.x, b.y};
}
// plain (coherent) loads for buffers written earlier in the same kernel sequence
__device__ __forceinline__ Vec4<float> ldc4(const Vec4<float> *p)
{
    const float4 v = *reinterpret_cast<const float4 *>(p);
    return {v.x, v.y, v.z, v.w};
}
__device__ __forceinline__ Vec4<double> ldc4(const Vec4<double> *p)
{
    const double2 *q = reinterpret_cast<const double2 *>(p);
    const double2 a = q[0], b = q[1];
    return {a.x, a.y, b.x, b.y};
}
__device__ __forceinline__ void st4(Vec4<float> *p, Vec4<float> v)
{
    *reinterpret_cast<float4 *>(p) = make_float4(v.x, v.y, v.z, v.w);
}
__device__ __forceinline__ void st4(Vec4<double> *p, Vec4<double> v)
{
    double2 *q = reinterpret_cast<double2 *>(p);
    q[0] = make_double2(v.x, v.y);
    q[1] = make_double2(v.z, v.w);
}
// Stores of what the density pass hands to the force pass (the neighbour masks and the force
// records), marked evict-last in L2 (createpolicy ... L2::evict_last with an L2::cache_hint
// store): they are read by the very next kernel, while the streams around them are read once.
__device__ __forceinline__ uint64_t l2_keep_policy()
{
    uint64_t p;
    asm volatile("createpolicy.fractional.L2::evict_last.b64 %0, 1.0;" : "=l"(p));
    return p;
}
__device__ __forceinline__ void st_keep(uint32_t *a, uint32_t v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.b32 [%0], %1, %2;" ::"l"(a), "r"(v), "l"(pol) : "memory");
}
__device__ __forceinline__ void st4_keep(Vec4<float> *p, Vec4<float> v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.v4.f32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w), "l"(pol)
                 : "memory");
}
__device__ __forceinline__ void st4_keep(Vec4<double> *p, Vec4<double> v, uint64_t) { st4(p, v); }
__device__ __forceinline__ void st_keep(uint4 *p, uint4 v, uint64_t pol)
{
    asm volatile("st.global.L2::cache_hint.v4.b32 [%0], {%1, %2, %3, %4}, %5;" ::"l"(p), "r"(v.x), "r"(v.y), "r"(v.z),
                 "r"(v.w), "l"(pol)
                 : "memory");
}

// The force passes start every row by loading the row's mask word, the head of that row's
// chain of dependent loads: the next row's word is fetched into L1 while a row is walked.
__device__ __forceinline__ void prefetch_l1(const void *p)
{
    asm volatile("prefetch.global.L1 [%0];" ::"l"(p));
}

// (q, 1/rho) of a neighbour: the upper half of its aux record
__device__ __forceinline__ void ld_qinv(const Vec4<float> *p, float &q, float &inv)
{
    const float2 v = __ldg(reinterpret_cast<const float2 *>(p) + 1);
    q = v.x;
    inv = v.y;
}
__device__ __forceinline__ void ld_qinv(const Vec4<double> *p, double &q, double &inv)
{
    const double2 v = __ldg(reinterpret_cast<const double2 *>(p) + 1);
    q = v.x;
    inv = v.y;
}

// .w fields carry 32-bit integers (scene index in positions, particle id in velocities)
__device__ __forceinline__ uint32_t wbits(float w) { return __float_as_uint(w); }
__device__ __forceinline__ uint32_t wbits(double w) { return (uint32_t) __double_as_longlong(w); }
template <class R>
__device__ __forceinline__ R mkw(uint32_t v);
template <>
__device__ __forceinline__ float mkw<float>(uint32_t v) { return __uint_as_float(v); }
template <>
__device__ __forceinline__ double mkw<double>(uint32_t v) { return __longlong_as_double((long long) v); }

// correctly rounded operations that the compiler may not fuse: the per-particle epilogue
// mirrors the reference's float expression order
__device__ __forceinline__ float radd(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double radd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float rsub(float a, float b) { return __fsub_rn(a, b); }
__device__ __forceinline__ double rsub(double a, double b) { return __dsub_rn(a, b); }
__device__ __forceinline__ float rmul(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double rmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ float rdiv(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double rdiv(double a, double b) { return __ddiv_rn(a, b); }
__device__ __forceinline__ float rfma(float a, float b, float c) { return __fmaf_rn(a, b, c); }
__device__ __forceinline__ double rfma(double a, double b, double c) { return __fma_rn(a, b, c); }
__device__ __forceinline__ float inv_sqrt(float x) { return rsqrtf(x); }
__device__ __forceinline__ double inv_sqrt(double x) { return 1.0 / sqrt(x); }

// The cell of a position in the step grid (cells h / cell multiple wide), and its global index.
template <class R>
__device__ __forceinline__ uint32_t hash_cell(const SceneDev &sc, R x, R y, R z, const Consts<R> &c, int &cx,
                                              int &cy, int &cz)
{
    cx = cell_axis(x, sc.half[0], c.inv_cell_f, c.cell_d, sc.res[0]);
    cy = cell_axis(y, sc.half[1], c.inv_cell_f, c.cell_d, sc.res[1]);
    cz = cell_axis(z, sc.half[2], c.inv_cell_f, c.cell_d, sc.res[2]);
    return sc.cell_base + (uint32_t) cx + (uint32_t) cy * (uint32_t) sc.res[0] +
           (uint32_t) cz * (uint32_t) sc.res[0] * (uint32_t) sc.res[1];
}

__device__ __forceinline__ SceneDev load_scene(const SceneDev *scenes, uint32_t s)
{
    SceneDev sc;
    const uint4 *src = reinterpret_cast<const uint4 *>(scenes + s);
    uint4 *dst = reinterpret_cast<uint4 *>(&sc);
#pragma unroll
    for (int k = 0; k < (int) (sizeof(SceneDev) / 16); k++) dst[k] = __ldg(src + k);
    return sc;
}

// (h^2 - r^2)^3 for r^2 <= h^2, else 0, branchless: t = h^2 - dx^2 - dy^2 - dz^2 clamped at 0.
// Every density kernel uses this one expression, so all launch variants give the same bits
// (a candidate outside a particle's own 27 cells is farther than h and adds exactly 0).
// Neighbour test shared by every kernel: r^2 < h^2 as h^2 - r^2 > 0 (the reference's r^2 <= h^2
// differs only for pairs at exactly r = h, whose density and force terms are 0).
// The neighbour test h^2 - r^2 > 0 and the poly6 sum, with every rounding explicit (fused
// multiply-adds in a fixed order) so that each kernel that evaluates them gets the same bits.
template <class R>
__device__ __forceinline__ R h2_minus_r2(R dx, R dy, R dz, R h2)
{
    R t = rfma(-dx, dx, h2);
    t = rfma(-dy, dy, t);
    return rfma(-dz, dz, t);
}
// acc + max(t, 0)^3
template <class R>
__device__ __forceinline__ R poly6_acc(R acc, R t)
{
    t = t > (R) 0 ? t : (R) 0;
    return rfma(rmul(t, t), t, acc);
}
template <class R>
__device__ __forceinline__ R poly6_add(R acc, R dx, R dy, R dz, R h2)
{
    return poly6_acc<R>(acc, h2_minus_r2<R>(dx, dy, dz, h2));
}
// The two walls of one axis (src/CCollisionGeometry.cpp:117-133 restated per component).
template <class R>
__device__ __forceinline__ void wall_axis(R p, R v, R half, const Consts<R> &c, R &acc)
{
    R d = radd(rmul(rsub(-half, p), (R) 1), c.wall_r);  // min wall, inverse normal +1
    if (d > (R) 0) acc = radd(radd(acc, rmul(rmul((R) 1, c.wall_k), d)), rmul((R) 1, rmul(c.wall_damp, rmul(v, (R) 1))));
    d = radd(rmul(rsub(half, p), (R) -1), c.wall_r);    // max wall, inverse normal -1
    if (d > (R) 0)
        acc = radd(radd(acc, rmul(rmul((R) -1, c.wall_k), d)), rmul((R) -1, rmul(c.wall_damp, rmul(v, (R) -1))));
}

// Acceleration of one particle in the force pass: total acceleration from the summed pressure and
// viscosity terms (src/CCPUParticleSimulator.cpp:189-193), walls (src/CCollisionGeometry.cpp:117-133),
// box obstacles, position-Verlet integration (src/CCPUParticleSimulator.cpp:211-229), and the
// cell hash of the new position for the next step. Float operations are explicitly rounded
// in the reference's order.
template <class R>
__device__ __forceinline__ void accel_of(const Vec4<R> &pi, const Vec4<R> &vi, R rho, const SceneDev &sc,
                                         const ObstacleDev *__restrict__ obstacles, const Consts<R> &c, R fpx,
                                         R fpy, R fpz, R fvx, R fvy, R fvz, R &ax, R &ay, R &az)
{
    const R sp = rmul(-c.mass, rho), sv = rmul(c.mu, c.mass);
    ax = rdiv(radd(radd(rmul(fpx, sp), rmul(fvx, sv)), rmul((R) sc.gravity[0], rho)), rho);
    ay = rdiv(radd(radd(rmul(fpy, sp), rmul(fvy, sv)), rmul((R) sc.gravity[1], rho)), rho);
    az = rdiv(radd(radd(rmul(fpz, sp), rmul(fvz, sv)), rmul((R) sc.gravity[2], rho)), rho);

    // walls at -+box/2 in the order left, bottom, back, right, top, front. Each wall acts on
    // one component only, so per axis: the min wall (inverse normal +1), then the max wall
    // (inverse normal -1); d = dot(wall - p, n_inv) + r, a += K n_inv d + damp dot(v, n_inv) n_inv.
    R wx = 0, wy = 0, wz = 0;
    wall_axis<R>(pi.x, vi.x, (R) sc.half[0], c, wx);
    wall_axis<R>(pi.y, vi.y, (R) sc.half[1], c, wy);
    wall_axis<R>(pi.z, vi.z, (R) sc.half[2], c, wz);
    // box obstacles: inside the obstacle grown by the particle radius, push out through the
    // nearest face with the wall spring and damping
    for (uint32_t o = 0; o < sc.n_obs; o++) {
        const ObstacleDev ob = obstacles[sc.obs_base + o];
        const R d0 = radd(rsub(pi.x, (R) ob.lo[0]), c.wall_r), d1 = radd(rsub(pi.y, (R) ob.lo[1]), c.wall_r);
        const R d2 = radd(rsub(pi.z, (R) ob.lo[2]), c.wall_r), d3 = radd(rsub((R) ob.hi[0], pi.x), c.wall_r);
        const R d4 = radd(rsub((R) ob.hi[1], pi.y), c.wall_r), d5 = radd(rsub((R) ob.hi[2], pi.z), c.wall_r);
        if (d0 <= (R) 0 || d1 <= (R) 0 || d2 <= (R) 0 || d3 <= (R) 0 || d4 <= (R) 0 || d5 <= (R) 0) continue;
        // first face with the smallest penetration, in face order
        R best = d0;
        int bf = 0;
        if (d1 < best) { best = d1; bf = 1; }
        if (d2 < best) { best = d2; bf = 2; }
        if (d3 < best) { best = d3; bf = 3; }
        if (d4 < best) { best = d4; bf = 4; }
        if (d5 < best) { best = d5; bf = 5; }
        const R sgn = bf < 3 ? (R) -1 : (R) 1;  // outward normal of the face
        const R kt = rmul(rmul(sgn, c.wall_k), best);
        const int a = bf % 3;
        const R v = a == 0 ? vi.x : (a == 1 ? vi.y : vi.z);
        const R dt = rmul(sgn, rmul(c.wall_damp, rmul(v, sgn)));
        if (a == 0) wx = radd(radd(wx, kt), dt);
        else if (a == 1) wy = radd(radd(wy, kt), dt);
        else wz = radd(radd(wz, kt), dt);
    }
    ax = radd(ax, wx);
    ay = radd(ay, wy);
    az = radd(az, wz);

}

// count[cell] += 1 and gsum[cell / kScanTile] += 1 with one atomic per cell and one per group
// among the warp's converged lanes (sorted particles of a warp mostly land in the same few cells)
__device__ __forceinline__ void count_add(uint32_t *__restrict__ count, uint32_t *__restrict__ gsum, uint32_t cell)
{
    const unsigned act = __activemask();
    const int lane = (int) (threadIdx.x & 31u);
    const unsigned peers = __match_any_sync(act, cell);
    if (lane == __ffs(peers) - 1) atomicAdd(count + cell, (uint32_t) __popc(peers));
    const uint32_t g = cell / kScanTile;
    const unsigned gpeers = __match_any_sync(act, g);
    if (lane == __ffs(gpeers) - 1) atomicAdd(gsum + g, (uint32_t) __popc(gpeers));
}

template <class R>
__device__ __forceinline__ void finish_particle(uint32_t i, const Vec4<R> &pi, const Vec4<R> &vi, R rho,
                                                const SceneDev &sc, const ObstacleDev *__restrict__ obstacles,
                                                const Consts<R> &c, R fpx, R fpy, R fpz, R fvx, R fvy, R fvz,
                                                Vec4<R> *__restrict__ pos_out, Vec4<R> *__restrict__ vel_out,
                                                Vec4<R> *__restrict__ acc_out, uint2 *__restrict__ cid_out,
                                                uint32_t *__restrict__ count)
{
    R ax, ay, az;
    accel_of<R>(pi, vi, rho, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, ax, ay, az);
    // x' = x + v dt + (a dt) dt ; v' = (x' - x) / dt
    const R dt = c.dt;
    const R nx = radd(radd(pi.x, rmul(vi.x, dt)), rmul(rmul(ax, dt), dt));
    const R ny = radd(radd(pi.y, rmul(vi.y, dt)), rmul(rmul(ay, dt), dt));
    const R nz = radd(radd(pi.z, rmul(vi.z, dt)), rmul(rmul(az, dt), dt));
    const R nvx = rdiv(rsub(nx, pi.x), dt), nvy = rdiv(rsub(ny, pi.y), dt), nvz = rdiv(rsub(nz, pi.z), dt);
    st4(pos_out + i, Vec4<R>{nx, ny, nz, pi.w});
    st4(vel_out + i, Vec4<R>{nvx, nvy, nvz, vi.w});
    if (acc_out) st4(acc_out + i, Vec4<R>{ax, ay, az, (R) 0});
    int qx, qy, qz;
    const uint32_t cell = hash_cell<R>(sc, nx, ny, nz, c, qx, qy, qz);
    count_add(count, c.gsum, cell);
    cid_out[i] = make_uint2(cell, wbits(vi.w));
}

template <class R>
__device__ __forceinline__ void pair_terms(const Vec4<R> &pi, const Vec4<R> &vi, R qi, const Vec4<R> &pj,
                                           const Vec4<R> &vj, R qj, R invj, const Consts<R> &c, R &fpx, R &fpy,
                                           R &fpz, R &fvx, R &fvy, R &fvz);

// The density pass's record of a particle: (rho, p, c_spiky p/rho^2, c_visc/rho). The last two
// are the per-particle factors of the force terms with the kernels' constants folded in, so
// that a pair costs two multiplications less (src/CCPUParticleSimulator.cpp:177-183).
template <class R>
__device__ __forceinline__ Vec4<R> aux_record(R rho, R p, const Consts<R> &c)
{
    return Vec4<R>{rho, p, rmul(c.c_spiky, rdiv(p, rmul(rho, rho))), rdiv(c.c_visc, rho)};
}

// Pressure and viscosity terms of one accepted neighbour (src/CCPUParticleSimulator.cpp:177-183).
template <class R>
__device__ __forceinline__ void pair_force(const Vec4<R> &pi, const Vec4<R> &vi, R qi, uint32_t j,
                                           const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                           const Vec4<R> *__restrict__ aux, const Consts<R> &c, R &fpx, R &fpy,
                                           R &fpz, R &fvx, R &fvy, R &fvz)
{
    const Vec4<R> pj = ld4(pos + j);
    const Vec4<R> vj = ld4(vel + j);
    R qj, invj;
    ld_qinv(aux + j, qj, invj);
    pair_terms<R>(pi, vi, qi, pj, vj, qj, invj, c, fpx, fpy, fpz, fvx, fvy, fvz);
}

// The same terms from a neighbour's records already loaded (pair_force's arithmetic).
template <class R>
__device__ __forceinline__ void pair_terms(const Vec4<R> &pi, const Vec4<R> &vi, R qi, const Vec4<R> &pj,
                                           const Vec4<R> &vj, R qj, R invj, const Consts<R> &c, R &fpx, R &fpy,
                                           R &fpz, R &fvx, R &fvy, R &fvz)
{
    const R dx = rsub(pi.x, pj.x), dy = rsub(pi.y, pj.y), dz = rsub(pi.z, pj.z);
    const R r2 = rfma(dz, dz, rfma(dy, dy, rmul(dx, dx)));
    const R rinv = inv_sqrt(r2);
    const R hr = rfma(-r2, rinv, c.h);
    // (p_i/rho_i^2 + p_j/rho_j^2) grad W and lap W / rho_j, the constants carried by qi, qj, invj
    const R w = rmul(radd(qi, qj), rmul(rmul(hr, hr), rinv));
    fpx = rfma(w, dx, fpx);
    fpy = rfma(w, dy, fpy);
    fpz = rfma(w, dz, fpz);
    const R l = rmul(hr, invj);
    fvx = rfma(rsub(vj.x, vi.x), l, fvx);
    fvy = rfma(rsub(vj.y, vi.y), l, fvy);
    fvz = rfma(rsub(vj.z, vi.z), l, fvz);
}

// TwoSum (Knuth): s + e == a + b exactly, s = fl(a + b); explicitly rounded operations.
__device__ __forceinline__ void two_sum(float a, float b, float &s, float &e)
{
    s = __fadd_rn(a, b);
    const float bp = __fsub_rn(s, a);
    e = __fadd_rn(__fsub_rn(a, __fsub_rn(s, bp)), __fsub_rn(b, bp));
}


// Rank of id among the ids of its cell, the slots tmp[b, e): the number of smaller ids. Cells of
// at most kBigCell particles are counted directly (occupancy^2 work per cell, trivial at such
// sizes). Larger cells, up to kBigCellMax, have had their slots sorted by k_sort_big, and the
// rank is a lower-bound search. Cells above kBigCellMax (thousands of times the rest density)
// keep the count.
__device__ __forceinline__ uint32_t rank_in_cell(const uint32_t *__restrict__ tmp, uint32_t b, uint32_t e,
                                                 uint32_t id)
{
    const uint32_t occ = e - b;
    if (occ > kBigCell && occ <= kBigCellMax) {
        uint32_t lo = b, hi = e;
        while (lo < hi) {
            const uint32_t mid = (lo + hi) >> 1;
            if (tmp[mid] < id) lo = mid + 1;
            else hi = mid;
        }
        return lo - b;
    }
    uint32_t r = 0;
    for (uint32_t k = b; k < e; k++) r += tmp[k] < id ? 1u : 0u;
    return r;
}

}  // namespace sph
