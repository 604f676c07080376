// sph_kernels.cu -- hand-written sm_103a kernels of the SPH grid step.
//
// One step is: scan (cell starts) -> slot + canonical rank + permute (sorted SoA)
// -> density/pressure -> forces + walls + integration + next step's cell hash.
// Semantics follow the reference's CPU simulator (src/CCPUParticleSimulator.cpp:32-229),
// which the OpenCL grid path (resources/kernels/sph_grid.cl, sph_common.cl) approximates;
// where the two differ (the OpenCL walls kernel's (1,1,0) start value, sph_common.cl:68,
// and its float cell hash, sph_grid.cl:31-40) this follows the CPU path.
//
// All kernels are templated on the arithmetic type R: float is the plain form, double
// the FP64 reference run of the same method.
#include <cuda_runtime.h>
#include <stdint.h>

#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {

// ------------------------------------------------------------------------------------
// ingest: host-staged float xyz/vel -> *_u records with scene/id bits, plus the hash.
// Replaces addParticle + the first H2D of updateGrid; ids follow upload order.
template <class R>
__global__ void __launch_bounds__(256) k_ingest(Vec4<R> *__restrict__ pos_u, Vec4<R> *__restrict__ vel_u,
                                                uint2 *__restrict__ cid_u, uint32_t *__restrict__ count,
                                                const SceneDev *__restrict__ scenes,
                                                const uint32_t *__restrict__ scene_off, uint32_t nscenes,
                                                const float *__restrict__ xyz, const float *__restrict__ vel,
                                                uint32_t first, uint32_t n, int32_t fixed_scene, uint32_t id0,
                                                Consts<R> c)
{
    const uint32_t k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= n) return;
    uint32_t s, id;
    if (fixed_scene >= 0) {
        s = (uint32_t) fixed_scene;
        id = id0 + k;
    } else {
        uint32_t lo = 0, hi = nscenes;  // largest s with scene_off[s] <= k
        while (hi - lo > 1) {
            const uint32_t mid = (lo + hi) >> 1;
            if (__ldg(scene_off + mid) <= k) lo = mid;
            else hi = mid;
        }
        s = lo;
        id = k - __ldg(scene_off + s);
    }
    const SceneDev sc = load_scene(scenes, s);
    const R x = (R) xyz[3 * k], y = (R) xyz[3 * k + 1], z = (R) xyz[3 * k + 2];
    R vx = 0, vy = 0, vz = 0;
    if (vel) {
        vx = (R) vel[3 * k];
        vy = (R) vel[3 * k + 1];
        vz = (R) vel[3 * k + 2];
    }
    int cx, cy, cz;
    const uint32_t cell = hash_cell<R>(sc, x, y, z, c, cx, cy, cz);
    count_add(count, c.gsum, cell);
    const uint32_t i = first + k;
    st4(pos_u + i, Vec4<R>{x, y, z, mkw<R>(s)});
    st4(vel_u + i, Vec4<R>{vx, vy, vz, mkw<R>(id)});
    cid_u[i] = make_uint2(cell, id);
}

// ------------------------------------------------------------------------------------
// Exclusive scan of the per-cell counts into cell starts: each tile's offset is the sum of the
// group sums before it (every hash adds to its cell's group beside the cell, so no pass over
// the counts precedes this one), then the tile scans itself.
// Replaces scan_local / increment_local_scans (resources/kernels/sph_grid.cl:71-121, 9-23)
// and its sums-buffer race. The counts are left as they are: the slot pass takes every slot
// by decrementing its cell's count, which leaves the counts at zero for the next hash; the
// crowded-cell sort clears the group sums.
// A tile is Q groups of 256 x 4 cells: each thread reads one 16-byte group of 4 counts per
// group (coalesced across the block) and the groups are scanned one after another. Q = 1 (1024
// cells) gives enough blocks to fill the GPU on grids of a few hundred thousand cells; grids of
// millions of cells (cells of h/2) take Q = 4, four 16-byte loads in flight per thread.
constexpr int SCAN_THREADS = 256;
constexpr int SCAN_GROUP = SCAN_THREADS * 4;
constexpr uint32_t kScanLargeGrid = 1u << 21;  // cells from which tiles of 4 groups are used
static_assert(SCAN_GROUP == (int) kScanTile, "the scan group and the group-count sizing agree");

// the 4 counts of a thread, 0 beyond ncells; one 16-byte load when the array is 16-byte
// aligned (vec, decided on the host from the pointers), else 4 scalar loads
__device__ __forceinline__ uint4 load_counts4(const uint32_t *__restrict__ count, uint32_t base, uint32_t ncells,
                                             bool vec)
{
    if (vec && base + 4 <= ncells) return __ldg(reinterpret_cast<const uint4 *>(count + base));
    if (base + 4 <= ncells) return make_uint4(count[base], count[base + 1], count[base + 2], count[base + 3]);
    uint4 v = make_uint4(0, 0, 0, 0);
    if (base < ncells) v.x = count[base];
    if (base + 1 < ncells) v.y = count[base + 1];
    if (base + 2 < ncells) v.z = count[base + 2];
    return v;
}

__device__ __forceinline__ uint32_t block_exclusive_scan(uint32_t v, uint32_t &total)
{
    __shared__ uint32_t warp_tot[SCAN_THREADS / 32];
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    uint32_t x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const uint32_t y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_tot[wid] = x;
    __syncthreads();
    if (wid == 0) {
        uint32_t t = lane < (SCAN_THREADS / 32) ? warp_tot[lane] : 0;
        uint32_t u = t;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, u, o);
            if (lane >= o) u += y;
        }
        if (lane < (SCAN_THREADS / 32)) warp_tot[lane] = u - t;  // exclusive warp offsets
    }
    __syncthreads();
    const uint32_t excl = warp_tot[wid] + x - v;
    // block total: last warp's exclusive offset + its inclusive sum
    __shared__ uint32_t tot;
    if (threadIdx.x == SCAN_THREADS - 1) tot = excl + v;
    __syncthreads();
    total = tot;
    __syncthreads();
    return excl;
}

template <int Q>
__global__ void __launch_bounds__(SCAN_THREADS) k_scan_apply(const uint32_t *__restrict__ count, uint32_t ncells,
                                                             const uint32_t *__restrict__ gsum,
                                                             uint32_t *__restrict__ start, bool vec,
                                                             uint32_t *__restrict__ big)
{
    chain_wait();
    uint4 c4[Q];
#pragma unroll
    for (int q = 0; q < Q; q++)
        c4[q] = load_counts4(count, (blockIdx.x * Q + q) * SCAN_GROUP + threadIdx.x * 4, ncells, vec);
    // this tile's offset: the sum of the earlier groups' counts (ncells / 1024 words at most,
    // read by every block, so held in L1 and L2)
    __shared__ uint32_t off_w[SCAN_THREADS / 32];
    uint32_t part = 0;
    for (uint32_t t = threadIdx.x; t < blockIdx.x * Q; t += SCAN_THREADS) part += __ldg(gsum + t);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) part += __shfl_xor_sync(0xffffffffu, part, o);
    if ((threadIdx.x & 31) == 0) off_w[threadIdx.x >> 5] = part;
    __syncthreads();
    uint32_t off = 0;
#pragma unroll
    for (int w = 0; w < SCAN_THREADS / 32; w++) off += off_w[w];
#pragma unroll
    for (int q = 0; q < Q; q++) {  // the groups in order, each offset by the ones before it
        const uint4 c = c4[q];
        const uint32_t base = (blockIdx.x * Q + q) * SCAN_GROUP + threadIdx.x * 4;
        uint32_t total;
        const uint32_t run = block_exclusive_scan(c.x + c.y + c.z + c.w, total) + off;
        off += total;
        const uint4 st4v = make_uint4(run, run + c.x, run + c.x + c.y, run + c.x + c.y + c.z);
        if (big) {  // cells above kBigCell particles get their slot ids sorted before the rank
            const uint32_t cv[4] = {c.x, c.y, c.z, c.w};
#pragma unroll
            for (int k = 0; k < 4; k++)
                if (cv[k] > kBigCell) big[1 + atomicAdd(big, 1u)] = base + (uint32_t) k;
        }
        if (vec && base + 4 <= ncells) {
            *reinterpret_cast<uint4 *>(start + base) = st4v;
        } else {
            const uint32_t sv[4] = {st4v.x, st4v.y, st4v.z, st4v.w};
            for (uint32_t k = 0; k < 4 && base + k < ncells; k++) start[base + k] = sv[k];
        }
    }
    if (blockIdx.x == gridDim.x - 1 && threadIdx.x == 0) start[ncells] = off;
}

// ------------------------------------------------------------------------------------
// Canonical counting sort: every particle takes a slot in its cell (arbitrary order),
// then its final position is the cell start plus the number of same-cell particles with
// a smaller id. The resulting order is ascending (cell, id) regardless of atomic order;
// the reference leaves the within-cell order unspecified (host std::sort,
// src/CGPUParticleSimulator.cpp:116-139; swap-remove lists, src/CCPUParticleSimulator.cpp:72-84).
// Slots are taken from the top of each cell down: the count still unclaimed in a cell is the
// end of its free slots, and the last slot taken returns the count to zero for the next hash.
// The kernel is bound by the latency of its load -> atomic -> store chain, not by its bytes, so
// each thread carries P particles, one from each of its block's P consecutive tiles of 256 (a
// warp still covers 32 consecutive particles per tile), and the P chains overlap.
constexpr int SLOT_PER = 4;
constexpr uint32_t kNoCell = 0xffffffffu;  // match key of lanes past n (no cell reaches 2^31)

template <int P>
__global__ void __launch_bounds__(256) k_slot(const uint2 *__restrict__ cid_u, uint32_t n,
                                              const uint32_t *__restrict__ start, uint32_t *__restrict__ count,
                                              uint32_t *__restrict__ tmp)
{
    chain_wait();
    const unsigned lane = threadIdx.x & 31u;
    uint2 cd[P];
#pragma unroll
    for (int k = 0; k < P; k++) {
        const uint32_t i = (blockIdx.x * P + k) * 256u + threadIdx.x;
        cd[k] = i < n ? cid_u[i] : make_uint2(kNoCell, 0);
    }
    // consecutive particles mostly share a cell: one atomic per cell and warp, each lane taking
    // its rank among the warp's lanes of that cell (the slot order is arbitrary anyway)
    unsigned peers[P];
    uint32_t left[P], first[P];
#pragma unroll
    for (int k = 0; k < P; k++) {
        peers[k] = __match_any_sync(0xffffffffu, cd[k].x);
        left[k] = 0;
        first[k] = 0;
        if (cd[k].x != kNoCell && (int) lane == __ffs(peers[k]) - 1) {
            left[k] = atomicSub(count + cd[k].x, (uint32_t) __popc(peers[k]));  // slots left-take .. left-1
            first[k] = __ldg(start + cd[k].x);
        }
    }
#pragma unroll
    for (int k = 0; k < P; k++) {
        const uint32_t base = __shfl_sync(0xffffffffu, first[k] + left[k] - (uint32_t) __popc(peers[k]),
                                          __ffs(peers[k]) - 1);
        const uint32_t t = base + (uint32_t) __popc(peers[k] & ((1u << lane) - 1u));
        if (cd[k].x != kNoCell && sph_check(t < n, CHK_SORT)) tmp[t] = cd[k].y;
    }
}

// Slot ids of the listed big cells sorted ascending in place (one block per cell at a time,
// bitonic sort in shared memory over the cell's ids padded to a power of two). Cells above
// kBigCellMax are left as they are: rank_in_cell counts them.
constexpr int SORT_THREADS = 256;

__global__ void __launch_bounds__(SORT_THREADS) k_sort_big(const uint32_t *__restrict__ start, uint32_t *__restrict__ tmp,
                                                           const uint32_t *__restrict__ big,
                                                           uint32_t *__restrict__ gsum, uint32_t ngroups)
{
    __shared__ uint32_t sk[kBigCellMax];
    chain_wait();
    // the scan has read the group sums: zero for the next hash
    for (uint32_t t = blockIdx.x * SORT_THREADS + threadIdx.x; t < ngroups; t += gridDim.x * SORT_THREADS) gsum[t] = 0;
    const uint32_t nbig = big[0];
    for (uint32_t q = blockIdx.x; q < nbig; q += gridDim.x) {
        const uint32_t cell = big[1 + q];
        const uint32_t b = start[cell], e = start[cell + 1], occ = e - b;
        if (occ <= kBigCell || occ > kBigCellMax) continue;
        uint32_t P = 2 * kBigCell;
        while (P < occ) P <<= 1;
        for (uint32_t t = threadIdx.x; t < P; t += SORT_THREADS) sk[t] = t < occ ? tmp[b + t] : 0xffffffffu;
        __syncthreads();
        for (uint32_t k = 2; k <= P; k <<= 1) {
            for (uint32_t j = k >> 1; j > 0; j >>= 1) {
                for (uint32_t t = threadIdx.x; t < P / 2; t += SORT_THREADS) {
                    const uint32_t lo = 2 * j * (t / j) + (t % j), hi = lo + j;  // lo has bit j clear
                    const uint32_t x = sk[lo], y = sk[hi];
                    if ((x > y) == ((lo & k) == 0)) {
                        sk[lo] = y;
                        sk[hi] = x;
                    }
                }
                __syncthreads();
            }
        }
        for (uint32_t t = threadIdx.x; t < occ; t += SORT_THREADS) tmp[b + t] = sk[t];
        __syncthreads();
    }
}

// One particle per thread here (more per thread measured slower: the rank loop's registers cost
// more occupancy than the overlap gains); the state loads are issued before the rank is counted.
template <class R>
__global__ void __launch_bounds__(256) k_rank_permute(const uint2 *__restrict__ cid_u, uint32_t n,
                                                      const uint32_t *__restrict__ start,
                                                      const uint32_t *__restrict__ tmp,
                                                      const Vec4<R> *__restrict__ pos_u,
                                                      const Vec4<R> *__restrict__ vel_u,
                                                      Vec4<R> *__restrict__ pos_s, Vec4<R> *__restrict__ vel_s,
                                                      uint32_t *__restrict__ big)
{
    chain_wait();
    if (blockIdx.x == 0 && threadIdx.x == 0) big[0] = 0;  // the crowded-cell list is used: empty for the next scan
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint2 cd = cid_u[i];
    const Vec4<R> p = ld4(pos_u + i), v = ld4(vel_u + i);
    const uint32_t b = start[cd.x], e = start[cd.x + 1];
    if (!sph_check(b <= e && e <= n, CHK_SORT)) return;
    const uint32_t dst = b + rank_in_cell(tmp, b, e, cd.y);
    if (!sph_check(dst < e, CHK_SORT)) return;
    st4(pos_s + dst, p);
    st4(vel_s + dst, v);
}

// ------------------------------------------------------------------------------------
// Neighbour walk: the 27 cells around a particle are 9 rows (dy, dz) of 3 cells along x,
// and in (cell, id) order each row is one contiguous range of the sorted arrays.
template <class R, class F>
__device__ __forceinline__ void for_each_row(const SceneDev &sc, const uint32_t *__restrict__ start, int cx, int cy,
                                             int cz, F &&f)
{
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx > 0 ? cx - 1 : 0;
    const int xh = cx + 1 < X ? cx + 1 : X - 1;
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
        const int z = cz + dz;
        if (z < 0 || z >= Z) continue;
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++) {
            const int y = cy + dy;
            if (y < 0 || y >= Y) continue;
            const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
            const uint32_t jb = __ldg(start + row + xl);
            const uint32_t je = __ldg(start + row + xh + 1);
            f(jb, je);
        }
    }
}

// Density and pressure (src/CCPUParticleSimulator.cpp:93-141): rho = m * poly6 * sum (h^2-r^2)^3
// over r^2 <= h^2, self included; p = k (rho - rho0). Also stores c_spiky p / rho^2 and
// c_visc / rho, the two per-neighbour factors of the force pass (aux_record).
template <class R>
__global__ void __launch_bounds__(256) k_density(const Vec4<R> *__restrict__ pos, Vec4<R> *__restrict__ aux,
                                                 const uint32_t *__restrict__ start,
                                                 const SceneDev *__restrict__ scenes, uint32_t n, Consts<R> c)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    R acc = 0;
    const R h2 = c.h2;
    for_each_row<R>(sc, start, cx, cy, cz, [&](uint32_t jb, uint32_t je) {
#pragma unroll 4
        for (uint32_t j = jb; j < je; j++) {
            const Vec4<R> pj = ld4(pos + j);
            acc = poly6_add<R>(acc, pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2);
        }
    });
    const R rho = rmul(rmul(acc, c.c_poly6), c.mass);
    const R p = rmul(c.k, rsub(rho, c.rho0));
    st4(aux + i, aux_record<R>(rho, p, c));
}

// Forces, first form: one thread per sorted particle, the pair terms evaluated inside the
// candidate loop.
template <class R>
__global__ void __launch_bounds__(256) k_forces(const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                                const Vec4<R> *__restrict__ aux, const uint32_t *__restrict__ start,
                                                const SceneDev *__restrict__ scenes,
                                                const ObstacleDev *__restrict__ obstacles, uint32_t n, Consts<R> c,
                                                Vec4<R> *__restrict__ pos_out, Vec4<R> *__restrict__ vel_out,
                                                Vec4<R> *__restrict__ acc_out, uint2 *__restrict__ cid_out,
                                                uint32_t *__restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const Vec4<R> vi = ld4(vel + i);
    const Vec4<R> ai = ld4(aux + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const R h2 = c.h2, qi = ai.z;
    R fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    for_each_row<R>(sc, start, cx, cy, cz, [&](uint32_t jb, uint32_t je) {
#pragma unroll 2
        for (uint32_t j = jb; j < je; j++) {
            const Vec4<R> pj = ld4(pos + j);
            if (h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2) > (R) 0 && j != i)
                pair_force<R>(pi, vi, qi, j, pos, vel, aux, c, fpx, fpy, fpz, fvx, fvy, fvz);
        }
    });
    finish_particle<R>(i, pi, vi, ai.x, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, pos_out, vel_out, acc_out,
                       cid_out, count);
}

// Forces, compacted form: the candidate scan only tests distances and appends accepted
// neighbours to a per-thread list in shared memory (column-major, so a warp's appends hit
// distinct banks); the pair terms then run over the list with every lane busy. A full
// list is drained in place, so any neighbour count is handled.
template <class R, int CAP, int BLOCK>
__global__ void __launch_bounds__(BLOCK) k_forces_list(
    const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel, const Vec4<R> *__restrict__ aux,
    const uint32_t *__restrict__ start, const SceneDev *__restrict__ scenes, const ObstacleDev *__restrict__ obstacles,
    uint32_t n, Consts<R> c, Vec4<R> *__restrict__ pos_out, Vec4<R> *__restrict__ vel_out,
    Vec4<R> *__restrict__ acc_out, uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    __shared__ uint32_t list[CAP][BLOCK];
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const Vec4<R> vi = ld4(vel + i);
    const Vec4<R> ai = ld4(aux + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const R h2 = c.h2, qi = ai.z;
    R fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    int cnt = 0;
    auto drain = [&]() {
        for (int k = 0; k < cnt; k++)
            pair_force<R>(pi, vi, qi, list[k][threadIdx.x], pos, vel, aux, c, fpx, fpy, fpz, fvx, fvy, fvz);
        cnt = 0;
    };
    for_each_row<R>(sc, start, cx, cy, cz, [&](uint32_t jb, uint32_t je) {
        // chunks of at most CAP candidates; the list is drained between chunks when the
        // next chunk might not fit, so it never overflows inside the candidate loop
        for (uint32_t cb = jb; cb < je; cb += CAP) {
            const uint32_t ce = min(je, cb + (uint32_t) CAP);
            if (cnt + (int) (ce - cb) > CAP) drain();
#pragma unroll 4
            for (uint32_t j = cb; j < ce; j++) {
                const Vec4<R> pj = ld4(pos + j);
                if (h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2) > (R) 0 && j != i)
                    list[cnt++][threadIdx.x] = j;
            }
        }
    });
    drain();
    finish_particle<R>(i, pi, vi, ai.x, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, pos_out, vel_out, acc_out,
                       cid_out, count);
}

// ------------------------------------------------------------------------------------
// Neighbour masks: the density pass already tests every candidate, so it records which ones
// it accepted. For each particle and each row of its stencil, the row's candidate window
// [start of cell x-RAD, end of cell x+RAD) is cut into 32-candidate chunks; chunk w of row r is
// one 32-bit word at masks[(r * WORDS + w) * n + i] (coalesced across particles). Bit k
// set = candidate window_start + 32 w + k is a neighbour (self included). Candidates past
// WORDS chunks are not recorded: the force pass tests them itself. RAD = 1 is the reference's
// 27 cells of size h; RAD = 2 walks 125 cells of size h/2 (42% less volume than 27 h^3).

template <class R, bool REC, int RAD = 1>
__global__ void __launch_bounds__(256) k_density_mask(const Vec4<R> *__restrict__ pos, Vec4<R> *__restrict__ aux,
                                                      const uint32_t *__restrict__ start,
                                                      const SceneDev *__restrict__ scenes, uint32_t n, Consts<R> c,
                                                      uint32_t *__restrict__ masks, const Vec4<R> *__restrict__ vel,
                                                      Vec4<R> *__restrict__ frec)
{
    using St = Stencil<RAD>;
    chain_wait();
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const R h2 = c.h2;
    R acc = 0;
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
                // bit k of the chunk's word = candidate cb + k; bits enter at the top and
                // move down one place per candidate
                const uint32_t ce = min(je, cb + 32u);
                uint32_t m = 0;
#pragma unroll 4
                for (uint32_t j = cb; j < ce; j++) {
                    const Vec4<R> pj = ld4(pos + j);
                    const R t = h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2);
                    m = (m >> 1) | (t > (R) 0 ? 0x80000000u : 0u);
                    acc = poly6_acc<R>(acc, t);
                }
                m >>= 32 - (ce - cb);
                if (w < St::WORDS) st_keep(masks + (size_t) (r * St::WORDS + w) * n + i, m, keep);
            }
        }
    }
    const R rho = rmul(rmul(acc, c.c_poly6), c.mass);
    const R p = rmul(c.k, rsub(rho, c.rho0));
    const Vec4<R> ar = aux_record<R>(rho, p, c);
    const R q = ar.z, inv = ar.w;
    st4(aux + i, ar);
    if (REC) {  // the force pass's view of this particle as a neighbour, in one 2 x 16-byte record
        const Vec4<R> vi = ld4(vel + i);
        st4_keep(frec + 2 * (size_t) i, Vec4<R>{pi.x, pi.y, pi.z, q}, keep);
        st4_keep(frec + 2 * (size_t) i + 1, Vec4<R>{vi.x, vi.y, vi.z, inv}, keep);
    }
}

// Forces driven by the density pass's masks: only accepted neighbours are visited, in the
// same candidate order as the scanning forms (so the sums are bit-identical).
template <class R, int MINB, bool REC>
__global__ void __launch_bounds__(256, MINB) k_forces_mask(
    const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel, const Vec4<R> *__restrict__ aux,
    const uint32_t *__restrict__ start, const SceneDev *__restrict__ scenes, const ObstacleDev *__restrict__ obstacles,
    uint32_t n, Consts<R> c, const uint32_t *__restrict__ masks, const Vec4<R> *__restrict__ frec,
    Vec4<R> *__restrict__ pos_out, Vec4<R> *__restrict__ vel_out, Vec4<R> *__restrict__ acc_out,
    uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const Vec4<R> vi = ld4(vel + i);
    const Vec4<R> ai = ld4(aux + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const R h2 = c.h2, qi = ai.z;
    R fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
    const int xl = cx > 0 ? cx - 1 : 0, xh = cx + 1 < X ? cx + 1 : X - 1;
#pragma unroll 1
    for (int dz = -1; dz <= 1; dz++) {
#pragma unroll 1
        for (int dy = -1; dy <= 1; dy++) {
            const int r = (dz + 1) * 3 + (dy + 1);
            const int z = cz + dz, y = cy + dy;
            if (z < 0 || z >= Z || y < 0 || y >= Y) continue;
            const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
            const uint32_t jb = __ldg(start + row + xl), je = __ldg(start + row + xh + 1);
            if (!sph_check(jb <= je && je <= n, CHK_ROW)) continue;
            const uint32_t nw = (je - jb + 31) / 32;
            for (uint32_t w = 0; w < nw; w++) {
                const uint32_t cb = jb + 32 * w;
                uint32_t m = 0;
                if (w < (uint32_t) Stencil<1>::WORDS) {
                    m = __ldg(masks + (size_t) (r * Stencil<1>::WORDS + w) * n + i);
                } else {  // beyond the recorded chunks: test the candidates here
                    const uint32_t ce = min(je, cb + 32u);
                    for (uint32_t j = ce; j-- > cb;) {
                        const Vec4<R> pj = ld4(pos + j);
                        m = (m << 1) | (h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2) > (R) 0 ? 1u : 0u);
                    }
                }
                while (m) {
                    const uint32_t j = cb + (uint32_t) (__ffs(m) - 1);
                    m &= m - 1;
                    if (j == i || !sph_check(j < je, CHK_NEIGHBOUR)) continue;
                    if (REC) {
                        const Vec4<R> pj = ld4(frec + 2 * (size_t) j), vj = ld4(frec + 2 * (size_t) j + 1);
                        pair_terms<R>(pi, vi, qi, pj, vj, pj.w, vj.w, c, fpx, fpy, fpz, fvx, fvy, fvz);
                    } else {
                        pair_force<R>(pi, vi, qi, j, pos, vel, aux, c, fpx, fpy, fpz, fvx, fvy, fvz);
                    }
                }
            }
        }
    }
    finish_particle<R>(i, pi, vi, ai.x, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, pos_out, vel_out, acc_out,
                       cid_out, count);
}

// Forces from the masks, two accepted neighbours per iteration: both neighbours' records are
// loaded before either's terms are added, so two gathers are in flight at once and the loop
// overhead is paid once per pair. The terms are still added one neighbour at a time in
// candidate order (the sums are the same bits as the other forms of the same cell multiple).
template <class R, int MINB, bool REC, int BLOCK = 256, int RAD = 1>
__global__ void __launch_bounds__(BLOCK, MINB) k_forces_mask2(
    const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel, const Vec4<R> *__restrict__ aux,
    const uint32_t *__restrict__ start, const SceneDev *__restrict__ scenes, const ObstacleDev *__restrict__ obstacles,
    uint32_t n, Consts<R> c, const uint32_t *__restrict__ masks, const Vec4<R> *__restrict__ frec,
    Vec4<R> *__restrict__ pos_out, Vec4<R> *__restrict__ vel_out, Vec4<R> *__restrict__ acc_out,
    uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    using St = Stencil<RAD>;
    chain_wait();
    const uint32_t i = blockIdx.x * BLOCK + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const Vec4<R> vi = ld4(vel + i);
    const Vec4<R> ai = ld4(aux + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    int cx, cy, cz;
    hash_cell<R>(sc, pi.x, pi.y, pi.z, c, cx, cy, cz);
    const R h2 = c.h2, qi = ai.z;
    R fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
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
                        const Vec4<R> pj = ld4(pos + j);
                        m = (m << 1) | (h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2) > (R) 0 ? 1u : 0u);
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
                    Vec4<R> p0, v0, p1, v1;
                    R q0, inv0, q1, inv1;
                    if (REC) {
                        p0 = ld4(frec + 2 * (size_t) j0);
                        v0 = ld4(frec + 2 * (size_t) j0 + 1);
                        p1 = ld4(frec + 2 * (size_t) j1);
                        v1 = ld4(frec + 2 * (size_t) j1 + 1);
                        q0 = p0.w, inv0 = v0.w, q1 = p1.w, inv1 = v1.w;
                    } else {
                        p0 = ld4(pos + j0), v0 = ld4(vel + j0);
                        p1 = ld4(pos + j1), v1 = ld4(vel + j1);
                        ld_qinv(aux + j0, q0, inv0);
                        ld_qinv(aux + j1, q1, inv1);
                    }
                    pair_terms<R>(pi, vi, qi, p0, v0, q0, inv0, c, fpx, fpy, fpz, fvx, fvy, fvz);
                    if (two) pair_terms<R>(pi, vi, qi, p1, v1, q1, inv1, c, fpx, fpy, fpz, fvx, fvy, fvz);
                }
            }
        }
    }
    // the scene record again rather than kept live across the pair loop (fewer registers)
    const SceneDev sc2 = load_scene(scenes, wbits(pi.w));
    finish_particle<R>(i, pi, vi, ai.x, sc2, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, pos_out, vel_out, acc_out,
                       cid_out, count);
}

// All-pairs forms, the reference's brute-force simulator (sph_brute.cl:9-57) restated: every
// particle of the scene is a candidate, visited in the sorted (cell, id) order. The neighbours
// accepted by the grid forms are exactly the candidates within h, and the sorted order visits
// them in the grid forms' candidate order, so both forms sum the same terms in the same order
// and give the same bits: an independent check of the grid build and the cell windows.
template <class R>
__device__ __forceinline__ void scene_range(const SceneDev &sc, const uint32_t *__restrict__ start, uint32_t &jb,
                                            uint32_t &je)
{
    jb = __ldg(start + sc.cell_base);
    je = __ldg(start + sc.cell_base + (uint32_t) sc.res[0] * (uint32_t) sc.res[1] * (uint32_t) sc.res[2]);
}

template <class R>
__global__ void __launch_bounds__(256) k_density_all(const Vec4<R> *__restrict__ pos, Vec4<R> *__restrict__ aux,
                                                     const uint32_t *__restrict__ start,
                                                     const SceneDev *__restrict__ scenes, uint32_t n, Consts<R> c)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    uint32_t jb, je;
    scene_range<R>(sc, start, jb, je);
    R acc = 0;
    const R h2 = c.h2;
#pragma unroll 4
    for (uint32_t j = jb; j < je; j++) {
        const Vec4<R> pj = ld4(pos + j);
        acc = poly6_add<R>(acc, pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2);
    }
    const R rho = rmul(rmul(acc, c.c_poly6), c.mass);
    const R p = rmul(c.k, rsub(rho, c.rho0));
    st4(aux + i, aux_record<R>(rho, p, c));
}

template <class R>
__global__ void __launch_bounds__(256) k_forces_all(const Vec4<R> *__restrict__ pos, const Vec4<R> *__restrict__ vel,
                                                    const Vec4<R> *__restrict__ aux,
                                                    const uint32_t *__restrict__ start,
                                                    const SceneDev *__restrict__ scenes,
                                                    const ObstacleDev *__restrict__ obstacles, uint32_t n,
                                                    Consts<R> c, Vec4<R> *__restrict__ pos_out,
                                                    Vec4<R> *__restrict__ vel_out, Vec4<R> *__restrict__ acc_out,
                                                    uint2 *__restrict__ cid_out, uint32_t *__restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> pi = ld4(pos + i);
    const Vec4<R> vi = ld4(vel + i);
    const Vec4<R> ai = ld4(aux + i);
    const SceneDev sc = load_scene(scenes, wbits(pi.w));
    uint32_t jb, je;
    scene_range<R>(sc, start, jb, je);
    const R h2 = c.h2, qi = ai.z;
    R fpx = 0, fpy = 0, fpz = 0, fvx = 0, fvy = 0, fvz = 0;
    for (uint32_t j = jb; j < je; j++) {
        const Vec4<R> pj = ld4(pos + j);
        if (j != i && h2_minus_r2<R>(pi.x - pj.x, pi.y - pj.y, pi.z - pj.z, h2) > (R) 0) {
            const Vec4<R> vj = ld4(vel + j);
            R qj, invj;
            ld_qinv(aux + j, qj, invj);
            pair_terms<R>(pi, vi, qi, pj, vj, qj, invj, c, fpx, fpy, fpz, fvx, fvy, fvz);
        }
    }
    finish_particle<R>(i, pi, vi, ai.x, sc, obstacles, c, fpx, fpy, fpz, fvx, fvy, fvz, pos_out, vel_out, acc_out,
                       cid_out, count);
}

// Density, blocked form: each thread owns P consecutive sorted particles. When they share a
// scene and a (y, z) row of cells (nearly always in sorted order) one candidate scan over the
// union x-range serves all of them: a candidate outside a particle's own 3 x 3 x 3 block is
// farther than h (cells are h wide and the clamp only moves particles outward), so the
// r^2 test alone selects the same neighbours. The test is branchless: t = h^2 - r^2
// clamped at 0 contributes t^3.
template <class R, int P>
__global__ void __launch_bounds__(256) k_density_blk(const Vec4<R> *__restrict__ pos, Vec4<R> *__restrict__ aux,
                                                     const uint32_t *__restrict__ start,
                                                     const SceneDev *__restrict__ scenes, uint32_t n, Consts<R> c)
{
    const uint32_t i0 = (blockIdx.x * blockDim.x + threadIdx.x) * P;
    if (i0 >= n) return;
    R px[P], py[P], pz[P], acc[P];
    int cxs[P];
    const Vec4<R> p0 = ld4(pos + i0);
    const uint32_t s0 = wbits(p0.w);
    const SceneDev sc = load_scene(scenes, s0);
    int cy0, cz0;
    bool same = true;
#pragma unroll
    for (int p = 0; p < P; p++) {
        const uint32_t i = i0 + p;
        acc[p] = 0;
        Vec4<R> q = p0;
        if (p > 0 && i < n) q = ld4(pos + i);
        px[p] = q.x; py[p] = q.y; pz[p] = q.z;
        if (p > 0 && i >= n) { px[p] = py[p] = pz[p] = (R) 1e30; cxs[p] = cxs[0]; continue; }
        int cx, cy, cz;
        if (p == 0 || wbits(q.w) == s0) {
            hash_cell<R>(sc, q.x, q.y, q.z, c, cx, cy, cz);
            if (p == 0) { cy0 = cy; cz0 = cz; }
            else same = same && cy == cy0 && cz == cz0;
        } else {
            same = false;
            cx = 0;
        }
        cxs[p] = cx;
    }
    const R h2 = c.h2;
    if (same) {
        int lo = cxs[0], hi = cxs[0];
#pragma unroll
        for (int p = 1; p < P; p++) { lo = min(lo, cxs[p]); hi = max(hi, cxs[p]); }
        const int X = sc.res[0], Y = sc.res[1], Z = sc.res[2];
        const int xl = lo > 0 ? lo - 1 : 0, xh = hi + 1 < X ? hi + 1 : X - 1;
#pragma unroll 1
        for (int dz = -1; dz <= 1; dz++) {
            const int z = cz0 + dz;
            if (z < 0 || z >= Z) continue;
#pragma unroll 1
            for (int dy = -1; dy <= 1; dy++) {
                const int y = cy0 + dy;
                if (y < 0 || y >= Y) continue;
                const uint32_t row = sc.cell_base + (uint32_t) y * (uint32_t) X + (uint32_t) z * (uint32_t) X * (uint32_t) Y;
                const uint32_t jb = __ldg(start + row + xl), je = __ldg(start + row + xh + 1);
#pragma unroll 2
                for (uint32_t j = jb; j < je; j++) {
                    const Vec4<R> pj = ld4(pos + j);
#pragma unroll
                    for (int p = 0; p < P; p++) acc[p] = poly6_add<R>(acc[p], px[p] - pj.x, py[p] - pj.y, pz[p] - pj.z, h2);
                }
            }
        }
    } else {
        // particles of different rows or scenes: one walk each
#pragma unroll
        for (int p = 0; p < P; p++) {
            const uint32_t i = i0 + p;
            if (i >= n) continue;
            const Vec4<R> q = ld4(pos + i);
            const SceneDev sq = load_scene(scenes, wbits(q.w));
            int cx, cy, cz;
            hash_cell<R>(sq, q.x, q.y, q.z, c, cx, cy, cz);
            R a = 0;
            for_each_row<R>(sq, start, cx, cy, cz, [&](uint32_t jb, uint32_t je) {
                for (uint32_t j = jb; j < je; j++) {
                    const Vec4<R> pj = ld4(pos + j);
                    a = poly6_add<R>(a, q.x - pj.x, q.y - pj.y, q.z - pj.z, h2);
                }
            });
            acc[p] = a;
        }
    }
#pragma unroll
    for (int p = 0; p < P; p++) {
        const uint32_t i = i0 + p;
        if (i >= n) continue;
        const R rho = rmul(rmul(acc[p], c.c_poly6), c.mass);
        const R pr = rmul(c.k, rsub(rho, c.rho0));
        st4(aux + i, aux_record<R>(rho, pr, c));
    }
}

// ------------------------------------------------------------------------------------
// rehash: the (cell, id) of every *_u particle again, its cell in the step grid (after the grid's
// cell multiple changed, or after the *_u arrays were refilled); the counts must have been zeroed.
template <class R>
__global__ void __launch_bounds__(256) k_rehash(const Vec4<R> *__restrict__ pos_u, const Vec4<R> *__restrict__ vel_u,
                                                uint2 *__restrict__ cid_u, uint32_t *__restrict__ count,
                                                const SceneDev *__restrict__ scenes, uint32_t n, Consts<R> c)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Vec4<R> p = ldc4(pos_u + i);
    const SceneDev sc = load_scene(scenes, wbits(p.w));
    int cx, cy, cz;
    const uint32_t cell = hash_cell<R>(sc, p.x, p.y, p.z, c, cx, cy, cz);
    count_add(count, c.gsum, cell);
    cid_u[i] = make_uint2(cell, wbits(ldc4(vel_u + i).w));
}

// ------------------------------------------------------------------------------------
// egress: any layout -> id-ordered, scene-major staging arrays for one D2H copy each.
template <class R>
__global__ void __launch_bounds__(256) k_egress(const Vec4<R> *__restrict__ posL, const Vec4<R> *__restrict__ velL,
                                                const Vec4<R> *__restrict__ posA, const Vec4<R> *__restrict__ velA,
                                                const Vec4<R> *__restrict__ aux, const Vec4<R> *__restrict__ pos_u,
                                                const Vec4<R> *__restrict__ vel_u, const Vec4<R> *__restrict__ acc,
                                                const uint32_t *__restrict__ scene_off, uint32_t n_state,
                                                uint32_t n_aux, uint32_t n_acc, R *xyz, R *v, R *rho, R *p, R *a)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n_state) {
        const Vec4<R> pp = ldc4(posL + i), vv = ldc4(velL + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        if (!sph_check(o < n_state, CHK_EGRESS)) return;
        xyz[3 * o] = pp.x; xyz[3 * o + 1] = pp.y; xyz[3 * o + 2] = pp.z;
        v[3 * o] = vv.x; v[3 * o + 1] = vv.y; v[3 * o + 2] = vv.z;
    }
    if (i < n_aux) {
        const Vec4<R> pp = ldc4(posA + i), vv = ldc4(velA + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        const Vec4<R> ax = ldc4(aux + i);
        rho[o] = ax.x;
        p[o] = ax.y;
    }
    if (acc && i < n_acc) {
        const Vec4<R> pp = ldc4(pos_u + i), vv = ldc4(vel_u + i);
        const uint32_t o = __ldg(scene_off + wbits(pp.w)) + wbits(vv.w);
        const Vec4<R> aa = ldc4(acc + i);
        a[3 * o] = aa.x; a[3 * o + 1] = aa.y; a[3 * o + 2] = aa.z;
    }
}

// FP64 reductions per scene in fixed order (deterministic): STATS_SPLIT blocks per scene
// each reduce a fixed slice of the scene's contiguous range into a partial record, then one
// block per scene adds the partials in slice order. Mass, momentum, kinetic energy, mean and
// max density.
constexpr int STATS_SPLIT = 64;
constexpr int STATS_THREADS = 256;

template <class R>
__global__ void __launch_bounds__(STATS_THREADS) k_stats_partial(const Vec4<R> *__restrict__ vel,
                                                                 const Vec4<R> *__restrict__ aux,
                                                                 const uint32_t *__restrict__ start,
                                                                 const SceneDev *__restrict__ scenes,
                                                                 double *__restrict__ partial)
{
    const uint32_t s = blockIdx.x / STATS_SPLIT, part = blockIdx.x % STATS_SPLIT;
    const SceneDev sc = load_scene(scenes, s);
    const uint32_t b = start[sc.cell_base], e = start[sc.cell_base + sc.ncells];
    const uint32_t len = e - b, chunk = (len + STATS_SPLIT - 1) / STATS_SPLIT;
    const uint32_t lo = b + part * chunk, hi = min(e, lo + chunk);
    double mx = 0, my = 0, mz = 0, ke = 0, rs = 0, rmax = -1e300;
    for (uint32_t i = lo + threadIdx.x; i < hi; i += STATS_THREADS) {
        const Vec4<R> v = ldc4(vel + i);
        const Vec4<R> a = ldc4(aux + i);
        const double vx = (double) v.x, vy = (double) v.y, vz = (double) v.z;
        mx += vx; my += vy; mz += vz;
        ke += vx * vx + vy * vy + vz * vz;
        rs += (double) a.x;
        rmax = fmax(rmax, (double) a.x);
    }
    __shared__ double red[6][STATS_THREADS];
    red[0][threadIdx.x] = mx; red[1][threadIdx.x] = my; red[2][threadIdx.x] = mz;
    red[3][threadIdx.x] = ke; red[4][threadIdx.x] = rs; red[5][threadIdx.x] = rmax;
    __syncthreads();
    for (int w = STATS_THREADS / 2; w > 0; w >>= 1) {
        if ((int) threadIdx.x < w) {
#pragma unroll
            for (int k = 0; k < 5; k++) red[k][threadIdx.x] += red[k][threadIdx.x + w];
            red[5][threadIdx.x] = fmax(red[5][threadIdx.x], red[5][threadIdx.x + w]);
        }
        __syncthreads();
    }
    if (threadIdx.x < 6) partial[6 * blockIdx.x + threadIdx.x] = red[threadIdx.x][0];
}

__global__ void k_stats_final(const double *__restrict__ partial, const uint32_t *__restrict__ start,
                              const SceneDev *__restrict__ scenes, double mass, double *__restrict__ out)
{
    const uint32_t s = blockIdx.x;
    if (threadIdx.x != 0) return;
    const SceneDev sc = load_scene(scenes, s);
    const double cnt = (double) (start[sc.cell_base + sc.ncells] - start[sc.cell_base]);
    double t[6] = {0, 0, 0, 0, 0, -1e300};
    for (int k = 0; k < STATS_SPLIT; k++) {
        const double *p = partial + 6 * ((size_t) s * STATS_SPLIT + k);
        for (int q = 0; q < 5; q++) t[q] += p[q];
        t[5] = fmax(t[5], p[5]);
    }
    double *o = out + 8 * s;
    o[0] = mass * cnt;
    o[1] = mass * t[0]; o[2] = mass * t[1]; o[3] = mass * t[2];
    o[4] = 0.5 * mass * t[3];
    o[5] = cnt > 0 ? t[4] / cnt : 0.0;
    o[6] = cnt > 0 ? t[5] : 0.0;
    o[7] = cnt;
}

// ------------------------------------------------------------------------------------
static inline unsigned nblk(uint32_t n, unsigned t) { return (unsigned) ((n + t - 1) / t); }

template <class R>
cudaError_t Launch<R>::ingest(const DevBufs &b, const float *xyz, const float *vel, uint32_t first, uint32_t n,
                              int32_t scene, uint32_t id0, uint32_t nscenes, Consts<R> c, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    k_ingest<R><<<nblk(n, 256), 256, 0, st>>>((Vec4<R> *) b.pos_u, (Vec4<R> *) b.vel_u, b.cid_u, b.count, b.scenes,
                                              b.scene_off, nscenes, xyz, vel, first, n, scene, id0, c);
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::scan(const DevBufs &b, uint32_t ncells, cudaStream_t st)
{
    // 16-byte accesses only where both arrays allow them (a caller's start array may not)
    const bool vec = ((reinterpret_cast<uintptr_t>(b.count) | reinterpret_cast<uintptr_t>(b.start)) & 15u) == 0;
    if (ncells >= kScanLargeGrid) {
        const uint32_t nb = (ncells + 4 * SCAN_GROUP - 1) / (4 * SCAN_GROUP);
        return launch_chained(k_scan_apply<4>, nb, SCAN_THREADS, st, b.count, ncells, b.bsum, b.start, vec, b.big);
    }
    const uint32_t nb = (ncells + SCAN_GROUP - 1) / SCAN_GROUP;
    return launch_chained(k_scan_apply<1>, nb, SCAN_THREADS, st, b.count, ncells, b.bsum, b.start, vec, b.big);
}

template <class R>
cudaError_t Launch<R>::permute(const DevBufs &b, uint32_t n, uint32_t ncells, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    cudaError_t e = launch_slot(b, n, ncells, st);
    if (e != cudaSuccess) return e;
    return launch_chained(k_rank_permute<R>, nblk(n, 256), 256, st, b.cid_u, n, b.start, b.tmp,
                          (const Vec4<R> *) b.pos_u, (const Vec4<R> *) b.vel_u, (Vec4<R> *) b.pos_s,
                          (Vec4<R> *) b.vel_s, b.big);
}

template <class R>
cudaError_t Launch<R>::rehash(const DevBufs &b, uint32_t n, Consts<R> c, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    k_rehash<R><<<nblk(n, 256), 256, 0, st>>>((const Vec4<R> *) b.pos_u, (const Vec4<R> *) b.vel_u, b.cid_u, b.count,
                                              b.scenes, n, c);
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::density(const DevBufs &b, uint32_t n, Consts<R> c, const Tune &t, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const Vec4<R> *pos = (const Vec4<R> *) b.pos_s;
    Vec4<R> *aux = (Vec4<R> *) b.aux;
    if (t.density_p == Tune::ALL_PAIRS) {
        k_density_all<R><<<nblk(n, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c);
        return cudaGetLastError();
    }
    if (t.forces_mode >= 7) {  // masks and force records
        if (t.cell_mult == 2) {
            if constexpr (sizeof(R) == 4)
                return launch_chained(k_density_mask<R, true, 2>, nblk(n, 256), 256, st, pos, aux, b.start, b.scenes,
                                      n, c, b.masks, (const Vec4<R> *) b.vel_s, (Vec4<R> *) b.frec);
            else
                return cudaErrorInvalidValue;  // the FP64 form runs on the reference's grid only
        } else {
            return launch_chained(k_density_mask<R, true, 1>, nblk(n, 256), 256, st, pos, aux, b.start, b.scenes, n,
                                  c, b.masks, (const Vec4<R> *) b.vel_s, (Vec4<R> *) b.frec);
        }
        return cudaGetLastError();
    }
    if (t.cell_mult != 1) return cudaErrorInvalidValue;  // cells of h/2: the record variants only
    if (t.forces_mode >= 3) {  // the mask-driven force passes need the masks
        k_density_mask<R, false><<<nblk(n, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c, b.masks, nullptr,
                                                               nullptr);
        return cudaGetLastError();
    }
    switch (t.density_p) {
    case 2: k_density_blk<R, 2><<<nblk((n + 1) / 2, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c); break;
    case 4: k_density_blk<R, 4><<<nblk((n + 3) / 4, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c); break;
    case 1: k_density_blk<R, 1><<<nblk(n, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c); break;
    default: k_density<R><<<nblk(n, 256), 256, 0, st>>>(pos, aux, b.start, b.scenes, n, c); break;
    }
    return cudaGetLastError();
}

// the record-reading force kernel of one (register budget, block size, stencil) choice
template <class R, int MINB, int BLOCK, int RAD>
static cudaError_t launch_forces_rec(const DevBufs &b, uint32_t n, Consts<R> c, Vec4<R> *ao, cudaStream_t st)
{
    return launch_chained(k_forces_mask2<R, MINB, true, BLOCK, RAD>, nblk(n, BLOCK), BLOCK, st,
                          (const Vec4<R> *) b.pos_s, (const Vec4<R> *) b.vel_s, (const Vec4<R> *) b.aux, b.start,
                          b.scenes, b.obstacles, n, c, b.masks, (const Vec4<R> *) b.frec, (Vec4<R> *) b.pos_u,
                          (Vec4<R> *) b.vel_u, ao, b.cid_u, b.count);
}

template <class R>
cudaError_t Launch<R>::forces(const DevBufs &b, uint32_t n, Consts<R> c, bool record_acc, const Tune &t,
                              cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const Vec4<R> *pos = (const Vec4<R> *) b.pos_s, *vel = (const Vec4<R> *) b.vel_s, *aux = (const Vec4<R> *) b.aux;
    Vec4<R> *po = (Vec4<R> *) b.pos_u, *vo = (Vec4<R> *) b.vel_u, *ao = record_acc ? (Vec4<R> *) b.acc : nullptr;
    if (t.cell_mult == 2) {  // cells of h/2: the record variants 7 to 11 (plain FP32 only)
        if constexpr (sizeof(R) == 4) {
            switch (t.forces_mode) {
            case 7: return launch_forces_rec<R, 1, 256, 2>(b, n, c, ao, st);
            case 8: return launch_forces_rec<R, 5, 256, 2>(b, n, c, ao, st);
            case 9: return launch_forces_rec<R, 6, 256, 2>(b, n, c, ao, st);
            case 10: return launch_forces_rec<R, 12, 128, 2>(b, n, c, ao, st);
            case 11: return launch_forces_rec<R, 10, 128, 2>(b, n, c, ao, st);
            default: return cudaErrorInvalidValue;
            }
        } else {
            return cudaErrorInvalidValue;
        }
    }
    switch (t.forces_mode) {
    case Tune::ALL_PAIRS:
        k_forces_all<R><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n, c, po, vo, ao,
                                                      b.cid_u, b.count);
        break;
    case 3:
        k_forces_mask<R, 0, false><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n,
                                                                 c, b.masks, nullptr, po, vo, ao, b.cid_u, b.count);
        break;
    case 4:
        k_forces_mask<R, 4, false><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n,
                                                                 c, b.masks, nullptr, po, vo, ao, b.cid_u, b.count);
        break;
    case 5:
        k_forces_mask2<R, 4, false><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n,
                                                                  c, b.masks, nullptr, po, vo, ao, b.cid_u, b.count);
        break;
    case 6:
        k_forces_mask2<R, 0, false><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n,
                                                                  c, b.masks, nullptr, po, vo, ao, b.cid_u, b.count);
        break;
    case 7: return launch_forces_rec<R, 0, 256, 1>(b, n, c, ao, st);
    case 8: return launch_forces_rec<R, 5, 256, 1>(b, n, c, ao, st);
    case 9: return launch_forces_rec<R, 6, 256, 1>(b, n, c, ao, st);
    case 10: return launch_forces_rec<R, 12, 128, 1>(b, n, c, ao, st);
    case 11: return launch_forces_rec<R, 10, 128, 1>(b, n, c, ao, st);
    case 1:
        k_forces_list<R, 32, 128><<<nblk(n, 128), 128, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n, c,
                                                                  po, vo, ao, b.cid_u, b.count);
        break;
    case 2:
        k_forces_list<R, 64, 128><<<nblk(n, 128), 128, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n, c,
                                                                  po, vo, ao, b.cid_u, b.count);
        break;
    default:
        k_forces<R><<<nblk(n, 256), 256, 0, st>>>(pos, vel, aux, b.start, b.scenes, b.obstacles, n, c, po, vo, ao,
                                                  b.cid_u, b.count);
        break;
    }
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::egress(const DevBufs &b, uint32_t n_state, uint32_t n_aux, uint32_t n_acc, int layout_sorted,
                              int aux_sorted, cudaStream_t st)
{
    if (!n_state) return cudaSuccess;
    const Vec4<R> *posL = (const Vec4<R> *) (layout_sorted ? b.pos_s : b.pos_u);
    const Vec4<R> *velL = (const Vec4<R> *) (layout_sorted ? b.vel_s : b.vel_u);
    const Vec4<R> *posA = (const Vec4<R> *) (aux_sorted ? b.pos_s : b.pos_u);
    const Vec4<R> *velA = (const Vec4<R> *) (aux_sorted ? b.vel_s : b.vel_u);
    R *xyz, *v, *rho, *p, *a;
    if (sizeof(R) == 8) {
        xyz = (R *) b.st_xyz64; v = (R *) b.st_vel64; rho = (R *) b.st_rho64; p = (R *) b.st_p64; a = (R *) b.st_acc64;
    } else {
        xyz = (R *) b.st_xyz; v = (R *) b.st_vel; rho = (R *) b.st_rho; p = (R *) b.st_p; a = (R *) b.st_acc;
    }
    k_egress<R><<<nblk(n_state, 256), 256, 0, st>>>(posL, velL, posA, velA, (const Vec4<R> *) b.aux,
                                                    (const Vec4<R> *) b.pos_u, (const Vec4<R> *) b.vel_u,
                                                    a ? (const Vec4<R> *) b.acc : nullptr, b.scene_off, n_state,
                                                    n_aux, n_acc, xyz, v, rho, p, a);
    return cudaGetLastError();
}

template <class R>
cudaError_t Launch<R>::stats(const DevBufs &b, uint32_t nscenes, Consts<R> c, int layout_sorted, cudaStream_t st)
{
    const Vec4<R> *vel = (const Vec4<R> *) (layout_sorted ? b.vel_s : b.vel_u);
    k_stats_partial<R><<<nscenes * STATS_SPLIT, STATS_THREADS, 0, st>>>(vel, (const Vec4<R> *) b.aux, b.start, b.scenes,
                                                                        b.stats_partial);
    k_stats_final<<<nscenes, 32, 0, st>>>(b.stats_partial, b.start, b.scenes, (double) c.mass, b.stats);
    return cudaGetLastError();
}

cudaError_t launch_slot(const DevBufs &b, uint32_t n, uint32_t ncells, cudaStream_t st)
{
    if (!n) return cudaSuccess;
    const cudaError_t e =
        launch_chained(k_slot<SLOT_PER>, nblk(n, 256 * SLOT_PER), 256, st, b.cid_u, n, b.start, b.count, b.tmp);
    return e == cudaSuccess ? launch_sort_big(b.start, b.tmp, b.big, b.bsum, ncells, st) : e;
}

cudaError_t launch_sort_big(const uint32_t *start, uint32_t *tmp, const uint32_t *big, uint32_t *gsum,
                            uint32_t ncells, cudaStream_t st)
{
    // a fixed grid walks the list (its length is known only on the device); with no big cell
    // every block only clears its share of the group sums
    return launch_chained(k_sort_big, 152, SORT_THREADS, st, start, tmp, big, gsum, ncells / kScanTile + 1);
}

template struct Launch<float>;
template struct Launch<double>;

SPH_CHECK_ACCESSOR(check_flags_kernels)

}  // namespace sph
