// sph_internal.h -- types shared by the host context and the sm_103a kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

namespace sph {

// Device-side descriptor of one scene of a batch. Cells of scene s occupy the global
// cell range [cell_base, cell_base + ncells) of the step's grid. With cell multiple 1 that is the
// reference's grid: (int) ceil(box / h) cells per axis, linear index x + y*X + z*X*Y
// (include/CGrid.h:25-28). With cell multiple m the step's cells are h/m wide and res is m times
// the reference's resolution (the same extent, split m ways per axis).
struct alignas(16) SceneDev {
    float half[3];      // box / 2 (exact in float), the wall positions
    uint32_t cell_base;
    int32_t res[3];
    uint32_t ncells;
    float gravity[3];
    uint32_t obs_base;  // first obstacle of this scene in the obstacle table
    uint32_t n_obs;
    uint32_t pad[3];
};

// Axis-aligned box obstacle: lo/hi corners.
struct alignas(16) ObstacleDev {
    float lo[3];
    float pad0;
    float hi[3];
    float pad1;
};

// Step constants in the arithmetic type R (float for the plain form, double for FP64).
template <class R>
struct Consts {
    R h, h2;           // smoothing length and its square
    R mass, k, rho0, mu;
    R dt;
    R c_poly6, c_spiky, c_visc;  // 315/(64 pi h^9), -45/(pi h^6), 45/(pi h^6)
    R wall_k, wall_damp, wall_r;
    float h_f, inv_h_f; // h as float, 1/h rounded (the mixed form's h-cell codes)
    double h_d;         // (double) h
    // the step grid's cell width h/m: the hash's float reciprocal (m times 1/h rounded, exactly)
    // and the divisor of its exact double formula
    float inv_cell_f;
    double cell_d;
    // particles per group of kScanTile cells of the step grid: every hash adds to it beside the
    // cell's count, the scan reads it for its tile offsets, the crowded-cell sort clears it
    uint32_t *gsum;
};

// Buffers of one context, in the layout of the precision form.
//   *_s : state in canonical sorted order, ascending (global cell, id)
//   *_u : state in the previous sorted order (output of the force pass / upload)
// .w of a position carries the scene index bits, .w of a velocity the particle id bits.
struct DevBufs {
    void *pos_s, *vel_s, *pos_u, *vel_u, *aux, *acc;  // R4 arrays
    uint2 *cid_u;          // (global cell, id) of every *_u particle
    uint32_t *tmp;         // ids scattered into cell slots, for the canonical rank
    uint32_t *count;       // particles per global cell (hash output; the slot pass counts it back to 0)
    uint32_t *start;       // exclusive scan of count, ncells_total + 1 entries
    uint32_t *bsum;        // particles per kScanTile-cell group (Consts::gsum), ncells / kScanTile + 1 words
    uint32_t *big;         // cells above kBigCell particles: count in word 0, then the cells (big_words(n) words)
    SceneDev *scenes;
    ObstacleDev *obstacles;
    uint32_t *scene_off;   // first output index of every scene (id-order downloads)
    int32_t *err;          // device error flag
    // staging for host transfers (ingest / egress)
    float *st_xyz, *st_vel, *st_rho, *st_p, *st_acc;
    double *st_xyz64, *st_vel64, *st_rho64, *st_p64, *st_acc64;
    double *stats;         // per-scene FP64 reductions, 8 doubles each
    double *stats_partial; // per-scene slices of the reductions (kSplit x 6 doubles each)
    uint32_t *masks;       // accepted-neighbour bit masks of the density pass, 36 words per particle
    void *frec;            // force records of the density pass: plain/FP64 variants 7-11 (x, y, z, c_spiky p/rho^2),
                           // (v, c_visc/rho); mixed: one 16-byte record per particle (sph_mixed.cu)
    uint32_t *inv;         // layout index of each particle in id order (downloads into pinned host memory)
    // mixed-precision form only
    void *lo_s, *lo_u;     // low parts of the hi/lo positions (float4, .w unused)
    uint2 *gpos;           // gathered positions: 16-bit codes x | y << 16, z (sorted order)
                           // (the mixed form's neighbour records, 16 bytes each, live in frec)
};

// ---- exact cell hash -------------------------------------------------------------
// The reference computes floor((p + box/2.0) / h) in double (src/CCPUParticleSimulator.cpp:46-48)
// and clamps to [0, res-1] (:50-69). Here the quotient is first taken in float; its
// relative error is below 3 * 2^-24, so whenever it lies farther than 4e-7 * max(|q|, 1)
// from an integer its floor equals the double result. Otherwise (and for NaN) the double
// formula is evaluated exactly as the reference does. NaN and negatives map to cell 0,
// values at or beyond res to res - 1.
__host__ __device__ inline int cell_axis(float p, float half, float inv_h, double h_d, int res)
{
    const float qf = (p + half) * inv_h;
    const float rq = rintf(qf);
    if (fabsf(qf - rq) > fmaxf(fabsf(qf), 1.0f) * 4.0e-7f) {
        if (qf < 0.0f) return 0;
        if (qf >= (float) res) return res - 1;
        return (int) floorf(qf);
    }
    const double q = ((double) p + (double) half) / h_d;
    if (!(q >= 0.0)) return 0;
    if (q >= (double) res) return res - 1;
    return (int) floor(q);
}

__host__ __device__ inline int cell_axis(double p, float half, float inv_h, double h_d, int res)
{
    const double q = (p + (double) half) / h_d;
    if (!(q >= 0.0)) return 0;
    if (q >= (double) res) return res - 1;
    return (int) floor(q);
}

// Constants of the mixed form, whose neighbour displacements are in code units of h / 8192.
struct MixConsts {
    float to_units;  // 8192 / h
    float poly6_q;   // 315 / (64 pi h^9) * (h / 8192)^6: the poly6 factor for (h^2 - r^2) in units^2
    float spiky_q;   // -45 / (pi h^6) * (h / 8192)^2
    float visc_q;    // 45 / (pi h^6) * (h / 8192)
};

// Launch variants of the neighbour kernels (picked per context; see the autotuner).
//   density_p : 0 = one particle per thread, first form; 1/2/4 = blocked branchless form
//               with that many consecutive particles per thread
//   forces_mode: 0 = pair terms inside the candidate loop; 1/2 = compacted neighbour list
//               of 32/64 entries per thread in shared memory; 3..11 = driven by the neighbour
//               masks that the density pass then writes (density_p is ignored): 3/4 one
//               neighbour per iteration without/with a 64-register cap, 5/6 two per
//               iteration with/without it, 7 as 6 with each neighbour's terms read from one
//               packed force record (two 16-byte loads from one 32-byte record), 8 and 9 as
//               7 at 48 and 40 registers, 10 and 11 as 9 and 8 in blocks of 128 threads
//   cell_mult : the step grid's cells are h / cell_mult wide (1 or 2); the neighbour passes walk
//               (2 cell_mult + 1)^2 rows of 2 cell_mult + 1 cells (only the mask-driven record
//               variants, 7 to 11 and the mixed form's, run on cells of h/2)
struct Tune {
    static constexpr int ALL_PAIRS = 16;  // both passes over every particle of the scene
    int density_p = 2;
    int forces_mode = 3;
    int cell_mult = 1;
};

// Neighbour rows of the stencil of radius RAD cells (RAD = cell multiple): (2 RAD + 1)^2 rows,
// each 2 RAD + 1 cells along x, with WORDS mask words of 32 candidates recorded per row. The
// mask buffer holds 36 words per particle: 9 rows x 4 words, or 25 rows x 1 word.
template <int RAD>
struct Stencil {
    static constexpr int ROWS = (2 * RAD + 1) * (2 * RAD + 1);
    static constexpr int WORDS = RAD == 1 ? 4 : 1;
    static_assert(ROWS * WORDS <= 36, "the masks fit the per-particle mask buffer");
};
constexpr int kMaskWordsPerParticle = 36;

// Cells of the cell-count scan's smallest tile (one block of 256 threads x 4 cells); larger
// grids use tiles of several such groups. The block-sum buffer holds one word per tile of this
// size (plus one), enough for any tile size, and is sized with it wherever it is allocated.
constexpr uint32_t kScanTile = 1024;

// Cells holding more than kBigCell particles are listed by the scan and their slot ids sorted
// (k_sort_big), so that the canonical rank is a search instead of an occupancy^2 count (cells up
// to kBigCell, 16 times the rest occupancy, are counted directly: at most 128 loads a particle).
// Sorting happens in shared memory for cells of up to kBigCellMax particles. The list holds its
// length in word 0 and at most n / kBigCell cells: big_words(n) words.
constexpr uint32_t kBigCell = 128;
constexpr uint32_t kBigCellMax = 4096;
__host__ __device__ constexpr uint64_t big_words(uint64_t n) { return n / kBigCell + 2; }

// ---- kernel launchers (sph_kernels.cu) --------------------------------------------
template <class R>
struct Launch {
    // xyz / vel: device staging arrays of n particles stored at [first, first + n).
    // scene >= 0: all belong to that scene with ids id0..; scene < 0: scene and id follow
    // the scene_off table (upload of every scene at once, first == 0).
    static cudaError_t ingest(const DevBufs &b, const float *xyz, const float *vel, uint32_t first, uint32_t n,
                              int32_t scene, uint32_t id0, uint32_t nscenes, Consts<R> c, cudaStream_t st);
    static cudaError_t scan(const DevBufs &b, uint32_t ncells, cudaStream_t st);
    static cudaError_t permute(const DevBufs &b, uint32_t n, uint32_t ncells, cudaStream_t st);
    // positions of the first n *_u particles hashed again into the step grid (after the cell
    // multiple changed): counts and the cells of cid_u
    static cudaError_t rehash(const DevBufs &b, uint32_t n, Consts<R> c, cudaStream_t st);
    static cudaError_t density(const DevBufs &b, uint32_t n, Consts<R> c, const Tune &t, cudaStream_t st);
    static cudaError_t forces(const DevBufs &b, uint32_t n, Consts<R> c, bool record_acc, const Tune &t,
                              cudaStream_t st);
    // state of the first n_state particles, density/pressure of the first n_aux, and
    // accelerations of the first n_acc (when recorded) into id-ordered staging arrays
    static cudaError_t egress(const DevBufs &b, uint32_t n_state, uint32_t n_aux, uint32_t n_acc, int layout_sorted,
                              int aux_sorted, cudaStream_t st);
    static cudaError_t stats(const DevBufs &b, uint32_t nscenes, Consts<R> c, int layout_sorted, cudaStream_t st);
};

// slot assignment of the counting sort alone (the mixed form has its own permute), on a grid
// of ncells cells
cudaError_t launch_slot(const DevBufs &b, uint32_t n, uint32_t ncells, cudaStream_t st);

// sorts the slot ids of every cell the scan listed in big (after the slots are taken) and
// clears the group sums gsum of a grid of ncells cells
cudaError_t launch_sort_big(const uint32_t *start, uint32_t *tmp, const uint32_t *big, uint32_t *gsum,
                            uint32_t ncells, cudaStream_t st);

// disc emitter on the device (sph_emit.cu): n particles into the float3 staging arrays
cudaError_t launch_emit_fountain(uint64_t seed, uint32_t step, uint32_t n, const float center[3], float radius,
                                 float speed, float sigma, float *xyz, float *vel, cudaStream_t st);

// id-ordered float3 positions (and velocities if v) of the first n particles (sph_handoff.cu)
template <class R>
cudaError_t launch_handoff(const DevBufs &b, uint32_t n, int layout_sorted, float *xyz, float *v, cudaStream_t st);

// id-ordered float3 positions and/or velocities written straight into pinned host arrays
// (device-accessible views), through b.inv (sph_handoff.cu)
template <class R>
cudaError_t launch_gather_host(const DevBufs &b, uint32_t n, int layout_sorted, float *xyz, float *v, cudaStream_t st);

// orthographic point splat of one scene into per-pixel counts and nearest depth (sph_handoff.cu)
template <class R>
cudaError_t launch_splat(const DevBufs &b, uint32_t n, int layout_sorted, uint32_t scene, int axis, float half_u,
                         float half_v, float scale_u, float scale_v, uint32_t width, uint32_t height,
                         uint32_t *count, float *depth, cudaStream_t st);

// Working memory of a reference-grid build of n particles and C cells: counts (C words), slot
// ids (n), group sums (C / kScanTile + 1), crowded cells (big_words(n)).
struct GridScratch {
    uint32_t *count, *tmp, *bsum, *big;
};
// the reference's grid (cells of size h) of n id-ordered float positions (sph_noalloc.cu)
cudaError_t ref_grid_build(const float *xyz, uint32_t n, int3 res, float3 half, float h, uint32_t *out_cell,
                           uint32_t *out_start, uint32_t *out_order, const GridScratch &g, cudaStream_t st);

// checked builds: OR each translation unit's device check flags into *out and clear them
cudaError_t check_flags_kernels(uint32_t *out);
cudaError_t check_flags_mixed(uint32_t *out);
cudaError_t check_flags_handoff(uint32_t *out);
cudaError_t check_flags_noalloc(uint32_t *out);

// mixed-precision passes (sph_mixed.cu)
cudaError_t mixed_permute(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, cudaStream_t st);
cudaError_t mixed_density(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, int cell_mult,
                          cudaStream_t st);
// variant: the mixed force pass's launch form, 0..kMixedVariants-1 (all give the same bits)
constexpr int kMixedVariants = 4;
cudaError_t mixed_forces(const DevBufs &b, uint32_t n, Consts<float> c, MixConsts mc, bool record_acc, int variant,
                         int cell_mult, cudaStream_t st);
cudaError_t mixed_egress(const DevBufs &b, uint32_t n_state, uint32_t n_aux, uint32_t n_acc, int layout_sorted,
                         int aux_sorted, bool f64, cudaStream_t st);

}  // namespace sph
