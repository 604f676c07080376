// sph_noalloc.cu -- a grid build that allocates no device memory.
//
// For callers that must not allocate once they are running: a host application that has
// already handed its GPU memory to its own pool allocator, or a per-frame callback in a
// real-time loop, where cudaMalloc/cudaFree would synchronise the device and stall the frame.
// The caller passes device arrays for the positions and for every output; the kernels'
// working memory (per-cell counts, per-particle slot ids, per-group counts, the list
// of crowded cells) lives in one file-scope device array of fixed size. The array belongs to
// the library's device code: CUDA creates it on a device when that code is loaded there, which
// under lazy module loading (the default) is the first call on that device. That first call
// also looks up the array's device address, so it belongs in the caller's setup: before its
// pool allocator takes the GPU's memory and before any stream capture. Every GPU that has run
// a call holds the array until the process exits. cudaDeviceReset is not supported between
// calls: the address looked up by the first call would then be stale.
//
// Limits: at most kMaxParticles particles and kMaxCells grid cells per call (about 8 MiB of
// scratch). Calls share the scratch array, which keeps the previous call's contents: each
// call clears what must start at zero, and two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on it and must not be issued.
#include <cuda_runtime.h>

#include <cmath>
#include <mutex>

#include "../../include/sph_cuda.h"
#include "sph_device.cuh"
#include "sph_internal.h"

namespace sph {
namespace {

constexpr uint32_t kMaxParticles = 1u << 20;
constexpr uint32_t kMaxCells = 1u << 20;
constexpr uint32_t kMaxBlocks = kMaxCells / kScanTile + 1;  // group sums of the scan
constexpr size_t kBigWords = big_words(kMaxParticles);       // crowded-cell list
// counts | slot ids | group sums | crowded cells, as 32-bit words
constexpr size_t kScratchWords = (size_t) kMaxCells + kMaxParticles + kMaxBlocks + kBigWords;

__device__ __align__(256) uint32_t g_grid_scratch[kScratchWords];

// Device address of g_grid_scratch per device ordinal, looked up once per device (the host
// symbol is only a stand-in and must not be passed to a kernel).
constexpr int kMaxDevices = 64;
uint32_t *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

__global__ void __launch_bounds__(256) k_hash_plain_xyz(const float *__restrict__ xyz, uint32_t n, float3 half,
                                                        int3 res, float inv_h, double h_d,
                                                        uint32_t *__restrict__ out_cell, uint32_t *__restrict__ count,
                                                        uint32_t *__restrict__ gsum)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cx = cell_axis(xyz[3 * i], half.x, inv_h, h_d, res.x);
    const int cy = cell_axis(xyz[3 * i + 1], half.y, inv_h, h_d, res.y);
    const int cz = cell_axis(xyz[3 * i + 2], half.z, inv_h, h_d, res.z);
    const uint32_t cell = (uint32_t) cx + (uint32_t) cy * (uint32_t) res.x + (uint32_t) cz * (uint32_t) res.x * (uint32_t) res.y;
    out_cell[i] = cell;
    count_add(count, gsum, cell);
}

// every id takes a slot of its cell, from the top down (the counts end at zero)
__global__ void __launch_bounds__(256) k_slot_ids(const uint32_t *__restrict__ cell, uint32_t n,
                                                  const uint32_t *__restrict__ start, uint32_t *__restrict__ count,
                                                  uint32_t *__restrict__ slot_ids)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = cell[i];
    slot_ids[start[c] + atomicSub(count + c, 1u) - 1u] = i;
}

// canonical (cell, id) order: position = cell start + number of same-cell ids below i
__global__ void __launch_bounds__(256) k_rank_ids(const uint32_t *__restrict__ cell, uint32_t n,
                                                  const uint32_t *__restrict__ start,
                                                  const uint32_t *__restrict__ slot_ids, uint32_t *__restrict__ order)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = cell[i], b = start[c], e = start[c + 1];
    const uint32_t dst = b + rank_in_cell(slot_ids, b, e, i);
    if (sph_check(dst < e && e <= n, CHK_SORT)) order[dst] = i;
}

}  // namespace

// The reference's grid of n particles (float xyz, id order) in a box of res cells per axis (cells
// of size h, linear index x + y*X + z*X*Y): the cell of every particle, the cell starts and the
// ids in ascending (cell, id) order, with the working memory g (counts, slot ids, group sums,
// crowded-cell list) supplied by the caller.
cudaError_t ref_grid_build(const float *xyz, uint32_t n, int3 res, float3 half, float h, uint32_t *out_cell,
                           uint32_t *out_start, uint32_t *out_order, const GridScratch &g, cudaStream_t st)
{
    const uint64_t ncells = (uint64_t) res.x * (uint64_t) res.y * (uint64_t) res.z;
    DevBufs b{};
    b.count = g.count;
    b.tmp = g.tmp;
    b.bsum = g.bsum;
    b.big = g.big;
    b.start = out_start;
    // counts, group sums and the crowded-cell list start empty (a previous call, or one that
    // failed, may have left values)
    cudaError_t e = cudaMemsetAsync(b.count, 0, 4 * ncells, st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.bsum, 0, 4 * (ncells / kScanTile + 1), st);
    if (e == cudaSuccess) e = cudaMemsetAsync(b.big, 0, 4, st);
    if (e != cudaSuccess) return e;
    const unsigned blocks = (unsigned) ((n + 255) / 256);
    if (n)
        k_hash_plain_xyz<<<blocks, 256, 0, st>>>(xyz, n, half, res, 1.0f / h, (double) h, out_cell, b.count, b.bsum);
    e = Launch<float>::scan(b, (uint32_t) ncells, st);  // starts
    if (e == cudaSuccess && n) {
        k_slot_ids<<<blocks, 256, 0, st>>>(out_cell, n, b.start, b.count, b.tmp);
        e = launch_sort_big(b.start, b.tmp, b.big, b.bsum, (uint32_t) ncells, st);
        if (e == cudaSuccess) {
            k_rank_ids<<<blocks, 256, 0, st>>>(out_cell, n, b.start, b.tmp, out_order);
            e = cudaGetLastError();
        }
    }
    return e;
}

SPH_CHECK_ACCESSOR(check_flags_noalloc)

}  // namespace sph

using namespace sph;

// The status code is the whole report: this entry point keeps no error text.
extern "C" int sph_grid_build_noalloc(const float *xyz, uint32_t n, const float box[3], float h, uint32_t *out_cell,
                                      uint32_t *out_start, uint32_t *out_order, void *stream)
{
    if (!box || !(h > 0) || !std::isfinite(h) || !out_start) return SPH_ERR_ARG;
    if (n && (!xyz || !out_cell || !out_order)) return SPH_ERR_ARG;
    // cells per axis as the context computes them (float quotient, then ceil), checked against
    // the scratch limit before the conversion to int so that no huge or infinite quotient is cast
    int r3[3];
    for (int a = 0; a < 3; a++) {
        if (!(box[a] > 0) || !std::isfinite(box[a])) return SPH_ERR_ARG;
        const float q = ceilf(box[a] / h);
        if (!(q <= (float) kMaxCells)) return SPH_ERR_CAPACITY;  // also an infinite quotient
        r3[a] = (int) q;
    }
    const int3 res = make_int3(r3[0], r3[1], r3[2]);
    const uint64_t ncells = (uint64_t) res.x * (uint64_t) res.y * (uint64_t) res.z;
    if (n > kMaxParticles || ncells > kMaxCells) return SPH_ERR_CAPACITY;  // beyond the fixed scratch
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) return SPH_ERR_CUDA;
    uint32_t *scratch = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_scratch_mu);
        if (!g_scratch_ptr[dev]) {
            // first call on this device (with it current): resolve the array's device address
            void *p = nullptr;
            if (cudaGetSymbolAddress(&p, g_grid_scratch) != cudaSuccess || !p) return SPH_ERR_CUDA;
            g_scratch_ptr[dev] = (uint32_t *) p;
        }
        scratch = g_scratch_ptr[dev];
    }
    GridScratch g;
    g.count = scratch;
    g.tmp = scratch + (size_t) kMaxCells;
    g.bsum = scratch + (size_t) kMaxCells + kMaxParticles;
    g.big = g.bsum + kMaxBlocks;
    const float3 half = make_float3(box[0] / 2.0f, box[1] / 2.0f, box[2] / 2.0f);
    const cudaError_t e = ref_grid_build(xyz, n, res, half, h, out_cell, out_start, out_order, g, (cudaStream_t) stream);
    return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
