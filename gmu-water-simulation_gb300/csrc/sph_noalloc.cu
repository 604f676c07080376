// sph_noalloc.cu -- a grid build that allocates no device memory.
//
// For callers that must not allocate once they are running: a host application that has
// already handed its GPU memory to its own pool allocator, or a per-frame callback in a
// real-time loop, where cudaMalloc/cudaFree would synchronise the device and stall the frame.
// The caller passes device arrays for the positions and for every output; the kernels'
// working memory (per-cell counts and cursors, per-particle slot ids, scan block sums) lives
// in one file-scope device array of fixed size, reserved when the library's module is loaded
// and held by every GPU that loads it until the process exits.
//
// Limits: at most kMaxParticles particles and kMaxCells grid cells per call (about 12 MiB of
// scratch). Calls share the scratch array, which keeps the previous call's contents: each
// call clears what must start at zero, and two calls whose work overlaps on the GPU (on
// different streams, or from different host threads) race on it and must not be issued.
#include <cuda_runtime.h>

#include <mutex>

#include "../../include/sph_cuda.h"
#include "sph_internal.h"

namespace sph {
namespace {

constexpr uint32_t kMaxParticles = 1u << 20;
constexpr uint32_t kMaxCells = 1u << 20;
constexpr uint32_t kMaxBlocks = kMaxCells / kScanTile + 1;  // scan block sums
// counts | cursors | slot ids | scan block sums, as 32-bit words
constexpr size_t kScratchWords = (size_t) kMaxCells + kMaxCells + kMaxParticles + kMaxBlocks;

__device__ __align__(256) uint32_t g_grid_scratch[kScratchWords];

// Device address of g_grid_scratch per device ordinal, looked up once per device (the host
// symbol is only a stand-in and must not be passed to a kernel).
constexpr int kMaxDevices = 64;
uint32_t *g_scratch_ptr[kMaxDevices] = {nullptr};
std::mutex g_scratch_mu;

__global__ void __launch_bounds__(256) k_hash_plain_xyz(const float *__restrict__ xyz, uint32_t n, float3 half,
                                                        int3 res, float inv_h, double h_d,
                                                        uint32_t *__restrict__ out_cell, uint32_t *__restrict__ count)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const int cx = cell_axis(xyz[3 * i], half.x, inv_h, h_d, res.x);
    const int cy = cell_axis(xyz[3 * i + 1], half.y, inv_h, h_d, res.y);
    const int cz = cell_axis(xyz[3 * i + 2], half.z, inv_h, h_d, res.z);
    const uint32_t cell = (uint32_t) cx + (uint32_t) cy * (uint32_t) res.x + (uint32_t) cz * (uint32_t) res.x * (uint32_t) res.y;
    out_cell[i] = cell;
    atomicAdd(count + cell, 1u);
}

__global__ void __launch_bounds__(256) k_slot_ids(const uint32_t *__restrict__ cell, uint32_t n,
                                                  uint32_t *__restrict__ cursor, uint32_t *__restrict__ slot_ids)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    slot_ids[atomicAdd(cursor + cell[i], 1u)] = i;
}

// canonical (cell, id) order: position = cell start + number of same-cell ids below i
__global__ void __launch_bounds__(256) k_rank_ids(const uint32_t *__restrict__ cell, uint32_t n,
                                                  const uint32_t *__restrict__ start,
                                                  const uint32_t *__restrict__ slot_ids, uint32_t *__restrict__ order)
{
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t c = cell[i], b = start[c], e = start[c + 1];
    uint32_t r = 0;
    for (uint32_t k = b; k < e; k++) r += slot_ids[k] < i ? 1u : 0u;
    order[b + r] = i;
}

}  // namespace
}  // namespace sph

using namespace sph;

// The status code is the whole report: this entry point keeps no error text.
extern "C" int sph_grid_build_noalloc(const float *xyz, uint32_t n, const float box[3], float h, uint32_t *out_cell,
                                      uint32_t *out_start, uint32_t *out_order, void *stream)
{
    if (!box || !(h > 0) || !out_start) return SPH_ERR_ARG;
    if (n && (!xyz || !out_cell || !out_order)) return SPH_ERR_ARG;
    for (int a = 0; a < 3; a++)
        if (!(box[a] > 0)) return SPH_ERR_ARG;
    int3 res;
    res.x = (int) ceilf(box[0] / h);
    res.y = (int) ceilf(box[1] / h);
    res.z = (int) ceilf(box[2] / h);
    const uint64_t ncells = (uint64_t) res.x * res.y * res.z;
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
    cudaStream_t st = (cudaStream_t) stream;
    DevBufs b{};
    b.count = scratch;
    b.cursor = scratch + kMaxCells;
    b.tmp = scratch + 2 * (size_t) kMaxCells;
    b.bsum = scratch + 2 * (size_t) kMaxCells + kMaxParticles;
    b.start = out_start;
    // counts must start at zero: the previous call's values remain in the array
    if (cudaMemsetAsync(b.count, 0, 4 * ncells, st) != cudaSuccess) return SPH_ERR_CUDA;
    const unsigned blocks = (unsigned) ((n + 255) / 256);
    if (n) {
        const float3 half = make_float3(box[0] / 2.0f, box[1] / 2.0f, box[2] / 2.0f);
        k_hash_plain_xyz<<<blocks, 256, 0, st>>>(xyz, n, half, res, 1.0f / h, (double) h, out_cell, b.count);
    }
    cudaError_t e = Launch<float>::scan(b, (uint32_t) ncells, st);  // starts; cursors = starts; counts back to 0
    if (e == cudaSuccess && n) {
        k_slot_ids<<<blocks, 256, 0, st>>>(out_cell, n, b.cursor, b.tmp);
        k_rank_ids<<<blocks, 256, 0, st>>>(out_cell, n, b.start, b.tmp, out_order);
        e = cudaGetLastError();
    }
    return e == cudaSuccess ? SPH_OK : SPH_ERR_CUDA;
}
