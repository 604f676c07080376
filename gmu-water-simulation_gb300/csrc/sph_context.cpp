// sph_context.cpp -- host side of the C ABI (include/sph_cuda.h): context, buffers,
// pass sequencing, CUDA-graph replay of whole steps, transfers and error reporting.
//
// Replaces CGPUBaseParticleSimulator / CGPUParticleSimulator and CLWrapper
// (src/CGPUBaseParticleSimulator.cpp, src/CGPUParticleSimulator.cpp, src/CLWrapper.cpp):
// one CUDA stream per context instead of one OpenCL queue, the whole step on the device
// instead of a host sort and four full-array copies per step.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <new>
#include <sstream>
#include <string>
#include <sys/stat.h>
#include <vector>

#include "../../include/sph_cuda.h"
#include "sph_internal.h"

using namespace sph;

namespace {

struct SceneHost {
    float box[3];
    int32_t res[3];
    uint32_t cell_base, ncells, cap, count;
    float gravity[3];
    std::vector<ObstacleDev> obs;
};

enum State { EMPTY = 0, HASHED = 1, SORTED = 2, DENSE = 3 };

constexpr int kOnlineN = 4;  // force variants tried by online tuning (one trial step each)
constexpr int kOnlineMax = kOnlineN + 1;  // ... and one trial on the other cell multiple

thread_local std::string g_create_error;

}  // namespace

struct sph_ctx {
    sph_params prm{};
    int device = 0;
    cudaStream_t stream = nullptr;
    std::vector<SceneHost> sc;
    uint64_t ctot = 0, ncap = 0;  // cells of the step grid (all scenes), particle capacity
    uint64_t ctot_ref = 0;        // cells of the reference grid (cells of size h)
    uint64_t ctot_cap = 0;        // cells the grid arrays hold: the finest grid this context may use
    uint32_t n = 0;         // particles held (including appended ones)
    uint32_t n_sorted = 0;  // particles covered by the last grid pass
    uint32_t n_forced = 0;  // particles covered by the last force pass (recorded accelerations)
    uint32_t n_dense = 0;   // particles covered by the last density pass (valid aux records)
    DevBufs b{};
    void *pool = nullptr;
    State state = EMPTY;
    bool appended = false;  // particles appended since the last grid pass
    std::string err, devname;
    cudaEvent_t ev[4] = {nullptr, nullptr, nullptr, nullptr};
    double ms[5] = {0, 0, 0, 0, 0};
    cudaGraphExec_t graph = nullptr;
    int graph_steps = 0;
    uint32_t graph_n = 0;
    std::vector<uint32_t> scene_off_host;
    Tune tune;
    bool tune_pinned = false;  // variants set explicitly: the cache does not override them
    bool cell_pinned = false;  // cell multiple set explicitly: the autotuner keeps it
    // front-end handoff (allocated by the first handoff or export)
    cudaStream_t ho_stream = nullptr;
    cudaEvent_t ho_ready = nullptr, ho_done = nullptr, ho_export = nullptr;
    float *ho_xyz = nullptr, *ho_vel = nullptr;
    bool ho_recorded = false;  // ho_done has been recorded at least once
    // online tuning of the mask-driven force variant (sph_set_online_tuning)
    int online_period = 0;     // steps between trials; 0 = off
    uint64_t steps_run = 0;    // whole steps run by this context
    int trial = -1;            // candidate being timed in this step, -1 = none
    int n_trials = 0;          // candidates of the current trial period
    float trial_ms[kOnlineMax] = {};  // one per online candidate
    int trial_m[kOnlineMax] = {}, trial_v[kOnlineMax] = {};  // its cell multiple and force variant
    int last_best_v[3] = {0, 10, 10};  // per cell multiple, the force variant its last trials kept
    cudaEvent_t on_ev[2] = {nullptr, nullptr};
    int graph_forces = -1;     // force variant captured in the graph
    std::vector<unsigned char *> canaries;  // checked builds: the guard region after each array
};

namespace {

int fail(sph_ctx *c, int code, const std::string &msg)
{
    if (c) c->err = msg;
    else g_create_error = msg;
    return code;
}

int cuda_fail(sph_ctx *c, cudaError_t e, const char *what)
{
    std::string m = std::string(what) + ": " + cudaGetErrorName(e) + " (" + cudaGetErrorString(e) + ")";
    return fail(c, SPH_ERR_CUDA, m);
}

#define CK(ctx, call)                                               \
    do {                                                            \
        cudaError_t e_ = (call);                                    \
        if (e_ != cudaSuccess) return cuda_fail((ctx), e_, #call);  \
    } while (0)

bool is_f64(const sph_ctx *c) { return c->prm.precision == SPH_F64; }
bool is_mixed(const sph_ctx *c) { return c->prm.precision == SPH_MIXED; }

MixConsts make_mix(const sph_params &p)
{
    MixConsts m{};
    const double h = (double) p.h, s = h / 8192.0;
    m.to_units = (float) (8192.0 / h);
    m.poly6_q = (float) (315.0 / (64.0 * M_PI * std::pow(h, 9)) * std::pow(s, 6));
    m.spiky_q = (float) (-45.0 / (M_PI * std::pow(h, 6)) * s * s);
    m.visc_q = (float) (45.0 / (M_PI * std::pow(h, 6)) * s);
    return m;
}
size_t r4_bytes(const sph_ctx *c) { return is_f64(c) ? 32 : 16; }

// The hash outputs of a grid of ncells cells cleared: the per-cell counts, their per-group sums
// and the crowded-cell list (the step's own passes leave all three empty between steps).
int clear_counts(sph_ctx *c, uint64_t ncells)
{
    CK(c, cudaMemsetAsync(c->b.count, 0, 4 * ncells, c->stream));
    CK(c, cudaMemsetAsync(c->b.bsum, 0, 4 * (ncells / kScanTile + 1), c->stream));
    CK(c, cudaMemsetAsync(c->b.big, 0, 4, c->stream));
    return SPH_OK;
}

template <class R>
Consts<R> make_consts(const sph_ctx *ctx, int cell_mult)
{
    const sph_params &p = ctx->prm;
    Consts<R> c{};
    const double h = (double) p.h;
    c.h = (R) p.h;
    if (sizeof(R) == 4) c.h2 = (R) (p.h * p.h);  // float product, as h*h in the reference
    else c.h2 = (R) (h * h);
    c.mass = (R) p.mass;
    c.k = (R) p.gas_stiffness;
    c.rho0 = (R) p.rest_density;
    c.mu = (R) p.viscosity;
    c.dt = (R) p.dt;
    c.c_poly6 = (R) (315.0 / (64.0 * M_PI * std::pow(h, 9)));
    c.c_spiky = (R) (-45.0 / (M_PI * std::pow(h, 6)));
    c.c_visc = (R) (45.0 / (M_PI * std::pow(h, 6)));
    c.wall_k = (R) (double) p.wall_k;
    c.wall_damp = sizeof(R) == 4 ? (R) p.wall_damping : (R) (p.wall_damping == -0.9f ? -0.9 : (double) p.wall_damping);
    c.wall_r = sizeof(R) == 4 ? (R) p.wall_radius : (R) (p.wall_radius == 0.01f ? 0.01 : (double) p.wall_radius);
    c.h_f = p.h;
    c.inv_h_f = 1.0f / p.h;
    c.h_d = (double) p.h;
    // the step grid's cells are h / cell_mult wide: its hash scales the float reciprocal and the
    // double divisor by the (power-of-two) multiple, both exactly
    c.inv_cell_f = c.inv_h_f * (float) cell_mult;
    c.cell_d = c.h_d / (double) cell_mult;
    c.gsum = ctx->b.bsum;
    return c;
}

// The scenes' descriptors on the device, in the step grid of the current cell multiple m: m
// times the reference resolution per axis, scenes' cell ranges consecutive.
int upload_scenes(sph_ctx *c)
{
    std::vector<SceneDev> sd(c->sc.size());
    uint32_t ob = 0;
    const int m = c->tune.cell_mult;
    uint64_t base = 0;
    for (size_t s = 0; s < c->sc.size(); s++) {
        const SceneHost &h = c->sc[s];
        SceneDev &d = sd[s];
        std::memset(&d, 0, sizeof(d));
        for (int a = 0; a < 3; a++) {
            d.half[a] = h.box[a] / 2.0f;
            d.res[a] = h.res[a] * m;
            d.gravity[a] = h.gravity[a];
        }
        d.cell_base = (uint32_t) base;
        d.ncells = (uint32_t) ((uint64_t) d.res[0] * d.res[1] * d.res[2]);
        base += d.ncells;
        d.obs_base = ob;
        d.n_obs = (uint32_t) h.obs.size();
        ob += d.n_obs;
    }
    c->ctot = base;
    CK(c, cudaMemcpyAsync(c->b.scenes, sd.data(), sd.size() * sizeof(SceneDev), cudaMemcpyHostToDevice, c->stream));
    if (ob) {
        std::vector<ObstacleDev> all;
        for (auto &h : c->sc) all.insert(all.end(), h.obs.begin(), h.obs.end());
        CK(c, cudaMemcpyAsync(c->b.obstacles, all.data(), all.size() * sizeof(ObstacleDev), cudaMemcpyHostToDevice,
                              c->stream));
    }
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

// Device-accessible view of a pinned (page-locked) host array, or nullptr for other memory.
// Kernels then read or write the caller's array over the host link directly: the transfer
// and the ingest (or the id-ordered gather) become one pass.
void *pinned_view(const void *p)
{
    if (!p) return nullptr;
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // not an error of the context: the copy path is taken
        return nullptr;
    }
    return a.type == cudaMemoryTypeHost ? a.devicePointer : nullptr;
}

// The scene-offset table on the device, copied only when the scene counts changed since the
// last copy (uploads and downloads of an unchanged batch skip the small pageable copy).
int upload_scene_off(sph_ctx *c)
{
    std::vector<uint32_t> off(c->sc.size() + 1, 0);
    for (size_t s = 0; s < c->sc.size(); s++) off[s + 1] = off[s] + c->sc[s].count;
    if (off == c->scene_off_host) return SPH_OK;
    // pageable source: staged before the call returns, so the local array may go
    CK(c, cudaMemcpyAsync(c->b.scene_off, off.data(), off.size() * sizeof(uint32_t), cudaMemcpyHostToDevice,
                          c->stream));
    c->scene_off_host = off;  // only once the copy is queued
    return SPH_OK;
}

void drop_graph(sph_ctx *c)
{
    if (c->graph) cudaGraphExecDestroy(c->graph);
    c->graph = nullptr;
    c->graph_steps = 0;
}

struct PoolItem {
    void **p;
    size_t bytes;
};

// Checked builds follow every array of the pool with a guard region of known bytes;
// sph_debug_check reports any that changed (an out-of-bounds write that escaped the checks).
#ifdef SPH_CHECKED
constexpr size_t kCanaryBytes = 256;
#else
constexpr size_t kCanaryBytes = 0;
#endif
constexpr unsigned char kCanary = 0xA5;

// The sub-arrays of a context's single device allocation (256-byte aligned); returns the
// total size. Needs only the configuration (no CUDA call), so a create can be refused before
// any device work and sph_memory_required can answer on the host.
size_t pool_layout(sph_ctx *c, std::vector<PoolItem> &items)
{
    const size_t r4 = r4_bytes(c), rs = is_f64(c) ? 8 : 4;
    const bool mixed = is_mixed(c);
    const uint64_t N = c->ncap, C = c->ctot_cap;
    const uint64_t nb = (C + kScanTile - 1) / kScanTile + 1;
    uint64_t nobs = 0;
    for (auto &h : c->sc) nobs += h.obs.size();
    DevBufs &b = c->b;
    const bool rec = (c->prm.flags & SPH_FLAG_RECORD_ACC) != 0;
    items = {
        {&b.pos_s, r4 * N}, {&b.vel_s, r4 * N}, {&b.pos_u, r4 * N}, {&b.vel_u, r4 * N}, {&b.aux, r4 * N},
        {&b.acc, rec ? r4 * N : 0},
        {(void **) &b.cid_u, 8 * N}, {(void **) &b.tmp, 4 * N},
        {(void **) &b.count, 4 * C}, {(void **) &b.start, 4 * (C + 1)},
        {(void **) &b.bsum, 4 * nb}, {(void **) &b.big, 4 * big_words(N)},
        {(void **) &b.scenes, sizeof(SceneDev) * c->sc.size()},
        {(void **) &b.obstacles, sizeof(ObstacleDev) * (nobs ? nobs : 1)},
        {(void **) &b.scene_off, 4 * (c->sc.size() + 1)}, {(void **) &b.err, 16},
        {(void **) &b.st_xyz, 12 * N}, {(void **) &b.st_vel, 12 * N},
        {(void **) &b.st_rho, rs == 4 ? 4 * N : 0}, {(void **) &b.st_p, rs == 4 ? 4 * N : 0},
        {(void **) &b.st_acc, rs == 4 && rec ? 12 * N : 0},
        {(void **) &b.st_xyz64, (rs == 8 || mixed) ? 24 * N : 0}, {(void **) &b.st_vel64, (rs == 8 || mixed) ? 24 * N : 0},
        {(void **) &b.st_rho64, (rs == 8 || mixed) ? 8 * N : 0}, {(void **) &b.st_p64, (rs == 8 || mixed) ? 8 * N : 0},
        {&b.lo_s, mixed ? 16 * N : 0}, {&b.lo_u, mixed ? 16 * N : 0},
        {(void **) &b.gpos, mixed ? 8 * N : 0},
        {(void **) &b.st_acc64, (rs == 8 || mixed) && rec ? 24 * N : 0},
        {(void **) &b.stats, 64 * c->sc.size()},
        {(void **) &b.stats_partial, 6 * 8 * 64 * c->sc.size()},
        {(void **) &b.masks, 4 * 36 * N},
        {(void **) &b.frec, mixed ? 16 * N : 2 * r4 * N},
        {(void **) &b.inv, 4 * N},
    };
    size_t total = 0;
    for (auto &it : items) total += ((it.bytes + 255) & ~size_t(255)) + kCanaryBytes;
    return total;
}

// SPH_DEVICE_MEMORY_LIMIT (bytes): an optional cap on a context's device allocation, e.g. to
// share a GPU with other work; 0 or unset = no cap
uint64_t memory_limit()
{
    const char *v = std::getenv("SPH_DEVICE_MEMORY_LIMIT");
    return v ? std::strtoull(v, nullptr, 10) : 0;
}

int allocate(sph_ctx *c)
{
    std::vector<PoolItem> items;
    const size_t total = pool_layout(c, items);
    DevBufs &b = c->b;
    const uint64_t N = c->ncap, C = c->ctot_cap;
    const size_t r4 = r4_bytes(c);
    cudaError_t e = cudaMalloc(&c->pool, total);
    if (e != cudaSuccess) {
        c->pool = nullptr;
        return fail(c, SPH_ERR_NOMEM, std::string("device allocation of ") + std::to_string(total) +
                                          " bytes failed: " + cudaGetErrorString(e));
    }
    char *p = (char *) c->pool;
    c->canaries.clear();
    for (auto &it : items) {
        *it.p = it.bytes ? (void *) p : nullptr;
        p += (it.bytes + 255) & ~size_t(255);
        if (kCanaryBytes) {
            c->canaries.push_back((unsigned char *) p);
            CK(c, cudaMemsetAsync(p, kCanary, kCanaryBytes, c->stream));
            p += kCanaryBytes;
        }
    }
    if (int rc = clear_counts(c, C)) return rc;
    CK(c, cudaMemsetAsync(b.aux, 0, r4 * N, c->stream));
    CK(c, cudaMemsetAsync(b.err, 0, 16, c->stream));
    return SPH_OK;
}

// the all-pairs form is O(n^2) per scene: a check for small scenes, not a production path
constexpr uint32_t kAllPairsMax = 131072;

// Cell multiples: 1 (the reference's cells of size h) or 2 (cells of h/2 with a 5-cell stencil per
// axis), for the plain FP32 and mixed forms' grid passes. The FP64 form (the reference run) and the
// all-pairs form stay on the reference's grid.
constexpr int kMaxCellMult = 2;
bool cell_mult_allowed(const sph_ctx *c, int m, uint64_t ctot_ref)
{
    if (m == 1) return true;
    if (m != 2) return false;
    if (c->prm.precision == SPH_F64 || (c->prm.flags & SPH_FLAG_ALL_PAIRS)) return false;
    return (uint64_t) m * m * m * ctot_ref < (1ull << 31);
}

// Validates the parameters and scenes and fills the host side of a context (scenes, cells,
// capacity, tune); no CUDA call. Errors are reported as create errors (sph_last_error(NULL)).
int parse_config(const sph_params *p, uint32_t n_scenes, const sph_scene_desc *scenes, sph_ctx *c)
{
    if (!p || !scenes || n_scenes == 0) return fail(nullptr, SPH_ERR_ARG, "params/scenes missing or n_scenes == 0");
    if (p->struct_size != sizeof(sph_params)) return fail(nullptr, SPH_ERR_ARG, "sph_params.struct_size mismatch");
    if (!(p->h > 0) || !(p->dt > 0) || !(p->mass > 0)) return fail(nullptr, SPH_ERR_ARG, "h, dt and mass must be > 0");
    if (p->precision != SPH_PLAIN_F32 && p->precision != SPH_F64 && p->precision != SPH_MIXED)
        return fail(nullptr, SPH_ERR_UNSUPPORTED, "unknown precision form");
    const bool all_pairs = (p->flags & SPH_FLAG_ALL_PAIRS) != 0;
    if (all_pairs && p->precision == SPH_MIXED)
        return fail(nullptr, SPH_ERR_UNSUPPORTED, "the all-pairs form has no mixed-precision variant");
    for (uint32_t s = 0; all_pairs && s < n_scenes; s++)
        if (scenes[s].max_particles > kAllPairsMax)
            return fail(nullptr, SPH_ERR_CAPACITY, "scene " + std::to_string(s) + ": the all-pairs form takes at most " +
                                                       std::to_string(kAllPairsMax) + " particles per scene");
    c->prm = *p;
    if (p->precision == SPH_MIXED) {  // the mixed form's own launch forms
        c->tune.density_p = 0;
        c->tune.forces_mode = 0;
    }
    if (all_pairs) {  // both passes over every particle of the scene; no variants to choose
        c->tune.density_p = Tune::ALL_PAIRS;
        c->tune.forces_mode = Tune::ALL_PAIRS;
        c->tune_pinned = true;
    }
    c->device = p->device;
    uint64_t ctot = 0, ncap = 0;
    for (uint32_t s = 0; s < n_scenes; s++) {
        const sph_scene_desc &d = scenes[s];
        SceneHost h{};
        for (int a = 0; a < 3; a++) {
            if (!(d.box[a] > 0) || !std::isfinite(d.box[a]))
                return fail(nullptr, SPH_ERR_ARG, "scene " + std::to_string(s) + ": box extents must be finite and > 0");
            h.box[a] = d.box[a];
            h.res[a] = (int32_t) std::ceil(d.box[a] / p->h);  // float division, then ceil
            h.gravity[a] = p->gravity[a];
        }
        const uint64_t nc = (uint64_t) h.res[0] * h.res[1] * h.res[2];
        h.cell_base = (uint32_t) ctot;
        h.ncells = (uint32_t) nc;
        h.cap = d.max_particles;
        h.count = 0;
        if (d.n_obstacles && !d.obstacles)
            return fail(nullptr, SPH_ERR_ARG, "scene " + std::to_string(s) + ": obstacles pointer is NULL");
        for (uint32_t o = 0; o < d.n_obstacles; o++) {
            ObstacleDev ob{};
            for (int a = 0; a < 3; a++) {
                ob.lo[a] = d.obstacles[6 * o + a];
                ob.hi[a] = d.obstacles[6 * o + 3 + a];
            }
            h.obs.push_back(ob);
        }
        ctot += nc;
        ncap += d.max_particles;
        c->sc.push_back(h);
    }
    if (ctot >= (1ull << 31) || ncap >= (1ull << 31) || ncap == 0)
        return fail(nullptr, SPH_ERR_ARG, "total cells and particle capacity must be in [1, 2^31)");
    c->ctot = ctot;
    c->ctot_ref = ctot;
    // room for the grid of cells h/2 where this form can use it (plain FP32 and mixed grid forms)
    c->ctot_cap = cell_mult_allowed(c, 2, ctot) ? kMaxCellMult * kMaxCellMult * kMaxCellMult * ctot : ctot;
    c->ncap = ncap;
    return SPH_OK;
}

int create_common(const sph_params *p, uint32_t n_scenes, const sph_scene_desc *scenes, sph_ctx **out)
{
    if (!out) return fail(nullptr, SPH_ERR_ARG, "out is NULL");
    *out = nullptr;
    sph_ctx *c = new (std::nothrow) sph_ctx();
    if (!c) return fail(nullptr, SPH_ERR_NOMEM, "host allocation failed");
    int prc = parse_config(p, n_scenes, scenes, c);
    if (prc) {
        delete c;
        return prc;
    }
    {
        std::vector<PoolItem> items;
        const uint64_t need = pool_layout(c, items), limit = memory_limit();
        c->b = DevBufs{};
        if (limit && need > limit) {
            delete c;
            return fail(nullptr, SPH_ERR_NOMEM, "the context needs " + std::to_string(need) +
                                                    " bytes of device memory, above SPH_DEVICE_MEMORY_LIMIT (" +
                                                    std::to_string(limit) + ")");
        }
    }
    cudaError_t e = cudaSetDevice(c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e != cudaSuccess) {
        std::string m = std::string("CUDA device ") + std::to_string(c->device) + " unavailable: " + cudaGetErrorString(e);
        delete c;
        return fail(nullptr, SPH_ERR_CUDA, m);
    }
    for (auto &ev : c->ev) cudaEventCreate(&ev);
    cudaDeviceProp prop{};
    if (cudaGetDeviceProperties(&prop, c->device) == cudaSuccess) {
        char buf[512];
        std::snprintf(buf, sizeof buf, "%s (CUDA sm_%d%d, %d SMs)", prop.name, prop.major, prop.minor,
                      prop.multiProcessorCount);
        c->devname = buf;
    }
    int rc = allocate(c);
    if (rc == SPH_OK) rc = upload_scenes(c);
    if (rc == SPH_OK) rc = upload_scene_off(c);
    if (rc == SPH_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) rc = fail(c, SPH_ERR_CUDA, "setup failed");
    if (rc != SPH_OK) {
        g_create_error = c->err;
        sph_destroy(c);
        return rc;
    }
    *out = c;
    return SPH_OK;
}

template <class R>
int run_grid(sph_ctx *c)
{
    CK(c, Launch<R>::scan(c->b, (uint32_t) c->ctot, c->stream));
    if (is_mixed(c)) {
        CK(c, launch_slot(c->b, c->n, (uint32_t) c->ctot, c->stream));
        CK(c, mixed_permute(c->b, c->n, make_consts<float>(c, c->tune.cell_mult), make_mix(c->prm), c->stream));
    } else {
        CK(c, Launch<R>::permute(c->b, c->n, (uint32_t) c->ctot, c->stream));
    }
    return SPH_OK;
}
template <class R>
int run_density(sph_ctx *c)
{
    if (is_mixed(c))
        CK(c, mixed_density(c->b, c->n, make_consts<float>(c, c->tune.cell_mult), make_mix(c->prm),
                            c->tune.cell_mult, c->stream));
    else CK(c, Launch<R>::density(c->b, c->n, make_consts<R>(c, c->tune.cell_mult), c->tune, c->stream));
    return SPH_OK;
}
template <class R>
int run_forces(sph_ctx *c)
{
    const bool rec = (c->prm.flags & SPH_FLAG_RECORD_ACC) != 0;
    if (is_mixed(c))
        CK(c, mixed_forces(c->b, c->n, make_consts<float>(c, c->tune.cell_mult), make_mix(c->prm), rec,
                           c->tune.forces_mode, c->tune.cell_mult, c->stream));
    else CK(c, Launch<R>::forces(c->b, c->n, make_consts<R>(c, c->tune.cell_mult), rec, c->tune, c->stream));
    return SPH_OK;
}

int pass_grid(sph_ctx *c)
{
    if (c->state != HASHED) return fail(c, SPH_ERR_STATE, "grid pass needs hashed particles (upload first)");
    int rc = is_f64(c) ? run_grid<double>(c) : run_grid<float>(c);
    if (rc) return rc;
    c->state = SORTED;
    c->n_sorted = c->n;
    c->appended = false;
    return SPH_OK;
}
int pass_density(sph_ctx *c)
{
    if (c->state != SORTED) return fail(c, SPH_ERR_STATE, "density pass must follow the grid pass");
    int rc = is_f64(c) ? run_density<double>(c) : run_density<float>(c);
    if (rc) return rc;
    c->state = DENSE;
    c->n_dense = c->n;
    return SPH_OK;
}
int pass_forces(sph_ctx *c)
{
    if (c->state != DENSE) return fail(c, SPH_ERR_STATE, "force pass must follow the density pass");
    int rc = is_f64(c) ? run_forces<double>(c) : run_forces<float>(c);
    if (rc) return rc;
    c->state = HASHED;
    c->n_forced = c->n;
    return SPH_OK;
}

int one_step(sph_ctx *c)
{
    int rc = pass_grid(c);
    if (!rc) rc = pass_density(c);
    if (!rc) rc = pass_forces(c);
    return rc;
}

// Steps per captured graph: small scenes are launch-bound, so one graph holds several steps.
int graph_unroll(uint32_t n) { return n < 262144 ? 8 : 2; }

int build_graph(sph_ctx *c, int steps)
{
    drop_graph(c);
    CK(c, cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    int rc = SPH_OK;
    for (int k = 0; k < steps && rc == SPH_OK; k++) rc = one_step(c);
    cudaGraph_t g = nullptr;
    cudaError_t e = cudaStreamEndCapture(c->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (e != cudaSuccess) return cuda_fail(c, e, "cudaStreamEndCapture");
    e = cudaGraphInstantiate(&c->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) {
        c->graph = nullptr;
        return cuda_fail(c, e, "cudaGraphInstantiate");
    }
    c->graph_steps = steps;
    c->graph_n = c->n;
    c->graph_forces = c->tune.forces_mode;
    return SPH_OK;
}

float elapsed(cudaEvent_t a, cudaEvent_t b)
{
    float ms = 0;
    if (cudaEventElapsedTime(&ms, a, b) != cudaSuccess) ms = 0;
    return ms;
}

// ---- online tuning: the mask-driven force variants compute the same bits, so real steps can
// try each in turn. The candidates are four record-reading variants of one kernel (7: no
// register cap, blocks of 256 threads; 9: 40 registers, blocks of 256; 10 and 11: 40 and 48
// registers, blocks of 128), whose order depends on how latency-bound the pass is: the
// collapsing dam break settles on 9 or 10, the dense fountain on 7. Every online_period steps, one step runs with each candidate,
// timed from the start of its grid pass to the end of its force pass; the fastest is kept
// until the next trial. A trial step waits for its own end (one host synchronisation per
// candidate).
// The mixed form's candidates are its four launch forms (blocks of 128 or 256 threads, with and
// without a 48-register cap).
constexpr int kOnlineCand[kOnlineN] = {7, 9, 10, 11};
constexpr int kOnlineCandMixed[kOnlineN] = {0, 1, 2, 3};
static_assert(kOnlineN == kMixedVariants, "every mixed variant is an online candidate");

int online_candidate(const sph_ctx *c, int k) { return is_mixed(c) ? kOnlineCandMixed[k] : kOnlineCand[k]; }

bool online_active(const sph_ctx *c)
{
    if (c->online_period <= 0) return false;
    return is_mixed(c) || (c->tune.forces_mode >= 3 && c->tune.forces_mode <= 11);
}

// before a step: start a due trial and set this step's candidate
int set_cell_mult(sph_ctx *c, int m);
bool cell_mult_allowed(const sph_ctx *c, int m, uint64_t ctot_ref);

// A trial period times the form's four variants on the current cell multiple and, unless the
// multiple was set by the caller, the other multiple once (with the variant its last trials
// kept): the column's state decides which grid is faster, and it changes over a run.
int online_begin_step(sph_ctx *c)
{
    if (!online_active(c)) return SPH_OK;
    if (c->trial < 0 && c->steps_run % (uint64_t) c->online_period == 0) {
        c->trial = 0;
        c->n_trials = 0;
        const int m = c->tune.cell_mult;
        for (int k = 0; k < kOnlineN; k++, c->n_trials++) {
            c->trial_m[c->n_trials] = m;
            c->trial_v[c->n_trials] = online_candidate(c, k);
        }
        const int other = m == 1 ? 2 : 1;
        if (!c->cell_pinned && cell_mult_allowed(c, other, c->ctot_ref)) {
            c->trial_m[c->n_trials] = other;
            c->trial_v[c->n_trials] = is_mixed(c) ? std::min(c->last_best_v[other], kMixedVariants - 1)
                                                  : std::max(7, c->last_best_v[other]);
            c->n_trials++;
        }
    }
    if (c->trial < 0) return SPH_OK;
    if (c->trial_m[c->trial] != c->tune.cell_mult) {  // re-hash into the other grid (not timed)
        const int rc = set_cell_mult(c, c->trial_m[c->trial]);
        if (rc) return rc;
    }
    c->tune.forces_mode = c->trial_v[c->trial];
    CK(c, cudaEventRecord(c->on_ev[0], c->stream));
    return SPH_OK;
}

// after a step: time a trial step; after the last candidate keep the fastest
int online_end_step(sph_ctx *c)
{
    c->steps_run++;
    if (c->trial < 0 || !online_active(c)) return SPH_OK;
    CK(c, cudaEventRecord(c->on_ev[1], c->stream));
    CK(c, cudaEventSynchronize(c->on_ev[1]));
    c->trial_ms[c->trial] = elapsed(c->on_ev[0], c->on_ev[1]);
    if (++c->trial < c->n_trials) return SPH_OK;
    int best = 0;
    for (int k = 1; k < c->n_trials; k++)
        if (c->trial_ms[k] < c->trial_ms[best]) best = k;
    // the best variant of each multiple tried, for that multiple's next trial
    for (int m = 1; m <= 2; m++) {
        int bm = -1;
        for (int k = 0; k < c->n_trials; k++)
            if (c->trial_m[k] == m && (bm < 0 || c->trial_ms[k] < c->trial_ms[bm])) bm = k;
        if (bm >= 0) c->last_best_v[m] = c->trial_v[bm];
    }
    c->trial = -1;
    if (c->trial_m[best] != c->tune.cell_mult) {
        const int rc = set_cell_mult(c, c->trial_m[best]);
        if (rc) return rc;
    }
    c->tune.forces_mode = c->trial_v[best];
    return SPH_OK;
}

bool valid_density(int v) { return v == 0 || v == 1 || v == 2 || v == 4; }
bool valid_forces(int v) { return v >= 0 && v <= 11; }
// the mixed form has its own force variants and one density pass (density variant 0); cells of
// h/2 run the plain form's record variants 7 to 11
bool valid_variant(const sph_ctx *c, int dv, int fv, int cell_mult)
{
    if (is_mixed(c)) return dv == 0 && fv >= 0 && fv < kMixedVariants;
    if (cell_mult == 2) return dv == 0 && fv >= 7 && fv <= 11;
    return valid_density(dv) && valid_forces(fv);
}

int bucket_of(uint64_t n)
{
    int b = 0;
    while (n > 1) {
        n >>= 1;
        b++;
    }
    return b;
}

std::string tune_cache_path()
{
    const char *env = std::getenv("SPH_TUNE_CACHE");
    if (env && *env) return env;
    const char *home = std::getenv("HOME");
    return std::string(home && *home ? home : "/tmp") + "/.cache/sph_gb300/tune.txt";
}

std::string tune_key(const sph_ctx *c, uint64_t n)
{
    std::string dev = c->devname;
    for (auto &ch : dev)
        if (ch == ' ' || ch == '|') ch = '_';
    return dev + "|p" + std::to_string(c->prm.precision) + "|b" + std::to_string(bucket_of(n));
}

// cached (density, forces, cell multiple) choice for key, if any; lines are "key d f m" (a line
// without m is cell multiple 1)
bool tune_lookup(const sph_ctx *c, const std::string &key, int &dv, int &fv, int &mv)
{
    std::ifstream f(tune_cache_path());
    std::string line;
    bool found = false;
    while (std::getline(f, line)) {
        std::istringstream is(line);
        std::string k;
        int d, fo, m = 1;
        if (!(is >> k >> d >> fo) || k != key) continue;
        if (!(is >> m)) m = 1;
        if (cell_mult_allowed(c, m, c->ctot_ref) && valid_variant(c, d, fo, m)) {
            dv = d;
            fv = fo;
            mv = m;
            found = true;  // the last entry wins
        }
    }
    return found;
}

void tune_store(const std::string &key, int dv, int fv, int mv)
{
    const std::string path = tune_cache_path();
    for (size_t p = path.find('/', 1); p != std::string::npos; p = path.find('/', p + 1))
        mkdir(path.substr(0, p).c_str(), 0755);
    std::ofstream f(path, std::ios::app);
    if (f) f << key << " " << dv << " " << fv << " " << mv << "\n";
}


// Switches the step grid to cells of h / m: the scenes' descriptors, the counts, and the cell of
// every held particle (the *_u arrays) in the new grid. Only between steps. Cells of h/2 run the
// record variants of the plain form (7 to 11); another plain variant becomes 10.
int set_cell_mult(sph_ctx *c, int m)
{
    if (m == c->tune.cell_mult) return SPH_OK;
    drop_graph(c);
    c->tune.cell_mult = m;
    if (m == 2 && !is_mixed(c) && c->tune.forces_mode < 7) {
        c->tune.density_p = 0;
        c->tune.forces_mode = 10;
    }
    int rc = upload_scenes(c);  // also sets c->ctot
    if (rc) return rc;
    if (int rc2 = clear_counts(c, c->ctot)) return rc2;
    if (c->state == HASHED && c->n) {
        if (is_f64(c)) CK(c, Launch<double>::rehash(c->b, c->n, make_consts<double>(c, m), c->stream));
        else CK(c, Launch<float>::rehash(c->b, c->n, make_consts<float>(c, m), c->stream));
    }
    return SPH_OK;
}

// After a grid pass: the unsorted arrays refilled from the sorted state (the trial force passes
// of the autotuner overwrite them), hashed again, ready for another grid pass of the same state.
int refill_unsorted(sph_ctx *c)
{
    const size_t r4 = r4_bytes(c);
    CK(c, cudaMemcpyAsync(c->b.pos_u, c->b.pos_s, r4 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    CK(c, cudaMemcpyAsync(c->b.vel_u, c->b.vel_s, r4 * c->n, cudaMemcpyDeviceToDevice, c->stream));
    if (is_mixed(c)) CK(c, cudaMemcpyAsync(c->b.lo_u, c->b.lo_s, 16ull * c->n, cudaMemcpyDeviceToDevice, c->stream));
    if (int rc = clear_counts(c, c->ctot)) return rc;
    if (is_f64(c)) CK(c, Launch<double>::rehash(c->b, c->n, make_consts<double>(c, c->tune.cell_mult), c->stream));
    else CK(c, Launch<float>::rehash(c->b, c->n, make_consts<float>(c, c->tune.cell_mult), c->stream));
    c->state = HASHED;
    return SPH_OK;
}

}  // namespace

// =====================================================================================
extern "C" {

void sph_params_default(sph_params *p)
{
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->struct_size = sizeof(sph_params);
    p->h = 0.0457f;            // include/CParticle.h:80
    p->viscosity = 3.5f;       // :81
    p->mass = 0.02f;           // :82
    p->gas_stiffness = 3.0f;   // :83
    p->rest_density = 998.29f; // :84
    p->dt = 0.01f;             // src/CBaseParticleSimulator.cpp:7
    p->gravity[0] = 0.0f;
    p->gravity[1] = -9.80665f; // include/CBaseParticleSimulator.h:19
    p->gravity[2] = 0.0f;
    p->wall_k = 10000.0f;      // include/CCollisionGeometry.h:20
    p->wall_damping = -0.9f;   // include/CCollisionGeometry.h:21
    p->wall_radius = 0.01f;    // src/CCollisionGeometry.cpp:124
    p->precision = SPH_PLAIN_F32;
    p->flags = 0;
    p->device = 0;
}

int sph_create(const sph_params *p, const float box[3], uint32_t max_particles, sph_ctx **out)
{
    try {
        if (!box) return fail(nullptr, SPH_ERR_ARG, "box is NULL");
        sph_scene_desc d{};
        for (int a = 0; a < 3; a++) d.box[a] = box[a];
        d.max_particles = max_particles;
        return create_common(p, 1, &d, out);
    } catch (...) {
        return fail(nullptr, SPH_ERR_NOMEM, "host exception in sph_create");
    }
}

int sph_batch_create(const sph_params *p, uint32_t n_scenes, const sph_scene_desc *scenes, sph_ctx **out)
{
    try {
        return create_common(p, n_scenes, scenes, out);
    } catch (...) {
        return fail(nullptr, SPH_ERR_NOMEM, "host exception in sph_batch_create");
    }
}

int sph_debug_check(sph_ctx *c, uint32_t *flags)
{
    if (!c || !flags) return c ? fail(c, SPH_ERR_ARG, "flags is NULL") : SPH_ERR_ARG;
#ifndef SPH_CHECKED
    return fail(c, SPH_ERR_UNSUPPORTED, "this library is built without checks (libsph_gb300_checked.so has them)");
#else
    CK(c, cudaSetDevice(c->device));
    CK(c, cudaStreamSynchronize(c->stream));
    *flags = 0;
    CK(c, check_flags_kernels(flags));
    CK(c, check_flags_mixed(flags));
    CK(c, check_flags_handoff(flags));
    CK(c, check_flags_noalloc(flags));
    std::vector<unsigned char> buf(kCanaryBytes);
    for (unsigned char *g : c->canaries) {
        CK(c, cudaMemcpy(buf.data(), g, kCanaryBytes, cudaMemcpyDeviceToHost));
        for (unsigned char v : buf)
            if (v != kCanary) {
                *flags |= SPH_CHECK_CANARY;
                break;
            }
    }
    return SPH_OK;
#endif
}

int sph_memory_required(const sph_params *p, uint32_t n_scenes, const sph_scene_desc *scenes, uint64_t *bytes)
{
    if (!bytes) return fail(nullptr, SPH_ERR_ARG, "bytes is NULL");
    try {
        sph_ctx c;  // host side only: no device, no stream
        const int rc = parse_config(p, n_scenes, scenes, &c);
        if (rc) return rc;
        std::vector<PoolItem> items;
        *bytes = pool_layout(&c, items);
        return SPH_OK;
    } catch (...) {
        return fail(nullptr, SPH_ERR_NOMEM, "host exception in sph_memory_required");
    }
}

void sph_destroy(sph_ctx *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    if (c->ho_stream) cudaStreamSynchronize(c->ho_stream);
    drop_graph(c);
    for (auto &ev : c->ev)
        if (ev) cudaEventDestroy(ev);
    for (cudaEvent_t ev : {c->ho_ready, c->ho_done, c->ho_export, c->on_ev[0], c->on_ev[1]})
        if (ev) cudaEventDestroy(ev);
    if (c->ho_stream) cudaStreamDestroy(c->ho_stream);
    if (c->ho_xyz) cudaFree(c->ho_xyz);
    if (c->ho_vel) cudaFree(c->ho_vel);
    if (c->pool) cudaFree(c->pool);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

const char *sph_last_error(const sph_ctx *c) { return c ? c->err.c_str() : g_create_error.c_str(); }

const char *sph_device_name(const sph_ctx *c) { return c ? c->devname.c_str() : ""; }

void *sph_stream(const sph_ctx *c) { return c ? (void *) c->stream : nullptr; }

int sph_upload(sph_ctx *c, const float *xyz, const float *vel, const uint32_t *counts)
{
    if (!c) return SPH_ERR_ARG;
    try {
        if (!counts) return fail(c, SPH_ERR_ARG, "counts is NULL");
        uint64_t total = 0;
        for (size_t s = 0; s < c->sc.size(); s++) {
            if (counts[s] > c->sc[s].cap)
                return fail(c, SPH_ERR_CAPACITY, "scene " + std::to_string(s) + ": " + std::to_string(counts[s]) +
                                                     " particles exceed its capacity " + std::to_string(c->sc[s].cap));
            total += counts[s];
        }
        if (total && !xyz) return fail(c, SPH_ERR_ARG, "xyz is NULL");
        CK(c, cudaSetDevice(c->device));
        drop_graph(c);
        for (size_t s = 0; s < c->sc.size(); s++) c->sc[s].count = counts[s];
        c->n = (uint32_t) total;
        // the cached choice of this particle-count bucket, its cell multiple before the hash
        int dv, fv, mv;
        if (!c->tune_pinned && tune_lookup(c, tune_key(c, total), dv, fv, mv)) {
            c->state = EMPTY;
            int rc = set_cell_mult(c, mv);
            if (rc) return rc;
            c->tune.density_p = dv;
            c->tune.forces_mode = fv;
        }
        int rc = upload_scene_off(c);
        if (rc) return rc;
        if (int rc2 = clear_counts(c, c->ctot)) return rc2;
        if (total) {
            if (is_mixed(c)) CK(c, cudaMemsetAsync(c->b.lo_u, 0, 16 * total, c->stream));
            // pinned caller arrays are read by the ingest kernel itself; others go through staging
            const float *sx = (const float *) pinned_view(xyz);
            const float *sv = vel ? (const float *) pinned_view(vel) : nullptr;
            if (!sx || (vel && !sv)) {
                CK(c, cudaMemcpyAsync(c->b.st_xyz, xyz, 12 * total, cudaMemcpyHostToDevice, c->stream));
                if (vel) CK(c, cudaMemcpyAsync(c->b.st_vel, vel, 12 * total, cudaMemcpyHostToDevice, c->stream));
                sx = c->b.st_xyz;
                sv = vel ? c->b.st_vel : nullptr;
            }
            if (is_f64(c))
                CK(c, Launch<double>::ingest(c->b, sx, sv, 0, c->n, -1, 0, (uint32_t) c->sc.size(),
                                             make_consts<double>(c, c->tune.cell_mult), c->stream));
            else
                CK(c, Launch<float>::ingest(c->b, sx, sv, 0, c->n, -1, 0, (uint32_t) c->sc.size(),
                                            make_consts<float>(c, c->tune.cell_mult), c->stream));
        }
        c->state = HASHED;
        c->n_sorted = 0;
        c->n_forced = 0;
        c->n_dense = 0;
        c->appended = false;
        return SPH_OK;
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_upload");
    }
}

namespace {

// checks shared by the two append paths
int append_check(sph_ctx *c, uint32_t scene, uint32_t n)
{
    if (scene >= c->sc.size()) return fail(c, SPH_ERR_ARG, "scene index out of range");
    if (n == 0) return SPH_OK;
    if (c->state != HASHED) return fail(c, SPH_ERR_STATE, "append needs a completed step (or an upload) first");
    const SceneHost &h = c->sc[scene];
    if ((uint64_t) h.count + n > h.cap)
        return fail(c, SPH_ERR_CAPACITY, "scene " + std::to_string(scene) + " would exceed its capacity");
    return SPH_OK;
}

// ingest n particles from the staging arrays as the tail of the scene
int append_ingest(sph_ctx *c, uint32_t scene, uint32_t n, bool has_vel)
{
    SceneHost &h = c->sc[scene];
    if (is_mixed(c)) CK(c, cudaMemsetAsync((char *) c->b.lo_u + 16ull * c->n, 0, 16ull * n, c->stream));
    if (is_f64(c))
        CK(c, Launch<double>::ingest(c->b, c->b.st_xyz, has_vel ? c->b.st_vel : nullptr, c->n, n, (int32_t) scene,
                                     h.count, (uint32_t) c->sc.size(), make_consts<double>(c, c->tune.cell_mult), c->stream));
    else
        CK(c, Launch<float>::ingest(c->b, c->b.st_xyz, has_vel ? c->b.st_vel : nullptr, c->n, n, (int32_t) scene,
                                    h.count, (uint32_t) c->sc.size(), make_consts<float>(c, c->tune.cell_mult), c->stream));
    h.count += n;
    c->n += n;
    c->appended = true;
    return SPH_OK;
}

}  // namespace

int sph_append(sph_ctx *c, uint32_t scene, const float *xyz, const float *vel, uint32_t n)
{
    if (!c) return SPH_ERR_ARG;
    if (n != 0 && !xyz) return fail(c, SPH_ERR_ARG, "xyz is NULL");
    int rc = append_check(c, scene, n);
    if (rc || n == 0) return rc;
    CK(c, cudaSetDevice(c->device));
    drop_graph(c);
    CK(c, cudaMemcpyAsync(c->b.st_xyz, xyz, 12ull * n, cudaMemcpyHostToDevice, c->stream));
    if (vel) CK(c, cudaMemcpyAsync(c->b.st_vel, vel, 12ull * n, cudaMemcpyHostToDevice, c->stream));
    rc = append_ingest(c, scene, n, vel != nullptr);
    if (rc) return rc;
    // the caller may reuse or free its host arrays once this returns
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

int sph_emit_fountain(sph_ctx *c, uint32_t scene, uint64_t seed, uint32_t step, uint32_t n, const float center[3],
                      float radius, float speed, float sigma)
{
    if (!c) return SPH_ERR_ARG;
    if (!center) return fail(c, SPH_ERR_ARG, "center is NULL");
    int rc = append_check(c, scene, n);
    if (rc || n == 0) return rc;
    CK(c, cudaSetDevice(c->device));
    drop_graph(c);
    CK(c, launch_emit_fountain(seed, step, n, center, radius, speed, sigma, c->b.st_xyz, c->b.st_vel, c->stream));
    return append_ingest(c, scene, n, true);
}

int sph_set_gravity(sph_ctx *c, int32_t scene, const float g[3])
{
    if (!c || !g) return c ? fail(c, SPH_ERR_ARG, "gravity is NULL") : SPH_ERR_ARG;
    if (scene >= (int32_t) c->sc.size()) return fail(c, SPH_ERR_ARG, "scene index out of range");
    for (size_t s = 0; s < c->sc.size(); s++)
        if (scene < 0 || (size_t) scene == s)
            for (int a = 0; a < 3; a++) c->sc[s].gravity[a] = g[a];
    CK(c, cudaSetDevice(c->device));
    return upload_scenes(c);
}

// Pass-by-pass calls. With SPH_FLAG_PROFILE each records CUDA events around its work and waits
// for its own end, so that its time (sProfilingEvent's grid, density or forces field) is known
// when the call returns, as each pass of the reference returns its own profiled duration
// (src/CBaseParticleSimulator.cpp:116-144).
int sph_pass_grid(sph_ctx *c)
{
    if (!c) return SPH_ERR_ARG;
    CK(c, cudaSetDevice(c->device));
    const bool prof = (c->prm.flags & SPH_FLAG_PROFILE) != 0;
    int rc = c->state == HASHED ? online_begin_step(c) : SPH_OK;
    if (rc) return rc;
    if (prof) CK(c, cudaEventRecord(c->ev[0], c->stream));
    rc = pass_grid(c);
    if (!rc && prof) {
        CK(c, cudaEventRecord(c->ev[1], c->stream));
        CK(c, cudaEventSynchronize(c->ev[1]));
        c->ms[0] = elapsed(c->ev[0], c->ev[1]);
    }
    return rc;
}
int sph_pass_density(sph_ctx *c)
{
    if (!c) return SPH_ERR_ARG;
    CK(c, cudaSetDevice(c->device));
    int rc = pass_density(c);
    if (!rc && (c->prm.flags & SPH_FLAG_PROFILE)) {
        CK(c, cudaEventRecord(c->ev[2], c->stream));
        CK(c, cudaEventSynchronize(c->ev[2]));
        c->ms[1] = elapsed(c->ev[1], c->ev[2]);
    }
    return rc;
}
int sph_pass_forces(sph_ctx *c)
{
    if (!c) return SPH_ERR_ARG;
    CK(c, cudaSetDevice(c->device));
    int rc = pass_forces(c);
    if (!rc && (c->prm.flags & SPH_FLAG_PROFILE)) {
        CK(c, cudaEventRecord(c->ev[3], c->stream));
        CK(c, cudaEventSynchronize(c->ev[3]));
        c->ms[2] = elapsed(c->ev[2], c->ev[3]);
        c->ms[3] = 0;
        c->ms[4] = 0;
    }
    if (!rc) rc = online_end_step(c);
    return rc;
}

int sph_step(sph_ctx *c, int32_t nsteps)
{
    if (!c) return SPH_ERR_ARG;
    if (nsteps < 0) return fail(c, SPH_ERR_ARG, "nsteps < 0");
    if (c->state != HASHED) return fail(c, SPH_ERR_STATE, "step needs uploaded particles and no pass in progress");
    CK(c, cudaSetDevice(c->device));
    if (c->prm.flags & SPH_FLAG_PROFILE) {
        for (int k = 0; k < nsteps; k++) {
            int rc = online_begin_step(c);
            if (rc) return rc;
            CK(c, cudaEventRecord(c->ev[0], c->stream));
            rc = pass_grid(c);
            if (rc) return rc;
            CK(c, cudaEventRecord(c->ev[1], c->stream));
            rc = pass_density(c);
            if (rc) return rc;
            CK(c, cudaEventRecord(c->ev[2], c->stream));
            rc = pass_forces(c);
            if (rc) return rc;
            CK(c, cudaEventRecord(c->ev[3], c->stream));
            rc = online_end_step(c);
            if (rc) return rc;
        }
        if (nsteps > 0) {
            CK(c, cudaEventSynchronize(c->ev[3]));
            c->ms[0] = elapsed(c->ev[0], c->ev[1]);
            c->ms[1] = elapsed(c->ev[1], c->ev[2]);
            c->ms[2] = elapsed(c->ev[2], c->ev[3]);
            c->ms[3] = 0;
            c->ms[4] = 0;
        }
        return SPH_OK;
    }
    const int unroll = graph_unroll(c->n);
    int done = 0;
    while (done < nsteps) {
        // trial steps of the online tuning run one by one, outside the graph
        if (online_active(c) && (c->trial >= 0 || c->steps_run % (uint64_t) c->online_period == 0)) {
            int rc = online_begin_step(c);
            if (!rc) rc = one_step(c);
            if (!rc) rc = online_end_step(c);
            if (rc) return rc;
            done++;
            continue;
        }
        int chunk = nsteps - done;
        if (online_active(c))
            chunk = (int) std::min<uint64_t>((uint64_t) chunk,
                                             c->online_period - c->steps_run % (uint64_t) c->online_period);
        int k = 0;
        if (chunk >= unroll) {
            if (!c->graph || c->graph_steps != unroll || c->graph_n != c->n || c->graph_forces != c->tune.forces_mode) {
                int rc = build_graph(c, unroll);
                if (rc) return rc;
                c->state = HASHED;
            }
            for (; chunk - k >= unroll; k += unroll) CK(c, cudaGraphLaunch(c->graph, c->stream));
            c->n_sorted = c->n_dense = c->n_forced = c->n;
            c->appended = false;
        }
        for (; k < chunk; k++) {
            int rc = one_step(c);
            if (rc) return rc;
        }
        c->steps_run += (uint64_t) chunk;
        done += chunk;
    }
    CK(c, cudaGetLastError());
    return SPH_OK;
}

int sph_set_online_tuning(sph_ctx *c, int32_t period)
{
    if (!c) return SPH_ERR_ARG;
    if (period != 0 && period < kOnlineN) return fail(c, SPH_ERR_ARG, "period must be 0 (off) or at least 4 steps");
    if (period && (c->prm.flags & SPH_FLAG_ALL_PAIRS))
        return fail(c, SPH_ERR_STATE, "this context has no force variants to tune");
    if (c->trial >= 0) return fail(c, SPH_ERR_STATE, "a tuning trial is in progress");
    CK(c, cudaSetDevice(c->device));
    for (auto &ev : c->on_ev)
        if (!ev) CK(c, cudaEventCreate(&ev));
    c->online_period = period;
    return SPH_OK;
}

int sph_set_variant(sph_ctx *c, int32_t density_variant, int32_t forces_variant)
{
    if (!c) return SPH_ERR_ARG;
    if (c->prm.flags & SPH_FLAG_ALL_PAIRS) return fail(c, SPH_ERR_STATE, "an all-pairs context has no launch variants");
    if (!valid_variant(c, density_variant, forces_variant, c->tune.cell_mult))
        return fail(c, SPH_ERR_ARG, is_mixed(c) ? "unknown launch variant (mixed form: density 0, forces 0-3)"
                                    : c->tune.cell_mult == 2 ? "unknown launch variant (cells of h/2: density 0, forces 7-11)"
                                                             : "unknown launch variant");
    c->tune.density_p = density_variant;
    c->tune.forces_mode = forces_variant;
    c->tune_pinned = true;
    drop_graph(c);
    return SPH_OK;
}

int sph_get_variant(const sph_ctx *c, int32_t out[2])
{
    if (!c || !out) return SPH_ERR_ARG;
    out[0] = c->tune.density_p;
    out[1] = c->tune.forces_mode;
    return SPH_OK;
}

int sph_autotune(sph_ctx *c, int32_t reps)
{
    if (!c) return SPH_ERR_ARG;
    if (reps < 1) return fail(c, SPH_ERR_ARG, "reps must be >= 1");
    if (c->prm.flags & SPH_FLAG_ALL_PAIRS) return fail(c, SPH_ERR_STATE, "an all-pairs context has no launch variants");
    if (c->state != HASHED) return fail(c, SPH_ERR_STATE, "autotune needs a completed step (or an upload)");
    if (c->n == 0) return fail(c, SPH_ERR_STATE, "autotune needs particles");
    CK(c, cudaSetDevice(c->device));
    drop_graph(c);
    // every (cell multiple, density, forces) choice on the same state: per cell multiple the grid
    // pass once, then each (density, forces) pair timed as density + forces on its sorted state;
    // the choice minimises grid + density + forces. Between cell multiples the unsorted arrays are
    // refilled from the sorted starting state (the trials' force passes overwrote them).
    struct Cfg { int d, f; };
    float best = 1e30f;
    int bm = c->tune.cell_mult, bd = c->tune.density_p, bf = c->tune.forces_mode;
    // a cell multiple set with sph_set_cell_multiple stays; else both are tried
    std::vector<int> mults = {c->tune.cell_mult};
    if (!c->cell_pinned)
        for (int m = 1; m <= kMaxCellMult; m++)
            if (m != c->tune.cell_mult && cell_mult_allowed(c, m, c->ctot_ref)) mults.push_back(m);
    for (size_t mi = 0; mi < mults.size(); mi++) {
        const int m = mults[mi];
        if (mi > 0) {
            int rc = refill_unsorted(c);
            if (!rc) rc = set_cell_mult(c, m);
            if (rc) return rc;
        } else if (m != c->tune.cell_mult) {
            int rc = set_cell_mult(c, m);
            if (rc) return rc;
        }
        CK(c, cudaEventRecord(c->ev[0], c->stream));
        int rc = pass_grid(c);
        if (rc) return rc;
        CK(c, cudaEventRecord(c->ev[1], c->stream));
        CK(c, cudaEventSynchronize(c->ev[1]));
        const float grid_ms = elapsed(c->ev[0], c->ev[1]);
        std::vector<Cfg> cfgs;
        if (is_mixed(c)) {
            for (int f = 0; f < kMixedVariants; f++) cfgs.push_back({0, f});
        } else if (m == 2) {
            for (int f = 7; f <= 11; f++) cfgs.push_back({0, f});
        } else {
            for (int d : {0, 1, 2, 4})
                for (int f = 0; f <= 2; f++) cfgs.push_back({d, f});
            for (int f = 3; f <= 11; f++) cfgs.push_back({0, f});
        }
        for (const Cfg &g : cfgs) {
            c->tune.density_p = g.d;
            c->tune.forces_mode = g.f;
            for (int r = 0; r <= reps; r++) {  // the first run is a warm-up
                if (int rc2 = clear_counts(c, c->ctot)) return rc2;  // the force pass adds to the counts
                CK(c, cudaEventRecord(c->ev[0], c->stream));
                c->state = SORTED;
                rc = pass_density(c);
                if (!rc) rc = pass_forces(c);
                if (rc) return rc;
                CK(c, cudaEventRecord(c->ev[1], c->stream));
                CK(c, cudaEventSynchronize(c->ev[1]));
                const float ms = grid_ms + elapsed(c->ev[0], c->ev[1]);
                if (r > 0 && ms < best) {
                    best = ms;
                    bm = m;
                    bd = g.d;
                    bf = g.f;
                }
            }
        }
    }
    // the step itself, with the chosen cell multiple and variants, from the starting state
    if (bm != c->tune.cell_mult) {
        int rc = refill_unsorted(c);
        if (!rc) rc = set_cell_mult(c, bm);
        if (!rc) rc = pass_grid(c);
        if (rc) return rc;
    }
    c->tune.density_p = bd;
    c->tune.forces_mode = bf;
    if (int rc2 = clear_counts(c, c->ctot)) return rc2;
    c->state = SORTED;
    int rc = pass_density(c);
    if (!rc) rc = pass_forces(c);
    if (rc) return rc;
    c->tune_pinned = true;
    c->steps_run++;  // the step above was a real one
    tune_store(tune_key(c, c->n), bd, bf, bm);
    return SPH_OK;
}

int sph_set_cell_multiple(sph_ctx *c, int32_t m)
{
    if (!c) return SPH_ERR_ARG;
    if (m != 1 && m != 2) return fail(c, SPH_ERR_ARG, "the cell multiple is 1 (cells of h) or 2 (cells of h/2)");
    if (!cell_mult_allowed(c, m, c->ctot_ref))
        return fail(c, SPH_ERR_UNSUPPORTED, "cells of h/2 are for the plain FP32 and mixed grid forms");
    if (c->state != HASHED && c->state != EMPTY)
        return fail(c, SPH_ERR_STATE, "the cell multiple changes between steps (not between passes)");
    CK(c, cudaSetDevice(c->device));
    const int rc = set_cell_mult(c, m);
    if (!rc) c->tune_pinned = c->cell_pinned = true;
    return rc;
}

int sph_get_cell_multiple(const sph_ctx *c) { return c ? c->tune.cell_mult : SPH_ERR_ARG; }

int sph_pass_times(sph_ctx *c, double ms[5])
{
    if (!c || !ms) return SPH_ERR_ARG;
    if (!(c->prm.flags & SPH_FLAG_PROFILE)) return fail(c, SPH_ERR_STATE, "context created without SPH_FLAG_PROFILE");
    for (int k = 0; k < 5; k++) ms[k] = c->ms[k];
    return SPH_OK;
}

int sph_get_counts(const sph_ctx *c, uint32_t *counts)
{
    if (!c || !counts) return SPH_ERR_ARG;
    for (size_t s = 0; s < c->sc.size(); s++) counts[s] = c->sc[s].count;
    return SPH_OK;
}

uint32_t sph_num_scenes(const sph_ctx *c) { return c ? (uint32_t) c->sc.size() : 0; }
uint64_t sph_num_particles(const sph_ctx *c) { return c ? c->n : 0; }

int sph_get_resolution(const sph_ctx *c, uint32_t scene, int32_t res[3])
{
    if (!c || !res || scene >= c->sc.size()) return SPH_ERR_ARG;
    for (int a = 0; a < 3; a++) res[a] = c->sc[scene].res[a];
    return SPH_OK;
}

static int download_impl(sph_ctx *c, void *xyz, void *vel, void *rho, void *p, void *acc, bool f64)
{
    if (!c) return SPH_ERR_ARG;
    if (f64 ? !(is_f64(c) || is_mixed(c)) : is_f64(c))
        return fail(c, SPH_ERR_ARG, f64 ? "context is neither FP64 nor mixed" : "FP64 context: use sph_download_f64");
    if (c->state == EMPTY) return fail(c, SPH_ERR_STATE, "nothing uploaded");
    if (acc && !(c->prm.flags & SPH_FLAG_RECORD_ACC))
        return fail(c, SPH_ERR_STATE, "accelerations need SPH_FLAG_RECORD_ACC");
    CK(c, cudaSetDevice(c->device));
    int rc = upload_scene_off(c);
    if (rc) return rc;
    const int layout_sorted = (c->state == SORTED || c->state == DENSE) ? 1 : 0;
    const int aux_sorted = c->state == DENSE ? 1 : 0;
    // plain FP32 positions and velocities into pinned arrays: written there by one gather
    if (!f64 && !is_f64(c) && !is_mixed(c) && !rho && !p && !acc && (xyz || vel)) {
        float *vx = xyz ? (float *) pinned_view(xyz) : nullptr;
        float *vv = vel ? (float *) pinned_view(vel) : nullptr;
        const bool aligned = ((reinterpret_cast<uintptr_t>(vx) | reinterpret_cast<uintptr_t>(vv)) & 15u) == 0;
        if ((!xyz || vx) && (!vel || vv) && aligned) {
            CK(c, launch_gather_host<float>(c->b, c->n, layout_sorted, vx, vv, c->stream));
            CK(c, cudaStreamSynchronize(c->stream));
            return SPH_OK;
        }
    }
    const size_t rs = f64 ? 8 : 4;
    const uint32_t n = c->n;
    DevBufs &b = c->b;
    void *sx = f64 ? (void *) b.st_xyz64 : (void *) b.st_xyz;
    void *sv = f64 ? (void *) b.st_vel64 : (void *) b.st_vel;
    void *sr = f64 ? (void *) b.st_rho64 : (void *) b.st_rho;
    void *sp = f64 ? (void *) b.st_p64 : (void *) b.st_p;
    void *sa = f64 ? (void *) b.st_acc64 : (void *) b.st_acc;
    CK(c, cudaMemsetAsync(sr, 0, rs * n, c->stream));
    CK(c, cudaMemsetAsync(sp, 0, rs * n, c->stream));
    if (sa) CK(c, cudaMemsetAsync(sa, 0, 3 * rs * n, c->stream));
    // particles appended after the last grid pass have no density yet (0, as addParticle
    // sets) and no acceleration
    // aux records are indexed like the *_u arrays except right after a density pass
    const uint32_t n_aux = c->n_dense;
    const uint32_t n_acc = c->n_forced;
    if (is_mixed(c)) CK(c, mixed_egress(b, n, n_aux, n_acc, layout_sorted, aux_sorted, f64, c->stream));
    else if (f64) CK(c, Launch<double>::egress(b, n, n_aux, n_acc, layout_sorted, aux_sorted, c->stream));
    else CK(c, Launch<float>::egress(b, n, n_aux, n_acc, layout_sorted, aux_sorted, c->stream));
    if (xyz) CK(c, cudaMemcpyAsync(xyz, sx, 3 * rs * n, cudaMemcpyDeviceToHost, c->stream));
    if (vel) CK(c, cudaMemcpyAsync(vel, sv, 3 * rs * n, cudaMemcpyDeviceToHost, c->stream));
    if (rho) CK(c, cudaMemcpyAsync(rho, sr, rs * n, cudaMemcpyDeviceToHost, c->stream));
    if (p) CK(c, cudaMemcpyAsync(p, sp, rs * n, cudaMemcpyDeviceToHost, c->stream));
    if (acc) CK(c, cudaMemcpyAsync(acc, sa, 3 * rs * n, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

namespace {

// handoff stream, events and the two float3 buffers of the context's capacity
int handoff_init(sph_ctx *c)
{
    if (c->ho_stream) return SPH_OK;
    CK(c, cudaStreamCreateWithFlags(&c->ho_stream, cudaStreamNonBlocking));
    CK(c, cudaEventCreateWithFlags(&c->ho_ready, cudaEventDisableTiming));
    CK(c, cudaEventCreateWithFlags(&c->ho_done, cudaEventDisableTiming));
    CK(c, cudaEventCreateWithFlags(&c->ho_export, cudaEventDisableTiming));
    CK(c, cudaMalloc(&c->ho_xyz, 12 * c->ncap));
    CK(c, cudaMalloc(&c->ho_vel, 12 * c->ncap));
    return SPH_OK;
}

// id-ordered float3 state of every particle into xyz (and vel if not NULL), queued on the
// context's stream
int handoff_egress(sph_ctx *c, float *xyz, float *vel)
{
    int rc = upload_scene_off(c);
    if (rc) return rc;
    const int layout_sorted = (c->state == SORTED || c->state == DENSE) ? 1 : 0;
    if (is_mixed(c)) {
        DevBufs hb = c->b;
        hb.st_xyz = xyz;
        hb.st_vel = vel ? vel : c->ho_vel;
        hb.st_acc = nullptr;
        CK(c, mixed_egress(hb, c->n, 0, 0, layout_sorted, 0, false, c->stream));
    } else if (is_f64(c)) {
        CK(c, launch_handoff<double>(c->b, c->n, layout_sorted, xyz, vel, c->stream));
    } else {
        CK(c, launch_handoff<float>(c->b, c->n, layout_sorted, xyz, vel, c->stream));
    }
    return SPH_OK;
}

}  // namespace

int sph_handoff_async(sph_ctx *c, float *xyz, float *vel)
{
    if (!c) return SPH_ERR_ARG;
    if (!xyz) return fail(c, SPH_ERR_ARG, "xyz is NULL");
    if (c->state == EMPTY) return fail(c, SPH_ERR_STATE, "nothing uploaded");
    try {
        CK(c, cudaSetDevice(c->device));
        int rc = handoff_init(c);
        if (rc) return rc;
        // the previous copy must have left the handoff buffers before they are rewritten
        if (c->ho_recorded) CK(c, cudaStreamWaitEvent(c->stream, c->ho_done, 0));
        rc = handoff_egress(c, c->ho_xyz, c->ho_vel);
        if (rc) return rc;
        CK(c, cudaEventRecord(c->ho_ready, c->stream));
        CK(c, cudaStreamWaitEvent(c->ho_stream, c->ho_ready, 0));
        const size_t bytes = 12ull * c->n;
        if (bytes) {
            CK(c, cudaMemcpyAsync(xyz, c->ho_xyz, bytes, cudaMemcpyDeviceToHost, c->ho_stream));
            if (vel) CK(c, cudaMemcpyAsync(vel, c->ho_vel, bytes, cudaMemcpyDeviceToHost, c->ho_stream));
        }
        CK(c, cudaEventRecord(c->ho_done, c->ho_stream));
        c->ho_recorded = true;
        return SPH_OK;
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_handoff_async");
    }
}

int sph_handoff_ready(sph_ctx *c)
{
    if (!c) return SPH_ERR_ARG;
    if (!c->ho_recorded) return 1;
    const cudaError_t e = cudaEventQuery(c->ho_done);
    if (e == cudaSuccess) return 1;
    if (e == cudaErrorNotReady) return 0;
    return cuda_fail(c, e, "sph_handoff_ready");
}

int sph_handoff_wait(sph_ctx *c)
{
    if (!c) return SPH_ERR_ARG;
    if (!c->ho_recorded) return SPH_OK;
    CK(c, cudaEventSynchronize(c->ho_done));
    return SPH_OK;
}

int sph_export_positions(sph_ctx *c, float *dev_xyz, float *dev_vel, void *consumer_stream)
{
    if (!c) return SPH_ERR_ARG;
    if (!dev_xyz) return fail(c, SPH_ERR_ARG, "dev_xyz is NULL");
    if (c->state == EMPTY) return fail(c, SPH_ERR_STATE, "nothing uploaded");
    try {
        CK(c, cudaSetDevice(c->device));
        int rc = handoff_init(c);
        if (rc) return rc;
        rc = handoff_egress(c, dev_xyz, dev_vel);
        if (rc) return rc;
        if (consumer_stream) {
            CK(c, cudaEventRecord(c->ho_export, c->stream));
            CK(c, cudaStreamWaitEvent((cudaStream_t) consumer_stream, c->ho_export, 0));
        }
        return SPH_OK;
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_export_positions");
    }
}

int sph_splat(sph_ctx *c, uint32_t scene, int32_t axis, uint32_t width, uint32_t height, uint32_t *dev_count,
              float *dev_depth, void *consumer_stream)
{
    if (!c) return SPH_ERR_ARG;
    if (scene >= c->sc.size()) return fail(c, SPH_ERR_ARG, "scene index out of range");
    if (axis < 0 || axis > 2) return fail(c, SPH_ERR_ARG, "axis must be 0, 1 or 2");
    if (width == 0 || height == 0 || (uint64_t) width * height > (1ull << 28))
        return fail(c, SPH_ERR_ARG, "image size must be in [1, 2^28] pixels");
    if (!dev_count && !dev_depth) return fail(c, SPH_ERR_ARG, "no output image");
    if (c->state == EMPTY) return fail(c, SPH_ERR_STATE, "nothing uploaded");
    CK(c, cudaSetDevice(c->device));
    const int au = axis == 0 ? 1 : 0, av = axis == 2 ? 1 : 2;
    const SceneHost &h = c->sc[scene];
    const float half_u = h.box[au] / 2.0f, half_v = h.box[av] / 2.0f;
    const float scale_u = (float) width / h.box[au], scale_v = (float) height / h.box[av];
    const int layout_sorted = (c->state == SORTED || c->state == DENSE) ? 1 : 0;
    if (is_f64(c))
        CK(c, launch_splat<double>(c->b, c->n, layout_sorted, scene, axis, half_u, half_v, scale_u, scale_v, width,
                                   height, dev_count, dev_depth, c->stream));
    else
        CK(c, launch_splat<float>(c->b, c->n, layout_sorted, scene, axis, half_u, half_v, scale_u, scale_v, width,
                                  height, dev_count, dev_depth, c->stream));
    if (consumer_stream) {
        if (!c->ho_export) CK(c, cudaEventCreateWithFlags(&c->ho_export, cudaEventDisableTiming));
        CK(c, cudaEventRecord(c->ho_export, c->stream));
        CK(c, cudaStreamWaitEvent((cudaStream_t) consumer_stream, c->ho_export, 0));
    }
    return SPH_OK;
}

int sph_download(sph_ctx *c, float *xyz, float *vel, float *rho, float *p, float *acc)
{
    try {
        return download_impl(c, xyz, vel, rho, p, acc, false);
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_download");
    }
}

int sph_download_f64(sph_ctx *c, double *xyz, double *vel, double *rho, double *p, double *acc)
{
    try {
        return download_impl(c, xyz, vel, rho, p, acc, true);
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_download_f64");
    }
}

namespace {

// The reference's grid (cells of size h) of the current sorted state when the step runs on cells
// of h/2: per scene, the id-ordered positions go through the same grid build as
// sph_grid_build_noalloc, with working memory allocated for the call.
int get_grid_ref(sph_ctx *c, uint32_t *cell_of_particle, uint32_t *cell_counts, uint32_t *sorted_ids)
{
    const uint32_t n = c->n;
    // id-ordered float positions of the sorted state (the mixed form's hi part: its hash input)
    if (is_mixed(c)) CK(c, mixed_egress(c->b, n, 0, 0, 1, 1, false, c->stream));
    else CK(c, Launch<float>::egress(c->b, n, 0, 0, 1, 1, c->stream));
    uint64_t nmax = 1, cmax = 1;
    for (auto &h : c->sc) {
        nmax = std::max<uint64_t>(nmax, h.count);
        cmax = std::max<uint64_t>(cmax, (uint64_t) h.res[0] * h.res[1] * h.res[2]);
    }
    const uint64_t nb = cmax / kScanTile + 1;
    const uint64_t words = nmax + (cmax + 1) + nmax + cmax + nmax + nb + big_words(nmax);
    uint32_t *mem = nullptr;
    CK(c, cudaMalloc(&mem, 4 * words));
    uint32_t *d_cell = mem, *d_start = d_cell + nmax, *d_order = d_start + cmax + 1;
    GridScratch g;
    g.count = d_order + nmax;
    g.tmp = g.count + cmax;
    g.bsum = g.tmp + nmax;
    g.big = g.bsum + nb;
    uint64_t off = 0, cbase = 0;
    cudaError_t e = cudaSuccess;
    std::vector<uint32_t> cell, start, order;
    for (size_t s = 0; s < c->sc.size() && e == cudaSuccess; s++) {
        const SceneHost &h = c->sc[s];
        const uint64_t nc = (uint64_t) h.res[0] * h.res[1] * h.res[2];
        const int3 res = make_int3(h.res[0], h.res[1], h.res[2]);
        const float3 half = make_float3(h.box[0] / 2.0f, h.box[1] / 2.0f, h.box[2] / 2.0f);
        e = ref_grid_build(c->b.st_xyz + 3 * off, h.count, res, half, c->prm.h, d_cell, d_start, d_order, g, c->stream);
        cell.resize(h.count);
        order.resize(h.count);
        start.resize(nc + 1);
        if (e == cudaSuccess && h.count) e = cudaMemcpyAsync(cell.data(), d_cell, 4ull * h.count, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess && h.count) e = cudaMemcpyAsync(order.data(), d_order, 4ull * h.count, cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaMemcpyAsync(start.data(), d_start, 4 * (nc + 1), cudaMemcpyDeviceToHost, c->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(c->stream);
        if (e != cudaSuccess) break;
        if (cell_of_particle) std::memcpy(cell_of_particle + off, cell.data(), 4ull * h.count);
        if (sorted_ids) std::memcpy(sorted_ids + off, order.data(), 4ull * h.count);
        if (cell_counts)
            for (uint64_t k = 0; k < nc; k++) cell_counts[cbase + k] = start[k + 1] - start[k];
        off += h.count;
        cbase += nc;
    }
    cudaFree(mem);
    if (e != cudaSuccess) return cuda_fail(c, e, "reference grid of the sorted state");
    return SPH_OK;
}

}  // namespace

int sph_get_grid(sph_ctx *c, uint32_t *cell_of_particle, uint32_t *cell_counts, uint32_t *sorted_ids)
{
    if (!c) return SPH_ERR_ARG;
    if (c->state != SORTED && c->state != DENSE) return fail(c, SPH_ERR_STATE, "the grid is available after a grid pass");
    try {
        CK(c, cudaSetDevice(c->device));
        if (c->tune.cell_mult != 1) return get_grid_ref(c, cell_of_particle, cell_counts, sorted_ids);
        const uint32_t n = c->n;
        std::vector<uint32_t> start(c->ctot + 1);
        CK(c, cudaMemcpyAsync(start.data(), c->b.start, 4 * (c->ctot + 1), cudaMemcpyDeviceToHost, c->stream));
        std::vector<uint2> cid(n);
        if (n) CK(c, cudaMemcpyAsync(cid.data(), c->b.cid_u, 8ull * n, cudaMemcpyDeviceToHost, c->stream));
        const size_t r4 = r4_bytes(c);
        std::vector<unsigned char> vs((size_t) n * r4);
        if (n) CK(c, cudaMemcpyAsync(vs.data(), c->b.vel_s, r4 * n, cudaMemcpyDeviceToHost, c->stream));
        CK(c, cudaStreamSynchronize(c->stream));
        std::vector<uint32_t> off(c->sc.size() + 1, 0);
        for (size_t s = 0; s < c->sc.size(); s++) off[s + 1] = off[s] + c->sc[s].count;
        if (cell_counts)
            for (uint64_t k = 0; k < c->ctot; k++) cell_counts[k] = start[k + 1] - start[k];
        if (cell_of_particle) {
            for (uint32_t i = 0; i < n; i++) {
                const uint32_t cell = cid[i].x, id = cid[i].y;
                size_t s = 0, hi = c->sc.size();
                while (hi - s > 1) {  // last scene with cell_base <= cell
                    size_t mid = (s + hi) / 2;
                    if (c->sc[mid].cell_base <= cell) s = mid;
                    else hi = mid;
                }
                cell_of_particle[off[s] + id] = cell - c->sc[s].cell_base;
            }
        }
        if (sorted_ids) {
            for (uint32_t k = 0; k < n; k++) {
                uint32_t w;
                std::memcpy(&w, vs.data() + (size_t) k * r4 + (r4 == 16 ? 12 : 24), 4);
                sorted_ids[k] = w;
            }
        }
        return SPH_OK;
    } catch (...) {
        return fail(c, SPH_ERR_NOMEM, "host exception in sph_get_grid");
    }
}

int sph_stats(sph_ctx *c, uint32_t scene, double out[8])
{
    if (!c || !out) return SPH_ERR_ARG;
    if (scene >= c->sc.size()) return fail(c, SPH_ERR_ARG, "scene index out of range");
    if (!(c->state == HASHED && c->n_sorted > 0) && c->state != DENSE)
        return fail(c, SPH_ERR_STATE, "statistics need a completed step or a density pass");
    CK(c, cudaSetDevice(c->device));
    const int layout_sorted = c->state == DENSE ? 1 : 0;
    if (is_f64(c)) CK(c, Launch<double>::stats(c->b, (uint32_t) c->sc.size(), make_consts<double>(c, c->tune.cell_mult), layout_sorted, c->stream));
    else CK(c, Launch<float>::stats(c->b, (uint32_t) c->sc.size(), make_consts<float>(c, c->tune.cell_mult), layout_sorted, c->stream));
    CK(c, cudaMemcpyAsync(out, c->b.stats + 8 * scene, 64, cudaMemcpyDeviceToHost, c->stream));
    CK(c, cudaStreamSynchronize(c->stream));
    return SPH_OK;
}

}  // extern "C"
