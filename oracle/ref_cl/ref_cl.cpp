// ref_cl.cpp -- the reference's own OpenCL grid kernels run on the CPU (test infrastructure:
// it pins the oracle and generates golden vectors; never the product path).
//
// The kernel sources are compiled where they lie in the reference tree (the recipe in
// oracle/oracle.py passes their directory with -I); cl_shim.h supplies the OpenCL C built-ins.
// The host side restates CGPUParticleSimulator's grid preparation
// (src/CGPUParticleSimulator.cpp:58-160 and update_grid_positions, sph_grid.cl:24-65): the
// cell of each particle from (position + box/2) / h in float, clamped per axis; the
// particle indices sorted by cell; the exclusive scan of the cell counts. Then
// density_pressure_step and forces_step (sph_grid.cl:124-225) run once per work-item, in
// that order, with the constants of CBaseParticleSimulator (src/CBaseParticleSimulator.cpp:23-25).
#include "cl_shim.h"

// the grid simulator's program (sph_common.cl + sph_grid.cl)
namespace clk {
using namespace clt;
#include "sph_common.cl"
#include "sph_grid.cl"
}  // namespace clk

// the brute-force simulator's program (sph_common.cl + sph_brute.cl) reuses the kernel
// names, so it gets a namespace of its own
namespace clb {
using namespace clt;
#include "sph_common.cl"
#include "sph_brute.cl"
}  // namespace clb

#include <algorithm>
#include <cmath>
#include <numeric>
#include <vector>

thread_local unsigned long clt::cl_shim_gid = 0;

using clt::float3;
using clt::int3;
using clt::uint;

extern "C" {

// One evaluation of the grid density/pressure and force kernels for n particles (input order):
// rho[n], p[n] and acc[3n] (before the walls and the integration). Returns 0, or -1 on a bad
// argument.
int refcl_density_forces(int n, const float *xyz, const float *vel, const float box[3], const float gravity[3],
                         float *rho, float *p, float *acc)
{
    if (n < 0 || (n > 0 && (!xyz || !vel || !rho || !p || !acc)) || !box || !gravity) return -1;
    const float h = clk::particle_h;
    int3 grid;
    grid.x = (int) std::ceil(box[0] / h);
    grid.y = (int) std::ceil(box[1] / h);
    grid.z = (int) std::ceil(box[2] / h);
    const float3 half(box[0] / 2.0f, box[1] / 2.0f, box[2] / 2.0f);
    const int cells = grid.x * grid.y * grid.z;
    std::vector<clk::ParticleCL> part((size_t) n);
    std::vector<int> counts((size_t) cells, 0);
    for (int i = 0; i < n; i++) {
        clk::ParticleCL &q = part[(size_t) i];
        q = clk::ParticleCL();
        q.position = float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        q.velocity = float3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        q.id = (uint) i;
        const float3 g = (q.position + half) / clk::particle_h;  // update_grid_positions
        int c[3] = {(int) clt::floor(g.x), (int) clt::floor(g.y), (int) clt::floor(g.z)};
        const int lim[3] = {grid.x, grid.y, grid.z};
        for (int a = 0; a < 3; a++) c[a] = c[a] < 0 ? 0 : (c[a] >= lim[a] ? lim[a] - 1 : c[a]);
        q.grid_position.x = c[0];
        q.grid_position.y = c[1];
        q.grid_position.z = c[2];
        q.cell_id = (uint) (c[0] + c[1] * grid.x + c[2] * grid.x * grid.y);
        counts[q.cell_id]++;
    }
    std::vector<int> sorted((size_t) n);
    std::iota(sorted.begin(), sorted.end(), 0);
    std::stable_sort(sorted.begin(), sorted.end(), [&](int a, int b) { return part[a].cell_id < part[b].cell_id; });
    std::vector<int> scan((size_t) cells, 0);
    for (int k = 1; k < cells; k++) scan[k] = scan[k - 1] + counts[k - 1];
    const float poly6 = (float) (315.0f / (64.0f * M_PI * std::pow(clk::particle_h, 9)));
    const float spiky = (float) (-45.0f / (M_PI * std::pow(clk::particle_h, 6)));
    const float viscl = (float) (45.0f / (M_PI * std::pow(clk::particle_h, 6)));
    for (int i = 0; i < n; i++) {
        clt::cl_shim_gid = (unsigned long) i;
        clk::density_pressure_step(part.data(), scan.data(), sorted.data(), n, grid, poly6);
    }
    const float3 gv(gravity[0], gravity[1], gravity[2]);
    for (int i = 0; i < n; i++) {
        clt::cl_shim_gid = (unsigned long) i;
        clk::forces_step(part.data(), scan.data(), sorted.data(), n, grid, gv, spiky, viscl);
    }
    for (int i = 0; i < n; i++) {
        rho[i] = part[(size_t) i].density;
        p[i] = part[(size_t) i].pressure;
        acc[3 * i] = part[(size_t) i].acceleration.x;
        acc[3 * i + 1] = part[(size_t) i].acceleration.y;
        acc[3 * i + 2] = part[(size_t) i].acceleration.z;
    }
    return 0;
}

// The all-pairs kernels of CGPUBruteParticleSimulator (sph_brute.cl:9-57) for the same
// state: every particle is a candidate, in input order. Same outputs as above.
int refcl_brute_density_forces(int n, const float *xyz, const float *vel, const float gravity[3], float *rho,
                               float *p, float *acc)
{
    if (n < 0 || (n > 0 && (!xyz || !vel || !rho || !p || !acc)) || !gravity) return -1;
    std::vector<clb::ParticleCL> part((size_t) n);
    for (int i = 0; i < n; i++) {
        clb::ParticleCL &q = part[(size_t) i];
        q = clb::ParticleCL();
        q.position = float3(xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]);
        q.velocity = float3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        q.id = (uint) i;
    }
    const float poly6 = (float) (315.0f / (64.0f * M_PI * std::pow(clb::particle_h, 9)));
    const float spiky = (float) (-45.0f / (M_PI * std::pow(clb::particle_h, 6)));
    const float viscl = (float) (45.0f / (M_PI * std::pow(clb::particle_h, 6)));
    for (int i = 0; i < n; i++) {
        clt::cl_shim_gid = (unsigned long) i;
        clb::density_pressure_step(part.data(), n, poly6);
    }
    const float3 gv(gravity[0], gravity[1], gravity[2]);
    for (int i = 0; i < n; i++) {
        clt::cl_shim_gid = (unsigned long) i;
        clb::forces_step(part.data(), n, gv, spiky, viscl);
    }
    for (int i = 0; i < n; i++) {
        rho[i] = part[(size_t) i].density;
        p[i] = part[(size_t) i].pressure;
        acc[3 * i] = part[(size_t) i].acceleration.x;
        acc[3 * i + 1] = part[(size_t) i].acceleration.y;
        acc[3 * i + 2] = part[(size_t) i].acceleration.z;
    }
    return 0;
}

}  // extern "C"
