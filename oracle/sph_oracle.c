/*
 * sph_oracle.c -- TEST INFRASTRUCTURE ONLY (the checker, never the product).
 *
 * A Qt-free CPU restatement of the reference's serial SPH grid step,
 * CCPUParticleSimulator (src/CCPUParticleSimulator.cpp:9-229), with the wall
 * response of CCollisionGeometry::inverseBoundingBoxBounce
 * (src/CCollisionGeometry.cpp:117-133), the grid resolution of
 * CBaseParticleSimulator's constructor (src/CBaseParticleSimulator.cpp:27-31),
 * the constants of include/CParticle.h:80-84 and the dam-break scene of
 * CBaseParticleSimulator::setupScene (src/CBaseParticleSimulator.cpp:38-74).
 * A CPU restatement of the all-pairs kernels (resources/kernels/sph_brute.cl:9-57)
 * serves as an independent second check.
 *
 * The reference's CPU path cannot be built here (it needs Qt5Gui QVector3D and
 * Qt3D, which are absent) and it ships no tests, fixtures or golden vectors. The
 * density, pressure and forces of this restatement are pinned to the reference's
 * own OpenCL grid kernels compiled for the CPU (oracle/ref_cl, golden vectors in
 * tests/golden/ref_cl_cases.npz); the walls, integration and cell hash to analytic
 * known answers (self density, hand-placed particle pairs evaluated independently
 * in high precision) and to the reference's own scene-count assert
 * (src/CBaseParticleSimulator.cpp:56).
 *
 * Arithmetic is restated operation by operation. Qt5's QVector3D stores floats;
 * its +, -, * float, / float, dotProduct and lengthSquared are float operations
 * evaluated left to right; a double scalar times a QVector3D is first converted to
 * float (QVector3D has only float-factor operators). The reference's double
 * scalars (Wpoly6, spiky and viscosity coefficients, the wall distance, the cell
 * hash) stay double here. Compile with -ffp-contract=off so that no multiply-add
 * is fused: the reference's x86-64 build has no FMA.
 *
 * Three modes:
 *   ORC_REF   float-faithful arithmetic and the reference's history-dependent
 *             per-cell particle order (swap-with-last re-binning, all particles
 *             start in cell (0,0,0) as addParticle puts them there);
 *   ORC_CANON float-faithful arithmetic, cell lists rebuilt every step in the
 *             canonical (cell, id) order;
 *   ORC_F64   the same method entirely in double, canonical order.
 *
 * Per-particle work of the density and force passes is independent, so those
 * passes may run on several threads (OpenMP) with results bit-identical to one
 * thread; the grid re-binning stays serial exactly as in the reference.
 */
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#ifndef M_PI
#define M_PI 3.14159265358979323846
#endif

/* include/CParticle.h:80-84 */
static const float P_H = 0.0457f;
static const float P_VISCOSITY = 3.5f;
static const float P_MASS = 0.02f;
static const float P_GAS_STIFFNESS = 3.0f;
static const float P_REST_DENSITY = 998.29f;
/* include/CCollisionGeometry.h:20-21 */
#define WALL_K 10000.0
#define WALL_DAMPING (-0.9)
/* src/CCollisionGeometry.cpp:124 particle radius */
#define WALL_RADIUS 0.01

enum { ORC_REF = 0, ORC_CANON = 1, ORC_F64 = 2 };

/* ---------------- QVector3D restatement (float storage) ---------------- */
typedef struct { float x, y, z; } v3f;
static inline v3f v3(float x, float y, float z) { v3f r = {x, y, z}; return r; }
static inline v3f v3_add(v3f a, v3f b) { return v3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3f v3_sub(v3f a, v3f b) { return v3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3f v3_mul(v3f a, float f) { return v3(a.x * f, a.y * f, a.z * f); }
static inline v3f v3_div(v3f a, float f) { return v3(a.x / f, a.y / f, a.z / f); }
static inline float v3_dot(v3f a, v3f b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline float v3_len2(v3f a) { return a.x * a.x + a.y * a.y + a.z * a.z; }
static inline float v3_norm(v3f a) { return sqrtf(v3_len2(a)); }

typedef struct { double x, y, z; } v3d;
static inline v3d d3(double x, double y, double z) { v3d r = {x, y, z}; return r; }
static inline v3d d3_add(v3d a, v3d b) { return d3(a.x + b.x, a.y + b.y, a.z + b.z); }
static inline v3d d3_sub(v3d a, v3d b) { return d3(a.x - b.x, a.y - b.y, a.z - b.z); }
static inline v3d d3_mul(v3d a, double f) { return d3(a.x * f, a.y * f, a.z * f); }
static inline v3d d3_div(v3d a, double f) { return d3(a.x / f, a.y / f, a.z / f); }
static inline double d3_dot(v3d a, v3d b) { return a.x * b.x + a.y * b.y + a.z * b.z; }
static inline double d3_norm(v3d a) { return sqrt(d3_dot(a, a)); }

/* ---------------- per-cell particle lists (std::vector<CParticle*>) ---------------- */
typedef struct { int32_t *d; int32_t n, cap; } ilist;
static void il_push(ilist *l, int32_t v)
{
    if (l->n == l->cap) {
        int32_t nc = l->cap ? 2 * l->cap : 8;
        l->d = (int32_t *) realloc(l->d, (size_t) nc * sizeof(int32_t));
        l->cap = nc;
    }
    l->d[l->n++] = v;
}

typedef struct orc_sim {
    int mode, nthreads;
    float box[3];
    int res[3];
    int64_t ncells;
    float dt;
    float gravity[3];
    int32_t n, cap;
    /* float state (REF / CANON) */
    v3f *pos, *vel, *acc;
    float *rho, *prs;
    /* double state (F64) */
    v3d *pos64, *vel64, *acc64;
    double *rho64, *prs64;
    float *ascale;   /* per-particle magnitude of the force terms, for tolerances */
    int nobs;        /* axis-aligned box obstacles: lo xyz, hi xyz */
    float *obs;
    int32_t *cell;   /* cell of each particle after the last grid update */
    ilist *cells;
} orc_sim;

/* Grid resolution: (int) ceil(box / h) evaluated in float
 * (src/CBaseParticleSimulator.cpp:27-31, the QVector3D then feeds CGrid's int ctor). */
int orc_grid_res(float box) { return (int) ceilf(box / P_H); }

/* Cell coordinate along one axis: (int) floor((p + box/2.0) / h) in double, clamped to
 * [0, res-1] (src/CCPUParticleSimulator.cpp:46-69). The reference's float->int conversion
 * is undefined for NaN and for |q| >= 2^31; here NaN and negatives map to 0 and anything
 * at or beyond res maps to res-1. */
int orc_cell_axis(float p, float box, int res)
{
    double q = ((double) p + (double) box / 2.0) / (double) P_H;
    if (!(q >= 0.0)) return 0;
    if (q >= (double) res) return res - 1;
    return (int) floor(q);
}

static int cell_axis_f64(double p, double box, int res)
{
    double q = (p + box / 2.0) / (double) P_H;
    if (!(q >= 0.0)) return 0;
    if (q >= (double) res) return res - 1;
    return (int) floor(q);
}

/* Restatement of setupScene's DAM_BREAK lattice (src/CBaseParticleSimulator.cpp:38-58):
 * y outer, x middle, z inner; loop counters are float incremented by a double. */
int orc_reference_dam_break(float box, float *out_xyz, int cap)
{
    double halfParticle = P_H / 2.0f;
    float off = -box / 2.0f;
    int n = 0;
    for (float y = 0; y < box; y += halfParticle)
        for (float x = 0; x < box / 4.0; x += halfParticle)
            for (float z = 0; z < box; z += halfParticle) {
                if (n < cap && out_xyz) {
                    out_xyz[3 * n + 0] = x + off;
                    out_xyz[3 * n + 1] = y + off;
                    out_xyz[3 * n + 2] = z + off;
                }
                n++;
            }
    return n;
}

/* calculatedCount of setupScene (src/CBaseParticleSimulator.cpp:40-41). */
unsigned orc_reference_dam_break_count(float box)
{
    double halfParticle = P_H / 2.0f;
    return (unsigned) (ceil(box / halfParticle) * ceil(box / halfParticle) * ceil(box / 4 / halfParticle));
}

orc_sim *orc_create(float bx, float by, float bz, int mode, int nthreads)
{
    orc_sim *s = (orc_sim *) calloc(1, sizeof(orc_sim));
    s->mode = mode;
    s->nthreads = nthreads > 0 ? nthreads : 1;
    s->box[0] = bx; s->box[1] = by; s->box[2] = bz;
    for (int a = 0; a < 3; a++) s->res[a] = orc_grid_res(s->box[a]);
    s->ncells = (int64_t) s->res[0] * s->res[1] * s->res[2];
    s->cells = (ilist *) calloc((size_t) s->ncells, sizeof(ilist));
    s->dt = 0.01f;                                  /* src/CBaseParticleSimulator.cpp:7 */
    s->gravity[0] = 0; s->gravity[1] = -9.80665f;   /* include/CBaseParticleSimulator.h:19 */
    s->gravity[2] = 0;
    return s;
}

void orc_destroy(orc_sim *s)
{
    if (!s) return;
    for (int64_t c = 0; c < s->ncells; c++) free(s->cells[c].d);
    free(s->cells);
    free(s->pos); free(s->vel); free(s->acc); free(s->rho); free(s->prs);
    free(s->pos64); free(s->vel64); free(s->acc64); free(s->rho64); free(s->prs64);
    free(s->ascale); free(s->cell); free(s->obs);
    free(s);
}

void orc_set_gravity(orc_sim *s, float gx, float gy, float gz)
{
    s->gravity[0] = gx; s->gravity[1] = gy; s->gravity[2] = gz;
}
void orc_set_dt(orc_sim *s, float dt) { s->dt = dt; }

/* Box obstacles (no reference counterpart: CCollisionGeometry only bounds the domain).
 * A particle inside an obstacle grown by the particle radius is pushed out through the
 * nearest face with the wall spring and damping constants; obstacles act after the walls,
 * in table order. boxes: 6 floats per obstacle (lo xyz, hi xyz). */
void orc_set_obstacles(orc_sim *s, int n, const float *boxes)
{
    free(s->obs);
    s->obs = NULL;
    s->nobs = n > 0 ? n : 0;
    if (s->nobs) {
        s->obs = (float *) malloc((size_t) n * 6 * sizeof(float));
        memcpy(s->obs, boxes, (size_t) n * 6 * sizeof(float));
    }
}
int orc_count(orc_sim *s) { return s->n; }
void orc_get_res(orc_sim *s, int *res3) { res3[0] = s->res[0]; res3[1] = s->res[1]; res3[2] = s->res[2]; }

static void grow(orc_sim *s, int32_t need)
{
    if (need <= s->cap) return;
    int32_t nc = s->cap ? s->cap : 1024;
    while (nc < need) nc *= 2;
#define RE(p, T) p = (T *) realloc(p, (size_t) nc * sizeof(T))
    RE(s->pos, v3f); RE(s->vel, v3f); RE(s->acc, v3f); RE(s->rho, float); RE(s->prs, float);
    RE(s->pos64, v3d); RE(s->vel64, v3d); RE(s->acc64, v3d); RE(s->rho64, double); RE(s->prs64, double);
    RE(s->ascale, float); RE(s->cell, int32_t);
#undef RE
    s->cap = nc;
}

/* addParticle (src/CBaseParticleSimulator.cpp:67-74): ids are assigned in call order and
 * every new particle is pushed onto grid cell (0,0,0). vel may be NULL (zero). */
int orc_add_particles(orc_sim *s, int n, const float *xyz, const float *vel)
{
    grow(s, s->n + n);
    for (int k = 0; k < n; k++) {
        int32_t i = s->n + k;
        s->pos[i] = v3(xyz[3 * k], xyz[3 * k + 1], xyz[3 * k + 2]);
        s->vel[i] = vel ? v3(vel[3 * k], vel[3 * k + 1], vel[3 * k + 2]) : v3(0, 0, 0);
        s->acc[i] = v3(0, 0, 0);
        s->rho[i] = 0; s->prs[i] = 0;
        s->pos64[i] = d3(s->pos[i].x, s->pos[i].y, s->pos[i].z);
        s->vel64[i] = d3(s->vel[i].x, s->vel[i].y, s->vel[i].z);
        s->acc64[i] = d3(0, 0, 0);
        s->rho64[i] = 0; s->prs64[i] = 0;
        s->ascale[i] = 0;
        s->cell[i] = 0;
        il_push(&s->cells[0], i);
    }
    s->n += n;
    return s->n;
}

static inline int64_t lin(const orc_sim *s, int x, int y, int z)
{
    return (int64_t) x + (int64_t) y * s->res[0] + (int64_t) z * s->res[0] * s->res[1]; /* include/CGrid.h:25-28 */
}

static void particle_cell(const orc_sim *s, int32_t i, int *cx, int *cy, int *cz)
{
    if (s->mode == ORC_F64) {
        *cx = cell_axis_f64(s->pos64[i].x, s->box[0], s->res[0]);
        *cy = cell_axis_f64(s->pos64[i].y, s->box[1], s->res[1]);
        *cz = cell_axis_f64(s->pos64[i].z, s->box[2], s->res[2]);
    } else {
        *cx = orc_cell_axis(s->pos[i].x, s->box[0], s->res[0]);
        *cy = orc_cell_axis(s->pos[i].y, s->box[1], s->res[1]);
        *cz = orc_cell_axis(s->pos[i].z, s->box[2], s->res[2]);
    }
}

/* updateGrid (src/CCPUParticleSimulator.cpp:32-91). REF: visit cells x outer, y, z inner;
 * a particle whose cell changed is pushed onto the new cell's list and replaced by the
 * list's last element, and the same slot is examined again. CANON / F64: lists rebuilt in
 * id order, which is the canonical (cell, id) order. */
void orc_update_grid(orc_sim *s)
{
    if (s->mode == ORC_REF) {
        for (int x = 0; x < s->res[0]; x++)
            for (int y = 0; y < s->res[1]; y++)
                for (int z = 0; z < s->res[2]; z++) {
                    ilist *l = &s->cells[lin(s, x, y, z)];
                    for (long p = 0; p < (long) l->n; p++) {
                        int32_t i = l->d[p];
                        int nx, ny, nz;
                        particle_cell(s, i, &nx, &ny, &nz);
                        if (x != nx || y != ny || z != nz) {
                            il_push(&s->cells[lin(s, nx, ny, nz)], i);
                            l = &s->cells[lin(s, x, y, z)];
                            l->d[p] = l->d[l->n - 1];
                            l->n--;
                            p--;
                        }
                    }
                }
    } else {
        for (int64_t c = 0; c < s->ncells; c++) s->cells[c].n = 0;
        for (int32_t i = 0; i < s->n; i++) {
            int nx, ny, nz;
            particle_cell(s, i, &nx, &ny, &nz);
            il_push(&s->cells[lin(s, nx, ny, nz)], i);
        }
    }
    for (int64_t c = 0; c < s->ncells; c++)
        for (int32_t k = 0; k < s->cells[c].n; k++) s->cell[s->cells[c].d[k]] = (int32_t) c;
}

/* ---------------- SPH kernel functions (src/CCPUParticleSimulator.cpp:9-30) ---------------- */
static double c_poly6, c_spiky, c_visc, h_sq;
static void init_constants(void)
{
    static int done = 0;
    if (done) return;
    c_poly6 = 315.0 / (64.0 * M_PI * pow(P_H, 9));
    c_spiky = -45.0 / (M_PI * pow(P_H, 6));
    c_visc = 45.0 / (M_PI * pow(P_H, 6));
    h_sq = P_H * P_H;  /* float product, then widened: static double hSquared = h * h */
    done = 1;
}
static inline double Wpoly6(double r2) { return c_poly6 * pow(h_sq - r2, 3); }
static inline v3f WspikyGradient(v3f d, double r2)
{
    double r = sqrt(r2);
    /* coefficient * pow(h - r, 2) * diffPosition / radius */
    return v3_div(v3_mul(d, (float) (c_spiky * pow(P_H - r, 2))), (float) r);
}
static inline double WviscLaplacian(double r2) { return c_visc * (P_H - sqrt(r2)); }

/* updateDensityPressure (src/CCPUParticleSimulator.cpp:93-141) for one particle in cell (x,y,z). */
static void density_one(orc_sim *s, int32_t i, int x, int y, int z)
{
    if (s->mode == ORC_F64) {
        const double hh = (double) P_H * (double) P_H;
        const double cp = 315.0 / (64.0 * M_PI * pow(P_H, 9));
        double rho = 0.0;
        for (int ox = -1; ox <= 1; ox++) {
            if (x + ox < 0) continue;
            if (x + ox >= s->res[0]) break;
            for (int oy = -1; oy <= 1; oy++) {
                if (y + oy < 0) continue;
                if (y + oy >= s->res[1]) break;
                for (int oz = -1; oz <= 1; oz++) {
                    if (z + oz < 0) continue;
                    if (z + oz >= s->res[2]) break;
                    const ilist *l = &s->cells[lin(s, x + ox, y + oy, z + oz)];
                    for (int32_t k = 0; k < l->n; k++) {
                        v3d d = d3_sub(s->pos64[i], s->pos64[l->d[k]]);
                        double r2 = d3_dot(d, d);
                        if (r2 <= hh) { double t = hh - r2; rho += cp * t * t * t; }
                    }
                }
            }
        }
        rho *= (double) P_MASS;
        s->rho64[i] = rho;
        s->prs64[i] = (double) P_GAS_STIFFNESS * (rho - (double) P_REST_DENSITY);
        return;
    }
    float rho = 0.0f;
    for (int ox = -1; ox <= 1; ox++) {
        if (x + ox < 0) continue;
        if (x + ox >= s->res[0]) break;
        for (int oy = -1; oy <= 1; oy++) {
            if (y + oy < 0) continue;
            if (y + oy >= s->res[1]) break;
            for (int oz = -1; oz <= 1; oz++) {
                if (z + oz < 0) continue;
                if (z + oz >= s->res[2]) break;
                const ilist *l = &s->cells[lin(s, x + ox, y + oy, z + oz)];
                for (int32_t k = 0; k < l->n; k++) {
                    v3f d = v3_sub(s->pos[i], s->pos[l->d[k]]);
                    double r2 = v3_len2(d);
                    if (r2 <= P_H * P_H) rho = (float) ((double) rho + Wpoly6(r2));
                }
            }
        }
    }
    rho *= P_MASS;
    s->rho[i] = rho;
    s->prs[i] = P_GAS_STIFFNESS * (rho - P_REST_DENSITY);
}

/* inverseBoundingBoxBounce (src/CCollisionGeometry.cpp:117-133). Walls come from the
 * bounding box of the grid's cuboid mesh, at +-box/2, in the order left, bottom, back,
 * right, top, front (include/CCollisionGeometry.h:237-250). */
static v3f wall_bounce(const orc_sim *s, v3f pos, v3f vel, float *mag)
{
    const float hx = s->box[0] / 2.0f, hy = s->box[1] / 2.0f, hz = s->box[2] / 2.0f;
    const v3f nrm[6] = {v3(-1, 0, 0), v3(0, -1, 0), v3(0, 0, -1), v3(1, 0, 0), v3(0, 1, 0), v3(0, 0, 1)};
    const v3f wp[6] = {v3(-hx, 0, 0), v3(0, -hy, 0), v3(0, 0, -hz), v3(hx, 0, 0), v3(0, hy, 0), v3(0, 0, hz)};
    v3f acc = v3(0, 0, 0);
    float m = 0.0f;
    for (int w = 0; w < 6; w++) {
        v3f inv = v3_mul(nrm[w], -1.0f);
        double d = (double) v3_dot(v3_sub(wp[w], pos), inv) + WALL_RADIUS;
        if (d > 0.0) {
            v3f t1 = v3_mul(v3_mul(inv, (float) WALL_K), (float) d);
            v3f t2 = v3_mul(inv, (float) (WALL_DAMPING * (double) v3_dot(vel, inv)));
            acc = v3_add(acc, t1);
            acc = v3_add(acc, t2);
            m += v3_norm(t1) + v3_norm(t2);
        }
    }
    for (int o = 0; o < s->nobs; o++) {
        const float *lo = s->obs + 6 * o, *hi = lo + 3;
        const float p3[3] = {pos.x, pos.y, pos.z}, vv[3] = {vel.x, vel.y, vel.z};
        float best = 1e30f;
        int bf = -1, outside = 0;
        for (int f = 0; f < 6; f++) {
            const int a = f % 3;
            const float dpen = f < 3 ? (p3[a] - lo[a]) + (float) WALL_RADIUS : (hi[a] - p3[a]) + (float) WALL_RADIUS;
            if (dpen <= 0.0f) outside = 1;
            else if (dpen < best) { best = dpen; bf = f; }
        }
        if (!outside && bf >= 0) {
            const int a = bf % 3;
            const float sgn = bf < 3 ? -1.0f : 1.0f;
            const float kt = (sgn * (float) WALL_K) * best;
            const float dt = sgn * ((float) WALL_DAMPING * (vv[a] * sgn));
            float *c = a == 0 ? &acc.x : (a == 1 ? &acc.y : &acc.z);
            *c = (*c + kt) + dt;
            m += fabsf(kt) + fabsf(dt);
        }
    }
    if (mag) *mag = m;
    return acc;
}

static v3d wall_bounce64(const orc_sim *s, v3d pos, v3d vel, double *mag)
{
    const double hx = s->box[0] / 2.0, hy = s->box[1] / 2.0, hz = s->box[2] / 2.0;
    const v3d nrm[6] = {d3(-1, 0, 0), d3(0, -1, 0), d3(0, 0, -1), d3(1, 0, 0), d3(0, 1, 0), d3(0, 0, 1)};
    const v3d wp[6] = {d3(-hx, 0, 0), d3(0, -hy, 0), d3(0, 0, -hz), d3(hx, 0, 0), d3(0, hy, 0), d3(0, 0, hz)};
    v3d acc = d3(0, 0, 0);
    double m = 0.0;
    for (int w = 0; w < 6; w++) {
        v3d inv = d3_mul(nrm[w], -1.0);
        double d = d3_dot(d3_sub(wp[w], pos), inv) + WALL_RADIUS;
        if (d > 0.0) {
            v3d t1 = d3_mul(inv, WALL_K * d);
            v3d t2 = d3_mul(inv, WALL_DAMPING * d3_dot(vel, inv));
            acc = d3_add(d3_add(acc, t1), t2);
            m += d3_norm(t1) + d3_norm(t2);
        }
    }
    for (int o = 0; o < s->nobs; o++) {
        const float *lo = s->obs + 6 * o, *hi = lo + 3;
        const double p3[3] = {pos.x, pos.y, pos.z}, vv[3] = {vel.x, vel.y, vel.z};
        double best = 1e300;
        int bf = -1, outside = 0;
        for (int f = 0; f < 6; f++) {
            const int a = f % 3;
            const double dpen = f < 3 ? (p3[a] - lo[a]) + WALL_RADIUS : (hi[a] - p3[a]) + WALL_RADIUS;
            if (dpen <= 0.0) outside = 1;
            else if (dpen < best) { best = dpen; bf = f; }
        }
        if (!outside && bf >= 0) {
            const int a = bf % 3;
            const double sgn = bf < 3 ? -1.0 : 1.0;
            const double kt = (sgn * WALL_K) * best;
            const double dt = sgn * (WALL_DAMPING * (vv[a] * sgn));
            double *c = a == 0 ? &acc.x : (a == 1 ? &acc.y : &acc.z);
            *c = (*c + kt) + dt;
            m += fabs(kt) + fabs(dt);
        }
    }
    if (mag) *mag = m;
    return acc;
}

/* updateForces (src/CCPUParticleSimulator.cpp:143-203) for one particle. Also records a
 * magnitude scale: the acceleration that the sum of the absolute values of every term
 * would give, used by the tests as the denominator of a relative error. */
static void forces_one(orc_sim *s, int32_t i, int x, int y, int z)
{
    if (s->mode == ORC_F64) {
        const double hh = (double) P_H * (double) P_H;
        const double cs = -45.0 / (M_PI * pow(P_H, 6)), cv = 45.0 / (M_PI * pow(P_H, 6));
        const double rho_i = s->rho64[i], p_i = s->prs64[i];
        v3d g = d3(s->gravity[0], s->gravity[1], s->gravity[2]);
        v3d fp = d3(0, 0, 0), fv = d3(0, 0, 0);
        double mp = 0, mv = 0;
        for (int ox = -1; ox <= 1; ox++) {
            if (x + ox < 0) continue;
            if (x + ox >= s->res[0]) break;
            for (int oy = -1; oy <= 1; oy++) {
                if (y + oy < 0) continue;
                if (y + oy >= s->res[1]) break;
                for (int oz = -1; oz <= 1; oz++) {
                    if (z + oz < 0) continue;
                    if (z + oz >= s->res[2]) break;
                    const ilist *l = &s->cells[lin(s, x + ox, y + oy, z + oz)];
                    for (int32_t k = 0; k < l->n; k++) {
                        int32_t j = l->d[k];
                        v3d d = d3_sub(s->pos64[i], s->pos64[j]);
                        double r2 = d3_dot(d, d);
                        if (r2 <= hh && i != j) {
                            double r = sqrt(r2);
                            v3d grad = d3_mul(d, cs * ((double) P_H - r) * ((double) P_H - r) / r);
                            double lap = cv * ((double) P_H - r);
                            double pij = p_i / (rho_i * rho_i) + s->prs64[j] / (s->rho64[j] * s->rho64[j]);
                            v3d tp = d3_mul(grad, pij);
                            v3d tv = d3_mul(d3_sub(s->vel64[j], s->vel64[i]), lap / s->rho64[j]);
                            fp = d3_add(fp, tp);
                            fv = d3_add(fv, tv);
                            mp += d3_norm(tp);
                            mv += d3_norm(tv);
                        }
                    }
                }
            }
        }
        fp = d3_mul(fp, -(double) P_MASS * rho_i);
        fv = d3_mul(fv, (double) P_VISCOSITY * (double) P_MASS);
        v3d a = d3_div(d3_add(d3_add(fp, fv), d3_mul(g, rho_i)), rho_i);
        double mw;
        a = d3_add(a, wall_bounce64(s, s->pos64[i], s->vel64[i], &mw));
        s->acc64[i] = a;
        s->ascale[i] = (float) ((mp * (double) P_MASS * fabs(rho_i) + mv * (double) P_VISCOSITY * (double) P_MASS)
                                / fabs(rho_i) + d3_norm(g) + mw);
        return;
    }
    const float rho_i = s->rho[i], p_i = s->prs[i];
    v3f g = v3(s->gravity[0], s->gravity[1], s->gravity[2]);
    v3f f_gravity = v3_mul(g, rho_i);
    v3f fp = v3(0, 0, 0), fv = v3(0, 0, 0);
    float mp = 0, mv = 0;
    for (int ox = -1; ox <= 1; ox++) {
        if (x + ox < 0) continue;
        if (x + ox >= s->res[0]) break;
        for (int oy = -1; oy <= 1; oy++) {
            if (y + oy < 0) continue;
            if (y + oy >= s->res[1]) break;
            for (int oz = -1; oz <= 1; oz++) {
                if (z + oz < 0) continue;
                if (z + oz >= s->res[2]) break;
                const ilist *l = &s->cells[lin(s, x + ox, y + oy, z + oz)];
                for (int32_t k = 0; k < l->n; k++) {
                    int32_t j = l->d[k];
                    v3f d = v3_sub(s->pos[i], s->pos[j]);
                    double r2 = v3_len2(d);
                    if (r2 <= P_H * P_H && i != j) {  /* ids are the particle indices */
                        v3f grad = WspikyGradient(d, r2);
                        double lap = WviscLaplacian(r2);
                        double pij = p_i / pow(rho_i, 2) + (s->prs[j] / pow(s->rho[j], 2));
                        v3f tp = v3_mul(grad, (float) pij);
                        v3f tv = v3_div(v3_mul(v3_sub(s->vel[j], s->vel[i]), (float) lap), s->rho[j]);
                        fp = v3_add(fp, tp);
                        fv = v3_add(fv, tv);
                        mp += v3_norm(tp);
                        mv += v3_norm(tv);
                    }
                }
            }
        }
    }
    fp = v3_mul(fp, -P_MASS * rho_i);
    fv = v3_mul(fv, P_VISCOSITY * P_MASS);
    v3f a = v3_div(v3_add(v3_add(fp, fv), f_gravity), rho_i);
    float mw;
    a = v3_add(a, wall_bounce(s, s->pos[i], s->vel[i], &mw));
    s->acc[i] = a;
    s->ascale[i] = (mp * P_MASS * fabsf(rho_i) + mv * P_VISCOSITY * P_MASS) / fabsf(rho_i) + v3_norm(g) + mw;
}

typedef void (*pass_fn)(orc_sim *, int32_t, int, int, int);
static void run_pass(orc_sim *s, pass_fn fn)
{
    init_constants();
    const int64_t C = s->ncells;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 256) num_threads(s->nthreads)
#endif
    for (int64_t c = 0; c < C; c++) {
        const int x = (int) (c % s->res[0]);
        const int y = (int) ((c / s->res[0]) % s->res[1]);
        const int z = (int) (c / ((int64_t) s->res[0] * s->res[1]));
        const ilist *l = &s->cells[c];
        for (int32_t k = 0; k < l->n; k++) fn(s, l->d[k], x, y, z);
    }
}

void orc_density(orc_sim *s) { run_pass(s, density_one); }
void orc_forces(orc_sim *s) { run_pass(s, forces_one); }

/* integrate (src/CCPUParticleSimulator.cpp:211-229): position Verlet in float. */
void orc_integrate(orc_sim *s)
{
    if (s->mode == ORC_F64) {
        const double dt = (double) s->dt;
        for (int32_t i = 0; i < s->n; i++) {
            v3d np = d3_add(d3_add(s->pos64[i], d3_mul(s->vel64[i], dt)), d3_mul(d3_mul(s->acc64[i], dt), dt));
            s->vel64[i] = d3_div(d3_sub(np, s->pos64[i]), dt);
            s->pos64[i] = np;
        }
        return;
    }
    const float dt = s->dt;
    for (int32_t i = 0; i < s->n; i++) {
        v3f np = v3_add(v3_add(s->pos[i], v3_mul(s->vel[i], dt)), v3_mul(v3_mul(s->acc[i], dt), dt));
        s->vel[i] = v3_div(v3_sub(np, s->pos[i]), dt);
        s->pos[i] = np;
    }
}

/* CBaseParticleSimulator::step (src/CBaseParticleSimulator.cpp:116-144): grid, density,
 * forces (walls included, updateCollisions is a no-op on the CPU), integrate. */
void orc_step(orc_sim *s, int nsteps)
{
    for (int k = 0; k < nsteps; k++) {
        orc_update_grid(s);
        orc_density(s);
        orc_forces(s);
        orc_integrate(s);
    }
}

/* State in id order. Any pointer may be NULL. Float getters of an F64 simulator round. */
void orc_get_state(orc_sim *s, float *pos, float *vel, float *acc, float *rho, float *prs, float *ascale)
{
    for (int32_t i = 0; i < s->n; i++) {
        if (s->mode == ORC_F64) {
            if (pos) { pos[3 * i] = (float) s->pos64[i].x; pos[3 * i + 1] = (float) s->pos64[i].y; pos[3 * i + 2] = (float) s->pos64[i].z; }
            if (vel) { vel[3 * i] = (float) s->vel64[i].x; vel[3 * i + 1] = (float) s->vel64[i].y; vel[3 * i + 2] = (float) s->vel64[i].z; }
            if (acc) { acc[3 * i] = (float) s->acc64[i].x; acc[3 * i + 1] = (float) s->acc64[i].y; acc[3 * i + 2] = (float) s->acc64[i].z; }
            if (rho) rho[i] = (float) s->rho64[i];
            if (prs) prs[i] = (float) s->prs64[i];
        } else {
            if (pos) { pos[3 * i] = s->pos[i].x; pos[3 * i + 1] = s->pos[i].y; pos[3 * i + 2] = s->pos[i].z; }
            if (vel) { vel[3 * i] = s->vel[i].x; vel[3 * i + 1] = s->vel[i].y; vel[3 * i + 2] = s->vel[i].z; }
            if (acc) { acc[3 * i] = s->acc[i].x; acc[3 * i + 1] = s->acc[i].y; acc[3 * i + 2] = s->acc[i].z; }
            if (rho) rho[i] = s->rho[i];
            if (prs) prs[i] = s->prs[i];
        }
        if (ascale) ascale[i] = s->ascale[i];
    }
}

void orc_get_state_f64(orc_sim *s, double *pos, double *vel, double *acc, double *rho, double *prs)
{
    for (int32_t i = 0; i < s->n; i++) {
        if (pos) { pos[3 * i] = s->pos64[i].x; pos[3 * i + 1] = s->pos64[i].y; pos[3 * i + 2] = s->pos64[i].z; }
        if (vel) { vel[3 * i] = s->vel64[i].x; vel[3 * i + 1] = s->vel64[i].y; vel[3 * i + 2] = s->vel64[i].z; }
        if (acc) { acc[3 * i] = s->acc64[i].x; acc[3 * i + 1] = s->acc64[i].y; acc[3 * i + 2] = s->acc64[i].z; }
        if (rho) rho[i] = s->rho64[i];
        if (prs) prs[i] = s->prs64[i];
    }
}

/* Replace the state (id order) without touching the cell lists: used to start the
 * oracle from a state produced elsewhere. Double inputs feed the F64 state and are
 * rounded for the float state. */
void orc_set_state(orc_sim *s, const float *pos, const float *vel)
{
    for (int32_t i = 0; i < s->n; i++) {
        s->pos[i] = v3(pos[3 * i], pos[3 * i + 1], pos[3 * i + 2]);
        s->vel[i] = v3(vel[3 * i], vel[3 * i + 1], vel[3 * i + 2]);
        s->pos64[i] = d3(s->pos[i].x, s->pos[i].y, s->pos[i].z);
        s->vel64[i] = d3(s->vel[i].x, s->vel[i].y, s->vel[i].z);
    }
}

/* The grid after the last orc_update_grid: the cell of every particle (id order), the
 * count of every cell, and the canonical order (ascending (cell, id)). */
void orc_get_grid(orc_sim *s, int32_t *cell_of_particle, int32_t *counts, int32_t *order)
{
    if (cell_of_particle) memcpy(cell_of_particle, s->cell, (size_t) s->n * sizeof(int32_t));
    if (counts)
        for (int64_t c = 0; c < s->ncells; c++) counts[c] = s->cells[c].n;
    if (order) {
        int64_t *start = (int64_t *) calloc((size_t) s->ncells + 1, sizeof(int64_t));
        for (int32_t i = 0; i < s->n; i++) start[s->cell[i] + 1]++;
        for (int64_t c = 0; c < s->ncells; c++) start[c + 1] += start[c];
        for (int32_t i = 0; i < s->n; i++) order[start[s->cell[i]]++] = i;
        free(start);
    }
}

/* ---------------- all-pairs second check (resources/kernels/sph_brute.cl:9-57) ----------------
 * float arithmetic as in the OpenCL C kernels; walls and integration follow the CPU path
 * (src/CCollisionGeometry.cpp:117-133, src/CCPUParticleSimulator.cpp:211-229). One step. */
void orc_brute_step(orc_sim *s)
{
    init_constants();
    const float poly6 = (float) (315.0f / (64.0f * M_PI * pow(P_H, 9)));   /* src/CBaseParticleSimulator.cpp:23-25 */
    const float spiky = (float) (-45.0f / (M_PI * pow(P_H, 6)));
    const float visc = (float) (45.0f / (M_PI * pow(P_H, 6)));
    const float h2 = 0.00208849f;                                          /* sph_common.cl:16 */
    const int32_t n = s->n;
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(s->nthreads)
#endif
    for (int32_t i = 0; i < n; i++) {
        float rho = 0.0f;
        for (int32_t j = 0; j < n; j++) {
            v3f d = v3_sub(s->pos[i], s->pos[j]);
            float r2 = v3_dot(d, d);
            if (r2 <= h2) rho += poly6 * powf(h2 - r2, 3);
        }
        rho *= P_MASS;
        s->rho[i] = rho;
        s->prs[i] = P_GAS_STIFFNESS * (rho - P_REST_DENSITY);
    }
#ifdef _OPENMP
#pragma omp parallel for schedule(dynamic, 64) num_threads(s->nthreads)
#endif
    for (int32_t i = 0; i < n; i++) {
        v3f fp = v3(0, 0, 0), fv = v3(0, 0, 0);
        for (int32_t j = 0; j < n; j++) {
            v3f d = v3_sub(s->pos[i], s->pos[j]);
            float r2 = v3_dot(d, d);
            if (r2 <= h2 && i != j) {
                float r = sqrtf(r2);
                v3f grad = v3_div(v3_mul(d, spiky * powf(P_H - r, 2)), r);
                float lap = visc * (P_H - sqrtf(r2));
                fp = v3_add(fp, v3_mul(grad, (s->prs[i] / powf(s->rho[i], 2)) + (s->prs[j] / powf(s->rho[j], 2))));
                fv = v3_add(fv, v3_div(v3_mul(v3_sub(s->vel[j], s->vel[i]), lap), s->rho[j]));
            }
        }
        fp = v3_mul(fp, -P_MASS * s->rho[i]);
        fv = v3_mul(fv, P_VISCOSITY * P_MASS);
        v3f g = v3(s->gravity[0], s->gravity[1], s->gravity[2]);
        v3f a = v3_div(v3_add(v3_add(fp, fv), v3_mul(g, s->rho[i])), s->rho[i]);
        a = v3_add(a, wall_bounce(s, s->pos[i], s->vel[i], NULL));
        s->acc[i] = a;
    }
    orc_integrate(s);
}
