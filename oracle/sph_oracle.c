/*
 * sph_oracle.c — CPU restatement of the reference's WCSPH step.
 *
 * TEST INFRASTRUCTURE ONLY. This file is the checker for the GPU library: it
 * is linked by the tests, by __graft_entry__.smoke() and by bench.py's CPU
 * baseline, never by the product. It restates, in plain C with OpenMP, the
 * algorithm of KemengHuang/Fast-General-GPU-SPH-framework (paths relative to
 * that project):
 *
 *   oracle_params_init   src/simulation/sph_hybrid_system.cpp:127-202
 *   oracle_lattice       src/simulation/sph_hybrid_system.cpp:441-464
 *   oracle_keys          src/core/sph_utils.cuh:44-99
 *   oracle_sort          src/grid/sph_arrangement.cu:1309-1395 (counting sort
 *                        by micro key; ties broken by previous index, which
 *                        is one of the orders the reference's atomic slots
 *                        can produce)
 *   oracle_block_req     src/io/gpu_model.cu:137-181
 *   oracle_split         src/grid/sph_arrangement.cu:87-107, 193-206, 358-384
 *   oracle_tasks         src/grid/sph_arrangement.cu:885-1022
 *   oracle_density       src/solver/density_kernels.cu:160-179, 278-295,
 *                        297-565 (FP64, full 27-cell search)
 *   oracle_force         src/solver/force_kernels.cu:378-435, 525-561,
 *                        725-1054 (FP64, full 27-cell search)
 *   oracle_force_model   the same with Monaghan's artificial viscosity
 *                        (Monaghan 1992) as an alternative to the reference's
 *                        Laplacian term; the reference has no such option
 *   oracle_integrate     src/solver/integration_kernels.cu:235-336 (FP64)
 *   oracle_step          src/simulation/sph_hybrid_system.cpp:253-339 (FP64)
 *
 * Integer results (keys, permutation, offsets, split, tasks) are exact.
 * Physics is evaluated in double precision from the same single-precision
 * coefficients the GPU uses, so it bounds the FP32 rounding error of the GPU.
 * The micro-cell pruning of the reference only removes pairs farther than h,
 * so the full 27-cell search here visits the same interacting pairs.
 *
 * Parity pins: the reference's own tests hold no golden vectors for this
 * path; the fixtures under tests/golden/ (see their generating script) pin
 * this restatement.
 */
#define _USE_MATH_DEFINES
#include <math.h>
#include <stdint.h>
#include <stdlib.h>
#include <string.h>

#ifdef _OPENMP
#include <omp.h>
#endif

#include "../include/gsph.h"

#define ORACLE_EXPORT __attribute__((visibility("default")))

/* ------------------------------------------------------------ params --- */
ORACLE_EXPORT int oracle_params_init(const gsph_scene *s, gsph_params *p) {
    memset(p, 0, sizeof(*p));
    p->kernel = isnan(s->kernel) ? 0.03f : s->kernel;
    p->mass = s->mass;
    p->kernel_2 = p->kernel * p->kernel;
    for (int a = 0; a < 3; ++a) p->world_size[a] = s->world[a];
    p->cell_size = p->kernel;
    p->inv_cell_size = 1.0f / p->cell_size;
    for (int a = 0; a < 3; ++a) {
        float g = ceilf(p->world_size[a] / p->cell_size);
        if (!(g >= 1.f) || g > 65535.f) return -1;
        p->grid_size[a] = (int32_t)g;
    }
    p->gravity[0] = 0.0f;
    p->gravity[1] = isnan(s->gravity_y) ? -9.8f : s->gravity_y;
    p->gravity[2] = 0.0f;
    p->wall_damping = -0.5f;
    p->rest_density = isnan(s->rest_density) ? 1000.0f : s->rest_density;
    p->gas_constant = isnan(s->gas_constant) ? 1.0f : s->gas_constant;
    p->viscosity = isnan(s->viscosity) ? 6.5f : s->viscosity;
    p->time_step = isnan(s->time_step) ? 0.003f : s->time_step;
    p->surface_normal = 0.1f;
    p->surface_coe = 0.2f;
    const double k = (double)p->kernel;
    p->poly6_value = (float)(315.0f / (64.0f * M_PI * pow(k, 9)));
    p->spiky_value = (float)(-45.0f / (M_PI * pow(k, 6)));
    p->visco_value = (float)(45.0f / (M_PI * pow(k, 6)));
    p->grad_poly6 = (float)(-945 / (32 * M_PI * pow(k, 9)));
    p->lplc_poly6 = (float)(945 / (8 * M_PI * pow(k, 9)));
    p->self_density = (float)((double)(p->mass * p->poly6_value) * pow(k, 6));
    p->inv_rest_density = 1.0f / p->rest_density;
    p->density_scale = p->mass * p->poly6_value;
    p->half_spiky_value = p->spiky_value * 0.5f;
    p->viscosity_visco_value = p->viscosity * p->visco_value;
    p->grad_color_scale = p->grad_poly6 * p->mass;
    p->lplc_color_scale = p->lplc_poly6 * p->mass;
    p->bound_interval = p->kernel;
    for (int a = 0; a < 3; ++a) {
        p->bound_min[a] = p->bound_interval;
        p->bound_max[a] = p->world_size[a] - p->bound_interval;
    }
    return 0;
}

/* Lattice without jitter: x outer, y, z inner, FP32 accumulation. Returns
 * the particle count; writes positions when pos4 != NULL. */
ORACLE_EXPORT long oracle_lattice(const gsph_scene *s, const gsph_params *p,
                                  float *pos4, long capacity) {
    const float step = p->kernel * s->interval;
    long n = 0;
    for (uint32_t b = 0; b < s->n_blocks; ++b)
        for (float x = s->block_begin[b][0]; x < s->block_end[b][0]; x += step)
            for (float y = s->block_begin[b][1]; y < s->block_end[b][1]; y += step)
                for (float z = s->block_begin[b][2]; z < s->block_end[b][2]; z += step) {
                    if (pos4) {
                        if (n >= capacity) return -1;
                        pos4[4 * n + 0] = x;
                        pos4[4 * n + 1] = y;
                        pos4[4 * n + 2] = z;
                        pos4[4 * n + 3] = 0.f;
                    }
                    ++n;
                }
    return n;
}

/* -------------------------------------------------------------- keys --- */
/* Micro coordinate along one axis: floorf(p * (4 * inv_cell)), single
 * precision (sph_utils.cuh:47-51). Out-of-grid values are clamped and
 * reported through *out. */
static inline int micro_coord(float p, float rat, int g, int *out) {
    const float f = floorf(p * rat);
    const float lim = (float)(g << 2);
    if (f >= 0.f && f < lim) return (int)f;
    *out = 1;
    if (!(f >= 0.f)) return 0;
    return (g << 2) - 1;
}

ORACLE_EXPORT int oracle_keys(const float *pos4, long n, const gsph_params *p,
                              uint32_t *key) {
    const float rat = 4.f * p->inv_cell_size;
    const int gx = p->grid_size[0], gy = p->grid_size[1], gz = p->grid_size[2];
    int bad = 0;
    for (long i = 0; i < n; ++i) {
        int o = 0;
        const int mx = micro_coord(pos4[4 * i + 0], rat, gx, &o);
        const int my = micro_coord(pos4[4 * i + 1], rat, gy, &o);
        const int mz = micro_coord(pos4[4 * i + 2], rat, gz, &o);
        bad |= o;
        const uint32_t c = (uint32_t)(mx >> 2) +
                           (uint32_t)gx * ((uint32_t)(my >> 2) + (uint32_t)gy * (uint32_t)(mz >> 2));
        /* idi = y + ((z + (x << 2)) << 2), sph_utils.cuh:95 */
        const uint32_t sub = (uint32_t)(my & 3) + (((uint32_t)(mz & 3) + ((uint32_t)(mx & 3) << 2)) << 2);
        key[i] = (c << 6) | sub;
    }
    return bad;
}

/* -------------------------------------------------------------- sort --- */
static int cmp_u64(const void *a, const void *b) {
    const uint64_t x = *(const uint64_t *)a, y = *(const uint64_t *)b;
    return (x > y) - (x < y);
}

/* Stable counting sort by micro key (ties keep the input order).
 * Outputs: key_sorted[n], perm[n] (source of each slot), cell_start[numc+1].
 * Returns 0, 1 if a particle was outside the grid (clamped), -2 on
 * allocation failure. */
ORACLE_EXPORT int oracle_sort(const float *pos4, long n, const gsph_params *p,
                              uint32_t *key_sorted, int32_t *perm,
                              int32_t *cell_start) {
    const long numc = (long)p->grid_size[0] * p->grid_size[1] * p->grid_size[2];
    uint32_t *key = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    uint64_t *pr = (uint64_t *)malloc(sizeof(uint64_t) * (size_t)(n > 0 ? n : 1));
    int32_t *fill = (int32_t *)malloc(sizeof(int32_t) * (size_t)(numc > 0 ? numc : 1));
    if (!key || !pr || !fill) {
        free(key);
        free(pr);
        free(fill);
        return -2;
    }
    const int bad = oracle_keys(pos4, n, p, key);
    /* counting sort over coarse cells ... */
    memset(cell_start, 0, sizeof(int32_t) * (size_t)(numc + 1));
    for (long i = 0; i < n; ++i) cell_start[(key[i] >> 6) + 1]++;
    for (long c = 0; c < numc; ++c) cell_start[c + 1] += cell_start[c];
    memcpy(fill, cell_start, sizeof(int32_t) * (size_t)numc);
    for (long i = 0; i < n; ++i)
        pr[fill[key[i] >> 6]++] = ((uint64_t)key[i] << 32) | (uint64_t)(uint32_t)i;
    /* ... then (micro key, input index) order inside every cell */
    for (long c = 0; c < numc; ++c) {
        const int32_t b = cell_start[c], e = cell_start[c + 1];
        if (e - b > 1) qsort(pr + b, (size_t)(e - b), sizeof(uint64_t), cmp_u64);
    }
    for (long i = 0; i < n; ++i) {
        key_sorted[i] = (uint32_t)(pr[i] >> 32);
        perm[i] = (int32_t)(pr[i] & 0xFFFFFFFFu);
    }
    free(key);
    free(pr);
    free(fill);
    return bad;
}

/* --------------------------------------------------- model and split --- */
ORACLE_EXPORT void oracle_block_req(const int32_t *cell_start,
                                    const gsph_params *p, int32_t *req) {
    const int gx = p->grid_size[0], gy = p->grid_size[1];
    const long slice = (long)gx * gy;
    const long numc = slice * p->grid_size[2];
    for (long idx = 0; idx < numc; ++idx) {
        const int self = cell_start[idx + 1] - cell_start[idx];
        if (self == 0) {
            req[idx] = 0;
            continue;
        }
        int total = self;
        const long x = idx % gx;
        const long y = (idx / gx) % gy;
#define CNT(c) (cell_start[(c) + 1] - cell_start[(c)])
        if (x > 0) total += CNT(idx - 1);
        if (x + 1 < gx) total += CNT(idx + 1);
        if (y > 0) total += CNT(idx - gx);
        if (y + 1 < gy) total += CNT(idx + gx);
        if (idx >= slice) total += CNT(idx - slice);
        if (idx + slice < numc) total += CNT(idx + slice);
#undef CNT
        if (total < 96 && self < 15)
            req[idx] = 0;
        else if (total < 60)
            req[idx] = (self + 27) >> 5;
        else
            req[idx] = (self + 31) >> 5;
    }
}

/* Compact index (TRA particles by cell, then SMS particles by cell) and the
 * split point "middle" (number of TRA particles). A particle is SMS when its
 * offset inside its cell is below 32*req. Returns middle. */
ORACLE_EXPORT long oracle_split(const int32_t *cell_start, const int32_t *req,
                                const gsph_params *p, int32_t *compact) {
    const long numc = (long)p->grid_size[0] * p->grid_size[1] * p->grid_size[2];
    long middle = 0;
    for (long c = 0; c < numc; ++c) {
        const int b = cell_start[c], n = cell_start[c + 1] - b;
        int sms = req[c] * 32;
        if (sms > n) sms = n;
        for (int j = sms; j < n; ++j) compact[middle++] = b + j;
    }
    long k = middle;
    for (long c = 0; c < numc; ++c) {
        const int b = cell_start[c], n = cell_start[c + 1] - b;
        int sms = req[c] * 32;
        if (sms > n) sms = n;
        for (int j = 0; j < sms; ++j) compact[k++] = b + j;
    }
    return middle;
}

static uint16_t pack_bounds(int a, int b, int c, int d, int e, int f) {
    return (uint16_t)(a | (b << 2) | (c << 4) | (d << 6) | (e << 8) | (f << 10));
}

/* knArrangeSmsTasks + judgeTask. tasks must hold T + 1 entries. Returns T. */
ORACLE_EXPORT long oracle_tasks(const uint32_t *key_sorted,
                                const int32_t *cell_start, const int32_t *req,
                                const gsph_params *p, gsph_block_task *tasks,
                                long capacity) {
    const int gx = p->grid_size[0], gy = p->grid_size[1];
    const long numc = (long)gx * gy * p->grid_size[2];
    long t = 0;
    for (long c = 0; c < numc; ++c) {
        const int b = cell_start[c], n = cell_start[c + 1] - b;
        for (int l = 0; l < req[c]; ++l) {
            if (t >= capacity - 1) return -1;
            const int off = l * 32;
            const int last = (off + 31 < n - 1) ? off + 31 : n - 1;
            const uint32_t fh = key_sorted[b + off], lh = key_sorted[b + last];
            gsph_block_task k;
            memset(&k, 0, sizeof(k));
            k.cellid = (int32_t)c;
            k.cell_pos[0] = (uint16_t)(c % gx);
            k.cell_pos[1] = (uint16_t)(c / gx % gy);
            k.cell_pos[2] = (uint16_t)(c / gx / gy);
            k.cell_begin = b;
            k.cell_particle_count = n;
            k.p_offset = (uint16_t)off;
            const int min_x = (fh >> 4) & 3, max_x = (lh >> 4) & 3;
            const int min_z = (fh >> 2) & 3, max_z = (lh >> 2) & 3;
            const int min_y = fh & 3, max_y = lh & 3;
            k.xxi = (int8_t)min_x;
            k.xxx = (int8_t)max_x;
            if (min_x == max_x) {
                k.zzi = (int8_t)min_z;
                k.zzz = (int8_t)max_z;
                if (min_z == max_z) {
                    k.yyi = (int8_t)min_y;
                    k.yyy = (int8_t)max_y;
                } else {
                    k.yyi = 0;
                    k.yyy = 3;
                }
            } else {
                k.zzi = 0;
                k.zzz = 3;
                k.yyi = 0;
                k.yyy = 3;
            }
            k.paired_bounds = pack_bounds(k.xxi, k.xxx, k.yyi, k.yyy, k.zzi, k.zzz);
            tasks[t++] = k;
        }
    }
    const long T = t;
    for (long first = 0; first < T; first += 2) {
        const long second = first + 1;
        if (second >= T) {
            gsph_block_task pad = tasks[first];
            tasks[first].is_same = 1;
            pad.is_same = 1;
            pad.p_offset = (uint16_t)(tasks[first].p_offset + 32);
            tasks[second] = pad;
            break;
        }
        if (tasks[first].cellid != tasks[second].cellid) {
            tasks[first].is_same = 0;
            tasks[second].is_same = 0;
            continue;
        }
        int zmin = tasks[first].zzi, zmax = tasks[first].zzz;
        if (tasks[first].xxi == tasks[second].xxx) {
            zmax = tasks[second].zzz;
        } else {
            zmin = 0;
            zmax = 3;
        }
        tasks[first].is_same = 1;
        tasks[second].is_same = 1;
        tasks[first].paired_bounds =
            pack_bounds(tasks[first].xxi, tasks[second].xxx, tasks[first].yyi,
                        tasks[first].yyy, zmin, zmax);
    }
    return T;
}

/* ----------------------------------------------------------- physics --- */
/* Coarse cell coordinates of a sorted particle, from its micro key. */
static inline void key_cell(uint32_t key, int gx, int gy, int *cx, int *cy,
                            int *cz) {
    const uint32_t c = key >> 6;
    *cx = (int)(c % (uint32_t)gx);
    *cy = (int)(c / (uint32_t)gx % (uint32_t)gy);
    *cz = (int)(c / (uint32_t)gx / (uint32_t)gy);
}

/* FP64 density core on double positions. */
static void density_d(const double *pos4, const uint32_t *key_sorted,
                      const int32_t *cell_start, long n, const gsph_params *p,
                      double *rho, double *pressure) {
    const int gx = p->grid_size[0], gy = p->grid_size[1], gz = p->grid_size[2];
    const double h2 = (double)p->kernel * (double)p->kernel;
    const double scale = (double)p->density_scale, self_d = (double)p->self_density;
#pragma omp parallel for schedule(dynamic, 1024)
    for (long i = 0; i < n; ++i) {
        int cx, cy, cz;
        key_cell(key_sorted[i], gx, gy, &cx, &cy, &cz);
        const double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        double s = 0.0;
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= gx || y >= gy || z >= gz) continue;
                    const long c = x + (long)gx * (y + (long)gy * z);
                    for (int j = cell_start[c]; j < cell_start[c + 1]; ++j) {
                        const double rx = xi - pos4[4 * j], ry = yi - pos4[4 * j + 1],
                                     rz = zi - pos4[4 * j + 2];
                        const double d2 = rx * rx + ry * ry + rz * rz;
                        if (d2 > h2 || d2 < 1e-12) continue;
                        const double t = h2 - d2;
                        s += t * t * t;
                    }
                }
        const double r = s * scale + self_d;
        rho[i] = r;
        pressure[i] = (pow(r * (1.0 / (double)p->rest_density), 7) - 1.0) *
                      (double)p->gas_constant;
    }
}

/* FP64 force core on double state (pos w = 1/rho, ev w = pressure). */
/* model: 0 = the reference's Laplacian viscosity (force_kernels.cu:378-435);
 * 1 = Monaghan's artificial viscosity (Monaghan 1992) in its place, with
 * art_coef = alpha * c0: for v_ij . r_ij < 0, mu = h v_ij . r_ij /
 * (r^2 + 0.01 h^2), Pi = -alpha c0 mu / ((rho_i + rho_j) / 2), force
 * -m rho_i sum_j Pi grad W_spiky(r_ij). */
static void force_d(const double *pos4, const double *ev4,
                    const uint32_t *key_sorted, const int32_t *cell_start,
                    long n, const gsph_params *p, int model, double art_coef,
                    double *acc3, double *mag) {
    const int gx = p->grid_size[0], gy = p->grid_size[1], gz = p->grid_size[2];
    const double h = (double)p->kernel, h2 = h * h;
    const double art_eps = (double)(0.01f * p->kernel_2);
#pragma omp parallel for schedule(dynamic, 1024)
    for (long i = 0; i < n; ++i) {
        int cx, cy, cz;
        key_cell(key_sorted[i], gx, gy, &cx, &cy, &cz);
        const double xi = pos4[4 * i], yi = pos4[4 * i + 1], zi = pos4[4 * i + 2];
        const double inv_rho_i = pos4[4 * i + 3];
        const double vxi = ev4[4 * i], vyi = ev4[4 * i + 1], vzi = ev4[4 * i + 2],
                     pi = ev4[4 * i + 3];
        double P[3] = {0, 0, 0}, Vs[3] = {0, 0, 0}, G[3] = {0, 0, 0}, L = 0.0;
        double Pm = 0.0, Vm = 0.0;   /* sums of |pair term| (conditioning) */
        for (int dz = -1; dz <= 1; ++dz)
            for (int dy = -1; dy <= 1; ++dy)
                for (int dx = -1; dx <= 1; ++dx) {
                    const int x = cx + dx, y = cy + dy, z = cz + dz;
                    if (x < 0 || y < 0 || z < 0 || x >= gx || y >= gy || z >= gz) continue;
                    const long c = x + (long)gx * (y + (long)gy * z);
                    for (int j = cell_start[c]; j < cell_start[c + 1]; ++j) {
                        const double rx = xi - pos4[4 * j], ry = yi - pos4[4 * j + 1],
                                     rz = zi - pos4[4 * j + 2];
                        const double d2 = rx * rx + ry * ry + rz * rz;
                        if (d2 > h2 || d2 < 1e-12) continue;
                        const double d = sqrt(d2);
                        const double V = pos4[4 * j + 3];
                        const double k = h - d;
                        const double pw = V * (pi + ev4[4 * j + 3]) * k * k / d;
                        P[0] -= rx * pw;
                        P[1] -= ry * pw;
                        P[2] -= rz * pw;
                        Pm += fabs(pw) * d;
                        const double wk = V * k;
                        double ux, uy, uz;
                        if (model == 1) {
                            const double vr = (vxi - ev4[4 * j]) * rx +
                                              (vyi - ev4[4 * j + 1]) * ry +
                                              (vzi - ev4[4 * j + 2]) * rz;
                            double w = 0.0;
                            if (vr < 0.0) {
                                const double mu = h * vr / (d2 + art_eps);
                                const double rho_mean = 0.5 * (1.0 / inv_rho_i + 1.0 / V);
                                w = -art_coef * mu / rho_mean * k * k / d;
                            }
                            ux = rx * w;
                            uy = ry * w;
                            uz = rz * w;
                        } else {
                            ux = (ev4[4 * j] - vxi) * wk;
                            uy = (ev4[4 * j + 1] - vyi) * wk;
                            uz = (ev4[4 * j + 2] - vzi) * wk;
                        }
                        Vs[0] += ux;
                        Vs[1] += uy;
                        Vs[2] += uz;
                        Vm += sqrt(ux * ux + uy * uy + uz * uz);
                        const double hr = h2 - d2;
                        const double gw = V * hr * hr;
                        G[0] += rx * gw;
                        G[1] += ry * gw;
                        G[2] += rz * gw;
                        L += V * hr * (d2 - 0.75 * hr);
                    }
                }
        const double vcoef = model == 1 ? -(double)p->spiky_value / inv_rho_i
                                        : (double)p->viscosity_visco_value;
        double F[3];
        for (int a = 0; a < 3; ++a)
            F[a] = (P[a] * (double)p->half_spiky_value + Vs[a] * vcoef) * (double)p->mass;
        for (int a = 0; a < 3; ++a) G[a] *= (double)p->grad_color_scale;
        L *= (double)p->lplc_color_scale * inv_rho_i;
        const double nrm = sqrt(G[0] * G[0] + G[1] * G[1] + G[2] * G[2]);
        for (int a = 0; a < 3; ++a) {
            double sf = 0.0;
            if (nrm > (double)p->surface_normal)
                sf = G[a] * (double)p->surface_coe * L / nrm;
            acc3[3 * i + a] = F[a] + sf;
        }
        if (mag)
            mag[i] = (Pm * fabs((double)p->half_spiky_value) + Vm * fabs(vcoef)) *
                     (double)p->mass;
    }
}

static double *widen(const float *a, long count) {
    double *d = (double *)malloc(sizeof(double) * (size_t)(count > 0 ? count : 1));
    if (!d) return NULL;
    for (long i = 0; i < count; ++i) d[i] = (double)a[i];
    return d;
}

/* Density of every sorted particle (FP64) from single-precision sorted
 * positions (key_sorted/cell_start from oracle_sort). Outputs rho[n] and
 * pressure[n] = ((rho/rho0)^7 - 1) * B. Returns 0, or -2 on allocation
 * failure. */
ORACLE_EXPORT int oracle_density(const float *pos4, const uint32_t *key_sorted,
                                 const int32_t *cell_start, long n,
                                 const gsph_params *p, double *rho,
                                 double *pressure) {
    double *pd = widen(pos4, 4 * n);
    if (!pd) return -2;
    density_d(pd, key_sorted, cell_start, n, p, rho, pressure);
    free(pd);
    return 0;
}

/* Force of every sorted particle (FP64) from single-precision inputs with
 * pos4.w = 1/rho and ev4.w = pressure as the density pass stores them.
 * Output acc3[3n]; mag[n] (may be NULL) receives the sum over pairs of the
 * magnitude of each pressure and viscosity pair term, i.e. the scale of the
 * rounding error of any summation of those terms. */
ORACLE_EXPORT int oracle_force(const float *pos4, const float *ev4,
                               const uint32_t *key_sorted,
                               const int32_t *cell_start, long n,
                               const gsph_params *p, double *acc3,
                               double *mag) {
    double *pd = widen(pos4, 4 * n), *ed = widen(ev4, 4 * n);
    if (!pd || !ed) {
        free(pd);
        free(ed);
        return -2;
    }
    force_d(pd, ed, key_sorted, cell_start, n, p, 0, 0.0, acc3, mag);
    free(pd);
    free(ed);
    return 0;
}

/* oracle_force with a choice of viscosity model (0: the reference's
 * Laplacian; 1: Monaghan's artificial viscosity with alpha and c0). */
ORACLE_EXPORT int oracle_force_model(const float *pos4, const float *ev4,
                                     const uint32_t *key_sorted,
                                     const int32_t *cell_start, long n,
                                     const gsph_params *p, int model, double alpha,
                                     double c0, double *acc3, double *mag) {
    double *pd = widen(pos4, 4 * n), *ed = widen(ev4, 4 * n);
    if (!pd || !ed) {
        free(pd);
        free(ed);
        return -2;
    }
    force_d(pd, ed, key_sorted, cell_start, n, p, model,
            (double)((float)alpha * (float)c0), acc3, mag);
    free(pd);
    free(ed);
    return 0;
}

/* knIntegrateVelocityE in FP64 on the given state (in place). pos4/vel4/ev4
 * are double[4n] (pos w = 1/rho, ev w = pressure), acc3 double[3n]. */
ORACLE_EXPORT void oracle_integrate(double *pos4, double *vel4, double *ev4,
                                    const double *acc3, long n,
                                    const gsph_params *p) {
    const double alpha = 20000000.0, beta = 200000.0;
    const double kernel = (double)(float)((double)p->kernel + 0.01);
    const double bmin[3] = {p->bound_min[0], p->bound_min[1], p->bound_min[2]};
    const double bmax[3] = {p->bound_max[0], p->bound_max[1], p->bound_max[2]};
    const double g[3] = {p->gravity[0], p->gravity[1], p->gravity[2]};
    const double dt = (double)p->time_step, damp = (double)p->wall_damping;
#pragma omp parallel for schedule(static)
    for (long i = 0; i < n; ++i) {
        double *x = pos4 + 4 * i, *v = vel4 + 4 * i, *e = ev4 + 4 * i;
        double a[3] = {acc3[3 * i], acc3[3 * i + 1], acc3[3 * i + 2]};
        /* penalty walls, order y, x, z (integration_kernels.cu:255-288) */
        static const int order[3] = {1, 0, 2};
        for (int q = 0; q < 3; ++q) {
            const int ax = order[q];
            double diff = kernel - (x[ax] - bmin[ax]);
            if (diff > 0.0) a[ax] += alpha * diff - beta * v[ax];
            diff = kernel - (bmax[ax] - x[ax]);
            if (diff > 0.0) a[ax] -= alpha * diff + beta * v[ax];
        }
        for (int q = 0; q < 3; ++q) a[q] = a[q] * x[3] + g[q];
        double sp = a[0] * a[0] + a[1] * a[1] + a[2] * a[2];
        if (sp > 3000000.0) {
            const double s = sqrt(3000000.0 / sp);
            for (int q = 0; q < 3; ++q) a[q] *= s;
        }
        double nv[3];
        for (int q = 0; q < 3; ++q) nv[q] = v[q] + a[q] * dt;
        sp = nv[0] * nv[0] + nv[1] * nv[1] + nv[2] * nv[2];
        if (sp > 36.0) {
            const double s = sqrt(36.0 / sp);
            for (int q = 0; q < 3; ++q) nv[q] *= s;
        }
        double np[3];
        for (int q = 0; q < 3; ++q) np[q] = x[q] + nv[q] * dt;
        for (int q = 0; q < 3; ++q) {
            if (np[q] >= bmax[q]) {
                nv[q] *= damp;
                np[q] = bmax[q] - kernel;
            }
            if (np[q] <= bmin[q]) {
                nv[q] *= damp;
                np[q] = bmin[q] + kernel;
            }
        }
        for (int q = 0; q < 3; ++q) {
            e[q] = (nv[q] + e[q]) * 0.5;
            x[q] = np[q];
            v[q] = nv[q];
        }
    }
}

/* One full frame (tick) on an FP64 state: sort, density, force, integrate.
 * State arrays are double[4n], reordered in place into sorted order. Keys
 * are computed from the single-precision rounding of the positions, exactly
 * as the device would see them. Returns 0, or 1 if a particle left the grid. */
ORACLE_EXPORT int oracle_step(double *pos4, double *vel4, double *ev4, long n,
                              const gsph_params *p) {
    const long numc = (long)p->grid_size[0] * p->grid_size[1] * p->grid_size[2];
    float *pf = (float *)malloc(sizeof(float) * 4 * (size_t)(n > 0 ? n : 1));
    uint32_t *ks = (uint32_t *)malloc(sizeof(uint32_t) * (size_t)(n > 0 ? n : 1));
    int32_t *perm = (int32_t *)malloc(sizeof(int32_t) * (size_t)(n > 0 ? n : 1));
    int32_t *cs = (int32_t *)malloc(sizeof(int32_t) * (size_t)(numc + 1));
    double *tmp = (double *)malloc(sizeof(double) * 12 * (size_t)(n > 0 ? n : 1));
    double *rho = (double *)malloc(sizeof(double) * 2 * (size_t)(n > 0 ? n : 1));
    double *acc = (double *)malloc(sizeof(double) * 3 * (size_t)(n > 0 ? n : 1));
    if (!pf || !ks || !perm || !cs || !tmp || !rho || !acc) {
        free(pf); free(ks); free(perm); free(cs); free(tmp); free(rho); free(acc);
        return -2;
    }
    for (long i = 0; i < 4 * n; ++i) pf[i] = (float)pos4[i];
    const int bad = oracle_sort(pf, n, p, ks, perm, cs);
    /* reorder the double state */
    memcpy(tmp, pos4, sizeof(double) * 4 * (size_t)n);
    memcpy(tmp + 4 * n, vel4, sizeof(double) * 4 * (size_t)n);
    memcpy(tmp + 8 * n, ev4, sizeof(double) * 4 * (size_t)n);
    for (long i = 0; i < n; ++i)
        for (int q = 0; q < 4; ++q) {
            pos4[4 * i + q] = tmp[4 * perm[i] + q];
            vel4[4 * i + q] = tmp[4 * n + 4 * perm[i] + q];
            ev4[4 * i + q] = tmp[8 * n + 4 * perm[i] + q];
        }
    density_d(pos4, ks, cs, n, p, rho, rho + n);
    for (long i = 0; i < n; ++i) {
        pos4[4 * i + 3] = 1.0 / rho[i];
        ev4[4 * i + 3] = rho[n + i];
    }
    force_d(pos4, ev4, ks, cs, n, p, 0, 0.0, acc, NULL);
    oracle_integrate(pos4, vel4, ev4, acc, n, p);
    free(pf); free(ks); free(perm); free(cs); free(tmp); free(rho); free(acc);
    return bad;
}

ORACLE_EXPORT int oracle_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}
