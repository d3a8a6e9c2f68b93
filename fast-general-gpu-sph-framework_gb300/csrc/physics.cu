// physics.cu — density, force and integration (rows A10-A12), plus the FP64
// state reductions.
//
// Reference behaviour (KemengHuang/Fast-General-GPU-SPH-framework):
//   density    src/solver/density_kernels.cu:160-179 (TRA loop), 278-295
//              (SMS batch), 297-565 (hybrid kernel; 1/rho -> position.w,
//              pressure -> evaluated_velocity.w)
//   force      src/solver/force_kernels.cu:378-435 (SMS batch), 525-561 (TRA
//              loop), 725-1054 (hybrid kernel: spiky pressure, Mueller
//              viscosity, colour-field surface tension -> acceleration)
//   rows       src/solver/kernel_common.cuh:69-112 (TRA row range),
//              614-674 (SMS row range from task micro bounds)
//   integrate  src/solver/integration_kernels.cu:235-336 (knIntegrateVelocityE)
//   checksum   src/simulation/sph_hybrid_system.cpp:43-62
//
// Design here: one persistent kernel per pass and path; each warp repeatedly
// takes a work unit from a device counter — 32 TRA particles (one per lane) or
// one 32-particle SMS task (candidates staged in batches in shared memory,
// evaluated two at a time with packed FP32x2 arithmetic by every lane). The
// grid is sized from the SM count, so the launch needs neither the host-side
// TRA/SMS counts nor a host synchronisation. Neighbour rows merge the three
// x-adjacent cells of each (dy, dz) row into one contiguous index range,
// pruned by micro-x slab as in the reference (SMS rows at dz = -1 / +1 are
// further cut to the micro-z groups that reach the task). Candidates are
// visited rows z-major, then in increasing sorted index; the TRA density pass
// records which interact as bit masks that the TRA force pass walks.
#include <algorithm>

#include "gsph_internal.h"

namespace gsph {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;
constexpr float kFloatSmall = 1e-12f;   // core/cuda_math.cuh:14

__device__ __forceinline__ float powf_7(float b) {
    // kernel_common.cuh:51-55, six sequential multiplies
    return b * b * b * b * b * b * b;
}

// Squared distance with one fixed rounding sequence (x^2, then + y^2, then
// + z^2, each fused), shared by the force passes.
__device__ __forceinline__ float sq_dist(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmul_rn(dx, dx)));
}

// The TRA density pass's cut-off test in one unsigned compare: with
// e = d^2 - kFloatSmall (the subtraction folded into the first fused
// multiply-add), the reference's kFloatSmall <= d^2 <= h^2 is
// 0 <= e <= h^2 - kFloatSmall, and for FP32 values that is
// bits(e) <= bits(h^2 - kFloatSmall) (a negative e has its sign bit set).
// The weight (h^2 - d^2) is then (h^2 - kFloatSmall) - e. Only roundings
// differ from the two-compare form; pairs at the cut-off contribute zero
// either way.
__device__ __forceinline__ float sq_dist_less_small(float dx, float dy, float dz) {
    return __fmaf_rn(dz, dz, __fmaf_rn(dy, dy, __fmaf_rn(dx, dx, -kFloatSmall)));
}

// Start of micro-x slab `lo` of cell c (0 = cell start).
__device__ __forceinline__ int slab_begin(const Frame &f, int c, int s, int e,
                                          int lo) {
    if (lo == 0) return s;
    const uint32_t xs = f.cell_xslab[c];
    if (xs == kXslabUnknown) return s;
    return s + min(int((xs >> (10 * (lo - 1))) & 1023u), e - s);
}
// End of micro-x slab `hi` of cell c (3 = cell end).
__device__ __forceinline__ int slab_end(const Frame &f, int c, int s, int e,
                                        int hi) {
    if (hi == 3) return e;
    const uint32_t xs = f.cell_xslab[c];
    if (xs == kXslabUnknown) return e;
    return s + min(int((xs >> (10 * hi)) & 1023u), e - s);
}

// Contiguous candidate range of one neighbour row: left cell from micro-x
// `lo`, the middle cell, right cell up to micro-x `hi` (kernel_common.cuh:
// 69-112 for TRA with lo = hi = own micro-x; 614-674 for SMS tasks).
__device__ __forceinline__ void row_range(const Frame &f, const SceneGeom &G,
                                          int m, int cx, int lo, int hi,
                                          int &begin, int &end) {
    const int sM = f.cell_start[m];
    const int eM = f.cell_start[m + 1];
    begin = sM;
    end = eM;
    if (cx > 0) begin = slab_begin(f, m - 1, f.cell_start[m - 1], sM, lo);
    if (cx + 1 < G.gx) end = slab_end(f, m + 1, eM, f.cell_start[m + 2], hi);
}

struct MicroPos {
    int cx, cy, cz, lmx;
};

__device__ __forceinline__ MicroPos micro_of(float4 p, const DevParams &P,
                                             const SceneGeom &G) {
    // Same float arithmetic as the key (grid.cu); positions are inside the
    // grid after the arrange stage has clamped/flagged them.
    int mx = int(floorf(p.x * P.rat));
    int my = int(floorf(p.y * P.rat));
    int mz = int(floorf(p.z * P.rat));
    mx = min(max(mx, 0), (G.gx << 2) - 1);
    my = min(max(my, 0), (G.gy << 2) - 1);
    mz = min(max(mz, 0), (G.gz << 2) - 1);
    MicroPos r;
    r.cx = mx >> 2;
    r.cy = my >> 2;
    r.cz = mz >> 2;
    r.lmx = mx & 3;
    return r;
}

struct ForceAcc {
    float px, py, pz;   // pressure sum
    float vx, vy, vz;   // viscosity sum
    float gx, gy, gz;   // colour gradient
    float lap;          // colour laplacian
};

// Monaghan's artificial viscosity of one interacting pair (the optional
// GSPH_VISCOSITY_ARTIFICIAL model, Monaghan 1992): for v_ij . r_ij < 0,
// mu = h v_ij . r_ij / (r^2 + 0.01 h^2), Pi = -alpha c0 mu / rho_mean with
// rho_mean = (rho_i + rho_j) / 2 = (V_i + V_j) / (2 V_i V_j), V = 1/rho.
// Returns Pi (h - r)^2 / r, the factor of r_ij in sum_j Pi grad W / spiky;
// zero for a separating pair.
__device__ __forceinline__ float artificial_pair(float vr, float d2, float k,
                                                 float inv_d, float vi, float vj,
                                                 const DevParams &P) {
    if (!(vr < 0.f)) return 0.f;
    const float mu = __fdividef(P.h * vr, d2 + P.art_eps);
    const float pij = __fdividef(-2.f * P.art_coef * mu * vi * vj, vi + vj);
    return pij * k * k * inv_d;
}

// kChecked = false for neighbours taken from the density pass's masks: the
// masks were set by the same squared distance and the same cut-off test, so
// the test would always pass. kArt: the viscosity slots of the accumulator
// hold Monaghan's sum_j Pi (h - r)^2 / r r_ij instead of the reference's
// Laplacian term.
template <bool kChecked = true, bool kArt = false>
__device__ __forceinline__ void force_pair(const float4 &self,
                                           const float4 &sev, const float4 &q,
                                           const float4 &qev,
                                           const DevParams &P, ForceAcc &a) {
    const float rx = self.x - q.x, ry = self.y - q.y, rz = self.z - q.z;
    const float d2 = sq_dist(rx, ry, rz);
    if (kChecked && (P.h2 < d2 || kFloatSmall > d2)) return;
    const float inv_d = rsqrtf(d2);
    const float d = d2 * inv_d;
    const float V = q.w;   // 1/rho_j
    const float k = P.h - d;
    const float wk = V * k;
    const float pw = wk * (sev.w + qev.w) * k;
    const float ps = pw * inv_d;
    a.px -= rx * ps;
    a.py -= ry * ps;
    a.pz -= rz * ps;
    if (kArt) {
        const float vr = (sev.x - qev.x) * rx + (sev.y - qev.y) * ry + (sev.z - qev.z) * rz;
        const float w = artificial_pair(vr, d2, k, inv_d, self.w, V, P);
        a.vx += rx * w;
        a.vy += ry * w;
        a.vz += rz * w;
    } else {
        a.vx += (qev.x - sev.x) * wk;
        a.vy += (qev.y - sev.y) * wk;
        a.vz += (qev.z - sev.z) * wk;
    }
    const float h2r2 = P.h2 - d2;
    const float wh = V * h2r2;
    const float gw = wh * h2r2;
    a.gx += rx * gw;
    a.gy += ry * gw;
    a.gz += rz * gw;
    a.lap += wh * (d2 - 0.75f * h2r2);
}

__device__ __forceinline__ void write_density(const Frame &f, const DevParams &P,
                                              int self, float sum, bool sms) {
    float rho = sum * P.density_scale + P.self_density;
    // The SMS path of the reference guards rho < 1e-12 before the reciprocal
    // (density_kernels.cu:540-541); the TRA path does not (:353-355).
    const float stored = (sms && rho < kFloatSmall) ? P.rest_density : rho;
    f.pos[self].w = __fdividef(1.0f, stored);
    f.ev[self].w = (powf_7(rho * P.inv_rest_density) - 1) * P.gas_constant;
}

// knIntegrateVelocityE (integration_kernels.cu:235-336), same operation order:
// penalty walls on the old velocity, a = F/rho + g, clamps, semi-implicit
// Euler, damped reflection, ev = (v_new + ev_old) / 2; 1/rho and pressure
// are kept.
__device__ __forceinline__ void integrate_one(const float4 tp, const float4 v4,
                                              const float4 ev, float ax, float ay,
                                              float az, const DevParams &P,
                                              const SceneGeom &G, float4 &pos_out,
                                              float4 &vel_out, float4 &ev_out) {
    float vx = v4.x, vy = v4.y, vz = v4.z;
    const float alpha = 20000000.f;
    const float beta = 200000.f;
    const float kernel = P.wall_kernel;
    float diff;
    diff = kernel - (tp.y - P.bmin);
    if (diff > 0.0f) ay += alpha * diff - beta * vy;
    diff = kernel - (G.bmax_y - tp.y);
    if (diff > 0.0f) ay -= alpha * diff + beta * vy;
    diff = kernel - (tp.x - P.bmin);
    if (diff > 0.0f) ax += alpha * diff - beta * vx;
    diff = kernel - (G.bmax_x - tp.x);
    if (diff > 0.0f) ax -= alpha * diff + beta * vx;
    diff = kernel - (tp.z - P.bmin);
    if (diff > 0.0f) az += alpha * diff - beta * vz;
    diff = kernel - (G.bmax_z - tp.z);
    if (diff > 0.0f) az -= alpha * diff + beta * vz;
    const float acc_limit = 3000000.f;
    const float vel_limit = 36.f;
    ax = ax * tp.w + P.gx_acc;
    ay = ay * tp.w + P.gy_acc;
    az = az * tp.w + P.gz_acc;
    float speed = ax * ax + ay * ay + az * az;
    if (speed > acc_limit) {
        const float s = sqrtf(acc_limit / speed);
        ax *= s;
        ay *= s;
        az *= s;
    }
    vx += ax * P.time_step;
    vy += ay * P.time_step;
    vz += az * P.time_step;
    speed = vx * vx + vy * vy + vz * vz;
    if (speed > vel_limit) {
        const float s = sqrtf(vel_limit / speed);
        vx *= s;
        vy *= s;
        vz *= s;
    }
    float px = tp.x + vx * P.time_step;
    float py = tp.y + vy * P.time_step;
    float pz = tp.z + vz * P.time_step;
    if (px >= G.bmax_x) { vx *= P.wall_damping; px = G.bmax_x - kernel; }
    if (px <= P.bmin) { vx *= P.wall_damping; px = P.bmin + kernel; }
    if (py >= G.bmax_y) { vy *= P.wall_damping; py = G.bmax_y - kernel; }
    if (py <= P.bmin) { vy *= P.wall_damping; py = P.bmin + kernel; }
    if (pz >= G.bmax_z) { vz *= P.wall_damping; pz = G.bmax_z - kernel; }
    if (pz <= P.bmin) { vz *= P.wall_damping; pz = P.bmin + kernel; }
    pos_out = make_float4(px, py, pz, tp.w);
    vel_out = make_float4(vx, vy, vz, 0.f);
    ev_out = make_float4((vx + ev.x) * 0.5f, (vy + ev.y) * 0.5f, (ev.z + vz) * 0.5f, ev.w);
}

// Writes the force; with f.pos_next set, also integrates the particle (the
// same arithmetic as k_integrate on the stored force) into the next buffers.
__device__ __forceinline__ void write_force(const Frame &f, const DevParams &P,
                                            int self, const float4 &p,
                                            const float4 &pev, const SceneGeom &G,
                                            const ForceAcc &a, bool sms) {
    float tx, ty, tz;
    if (P.visc_artificial) {
        // -m rho_i sum Pi grad W: the mass is applied below with the rest
        const float c = -P.spiky * __fdividef(1.0f, p.w);
        tx = a.px * P.half_spiky + a.vx * c;
        ty = a.py * P.half_spiky + a.vy * c;
        tz = a.pz * P.half_spiky + a.vz * c;
    } else {
        tx = a.px * P.half_spiky + a.vx * P.visco_coef;
        ty = a.py * P.half_spiky + a.vy * P.visco_coef;
        tz = a.pz * P.half_spiky + a.vz * P.visco_coef;
    }
    const float gx = a.gx * P.grad_color_scale;
    const float gy = a.gy * P.grad_color_scale;
    const float gz = a.gz * P.grad_color_scale;
    float lap = a.lap * P.lplc_color_scale;
    lap *= p.w;   // 1/rho_i
    float sx = 0.f, sy = 0.f, sz = 0.f;
    const float n2 = gx * gx + gy * gy + gz * gz;
    if (sms) {
        // force_kernels.cu:1030-1043
        const float inv_n = rsqrtf(n2);
        const float nrm = n2 * inv_n;
        if (nrm > P.surface_normal) {
            const float s = P.surface_coe * lap * inv_n;
            sx = gx * s;
            sy = gy * s;
            sz = gz * s;
        }
    } else {
        // force_kernels.cu:796-805
        const float nrm = sqrtf(n2);
        if (nrm > P.surface_normal) {
            sx = gx * P.surface_coe * lap / nrm;
            sy = gy * P.surface_coe * lap / nrm;
            sz = gz * P.surface_coe * lap / nrm;
        }
    }
    tx *= P.mass;
    ty *= P.mass;
    tz *= P.mass;
    const float4 acc = make_float4(tx + sx, ty + sy, tz + sz, 0.f);
    if (f.acc) f.acc[self] = acc;   // null in the fused frames of a step but its last
    if (f.pos_next) {
        float4 po, vo, eo;
        integrate_one(p, f.vel[self], pev, acc.x, acc.y, acc.z, P, G, po, vo, eo);
        f.pos_next[self] = po;
        f.vel_next[self] = vo;
        f.ev_next[self] = eo;
        if (f.hash_next && !sms) {   // SMS particles: launch_hash_sms
            const uint32_t key = micro_key(po, P, G, f.ctr, self);
            f.key_in[self] = key;
            f.slot[self] = cell_slot(f.cell_count, key >> 6, __activemask());
        }
    }
}

// Cell-array bytes past which the TRA density pass prefetches its rows'
// offsets: about half of the GB300's L2.
constexpr size_t kRowPrefetchCellBytes = size_t(64) << 20;

// Warps per block of the density and force kernels: 8 by default; each
// kernel is also built for 4 (gsph_tuning.warps_per_block), with twice the
// CTAs per SM for the same occupancy.
constexpr int kWarpsPerBlock = 8;
// SMS candidates staged per batch (two per lane).
constexpr int kSmsBatch = 64;
constexpr int kDenBatch = 256;   // SMS density: candidates staged per batch
// Coordinate of padding candidates: far outside any kernel radius.
constexpr float kFar = 1.0e18f;

// Next work unit of a warp from a device counter (one atomic per unit).
__device__ __forceinline__ int next_unit(int *counter) {
    int u = 0;
    if ((threadIdx.x & 31) == 0) u = atomicAdd(counter, 1);
    return __shfl_sync(kFull, u, 0);
}

// ------------------------------------------------------------ density TRA --
// One particle per lane, 32 consecutive TRA particles per work unit
// (density_kernels.cu:318-366). Which candidates of each row interact is also
// recorded as a bit mask for the force pass.
//
// kRowPrefetch: each lane first prefetches its nine rows' cell offsets and
// slab words into L1, so that the per-row set-up inside the row loop waits on
// L1 rather than DRAM. Chosen on the host when the cell arrays are too large
// to stay in L2 (large batches); otherwise the extra instructions cost more
// than they save.
template <int W, bool kRowPrefetch>
__global__ void __launch_bounds__(W * 32, 6 * kWarpsPerBlock / W)
k_density_tra(Frame f, DevParams P) {
    const int lane = threadIdx.x & 31;
    const int middle = f.ctr->middle;
    const int units = (middle + 31) >> 5;
    const bool ident = !f.ctr->any_sms;   // all TRA: compact is the identity
    for (;;) {
        const int u = next_unit(&f.ctr->work_density);
        if (u >= units) break;
        const int idx = (u << 5) + lane;
        if (idx >= middle) continue;
        const int self = ident ? idx : f.compact[idx];
        const float4 p = f.pos[self];
        const SceneGeom G = geom_of_particle(f.scenes, self);
        const MicroPos mp = micro_of(p, P, G);
        uint32_t *masks = f.nbr_mask + size_t(u) * 9 * 32 + lane;
        int incomplete = 0;
        int found = 0;
        float sum = 0.f;
        const float cut = P.h2 - kFloatSmall;
        const uint32_t cut_bits = __float_as_uint(cut);
        if (kRowPrefetch) {
            const int left = mp.cx > 0 ? 1 : 0;
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                const int ny = mp.cy + (r % 3) - 1;
                const int nz = mp.cz + (r / 3) - 1;
                if (ny >= 0 && ny < G.gy && nz >= 0 && nz < G.gz) {
                    const int m = G.cbase + mp.cx - left + G.gx * (ny + G.gy * nz);
                    asm volatile("prefetch.global.L1 [%0];" :: "l"(f.cell_start + m));
                    asm volatile("prefetch.global.L1 [%0];" :: "l"(f.cell_xslab + m));
                }
            }
        }
        for (int r = 0; r < 9; ++r) {
            const int ny = mp.cy + (r % 3) - 1;
            const int nz = mp.cz + (r / 3) - 1;
            uint32_t mask = 0u;
            if (ny >= 0 && ny < G.gy && nz >= 0 && nz < G.gz) {
                const int m = G.cbase + mp.cx + G.gx * (ny + G.gy * nz);
                int begin, end;
                row_range(f, G, m, mp.cx, mp.lmx, mp.lmx, begin, end);
                incomplete |= (end - begin > kMaskRowMax);
                uint32_t bit = 1u;
#pragma unroll 8
                for (int j = begin; j < end; ++j, bit <<= 1) {
                    const float4 q = f.pos[j];
                    const float dx = p.x - q.x, dy = p.y - q.y, dz = p.z - q.z;
                    const float e = sq_dist_less_small(dx, dy, dz);
                    if (__float_as_uint(e) > cut_bits) continue;
                    const float t = cut - e;
                    sum += t * t * t;
                    mask |= bit;
                }
            }
            masks[r * 32] = mask;
            found += __popc(mask);
        }
        f.nbr_flag[idx] = incomplete ? -1 : found;
        write_density(f, P, self, sum, false);
    }
}

// ------------------------------------------------------- SMS candidates --
// The candidates of an SMS task, row by row (rows z-major as in the
// reference), each row in increasing sorted index. Rows at dz = 0 are the
// reference's x-merged range (micro-x slabs pruned by the task's x bounds,
// kernel_common.cuh:614-674). Rows at dz = -1 / +1 are further pruned in z: a
// particle of the cell below (above) whose micro-z is below (above) every
// task particle's own micro-z is at least h away from all of them, so only
// the micro-z groups [zmin, 3] ([0, zmax]) of each micro-x slab are kept,
// using the per-cell (micro-x, micro-z) group offsets of the sort. Pruned
// candidates never interact, so the interacting set and its order are the
// same as the reference's.
//
// Segment of lane l (< 12) of row cell m: cell m - 1 + l / 4, micro-x slab
// l % 4, micro-z groups [zlo, zhi]; empty where the slab is outside the
// task's x bounds or the cell outside the grid. A cell whose groups are
// unknown (> 65,535 particles) is taken whole by its first lane.
__device__ __forceinline__ void sms_segment(const Frame &f, const SceneGeom &G, int m,
                                            int cx, int xlo, int xhi, int zlo,
                                            int zhi, int lane, int &sb, int &sl) {
    sb = 0;
    sl = 0;
    if (lane >= 12) return;
    const int k = lane >> 2, mx = lane & 3;
    if (k == 0 && (cx == 0 || mx < xlo)) return;
    if (k == 2 && (cx + 1 >= G.gx || mx > xhi)) return;
    const int c = m + k - 1;
    const int cs = f.cell_start[c];
    const int cnt = f.cell_start[c + 1] - cs;
    if (cnt <= 0) return;
    const uint16_t *g = f.cell_grp + size_t(c) * 16;
    int b, e;
    if (g[0] == kGroupsUnknown) {
        if (mx != (k == 0 ? xlo : 0)) return;
        b = k == 0 ? slab_begin(f, c, cs, cs + cnt, xlo) - cs : 0;
        e = k == 2 ? slab_end(f, c, cs, cs + cnt, xhi) - cs : cnt;
    } else {
        b = g[mx * 4 + zlo];
        e = zhi < 3 ? g[mx * 4 + zhi + 1] : (mx < 3 ? g[mx * 4 + 4] : cnt);
        b = min(b, cnt);
        e = min(e, cnt);
    }
    if (e > b) {
        sb = cs + b;
        sl = e - b;
    }
}

// Streams a task's candidates through a warp's kDenBatch-slot staging batch:
// stage(slot, index) fills one slot, run(pairs) evaluates the staged slots
// two at a time; batches run full except the last (its odd slot is padded
// by pad(slot)). Control flow is warp-uniform.
template <class Stage, class Pad, class Run>
__device__ __forceinline__ void sms_stream(const Frame &f, const SceneGeom &G,
                                           const gsph_block_task &task, int zmin,
                                           int zmax, int lane, Stage stage, Pad pad,
                                           Run run) {
    const int cx = task.cell_pos[0], cy = task.cell_pos[1], cz = task.cell_pos[2];
    int fill = 0;
    auto take_range = [&](int b, int len) {
        int o = 0;
        while (o < len) {
            const int n = min(len - o, kDenBatch - fill);
            for (int t = lane; t < n; t += 32) stage(fill + t, b + o + t);
            fill += n;
            o += n;
            if (fill == kDenBatch) {
                __syncwarp();
                run(kDenBatch / 2);
                __syncwarp();
                fill = 0;
            }
        }
    };
    for (int r = 0; r < 9; ++r) {
        const int ny = cy + (r % 3) - 1;
        const int nz = cz + (r / 3) - 1;
        if (ny < 0 || ny >= G.gy || nz < 0 || nz >= G.gz) continue;
        const int m = G.cbase + cx + G.gx * (ny + G.gy * nz);
        const int dz = r / 3 - 1;
        const int zlo = dz < 0 ? zmin : 0, zhi = dz > 0 ? zmax : 3;
        if ((zlo == 0 && zhi == 3) || !f.cell_grp) {
            int begin, end;
            row_range(f, G, m, cx, task.xxi, task.xxx, begin, end);
            take_range(begin, end - begin);
        } else {
            int sb, sl;
            sms_segment(f, G, m, cx, task.xxi, task.xxx, zlo, zhi, lane, sb, sl);
            const unsigned nonempty = __ballot_sync(kFull, sl > 0);
            for (unsigned w = nonempty; w; w &= w - 1) {
                const int src = __ffs(w) - 1;
                take_range(__shfl_sync(kFull, sb, src), __shfl_sync(kFull, sl, src));
            }
        }
    }
    if (fill > 0) {
        if ((fill & 1) && lane == 0) pad(fill);
        __syncwarp();
        run((fill + 1) >> 1);
        __syncwarp();
    }
}

// Micro-z range of a task's particles (warp-wide; inactive lanes neutral).
__device__ __forceinline__ void task_z_range(const Frame &f, int self, bool active,
                                             int &zmin, int &zmax) {
    const int mz = active ? int((f.key[self] >> 2) & 3u) : -1;
    zmin = int(__reduce_min_sync(kFull, unsigned(active ? mz : 3)));
    zmax = __reduce_max_sync(kFull, active ? mz : 0);
}

// ------------------------------------------------------------ density SMS --
// One 32-particle task per warp (density_kernels.cu:368-565). Candidates are
// streamed 256 at a time into shared memory, each pair (slots 2k, 2k+1) as an
// (x, x, y, y) float4 and a (z, z) float2; every lane evaluates them two at a
// time with packed FP32x2 arithmetic and the TRA pass's one-compare cut-off
// test.
template <int W>
__global__ void __launch_bounds__(W * 32, 4 * kWarpsPerBlock / W)
k_density_sms(Frame f, DevParams P) {
    // candidate pair k (slots 2k, 2k+1): (x, x, y, y) and (z, z)
    __shared__ __align__(16) float4 sms_xy[W][kDenBatch / 2];
    __shared__ __align__(16) float2 sms_zz[W][kDenBatch / 2];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int task_count = f.ctr->task_count;
    if (task_count == 0) return;   // no SMS work: skip the queue atomics
    float *fxy = reinterpret_cast<float *>(sms_xy[warp]);
    float *fz = reinterpret_cast<float *>(sms_zz[warp]);
    const float4 *sxy = sms_xy[warp];
    const float2 *szz = sms_zz[warp];
    for (;;) {
        const int u = next_unit(&f.ctr->work_density_sms);
        if (u >= task_count) break;
        const gsph_block_task task = f.tasks[u];
        const int cb = task.cell_begin;
        const int cend = cb + task.cell_particle_count;
        const int self = cb + task_offset(task) + lane;
        const bool active = self < cend;
        if (cb + task_offset(task) >= cend) continue;   // warp-uniform
        const float4 p = f.pos[active ? self : cend - 1];
        const SceneGeom G = geom_of_cell(f.scenes, task.cellid);
        int zmin, zmax;
        task_z_range(f, self, active, zmin, zmax);
        const float2 npx = make_float2(-p.x, -p.x);
        const float2 npy = make_float2(-p.y, -p.y);
        const float2 npz = make_float2(-p.z, -p.z);
        const float cut = P.h2 - kFloatSmall;
        const uint32_t cut_bits = __float_as_uint(cut);
        const float2 cutv = make_float2(cut, cut);
        const float2 msm = make_float2(-kFloatSmall, -kFloatSmall);
        const float2 m1 = make_float2(-1.f, -1.f);
        float2 acc = make_float2(0.f, 0.f);
        sms_stream(
            f, G, task, zmin, zmax, lane,
            [&](int slot, int j) {
                const float4 q = f.pos[j];
                const int o = (slot >> 1) * 4 + (slot & 1);
                fxy[o] = q.x;
                fxy[o + 2] = q.y;
                fz[slot] = q.z;
            },
            [&](int slot) {
                const int o = (slot >> 1) * 4 + (slot & 1);
                fxy[o] = kFar;
                fxy[o + 2] = kFar;
                fz[slot] = kFar;
            },
            [&](int pairs) {
#pragma unroll 32
                for (int k = 0; k < pairs; ++k) {
                    const float4 qa = sxy[k];
                    const float2 dx = __fadd2_rn(make_float2(qa.x, qa.y), npx);
                    const float2 dy = __fadd2_rn(make_float2(qa.z, qa.w), npy);
                    const float2 dz = __fadd2_rn(szz[k], npz);
                    // the cut-off test of sq_dist_less_small, per half
                    float2 e = __ffma2_rn(dx, dx, msm);
                    e = __ffma2_rn(dy, dy, e);
                    e = __ffma2_rn(dz, dz, e);
                    float2 t = __ffma2_rn(e, m1, cutv);
                    t.x = __float_as_uint(e.x) > cut_bits ? 0.f : t.x;
                    t.y = __float_as_uint(e.y) > cut_bits ? 0.f : t.y;
                    acc = __ffma2_rn(__fmul2_rn(t, t), t, acc);
                }
            });
        if (active) write_density(f, P, self, acc.x + acc.y, true);
    }
}

// -------------------------------------------------------------- force TRA --
// The neighbours the density pass found, in the same order (rows in sequence,
// set bits in increasing candidate index). Each lane stages its 9 (row start,
// mask) pairs in shared memory and walks all its neighbours in one loop, so
// lanes stay converged across rows. Without masks (or with a row longer than
// 32 candidates) the lane scans its candidates as the reference does.
template <bool kArt, int W>
__global__ void __launch_bounds__(W * 32, 4 * kWarpsPerBlock / W)
k_force_tra(Frame f, DevParams P, bool fresh) {
    __shared__ uint32_t row_mask[9][W * 32];
    __shared__ int row_start[9][W * 32];
    const int lane = threadIdx.x & 31;
    const int middle = f.ctr->middle;
    const int units = (middle + 31) >> 5;
    const bool ident = !f.ctr->any_sms;   // all TRA: compact is the identity
    if (units == 0) return;        // no TRA work: skip the queue atomics
    for (;;) {
        const int u = next_unit(&f.ctr->work_force);
        if (u >= units) break;
        const int idx = (u << 5) + lane;
        if (idx >= middle) continue;
        const int self = ident ? idx : f.compact[idx];
        const float4 p = f.pos[self];
        const float4 pev = f.ev[self];
        const SceneGeom G = geom_of_particle(f.scenes, self);
        const MicroPos mp = micro_of(p, P, G);
        ForceAcc a = {0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f};
        const int found = fresh ? f.nbr_flag[idx] : -1;
        if (found >= 0) {
            // all nine masks, then every row's offsets and slab word, loaded
            // without conditions (a row without neighbours reads the
            // particle's own cell) so that the loads are in flight together
            const uint32_t *masks = f.nbr_mask + size_t(u) * 9 * 32 + lane;
            uint32_t mk[9];
#pragma unroll
            for (int r = 0; r < 9; ++r) mk[r] = masks[r * 32];
            const int own = G.cbase + mp.cx + G.gx * (mp.cy + G.gy * mp.cz);
            const int left = mp.cx > 0 ? 1 : 0;
#pragma unroll
            for (int r = 0; r < 9; ++r) {
                const int m = mk[r] ? own + G.gx * ((r % 3) - 1 + G.gy * ((r / 3) - 1)) : own;
                const int s0 = f.cell_start[m - left];
                const int s1 = f.cell_start[m];
                const uint32_t xs = f.cell_xslab[m - left];
                int start = s0;
                if (left && mp.lmx > 0 && xs != kXslabUnknown)
                    start = s0 + min(int((xs >> (10 * (mp.lmx - 1))) & 1023u), s1 - s0);
                row_mask[r][threadIdx.x] = mk[r];
                row_start[r][threadIdx.x] = start;
            }
            int r = 0;
            uint32_t mask = row_mask[0][threadIdx.x];
            int base = row_start[0][threadIdx.x];
            // two neighbours per iteration: both loads are in flight before
            // the first pair is evaluated (the order of the sums is unchanged)
            int k = 0;
            for (; k + 1 < found; k += 2) {
                while (!mask) {
                    ++r;
                    mask = row_mask[r][threadIdx.x];
                    base = row_start[r][threadIdx.x];
                }
                const int j0 = base + __ffs(mask) - 1;
                mask &= mask - 1u;
                while (!mask) {
                    ++r;
                    mask = row_mask[r][threadIdx.x];
                    base = row_start[r][threadIdx.x];
                }
                const int j1 = base + __ffs(mask) - 1;
                mask &= mask - 1u;
                const float4 q0 = f.pos[j0], e0 = f.ev[j0];
                const float4 q1 = f.pos[j1], e1 = f.ev[j1];
                force_pair<false, kArt>(p, pev, q0, e0, P, a);
                force_pair<false, kArt>(p, pev, q1, e1, P, a);
            }
            if (k < found) {
                while (!mask) {
                    ++r;
                    mask = row_mask[r][threadIdx.x];
                    base = row_start[r][threadIdx.x];
                }
                const int j = base + __ffs(mask) - 1;
                force_pair<false, kArt>(p, pev, f.pos[j], f.ev[j], P, a);
            }
        } else {
            for (int r = 0; r < 9; ++r) {
                const int ny = mp.cy + (r % 3) - 1;
                const int nz = mp.cz + (r / 3) - 1;
                if (ny < 0 || ny >= G.gy || nz < 0 || nz >= G.gz) continue;
                const int m = G.cbase + mp.cx + G.gx * (ny + G.gy * nz);
                int begin, end;
                row_range(f, G, m, mp.cx, mp.lmx, mp.lmx, begin, end);
                for (int j = begin; j < end; ++j) {
                    const float4 q = f.pos[j];
                    const float rx = p.x - q.x, ry = p.y - q.y, rz = p.z - q.z;
                    const float d2 = sq_dist(rx, ry, rz);
                    if (P.h2 < d2 || kFloatSmall > d2) continue;
                    force_pair<true, kArt>(p, pev, q, f.ev[j], P, a);
                }
            }
        }
        write_force(f, P, self, p, pev, G, a, false);
    }
}

// -------------------------------------------------------------- force SMS --
// One 32-particle task per warp (force_kernels.cu:830-1054). The candidates
// are the density pass's: x-merged rows, those at dz = -1 / +1 cut to the
// micro-z groups that can reach the task, one (cell, micro-x slab) segment at
// a time. They are staged 64 at a time in shared memory, each candidate pair
// as four float4s (one 16-byte broadcast load per pair and quantity group),
// and evaluated two at a time with packed FP32x2 arithmetic; a pair is
// skipped when no lane of the warp interacts with either candidate. Each
// term rounds as the reference's scalar expression; the two halves of every
// accumulator are summed at the end.
template <bool kArt, int W>
__global__ void __launch_bounds__(W * 32, 4 * kWarpsPerBlock / W)
k_force_sms(Frame f, DevParams P) {
    // candidate pair k (slots 2k, 2k+1) as four float4s: (x, x, y, y),
    // (z, z, 1/rho, 1/rho), (vx, vx, vy, vy), (vz, vz, p, p)
    __shared__ __align__(16) float4 sm[4][W][kSmsBatch / 2];
    const int lane = threadIdx.x & 31;
    const int warp = threadIdx.x >> 5;
    const int task_count = f.ctr->task_count;
    if (task_count == 0) return;   // no SMS work: skip the queue atomics
    float4 *sa = sm[0][warp], *sb4 = sm[1][warp], *sc = sm[2][warp], *sd = sm[3][warp];
    for (;;) {
        const int u = next_unit(&f.ctr->work_force_sms);
        if (u >= task_count) break;
        const gsph_block_task task = f.tasks[u];
        const int cb = task.cell_begin;
        const int cend = cb + task.cell_particle_count;
        const int self = cb + task_offset(task) + lane;
        const bool active = self < cend;
        if (cb + task_offset(task) >= cend) continue;
        const int safe = active ? self : cend - 1;
        const float4 p = f.pos[safe];
        const float4 pev = f.ev[safe];
        const SceneGeom G = geom_of_cell(f.scenes, task.cellid);
        const int cx = task.cell_pos[0], cy = task.cell_pos[1],
                  cz = task.cell_pos[2];
        const float2 npx = make_float2(-p.x, -p.x);
        const float2 npy = make_float2(-p.y, -p.y);
        const float2 npz = make_float2(-p.z, -p.z);
        const float2 nvx = make_float2(-pev.x, -pev.x);
        const float2 nvy = make_float2(-pev.y, -pev.y);
        const float2 nvz = make_float2(-pev.z, -pev.z);
        int zmin, zmax;
        task_z_range(f, self, active, zmin, zmax);
        const float2 pi2 = make_float2(pev.w, pev.w);
        const float2 h2v = make_float2(P.h2, P.h2);
        const float2 hv = make_float2(P.h, P.h);
        const float2 m1 = make_float2(-1.f, -1.f);
        const float2 m075 = make_float2(-0.75f, -0.75f);
        const float2 zero = make_float2(0.f, 0.f);
        // pressure sum gets -r*ps = d*ps with d = q - p; the colour
        // gradient is accumulated with the opposite sign and negated at the end
        float2 Px = zero, Py = zero, Pz = zero, Vx = zero, Vy = zero, Vz = zero;
        float2 Gx = zero, Gy = zero, Gz = zero, L = zero;
        for (int r = 0; r < 9; ++r) {
            const int ny = cy + (r % 3) - 1;
            const int nz = cz + (r / 3) - 1;
            if (ny < 0 || ny >= G.gy || nz < 0 || nz >= G.gz) continue;
            const int m = G.cbase + cx + G.gx * (ny + G.gy * nz);
            // rows at dz = -1 / +1 keep only the micro-z groups that can
            // reach the task (as the density pass's candidate stream)
            const int rdz = r / 3 - 1;
            const int zlo = rdz < 0 ? zmin : 0, zhi = rdz > 0 ? zmax : 3;
            const bool zcut = f.cell_grp && !(zlo == 0 && zhi == 3);
            int begin = 0, end = 0;
            if (!zcut) row_range(f, G, m, cx, task.xxi, task.xxx, begin, end);
            const int nseg = zcut ? 12 : 1;
            for (int sg = 0; sg < nseg; ++sg) {
                if (zcut) {
                    int sb, sl;
                    sms_segment(f, G, m, cx, task.xxi, task.xxx, zlo, zhi, sg, sb, sl);
                    begin = sb;
                    end = sb + sl;
                }
                for (int base = begin; base < end; base += kSmsBatch) {
                    const int cnt = min(kSmsBatch, end - base);
#pragma unroll
                    for (int hh = 0; hh < kSmsBatch; hh += 32) {
                        const int t = hh + lane;
                        float4 q = make_float4(kFar, kFar, kFar, 0.f);
                        float4 qv = make_float4(0.f, 0.f, 0.f, 0.f);
                        if (t < cnt) {
                            q = f.pos[base + t];
                            qv = f.ev[base + t];
                        }
                        const int o = (t >> 1) * 4 + (t & 1);
                        float *fa = reinterpret_cast<float *>(sa), *fb = reinterpret_cast<float *>(sb4);
                        float *fc = reinterpret_cast<float *>(sc), *fd = reinterpret_cast<float *>(sd);
                        fa[o] = q.x; fa[o + 2] = q.y; fb[o] = q.z; fb[o + 2] = q.w;
                        fc[o] = qv.x; fc[o + 2] = qv.y; fd[o] = qv.z; fd[o + 2] = qv.w;
                    }
                    __syncwarp();
                    const int pairs = (cnt + 1) >> 1;
#pragma unroll 8
                    for (int k = 0; k < pairs; ++k) {
                        const float4 qa = sa[k], qb = sb4[k];
                        const float2 dx = __fadd2_rn(make_float2(qa.x, qa.y), npx);
                        const float2 dy = __fadd2_rn(make_float2(qa.z, qa.w), npy);
                        const float2 dz = __fadd2_rn(make_float2(qb.x, qb.y), npz);
                        float2 d2 = __fmul2_rn(dx, dx);
                        d2 = __ffma2_rn(dy, dy, d2);
                        d2 = __ffma2_rn(dz, dz, d2);
                        const float2 t = __ffma2_rn(d2, m1, h2v);   // h^2 - r^2
                        const bool okx = t.x >= 0.f && d2.x >= kFloatSmall;
                        const bool oky = t.y >= 0.f && d2.y >= kFloatSmall;
                        if (!__any_sync(kFull, active && (okx || oky))) continue;
                        const float2 d2s = make_float2(okx ? d2.x : 1.f, oky ? d2.y : 1.f);
                        const float2 inv = make_float2(rsqrtf(d2s.x), rsqrtf(d2s.y));
                        const float2 d = __fmul2_rn(d2s, inv);
                        const float2 kk = __ffma2_rn(d, m1, hv);       // h - r
                        // 1/rho of the candidate, zero where it does not interact:
                        // the pressure, viscosity and colour terms vanish with it
                        const float2 V = make_float2(okx ? qb.z : 0.f, oky ? qb.w : 0.f);
                        const float4 qc = sc[k], qd = sd[k];
                        const float2 wk = __fmul2_rn(V, kk);
                        const float2 psum = __fadd2_rn(pi2, make_float2(qd.z, qd.w));
                        const float2 ps = __fmul2_rn(__fmul2_rn(__fmul2_rn(wk, psum), kk), inv);
                        Px = __ffma2_rn(dx, ps, Px);
                        Py = __ffma2_rn(dy, ps, Py);
                        Pz = __ffma2_rn(dz, ps, Pz);
                        const float2 dvx = __fadd2_rn(make_float2(qc.x, qc.y), nvx);
                        const float2 dvy = __fadd2_rn(make_float2(qc.z, qc.w), nvy);
                        const float2 dvz = __fadd2_rn(make_float2(qd.x, qd.y), nvz);
                        if (kArt) {
                            // v_ij . r_ij = (v_j - v_i) . (x_j - x_i); the sum is
                            // kept against d = x_j - x_i and negated at the end
                            float2 vr = __fmul2_rn(dvx, dx);
                            vr = __ffma2_rn(dvy, dy, vr);
                            vr = __ffma2_rn(dvz, dz, vr);
                            const float2 w = make_float2(
                                okx ? artificial_pair(vr.x, d2s.x, kk.x, inv.x, p.w, qb.z, P)
                                    : 0.f,
                                oky ? artificial_pair(vr.y, d2s.y, kk.y, inv.y, p.w, qb.w, P)
                                    : 0.f);
                            Vx = __ffma2_rn(dx, w, Vx);
                            Vy = __ffma2_rn(dy, w, Vy);
                            Vz = __ffma2_rn(dz, w, Vz);
                        } else {
                            Vx = __ffma2_rn(dvx, wk, Vx);
                            Vy = __ffma2_rn(dvy, wk, Vy);
                            Vz = __ffma2_rn(dvz, wk, Vz);
                        }
                        const float2 wh = __fmul2_rn(V, t);
                        const float2 gw = __fmul2_rn(wh, t);
                        Gx = __ffma2_rn(dx, gw, Gx);
                        Gy = __ffma2_rn(dy, gw, Gy);
                        Gz = __ffma2_rn(dz, gw, Gz);
                        L = __ffma2_rn(wh, __ffma2_rn(t, m075, d2), L);
                    }
                    __syncwarp();
                }
            }
        }
        if (active) {
            ForceAcc a;
            a.px = Px.x + Px.y;
            a.py = Py.x + Py.y;
            a.pz = Pz.x + Pz.y;
            a.vx = kArt ? -(Vx.x + Vx.y) : Vx.x + Vx.y;
            a.vy = kArt ? -(Vy.x + Vy.y) : Vy.x + Vy.y;
            a.vz = kArt ? -(Vz.x + Vz.y) : Vz.x + Vz.y;
            a.gx = -(Gx.x + Gx.y);
            a.gy = -(Gy.x + Gy.y);
            a.gz = -(Gz.x + Gz.y);
            a.lap = L.x + L.y;
            write_force(f, P, self, p, pev, G, a, true);
        }
    }
}

// -------------------------------------------------------------- integrate --
__global__ void __launch_bounds__(256)
k_integrate(Frame f, DevParams P) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= f.n) return;
    const float4 tp = f.pos[i];
    const float4 ev = f.ev[i];
    const SceneGeom G = geom_of_particle(f.scenes, i);
    const float4 v4 = f.vel[i];
    const float4 a4 = f.acc[i];
    float4 po, vo, eo;
    integrate_one(tp, v4, ev, a4.x, a4.y, a4.z, P, G, po, vo, eo);
    f.pos[i] = po;
    f.vel[i] = vo;
    f.ev[i] = eo;
}

// ---------------------------------------------------------------- render --
// COLORA (kernel_common.cuh:58): a * 255 << 24 | b << 16 | g << 8 | r, each
// channel clamped to [0, 255] (the device conversion of the reference
// saturates the same way).
__device__ __forceinline__ uint32_t colora(float r, float g, float b, float a) {
    auto ch = [](float v) { return uint32_t(fminf(fmaxf(v * 255.0f, 0.f), 255.f)); };
    return (ch(a) << 24) | (ch(b) << 16) | (ch(g) << 8) | ch(r);
}

__device__ __forceinline__ float density_color(const Frame &f, int i) {
    return (5000.f - 1.0f / f.pos[i].w) / 6000.f;
}

__global__ void __launch_bounds__(256)
k_render_tra(Frame f, uint32_t *color) {
    const int middle = f.ctr->middle;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < middle;
         k += gridDim.x * blockDim.x) {
        const int i = f.ctr->any_sms ? f.compact[k] : k;
        const float c = density_color(f, i);
        color[i] = colora(c, 0.f, c, 1.f);
    }
}

__global__ void __launch_bounds__(256)
k_render_sms(Frame f, uint32_t *color) {
    const int tasks = f.ctr->task_count;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < tasks * kSmsTaskParticles;
         k += gridDim.x * blockDim.x) {
        const gsph_block_task t = f.tasks[k / kSmsTaskParticles];
        const int i = t.cell_begin + task_offset(t) + k % kSmsTaskParticles;
        if (i >= t.cell_begin + t.cell_particle_count) continue;
        const float c = density_color(f, i);
        color[i] = t.is_same ? colora(0.f, c, c, 1.f) : colora(c, c, 0.f, 1.f);
    }
}

__global__ void __launch_bounds__(256)
k_final_position(Frame f, float3 ratio, float3 origin, float4 *out) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < f.n;
         i += gridDim.x * blockDim.x) {
        const float4 p = f.pos[i];
        out[i] = make_float4(p.x * ratio.x + origin.x, p.y * ratio.y + origin.y,
                             p.z * ratio.z + origin.z, 1.f);
    }
}

// ------------------------------------------------------- FP64 reductions --
// Deterministic two-level tree: fixed per-block partials, then one block.
constexpr int kRedThreads = 256;
constexpr int kRedBlocks = 512;

template <int K>
__device__ __forceinline__ void block_sum(double (&v)[K], double *out) {
    __shared__ double sh[K][kRedThreads / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_down_sync(kFull, x, o);
        if (lane == 0) sh[k][warp] = x;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int w = 0; w < kRedThreads / 32; ++w) t += sh[threadIdx.x][w];
        out[threadIdx.x] = t;
    }
}

__global__ void __launch_bounds__(kRedThreads)
k_checksum_partial(const float4 *__restrict__ pos, int n,
                   double *__restrict__ part) {
    double v[5] = {0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n;
         i += gridDim.x * kRedThreads) {
        const float4 p = pos[i];
        v[0] += p.x;
        v[1] += p.y;
        v[2] += p.z;
        v[3] += p.w;
        v[4] += double((unsigned(i) & 1023u) + 1u) *
                (double(p.x) + 3.0 * double(p.y) + 7.0 * double(p.z));
    }
    block_sum<5>(v, part + 5 * blockIdx.x);
}

__global__ void __launch_bounds__(kRedThreads)
k_reduce_partial(const float4 *__restrict__ pos, const float4 *__restrict__ vel,
                 int n, double mass, double *__restrict__ part) {
    double v[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (int i = blockIdx.x * kRedThreads + threadIdx.x; i < n;
         i += gridDim.x * kRedThreads) {
        const float4 p = pos[i];
        const float4 u = vel[i];
        v[0] += mass;
        v[1] += mass * u.x;
        v[2] += mass * u.y;
        v[3] += mass * u.z;
        v[4] += 0.5 * mass * (double(u.x) * u.x + double(u.y) * u.y +
                              double(u.z) * u.z);
        v[5] += p.x;
        v[6] += p.y;
        v[7] += p.z;
    }
    block_sum<8>(v, part + 8 * blockIdx.x);
}

template <int K>
__global__ void __launch_bounds__(kRedThreads)
k_final_sum(const double *__restrict__ part, int nparts, double *__restrict__ out) {
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
    for (int b = threadIdx.x; b < nparts; b += kRedThreads)
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] += part[K * b + k];
    block_sum<K>(v, out);
}

// Shared-memory carveout of one kernel: what `ctas` resident CTAs of it need
// (static shared memory plus the 1 KB the SM reserves per CTA), so that the
// rest of the SM's unified L1/shared storage stays L1 for candidate reads.
template <class Kernel>
cudaError_t set_carveout(Kernel kernel, int ctas, int smem_per_sm, int threads) {
    cudaFuncAttributes a{};
    cudaError_t e = cudaFuncGetAttributes(&a, kernel);
    if (e != cudaSuccess) return e;
    int pct = 0;
    if (a.sharedSizeBytes > 0 && smem_per_sm > 0) {
        const long long need = (long long)(a.sharedSizeBytes + 1024) * ctas;
        pct = int(std::min<long long>(100, (need * 100 + smem_per_sm - 1) / smem_per_sm));
    }
    e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, pct);
    if (e != cudaSuccess) return e;
    // the hint is rounded to a supported split; keep the default if the
    // rounded one would hold fewer CTAs
    int fit = 0;
    e = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&fit, kernel, threads, 0);
    if (e != cudaSuccess) return e;
    if (fit < ctas)
        e = cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout,
                                 int(cudaSharedmemCarveoutDefault));
    return e;
}

template <int W>
cudaError_t configure_shape(int smem) {
    const int k = kWarpsPerBlock / W;   // CTAs per SM scale with the block size
    cudaError_t e;
    if ((e = set_carveout(k_density_tra<W, false>, kMaxShape.density_tra * k, smem, W * 32)))
        return e;
    if ((e = set_carveout(k_density_tra<W, true>, kMaxShape.density_tra * k, smem, W * 32)))
        return e;
    if ((e = set_carveout(k_density_sms<W>, kMaxShape.density_sms * k, smem, W * 32)))
        return e;
    if ((e = set_carveout(k_force_tra<false, W>, kMaxShape.force_tra * k, smem, W * 32)))
        return e;
    if ((e = set_carveout(k_force_tra<true, W>, kMaxShape.force_tra * k, smem, W * 32)))
        return e;
    if ((e = set_carveout(k_force_sms<false, W>, kMaxShape.force_sms * k, smem, W * 32)))
        return e;
    return set_carveout(k_force_sms<true, W>, kMaxShape.force_sms * k, smem, W * 32);
}

template <int W>
void launch_density_w(const Frame &f, const DevParams &P, int num_sms,
                      const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms,
                      bool row_prefetch) {
    k_density_sms<W><<<num_sms * shape.density_sms, W * 32, 0, s_sms>>>(f, P);
    if (row_prefetch)
        k_density_tra<W, true><<<num_sms * shape.density_tra, W * 32, 0, s>>>(f, P);
    else
        k_density_tra<W, false><<<num_sms * shape.density_tra, W * 32, 0, s>>>(f, P);
}

template <bool kArt, int W>
void launch_force_w(const Frame &f, const DevParams &P, int num_sms, bool fresh,
                    const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms) {
    k_force_sms<kArt, W><<<num_sms * shape.force_sms, W * 32, 0, s_sms>>>(f, P);
    k_force_tra<kArt, W><<<num_sms * shape.force_tra, W * 32, 0, s>>>(f, P, fresh);
}

}  // namespace

cudaError_t configure_physics_kernels(int device) {
    int smem = 0;
    cudaError_t e = cudaDeviceGetAttribute(
        &smem, cudaDevAttrMaxSharedMemoryPerMultiprocessor, device);
    if (e != cudaSuccess) return e;
    if ((e = configure_shape<kWarpsPerBlock>(smem))) return e;
    return configure_shape<kWarpsPerBlock / 2>(smem);
}

void launch_density(const Frame &f, const DevParams &P, int num_sms,
                    const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms) {
    if (f.n <= 0) return;
    // cell offsets and slab words: 8 bytes per cell
    const bool row_prefetch = size_t(P.numc) * 8 > kRowPrefetchCellBytes;
    if (shape.warps == kWarpsPerBlock / 2)
        launch_density_w<kWarpsPerBlock / 2>(f, P, num_sms, shape, s, s_sms, row_prefetch);
    else
        launch_density_w<kWarpsPerBlock>(f, P, num_sms, shape, s, s_sms, row_prefetch);
}

void launch_force(const Frame &f, const DevParams &P, int num_sms, bool fresh,
                  const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms) {
    if (f.n <= 0) return;
    const bool half = shape.warps == kWarpsPerBlock / 2;
    if (P.visc_artificial) {
        if (half)
            launch_force_w<true, kWarpsPerBlock / 2>(f, P, num_sms, fresh, shape, s, s_sms);
        else
            launch_force_w<true, kWarpsPerBlock>(f, P, num_sms, fresh, shape, s, s_sms);
    } else {
        if (half)
            launch_force_w<false, kWarpsPerBlock / 2>(f, P, num_sms, fresh, shape, s, s_sms);
        else
            launch_force_w<false, kWarpsPerBlock>(f, P, num_sms, fresh, shape, s, s_sms);
    }
}

void launch_integrate(const Frame &f, const DevParams &P, cudaStream_t s) {
    if (f.n <= 0) return;
    k_integrate<<<(f.n + 255) / 256, 256, 0, s>>>(f, P);
}

// out5 must hold 5 + 5*kRedBlocks doubles (partials follow the result).
void launch_checksum(const float4 *pos, int n, double *out5, cudaStream_t s) {
    k_checksum_partial<<<kRedBlocks, kRedThreads, 0, s>>>(pos, n, out5 + 8);
    k_final_sum<5><<<1, kRedThreads, 0, s>>>(out5 + 8, kRedBlocks, out5);
}

// out8 must hold 8 + 8*kRedBlocks doubles.
void launch_render(const Frame &f, float3 ratio, float3 origin, uint32_t *color,
                   float4 *final_pos, cudaStream_t s) {
    if (f.n <= 0) return;
    const int blocks = std::min((f.n + 255) / 256, 4096);
    if (color) {
        k_render_tra<<<blocks, 256, 0, s>>>(f, color);
        k_render_sms<<<blocks, 256, 0, s>>>(f, color);
    }
    if (final_pos) k_final_position<<<blocks, 256, 0, s>>>(f, ratio, origin, final_pos);
}

void launch_reductions(const float4 *pos, const float4 *vel, int n, float mass,
                       double *out8, cudaStream_t s) {
    k_reduce_partial<<<kRedBlocks, kRedThreads, 0, s>>>(pos, vel, n, mass,
                                                        out8 + 8);
    k_final_sum<8><<<1, kRedThreads, 0, s>>>(out8 + 8, kRedBlocks, out8);
}

}  // namespace gsph
