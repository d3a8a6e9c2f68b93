// gsph_internal.h — types shared by the host runtime and the device kernels.
//
// Layout of one scene in HBM (structure of arrays, 16-byte particle records):
//   pos[2]  float4[N]  x,y,z, w = 1/rho (ping-pong: the grid sort writes the
//                      sorted copy into the other buffer)
//   vel[2]  float4[N]  velocity (w unused; float4 keeps every access 16 B)
//   ev[2]   float4[N]  evaluated velocity, w = pressure
//   acc     float4[N]  pressure+viscosity+surface force ("acceleration")
//   key     uint32[N]  micro-cell key of the sorted particles
//   cell_start int32[numc+1], cell_xslab uint32[numc]
#ifndef GSPH_INTERNAL_H_
#define GSPH_INTERNAL_H_

#include <cstdint>
#include <vector>
#include <cuda_runtime.h>

#include "../../include/gsph.h"

namespace gsph {

// Cells with more particles than this are ordered by the block-level sort.
constexpr int kSmallCellMax = 32;
// Largest cell the block-level sort keeps in shared memory.
constexpr int kBigCellSmem = 4096;
// SMS task width (reference sph_utils.cuh:35).
constexpr int kSmsTaskParticles = 32;
// Sentinel for cell_xslab: slab boundaries unknown, search the whole cell.
constexpr uint32_t kXslabUnknown = 0xFFFFFFFFu;
constexpr uint16_t kGroupsUnknown = 0xFFFFu;
// Largest particle offset of an SMS task inside its cell: the descriptor's
// 16-bit p_offset (the reference's field, which wraps past 65,535 particles)
// plus bits 16-23 in the descriptor's padding byte.
constexpr int kTaskOffsetLimit = 1 << 24;
// Neighbour masks of TRA particles: the density pass records, for each of the
// 9 neighbour rows of a TRA particle, a 32-bit mask of which candidates of the
// row interact; the force pass walks the set bits instead of re-testing every
// candidate. A particle with a row longer than 32 candidates is flagged and
// the force pass scans its candidates instead.
constexpr int kMaskRowMax = 32;
// Scan tile (items per CTA) for the reduce-then-scan kernels.
constexpr int kScanThreads = 256;
constexpr int kScanItems = 16;
constexpr int kScanTile = kScanThreads * kScanItems;
// Tiles of the per-occupied-cell {tasks, SMS, TRA} scan of the split.
constexpr int kValItems = 4;
constexpr int kValTile = kScanThreads * kValItems;

// Error bits raised by kernels into Counters::err.
enum : uint32_t {
    kErrOutOfDomain = 1u,     // a particle's micro cell was outside the grid
    kErrTaskCapacity = 2u,    // more SMS tasks than the task buffer holds
};

// Physical parameters as the kernels see them (passed by value: one constant
// bank per launch, so several handles can coexist in one process). Every
// scene of a batch shares them; per-scene geometry lives in SceneGeom.
struct DevParams {
    float h, h2, rat;            // rat = 4 * inv_cell_size (micro cells)
    int numc;                    // cells of all scenes
    float density_scale, self_density, rest_density, inv_rest_density;
    float gas_constant;
    float half_spiky, visco_coef, grad_color_scale, lplc_color_scale;
    float surface_normal, surface_coe, mass;
    float time_step, wall_damping, wall_kernel;   // wall_kernel = h + 0.01
    float gx_acc, gy_acc, gz_acc;                 // gravity
    float bmin;                                   // lower wall (= h) on every axis
    int sparse_total, sparse_self, mid_total;     // split thresholds (gsph_tuning)
    // Artificial viscosity (GSPH_VISCOSITY_ARTIFICIAL): visc_artificial set,
    // art_coef = alpha * c0, art_eps = 0.01 h^2, spiky = the spiky gradient
    // constant. Unused by the reference's Laplacian model.
    int visc_artificial;
    float art_coef, art_eps, spiky;
};

// Geometry of one scene of a batch. Particles of scene s occupy
// [pbase, pbase + n) and its cells [cbase, cbase + gx*gy*gz) of the
// concatenated arrays; positions are in the scene's own coordinates. A single
// scene is a batch of one.
struct SceneGeom {
    int gx, gy, gz;
    int cbase;
    float bmax_x, bmax_y, bmax_z;
    int pad;
};

// Scenes of a batch. With one scene (count == 1) the geometry travels in the
// kernel parameter itself (`single`) and the device arrays are not read.
struct SceneTable {
    const SceneGeom *geom;   // [count]
    const int *pbase;        // [count + 1] particle offsets
    const int *cbase;        // [count + 1] cell offsets
    int count;
    SceneGeom single;
};

// Geometry of the scene holding sorted particle i / global cell c.
__device__ __forceinline__ int scene_of(const int *base, int count, int i);
__device__ __forceinline__ SceneGeom geom_of_particle(const SceneTable &T, int i) {
    return T.count == 1 ? T.single : T.geom[scene_of(T.pbase, T.count, i)];
}
__device__ __forceinline__ SceneGeom geom_of_cell(const SceneTable &T, int c) {
    return T.count == 1 ? T.single : T.geom[scene_of(T.cbase, T.count, c)];
}

// Scene of sorted particle i / of global cell c (the last scene whose range
// starts at or before it; empty scenes are skipped by construction).
__device__ __forceinline__ int scene_of(const int *base, int count, int i) {
    if (count == 1) return 0;
    int lo = 0, hi = count - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (base[mid] <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    return lo;
}

// Device-resident counters of one frame (one 128-byte line).
struct Counters {
    int32_t num_occ;        // occupied cells
    int32_t num_big;        // cells sorted by the block-level path
    int32_t task_count;     // SMS tasks (T)
    int32_t middle;         // TRA particles
    int32_t n_sms;          // SMS particles
    int32_t work_density;   // work counters of the persistent kernels:
    int32_t work_force;     //   TRA units of density / force,
    uint32_t err;           // error bits
    int32_t err_index;      // first offending particle (best effort)
    int32_t work_density_sms;   //   SMS tasks of density / force
    int32_t work_force_sms;
    // Set when some cell takes the SMS path this frame; when clear, every
    // particle is TRA, the compact index is the identity and the TRA/SMS
    // compaction is skipped.
    int32_t any_sms;
    // CTAs of the cell-count reduction / of the performance model that have
    // written their tile sums; the last one scans the tiles (and resets it).
    int32_t scan_done;
    int32_t model_done;
    int32_t pad[18];
};

// Per-frame device pointers of one batch of scenes.
struct Frame {
    int n;
    SceneTable scenes;
    const float4 *pos_in, *vel_in, *ev_in;     // unsorted (previous order)
    float4 *pos, *vel, *ev, *acc;              // sorted (current order)
    // When set, the force pass also integrates each particle (the reference's
    // advance) and writes the new state here instead of leaving it to a
    // separate integration launch; the arrays must not alias pos/vel/ev.
    float4 *pos_next, *vel_next, *ev_next;
    // With pos_next set and hash_next true, the TRA force pass also computes
    // the next frame's micro key and cell slot of its particles (key_in, slot,
    // cell_count); launch_hash_sms does the same for the SMS particles after
    // the SMS force pass.
    bool hash_next;
    uint32_t *key_in, *slot;                   // per source particle
    unsigned long long *pairs;                 // (key << 32 | src), by cell
    uint32_t *key;                             // sorted keys
    int32_t *perm;                             // source of each sorted slot
    int32_t *cell_count, *cell_start;
    uint32_t *cell_xslab;
    // Per cell, 16 offsets (relative to the cell start) of the first particle
    // of each (micro-x, micro-z) group, group g = mx * 4 + mz, in sort order;
    // entry 0 is kGroupsUnknown for cells above 65,535 particles. Null when the
    // caller does not keep it.
    uint16_t *cell_grp;
    int32_t *occ_list, *big_list;
    int4 *cell_val;                            // per occupied cell {req,sms,tra}
    int4 *cell_prefix;                         // exclusive prefix of cell_val
    gsph_block_task *tasks;
    int32_t task_capacity;
    int32_t *compact;
    // TRA neighbour masks, interleaved by 32-particle chunk of the compact
    // index: row r of compact index i at nbr_mask[((i >> 5) * 9 + r) * 32 +
    // (i & 31)]; nbr_flag[i] = number of neighbours, or -1 where the masks
    // are incomplete.
    uint32_t *nbr_mask;
    int32_t *nbr_flag;
    unsigned long long *scan_tiles;            // tile sums, cell scan
    int4 *scan_tiles4;                         // tile sums, task scan
    Counters *ctr;
};

// ---- shared device helpers (grid sort and the force pass's look-ahead hash) ----
// Particle offset of an SMS task inside its cell (see kTaskOffsetLimit).
inline __host__ __device__ int task_offset(const gsph_block_task &t) {
    return int(t.p_offset) | (int(t.pad_) << 16);
}
inline __host__ __device__ void set_task_offset(gsph_block_task &t, int off) {
    t.p_offset = uint16_t(off & 0xFFFF);
    t.pad_ = uint8_t(off >> 16);
}

#ifdef __CUDACC__
__device__ __forceinline__ unsigned lanemask_lt() {
    unsigned m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Micro key of one position (sph_utils.cuh:44-99), in the global cell space
// of a batch: the scene's cell base is added to the reference's cell index.
// Positions outside the scene's grid raise kErrOutOfDomain and are clamped to
// the nearest cell so that no index ever leaves the tables.
__device__ __forceinline__ uint32_t micro_key(float4 p, const DevParams &P,
                                              const SceneGeom &G,
                                              Counters *ctr, int i) {
    const float fx = floorf(p.x * P.rat);
    const float fy = floorf(p.y * P.rat);
    const float fz = floorf(p.z * P.rat);
    const float lx = float(G.gx << 2), ly = float(G.gy << 2),
                lz = float(G.gz << 2);
    int mx, my, mz;
    if (fx >= 0.f && fx < lx && fy >= 0.f && fy < ly && fz >= 0.f && fz < lz) {
        mx = int(fx);
        my = int(fy);
        mz = int(fz);
    } else {
        mx = (fx >= 0.f) ? min(int(fminf(fx, lx - 1.f)), (G.gx << 2) - 1) : 0;
        my = (fy >= 0.f) ? min(int(fminf(fy, ly - 1.f)), (G.gy << 2) - 1) : 0;
        mz = (fz >= 0.f) ? min(int(fminf(fz, lz - 1.f)), (G.gz << 2) - 1) : 0;
        if (atomicOr(&ctr->err, kErrOutOfDomain) == 0u) ctr->err_index = i;
    }
    const uint32_t c = uint32_t(G.cbase) + uint32_t(mx >> 2) +
                       uint32_t(G.gx) * (uint32_t(my >> 2) + uint32_t(G.gy) * uint32_t(mz >> 2));
    const uint32_t sub = uint32_t(my & 3) | (uint32_t(mz & 3) << 2) | (uint32_t(mx & 3) << 4);
    return (c << 6) | sub;
}

// Slot of a particle among its cell's particles: one atomic per cell per warp
// (lanes in `active` with the same cell share it, match.any).
__device__ __forceinline__ uint32_t cell_slot(int32_t *cell_count, uint32_t cell,
                                              unsigned active) {
    const unsigned peers = __match_any_sync(active, cell);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    int base = 0;
    if (lane == leader) base = atomicAdd(&cell_count[cell], __popc(peers));
    base = __shfl_sync(peers, base, leader);
    return uint32_t(base + __popc(peers & lanemask_lt()));
}
#endif  // __CUDACC__

// ---- launchers (grid.cu) ----
void launch_hash_count(const Frame &f, const DevParams &P, cudaStream_t s);
// Hash of the previous split's SMS particles only (compact[middle, n)).
// Keys and cell slots ahead for the split's SMS particles (compact[middle,
// n)) from their integrated positions `pos`.
void launch_hash_sms(const Frame &f, const float4 *pos, const DevParams &P,
                     cudaStream_t s);
void launch_cell_scan(const Frame &f, const DevParams &P, cudaStream_t s);
void launch_scatter_pairs(const Frame &f, cudaStream_t s);
void launch_cell_sort(const Frame &f, int num_sms, cudaStream_t s);
// ---- launchers (split.cu) ----
// Performance model, TRA/SMS partition and SMS tasks; launch_judge then
// pairs the tasks (judgeTask), which only the SMS passes read.
void launch_split(const Frame &f, const DevParams &P, int max_occ, int num_sms,
                  cudaStream_t s);
void launch_judge(const Frame &f, int max_occ, int num_sms, cudaStream_t s);
// ---- launchers (physics.cu) ----
// Launch shapes of the density and force passes: CTAs per SM of each kernel.
struct LaunchShape {
    int density_tra, density_sms, force_tra, force_sms;
    int warps;   // warps per block: 8, or 4 (then up to twice the CTAs per SM)
};
constexpr LaunchShape kMaxShape = {6, 4, 4, 4, 8};   // the kernels' launch bounds

// Shared-memory carveouts of the density and force kernels (once per
// device, before their first launch).
cudaError_t configure_physics_kernels(int device);
// The TRA pass on s, the SMS pass on s_sms (the two touch disjoint particles
// and work counters; the caller joins them before the results are read).
void launch_density(const Frame &f, const DevParams &P, int num_sms,
                    const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms);
// fresh: the density pass ran on the current state, so the TRA neighbour
// masks are valid.
void launch_force(const Frame &f, const DevParams &P, int num_sms, bool fresh,
                  const LaunchShape &shape, cudaStream_t s, cudaStream_t s_sms);
void launch_integrate(const Frame &f, const DevParams &P, cudaStream_t s);
// Render-side buffers (headless): packed RGBA colour per particle from its
// density and its path (TRA, paired SMS, single SMS), and render-space
// positions.
void launch_render(const Frame &f, float3 ratio, float3 origin, uint32_t *color,
                   float4 *final_pos, cudaStream_t s);
void launch_reductions(const float4 *pos, const float4 *vel, int n,
                       float mass, double *out8, cudaStream_t s);
void launch_checksum(const float4 *pos, int n, double *out5, cudaStream_t s);

// Host-side helpers (scene.cpp).
DevParams make_dev_params(const gsph_params &p);
// Checks a scene's grid before any kernel sees it: every dimension in
// [1, 65535] and the cell count, computed in 64 bits, below kMaxCells (32-bit
// micro keys hold the cell index in their upper 26 bits). On success stores
// the cell count in *numc; otherwise sets the error string (prefixed by
// `who`) and returns GSPH_ERR_INVALID_ARG or GSPH_ERR_CAPACITY.
constexpr long long kMaxCells = 1LL << 26;
gsph_status check_grid(const gsph_params &p, const char *who, long long *numc);
SceneGeom make_scene_geom(const gsph_params &p, int cbase);
void set_error(const char *fmt, ...);

// Snapshot file format (snapshot.cpp).
gsph_status snapshot_write(const char *path, const gsph_params *plist,
                           const uint32_t *counts, uint32_t n_scenes,
                           const float *pos4, const float *vel4, const float *ev4,
                           uint64_t frames);
gsph_status snapshot_header(const char *path, uint32_t *n_scenes,
                            uint64_t *n_particles, uint64_t *frames);
gsph_status snapshot_read(const char *path, std::vector<gsph_params> &plist,
                          std::vector<uint32_t> &counts, std::vector<float> &pos4,
                          std::vector<float> &vel4, std::vector<float> &ev4,
                          uint64_t &frames);

}  // namespace gsph

#endif  // GSPH_INTERNAL_H_
