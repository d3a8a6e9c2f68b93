/*
 * gsph.h — C ABI of the GB300-native weakly-compressible SPH step.
 *
 * This is the drop-in boundary for the reference's single-scene hot path
 * (KemengHuang/Fast-General-GPU-SPH-framework). Every entry point below names
 * the reference interface it replaces (path:line in that project):
 *
 *   reference                                   here
 *   -----------------------------------------   -------------------------------
 *   readSceneFromJsonFile  sph_hybrid_system.cpp:69-126      gsph_scene_load_json
 *   defaultInitializeSPHSysPara  sph_hybrid_system.cpp:127-202 gsph_params_init
 *   initializeScene lattice  sph_hybrid_system.cpp:432-473   gsph_lattice_count/fill
 *   HybridSystem ctor  sph_hybrid_system.cpp:209-240          gsph_create*
 *   HybridSystem::tick  sph_hybrid_system.cpp:253-339         gsph_step
 *   Arrangement::arrangeHybridFrame  sph_arrangement.cu:1493  gsph_arrange
 *   computeDensityHybrid  kernel_dispatch.cu:206-222          gsph_density
 *   computeForceHybrid  kernel_dispatch.cu:224-253            gsph_force
 *   advance  kernel_dispatch.cu:314-323                       gsph_advance
 *   HybridSystem::runBenchmark  sph_hybrid_system.cpp:341-430 gsph_benchmark
 *   computeBenchmarkStateChecksum  sph_hybrid_system.cpp:43-62 gsph_checksum
 *   getNumParticles / getPosition  sph_hybrid_system.h        gsph_get_info / gsph_copy_out
 *   Arrangement getters  sph_arrangement.h:41-59              gsph_copy_out fields
 *
 * Conventions: every function returns gsph_status (0 = success, negative =
 * error) and never exits the process; gsph_last_error() returns the message of
 * the calling thread's last failure. A handle owns its device memory and one
 * CUDA stream; all work is asynchronous on that stream until a call that
 * returns host data (copy_out, checksum, benchmark, sync). A handle may be used
 * from one thread at a time; different handles are independent (parameters
 * live in each handle, not in a process-global constant bank).
 * There is no CPU fallback: without a usable CUDA device, creation fails with
 * GSPH_ERR_NO_DEVICE.
 */
#ifndef GSPH_H_
#define GSPH_H_

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define GSPH_ABI_VERSION 1
#define GSPH_MAX_FLUID_BLOCKS 64

typedef int gsph_status;
enum {
    GSPH_OK = 0,
    GSPH_ERR_INVALID_ARG = -1,
    GSPH_ERR_IO = -2,
    GSPH_ERR_PARSE = -3,
    GSPH_ERR_CUDA = -4,
    GSPH_ERR_OUT_OF_MEMORY = -5,
    GSPH_ERR_CAPACITY = -6,
    GSPH_ERR_DOMAIN = -7,     /* a particle left the grid (device flag) */
    GSPH_ERR_NO_DEVICE = -8,
    GSPH_ERR_STATE = -9
};

typedef struct gsph_system *gsph_handle;

/* Scene file contents (reference Scene, sph_hybrid_system.h:37-44, and the
 * JSON keys read at sph_hybrid_system.cpp:83-117). Defaults as in the
 * reference: interval 0.5, mass 0.02, recomm_nump 65536, box 0. */
typedef struct {
    float world[3];                 /* "xx","yy","zz" */
    float mass;                     /* "mass" */
    float interval;                 /* "interval" (lattice step / h) */
    uint32_t recomm_nump;           /* "recomm_nump" */
    uint32_t n_blocks;              /* "fluid_block" entries */
    float block_begin[GSPH_MAX_FLUID_BLOCKS][3];
    float block_end[GSPH_MAX_FLUID_BLOCKS][3];
    /* Optional physics keys (not in the reference's files; absent = NaN,
     * meaning "use the reference's hard-coded value"). */
    float kernel;                   /* "kernel" (h) */
    float rest_density;             /* "rest_density" */
    float gas_constant;             /* "gas_constant" */
    float viscosity;                /* "viscosity" */
    float time_step;                /* "time_step" */
    float gravity_y;                /* "gravity_y" */
    float jitter;                   /* "jitter" (fraction of lattice step) */
    uint64_t seed;                  /* "seed" */
} gsph_scene;

/* Physical parameters, the live subset of the reference SystemParameter
 * (core/sph_parameter.h:18-90) with its derived coefficients. */
typedef struct {
    float world_size[3];
    float cell_size, inv_cell_size;
    int32_t grid_size[3];
    float kernel, kernel_2, mass;
    float gravity[3];
    float wall_damping, rest_density, gas_constant, viscosity, time_step;
    float surface_normal, surface_coe;
    float poly6_value, spiky_value, visco_value, grad_poly6, lplc_poly6;
    float self_density;
    float inv_rest_density, density_scale, half_spiky_value;
    float viscosity_visco_value, grad_color_scale, lplc_color_scale;
    float bound_interval, bound_min[3], bound_max[3];
} gsph_params;

/* BlockTask, the reference's 32-byte SMS task descriptor
 * (particle/particle_buffer.h:60-87), same field layout. p_offset is 16 bits
 * there and wraps in cells of more than 65,535 particles; here the padding
 * byte after is_same holds bits 16-23 of the task's particle offset (the
 * reference leaves that byte undefined), so such cells still run. */
typedef struct {
    int8_t is_same;
    uint8_t pad_;                /* bits 16-23 of the particle offset */
    uint16_t paired_bounds;
    int32_t cellid;
    uint16_t cell_pos[3];
    uint16_t p_offset;
    int8_t xxi, xxx, yyi, yyy, zzi, zzz;
    int32_t cell_begin;
    int32_t cell_particle_count;
} gsph_block_task;

typedef struct {
    uint32_t n_particles;
    uint32_t n_cells;            /* numc = gx*gy*gz */
    int32_t grid_size[3];
    int32_t tra_particles;       /* "middle" after the last arrange */
    int32_t sms_tasks;           /* SMS task count after the last arrange */
    int32_t occupied_cells;
    int32_t big_cells;           /* cells sorted by the block-level path */
    uint64_t frames;             /* ticks executed */
    uint64_t device_bytes;       /* device memory held by the handle */
    uint32_t n_scenes;           /* scenes in the handle (1 unless batched) */
    uint32_t reserved_;
} gsph_info;

/* Report of gsph_benchmark (the print block of runBenchmark,
 * sph_hybrid_system.cpp:397-429). */
typedef struct {
    int32_t measured_frames, warmup_frames;
    double total_wall_ms, avg_frame_ms, fps;
    double checksum[5];          /* x, y, z, 1/rho, weighted */
    int32_t tra_particles, sms_tasks;
    int32_t is_same_pairs, total_pairs, same_cell_pairs;
    int32_t full_is_same_pairs, partial_is_same_pairs;
    int32_t compact_is_same_pairs, widened_is_same_pairs;
    double arrange_ms, density_ms, force_ms, integrate_ms, total_kernel_ms;
    double particle_steps_per_s;
} gsph_bench_report;

/* Tunables of the TRA/SMS split and of the density/force launches. The
 * defaults (gsph_tuning_default) are the reference's performance model
 * (gpu_model.cu:172-180: a cell stays TRA while its 7-cell total is below
 * sparse_total and its own count below sparse_self; below mid_total it gets
 * (n+27)>>5 SMS tasks, else (n+31)>>5) and this library's launch shapes (CTAs
 * per SM of the TRA density, SMS density, TRA force and SMS force passes, at
 * most 6 / 4 / 4 / 4 with 8 warps per block, twice that with 4; the blocks of
 * 4 warps are the same kernels built for that shape). Other thresholds change which
 * cells take the SMS path: results stay within the parity tolerances but the
 * split is no longer the reference's. */
typedef struct {
    int32_t sparse_total, sparse_self, mid_total;
    int32_t ctas_density_tra, ctas_density_sms, ctas_force_tra, ctas_force_sms;
    int32_t warps_per_block;   /* 8 (0 reads as 8) or 4; with 4 the CTA counts
                                * may go up to twice the limits above */
} gsph_tuning;

/* Fields for gsph_copy_out / gsph_copy_in. All particle fields are in the
 * handle's current (sorted) order. */
typedef enum {
    GSPH_FIELD_POSITION = 0,      /* float4[N]  x,y,z, w = 1/rho             */
    GSPH_FIELD_VELOCITY = 1,      /* float4[N]  x,y,z, w unused             */
    GSPH_FIELD_EVAL_VELOCITY = 2, /* float4[N]  x,y,z, w = pressure          */
    GSPH_FIELD_ACCELERATION = 3,  /* float4[N]  force/acceleration, w unused */
    GSPH_FIELD_KEY = 4,           /* uint32[N]  sorted micro-cell key        */
    GSPH_FIELD_PERMUTATION = 5,   /* int32[N]   source index of each slot    */
    GSPH_FIELD_CELL_START = 6,    /* int32[numc+1] coarse cell offsets       */
    GSPH_FIELD_CELL_COUNT = 7,    /* int32[numc] coarse cell counts          */
    GSPH_FIELD_MICRO_START = 8,   /* int32[numc*64+1] dense micro offsets    */
    GSPH_FIELD_BLOCK_REQ = 9,     /* int32[numc] SMS tasks per cell          */
    GSPH_FIELD_COMPACT_INDEX = 10,/* int32[N] TRA particles then SMS ones    */
    GSPH_FIELD_TASKS = 11,        /* gsph_block_task[T + (T&1)]              */
    GSPH_FIELD_SPLIT = 12,        /* int32[2] {middle, task count}           */
    /* Headless render-side buffers, computed on demand from the current state
     * and the last arrange (the reference writes them every frame for its GL
     * view, density_kernels.cu:361-365,547-562, integration_kernels.cu:331-335;
     * its headless build leaves them out): */
    GSPH_FIELD_COLOR = 13,        /* uint32[N] RGBA8, COLORA of (5000-rho)/6000:
                                     TRA (c,0,c), paired SMS (0,c,c), single
                                     SMS (c,c,0)                              */
    GSPH_FIELD_FINAL_POSITION = 14,/* float4[N] position * ratio + origin, w=1 */
    /* Diagnostic of the last density pass on the current grid: */
    GSPH_FIELD_NEIGHBOR_COUNT = 15 /* int32[N] neighbours (0 < d^2 <= h^2) the
                                     density pass found for each TRA particle;
                                     -1 for SMS particles and where a
                                     neighbour row held more than 32
                                     candidates (no neighbour record)       */
} gsph_field;

const char *gsph_last_error(void);
int gsph_abi_version(void);

/* Scene + parameters + initial lattice (host-side; no device needed). */
gsph_status gsph_scene_default(gsph_scene *out);
gsph_status gsph_scene_load_json(const char *path, gsph_scene *out);
gsph_status gsph_scene_parse_json(const char *text, size_t len, gsph_scene *out);
gsph_status gsph_params_init(const gsph_scene *scene, gsph_params *out);
gsph_status gsph_lattice_count(const gsph_scene *scene, const gsph_params *p,
                               uint32_t *count);
/* Writes count float4 positions (w = 0), in the reference's x -> y -> z loop
 * order with FP32 accumulation; applies the scene's seeded jitter if any. */
gsph_status gsph_lattice_fill(const gsph_scene *scene, const gsph_params *p,
                              float *pos4, uint32_t capacity, uint32_t *count);

/* Lifetime. pos4/vel4 are host float4 arrays (vel4 may be NULL: zero). */
gsph_status gsph_create(const gsph_params *p, const float *pos4,
                        const float *vel4, uint32_t n, int device,
                        gsph_handle *out);
gsph_status gsph_create_from_json(const char *scene_path, int device,
                                  gsph_handle *out);
gsph_status gsph_destroy(gsph_handle h);

/* Snapshot / restart. gsph_snapshot_save writes every scene's parameters and
 * particle count and the particle state (position with w = 1/rho, velocity,
 * evaluated velocity with w = pressure) in the handle's current order, plus
 * the frame counter, to a versioned binary file with a payload checksum.
 * gsph_snapshot_load creates a handle (a batch when the file holds several
 * scenes) that continues the run bit for bit: stepping it K frames gives the
 * same state as stepping the saved handle K frames. gsph_snapshot_info reads
 * the header only. Corrupted or foreign files fail with GSPH_ERR_PARSE. The
 * reference has no restart path (its scenes always start from the JSON
 * lattice, sph_hybrid_system.cpp:432-473). */
gsph_status gsph_snapshot_save(gsph_handle h, const char *path);
gsph_status gsph_snapshot_load(const char *path, int device, gsph_handle *out);
gsph_status gsph_snapshot_info(const char *path, uint32_t *n_scenes,
                               uint64_t *n_particles, uint64_t *frames);

/* Batched step: num_scenes independent scenes stepped together, one launch
 * per stage for all of them (segmented grid sort over the concatenated cell
 * space, persistent density/force kernels over one work queue). params[k] is
 * scene k's parameter set; all scenes must share the physical parameters and
 * may differ in their box (world size, grid, walls). pos4/vel4 hold the
 * scenes' particles one after another (counts[k] each, float4; vel4 may be
 * NULL). Each scene evolves exactly as it would alone: same sort order, same
 * neighbour order, same arithmetic (bit-identical results). The reference
 * steps one scene per process and has no counterpart. */
gsph_status gsph_batch_create(const gsph_params *params, const uint32_t *counts,
                              uint32_t num_scenes, const float *pos4,
                              const float *vel4, int device, gsph_handle *out);
/* gsph_batch_create with room to grow: buffers sized for particle_capacity
 * particles, cell_capacity cells and scene_capacity scenes (each at least
 * the initial batch's), so gsph_batch_repack can change the scene set
 * without reallocating. */
gsph_status gsph_batch_create_ex(const gsph_params *params, const uint32_t *counts,
                                 uint32_t num_scenes, const float *pos4,
                                 const float *vel4, uint64_t particle_capacity,
                                 uint64_t cell_capacity, uint32_t scene_capacity,
                                 int device, gsph_handle *out);
/* Changes the scene set between frames: the scenes listed in keep (current
 * indices) stay, in that order, followed by n_add new scenes (parameters,
 * counts, concatenated float4 positions / velocities; velocities may be
 * NULL). Kept scenes continue exactly as if stepped alone. Fails with
 * GSPH_ERR_CAPACITY, leaving the batch unchanged, when the new set does not
 * fit the capacity. No counterpart in the reference (used by a serving loop
 * that admits and retires scenes). */
gsph_status gsph_batch_repack(gsph_handle h, const uint32_t *keep, uint32_t n_keep,
                              const gsph_params *add_params, const uint32_t *add_counts,
                              uint32_t n_add, const float *add_pos4,
                              const float *add_vel4);
/* Continuous-batching scene server (no counterpart in the reference, which
 * steps one scene per process). Requests — a scene's parameters, initial
 * positions (and velocities) and a number of frames — wait in a FIFO queue;
 * gsph_server_step admits the queued requests that fit the memory budget and
 * a batch's capacity (opening batches up to max_batches), steps every resident
 * scene together up to the earliest
 * completion (at most chunk_frames frames), and keeps the finished requests'
 * final state for gsph_server_take. Each request is stepped exactly its
 * frames, and its result is bit-identical to the scene stepped alone. A
 * request that cannot fit even alone is rejected (counted in the stats).
 * submit / poll / take / get_stats may be called from other threads while
 * one thread calls gsph_server_step. All requests share the physical
 * parameters of the first one admitted (see gsph_batch_create). */
typedef struct gsph_server *gsph_server_handle;
typedef struct {
    uint64_t budget_bytes;         /* device bytes the resident scenes may use */
    uint64_t particle_capacity;    /* capacity of each batch: particles, cells, */
    uint64_t cell_capacity;        /* scenes (a batch holds < 2^26 cells)       */
    uint32_t scene_capacity;
    int32_t chunk_frames;          /* most frames between admissions (>= 1) */
    int32_t device;
    int32_t max_batches;           /* batches the server may open (0 or 1: one).
                                    * Each opened batch allocates its capacity;
                                    * the batches step concurrently on their
                                    * own streams, and the budget bounds the
                                    * resident bytes of all of them together. */
} gsph_server_config;
typedef struct {
    uint64_t submitted, finished, rejected;
    uint64_t frames, chunks, particle_steps;
    uint64_t queued, resident, resident_particles, resident_bytes;
    uint64_t batches;              /* batches holding resident scenes */
} gsph_server_stats;
gsph_status gsph_server_create(const gsph_server_config *cfg, gsph_server_handle *out);
gsph_status gsph_server_destroy(gsph_server_handle s);
gsph_status gsph_server_submit(gsph_server_handle s, uint64_t id, const gsph_params *p,
                               const float *pos4, const float *vel4, uint32_t n,
                               uint32_t frames);
/* frames_stepped (may be NULL) receives the frames of this chunk (0: idle). */
gsph_status gsph_server_step(gsph_server_handle s, int *frames_stepped);
/* The oldest finished request not yet taken (GSPH_ERR_STATE if none). */
gsph_status gsph_server_poll(gsph_server_handle s, uint64_t *id, uint32_t *n);
/* Copies a finished request's final positions / velocities (float4 each,
 * either may be NULL) and releases it. */
gsph_status gsph_server_take(gsph_server_handle s, uint64_t id, float *pos4, float *vel4);
gsph_status gsph_server_get_stats(gsph_server_handle s, gsph_server_stats *out);

/* Particle and cell offsets of the scenes: pbase_out[num_scenes + 1],
 * cbase_out[num_scenes + 1] (either may be NULL). Scene k's particles are
 * rows [pbase[k], pbase[k+1]) of every particle field. */
gsph_status gsph_batch_ranges(gsph_handle h, int32_t *pbase_out,
                              int32_t *cbase_out);
/* gsph_copy_out restricted to one scene, in that scene's own numbering
 * (particle fields: the scene's rows; KEY: the scene's own micro keys;
 * PERMUTATION: indices within the scene; CELL_START/CELL_COUNT: the scene's
 * cells, offsets from its first particle). */
gsph_status gsph_copy_out_scene(gsph_handle h, uint32_t scene, gsph_field field,
                                void *host_dst, size_t bytes);

/* One frame = arrange + density + force + advance (tick). gsph_density and
 * gsph_force need the grid of the current positions: they fail with
 * GSPH_ERR_STATE after gsph_advance, a frame, or a position copy-in until
 * gsph_arrange has run again. */
gsph_status gsph_step(gsph_handle h, int n_steps);
gsph_status gsph_arrange(gsph_handle h);
gsph_status gsph_density(gsph_handle h);
gsph_status gsph_force(gsph_handle h);
gsph_status gsph_advance(gsph_handle h);
/* frames > 0: gsph_step launches captured CUDA graphs of that many whole
 * frames (any remainder frame by frame); 0: kernels are launched one by one.
 * A frame needs no host synchronisation, so any number of frames can be
 * captured. */
gsph_status gsph_set_graph_mode(gsph_handle h, int frames);
gsph_status gsph_sync(gsph_handle h);
/* The handle's CUDA stream (a cudaStream_t), for callers that order their own
 * work or timing events against the handle's kernels. Some kernels of a frame
 * run on a second, internal stream, which every call joins back into this one
 * before it returns, so work ordered after this stream sees all of them. */
gsph_status gsph_stream(gsph_handle h, void **stream_out);

gsph_status gsph_get_info(gsph_handle h, gsph_info *out);
gsph_status gsph_get_params(gsph_handle h, gsph_params *out);
gsph_status gsph_copy_out(gsph_handle h, gsph_field field, void *host_dst,
                          size_t bytes);
/* Overwrites particle state (POSITION, VELOCITY, EVAL_VELOCITY,
 * ACCELERATION only) in the current order. */
gsph_status gsph_copy_in(gsph_handle h, gsph_field field, const void *host_src,
                         size_t bytes);
/* Asynchronous pinned-host copies on the handle's stream (host buffers must
 * stay valid until the next gsph_sync). */
gsph_status gsph_copy_in_async(gsph_handle h, gsph_field field,
                               const void *host_src, size_t bytes);
gsph_status gsph_copy_out_async(gsph_handle h, gsph_field field,
                                void *host_dst, size_t bytes);
/* A step on host-resident state: uploads position, velocity and evaluated
 * velocity (float4[N] each, the handle's current order, pinned memory) from
 * the three arrays, runs `frames` frames and downloads the new state into the
 * same arrays (HybridSystem::tick with the state kept on the host). Asynchronous:
 * the arrays are complete after gsph_sync. The downloads run on an internal
 * stream, so the upload of an array by the next call waits only for that
 * array's own download (the three round trips overlap); every other call on
 * the handle first waits for all of them. */
gsph_status gsph_step_host_async(gsph_handle h, int frames, void *pos4, void *vel4,
                                 void *ev4);

/* Render-space transform of GSPH_FIELD_FINAL_POSITION (the reference's
 * sim_ratio / sim_origin, sph_hybrid_system.cpp:221-224); default ratio 1,
 * origin 0. */
gsph_status gsph_set_render_transform(gsph_handle h, const float ratio[3],
                                      const float origin[3]);

/* Split thresholds and launch shapes (see gsph_tuning). */
gsph_status gsph_tuning_default(gsph_tuning *out);
gsph_status gsph_get_tuning(gsph_handle h, gsph_tuning *out);
gsph_status gsph_set_tuning(gsph_handle h, const gsph_tuning *t);

/* Viscosity model of the force pass (every scene of a handle).
 * GSPH_VISCOSITY_LAPLACIAN (the default) is the reference's: mu * visco_value
 * * sum_j V_j (v_j - v_i)(h - r) with V_j = 1/rho_j (force_kernels.cu:378-435,
 * 525-561), mu = gsph_params.viscosity.
 * GSPH_VISCOSITY_ARTIFICIAL is Monaghan's artificial viscosity (Monaghan
 * 1992) in place of it: for a pair approaching each other (v_ij . r_ij < 0,
 * v_ij = v_i - v_j, r_ij = x_i - x_j, velocities = evaluated velocities),
 *   mu_ij = h v_ij . r_ij / (r^2 + 0.01 h^2),
 *   Pi_ij = -alpha c0 mu_ij / ((rho_i + rho_j) / 2),
 * and the particle's force (the quantity the integrator divides by rho_i)
 * gains -m rho_i sum_j Pi_ij grad W(r_ij), with the spiky gradient the
 * pressure term uses. alpha > 0 and c0 > 0 (the speed of sound) are given.
 * The reference has no such term (it is an option of this library, checked
 * against the FP64 oracle). The model is a handle setting: it is not stored
 * in snapshots, and scene servers use the default. */
typedef enum {
    GSPH_VISCOSITY_LAPLACIAN = 0,
    GSPH_VISCOSITY_ARTIFICIAL = 1
} gsph_viscosity_model;
gsph_status gsph_set_viscosity_model(gsph_handle h, int model, float alpha, float c0);
/* Times n_candidates tunings (NULL: a built-in grid of split thresholds and
 * CTAs per SM) on the handle's current state, frames_per_trial frames each
 * after one warm-up frame, restoring the state after every trial, and
 * installs the fastest. best_out / best_ms_out (either may be NULL) receive
 * it and its device time per frame. The state, frame counter and results of
 * the handle are as before the call. Replaces the reference's fixed
 * thresholds; no counterpart in the reference. */
gsph_status gsph_autotune(gsph_handle h, int frames_per_trial,
                          const gsph_tuning *candidates, int n_candidates,
                          gsph_tuning *best_out, float *best_ms_out);

/* FP64 state checksum as the reference's benchmark prints it:
 * {sum x, sum y, sum z, sum w, sum ((i&1023)+1)*(x+3y+7z)}. */
gsph_status gsph_checksum(gsph_handle h, double out[5]);
/* Order-independent FP64 reductions on the device: {sum m, sum m*v.x, .y, .z,
 * kinetic energy, sum x, sum y, sum z}. */
gsph_status gsph_reductions(gsph_handle h, double out[8]);

gsph_status gsph_benchmark(gsph_handle h, int frames, gsph_bench_report *out);
/* Stage timing: while enabled, every frame records CUDA events on the
 * handle's stream between its stages (frames then run without graphs).
 * gsph_stage_times waits for the stream and returns the mean device time (ms)
 * per frame since the previous call: {arrange, density, force, integrate};
 * density and force are one kernel launch each. */
gsph_status gsph_set_stage_timing(gsph_handle h, int enabled);
gsph_status gsph_stage_times(gsph_handle h, float out[4]);

/* Kernel-level entry: the grid sort (arrange stage, A2-A5) over caller-owned
 * device buffers (the Arrangement path, sph_arrangement.cu:1352-1395).
 * Positions/velocities/evaluated velocities are float4 device arrays of n
 * particles; the sorted copies go to the *_out arrays; key_out (uint32[n]),
 * perm_out (int32[n]) and cell_start_out (int32[numc+1]) receive the grid.
 * scratch/scratch_bytes is caller-owned device memory of at least
 * gsph_grid_sort_scratch_bytes(n, numc) bytes. stream is a cudaStream_t. */
size_t gsph_grid_sort_scratch_bytes(uint32_t n, uint32_t numc);
gsph_status gsph_grid_sort_dev(const gsph_params *p, uint32_t n,
                               const float *pos_in, const float *vel_in,
                               const float *ev_in, float *pos_out,
                               float *vel_out, float *ev_out,
                               uint32_t *key_out, int32_t *perm_out,
                               int32_t *cell_start_out, void *scratch,
                               size_t scratch_bytes, void *stream);

/* The same grid sort for callers that cannot allocate device memory at the
 * call site: hosts that run under a fixed device-memory budget kept by their
 * own pool allocator (a raw cudaMalloc would fail or escape the budget), and
 * real-time loops that cannot pay cudaMalloc's implicit synchronisation.
 * No counterpart in the reference: it is an addition of this library.
 * The caller passes inputs and outputs only; the scratch is a fixed
 * file-scope device array of GSPH_NOALLOC_SCRATCH_BYTES that every GPU which
 * loads the library holds until the process exits. Limits: at most
 * GSPH_NOALLOC_MAX_PARTICLES particles and GSPH_NOALLOC_MAX_CELLS cells;
 * larger inputs return GSPH_ERR_CAPACITY without launching anything. The
 * first call on a device looks up the array's device address on that device
 * (make that first call before any stream capture). Calls share the array:
 * each call clears what it accumulates into, but calls that overlap on the
 * GPU (different streams, or different host threads) race. Allocates
 * nothing: no cudaMalloc, cudaFree or allocating library routine. */
#define GSPH_NOALLOC_MAX_PARTICLES 262144u
#define GSPH_NOALLOC_MAX_CELLS 524288u
#define GSPH_NOALLOC_SCRATCH_BYTES 10487040u
gsph_status gsph_grid_sort_dev_noalloc(const gsph_params *p, uint32_t n,
                                       const float *pos_in, const float *vel_in,
                                       const float *ev_in, float *pos_out,
                                       float *vel_out, float *ev_out,
                                       uint32_t *key_out, int32_t *perm_out,
                                       int32_t *cell_start_out, void *stream);

#ifdef __cplusplus
}
#endif

#endif /* GSPH_H_ */
