// system.cu — the scene runtime behind the C ABI: device buffers, the frame
// (tick) pipeline, CUDA-graph capture, timing, checksums and copy-out.
//
// Reference counterparts (KemengHuang/Fast-General-GPU-SPH-framework):
//   HybridSystem ctor / initializeScene  src/simulation/sph_hybrid_system.cpp:209-240, 432-473
//   HybridSystem::tick                   src/simulation/sph_hybrid_system.cpp:253-339
//   HybridSystem::runBenchmark           src/simulation/sph_hybrid_system.cpp:341-430
//   Arrangement ctor (buffers)           src/grid/sph_arrangement.cu:607-673
//   Arrangement::arrangeHybridFrame      src/grid/sph_arrangement.cu:1493-1506
//   getSmsTaskPairStats                  src/grid/sph_arrangement.cu:1595-1636
//   knInit (zero ev, acc)                src/solver/integration_kernels.cu:6-17
//
// Unlike the reference, a frame needs no host synchronisation (the TRA/SMS
// counts stay on the device), so whole frames can be captured as CUDA graphs.
#include <algorithm>
#include <cmath>
#include <chrono>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <vector>

#include "gsph_internal.h"

namespace gsph {

namespace {

#define GSPH_CUDA(call)                                                         \
    do {                                                                        \
        cudaError_t e_ = (call);                                                \
        if (e_ != cudaSuccess) {                                                \
            set_error("%s failed: %s (%s:%d)", #call, cudaGetErrorString(e_),  \
                      __FILE__, __LINE__);                                      \
            return GSPH_ERR_CUDA;                                               \
        }                                                                       \
    } while (0)

size_t align_up(size_t x, size_t a) { return (x + a - 1) / a * a; }

int device_sm_count(int device) {
    int v = 0;
    if (cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, device) !=
            cudaSuccess ||
        v <= 0)
        v = 1;
    return v;
}

// Repack: gathers the kept scenes' particle state into the front of the
// other buffer set. Kept scene k moves from [src_base[k], +count) to
// [dst_base[k], dst_base[k+1]); one thread per destination particle finds
// its scene by binary search over dst_base (empty scenes are skipped by
// taking the last base <= i).
__global__ void __launch_bounds__(256)
k_repack_gather(const float4 *__restrict__ pos_s, const float4 *__restrict__ vel_s,
                const float4 *__restrict__ ev_s, float4 *__restrict__ pos_d,
                float4 *__restrict__ vel_d, float4 *__restrict__ ev_d,
                const int *__restrict__ dst_base, const int *__restrict__ src_base,
                int n_keep, int total) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= total) return;
    int lo = 0, hi = n_keep - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (dst_base[mid] <= i)
            lo = mid;
        else
            hi = mid - 1;
    }
    const int src = src_base[lo] + (i - dst_base[lo]);
    pos_d[i] = pos_s[src];
    vel_d[i] = vel_s[src];
    ev_d[i] = ev_s[src];
}

}  // namespace

struct System {
    gsph_params params{};
    DevParams dp{};
    int device = 0;
    int num_sms = 1;
    int n = 0;
    int numc = 0;
    int max_occ = 0;
    int task_capacity = 0;
    cudaStream_t stream = nullptr;
    std::vector<void *> allocs;
    size_t device_bytes = 0;

    float4 *pos[2] = {nullptr, nullptr};
    float4 *vel[2] = {nullptr, nullptr};
    float4 *ev[2] = {nullptr, nullptr};
    float4 *acc = nullptr;
    int cur = 0;   // buffer index that holds the current (sorted) state
    Frame fr{};    // pointers shared by both parities
    double *red = nullptr;   // reductions workspace
    bool arranged = false;   // sorted state + split valid
    bool grid_current = false;   // no position changed since the last arrange
    bool lists_valid = false;   // TRA neighbour masks match the state
    // hashed: key_in / slot / cell_count hold the micro keys and cell slots
    // of the current state (computed ahead by the last frame's force pass),
    // so the next arrange skips its hash launch. counts_dirty: cell_count may
    // hold counts that no arrange will consume (cleared before a new hash).
    bool hashed = false;
    bool counts_dirty = false;
    uint64_t frames = 0;

    LaunchShape shape = kMaxShape;   // CTAs per SM of the density/force kernels
    float3 render_ratio = make_float3(1.f, 1.f, 1.f);
    float3 render_origin = make_float3(0.f, 0.f, 0.f);
    uint32_t *render_color = nullptr;    // allocated on first use
    float4 *render_pos = nullptr;
    int graph_frames = 0;   // frames per captured CUDA graph (0: stream launches)
    cudaGraphExec_t graph[2] = {nullptr, nullptr};   // by starting parity

    bool timing = false;
    std::vector<cudaEvent_t> ev_pool;

    // gsph_step_host_async: the state's return copies run on their own
    // stream, one event per array, so that the next call's upload of an array
    // waits only for that array's return copy. Every other entry point joins
    // them into the main stream first (join_xfer).
    cudaStream_t xfer = nullptr;
    cudaEvent_t xfer_done[3] = {nullptr, nullptr, nullptr};
    cudaEvent_t frames_done = nullptr;
    bool xfer_pending = false;

    void join_xfer() {
        if (!xfer_pending) return;
        for (cudaEvent_t e : xfer_done) cudaStreamWaitEvent(stream, e, 0);
        xfer_pending = false;
    }
    std::vector<std::vector<cudaEvent_t>> ev_pending;   // 5 events per frame

    // The SMS side of the density and force stages (task pairing, SMS
    // density, SMS force) runs on a second stream beside the TRA passes:
    // fork() orders it after the main stream's work so far, join() orders
    // the main stream after it. Inside a capture the pair becomes a fork
    // and a join of the graph. In an all-TRA frame the SMS launches, which
    // find no work, then cost the frame nothing.
    cudaStream_t aux = nullptr;
    cudaEvent_t fork_ev = nullptr, join_ev = nullptr;
    void fork() {
        cudaEventRecord(fork_ev, stream);
        cudaStreamWaitEvent(aux, fork_ev, 0);
    }
    void join() {
        cudaEventRecord(join_ev, aux);
        cudaStreamWaitEvent(stream, join_ev, 0);
    }

    ~System() { release(); }

    void release() {
        if (device >= 0) cudaSetDevice(device);
        for (auto &g : graph)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
        for (auto &v : ev_pending)
            for (auto e : v) cudaEventDestroy(e);
        ev_pending.clear();
        for (auto e : ev_pool) cudaEventDestroy(e);
        ev_pool.clear();
        if (xfer) {
            cudaStreamSynchronize(xfer);
            cudaStreamDestroy(xfer);
            xfer = nullptr;
        }
        for (auto &e : xfer_done)
            if (e) {
                cudaEventDestroy(e);
                e = nullptr;
            }
        if (frames_done) {
            cudaEventDestroy(frames_done);
            frames_done = nullptr;
        }
        if (aux) {
            cudaStreamSynchronize(aux);
            cudaStreamDestroy(aux);
            aux = nullptr;
        }
        for (cudaEvent_t *e : {&fork_ev, &join_ev})
            if (*e) {
                cudaEventDestroy(*e);
                *e = nullptr;
            }
        xfer_pending = false;
        for (void *p : allocs) cudaFree(p);
        allocs.clear();
        if (stream) {
            cudaStreamDestroy(stream);
            stream = nullptr;
        }
    }

    gsph_status alloc(void **p, size_t bytes) {
        bytes = std::max<size_t>(align_up(bytes, 256), 256);
        cudaError_t e = cudaMalloc(p, bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            set_error("cudaMalloc of %zu bytes failed: %s", bytes,
                      cudaGetErrorString(e));
            return e == cudaErrorMemoryAllocation ? GSPH_ERR_OUT_OF_MEMORY
                                                  : GSPH_ERR_CUDA;
        }
        allocs.push_back(*p);
        device_bytes += bytes;
        return GSPH_OK;
    }

    template <typename T>
    gsph_status alloc_n(T **p, size_t count) {
        return alloc(reinterpret_cast<void **>(p), count * sizeof(T));
    }

    // Scenes of the batch (a single scene is a batch of one).
    std::vector<gsph_params> scene_params;
    std::vector<int> pbase, cbase;          // [S + 1] particle / cell offsets
    std::vector<SceneGeom> geom;            // [S]
    SceneGeom *d_geom = nullptr;
    int *d_pbase = nullptr, *d_cbase = nullptr;
    int *d_repack = nullptr;   // repack gather table: dst bases, src bases
    int n_cap = 0, c_cap = 0, s_cap = 0;    // capacities of the buffers

    // Every scene of a batch must share the physical parameters; only the box
    // (world size, grid, upper walls) may differ.
    static bool same_physics(const gsph_params &a, const gsph_params &b) {
        gsph_params x = a, y = b;
        for (gsph_params *q : {&x, &y}) {
            for (int k = 0; k < 3; ++k) {
                q->world_size[k] = 0.f;
                q->grid_size[k] = 0;
                q->bound_max[k] = 0.f;
            }
        }
        return std::memcmp(&x, &y, sizeof(x)) == 0;
    }

    // Scene table for `count` scenes of the given sizes (host side).
    gsph_status layout(const gsph_params *plist, const uint32_t *counts,
                       int count, long long &n_total, long long &c_total) {
        scene_params.assign(plist, plist + count);
        pbase.assign(size_t(count) + 1, 0);
        cbase.assign(size_t(count) + 1, 0);
        geom.resize(size_t(count));
        n_total = 0;
        c_total = 0;
        for (int k = 0; k < count; ++k) {
            const gsph_params &q = plist[k];
            if (!same_physics(q, plist[0])) {
                set_error("scene %d of the batch has physical parameters that "
                          "differ from scene 0 (only the box may differ)", k);
                return GSPH_ERR_INVALID_ARG;
            }
            const long long cells =
                (long long)q.grid_size[0] * q.grid_size[1] * q.grid_size[2];
            if (cells <= 0) {
                set_error("scene %d has an empty grid", k);
                return GSPH_ERR_INVALID_ARG;
            }
            geom[size_t(k)] = make_scene_geom(q, int(c_total));
            n_total += counts[k];
            c_total += cells;
            pbase[size_t(k) + 1] = int(std::min<long long>(n_total, 0x7FFFFFFF));
            cbase[size_t(k) + 1] = int(std::min<long long>(c_total, 0x7FFFFFFF));
        }
        if (n_total > 0x7FFFFFFFLL) {
            set_error("batch holds %lld particles; at most 2^31-1", n_total);
            return GSPH_ERR_CAPACITY;
        }
        if (c_total >= 67108864LL) {   // 32-bit micro keys: cells * 64 < 2^32
            set_error("batch holds %lld cells; at most 2^26", c_total);
            return GSPH_ERR_CAPACITY;
        }
        return GSPH_OK;
    }

    gsph_status upload_table() {
        const int S = int(geom.size());
        if (S > s_cap) {
            set_error("batch of %d scenes exceeds its capacity of %d", S, s_cap);
            return GSPH_ERR_CAPACITY;
        }
        GSPH_CUDA(cudaMemcpyAsync(d_geom, geom.data(), sizeof(SceneGeom) * S,
                                  cudaMemcpyHostToDevice, stream));
        GSPH_CUDA(cudaMemcpyAsync(d_pbase, pbase.data(), sizeof(int) * (S + 1),
                                  cudaMemcpyHostToDevice, stream));
        GSPH_CUDA(cudaMemcpyAsync(d_cbase, cbase.data(), sizeof(int) * (S + 1),
                                  cudaMemcpyHostToDevice, stream));
        fr.scenes.geom = d_geom;
        fr.scenes.pbase = d_pbase;
        fr.scenes.cbase = d_cbase;
        fr.scenes.count = S;
        if (S > 0) fr.scenes.single = geom[0];
        return GSPH_OK;
    }

    // Sizes that depend on the particle and cell counts of the current layout.
    void set_counts(int n_particles, int n_cells) {
        n = n_particles;
        numc = n_cells;
        dp.numc = n_cells;
        max_occ = std::max(1, std::min(numc, n));
        task_capacity = (n + kSmsTaskParticles - 1) / kSmsTaskParticles + max_occ + 2;
        fr.n = n;
        fr.task_capacity = task_capacity;
        params = scene_params.empty() ? params : scene_params[0];
        drop_graphs();
    }

    gsph_status init(const gsph_params *plist, const uint32_t *counts, int count,
                     const float *pos4, const float *vel4, int dev,
                     long long n_capacity = 0, long long c_capacity = 0,
                     int s_capacity = 0) {
        device = dev;
        GSPH_CUDA(cudaSetDevice(device));
        num_sms = device_sm_count(device);
        GSPH_CUDA(configure_physics_kernels(device));
        GSPH_CUDA(cudaStreamCreateWithFlags(&stream, cudaStreamNonBlocking));
        GSPH_CUDA(cudaStreamCreateWithFlags(&aux, cudaStreamNonBlocking));
        GSPH_CUDA(cudaEventCreateWithFlags(&fork_ev, cudaEventDisableTiming));
        GSPH_CUDA(cudaEventCreateWithFlags(&join_ev, cudaEventDisableTiming));
        long long n_total = 0, c_total = 0;
        if (count < 1) {
            set_error("a batch needs at least one scene at creation");
            return GSPH_ERR_INVALID_ARG;
        }
        gsph_status st = layout(plist, counts, count, n_total, c_total);
        if (st) return st;
        dp = make_dev_params(plist[0]);
        params = plist[0];
        n_cap = int(std::max<long long>(std::max(n_total, n_capacity), 1));
        c_cap = int(std::max(c_total, c_capacity));
        s_cap = std::max(count, s_capacity);
        const int occ_cap = std::max(1, std::min(c_cap, n_cap));
        const int task_cap =
            (n_cap + kSmsTaskParticles - 1) / kSmsTaskParticles + occ_cap + 2;
        const size_t N = size_t(n_cap), C = size_t(c_cap);
        for (int b = 0; b < 2; ++b) {
            if ((st = alloc_n(&pos[b], N)) || (st = alloc_n(&vel[b], N)) ||
                (st = alloc_n(&ev[b], N)))
                return st;
        }
        if ((st = alloc_n(&acc, N)) || (st = alloc_n(&fr.key_in, N)) ||
            (st = alloc_n(&fr.slot, N)) || (st = alloc_n(&fr.pairs, N)) ||
            (st = alloc_n(&fr.key, N)) || (st = alloc_n(&fr.perm, N)) ||
            (st = alloc_n(&fr.cell_count, C)) ||
            (st = alloc_n(&fr.cell_start, C + 1)) ||
            (st = alloc_n(&fr.cell_xslab, C)) ||
            (st = alloc_n(&fr.cell_grp, C * 16)) ||
            (st = alloc_n(&fr.occ_list, size_t(occ_cap))) ||
            (st = alloc_n(&fr.big_list, size_t(occ_cap))) ||
            (st = alloc_n(&fr.cell_val, size_t(occ_cap))) ||
            (st = alloc_n(&fr.cell_prefix, size_t(occ_cap))) ||
            (st = alloc_n(&fr.tasks, size_t(task_cap))) ||
            (st = alloc_n(&fr.compact, N)) ||
            (st = alloc_n(&fr.nbr_mask, ((N + 31) / 32) * 32 * 9)) ||
            (st = alloc_n(&fr.nbr_flag, N)) ||
            (st = alloc_n(&fr.scan_tiles, (C + kScanTile - 1) / kScanTile)) ||
            (st = alloc_n(&fr.scan_tiles4, size_t((occ_cap + kValTile - 1) / kValTile))) ||
            (st = alloc_n(&fr.ctr, 1)) ||
            (st = alloc_n(&red, size_t(8 + 8 * 512))) ||
            (st = alloc_n(&d_geom, size_t(s_cap))) ||
            (st = alloc_n(&d_pbase, size_t(s_cap) + 1)) ||
            (st = alloc_n(&d_cbase, size_t(s_cap) + 1)) ||
            (st = alloc_n(&d_repack, 2 * size_t(s_cap) + 2)))
            return st;
        fr.acc = acc;
        set_counts(int(n_total), int(c_total));
        if ((st = upload_table())) return st;
        GSPH_CUDA(cudaMemsetAsync(fr.cell_count, 0, sizeof(int32_t) * C, stream));
        GSPH_CUDA(cudaMemsetAsync(fr.cell_xslab, 0xFF, sizeof(uint32_t) * C, stream));
        GSPH_CUDA(cudaMemsetAsync(fr.ctr, 0, sizeof(Counters), stream));
        GSPH_CUDA(cudaMemsetAsync(fr.tasks, 0, sizeof(gsph_block_task) * task_cap, stream));
        for (int b = 0; b < 2; ++b) {
            GSPH_CUDA(cudaMemsetAsync(pos[b], 0, sizeof(float4) * N, stream));
            GSPH_CUDA(cudaMemsetAsync(vel[b], 0, sizeof(float4) * N, stream));
            GSPH_CUDA(cudaMemsetAsync(ev[b], 0, sizeof(float4) * N, stream));
        }
        GSPH_CUDA(cudaMemsetAsync(acc, 0, sizeof(float4) * N, stream));
        if (n > 0) {
            GSPH_CUDA(cudaMemcpyAsync(pos[0], pos4, sizeof(float4) * n,
                                      cudaMemcpyHostToDevice, stream));
            if (vel4)
                GSPH_CUDA(cudaMemcpyAsync(vel[0], vel4, sizeof(float4) * n,
                                          cudaMemcpyHostToDevice, stream));
        }
        cur = 0;
        GSPH_CUDA(cudaStreamSynchronize(stream));
        return GSPH_OK;
    }

    // New scene set: the kept scenes (by current index, in the given order)
    // followed by new ones. The kept scenes' state is copied on the device
    // in its current order, so each continues exactly as if alone.
    gsph_status repack(const uint32_t *keep, int n_keep, const gsph_params *add_p,
                       const uint32_t *add_n, int n_add, const float *add_pos4,
                       const float *add_vel4) {
        const int S_old = int(geom.size());
        std::vector<gsph_params> plist;
        std::vector<uint32_t> counts;
        std::vector<int> src_base;
        for (int k = 0; k < n_keep; ++k) {
            if (keep[k] >= uint32_t(S_old)) {
                set_error("repack: scene %u out of range", keep[k]);
                return GSPH_ERR_INVALID_ARG;
            }
            plist.push_back(scene_params[keep[k]]);
            counts.push_back(uint32_t(pbase[keep[k] + 1] - pbase[keep[k]]));
            src_base.push_back(pbase[keep[k]]);
        }
        for (int k = 0; k < n_add; ++k) {
            plist.push_back(add_p[k]);
            counts.push_back(add_n[k]);
        }
        const int S = n_keep + n_add;
        if (S > 0 && !same_physics(plist[0], params)) {
            set_error("repack: new scenes must share the batch's physical parameters");
            return GSPH_ERR_INVALID_ARG;
        }
        if (S > s_cap) {
            set_error("repack: %d scenes exceed the capacity of %d", S, s_cap);
            return GSPH_ERR_CAPACITY;
        }
        // validate before touching any state
        std::vector<gsph_params> old_params = scene_params;
        std::vector<int> old_pbase = pbase, old_cbase = cbase;
        std::vector<SceneGeom> old_geom = geom;
        long long n_total = 0, c_total = 0;
        gsph_status st = S > 0 ? layout(plist.data(), counts.data(), S, n_total, c_total)
                               : GSPH_OK;
        if (st == GSPH_OK && (n_total > n_cap || c_total > c_cap)) {
            set_error("repack: %lld particles / %lld cells exceed the capacity "
                      "(%d / %d)", n_total, c_total, n_cap, c_cap);
            st = GSPH_ERR_CAPACITY;
        }
        if (st) {
            scene_params = old_params;
            pbase = old_pbase;
            cbase = old_cbase;
            geom = old_geom;
            return st;
        }
        if (S == 0) {
            scene_params.clear();
            pbase.assign(1, 0);
            cbase.assign(1, 0);
            geom.clear();
        }
        const int dst = 1 - cur;
        // kept scenes: one gather launch into the front of the other buffers
        const int kept_total = n_keep > 0 ? pbase[size_t(n_keep)] : 0;
        if (kept_total > 0) {
            std::vector<int> table(size_t(2 * n_keep + 1));
            for (int k = 0; k <= n_keep; ++k) table[size_t(k)] = pbase[size_t(k)];
            for (int k = 0; k < n_keep; ++k)
                table[size_t(n_keep + 1 + k)] = src_base[size_t(k)];
            GSPH_CUDA(cudaMemcpyAsync(d_repack, table.data(), sizeof(int) * table.size(),
                                      cudaMemcpyHostToDevice, stream));
            k_repack_gather<<<(kept_total + 255) / 256, 256, 0, stream>>>(
                pos[cur], vel[cur], ev[cur], pos[dst], vel[dst], ev[dst], d_repack,
                d_repack + n_keep + 1, n_keep, kept_total);
            GSPH_CUDA(cudaGetLastError());
        }
        // new scenes: contiguous after the kept ones, one copy per array
        const size_t added = size_t(n_total - kept_total);
        if (added > 0) {
            GSPH_CUDA(cudaMemcpyAsync(pos[dst] + kept_total, add_pos4,
                                      sizeof(float4) * added, cudaMemcpyHostToDevice,
                                      stream));
            if (add_vel4)
                GSPH_CUDA(cudaMemcpyAsync(vel[dst] + kept_total, add_vel4,
                                          sizeof(float4) * added,
                                          cudaMemcpyHostToDevice, stream));
            else
                GSPH_CUDA(cudaMemsetAsync(vel[dst] + kept_total, 0,
                                          sizeof(float4) * added, stream));
            GSPH_CUDA(cudaMemsetAsync(ev[dst] + kept_total, 0, sizeof(float4) * added,
                                      stream));
        }
        cur = dst;
        set_counts(int(n_total), int(c_total));
        if ((st = upload_table())) return st;
        arranged = false;
        grid_current = false;
        lists_valid = false;
        hashed = false;
        counts_dirty = true;
        GSPH_CUDA(cudaStreamSynchronize(stream));
        return GSPH_OK;
    }

    // Frame descriptor of the arrange stage reading buffer `in`.
    Frame frame_arrange(int in) const {
        Frame f = fr;
        f.pos_in = pos[in];
        f.vel_in = vel[in];
        f.ev_in = ev[in];
        f.pos = pos[1 - in];
        f.vel = vel[1 - in];
        f.ev = ev[1 - in];
        return f;
    }
    // Frame descriptor of the physics stages on buffer `b`.
    Frame frame_physics(int b) const {
        Frame f = fr;
        f.pos_in = pos[b];
        f.vel_in = vel[b];
        f.ev_in = ev[b];
        f.pos = pos[b];
        f.vel = vel[b];
        f.ev = ev[b];
        return f;
    }

    // Hash of the current state into key_in / slot / cell_count.
    void enqueue_hash(int in) {
        if (counts_dirty)
            cudaMemsetAsync(fr.cell_count, 0, sizeof(int32_t) * size_t(c_cap), stream);
        launch_hash_count(frame_arrange(in), dp, stream);
        hashed = true;
        counts_dirty = true;
    }

    // pair_tasks: also pair the SMS tasks (judgeTask) here; a frame leaves
    // that to its density stage, on the second stream.
    void enqueue_arrange(int in, bool pair_tasks = true) {
        lists_valid = false;
        const Frame f = frame_arrange(in);
        if (!hashed) enqueue_hash(in);
        launch_cell_scan(f, dp, stream);
        launch_scatter_pairs(f, stream);
        launch_cell_sort(f, num_sms, stream);
        launch_split(f, dp, max_occ, num_sms, stream);
        if (pair_tasks) launch_judge(f, max_occ, num_sms, stream);
        hashed = false;          // consumed; the sort cleared the counts
        counts_dirty = false;
    }
    // pair_tasks: the arrange left the task pairing to this stage.
    void enqueue_density(int b, bool pair_tasks = false) {
        const Frame f = frame_physics(b);
        fork();
        if (pair_tasks) launch_judge(f, max_occ, num_sms, aux);
        launch_density(f, dp, num_sms, shape, stream, aux);
        join();
        lists_valid = true;
    }
    void enqueue_force(int b) {
        fork();
        launch_force(frame_physics(b), dp, num_sms, lists_valid, shape, stream, aux);
        join();
    }
    // Force on buffer b with the integration fused in: the new state goes to
    // buffer 1 - b (the previous frame's unsorted copy, no longer read), in
    // buffer b's order. keep_acc: also store the acceleration (the last frame
    // of a step does, so GSPH_FIELD_ACCELERATION holds it afterwards).
    void enqueue_force_advance(int b, bool keep_acc = true) {
        Frame f = frame_physics(b);
        if (!keep_acc) f.acc = nullptr;
        f.pos_next = pos[1 - b];
        f.vel_next = vel[1 - b];
        f.ev_next = ev[1 - b];
        f.hash_next = true;
        fork();
        launch_force(f, dp, num_sms, lists_valid, shape, stream, aux);
        // the SMS particles' keys ahead, after their force pass on the
        // second stream (beside the TRA force pass, which hashes its own)
        launch_hash_sms(f, f.pos_next, dp, aux);
        join();
        lists_valid = false;
        hashed = true;
        counts_dirty = true;
    }
    void enqueue_advance(int b) {
        launch_integrate(frame_physics(b), dp, stream);
        lists_valid = false;
        hashed = false;
    }

    gsph_status check_launch() {
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) {
            set_error("kernel launch failed: %s", cudaGetErrorString(e));
            return GSPH_ERR_CUDA;
        }
        return GSPH_OK;
    }

    cudaEvent_t take_event() {
        if (!ev_pool.empty()) {
            cudaEvent_t e = ev_pool.back();
            ev_pool.pop_back();
            return e;
        }
        cudaEvent_t e = nullptr;
        cudaEventCreate(&e);
        return e;
    }

    // Capture graph_frames whole frames starting from buffer `parity`.
    gsph_status build_graph(int parity) {
        cudaGraph_t g = nullptr;
        GSPH_CUDA(cudaStreamBeginCapture(stream, cudaStreamCaptureModeThreadLocal));
        // graph launches are preceded by a complete hash of the state
        hashed = true;
        for (int k = 0; k < graph_frames; ++k) {
            enqueue_arrange(parity, false);
            enqueue_density(1 - parity, true);
            enqueue_force_advance(1 - parity, k == graph_frames - 1);
        }
        cudaError_t e = cudaStreamEndCapture(stream, &g);
        if (e != cudaSuccess) {
            set_error("graph capture failed: %s", cudaGetErrorString(e));
            if (g) cudaGraphDestroy(g);
            return GSPH_ERR_CUDA;
        }
        e = cudaGraphInstantiate(&graph[parity], g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            set_error("graph instantiate failed: %s", cudaGetErrorString(e));
            graph[parity] = nullptr;
            return GSPH_ERR_CUDA;
        }
        return GSPH_OK;
    }

    void drop_graphs() {
        for (auto &g : graph)
            if (g) {
                cudaGraphExecDestroy(g);
                g = nullptr;
            }
    }

    // One frame launched kernel by kernel (with stage events when timing):
    // the sort moves the state from buffer `cur` into the other buffer, and
    // the force pass, which also integrates, writes the new state back into
    // buffer `cur` in the sorted order. The integrate stage time is then 0
    // (it is part of the force pass).
    gsph_status tick(bool keep_acc = true) {
        if (numc == 0) return GSPH_OK;   // a batch without scenes
        const int in = cur, out = 1 - cur;
        std::vector<cudaEvent_t> evs;
        if (timing) {
            for (int k = 0; k < 5; ++k) evs.push_back(take_event());
            cudaEventRecord(evs[0], stream);
        }
        enqueue_arrange(in, false);
        if (timing) cudaEventRecord(evs[1], stream);
        enqueue_density(out, true);
        if (timing) cudaEventRecord(evs[2], stream);
        enqueue_force_advance(out, keep_acc);
        if (timing) {
            cudaEventRecord(evs[3], stream);
            cudaEventRecord(evs[4], stream);
            ev_pending.push_back(std::move(evs));
        }
        gsph_status st = check_launch();
        if (st) return st;
        cur = in;
        arranged = true;
        grid_current = false;
        ++frames;
        return GSPH_OK;
    }

    // n frames: whole captured graphs while they fit, single frames after.
    gsph_status step(int n) {
        if (numc == 0) return GSPH_OK;   // a batch without scenes
        if (graph_frames > 0 && !timing) {
            // captured frames start from a hashed state and leave one behind
            if (n >= graph_frames && !hashed) enqueue_hash(cur);
            GSPH_CUDA(cudaGetLastError());
            while (n >= graph_frames) {
                if (!graph[cur]) {
                    gsph_status st = build_graph(cur);
                    if (st) return st;
                }
                GSPH_CUDA(cudaGraphLaunch(graph[cur], stream));
                hashed = true;
                counts_dirty = true;
                arranged = true;
                grid_current = false;
                lists_valid = false;
                frames += uint64_t(graph_frames);
                n -= graph_frames;
            }
        }
        for (int k = 0; k < n; ++k) {
            gsph_status st = tick(k == n - 1);
            if (st) return st;
        }
        return GSPH_OK;
    }

    gsph_status read_counters(Counters &c) {
        GSPH_CUDA(cudaMemcpyAsync(&c, fr.ctr, sizeof(Counters),
                                  cudaMemcpyDeviceToHost, stream));
        GSPH_CUDA(cudaStreamSynchronize(stream));
        return GSPH_OK;
    }

    gsph_status sync_and_check() {
        join_xfer();
        GSPH_CUDA(cudaStreamSynchronize(stream));
        Counters c;
        gsph_status st = read_counters(c);
        if (st) return st;
        if (c.err & kErrOutOfDomain) {
            set_error("a particle left the simulation grid (first index %d); it "
                      "was clamped into the boundary cell",
                      c.err_index);
            clear_err();
            return GSPH_ERR_DOMAIN;
        }
        if (c.err & kErrTaskCapacity) {
            set_error("SMS task buffer overflow");
            clear_err();
            return GSPH_ERR_CAPACITY;
        }
        return GSPH_OK;
    }

    void clear_err() {
        uint32_t z[2] = {0, 0};
        cudaMemcpyAsync(&fr.ctr->err, z, sizeof(z), cudaMemcpyHostToDevice, stream);
        cudaStreamSynchronize(stream);
    }

    gsph_tuning tuning() const {
        gsph_tuning t{};
        t.sparse_total = dp.sparse_total;
        t.sparse_self = dp.sparse_self;
        t.mid_total = dp.mid_total;
        t.ctas_density_tra = shape.density_tra;
        t.ctas_density_sms = shape.density_sms;
        t.ctas_force_tra = shape.force_tra;
        t.ctas_force_sms = shape.force_sms;
        t.warps_per_block = shape.warps;
        return t;
    }

    gsph_status set_tuning(const gsph_tuning &t) {
        const int warps = t.warps_per_block == 0 ? kMaxShape.warps : t.warps_per_block;
        const int k = (warps == kMaxShape.warps / 2) ? 2 : 1;
        if ((warps != kMaxShape.warps && warps != kMaxShape.warps / 2) ||
            t.sparse_total < 0 || t.sparse_self < 0 || t.mid_total < 0 ||
            t.ctas_density_tra < 1 || t.ctas_density_tra > k * kMaxShape.density_tra ||
            t.ctas_density_sms < 1 || t.ctas_density_sms > k * kMaxShape.density_sms ||
            t.ctas_force_tra < 1 || t.ctas_force_tra > k * kMaxShape.force_tra ||
            t.ctas_force_sms < 1 || t.ctas_force_sms > k * kMaxShape.force_sms) {
            set_error("gsph_set_tuning: thresholds must be >= 0, warps per block %d or %d, "
                      "and CTAs per SM in [1, %d/%d/%d/%d] (twice that with %d warps)",
                      kMaxShape.warps, kMaxShape.warps / 2, kMaxShape.density_tra,
                      kMaxShape.density_sms, kMaxShape.force_tra, kMaxShape.force_sms,
                      kMaxShape.warps / 2);
            return GSPH_ERR_INVALID_ARG;
        }
        dp.sparse_total = t.sparse_total;
        dp.sparse_self = t.sparse_self;
        dp.mid_total = t.mid_total;
        shape = {t.ctas_density_tra, t.ctas_density_sms, t.ctas_force_tra,
                 t.ctas_force_sms, warps};
        drop_graphs();   // the captured launches carry the old values
        return GSPH_OK;
    }

    // Times each candidate on a saved copy of the current state (one warm-up
    // frame, then `trial` frames between events), restores the state after
    // every trial and installs the fastest candidate.
    gsph_status autotune(int trial, const gsph_tuning *cand, int nc, gsph_tuning *best,
                         float *best_ms) {
        if (trial < 1 || nc < 1 || !cand) {
            set_error("gsph_autotune: need frames_per_trial >= 1 and a candidate");
            return GSPH_ERR_INVALID_ARG;
        }
        for (int k = 0; k < nc; ++k) {
            gsph_tuning probe = cand[k];
            const gsph_tuning keep = tuning();
            gsph_status st = set_tuning(probe);
            set_tuning(keep);
            if (st) return st;
        }
        GSPH_CUDA(cudaStreamSynchronize(stream));
        const gsph_tuning start = tuning();
        if (numc == 0 || n == 0) {
            if (best) *best = start;
            if (best_ms) *best_ms = 0.f;
            return GSPH_OK;
        }
        const size_t bytes = sizeof(float4) * size_t(n);
        float4 *saved = nullptr;
        GSPH_CUDA(cudaMalloc(&saved, 3 * bytes));
        const int cur0 = cur;
        const uint64_t frames0 = frames;
        const bool arranged0 = arranged;
        const int graphs0 = graph_frames;
        const bool timing0 = timing;
        auto restore = [&]() -> gsph_status {
            cur = cur0;
            GSPH_CUDA(cudaMemcpyAsync(pos[cur], saved, bytes, cudaMemcpyDeviceToDevice, stream));
            GSPH_CUDA(cudaMemcpyAsync(vel[cur], saved + n, bytes, cudaMemcpyDeviceToDevice,
                                      stream));
            GSPH_CUDA(cudaMemcpyAsync(ev[cur], saved + 2 * size_t(n), bytes,
                                      cudaMemcpyDeviceToDevice, stream));
            return GSPH_OK;
        };
        gsph_status st = GSPH_OK;
        cudaEvent_t e0 = nullptr, e1 = nullptr;
        int best_k = -1;
        float best_t = 0.f;
        do {
            cudaError_t ce = cudaMemcpyAsync(saved, pos[cur], bytes, cudaMemcpyDeviceToDevice,
                                             stream);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(saved + n, vel[cur], bytes, cudaMemcpyDeviceToDevice,
                                     stream);
            if (ce == cudaSuccess)
                ce = cudaMemcpyAsync(saved + 2 * size_t(n), ev[cur], bytes,
                                     cudaMemcpyDeviceToDevice, stream);
            if (ce == cudaSuccess) ce = cudaEventCreate(&e0);
            if (ce == cudaSuccess) ce = cudaEventCreate(&e1);
            if (ce != cudaSuccess) {
                set_error("gsph_autotune: %s", cudaGetErrorString(ce));
                st = GSPH_ERR_CUDA;
                break;
            }
            graph_frames = 0;
            timing = false;
            for (int k = 0; k < nc && !st; ++k) {
                if ((st = restore()) || (st = set_tuning(cand[k])) || (st = tick())) break;
                cudaEventRecord(e0, stream);
                for (int f = 0; f < trial && !st; ++f) st = tick();
                cudaEventRecord(e1, stream);
                if (st || (st = sync_and_check())) break;
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                ms /= float(trial);
                if (best_k < 0 || ms < best_t) {
                    best_k = k;
                    best_t = ms;
                }
            }
        } while (false);
        gsph_status rs = restore();
        set_tuning(best_k >= 0 && !st ? cand[best_k] : start);
        frames = frames0;
        arranged = arranged0;
        // the trials' sorts rewrote the grid arrays (offsets, keys, tasks):
        // the restored state needs a new arrange
        grid_current = false;
        lists_valid = false;
        hashed = false;
        counts_dirty = true;
        graph_frames = graphs0;
        timing = timing0;
        cudaStreamSynchronize(stream);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        cudaFree(saved);
        if (st) return st;
        if (rs) return rs;
        if (best) *best = cand[best_k];
        if (best_ms) *best_ms = best_t;
        return GSPH_OK;
    }

    gsph_status stage_times(float out[4]) {
        GSPH_CUDA(cudaStreamSynchronize(stream));
        double acc4[4] = {0, 0, 0, 0};
        const size_t nf = ev_pending.size();
        for (auto &evs : ev_pending) {
            for (int k = 0; k < 4; ++k) {
                float ms = 0.f;
                cudaEventElapsedTime(&ms, evs[k], evs[k + 1]);
                acc4[k] += ms;
            }
            for (auto e : evs) ev_pool.push_back(e);
        }
        ev_pending.clear();
        for (int k = 0; k < 4; ++k) out[k] = nf ? float(acc4[k] / nf) : 0.f;
        return GSPH_OK;
    }
};

}  // namespace gsph

using namespace gsph;

struct gsph_system {
    System sys;
};

namespace {

// Validates the handle and makes it current. join: order the main stream
// after any state return copies still in flight (every entry point but
// gsph_step_host_async, which waits array by array).
gsph_status check_handle(gsph_handle h, bool join = true) {
    if (!h) {
        set_error("null gsph handle");
        return GSPH_ERR_INVALID_ARG;
    }
    cudaError_t e = cudaSetDevice(h->sys.device);
    if (e != cudaSuccess) {
        set_error("cudaSetDevice(%d) failed: %s", h->sys.device,
                  cudaGetErrorString(e));
        return GSPH_ERR_CUDA;
    }
    if (join) h->sys.join_xfer();
    return GSPH_OK;
}

size_t field_bytes(const System &s, gsph_field f, gsph_status &st) {
    st = GSPH_OK;
    const size_t N = size_t(s.n);
    switch (f) {
        case GSPH_FIELD_POSITION:
        case GSPH_FIELD_VELOCITY:
        case GSPH_FIELD_EVAL_VELOCITY:
        case GSPH_FIELD_ACCELERATION: return N * sizeof(float4);
        case GSPH_FIELD_KEY:
        case GSPH_FIELD_PERMUTATION:
        case GSPH_FIELD_COMPACT_INDEX: return N * 4;
        case GSPH_FIELD_CELL_START: return (size_t(s.numc) + 1) * 4;
        case GSPH_FIELD_CELL_COUNT:
        case GSPH_FIELD_BLOCK_REQ: return size_t(s.numc) * 4;
        case GSPH_FIELD_MICRO_START: return (size_t(s.numc) * 64 + 1) * 4;
        case GSPH_FIELD_SPLIT: return 8;
        case GSPH_FIELD_COLOR: return N * 4;
        case GSPH_FIELD_FINAL_POSITION: return N * sizeof(float4);
        case GSPH_FIELD_NEIGHBOR_COUNT: return N * 4;
        case GSPH_FIELD_TASKS: return 0;   // variable, checked separately
    }
    st = GSPH_ERR_INVALID_ARG;
    set_error("unknown field %d", int(f));
    return 0;
}

float4 *state_ptr(System &s, gsph_field f) {
    switch (f) {
        case GSPH_FIELD_POSITION: return s.pos[s.cur];
        case GSPH_FIELD_VELOCITY: return s.vel[s.cur];
        case GSPH_FIELD_EVAL_VELOCITY: return s.ev[s.cur];
        case GSPH_FIELD_ACCELERATION: return s.acc;
        default: return nullptr;
    }
}

}  // namespace

extern "C" {

gsph_status gsph_create(const gsph_params *p, const float *pos4,
                        const float *vel4, uint32_t n, int device,
                        gsph_handle *out) {
    if (!p || !out || (n > 0 && !pos4)) {
        set_error("gsph_create: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (n > 0x7FFFFFFFu) {
        set_error("gsph_create: %u particles exceed 2^31-1", n);
        return GSPH_ERR_CAPACITY;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error("There is no CUDA device (%s).",
                  e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return GSPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        set_error("device %d out of range [0, %d)", device, count);
        return GSPH_ERR_INVALID_ARG;
    }
    {
        const gsph_status gs = check_grid(*p, "gsph_create", nullptr);
        if (gs) return gs;
    }
    gsph_system *h = new (std::nothrow) gsph_system();
    if (!h) {
        set_error("gsph_create: host allocation failed");
        return GSPH_ERR_OUT_OF_MEMORY;
    }
    const uint32_t counts[1] = {n};
    gsph_status st = h->sys.init(p, counts, 1, pos4, vel4, device);
    if (st) {
        delete h;
        return st;
    }
    *out = h;
    return GSPH_OK;
}

gsph_status gsph_create_from_json(const char *scene_path, int device,
                                  gsph_handle *out) {
    if (!scene_path || !out) {
        set_error("gsph_create_from_json: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_scene sc;
    gsph_status st = gsph_scene_load_json(scene_path, &sc);
    if (st) return st;
    gsph_params p;
    if ((st = gsph_params_init(&sc, &p))) return st;
    uint32_t n = 0;
    if ((st = gsph_lattice_count(&sc, &p, &n))) return st;
    std::vector<float> pos(size_t(n) * 4 + 4);
    if ((st = gsph_lattice_fill(&sc, &p, pos.data(), n, &n))) return st;
    return gsph_create(&p, pos.data(), nullptr, n, device, out);
}

gsph_status gsph_batch_create(const gsph_params *params, const uint32_t *counts,
                              uint32_t num_scenes, const float *pos4,
                              const float *vel4, int device, gsph_handle *out) {
    if (!params || !counts || !out || num_scenes == 0) {
        set_error("gsph_batch_create: null argument or no scene");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = nullptr;
    unsigned long long total = 0;
    for (uint32_t k = 0; k < num_scenes; ++k) total += counts[k];
    if (total > 0 && !pos4) {
        set_error("gsph_batch_create: null positions");
        return GSPH_ERR_INVALID_ARG;
    }
    if (total > 0x7FFFFFFFull) {
        set_error("gsph_batch_create: %llu particles exceed 2^31-1", total);
        return GSPH_ERR_CAPACITY;
    }
    if (num_scenes > 1000000u) {
        set_error("gsph_batch_create: too many scenes (%u)", num_scenes);
        return GSPH_ERR_CAPACITY;
    }
    int count = 0;
    cudaError_t e = cudaGetDeviceCount(&count);
    if (e != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error("There is no CUDA device (%s).",
                  e == cudaSuccess ? "count 0" : cudaGetErrorString(e));
        return GSPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        set_error("device %d out of range [0, %d)", device, count);
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_system *h = new (std::nothrow) gsph_system();
    if (!h) {
        set_error("gsph_batch_create: host allocation failed");
        return GSPH_ERR_OUT_OF_MEMORY;
    }
    gsph_status st = h->sys.init(params, counts, int(num_scenes), pos4, vel4, device);
    if (st) {
        delete h;
        return st;
    }
    *out = h;
    return GSPH_OK;
}

gsph_status gsph_batch_ranges(gsph_handle h, int32_t *pbase_out,
                              int32_t *cbase_out) {
    if (!h) {
        set_error("null gsph handle");
        return GSPH_ERR_INVALID_ARG;
    }
    const System &s = h->sys;
    if (pbase_out) std::copy(s.pbase.begin(), s.pbase.end(), pbase_out);
    if (cbase_out) std::copy(s.cbase.begin(), s.cbase.end(), cbase_out);
    return GSPH_OK;
}

gsph_status gsph_batch_create_ex(const gsph_params *params, const uint32_t *counts,
                                 uint32_t num_scenes, const float *pos4,
                                 const float *vel4, uint64_t particle_capacity,
                                 uint64_t cell_capacity, uint32_t scene_capacity,
                                 int device, gsph_handle *out) {
    if (!params || !counts || !out || num_scenes == 0) {
        set_error("gsph_batch_create_ex: null argument or no scene");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = nullptr;
    if (particle_capacity > 0x7FFFFFFFull || cell_capacity >= 67108864ull ||
        scene_capacity > 1000000u) {
        set_error("gsph_batch_create_ex: capacity out of range");
        return GSPH_ERR_CAPACITY;
    }
    int count = 0;
    if (cudaGetDeviceCount(&count) != cudaSuccess || count == 0) {
        cudaGetLastError();
        set_error("There is no CUDA device.");
        return GSPH_ERR_NO_DEVICE;
    }
    if (device < 0 || device >= count) {
        set_error("device %d out of range [0, %d)", device, count);
        return GSPH_ERR_INVALID_ARG;
    }
    gsph_system *h = new (std::nothrow) gsph_system();
    if (!h) {
        set_error("gsph_batch_create_ex: host allocation failed");
        return GSPH_ERR_OUT_OF_MEMORY;
    }
    gsph_status st = h->sys.init(params, counts, int(num_scenes), pos4, vel4, device,
                                 (long long)particle_capacity, (long long)cell_capacity,
                                 int(scene_capacity));
    if (st) {
        delete h;
        return st;
    }
    *out = h;
    return GSPH_OK;
}

gsph_status gsph_batch_repack(gsph_handle h, const uint32_t *keep, uint32_t n_keep,
                              const gsph_params *add_params, const uint32_t *add_counts,
                              uint32_t n_add, const float *add_pos4,
                              const float *add_vel4) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if ((n_keep && !keep) || (n_add && (!add_params || !add_counts))) {
        set_error("gsph_batch_repack: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    unsigned long long added = 0;
    for (uint32_t k = 0; k < n_add; ++k) added += add_counts[k];
    if (added && !add_pos4) {
        set_error("gsph_batch_repack: null positions");
        return GSPH_ERR_INVALID_ARG;
    }
    System &s = h->sys;
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    return s.repack(keep, int(n_keep), add_params, add_counts, int(n_add), add_pos4,
                    add_vel4);
}

gsph_status gsph_destroy(gsph_handle h) {
    if (!h) return GSPH_OK;
    delete h;
    return GSPH_OK;
}

gsph_status gsph_step(gsph_handle h, int n_steps) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (n_steps < 0) {
        set_error("gsph_step: negative step count");
        return GSPH_ERR_INVALID_ARG;
    }
    return h->sys.step(n_steps);
}

gsph_status gsph_arrange(gsph_handle h) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    s.enqueue_arrange(s.cur);
    if ((st = s.check_launch())) return st;
    s.cur = 1 - s.cur;
    s.arranged = true;
    s.grid_current = true;
    return GSPH_OK;
}

static gsph_status need_arranged(System &s) {
    if (!s.arranged || !s.grid_current) {
        set_error("positions changed since the last arrange (call gsph_arrange)");
        return GSPH_ERR_STATE;
    }
    return GSPH_OK;
}

gsph_status gsph_density(gsph_handle h) {
    gsph_status st = check_handle(h);
    if (st || (st = need_arranged(h->sys))) return st;
    h->sys.enqueue_density(h->sys.cur);
    return h->sys.check_launch();
}

gsph_status gsph_force(gsph_handle h) {
    gsph_status st = check_handle(h);
    if (st || (st = need_arranged(h->sys))) return st;
    h->sys.enqueue_force(h->sys.cur);
    return h->sys.check_launch();
}

gsph_status gsph_advance(gsph_handle h) {
    gsph_status st = check_handle(h);
    if (st) return st;
    h->sys.enqueue_advance(h->sys.cur);
    h->sys.grid_current = false;
    return h->sys.check_launch();
}

gsph_status gsph_set_graph_mode(gsph_handle h, int enabled) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (enabled < 0) {
        set_error("gsph_set_graph_mode: negative frame count");
        return GSPH_ERR_INVALID_ARG;
    }
    if (enabled != h->sys.graph_frames) h->sys.drop_graphs();
    h->sys.graph_frames = enabled;
    return GSPH_OK;
}

gsph_status gsph_sync(gsph_handle h) {
    gsph_status st = check_handle(h);
    if (st) return st;
    return h->sys.sync_and_check();
}

gsph_status gsph_stream(gsph_handle h, void **stream_out) {
    if (!h || !stream_out) {
        set_error("gsph_stream: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    *stream_out = static_cast<void *>(h->sys.stream);
    return GSPH_OK;
}

gsph_status gsph_get_info(gsph_handle h, gsph_info *out) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (!out) {
        set_error("gsph_get_info: null output");
        return GSPH_ERR_INVALID_ARG;
    }
    System &s = h->sys;
    Counters c;
    if ((st = s.read_counters(c))) return st;
    std::memset(out, 0, sizeof(*out));
    out->n_particles = uint32_t(s.n);
    out->n_cells = uint32_t(s.numc);
    for (int a = 0; a < 3; ++a) out->grid_size[a] = s.params.grid_size[a];
    out->tra_particles = s.arranged ? c.middle : s.n;
    out->sms_tasks = s.arranged ? c.task_count : 0;
    out->occupied_cells = c.num_occ;
    out->big_cells = c.num_big;
    out->frames = s.frames;
    out->device_bytes = s.device_bytes;
    out->n_scenes = uint32_t(s.geom.size());
    return GSPH_OK;
}

gsph_status gsph_get_params(gsph_handle h, gsph_params *out) {
    if (!h || !out) {
        set_error("gsph_get_params: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = h->sys.params;
    return GSPH_OK;
}

gsph_status gsph_copy_out(gsph_handle h, gsph_field field, void *host_dst,
                          size_t bytes) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (!host_dst) {
        set_error("gsph_copy_out: null destination");
        return GSPH_ERR_INVALID_ARG;
    }
    System &s = h->sys;
    if ((st = s.sync_and_check()) && st != GSPH_ERR_DOMAIN) return st;
    Counters c;
    if ((st = s.read_counters(c))) return st;
    const int T = s.arranged ? c.task_count : 0;
    if (field == GSPH_FIELD_TASKS) {
        const size_t need = size_t(T + (T & 1)) * sizeof(gsph_block_task);
        if (bytes != need) {
            set_error("gsph_copy_out(TASKS): %zu bytes given, %zu needed", bytes,
                      need);
            return GSPH_ERR_INVALID_ARG;
        }
        if (need)
            GSPH_CUDA(cudaMemcpy(host_dst, s.fr.tasks, need, cudaMemcpyDeviceToHost));
        return GSPH_OK;
    }
    const size_t need = field_bytes(s, field, st);
    if (st) return st;
    if (bytes != need) {
        set_error("gsph_copy_out(%d): %zu bytes given, %zu needed", int(field),
                  bytes, need);
        return GSPH_ERR_INVALID_ARG;
    }
    const int numc = s.numc;
    switch (field) {
        case GSPH_FIELD_POSITION:
        case GSPH_FIELD_VELOCITY:
        case GSPH_FIELD_EVAL_VELOCITY:
        case GSPH_FIELD_ACCELERATION:
            if (need)
                GSPH_CUDA(cudaMemcpy(host_dst, state_ptr(s, field), need,
                                     cudaMemcpyDeviceToHost));
            return GSPH_OK;
        case GSPH_FIELD_KEY:
            if (need) GSPH_CUDA(cudaMemcpy(host_dst, s.fr.key, need, cudaMemcpyDeviceToHost));
            return GSPH_OK;
        case GSPH_FIELD_PERMUTATION:
            if (need) GSPH_CUDA(cudaMemcpy(host_dst, s.fr.perm, need, cudaMemcpyDeviceToHost));
            return GSPH_OK;
        case GSPH_FIELD_COMPACT_INDEX:
            if (s.arranged && !c.any_sms) {   // all TRA: the identity, not stored
                int32_t *o = static_cast<int32_t *>(host_dst);
                for (int i = 0; i < s.n; ++i) o[i] = i;
                return GSPH_OK;
            }
            if (need) GSPH_CUDA(cudaMemcpy(host_dst, s.fr.compact, need, cudaMemcpyDeviceToHost));
            return GSPH_OK;
        case GSPH_FIELD_CELL_START:
            GSPH_CUDA(cudaMemcpy(host_dst, s.fr.cell_start, need, cudaMemcpyDeviceToHost));
            return GSPH_OK;
        case GSPH_FIELD_CELL_COUNT: {
            std::vector<int32_t> st1(size_t(numc) + 1);
            GSPH_CUDA(cudaMemcpy(st1.data(), s.fr.cell_start, st1.size() * 4,
                                 cudaMemcpyDeviceToHost));
            int32_t *o = static_cast<int32_t *>(host_dst);
            for (int i = 0; i < numc; ++i) o[i] = st1[i + 1] - st1[i];
            return GSPH_OK;
        }
        case GSPH_FIELD_MICRO_START: {
            // Dense micro offsets (the reference's d_cell_offset_M) rebuilt
            // from the sorted keys: exclusive sum of the micro counts.
            std::vector<uint32_t> keys(size_t(s.n));
            if (s.n)
                GSPH_CUDA(cudaMemcpy(keys.data(), s.fr.key, size_t(s.n) * 4,
                                     cudaMemcpyDeviceToHost));
            int32_t *o = static_cast<int32_t *>(host_dst);
            const size_t m = size_t(numc) * 64;
            std::memset(o, 0, (m + 1) * 4);
            for (uint32_t k : keys)
                if (k < m) ++o[k + 1];
            for (size_t i = 1; i <= m; ++i) o[i] += o[i - 1];
            return GSPH_OK;
        }
        case GSPH_FIELD_BLOCK_REQ: {
            int32_t *o = static_cast<int32_t *>(host_dst);
            std::memset(o, 0, size_t(numc) * 4);
            if (!s.arranged || c.num_occ <= 0) return GSPH_OK;
            std::vector<int32_t> occ(size_t(c.num_occ));
            std::vector<int4> val(size_t(c.num_occ));
            GSPH_CUDA(cudaMemcpy(occ.data(), s.fr.occ_list, occ.size() * 4,
                                 cudaMemcpyDeviceToHost));
            GSPH_CUDA(cudaMemcpy(val.data(), s.fr.cell_val, val.size() * sizeof(int4),
                                 cudaMemcpyDeviceToHost));
            for (size_t k = 0; k < occ.size(); ++k) o[occ[k]] = val[k].x;
            return GSPH_OK;
        }
        case GSPH_FIELD_NEIGHBOR_COUNT: {
            if (!s.arranged) {
                set_error("gsph_copy_out(NEIGHBOR_COUNT): no arranged frame yet");
                return GSPH_ERR_STATE;
            }
            int32_t *o = static_cast<int32_t *>(host_dst);
            for (int i = 0; i < s.n; ++i) o[i] = -1;
            const int mid = std::min(std::max(c.middle, 0), s.n);
            if (!mid) return GSPH_OK;
            std::vector<int32_t> flag(static_cast<size_t>(mid)), slot(static_cast<size_t>(mid));
            GSPH_CUDA(cudaMemcpy(flag.data(), s.fr.nbr_flag, size_t(mid) * 4,
                                 cudaMemcpyDeviceToHost));
            if (c.any_sms)
                GSPH_CUDA(cudaMemcpy(slot.data(), s.fr.compact, size_t(mid) * 4,
                                     cudaMemcpyDeviceToHost));
            else
                for (int i = 0; i < mid; ++i) slot[size_t(i)] = i;
            for (int i = 0; i < mid; ++i) {
                const int k = slot[size_t(i)];
                if (k >= 0 && k < s.n) o[k] = flag[size_t(i)];
            }
            return GSPH_OK;
        }
        case GSPH_FIELD_SPLIT: {
            int32_t *o = static_cast<int32_t *>(host_dst);
            o[0] = s.arranged ? c.middle : s.n;
            o[1] = T;
            return GSPH_OK;
        }
        case GSPH_FIELD_COLOR:
        case GSPH_FIELD_FINAL_POSITION: {
            if (!need) return GSPH_OK;
            const bool color = field == GSPH_FIELD_COLOR;
            if (color && !s.arranged) {
                set_error("gsph_copy_out(COLOR): no arranged frame yet");
                return GSPH_ERR_STATE;
            }
            if (color && !s.render_color &&
                (st = s.alloc_n(&s.render_color, size_t(s.n_cap))))
                return st;
            if (!color && !s.render_pos && (st = s.alloc_n(&s.render_pos, size_t(s.n_cap))))
                return st;
            Frame f = s.fr;
            f.pos = s.pos[s.cur];
            launch_render(f, s.render_ratio, s.render_origin,
                          color ? s.render_color : nullptr,
                          color ? nullptr : s.render_pos, s.stream);
            GSPH_CUDA(cudaGetLastError());
            GSPH_CUDA(cudaStreamSynchronize(s.stream));
            GSPH_CUDA(cudaMemcpy(host_dst, color ? static_cast<void *>(s.render_color)
                                                 : static_cast<void *>(s.render_pos),
                                 need, cudaMemcpyDeviceToHost));
            return GSPH_OK;
        }
        default: break;
    }
    set_error("gsph_copy_out: unsupported field %d", int(field));
    return GSPH_ERR_INVALID_ARG;
}

gsph_status gsph_copy_out_scene(gsph_handle h, uint32_t scene, gsph_field field,
                                void *host_dst, size_t bytes) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    if (!host_dst || scene >= s.geom.size()) {
        set_error("gsph_copy_out_scene: null destination or scene %u out of range",
                  scene);
        return GSPH_ERR_INVALID_ARG;
    }
    if ((st = s.sync_and_check()) && st != GSPH_ERR_DOMAIN) return st;
    const int p0 = s.pbase[scene], p1 = s.pbase[scene + 1];
    const int c0 = s.cbase[scene], c1 = s.cbase[scene + 1];
    const size_t np = size_t(p1 - p0), nc = size_t(c1 - c0);
    switch (field) {
        case GSPH_FIELD_POSITION:
        case GSPH_FIELD_VELOCITY:
        case GSPH_FIELD_EVAL_VELOCITY:
        case GSPH_FIELD_ACCELERATION: {
            if (bytes != np * sizeof(float4)) break;
            if (np)
                GSPH_CUDA(cudaMemcpy(host_dst, state_ptr(s, field) + p0, bytes,
                                     cudaMemcpyDeviceToHost));
            return GSPH_OK;
        }
        case GSPH_FIELD_KEY:
        case GSPH_FIELD_PERMUTATION: {
            if (bytes != np * 4) break;
            if (!np) return GSPH_OK;
            const bool key = field == GSPH_FIELD_KEY;
            GSPH_CUDA(cudaMemcpy(host_dst, key ? (const void *)(s.fr.key + p0)
                                               : (const void *)(s.fr.perm + p0),
                                 bytes, cudaMemcpyDeviceToHost));
            uint32_t *o = static_cast<uint32_t *>(host_dst);
            const uint32_t shift = key ? uint32_t(c0) << 6 : uint32_t(p0);
            for (size_t i = 0; i < np; ++i) o[i] -= shift;
            return GSPH_OK;
        }
        case GSPH_FIELD_CELL_START:
        case GSPH_FIELD_CELL_COUNT: {
            const bool start = field == GSPH_FIELD_CELL_START;
            if (bytes != (start ? nc + 1 : nc) * 4) break;
            std::vector<int32_t> st1(nc + 1);
            GSPH_CUDA(cudaMemcpy(st1.data(), s.fr.cell_start + c0, (nc + 1) * 4,
                                 cudaMemcpyDeviceToHost));
            int32_t *o = static_cast<int32_t *>(host_dst);
            for (size_t i = 0; i < nc; ++i)
                o[i] = start ? st1[i] - p0 : st1[i + 1] - st1[i];
            if (start) o[nc] = st1[nc] - p0;
            return GSPH_OK;
        }
        default:
            set_error("gsph_copy_out_scene: field %d has no per-scene form", int(field));
            return GSPH_ERR_INVALID_ARG;
    }
    set_error("gsph_copy_out_scene: %zu bytes given for field %d of scene %u", bytes,
              int(field), scene);
    return GSPH_ERR_INVALID_ARG;
}

gsph_status gsph_copy_in(gsph_handle h, gsph_field field, const void *host_src,
                         size_t bytes) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    float4 *dst = state_ptr(s, field);
    if (!dst || !host_src) {
        set_error("gsph_copy_in: field %d is not writable or source is null",
                  int(field));
        return GSPH_ERR_INVALID_ARG;
    }
    if (bytes != size_t(s.n) * sizeof(float4)) {
        set_error("gsph_copy_in: %zu bytes given, %zu needed", bytes,
                  size_t(s.n) * sizeof(float4));
        return GSPH_ERR_INVALID_ARG;
    }
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    if (bytes) GSPH_CUDA(cudaMemcpy(dst, host_src, bytes, cudaMemcpyHostToDevice));
    s.lists_valid = false;   // the masks describe the old state
    // new positions need a new grid (cell lists and the sorted x/y/z copy)
    if (field == GSPH_FIELD_POSITION) {
        s.grid_current = false;
        s.hashed = false;
    }
    return GSPH_OK;
}

gsph_status gsph_copy_in_async(gsph_handle h, gsph_field field,
                               const void *host_src, size_t bytes) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    float4 *dst = state_ptr(s, field);
    if (!dst || !host_src || bytes != size_t(s.n) * sizeof(float4)) {
        set_error("gsph_copy_in_async: bad field, source or size");
        return GSPH_ERR_INVALID_ARG;
    }
    if (bytes)
        GSPH_CUDA(cudaMemcpyAsync(dst, host_src, bytes, cudaMemcpyHostToDevice,
                                  s.stream));
    s.lists_valid = false;   // the masks describe the old state
    if (field == GSPH_FIELD_POSITION) {
        s.grid_current = false;
        s.hashed = false;
    }
    return GSPH_OK;
}

gsph_status gsph_step_host_async(gsph_handle h, int frames, void *pos4, void *vel4,
                                 void *ev4) {
    gsph_status st = check_handle(h, false);
    if (st) return st;
    System &s = h->sys;
    if (frames < 0 || !pos4 || !vel4 || !ev4) {
        set_error("gsph_step_host_async: negative frame count or null array");
        return GSPH_ERR_INVALID_ARG;
    }
    if (!s.xfer) {
        GSPH_CUDA(cudaStreamCreateWithFlags(&s.xfer, cudaStreamNonBlocking));
        for (auto &e : s.xfer_done)
            GSPH_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        GSPH_CUDA(cudaEventCreateWithFlags(&s.frames_done, cudaEventDisableTiming));
    }
    const gsph_field fields[3] = {GSPH_FIELD_POSITION, GSPH_FIELD_VELOCITY,
                                  GSPH_FIELD_EVAL_VELOCITY};
    void *host[3] = {pos4, vel4, ev4};
    const size_t bytes = size_t(s.n) * sizeof(float4);
    // upload: each array after its previous return copy (if any) is done
    for (int k = 0; k < 3; ++k) {
        if (s.xfer_pending) GSPH_CUDA(cudaStreamWaitEvent(s.stream, s.xfer_done[k], 0));
        if (bytes)
            GSPH_CUDA(cudaMemcpyAsync(state_ptr(s, fields[k]), host[k], bytes,
                                      cudaMemcpyHostToDevice, s.stream));
    }
    s.xfer_pending = false;
    s.lists_valid = false;
    s.grid_current = false;
    s.hashed = false;
    if ((st = s.step(frames))) return st;
    if ((st = s.check_launch())) return st;
    // return copies on the transfer stream, after the frames
    GSPH_CUDA(cudaEventRecord(s.frames_done, s.stream));
    GSPH_CUDA(cudaStreamWaitEvent(s.xfer, s.frames_done, 0));
    for (int k = 0; k < 3; ++k) {
        if (bytes)
            GSPH_CUDA(cudaMemcpyAsync(host[k], state_ptr(s, fields[k]), bytes,
                                      cudaMemcpyDeviceToHost, s.xfer));
        GSPH_CUDA(cudaEventRecord(s.xfer_done[k], s.xfer));
    }
    s.xfer_pending = true;
    return GSPH_OK;
}

gsph_status gsph_copy_out_async(gsph_handle h, gsph_field field, void *host_dst,
                                size_t bytes) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    float4 *src = state_ptr(s, field);
    if (!src || !host_dst || bytes != size_t(s.n) * sizeof(float4)) {
        set_error("gsph_copy_out_async: bad field, destination or size");
        return GSPH_ERR_INVALID_ARG;
    }
    if (bytes)
        GSPH_CUDA(cudaMemcpyAsync(host_dst, src, bytes, cudaMemcpyDeviceToHost,
                                  s.stream));
    return GSPH_OK;
}

gsph_status gsph_snapshot_save(gsph_handle h, const char *path) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    const size_t n = size_t(s.n);
    std::vector<float> pos(n * 4), vel(n * 4), ev(n * 4);
    if (n) {
        GSPH_CUDA(cudaMemcpy(pos.data(), s.pos[s.cur], n * 16, cudaMemcpyDeviceToHost));
        GSPH_CUDA(cudaMemcpy(vel.data(), s.vel[s.cur], n * 16, cudaMemcpyDeviceToHost));
        GSPH_CUDA(cudaMemcpy(ev.data(), s.ev[s.cur], n * 16, cudaMemcpyDeviceToHost));
    }
    const uint32_t S = uint32_t(s.scene_params.size());
    std::vector<uint32_t> counts(S);
    for (uint32_t k = 0; k < S; ++k) counts[k] = uint32_t(s.pbase[k + 1] - s.pbase[k]);
    return snapshot_write(path, s.scene_params.data(), counts.data(), S, pos.data(),
                          vel.data(), ev.data(), s.frames);
}

gsph_status gsph_snapshot_info(const char *path, uint32_t *n_scenes,
                               uint64_t *n_particles, uint64_t *frames) {
    return snapshot_header(path, n_scenes, n_particles, frames);
}

gsph_status gsph_snapshot_load(const char *path, int device, gsph_handle *out) {
    if (!out) {
        set_error("gsph_snapshot_load: null handle pointer");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = nullptr;
    std::vector<gsph_params> plist;
    std::vector<uint32_t> counts;
    std::vector<float> pos, vel, ev;
    uint64_t frames = 0;
    gsph_status st = snapshot_read(path, plist, counts, pos, vel, ev, frames);
    if (st) return st;
    if (plist.empty()) {
        set_error("snapshot %s holds no scene", path);
        return GSPH_ERR_PARSE;
    }
    gsph_handle h = nullptr;
    if (plist.size() == 1)
        st = gsph_create(plist.data(), pos.data(), vel.data(), counts[0], device, &h);
    else
        st = gsph_batch_create(plist.data(), counts.data(), uint32_t(plist.size()),
                               pos.data(), vel.data(), device, &h);
    if (st) return st;
    System &s = h->sys;
    if (s.n > 0) {
        cudaError_t e = cudaMemcpy(s.ev[s.cur], ev.data(), size_t(s.n) * 16,
                                   cudaMemcpyHostToDevice);
        if (e != cudaSuccess) {
            set_error("gsph_snapshot_load: %s", cudaGetErrorString(e));
            gsph_destroy(h);
            return GSPH_ERR_CUDA;
        }
    }
    s.frames = frames;
    *out = h;
    return GSPH_OK;
}

gsph_status gsph_set_render_transform(gsph_handle h, const float ratio[3],
                                      const float origin[3]) {
    if (!h || !ratio || !origin) {
        set_error("gsph_set_render_transform: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    h->sys.render_ratio = make_float3(ratio[0], ratio[1], ratio[2]);
    h->sys.render_origin = make_float3(origin[0], origin[1], origin[2]);
    return GSPH_OK;
}

gsph_status gsph_tuning_default(gsph_tuning *out) {
    if (!out) {
        set_error("gsph_tuning_default: null output");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = gsph_tuning{};
    out->sparse_total = 96;   // gpu_model.cu:172-180
    out->sparse_self = 15;
    out->mid_total = 60;
    out->ctas_density_tra = kMaxShape.density_tra;
    out->ctas_density_sms = kMaxShape.density_sms;
    out->ctas_force_tra = kMaxShape.force_tra;
    out->ctas_force_sms = kMaxShape.force_sms;
    out->warps_per_block = kMaxShape.warps;
    return GSPH_OK;
}

gsph_status gsph_get_tuning(gsph_handle h, gsph_tuning *out) {
    if (!h || !out) {
        set_error("gsph_get_tuning: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    *out = h->sys.tuning();
    return GSPH_OK;
}

gsph_status gsph_set_tuning(gsph_handle h, const gsph_tuning *t) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (!t) {
        set_error("gsph_set_tuning: null tuning");
        return GSPH_ERR_INVALID_ARG;
    }
    GSPH_CUDA(cudaStreamSynchronize(h->sys.stream));
    return h->sys.set_tuning(*t);
}

gsph_status gsph_set_viscosity_model(gsph_handle h, int model, float alpha, float c0) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (model != GSPH_VISCOSITY_LAPLACIAN && model != GSPH_VISCOSITY_ARTIFICIAL) {
        set_error("gsph_set_viscosity_model: unknown model %d", model);
        return GSPH_ERR_INVALID_ARG;
    }
    if (model == GSPH_VISCOSITY_ARTIFICIAL &&
        !(alpha > 0.f && c0 > 0.f && std::isfinite(alpha * c0))) {
        set_error("gsph_set_viscosity_model: alpha and c0 must be positive and finite");
        return GSPH_ERR_INVALID_ARG;
    }
    System &s = h->sys;
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    s.dp.visc_artificial = model == GSPH_VISCOSITY_ARTIFICIAL;
    s.dp.art_coef = model == GSPH_VISCOSITY_ARTIFICIAL ? alpha * c0 : 0.f;
    s.drop_graphs();   // the captured launches carry the old parameters
    return GSPH_OK;
}

// Built-in candidates: four split-threshold sets (the reference's, all TRA,
// SMS-leaning, TRA-leaning), each with block shapes of 8 and 4 warps, the
// largest and a smaller CTA count for each TRA pass, and for the SMS passes
// (with 8 warps) the largest and a smaller count: 4 x (2 x 2 x 2 + 2) = 40.
static std::vector<gsph_tuning> default_candidates() {
    std::vector<gsph_tuning> c;
    const int thr[4][3] = {{96, 15, 60}, {0x7FFFFFFF, 0x7FFFFFFF, 60},
                           {48, 8, 30}, {192, 30, 120}};
    auto add = [&](const int *t, int warps, int dt, int ds, int ft, int fs) {
        gsph_tuning g{};
        g.sparse_total = t[0];
        g.sparse_self = t[1];
        g.mid_total = t[2];
        g.ctas_density_tra = dt;
        g.ctas_density_sms = ds;
        g.ctas_force_tra = ft;
        g.ctas_force_sms = fs;
        g.warps_per_block = warps;
        c.push_back(g);
    };
    const LaunchShape m = kMaxShape;
    for (const auto &t : thr) {
        for (int w : {m.warps, m.warps / 2}) {
            const int k = w == m.warps ? 1 : 2;
            for (int dt : {k * m.density_tra, k * (m.density_tra - 2)})
                for (int ft : {k * m.force_tra, k * (m.force_tra - 1)})
                    add(t, w, dt, k * m.density_sms, ft, k * m.force_sms);
        }
        add(t, m.warps, m.density_tra, m.density_sms - 1, m.force_tra, m.force_sms - 1);
        add(t, m.warps, m.density_tra, m.density_sms - 2, m.force_tra, m.force_sms - 2);
    }
    return c;
}

gsph_status gsph_autotune(gsph_handle h, int frames_per_trial,
                          const gsph_tuning *candidates, int n_candidates,
                          gsph_tuning *best_out, float *best_ms_out) {
    gsph_status st = check_handle(h);
    if (st) return st;
    std::vector<gsph_tuning> builtin;
    if (!candidates) {
        builtin = default_candidates();
        candidates = builtin.data();
        n_candidates = int(builtin.size());
    }
    return h->sys.autotune(frames_per_trial, candidates, n_candidates, best_out,
                           best_ms_out);
}

gsph_status gsph_checksum(gsph_handle h, double out[5]) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    launch_checksum(s.pos[s.cur], s.n, s.red, s.stream);
    if ((st = s.check_launch())) return st;
    GSPH_CUDA(cudaMemcpyAsync(out, s.red, 5 * sizeof(double),
                              cudaMemcpyDeviceToHost, s.stream));
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    return GSPH_OK;
}

gsph_status gsph_reductions(gsph_handle h, double out[8]) {
    gsph_status st = check_handle(h);
    if (st) return st;
    System &s = h->sys;
    launch_reductions(s.pos[s.cur], s.vel[s.cur], s.n, s.params.mass, s.red,
                      s.stream);
    if ((st = s.check_launch())) return st;
    GSPH_CUDA(cudaMemcpyAsync(out, s.red, 8 * sizeof(double),
                              cudaMemcpyDeviceToHost, s.stream));
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    return GSPH_OK;
}

gsph_status gsph_set_stage_timing(gsph_handle h, int enabled) {
    gsph_status st = check_handle(h);
    if (st) return st;
    h->sys.timing = enabled != 0;
    return GSPH_OK;
}

gsph_status gsph_stage_times(gsph_handle h, float out[4]) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (!out) {
        set_error("gsph_stage_times: null output");
        return GSPH_ERR_INVALID_ARG;
    }
    return h->sys.stage_times(out);
}

gsph_status gsph_benchmark(gsph_handle h, int frames, gsph_bench_report *out) {
    gsph_status st = check_handle(h);
    if (st) return st;
    if (!out || frames <= 0) {
        set_error("gsph_benchmark: frame count must be positive");
        return GSPH_ERR_INVALID_ARG;
    }
    System &s = h->sys;
    std::memset(out, 0, sizeof(*out));
    // Warm-up frames with per-stage events (sph_hybrid_system.cpp:356-370).
    const int warm = frames < 5 ? frames : 5;
    const bool old_timing = s.timing;
    float stage[4] = {0, 0, 0, 0};
    s.timing = true;
    {
        float tmp[4];
        s.stage_times(tmp);   // drop anything pending
    }
    for (int i = 0; i < warm; ++i)
        if ((st = s.tick())) return st;
    s.stage_times(stage);
    s.timing = false;
    const int measured = frames - warm;
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    const auto t0 = std::chrono::steady_clock::now();
    if ((st = s.step(measured))) return st;
    GSPH_CUDA(cudaStreamSynchronize(s.stream));
    const auto t1 = std::chrono::steady_clock::now();
    s.timing = old_timing;
    const double elapsed = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const double total_kernel = stage[0] + stage[1] + stage[2] + stage[3];
    out->measured_frames = measured;
    out->warmup_frames = warm;
    out->total_wall_ms = elapsed;
    out->avg_frame_ms = measured > 0 ? elapsed / measured : total_kernel;
    out->fps = out->avg_frame_ms > 0 ? 1000.0 / out->avg_frame_ms : 0.0;
    out->particle_steps_per_s =
        out->avg_frame_ms > 0 ? double(s.n) * 1000.0 / out->avg_frame_ms : 0.0;
    out->arrange_ms = stage[0];
    out->density_ms = stage[1];
    out->force_ms = stage[2];
    out->integrate_ms = stage[3];
    out->total_kernel_ms = total_kernel;
    if ((st = gsph_checksum(h, out->checksum))) return st;
    if ((st = s.sync_and_check())) return st;
    Counters c;
    if ((st = s.read_counters(c))) return st;
    out->tra_particles = c.middle;
    out->sms_tasks = c.task_count;
    // Pair statistics (getSmsTaskPairStats, sph_arrangement.cu:1595-1636).
    const int T = c.task_count;
    if (T > 0) {
        std::vector<gsph_block_task> tasks(size_t(T + (T & 1)));
        GSPH_CUDA(cudaMemcpy(tasks.data(), s.fr.tasks,
                             tasks.size() * sizeof(gsph_block_task),
                             cudaMemcpyDeviceToHost));
        out->total_pairs = (T + 1) / 2;
        for (int i = 0; i < T; i += 2) {
            const gsph_block_task &a = tasks[size_t(i)];
            const gsph_block_task &b = tasks[size_t(i) + 1];
            if (a.is_same) {
                ++out->is_same_pairs;
                if (a.cell_particle_count - task_offset(b) >= kSmsTaskParticles)
                    ++out->full_is_same_pairs;
                else
                    ++out->partial_is_same_pairs;
                if (a.xxi == b.xxx)
                    ++out->compact_is_same_pairs;
                else
                    ++out->widened_is_same_pairs;
            }
            if (a.cellid == b.cellid) ++out->same_cell_pairs;
        }
    }
    return GSPH_OK;
}

// ------------------------------------------------------- kernel-level API --
size_t gsph_grid_sort_scratch_bytes(uint32_t n, uint32_t numc) {
    const size_t N = std::max<size_t>(n, 1), C = std::max<size_t>(numc, 1);
    const size_t occ = std::max<size_t>(std::min(N, C), 1);
    const size_t tiles = (C + kScanTile - 1) / kScanTile;
    size_t b = 0;
    b += align_up(N * 4, 256);      // key_in
    b += align_up(N * 4, 256);      // slot
    b += align_up(N * 8, 256);      // pairs
    b += align_up(C * 4, 256);      // cell_count
    b += align_up(C * 4, 256);      // cell_xslab
    b += align_up(occ * 4, 256);    // occ_list
    b += align_up(occ * 4, 256);    // big_list
    b += align_up(tiles * 8, 256);  // scan tiles
    b += align_up(sizeof(Counters), 256);
    return b;
}

gsph_status gsph_grid_sort_dev(const gsph_params *p, uint32_t n,
                               const float *pos_in, const float *vel_in,
                               const float *ev_in, float *pos_out,
                               float *vel_out, float *ev_out, uint32_t *key_out,
                               int32_t *perm_out, int32_t *cell_start_out,
                               void *scratch, size_t scratch_bytes,
                               void *stream) {
    if (!p || !pos_in || !vel_in || !ev_in || !pos_out || !vel_out || !ev_out ||
        !key_out || !perm_out || !cell_start_out || !scratch) {
        set_error("gsph_grid_sort_dev: null argument");
        return GSPH_ERR_INVALID_ARG;
    }
    {
        const gsph_status gs = check_grid(*p, "gsph_grid_sort_dev", nullptr);
        if (gs) return gs;
    }
    const DevParams dp = make_dev_params(*p);
    if (n > 0x7FFFFFFFu) {
        set_error("gsph_grid_sort_dev: too many particles");
        return GSPH_ERR_INVALID_ARG;
    }
    const size_t need = gsph_grid_sort_scratch_bytes(n, uint32_t(dp.numc));
    if (scratch_bytes < need) {
        set_error("gsph_grid_sort_dev: scratch of %zu bytes, %zu needed",
                  scratch_bytes, need);
        return GSPH_ERR_INVALID_ARG;
    }
    if (reinterpret_cast<uintptr_t>(scratch) % 256 != 0) {
        set_error("gsph_grid_sort_dev: scratch must be 256-byte aligned");
        return GSPH_ERR_INVALID_ARG;
    }
    int dev = 0;
    GSPH_CUDA(cudaGetDevice(&dev));
    const size_t N = std::max<size_t>(n, 1), C = size_t(dp.numc);
    const size_t occ = std::max<size_t>(std::min(N, C), 1);
    const size_t tiles = (C + kScanTile - 1) / kScanTile;
    char *w = static_cast<char *>(scratch);
    auto carve = [&](size_t bytes) {
        char *r = w;
        w += align_up(bytes, 256);
        return r;
    };
    Frame f{};
    f.n = int(n);
    f.scenes.count = 1;   // one scene: geometry passed inline, no device table
    f.scenes.single = make_scene_geom(*p, 0);
    f.pos_in = reinterpret_cast<const float4 *>(pos_in);
    f.vel_in = reinterpret_cast<const float4 *>(vel_in);
    f.ev_in = reinterpret_cast<const float4 *>(ev_in);
    f.pos = reinterpret_cast<float4 *>(pos_out);
    f.vel = reinterpret_cast<float4 *>(vel_out);
    f.ev = reinterpret_cast<float4 *>(ev_out);
    f.key = key_out;
    f.perm = perm_out;
    f.cell_start = cell_start_out;
    f.key_in = reinterpret_cast<uint32_t *>(carve(N * 4));
    f.slot = reinterpret_cast<uint32_t *>(carve(N * 4));
    f.pairs = reinterpret_cast<unsigned long long *>(carve(N * 8));
    f.cell_count = reinterpret_cast<int32_t *>(carve(C * 4));
    f.cell_xslab = reinterpret_cast<uint32_t *>(carve(C * 4));
    f.occ_list = reinterpret_cast<int32_t *>(carve(occ * 4));
    f.big_list = reinterpret_cast<int32_t *>(carve(occ * 4));
    f.scan_tiles = reinterpret_cast<unsigned long long *>(carve(tiles * 8));
    f.ctr = reinterpret_cast<Counters *>(carve(sizeof(Counters)));
    cudaStream_t s = static_cast<cudaStream_t>(stream);
    GSPH_CUDA(cudaMemsetAsync(f.cell_count, 0, C * 4, s));
    GSPH_CUDA(cudaMemsetAsync(f.ctr, 0, sizeof(Counters), s));
    launch_hash_count(f, dp, s);
    launch_cell_scan(f, dp, s);
    launch_scatter_pairs(f, s);
    launch_cell_sort(f, device_sm_count(dev), s);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) {
        set_error("gsph_grid_sort_dev: launch failed: %s", cudaGetErrorString(e));
        return GSPH_ERR_CUDA;
    }
    return GSPH_OK;
}

}  // extern "C"
