// split.cu — the hybrid SMS/TRA split and SMS task generation (rows A6-A9).
//
// Reference behaviour (KemengHuang/Fast-General-GPU-SPH-framework):
//   performance model  src/io/gpu_model.cu:137-181
//                      (knCalculateBlockRequirementHybridMode)
//   TRA/SMS partition  src/grid/sph_arrangement.cu:87-107, 193-206, 358-384,
//                      1459-1482 (bucket = cell (TRA) or cell+numc (SMS);
//                      compact index = TRA particles, then SMS particles;
//                      "middle" = number of TRA particles)
//   task scan + tasks  src/grid/sph_arrangement.cu:1499-1500, 885-965
//                      (knArrangeSmsTasks)
//   pairing            src/grid/sph_arrangement.cu:966-1022 (judgeTask)
//
// Design here: the work is indexed by OCCUPIED cells (compacted by the grid
// scan) instead of all numc cells, one scan of the triple {tasks, SMS
// particles, TRA particles} per occupied cell replaces the reference's second
// counting sort, and no host synchronisation is needed: counts stay on the
// device for the persistent density/force kernels.
#include <algorithm>

#include "gsph_internal.h"

namespace gsph {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

__device__ __forceinline__ int cell_n(const int32_t *__restrict__ start, int c) {
    return start[c + 1] - start[c];
}

// A6: SMS task count of one cell (gpu_model.cu:137-181, same neighbour
// bounds tests; the thresholds are the reference's unless tuned), with the
// cell's SMS and TRA particle counts: {req, sms, tra, 0}.
__device__ __forceinline__ int4 cell_model(int gidx, const int32_t *__restrict__ start,
                                           const SceneTable &T, int3 thr) {
    const SceneGeom G = geom_of_cell(T, gidx);
    const int idx = gidx - G.cbase;           // the scene's own cell index
    const int grid_x = G.gx, grid_y = G.gy;
    const int slice = grid_x * grid_y;
    const int numc = slice * G.gz;
    const int self = cell_n(start, gidx);
    int totaln = self;
    const int x = idx % grid_x;
    const int y = (idx / grid_x) % grid_y;
    if (x > 0) totaln += cell_n(start, gidx - 1);
    if (x + 1 < grid_x) totaln += cell_n(start, gidx + 1);
    if (y > 0) totaln += cell_n(start, gidx - grid_x);
    if (y + 1 < grid_y) totaln += cell_n(start, gidx + grid_x);
    if (idx >= slice) totaln += cell_n(start, gidx - slice);
    if (idx + slice < numc) totaln += cell_n(start, gidx + slice);
    int req;
    if (totaln < thr.x && self < thr.y)     // reference: 96, 15
        req = 0;
    else if (totaln < thr.z)                // reference: 60
        req = (self + 27) >> 5;
    else
        req = (self + 31) >> 5;
    const int sms = min(req * kSmsTaskParticles, self);
    return make_int4(req, sms, self - sms, 0);
}

__device__ __forceinline__ int4 add4(int4 a, int4 b) {
    return make_int4(a.x + b.x, a.y + b.y, a.z + b.z, a.w + b.w);
}
__device__ __forceinline__ int4 shfl_up4(int4 v, int o) {
    return make_int4(__shfl_up_sync(kFull, v.x, o), __shfl_up_sync(kFull, v.y, o),
                     __shfl_up_sync(kFull, v.z, o), __shfl_up_sync(kFull, v.w, o));
}
__device__ __forceinline__ int4 shfl_down4(int4 v, int o) {
    return make_int4(__shfl_down_sync(kFull, v.x, o),
                     __shfl_down_sync(kFull, v.y, o),
                     __shfl_down_sync(kFull, v.z, o),
                     __shfl_down_sync(kFull, v.w, o));
}

// Exclusive scan, in place, of the int4 tile sums by one block; returns the
// grand total. The tiles were written by other CTAs of the same launch, so
// they are read from L2.
__device__ int4 scan_val_tiles(int4 *tiles, int ntiles) {
    __shared__ int4 ws[32];
    __shared__ int4 carry;
    if (threadIdx.x == 0) carry = make_int4(0, 0, 0, 0);
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = int(blockDim.x >> 5);
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        const int4 v = t < ntiles ? __ldcg(tiles + t) : make_int4(0, 0, 0, 0);
        int4 x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            int4 y = shfl_up4(x, o);
            if (lane >= o) x = add4(x, y);
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            int4 w = lane < nw ? ws[lane] : make_int4(0, 0, 0, 0);
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                int4 y = shfl_up4(w, o);
                if (lane >= o) w = add4(w, y);
            }
            if (lane < nw) ws[lane] = w;
        }
        __syncthreads();
        const int4 wprefix = warp > 0 ? ws[warp - 1] : make_int4(0, 0, 0, 0);
        int4 excl = add4(carry, wprefix);
        excl = make_int4(excl.x + x.x - v.x, excl.y + x.y - v.y, excl.z + x.z - v.z, 0);
        if (t < ntiles) tiles[t] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = add4(excl, v);
        __syncthreads();
    }
    return carry;
}

// A6 + the reduction of A7: the performance model of every occupied cell
// ({req, sms, tra} per cell, kValTile cells per tile) and each tile's sum.
// The last CTA to finish (a counter, no waiting) scans the tile sums and
// sets the task count, the SMS particle count and the middle value; in a
// frame where no cell takes the SMS path it only records that.
__global__ void __launch_bounds__(kScanThreads)
k_cell_model(const int32_t *__restrict__ occ, Counters *ctr,
             const int32_t *__restrict__ start, SceneTable T, int3 thr,
             int4 *__restrict__ val, int4 *__restrict__ tiles, int task_capacity,
             int n_particles) {
    const int n = ctr->num_occ;
    __shared__ int4 ws[kScanThreads / 32];
    __shared__ bool last;
    bool any = false;
    for (int tile = blockIdx.x; tile * kValTile < n; tile += gridDim.x) {
        const int first = tile * kValTile + threadIdx.x;
        int4 s = make_int4(0, 0, 0, 0);
        // consecutive threads take consecutive cells (coalesced)
#pragma unroll
        for (int q = 0; q < kValItems; ++q) {
            const int k = first + q * kScanThreads;
            if (k < n) {
                const int4 v = cell_model(occ[k], start, T, thr);
                val[k] = v;
                any |= v.x > 0;
                s = add4(s, v);
            }
        }
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) s = add4(s, shfl_down4(s, o));
        if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
        __syncthreads();
        if (threadIdx.x == 0) {
            int4 t = make_int4(0, 0, 0, 0);
            for (int w = 0; w < kScanThreads / 32; ++w) t = add4(t, ws[w]);
            tiles[tile] = t;
        }
        __syncthreads();
    }
    if (__any_sync(kFull, any) && (threadIdx.x & 31) == 0) atomicOr(&ctr->any_sms, 1);
    __syncthreads();
    if (threadIdx.x == 0) {
        __threadfence();
        last = atomicAdd(&ctr->model_done, 1) == int(gridDim.x) - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const bool sms = atomicAdd(&ctr->any_sms, 0) != 0;
    if (!sms) {   // all TRA: nothing to compact
        if (threadIdx.x == 0) {
            ctr->task_count = 0;
            ctr->n_sms = 0;
            ctr->middle = n_particles;
            ctr->model_done = 0;
        }
        return;
    }
    const int4 total = scan_val_tiles(tiles, (n + kValTile - 1) / kValTile);
    if (threadIdx.x == 0) {
        int tasks = total.x;
        if (tasks + 1 > task_capacity) {   // +1: odd-tail descriptor
            atomicOr(&ctr->err, kErrTaskCapacity);
            tasks = task_capacity - 1;
        }
        ctr->task_count = tasks;
        ctr->n_sms = total.y;
        ctr->middle = total.z;
        ctr->model_done = 0;
    }
}

__global__ void __launch_bounds__(kScanThreads)
k_val_scan_apply(const int4 *__restrict__ in, const Counters *ctr,
                 const int4 *__restrict__ tiles, int4 *__restrict__ out) {
    if (!ctr->any_sms) return;
    const int n = ctr->num_occ;
    __shared__ int4 ws[kScanThreads / 32];
    for (int tile = blockIdx.x; tile * kValTile < n; tile += gridDim.x) {
    const int first = tile * kValTile + threadIdx.x * kValItems;
    int4 v[kValItems];
    int4 s = make_int4(0, 0, 0, 0);
#pragma unroll
    for (int q = 0; q < kValItems; ++q) {
        v[q] = (first + q < n) ? in[first + q] : make_int4(0, 0, 0, 0);
        s = add4(s, v[q]);
    }
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    int4 x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        int4 y = shfl_up4(x, o);
        if (lane >= o) x = add4(x, y);
    }
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    int4 run = tiles[tile];
    for (int w = 0; w < warp; ++w) run = add4(run, ws[w]);
    run = make_int4(run.x + x.x - s.x, run.y + x.y - s.y, run.z + x.z - s.z, 0);
#pragma unroll
    for (int q = 0; q < kValItems; ++q) {
        if (first + q < n) out[first + q] = run;
        run = add4(run, v[q]);
    }
    __syncthreads();
    }
}

__host__ __device__ __forceinline__ uint16_t pack_bounds(int min_x, int max_x,
                                                         int min_y, int max_y,
                                                         int min_z, int max_z) {
    // packSmsTaskBounds, particle/particle_buffer.h:89-95
    return uint16_t(min_x | (max_x << 2) | (min_y << 4) | (max_y << 6) |
                    (min_z << 8) | (max_z << 10));
}

// A7/A8: compact index and task descriptors of each occupied cell.
__global__ void __launch_bounds__(128)
k_cell_emit(const int32_t *__restrict__ occ, Counters *ctr,
            const int32_t *__restrict__ start, const uint32_t *__restrict__ key,
            const int4 *__restrict__ val, const int4 *__restrict__ prefix,
            SceneTable T, int32_t *__restrict__ compact,
            gsph_block_task *__restrict__ tasks) {
    if (!ctr->any_sms) return;   // all TRA: the compact index is the identity
    const int num_occ = ctr->num_occ;
    for (int k = blockIdx.x * blockDim.x + threadIdx.x; k < num_occ;
         k += gridDim.x * blockDim.x) {
    const int cell = occ[k];
    const int b = start[cell];
    const int n = start[cell + 1] - b;
    const int4 v = val[k];
    const int4 pre = prefix[k];
    const int middle = ctr->middle;
    const int task_count = ctr->task_count;
    for (int j = 0; j < v.z; ++j) compact[pre.z + j] = b + v.y + j;
    for (int j = 0; j < v.y; ++j) compact[middle + pre.y + j] = b + j;
    if (v.x == 0) continue;
    const SceneGeom G = geom_of_cell(T, cell);
    const int local = cell - G.cbase;
    const uint16_t cx = uint16_t(local % G.gx);
    const uint16_t cy = uint16_t(local / G.gx % G.gy);
    const uint16_t cz = uint16_t(local / G.gx / G.gy);
    for (int t = 0; t < v.x; ++t) {
        const int ti = pre.x + t;
        if (ti >= task_count) break;   // capacity guard (error already raised)
        const int off = t * kSmsTaskParticles;
        if (off >= kTaskOffsetLimit) {   // a cell beyond 2^24 particles
            atomicOr(&ctr->err, kErrTaskCapacity);
            break;
        }
        const uint32_t first_hash = key[b + off];
        const uint32_t last_hash = key[b + min(off + kSmsTaskParticles - 1, n - 1)];
        const int min_x = (first_hash >> 4) & 3, max_x = (last_hash >> 4) & 3;
        const int min_z = (first_hash >> 2) & 3, max_z = (last_hash >> 2) & 3;
        const int min_y = first_hash & 3, max_y = last_hash & 3;
        gsph_block_task task;
        task.is_same = 0;
        task.cellid = cell;
        task.cell_pos[0] = cx;
        task.cell_pos[1] = cy;
        task.cell_pos[2] = cz;
        set_task_offset(task, off);
        task.cell_begin = b;
        task.cell_particle_count = n;
        task.xxi = int8_t(min_x);
        task.xxx = int8_t(max_x);
        if (min_x == max_x) {
            task.zzi = int8_t(min_z);
            task.zzz = int8_t(max_z);
            if (min_z == max_z) {
                task.yyi = int8_t(min_y);
                task.yyy = int8_t(max_y);
            } else {
                task.yyi = 0;
                task.yyy = 3;
            }
        } else {
            task.zzi = 0;
            task.zzz = 3;
            task.yyi = 0;
            task.yyy = 3;
        }
        task.paired_bounds =
            pack_bounds(task.xxi, task.xxx, task.yyi, task.yyy, task.zzi, task.zzz);
        tasks[ti] = task;
    }
    }
}

// One pair (first, first + 1) of the historical same-cell pairing.
__device__ __forceinline__ void judge_pair(gsph_block_task *__restrict__ tasks,
                                           int first, int task_count) {
    const int second = first + 1;
    gsph_block_task a = tasks[first];
    if (second >= task_count) {
        // Odd tail (sph_arrangement.cu:976-991): a fabricated descriptor of
        // the next 32 particles of the same cell. Fields the reference leaves
        // stale are copied from the last task here.
        gsph_block_task t = a;
        a.is_same = 1;
        t.is_same = 1;
        set_task_offset(t, task_offset(a) + kSmsTaskParticles);
        tasks[first] = a;
        tasks[second] = t;
        return;
    }
    gsph_block_task b = tasks[second];
    if (a.cellid != b.cellid) {
        tasks[first].is_same = 0;
        tasks[second].is_same = 0;
        return;
    }
    int pmin_z = a.zzi, pmax_z = a.zzz;
    if (a.xxi == b.xxx) {
        pmax_z = b.zzz;
    } else {
        pmin_z = 0;
        pmax_z = 3;
    }
    tasks[first].is_same = 1;
    tasks[second].is_same = 1;
    tasks[first].paired_bounds =
        pack_bounds(a.xxi, b.xxx, a.yyi, a.yyy, pmin_z, pmax_z);
}

// A9: historical same-cell pairing of tasks (2k, 2k+1), odd-tail descriptor.
__global__ void __launch_bounds__(128)
k_judge(gsph_block_task *__restrict__ tasks, const Counters *ctr) {
    const int task_count = ctr->task_count;
    for (int pair = blockIdx.x * blockDim.x + threadIdx.x; (pair << 1) < task_count;
         pair += gridDim.x * blockDim.x)
        judge_pair(tasks, pair << 1, task_count);
}}  // namespace

void launch_split(const Frame &f, const DevParams &P, int max_occ, int num_sms,
                  cudaStream_t s) {
    if (f.n <= 0 || max_occ <= 0) return;
    // grid-stride kernels over the device-side counts, sized for the capacity
    // but at most a few CTAs per SM
    const int cap128 = std::min((max_occ + 127) / 128, num_sms * 16);
    const int ntiles = std::min((max_occ + kValTile - 1) / kValTile, num_sms * 8);
    k_cell_model<<<ntiles, kScanThreads, 0, s>>>(
        f.occ_list, f.ctr, f.cell_start, f.scenes,
        make_int3(P.sparse_total, P.sparse_self, P.mid_total), f.cell_val, f.scan_tiles4,
        f.task_capacity, f.n);
    k_val_scan_apply<<<ntiles, kScanThreads, 0, s>>>(f.cell_val, f.ctr,
                                                    f.scan_tiles4, f.cell_prefix);
    k_cell_emit<<<cap128, 128, 0, s>>>(
        f.occ_list, f.ctr, f.cell_start, f.key, f.cell_val, f.cell_prefix,
        f.scenes, f.compact, f.tasks);
}

void launch_judge(const Frame &f, int max_occ, int num_sms, cudaStream_t s) {
    if (f.n <= 0 || max_occ <= 0) return;   // as launch_split: no tasks made
    const int max_pairs = (f.task_capacity + 1) / 2;
    k_judge<<<std::min((max_pairs + 127) / 128, num_sms * 8), 128, 0, s>>>(f.tasks,
                                                                          f.ctr);
}

}  // namespace gsph
