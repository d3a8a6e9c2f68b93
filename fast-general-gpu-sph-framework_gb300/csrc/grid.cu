// grid.cu — uniform-grid hash and deterministic counting sort (arrange stage,
// rows A2-A5 of the hot path).
//
// Reference behaviour (KemengHuang/Fast-General-GPU-SPH-framework):
//   micro key      src/core/sph_utils.cuh:44-99  (ParticlePos2CellPosM,
//                  CellPos2CellIdxM): key = (cell << 6) | (mx << 4) | (mz << 2) | my
//   count          src/grid/sph_arrangement.cu:1331-1341 (CountingSort_Cell_SumM)
//   offsets        src/grid/sph_arrangement.cu:1370-1371 (CUB ExclusiveSum over
//                  a dense numc*64+1 micro table)
//   reorder        src/grid/sph_arrangement.cu:1309-1330 (CountingSort_Result_M)
//   cell info      src/grid/sph_arrangement.cu:1342-1351 (calculate_cell_info)
//
// Design here (not a translation):
//   * counting is per COARSE cell (numc ints, not numc*64), with warp-aggregated
//     atomics (match.any) so a warp of sorted particles issues one atomic per
//     cell it touches;
//   * the coarse scan is reduce-then-scan (no inter-CTA spin waits) and also
//     compacts the occupied cells and the list of large cells;
//   * the order inside a coarse cell is canonical: (micro key, previous index).
//     The reference's atomic slot order varies run to run; this one does not,
//     so two runs (and the CPU restatement) give the same permutation;
//   * per cell, the three micro-x slab boundaries are kept (10 bits each) in
//     place of the dense micro table; stale entries of empty cells are harmless
//     because every use clamps them by the cell's count.
#include <algorithm>

#include "gsph_internal.h"

namespace gsph {

namespace {

constexpr unsigned kFull = 0xFFFFFFFFu;

// ---------------------------------------------------------------------------
// A2: key + per-coarse-cell slot (warp-aggregated atomics).
__global__ void __launch_bounds__(256)
k_hash_count(const float4 *__restrict__ pos, int n, DevParams P, SceneTable T,
             uint32_t *__restrict__ key_out, uint32_t *__restrict__ slot_out,
             int32_t *__restrict__ cell_count, Counters *ctr) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const bool valid = i < n;
    const unsigned active = __ballot_sync(kFull, valid);
    if (!valid) return;
    const SceneGeom G = geom_of_particle(T, i);
    const uint32_t key = micro_key(pos[i], P, G, ctr, i);
    key_out[i] = key;
    slot_out[i] = cell_slot(cell_count, key >> 6, active);
}

// The particles the split sent to SMS tasks (compact[middle, n)), hashed
// ahead from their integrated positions after the SMS force pass (the TRA
// force pass hashes its own particles).
__global__ void __launch_bounds__(256)
k_hash_sms(const float4 *__restrict__ pos, int n, DevParams P, SceneTable T,
           const int32_t *__restrict__ compact, uint32_t *__restrict__ key_out,
           uint32_t *__restrict__ slot_out, int32_t *__restrict__ cell_count,
           Counters *ctr) {
    const int middle = ctr->middle;
    const int lane = threadIdx.x & 31;
    const int warp = (blockIdx.x * blockDim.x + threadIdx.x) >> 5;
    const int warps = (gridDim.x * blockDim.x) >> 5;
    // warp-uniform loop: every lane of a warp sees the same base
    for (int base = middle + warp * 32; base < n; base += warps * 32) {
        const int k = base + lane;
        const bool valid = k < n;
        const unsigned active = __ballot_sync(kFull, valid);
        if (valid) {
            const int i = compact[k];
            const SceneGeom G = geom_of_particle(T, i);
            const uint32_t key = micro_key(pos[i], P, G, ctr, i);
            key_out[i] = key;
            slot_out[i] = cell_slot(cell_count, key >> 6, active);
        }
    }
}

// ---------------------------------------------------------------------------
// A3/A5: reduce-then-scan over the coarse counts. Values are packed
// (occupied << 32) | count so one scan yields the cell offsets and the
// occupied-cell compaction.
__device__ __forceinline__ unsigned long long pack_cell(int cnt) {
    return (cnt > 0 ? (1ull << 32) : 0ull) | (unsigned long long)(unsigned)cnt;
}

__device__ __forceinline__ void load_tile_counts(const int32_t *__restrict__ in,
                                                 int n, int first,
                                                 int (&v)[kScanItems]) {
    if (first + kScanItems <= n) {
        const int4 *p4 = reinterpret_cast<const int4 *>(in + first);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q) {
            int4 t = p4[q];
            v[4 * q + 0] = t.x;
            v[4 * q + 1] = t.y;
            v[4 * q + 2] = t.z;
            v[4 * q + 3] = t.w;
        }
    } else {
#pragma unroll
        for (int q = 0; q < kScanItems; ++q)
            v[q] = (first + q < n) ? in[first + q] : 0;
    }
}

// Exclusive scan of the packed tile sums by one block (any multiple of 32
// threads), in place; returns the grand total to thread 0. The tiles were
// written by other CTAs of the same launch, so they are read from L2.
__device__ unsigned long long scan_tile_sums(unsigned long long *tiles, int ntiles) {
    __shared__ unsigned long long ws[32];
    __shared__ unsigned long long carry;
    if (threadIdx.x == 0) carry = 0;
    __syncthreads();
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int nw = int(blockDim.x >> 5);
    for (int base = 0; base < ntiles; base += blockDim.x) {
        const int t = base + threadIdx.x;
        const unsigned long long v = t < ntiles ? __ldcg(tiles + t) : 0ull;
        unsigned long long x = v;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            unsigned long long y = __shfl_up_sync(kFull, x, o);
            if (lane >= o) x += y;
        }
        if (lane == 31) ws[warp] = x;
        __syncthreads();
        if (warp == 0) {
            unsigned long long w = lane < nw ? ws[lane] : 0ull;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                unsigned long long y = __shfl_up_sync(kFull, w, o);
                if (lane >= o) w += y;
            }
            if (lane < nw) ws[lane] = w;
        }
        __syncthreads();
        const unsigned long long wprefix = warp > 0 ? ws[warp - 1] : 0ull;
        const unsigned long long excl = carry + wprefix + x - v;
        if (t < ntiles) tiles[t] = excl;
        __syncthreads();
        if (threadIdx.x == blockDim.x - 1) carry = excl + v;
        __syncthreads();
    }
    return carry;
}

// Tile sums of the packed (occupied, count) values; the last CTA to finish
// (a counter, no waiting) scans the tile sums, writes the grand total and
// resets the frame's work counters.
__global__ void __launch_bounds__(kScanThreads)
k_cell_scan_reduce(const int32_t *__restrict__ count, int numc,
                   unsigned long long *__restrict__ tiles, int32_t *__restrict__ cell_start,
                   Counters *ctr) {
    const int first = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    load_tile_counts(count, numc, first, v);
    unsigned long long s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) s += pack_cell(v[q]);
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) s += __shfl_down_sync(kFull, s, o);
    __shared__ unsigned long long ws[kScanThreads / 32];
    __shared__ bool last;
    if ((threadIdx.x & 31) == 0) ws[threadIdx.x >> 5] = s;
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long t = 0;
        for (int w = 0; w < kScanThreads / 32; ++w) t += ws[w];
        tiles[blockIdx.x] = t;
        __threadfence();
        last = atomicAdd(&ctr->scan_done, 1) == int(gridDim.x) - 1;
    }
    __syncthreads();
    if (!last) return;
    __threadfence();
    const unsigned long long total = scan_tile_sums(tiles, int(gridDim.x));
    if (threadIdx.x == 0) {
        cell_start[numc] = int32_t(total & 0xFFFFFFFFull);
        ctr->num_occ = int32_t(total >> 32);
        ctr->num_big = 0;
        ctr->work_density = 0;
        ctr->work_force = 0;
        ctr->work_density_sms = 0;
        ctr->work_force_sms = 0;
        ctr->any_sms = 0;
        ctr->scan_done = 0;
    }
}

__global__ void __launch_bounds__(kScanThreads)
k_cell_scan_apply(const int32_t *__restrict__ count, int numc,
                  const unsigned long long *__restrict__ tiles,
                  int32_t *__restrict__ cell_start,
                  int32_t *__restrict__ occ_list,
                  int32_t *__restrict__ big_list, Counters *ctr) {
    const int first = blockIdx.x * kScanTile + threadIdx.x * kScanItems;
    int v[kScanItems];
    load_tile_counts(count, numc, first, v);
    unsigned long long s = 0;
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) s += pack_cell(v[q]);
    // block exclusive scan of per-thread sums
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    unsigned long long x = s;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned long long y = __shfl_up_sync(kFull, x, o);
        if (lane >= o) x += y;
    }
    __shared__ unsigned long long ws[kScanThreads / 32];
    if (lane == 31) ws[warp] = x;
    __syncthreads();
    unsigned long long wprefix = 0;
    for (int w = 0; w < warp; ++w) wprefix += ws[w];
    unsigned long long run = tiles[blockIdx.x] + wprefix + x - s;
    int out[kScanItems];
#pragma unroll
    for (int q = 0; q < kScanItems; ++q) {
        const int c = first + q;
        out[q] = int32_t(run & 0xFFFFFFFFull);
        if (c < numc && v[q] > 0) {
            occ_list[run >> 32] = c;
            if (v[q] > kSmallCellMax) big_list[atomicAdd(&ctr->num_big, 1)] = c;
        }
        run += pack_cell(v[q]);
    }
    if (first + kScanItems <= numc) {
        // a thread's cells are contiguous: 16-byte stores
        int4 *dst = reinterpret_cast<int4 *>(cell_start + first);
#pragma unroll
        for (int q = 0; q < kScanItems / 4; ++q)
            dst[q] = make_int4(out[4 * q], out[4 * q + 1], out[4 * q + 2], out[4 * q + 3]);
    } else {
#pragma unroll
        for (int q = 0; q < kScanItems; ++q)
            if (first + q < numc) cell_start[first + q] = out[q];
    }
}

// ---------------------------------------------------------------------------
// Scatter (key, source) pairs to their coarse-cell range (slot order).
__global__ void __launch_bounds__(256)
k_scatter_pairs(const uint32_t *__restrict__ key_in,
                const uint32_t *__restrict__ slot, int n,
                const int32_t *__restrict__ cell_start,
                unsigned long long *__restrict__ pairs) {
    // two particles per thread, a block-width apart: both chains of loads
    // are in flight together
    const int i0 = blockIdx.x * (2 * blockDim.x) + threadIdx.x;
    const int i1 = i0 + blockDim.x;
    uint32_t k0 = 0, k1 = 0, s0 = 0, s1 = 0;
    if (i0 < n) { k0 = key_in[i0]; s0 = slot[i0]; }
    if (i1 < n) { k1 = key_in[i1]; s1 = slot[i1]; }
    int c0 = 0, c1 = 0;
    if (i0 < n) c0 = cell_start[k0 >> 6];
    if (i1 < n) c1 = cell_start[k1 >> 6];
    if (i0 < n) pairs[c0 + int(s0)] = ((unsigned long long)k0 << 32) | (unsigned)i0;
    if (i1 < n) pairs[c1 + int(s1)] = ((unsigned long long)k1 << 32) | (unsigned)i1;
}

__device__ __forceinline__ uint32_t pack_xslab(int s1, int s2, int s3, int cnt) {
    if (cnt > 1023) return kXslabUnknown;
    return uint32_t(s1) | (uint32_t(s2) << 10) | (uint32_t(s3) << 20);
}

// Writes the 16 (micro-x, micro-z) group offsets of a cell from its group
// counts, and the three micro-x slab boundaries derived from them.
__device__ __forceinline__ void write_groups(const Frame &f, uint32_t cell,
                                             const int (&n16)[16], int cnt) {
    int off[17];
    off[0] = 0;
#pragma unroll
    for (int g = 0; g < 16; ++g) off[g + 1] = off[g] + n16[g];
    f.cell_xslab[cell] = pack_xslab(off[4], off[8], off[12], cnt);
    if (!f.cell_grp) return;
    uint32_t w[8];
#pragma unroll
    for (int k = 0; k < 8; ++k)
        w[k] = uint32_t(off[2 * k] & 0xFFFF) | (uint32_t(off[2 * k + 1] & 0xFFFF) << 16);
    if (cnt > 65535) w[0] = (w[0] & 0xFFFF0000u) | kGroupsUnknown;
    uint4 *dst = reinterpret_cast<uint4 *>(f.cell_grp + size_t(cell) * 16);
    dst[0] = make_uint4(w[0], w[1], w[2], w[3]);
    dst[1] = make_uint4(w[4], w[5], w[6], w[7]);
}

__device__ __forceinline__ void move_particle(const Frame &f, int dst,
                                              unsigned long long e) {
    const int src = int(e & 0xFFFFFFFFull);
    f.key[dst] = uint32_t(e >> 32);
    f.perm[dst] = src;
    f.pos[dst] = f.pos_in[src];
    f.vel[dst] = f.vel_in[src];
    f.ev[dst] = f.ev_in[src];
}

// Group offsets and slab words of a small cell, written by the thread of the
// cell's first particle, which also clears the cell's count.
__device__ __forceinline__ void small_cell_groups(const Frame &f, uint32_t cell, int b,
                                                  int cnt) {
    // group counts, 8 bits each (cnt <= 32), packed in two words
    unsigned long long lo = 0, hi = 0;
    for (int j = 0; j < cnt; ++j) {
        const int g = int((f.pairs[b + j] >> 34) & 15ull);
        if (g < 8)
            lo += 1ull << (8 * g);
        else
            hi += 1ull << (8 * (g - 8));
    }
    int n16[16];
#pragma unroll
    for (int g = 0; g < 8; ++g) {
        n16[g] = int((lo >> (8 * g)) & 0xFF);
        n16[g + 8] = int((hi >> (8 * g)) & 0xFF);
    }
    write_groups(f, cell, n16, cnt);
    f.cell_count[cell] = 0;   // ready for the next frame's atomics
}

// Cells with at most kSmallCellMax particles: one thread per particle ranks
// its pair among the cell's pairs (all distinct: sources are unique). Each
// thread takes two particles a block-width apart and issues both particles'
// loads (pair, cell bounds, state, the cell's pairs) before any store, so
// that the two chains of loads are in flight together.
__global__ void __launch_bounds__(256) k_sort_small(Frame f) {
    int s[2];
    s[0] = blockIdx.x * (2 * blockDim.x) + threadIdx.x;
    s[1] = s[0] + blockDim.x;
    unsigned long long e[2] = {0ull, 0ull};
    int b[2] = {0, 0}, cnt[2] = {0, 0}, rank[2] = {0, 0};
    bool live[2];
    float4 pos[2], vel[2], ev[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        live[k] = s[k] < f.n;
        if (live[k]) e[k] = f.pairs[s[k]];
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (live[k]) {
            const uint32_t cell = uint32_t(e[k] >> 38);
            b[k] = f.cell_start[cell];
            cnt[k] = f.cell_start[cell + 1] - b[k];
            live[k] = cnt[k] <= kSmallCellMax;
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (live[k]) {
            const int src = int(e[k] & 0xFFFFFFFFull);
            pos[k] = f.pos_in[src];
            vel[k] = f.vel_in[src];
            ev[k] = f.ev_in[src];
        }
    }
#pragma unroll
    for (int k = 0; k < 2; ++k)
        if (live[k])
            for (int j = 0; j < cnt[k]; ++j) rank[k] += (f.pairs[b[k] + j] < e[k]) ? 1 : 0;
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        if (!live[k]) continue;
        const int dst = b[k] + rank[k];
        f.key[dst] = uint32_t(e[k] >> 32);
        f.perm[dst] = int(e[k] & 0xFFFFFFFFull);
        f.pos[dst] = pos[k];
        f.vel[dst] = vel[k];
        f.ev[dst] = ev[k];
        if (rank[k] == 0) small_cell_groups(f, uint32_t(e[k] >> 38), b[k], cnt[k]);
    }
}

// Buckets of the block-level sort past kBigCellSmem particles: 64 micro
// cells x kSrcBuckets source-index ranges; counts and starts fit in the
// shared staging array.
constexpr int kSrcBuckets = 32;
constexpr int kBuckets = 64 * kSrcBuckets;
static_assert((2 * kBuckets + 1) * sizeof(int) <= kBigCellSmem * sizeof(unsigned long long),
              "bucket tables must fit in the staging array");

// Exclusive scan of in[0, n) into out[0, n] (out[n] = total) by the whole
// block (blockDim.x = 256, n a multiple of 256). Ends with __syncthreads.
__device__ void block_exclusive_scan(const int *in, int *out, int n) {
    __shared__ int warp_sum[8];
    __shared__ int carry;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int per = n / blockDim.x;          // items per thread, contiguous
    const int first = threadIdx.x * per;
    int sum = 0;
    for (int q = 0; q < per; ++q) sum += in[first + q];
    int x = sum;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
        if (lane >= o) x += y;
    }
    if (lane == 31) warp_sum[warp] = x;
    __syncthreads();
    if (threadIdx.x == 0) {
        int run = 0;
        for (int w = 0; w < int(blockDim.x >> 5); ++w) {
            const int v = warp_sum[w];
            warp_sum[w] = run;
            run += v;
        }
        carry = run;
    }
    __syncthreads();
    int run = warp_sum[warp] + x - sum;
    for (int q = 0; q < per; ++q) {
        out[first + q] = run;
        run += in[first + q];
    }
    if (threadIdx.x == 0) out[n] = carry;
    __syncthreads();
}

// Cells with more than kSmallCellMax particles: one CTA per cell. Pairs
// compare as (micro cell, source index) inside a cell, so up to kBigCellSmem
// particles the pairs are staged in shared memory, bucketed by their 6-bit
// micro cell (counts, scan, scatter) and ranked by value inside their bucket
// only. Larger cells do the same in global memory with finer buckets.
__global__ void __launch_bounds__(256) k_sort_big(Frame f) {
    __shared__ unsigned long long sp[kBigCellSmem];
    __shared__ uint16_t order[kBigCellSmem];
    __shared__ int mcount[64], mfill[64], mstart[65];
    __shared__ int grp[16];
    const int nbig = f.ctr->num_big;
    for (int q = blockIdx.x; q < nbig; q += gridDim.x) {
        const int cell = f.big_list[q];
        const int b = f.cell_start[cell];
        const int cnt = f.cell_start[cell + 1] - b;
        if (cnt <= kBigCellSmem) {
            if (threadIdx.x < 64) {
                mcount[threadIdx.x] = 0;
                mfill[threadIdx.x] = 0;
            }
            for (int j = threadIdx.x; j < cnt; j += blockDim.x) sp[j] = f.pairs[b + j];
            __syncthreads();
            for (int j = threadIdx.x; j < cnt; j += blockDim.x)
                atomicAdd(&mcount[int((sp[j] >> 32) & 63ull)], 1);
            __syncthreads();
            if (threadIdx.x < 32) {   // exclusive scan of the 64 counts
                const int l = threadIdx.x;
                const int c0 = mcount[2 * l], c1 = mcount[2 * l + 1];
                int x = c0 + c1;
#pragma unroll
                for (int o = 1; o < 32; o <<= 1) {
                    const int y = __shfl_up_sync(0xFFFFFFFFu, x, o);
                    if (l >= o) x += y;
                }
                const int excl = x - c0 - c1;
                mstart[2 * l] = excl;
                mstart[2 * l + 1] = excl + c0;
                if (l == 31) mstart[64] = x;
            }
            __syncthreads();
            for (int j = threadIdx.x; j < cnt; j += blockDim.x) {
                const int m = int((sp[j] >> 32) & 63ull);
                order[mstart[m] + atomicAdd(&mfill[m], 1)] = uint16_t(j);
            }
            __syncthreads();
            for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
                const unsigned long long e = sp[order[t]];
                const int m = int((e >> 32) & 63ull);
                int rank = mstart[m];
                for (int k = mstart[m]; k < mstart[m + 1]; ++k)
                    rank += (sp[order[k]] < e) ? 1 : 0;
                move_particle(f, b + rank, e);
            }
            if (threadIdx.x == 0) {
                int n16[16];
#pragma unroll
                for (int g = 0; g < 16; ++g)
                    n16[g] = mcount[4 * g] + mcount[4 * g + 1] + mcount[4 * g + 2] +
                             mcount[4 * g + 3];
                write_groups(f, uint32_t(cell), n16, cnt);
                f.cell_count[cell] = 0;
            }
            __syncthreads();
            continue;
        }
        // Past kBigCellSmem particles: bucket the cell's pairs by (micro
        // cell, source index scaled into kSrcBuckets ranges) — an order-
        // preserving bucket of (micro key, source) — with counts and a scan in
        // shared memory (over the staging array) and the bucketed order in
        // the cell's own range of f.slot (free during the sort: the hash that
        // fills it ran before the scatter), then rank each pair inside its
        // bucket only.
        if (threadIdx.x < 16) grp[threadIdx.x] = 0;
        int *bcount = reinterpret_cast<int *>(sp);          // [kBuckets]
        int *bstart = bcount + kBuckets;                     // [kBuckets + 1]
        for (int k = threadIdx.x; k < kBuckets; k += blockDim.x) bcount[k] = 0;
        __syncthreads();
        const unsigned long long *src = f.pairs + b;
        const unsigned long long nsrc = (unsigned long long)f.n;
        auto bucket_of = [&](unsigned long long e) {
            const int micro = int((e >> 32) & 63ull);
            const int sub = int(((e & 0xFFFFFFFFull) * kSrcBuckets) / nsrc);
            return micro * kSrcBuckets + sub;
        };
        for (int i = threadIdx.x; i < cnt; i += blockDim.x)
            atomicAdd(&bcount[bucket_of(src[i])], 1);
        __syncthreads();
        block_exclusive_scan(bcount, bstart, kBuckets);   // bstart[kBuckets] = cnt
        for (int k = threadIdx.x; k < kBuckets; k += blockDim.x) bcount[k] = 0;
        __syncthreads();
        uint32_t *order_g = f.slot + b;
        for (int i = threadIdx.x; i < cnt; i += blockDim.x) {
            const int k = bucket_of(src[i]);
            order_g[bstart[k] + atomicAdd(&bcount[k], 1)] = uint32_t(i);
        }
        __syncthreads();
        for (int t = threadIdx.x; t < cnt; t += blockDim.x) {
            const unsigned long long e = src[order_g[t]];
            const int k = bucket_of(e);
            int rank = bstart[k];
            for (int q = bstart[k]; q < bstart[k + 1]; ++q)
                rank += (src[order_g[q]] < e) ? 1 : 0;
            move_particle(f, b + rank, e);
            atomicAdd(&grp[int((e >> 34) & 15ull)], 1);
        }
        __syncthreads();
        if (threadIdx.x == 0) {
            int n16[16];
#pragma unroll
            for (int g = 0; g < 16; ++g) n16[g] = grp[g];
            write_groups(f, uint32_t(cell), n16, cnt);
            f.cell_count[cell] = 0;
        }
        __syncthreads();
    }
}

}  // namespace

void launch_hash_sms(const Frame &f, const float4 *pos, const DevParams &P,
                     cudaStream_t s) {
    if (f.n <= 0) return;
    k_hash_sms<<<std::min((f.n + 255) / 256, 4096), 256, 0, s>>>(
        pos, f.n, P, f.scenes, f.compact, f.key_in, f.slot, f.cell_count, f.ctr);
}

void launch_hash_count(const Frame &f, const DevParams &P, cudaStream_t s) {
    if (f.n <= 0) return;
    k_hash_count<<<(f.n + 255) / 256, 256, 0, s>>>(f.pos_in, f.n, P, f.scenes,
                                                  f.key_in, f.slot, f.cell_count,
                                                  f.ctr);
}

void launch_cell_scan(const Frame &f, const DevParams &P, cudaStream_t s) {
    const int ntiles = (P.numc + kScanTile - 1) / kScanTile;
    k_cell_scan_reduce<<<ntiles, kScanThreads, 0, s>>>(f.cell_count, P.numc,
                                                       f.scan_tiles, f.cell_start, f.ctr);
    k_cell_scan_apply<<<ntiles, kScanThreads, 0, s>>>(
        f.cell_count, P.numc, f.scan_tiles, f.cell_start, f.occ_list,
        f.big_list, f.ctr);
}

void launch_scatter_pairs(const Frame &f, cudaStream_t s) {
    if (f.n <= 0) return;
    k_scatter_pairs<<<(f.n + 511) / 512, 256, 0, s>>>(f.key_in, f.slot, f.n,
                                                     f.cell_start, f.pairs);
}

void launch_cell_sort(const Frame &f, int num_sms, cudaStream_t s) {
    if (f.n <= 0) return;
    k_sort_small<<<(f.n + 511) / 512, 256, 0, s>>>(f);
    k_sort_big<<<num_sms * 4, 256, 0, s>>>(f);
}

}  // namespace gsph
