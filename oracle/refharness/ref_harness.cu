// ref_harness.cu — runs the reference's own CUDA kernels on the GPU.
//
// TEST INFRASTRUCTURE ONLY: a checker used to record golden fixtures and to
// time the reference's path on the same GPU. It is never linked into or called
// by the product.
//
// The kernels come from the device image oracle/_ref/ref_device.cubin, built
// from the reference's unmodified sources (ref_device.cu). This program is the
// host side the reference cannot be compiled with here (it needs jsoncpp and
// Windows timers): it reproduces, call for call, the launches of
//   Arrangement::arrangeHybridFrame  src/grid/sph_arrangement.cu:1352-1506
//     (CountingSort_O_M, gpu_model::calculateBlockRequirementHybridMode,
//      CountingSortCUDA_Two9_M, the task scan, arrangeSmsTasks + judgeTask)
//   computeDensityHybrid / computeForceHybrid  src/solver/kernel_dispatch.cu:182-253
//   advance                                   src/solver/kernel_dispatch.cu:314-323
//   HybridSystem::tick / runBenchmark         src/simulation/sph_hybrid_system.cpp:253-430
// with the same grid shapes, the same per-frame host synchronisation and the
// same buffer aliasing (the sort's temporary buffer shares acceleration and
// final_position with the main one, particle_buffer.cpp:137-162). Scans use
// CUB's DeviceScan as the reference does.
//
// Usage:
//   ref_harness <cubin> tick  <input.bin> <out_dir>
//   ref_harness <cubin> bench <input.bin> <frames>
//   ref_harness <cubin> run   <input.bin> <frames> <out_dir>
// input.bin: "GSPHREF1", gsph_params, int32 n, float4 pos[n], float4 vel[n],
// float4 ev[n]. tick writes raw arrays + meta.txt into out_dir; bench prints
// one JSON line with the reference's benchmark fields; run steps whole frames
// (tick) and writes the final position, velocity and evaluated velocity.
#include <cuda.h>
#include <cuda_runtime.h>

#include <chrono>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <cub/device/device_scan.cuh>

#include "../../include/gsph.h"
#include "ref_layout.h"

using namespace refh;

#define CK(x)                                                                 \
    do {                                                                      \
        cudaError_t e_ = (x);                                                 \
        if (e_ != cudaSuccess) {                                              \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x,    \
                         cudaGetErrorString(e_));                             \
            std::exit(2);                                                     \
        }                                                                     \
    } while (0)
#define CU(x)                                                                 \
    do {                                                                      \
        CUresult r_ = (x);                                                    \
        if (r_ != CUDA_SUCCESS) {                                             \
            const char *s_ = nullptr;                                         \
            cuGetErrorString(r_, &s_);                                        \
            std::fprintf(stderr, "%s:%d %s: %s\n", __FILE__, __LINE__, #x,    \
                         s_ ? s_ : "?");                                      \
            std::exit(2);                                                     \
        }                                                                     \
    } while (0)

static int ceil_int(int a, int b) { return (a + b - 1) / b; }

struct Kernels {
    CUfunction init, cell_sum_m, result_m, cell_info, block_req, cell_sum_two_m,
        result_two9, middle, arrange_tasks, judge, density[2], force[2],
        integrate;
    CUdeviceptr sys_para = 0;
    size_t sys_para_size = 0;
};

// Kernels are found by their mangled name prefix: _ZN<len(ns)><ns><len(name)><name>
// followed by E (plain function) or I (template arguments, matched by `tail`).
static CUfunction find_kernel(const std::vector<CUfunction> &fns,
                              const std::vector<std::string> &names,
                              const char *ns, const char *name,
                              const char *tail = "E") {
    const std::string prefix = "_ZN" + std::to_string(std::strlen(ns)) + ns +
                               std::to_string(std::strlen(name)) + name + tail;
    CUfunction hit = nullptr;
    for (size_t i = 0; i < fns.size(); ++i) {
        if (names[i].compare(0, prefix.size(), prefix) != 0) continue;
        if (hit) {
            std::fprintf(stderr, "ambiguous kernel name %s\n", prefix.c_str());
            std::exit(2);
        }
        hit = fns[i];
    }
    if (!hit) {
        std::fprintf(stderr, "kernel %s not found in the device image\n", prefix.c_str());
        std::exit(2);
    }
    return hit;
}

static Kernels load_kernels(const char *cubin) {
    CU(cuInit(0));
    CK(cudaSetDevice(0));
    CK(cudaFree(nullptr));   // make the primary context current
    CUmodule mod;
    CU(cuModuleLoad(&mod, cubin));
    unsigned int count = 0;
    CU(cuModuleGetFunctionCount(&count, mod));
    std::vector<CUfunction> fns(count);
    CU(cuModuleEnumerateFunctions(fns.data(), count, mod));
    std::vector<std::string> names(count);
    for (unsigned i = 0; i < count; ++i) {
        const char *nm = nullptr;
        CU(cuFuncGetName(&nm, fns[i]));
        names[i] = nm ? nm : "";
    }
    Kernels k;
    k.init = find_kernel(fns, names, "sph", "knInit");
    k.cell_sum_m = find_kernel(fns, names, "sph", "CountingSort_Cell_SumM");
    k.result_m = find_kernel(fns, names, "sph", "CountingSort_Result_M");
    k.cell_info = find_kernel(fns, names, "sph", "calculate_cell_info");
    k.block_req = find_kernel(fns, names, "gpu_model", "knCalculateBlockRequirementHybridMode");
    k.cell_sum_two_m = find_kernel(fns, names, "sph", "CountingSort_Cell_Sum_two_M");
    k.result_two9 = find_kernel(fns, names, "sph", "CountingSort_Result_two9");
    k.middle = find_kernel(fns, names, "sph", "knFindHybridModeMiddleValue");
    k.arrange_tasks = find_kernel(fns, names, "sph", "knArrangeSmsTasks");
    k.judge = find_kernel(fns, names, "sph", "judgeTask");
    k.density[0] = find_kernel(fns, names, "sph", "computeDensityHybridKernel", "ILb0E");
    k.density[1] = find_kernel(fns, names, "sph", "computeDensityHybridKernel", "ILb1E");
    k.force[0] = find_kernel(fns, names, "sph", "computeForceHybridKernel", "ILb0E");
    k.force[1] = find_kernel(fns, names, "sph", "computeForceHybridKernel", "ILb1E");
    k.integrate = find_kernel(fns, names, "sph", "knIntegrateVelocityE");
    // sph::kDevSysPara, the reference's __constant__ SystemParameter
    // (device_context.cu:10)
    const std::string para = std::string("_ZN3sph") + std::to_string(std::strlen("kDevSysPara")) +
                             "kDevSysPara" + "E";
    CU(cuModuleGetGlobal(&k.sys_para, &k.sys_para_size, mod, para.c_str()));
    if (k.sys_para_size != sizeof(SysPara)) {
        std::fprintf(stderr, "kDevSysPara size %zu != %zu\n", k.sys_para_size,
                     sizeof(SysPara));
        std::exit(2);
    }
    return k;
}

static void launch(CUfunction f, int blocks, int threads, unsigned smem,
                   std::vector<void *> args) {
    if (blocks <= 0) return;
    CU(cuLaunchKernel(f, blocks, 1, 1, threads, 1, 1, smem, nullptr, args.data(),
                      nullptr));
}

// SystemParameter from the library's parameter struct (same values as
// defaultInitializeSPHSysPara, sph_hybrid_system.cpp:127-202).
static SysPara to_sys_para(const gsph_params &p) {
    SysPara s;
    std::memset(&s, 0, sizeof(s));
    s.world_size = {p.world_size[0], p.world_size[1], p.world_size[2]};
    s.cell_size = p.cell_size;
    s.inv_cell_size = p.inv_cell_size;
    s.grid_size = {uint16_t(p.grid_size[0]), uint16_t(p.grid_size[1]),
                   uint16_t(p.grid_size[2])};
    s.kernel = p.kernel;
    s.kernel_2 = p.kernel_2;
    s.mass = p.mass;
    s.rest_density1 = 1000.0f;
    s.rest_density2 = 1000.0f;
    s.to = 0.0000005f;
    s.limita = 0.0005f;
    s.viscosity1 = 6.5f;
    s.viscosity2 = 6.5f;
    s.gravity = {p.gravity[0], p.gravity[1], p.gravity[2]};
    s.wall_damping = p.wall_damping;
    s.rest_density = p.rest_density;
    s.gas_constant = p.gas_constant;
    s.viscosity = p.viscosity;
    s.time_step = p.time_step;
    s.surface_normal = p.surface_normal;
    s.surface_coe = p.surface_coe;
    s.poly6_value = p.poly6_value;
    s.spiky_value = p.spiky_value;
    s.visco_value = p.visco_value;
    s.grad_poly6 = p.grad_poly6;
    s.lplc_poly6 = p.lplc_poly6;
    s.self_density = p.self_density;
    s.self_lplc_color = 0.0f;   // integer 3 / 4 == 0 in the reference formula
    s.inv_rest_density = p.inv_rest_density;
    s.density_scale = p.density_scale;
    s.half_spiky_value = p.half_spiky_value;
    s.viscosity_visco_value = p.viscosity_visco_value;
    s.grad_color_scale = p.grad_color_scale;
    s.lplc_color_scale = p.lplc_color_scale;
    s.sim_ratio = {1.f, 1.f, 1.f};
    s.bound_interval = p.bound_interval;
    s.bound_min = {p.bound_min[0], p.bound_min[1], p.bound_min[2]};
    s.bound_max = {p.bound_max[0], p.bound_max[1], p.bound_max[2]};
    return s;
}

struct Scene {
    gsph_params p;
    int n = 0;
    std::vector<F4> pos, vel, ev;
};

static Scene read_input(const char *path) {
    Scene sc;
    FILE *f = std::fopen(path, "rb");
    if (!f) {
        std::fprintf(stderr, "cannot open %s\n", path);
        std::exit(2);
    }
    char magic[8];
    if (std::fread(magic, 1, 8, f) != 8 || std::memcmp(magic, "GSPHREF1", 8) ||
        std::fread(&sc.p, sizeof(sc.p), 1, f) != 1 ||
        std::fread(&sc.n, sizeof(int), 1, f) != 1 || sc.n < 0) {
        std::fprintf(stderr, "bad input file %s\n", path);
        std::exit(2);
    }
    sc.pos.resize(sc.n);
    sc.vel.resize(sc.n);
    sc.ev.resize(sc.n);
    size_t n = size_t(sc.n);
    if (std::fread(sc.pos.data(), sizeof(F4), n, f) != n ||
        std::fread(sc.vel.data(), sizeof(F4), n, f) != n ||
        std::fread(sc.ev.data(), sizeof(F4), n, f) != n) {
        std::fprintf(stderr, "truncated input file %s\n", path);
        std::exit(2);
    }
    std::fclose(f);
    return sc;
}

// Device state of one scene, laid out as the reference allocates it
// (Arrangement ctor sph_arrangement.cu:607-673, ParticleBufferObject).
struct RefState {
    int n = 0, numc = 0;
    US3 grid;
    BufList buf{}, tmp{};
    int *d_hash = nullptr, *hashp = nullptr, *d_hash_p = nullptr;
    int *d_index = nullptr, *d_p_offset = nullptr, *d_p_offset_p = nullptr;
    int *d_block_reqs = nullptr, *d_task_offset = nullptr, *cell_num_two = nullptr;
    int *d_cell_offset = nullptr, *d_cell_nump = nullptr;
    int *d_cell_offset_M = nullptr, *d_cell_nump_M = nullptr;
    int *d_counts = nullptr;   // {middle, task count}
    int *h_counts = nullptr;   // pinned
    Task *d_tasks = nullptr;
    void *cub_temp = nullptr;
    size_t cub_bytes = 0;
    int middle = 0, task_count = 0;
};

template <typename T>
static T *dalloc(size_t count) {
    T *p = nullptr;
    CK(cudaMalloc(&p, std::max<size_t>(count, 1) * sizeof(T)));
    return p;
}

static RefState make_state(const Scene &sc, const Kernels &k) {
    RefState st;
    st.n = sc.n;
    st.grid = {uint16_t(sc.p.grid_size[0]), uint16_t(sc.p.grid_size[1]),
               uint16_t(sc.p.grid_size[2])};
    st.numc = st.grid.x * st.grid.y * st.grid.z;
    const size_t N = size_t(sc.n), C = size_t(st.numc);
    // main particle buffer
    st.buf.position_d = dalloc<F4>(N);
    st.buf.velocity = dalloc<F3>(N);
    st.buf.acceleration = dalloc<F3>(N);
    st.buf.evaluated_velocity = dalloc<F4>(N);
    st.buf.final_position = dalloc<F3>(N);
    st.buf.color = dalloc<unsigned>(N);
    // sort target: own pos/vel/ev/color, shared acceleration/final_position
    st.tmp.position_d = dalloc<F4>(N);
    st.tmp.velocity = dalloc<F3>(N);
    st.tmp.evaluated_velocity = dalloc<F4>(N);
    st.tmp.color = dalloc<unsigned>(N);
    st.tmp.acceleration = st.buf.acceleration;
    st.tmp.final_position = st.buf.final_position;
    st.d_hash = dalloc<int>(N);
    st.hashp = dalloc<int>(N);
    st.d_hash_p = dalloc<int>(N);
    st.d_index = dalloc<int>(N);
    st.d_p_offset = dalloc<int>(N);
    st.d_p_offset_p = dalloc<int>(N);
    st.d_block_reqs = dalloc<int>(C);
    st.d_task_offset = dalloc<int>(C);
    st.cell_num_two = dalloc<int>(2 * C + 1);
    st.d_cell_offset = dalloc<int>(C + 1);
    st.d_cell_nump = dalloc<int>(C);
    st.d_cell_offset_M = dalloc<int>(C * 64 + 1);
    st.d_cell_nump_M = dalloc<int>(C * 64 + 1);
    st.d_counts = dalloc<int>(2);
    CK(cudaMallocHost(&st.h_counts, 2 * sizeof(int)));
    const size_t task_cap = size_t(ceil_int(sc.n, 32)) + C + 2;
    st.d_tasks = dalloc<Task>(task_cap);
    CK(cudaMemset(st.d_tasks, 0, task_cap * sizeof(Task)));
    CK(cudaMemset(st.d_counts + 1, 0, sizeof(int)));
    size_t b1 = 0, b2 = 0, b3 = 0;
    CK(cub::DeviceScan::ExclusiveSum(nullptr, b1, st.d_cell_nump_M, st.d_cell_offset_M,
                                     int(C * 64 + 1)));
    CK(cub::DeviceScan::ExclusiveSum(nullptr, b2, st.d_block_reqs, st.d_task_offset, int(C)));
    CK(cub::DeviceScan::InclusiveSum(nullptr, b3, st.cell_num_two, st.cell_num_two, int(2 * C)));
    st.cub_bytes = std::max(b1, std::max(b2, b3));
    CK(cudaMalloc(&st.cub_temp, st.cub_bytes));
    // initial state: transSysParaToDevice, host data as float4/float3, knInit
    const SysPara sp = to_sys_para(sc.p);
    CU(cuMemcpyHtoD(k.sys_para, &sp, sizeof(sp)));
    std::vector<F3> v3(N);
    for (size_t i = 0; i < N; ++i) v3[i] = {sc.vel[i].x, sc.vel[i].y, sc.vel[i].z};
    CK(cudaMemcpy(st.buf.position_d, sc.pos.data(), N * sizeof(F4), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(st.buf.velocity, v3.data(), N * sizeof(F3), cudaMemcpyHostToDevice));
    int n = sc.n;
    launch(k.init, ceil_int(n, 256), 256, 0, {&st.buf, &n});   // BuffInit
    // evaluated velocity given by the caller (knInit zeroes it)
    CK(cudaMemcpy(st.buf.evaluated_velocity, sc.ev.data(), N * sizeof(F4),
                  cudaMemcpyHostToDevice));
    CK(cudaDeviceSynchronize());
    return st;
}

// Arrangement::arrangeHybridFrame, sph_arrangement.cu:1493-1506.
static void arrange(RefState &st, const Kernels &k, float inv_cell) {
    const int nt = 256;
    int n = st.n, numc = st.numc;
    int numCN = numc << 6;
    // CountingSort_O_M (:1352-1395)
    CK(cudaMemsetAsync(st.d_cell_nump_M, 0, sizeof(int) * (size_t(numCN) + 1), 0));
    launch(k.cell_sum_m, ceil_int(n, nt), nt, 0,
           {&st.d_p_offset, &st.d_hash, &st.d_cell_nump_M, &n, &st.buf.position_d,
            &inv_cell, &st.grid});
    CK(cub::DeviceScan::ExclusiveSum(st.cub_temp, st.cub_bytes, st.d_cell_nump_M,
                                     st.d_cell_offset_M, numCN + 1));
    launch(k.result_m, ceil_int(n, nt), nt, 0,
           {&st.d_p_offset, &st.d_hash, &st.hashp, &st.d_cell_offset_M, &n, &st.buf,
            &st.tmp});
    launch(k.cell_info, ceil_int(numc, nt), nt, 0,
           {&st.d_cell_nump, &st.d_cell_offset, &st.d_cell_offset_M, &numc});
    std::swap(st.d_hash, st.hashp);
    std::swap(st.buf, st.tmp);
    // gpu_model::calculateBlockRequirementHybridMode (gpu_model.cu:309-319)
    launch(k.block_req, ceil_int(numc, 256), 256, 0,
           {&st.d_cell_nump, &st.d_block_reqs, &st.grid});
    // CountingSortCUDA_Two9_M (:1459-1482)
    int numCell = numc << 1;
    CK(cudaMemsetAsync(st.cell_num_two, 0, sizeof(int) * size_t(numCell), 0));
    launch(k.cell_sum_two_m, ceil_int(n, nt), nt, 0,
           {&st.d_hash_p, &st.d_p_offset_p, &st.d_hash, &st.cell_num_two, &n,
            &st.d_block_reqs, &numc, &st.d_cell_offset});
    CK(cub::DeviceScan::InclusiveSum(st.cub_temp, st.cub_bytes, st.cell_num_two,
                                     st.cell_num_two, numCell));
    launch(k.result_two9, ceil_int(n, nt), nt, 0,
           {&st.d_p_offset_p, &st.d_hash_p, &st.hashp, &st.cell_num_two, &st.d_index,
            &n});
    CK(cudaMemsetAsync(st.d_counts, 0xFF, sizeof(int), 0));
    unsigned nump = unsigned(n);
    launch(k.middle, ceil_int(n, nt), nt, (nt + 1) * sizeof(int),
           {&numc, &st.d_counts, &st.hashp, &nump});
    // task offsets (:1499-1500) and arrangeSmsTasks (:1034-1071)
    CK(cub::DeviceScan::ExclusiveSum(st.cub_temp, st.cub_bytes, st.d_block_reqs,
                                     st.d_task_offset, numc));
    int *task_count_ptr = st.d_counts + 1;
    launch(k.arrange_tasks, ceil_int(numc, 128), 128, 0,
           {&st.d_hash, &st.d_cell_offset, &st.d_cell_nump, &st.d_tasks, &task_count_ptr,
            &st.d_block_reqs, &st.d_task_offset, &numc, &st.grid});
    CK(cudaMemcpyAsync(st.h_counts, st.d_counts, 2 * sizeof(int), cudaMemcpyDeviceToHost, 0));
    CK(cudaStreamSynchronize(0));
    st.task_count = st.h_counts[1];
    st.middle = st.h_counts[0];
    const int pair_count = ceil_int(st.task_count, 2);
    launch(k.judge, ceil_int(pair_count, 128), 128, 0, {&st.d_tasks, &task_count_ptr});
}

// computeDensityHybrid / computeForceHybrid (kernel_dispatch.cu:182-253) and
// HybridSystem::tick's clamp of the split point (sph_hybrid_system.cpp:281-286).
static void physics(RefState &st, const Kernels &k, CUfunction *fam) {
    int middle = st.middle;
    if (middle < 0 || middle > st.n) middle = st.n;
    IdxRange tra{0, middle};
    const int blocks = ceil_int(middle, 64) + ceil_int(st.task_count, 2);
    const bool sms_only = middle == 0;
    int *d_T = st.d_counts + 1, *d_mid = st.d_counts;
    launch(fam[sms_only ? 1 : 0], blocks, 64, 0,
           {&st.d_cell_offset_M, &tra, &st.buf, &st.d_index, &st.d_cell_offset,
            &st.d_cell_nump, &st.d_tasks, &d_T, &d_mid});
}

static void advance(RefState &st, const Kernels &k) {
    unsigned nump = unsigned(st.n);
    launch(k.integrate, ceil_int(st.n, 128), 128, 0, {&st.buf, &nump});
}

template <typename T>
static void dump(const std::string &dir, const char *name, const void *dptr,
                 size_t count, FILE *meta, const char *dtype, int cols = 1) {
    std::vector<T> h(std::max<size_t>(count, 1));
    if (count)
        CK(cudaMemcpy(h.data(), dptr, count * sizeof(T), cudaMemcpyDeviceToHost));
    const std::string path = dir + "/" + name + ".bin";
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    if (count) std::fwrite(h.data(), sizeof(T), count, f);
    std::fclose(f);
    std::fprintf(meta, "%s %s %zu %d\n", name, dtype, count / size_t(cols), cols);
}

static void write_host(const std::string &dir, const char *name, const void *h,
                       size_t bytes, size_t rows, FILE *meta, const char *dtype) {
    const std::string path = dir + "/" + name + ".bin";
    FILE *f = std::fopen(path.c_str(), "wb");
    if (!f) {
        std::fprintf(stderr, "cannot write %s\n", path.c_str());
        std::exit(2);
    }
    if (bytes) std::fwrite(h, 1, bytes, f);
    std::fclose(f);
    std::fprintf(meta, "%s %s %zu 1\n", name, dtype, rows);
}

// The dense micro-cell offset table (cells * 64 + 1 ints: 810 MB for a
// 3.16M-cell grid) written sparsely: the index, start and count of every
// occupied micro cell, and the total.
static void dump_micro_sparse(const std::string &dir, const int *d_off,
                              size_t micro_cells, FILE *meta) {
    std::vector<int> h(micro_cells + 1);
    CK(cudaMemcpy(h.data(), d_off, h.size() * sizeof(int), cudaMemcpyDeviceToHost));
    std::vector<long long> idx;
    std::vector<int> start, count;
    for (size_t m = 0; m < micro_cells; ++m) {
        const int c = h[m + 1] - h[m];
        if (c != 0) {
            idx.push_back((long long)m);
            start.push_back(h[m]);
            count.push_back(c);
        }
    }
    std::fprintf(meta, "micro_total %d\n", h[micro_cells]);
    write_host(dir, "micro_index", idx.data(), idx.size() * 8, idx.size(), meta, "int64");
    write_host(dir, "micro_start", start.data(), start.size() * 4, start.size(), meta,
               "int32");
    write_host(dir, "micro_count", count.data(), count.size() * 4, count.size(), meta,
               "int32");
}

static int run_tick(const Kernels &k, const Scene &sc, const std::string &dir) {
    RefState st = make_state(sc, k);
    const float inv_cell = sc.p.inv_cell_size;
    FILE *meta = std::fopen((dir + "/meta.txt").c_str(), "w");
    if (!meta) {
        std::fprintf(stderr, "cannot write into %s\n", dir.c_str());
        return 2;
    }
    const size_t N = size_t(st.n), C = size_t(st.numc);
    arrange(st, k, inv_cell);
    CK(cudaDeviceSynchronize());
    std::fprintf(meta, "middle %d\ntask_count %d\n", st.middle, st.task_count);
    dump<int>(dir, "hash", st.d_hash, N, meta, "int32");
    dump<int>(dir, "cell_offset", st.d_cell_offset, C, meta, "int32");
    dump<int>(dir, "cell_nump", st.d_cell_nump, C, meta, "int32");
    dump_micro_sparse(dir, st.d_cell_offset_M, C * 64, meta);
    dump<int>(dir, "block_req", st.d_block_reqs, C, meta, "int32");
    dump<int>(dir, "index", st.d_index, N, meta, "int32");
    const int T = st.task_count;
    dump<Task>(dir, "tasks", st.d_tasks, size_t(T + (T & 1)), meta, "task");
    dump<float>(dir, "sorted_pos", st.buf.position_d, N * 4, meta, "float32", 4);
    dump<float>(dir, "sorted_vel", st.buf.velocity, N * 3, meta, "float32", 3);
    dump<float>(dir, "sorted_ev", st.buf.evaluated_velocity, N * 4, meta, "float32", 4);
    physics(st, k, const_cast<CUfunction *>(k.density));
    CK(cudaDeviceSynchronize());
    dump<float>(dir, "density_pos", st.buf.position_d, N * 4, meta, "float32", 4);
    dump<float>(dir, "density_ev", st.buf.evaluated_velocity, N * 4, meta, "float32", 4);
    physics(st, k, const_cast<CUfunction *>(k.force));
    CK(cudaDeviceSynchronize());
    dump<float>(dir, "force_acc", st.buf.acceleration, N * 3, meta, "float32", 3);
    advance(st, k);
    CK(cudaDeviceSynchronize());
    dump<float>(dir, "final_pos", st.buf.position_d, N * 4, meta, "float32", 4);
    dump<float>(dir, "final_vel", st.buf.velocity, N * 3, meta, "float32", 3);
    dump<float>(dir, "final_ev", st.buf.evaluated_velocity, N * 4, meta, "float32", 4);
    std::fclose(meta);
    return 0;
}

// HybridSystem::runBenchmark (sph_hybrid_system.cpp:341-430).
static int run_bench(const Kernels &k, const Scene &sc, int frames) {
    RefState st = make_state(sc, k);
    const float inv_cell = sc.p.inv_cell_size;
    cudaEvent_t ev[5];
    for (auto &e : ev) CK(cudaEventCreate(&e));
    const int warm = frames < 5 ? frames : 5;
    double acc[4] = {0, 0, 0, 0};
    auto tick = [&](bool timed) {
        if (timed) CK(cudaEventRecord(ev[0], 0));
        arrange(st, k, inv_cell);
        if (timed) CK(cudaEventRecord(ev[1], 0));
        physics(st, k, const_cast<CUfunction *>(k.density));
        if (timed) CK(cudaEventRecord(ev[2], 0));
        physics(st, k, const_cast<CUfunction *>(k.force));
        if (timed) CK(cudaEventRecord(ev[3], 0));
        advance(st, k);
        if (timed) {
            CK(cudaEventRecord(ev[4], 0));
            CK(cudaEventSynchronize(ev[4]));
            float a, d, f, t;
            CK(cudaEventElapsedTime(&a, ev[0], ev[1]));
            CK(cudaEventElapsedTime(&d, ev[1], ev[2]));
            CK(cudaEventElapsedTime(&f, ev[2], ev[3]));
            CK(cudaEventElapsedTime(&t, ev[0], ev[4]));
            acc[0] += a;
            acc[1] += d;
            acc[2] += f;
            acc[3] += t;
        }
    };
    for (int i = 0; i < warm; ++i) tick(true);
    const int measured = frames - warm;
    CK(cudaDeviceSynchronize());
    const auto t0 = std::chrono::steady_clock::now();
    CK(cudaEventRecord(ev[0], 0));
    for (int i = 0; i < measured; ++i) tick(false);
    CK(cudaEventRecord(ev[4], 0));
    CK(cudaDeviceSynchronize());
    const auto t1 = std::chrono::steady_clock::now();
    float dev_ms = 0.f;
    CK(cudaEventElapsedTime(&dev_ms, ev[0], ev[4]));
    const double wall = std::chrono::duration<double, std::milli>(t1 - t0).count();
    const double avg = measured > 0 ? wall / measured : acc[3] / warm;
    // state checksum (sph_hybrid_system.cpp:43-62)
    std::vector<F4> h(st.n);
    CK(cudaMemcpy(h.data(), st.buf.position_d, size_t(st.n) * sizeof(F4),
                  cudaMemcpyDeviceToHost));
    double cs[5] = {0, 0, 0, 0, 0};
    for (int i = 0; i < st.n; ++i) {
        cs[0] += h[i].x;
        cs[1] += h[i].y;
        cs[2] += h[i].z;
        cs[3] += h[i].w;
        cs[4] += double((unsigned(i) & 1023u) + 1u) *
                 (h[i].x + 3.0 * h[i].y + 7.0 * h[i].z);
    }
    std::printf("{\"impl\": \"reference-gpu\", \"particles\": %d, \"frames\": %d, "
                "\"measured_frames\": %d, \"avg_frame_ms\": %.6f, "
                "\"device_ms_per_frame\": %.6f, \"particle_steps_per_s\": %.6e, "
                "\"arrange_ms\": %.6f, \"density_ms\": %.6f, \"force_ms\": %.6f, "
                "\"total_kernel_ms\": %.6f, \"tra_particles\": %d, \"sms_tasks\": %d, "
                "\"checksum\": [%.17g, %.17g, %.17g, %.17g, %.17g]}\n",
                st.n, frames, measured, avg, measured > 0 ? dev_ms / measured : 0.0,
                avg > 0 ? st.n * 1000.0 / avg : 0.0, acc[0] / warm, acc[1] / warm,
                acc[2] / warm, acc[3] / warm, st.middle, st.task_count, cs[0], cs[1],
                cs[2], cs[3], cs[4]);
    return 0;
}

// `frames` whole reference frames (tick, sph_hybrid_system.cpp:253-339),
// then the final state.
static int run_frames(const Kernels &k, const Scene &sc, int frames,
                      const std::string &dir) {
    RefState st = make_state(sc, k);
    const float inv_cell = sc.p.inv_cell_size;
    FILE *meta = std::fopen((dir + "/meta.txt").c_str(), "w");
    if (!meta) {
        std::fprintf(stderr, "cannot write into %s\n", dir.c_str());
        return 2;
    }
    for (int i = 0; i < frames; ++i) {
        arrange(st, k, inv_cell);
        physics(st, k, const_cast<CUfunction *>(k.density));
        physics(st, k, const_cast<CUfunction *>(k.force));
        advance(st, k);
    }
    CK(cudaDeviceSynchronize());
    const size_t N = size_t(st.n);
    std::fprintf(meta, "middle %d\ntask_count %d\n", st.middle, st.task_count);
    dump<float>(dir, "final_pos", st.buf.position_d, N * 4, meta, "float32", 4);
    dump<float>(dir, "final_vel", st.buf.velocity, N * 3, meta, "float32", 3);
    dump<float>(dir, "final_ev", st.buf.evaluated_velocity, N * 4, meta, "float32", 4);
    std::fclose(meta);
    return 0;
}

int main(int argc, char **argv) {
    if (argc < 5) {
        std::fprintf(stderr,
                     "usage: %s <cubin> tick <input.bin> <out_dir>\n"
                     "       %s <cubin> bench <input.bin> <frames>\n"
                     "       %s <cubin> run <input.bin> <frames> <out_dir>\n",
                     argv[0], argv[0], argv[0]);
        return 2;
    }
    const Kernels k = load_kernels(argv[1]);
    const Scene sc = read_input(argv[3]);
    if (!std::strcmp(argv[2], "tick")) return run_tick(k, sc, argv[4]);
    if (!std::strcmp(argv[2], "bench")) return run_bench(k, sc, std::atoi(argv[4]));
    if (!std::strcmp(argv[2], "run") && argc >= 6)
        return run_frames(k, sc, std::atoi(argv[4]), argv[5]);
    std::fprintf(stderr, "unknown mode %s\n", argv[2]);
    return 2;
}
