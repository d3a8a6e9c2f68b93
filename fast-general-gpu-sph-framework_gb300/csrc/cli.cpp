// cli.cpp — the `gsph` command: headless benchmark of one scene.
//
// Same flags and output block as the reference's executable
// (src/main.cpp:42-85 parseBenchmarkFrames / runHeadlessBenchmark and the print
// block of HybridSystem::runBenchmark, src/simulation/sph_hybrid_system.cpp:
// 397-429), plus --scene PATH (the reference compiles the scene path in),
// --device D, --graph (launch whole frames as CUDA graphs of 10 frames),
// --artificial-viscosity ALPHA C0 (Monaghan's artificial viscosity in place of
// the reference's Laplacian term) and --autotune (time the built-in tunings
// on the scene and keep the fastest before the benchmark).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/gsph.h"

namespace {

int parse_frames(int argc, char **argv) {
    int frames = 200;   // headless default (main.cpp:44)
    for (int i = 1; i + 1 < argc; ++i)
        if (!std::strcmp(argv[i], "--headless") || !std::strcmp(argv[i], "--benchmark"))
            frames = std::atoi(argv[++i]);
    return frames;
}

std::string arg_value(int argc, char **argv, const char *key, const char *dflt) {
    for (int i = 1; i + 1 < argc; ++i)
        if (!std::strcmp(argv[i], key)) return argv[i + 1];
    return dflt ? dflt : "";
}

bool has_flag(int argc, char **argv, const char *key) {
    for (int i = 1; i < argc; ++i)
        if (!std::strcmp(argv[i], key)) return true;
    return false;
}

}  // namespace

int main(int argc, char **argv) {
    const int frames = parse_frames(argc, argv);
    if (frames <= 0) {
        std::fprintf(stderr, "Benchmark frame count must be positive.\n");
        return EXIT_FAILURE;
    }
    const std::string scene = arg_value(argc, argv, "--scene", "scenes/scene_default.json");
    const int device = std::atoi(arg_value(argc, argv, "--device", "0").c_str());
    gsph_handle h = nullptr;
    gsph_status st = gsph_create_from_json(scene.c_str(), device, &h);
    if (st) {
        std::fprintf(stderr, "%s\n", gsph_last_error());
        return EXIT_FAILURE;
    }
    std::printf("CUDA initialized.\n");
    gsph_info info;
    gsph_get_info(h, &info);
    std::printf("Number of particles: %u\n", info.n_particles);
    for (int i = 1; i + 2 < argc; ++i)
        if (!std::strcmp(argv[i], "--artificial-viscosity")) {
            st = gsph_set_viscosity_model(h, GSPH_VISCOSITY_ARTIFICIAL,
                                          float(std::atof(argv[i + 1])),
                                          float(std::atof(argv[i + 2])));
            if (st) {
                std::fprintf(stderr, "%s\n", gsph_last_error());
                gsph_destroy(h);
                return EXIT_FAILURE;
            }
            std::printf("Artificial viscosity: alpha %s, c0 %s\n", argv[i + 1], argv[i + 2]);
        }
    if (has_flag(argc, argv, "--autotune")) {
        gsph_tuning best;
        float ms = 0.f;
        st = gsph_autotune(h, 3, nullptr, 0, &best, &ms);
        if (st) {
            std::fprintf(stderr, "%s\n", gsph_last_error());
            gsph_destroy(h);
            return EXIT_FAILURE;
        }
        std::printf("Autotuned: thresholds %d/%d/%d, CTAs per SM %d/%d/%d/%d, %d warps per "
                    "block (%.4f ms per trial frame)\n",
                    best.sparse_total, best.sparse_self, best.mid_total, best.ctas_density_tra,
                    best.ctas_density_sms, best.ctas_force_tra, best.ctas_force_sms,
                    best.warps_per_block, double(ms));
    }
    // --graph: whole frames launched as CUDA graphs of 10 frames
    if (has_flag(argc, argv, "--graph")) gsph_set_graph_mode(h, 10);
    gsph_bench_report r;
    st = gsph_benchmark(h, frames, &r);
    if (st) {
        std::fprintf(stderr, "%s\n", gsph_last_error());
        gsph_destroy(h);
        return EXIT_FAILURE;
    }
    std::printf("\n========== Headless benchmark (%d measured + %d warm-up frames) ==========\n",
                r.measured_frames, r.warmup_frames);
    std::printf("Total wall time: %g ms\n", r.total_wall_ms);
    std::printf("Average frame time: %g ms\n", r.avg_frame_ms);
    std::printf("FPS: %g\n", r.fps);
    std::printf("State checksum: %.17g, %.17g, %.17g, %.17g, %.17g\n", r.checksum[0],
                r.checksum[1], r.checksum[2], r.checksum[3], r.checksum[4]);
    std::printf("Hybrid split: %d TRA particles, %d SMS tasks\n", r.tra_particles,
                r.sms_tasks);
    std::printf("judgeTask isSame SMS pairs: %d / %d (same-cell pairs: %d, full: %d, "
                "partial: %d, compact: %d, widened: %d)\n",
                r.is_same_pairs, r.total_pairs, r.same_cell_pairs, r.full_is_same_pairs,
                r.partial_is_same_pairs, r.compact_is_same_pairs, r.widened_is_same_pairs);
    std::printf("Per-stage averages (CUDA events, warm-up frames):\n");
    std::printf("  arrange/grid : %g ms\n", r.arrange_ms);
    std::printf("  density      : %g ms\n", r.density_ms);
    std::printf("  force        : %g ms\n", r.force_ms);
    std::printf("  integrate    : %g ms\n", r.integrate_ms);
    std::printf("  total kernel : %g ms\n", r.total_kernel_ms);
    std::printf("Particle-steps/s: %.6g\n", r.particle_steps_per_s);
    std::printf("==================================================\n\n");
    gsph_destroy(h);
    return EXIT_SUCCESS;
}
