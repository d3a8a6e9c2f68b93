// ref_layout.h — host-side mirrors of the reference's kernel argument types.
//
// TEST INFRASTRUCTURE ONLY. The reference-kernel harness passes these by value
// to kernels compiled from the reference's sources, so their layouts must be
// identical to the reference's types:
//   SystemParameter      src/core/sph_parameter.h:18-90
//   ParticleBufferList   src/particle/particle_buffer.h:116-145
//   BlockTask            src/particle/particle_buffer.h:60-87
//   ParticleIdxRange     src/particle/particle_buffer.h:110-114
// layout_check.cu verifies every size and offset against the reference
// headers when the reference tree is available.
#ifndef GSPH_REF_LAYOUT_H_
#define GSPH_REF_LAYOUT_H_

#include <cstdint>

namespace refh {

struct F3 { float x, y, z; };
struct US3 { uint16_t x, y, z; };
struct F4 { float x, y, z, w; };

struct SysPara {
    F3 world_size;
    float cell_size;
    float inv_cell_size;
    US3 grid_size;
    float kernel;
    float kernel_2;
    float mass;
    float mass1;
    float mass2;
    float rest_density1;
    float rest_density2;
    float to;
    float limita;
    float viscosity1;
    float viscosity2;
    F3 gravity;
    float wall_damping;
    float rest_density;
    float gas_constant;
    float viscosity;
    float time_step;
    float surface_normal;
    float surface_coe;
    float poly6_value;
    float spiky_value;
    float visco_value;
    float grad_poly6;
    float lplc_poly6;
    float self_density;
    float self_lplc_color;
    float inv_rest_density;
    float density_scale;
    float half_spiky_value;
    float viscosity_visco_value;
    float grad_color_scale;
    float lplc_color_scale;
    F3 sim_ratio;
    F3 sim_origin;
    float bound_interval;
    F3 bound_min;
    F3 bound_max;
    float spacing_fluid;
    int pcisph_min_loops;
    int pcisph_max_loops;
    float pcisph_max_density_error_allowed;
    float pcisph_density_error_factor;
};

struct BufList {
    void *position_d;          // float4
    void *evaluated_velocity;  // float4
    void *velocity;            // float3
    void *acceleration;        // float3
    void *final_position;      // float3
    void *predicted_pos;
    void *correction_pressure_force;
    void *pressure;
    void *predicted_density;
    void *densityError;
    void *correction_pressure;
    void *color;               // unsigned int
    void *phase;
    void *vlfrt;
    void *mixV;
    void *Vm;
    void *mixP;
    void *mixM;
    void *Mixden;
};

struct Task {
    int8_t isSame;
    uint16_t paired_bounds;
    int32_t cellid;
    US3 cell_pos;
    uint16_t p_offset;
    int8_t xxi, xxx, yyi, yyy, zzi, zzz;
    int32_t cell_begin;
    int32_t cell_particle_count;
};

struct IdxRange {
    int begin, end;
};

static_assert(sizeof(Task) == 32, "Task layout");

}  // namespace refh

#endif  // GSPH_REF_LAYOUT_H_
