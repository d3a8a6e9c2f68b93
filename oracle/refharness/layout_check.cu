// layout_check.cu — compile-time proof that ref_layout.h matches the
// reference's own type layouts (compiled with -fsyntax-only wherever the
// reference tree is present). TEST INFRASTRUCTURE ONLY.
#include <cstddef>

#include "core/sph_parameter.h"
#include "particle/particle_buffer.h"
#include "ref_layout.h"

#define SAME(A, B, F) static_assert(offsetof(A, F) == offsetof(B, F), #F)

static_assert(sizeof(sph::SystemParameter) == sizeof(refh::SysPara), "SystemParameter size");
SAME(sph::SystemParameter, refh::SysPara, world_size);
SAME(sph::SystemParameter, refh::SysPara, grid_size);
SAME(sph::SystemParameter, refh::SysPara, kernel);
SAME(sph::SystemParameter, refh::SysPara, gravity);
SAME(sph::SystemParameter, refh::SysPara, rest_density);
SAME(sph::SystemParameter, refh::SysPara, poly6_value);
SAME(sph::SystemParameter, refh::SysPara, self_density);
SAME(sph::SystemParameter, refh::SysPara, inv_rest_density);
SAME(sph::SystemParameter, refh::SysPara, lplc_color_scale);
SAME(sph::SystemParameter, refh::SysPara, sim_ratio);
SAME(sph::SystemParameter, refh::SysPara, bound_interval);
SAME(sph::SystemParameter, refh::SysPara, bound_min);
SAME(sph::SystemParameter, refh::SysPara, bound_max);
SAME(sph::SystemParameter, refh::SysPara, pcisph_density_error_factor);

static_assert(sizeof(sph::ParticleBufferList) == sizeof(refh::BufList), "ParticleBufferList size");
SAME(sph::ParticleBufferList, refh::BufList, position_d);
SAME(sph::ParticleBufferList, refh::BufList, evaluated_velocity);
SAME(sph::ParticleBufferList, refh::BufList, velocity);
SAME(sph::ParticleBufferList, refh::BufList, acceleration);
SAME(sph::ParticleBufferList, refh::BufList, final_position);
SAME(sph::ParticleBufferList, refh::BufList, color);
SAME(sph::ParticleBufferList, refh::BufList, Mixden);

static_assert(sizeof(sph::BlockTask) == sizeof(refh::Task), "BlockTask size");
SAME(sph::BlockTask, refh::Task, isSame);
SAME(sph::BlockTask, refh::Task, paired_bounds);
SAME(sph::BlockTask, refh::Task, cellid);
SAME(sph::BlockTask, refh::Task, cell_pos);
SAME(sph::BlockTask, refh::Task, p_offset);
SAME(sph::BlockTask, refh::Task, xxi);
SAME(sph::BlockTask, refh::Task, zzz);
SAME(sph::BlockTask, refh::Task, cell_begin);
SAME(sph::BlockTask, refh::Task, cell_particle_count);

static_assert(sizeof(sph::ParticleIdxRange) == sizeof(refh::IdxRange), "ParticleIdxRange size");
