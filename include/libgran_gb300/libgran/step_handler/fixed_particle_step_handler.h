// fixed_particle_step_handler.h (libgran_gb300 drop-in) -- the step handler of libgran's custom
// step-handler tutorial (Custom-step-handler.md:44-97) with its template and constructor
// signatures: increment_v of the fixed particle is skipped, every other increment goes to the base
// handler. A granular_system built with it gives the engine a hold mask with LG_HOLD_V for that
// particle; held_particles_step_handler generalises it to any LG_HOLD_* bits per particle.
#ifndef LIBGRAN_GB300_FIXED_PARTICLE_STEP_HANDLER_H
#define LIBGRAN_GB300_FIXED_PARTICLE_STEP_HANDLER_H
#include <cstdint>
#include <utility>
#include <vector>
#include "../gb300_functor_base.h"

template <typename field_container_t, typename field_value_t,
          template <typename _field_container_t, typename _field_value_t> typename base_step_handler_t>
struct fixed_particle_step_handler {
    fixed_particle_step_handler(size_t fixed_particle,
                                base_step_handler_t<field_container_t, field_value_t> base_step_handler)
        : fixed_particle(fixed_particle), base_step_handler(std::move(base_step_handler)) {}

    std::vector<uint8_t> hold_mask(size_t n) const {
        std::vector<uint8_t> m(n, 0);
        if (fixed_particle < n) m[fixed_particle] = LG_HOLD_V;
        return m;
    }

    const size_t fixed_particle;
    base_step_handler_t<field_container_t, field_value_t> base_step_handler;
};

// Any set of held increments: mask[i] holds LG_HOLD_X / V / THETA / OMEGA bits of particle i.
template <typename field_container_t, typename field_value_t>
struct held_particles_step_handler {
    explicit held_particles_step_handler(std::vector<uint8_t> mask) : mask(std::move(mask)) {}
    std::vector<uint8_t> hold_mask(size_t n) const {
        std::vector<uint8_t> m(mask);
        m.resize(n, 0);
        return m;
    }
    std::vector<uint8_t> mask;
};

#endif
