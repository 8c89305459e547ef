// C ABI of the FFP3 fluid-particle output and the particle id attribute
// (c_bindings/fluidsimulation_c.cpp:348-455, 833-874, 3716-3768, 4402-4450, 4757-4764, 4944-4950).
#include <cstring>

#include "capi_internal.h"

using ffgpu::Engine;
using ffgpu::guarded;

static Engine &E(FluidSimulation *obj) {
    if (!obj) throw std::invalid_argument("Error: null FluidSimulation handle.\n");
    return obj->eng;
}

extern "C" {

void FluidSimulation_enable_fluid_particle_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp_output = true; });
}

void FluidSimulation_disable_fluid_particle_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp_output = false; });
}

int FluidSimulation_is_fluid_particle_output_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).ffp_output ? 1 : 0; });
}

double FluidSimulation_get_fluid_particle_output_amount(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).ffp_amount; });
}

// FluidSimulation::setFluidParticleOutputAmount (fluidsimulation.cpp:338-352): negative amounts are
// refused, the rest clamped to [0, 1]
void FluidSimulation_set_fluid_particle_output_amount(FluidSimulation *obj, double value, int *err) {
    guarded(err, [&] {
        if (value < 0.0)
            throw std::domain_error("Error: amount must be greater than or equal to 0.0.\nOutput Amount: " +
                                    std::to_string(value) + "\n");
        E(obj).ffp_amount = std::max(std::min(value, 1.0), 0.0);
    });
}

static void set_bit(Engine &e, int bit, bool on) { e.ffp.enabled = on ? (e.ffp.enabled | bit) : (e.ffp.enabled & ~bit); }

void FluidSimulation_enable_fluid_particle_surface_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 1, true); });
}
void FluidSimulation_disable_fluid_particle_surface_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 1, false); });
}
int FluidSimulation_is_fluid_particle_surface_output_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (E(obj).ffp.enabled & 1) ? 1 : 0; });
}
void FluidSimulation_enable_fluid_particle_boundary_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 2, true); });
}
void FluidSimulation_disable_fluid_particle_boundary_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 2, false); });
}
int FluidSimulation_is_fluid_particle_boundary_output_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (E(obj).ffp.enabled & 2) ? 1 : 0; });
}
void FluidSimulation_enable_fluid_particle_interior_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 4, true); });
}
void FluidSimulation_disable_fluid_particle_interior_output(FluidSimulation *obj, int *err) {
    guarded(err, [&] { set_bit(E(obj), 4, false); });
}
int FluidSimulation_is_fluid_particle_interior_output_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (E(obj).ffp.enabled & 4) ? 1 : 0; });
}

void FluidSimulation_enable_fluid_particle_velocity_attribute(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp.velocity = true; });
}
void FluidSimulation_disable_fluid_particle_velocity_attribute(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp.velocity = false; });
}
int FluidSimulation_is_fluid_particle_velocity_attribute_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).ffp.velocity ? 1 : 0; });
}
void FluidSimulation_enable_fluid_particle_speed_attribute(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp.speed = true; });
}
void FluidSimulation_disable_fluid_particle_speed_attribute(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).ffp.speed = false; });
}
int FluidSimulation_is_fluid_particle_speed_attribute_enabled(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).ffp.speed ? 1 : 0; });
}

// The FFP3 bytes of the last output (empty before the first output or when the attribute is off)
int FluidSimulation_get_fluid_particle_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (int)E(obj).ffp3_bytes(0); });
}
int FluidSimulation_get_fluid_particle_id_attribute_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (int)E(obj).ffp3_bytes(1); });
}
int FluidSimulation_get_fluid_particle_velocity_attribute_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (int)E(obj).ffp3_bytes(2); });
}
int FluidSimulation_get_fluid_particle_speed_attribute_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (int)E(obj).ffp3_bytes(3); });
}
void FluidSimulation_get_fluid_particle_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { E(obj).read_ffp3(0, c_data); });
}
void FluidSimulation_get_fluid_particle_id_attribute_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { E(obj).read_ffp3(1, c_data); });
}
void FluidSimulation_get_fluid_particle_velocity_attribute_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { E(obj).read_ffp3(2, c_data); });
}
void FluidSimulation_get_fluid_particle_speed_attribute_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { E(obj).read_ffp3(3, c_data); });
}

void FluidSimulation_load_marker_particle_id_data(FluidSimulation *obj, FluidSimulationMarkerParticleIDData data,
                                                  int *err) {
    guarded(err, [&] {
        if (data.size < 0) throw std::domain_error("Error: id data count must be non-negative.\n");
        E(obj).load_ids(reinterpret_cast<const uint16_t *>(data.id), data.size);
    });
}

void FluidSimulation_get_marker_particle_id_data_range(FluidSimulation *obj, int start_idx, int end_idx, char *c_data,
                                                       int *err) {
    guarded(err, [&] { E(obj).get_ids(reinterpret_cast<uint16_t *>(c_data), start_idx, end_idx); });
}

}  // extern "C"
