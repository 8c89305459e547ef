// C ABI, part 1: the drop-in subset of the reference engine's FluidSimulation_* API
// (src/engine/c_bindings/fluidsimulation_c.cpp) over the GB300 engine.  Exceptions
// become *err = 0 with the message readable through CBindings_get_error_message(),
// the reference's convention (cbindings.h:37-160, cbindings.cpp:35-44).
#include <cstring>
#include <string>

#include "capi_internal.h"

namespace ffgpu {
// The reference keeps one static 4096-byte message buffer; here it is per thread.
thread_local char g_error[4096];

void set_error(const std::exception &ex) {
    std::strncpy(g_error, ex.what(), sizeof(g_error) - 1);
    g_error[sizeof(g_error) - 1] = '\0';
}
}  // namespace ffgpu

using namespace ffgpu;

extern "C" {

char *CBindings_get_error_message(void) { return g_error; }

FluidSimulation *FluidSimulation_new_from_dimensions(int isize, int jsize, int ksize, double dx, int *err) {
    return guarded(err, [&]() -> FluidSimulation * { return new FluidSimulation(isize, jsize, ksize, dx); });
}

void FluidSimulation_destroy(FluidSimulation *obj) { delete obj; }

void FluidSimulation_get_version(FluidSimulation *obj, int *major, int *minor, int *revision, int *err) {
    guarded(err, [&] { E(obj); *major = 1; *minor = 8; *revision = 5; });
}

void FluidSimulation_initialize(FluidSimulation *obj, int *err) { guarded(err, [&] { E(obj).initialize(); }); }

int FluidSimulation_is_initialized(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).initialized() ? 1 : 0; });
}

void FluidSimulation_update(FluidSimulation *obj, double dt, int *err) { guarded(err, [&] { E(obj).update(dt); }); }

int FluidSimulation_get_current_frame(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).current_frame; });
}

double FluidSimulation_get_cell_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).dx; });
}

void FluidSimulation_get_grid_dimensions(FluidSimulation *obj, int *i, int *j, int *k, int *err) {
    guarded(err, [&] { Engine &e = E(obj); *i = e.ni; *j = e.nj; *k = e.nk; });
}

void FluidSimulation_get_simulation_dimensions(FluidSimulation *obj, double *width, double *height, double *depth,
                                               int *err) {
    guarded(err, [&] { Engine &e = E(obj); *width = e.ni * e.dx; *height = e.nj * e.dx; *depth = e.nk * e.dx; });
}

int FluidSimulation_get_pressure_solver_max_iterations(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).max_iterations; });
}

void FluidSimulation_set_pressure_solver_max_iterations(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] {
        if (n < 1) throw std::domain_error("Error: max iterations must be greater than or equal to 1.\n");
        E(obj).max_iterations = n;
    });
}

// Console output and surface reconstruction are outside this library's path; the toggles
// are accepted so callers run unchanged.
void FluidSimulation_enable_console_output(FluidSimulation *obj, int *err) { guarded(err, [&] { E(obj); }); }
void FluidSimulation_disable_console_output(FluidSimulation *obj, int *err) { guarded(err, [&] { E(obj); }); }
void FluidSimulation_enable_surface_reconstruction(FluidSimulation *obj, int *err) {
    guarded(err, [&] {
        E(obj);
        throw std::runtime_error("Error: surface reconstruction is not part of the GB300 substep library.\n");
    });
}
void FluidSimulation_disable_surface_reconstruction(FluidSimulation *obj, int *err) { guarded(err, [&] { E(obj); }); }

int FluidSimulation_get_max_thread_count(FluidSimulation *obj, int *err) { return guarded(err, [&] { E(obj); return 1; }); }
void FluidSimulation_set_max_thread_count(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] {
        E(obj);
        if (n < 1) throw std::domain_error("Error: thread count must be greater than or equal to 1.\n");
    });
}

void FluidSimulation_add_body_force(FluidSimulation *obj, double fx, double fy, double fz, int *err) {
    // fluidsimulation.cpp: forces are stored as float vectors and summed in float
    guarded(err, [&] { Engine &e = E(obj); e.gx += (float)fx; e.gy += (float)fy; e.gz += (float)fz; });
}

void FluidSimulation_reset_body_force(FluidSimulation *obj, int *err) {
    guarded(err, [&] { Engine &e = E(obj); e.gx = e.gy = e.gz = 0.0f; });
}

int FluidSimulation_get_CFL_condition_number(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (int)E(obj).cfl; });
}

void FluidSimulation_set_CFL_condition_number(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] {
        if (n < 1) throw std::domain_error("Error: CFL condition number must be greater than or equal to 1.\n");
        E(obj).cfl = n;
    });
}

int FluidSimulation_get_min_time_steps_per_frame(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).min_substeps; });
}

void FluidSimulation_set_min_time_steps_per_frame(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] {
        if (n < 1) throw std::domain_error("Error: min step count must be greater than or equal to 1.\n");
        E(obj).min_substeps = n;
    });
}

int FluidSimulation_get_max_time_steps_per_frame(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).max_substeps; });
}

void FluidSimulation_set_max_time_steps_per_frame(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] {
        if (n < 1) throw std::domain_error("Error: max step count must be greater than or equal to 1.\n");
        E(obj).max_substeps = n;
    });
}

void FluidSimulation_enable_extreme_velocity_removal(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).extreme_velocity_removal = true; });
}

void FluidSimulation_disable_extreme_velocity_removal(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).extreme_velocity_removal = false; });
}

void FluidSimulation_set_velocity_transfer_method_FLIP(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).apic = false; });
}

int FluidSimulation_get_viscosity_solver_max_iterations(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).visc_max_iterations; });
}

void FluidSimulation_set_viscosity_solver_max_iterations(FluidSimulation *obj, int n, int *err) {
    guarded(err, [&] { E(obj).visc_max_iterations = n; });
}

double FluidSimulation_get_viscosity(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).viscosity; });
}

double FluidSimulation_get_surface_tension(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).surface_tension; });
}

void FluidSimulation_set_surface_tension(FluidSimulation *obj, double k, int *err) {
    guarded(err, [&] {
        if (k < 0.0)
            throw std::domain_error("Error: surface tension must be greater than or equal to 0.\nsurface tension: " +
                                    std::to_string(k) + "\n");
        E(obj).surface_tension = k;
    });
}

double FluidSimulation_get_surface_tension_condition_number(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).tension_cfl; });
}

void FluidSimulation_set_surface_tension_condition_number(FluidSimulation *obj, double n, int *err) {
    guarded(err, [&] {
        if (n <= 0.0)
            throw std::domain_error("Error: condition number must be greater than 0.0.\nnumber: " + std::to_string(n) +
                                    "\n");
        E(obj).tension_cfl = n;
    });
}

void FluidSimulation_set_viscosity(FluidSimulation *obj, double v, int *err) {
    guarded(err, [&] {
        if (v < 0.0)
            throw std::domain_error("Error: viscosity must be greater than or equal to 0.\nviscosity: " +
                                    std::to_string(v) + "\n");
        Engine &e = E(obj);
        e.viscosity_enabled = true;
        e.viscosity = v;
    });
}

double FluidSimulation_get_viscosity_solver_error_tolerance(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).visc_tolerance; });
}

void FluidSimulation_set_viscosity_solver_error_tolerance(FluidSimulation *obj, double tol, int *err) {
    guarded(err, [&] {
        if (tol < 0.0)
            throw std::domain_error("Error: viscosity solver error tolerance must be greater than or equal to 0.\n"
                                    "error tolerance: " + std::to_string(tol) + "\n");
        E(obj).visc_tolerance = tol;
    });
}

void FluidSimulation_set_velocity_transfer_method_APIC(FluidSimulation *obj, int *err) {
    guarded(err, [&] { E(obj).apic = true; });
}

int FluidSimulation_is_velocity_transfer_method_FLIP(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).apic ? 0 : 1; });
}

int FluidSimulation_is_velocity_transfer_method_APIC(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).apic ? 1 : 0; });
}

double FluidSimulation_get_PICAPIC_ratio(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).pic_apic_ratio; });
}

void FluidSimulation_set_PICAPIC_ratio(FluidSimulation *obj, double ratio, int *err) {
    guarded(err, [&] {
        if (ratio < 0.0 || ratio > 1.0) throw std::domain_error("Error: PICAPIC ratio must be in range [0.0, 1.0].\n");
        E(obj).pic_apic_ratio = ratio;
    });
}

double FluidSimulation_get_PICFLIP_ratio(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).pic_ratio; });
}

void FluidSimulation_set_PICFLIP_ratio(FluidSimulation *obj, double ratio, int *err) {
    guarded(err, [&] {
        if (ratio < 0.0 || ratio > 1.0) throw std::domain_error("Error: PICFLIP ratio must be in range [0.0, 1.0].\n");
        E(obj).pic_ratio = ratio;
    });
}

int FluidSimulation_get_num_marker_particles(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return E(obj).num_particles(); });
}

unsigned int FluidSimulation_get_marker_particle_position_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (unsigned int)(E(obj).num_particles() * 3 * sizeof(float)); });
}

unsigned int FluidSimulation_get_marker_particle_velocity_data_size(FluidSimulation *obj, int *err) {
    return guarded(err, [&] { return (unsigned int)(E(obj).num_particles() * 3 * sizeof(float)); });
}

FluidSimulationFrameStats FluidSimulation_get_frame_stats_data(FluidSimulation *obj, int *err) {
    return guarded(err, [&] {
        Engine &e = E(obj);
        FluidSimulationFrameStats s;
        std::memset(&s, 0, sizeof(s));
        FluidSimulationMeshStats ms{0, -1, -1, 0};
        FluidSimulationMeshStats *m = &s.surface;
        FluidSimulationMeshStats *mend = &s.forcefield;
        for (; m <= mend; m++) *m = ms;
        s.frame = e.current_frame - 1;
        s.substeps = e.frame_substeps;
        s.deltaTime = e.last_frame_dt;
        s.fluidParticles = e.num_particles();
        s.performanceScore = e.performance_score;
        s.pressureSolverEnabled = 1;
        s.pressureSolverSuccess = e.frame_solve.success ? 1 : 0;
        s.pressureSolverError = (double)(float)e.frame_solve.error;
        s.pressureSolverIterations = e.frame_solve.iterations;
        s.pressureSolverMaxIterations = e.max_iterations;
        s.viscositySolverEnabled = e.viscosity_enabled ? 1 : 0;
        s.viscositySolverSuccess = e.frame_visc.success ? 1 : 0;
        s.viscositySolverError = (double)e.frame_visc.error;
        s.viscositySolverIterations = e.frame_visc.iterations;
        s.viscositySolverMaxIterations = e.visc_max_iterations;
        s.timing.total = e.frame_time;
        s.timing.pressure = 0.0;
        return s;
    });
}

void FluidSimulation_get_marker_particle_position_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                             char *c_data, int *err) {
    guarded(err, [&] { E(obj).get_positions(reinterpret_cast<float *>(c_data), start_idx, end_idx); });
}

void FluidSimulation_get_marker_particle_velocity_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                             char *c_data, int *err) {
    guarded(err, [&] { E(obj).get_velocities(reinterpret_cast<float *>(c_data), start_idx, end_idx); });
}

void FluidSimulation_get_marker_particle_affinex_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err) {
    guarded(err, [&] { E(obj).get_affine(0, reinterpret_cast<float *>(c_data), start_idx, end_idx); });
}

void FluidSimulation_get_marker_particle_affiney_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err) {
    guarded(err, [&] { E(obj).get_affine(1, reinterpret_cast<float *>(c_data), start_idx, end_idx); });
}

void FluidSimulation_get_marker_particle_affinez_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err) {
    guarded(err, [&] { E(obj).get_affine(2, reinterpret_cast<float *>(c_data), start_idx, end_idx); });
}

void FluidSimulation_get_marker_particle_position_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { Engine &e = E(obj); e.get_positions(reinterpret_cast<float *>(c_data), 0, e.num_particles()); });
}

void FluidSimulation_get_marker_particle_velocity_data(FluidSimulation *obj, char *c_data, int *err) {
    guarded(err, [&] { Engine &e = E(obj); e.get_velocities(reinterpret_cast<float *>(c_data), 0, e.num_particles()); });
}

void FluidSimulation_load_marker_particle_data(FluidSimulation *obj, FluidSimulationMarkerParticleData data, int *err) {
    guarded(err, [&] {
        if (data.size < 0) throw std::domain_error("Error: particle count must be non-negative.\n");
        if (data.size == 0) return;
        E(obj).load_particles(reinterpret_cast<const float *>(data.positions),
                              reinterpret_cast<const float *>(data.velocities), data.size);
    });
}

void FluidSimulation_load_marker_particle_affine_data(FluidSimulation *obj, FluidSimulationMarkerParticleAffineData data,
                                                      int *err) {
    guarded(err, [&] {
        if (data.size < 0) throw std::domain_error("Error: affine data count must be non-negative.\n");
        E(obj).load_affine(reinterpret_cast<const float *>(data.affineX), reinterpret_cast<const float *>(data.affineY),
                           reinterpret_cast<const float *>(data.affineZ), data.size);
    });
}

}  // extern "C"
