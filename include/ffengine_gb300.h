/*
 * C ABI of the GB300 FLIP substep library (libffengine_gb300.so).
 *
 * Part 1 is the drop-in subset of the FLIP Fluids engine's C API
 * (rlguy/Blender-FLIP-Fluids src/engine/c_bindings/fluidsimulation_c.cpp): same names,
 * same argument meaning, same error convention -- every call but _destroy takes a
 * trailing `int *err`, set to 1 on success and 0 on failure, with the message readable
 * through CBindings_get_error_message() (src/engine/c_bindings/cbindings.cpp:35-44,101).
 * The reference's ctypes loader picks the longest library name starting with
 * "libffengine" (src/engine/ffengine/ffengine.py:59-107), so this library is selected
 * without changes to the caller.
 *
 * Part 2 adds GB300 entry points with no reference counterpart: solver selection,
 * statistics, particle replacement, analytic obstacles, and stage-level functions that
 * run one kernel group on host arrays (used by the parity tests).
 *
 * Grids are x-fastest (index i + ni*(j + nj*k)); face grids are (ni+1)*nj*nk (U),
 * ni*(nj+1)*nk (V), ni*nj*(nk+1) (W); the solid level set is nodal (ni+1)(nj+1)(nk+1).
 */
#ifndef FFENGINE_GB300_H
#define FFENGINE_GB300_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct FluidSimulation FluidSimulation;   /* opaque handle */
typedef struct MeshObject MeshObject;             /* opaque handle */

/* meshutils.h:34-39 */
typedef struct TriangleMesh_t {
    float *vertices;     /* numVertices * 3 float32, interleaved xyz */
    int *triangles;      /* numTriangles * 3 vertex indices */
    int numVertices;
    int numTriangles;
} TriangleMesh_t;

/* fluidsimulation.h:153-157 */
typedef struct FluidSimulationMarkerParticleData {
    int size;
    char *positions;    /* size * 3 float32, interleaved xyz */
    char *velocities;   /* size * 3 float32 */
} FluidSimulationMarkerParticleData;

/* fluidsimulation.h:159-164: three arrays of size xyz float32 triples, the affine vectors of the
 * x, y and z velocity components */
typedef struct FluidSimulationMarkerParticleAffineData {
    int size;
    char *affineX;
    char *affineY;
    char *affineZ;
} FluidSimulationMarkerParticleAffineData;

/* fluidsimulation.h:201-204: size uint16 particle ids */
typedef struct FluidSimulationMarkerParticleIDData {
    int size;
    char *id;
} FluidSimulationMarkerParticleIDData;

/* fluidsimulation.h:62-78 */
typedef struct FluidSimulationMeshStats {
    int enabled;
    int vertices;
    int triangles;
    unsigned int bytes;
} FluidSimulationMeshStats;

typedef struct FluidSimulationTimingStats {
    double total, mesh, advection, particles, pressure, diffuse, viscosity, objects;
} FluidSimulationTimingStats;

/* fluidsimulation.h:80-152 (field order and types preserved for by-value ABI) */
typedef struct FluidSimulationFrameStats {
    int frame;
    int substeps;
    double deltaTime;
    int fluidParticles;
    int diffuseParticles;
    int performanceScore;
    int pressureSolverEnabled;
    int pressureSolverSuccess;
    double pressureSolverError;
    int pressureSolverIterations;
    int pressureSolverMaxIterations;
    int viscositySolverEnabled;
    int viscositySolverSuccess;
    double viscositySolverError;
    int viscositySolverIterations;
    int viscositySolverMaxIterations;
    FluidSimulationMeshStats surface, preview, surfaceblur, surfacevelocity, surfacevorticity, surfacespeed,
        surfaceage, surfacelifetime, surfacewhitewaterproximity, surfacecolor, surfacesourceid,
        surfaceviscosity, surfacedensity, foam, bubble, spray, dust, foamblur, bubbleblur, sprayblur,
        dustblur, foamvelocity, bubblevelocity, sprayvelocity, dustvelocity, foamid, bubbleid, sprayid,
        dustid, foamlifetime, bubblelifetime, spraylifetime, dustlifetime, fluidparticles,
        fluidparticlesid, fluidparticlesuid, fluidparticlesvelocity, fluidparticlesspeed,
        fluidparticlesvorticity, fluidparticlescolor, fluidparticlesage, fluidparticleslifetime,
        fluidparticlesviscosity, fluidparticlesdensity, fluidparticlesdensityaverage,
        fluidparticleswhitewaterproximity, fluidparticlessourceid, particles, obstacle, forcefield;
    FluidSimulationTimingStats timing;
} FluidSimulationFrameStats;

/* ---------------- Part 1: drop-in subset (fluidsimulation_c.cpp) ---------------- */
char *CBindings_get_error_message(void);                                                 /* cbindings.cpp:101 */
FluidSimulation *FluidSimulation_new_from_dimensions(int isize, int jsize, int ksize, double dx, int *err); /* :56 */
void FluidSimulation_destroy(FluidSimulation *obj);                                       /* :71 */
void FluidSimulation_get_version(FluidSimulation *obj, int *major, int *minor, int *revision, int *err); /* :75 */
void FluidSimulation_initialize(FluidSimulation *obj, int *err);                         /* :97 */
int FluidSimulation_is_initialized(FluidSimulation *obj, int *err);                      /* :101 */
void FluidSimulation_update(FluidSimulation *obj, double dt, int *err);                  /* :115 */
int FluidSimulation_get_current_frame(FluidSimulation *obj, int *err);                   /* :121 */
double FluidSimulation_get_cell_size(FluidSimulation *obj, int *err);                    /* :155 */
void FluidSimulation_get_grid_dimensions(FluidSimulation *obj, int *i, int *j, int *k, int *err); /* :161 */
void FluidSimulation_get_simulation_dimensions(FluidSimulation *obj, double *width, double *height,
                                               double *depth, int *err);                 /* :186 */
int FluidSimulation_get_pressure_solver_max_iterations(FluidSimulation *obj, int *err);  /* :318 */
void FluidSimulation_set_pressure_solver_max_iterations(FluidSimulation *obj, int n, int *err); /* :325 */
void FluidSimulation_enable_console_output(FluidSimulation *obj, int *err);              /* :586 */
void FluidSimulation_disable_console_output(FluidSimulation *obj, int *err);             /* :593 */
void FluidSimulation_enable_surface_reconstruction(FluidSimulation *obj, int *err);      /* :607 */
void FluidSimulation_disable_surface_reconstruction(FluidSimulation *obj, int *err);     /* :614 */
int FluidSimulation_get_max_thread_count(FluidSimulation *obj, int *err);                /* :2583 */
void FluidSimulation_set_max_thread_count(FluidSimulation *obj, int n, int *err);        /* :2591 */
void FluidSimulation_add_body_force(FluidSimulation *obj, double fx, double fy, double fz, int *err); /* :2599 */
void FluidSimulation_reset_body_force(FluidSimulation *obj, int *err);                   /* :2615 */
int FluidSimulation_get_CFL_condition_number(FluidSimulation *obj, int *err);            /* :2825 */
void FluidSimulation_set_CFL_condition_number(FluidSimulation *obj, int n, int *err);    /* :2833 */
int FluidSimulation_get_min_time_steps_per_frame(FluidSimulation *obj, int *err);        /* :2878 */
void FluidSimulation_set_min_time_steps_per_frame(FluidSimulation *obj, int n, int *err); /* :2886 */
int FluidSimulation_get_max_time_steps_per_frame(FluidSimulation *obj, int *err);        /* :2894 */
void FluidSimulation_set_max_time_steps_per_frame(FluidSimulation *obj, int n, int *err); /* :2902 */
void FluidSimulation_enable_extreme_velocity_removal(FluidSimulation *obj, int *err);    /* :2952 */
void FluidSimulation_disable_extreme_velocity_removal(FluidSimulation *obj, int *err);   /* :2959 */
void FluidSimulation_set_velocity_transfer_method_FLIP(FluidSimulation *obj, int *err);  /* :2973 */
/* Viscosity solve before the pressure projection (fluidsimulation.cpp:5983-6064,
 * viscositysolver.cpp): setting a viscosity enables it; a constant viscosity field */
int FluidSimulation_get_viscosity_solver_max_iterations(FluidSimulation *obj, int *err);  /* :333 */
void FluidSimulation_set_viscosity_solver_max_iterations(FluidSimulation *obj, int n, int *err); /* :340 */
double FluidSimulation_get_surface_tension(FluidSimulation *obj, int *err);              /* :2757 */
void FluidSimulation_set_surface_tension(FluidSimulation *obj, double k, int *err);      /* :2763 */
double FluidSimulation_get_surface_tension_condition_number(FluidSimulation *obj, int *err); /* :2841 */
void FluidSimulation_set_surface_tension_condition_number(FluidSimulation *obj, double n, int *err); /* :2849 */
double FluidSimulation_get_viscosity(FluidSimulation *obj, int *err);                    /* :2728 */
void FluidSimulation_set_viscosity(FluidSimulation *obj, double v, int *err);            /* :2734 */
double FluidSimulation_get_viscosity_solver_error_tolerance(FluidSimulation *obj, int *err); /* :2742 */
void FluidSimulation_set_viscosity_solver_error_tolerance(FluidSimulation *obj, double tol, int *err); /* :2748 */
/* APIC transfer (velocityadvector.cpp:543-623, fluidsimulation.cpp:6791-6843); select it before
 * FluidSimulation_initialize for loaded affine data to be kept */
void FluidSimulation_set_velocity_transfer_method_APIC(FluidSimulation *obj, int *err);  /* :2980 */
int FluidSimulation_is_velocity_transfer_method_FLIP(FluidSimulation *obj, int *err);    /* :2987 */
int FluidSimulation_is_velocity_transfer_method_APIC(FluidSimulation *obj, int *err);    /* :2994 */
double FluidSimulation_get_PICAPIC_ratio(FluidSimulation *obj, int *err);                /* :3014 */
void FluidSimulation_set_PICAPIC_ratio(FluidSimulation *obj, double ratio, int *err);    /* :3020 */
double FluidSimulation_get_PICFLIP_ratio(FluidSimulation *obj, int *err);                /* :3001 */
void FluidSimulation_set_PICFLIP_ratio(FluidSimulation *obj, double ratio, int *err);    /* :3007 */
int FluidSimulation_get_num_marker_particles(FluidSimulation *obj, int *err);            /* :3151 */
unsigned int FluidSimulation_get_marker_particle_position_data_size(FluidSimulation *obj, int *err); /* :3952 */
unsigned int FluidSimulation_get_marker_particle_velocity_data_size(FluidSimulation *obj, int *err); /* :3958 */
FluidSimulationFrameStats FluidSimulation_get_frame_stats_data(FluidSimulation *obj, int *err); /* :4618 */
void FluidSimulation_get_marker_particle_position_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                             char *c_data, int *err);    /* :4625 */
void FluidSimulation_get_marker_particle_velocity_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                             char *c_data, int *err);    /* :4636 */
/* affine vectors (xyz float32 triples) of particles [start_idx, end_idx); APIC only */
void FluidSimulation_get_marker_particle_affinex_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err);     /* :4647 */
void FluidSimulation_get_marker_particle_affiney_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err);     /* :4658 */
void FluidSimulation_get_marker_particle_affinez_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                            char *c_data, int *err);     /* :4669 */
void FluidSimulation_get_marker_particle_position_data(FluidSimulation *obj, char *c_data, int *err); /* :4823 */
void FluidSimulation_get_marker_particle_velocity_data(FluidSimulation *obj, char *c_data, int *err); /* :4830 */
void FluidSimulation_load_marker_particle_data(FluidSimulation *obj, FluidSimulationMarkerParticleData data,
                                               int *err);                                /* :4872 */
void FluidSimulation_load_marker_particle_affine_data(FluidSimulation *obj,
                                                      FluidSimulationMarkerParticleAffineData data,
                                                      int *err);                         /* :4880 */

/* FFP3 fluid-particle output (fluidsimulation.cpp:9477-9800): enabling it gives the particles a
 * uint16 id (loaded with load_marker_particle_id_data, paired with the particle batch of the same
 * position and size, else random) and, after the first substep of every update, an FFP3 output of
 * the particles grouped surface / boundary / interior, then by id, for ids below
 * round(65536 * output amount).  The bytes stay on the device until read; sizes are 0 before the
 * first output and for attributes that are off.  The meshing volume, the source-id blacklist and
 * the domain offset / scale (identity here) are not part of this output. */
void FluidSimulation_enable_fluid_particle_output(FluidSimulation *obj, int *err);                /* :348 */
void FluidSimulation_disable_fluid_particle_output(FluidSimulation *obj, int *err);               /* :355 */
int FluidSimulation_is_fluid_particle_output_enabled(FluidSimulation *obj, int *err);             /* :362 */
double FluidSimulation_get_fluid_particle_output_amount(FluidSimulation *obj, int *err);          /* :369 */
void FluidSimulation_set_fluid_particle_output_amount(FluidSimulation *obj, double value, int *err); /* :375 */
void FluidSimulation_enable_fluid_particle_surface_output(FluidSimulation *obj, int *err);        /* :381 */
void FluidSimulation_disable_fluid_particle_surface_output(FluidSimulation *obj, int *err);       /* :388 */
int FluidSimulation_is_fluid_particle_surface_output_enabled(FluidSimulation *obj, int *err);     /* :395 */
void FluidSimulation_enable_fluid_particle_boundary_output(FluidSimulation *obj, int *err);       /* :402 */
void FluidSimulation_disable_fluid_particle_boundary_output(FluidSimulation *obj, int *err);      /* :409 */
int FluidSimulation_is_fluid_particle_boundary_output_enabled(FluidSimulation *obj, int *err);    /* :416 */
void FluidSimulation_enable_fluid_particle_interior_output(FluidSimulation *obj, int *err);       /* :423 */
void FluidSimulation_disable_fluid_particle_interior_output(FluidSimulation *obj, int *err);      /* :430 */
int FluidSimulation_is_fluid_particle_interior_output_enabled(FluidSimulation *obj, int *err);    /* :437 */
void FluidSimulation_enable_fluid_particle_velocity_attribute(FluidSimulation *obj, int *err);    /* :833 */
void FluidSimulation_disable_fluid_particle_velocity_attribute(FluidSimulation *obj, int *err);   /* :840 */
int FluidSimulation_is_fluid_particle_velocity_attribute_enabled(FluidSimulation *obj, int *err); /* :847 */
void FluidSimulation_enable_fluid_particle_speed_attribute(FluidSimulation *obj, int *err);       /* :854 */
void FluidSimulation_disable_fluid_particle_speed_attribute(FluidSimulation *obj, int *err);      /* :861 */
int FluidSimulation_is_fluid_particle_speed_attribute_enabled(FluidSimulation *obj, int *err);    /* :868 */
int FluidSimulation_get_fluid_particle_data_size(FluidSimulation *obj, int *err);                 /* :3716 */
int FluidSimulation_get_fluid_particle_id_attribute_data_size(FluidSimulation *obj, int *err);    /* :3729 */
int FluidSimulation_get_fluid_particle_velocity_attribute_data_size(FluidSimulation *obj, int *err); /* :3742 */
int FluidSimulation_get_fluid_particle_speed_attribute_data_size(FluidSimulation *obj, int *err); /* :3755 */
void FluidSimulation_get_fluid_particle_data(FluidSimulation *obj, char *c_data, int *err);       /* :4402 */
void FluidSimulation_get_fluid_particle_id_attribute_data(FluidSimulation *obj, char *c_data, int *err); /* :4414 */
void FluidSimulation_get_fluid_particle_velocity_attribute_data(FluidSimulation *obj, char *c_data,
                                                                int *err);                       /* :4426 */
void FluidSimulation_get_fluid_particle_speed_attribute_data(FluidSimulation *obj, char *c_data, int *err); /* :4438 */
void FluidSimulation_load_marker_particle_id_data(FluidSimulation *obj, FluidSimulationMarkerParticleIDData data,
                                                  int *err);                                     /* :4944 */
void FluidSimulation_get_marker_particle_id_data_range(FluidSimulation *obj, int start_idx, int end_idx,
                                                       char *c_data, int *err);                  /* :4757 */

/* ---------------- Part 2: GB300 extensions (no reference counterpart) ---------------- */
/* Pressure solver: 0 = FP64 PCG with the reference's MIC(0) and float step lengths,
 * 1 = mixed precision (FP32 PCG inner solve, FP64 dots, FP64 iterative refinement). */
void FluidSimulation_gb300_set_pressure_solver_mode(FluidSimulation *obj, int mode, int *err);
/* The reference's tolerance (1e-9, inf-norm relative to ||b||_inf) has no C setter. */
void FluidSimulation_gb300_set_pressure_solver_tolerance(FluidSimulation *obj, double tol, int *err);
/* Mixed-precision mode: reliable-update factor in (0, 1).  The FP32 iteration folds its
 * iterate into the FP64 solution and restarts from the FP64 true residual (keeping its search
 * direction) whenever its own residual has dropped by this factor (default 0.1). */
void FluidSimulation_gb300_set_mixed_inner_tolerance(FluidSimulation *obj, double rel, int *err);
/* Static analytic sphere obstacle (centre, radius) added to the solid level set; call before initialize. */
void FluidSimulation_gb300_add_sphere_obstacle(FluidSimulation *obj, double cx, double cy, double cz, double r, int *err);
/* Replaces the static solid level set with a caller-computed nodal one (e.g. a mesh SDF). */
void FluidSimulation_gb300_set_solid_level_set(FluidSimulation *obj, const float *phi, int *err);
/* Replaces the marker particles from host buffers (positions/velocities interleaved xyz). */
void FluidSimulation_gb300_set_marker_particle_data(FluidSimulation *obj, FluidSimulationMarkerParticleData data, int *err);
/* out[0..5]: iterations, success, outer passes, box cells, error, relative residual of the last substep. */
void FluidSimulation_gb300_get_pressure_solver_stats(FluidSimulation *obj, double *out6, int *err);
/* Enables per-stage CUDA-event timing; out[0..11] in ms (sort, sdf, p2g, extrap, build, factor, pcg,
 * project, g2p, advect, remove, total) of the last substep. */
/* Save-state particle files (the bake script's format, bake.py:2864-2905): attribute 0 position,
 * 1 velocity, 2/3/4 affine x/y/z, written as interleaved float32 xyz in particle order straight
 * from device memory (chunks of 2^21 particles through two pinned buffers, copy overlapping the
 * write); append != 0 appends to the file. */
void FluidSimulation_gb300_write_marker_particle_file(FluidSimulation *obj, int attribute, const char *path,
                                                      int append, int *err);
/* Reads save-state files back as the bake script's loader does (bake.py:554-721): chunks of 2^21
 * particles, each one load_marker_particle_data batch and, when the three affine paths are
 * given, one load_marker_particle_affine_data batch.  Returns the number of particles read. */
long long FluidSimulation_gb300_load_marker_particle_files(FluidSimulation *obj, const char *position_path,
                                                           const char *velocity_path, const char *affinex_path,
                                                           const char *affiney_path, const char *affinez_path,
                                                           int *err);
/* Error report of every solve against an FP64 reference solve (reference_tolerance > 0; 0 turns
 * it off).  Each substep then also solves its pressure system with the FP64 PCG -- same operator,
 * same FP64 MIC(0) factor -- to ||b - A p||_inf <= reference_tolerance * ||b||_inf, projects the
 * velocity field with that pressure into separate buffers and compares; the substep itself keeps
 * its own solve.  get_solve_check gives, for the last substep: {valid, pressure relative L2,
 * velocity relative L2 over the projected faces, max weighted divergence after the projection /
 * ||b||_inf, the same for the reference-projected field, ||b||_inf, reference iterations,
 * reference relative residual}. */
void FluidSimulation_gb300_set_solve_check(FluidSimulation *obj, double reference_tolerance, int *err);
void FluidSimulation_gb300_get_solve_check(FluidSimulation *obj, double *out8, int *err);
/* Lengths of the last update's substeps, in order (FluidSimulation::update's CFL substepping,
 * fluidsimulation.cpp:10455-10470): writes up to `capacity` of them into out (may be NULL) and
 * returns how many there were. */
int FluidSimulation_gb300_get_frame_substep_times(FluidSimulation *obj, double *out, int capacity, int *err);
/* viscosity solve of the last substep: {rows, iterations, final residual, success} */
void FluidSimulation_gb300_get_viscosity_solver_stats(FluidSimulation *obj, double *out, int *err);
/* with stage timing on (FluidSimulation_gb300_enable_stage_timing): milliseconds of the last
 * viscosity solve's system build, factor (and preconditioner setup) and PCG iterations */
void FluidSimulation_gb300_get_viscosity_solver_times(FluidSimulation *obj, float *out, int *err);
void FluidSimulation_gb300_enable_stage_timing(FluidSimulation *obj, int enable, int *err);
void FluidSimulation_gb300_get_stage_times(FluidSimulation *obj, float *out12, int *err);
/* Number of kernels this handle has launched so far. */
unsigned long long FluidSimulation_gb300_get_kernel_launch_count(FluidSimulation *obj, int *err);
/* Runs k substeps of length dt and returns their device time in ms (CUDA events on the
 * engine's stream). */
float FluidSimulation_gb300_run_substeps_timed(FluidSimulation *obj, int k, double dt, int *err);
/* Re-runs one kernel group `reps` times on the current state and returns its mean device
 * time in ms; *bytes receives its algorithmic bytes per run.  Ids: 0 P2G (U component),
 * 1 liquid SDF, 2 FP32 SpMV + dot (operator as hi + lo floats), 3 FP32 MIC(0) forward + backward substitution,
 * 4 extrapolation (U, all layers), 5 G2P, 6 RK3 advection + collision, 7 particle sort. */
float FluidSimulation_gb300_time_kernel(FluidSimulation *obj, int kernel_id, int reps, double *bytes, int *err);
/* Differentiable substep: one substep without marker removal that records the transfer
 * weights, extrapolation layers and solver operator, so that FluidSimulation_gb300_adjoint
 * can map dL/dv1 (particle velocities after the substep) to dL/dv0 (before it).  With
 * grad_v1 == NULL the loss is L = mean over particles with y > loss_ymin of vy^2 (after the
 * substep) and the return value is the number of those particles.  Host arrays are
 * interleaved xyz float32.  The adjoint's projection is a second PCG solve on the same
 * operator and MIC(0) factor, to the adjoint tolerance. */
void FluidSimulation_gb300_substep_differentiable(FluidSimulation *obj, double dt, int *err);
int FluidSimulation_gb300_adjoint(FluidSimulation *obj, const float *grad_v1, double loss_ymin, float *grad_v0,
                                  int *err);
void FluidSimulation_gb300_set_adjoint_tolerance(FluidSimulation *obj, double tol, int *err);
/* Differentiable rollout: k differentiable substeps of length dt from the current particle
 * state, keeping a device checkpoint of (x, v) before each (24 bytes per particle per substep).
 * The particle state afterwards is the rollout's final state. */
void FluidSimulation_gb300_rollout_forward(FluidSimulation *obj, int k, double dt, int *err);
/* Maps dL/dx_k and dL/dv_k (the state after the rollout) to dL/dx_0 and dL/dv_0, walking the
 * substeps backwards and recomputing each from its checkpoint.  Host arrays are interleaved
 * xyz float32 in particle order.  grad_xk == NULL means zero; grad_vk == NULL selects the
 * built-in loss, mean vy^2 over particles with y > loss_ymin after the rollout, and the
 * return value is the number of those particles (otherwise -1).  NULL outputs are skipped. */
int FluidSimulation_gb300_rollout_adjoint(FluidSimulation *obj, const float *grad_xk, const float *grad_vk,
                                          double loss_ymin, float *grad_x0, float *grad_v0, int *err);
/* k x (differentiable substep + the adjoint of one rollout substep: the built-in loss on v1
 * and a non-zero position cotangent); device time in ms. */
float FluidSimulation_gb300_run_forward_adjoint_timed(FluidSimulation *obj, int k, double dt, double loss_ymin,
                                                      int *err);
/* Runs exactly one substep of length dt (no CFL substepping). */
void FluidSimulation_gb300_substep(FluidSimulation *obj, double dt, int *err);

/* Stage-level functions on host arrays (one kernel group each). */
void ffgpu_solid_phi(int ni, int nj, int nk, double dx, int nspheres, const double *spheres, float *phi, int *err);
void ffgpu_face_weights(int ni, int nj, int nk, const float *solid, float *wu, float *wv, float *ww, int *err);
void ffgpu_sort_particles(int ni, int nj, int nk, double dx, int np, const float *pos, int *cell_start,
                          int *sorted_index, int *err);
void ffgpu_liquid_sdf(int ni, int nj, int nk, double dx, int np, const float *pos, const float *solid,
                      int postprocess, float *phi, int *err);
void ffgpu_p2g(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, float *u, float *v,
               float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err);
/* as ffgpu_p2g with one launch per component (the differentiable substep's kernel); the three-component
 * pass ffgpu_p2g runs gives the same values bit for bit */
void ffgpu_p2g_components(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, float *u,
                          float *v, float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err);
void ffgpu_extrapolate(int w, int h, int d, float *grid, const unsigned char *valid, int layers, int *err);
/* mode: bit 0 mixed precision (else FP64), bit 1 apply MIC(0) one i+j+k hyperplane per launch
 * (else the pipelined wavefront kernel), bit 2 keep the grid's axis order in the mixed solve (else
 * the shortest box axis is swept, FluidSimulation_gb300_set_pressure_axis_order).  stats: iterations, success, outer passes, box cells;
 * errs: error, relative FP64 residual, ||b||_inf */
void ffgpu_pressure_solve(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                          const float *wv, const float *ww, const float *u, const float *v, const float *w,
                          double tol, int maxit, int mode, float *pressure, double *pressure64, int *stats,
                          double *errs, int *err);
void ffgpu_apply_pressure(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                          const float *wv, const float *ww, const float *pressure, float *u, float *v, float *w,
                          unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err);
void ffgpu_g2p(int ni, int nj, int nk, double dx, double pic, int np, const float *pos, float *vel, const float *u,
               const float *v, const float *w, const float *su, const float *sv, const float *sw, int *err);
void ffgpu_advect(int ni, int nj, int nk, double dx, double dt, int cfl, int np, const float *pos, const float *u,
                  const float *v, const float *w, const float *solid, float *out, int *err);
int ffgpu_remove(int ni, int nj, int nk, double dx, int np, float *pos, float *vel, const float *solid,
                 int max_per_cell, int *err);
/* Axis order of the mixed-precision solve: 1 (default) runs it in a copy of the pressure box whose
 * shortest axis is the one the MIC(0) wavefront sweeps, when that axis is under 4/5 of the box's z
 * extent; 0 keeps the grid's order.  The FP64 solver always keeps the grid's order. */
void FluidSimulation_gb300_set_pressure_axis_order(FluidSimulation *obj, int mode, int *err);
/* 2 (default): the mixed-precision solve starts from the linear extrapolation in time of the last
 * two substeps' pressures on the current pressure cells (p dt extrapolated, with the substep lengths;
 * the last pressure alone until two are known) instead of zero; the stopping rule (relative to
 * ||b||_inf) is unchanged.  1: from the previous substep's pressure, scaled by the ratio of the
 * substep lengths.  0: zero start, as the reference's PCG.  Other values fail with a domain error. */
void FluidSimulation_gb300_set_pressure_warm_start(FluidSimulation *obj, int on, int *err);
/* 1 (default): the mixed-precision solve replays its batches of iterations (8 a host check) from a CUDA
 * graph captured once per solve; 0: launches them one by one.  The results are the same bit for bit. */
void FluidSimulation_gb300_set_pcg_graphs(FluidSimulation *obj, int on, int *err);
/* MIC(0) preconditioner of the viscosity solve: 0 (default) each velocity component's block swept by
 * the tiled wavefront of the pressure solve along its box's shortest axis, the couplings between
 * components applied between the sweeps; 1 one launch per level of the reference's row order; 2 those
 * levels in one cooperative launch; 3 as 0 but swept along the grid's z axis.  Forms 1, 2 and 3 give
 * a bit-identical forward sweep; 3's backward sweep applies the couplings to the later components
 * before a row's own neighbours, and 0 also subtracts a row's own neighbours in its box's axis order
 * (other rounding orders of the same operator). */
void FluidSimulation_gb300_set_viscosity_preconditioner(FluidSimulation *obj, int form, int *err);
/* 1 (default): the viscosity solve's PCG starts from the velocity field before the solve (each row's
 * face value) instead of zero; the stop stays |r|inf <= tolerance * |b|inf, the zero start's, so the
 * solution meets the same accuracy with fewer iterations.  0: zero start, as the reference's
 * ViscositySolver (its iteration counts). */
void FluidSimulation_gb300_set_viscosity_warm_start(FluidSimulation *obj, int on, int *err);

/* Failure handling.  set_wait_limit: polls before a wait of the MIC(0) factor or wavefront
 * preconditioner kernels gives up (0 restores the default of about a second); a wait that gives up
 * makes the pressure solve fail with *err = 0 and the message "... wavefront wait timed out ...",
 * and the handle stays usable.  inject_allocation_failure: the after-th next device allocation of
 * any engine in the process fails as if the device were out of memory (0 cancels). */
void FluidSimulation_gb300_set_wait_limit(FluidSimulation *obj, long long polls, int *err);
void ffgpu_inject_allocation_failure(long long after, int *err);
/* One wavefront wait on a flag that nothing sets, bounded by limit polls (1 .. 2^24): returns the
 * error bits the kernel raised (1: the wait timed out); the device context stays usable. */
int ffgpu_wait_probe(long long limit, int *err);

/* Surface tension stages on host arrays (ni*nj*nk cell grids).  curvature_grid: the curvature
 * grid of a post-processed liquid level set (ParticleLevelSet::calculateCurvatureGrid,
 * particlelevelset.cpp:196-291) and its re-initialised surface level set.  cluster_status: the
 * per-cell status of PressureSolver::_initializeSurfaceTensionClusterData (pressuresolver.cpp:314-605):
 * 0x01 / 0x02 ok inside / outside, 0x04 / 0x08 bad inside / outside, 0x10 border.
 * pressure_solve_tension / apply_pressure_tension: ffgpu_pressure_solve / ffgpu_apply_pressure with
 * the surface tension term of the curvature grid and constant k_st (pressuresolver.cpp:659-749, 1047-1205). */
void ffgpu_curvature_grid(int ni, int nj, int nk, double dx, const float *phi, float *surface_phi, float *curvature,
                          int *err);
void ffgpu_cluster_status(int ni, int nj, int nk, const float *phi, unsigned char *status, int *err);
void ffgpu_pressure_solve_tension(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                                  const float *wv, const float *ww, const float *u, const float *v, const float *w,
                                  const float *curvature, double k_st, double tol, int maxit, int mode,
                                  float *pressure, double *pressure64, int *stats, double *errs, int *err);
void ffgpu_apply_pressure_tension(int ni, int nj, int nk, double dx, double dt, const float *phi, const float *wu,
                                  const float *wv, const float *ww, const float *pressure, const float *curvature,
                                  double k_st, float *u, float *v, float *w, unsigned char *vu, unsigned char *vv,
                                  unsigned char *vw, int *err);
/* Mesh obstacles (meshobject_c.cpp:38-192, fluidsimulation_c.cpp:3113-3134).  Static meshes only:
 * MeshObject_update_mesh_animated fails.  The obstacle is copied on update and read before each
 * substep; the solid level set (domain box and obstacles) is rebuilt on the GPU when the obstacle
 * list, a mesh or a switch changed. */
MeshObject *MeshObject_new(int i, int j, int k, double dx, int *err);                        /* :38 */
void MeshObject_destroy(MeshObject *obj);                                                    /* :52 */
void MeshObject_update_mesh_static(MeshObject *obj, TriangleMesh_t mesh_data, int *err);     /* :56 */
void MeshObject_update_mesh_animated(MeshObject *obj, TriangleMesh_t mesh_data_previous,
                                     TriangleMesh_t mesh_data_current, TriangleMesh_t mesh_data_next,
                                     int *err);                                              /* :71 */
void MeshObject_enable(MeshObject *obj, int *err);                                           /* :90 */
void MeshObject_disable(MeshObject *obj, int *err);                                          /* :96 */
int MeshObject_is_enabled(MeshObject *obj, int *err);                                        /* :102 */
void MeshObject_inverse(MeshObject *obj, int *err);                                          /* :108 */
int MeshObject_is_inversed(MeshObject *obj, int *err);                                       /* :114 */
float MeshObject_get_friction(MeshObject *obj, int *err);                                    /* :120 */
void MeshObject_set_friction(MeshObject *obj, float f, int *err);                            /* :126 */
float MeshObject_get_mesh_expansion(MeshObject *obj, int *err);                              /* :180 */
void MeshObject_set_mesh_expansion(MeshObject *obj, float ex, int *err);                     /* :186 */
void FluidSimulation_add_mesh_obstacle(FluidSimulation *obj, MeshObject *obstacle, int *err);    /* :3113 */
void FluidSimulation_remove_mesh_obstacle(FluidSimulation *obj, MeshObject *obstacle, int *err); /* :3121 */
void FluidSimulation_remove_mesh_obstacles(FluidSimulation *obj, int *err);                     /* :3129 */

/* Solid level set (nodal, (ni+1)(nj+1)(nk+1)) of the closed domain and nobj static meshes given as
 * concatenated arrays (object o: nverts[o] xyz vertices, ntris[o] triangles indexing its own
 * vertices; flags[o] bit0 inverted, bit1 disabled; expansion[o] its mesh expansion), as the solid
 * level set the engine builds (fluidsimulation.cpp:5277-5333).  jitter: njitter xyz offsets of the
 * inside tests' z lines in call order, the fixed offset after that. */
void ffgpu_solid_level_set(int ni, int nj, int nk, double dx, int nobj, const int *nverts, const int *ntris,
                           const float *verts, const int *tris, const int *flags, const float *expansion,
                           int njitter, const float *jitter, float *phi, int *err);

/* Marker removal with the extreme-velocity rule on (fluidsimulation.cpp:7723-7851): the speed
 * limit of an update of length frame_dt allowing max_substeps substeps at this CFL number is
 * written to *limit; returns the new particle count. */
int ffgpu_remove_extreme(int ni, int nj, int nk, double dx, int np, float *pos, float *vel, const float *solid,
                         int max_per_cell, double frame_dt, int cfl, int max_substeps, float *limit, int *err);
/* Pressure-cell classification (pressuresolver.cpp:138-147): fluid[c] = 1 for interior cells with
 * liquid phi < 0, else 0 (ni*nj*nk bytes); bbox6 = {i0, j0, k0, i1, j1, k1} of those cells
 * ({INT_MAX x3, -1 x3} when there are none). */
void ffgpu_classify(int ni, int nj, int nk, const float *phi, unsigned char *fluid, int *bbox6, int *err);
/* One full substep on host arrays; solid may be NULL (closed box); mode as ffgpu_pressure_solve;
 * returns the new particle count. */
int ffgpu_substep(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy, float gz,
                  const float *solid, double tol, int maxit, int mode, int np, float *pos, float *vel, int *stats,
                  double *errs, int *err);
/* APIC stages: aff9 holds 9 float32 per particle, component c's affine vector at 3c .. 3c+2. */
void ffgpu_p2g_apic(int ni, int nj, int nk, double dx, int np, const float *pos, const float *vel, const float *aff9,
                    float *u, float *v, float *w, unsigned char *vu, unsigned char *vv, unsigned char *vw, int *err);
/* vel and aff9 are outputs (the PIC velocity and the affine vectors); inputs read for the load only */
void ffgpu_g2p_apic(int ni, int nj, int nk, double dx, int np, const float *pos, float *vel, float *aff9,
                    const float *u, const float *v, const float *w, int *err);
/* Viscosity solve on host arrays (constrained u, v, w in/out; liquid: cell-centred level set,
 * solid: nodal level set, visc: constant viscosity).  stats <- {rows, iterations, success};
 * *res <- final residual.  Optional outputs (NULL to skip), sized as the oracle's: the seven
 * volume grids (centre, U, V, W, edgeU, edgeV, edgeW), the face -> row table, the system
 * (CSR: rows + 1, 15 rows, 15 rows), rhs, the MIC(0) factor (pivots, column starts, row indices,
 * values of the lower part by columns) and the solution. */
void ffgpu_viscosity(int ni, int nj, int nk, double dx, double dt, const float *liquid, const float *solid,
                     double visc, double tol, int maxit, float *u, float *v, float *w, int *stats, float *res,
                     float *vol7, int *index, unsigned *rowstart, unsigned *col, float *val, float *rhs,
                     float *ic_invdiag, unsigned *ic_colstart, unsigned *ic_rowindex, float *ic_value, float *soln,
                     int *err);
/* FFP3 output of the given particles (positions in the domain; ids uint16) as an update writes it
 * after its first substep (liquid level set post-processed against solid, its surface level set,
 * classification, grouping).  flags: bit0..2 surface, boundary, interior output, bit3 velocity, bit4
 * speed attribute.  Four outputs (positions, ids, velocities, speeds) of at least
 * 16 + 12 * 65536 + 12 np bytes; sizes <- their byte counts (0: not produced); types (optional)
 * <- per particle 0 surface, 1 boundary, 2 interior, 3 unset. */
void ffgpu_ffp3(int ni, int nj, int nk, double dx, const float *solid, int np, const float *pos, const float *vel,
                const uint16_t *ids, int flags, double amount, char *out_pos, char *out_id, char *out_vel,
                char *out_speed, long long *sizes, unsigned char *types, int *err);
/* The viscosity system and MIC(0) factor of the same inputs, then one preconditioner application to
 * the system's right-hand side: form 0 tiled wavefront blocks, 1 per-level launches, 2 one cooperative
 * launch (both sweeps only), 3 tiled wavefront blocks swept along the grid's z axis; sweeps 1 = L z = b,
 * 2 = (L L^T) z = b.  z <- the rows' values (as many
 * as the system has rows, at most the face count); returns the row count. */
int ffgpu_viscosity_precondition(int ni, int nj, int nk, double dx, double dt, const float *liquid,
                                 const float *solid, double visc, const float *u, const float *v, const float *w,
                                 int form, int sweeps, float *z, int *err);
int ffgpu_substep_apic(int ni, int nj, int nk, double dx, double dt, int cfl, float gx, float gy, float gz,
                       const float *solid, double tol, int maxit, int mode, int np, float *pos, float *vel, float *aff9,
                       int *stats, double *errs, int *err);

/* Allocation-free layered extrapolation (no counterpart in the reference engine).
 * Same result as ffgpu_extrapolate, but on caller-owned DEVICE buffers (grid: w*h*d float32,
 * updated in place; valid: w*h*d bytes) on the caller's CUDA stream (cudaStream_t passed as
 * void*, NULL = default stream), and it allocates nothing: no cudaMalloc/cudaFree and no
 * allocating library call.  It is for callers that cannot allocate device memory while they
 * run: hosts whose device memory belongs to another framework's pool, and real-time loops
 * that forbid allocator calls after set-up (an allocation can block for milliseconds).
 * Limit: w*h*d <= 4,194,304 cells (4 Mi); larger grids are rejected with an error.  Its
 * scratch is a fixed 8 MiB device array inside the library, held by every GPU that loads the
 * library until the process exits.  The first call on each device looks up that array's
 * device address (cudaGetSymbolAddress) and keeps it for the life of the process, so do not
 * call it again on a device after cudaDeviceReset; make that first call before any stream
 * capture.  A CUDA error still pending from an earlier call makes it fail without launching.
 * All calls share the array: calls that overlap on the GPU (different streams, or threads
 * without ordering) race and corrupt each other's results -- serialise them. */
void ffgpu_extrapolate_noalloc(int w, int h, int d, float *grid, const unsigned char *valid, int layers,
                               void *stream, int *err);

#ifdef __cplusplus
}
#endif
#endif
