// Oracle (test infrastructure only): one full substep in the reference's stage order
// (FluidSimulation::_stepFluid, fluidsimulation.cpp:10078-10121) for a static solid level
// set, unit density, FLIP or APIC transfer, no surface tension, viscosity or whitewater.
#include "oracle.h"

#include <cmath>
#include <vector>

extern "C" {
void oracle_liquid_sdf(int, int, int, double, double, int, const float *, float *);
void oracle_postprocess_sdf(int, int, int, double, const float *, float *);
void oracle_p2g_component(int, int, int, double, double, int, const float *, const float *, int, float *, unsigned char *);
void oracle_extrapolate(int, int, int, float *, const unsigned char *, int);
void oracle_body_force(int, int, int, double, float, float, float, float *, float *, float *);
void oracle_face_weights(int, int, int, const float *, float *, float *, float *);
int oracle_pressure_solve(int, int, int, double, double, const float *, const float *, const float *, const float *,
                          const float *, const float *, const float *, double, int, int, float *, int *, double *);
void oracle_apply_pressure(int, int, int, double, double, const float *, const float *, const float *, const float *,
                           const float *, float *, float *, float *, unsigned char *, unsigned char *, unsigned char *);
void oracle_apply_pressure_tension(int, int, int, double, double, const float *, const float *, const float *,
                                   const float *, const float *, const float *, double, float *, float *, float *,
                                   unsigned char *, unsigned char *, unsigned char *);
void oracle_constrain(int, int, int, const float *, const float *, const float *, float *, float *, float *);
void oracle_g2p(int, int, int, double, double, int, const float *, float *, const float *, const float *,
                const float *, const float *, const float *, const float *);
void oracle_advect(int, int, int, double, double, int, int, const float *, const float *, const float *,
                   const float *, const float *, float *);
int oracle_remove(int, int, int, double, int, float *, float *, const float *, int);
int oracle_remove_attr(int, int, int, double, int, float *, float *, float *, int, const float *, int);
float oracle_speed_limit(int, const float *, double, double, double, int);
int oracle_remove_extreme(int, int, int, double, int, float *, float *, const float *, int, float);
void oracle_p2g_apic_component(int, int, int, double, double, int, const float *, const float *, const float *, int,
                               float *, unsigned char *);
void oracle_g2p_apic(int, int, int, double, int, const float *, float *, float *, const float *, const float *,
                     const float *);
void oracle_curvature_grid(int, int, int, double, const float *, float *, float *);
int oracle_pressure_solve_tension(int, int, int, double, double, const float *, const float *, const float *,
                                  const float *, const float *, const float *, const float *, const float *, double,
                                  double, int, int, float *, int *, double *);
void oracle_viscosity(int, int, int, double, double, const float *, const float *, const float *, double, int, float *,
                      float *, float *, int *, float *, float *, int *, unsigned *, unsigned *, float *, float *,
                      float *, unsigned *, unsigned *, float *, float *);

// Advances np particles (pos/vel, in/out) by one substep of length dt.  solid_phi is the
// nodal (ni+1)(nj+1)(nk+1) solid level set.  stats <- {pressure iterations, success,
// fluid cells}; *err <- final pressure residual.  Returns the new particle count.
// aff9 (9 floats per particle, in/out) selects the APIC transfer when not null
// (velocityadvector.cpp:543-623, fluidsimulation.cpp:6791-6843); otherwise PIC/FLIP.
// visc > 0 applies the viscosity solve with that constant viscosity after the body force
// (fluidsimulation.cpp:5983-6064: velocity constraint, then ViscositySolver with tolerance 1e-4
// and at most 900 iterations).
int oracle_substep_tension(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                           float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                           float *aff9, double visc, double tension, int *stats, double *err);

int oracle_substep_full(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                        float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                        float *aff9, double visc, int *stats, double *err) {
    return oracle_substep_tension(ni, nj, nk, dx, dt, pic, cfl, gx, gy, gz, solid_phi, tol, maxit, np, pos, vel, aff9,
                                  visc, 0.0, stats, err);
}

static int substep_impl(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                        float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                        float *aff9, double visc, double tension, double evr_frame_dt, int evr_max_steps, int *stats,
                        double *err);

// tension > 0 adds surface tension: the curvature grid of the post-processed liquid level set
// (particlelevelset.cpp:196-291) and the ghost-fluid tension term in the pressure rhs
// (pressuresolver.cpp:314-749)
int oracle_substep_tension(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                           float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                           float *aff9, double visc, double tension, int *stats, double *err) {
    return substep_impl(ni, nj, nk, dx, dt, pic, cfl, gx, gy, gz, solid_phi, tol, maxit, np, pos, vel, aff9, visc,
                        tension, 0.0, 0, stats, err);
}

// A PIC/FLIP substep with extreme-velocity removal on (the engine's default): the removal
// applies the speed limit of the post-transfer velocities for an update of length frame_dt
// with at most max_steps substeps (fluidsimulation.cpp:7723-7851; the engine passes the
// frame's delta time, :7892).
int oracle_substep_evr(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                       float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                       double frame_dt, int max_steps, int *stats, double *err) {
    return substep_impl(ni, nj, nk, dx, dt, pic, cfl, gx, gy, gz, solid_phi, tol, maxit, np, pos, vel, nullptr, 0.0,
                        0.0, frame_dt, max_steps, stats, err);
}

static int substep_impl(int ni, int nj, int nk, double dx, double dt, double pic, int cfl, float gx, float gy,
                        float gz, const float *solid_phi, double tol, int maxit, int np, float *pos, float *vel,
                        float *aff9, double visc, double tension, double evr_frame_dt, int evr_max_steps, int *stats,
                        double *err) {
    size_t nc = (size_t)ni * nj * nk;
    size_t nu = (size_t)(ni + 1) * nj * nk, nv = (size_t)ni * (nj + 1) * nk, nw = (size_t)ni * nj * (nk + 1);
    std::vector<float> wu(nu), wv(nv), ww(nw);
    oracle_face_weights(ni, nj, nk, solid_phi, wu.data(), wv.data(), ww.data());
    double radius = 0.5 * 1.0 * dx * std::sqrt(3.0);   // fluidsimulation.cpp:4351
    std::vector<float> phi(nc);
    oracle_liquid_sdf(ni, nj, nk, dx, radius, np, pos, phi.data());
    oracle_postprocess_sdf(ni, nj, nk, dx, solid_phi, phi.data());
    std::vector<float> u(nu), v(nv), w(nw);
    std::vector<unsigned char> vu(nu), vv(nv), vw(nw);
    if (aff9) {
        oracle_p2g_apic_component(ni, nj, nk, dx, radius, np, pos, vel, aff9, 0, u.data(), vu.data());
        oracle_p2g_apic_component(ni, nj, nk, dx, radius, np, pos, vel, aff9, 1, v.data(), vv.data());
        oracle_p2g_apic_component(ni, nj, nk, dx, radius, np, pos, vel, aff9, 2, w.data(), vw.data());
    } else {
        oracle_p2g_component(ni, nj, nk, dx, radius, np, pos, vel, 0, u.data(), vu.data());
        oracle_p2g_component(ni, nj, nk, dx, radius, np, pos, vel, 1, v.data(), vv.data());
        oracle_p2g_component(ni, nj, nk, dx, radius, np, pos, vel, 2, w.data(), vw.data());
    }
    int layers = (int)std::ceil(std::sqrt(3) * cfl) + 3;   // fluidsimulation.cpp:6284
    oracle_extrapolate(ni + 1, nj, nk, u.data(), vu.data(), layers);
    oracle_extrapolate(ni, nj + 1, nk, v.data(), vv.data(), layers);
    oracle_extrapolate(ni, nj, nk + 1, w.data(), vw.data(), layers);
    std::vector<float> su = u, sv = v, sw = w;   // _saveVelocityField
    oracle_body_force(ni, nj, nk, dt, gx, gy, gz, u.data(), v.data(), w.data());
    if (visc > 0) {
        oracle_constrain(ni, nj, nk, wu.data(), wv.data(), ww.data(), u.data(), v.data(), w.data());
        std::vector<float> vg((size_t)(ni + 1) * (nj + 1) * (nk + 1), (float)visc);
        int vst[3];
        float verr;
        oracle_viscosity(ni, nj, nk, dx, dt, phi.data(), solid_phi, vg.data(), 1e-4, 900, u.data(), v.data(), w.data(),
                         vst, &verr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr, nullptr,
                         nullptr, nullptr);
    }
    std::vector<float> pressure(nc);
    int pst[2] = {0, 1};
    double perr = 0.0;
    int ncells;
    std::vector<float> surf, curv;
    if (tension > 0) {
        surf.resize(nc); curv.resize(nc);
        oracle_curvature_grid(ni, nj, nk, dx, phi.data(), surf.data(), curv.data());
        ncells = oracle_pressure_solve_tension(ni, nj, nk, dx, dt, phi.data(), wu.data(), wv.data(), ww.data(), u.data(),
                                               v.data(), w.data(), curv.data(), tension, tol, maxit, 1, pressure.data(),
                                               pst, &perr);
    } else {
        ncells = oracle_pressure_solve(ni, nj, nk, dx, dt, phi.data(), wu.data(), wv.data(), ww.data(), u.data(),
                                       v.data(), w.data(), tol, maxit, 1, pressure.data(), pst, &perr);
    }
    if (pst[1]) {
        oracle_apply_pressure_tension(ni, nj, nk, dx, dt, phi.data(), wu.data(), wv.data(), ww.data(), pressure.data(),
                                      tension > 0 ? curv.data() : nullptr, tension, u.data(), v.data(), w.data(),
                                      vu.data(), vv.data(), vw.data());
    }
    oracle_extrapolate(ni + 1, nj, nk, u.data(), vu.data(), layers);
    oracle_extrapolate(ni, nj + 1, nk, v.data(), vv.data(), layers);
    oracle_extrapolate(ni, nj, nk + 1, w.data(), vw.data(), layers);
    oracle_constrain(ni, nj, nk, wu.data(), wv.data(), ww.data(), su.data(), sv.data(), sw.data());
    oracle_constrain(ni, nj, nk, wu.data(), wv.data(), ww.data(), u.data(), v.data(), w.data());
    if (aff9) oracle_g2p_apic(ni, nj, nk, dx, np, pos, vel, aff9, u.data(), v.data(), w.data());
    else oracle_g2p(ni, nj, nk, dx, pic, np, pos, vel, u.data(), v.data(), w.data(), su.data(), sv.data(), sw.data());
    std::vector<float> np_pos(3 * (size_t)np);
    oracle_advect(ni, nj, nk, dx, dt, cfl, np, pos, u.data(), v.data(), w.data(), solid_phi, np_pos.data());
    for (size_t t = 0; t < np_pos.size(); t++) pos[t] = np_pos[t];
    int out;
    if (evr_frame_dt > 0.0) {
        float limit = oracle_speed_limit(np, vel, cfl, dx, evr_frame_dt, evr_max_steps);
        out = oracle_remove_extreme(ni, nj, nk, dx, np, pos, vel, solid_phi, 250, limit);
    } else {
        out = oracle_remove_attr(ni, nj, nk, dx, np, pos, vel, aff9, 9, solid_phi, 250);
    }
    stats[0] = pst[0]; stats[1] = pst[1]; stats[2] = ncells;
    *err = perr;
    return out;
}

int oracle_substep_transfer(int ni, int nj, int nk, double dx, double dt, double pic, int cfl,
                            float gx, float gy, float gz, const float *solid_phi, double tol, int maxit,
                            int np, float *pos, float *vel, float *aff9, int *stats, double *err) {
    return oracle_substep_full(ni, nj, nk, dx, dt, pic, cfl, gx, gy, gz, solid_phi, tol, maxit, np, pos, vel, aff9,
                               0.0, stats, err);
}

int oracle_substep(int ni, int nj, int nk, double dx, double dt, double pic, int cfl,
                   float gx, float gy, float gz, const float *solid_phi, double tol, int maxit,
                   int np, float *pos, float *vel, int *stats, double *err) {
    return oracle_substep_transfer(ni, nj, nk, dx, dt, pic, cfl, gx, gy, gz, solid_phi, tol, maxit, np, pos, vel,
                                   nullptr, stats, err);
}

}  // extern "C"
