// Shared pieces of the C ABI translation units: the opaque handle and the error guard
// that turns C++ exceptions into the reference's (*err, message) convention.
#pragma once
#include <exception>
#include <stdexcept>
#include <type_traits>

#include "../../include/ffengine_gb300.h"
#include "engine.h"

struct FluidSimulation {
    ffgpu::Engine eng;
    FluidSimulation(int i, int j, int k, double dx) : eng(i, j, k, dx) {}
};

// MeshObject handle (meshobject.h): a static obstacle mesh and its switches
struct MeshObject {
    ffgpu::Obstacle ob;
    int ni, nj, nk;
    double dx;
};

namespace ffgpu {

void set_error(const std::exception &ex);

template <typename F>
auto guarded(int *err, F f) -> decltype(f()) {
    using R = decltype(f());
    if (err) *err = 1;
    try {
        return f();
    } catch (const std::exception &ex) {
        set_error(ex);
        if (err) *err = 0;
    } catch (...) {
        set_error(std::runtime_error("unknown error"));
        if (err) *err = 0;
    }
    if constexpr (!std::is_void<R>::value) return R{};
}

inline Engine &E(FluidSimulation *o) {
    if (!o) throw std::invalid_argument("Error: FluidSimulation handle is null.\n");
    return o->eng;
}

}  // namespace ffgpu
