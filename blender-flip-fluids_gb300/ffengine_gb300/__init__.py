"""Python host side of the GB300 FLIP substep library.

Mirrors the part of the reference's ctypes package (rlguy/Blender-FLIP-Fluids
src/engine/ffengine/fluidsimulation.py) that drives the simulation update: the same
method and property names, the same argument meaning, and the same error behaviour
(a failing C call raises RuntimeError with the library's message, as
src/engine/ffengine/pybindings.py:26-31 does).  All computation happens in
libffengine_gb300.so on the GPU; there is no CPU fallback: if the library cannot be
loaded, every call raises LibraryLoadError.
"""
import ctypes
import os
from ctypes import byref, c_char, c_char_p, c_double, c_float, c_int, c_longlong, c_uint, c_ulonglong, c_void_p

LIB_DIR = os.path.join(os.path.dirname(os.path.abspath(__file__)), "lib")
LIB_NAME = "libffengine_gb300.so"


class LibraryLoadError(Exception):
    pass


_lib = None


def library_path():
    """ffengine_gb300/lib/libffengine_gb300.so, or the file named by FFENGINE_GB300_LIBRARY."""
    return os.environ.get("FFENGINE_GB300_LIBRARY") or os.path.join(LIB_DIR, LIB_NAME)


def load_library():
    """Loads libffengine_gb300.so from ffengine_gb300/lib (built by ffengine_gb300.build)."""
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise LibraryLoadError("Cannot find fluid engine library <%s>: build it with "
                                   "ffengine_gb300.build.build()" % path)
        _lib = ctypes.CDLL(path)
    return _lib


class _Lib:
    def __getattr__(self, name):
        return getattr(load_library(), name)


lib = _Lib()


def _check(success, prefix):
    if not success.value:
        f = load_library().CBindings_get_error_message
        f.restype = c_char_p
        raise RuntimeError(prefix + f().decode("utf-8"))


def call(name, argtypes, restype, *args):
    """Calls a C-ABI function with the trailing int* err and raises on failure."""
    f = getattr(load_library(), name)
    f.argtypes = list(argtypes) + [c_void_p]
    f.restype = restype
    err = c_int(1)
    r = f(*args, byref(err))
    _check(err, name + " - ")
    return r


class FluidSimulationMarkerParticleData_t(ctypes.Structure):
    _fields_ = [("size", c_int), ("positions", c_char_p), ("velocities", c_char_p)]


class FluidSimulationMarkerParticleAffineData_t(ctypes.Structure):
    _fields_ = [("size", c_int), ("affinex", c_char_p), ("affiney", c_char_p), ("affinez", c_char_p)]


class FluidSimulationMarkerParticleIDData_t(ctypes.Structure):
    _fields_ = [("size", c_int), ("id", c_char_p)]


class FluidSimulationMeshStats_t(ctypes.Structure):
    _fields_ = [("enabled", c_int), ("vertices", c_int), ("triangles", c_int), ("bytes", c_uint)]


class FluidSimulationTimingStats_t(ctypes.Structure):
    _fields_ = [(n, c_double) for n in ("total", "mesh", "advection", "particles", "pressure", "diffuse",
                                          "viscosity", "objects")]


_MESH_STATS = ("surface preview surfaceblur surfacevelocity surfacevorticity surfacespeed surfaceage "
               "surfacelifetime surfacewhitewaterproximity surfacecolor surfacesourceid surfaceviscosity "
               "surfacedensity foam bubble spray dust foamblur bubbleblur sprayblur dustblur foamvelocity "
               "bubblevelocity sprayvelocity dustvelocity foamid bubbleid sprayid dustid foamlifetime "
               "bubblelifetime spraylifetime dustlifetime fluidparticles fluidparticlesid fluidparticlesuid "
               "fluidparticlesvelocity fluidparticlesspeed fluidparticlesvorticity fluidparticlescolor "
               "fluidparticlesage fluidparticleslifetime fluidparticlesviscosity fluidparticlesdensity "
               "fluidparticlesdensityaverage fluidparticleswhitewaterproximity fluidparticlessourceid "
               "particles obstacle forcefield").split()


class FluidSimulationFrameStats_t(ctypes.Structure):
    _fields_ = ([("frame", c_int), ("substeps", c_int), ("deltaTime", c_double), ("fluidParticles", c_int),
                 ("diffuseParticles", c_int), ("performanceScore", c_int), ("pressureSolverEnabled", c_int),
                 ("pressureSolverSuccess", c_int), ("pressureSolverError", c_double),
                 ("pressureSolverIterations", c_int), ("pressureSolverMaxIterations", c_int),
                 ("viscositySolverEnabled", c_int), ("viscositySolverSuccess", c_int),
                 ("viscositySolverError", c_double), ("viscositySolverIterations", c_int),
                 ("viscositySolverMaxIterations", c_int)]
                + [(n, FluidSimulationMeshStats_t) for n in _MESH_STATS]
                + [("timing", FluidSimulationTimingStats_t)])


class TriangleMesh_t(ctypes.Structure):
    """meshutils.h:34-39 (the reference's trianglemesh.py TriangleMesh_t)."""
    _fields_ = [("vertices", c_void_p), ("triangles", c_void_p), ("num_vertices", c_int),
                ("num_triangles", c_int)]


class TriangleMesh:
    """Vertices (x, y, z float32 triples) and triangles (three int32 vertex indices), as the
    reference's ffengine.TriangleMesh; `to_struct` keeps the arrays alive on the struct."""

    def __init__(self, vertices=(), triangles=()):
        import array
        self.vertices = array.array("f", [float(x) for x in _flat(vertices)])
        self.triangles = array.array("i", [int(x) for x in _flat(triangles)])

    def translate(self, tx, ty, tz):
        for i in range(0, len(self.vertices), 3):
            self.vertices[i] += tx
            self.vertices[i + 1] += ty
            self.vertices[i + 2] += tz

    def scale(self, s):
        for i in range(len(self.vertices)):
            self.vertices[i] *= s

    def to_struct(self):
        vdata = (ctypes.c_float * len(self.vertices)).from_buffer_copy(self.vertices.tobytes()) \
            if len(self.vertices) else (ctypes.c_float * 1)()
        tdata = (ctypes.c_int * len(self.triangles)).from_buffer_copy(self.triangles.tobytes()) \
            if len(self.triangles) else (ctypes.c_int * 1)()
        st = TriangleMesh_t(ctypes.cast(vdata, c_void_p), ctypes.cast(tdata, c_void_p), len(self.vertices) // 3,
                            len(self.triangles) // 3)
        st._keep = (vdata, tdata)
        return st


def _flat(a):
    try:
        import numpy as np
        return np.asarray(a).reshape(-1).tolist()
    except ImportError:
        return [x for row in a for x in (row if hasattr(row, "__len__") else [row])]


class MeshObject:
    """GB300 counterpart of ffengine.MeshObject (meshobject.py) for static obstacles."""

    def __init__(self, i, j, k, dx):
        f = load_library().MeshObject_new
        f.argtypes = [c_int, c_int, c_int, c_double, c_void_p]
        f.restype = c_void_p
        err = c_int(1)
        self._obj = f(int(i), int(j), int(k), float(dx), byref(err))
        _check(err, "MeshObject_new - ")

    def __call__(self):
        return self._obj

    def __del__(self):
        obj = getattr(self, "_obj", None)
        if obj:
            f = load_library().MeshObject_destroy
            f.argtypes = [c_void_p]
            f.restype = None
            f(obj)
            self._obj = None

    def _m(self, name, *args, argtypes=(), restype=None):
        return call("MeshObject_" + name, [c_void_p] + list(argtypes), restype, self._obj, *args)

    def update_mesh_static(self, mesh):
        self._m("update_mesh_static", mesh.to_struct(), argtypes=[TriangleMesh_t])

    def update_mesh_animated(self, mesh_previous, mesh_current, mesh_next):
        self._m("update_mesh_animated", mesh_previous.to_struct(), mesh_current.to_struct(), mesh_next.to_struct(),
                argtypes=[TriangleMesh_t] * 3)

    @property
    def enable(self):
        return bool(self._m("is_enabled", restype=c_int))

    @enable.setter
    def enable(self, on):
        self._m("enable" if on else "disable")

    @property
    def inverse(self):
        return bool(self._m("is_inversed", restype=c_int))

    @inverse.setter
    def inverse(self, on):
        if bool(on) != self.inverse:
            self._m("inverse")

    @property
    def friction(self):
        return self._m("get_friction", restype=c_float)

    @friction.setter
    def friction(self, value):
        self._m("set_friction", float(value), argtypes=[c_float])

    @property
    def mesh_expansion(self):
        return self._m("get_mesh_expansion", restype=c_float)

    @mesh_expansion.setter
    def mesh_expansion(self, value):
        self._m("set_mesh_expansion", float(value), argtypes=[c_float])


class FluidSimulation:
    """GB300 counterpart of ffengine.FluidSimulation for the simulation-update path."""

    def __init__(self, isize, jsize, ksize, dx):
        if not all(isinstance(x, int) for x in (isize, jsize, ksize)):
            raise TypeError("FluidSimulation must be initialized with int grid dimensions and a real dx")
        f = load_library().FluidSimulation_new_from_dimensions
        f.argtypes = [c_int, c_int, c_int, c_double, c_void_p]
        f.restype = c_void_p
        err = c_int(1)
        self._obj = f(isize, jsize, ksize, float(dx), byref(err))
        _check(err, "FluidSimulation_new_from_dimensions - ")

    def __call__(self):
        return self._obj

    def __del__(self):
        obj = getattr(self, "_obj", None)
        if obj:
            f = load_library().FluidSimulation_destroy
            f.argtypes = [c_void_p]
            f.restype = None
            f(obj)
            self._obj = None

    def _v(self, name, *args, argtypes=(), restype=None):
        return call("FluidSimulation_" + name, [c_void_p] + list(argtypes), restype, self._obj, *args)

    # lifecycle (fluidsimulation.py:116-145)
    def initialize(self):
        self._v("initialize")

    def is_initialized(self):
        return bool(self._v("is_initialized", restype=c_int))

    def update(self, dt):
        self._v("update", dt, argtypes=[c_double])

    def get_current_frame(self):
        return self._v("get_current_frame", restype=c_int)

    def get_version(self):
        a, b, c = c_int(), c_int(), c_int()
        self._v("get_version", byref(a), byref(b), byref(c), argtypes=[c_void_p, c_void_p, c_void_p])
        return a.value, b.value, c.value

    # configuration
    @property
    def pressure_solver_max_iterations(self):
        return self._v("get_pressure_solver_max_iterations", restype=c_int)

    @pressure_solver_max_iterations.setter
    def pressure_solver_max_iterations(self, n):
        self._v("set_pressure_solver_max_iterations", int(n), argtypes=[c_int])

    @property
    def CFL_condition_number(self):
        return self._v("get_CFL_condition_number", restype=c_int)

    @CFL_condition_number.setter
    def CFL_condition_number(self, n):
        self._v("set_CFL_condition_number", int(n), argtypes=[c_int])

    @property
    def min_time_steps_per_frame(self):
        return self._v("get_min_time_steps_per_frame", restype=c_int)

    @min_time_steps_per_frame.setter
    def min_time_steps_per_frame(self, n):
        self._v("set_min_time_steps_per_frame", int(n), argtypes=[c_int])

    @property
    def max_time_steps_per_frame(self):
        return self._v("get_max_time_steps_per_frame", restype=c_int)

    @max_time_steps_per_frame.setter
    def max_time_steps_per_frame(self, n):
        self._v("set_max_time_steps_per_frame", int(n), argtypes=[c_int])

    @property
    def PICFLIP_ratio(self):
        return self._v("get_PICFLIP_ratio", restype=c_double)

    @PICFLIP_ratio.setter
    def PICFLIP_ratio(self, r):
        self._v("set_PICFLIP_ratio", float(r), argtypes=[c_double])

    @property
    def enable_extreme_velocity_removal(self):
        raise AttributeError("write-only in this library")

    @enable_extreme_velocity_removal.setter
    def enable_extreme_velocity_removal(self, boolval):
        self._v("enable_extreme_velocity_removal" if boolval else "disable_extreme_velocity_removal")

    def set_velocity_transfer_method_FLIP(self):
        self._v("set_velocity_transfer_method_FLIP")

    def set_velocity_transfer_method_APIC(self):
        self._v("set_velocity_transfer_method_APIC")

    def is_velocity_transfer_method_FLIP(self):
        return bool(self._v("is_velocity_transfer_method_FLIP", restype=c_int))

    def is_velocity_transfer_method_APIC(self):
        return bool(self._v("is_velocity_transfer_method_APIC", restype=c_int))

    @property
    def viscosity(self):
        return self._v("get_viscosity", restype=c_double)

    @viscosity.setter
    def viscosity(self, value):
        self._v("set_viscosity", float(value), argtypes=[c_double])

    @property
    def surface_tension(self):
        return self._v("get_surface_tension", restype=c_double)

    @surface_tension.setter
    def surface_tension(self, value):
        self._v("set_surface_tension", float(value), argtypes=[c_double])

    @property
    def surface_tension_condition_number(self):
        return self._v("get_surface_tension_condition_number", restype=c_double)

    @surface_tension_condition_number.setter
    def surface_tension_condition_number(self, value):
        self._v("set_surface_tension_condition_number", float(value), argtypes=[c_double])

    @property
    def viscosity_solver_error_tolerance(self):
        return self._v("get_viscosity_solver_error_tolerance", restype=c_double)

    @viscosity_solver_error_tolerance.setter
    def viscosity_solver_error_tolerance(self, value):
        self._v("set_viscosity_solver_error_tolerance", float(value), argtypes=[c_double])

    @property
    def viscosity_solver_max_iterations(self):
        return self._v("get_viscosity_solver_max_iterations", restype=c_int)

    @viscosity_solver_max_iterations.setter
    def viscosity_solver_max_iterations(self, n):
        self._v("set_viscosity_solver_max_iterations", int(n), argtypes=[c_int])

    @property
    def PICAPIC_ratio(self):
        return self._v("get_PICAPIC_ratio", restype=c_double)

    @PICAPIC_ratio.setter
    def PICAPIC_ratio(self, r):
        self._v("set_PICAPIC_ratio", float(r), argtypes=[c_double])

    def add_body_force(self, fx, fy, fz):
        self._v("add_body_force", float(fx), float(fy), float(fz), argtypes=[c_double] * 3)

    def reset_body_force(self):
        self._v("reset_body_force")

    @property
    def enable_surface_reconstruction(self):
        raise AttributeError("write-only in this library")

    @enable_surface_reconstruction.setter
    def enable_surface_reconstruction(self, boolval):
        self._v("enable_surface_reconstruction" if boolval else "disable_surface_reconstruction")

    @property
    def enable_console_output(self):
        raise AttributeError("write-only in this library")

    @enable_console_output.setter
    def enable_console_output(self, boolval):
        self._v("enable_console_output" if boolval else "disable_console_output")

    # particles (fluidsimulation.py:2610, 2934-2938, 3092-3103)
    def get_num_marker_particles(self):
        return self._v("get_num_marker_particles", restype=c_int)

    def load_marker_particle_data(self, num_particles, position_data, velocity_data):
        c_pos = (c_char * len(position_data)).from_buffer_copy(position_data)
        c_vel = (c_char * len(velocity_data)).from_buffer_copy(velocity_data)
        d = FluidSimulationMarkerParticleData_t()
        d.size = c_int(num_particles)
        d.positions = ctypes.cast(c_pos, c_char_p)
        d.velocities = ctypes.cast(c_vel, c_char_p)
        self._v("load_marker_particle_data", d, argtypes=[FluidSimulationMarkerParticleData_t])

    def load_marker_particle_affine_data(self, num_particles, affinex_data, affiney_data, affinez_data):
        bufs = [(c_char * len(b)).from_buffer_copy(b) for b in (affinex_data, affiney_data, affinez_data)]
        d = FluidSimulationMarkerParticleAffineData_t()
        d.size = c_int(num_particles)
        d.affinex, d.affiney, d.affinez = (ctypes.cast(b, c_char_p) for b in bufs)
        self._v("load_marker_particle_affine_data", d, argtypes=[FluidSimulationMarkerParticleAffineData_t])

    def load_marker_particle_id_data(self, num_particles, id_data):
        c_id = (c_char * len(id_data)).from_buffer_copy(id_data)
        d = FluidSimulationMarkerParticleIDData_t()
        d.size = c_int(num_particles)
        d.id = ctypes.cast(c_id, c_char_p)
        self._v("load_marker_particle_id_data", d, argtypes=[FluidSimulationMarkerParticleIDData_t])

    def get_marker_particle_id_data_range(self, start_idx, end_idx):
        buf = (c_char * (max(end_idx - start_idx, 0) * 2))()
        self._v("get_marker_particle_id_data_range", start_idx, end_idx, buf, argtypes=[c_int, c_int, c_void_p])
        return bytes(buf)

    # FFP3 fluid-particle output (fluidsimulation.py:349-420, 718-747, 2855-2869)
    def _toggle(name):
        def get(self):
            return bool(self._v("is_" + name + "_enabled", restype=c_int))

        def put(self, boolval):
            self._v(("enable_" if boolval else "disable_") + name)
        return property(get, put)

    enable_fluid_particle_output = _toggle("fluid_particle_output")
    enable_fluid_particle_surface_output = _toggle("fluid_particle_surface_output")
    enable_fluid_particle_boundary_output = _toggle("fluid_particle_boundary_output")
    enable_fluid_particle_interior_output = _toggle("fluid_particle_interior_output")
    enable_fluid_particle_velocity_attribute = _toggle("fluid_particle_velocity_attribute")
    enable_fluid_particle_speed_attribute = _toggle("fluid_particle_speed_attribute")
    del _toggle

    @property
    def fluid_particle_output_amount(self):
        return self._v("get_fluid_particle_output_amount", restype=c_double)

    @fluid_particle_output_amount.setter
    def fluid_particle_output_amount(self, value):
        self._v("set_fluid_particle_output_amount", float(value), argtypes=[c_double])

    def get_fluid_particle_data(self):
        return self._output("get_fluid_particle_data")

    def get_fluid_particle_id_attribute_data(self):
        return self._output("get_fluid_particle_id_attribute_data")

    def get_fluid_particle_velocity_attribute_data(self):
        return self._output("get_fluid_particle_velocity_attribute_data")

    def get_fluid_particle_speed_attribute_data(self):
        return self._output("get_fluid_particle_speed_attribute_data")

    def _output(self, name):
        size = self._v(name + "_size", restype=c_uint)
        buf = (c_char * size)()
        self._v(name, buf, argtypes=[c_void_p])
        return bytes(buf)

    def get_marker_particle_position_data(self):
        return self._output("get_marker_particle_position_data")

    def get_marker_particle_velocity_data(self):
        return self._output("get_marker_particle_velocity_data")

    def get_marker_particle_position_data_range(self, start_idx, end_idx):
        buf = (c_char * ((end_idx - start_idx) * 12))()
        self._v("get_marker_particle_position_data_range", start_idx, end_idx, buf,
                argtypes=[c_int, c_int, c_void_p])
        return bytes(buf)

    def get_marker_particle_velocity_data_range(self, start_idx, end_idx):
        buf = (c_char * ((end_idx - start_idx) * 12))()
        self._v("get_marker_particle_velocity_data_range", start_idx, end_idx, buf,
                argtypes=[c_int, c_int, c_void_p])
        return bytes(buf)

    def _range(self, name, start_idx, end_idx):
        buf = (c_char * (max(end_idx - start_idx, 0) * 12))()
        self._v(name, start_idx, end_idx, buf, argtypes=[c_int, c_int, c_void_p])
        return bytes(buf)

    def get_marker_particle_affinex_data_range(self, start_idx, end_idx):
        return self._range("get_marker_particle_affinex_data_range", start_idx, end_idx)

    def get_marker_particle_affiney_data_range(self, start_idx, end_idx):
        return self._range("get_marker_particle_affiney_data_range", start_idx, end_idx)

    def get_marker_particle_affinez_data_range(self, start_idx, end_idx):
        return self._range("get_marker_particle_affinez_data_range", start_idx, end_idx)

    def get_frame_stats_data(self):
        return self._v("get_frame_stats_data", restype=FluidSimulationFrameStats_t)

    # ---- GB300 extensions ----
    def set_pressure_solver_mode(self, mode):
        """0: FP64 PCG as the reference; 1: mixed precision with FP64 refinement."""
        self._v("gb300_set_pressure_solver_mode", int(mode), argtypes=[c_int])

    def set_pressure_solver_tolerance(self, tol):
        self._v("gb300_set_pressure_solver_tolerance", float(tol), argtypes=[c_double])

    def set_mixed_inner_tolerance(self, rel):
        self._v("gb300_set_mixed_inner_tolerance", float(rel), argtypes=[c_double])

    # mesh obstacles (fluidsimulation.py:2589-2602); the engine reads an added MeshObject before
    # every substep, so the simulation keeps it alive until it is removed
    def add_mesh_obstacle(self, mesh_object):
        self._v("add_mesh_obstacle", mesh_object(), argtypes=[c_void_p])
        self.__dict__.setdefault("_obstacles", []).append(mesh_object)

    def remove_mesh_obstacle(self, mesh_object):
        self._v("remove_mesh_obstacle", mesh_object(), argtypes=[c_void_p])
        held = self.__dict__.get("_obstacles", [])
        if mesh_object in held:
            held.remove(mesh_object)

    def remove_mesh_obstacles(self):
        self._v("remove_mesh_obstacles")
        self.__dict__["_obstacles"] = []

    def add_sphere_obstacle(self, cx, cy, cz, r):
        self._v("gb300_add_sphere_obstacle", float(cx), float(cy), float(cz), float(r), argtypes=[c_double] * 4)

    def set_solid_level_set(self, phi_float32_bytes):
        self._v("gb300_set_solid_level_set", phi_float32_bytes, argtypes=[c_char_p])

    def set_marker_particle_data(self, num_particles, position_data, velocity_data):
        c_pos = (c_char * len(position_data)).from_buffer_copy(position_data)
        c_vel = (c_char * len(velocity_data)).from_buffer_copy(velocity_data)
        d = FluidSimulationMarkerParticleData_t()
        d.size = c_int(num_particles)
        d.positions = ctypes.cast(c_pos, c_char_p)
        d.velocities = ctypes.cast(c_vel, c_char_p)
        self._v("gb300_set_marker_particle_data", d, argtypes=[FluidSimulationMarkerParticleData_t])

    def get_pressure_solver_stats(self):
        out = (c_double * 6)()
        self._v("gb300_get_pressure_solver_stats", out, argtypes=[c_void_p])
        keys = ("iterations", "success", "outer", "box_cells", "error", "rel_residual")
        return dict(zip(keys, list(out)))

    def set_solve_check(self, reference_tolerance):
        """Compare every solve with an FP64 reference solve to this relative residual (0: off)."""
        self._v("gb300_set_solve_check", float(reference_tolerance), argtypes=[c_double])

    def get_solve_check(self):
        out = (c_double * 8)()
        self._v("gb300_get_solve_check", out, argtypes=[c_void_p])
        keys = ("valid", "p_rel_l2", "u_rel_l2", "div_rel", "div_ref_rel", "bnorm", "ref_iterations",
                "ref_rel_residual")
        return dict(zip(keys, list(out)))

    def get_frame_substep_times(self):
        """Lengths of the last update's substeps, in order."""
        n = self._v("gb300_get_frame_substep_times", None, 0, argtypes=[c_void_p, c_int], restype=c_int)
        out = (c_double * max(n, 1))()
        self._v("gb300_get_frame_substep_times", out, n, argtypes=[c_void_p, c_int], restype=c_int)
        return list(out)[:n]

    def enable_stage_timing(self, enable=True):
        self._v("gb300_enable_stage_timing", 1 if enable else 0, argtypes=[c_int])

    # save-state particle files (bake.py:2864-2905, 554-721)
    SAVE_STATE_ATTRIBUTES = {"position": 0, "velocity": 1, "affinex": 2, "affiney": 3, "affinez": 4}

    def write_marker_particle_file(self, attribute, path, append=False):
        self._v("gb300_write_marker_particle_file", int(self.SAVE_STATE_ATTRIBUTES.get(attribute, attribute)),
                os.fsencode(path), 1 if append else 0, argtypes=[c_int, c_char_p, c_int])

    def load_marker_particle_files(self, position_path, velocity_path, affinex_path=None, affiney_path=None,
                                   affinez_path=None):
        enc = lambda p_: os.fsencode(p_) if p_ is not None else None
        return self._v("gb300_load_marker_particle_files", enc(position_path), enc(velocity_path),
                       enc(affinex_path), enc(affiney_path), enc(affinez_path), argtypes=[c_char_p] * 5,
                       restype=ctypes.c_longlong)

    def get_viscosity_solver_stats(self):
        out = (c_double * 4)()
        self._v("gb300_get_viscosity_solver_stats", out, argtypes=[c_void_p])
        return dict(rows=int(out[0]), iterations=int(out[1]), error=out[2], success=bool(out[3]))

    def get_viscosity_solver_times(self):
        """Milliseconds of the last viscosity solve (stage timing on): system, factor, PCG."""
        out = (c_float * 3)()
        self._v("gb300_get_viscosity_solver_times", out, argtypes=[c_void_p])
        return dict(build=out[0], factor=out[1], pcg=out[2])

    def get_stage_times(self):
        out = (c_float * 12)()
        self._v("gb300_get_stage_times", out, argtypes=[c_void_p])
        keys = ("sort", "sdf", "p2g", "extrap", "pressure_build", "factor", "pcg", "project", "g2p", "advect",
                "remove", "total")
        return dict(zip(keys, list(out)))

    def get_kernel_launch_count(self):
        return self._v("gb300_get_kernel_launch_count", restype=c_ulonglong)

    def substep(self, dt):
        self._v("gb300_substep", float(dt), argtypes=[c_double])

    def substep_differentiable(self, dt):
        """One substep without marker removal that records what the adjoint needs."""
        self._v("gb300_substep_differentiable", float(dt), argtypes=[c_double])

    def set_pressure_axis_order(self, mode):
        """1: the mixed solve sweeps the pressure box's shortest axis (default); 0: the grid's order."""
        self._v("gb300_set_pressure_axis_order", int(mode), argtypes=[c_int])

    def set_pressure_warm_start(self, mode):
        """Start of the mixed solve: 2 the linear extrapolation of the last two substeps' pressures
        (default), 1 (or True) the previous substep's pressure, 0 (or False) zero."""
        self._v("gb300_set_pressure_warm_start", int(mode), argtypes=[c_int])

    def set_pcg_graphs(self, on):
        """Replay the mixed solve's batches of iterations from a graph (default) or launch them one by one."""
        self._v("gb300_set_pcg_graphs", 1 if on else 0, argtypes=[c_int])

    def set_viscosity_preconditioner(self, form):
        """0 tiled wavefront blocks (default), 1 per-level launches, 2 one cooperative launch,
        3 tiled wavefront blocks swept along the grid's z axis."""
        self._v("gb300_set_viscosity_preconditioner", int(form), argtypes=[c_int])

    def set_viscosity_warm_start(self, on):
        """Start the viscosity PCG from the field before the solve (default) or from zero."""
        self._v("gb300_set_viscosity_warm_start", 1 if on else 0, argtypes=[c_int])

    def set_wait_limit(self, polls):
        """Polls before a wavefront wait of the pressure or viscosity solve gives up (0: the default)."""
        self._v("gb300_set_wait_limit", int(polls), argtypes=[c_longlong])

    def set_adjoint_tolerance(self, tol):
        self._v("gb300_set_adjoint_tolerance", float(tol), argtypes=[c_double])

    def adjoint(self, grad_v1=None, loss_ymin=0.5):
        """dL/dv0 as an (N, 3) float32 array.  grad_v1: (N, 3) float32 dL/dv1, or None for
        L = mean over particles with y > loss_ymin of vy^2 (returns (grad, count))."""
        import numpy as np
        n = self.get_num_marker_particles()
        out = np.zeros((n, 3), np.float32)
        g = None if grad_v1 is None else np.ascontiguousarray(grad_v1, np.float32)
        cnt = self._v("gb300_adjoint", g.ctypes.data_as(c_void_p) if g is not None else None, float(loss_ymin),
                      out.ctypes.data_as(c_void_p), argtypes=[c_void_p, c_double, c_void_p], restype=c_int)
        return out, cnt

    def rollout_forward(self, k, dt):
        """k differentiable substeps with a device checkpoint of (x, v) before each."""
        self._v("gb300_rollout_forward", int(k), float(dt), argtypes=[c_int, c_double])

    def rollout_adjoint(self, grad_xk=None, grad_vk=None, loss_ymin=0.5):
        """(dL/dx0, dL/dv0, count) as (N, 3) float32 arrays for the last rollout.  grad_xk /
        grad_vk: (N, 3) float32 gradients of the loss on the final state (None = zero for
        grad_xk; grad_vk None selects L = mean over particles with y > loss_ymin of vy^2,
        and count is their number, else -1)."""
        import numpy as np
        n = self.get_num_marker_particles()
        gx0 = np.zeros((n, 3), np.float32)
        gv0 = np.zeros((n, 3), np.float32)
        gx = None if grad_xk is None else np.ascontiguousarray(grad_xk, np.float32)
        gv = None if grad_vk is None else np.ascontiguousarray(grad_vk, np.float32)
        ptr = lambda a: a.ctypes.data_as(c_void_p) if a is not None else None
        cnt = self._v("gb300_rollout_adjoint", ptr(gx), ptr(gv), float(loss_ymin), ptr(gx0), ptr(gv0),
                      argtypes=[c_void_p, c_void_p, c_double, c_void_p, c_void_p], restype=c_int)
        return gx0, gv0, cnt
