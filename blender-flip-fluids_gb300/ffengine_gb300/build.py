"""Builds libffengine_gb300.so (all CUDA sources, sm_103a) in-tree.

Objects go to blender-flip-fluids_gb300/_build/, the library to ffengine_gb300/lib/,
the directory the reference's ctypes loader scans for libffengine*.so.  Each translation
unit compiles in parallel with one -gencode; -fmad=false keeps float/double rounding
identical to the reference engine's (no fused multiply-add unless a kernel asks for one).
"""
import concurrent.futures
import os
import shutil
import subprocess

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
ROOT_DIR = os.path.dirname(PKG_DIR)                     # blender-flip-fluids_gb300/
CSRC = os.path.join(ROOT_DIR, "csrc")
INCLUDE = os.path.join(os.path.dirname(ROOT_DIR), "include")
BUILD_DIR = os.path.join(ROOT_DIR, "_build")
LIB_DIR = os.path.join(PKG_DIR, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libffengine_gb300.so")

SOURCES = ["grid_kernels.cu", "sort_kernels.cu", "p2g_kernels.cu", "particle_kernels.cu", "pressure_build.cu",
           "tension_kernels.cu", "mesh_sdf.cu", "pcg_kernels.cu", "pcg_permute.cu", "mic_wavefront.cu", "adjoint_kernels.cu", "apic_kernels.cu",
           "viscosity_kernels.cu", "engine.cu", "engine_stages.cu", "engine_adjoint.cu", "capi.cu", "capi_stages.cu", "capi_mesh.cu",
           "ffp3_kernels.cu", "capi_ffp3.cu", "noalloc.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "--extended-lambda", "-Xcompiler", "-fPIC",
         "-Xcompiler", "-ffp-contract=off"]


def nvcc():
    path = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(path):
        raise RuntimeError("nvcc not found: the GB300 library needs the CUDA toolkit to build")
    return path


def _headers():
    hs = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    hs += [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE) if f.endswith(".h")]
    return hs


def _stale(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, jobs=None):
    """Compiles every CUDA translation unit and links the shared library; returns its path."""
    os.makedirs(BUILD_DIR, exist_ok=True)
    os.makedirs(LIB_DIR, exist_ok=True)
    headers = _headers()
    cc = nvcc()
    objs, cmds = [], []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD_DIR, src.replace(".cu", ".o"))
        objs.append(o)
        if _stale(o, [s] + headers):
            cmds.append([cc] + ARCH + FLAGS + ["-I", CSRC, "-I", INCLUDE, "-c", s, "-o", o])

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            print(r.stdout + r.stderr)

    with concurrent.futures.ThreadPoolExecutor(max_workers=jobs or max(1, os.cpu_count() or 1)) as ex:
        list(ex.map(run, cmds))
    if cmds or _stale(LIB_PATH, objs):
        run([cc] + ARCH + ["-shared", "-o", LIB_PATH] + objs + ["-lcudart_static", "-lrt", "-ldl", "-lpthread"])
    return LIB_PATH


if __name__ == "__main__":
    print(build(verbose=True))
