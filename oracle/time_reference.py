"""Times the reference engine's own update() beside the oracle port on this host (test
infrastructure: it calibrates how far the CPU port stands in for the reference as the benchmark's
CPU baseline).  Needs the reference built by oracle/build_ref.sh (oracle/_ref/ref_harness).

The workload is the benchmark's: the 256^3 dam break (x < 0.35, y < 0.5, 8 particles per cell,
seed 0) with the icosphere obstacle (0.6, 0.3, 0.5) r = 0.15, PCG tolerance 1e-6, one substep of
1/240 s per update, extreme-velocity removal off.  The reference runs with its default thread
count (every core); the port with OpenMP on every core.

Usage: python oracle/time_reference.py [--n 256] [--updates 2]
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import time

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
sys.path.insert(0, os.path.join(ROOT, "tests", "golden"))
sys.path.insert(0, os.path.join(ROOT, "tests"))
import make_golden  # noqa: E402
import struct  # noqa: E402


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--n", type=int, default=256)
    ap.add_argument("--updates", type=int, default=2)
    args = ap.parse_args()
    from ffengine_gb300 import scenes
    n = args.n
    sphere = (0.6, 0.3, 0.5, 0.15)
    pos, vel = scenes.dam_break_particles(n, 0.35, 0.5, seed=0)
    with tempfile.TemporaryDirectory() as tmp:
        inp = os.path.join(tmp, "time.in")
        make_golden.write_input(inp, n, pos, vel, sphere, args.updates)
        with open(inp, "r+b") as f:   # set mode_flags bit7 and append the tolerance
            f.seek(8)
            flags = struct.unpack("<i", f.read(4))[0]
            f.seek(8)
            f.write(struct.pack("<i", flags | 128))
            f.seek(0, 2)
            f.write(struct.pack("<d", 1e-6))
        out = subprocess.run([make_golden.HARNESS, "time", inp, tmp], check=True, capture_output=True, text=True)
        ref = json.loads(out.stdout.strip().splitlines()[-1])
    import oracle_api as O
    objs = [(*scenes.icosphere(*sphere, 4), 0, 0.0)]
    solid = O.solid_level_set(n, 1.0 / n, objs)
    t0 = time.perf_counter()
    O.substep(n, 1.0 / n, 1.0 / 240.0, 0.05, 5, (0.0, -9.81, 0.0), solid, pos, vel, tol=1e-6)
    port_s = time.perf_counter() - t0
    print(json.dumps({"workload": "dam_break_sphere_%d" % n, "particles": int(pos.shape[0]),
                      "reference_update_s": ref["update_s"], "reference_threads": ref["threads"],
                      "reference_pressure_iterations": ref["last_pressure_iterations"],
                      "port_substep_s": port_s, "port_threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())),
                      "host_cpus": os.cpu_count()}))


if __name__ == "__main__":
    main()
