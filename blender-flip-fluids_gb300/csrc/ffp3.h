// FFP3 fluid-particle output (ffp3_kernels.cu): settings, work buffers and the launch.
#pragma once
#include <cuda_runtime.h>

#include "common.cuh"
#include "devbuf.h"

namespace ffgpu {

struct Ffp3Params {
    int id_limit = 65536;             // round(65536 * output amount) (fluidsimulation.h:2131-2133)
    int enabled = 7;                  // bit0 surface, bit1 boundary, bit2 interior output
    int boundary_width = 1;           // cells (fluidsimulation.h:2264)
    float surface_width_cells = 0.90f;   // (fluidsimulation.h:2263)
    bool velocity = false, speed = false;   // attribute outputs
};

struct Ffp3Work {
    DevBuf<unsigned char> type;   // per particle: 0 surface, 1 boundary, 2 interior, 3 unset
    DevBuf<int> key, flag, off, keys[2], idx[2], key_start, counts, coff, scan_tmp;
    DevBuf<char> out[4];          // FFP3 bytes: positions, ids, velocities, speeds
};

struct Ffp3Counts {
    int total = 0, surface = 0, boundary = 0, interior = 0;
    size_t bytes[4] = {0, 0, 0, 0};   // size of each output (0: not produced)
};

// Classifies the np particles against the cell-centred surface level set and writes the FFP3 bytes
// of positions, ids (uint16) and, when asked, velocities and speeds into w.out.  ids: one 32-bit
// slot per particle holding the uint16 id.
Ffp3Counts launch_ffp3(Dims d, double dx, const float *surface, int np, const float *px, const float *py,
                       const float *pz, const float *vx, const float *vy, const float *vz, const unsigned int *ids,
                       const Ffp3Params &prm, Ffp3Work &w, cudaStream_t st, unsigned long long &launches);

}  // namespace ffgpu
