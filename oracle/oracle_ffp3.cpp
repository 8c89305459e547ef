// CPU oracle (test infrastructure only): the FFP3 fluid-particle output of the marker particles.
//
//   FluidSimulation::_classifyFluidParticleTypes[Thread] (fluidsimulation.cpp:9477-9552): a
//     particle whose cell lies within 2 + boundary width cells of a grid side is a boundary
//     particle; otherwise the surface level set sampled at p - dx/2 (the cell-centred trilinear
//     interpolation, interpolation.cpp:72-110) decides: >= -surface width dx is surface, below
//     is interior (a NaN sample leaves the particle unset).  No meshing volume.
//   FluidSimulation::_generateFluidParticleDataFFP3 (fluidsimulation.cpp:9554-9676): particles
//     with id < round(65536 * output amount) and an enabled type are grouped surface, boundary,
//     interior; inside a type by id; inside an id in particle order.  Per type and id the header
//     holds the end of the id's run within its type.
//   FluidSimulation::_generateFluidParticleFFP3FileData (fluidsimulation.h:2036-2068): the bytes,
//     4 uint32 (surface, boundary, interior counts, id limit), 3 uint32 per id (the surface,
//     boundary, interior run ends), then the grouped records.
// Written in the reference's float / double arithmetic.
#include <cmath>
#include <cstdint>
#include <cstring>
#include <vector>

#include "oracle.h"

namespace {

enum PType { SURFACE = 0, BOUNDARY = 1, INTERIOR = 2, UNSET = 3 };

// Interpolation::trilinearInterpolate(p - hdx, dx, grid) for a cell-centred grid
double sample_centred(const float *g, int ni, int nj, int nk, double dx, float px, float py, float pz) {
    const float sh = (float)(0.5 * dx);   // vmath::vec3 hdx(0.5 dx, ...)
    const float x = px - sh, y = py - sh, z = pz - sh;
    const double inv = 1.0 / dx;
    const int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
    const float gx = (float)((double)(float)i * dx), gy = (float)((double)(float)j * dx),
                gz = (float)((double)(float)k * dx);   // GridIndexToPosition (grid3d.h:80-84)
    const double ix = (x - gx) * inv, iy = (y - gy) * inv, iz = (z - gz) * inv;
    const int off[8][3] = {{0, 0, 0}, {1, 0, 0}, {0, 1, 0}, {0, 0, 1}, {1, 0, 1}, {0, 1, 1}, {1, 1, 0}, {1, 1, 1}};
    double p[8];
    for (int c = 0; c < 8; c++) {
        const int a = i + off[c][0], b = j + off[c][1], e = k + off[c][2];
        const bool in = a >= 0 && b >= 0 && e >= 0 && a < ni && b < nj && e < nk;
        p[c] = in ? (double)g[(size_t)a + (size_t)ni * ((size_t)b + (size_t)nj * e)] : 0.0;
    }
    return p[0] * (1 - ix) * (1 - iy) * (1 - iz) + p[1] * ix * (1 - iy) * (1 - iz) + p[2] * (1 - ix) * iy * (1 - iz) +
           p[3] * (1 - ix) * (1 - iy) * iz + p[4] * ix * (1 - iy) * iz + p[5] * (1 - ix) * iy * iz +
           p[6] * ix * iy * (1 - iz) + p[7] * ix * iy * iz;
}

template <typename T>
void file_data(const std::vector<T> &attr, const std::vector<int> &table, unsigned int counts[3], int id_limit,
               const std::vector<unsigned int> (&header)[3], char *out, long long *size) {
    const size_t total = (size_t)counts[0] + counts[1] + counts[2];
    std::vector<T> sorted(total);
    for (size_t i = 0; i < table.size(); i++)
        if (table[i] >= 0) sorted[(size_t)table[i]] = attr[i];
    const size_t head = 4 * sizeof(unsigned int) + (size_t)id_limit * 3 * sizeof(unsigned int);
    std::vector<unsigned int> h(4 + 3 * (size_t)id_limit);
    h[0] = counts[0]; h[1] = counts[1]; h[2] = counts[2]; h[3] = (unsigned int)id_limit;
    for (int i = 0; i < id_limit; i++)
        for (int t = 0; t < 3; t++) h[4 + 3 * (size_t)i + t] = header[t][(size_t)i];
    std::memcpy(out, h.data(), head);
    std::memcpy(out + head, sorted.data(), total * sizeof(T));
    *size = (long long)(head + total * sizeof(T));
}

}  // namespace

extern "C" {

// surface: the cell-centred surface level set (ParticleLevelSet::calculateCurvatureGrid's first
// output); ids: the particles' uint16 ids; flags: bit0 surface, bit1 boundary, bit2 interior
// output.  types <- per particle 0 surface, 1 boundary, 2 interior, 3 unset.  The four outputs
// hold at most 16 + 12 * 65536 + np * 12 bytes each; sizes <- their byte counts.
void oracle_ffp3(int ni, int nj, int nk, double dx, const float *surface, int np, const float *pos, const float *vel,
                 const uint16_t *ids, int boundary_width, float surface_width_cells, double amount, int flags,
                 unsigned char *types, char *pos_out, char *id_out, char *vel_out, char *speed_out, long long *sizes) {
    const int bw = 2 + boundary_width;
    const float surface_width = (float)(surface_width_cells * dx);
    const double inv = 1.0 / dx;
    for (int p = 0; p < np; p++) {
        const float x = pos[3 * p], y = pos[3 * p + 1], z = pos[3 * p + 2];
        const int i = (int)std::floor(x * inv), j = (int)std::floor(y * inv), k = (int)std::floor(z * inv);
        const bool in = i >= 0 && j >= 0 && k >= 0 && i < ni && j < nj && k < nk;
        const bool interior_cell = i >= bw && j >= bw && k >= bw && i < ni - bw && j < nj - bw && k < nk - bw;
        if (in && !interior_cell) { types[p] = BOUNDARY; continue; }
        const float d = (float)sample_centred(surface, ni, nj, nk, dx, x, y, z);
        if (d >= -surface_width) types[p] = SURFACE;
        else if (d < -surface_width) types[p] = INTERIOR;
        else types[p] = UNSET;
    }
    const int id_limit = (int)std::round(65536 * amount);   // _getFluidParticleOutputIDLimit
    const bool enabled[3] = {(flags & 1) != 0, (flags & 2) != 0, (flags & 4) != 0};
    unsigned int counts[3] = {0, 0, 0};
    std::vector<unsigned int> runs[3];
    for (auto &r : runs) r.assign((size_t)id_limit, 0u);
    for (int p = 0; p < np; p++) {
        const int t = types[p];
        if (t == UNSET || (int)ids[p] >= id_limit || !enabled[t]) continue;
        counts[t]++;
        runs[t][ids[p]]++;
    }
    std::vector<unsigned int> start[3];
    for (int t = 0; t < 3; t++) {
        start[t].assign((size_t)id_limit, 0u);
        unsigned int c = 0;
        for (int i = 0; i < id_limit; i++) { start[t][(size_t)i] = c; c += runs[t][(size_t)i]; }
    }
    const unsigned int offset[3] = {0, counts[0], counts[0] + counts[1]};
    std::vector<int> table((size_t)np, -1);
    for (int p = 0; p < np; p++) {
        const int t = types[p];
        if (t == UNSET || (int)ids[p] >= id_limit || !enabled[t]) continue;
        table[(size_t)p] = (int)(offset[t] + start[t][ids[p]]);
        start[t][ids[p]]++;   // ends up holding the run ends: the header
    }
    std::vector<float> P(pos, pos + 3 * (size_t)np);
    struct V3 { float x, y, z; };
    std::vector<V3> pv((size_t)np), vv((size_t)np);
    std::vector<uint16_t> iv(ids, ids + np);
    std::vector<float> sv((size_t)np);
    for (int p = 0; p < np; p++) {
        pv[(size_t)p] = V3{pos[3 * p], pos[3 * p + 1], pos[3 * p + 2]};   // domain scale 1, offset 0
        vv[(size_t)p] = V3{vel[3 * p], vel[3 * p + 1], vel[3 * p + 2]};
        const float a = vel[3 * p], b = vel[3 * p + 1], c = vel[3 * p + 2];
        sv[(size_t)p] = std::sqrt(a * a + b * b + c * c);   // vmath::vec3::length
    }
    file_data(pv, table, counts, id_limit, start, pos_out, sizes + 0);
    file_data(iv, table, counts, id_limit, start, id_out, sizes + 1);
    file_data(vv, table, counts, id_limit, start, vel_out, sizes + 2);
    file_data(sv, table, counts, id_limit, start, speed_out, sizes + 3);
}

}  // extern "C"
