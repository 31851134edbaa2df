// Coarse occupancy blocks: the occupied interval of a ray over blocks of 8^3 occupancy cells
// (each block marked when any cell of the block, grown by one cell on every side, is occupied).
// Shared by the proposal sampler and the marcher's shortcut for rays that can have no sample.
// Built without FMA contraction in every including file (one rounding per operation, the order
// of oracle/proposal.py).
#pragma once

#include <cstdint>

namespace ngp {

// The ray's occupied interval over the coarse grid (a 3D DDA, x/y/z order on ties).
__device__ __forceinline__ bool coarse_ray_interval(float ox, float oy, float oz, float dx, float dy, float dz, float t0,
                                             float t1, const std::uint8_t *__restrict__ coarse, int Gc, float mb,
                                             float &ta, float &tb) {
    ta = 0.f;
    tb = 0.f;
    if (!(t0 < t1)) return false;
    const float o[3] = {ox, oy, oz}, d[3] = {dx, dy, dz};
    const float scale = (float)Gc / (2.0f * mb);
    int cell[3], step[3];
    float tmax[3], tdel[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const float g = ((o[a] + t0 * d[a]) + mb) * scale;
        cell[a] = min(max((int)floorf(g), 0), Gc - 1);
        if (d[a] > 0.f) {
            step[a] = 1;
            tmax[a] = (((float)(cell[a] + 1) / scale - mb) - o[a]) / d[a];
            tdel[a] = (1.0f / scale) / d[a];
        } else if (d[a] < 0.f) {
            step[a] = -1;
            tmax[a] = (((float)cell[a] / scale - mb) - o[a]) / d[a];
            tdel[a] = (-1.0f / scale) / d[a];
        } else {
            step[a] = 0;
            tmax[a] = __int_as_float(0x7f800000);
            tdel[a] = __int_as_float(0x7f800000);
        }
    }
    float t = t0;
    bool hit = false;
    for (int it = 0; it < 3 * Gc + 3; ++it) {
        if (!(t < t1)) break;
        const float m = fminf(tmax[0], fminf(tmax[1], tmax[2]));
        const int a = tmax[0] == m ? 0 : (tmax[1] == m ? 1 : 2);
        const float tn = fminf(m, t1);
        if (coarse[cell[0] + cell[1] * Gc + cell[2] * Gc * Gc]) {
            if (!hit) ta = t;
            hit = true;
            tb = tn;
        }
        cell[a] += step[a];
        if (cell[a] < 0 || cell[a] >= Gc) break;
        t = m;
        tmax[a] = tmax[a] + tdel[a];
    }
    return hit;
}

}  // namespace ngp
