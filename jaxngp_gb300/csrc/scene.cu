// Ground-truth images of the synthetic scenes (Gaussian density blobs, optional thin shells).
//
// The training scenes are procedural stand-ins for the reference's NeRF-synthetic captures: RGBA
// photographs of an object in a unit box, 800x800 pinhole views.  Each pixel is the midpoint
// quadrature (n_steps across the box) of the emission-absorption integral with density
//     sigma(x) = sum_b peak_b exp(-|x - c_b|^2 / (2 s_b^2))  +  shells
// and colour the density-weighted mean of the blob colours.  Output alpha is the opacity and
// colour is straight (unpremultiplied), so blending over a background matches
// utils/data.py:443-465.  Blobs farther than 5 s_b from the ray are culled per ray.
#include "common.cuh"

namespace ngp {
namespace {

constexpr int kMaxBlobs = 1024;

__global__ void __launch_bounds__(128) render_blobs_kernel(NgpRenderBlobsDescriptor d, const float *__restrict__ transforms,
                                                           const float *__restrict__ blobs, const float *__restrict__ shells,
                                                           std::uint8_t *__restrict__ rgba) {
    const std::uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= d.n_rays) return;
    const std::uint64_t n_pix = (std::uint64_t)d.width * d.height;
    const std::uint64_t p = (std::uint64_t)d.view0 * n_pix + i;
    const std::uint32_t view = (std::uint32_t)(p / n_pix), pix = (std::uint32_t)(p % n_pix);
    const float px = (float)(pix % d.width), py = (float)(pix / d.width);
    float cx = ((px + 0.5f) - d.cx) / d.fx, cy = -(((py + 0.5f) - d.cy) / d.fy), cz = -1.f;
    const float inv = rsqrtf(cx * cx + cy * cy + cz * cz);
    cx *= inv;
    cy *= inv;
    cz *= inv;
    const float *T = transforms + (std::size_t)view * 12;
    const float dx = cx * T[0] + cy * T[1] + cz * T[2];
    const float dy = cx * T[3] + cy * T[4] + cz * T[5];
    const float dz = cx * T[6] + cy * T[7] + cz * T[8];
    const float ox = T[9], oy = T[10], oz = T[11];
    // box intersection
    const float b = d.bound;
    float t0 = 0.f, t1 = 1e30f;
    const float o3[3] = {ox, oy, oz}, d3[3] = {dx, dy, dz};
    for (int a = 0; a < 3; ++a) {
        const float id = 1.f / (fabsf(d3[a]) > 1e-12f ? d3[a] : copysignf(1e-12f, d3[a]));
        const float ta = (-b - o3[a]) * id, tb = (b - o3[a]) * id;
        t0 = fmaxf(t0, fminf(ta, tb));
        t1 = fminf(t1, fmaxf(ta, tb));
    }
    float R = 0.f, Gc = 0.f, B = 0.f, Tr = 1.f;
    if (t1 > t0) {
        // cull blobs: keep those whose 5-sigma ball meets the ray segment (a per-thread list in
        // local memory, up to every blob)
        std::uint16_t keep[kMaxBlobs];
        int n_keep = 0;
        for (std::uint32_t k = 0; k < d.n_blobs; ++k) {
            const float *bl = blobs + (std::size_t)k * 8;
            const float vx = bl[0] - ox, vy = bl[1] - oy, vz = bl[2] - oz;
            const float tc = vx * dx + vy * dy + vz * dz;
            const float qx = vx - tc * dx, qy = vy - tc * dy, qz = vz - tc * dz;
            const float r = 5.f * bl[3];
            if (qx * qx + qy * qy + qz * qz <= r * r && tc + r >= t0 && tc - r <= t1) keep[n_keep++] = (std::uint16_t)k;
        }
        const float dt = (t1 - t0) / (float)d.n_steps;
        for (std::uint32_t s = 0; s < d.n_steps && Tr > 1e-6f; ++s) {
            const float t = t0 + (s + 0.5f) * dt;
            const float x = ox + t * dx, y = oy + t * dy, z = oz + t * dz;
            float sig = 0.f, cr = 0.f, cg = 0.f, cb = 0.f;
            for (int q = 0; q < n_keep; ++q) {
                const float *bl = blobs + (std::size_t)keep[q] * 8;
                const float ex = x - bl[0], ey = y - bl[1], ez = z - bl[2];
                const float w = bl[4] * __expf(-(ex * ex + ey * ey + ez * ez) / (2.f * bl[3] * bl[3]));
                sig += w;
                cr += w * bl[5];
                cg += w * bl[6];
                cb += w * bl[7];
            }
            for (std::uint32_t q = 0; q < d.n_shells; ++q) {
                const float *sh = shells + (std::size_t)q * 8;
                const float ex = x - sh[0], ey = y - sh[1], ez = z - sh[2];
                const float dist = sqrtf(ex * ex + ey * ey + ez * ez) - sh[3];
                if (fabsf(dist) <= sh[4]) {  // shell colour (c0, c0, c1)
                    sig += sh[5];
                    cr += sh[5] * sh[6];
                    cg += sh[5] * sh[6];
                    cb += sh[5] * sh[7];
                }
            }
            if (sig <= 0.f) continue;
            const float alpha = 1.f - __expf(-sig * dt);
            const float w = Tr * alpha / sig;
            R += w * cr;
            Gc += w * cg;
            B += w * cb;
            Tr *= 1.f - alpha;
        }
    }
    const float A = 1.f - Tr;
    const float ia = A > 1e-6f ? 1.f / A : 0.f;
    auto q8 = [](float v) { return (std::uint8_t)fminf(fmaxf(rintf(v * 255.f), 0.f), 255.f); };
    reinterpret_cast<uchar4 *>(rgba)[i] = make_uchar4(q8(R * ia), q8(Gc * ia), q8(B * ia), q8(A));
}

}  // namespace

int launch_render_blobs(cudaStream_t stream, const NgpRenderBlobsDescriptor &d, const float *transforms,
                        const float *blobs, const float *shells, std::uint8_t *rgba) {
    NGP_CHECK_ARG(d.n_blobs <= kMaxBlobs && d.n_steps > 0 && d.width > 0 && d.height > 0, "render_blobs: bad sizes");
    NGP_CHECK_ARG((std::uint64_t)d.view0 * d.width * d.height + d.n_rays <= (std::uint64_t)d.n_views * d.width * d.height,
                  "render_blobs: pixel range past the last view");
    NGP_CHECK_ARG(((std::uintptr_t)rgba & 3u) == 0, "render_blobs: rgba must be 4-byte aligned");
    if (d.n_rays > 0) {
        render_blobs_kernel<<<(d.n_rays + 127) / 128, 128, 0, stream>>>(d, transforms, blobs, shells, rgba);
        count_launches(1);
    }
    return launch_status();
}

}  // namespace ngp
