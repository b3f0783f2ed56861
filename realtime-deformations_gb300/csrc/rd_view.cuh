// Headless viewer feed: the streams drawParticles fills for OpenGL
// (main.cpp:255-271: xyzs = (x, y, z, size) and rgba8 per particle) and a
// point-splat image of them made with CUDA alone (no graphics API): each
// particle covers the disc its camera-facing billboard of side `size`
// projects to (Particle.vertexshader: centre + right * sx * size + up * sy *
// size, sx, sy in [-1/2, 1/2]); the nearest particle wins each pixel (a 64-bit
// atomicMin of (depth, id), so the image does not depend on launch order) and
// is shaded as a sphere impostor.
#pragma once

#include "rd_kernels.cuh"

namespace rd {

struct ViewDev {
    float vp[16];            // view-projection, column-major: clip = VP * (x, y, z, 1)
    float right[3], up[3];   // camera axes in world space
    int width, height;
    uint32_t background;     // rgba8
    int max_radius;          // pixels
};

__device__ __forceinline__ void project(const ViewDev& V, float x, float y, float z, float& px, float& py,
                                        float& depth, float& w) {
    const float cx = V.vp[0] * x + V.vp[4] * y + V.vp[8] * z + V.vp[12];
    const float cy = V.vp[1] * x + V.vp[5] * y + V.vp[9] * z + V.vp[13];
    const float cz = V.vp[2] * x + V.vp[6] * y + V.vp[10] * z + V.vp[14];
    w = V.vp[3] * x + V.vp[7] * y + V.vp[11] * z + V.vp[15];
    const float iw = 1.0f / w;
    px = (cx * iw * 0.5f + 0.5f) * (float)V.width;
    py = (0.5f - cy * iw * 0.5f) * (float)V.height;  // image rows from the top
    depth = cz * iw * 0.5f + 0.5f;
}

// Pixel radius of a particle's billboard (the larger projected half side).
__device__ __forceinline__ float splat_radius(const ViewDev& V, float x, float y, float z, float size, float px,
                                              float py) {
    float ax, ay, d, w;
    project(V, x + V.right[0] * size * 0.5f, y + V.right[1] * size * 0.5f, z + V.right[2] * size * 0.5f, ax, ay, d, w);
    float bx, by;
    project(V, x + V.up[0] * size * 0.5f, y + V.up[1] * size * 0.5f, z + V.up[2] * size * 0.5f, bx, by, d, w);
    const float r1 = sqrtf((ax - px) * (ax - px) + (ay - py) * (ay - py));
    const float r2 = sqrtf((bx - px) * (bx - px) + (by - py) * (by - py));
    return fmaxf(r1, r2);
}

__global__ void k_splat_clear(unsigned long long* __restrict__ zid, int npix) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < npix) zid[i] = ~0ull;
}

// One thread per particle (original order): the pixels whose centres lie in
// its disc get min((depth bits << 32) | id).
__global__ void __launch_bounds__(256) k_splat(ViewDev V, int n, const float4* __restrict__ xyzs,
                                               unsigned long long* __restrict__ zid) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float4 p = xyzs[i];
    float px, py, depth, w;
    project(V, p.x, p.y, p.z, px, py, depth, w);
    if (!(w > 0.0f) || !(depth >= 0.0f && depth <= 1.0f)) return;  // behind the camera or clipped
    const float r = fminf(splat_radius(V, p.x, p.y, p.z, p.w, px, py), (float)V.max_radius);
    if (!(r > 0.0f)) return;
    const int x0 = max(0, (int)floorf(px - r)), x1 = min(V.width - 1, (int)floorf(px + r));
    const int y0 = max(0, (int)floorf(py - r)), y1 = min(V.height - 1, (int)floorf(py + r));
    const unsigned long long key = ((unsigned long long)__float_as_uint(depth) << 32) | (unsigned)i;
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
            const float dx = (float)x + 0.5f - px, dy = (float)y + 0.5f - py;
            if (dx * dx + dy * dy <= r * r) atomicMin(zid + (size_t)y * V.width + x, key);
        }
}

// The nearest particle's colour per pixel, shaded by the height of a sphere
// over its disc: rgb * (0.35 + 0.65 * sqrt(1 - (d / r)^2)), alpha 255.
__global__ void k_splat_resolve(ViewDev V, int n, const float4* __restrict__ xyzs, const uint32_t* __restrict__ rgba,
                                const unsigned long long* __restrict__ zid, uint32_t* __restrict__ image) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    const int npix = V.width * V.height;
    if (i >= npix) return;
    const unsigned long long key = zid[i];
    if (key == ~0ull) { image[i] = V.background; return; }
    const int id = (int)(key & 0xffffffffull);
    if (id >= n) { image[i] = V.background; return; }
    const float4 p = xyzs[id];
    float px, py, depth, w;
    project(V, p.x, p.y, p.z, px, py, depth, w);
    const float r = fminf(splat_radius(V, p.x, p.y, p.z, p.w, px, py), (float)V.max_radius);
    const int x = i % V.width, y = i / V.width;
    const float dx = (float)x + 0.5f - px, dy = (float)y + 0.5f - py;
    const float q = r > 0.0f ? fminf(1.0f, (dx * dx + dy * dy) / (r * r)) : 1.0f;
    const float shade = 0.35f + 0.65f * sqrtf(1.0f - q);
    const uint32_t c = rgba[id];
    const uint32_t cr = (uint32_t)fminf(255.0f, (float)(c & 0xff) * shade + 0.5f);
    const uint32_t cg = (uint32_t)fminf(255.0f, (float)((c >> 8) & 0xff) * shade + 0.5f);
    const uint32_t cb = (uint32_t)fminf(255.0f, (float)((c >> 16) & 0xff) * shade + 0.5f);
    image[i] = cr | (cg << 8) | (cb << 16) | (0xffu << 24);
}

}  // namespace rd
