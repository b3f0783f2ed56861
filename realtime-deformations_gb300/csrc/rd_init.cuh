// The reference's particle initialiser, initializeParticles
// (material_point_method.cpp:18-63 with utils.h:110-127), on the device: the
// cells within `width / h` of the origin, 8 points per cell at quarter offsets
// (ds = 1 or 3 quarters per axis), each jittered inside a ball of a quarter
// cell (phi, cos theta, u drawn uniformly, radius 0.25 cbrt(u)), kept where
// within `width` of the origin, filling particles from the last index down.
//
// RD_INIT_REFERENCE draws the jitter from the C library's rand() exactly as the
// reference does, so it reproduces the reference's particles: rand() is
// glibc's additive feedback generator (TYPE_3, the default of srand/rand):
//   r_0 = seed, r_i = 16807 r_{i-1} mod (2^31 - 1) for i = 1..30,
//   r_i = r_{i-31} for i = 31..33, r_i = r_{i-31} + r_{i-3} mod 2^32 after,
//   and the k-th rand() is r_{k+344} >> 1
// (the published description of glibc's random(), e.g. P. Selinger, "The
// GLIBC pseudo-random number generator", 2007).  Each candidate takes three
// values and each placed particle three more (its colour), so the stream is
// sequential: one device thread walks it, with the reference's float/double
// types and rounding (explicit _rn operations, no FMA contraction).
// RD_INIT_PARALLEL draws the jitter from a counter-based hash per candidate
// (SplitMix64 finaliser, Steele, Lea & Flood 2014) and places the accepted
// points in candidate order through a prefix sum: any size, one thread per
// candidate, not the reference's stream.
#pragma once

#include "rd_kernels.cuh"

namespace rd {

struct GlibcRand {
    int32_t r[34];  // the last 34 values, ring buffer
    int head;       // index of the oldest value
    __device__ void seed(uint32_t s) {
        if (s == 0) s = 1;
        int64_t w = (int32_t)s;
        r[0] = (int32_t)w;
        for (int i = 1; i < 31; ++i) {
            // 16807 * r mod (2^31 - 1), the sign kept as glibc's srandom_r does
            const int64_t hi = w / 127773, lo = w % 127773;
            w = 16807 * lo - 2836 * hi;
            if (w < 0) w += 2147483647;
            r[i] = (int32_t)w;
        }
        for (int i = 31; i < 34; ++i) r[i] = r[i - 31];
        head = 0;
        for (int k = 0; k < 310; ++k) next_raw();
    }
    __device__ uint32_t next_raw() {  // r_i = r_{i-31} + r_{i-3}
        const int i31 = (head + 3) % 34, i3 = (head + 31) % 34;  // r_{i-31}, r_{i-3}; head holds r_{i-34}
        const uint32_t v = (uint32_t)r[i31] + (uint32_t)r[i3];
        r[head] = (int32_t)v;
        head = (head + 1) % 34;
        return v;
    }
    __device__ int next() { return (int)(next_raw() >> 1); }
};

// utils.h:110-112: low + (rand() % 2000) / 2000.0 * (high - low), as float.
__device__ __forceinline__ float rand_float(GlibcRand& g, float lo, float hi) {
    const double q = __ddiv_rn((double)(g.next() % 2000), 2000.0);
    return (float)__dadd_rn((double)lo, __dmul_rn(q, (double)__fsub_rn(hi, lo)));
}

template <typename T>
__device__ __forceinline__ void place_particle(vec4<T>* pl, int n, int slot, const float pos[3], const float vel[3],
                                               float mass) {
    Particle<T> p;
#pragma unroll
    for (int a = 0; a < 3; ++a) { p.x[a] = (T)pos[a]; p.v[a] = (T)vel[a]; }
#pragma unroll
    for (int e = 0; e < 9; ++e) { p.B[e] = T(0); p.F[e] = (e % 4 == 0) ? T(1) : T(0); }
    p.Jp = T(1);
    p.m = (T)mass;
    p.vol = T(0);
    p.id = (uint32_t)slot;
    store_particle(pl, (size_t)n, (size_t)slot, p);
}

struct InitSpec {
    float origin[3], vel[3];
    float width, mass, h;
    uint32_t seed;
    int cx, cy, cz, wic;  // origin cell, width in cells
};

// Every particle at the origin with no mass until a point is placed in it.
template <typename T>
__global__ void k_init_defaults(InitSpec S, int n, vec4<T>* __restrict__ pl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) place_particle<T>(pl, n, i, S.origin, S.vel, 0.0f);
}

// RD_INIT_REFERENCE: one thread walks the candidates in the reference's order.
template <typename T>
__global__ void k_init_reference(InitSpec S, int n, vec4<T>* __restrict__ pl, int* __restrict__ need_more) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    GlibcRand g;
    g.seed(S.seed);
    const float q4 = 1.0f / 4.0f;
    int left = n, more = 0;
    for (int i = S.cx - S.wic; i < S.cx + S.wic; ++i)
        for (int j = S.cy - S.wic; j < S.cy + S.wic; ++j)
            for (int k = S.cz - S.wic; k < S.cz + S.wic; ++k)
                for (int d = 0; d < 8; ++d) {
                    const float dsx = (d & 4) ? 3.0f : 1.0f, dsy = (d & 2) ? 3.0f : 1.0f, dsz = (d & 1) ? 3.0f : 1.0f;
                    // generateRandomInsideUnitBall(0.25): phi float, cos theta double, u float
                    const float phi = rand_float(g, 0.0f, (float)(2.0 * 3.1415));
                    const double costheta = __dsub_rn((double)rand_float(g, 0.0f, 2.0f), 1.0);
                    const float u = rand_float(g, 0.0f, 1.0f);
                    const double theta = acos(costheta);
                    const float r = __fmul_rn(0.25f, cbrtf(u));
                    const double st = sin(theta);
                    const float jx = (float)__dmul_rn(__dmul_rn((double)r, st), cos((double)phi));
                    const float jy = (float)__dmul_rn(__dmul_rn((double)r, st), sin((double)phi));
                    const float jz = (float)__dmul_rn((double)r, cos(theta));
                    const float pos[3] = {__fmul_rn(__fadd_rn(__fadd_rn((float)i, __fmul_rn(dsx, q4)), jx), S.h),
                                          __fmul_rn(__fadd_rn(__fadd_rn((float)j, __fmul_rn(dsy, q4)), jy), S.h),
                                          __fmul_rn(__fadd_rn(__fadd_rn((float)k, __fmul_rn(dsz, q4)), jz), S.h)};
                    const float dx = __fsub_rn(pos[0], S.origin[0]), dy = __fsub_rn(pos[1], S.origin[1]),
                                dz = __fsub_rn(pos[2], S.origin[2]);
                    const float len = __fsqrt_rn(__fadd_rn(__fadd_rn(__fmul_rn(dx, dx), __fmul_rn(dy, dy)), __fmul_rn(dz, dz)));
                    if (len > S.width) continue;
                    if (!left) { ++more; continue; }
                    place_particle<T>(pl, n, --left, pos, S.vel, S.mass);
                    for (int c = 0; c < 3; ++c) (void)g.next();  // p.r, p.g, p.b (then set to white)
                }
    *need_more = more;
}

// SplitMix64 finaliser of (seed, candidate, draw) -> uniform in [0, 1).
__device__ __forceinline__ float hash_uniform(uint32_t seed, uint32_t cand, uint32_t draw) {
    uint64_t z = ((uint64_t)seed << 32 | cand) * 3ull + draw + 0x9E3779B97F4A7C15ull;
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    z ^= z >> 31;
    return (float)(z >> 40) * (1.0f / 16777216.0f);
}

// RD_INIT_PARALLEL candidate c: its jittered point and whether it is kept.
__device__ __forceinline__ bool parallel_candidate(const InitSpec& S, uint32_t c, float pos[3]) {
    const int side = 2 * S.wic;
    const int d = (int)(c % 8u);
    const int cell = (int)(c / 8u);
    const int k = cell % side, j = (cell / side) % side, i = cell / (side * side);
    const float dsx = (d & 4) ? 3.0f : 1.0f, dsy = (d & 2) ? 3.0f : 1.0f, dsz = (d & 1) ? 3.0f : 1.0f;
    const float phi = 6.2830f * hash_uniform(S.seed, c, 0);
    const float costheta = 2.0f * hash_uniform(S.seed, c, 1) - 1.0f;
    const float u = hash_uniform(S.seed, c, 2);
    const float r = 0.25f * cbrtf(u);
    const float st = sqrtf(fmaxf(0.0f, 1.0f - costheta * costheta));
    pos[0] = ((float)(S.cx - S.wic + i) + dsx * 0.25f + r * st * cosf(phi)) * S.h;
    pos[1] = ((float)(S.cy - S.wic + j) + dsy * 0.25f + r * st * sinf(phi)) * S.h;
    pos[2] = ((float)(S.cz - S.wic + k) + dsz * 0.25f + r * costheta) * S.h;
    const float dx = pos[0] - S.origin[0], dy = pos[1] - S.origin[1], dz = pos[2] - S.origin[2];
    return sqrtf(dx * dx + dy * dy + dz * dz) <= S.width;
}

// Kept candidates per chunk of 1024 (one CTA per chunk).
__global__ void __launch_bounds__(1024) k_init_count(InitSpec S, uint32_t ncand, uint32_t* __restrict__ chunk) {
    __shared__ uint32_t part[32];
    const uint32_t c = blockIdx.x * 1024u + threadIdx.x;
    float pos[3];
    const bool keep = c < ncand && parallel_candidate(S, c, pos);
    const uint32_t b = __ballot_sync(0xffffffffu, keep);
    if ((threadIdx.x & 31) == 0) part[threadIdx.x >> 5] = (uint32_t)__popc(b);
    __syncthreads();
    if (threadIdx.x == 0) {
        uint32_t t = 0;
        for (int w = 0; w < 32; ++w) t += part[w];
        chunk[blockIdx.x] = t;
    }
}

// Places the kept candidates of each chunk at their rank (chunk prefix + rank
// in the chunk), filling particles from the last index down.
template <typename T>
__global__ void __launch_bounds__(1024) k_init_place(InitSpec S, uint32_t ncand, const uint32_t* __restrict__ pre,
                                                     int n, vec4<T>* __restrict__ pl) {
    __shared__ uint32_t part[32];
    const uint32_t c = blockIdx.x * 1024u + threadIdx.x;
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    float pos[3];
    const bool keep = c < ncand && parallel_candidate(S, c, pos);
    const uint32_t b = __ballot_sync(0xffffffffu, keep);
    if (lane == 0) part[wid] = (uint32_t)__popc(b);
    __syncthreads();
    uint32_t before = 0;
    for (int w = 0; w < wid; ++w) before += part[w];
    const uint32_t rank = pre[blockIdx.x] + before + (uint32_t)__popc(b & ((1u << lane) - 1u));
    if (keep && rank < (uint32_t)n) place_particle<T>(pl, n, n - 1 - (int)rank, pos, S.vel, S.mass);
}

}  // namespace rd
