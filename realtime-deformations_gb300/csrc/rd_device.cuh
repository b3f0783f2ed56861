// Device-side building blocks of the sm_103a MPM step: vector types, the
// particle state planes, cubic B-spline weights, 3x3 helpers and the
// register-resident SVD that replaces the reference's Eigen::JacobiSVD.
#pragma once
#include <cuda_runtime.h>
#include <stdint.h>

namespace rd {

// ---------------------------------------------------------------- vectors
struct __align__(32) dvec4 { double x, y, z, w; };
template <typename T> struct V4T;
template <> struct V4T<float> { using type = float4; };
template <> struct V4T<double> { using type = dvec4; };
template <typename T> using vec4 = typename V4T<T>::type;

template <typename T> __device__ __forceinline__ vec4<T> mk4(T a, T b, T c, T d) {
    vec4<T> r; r.x = a; r.y = b; r.z = c; r.w = d; return r;
}

// Streaming loads/stores for particle planes: each plane element is read once
// and written once per kernel, so keep them out of L1 and mark them evict-first.
__device__ __forceinline__ float4 ld_stream(const float4* p) { return __ldcs(p); }
__device__ __forceinline__ dvec4 ld_stream(const dvec4* p) {
    const double2* q = reinterpret_cast<const double2*>(p);
    double2 a = __ldcs(q), b = __ldcs(q + 1);
    dvec4 r; r.x = a.x; r.y = a.y; r.z = b.x; r.w = b.y; return r;
}
__device__ __forceinline__ void st_stream(float4* p, float4 v) { __stcs(p, v); }
// Half k (0: x, y; 1: z, w) of a plane element.
__device__ __forceinline__ void st_stream_half(float4* p, int k, float a, float b) {
    __stcs(reinterpret_cast<float2*>(p) + k, make_float2(a, b));
}
__device__ __forceinline__ void st_stream(dvec4* p, dvec4 v) {
    double2* q = reinterpret_cast<double2*>(p);
    __stcs(q, make_double2(v.x, v.y)); __stcs(q + 1, make_double2(v.z, v.w));
}
__device__ __forceinline__ void st_stream_half(dvec4* p, int k, double a, double b) {
    __stcs(reinterpret_cast<double2*>(p) + k, make_double2(a, b));
}

// ---------------------------------------------------------------- bounds
// Bounds-checked build (nvcc -DRD_BOUNDS_CHECK: librd_mpm_checked.so): before
// each access at the checked sites - the fused kernel's and the P2G's shared
// tiles and records, the particle and grid indexes they compute - the index is
// tested against its buffer; one outside it is counted in rd_bounds_count
// (rd_debug_bounds_violations reads it) and the access skipped.  In the
// normal build RD_IN_BOUNDS is `true` and the tests compile away.
#ifdef RD_BOUNDS_CHECK
__device__ unsigned long long rd_bounds_count;
__device__ __forceinline__ bool in_bounds(long long i, long long n) {
    if (i >= 0 && i < n) return true;
    atomicAdd(&rd_bounds_count, 1ull);
    return false;
}
#define RD_IN_BOUNDS(i, n) ::rd::in_bounds((long long)(i), (long long)(n))
#else
#define RD_IN_BOUNDS(i, n) true
#endif

// ---------------------------------------------------------------- state
// Particle state: 7 planes of vec4 (structure of arrays of 16/32-byte
// vectors, so every plane access of a warp is one fully coalesced request):
//   0: x y z mass      1: vx vy vz volume
//   2: B00 B01 B02 B10 3: B11 B12 B20 B21   4: F00 F01 F02 F10
//   5: F11 F12 F20 F21 6: F22 Jp B22 id
// B is the reference's APIC matrix (C = B * DpInverse), F the elastic F_E,
// Jp = det F_P, id the particle's original index.  With track_fp three more
// planes carry the full plastic F_P: 7: P00 P01 P02 P10  8: P11 P12 P20 P21
// 9: P22 - - -.
constexpr int kPlanes = 7;
constexpr int kPlanesFP = 10;

template <typename T> struct Particle {
    T x[3], m, v[3], vol, B[9], F[9], Jp;
    uint32_t id;
};

template <typename T> __device__ __forceinline__ T id_to_real(uint32_t id);
template <> __device__ __forceinline__ float id_to_real<float>(uint32_t id) { return __uint_as_float(id); }
template <> __device__ __forceinline__ double id_to_real<double>(uint32_t id) { return (double)id; }
template <typename T> __device__ __forceinline__ uint32_t real_to_id(T v);
template <> __device__ __forceinline__ uint32_t real_to_id<float>(float v) { return __float_as_uint(v); }
template <> __device__ __forceinline__ uint32_t real_to_id<double>(double v) { return (uint32_t)v; }

template <typename T>
__device__ __forceinline__ void load_particle(const vec4<T>* __restrict__ pl, size_t n, size_t i, Particle<T>& p) {
    vec4<T> a = ld_stream(pl + 0 * n + i), b = ld_stream(pl + 1 * n + i), c = ld_stream(pl + 2 * n + i),
            d = ld_stream(pl + 3 * n + i), e = ld_stream(pl + 4 * n + i), f = ld_stream(pl + 5 * n + i),
            g = ld_stream(pl + 6 * n + i);
    p.x[0] = a.x; p.x[1] = a.y; p.x[2] = a.z; p.m = a.w;
    p.v[0] = b.x; p.v[1] = b.y; p.v[2] = b.z; p.vol = b.w;
    p.B[0] = c.x; p.B[1] = c.y; p.B[2] = c.z; p.B[3] = c.w;
    p.B[4] = d.x; p.B[5] = d.y; p.B[6] = d.z; p.B[7] = d.w;
    p.F[0] = e.x; p.F[1] = e.y; p.F[2] = e.z; p.F[3] = e.w;
    p.F[4] = f.x; p.F[5] = f.y; p.F[6] = f.z; p.F[7] = f.w;
    p.F[8] = g.x; p.Jp = g.y; p.B[8] = g.z; p.id = real_to_id<T>(g.w);
}

// The F_E / J_P part of a particle (planes 4 and 5 and the first half of
// plane 6) is final before the G2P gather and is stored apart from the rest
// (planes 0-3 and the second half of plane 6), so none of F is live across
// the gather.
template <typename T>
__device__ __forceinline__ void store_particle_front(vec4<T>* __restrict__ pl, size_t n, size_t i,
                                                     const Particle<T>& p) {
    st_stream(pl + 0 * n + i, mk4<T>(p.x[0], p.x[1], p.x[2], p.m));
    st_stream(pl + 1 * n + i, mk4<T>(p.v[0], p.v[1], p.v[2], p.vol));
    st_stream(pl + 2 * n + i, mk4<T>(p.B[0], p.B[1], p.B[2], p.B[3]));
    st_stream(pl + 3 * n + i, mk4<T>(p.B[4], p.B[5], p.B[6], p.B[7]));
    st_stream_half(pl + 6 * n + i, 1, p.B[8], id_to_real<T>(p.id));
}
template <typename T>
__device__ __forceinline__ void store_particle_back(vec4<T>* __restrict__ pl, size_t n, size_t i,
                                                    const Particle<T>& p) {
    st_stream(pl + 4 * n + i, mk4<T>(p.F[0], p.F[1], p.F[2], p.F[3]));
    st_stream(pl + 5 * n + i, mk4<T>(p.F[4], p.F[5], p.F[6], p.F[7]));
    st_stream_half(pl + 6 * n + i, 0, p.F[8], p.Jp);
}
template <typename T>
__device__ __forceinline__ void store_particle(vec4<T>* __restrict__ pl, size_t n, size_t i, const Particle<T>& p) {
    st_stream(pl + 0 * n + i, mk4<T>(p.x[0], p.x[1], p.x[2], p.m));
    st_stream(pl + 1 * n + i, mk4<T>(p.v[0], p.v[1], p.v[2], p.vol));
    st_stream(pl + 2 * n + i, mk4<T>(p.B[0], p.B[1], p.B[2], p.B[3]));
    st_stream(pl + 3 * n + i, mk4<T>(p.B[4], p.B[5], p.B[6], p.B[7]));
    st_stream(pl + 4 * n + i, mk4<T>(p.F[0], p.F[1], p.F[2], p.F[3]));
    st_stream(pl + 5 * n + i, mk4<T>(p.F[4], p.F[5], p.F[6], p.F[7]));
    st_stream(pl + 6 * n + i, mk4<T>(p.F[8], p.Jp, p.B[8], id_to_real<T>(p.id)));
}

// The plastic split F* = U diag(s) V^T of one particle (U, V row-major) and
// s - 1 (formed without cancellation), as 6 vec4 planes:
// U0..U3 | U4..U7 | U8 s0 s1 s2 | V0..V3 | V4..V7 | V8 (s-1)0 (s-1)1 (s-1)2.
template <typename T>
__device__ __forceinline__ void store_split(vec4<T>* __restrict__ pl, size_t n, size_t i, const T U[9], const T s[3],
                                            const T sm1[3], const T V[9]) {
    st_stream(pl + 0 * n + i, mk4<T>(U[0], U[1], U[2], U[3]));
    st_stream(pl + 1 * n + i, mk4<T>(U[4], U[5], U[6], U[7]));
    st_stream(pl + 2 * n + i, mk4<T>(U[8], s[0], s[1], s[2]));
    st_stream(pl + 3 * n + i, mk4<T>(V[0], V[1], V[2], V[3]));
    st_stream(pl + 4 * n + i, mk4<T>(V[4], V[5], V[6], V[7]));
    st_stream(pl + 5 * n + i, mk4<T>(V[8], sm1[0], sm1[1], sm1[2]));
}
template <typename T>
__device__ __forceinline__ void load_split(const vec4<T>* __restrict__ pl, size_t n, size_t i, T U[9], T s[3], T sm1[3],
                                           T V[9]) {
    const vec4<T> a = ld_stream(pl + 0 * n + i), b = ld_stream(pl + 1 * n + i), c = ld_stream(pl + 2 * n + i),
                  d = ld_stream(pl + 3 * n + i), e = ld_stream(pl + 4 * n + i), f = ld_stream(pl + 5 * n + i);
    U[0] = a.x; U[1] = a.y; U[2] = a.z; U[3] = a.w; U[4] = b.x; U[5] = b.y; U[6] = b.z; U[7] = b.w; U[8] = c.x;
    s[0] = c.y; s[1] = c.z; s[2] = c.w;
    V[0] = d.x; V[1] = d.y; V[2] = d.z; V[3] = d.w; V[4] = e.x; V[5] = e.y; V[6] = e.z; V[7] = e.w; V[8] = f.x;
    sm1[0] = f.y; sm1[1] = f.z; sm1[2] = f.w;
}
constexpr int kSplitPlanes = 6;

template <typename T>
__device__ __forceinline__ void load_fp(const vec4<T>* __restrict__ pl, size_t n, size_t i, T P[9]) {
    vec4<T> a = ld_stream(pl + 7 * n + i), b = ld_stream(pl + 8 * n + i), c = ld_stream(pl + 9 * n + i);
    P[0] = a.x; P[1] = a.y; P[2] = a.z; P[3] = a.w; P[4] = b.x; P[5] = b.y; P[6] = b.z; P[7] = b.w; P[8] = c.x;
}
template <typename T>
__device__ __forceinline__ void store_fp(vec4<T>* __restrict__ pl, size_t n, size_t i, const T P[9]) {
    st_stream(pl + 7 * n + i, mk4<T>(P[0], P[1], P[2], P[3]));
    st_stream(pl + 8 * n + i, mk4<T>(P[4], P[5], P[6], P[7]));
    st_stream(pl + 9 * n + i, mk4<T>(P[8], T(0), T(0), T(0)));
}

// ---------------------------------------------------------------- weights
// Cubic B-spline N(x) (material_point_method.hpp:20-31) at the four non-zero
// stencil offsets o = -1, 0, 1, 2 of node base + o, for t = x / h.  Both
// f = t - base and g = (base + 1) - t are exact in floating point (t and the
// integer node coordinate are multiples of ulp(t)), which is also what the
// reference's pos / h - idx evaluates to, so the polynomial pieces are chosen
// without branching: |t - (base-1)| = 1 + f uses (2 - a)^3 / 6 = g^3 / 6, and
// so on.  The node at offset -2 of the reference's 125-node stencil has
// |t - node| >= 2 and weight exactly 0.
template <typename T>
__device__ __forceinline__ void bspline4(T t, int base, T w[4]) {
    const T f = t - (T)base;
    const T g = (T)(base + 1) - t;
    const T f2 = f * f, f3 = f2 * f, g2 = g * g, g3 = g2 * g;
    const T sixth = T(1.0 / 6.0), two3 = T(2.0 / 3.0);
    w[0] = g3 * sixth;
    w[1] = T(0.5) * f3 - f2 + two3;
    w[2] = T(0.5) * g3 - g2 + two3;
    w[3] = f3 * sixth;
}

// IEEE divide then truncation toward zero: getParticleNeighs
// (material_point_method.cpp:83) computes ivec3(pos / h) the same way.
__device__ __forceinline__ int base_of(float x, float h) { return (int)__fdiv_rn(x, h); }
__device__ __forceinline__ int base_of(double x, double h) { return (int)__ddiv_rn(x, h); }
__device__ __forceinline__ float div_rn(float a, float b) { return __fdiv_rn(a, b); }
__device__ __forceinline__ double div_rn(double a, double b) { return __ddiv_rn(a, b); }

// ---------------------------------------------------------------- 3x3
// Determinant in glm's cofactor order (glm compute_determinant<tmat3x3>).
template <typename T> __device__ __forceinline__ T det3(const T M[9]) {
    return +M[0] * (M[4] * M[8] - M[5] * M[7]) - M[1] * (M[3] * M[8] - M[5] * M[6]) +
           M[2] * (M[3] * M[7] - M[4] * M[6]);
}
template <typename T> __device__ __forceinline__ void matmul3(T R[9], const T A[9], const T B[9]) {
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) R[3 * r + c] = A[3 * r] * B[c] + A[3 * r + 1] * B[3 + c] + A[3 * r + 2] * B[6 + c];
}

__device__ __forceinline__ float rsqrt_(float x) { return 1.0f / sqrtf(x); }
__device__ __forceinline__ double rsqrt_(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float sqrt_(float x) { return sqrtf(x); }
__device__ __forceinline__ double sqrt_(double x) { return sqrt(x); }
__device__ __forceinline__ float exp_(float x) { return expf(x); }
__device__ __forceinline__ double exp_(double x) { return exp(x); }
__device__ __forceinline__ float abs_(float x) { return fabsf(x); }
__device__ __forceinline__ double abs_(double x) { return fabs(x); }

template <typename T> struct SvdTol;
template <> struct SvdTol<float> { static constexpr float eps = 2e-7f; static constexpr int sweeps = 8; };
template <> struct SvdTol<double> { static constexpr double eps = 4e-16; static constexpr int sweeps = 14; };

// One-sided (Hestenes) Jacobi SVD, F = U diag(s) V^T with s >= 0, U and V
// orthogonal (U is a reflection when det F < 0): the convention of the
// JacobiSVD the reference calls (material_point_method.cpp:312).  Columns of
// A = F V are rotated pairwise until they are orthogonal to working precision;
// then s_i = |a_i| and u_i = a_i / s_i.  The singular values are not sorted:
// every use here (the plasticity clamp, det, the stress) is invariant to a
// consistent permutation.  The rotation is the standard one-sided Jacobi
// update (Demmel & Veselic 1992, Matrix Anal. Appl. 13(4)).
template <typename T>
__device__ __forceinline__ void svd3(const T F[9], T U[9], T s[3], T V[9]) {
    T a[3][3];  // a[col][row]
    T v[3][3];
#pragma unroll
    for (int c = 0; c < 3; ++c)
#pragma unroll
        for (int r = 0; r < 3; ++r) { a[c][r] = F[3 * r + c]; v[c][r] = (r == c) ? T(1) : T(0); }
    for (int sweep = 0; sweep < SvdTol<T>::sweeps; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const T al = a[p][0] * a[p][0] + a[p][1] * a[p][1] + a[p][2] * a[p][2];
            const T be = a[q][0] * a[q][0] + a[q][1] * a[q][1] + a[q][2] * a[q][2];
            const T ga = a[p][0] * a[q][0] + a[p][1] * a[q][1] + a[p][2] * a[q][2];
            if (abs_(ga) > SvdTol<T>::eps * sqrt_(al * be)) {
                rotated = true;
                const T zeta = (be - al) / (T(2) * ga);
                const T t = copysign(T(1), zeta) / (abs_(zeta) + sqrt_(T(1) + zeta * zeta));
                const T c = rsqrt_(T(1) + t * t);
                const T sn = c * t;
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    const T ap = a[p][r], aq = a[q][r];
                    a[p][r] = c * ap - sn * aq;
                    a[q][r] = sn * ap + c * aq;
                    const T vp = v[p][r], vq = v[q][r];
                    v[p][r] = c * vp - sn * vq;
                    v[q][r] = sn * vp + c * vq;
                }
            }
        }
        if (!rotated) break;
    }
    T smax = T(0);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        s[c] = sqrt_(a[c][0] * a[c][0] + a[c][1] * a[c][1] + a[c][2] * a[c][2]);
        smax = s[c] > smax ? s[c] : smax;
    }
    int kmin = 0;
#pragma unroll
    for (int c = 1; c < 3; ++c) kmin = s[c] < s[kmin] ? c : kmin;
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T inv = s[c] > T(0) ? T(1) / s[c] : T(0);
#pragma unroll
        for (int r = 0; r < 3; ++r) { U[3 * r + c] = a[c][r] * inv; V[3 * r + c] = v[c][r]; }
    }
    // A (nearly) vanishing singular value leaves its column of U undefined or
    // inaccurate: complete it as the cross product of the other two, keeping
    // the direction of a_kmin where that is still non-zero.
    if (!(s[kmin] > smax * (sizeof(T) == 4 ? T(1e-6) : T(1e-12)))) {
        const int i1 = (kmin + 1) % 3, i2 = (kmin + 2) % 3;
        T u0 = U[3 * 1 + i1] * U[3 * 2 + i2] - U[3 * 2 + i1] * U[3 * 1 + i2];
        T u1 = U[3 * 2 + i1] * U[3 * 0 + i2] - U[3 * 0 + i1] * U[3 * 2 + i2];
        T u2 = U[3 * 0 + i1] * U[3 * 1 + i2] - U[3 * 1 + i1] * U[3 * 0 + i2];
        const T nn = sqrt_(u0 * u0 + u1 * u1 + u2 * u2);
        T inv = nn > T(0) ? T(1) / nn : T(0);
        if (u0 * a[kmin][0] + u1 * a[kmin][1] + u2 * a[kmin][2] < T(0)) inv = -inv;
        U[kmin] = u0 * inv; U[3 + kmin] = u1 * inv; U[6 + kmin] = u2 * inv;
    }
}

// rsqrt with one Newton step: within about an ulp of 1/sqrt(x), so the
// Jacobi rotations below stay orthogonal to working precision.
__device__ __forceinline__ float rsqrt_acc(float x) {
    const float r = rsqrtf(x);
    return r * fmaf(-0.5f * x * r, r, 1.5f);
}
__device__ __forceinline__ double rsqrt_acc(double x) { return 1.0 / sqrt(x); }
__device__ __forceinline__ float div_fast(float a, float b) { return __fdividef(a, b); }
__device__ __forceinline__ double div_fast(double a, double b) { return a / b; }
// Reciprocal within about an ulp in FP32 (the hardware approximation, no
// IEEE rounding step); exact division in FP64.
__device__ __forceinline__ float rcp_fast(float x) { return __fdividef(1.0f, x); }
__device__ __forceinline__ double rcp_fast(double x) { return 1.0 / x; }
// Square root for a Jacobi rotation angle, which only needs to be close:
// the hardware approximation in FP32.
__device__ __forceinline__ float sqrt_approx(float x) {
    float r;
    asm("sqrt.approx.f32 %0, %1;" : "=f"(r) : "f"(x));
    return r;
}
__device__ __forceinline__ double sqrt_approx(double x) { return sqrt(x); }

// SVD of an F that is close to a rotation (the elastic F_E of the snow model
// stays within the plasticity clamp): F = U diag(s) V^T together with s - 1
// formed without cancellation.  With G = F - I (exact), the symmetric
// S = F^T F - I = G + G^T + G^T G is small and exactly representable to its own
// relative precision; its cyclic Jacobi eigen-decomposition (Golub & Van Loan,
// Matrix Computations, 8.5; rotations in the form of Rutishauser) gives
// V and e_i = s_i^2 - 1, so s_i = sqrt(1 + e_i) and s_i - 1 = e_i / (1 + s_i);
// u_i = F v_i / s_i.  The rotation angle only needs to be approximately right
// (an inexact angle leaves some off-diagonal for the next sweep); the cosine
// is formed accurately from the same tangent, so every rotation is orthogonal.
// When F is far from a rotation (|s_i^2 - 1| > 1/4) the one-sided Jacobi
// svd3 above is used, which keeps small singular values accurate.
template <typename T>
__device__ __forceinline__ void svd3_near(const T F[9], T U[9], T s[3], T sm1[3], T V[9]) {
    T G[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) G[e] = F[e];
    G[0] -= T(1); G[4] -= T(1); G[8] -= T(1);
    T A[3][3];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = r; c < 3; ++c) {
            A[r][c] = (G[3 * r + c] + G[3 * c + r]) + (G[r] * G[c] + G[3 + r] * G[3 + c] + G[6 + r] * G[6 + c]);
            A[c][r] = A[r][c];
        }
    const T dmax = fmax(abs_(A[0][0]), fmax(abs_(A[1][1]), abs_(A[2][2])));
    if (!(dmax <= T(0.25))) {  // far from a rotation (or non-finite): one-sided Jacobi on F
        svd3(F, U, s, V);
#pragma unroll
        for (int c = 0; c < 3; ++c) sm1[c] = s[c] - T(1);
        return;
    }
    T v[3][3];  // v[row][col]
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) v[r][c] = (r == c) ? T(1) : T(0);
    const T fro = sqrt_(A[0][0] * A[0][0] + A[1][1] * A[1][1] + A[2][2] * A[2][2] +
                        T(2) * (A[0][1] * A[0][1] + A[0][2] * A[0][2] + A[1][2] * A[1][2]));
    const T tol = SvdTol<T>::eps * fro;
    for (int sweep = 0; sweep < SvdTol<T>::sweeps; ++sweep) {
        bool rotated = false;
#pragma unroll
        for (int pq = 0; pq < 3; ++pq) {
            const int p = pq == 2 ? 1 : 0;
            const int q = pq == 0 ? 1 : 2;
            const int r = 3 - p - q;
            const T apq = A[p][q];
            if (abs_(apq) > tol) {
                rotated = true;
                const T theta = div_fast(A[q][q] - A[p][p], T(2) * apq);
                const T t = div_fast(copysign(T(1), theta), abs_(theta) + sqrt_approx(fma(theta, theta, T(1))));
                const T c = rsqrt_acc(fma(t, t, T(1)));
                const T sn = t * c;
                const T tau = div_fast(sn, T(1) + c);
                A[p][p] -= t * apq;
                A[q][q] += t * apq;
                A[p][q] = A[q][p] = T(0);
                const T arp = A[r][p], arq = A[r][q];
                A[r][p] = A[p][r] = arp - sn * (arq + tau * arp);
                A[r][q] = A[q][r] = arq + sn * (arp - tau * arq);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    const T vkp = v[k][p], vkq = v[k][q];
                    v[k][p] = vkp - sn * (vkq + tau * vkp);
                    v[k][q] = vkq + sn * (vkp - tau * vkq);
                }
            }
        }
        if (!rotated) break;
    }
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T e = A[c][c];
        s[c] = sqrt_(T(1) + e);
        sm1[c] = e * rcp_fast(T(1) + s[c]);
        const T inv = rcp_fast(s[c]);
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            V[3 * r + c] = v[r][c];
            U[3 * r + c] = (F[3 * r] * v[0][c] + F[3 * r + 1] * v[1][c] + F[3 * r + 2] * v[2][c]) * inv;
        }
    }
}

// ---------------------------------------------------------------- TMA
// Tile copies with the tensor memory accelerator: cp.async.bulk.tensor into
// shared memory, completion tracked by an mbarrier (one arrival with the
// expected byte count per copy).  The tensor map is a kernel parameter.
__device__ __forceinline__ uint32_t smem_addr(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(uint64_t* bar) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(bar)) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// One elected thread: the 4-D box at (0, z, y, x) of the tensor map into dst
// (128-byte aligned), signalling bar with `bytes`.  The innermost coordinate
// is 0, so the copy starts on a 16-byte boundary whatever the box origin;
// parts of the box outside the tensor read as zero.
__device__ __forceinline__ void tma_load_4d(void* dst, const void* tmap, uint64_t* bar, uint32_t bytes, int z, int y,
                                            int x) {
    const uint32_t b = smem_addr(bar);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(b), "r"(bytes) : "memory");
    asm volatile(
        "cp.async.bulk.tensor.4d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4, %5}], "
        "[%6];" ::"r"(smem_addr(dst)),
        "l"(tmap), "r"(0), "r"(z), "r"(y), "r"(x), "r"(b)
        : "memory");
}

// Waits for the phase `parity` of bar to complete, for at most `tries`
// polls; false when it gave up.
__device__ __forceinline__ bool mbar_wait(uint64_t* bar, uint32_t parity, int tries) {
    const uint32_t b = smem_addr(bar);
    for (int i = 0; i < tries; ++i) {
        uint32_t done;
        asm volatile(
            "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\tselp.u32 %0, 1, 0, p;\n\t}"
            : "=r"(done)
            : "r"(b), "r"(parity)
            : "memory");
        if (done) return true;
    }
    return false;
}

// ---------------------------------------------------------------- misc
__device__ __forceinline__ uint32_t lanemask_lt() {
    uint32_t m;
    asm("mov.u32 %0, %%lanemask_lt;" : "=r"(m));
    return m;
}

// Vector reduction of four FP32 values into global memory (sm_90+): one
// 16-byte atomic per grid cell instead of four.
__device__ __forceinline__ void red_add4(float4* addr, float4 v) {
    asm volatile("red.global.add.v4.f32 [%0], {%1, %2, %3, %4};" ::"l"(addr), "f"(v.x), "f"(v.y), "f"(v.z),
                 "f"(v.w)
                 : "memory");
}
__device__ __forceinline__ void red_add4(dvec4* addr, dvec4 v) {
    double* a = reinterpret_cast<double*>(addr);
    atomicAdd(a + 0, v.x); atomicAdd(a + 1, v.y); atomicAdd(a + 2, v.z); atomicAdd(a + 3, v.w);
}

}  // namespace rd
