// Kernels of the implicit time integration (rd_time_integration): the energy
// the reference minimises over the grid velocities in timeIntegration
// (material_point_method.cpp:160-233), its gradient, and the vector
// operations of an L-BFGS minimiser that the host drives.  The unknowns are
// the velocities of the cells with mass, kept as a compact vector (3 reals a
// cell); the velocity field the particles read is the stage-mode grid itself.
#pragma once
#include "rd_kernels.cuh"

namespace rd {

// Constants of the energy density Psi = mu ||F - R||^2 + lambda / 2 (J - 1)^2
// with mu = mu0 e, lambda = lambda0 e, e = exp(xi - J_P) as the reference
// writes it (its exp(xi * 1 - det F_P), material_point_method.cpp:194-199) or
// e = exp(xi (1 - J_P)) (intended).
template <typename T> struct ImpParams {
    T dt, mu0, lambda0, xi;
    int intended;
};

// Derivative of the cubic B-spline N at the four offsets -1..2 of node
// base + o for t = x / h, written with f = t - base and g = base + 1 - t
// (both exact): N'(1 + f) = -(1 - f)^2 / 2, N'(f) = 3/2 f^2 - 2 f,
// N'(f - 1) = -3/2 g^2 + 2 g, N'(f - 2) = (1 - g)^2 / 2 = f^2 / 2
// (weightNxDerivative, material_point_method.hpp:32-51, evaluated at
// u = t - node).
template <typename T>
__device__ __forceinline__ void bspline4_deriv(T t, int base, T d[4]) {
    const T f = t - (T)base;
    const T g = (T)(base + 1) - t;
    d[0] = T(-0.5) * g * g;
    d[1] = T(1.5) * f * f - T(2) * f;
    d[2] = T(-1.5) * g * g + T(2) * g;
    d[3] = T(0.5) * f * f;
}

// Block-wide sum of a double into *acc (one atomic per block).  Every thread
// of the block calls it; it may be called again in the same kernel.
__device__ __forceinline__ void block_add(double v, double* acc) {
    __shared__ double part[32];
    __syncthreads();  // a previous call's readers are done with part
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    if (lane == 0) part[wid] = v;
    __syncthreads();
    if (wid == 0) {
        v = lane < (int)(blockDim.x >> 5) ? part[lane] : 0.0;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if (lane == 0 && v != 0.0) atomicAdd(acc, v);
    }
}

// Cells with mass: their indices (in no particular order) and count.
template <typename T>
__global__ void __launch_bounds__(256) k_imp_used(const vec4<T>* __restrict__ grid, size_t ncells,
                                                  uint32_t* __restrict__ idx, uint32_t* count) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const bool used = c < ncells && grid[c].x != T(0);
    const uint32_t m = __ballot_sync(0xffffffffu, used);
    if (!m) return;
    const int lane = threadIdx.x & 31;
    uint32_t base = 0;
    if (lane == __ffs(m) - 1) base = atomicAdd(count, (uint32_t)__popc(m));
    base = __shfl_sync(0xffffffffu, base, __ffs(m) - 1);
    if (used) idx[base + __popc(m & lanemask_lt())] = (uint32_t)c;
}

// x[k] = velocity of cell idx[k] (3 reals a cell).
template <typename T>
__global__ void k_imp_gather(const vec4<T>* __restrict__ grid, const uint32_t* __restrict__ idx, int nused,
                             T* __restrict__ x) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nused) return;
    const vec4<T> g = grid[idx[k]];
    x[3 * k] = g.y; x[3 * k + 1] = g.z; x[3 * k + 2] = g.w;
}

// x[k] = dense[idx[k]] (dense: 3 reals a cell).
template <typename T>
__global__ void k_imp_take(const T* __restrict__ dense, const uint32_t* __restrict__ idx, int nused,
                           T* __restrict__ x) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nused) return;
    const size_t c = idx[k];
    x[3 * k] = dense[3 * c]; x[3 * k + 1] = dense[3 * c + 1]; x[3 * k + 2] = dense[3 * c + 2];
}

// dense[idx[k]] = x[k] (dense: 3 reals a cell).
template <typename T>
__global__ void k_imp_spread(T* __restrict__ dense, const uint32_t* __restrict__ idx, int nused,
                             const T* __restrict__ x) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nused) return;
    const size_t c = idx[k];
    dense[3 * c] = x[3 * k]; dense[3 * c + 1] = x[3 * k + 1]; dense[3 * c + 2] = x[3 * k + 2];
}

// Velocity of cell idx[k] = x[k] + a d[k] (d may be null); the mass stays.
template <typename T>
__global__ void k_imp_put(vec4<T>* __restrict__ grid, const uint32_t* __restrict__ idx, int nused,
                          const T* __restrict__ x, T a, const T* __restrict__ d) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nused) return;
    vec4<T>& g = grid[idx[k]];
    if (d) {
        g.y = x[3 * k] + a * d[3 * k];
        g.z = x[3 * k + 1] + a * d[3 * k + 1];
        g.w = x[3 * k + 2] + a * d[3 * k + 2];
    } else {
        g.y = x[3 * k]; g.z = x[3 * k + 1]; g.w = x[3 * k + 2];
    }
}

// The particles' part of the energy at the grid's current velocities:
// Fhat = (I + dt sum_i v_i grad w_ip^T) F_E over the 64 nodes with a non-zero
// weight gradient (ElasticPotential, material_point_method.cpp:175-190), the
// density with the polar rotation of Fhat, V Psi summed into energy[0].
// GRAD: also dt V P F_E^T grad w_ip added to each node's entry of gacc, with
// P = 2 mu (Fhat - R) + lambda (J - 1) J Fhat^-T.  A thread per particle.
template <typename T, bool GRAD>
__global__ void __launch_bounds__(kThreads) k_imp_particles(DevParams<T> P, ImpParams<T> Q,
                                                            const vec4<T>* __restrict__ pl,
                                                            const vec4<T>* __restrict__ grid,
                                                            vec4<T>* __restrict__ gacc, double* energy) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (p < P.n) {
        Particle<T> q;
        load_particle(pl, (size_t)P.n, (size_t)p, q);
        T w[3][4], dw[3][4];
        int b[3];
#pragma unroll
        for (int a = 0; a < 3; ++a) {
            const T t = P.hinv_pow2 != T(0) ? q.x[a] * P.hinv_pow2 : div_rn(q.x[a], P.h);
            b[a] = (int)t;
            bspline4(t, b[a], w[a]);
            bspline4_deriv(t, b[a], dw[a]);
        }
        const T ih = T(1) / P.h;
        // G = sum_i v_i grad w_i^T, separably: grad w = (dwx wy wz, wx dwy wz, wx wy dwz) / h
        T Gm[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) Gm[e] = T(0);
        for (int ox = 0; ox < 4; ++ox) {
            const int gx = b[0] - 1 + ox;
            T s0[3] = {T(0), T(0), T(0)}, s1[3] = {T(0), T(0), T(0)}, s2[3] = {T(0), T(0), T(0)};
            for (int oy = 0; oy < 4; ++oy) {
                const int gy = b[1] - 1 + oy;
                T c0[3] = {T(0), T(0), T(0)}, c1[3] = {T(0), T(0), T(0)};
#pragma unroll
                for (int oz = 0; oz < 4; ++oz) {
                    const int gz = b[2] - 1 + oz;
                    if (gx < 0 || gy < 0 || gz < 0 || gx >= P.M[0] || gy >= P.M[1] || gz >= P.M[2]) continue;
                    const vec4<T> g = grid[((size_t)gx * P.M[1] + gy) * P.M[2] + gz];
                    const T v[3] = {g.y, g.z, g.w};
#pragma unroll
                    for (int r = 0; r < 3; ++r) {
                        c0[r] += w[2][oz] * v[r];
                        c1[r] += dw[2][oz] * v[r];
                    }
                }
#pragma unroll
                for (int r = 0; r < 3; ++r) {
                    s0[r] += w[1][oy] * c0[r];
                    s1[r] += dw[1][oy] * c0[r];
                    s2[r] += w[1][oy] * c1[r];
                }
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                Gm[3 * r + 0] += dw[0][ox] * s0[r];
                Gm[3 * r + 1] += w[0][ox] * s1[r];
                Gm[3 * r + 2] += w[0][ox] * s2[r];
            }
        }
        T A[9];
#pragma unroll
        for (int e = 0; e < 9; ++e) A[e] = Q.dt * ih * Gm[e];
        A[0] += T(1); A[4] += T(1); A[8] += T(1);
        T Fh[9];
        matmul3(Fh, A, q.F);
        T U[9], s[3], sm1[3], V[9];
        svd3_near(Fh, U, s, sm1, V);
        // the proper rotation of the polar decomposition: U D V^T, D flipping
        // the smallest singular value's column when det Fhat < 0
        const T J = det3(Fh);
        int kmin = 0;
#pragma unroll
        for (int c = 1; c < 3; ++c) kmin = s[c] < s[kmin] ? c : kmin;
        T R[9];
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c) {
                T acc = T(0);
#pragma unroll
                for (int k = 0; k < 3; ++k) acc += (J < T(0) && k == kmin ? -U[3 * r + k] : U[3 * r + k]) * V[3 * c + k];
                R[3 * r + c] = acc;
            }
        const T jp = q.Jp;
        const T ex = Q.intended ? Q.xi * (T(1) - jp) : Q.xi - jp;
        const T hard = exp_(ex);
        const T mu = Q.mu0 * hard, lam = Q.lambda0 * hard;
        T n2 = T(0);
#pragma unroll
        for (int e = 0; e < 9; ++e) n2 += (Fh[e] - R[e]) * (Fh[e] - R[e]);
        const T psi = mu * n2 + lam / T(2) * (J - T(1)) * (J - T(1));
        e_out = (double)(q.vol * psi);
        if (GRAD) {
            // dt V P F_E^T, then its product with each node's weight gradient
            const T cof[9] = {Fh[4] * Fh[8] - Fh[5] * Fh[7], Fh[5] * Fh[6] - Fh[3] * Fh[8],
                              Fh[3] * Fh[7] - Fh[4] * Fh[6], Fh[2] * Fh[7] - Fh[1] * Fh[8],
                              Fh[0] * Fh[8] - Fh[2] * Fh[6], Fh[1] * Fh[6] - Fh[0] * Fh[7],
                              Fh[1] * Fh[5] - Fh[2] * Fh[4], Fh[2] * Fh[3] - Fh[0] * Fh[5],
                              Fh[0] * Fh[4] - Fh[1] * Fh[3]};
            T Pm[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) Pm[e] = T(2) * mu * (Fh[e] - R[e]) + lam * (J - T(1)) * cof[e];
            T Ft[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) Ft[3 * r + c] = q.F[3 * c + r];
            T Am[9];
            matmul3(Am, Pm, Ft);
            const T sc = Q.dt * q.vol * ih;
#pragma unroll
            for (int e = 0; e < 9; ++e) Am[e] *= sc;
            for (int ox = 0; ox < 4; ++ox)
                for (int oy = 0; oy < 4; ++oy)
#pragma unroll
                    for (int oz = 0; oz < 4; ++oz) {
                        const int gx = b[0] - 1 + ox, gy = b[1] - 1 + oy, gz = b[2] - 1 + oz;
                        if (gx < 0 || gy < 0 || gz < 0 || gx >= P.M[0] || gy >= P.M[1] || gz >= P.M[2]) continue;
                        const T gw[3] = {dw[0][ox] * w[1][oy] * w[2][oz], w[0][ox] * dw[1][oy] * w[2][oz],
                                         w[0][ox] * w[1][oy] * dw[2][oz]};
                        if (gw[0] == T(0) && gw[1] == T(0) && gw[2] == T(0)) continue;
                        const vec4<T> add = mk4<T>(T(0), Am[0] * gw[0] + Am[1] * gw[1] + Am[2] * gw[2],
                                                   Am[3] * gw[0] + Am[4] * gw[1] + Am[5] * gw[2],
                                                   Am[6] * gw[0] + Am[7] * gw[1] + Am[8] * gw[2]);
                        red_add4(gacc + ((size_t)gx * P.M[1] + gy) * P.M[2] + gz, add);
                    }
        }
    }
    block_add(e_out, energy);
}

// The kinetic part over the cells with mass, 1/2 m |v - v*|^2 (Energy,
// material_point_method.cpp:160-173), summed into energy[0]; GRAD: the
// compact gradient g[k] = m (v - v*) + the particles' part gathered from gacc,
// whose entry is cleared for the next evaluation.  v: the compact trial
// point x + a d (d may be null).
template <typename T, bool GRAD>
__global__ void __launch_bounds__(256) k_imp_cells(const vec4<T>* __restrict__ grid, const uint32_t* __restrict__ idx,
                                                   int nused, const T* __restrict__ vstar, const T* __restrict__ x,
                                                   T a, const T* __restrict__ d, vec4<T>* __restrict__ gacc,
                                                   T* __restrict__ g, double* energy) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    double e_out = 0.0;
    if (k < nused) {
        const uint32_t c = idx[k];
        const T m = grid[c].x;
        T dv[3];
#pragma unroll
        for (int r = 0; r < 3; ++r) dv[r] = (d ? x[3 * k + r] + a * d[3 * k + r] : x[3 * k + r]) - vstar[3 * k + r];
        e_out = 0.5 * (double)m * ((double)dv[0] * dv[0] + (double)dv[1] * dv[1] + (double)dv[2] * dv[2]);
        if (GRAD) {
            const vec4<T> ga = gacc[c];
            g[3 * k] = m * dv[0] + ga.y;
            g[3 * k + 1] = m * dv[1] + ga.z;
            g[3 * k + 2] = m * dv[2] + ga.w;
            gacc[c] = mk4<T>(T(0), T(0), T(0), T(0));
        }
    }
    block_add(e_out, energy);
}

// out[0] += sum a . b, out[1] += sum b . b (n reals); b may alias a.
template <typename T>
__global__ void __launch_bounds__(256) k_imp_dot(const T* __restrict__ a, const T* __restrict__ b, int n,
                                                 double* out) {
    double ab = 0.0, bb = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        ab += (double)a[i] * (double)b[i];
        bb += (double)b[i] * (double)b[i];
    }
    block_add(ab, out);
    block_add(bb, out + 1);
}

// y = y + a x (n reals).
template <typename T>
__global__ void __launch_bounds__(256) k_imp_axpy(T* __restrict__ y, T a, const T* __restrict__ x, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] += a * x[i];
}

// y = a y (n reals).
template <typename T>
__global__ void __launch_bounds__(256) k_imp_scale(T* __restrict__ y, T a, int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) y[i] *= a;
}

// z = x - y (n reals).
template <typename T>
__global__ void __launch_bounds__(256) k_imp_sub(T* __restrict__ z, const T* __restrict__ x, const T* __restrict__ y,
                                                 int n) {
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) z[i] = x[i] - y[i];
}

// Largest |x_i| (n reals) into *out as the bits of a non-negative double.
template <typename T>
__global__ void __launch_bounds__(256) k_imp_absmax(const T* __restrict__ x, int n, unsigned long long* out) {
    double m = 0.0;
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x)
        m = fmax(m, fabs((double)x[i]));
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_xor_sync(0xffffffffu, m, o));
    if ((threadIdx.x & 31) == 0 && m > 0.0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

}  // namespace rd
