// Reverse-mode kernels of the explicit MLS-MPM step (the step of rd_step,
// lagged-B order): the adjoint of every stage of
//   P2G + forces  (material_point_method.cpp:94-129,235-254)
//   grid update   (:256-262, sticky walls)
//   F update      (:306-330, plastic clamp of the singular values)
//   G2P, advection(:332-350, position clamp :381-388)
// for one step n, given the adjoint of the state after the step.
//
// Forward step n, per particle p with stencil nodes i, w_ip the cubic
// B-spline weight and d_ip = x_i - x_p:
//   m_i = sum w m_p,  q_i = sum w (m_p v_p + A_p d_ip),
//   A_p = m_p D B_p - dt V_p D tau(F_p, J_P),  D = DpInverse (a scalar)
//   vh_i = q_i / m_i + dt g  (0 where m_i = 0 and on walls)
//   v'_p = sum w vh_i,  B'_p = sum w vh_i d_ip^T
//   F* = (I + dt D B_p) F_p = U S V^T,  F'_p = U clamp(S) V^T,
//   J_P' = J_P prod S_k / clamp(S_k)
//   x'_p = clamp(x_p + dt v'_p)
// tau = P F^T = 2 mu (F F^T - U S U^T) + lambda J (J - 1) I (fixed corotated,
// mu, lambda = (mu0, lambda0) exp(xi (1 - J_P))).
//
// Reverse, two kernels per step (adjoints carry a trailing "b"):
//   k_adj_g2p  advection and clamp, the G2P gather turned into a scatter of
//              vh_b to the grid, and the backward of the plastic split (SVD
//              derivative with the clamp's subgradient).
//   k_adj_p2g  vh_b -> (m_b, q_b) per node while the tile is staged, then the
//              P2G scatter turned into a gather of (m_b, q_b), A_b -> B_b and
//              the stress backward.
// Both run a CTA per work item of the step-n state's sort, with the grid
// around the item's block staged in shared memory like the forward kernels.
// The adjoint of state n is indexed like the particle planes of state n
// (slot order).  Step n's fused kernel moved the particle in slot perm[s] of
// state n to slot s of state n + 1, so a thread handling sorted position s
// reads the adjoint of state n + 1 at s (coalesced), keeps its partial
// results at s, and stores the adjoint of state n at slot perm[s].
#pragma once

#include "rd_kernels.cuh"

namespace rd {

// v / h, exactly: a product where h is a power of two, else the division.
template <typename T>
__device__ __forceinline__ T over_h(const DevParams<T>& P, T v) {
    return P.hinv_pow2 != T(0) ? v * P.hinv_pow2 : v / P.h;
}
template <typename T>
__device__ __forceinline__ T x_over_h(const DevParams<T>& P, T x) {
    return P.hinv_pow2 != T(0) ? x * P.hinv_pow2 : div_rn(x, P.h);
}

// d w / d t of bspline4's four weights (t = x / h, f = t - base, g = 1 - f).
template <typename T>
__device__ __forceinline__ void bspline4_dt(T t, int base, T dw[4]) {
    const T f = t - (T)base;
    const T g = (T)(base + 1) - t;
    dw[0] = -T(0.5) * g * g;
    dw[1] = T(1.5) * f * f - T(2) * f;
    dw[2] = -(T(1.5) * g * g - T(2) * g);
    dw[3] = T(0.5) * f * f;
}

// Grid velocity of step n as k_g2p2g stages it: vh = p / m + dt g, zero where
// m = 0 and on sticky walls.
template <typename T>
__device__ __forceinline__ bool node_velocity(const DevParams<T>& P, const vec4<T>& g4, int gx, int gy, int gz,
                                              T vh[3]) {
    vh[0] = vh[1] = vh[2] = T(0);
    if (g4.x == T(0)) return false;
    if (P.bc == 1 && wall_node(P, gx, gy, gz)) return false;
    vh[0] = g4.y / g4.x + P.dt * P.g[0];
    vh[1] = g4.z / g4.x + P.dt * P.g[1];
    vh[2] = g4.w / g4.x + P.dt * P.g[2];
    return true;
}

// Adjoint state of all particles in slot order: kAdjPlanes vec4 planes of n
// entries, so a thread moves its particle's 25 values with 8 coalesced
// 16-byte accesses: 0: x0 x1 x2 J_P | 1: v0 v1 v2 - | 2-4: B row-major |
// 5-7: F row-major (the last entry of each matrix's third plane is spare).
constexpr int kAdjPlanes = 8;
constexpr int kAdjB = 2, kAdjF = 5;
template <typename T> struct AdjState {
    vec4<T>* p;
    size_t n;
};

template <typename T>
__device__ __forceinline__ void adj_load_xj(const AdjState<T>& A, size_t i, T x[3], T& Jp) {
    const vec4<T> a = A.p[i];
    x[0] = a.x; x[1] = a.y; x[2] = a.z; Jp = a.w;
}
template <typename T>
__device__ __forceinline__ void adj_load_v(const AdjState<T>& A, size_t i, T v[3]) {
    const vec4<T> a = A.p[A.n + i];
    v[0] = a.x; v[1] = a.y; v[2] = a.z;
}
template <typename T>
__device__ __forceinline__ void adj_load_mat(const AdjState<T>& A, int plane, size_t i, T M[9]) {
    const vec4<T> a = A.p[plane * A.n + i], b = A.p[(plane + 1) * A.n + i], c = A.p[(plane + 2) * A.n + i];
    M[0] = a.x; M[1] = a.y; M[2] = a.z; M[3] = a.w; M[4] = b.x; M[5] = b.y; M[6] = b.z; M[7] = b.w; M[8] = c.x;
}
template <typename T>
__device__ __forceinline__ void adj_store_xj(const AdjState<T>& A, size_t i, const T x[3], T Jp) {
    A.p[i] = mk4<T>(x[0], x[1], x[2], Jp);
}
template <typename T>
__device__ __forceinline__ void adj_store_v(const AdjState<T>& A, size_t i, const T v[3]) {
    A.p[A.n + i] = mk4<T>(v[0], v[1], v[2], T(0));
}
template <typename T>
__device__ __forceinline__ void adj_store_mat(const AdjState<T>& A, int plane, size_t i, const T M[9]) {
    A.p[plane * A.n + i] = mk4<T>(M[0], M[1], M[2], M[3]);
    A.p[(plane + 1) * A.n + i] = mk4<T>(M[4], M[5], M[6], M[7]);
    A.p[(plane + 2) * A.n + i] = mk4<T>(M[8], T(0), T(0), T(0));
}

// Per scene: sums of mu0_b, lambda0_b, theta_c_b, theta_s_b.
constexpr int kAccPerScene = 4;

// Per-scene parameter adjoints are summed per sorted position over all steps
// (position s belongs to the same scene in every step) and reduced per scene
// at the end.  pacc holds two double2 planes of n: (mu0, lambda0) at s and
// (theta_c, theta_s) at n + s, so each reverse kernel adds its pair with one
// coalesced 16-byte read-modify-write.
__device__ __forceinline__ void acc_add2(double* pacc, size_t plane_off, double a, double b) {
    double2* q = reinterpret_cast<double2*>(pacc) + plane_off;
    const double2 o = *q;
    *q = make_double2(o.x + a, o.y + b);
}

__global__ void __launch_bounds__(256) k_reduce_acc(const double* __restrict__ pacc,
                                                    const uint32_t* __restrict__ spoff, int nscenes, int n,
                                                    double* __restrict__ acc) {
    __shared__ double part[kAccPerScene][8];
    const int s = blockIdx.x;
    if (s >= nscenes) return;
    const int lo = spoff ? (int)spoff[s] : 0, hi = spoff ? (int)spoff[s + 1] : n;
    double sum[kAccPerScene] = {0.0, 0.0, 0.0, 0.0};
    const double2* pp = reinterpret_cast<const double2*>(pacc);
    for (int i = lo + threadIdx.x; i < hi; i += blockDim.x) {
        const double2 ml = pp[i], th = pp[(size_t)n + i];
        sum[0] += ml.x; sum[1] += ml.y; sum[2] += th.x; sum[3] += th.y;
    }
#pragma unroll
    for (int k = 0; k < kAccPerScene; ++k) {
        double v = sum[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
        if ((threadIdx.x & 31) == 0) part[k][threadIdx.x >> 5] = v;
    }
    __syncthreads();
    if (threadIdx.x < kAccPerScene) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[threadIdx.x][w];
        acc[kAccPerScene * s + threadIdx.x] = t;
    }
}

// Backward of the plastic split F' = U clamp(S) V^T, J_P' = J_P prod S / clamp(S)
// of F* = U S V^T.  Fb' and Jpb' are the adjoints of the outputs; returns
// F*_b, the factor J_P' / J_P (for J_P_b) and the theta adjoints.  In the SVD
// basis, M = U^T Fb' V: diagonal k gets g'_k M_kk (g' = 1 unclamped, 0
// clamped) plus Jpb' J_P' (1 / S_k - g'_k / g_k); each off-diagonal pair
// (k, l) gets ((a s + b t), (a s - b t)) / 2 with s = M_kl + M_lk,
// t = M_kl - M_lk, a = (g_k - g_l) / (S_k - S_l), b = (g_k + g_l) / (S_k + S_l).
template <typename T>
__device__ __forceinline__ void split_backward(const DevParams<T>& P, const T U[9], const T s[3], const T V[9],
                                               const T Fb[9], T Jpb_out, T Jp_old, T Fsb[9], T& ratio, T& thc_b,
                                               T& ths_b) {
    T g[3], gp[3];
    ratio = T(1);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if (s[k] < P.lo) { g[k] = P.lo; gp[k] = T(0); }
        else if (s[k] > P.hi) { g[k] = P.hi; gp[k] = T(0); }
        else { g[k] = s[k]; gp[k] = T(1); }
        ratio *= s[k] / g[k];
    }
    const T Jp_new = Jp_old * ratio;
    // M = U^T Fb V
    T t1[9], M[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            t1[3 * r + c] = U[r] * Fb[c] + U[3 + r] * Fb[3 + c] + U[6 + r] * Fb[6 + c];  // (U^T Fb)_rc
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            M[3 * r + c] = t1[3 * r] * V[c] + t1[3 * r + 1] * V[3 + c] + t1[3 * r + 2] * V[6 + c];
    T G[9];
    thc_b = ths_b = T(0);
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        G[4 * k] = gp[k] * M[4 * k] + Jpb_out * Jp_new * (T(1) / s[k] - gp[k] / g[k]);
        const T dg = M[4 * k] - Jpb_out * Jp_new / g[k];  // d L / d g_k
        if (s[k] < P.lo) thc_b -= dg;
        else if (s[k] > P.hi) ths_b += dg;
    }
    const int pk[3] = {0, 0, 1}, pl[3] = {1, 2, 2};
#pragma unroll
    for (int q = 0; q < 3; ++q) {
        const int k = pk[q], l = pl[q];
        const T ds = s[k] - s[l];
        T a;
        if (gp[k] == T(1) && gp[l] == T(1)) a = T(1);
        else if (fabs(ds) > T(1e-6) * (s[k] + s[l])) a = (g[k] - g[l]) / ds;
        else a = T(0.5) * (gp[k] + gp[l]);
        const T b = (g[k] + g[l]) / (s[k] + s[l]);
        const T sm = M[3 * k + l] + M[3 * l + k], df = M[3 * k + l] - M[3 * l + k];
        G[3 * k + l] = T(0.5) * (a * sm + b * df);
        G[3 * l + k] = T(0.5) * (a * sm - b * df);
    }
    // Fsb = U G V^T
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            t1[3 * r + c] = U[3 * r] * G[c] + U[3 * r + 1] * G[3 + c] + U[3 * r + 2] * G[6 + c];  // (U G)_rc
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            Fsb[3 * r + c] = t1[3 * r] * V[3 * c] + t1[3 * r + 1] * V[3 * c + 1] + t1[3 * r + 2] * V[3 * c + 2];
}

// Backward of tau = 2 mu (F F^T - U S U^T) + lambda J (J - 1) I for the
// adjoint tb of tau (only its symmetric part matters).  Adds to Fb and
// returns the adjoints of J_P, mu0 and lambda0.  With F F^T = U S^2 U^T, the
// left stretch U S U^T = sqrt(F F^T) has the derivative
// (U^T d(FF^T) U)_kl / (S_k + S_l) in the U basis, which stays finite at
// repeated singular values.  U, S (and S - 1) are the SVD the forward stress
// used.  Assumes det F > 0 (no inverted particles).
template <typename T>
__device__ __forceinline__ void stress_backward(const DevParams<T>& P, const T F[9], T Jp, const T U[9],
                                                const T s[3], const T sm1[3], const T tb[9], T Fb[9], T& Jpb,
                                                T& mu0b, T& lam0b) {
    T ts[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c) ts[3 * r + c] = T(0.5) * (tb[3 * r + c] + tb[3 * c + r]);
    const T J = det3(F);
    const T hard = exp_(P.xi * (T(1) - Jp));
    const T mu = P.mu0 * hard, lam = P.lambda0 * hard;
    // mu_b = 2 ts : U (S^2 - S) U^T,  lambda_b = tr(ts) J (J - 1)
    T Mt[9], t1[9];  // U^T ts U
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            t1[3 * r + c] = U[r] * ts[c] + U[3 + r] * ts[3 + c] + U[6 + r] * ts[6 + c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            Mt[3 * r + c] = t1[3 * r] * U[c] + t1[3 * r + 1] * U[3 + c] + t1[3 * r + 2] * U[6 + c];
    const T tr = ts[0] + ts[4] + ts[8];
    const T mub = T(2) * (Mt[0] * sm1[0] * s[0] + Mt[4] * sm1[1] * s[1] + Mt[8] * sm1[2] * s[2]);
    const T lamb = tr * J * (J - T(1));
    // F F^T term: 4 mu ts F; left stretch: b_b = U ((-2 mu Mt) / (S_k + S_l)) U^T, Fb += 2 b_b F
    T Bs[9];
#pragma unroll
    for (int k = 0; k < 3; ++k)
#pragma unroll
        for (int l = 0; l < 3; ++l) Bs[3 * k + l] = -T(2) * mu * Mt[3 * k + l] / (s[k] + s[l]);
    T bb[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            t1[3 * r + c] = U[3 * r] * Bs[c] + U[3 * r + 1] * Bs[3 + c] + U[3 * r + 2] * Bs[6 + c];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            bb[3 * r + c] = t1[3 * r] * U[3 * c] + t1[3 * r + 1] * U[3 * c + 1] + t1[3 * r + 2] * U[3 * c + 2];
    T K[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) K[e] = T(4) * mu * ts[e] + T(2) * bb[e];
    T KF[9];
    matmul3(KF, K, F);
    // lambda term: tr(ts) lambda (2J - 1) cof(F)
    const T cl = tr * lam * (T(2) * J - T(1));
    T cof[9];
    cof[0] = F[4] * F[8] - F[5] * F[7]; cof[1] = F[5] * F[6] - F[3] * F[8]; cof[2] = F[3] * F[7] - F[4] * F[6];
    cof[3] = F[2] * F[7] - F[1] * F[8]; cof[4] = F[0] * F[8] - F[2] * F[6]; cof[5] = F[1] * F[6] - F[0] * F[7];
    cof[6] = F[1] * F[5] - F[2] * F[4]; cof[7] = F[2] * F[3] - F[0] * F[5]; cof[8] = F[0] * F[4] - F[1] * F[3];
#pragma unroll
    for (int e = 0; e < 9; ++e) Fb[e] += KF[e] + cl * cof[e];
    Jpb += -P.xi * (mu * mub + lam * lamb);
    mu0b = mub * hard;
    lam0b = lamb * hard;
}

// ---------------------------------------------------------------- tiled reverse step
// Both reverse kernels walk the work items of the sort of the step-n state
// (kept from the recompute): a CTA per item, one particle per thread.
constexpr int kAdjThreads = 256;
// Two resident CTAs per SM in FP32 (at most 128 registers a thread; the batch
// instantiations would otherwise take more and run one CTA, half the warps);
// FP64 needs over 200 registers a thread and runs one.
template <typename T> constexpr int kAdjMinBlocks = sizeof(T) == 4 ? 2 : 1;
static_assert(WorkP<float>::value <= kAdjThreads && WorkP<double>::value <= kAdjThreads,
              "one particle per thread");

template <typename T> struct AdjG2PShared {
    vec4<T> gv[kTileCells];   // grid velocity of step n around the item's block
    P2GTile<T, kBlk> p;       // records of the vh_b scatter
    DevParams<T> par;
};

// Reverse of G2P, advection and the plastic split for one work item.  The
// scatter of vh_b_i = w (v'_b + B'_b d_i) has the form of a P2G record
// (q' = v'_b + B'_b e, A = B'_b, no mass), so it goes through the same
// cell-sorted register accumulation and tile flush as the forward P2G.
template <typename T>
__device__ __forceinline__ void adj_g2p_item(const DevParams<T>& P, const DevBufs& D, AdjG2PShared<T>& S,
                                             const int4 it, const vec4<T>* __restrict__ st,
                                             const vec4<T>* __restrict__ grid0, vec4<T>* __restrict__ agrid0,
                                             const AdjState<T>& nxt, const AdjState<T>& part,
                                             double* __restrict__ pacc, const vec4<T>* __restrict__ split) {
    const vec4<T>* grid = grid0 + P.goff;
    vec4<T>* agrid = agrid0 + P.goff;
    int org[3];
    tile_origin(P, it.x, org);
    const int count = min(it.z, min(WorkP<T>::value, P.n - it.y));
    for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
        size_t lin;
        T vh[3] = {T(0), T(0), T(0)};
        if (cell_of_tile(P, org, c, lin)) {
            const int ix = c / (kTile * kTile), iy = (c / kTile) % kTile, iz = c % kTile;
            node_velocity(P, grid[lin], org[0] + ix, org[1] + iy, org[2] + iz, vh);
        }
        S.gv[c] = mk4<T>(vh[0], vh[1], vh[2], T(0));
    }
    zero_tile(S.p);
    for (int c = threadIdx.x; c < P2GTile<T, kBlk>::NC; c += blockDim.x) S.p.cnt[c] = 0;
    __syncthreads();
    const int j = threadIdx.x;
    int rcell = 0xff, rrank = 0;  // this thread's record: cell and rank within it
    if (j < count) {
        const uint32_t sp = (uint32_t)(it.y + j);  // sorted position: slot of this particle in state n + 1
        const uint32_t idx = D.perm[sp];
        Particle<T> p;
        load_particle(st, (size_t)P.n, idx, p);
        Stencil<T> St;
        const bool ok = idx < (uint32_t)P.n && make_stencil(P, p.x, org, St);
        if (!ok) {
            raise_flag(D.flags, 4u);
            S.p.cellof[j] = 0xff;
        } else {
            T dw[3][4];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                bspline4_dt(x_over_h(P, p.x[a]), St.b[a], dw[a]);
#pragma unroll
                for (int o = 0; o < 4; ++o) dw[a][o] = over_h(P, dw[a][o]);
            }
            T vn[3], Bn[9];
            g2p_gather(S.gv, St, vn, Bn);
            // advection x' = clamp(x + dt v')
            T xb[3], vb[3], Bb[9], Jpb1;
            adj_load_xj(nxt, sp, xb, Jpb1);
            adj_load_v(nxt, sp, vb);
            adj_load_mat(nxt, kAdjB, sp, Bb);
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                const T xn = p.x[a] + vn[a] * P.dt;
                const T mask = (xn >= P.xlo && xn <= P.xhi[a]) ? T(1) : T(0);
                xb[a] *= mask;
                vb[a] += P.dt * xb[a];
            }
#pragma unroll
            for (int c = 0; c < 3; ++c) xb[c] -= Bb[c] * vn[0] + Bb[3 + c] * vn[1] + Bb[6 + c] * vn[2];
            // x_b += sum_i grad w_i s_i with s_i = vh_i . u_i, u_i = v'_b + B'_b d_i.
            // Separably: for each (ox, oy) column u = (v'_b + B'_b[:,0] d_x +
            // B'_b[:,1] d_y) + B'_b[:,2] d_z, and the z sums c0 = sum w_z s,
            // c1 = sum dw_z s come first, then the y sums, then the x sums.
            for (int ox = 0; ox < 4; ++ox) {
                T ax = T(0), ay = T(0), az = T(0);
                for (int oy = 0; oy < 4; ++oy) {
                    const int rowc = ((St.rel[0] + ox) * kTile + (St.rel[1] + oy)) * kTile + St.rel[2];
                    T ucol[3];
#pragma unroll
                    for (int r = 0; r < 3; ++r)
                        ucol[r] = vb[r] + Bb[3 * r] * St.d[0][ox] + Bb[3 * r + 1] * St.d[1][oy];
                    T c0 = T(0), c1 = T(0);
#pragma unroll
                    for (int oz = 0; oz < 4; ++oz) {
                        const vec4<T> v4 = S.gv[rowc + oz];
                        const T dz = St.d[2][oz];
                        const T sdot = v4.x * (ucol[0] + Bb[2] * dz) + v4.y * (ucol[1] + Bb[5] * dz) +
                                       v4.z * (ucol[2] + Bb[8] * dz);
                        c0 += St.w[2][oz] * sdot;
                        c1 += dw[2][oz] * sdot;
                    }
                    ax += St.w[1][oy] * c0;
                    ay += dw[1][oy] * c0;
                    az += St.w[1][oy] * c1;
                }
                xb[0] += dw[0][ox] * ax;
                xb[1] += St.w[0][ox] * ay;
                xb[2] += St.w[0][ox] * az;
            }
            // the vh_b scatter as a record: q' = v'_b + B'_b e, A = B'_b
            write_record<T, false>(&S.p.rec[j * kRecV4], St, p.x, Bb, vb, T(0), P.h);
            rcell = (St.rel[0] * kBlk + St.rel[1]) * kBlk + St.rel[2];
            S.p.cellof[j] = (uint8_t)rcell;
            rrank = atomicAdd(&S.p.cnt[rcell], 1);
            // plastic split of F* = (I + dt D B) F (lagged B)
            T A[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) A[e] = p.B[e] * P.dinv * P.dt;
            A[0] += T(1); A[4] += T(1); A[8] += T(1);
            // the SVD of F* = A F the forward made in this step (the recompute
            // keeps it per sorted slot): no second SVD here
            T U[9], s[3], V[9];
            {
                T sm1[3];
                load_split(split, (size_t)P.n, sp, U, s, sm1, V);
            }
            T Fb1[9];
            adj_load_mat(nxt, kAdjF, sp, Fb1);
            T Fsb[9], g_ratio, thc_b, ths_b;
            split_backward(P, U, s, V, Fb1, Jpb1, p.Jp, Fsb, g_ratio, thc_b, ths_b);
            T pF[9], pB[9];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) {
                    pF[3 * r + c] = A[r] * Fsb[c] + A[3 + r] * Fsb[3 + c] + A[6 + r] * Fsb[6 + c];
                    pB[3 * r + c] =
                        P.dt * P.dinv *
                        (Fsb[3 * r] * p.F[3 * c] + Fsb[3 * r + 1] * p.F[3 * c + 1] + Fsb[3 * r + 2] * p.F[3 * c + 2]);
                }
            adj_store_mat(part, kAdjF, sp, pF);
            adj_store_mat(part, kAdjB, sp, pB);
            adj_store_xj(part, sp, xb, Jpb1 * g_ratio);
            acc_add2(pacc, (size_t)P.n + sp, (double)thc_b, (double)ths_b);
        }
    }
    sort_ranked<T, kBlk>(S.p, j, rcell, rrank);
    p2g_runs<T, false, kBlk>(S.p, sorted_total(S.p));
    __syncthreads();
    p2g_flush<T, kBlk>(P, S.p, org, agrid);
    __syncthreads();
}

template <typename T, bool BATCH>
__global__ void __launch_bounds__(kAdjThreads, kAdjMinBlocks<T>) k_adj_g2p(DevParams<T> P0, DevBufs D, const vec4<T>* __restrict__ st,
                                                        const vec4<T>* __restrict__ grid0,
                                                        vec4<T>* __restrict__ agrid0, AdjState<T> nxt,
                                                        AdjState<T> part, double* __restrict__ pacc,
                                                        const vec4<T>* __restrict__ split) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    AdjG2PShared<T>& S = *reinterpret_cast<AdjG2PShared<T>*>(smem_raw);
    uint32_t nf, nb;
    work_counts(D, nf, nb);
    const uint32_t nw = nf + nb;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = work_item(D, nf, wi);
        if constexpr (BATCH) {
            copy_scene(S.par, D.scenes, it.w);
            __syncthreads();
            adj_g2p_item<T>(S.par, D, S, it, st, grid0, agrid0, nxt, part, pacc, split);
        } else {
            adj_g2p_item<T>(P0, D, S, it, st, grid0, agrid0, nxt, part, pacc, split);
        }
    }
}

template <typename T> struct AdjP2GShared {
    vec4<T> ag[kTileCells];  // (m_b, q_b) around the item's block
    DevParams<T> par;
};

// Reverse of P2G + forces for one work item.  The (m_b, q_b) tile comes from
// vh_b and the step's grid while it is staged: vh = q / m + dt g gives
// q_b = vh_b / m, m_b = -(q / m) . vh_b / m (zero where vh was set to zero).
template <typename T>
__device__ __forceinline__ void adj_p2g_item(const DevParams<T>& P, const DevBufs& D, AdjP2GShared<T>& S,
                                             const int4 it, const vec4<T>* __restrict__ st,
                                             const vec4<T>* __restrict__ grid0, const vec4<T>* __restrict__ agrid0,
                                             const AdjState<T>& part, const AdjState<T>& cur,
                                             double* __restrict__ pacc, const vec4<T>* __restrict__ prev_split) {
    const vec4<T>* grid = grid0 + P.goff;
    const vec4<T>* agrid = agrid0 + P.goff;
    int org[3];
    tile_origin(P, it.x, org);
    const int count = min(it.z, min(WorkP<T>::value, P.n - it.y));
    for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
        size_t lin;
        vec4<T> out = mk4<T>(T(0), T(0), T(0), T(0));
        if (cell_of_tile(P, org, c, lin)) {
            const int ix = c / (kTile * kTile), iy = (c / kTile) % kTile, iz = c % kTile;
            const vec4<T> g4 = grid[lin];
            if (g4.x != T(0) && !(P.bc == 1 && wall_node(P, org[0] + ix, org[1] + iy, org[2] + iz))) {
                const vec4<T> ab = agrid[lin];
                const T im = T(1) / g4.x;
                out.y = ab.y * im;
                out.z = ab.z * im;
                out.w = ab.w * im;
                out.x = -(g4.y * out.y + g4.z * out.z + g4.w * out.w) * im;
            }
        }
        S.ag[c] = out;
    }
    __syncthreads();
    const int j = threadIdx.x;
    if (j < count) {
        const uint32_t sp = (uint32_t)(it.y + j);
        const uint32_t idx = D.perm[sp];
        Particle<T> p;
        load_particle(st, (size_t)P.n, idx, p);
        Stencil<T> St;
        if (idx < (uint32_t)P.n && make_stencil(P, p.x, org, St)) {
            T dw[3][4];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                bspline4_dt(x_over_h(P, p.x[a]), St.b[a], dw[a]);
#pragma unroll
                for (int o = 0; o < 4; ++o) dw[a][o] = over_h(P, dw[a][o]);
            }
            T U[9], sv[3], svm1[3], tau[9], A[9], mv[3];
            if (prev_split) {
                // F of this state is U clamp(S) V^T of the previous step's split
                // (kept at this state's slot by the recompute): its SVD as is
                T V[9];
                load_split(prev_split, (size_t)P.n, idx, U, sv, svm1, V);
#pragma unroll
                for (int k = 0; k < 3; ++k) {
                    if (sv[k] < P.lo) { sv[k] = P.lo; svm1[k] = P.lo - T(1); }
                    else if (sv[k] > P.hi) { sv[k] = P.hi; svm1[k] = P.hi - T(1); }
                }
            } else {
                T V[9];
                svd3_near(p.F, U, sv, svm1, V);
            }
            stress_PFt_svd(P, p.F, p.Jp, U, sv, svm1, tau);
            const T fs = P.dt * p.vol * P.dinv;
#pragma unroll
            for (int e = 0; e < 9; ++e) A[e] = p.m * (p.B[e] * P.dinv) - fs * tau[e];
#pragma unroll
            for (int a = 0; a < 3; ++a) mv[a] = p.m * p.v[a];
            T swq[3] = {T(0), T(0), T(0)}, Ab[9], xb[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int e = 0; e < 9; ++e) Ab[e] = T(0);
            for (int ox = 0; ox < 4; ++ox)
                for (int oy = 0; oy < 4; ++oy) {
                    const int rowc = ((St.rel[0] + ox) * kTile + (St.rel[1] + oy)) * kTile + St.rel[2];
                    const T wxy = St.w[0][ox] * St.w[1][oy];
#pragma unroll
                    for (int oz = 0; oz < 4; ++oz) {
                        const vec4<T> a4 = S.ag[rowc + oz];
                        const T d[3] = {St.d[0][ox], St.d[1][oy], St.d[2][oz]};
                        const T w = wxy * St.w[2][oz];
                        const T qb[3] = {a4.y, a4.z, a4.w};
#pragma unroll
                        for (int r = 0; r < 3; ++r) {
                            const T wq = w * qb[r];
                            swq[r] += wq;
                            Ab[3 * r] += wq * d[0];
                            Ab[3 * r + 1] += wq * d[1];
                            Ab[3 * r + 2] += wq * d[2];
                        }
                        T q[3];
#pragma unroll
                        for (int r = 0; r < 3; ++r)
                            q[r] = mv[r] + (A[3 * r] * d[0] + A[3 * r + 1] * d[1] + A[3 * r + 2] * d[2]);
                        const T sdot = p.m * a4.x + qb[0] * q[0] + qb[1] * q[1] + qb[2] * q[2];
                        xb[0] += sdot * (dw[0][ox] * St.w[1][oy] * St.w[2][oz]);
                        xb[1] += sdot * (St.w[0][ox] * dw[1][oy] * St.w[2][oz]);
                        xb[2] += sdot * (wxy * dw[2][oz]);
                    }
                }
            // d_ip = x_i - x_p: x_b -= A^T sum w q_b
#pragma unroll
            for (int c = 0; c < 3; ++c) xb[c] -= A[c] * swq[0] + A[3 + c] * swq[1] + A[6 + c] * swq[2];
            T tb[9], Fb[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) { tb[e] = -fs * Ab[e]; Fb[e] = T(0); }
            T Jpb = T(0), mu0b = T(0), lam0b = T(0);
            stress_backward(P, p.F, p.Jp, U, sv, svm1, tb, Fb, Jpb, mu0b, lam0b);
            {
                T px[3], pJp, vo[3];
                adj_load_xj(part, sp, px, pJp);
#pragma unroll
                for (int a = 0; a < 3; ++a) { px[a] += xb[a]; vo[a] = p.m * swq[a]; }
                adj_store_xj(cur, idx, px, pJp + Jpb);
                adj_store_v(cur, idx, vo);
            }
            {
                T M[9];
                adj_load_mat(part, kAdjB, sp, M);
#pragma unroll
                for (int e = 0; e < 9; ++e) M[e] += p.m * P.dinv * Ab[e];
                adj_store_mat(cur, kAdjB, idx, M);
                adj_load_mat(part, kAdjF, sp, M);
#pragma unroll
                for (int e = 0; e < 9; ++e) M[e] += Fb[e];
                adj_store_mat(cur, kAdjF, idx, M);
            }
            acc_add2(pacc, sp, (double)mu0b, (double)lam0b);
        } else {
            raise_flag(D.flags, 4u);
        }
    }
    __syncthreads();
}

template <typename T, bool BATCH>
__global__ void __launch_bounds__(kAdjThreads, kAdjMinBlocks<T>) k_adj_p2g(DevParams<T> P0, DevBufs D, const vec4<T>* __restrict__ st,
                                                        const vec4<T>* __restrict__ grid0,
                                                        const vec4<T>* __restrict__ agrid0, AdjState<T> part,
                                                        AdjState<T> cur, double* __restrict__ pacc,
                                                        const vec4<T>* __restrict__ prev_split) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    AdjP2GShared<T>& S = *reinterpret_cast<AdjP2GShared<T>*>(smem_raw);
    uint32_t nf, nb;
    work_counts(D, nf, nb);
    const uint32_t nw = nf + nb;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = work_item(D, nf, wi);
        if constexpr (BATCH) {
            copy_scene(S.par, D.scenes, it.w);
            __syncthreads();
            adj_p2g_item<T>(S.par, D, S, it, st, grid0, agrid0, part, cur, pacc, prev_split);
        } else {
            adj_p2g_item<T>(P0, D, S, it, st, grid0, agrid0, part, cur, pacc, prev_split);
        }
    }
}

// The adjoint of the final state in its slot order from dL/dx, dL/dv given in
// particle id order (either may be NULL: zero).
template <typename T>
__global__ void k_adj_seed(int n, const vec4<T>* __restrict__ st, const T* __restrict__ gx,
                           const T* __restrict__ gv, AdjState<T> A) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = real_to_id<T>(st[6 * (size_t)n + i].w);
    T x[3], v[3], Z[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        x[a] = (gx && id < (uint32_t)n) ? gx[3 * id + a] : T(0);
        v[a] = (gv && id < (uint32_t)n) ? gv[3 * id + a] : T(0);
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) Z[e] = T(0);
    adj_store_xj(A, i, x, T(0));
    adj_store_v(A, i, v);
    adj_store_mat(A, kAdjB, i, Z);
    adj_store_mat(A, kAdjF, i, Z);
}

// Slot order -> particle id order (into a scratch adjoint) and back, for the
// step between two copies of one state whose sorts placed particles in
// different slots (a checkpoint and its recomputation).
template <typename T>
__global__ void k_adj_to_id(int n, const vec4<T>* __restrict__ st, AdjState<T> from, AdjState<T> by_id) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = real_to_id<T>(st[6 * (size_t)n + i].w);
    if (id >= (uint32_t)n) return;
#pragma unroll
    for (int k = 0; k < kAdjPlanes; ++k) by_id.p[k * by_id.n + id] = from.p[k * from.n + i];
}

template <typename T>
__global__ void k_adj_from_id(int n, const vec4<T>* __restrict__ st, AdjState<T> by_id, AdjState<T> to) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = real_to_id<T>(st[6 * (size_t)n + i].w);
    if (id >= (uint32_t)n) return;
#pragma unroll
    for (int k = 0; k < kAdjPlanes; ++k) to.p[k * to.n + i] = by_id.p[k * by_id.n + id];
}

// dL/dv of the start state, from its slot order to particle id order.
template <typename T>
__global__ void k_adj_out(int n, const vec4<T>* __restrict__ st, AdjState<T> A, T* __restrict__ v0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = real_to_id<T>(st[6 * (size_t)n + i].w);
    if (id >= (uint32_t)n) return;
    T v[3];
    adj_load_v(A, i, v);
#pragma unroll
    for (int a = 0; a < 3; ++a) v0[3 * id + a] = v[a];
}

}  // namespace rd
