// sm_103a kernels of the MPM step.  One step of rd_step is
//   k_keys (only when positions changed outside a step) -> k_scan -> k_scatter
//   -> memset(grid) -> k_p2g<fused> -> k_g2p_fused
// and the stage kernels serve rd_stage, which runs the reference's seven
// stages one by one (material_point_method.cpp:94-350).
#pragma once
#include "rd_device.cuh"

namespace rd {

// Particles are bucketed by 4x4x4-cell blocks of their base cell; a work item
// is (block key, first sorted index, count <= WorkP<T>).  Every stencil node of a
// particle whose base cell lies in block b is inside the 7^3-node tile whose
// origin is 4b - 1, so P2G and G2P never leave their shared-memory tile.
constexpr int kBlk = 4;
constexpr int kTile = kBlk + 3;
constexpr int kTileCells = kTile * kTile * kTile;
constexpr int kThreads = 128;

template <typename T> struct DevParams {
    int M[3];      // grid nodes per axis
    int NB[3];     // blocks per axis
    int nkeys;
    int n;         // particles
    T h, dinv, dt;
    T mu0, lambda0, xi;
    T lo, hi;      // singular value clamp
    T g[3];
    T xlo, xhi[3]; // position clamp (material_point_method.cpp:381-388)
    T fscale;      // force scale in P2G: dt when fused with the momentum, 1 alone
    int bc, bc_width;
    int lagged;
};

struct DevBufs {
    const void* pin;   // particle planes read
    void* pout;        // particle planes written (fused G2P: sorted order)
    const uint32_t* perm;
    uint32_t* keys_out;
    uint32_t* counts;
    const int4* work;
    const uint32_t* nwork;
    void* grid;        // vec4 per cell
    void* gforce;      // vec4 per cell (stage mode forces)
    uint32_t* flags;
};

__device__ __forceinline__ void raise_flag(uint32_t* flags, uint32_t f) {
    if ((__ldcg(flags) & f) == 0) atomicOr(flags, f);
}

// Block key of base cell b (clamped into the grid; the caller flags
// out-of-range particles).
template <typename T>
__device__ __forceinline__ uint32_t block_key(const DevParams<T>& P, const int b[3]) {
    int k[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        int c = b[a] < 0 ? 0 : (b[a] > P.M[a] - 1 ? P.M[a] - 1 : b[a]);
        k[a] = c / kBlk;
    }
    return ((uint32_t)k[0] * P.NB[1] + k[1]) * P.NB[2] + k[2];
}

template <typename T>
__device__ __forceinline__ bool stencil_in_grid(const DevParams<T>& P, const int b[3]) {
    return b[0] >= 1 && b[1] >= 1 && b[2] >= 1 && b[0] + 2 < P.M[0] && b[1] + 2 < P.M[1] && b[2] + 2 < P.M[2];
}

// One atomic per distinct key among the active lanes of the warp.
__device__ __forceinline__ void count_key(uint32_t* counts, uint32_t key) {
    const uint32_t peers = __match_any_sync(__activemask(), key);
    const int leader = __ffs(peers) - 1;
    if ((int)(threadIdx.x & 31) == leader) atomicAdd(counts + key, (uint32_t)__popc(peers));
}

// ---------------------------------------------------------------- sorting
template <typename T>
__global__ void __launch_bounds__(256) k_keys(DevParams<T> P, const vec4<T>* __restrict__ pl,
                                              uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                                              uint32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const vec4<T> x = ld_stream(pl + i);
    const int b[3] = {base_of(x.x, P.h), base_of(x.y, P.h), base_of(x.z, P.h)};
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    const uint32_t key = block_key(P, b);
    keys[i] = key;
    count_key(counts, key);
}

// Exclusive scan of the per-block counts into starts (and the scatter cursor),
// emission of the work items, reset of the counts for the next histogram.  One
// CTA of 1024 threads sweeps the key range in chunks of 1024 x kScanK keys.
constexpr int kScanK = 16;
__global__ void __launch_bounds__(1024) k_scan(uint32_t* __restrict__ counts, uint32_t* __restrict__ cursor,
                                               int4* __restrict__ work, uint32_t* __restrict__ nwork, int nkeys,
                                               uint32_t n_expected, uint32_t work_cap, uint32_t wp,
                                               uint32_t* flags) {
    __shared__ uint32_t s_c[32], s_i[32];
    __shared__ uint32_t carry_c, carry_i;
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) { carry_c = 0; carry_i = 0; }
    __syncthreads();
    for (int chunk = 0; chunk < nkeys; chunk += 1024 * kScanK) {
        const int k0 = chunk + tid * kScanK;
        uint32_t c[kScanK];
        uint32_t tc = 0, ti = 0;
#pragma unroll
        for (int k = 0; k < kScanK; ++k) {
            c[k] = (k0 + k < nkeys) ? counts[k0 + k] : 0u;
            tc += c[k];
            ti += (c[k] + wp - 1) / wp;
        }
        // inclusive warp scan of (tc, ti)
        uint32_t ic = tc, ii = ti;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t yc = __shfl_up_sync(0xffffffffu, ic, o), yi = __shfl_up_sync(0xffffffffu, ii, o);
            if (lane >= o) { ic += yc; ii += yi; }
        }
        if (lane == 31) { s_c[wid] = ic; s_i[wid] = ii; }
        __syncthreads();
        if (wid == 0) {
            uint32_t wc = s_c[lane], wi = s_i[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t yc = __shfl_up_sync(0xffffffffu, wc, o), yi = __shfl_up_sync(0xffffffffu, wi, o);
                if (lane >= o) { wc += yc; wi += yi; }
            }
            s_c[lane] = wc; s_i[lane] = wi;
        }
        __syncthreads();
        uint32_t oc = carry_c + (wid ? s_c[wid - 1] : 0u) + ic - tc;
        uint32_t oi = carry_i + (wid ? s_i[wid - 1] : 0u) + ii - ti;
#pragma unroll
        for (int k = 0; k < kScanK; ++k) {
            const int key = k0 + k;
            if (key >= nkeys) break;
            cursor[key] = oc;
            counts[key] = 0u;
            for (uint32_t j = 0; j < c[k]; j += wp) {
                const uint32_t cnt = (c[k] - j) < wp ? (c[k] - j) : wp;
                if (oi < work_cap) work[oi] = make_int4(key, (int)(oc + j), (int)cnt, 0);
                ++oi;
            }
            oc += c[k];
        }
        __syncthreads();
        if (tid == 1023) {
            carry_c += s_c[31];
            carry_i += s_i[31];
        }
        __syncthreads();
    }
    if (tid == 0) {
        // A histogram that does not add up to n would index past the buffers:
        // run no work items and report it instead.
        const bool bad = carry_c != n_expected || carry_i > work_cap;
        *nwork = bad ? 0u : carry_i;
        if (bad) atomicOr(flags, 4u);
    }
}

// perm[sorted position] = particle index.  Within a block the order is that of
// the atomics, so it varies from run to run; the block keys themselves (and
// hence the sorted key sequence) are bit-exact against a CPU sort.
__global__ void __launch_bounds__(256) k_scatter(int n, const uint32_t* __restrict__ keys,
                                                 uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t key = keys[i];
    const uint32_t peers = __match_any_sync(__activemask(), key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t pos = base + __popc(peers & lanemask_lt());
    if (pos < (uint32_t)n) perm[pos] = (uint32_t)i;
}

// ---------------------------------------------------------------- particle math
template <typename T> struct Stencil {
    int b[3];      // base cell
    int rel[3];    // base - 1 - tile origin, in [0, 3]
    T w[3][4];     // weights per axis at offsets -1..2
    T d[3][4];     // x_i - x_p per axis, (base + o) h - x as the reference computes it
};

template <typename T>
__device__ __forceinline__ bool make_stencil(const DevParams<T>& P, const T x[3], const int org[3], Stencil<T>& S) {
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t = div_rn(x[a], P.h);
        S.b[a] = (int)t;
        bspline4(t, S.b[a], S.w[a]);
#pragma unroll
        for (int o = 0; o < 4; ++o) S.d[a][o] = (T)(S.b[a] - 1 + o) * P.h - x[a];
        S.rel[a] = S.b[a] - 1 - org[a];
        ok = ok && S.rel[a] >= 0 && S.rel[a] <= kTile - 4;
    }
    return ok;
}

// P F^T of the fixed-corotated stress with the reference's hardening
// (material_point_method.cpp:239-248): P = 2 mu (F - R) + lambda (J - 1) J F^-T,
// so P F^T = 2 mu (F - R) F^T + lambda (J - 1) J I.  With F = U S V^T and the
// reference's proper rotation R = U D V^T (D = I, or diag(.., -1) on the
// smallest singular value when det F < 0), (F - R) F^T = U (S - D) S U^T.
// F stays within a few 1e-3 of a rotation, so s - 1 and J - 1 are formed
// without cancellation from G = F - I (exact in floating point):
// s_i^2 - 1 = v_i^T (G + G^T + G^T G) v_i and
// J - 1 = tr G + (sum of the principal 2x2 minors of G) + det G.
template <typename T>
__device__ __forceinline__ void stress_PFt(const DevParams<T>& P, const T F[9], T Jp, T out[9]) {
    T U[9], s[3], V[9];
    svd3(F, U, s, V);
    T G[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) G[e] = F[e];
    G[0] -= T(1); G[4] -= T(1); G[8] -= T(1);
    T S[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            S[3 * r + c] = (G[3 * r + c] + G[3 * c + r]) + (G[r] * G[c] + G[3 + r] * G[3 + c] + G[6 + r] * G[6 + c]);
    const T jm1 = (G[0] + G[4] + G[8]) +
                  ((G[0] * G[4] - G[1] * G[3]) + (G[0] * G[8] - G[2] * G[6]) + (G[4] * G[8] - G[5] * G[7])) +
                  det3(G);
    const T J = T(1) + jm1;
    const T hard = exp_(P.xi * (T(1) - Jp));
    const T mu = P.mu0 * hard, lam = P.lambda0 * hard;
    int kmin = 0;
#pragma unroll
    for (int c = 1; c < 3; ++c) kmin = s[c] < s[kmin] ? c : kmin;
    T dg[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T v0 = V[c], v1 = V[3 + c], v2 = V[6 + c];
        const T e = v0 * (S[0] * v0 + S[1] * v1 + S[2] * v2) + v1 * (S[3] * v0 + S[4] * v1 + S[5] * v2) +
                    v2 * (S[6] * v0 + S[7] * v1 + S[8] * v2);
        const T sm = (J < T(0) && c == kmin) ? (s[c] + T(1)) : e / (s[c] + T(1));  // s - d
        dg[c] = T(2) * mu * sm * s[c];
    }
    const T iso = lam * jm1 * J;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            out[3 * r + c] = U[3 * r] * dg[0] * U[3 * c] + U[3 * r + 1] * dg[1] * U[3 * c + 1] +
                             U[3 * r + 2] * dg[2] * U[3 * c + 2] + (r == c ? iso : T(0));
}

// updateDeformationGradient (material_point_method.cpp:306-330) for one
// particle: F_E* = (I + dt B D^-1) F_E = U S V^T, F_E <- U clamp(S) V^T, and
// det F_P *= prod S / prod clamp(S) (the reference's F_P <- F_E^-1 Fhat with
// Fhat = F_E* F_P); with the full F_P, F_P <- V (S / clamp(S)) V^T F_P.
template <typename T, bool TRACK_FP>
__device__ __forceinline__ void update_F(const DevParams<T>& P, const T Bm[9], T F[9], T& Jp, T FP[9]) {
    T A[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) A[e] = Bm[e] * P.dinv * P.dt;
    A[0] += T(1); A[4] += T(1); A[8] += T(1);
    T Fs[9];
    matmul3(Fs, A, F);
    T U[9], s[3], V[9];
    svd3(Fs, U, s, V);
    T sc[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) sc[c] = s[c] < P.lo ? P.lo : (s[c] > P.hi ? P.hi : s[c]);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = 0; c < 3; ++c)
            F[3 * r + c] = U[3 * r] * sc[0] * V[3 * c] + U[3 * r + 1] * sc[1] * V[3 * c + 1] +
                           U[3 * r + 2] * sc[2] * V[3 * c + 2];
    Jp = Jp * ((s[0] * s[1] * s[2]) / (sc[0] * sc[1] * sc[2]));
    if (TRACK_FP) {
        T r[3], Mv[9], out[9];
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] = s[c] / sc[c];
#pragma unroll
        for (int a = 0; a < 3; ++a)
#pragma unroll
            for (int b = 0; b < 3; ++b)
                Mv[3 * a + b] = V[3 * a] * r[0] * V[3 * b] + V[3 * a + 1] * r[1] * V[3 * b + 1] +
                                V[3 * a + 2] * r[2] * V[3 * b + 2];
        matmul3(out, Mv, FP);
#pragma unroll
        for (int e = 0; e < 9; ++e) FP[e] = out[e];
    }
}

template <typename T>
__device__ __forceinline__ T clampx(T x, T lo, T hi) { return x < lo ? lo : (hi < x ? hi : x); }

template <typename T>
__device__ __forceinline__ bool wall_node(const DevParams<T>& P, int i, int j, int k) {
    const int w = P.bc_width;
    return i < w || j < w || k < w || i >= P.M[0] - w || j >= P.M[1] - w || k >= P.M[2] - w;
}

template <typename T>
__device__ __forceinline__ void tile_origin(const DevParams<T>& P, int key, int org[3]) {
    const int bz = key % P.NB[2];
    const int by = (key / P.NB[2]) % P.NB[1];
    const int bx = key / (P.NB[1] * P.NB[2]);
    org[0] = bx * kBlk - 1; org[1] = by * kBlk - 1; org[2] = bz * kBlk - 1;
}

template <typename T>
__device__ __forceinline__ bool cell_of_tile(const DevParams<T>& P, const int org[3], int c, size_t& lin) {
    const int ix = c / (kTile * kTile), iy = (c / kTile) % kTile, iz = c % kTile;
    const int gx = org[0] + ix, gy = org[1] + iy, gz = org[2] + iz;
    lin = ((size_t)gx * P.M[1] + gy) * P.M[2] + gz;
    return gx >= 0 && gy >= 0 && gz >= 0 && gx < P.M[0] && gy < P.M[1] && gz < P.M[2];
}

// ---------------------------------------------------------------- P2G
// rasterizeParticlesToGrid + computeExplicitGridForces
// (material_point_method.cpp:94-129,235-254) for one work item per loop trip.
// Particle p adds w_ip m_p to the mass and w_ip (m v + A (x_i - x_p)) to the
// momentum of the 64 nodes i of its stencil, with
// A = m B D^-1 - fscale V D^-1 P F^T:
//   MOM && FORCE : fused step, q = m v + dt f       (fscale = dt)
//   MOM only     : rasterize stage, q = m v
//   FORCE only   : force stage, q = f                (fscale = 1, into gforce)
//
// Cell-owned accumulation.  Phase 1 (a thread per particle) turns each
// particle into a shared-memory record: its 12 separable weights,
// q' = m v + A e with e = (base - 1) h - x, h A, and m, so that node
// base - 1 + o receives w_o (m, q' + h A o).  The records are counting-sorted
// by base cell.  Phase 2 runs one task per (cell, x offset): a thread sums the
// contributions of every particle of that cell to the 16 nodes of that x
// layer in registers and adds them to the shared tile once, so the shared
// atomics per cell are 64 rather than 256 per particle.  The tile then goes to
// the grid with one 16-byte vector reduction per touched node.
template <typename T> struct WorkP;
template <> struct WorkP<float> { static constexpr int value = 512; };
template <> struct WorkP<double> { static constexpr int value = 128; };

constexpr int kRecV4 = 7;
constexpr int kCells = kBlk * kBlk * kBlk;

template <typename T> struct P2GShared {
    T tile[4 * kTileCells];
    vec4<T> rec[WorkP<T>::value * kRecV4];
    int cnt[kCells];
    int off[kCells];
    uint16_t order[WorkP<T>::value];
    uint8_t cellof[WorkP<T>::value];
};

template <typename T> __device__ __forceinline__ T pick4(const vec4<T>& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// Phase 2 for one (cell, x offset) task; adds 16 nodes x (m, q) to the tile.
template <typename T, bool MOM>
__device__ __forceinline__ void p2g_cell_task(P2GShared<T>& S, int c, int ox) {
    const int n_c = S.cnt[c];
    if (n_c == 0) return;
    const int cz = c % kBlk, cy = (c / kBlk) % kBlk, cx = c / (kBlk * kBlk);
    T am[4][4], aq[4][4][3];
#pragma unroll
    for (int a = 0; a < 4; ++a)
#pragma unroll
        for (int b = 0; b < 4; ++b) {
            am[a][b] = T(0);
            aq[a][b][0] = aq[a][b][1] = aq[a][b][2] = T(0);
        }
    const T fox = (T)ox;
    const int k0 = S.off[c];
    for (int k = k0; k < k0 + n_c; ++k) {
        const vec4<T>* r = &S.rec[(int)S.order[k] * kRecV4];
        const vec4<T> wx4 = r[0], wy4 = r[1], wz4 = r[2], qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
        const T wx = pick4<T>(wx4, ox);
        const T wy[4] = {wy4.x, wy4.y, wy4.z, wy4.w};
        const T wz[4] = {wz4.x, wz4.y, wz4.z, wz4.w};
        // h A columns: x (a4.x, a4.y, a4.z), y (a4.w, b4.x, b4.y), z (b4.z, b4.w, c4.x)
        T t1[3] = {qm.x + a4.x * fox, qm.y + a4.y * fox, qm.z + a4.z * fox};
        const T ay[3] = {a4.w, b4.x, b4.y};
        const T az[3] = {b4.z, b4.w, c4.x};
#pragma unroll
        for (int oy = 0; oy < 4; ++oy) {
            const T wxy = wx * wy[oy];
            T t3[3] = {t1[0], t1[1], t1[2]};
#pragma unroll
            for (int oz = 0; oz < 4; ++oz) {
                const T w = wxy * wz[oz];
                if (MOM) am[oy][oz] += w * qm.w;
#pragma unroll
                for (int q = 0; q < 3; ++q) {
                    aq[oy][oz][q] += w * t3[q];
                    t3[q] += az[q];
                }
            }
#pragma unroll
            for (int q = 0; q < 3; ++q) t1[q] += ay[q];
        }
    }
#pragma unroll
    for (int oy = 0; oy < 4; ++oy)
#pragma unroll
        for (int oz = 0; oz < 4; ++oz) {
            const int cell = ((cx + ox) * kTile + (cy + oy)) * kTile + (cz + oz);
            if (MOM) atomicAdd(&S.tile[cell], am[oy][oz]);
            atomicAdd(&S.tile[kTileCells + cell], aq[oy][oz][0]);
            atomicAdd(&S.tile[2 * kTileCells + cell], aq[oy][oz][1]);
            atomicAdd(&S.tile[3 * kTileCells + cell], aq[oy][oz][2]);
        }
}

template <typename T, bool MOM, bool FORCE>
__global__ void __launch_bounds__(kThreads) k_p2g(DevParams<T> P, DevBufs D) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    P2GShared<T>& S = *reinterpret_cast<P2GShared<T>*>(smem_raw);
    const vec4<T>* __restrict__ pl = static_cast<const vec4<T>*>(D.pin);
    vec4<T>* __restrict__ grid = static_cast<vec4<T>*>(MOM ? D.grid : D.gforce);
    const uint32_t nw = *D.nwork;
    const size_t n = (size_t)P.n;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = D.work[wi];
        for (int c = threadIdx.x; c < 4 * kTileCells; c += blockDim.x) S.tile[c] = T(0);
        for (int c = threadIdx.x; c < kCells; c += blockDim.x) S.cnt[c] = 0;
        int org[3];
        tile_origin(P, it.x, org);
        const int count = min(it.z, min(WorkP<T>::value, P.n - it.y));
        __syncthreads();
        // phase 1: a record per particle
        for (int j = threadIdx.x; j < count; j += blockDim.x) {
            Particle<T> p;
            load_particle(pl, n, D.perm[it.y + j], p);
            Stencil<T> St;
            if (!make_stencil(P, p.x, org, St)) {
                raise_flag(D.flags, 4u);
                S.cellof[j] = 0xff;
                continue;
            }
            if (!stencil_in_grid(P, St.b)) raise_flag(D.flags, 1u);
            T A[9];
            T mv[3] = {T(0), T(0), T(0)};
#pragma unroll
            for (int e = 0; e < 9; ++e) A[e] = T(0);
            if (MOM) {
#pragma unroll
                for (int e = 0; e < 9; ++e) A[e] = p.m * (p.B[e] * P.dinv);
#pragma unroll
                for (int a = 0; a < 3; ++a) mv[a] = p.m * p.v[a];
            }
            if (FORCE) {
                T G[9];
                stress_PFt(P, p.F, p.Jp, G);
                const T sc = P.fscale * (p.vol * P.dinv);
#pragma unroll
                for (int e = 0; e < 9; ++e) A[e] -= sc * G[e];
            }
            T e3[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) e3[a] = (T)(St.b[a] - 1) * P.h - p.x[a];
            T qp[3];
#pragma unroll
            for (int r = 0; r < 3; ++r) qp[r] = mv[r] + (A[3 * r] * e3[0] + A[3 * r + 1] * e3[1] + A[3 * r + 2] * e3[2]);
            vec4<T>* r = &S.rec[j * kRecV4];
            r[0] = mk4<T>(St.w[0][0], St.w[0][1], St.w[0][2], St.w[0][3]);
            r[1] = mk4<T>(St.w[1][0], St.w[1][1], St.w[1][2], St.w[1][3]);
            r[2] = mk4<T>(St.w[2][0], St.w[2][1], St.w[2][2], St.w[2][3]);
            r[3] = mk4<T>(qp[0], qp[1], qp[2], MOM ? p.m : T(0));
            r[4] = mk4<T>(P.h * A[0], P.h * A[3], P.h * A[6], P.h * A[1]);
            r[5] = mk4<T>(P.h * A[4], P.h * A[7], P.h * A[2], P.h * A[5]);
            r[6] = mk4<T>(P.h * A[8], T(0), T(0), T(0));
            const int cell = (St.rel[0] * kBlk + St.rel[1]) * kBlk + St.rel[2];
            S.cellof[j] = (uint8_t)cell;
            atomicAdd(&S.cnt[cell], 1);
        }
        __syncthreads();
        if (threadIdx.x < 32) {  // exclusive scan of the 64 cell counts
            const int l = threadIdx.x;
            const int a = S.cnt[2 * l], b = S.cnt[2 * l + 1];
            int x = a + b;
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const int y = __shfl_up_sync(0xffffffffu, x, o);
                if (l >= o) x += y;
            }
            S.off[2 * l] = x - a - b;
            S.off[2 * l + 1] = x - b;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < kCells; c += blockDim.x) S.cnt[c] = S.off[c];  // cursor
        __syncthreads();
        for (int j = threadIdx.x; j < count; j += blockDim.x) {
            const int c = S.cellof[j];
            if (c != 0xff) S.order[atomicAdd(&S.cnt[c], 1)] = (uint16_t)j;
        }
        __syncthreads();
        for (int c = threadIdx.x; c < kCells; c += blockDim.x) S.cnt[c] -= S.off[c];  // counts again
        __syncthreads();
        // phase 2: (cell, x offset) tasks
        for (int task = threadIdx.x; task < kCells * 4; task += blockDim.x)
            p2g_cell_task<T, MOM>(S, task % kCells, task / kCells);
        __syncthreads();
        for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
            size_t lin;
            if (!cell_of_tile(P, org, c, lin)) continue;
            const vec4<T> v = mk4<T>(S.tile[c], S.tile[kTileCells + c], S.tile[2 * kTileCells + c],
                                     S.tile[3 * kTileCells + c]);
            if (v.x != T(0) || v.y != T(0) || v.z != T(0) || v.w != T(0)) red_add4(grid + lin, v);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- fused G2P
// gridVelocitiesUpdate + updateDeformationGradient + updateParticleVelocities +
// updateParticlePositions (material_point_method.cpp:256-262,306-350) for one
// work item per loop trip.  The grid tile arrives as (m, p = m v + dt f) and is
// turned into v = p / m + dt g (zero where m = 0 and on sticky walls) while it
// is staged in shared memory.  The particle is written at its sorted position
// into the other plane buffer, and its next block key is counted.
template <typename T, bool TRACK_FP>
__global__ void __launch_bounds__(kThreads) k_g2p_fused(DevParams<T> P, DevBufs D) {
    __shared__ T sv[3 * kTileCells];
    const vec4<T>* __restrict__ pin = static_cast<const vec4<T>*>(D.pin);
    vec4<T>* __restrict__ pout = static_cast<vec4<T>*>(D.pout);
    const vec4<T>* __restrict__ grid = static_cast<const vec4<T>*>(D.grid);
    const uint32_t nw = *D.nwork;
    const size_t n = (size_t)P.n;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = D.work[wi];
        int org[3];
        tile_origin(P, it.x, org);
        for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
            size_t lin;
            T v0 = T(0), v1 = T(0), v2 = T(0);
            if (cell_of_tile(P, org, c, lin)) {
                const vec4<T> g4 = grid[lin];
                if (g4.x != T(0)) {
                    v0 = g4.y / g4.x + P.dt * P.g[0];
                    v1 = g4.z / g4.x + P.dt * P.g[1];
                    v2 = g4.w / g4.x + P.dt * P.g[2];
                    if (P.bc == 1) {
                        const int ix = c / (kTile * kTile), iy = (c / kTile) % kTile, iz = c % kTile;
                        if (wall_node(P, org[0] + ix, org[1] + iy, org[2] + iz)) v0 = v1 = v2 = T(0);
                    }
                }
            }
            sv[c] = v0; sv[kTileCells + c] = v1; sv[2 * kTileCells + c] = v2;
        }
        __syncthreads();
        const int send = min(it.y + it.z, P.n);
        for (int s = it.y + threadIdx.x; s < send; s += blockDim.x) {
            Particle<T> p;
            const uint32_t src = D.perm[s];
            load_particle(pin, n, src, p);
            T FP[9];
            if (TRACK_FP) load_fp(pin, n, src, FP);
            Stencil<T> S;
            const bool ok = make_stencil(P, p.x, org, S);
            if (!ok) raise_flag(D.flags, 4u);
            if (P.lagged) update_F<T, TRACK_FP>(P, p.B, p.F, p.Jp, FP);
            T vp[3] = {T(0), T(0), T(0)};
            T Bp[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) Bp[e] = T(0);
            if (ok) {
#pragma unroll
                for (int ox = 0; ox < 4; ++ox)
#pragma unroll
                    for (int oy = 0; oy < 4; ++oy) {
                        const T wxy = S.w[0][ox] * S.w[1][oy];
                        const int rowc = ((S.rel[0] + ox) * kTile + (S.rel[1] + oy)) * kTile + S.rel[2];
#pragma unroll
                        for (int oz = 0; oz < 4; ++oz) {
                            const T w = wxy * S.w[2][oz];
                            const int cell = rowc + oz;
                            const T vi[3] = {sv[cell], sv[kTileCells + cell], sv[2 * kTileCells + cell]};
                            const T dd[3] = {S.d[0][ox], S.d[1][oy], S.d[2][oz]};
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
                                vp[r] += vi[r] * w;
#pragma unroll
                                for (int c = 0; c < 3; ++c) Bp[3 * r + c] += w * (vi[r] * dd[c]);
                            }
                        }
                    }
            }
            if (!P.lagged) update_F<T, TRACK_FP>(P, Bp, p.F, p.Jp, FP);
#pragma unroll
            for (int a = 0; a < 3; ++a) p.v[a] = vp[a];
#pragma unroll
            for (int e = 0; e < 9; ++e) p.B[e] = Bp[e];
#pragma unroll
            for (int a = 0; a < 3; ++a) p.x[a] = clampx(p.x[a] + p.v[a] * P.dt, P.xlo, P.xhi[a]);
            store_particle(pout, n, s, p);
            if (TRACK_FP) store_fp(pout, n, s, FP);
            const int b[3] = {base_of(p.x[0], P.h), base_of(p.x[1], P.h), base_of(p.x[2], P.h)};
            const uint32_t key = block_key(P, b);
            D.keys_out[s] = key;
            count_key(D.counts, key);
            bool finite = isfinite(p.x[0]) && isfinite(p.x[1]) && isfinite(p.x[2]) && isfinite(p.v[0]) &&
                          isfinite(p.v[1]) && isfinite(p.v[2]) && isfinite(p.Jp);
#pragma unroll
            for (int e = 0; e < 9; ++e) finite = finite && isfinite(p.F[e]) && isfinite(p.B[e]);
            if (!finite) raise_flag(D.flags, 2u);
        }
        __syncthreads();
    }
}

// ---------------------------------------------------------------- stage kernels
// rasterize stage: v_i = (m v)_i / m_i on cells with m != 0 (material_point_method.cpp:118-121).
template <typename T>
__global__ void k_grid_normalize(vec4<T>* __restrict__ grid, size_t ncells) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= ncells) return;
    vec4<T> g = grid[c];
    if (g.x != T(0)) { g.y /= g.x; g.z /= g.x; g.w /= g.x; grid[c] = g; }
}

// gridVelocitiesUpdate (material_point_method.cpp:256-262) + optional walls.
template <typename T>
__global__ void k_grid_velocities(DevParams<T> P, vec4<T>* __restrict__ grid, const vec4<T>* __restrict__ force) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nc = (size_t)P.M[0] * P.M[1] * P.M[2];
    if (c >= nc) return;
    vec4<T> g = grid[c];
    if (g.x == T(0)) return;
    const vec4<T> f = force[c];
    g.y += P.dt * (f.y / g.x + P.g[0]);
    g.z += P.dt * (f.z / g.x + P.g[1]);
    g.w += P.dt * (f.w / g.x + P.g[2]);
    if (P.bc == 1) {
        const int k = (int)(c % P.M[2]), j = (int)((c / P.M[2]) % P.M[1]), i = (int)(c / ((size_t)P.M[1] * P.M[2]));
        if (wall_node(P, i, j, k)) g.y = g.z = g.w = T(0);
    }
    grid[c] = g;
}

// updateDeformationGradient as its own stage, in place.
template <typename T, bool TRACK_FP>
__global__ void __launch_bounds__(kThreads) k_update_F(DevParams<T> P, vec4<T>* __restrict__ pl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const size_t n = (size_t)P.n;
    Particle<T> p;
    load_particle(pl, n, i, p);
    T FP[9];
    if (TRACK_FP) load_fp(pl, n, i, FP);
    update_F<T, TRACK_FP>(P, p.B, p.F, p.Jp, FP);
    store_particle(pl, n, i, p);
    if (TRACK_FP) store_fp(pl, n, i, FP);
}

// updateParticleVelocities as its own stage (grid holds (m, v)), in place.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_g2p_stage(DevParams<T> P, DevBufs D) {
    __shared__ T sv[3 * kTileCells];
    vec4<T>* __restrict__ pl = static_cast<vec4<T>*>(D.pout);
    const vec4<T>* __restrict__ grid = static_cast<const vec4<T>*>(D.grid);
    const uint32_t nw = *D.nwork;
    const size_t n = (size_t)P.n;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = D.work[wi];
        int org[3];
        tile_origin(P, it.x, org);
        for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
            size_t lin;
            T v0 = T(0), v1 = T(0), v2 = T(0);
            if (cell_of_tile(P, org, c, lin)) {
                const vec4<T> g4 = grid[lin];
                v0 = g4.y; v1 = g4.z; v2 = g4.w;
            }
            sv[c] = v0; sv[kTileCells + c] = v1; sv[2 * kTileCells + c] = v2;
        }
        __syncthreads();
        const int send = min(it.y + it.z, P.n);
        for (int s = it.y + threadIdx.x; s < send; s += blockDim.x) {
            const uint32_t idx = D.perm[s];
            Particle<T> p;
            load_particle(pl, n, idx, p);
            Stencil<T> S;
            T vp[3] = {T(0), T(0), T(0)};
            T Bp[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) Bp[e] = T(0);
            if (make_stencil(P, p.x, org, S)) {
#pragma unroll
                for (int ox = 0; ox < 4; ++ox)
#pragma unroll
                    for (int oy = 0; oy < 4; ++oy) {
                        const T wxy = S.w[0][ox] * S.w[1][oy];
                        const int rowc = ((S.rel[0] + ox) * kTile + (S.rel[1] + oy)) * kTile + S.rel[2];
#pragma unroll
                        for (int oz = 0; oz < 4; ++oz) {
                            const T w = wxy * S.w[2][oz];
                            const int cell = rowc + oz;
                            const T vi[3] = {sv[cell], sv[kTileCells + cell], sv[2 * kTileCells + cell]};
                            const T dd[3] = {S.d[0][ox], S.d[1][oy], S.d[2][oz]};
#pragma unroll
                            for (int r = 0; r < 3; ++r) {
                                vp[r] += vi[r] * w;
#pragma unroll
                                for (int c = 0; c < 3; ++c) Bp[3 * r + c] += w * (vi[r] * dd[c]);
                            }
                        }
                    }
            } else {
                raise_flag(D.flags, 4u);
            }
#pragma unroll
            for (int a = 0; a < 3; ++a) p.v[a] = vp[a];
#pragma unroll
            for (int e = 0; e < 9; ++e) p.B[e] = Bp[e];
            store_particle(pl, n, idx, p);
        }
        __syncthreads();
    }
}

// updateParticlePositions (material_point_method.cpp:344-350,381-388), in place.
template <typename T>
__global__ void k_advect(DevParams<T> P, vec4<T>* __restrict__ pl) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    vec4<T> x = pl[i];
    const vec4<T> v = pl[(size_t)P.n + i];
    x.x = clampx(x.x + v.x * P.dt, P.xlo, P.xhi[0]);
    x.y = clampx(x.y + v.y * P.dt, P.xlo, P.xhi[1]);
    x.z = clampx(x.z + v.z * P.dt, P.xlo, P.xhi[2]);
    pl[i] = x;
}

// computeParticleVolumesAndDensities (material_point_method.cpp:131-142):
// rho_p = sum m_i w_ip / h^3, V_p = m_p / rho_p (0 where rho_p = 0).
template <typename T>
__global__ void k_volumes(DevParams<T> P, vec4<T>* __restrict__ pl, const vec4<T>* __restrict__ grid,
                          uint32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const vec4<T> x4 = pl[i];
    const T x[3] = {x4.x, x4.y, x4.z};
    int b[3];
    T w[3][4];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t = div_rn(x[a], P.h);
        b[a] = (int)t;
        bspline4(t, b[a], w[a]);
    }
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    T density = T(0);
    for (int ox = 0; ox < 4; ++ox)
        for (int oy = 0; oy < 4; ++oy)
            for (int oz = 0; oz < 4; ++oz) {
                const int gx = b[0] - 1 + ox, gy = b[1] - 1 + oy, gz = b[2] - 1 + oz;
                if (gx < 0 || gy < 0 || gz < 0 || gx >= P.M[0] || gy >= P.M[1] || gz >= P.M[2]) continue;
                const T m = grid[((size_t)gx * P.M[1] + gy) * P.M[2] + gz].x;
                density += m * ((w[0][ox] * w[1][oy]) * w[2][oz]);
            }
    density /= (P.h * P.h * P.h);
    vec4<T> v = pl[(size_t)P.n + i];
    v.w = density != T(0) ? x4.w / density : T(0);
    pl[(size_t)P.n + i] = v;
}

// Grid export: mass and velocity per cell as the reference holds them; in
// fused mode (m, p) -> v = p / m + dt g (+ walls) as k_g2p_fused stages it.
template <typename T, bool FUSED>
__global__ void k_grid_export(DevParams<T> P, const vec4<T>* __restrict__ grid, T* __restrict__ mass,
                              T* __restrict__ vel) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nc = (size_t)P.M[0] * P.M[1] * P.M[2];
    if (c >= nc) return;
    const vec4<T> g = grid[c];
    T v0 = g.y, v1 = g.z, v2 = g.w;
    if (FUSED) {
        v0 = v1 = v2 = T(0);
        if (g.x != T(0)) {
            v0 = g.y / g.x + P.dt * P.g[0];
            v1 = g.z / g.x + P.dt * P.g[1];
            v2 = g.w / g.x + P.dt * P.g[2];
            const int k = (int)(c % P.M[2]), j = (int)((c / P.M[2]) % P.M[1]),
                      i = (int)(c / ((size_t)P.M[1] * P.M[2]));
            if (P.bc == 1 && wall_node(P, i, j, k)) v0 = v1 = v2 = T(0);
        }
    }
    if (mass) mass[c] = g.x;
    if (vel) { vel[3 * c] = v0; vel[3 * c + 1] = v1; vel[3 * c + 2] = v2; }
}

// Viewer stream (main.cpp:259-271): float4 (x, y, z, size) in original order.
template <typename T>
__global__ void k_xyzs(int n, const vec4<T>* __restrict__ pl, float4* __restrict__ out, float size) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const vec4<T> x = pl[i];
    const uint32_t id = real_to_id<T>(pl[6 * (size_t)n + i].w);
    if (id < (uint32_t)n) out[id] = make_float4((float)x.x, (float)x.y, (float)x.z, size);
}

}  // namespace rd
