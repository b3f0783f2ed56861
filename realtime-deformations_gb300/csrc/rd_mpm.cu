// Host side of the C ABI declared in include/rd_mpm.h: the handle, its device
// buffers (allocated once in rd_create), parameter preparation and the launch
// sequences for the fused step and for the reference's individual stages.
#include <cuda_runtime.h>

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include "rd_kernels.cuh"
#include "../../include/rd_mpm.h"

using namespace rd;

namespace {

enum GridMode { GRID_NONE = 0, GRID_FUSED = 1, GRID_MV = 2, GRID_V = 3 };

template <typename T>
__global__ void k_pack(int n, const T* __restrict__ x, const T* __restrict__ v, const T* __restrict__ B,
                       const T* __restrict__ FE, const T* __restrict__ FP, const T* __restrict__ Jp,
                       const T* __restrict__ mass, const T* __restrict__ vol, vec4<T>* __restrict__ pl,
                       int track_fp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Particle<T> p;
    T P[9];
#pragma unroll
    for (int a = 0; a < 3; ++a) { p.x[a] = x[3 * i + a]; p.v[a] = v[3 * i + a]; }
    p.m = mass[i];
    p.vol = vol ? vol[i] : T(0);
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        p.B[e] = B ? B[9 * i + e] : T(0);
        p.F[e] = FE ? FE[9 * i + e] : ((e % 4 == 0) ? T(1) : T(0));
        P[e] = FP ? FP[9 * i + e] : ((e % 4 == 0) ? T(1) : T(0));
    }
    p.Jp = Jp ? Jp[i] : (FP ? det3(P) : T(1));
    p.id = (uint32_t)i;
    store_particle(pl, (size_t)n, (size_t)i, p);
    if (track_fp) store_fp(pl, (size_t)n, (size_t)i, P);
}

template <typename T>
__global__ void k_unpack(int n, const vec4<T>* __restrict__ pl, T* __restrict__ x, T* __restrict__ v,
                         T* __restrict__ B, T* __restrict__ FE, T* __restrict__ FP, T* __restrict__ Jp,
                         T* __restrict__ mass, T* __restrict__ vol, int track_fp) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    Particle<T> p;
    load_particle(pl, (size_t)n, (size_t)i, p);
    const uint32_t o = p.id;
    if (o >= (uint32_t)n) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        if (x) x[3 * o + a] = p.x[a];
        if (v) v[3 * o + a] = p.v[a];
    }
#pragma unroll
    for (int e = 0; e < 9; ++e) {
        if (B) B[9 * o + e] = p.B[e];
        if (FE) FE[9 * o + e] = p.F[e];
    }
    if (FP) {
        T P[9];
        if (track_fp) {
            load_fp(pl, (size_t)n, (size_t)i, P);
        } else {  // only det F_P is carried: report the isotropic F_P with that det
            const T c = cbrt(p.Jp);
#pragma unroll
            for (int e = 0; e < 9; ++e) P[e] = (e % 4 == 0) ? c : T(0);
        }
#pragma unroll
        for (int e = 0; e < 9; ++e) FP[9 * o + e] = P[e];
    }
    if (Jp) Jp[o] = p.Jp;
    if (mass) mass[o] = p.m;
    if (vol) vol[o] = p.vol;
}

template <typename T>
__global__ void k_debug_sort(int n, const vec4<T>* __restrict__ pl, const uint32_t* __restrict__ keys,
                             const uint32_t* __restrict__ perm, uint32_t* __restrict__ keys_orig,
                             uint32_t* __restrict__ order) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t id = real_to_id<T>(pl[6 * (size_t)n + i].w);
    if (id < (uint32_t)n) keys_orig[id] = keys[i];
    order[i] = real_to_id<T>(pl[6 * (size_t)n + perm[i]].w);
}

inline size_t align_up(size_t v, size_t a) { return (v + a - 1) / a * a; }

}  // namespace

struct rd_handle {
    rd_params prm{};
    cudaStream_t stream = nullptr;
    int sms = 0;
    int n = 0;
    size_t ncells = 0;
    int NB[3] = {0, 0, 0};
    int nblocks = 0;  // 4x4x4-cell blocks
    int nkeys = 0;    // sort keys: blocks x 64 cells
    int planes = kPlanes;
    size_t esize = 4;
    void* pl[2] = {nullptr, nullptr};
    int cur = 0;
    uint32_t* keys[2] = {nullptr, nullptr};
    uint32_t* perm = nullptr;
    uint32_t* counts = nullptr;
    uint32_t* cursor = nullptr;
    int4* work = nullptr;
    uint32_t* nwork2 = nullptr;  // two item counters: the current sort's and the next's
    int nb = 0;                  // nwork2[nb] belongs to the last sort
    uint32_t* tile_sums = nullptr;
    size_t work_cap = 0;
    void* grid[2] = {nullptr, nullptr};  // (m, p) of this step / the next (fused); (m, v) in stage mode
    int g = 0;                           // current grid buffer
    bool fgrid_valid = false;            // grid[g] holds P2G(x) for rd_step with fgrid_dt
    double fgrid_dt = 0.0;
    void* gforce = nullptr;
    uint32_t* flags = nullptr;
    float4* xyzs = nullptr;
    void* io = nullptr;  // device SoA staging for set/get (36 reals per particle)
    void* grid_io = nullptr;  // device staging for rd_get_grid to host (7 reals per cell)
    bool keys_valid = false;
    bool sorted = false;
    int grid_mode = GRID_NONE;
    double last_dt = 0.0;
    uint64_t launches = 0;
    int occ_p2g = 1, occ_g2p = 1;
    std::string err;
    // per-kernel event timing (rd_set_kernel_timing)
    bool timing = false;
    std::vector<cudaEvent_t> ev;      // pool, pairs (start, stop)
    std::vector<int> ev_kernel;       // kernel id per pair
    size_t ev_used = 0;               // pairs recorded since the last harvest
    uint64_t t_launches[RD_KERNEL_COUNT] = {};
    double t_ms[RD_KERNEL_COUNT] = {};
};

namespace {

rd_status fail(rd_handle* h, rd_status s, const std::string& msg) {
    if (h) h->err = msg;
    return s;
}

rd_status check_cuda(rd_handle* h, cudaError_t e, const char* what) {
    if (e == cudaSuccess) return RD_OK;
    return fail(h, e == cudaErrorMemoryAllocation ? RD_OOM : RD_CUDA_ERROR,
                std::string(what) + ": " + cudaGetErrorString(e));
}

#define RD_TRY(expr)                          \
    do {                                      \
        rd_status _s = (expr);                \
        if (_s != RD_OK) return _s;           \
    } while (0)

// DpInverse[0][0] as the reference evaluates it: glm::inverse of the diagonal
// matrix mat3(1) * (1/3f) * h * h (material_point_method.hpp:177; cofactor
// times 1/det in glm's order).  volatile keeps every product rounded to the
// declared type.
template <typename T> T reference_dinv(T h) {
    volatile T d = T(1) * (T)(1.0f / 3.0f);
    if (sizeof(T) == 8) d = T(1.0 / 3.0);
    d = d * h;
    d = d * h;
    volatile T dd = d * d;
    volatile T det = d * dd;
    volatile T od = T(1) / det;
    volatile T r = dd * od;
    return r;
}

template <typename T> DevParams<T> make_params(const rd_handle* h, double dt, T fscale) {
    const rd_params& p = h->prm;
    DevParams<T> P{};
    P.M[0] = p.max_i; P.M[1] = p.max_j; P.M[2] = p.max_k;
    P.NB[0] = h->NB[0]; P.NB[1] = h->NB[1]; P.NB[2] = h->NB[2];
    P.nkeys = h->nkeys;
    P.n = h->n;
    const T hh = (T)p.h;
    P.h = hh;
    P.dinv = reference_dinv<T>(hh);
    P.dt = (T)dt;
    // material_point_method.cpp:237-242, in the element type
    volatile T E = (T)p.E, nu = (T)p.nu;
    volatile T one_nu = T(1) + nu;
    volatile T mu0 = E / (T(2) * one_nu);
    volatile T en = E * nu;
    volatile T two_nu = T(2) * nu;
    volatile T den = one_nu * (T(1) - two_nu);
    volatile T lam0 = en / den;
    P.mu0 = mu0;
    P.lambda0 = lam0;
    P.xi = (T)p.xi;
    // material_point_method.cpp:320: (float)(1 - theta) evaluated in double
    P.lo = (T)(1.0 - p.theta_c);
    P.hi = (T)(1.0 + p.theta_s);
    for (int a = 0; a < 3; ++a) P.g[a] = (T)p.gravity[a];
    volatile T xl = T(3) * hh;
    P.xlo = xl;
    volatile T x0 = (T)(p.max_i - 3) * hh, x1 = (T)(p.max_j - 3) * hh, x2 = (T)(p.max_k - 3) * hh;
    P.xhi[0] = x0; P.xhi[1] = x1; P.xhi[2] = x2;
    P.fscale = fscale;
    P.bc = p.bc;
    P.bc_width = p.bc_width;
    P.lagged = p.lagged_b;
    return P;
}

template <typename T> DevBufs bufs(rd_handle* h) {
    DevBufs D{};
    D.pin = h->pl[h->cur];
    D.pout = h->pl[h->cur ^ 1];
    D.perm = h->perm;
    D.keys_out = h->keys[h->cur ^ 1];
    D.counts = h->counts;
    D.work = h->work;
    D.nwork = h->nwork2 + h->nb;
    D.work_cap = (uint32_t)h->work_cap;
    D.grid = h->grid[h->g];
    D.grid_next = h->grid[h->g ^ 1];
    D.gforce = h->gforce;
    D.flags = h->flags;
    return D;
}

inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)std::max<size_t>(1, (n + t - 1) / t); }

rd_status launched(rd_handle* h, const char* what, int count = 1) {
    h->launches += (uint64_t)count;
    return check_cuda(h, cudaGetLastError(), what);
}

constexpr size_t kEventPairs = 4096;

// Adds the elapsed time of every recorded pair to the per-kernel totals.
rd_status harvest_timing(rd_handle* h) {
    if (h->ev_used == 0) return RD_OK;
    RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    for (size_t i = 0; i < h->ev_used; ++i) {
        float ms = 0.f;
        RD_TRY(check_cuda(h, cudaEventElapsedTime(&ms, h->ev[2 * i], h->ev[2 * i + 1]), "event time"));
        h->t_ms[h->ev_kernel[i]] += ms;
        h->t_launches[h->ev_kernel[i]] += 1;
    }
    h->ev_used = 0;
    return RD_OK;
}

// Records the start event of a timed launch; returns the pair index or -1.
long tmark_begin(rd_handle* h, int kernel) {
    if (!h->timing) return -1;
    if (h->ev_used == kEventPairs && harvest_timing(h) != RD_OK) return -1;
    const size_t i = h->ev_used++;
    h->ev_kernel[i] = kernel;
    cudaEventRecord(h->ev[2 * i], h->stream);
    return (long)i;
}
void tmark_end(rd_handle* h, long i) {
    if (i >= 0) cudaEventRecord(h->ev[2 * i + 1], h->stream);
}

// Sort by block key: histogram (unless the last fused G2P already counted),
// scan + work items, scatter into perm.
template <typename T> rd_status sort_particles(rd_handle* h) {
    if (h->n == 0) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->nwork2, 0, 2 * sizeof(uint32_t), h->stream), "memset nwork"));
        h->sorted = true;
        return RD_OK;
    }
    DevParams<T> P = make_params<T>(h, 0.0, T(0));
    if (!h->keys_valid) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->counts, 0, sizeof(uint32_t) * h->nkeys, h->stream), "memset counts"));
        long t = tmark_begin(h, RD_KERNEL_KEYS);
        k_keys<T><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->pl[h->cur]),
                                                                  h->keys[h->cur], h->counts, h->flags);
        tmark_end(h, t);
        RD_TRY(launched(h, "k_keys"));
    }
    const int ntiles = (h->nkeys + kScanTile - 1) / kScanTile;
    // this sort fills nwork2[nb ^ 1] (cleared by the previous sort or at
    // creation) and clears nwork2[nb] for the next one
    uint32_t* nw = h->nwork2 + (h->nb ^ 1);
    uint32_t* nw_next = h->nwork2 + h->nb;
    long t = tmark_begin(h, RD_KERNEL_SCAN);
    k_tile_sums<<<ntiles, 256, 0, h->stream>>>(h->counts, h->nkeys, h->tile_sums);
    k_scan<<<ntiles, kScanThreads, 0, h->stream>>>(h->counts, h->cursor, h->tile_sums, h->nkeys, h->work, nw, nw_next,
                                                (uint32_t)h->n, (uint32_t)h->work_cap, (uint32_t)WorkP<T>::value,
                                                h->flags);
    tmark_end(h, t);
    RD_TRY(launched(h, "k_scan", 2));
    h->nb ^= 1;
    t = tmark_begin(h, RD_KERNEL_SCATTER);
    k_scatter<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->n, h->keys[h->cur], h->cursor, h->perm);
    tmark_end(h, t);
    RD_TRY(launched(h, "k_scatter"));
    h->keys_valid = false;  // counts consumed
    h->sorted = true;
    return RD_OK;
}

template <typename T> unsigned persistent_grid(const rd_handle* h, int occ) {
    const size_t max_items = (size_t)h->n / WorkP<T>::value + (size_t)std::min<int64_t>(h->nblocks, h->n) + 1;
    return (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)h->sms * occ));
}

template <typename T> rd_status step_fused(rd_handle* h, double dt) {
    const size_t gbytes = h->ncells * sizeof(vec4<T>);
    if (h->n == 0) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->grid[h->g ^ 1], 0, gbytes, h->stream), "memset grid"));
        h->g ^= 1;
        h->grid_mode = GRID_FUSED;
        h->last_dt = dt;
        return RD_OK;
    }
    if (!h->sorted) RD_TRY(sort_particles<T>(h));
    DevParams<T> P = make_params<T>(h, dt, (T)dt);
    long t;
    if (!(h->fgrid_valid && h->fgrid_dt == dt)) {  // P2G of the current state
        t = tmark_begin(h, RD_KERNEL_GRID_CLEAR);
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->grid[h->g], 0, gbytes, h->stream), "memset grid"));
        tmark_end(h, t);
        DevBufs D = bufs<T>(h);
        t = tmark_begin(h, RD_KERNEL_P2G);
        k_p2g<T, true, true><<<persistent_grid<T>(h, h->occ_p2g), kThreads, sizeof(P2GTile<T, kBlk>), h->stream>>>(P, D);
        tmark_end(h, t);
        RD_TRY(launched(h, "k_p2g"));
    }
    t = tmark_begin(h, RD_KERNEL_GRID_CLEAR);
    RD_TRY(check_cuda(h, cudaMemsetAsync(h->grid[h->g ^ 1], 0, gbytes, h->stream), "memset grid"));
    tmark_end(h, t);
    DevBufs D = bufs<T>(h);
    t = tmark_begin(h, RD_KERNEL_G2P2G);
    if (h->prm.track_fp)
        k_g2p2g<T, true><<<persistent_grid<T>(h, h->occ_g2p), kFusedThreads, sizeof(FusedShared<T>), h->stream>>>(P, D);
    else
        k_g2p2g<T, false><<<persistent_grid<T>(h, h->occ_g2p), kFusedThreads, sizeof(FusedShared<T>), h->stream>>>(P, D);
    tmark_end(h, t);
    RD_TRY(launched(h, "k_g2p2g"));
    h->cur ^= 1;
    h->g ^= 1;
    h->keys_valid = true;  // k_g2p2g wrote keys[cur] and counted them
    h->sorted = false;
    h->fgrid_valid = true;
    h->fgrid_dt = dt;
    h->grid_mode = GRID_FUSED;
    h->last_dt = dt;
    return RD_OK;
}

template <typename T> rd_status stage_impl(rd_handle* h, int stage, double dt) {
    const size_t nc = h->ncells;
    const unsigned cb = blocks_for(nc, 256);
    DevParams<T> P = make_params<T>(h, dt, T(1));
    h->fgrid_valid = false;
    switch (stage) {
        case RD_STAGE_RASTERIZE: {
            if (!h->sorted) RD_TRY(sort_particles<T>(h));
            RD_TRY(check_cuda(h, cudaMemsetAsync(h->grid[h->g], 0, nc * sizeof(vec4<T>), h->stream), "memset grid"));
            RD_TRY(check_cuda(h, cudaMemsetAsync(h->gforce, 0, nc * sizeof(vec4<T>), h->stream), "memset force"));
            if (h->n > 0) {
                DevBufs D = bufs<T>(h);
                k_p2g<T, true, false><<<persistent_grid<T>(h, h->occ_p2g), kThreads, sizeof(P2GTile<T, kBlk>), h->stream>>>(P, D);
                RD_TRY(launched(h, "k_p2g<rasterize>"));
            }
            k_grid_normalize<T><<<cb, 256, 0, h->stream>>>(static_cast<vec4<T>*>(h->grid[h->g]), nc);
            RD_TRY(launched(h, "k_grid_normalize"));
            h->grid_mode = GRID_V;
            return RD_OK;
        }
        case RD_STAGE_FORCES: {
            if (h->grid_mode != GRID_V) return fail(h, RD_INVALID_ARG, "forces stage needs a rasterized grid");
            if (!h->sorted) RD_TRY(sort_particles<T>(h));
            if (h->n > 0) {
                DevBufs D = bufs<T>(h);
                k_p2g<T, false, true><<<persistent_grid<T>(h, h->occ_p2g), kThreads, sizeof(P2GTile<T, kBlk>), h->stream>>>(P, D);
                RD_TRY(launched(h, "k_p2g<forces>"));
            }
            return RD_OK;
        }
        case RD_STAGE_GRID_VELOCITIES:
            if (h->grid_mode != GRID_V) return fail(h, RD_INVALID_ARG, "grid velocity stage needs a rasterized grid");
            k_grid_velocities<T><<<cb, 256, 0, h->stream>>>(P, static_cast<vec4<T>*>(h->grid[h->g]),
                                                             static_cast<const vec4<T>*>(h->gforce));
            return launched(h, "k_grid_velocities");
        case RD_STAGE_COLLISIONS:
            return RD_OK;  // empty collider list: bodyCollision is the identity
        case RD_STAGE_DEFORMATION:
            if (h->n == 0) return RD_OK;
            if (h->prm.track_fp)
                k_update_F<T, true><<<blocks_for(h->n, kThreads), kThreads, 0, h->stream>>>(
                    P, static_cast<vec4<T>*>(h->pl[h->cur]));
            else
                k_update_F<T, false><<<blocks_for(h->n, kThreads), kThreads, 0, h->stream>>>(
                    P, static_cast<vec4<T>*>(h->pl[h->cur]));
            return launched(h, "k_update_F");
        case RD_STAGE_PARTICLE_VELOCITIES: {
            if (h->grid_mode != GRID_V) return fail(h, RD_INVALID_ARG, "particle velocity stage needs a grid");
            if (!h->sorted) RD_TRY(sort_particles<T>(h));
            if (h->n == 0) return RD_OK;
            DevBufs D = bufs<T>(h);
            D.pout = h->pl[h->cur];
            k_g2p_stage<T><<<persistent_grid<T>(h, h->occ_g2p), kThreads, 0, h->stream>>>(P, D);
            return launched(h, "k_g2p_stage");
        }
        case RD_STAGE_POSITIONS:
            if (h->n == 0) return RD_OK;
            k_advect<T><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, static_cast<vec4<T>*>(h->pl[h->cur]));
            h->sorted = false;
            h->keys_valid = false;
            return launched(h, "k_advect");
        case RD_STAGE_VOLUMES:
            if (h->grid_mode != GRID_V && h->grid_mode != GRID_MV)
                return fail(h, RD_INVALID_ARG, "volume stage needs a rasterized grid");
            if (h->n == 0) return RD_OK;
            k_volumes<T><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, static_cast<vec4<T>*>(h->pl[h->cur]),
                                                                        static_cast<const vec4<T>*>(h->grid[h->g]),
                                                                        h->flags);
            return launched(h, "k_volumes");
        default:
            return fail(h, RD_INVALID_ARG, "unknown stage id");
    }
}

template <typename T> rd_status set_particles_impl(rd_handle* h, const rd_particles* in, int where) {
    const size_t n = (size_t)h->n;
    if (!in->x || !in->v || !in->mass) return fail(h, RD_INVALID_ARG, "x, v and mass are required");
    T* io = static_cast<T*>(h->io);
    // io layout: x 3n | v 3n | B 9n | FE 9n | FP 9n | Jp n | mass n | vol n
    T* d[8] = {io, io + 3 * n, io + 6 * n, io + 15 * n, io + 24 * n, io + 33 * n, io + 34 * n, io + 35 * n};
    const void* src[8] = {in->x, in->v, in->B, in->FE, in->FP, in->Jp, in->mass, in->volume};
    const size_t cnt[8] = {3 * n, 3 * n, 9 * n, 9 * n, 9 * n, n, n, n};
    const T* ptr[8];
    for (int k = 0; k < 8; ++k) {
        if (!src[k] || n == 0) { ptr[k] = nullptr; continue; }
        if (where == RD_HOST) {
            RD_TRY(check_cuda(h, cudaMemcpyAsync(d[k], src[k], cnt[k] * sizeof(T), cudaMemcpyHostToDevice, h->stream),
                              "upload"));
            ptr[k] = d[k];
        } else {
            ptr[k] = static_cast<const T*>(src[k]);
        }
    }
    if (n > 0) {
        k_pack<T><<<blocks_for(n, 256), 256, 0, h->stream>>>((int)n, ptr[0], ptr[1], ptr[2], ptr[3], ptr[4], ptr[5],
                                                             ptr[6], ptr[7], static_cast<vec4<T>*>(h->pl[h->cur]),
                                                             h->prm.track_fp);
        RD_TRY(launched(h, "k_pack"));
    }
    h->keys_valid = false;
    h->sorted = false;
    h->fgrid_valid = false;
    h->grid_mode = GRID_NONE;
    return RD_OK;
}

template <typename T> rd_status get_particles_impl(rd_handle* h, rd_particles* out, int where) {
    const size_t n = (size_t)h->n;
    if (n == 0) return RD_OK;
    T* io = static_cast<T*>(h->io);
    T* d[8] = {io, io + 3 * n, io + 6 * n, io + 15 * n, io + 24 * n, io + 33 * n, io + 34 * n, io + 35 * n};
    void* dst[8] = {out->x, out->v, out->B, out->FE, out->FP, out->Jp, out->mass, out->volume};
    const size_t cnt[8] = {3 * n, 3 * n, 9 * n, 9 * n, 9 * n, n, n, n};
    T* tgt[8];
    for (int k = 0; k < 8; ++k) tgt[k] = dst[k] ? (where == RD_HOST ? d[k] : static_cast<T*>(dst[k])) : nullptr;
    k_unpack<T><<<blocks_for(n, 256), 256, 0, h->stream>>>((int)n, static_cast<const vec4<T>*>(h->pl[h->cur]), tgt[0],
                                                           tgt[1], tgt[2], tgt[3], tgt[4], tgt[5], tgt[6], tgt[7],
                                                           h->prm.track_fp);
    RD_TRY(launched(h, "k_unpack"));
    if (where == RD_HOST) {
        for (int k = 0; k < 8; ++k)
            if (dst[k])
                RD_TRY(check_cuda(h, cudaMemcpyAsync(dst[k], d[k], cnt[k] * sizeof(T), cudaMemcpyDeviceToHost, h->stream),
                                  "download"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    }
    return RD_OK;
}

template <typename T> rd_status get_grid_impl(rd_handle* h, void* mass, void* vel, void* force, int where) {
    const size_t nc = h->ncells;
    if (h->grid_mode == GRID_NONE) return fail(h, RD_INVALID_ARG, "no grid computed yet");
    const bool host = where == RD_HOST;
    if (host && !h->grid_io) {  // allocated on first use only: a debugging / parity path
        RD_TRY(check_cuda(h, cudaMalloc(&h->grid_io, 7 * nc * sizeof(T)), "grid export buffer"));
    }
    T* scratch = static_cast<T*>(h->grid_io);
    T* m_d = host ? scratch : static_cast<T*>(mass);
    T* v_d = host ? scratch + nc : static_cast<T*>(vel);
    DevParams<T> P = make_params<T>(h, h->last_dt, T(1));
    const unsigned cb = blocks_for(nc, 256);
    if (h->grid_mode == GRID_FUSED)  // the grid the last step's G2P read
        k_grid_export<T, true><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g ^ 1]),
                                                          mass ? m_d : nullptr, vel ? v_d : nullptr);
    else
        k_grid_export<T, false><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g]),
                                                           mass ? m_d : nullptr, vel ? v_d : nullptr);
    RD_TRY(launched(h, "k_grid_export"));
    T* f_d = nullptr;
    if (force) {
        f_d = host ? scratch + 4 * nc : static_cast<T*>(force);
        if (h->grid_mode == GRID_FUSED) {
            RD_TRY(check_cuda(h, cudaMemsetAsync(f_d, 0, 3 * nc * sizeof(T), h->stream), "force"));
        } else {
            k_grid_export<T, false><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->gforce), nullptr, f_d);
            RD_TRY(launched(h, "k_grid_export<force>"));
        }
    }
    if (host) {
        if (mass) RD_TRY(check_cuda(h, cudaMemcpyAsync(mass, m_d, nc * sizeof(T), cudaMemcpyDeviceToHost, h->stream), "d2h"));
        if (vel) RD_TRY(check_cuda(h, cudaMemcpyAsync(vel, v_d, 3 * nc * sizeof(T), cudaMemcpyDeviceToHost, h->stream), "d2h"));
        if (force) RD_TRY(check_cuda(h, cudaMemcpyAsync(force, f_d, 3 * nc * sizeof(T), cudaMemcpyDeviceToHost, h->stream), "d2h"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    }
    return RD_OK;
}

template <typename T> rd_status xyzs_impl(rd_handle* h, float** out) {
    if (h->n > 0) {
        k_xyzs<T><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->n, static_cast<const vec4<T>*>(h->pl[h->cur]),
                                                                h->xyzs, 0.02f);
        RD_TRY(launched(h, "k_xyzs"));
    }
    *out = reinterpret_cast<float*>(h->xyzs);
    return RD_OK;
}

template <typename T> rd_status debug_sort_impl(rd_handle* h, uint32_t* keys, uint32_t* order, int where) {
    if (h->n == 0) return RD_OK;
    // keys[cur] must describe the current positions: recount them, then sort.
    h->keys_valid = false;
    RD_TRY(sort_particles<T>(h));
    uint32_t* kd = static_cast<uint32_t*>(h->io);
    uint32_t* od = kd + h->n;
    if (where == RD_DEVICE) { kd = keys; od = order; }
    k_debug_sort<T><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->n, static_cast<const vec4<T>*>(h->pl[h->cur]),
                                                                  h->keys[h->cur], h->perm, kd, od);
    RD_TRY(launched(h, "k_debug_sort"));
    if (where == RD_HOST) {
        RD_TRY(check_cuda(h, cudaMemcpyAsync(keys, kd, 4 * (size_t)h->n, cudaMemcpyDeviceToHost, h->stream), "d2h"));
        RD_TRY(check_cuda(h, cudaMemcpyAsync(order, od, 4 * (size_t)h->n, cudaMemcpyDeviceToHost, h->stream), "d2h"));
    }
    return check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
}

template <typename T> rd_status init_volumes_impl(rd_handle* h) {
    RD_TRY(stage_impl<T>(h, RD_STAGE_RASTERIZE, 0.0));
    return stage_impl<T>(h, RD_STAGE_VOLUMES, 0.0);
}

template <typename T> rd_status occupancy(rd_handle* h) {
    int o = 0;
    const int sm = (int)sizeof(P2GTile<T, kBlk>);
    RD_TRY(check_cuda(h, cudaFuncSetAttribute(k_p2g<T, true, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm), "smem attr"));
    RD_TRY(check_cuda(h, cudaFuncSetAttribute(k_p2g<T, true, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm), "smem attr"));
    RD_TRY(check_cuda(h, cudaFuncSetAttribute(k_p2g<T, false, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, sm), "smem attr"));
    RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_p2g<T, true, true>, kThreads, sm), "occ"));
    h->occ_p2g = std::max(1, o);
    const int fsm = (int)sizeof(FusedShared<T>);
    RD_TRY(check_cuda(h, cudaFuncSetAttribute(k_g2p2g<T, true>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm), "smem attr"));
    RD_TRY(check_cuda(h, cudaFuncSetAttribute(k_g2p2g<T, false>, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm), "smem attr"));
    if (h->prm.track_fp)
        RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_g2p2g<T, true>, kFusedThreads, fsm), "occ"));
    else
        RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_g2p2g<T, false>, kFusedThreads, fsm), "occ"));
    h->occ_g2p = std::max(1, o);
    return RD_OK;
}

void release(rd_handle* h) {
    for (cudaEvent_t e : h->ev)
        if (e) cudaEventDestroy(e);
    h->ev.clear();
    void* ptrs[] = {h->pl[0], h->pl[1], h->keys[0], h->keys[1], h->perm, h->counts, h->cursor, h->work,
                    h->nwork2, h->tile_sums, h->grid[0], h->grid[1], h->gforce, h->flags, h->xyzs, h->io, h->grid_io};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->stream) cudaStreamDestroy(h->stream);
}

}  // namespace

extern "C" {

void rd_default_params(rd_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->max_i = p->max_j = p->max_k = 20;       // main.cpp:205
    p->num_particles = 270 + 1877;              // main.cpp:203
    p->h = 0.05;                                // material_point_method.cpp:17
    p->E = 1.4e5f;                              // material_point_method.cpp:238
    p->nu = 0.2f;                               // :237
    p->xi = 10.0f;                              // material_point_method.hpp:213
    p->theta_c = 2.5f * 1e-2;                   // material_point_method.cpp:320
    p->theta_s = 5.0f * 1e-3;
    p->gravity[0] = 0.0; p->gravity[1] = -9.8; p->gravity[2] = 0.0;  // :260
    p->bc = RD_BC_NONE;
    p->bc_width = 3;
    p->lagged_b = 1;
    p->track_fp = 0;
    p->precision = RD_FP32;
    p->device = 0;
}

rd_status rd_create(const rd_params* params, rd_handle** out) {
    if (!params || !out) return RD_INVALID_ARG;
    *out = nullptr;
    const rd_params& p = *params;
    if (p.max_i < 8 || p.max_j < 8 || p.max_k < 8 || p.num_particles < 0 || !(p.h > 0) ||
        (p.precision != RD_FP32 && p.precision != RD_FP64) || p.bc_width < 0 ||
        (int64_t)p.max_i * p.max_j * p.max_k > (int64_t)1 << 30)
        return RD_INVALID_ARG;
    rd_handle* h = new (std::nothrow) rd_handle;
    if (!h) return RD_OOM;
    h->prm = p;
    h->n = p.num_particles;
    h->esize = p.precision == RD_FP64 ? 8 : 4;
    h->planes = p.track_fp ? kPlanesFP : kPlanes;
    h->ncells = (size_t)p.max_i * p.max_j * p.max_k;
    h->NB[0] = (p.max_i + kBlk - 1) / kBlk;
    h->NB[1] = (p.max_j + kBlk - 1) / kBlk;
    h->NB[2] = (p.max_k + kBlk - 1) / kBlk;
    h->nblocks = h->NB[0] * h->NB[1] * h->NB[2];
    h->nkeys = h->nblocks * kCellsPerBlock;
    auto bail = [&](rd_status s) { release(h); delete h; return s; };
    if (cudaSetDevice(p.device) != cudaSuccess) return bail(RD_CUDA_ERROR);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p.device) != cudaSuccess) return bail(RD_CUDA_ERROR);
    h->sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RD_CUDA_ERROR);
    const size_t n = std::max<size_t>(1, (size_t)h->n);
    const size_t v4 = 4 * h->esize;
    const size_t wp = p.precision == RD_FP64 ? WorkP<double>::value : WorkP<float>::value;
    h->work_cap = n / wp + std::min<size_t>((size_t)h->nblocks, n) + 2;
    struct { void** ptr; size_t bytes; } allocs[] = {
        {&h->pl[0], (size_t)h->planes * n * v4},
        {&h->pl[1], (size_t)h->planes * n * v4},
        {(void**)&h->keys[0], n * 4},
        {(void**)&h->keys[1], n * 4},
        {(void**)&h->perm, n * 4},
        {(void**)&h->counts, (size_t)h->nkeys * 4},
        {(void**)&h->cursor, (size_t)h->nkeys * 4},
        {(void**)&h->work, h->work_cap * sizeof(int4)},
        {(void**)&h->nwork2, 8},
        {(void**)&h->tile_sums, (size_t)((h->nkeys + kScanTile - 1) / kScanTile) * 4},
        {&h->grid[0], h->ncells * v4},
        {&h->grid[1], h->ncells * v4},
        {&h->gforce, h->ncells * v4},
        {(void**)&h->flags, 4},
        {(void**)&h->xyzs, n * sizeof(float4)},
        {&h->io, align_up(36 * n * h->esize, 256)},
    };
    for (auto& a : allocs) {
        cudaError_t e = cudaMalloc(a.ptr, a.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return bail(e == cudaErrorMemoryAllocation ? RD_OOM : RD_CUDA_ERROR);
        }
    }
    cudaMemsetAsync(h->counts, 0, (size_t)h->nkeys * 4, h->stream);
    cudaMemsetAsync(h->perm, 0, n * 4, h->stream);  // every entry is a valid index from the start
    cudaMemsetAsync(h->flags, 0, 4, h->stream);
    cudaMemsetAsync(h->nwork2, 0, 8, h->stream);
    rd_status s = p.precision == RD_FP64 ? occupancy<double>(h) : occupancy<float>(h);
    if (s != RD_OK) return bail(s);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(RD_CUDA_ERROR);
    *out = h;
    return RD_OK;
}

rd_status rd_destroy(rd_handle* h) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    release(h);
    delete h;
    return RD_OK;
}

#define RD_DISPATCH(h, fn, ...) ((h)->prm.precision == RD_FP64 ? fn<double>(__VA_ARGS__) : fn<float>(__VA_ARGS__))

rd_status rd_set_particles(rd_handle* h, const rd_particles* in, int where) {
    if (!h || !in || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, set_particles_impl, h, in, where);
}

rd_status rd_get_particles(rd_handle* h, rd_particles* out, int where) {
    if (!h || !out || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_particles_impl, h, out, where);
}

rd_status rd_init_volumes(rd_handle* h) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, init_volumes_impl, h);
}

rd_status rd_step(rd_handle* h, double dt, int32_t nsteps) {
    if (!h || nsteps < 0 || !std::isfinite(dt)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    for (int s = 0; s < nsteps; ++s) {
        rd_status st = RD_DISPATCH(h, step_fused, h, dt);
        if (st != RD_OK) return st;
    }
    return RD_OK;
}

rd_status rd_stage(rd_handle* h, int32_t stage, double dt) {
    if (!h || !std::isfinite(dt)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, stage_impl, h, stage, dt);
}

rd_status rd_get_grid(rd_handle* h, void* mass, void* velocity, void* force, int where) {
    if (!h || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_grid_impl, h, mass, velocity, force, where);
}

rd_status rd_device_xyzs(rd_handle* h, float** xyzs) {
    if (!h || !xyzs) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, xyzs_impl, h, xyzs);
}

rd_status rd_get_flags(rd_handle* h, uint32_t* flags) {
    if (!h || !flags) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    RD_TRY(check_cuda(h, cudaMemcpyAsync(flags, h->flags, 4, cudaMemcpyDeviceToHost, h->stream), "flags"));
    return check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
}

rd_status rd_clear_flags(rd_handle* h) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return check_cuda(h, cudaMemsetAsync(h->flags, 0, 4, h->stream), "clear flags");
}

rd_status rd_synchronize(rd_handle* h) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
}

rd_status rd_get_stream(rd_handle* h, void** stream) {
    if (!h || !stream) return RD_INVALID_ARG;
    *stream = (void*)h->stream;
    return RD_OK;
}

rd_status rd_last_error(rd_handle* h, char* buf, size_t len) {
    if (!h || !buf || len == 0) return RD_INVALID_ARG;
    std::snprintf(buf, len, "%s", h->err.c_str());
    return RD_OK;
}

rd_status rd_debug_sort(rd_handle* h, uint32_t* keys, uint32_t* order, int where) {
    if (!h || !keys || !order || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, debug_sort_impl, h, keys, order, where);
}

rd_status rd_set_kernel_timing(rd_handle* h, int enable) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    if (enable && h->ev.empty()) {  // created once, on first enable
        h->ev.assign(2 * kEventPairs, nullptr);
        h->ev_kernel.assign(kEventPairs, 0);
        for (auto& e : h->ev) RD_TRY(check_cuda(h, cudaEventCreate(&e), "event create"));
    }
    if (!enable) RD_TRY(harvest_timing(h));
    h->timing = enable != 0;
    h->ev_used = 0;
    for (int k = 0; k < RD_KERNEL_COUNT; ++k) { h->t_launches[k] = 0; h->t_ms[k] = 0.0; }
    return RD_OK;
}

rd_status rd_kernel_timing(rd_handle* h, int kernel, uint64_t* launches, double* total_ms) {
    if (!h || kernel < 0 || kernel >= RD_KERNEL_COUNT || !launches || !total_ms) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    RD_TRY(harvest_timing(h));
    *launches = h->t_launches[kernel];
    *total_ms = h->t_ms[kernel];
    return RD_OK;
}

rd_status rd_launch_count(rd_handle* h, uint64_t* count) {
    if (!h || !count) return RD_INVALID_ARG;
    *count = h->launches;
    return RD_OK;
}

}  // extern "C"

// ---------------------------------------------------------------------------
// Allocation-free rasterize (rd_rasterize_noalloc).  The sort scratch lives in
// one file-scope device array sized for the limits below; every GPU that loads
// this library holds it until the process exits.
namespace {

constexpr int kNaMaxParticles = 1 << 16;  // 65,536 particles
constexpr int kNaMaxKeys = 1 << 18;       // 262,144 cell keys (4x4x4 blocks x 64), e.g. a 64^3 grid
constexpr int kNaMaxTiles = kNaMaxKeys / kScanTile;
constexpr int kNaMaxWork = kNaMaxParticles / WorkP<float>::value + kNaMaxKeys / kCellsPerBlock + 2;

struct NaScratch {
    int4 work[kNaMaxWork];
    uint32_t keys[kNaMaxParticles];
    uint32_t perm[kNaMaxParticles];
    uint32_t counts[kNaMaxKeys];
    uint32_t cursor[kNaMaxKeys];
    uint32_t tile_sums[kNaMaxTiles];
    uint32_t nwork[2];
    uint32_t flags;
};

// Block key and histogram of particles given as device arrays (x: n x 3).
__global__ void __launch_bounds__(256) k_na_keys(DevParams<float> P, const float* __restrict__ x,
                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                                                 uint32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int b[3] = {base_of(x[3 * i], P.h), base_of(x[3 * i + 1], P.h), base_of(x[3 * i + 2], P.h)};
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    const uint32_t key = sort_key(P, b);
    keys[i] = key;
    count_key(counts, key);
}

// The rasterize P2G of k_p2g<float, true, false>, reading x, v, B and mass from
// the caller's structure-of-arrays device buffers instead of particle planes.
__global__ void __launch_bounds__(kThreads) k_na_p2g(DevParams<float> P, const float* __restrict__ x,
                                                     const float* __restrict__ v, const float* __restrict__ B,
                                                     const float* __restrict__ mass, const uint32_t* __restrict__ perm,
                                                     const int4* __restrict__ work, const uint32_t* nwork,
                                                     uint32_t work_cap, float4* __restrict__ grid, uint32_t* flags) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    P2GTile<float, kBlk>& S = *reinterpret_cast<P2GTile<float, kBlk>*>(smem_raw);
    const uint32_t nw = min(*nwork, work_cap);
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = work[wi];
        for (int c = threadIdx.x; c < 4 * P2GTile<float, kBlk>::TC; c += blockDim.x) S.tile[c] = 0.f;
        for (int c = threadIdx.x; c < P2GTile<float, kBlk>::NC; c += blockDim.x) S.cnt[c] = 0;
        int org[3];
        tile_origin(P, it.x, org);
        const int count = min(it.z, min(WorkP<float>::value, P.n - it.y));
        __syncthreads();
        for (int j = threadIdx.x; j < count; j += blockDim.x) {
            const uint32_t i = perm[it.y + j];
            const float px[3] = {x[3 * i], x[3 * i + 1], x[3 * i + 2]};
            Stencil<float> St;
            if (!make_stencil(P, px, org, St)) {
                raise_flag(flags, 4u);
                S.cellof[j] = 0xff;
                continue;
            }
            const float m = mass[i];
            float A[9], mv[3];
#pragma unroll
            for (int e = 0; e < 9; ++e) A[e] = B ? m * (B[9 * i + e] * P.dinv) : 0.f;
#pragma unroll
            for (int a = 0; a < 3; ++a) mv[a] = m * v[3 * i + a];
            write_record<float, true>(&S.rec[j * kRecV4], St, px, A, mv, m, P.h);
            const int cell = (St.rel[0] * kBlk + St.rel[1]) * kBlk + St.rel[2];
            S.cellof[j] = (uint8_t)cell;
            atomicAdd(&S.cnt[cell], 1);
        }
        sort_records<float, kBlk>(S, count);
        p2g_tasks<float, true, kBlk>(S, count);
        __syncthreads();
        p2g_flush<float, kBlk>(P, S, org, grid);
        __syncthreads();
    }
}

struct NaDevice {
    NaScratch* scratch = nullptr;
    int sms = 0;
    int occ = 1;
};
std::mutex g_na_mutex;
NaDevice g_na[64];

}  // namespace

static __device__ __align__(256) unsigned char rd_noalloc_scratch[sizeof(NaScratch)];

extern "C" rd_status rd_rasterize_noalloc(const rd_params* params, const rd_particles* in, float* grid_out,
                                          void* stream) {
    if (!params || !in || !in->x || !in->v || !in->mass || !grid_out) return RD_INVALID_ARG;
    const rd_params& p = *params;
    if (p.precision != RD_FP32) return RD_NOT_SUPPORTED;
    if (p.max_i < 8 || p.max_j < 8 || p.max_k < 8 || p.num_particles < 0 || !(p.h > 0)) return RD_INVALID_ARG;
    const int64_t cells = (int64_t)p.max_i * p.max_j * p.max_k;
    const int64_t nblocks = (int64_t)((p.max_i + kBlk - 1) / kBlk) * ((p.max_j + kBlk - 1) / kBlk) *
                            ((p.max_k + kBlk - 1) / kBlk);
    if (p.num_particles > kNaMaxParticles || cells > kNaMaxKeys || nblocks * kCellsPerBlock > kNaMaxKeys)
        return RD_TOO_LARGE;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RD_CUDA_ERROR;
    NaDevice nd;
    {
        // once per device, with that device current: the scratch array's device
        // address (the host-side name is only a stand-in) and the launch shape
        std::lock_guard<std::mutex> lock(g_na_mutex);
        if (!g_na[dev].scratch) {
            void* ptr = nullptr;
            if (cudaGetSymbolAddress(&ptr, rd_noalloc_scratch) != cudaSuccess || !ptr) return RD_CUDA_ERROR;
            int sms = 0, occ = 0;
            if (cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess) return RD_CUDA_ERROR;
            if (cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, k_na_p2g, kThreads, sizeof(P2GTile<float, kBlk>)) !=
                cudaSuccess)
                return RD_CUDA_ERROR;
            g_na[dev].sms = sms;
            g_na[dev].occ = std::max(1, occ);
            g_na[dev].scratch = static_cast<NaScratch*>(ptr);
        }
        nd = g_na[dev];
    }
    NaScratch* sc = nd.scratch;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    rd_handle hp;  // parameters only; owns no device memory
    hp.prm = p;
    hp.n = p.num_particles;
    hp.NB[0] = (p.max_i + kBlk - 1) / kBlk;
    hp.NB[1] = (p.max_j + kBlk - 1) / kBlk;
    hp.NB[2] = (p.max_k + kBlk - 1) / kBlk;
    hp.nblocks = (int)nblocks;
    hp.nkeys = (int)nblocks * kCellsPerBlock;
    DevParams<float> P = make_params<float>(&hp, 0.0, 0.0f);
    const int n = p.num_particles;
    // the scratch keeps the previous call's contents: clear what must start at zero
    if (cudaMemsetAsync(grid_out, 0, (size_t)cells * sizeof(float4), st) != cudaSuccess ||
        cudaMemsetAsync(sc->counts, 0, (size_t)hp.nkeys * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(sc->nwork, 0, 2 * sizeof(uint32_t) + sizeof(uint32_t), st) != cudaSuccess)
        return RD_CUDA_ERROR;
    if (n > 0) {
        const int ntiles = (hp.nkeys + kScanTile - 1) / kScanTile;
        const uint32_t work_cap = (uint32_t)kNaMaxWork;
        k_na_keys<<<blocks_for(n, 256), 256, 0, st>>>(P, static_cast<const float*>(in->x), sc->keys, sc->counts,
                                                      &sc->flags);
        k_tile_sums<<<ntiles, 256, 0, st>>>(sc->counts, hp.nkeys, sc->tile_sums);
        k_scan<<<ntiles, kScanThreads, 0, st>>>(sc->counts, sc->cursor, sc->tile_sums, hp.nkeys, sc->work, &sc->nwork[0],
                                                &sc->nwork[1], (uint32_t)n, work_cap, (uint32_t)WorkP<float>::value,
                                                &sc->flags);
        k_scatter<<<blocks_for(n, 256), 256, 0, st>>>(n, sc->keys, sc->cursor, sc->perm);
        const size_t max_items = (size_t)n / WorkP<float>::value + (size_t)std::min<int64_t>(nblocks, n) + 1;
        const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)nd.sms * nd.occ));
        k_na_p2g<<<grid, kThreads, sizeof(P2GTile<float, kBlk>), st>>>(
            P, static_cast<const float*>(in->x), static_cast<const float*>(in->v), static_cast<const float*>(in->B),
            static_cast<const float*>(in->mass), sc->perm, sc->work, &sc->nwork[0], work_cap,
            reinterpret_cast<float4*>(grid_out), &sc->flags);
    }
    return cudaGetLastError() == cudaSuccess ? RD_OK : RD_CUDA_ERROR;
}
