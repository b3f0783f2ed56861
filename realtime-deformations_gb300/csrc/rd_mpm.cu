// Host side of the C ABI declared in include/rd_mpm.h: the handle, its device
// buffers (allocated once in rd_create), parameter preparation and the launch
// sequences for the fused step and for the reference's individual stages.
#include <cuda.h>  // CUtensorMap and its enums (the encoder is fetched from the driver at run time)
#include <cuda_runtime.h>
#include <cudaTypedefs.h>

#include <algorithm>
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstring>
#include <mutex>
#include <new>
#include <string>
#include <vector>

#include <nvtx3/nvToolsExt.h>

#include "rd_adjoint.cuh"
#include "rd_implicit.cuh"
#include "rd_kernels.cuh"
#include "rd_init.cuh"
#include "rd_view.cuh"
#include "../../include/rd_mpm.h"

using namespace rd;

namespace {

// A named range in profiler timelines (no cost without a profiler attached).
struct NvtxRange {
    explicit NvtxRange(const char* name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

enum GridMode { GRID_NONE = 0, GRID_FUSED = 1, GRID_MV = 2, GRID_V = 3 };

// Rows of K reals per particle (x, v: K = 3; B, F_E, F_P: K = 9) of the
// caller's structure-of-arrays buffers move through shared memory, so that
// consecutive threads touch consecutive words of the K-strided row array.
// Called by every thread of a 256-thread block; rows r0 .. r0 + cnt - 1 are
// the block's, thread t's row is r0 + t.
constexpr int kIoThreads = 256;
// `count` reals from src to dst by the whole block, as 16-byte vectors when
// both addresses allow it (fewer, larger requests over the host link).
template <typename T>
__device__ __forceinline__ void block_copy(T* __restrict__ dst, const T* __restrict__ src, int count) {
    constexpr int V = 16 / (int)sizeof(T);
    int e0 = 0;
    if (((reinterpret_cast<uintptr_t>(src) | reinterpret_cast<uintptr_t>(dst)) & 15u) == 0) {
        const int nv = count / V;
        const float4* __restrict__ s4 = reinterpret_cast<const float4*>(src);
        float4* __restrict__ d4 = reinterpret_cast<float4*>(dst);
        for (int e = threadIdx.x; e < nv; e += blockDim.x) d4[e] = s4[e];
        e0 = nv * V;
    }
    for (int e = e0 + threadIdx.x; e < count; e += blockDim.x) dst[e] = src[e];
}
template <typename T, int K>
__device__ __forceinline__ void load_rows(const T* __restrict__ src, int r0, int cnt, T (&val)[K], T* sh) {
    __syncthreads();  // the previous use of sh is done
    block_copy(sh, src + (size_t)r0 * K, cnt * K);
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) val[k] = sh[threadIdx.x * K + k];  // rows past cnt: not used
}
template <typename T, int K>
__device__ __forceinline__ void store_rows(T* __restrict__ dst, int r0, int cnt, const T (&val)[K], T* sh) {
    __syncthreads();
#pragma unroll
    for (int k = 0; k < K; ++k) sh[threadIdx.x * K + k] = val[k];
    __syncthreads();
    block_copy(dst + (size_t)r0 * K, sh, cnt * K);
}

// The particle of row r0 + threadIdx.x of the caller's structure-of-arrays
// input (r0: the block's first row); absent fields take their defaults
// (B = 0, F_E = F_P = I, J_P = det F_P or 1, V = 0).  Called by every thread
// of a kIoThreads block; false for a row past n.  p.id is not set.
template <typename T>
__device__ __forceinline__ bool pack_row(int n, int r0, const T* __restrict__ x, const T* __restrict__ v,
                                         const T* __restrict__ B, const T* __restrict__ FE, const T* __restrict__ FP,
                                         const T* __restrict__ Jp, const T* __restrict__ mass,
                                         const T* __restrict__ vol, Particle<T>& p, T (&FPm)[9], T* sh) {
    const int i = r0 + threadIdx.x;
    const int cnt = min((int)blockDim.x, n - r0);
    T t3[3];
    load_rows(x, r0, cnt, t3, sh);
#pragma unroll
    for (int a = 0; a < 3; ++a) p.x[a] = t3[a];
    load_rows(v, r0, cnt, t3, sh);
#pragma unroll
    for (int a = 0; a < 3; ++a) p.v[a] = t3[a];
    if (B) {
        load_rows(B, r0, cnt, p.B, sh);
    } else {
#pragma unroll
        for (int e = 0; e < 9; ++e) p.B[e] = T(0);
    }
    if (FE) {
        load_rows(FE, r0, cnt, p.F, sh);
    } else {
#pragma unroll
        for (int e = 0; e < 9; ++e) p.F[e] = (e % 4 == 0) ? T(1) : T(0);
    }
    if (FP) {
        load_rows(FP, r0, cnt, FPm, sh);
    } else {
#pragma unroll
        for (int e = 0; e < 9; ++e) FPm[e] = (e % 4 == 0) ? T(1) : T(0);
    }
    if (i >= n) return false;
    p.m = mass[i];
    p.vol = vol ? vol[i] : T(0);
    p.Jp = Jp ? Jp[i] : (FP ? det3(FPm) : T(1));
    return true;
}

// Particles off .. off + n - 1 of planes holding ntot particles (one scene of
// a batch, or all of a single scene), from structure-of-arrays input in
// particle id order; particle i goes to slot off + i.  With keys (a single
// scene, P its parameters) it also writes the first sort's keys and
// histogram, as k_keys would: the loads from host memory bound this kernel,
// so the keys cost nothing here.
template <typename T>
__global__ void __launch_bounds__(kIoThreads)
    k_pack(int n, int off, int ntot, const T* __restrict__ x, const T* __restrict__ v, const T* __restrict__ B,
           const T* __restrict__ FE, const T* __restrict__ FP, const T* __restrict__ Jp, const T* __restrict__ mass,
           const T* __restrict__ vol, vec4<T>* __restrict__ pl, int track_fp, DevParams<T> P,
           uint32_t* __restrict__ keys, uint32_t* __restrict__ counts, uint32_t* __restrict__ bcount,
           uint32_t* __restrict__ flags) {
    __shared__ __align__(16) T sh[9 * kIoThreads];
    const int r0 = blockIdx.x * blockDim.x, i = r0 + threadIdx.x;
    Particle<T> p;
    T FPm[9];
    if (!pack_row(n, r0, x, v, B, FE, FP, Jp, mass, vol, p, FPm, sh)) return;
    p.id = (uint32_t)(off + i);
    store_particle(pl, (size_t)ntot, (size_t)(off + i), p);
    if (track_fp) store_fp(pl, (size_t)ntot, (size_t)(off + i), FPm);
    if (keys) {
        const int b[3] = {base_of(p.x[0], P.h), base_of(p.x[1], P.h), base_of(p.x[2], P.h)};
        if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
        const uint32_t key = sort_key(P, b);
        keys[off + i] = key;
        count_key(counts, bcount, key);
    }
}

// An upload in sorted order (a single scene of n particles), pass 1: the
// positions alone, for the sort's keys and histogram (as k_pack writes them);
// xcopy (may be null) keeps the rows on the device for pass 2, so the host
// link carries them once.
template <typename T>
__global__ void __launch_bounds__(kIoThreads)
    k_pack_keys(int n, const T* __restrict__ x, T* __restrict__ xcopy, DevParams<T> P, uint32_t* __restrict__ keys,
                uint32_t* __restrict__ counts, uint32_t* __restrict__ bcount, uint32_t* __restrict__ flags) {
    __shared__ __align__(16) T sh[3 * kIoThreads];
    const int r0 = blockIdx.x * blockDim.x, i = r0 + threadIdx.x;
    const int cnt = min((int)blockDim.x, n - r0);
    T t3[3];
    load_rows(x, r0, cnt, t3, sh);
    if (xcopy) store_rows(xcopy, r0, cnt, t3, sh);
    if (i >= n) return;
    const int b[3] = {base_of(t3[0], P.h), base_of(t3[1], P.h), base_of(t3[2], P.h)};
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    const uint32_t key = sort_key(P, b);
    keys[i] = key;
    count_key(counts, bcount, key);
}

// Pass 2 (after the scan): each particle goes straight to its sorted slot -
// the scan's cursor of its key, taken as k_scatter takes it - so the
// permutation is the identity and the first step's P2G reads the particles
// in order; with `stress`, also its P F^T (stress_PFt, P the scene's
// material), which that P2G then reads instead of computing.  The host link
// bounds the pass, so the SVD costs nothing here; the scattered 16-byte
// stores merge in L2.
template <typename T>
__global__ void __launch_bounds__(kIoThreads)
    k_pack_place(int n, const T* __restrict__ x, const T* __restrict__ v, const T* __restrict__ B,
                 const T* __restrict__ FE, const T* __restrict__ FP, const T* __restrict__ Jp,
                 const T* __restrict__ mass, const T* __restrict__ vol, vec4<T>* __restrict__ pl, int track_fp,
                 const uint32_t* __restrict__ keys, uint32_t* __restrict__ cursor, uint32_t* __restrict__ perm,
                 uint32_t* __restrict__ flags, DevParams<T> P, vec4<T>* __restrict__ stress,
                 uint32_t* __restrict__ slot_of) {
    __shared__ __align__(16) T sh[9 * kIoThreads];
    const int r0 = blockIdx.x * blockDim.x, i = r0 + threadIdx.x;
    Particle<T> p;
    T FPm[9];
    if (!pack_row(n, r0, x, v, B, FE, FP, Jp, mass, vol, p, FPm, sh)) return;
    p.id = (uint32_t)i;
    const uint32_t key = keys[i];
    const uint32_t peers = __match_any_sync(__activemask(), key);
    const int lane = threadIdx.x & 31;
    const int leader = __ffs(peers) - 1;
    uint32_t base = 0;
    if (lane == leader) base = atomicAdd(cursor + key, (uint32_t)__popc(peers));
    base = __shfl_sync(peers, base, leader);
    const uint32_t slot = base + __popc(peers & lanemask_lt());
    if (slot >= (uint32_t)n) {  // counts that do not add up to n (flagged by the scan too)
        raise_flag(flags, 4u);
        return;
    }
    store_particle(pl, (size_t)n, (size_t)slot, p);
    if (track_fp) store_fp(pl, (size_t)n, (size_t)slot, FPm);
    perm[slot] = slot;
    slot_of[i] = slot;
    if (stress) {
        T G[9];
        stress_PFt(P, p.F, p.Jp, G);
        store_stress(stress, (size_t)n, (size_t)slot, G);
    }
}

// The slot of each particle of a scene (particles off .. off + n - 1 in
// slots off .. off + n - 1, in any order): slot[id - off].
template <typename T>
__global__ void k_slot_of_id(int n, int off, int ntot, const vec4<T>* __restrict__ pl, uint32_t* __restrict__ slot) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const uint32_t o = real_to_id<T>(pl[6 * (size_t)ntot + off + i].w) - (uint32_t)off;
    if (o < (uint32_t)n) slot[o] = (uint32_t)(off + i);
}

// The scene's particles in id order: thread o gathers particle id off + o
// from its slot and the rows go out coalesced (a slot outside the scene's,
// which a consistent state never holds, gives a zero row).
template <typename T>
__global__ void __launch_bounds__(kIoThreads)
    k_unpack(int n, int off, int ntot, const vec4<T>* __restrict__ pl, const uint32_t* __restrict__ slot,
             T* __restrict__ x, T* __restrict__ v, T* __restrict__ B, T* __restrict__ FE, T* __restrict__ FP,
             T* __restrict__ Jp, T* __restrict__ mass, T* __restrict__ vol, int track_fp) {
    __shared__ __align__(16) T sh[9 * kIoThreads];
    const int r0 = blockIdx.x * blockDim.x, o = r0 + threadIdx.x;
    const int cnt = min((int)blockDim.x, n - r0);
    Particle<T> p;
    T P[9];
    const uint32_t s = o < n ? slot[o] : 0xffffffffu;
    const bool ok = s - (uint32_t)off < (uint32_t)n;
    if (ok) {
        load_particle(pl, (size_t)ntot, (size_t)s, p);
        if (track_fp) {
            load_fp(pl, (size_t)ntot, (size_t)s, P);
        } else {  // only det F_P is carried: report the isotropic F_P with that det
            const T c = cbrt(p.Jp);
#pragma unroll
            for (int e = 0; e < 9; ++e) P[e] = (e % 4 == 0) ? c : T(0);
        }
    } else {
        p.x[0] = p.x[1] = p.x[2] = p.v[0] = p.v[1] = p.v[2] = p.m = p.vol = p.Jp = T(0);
#pragma unroll
        for (int e = 0; e < 9; ++e) p.B[e] = p.F[e] = P[e] = T(0);
    }
    if (x) store_rows(x, r0, cnt, p.x, sh);
    if (v) store_rows(v, r0, cnt, p.v, sh);
    if (B) store_rows(B, r0, cnt, p.B, sh);
    if (FE) store_rows(FE, r0, cnt, p.F, sh);
    if (FP) store_rows(FP, r0, cnt, P, sh);
    if (o >= n) return;
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

// One scene of a handle: its parameters and where its particles, grid nodes
// and 4x4x4 blocks start in the handle's shared arrays.
struct rd_scene_info {
    rd_params prm{};
    int n = 0;
    uint32_t poff = 0;
    size_t ncells = 0;
    size_t goff = 0;
    int NB[3] = {0, 0, 0};
    int nblocks = 0;
    uint32_t block_base = 0;
    bool set = false;  // particles uploaded
};

// Two steady steps captured as one CUDA graph, for one assignment of the
// ping-pong buffers and one dt.
struct rd_graph {
    int key = 0;
    double dt = 0.0;
    cudaGraphExec_t exec = nullptr;
    uint64_t launches = 0;
};

// Reverse-mode rollout: checkpoints of the forward states, the per-segment
// stores of the recomputed states and grids, and the adjoint buffers.
// Buffers of rd_time_integration, allocated on its first call: the list of
// cells with mass and a dense gradient accumulator (per cell), the compact
// L-BFGS vectors (3 reals per cell with mass; grown when a call needs more)
// and the reduction words.
struct rd_implicit_data {
    uint32_t* idx = nullptr;  // cells with mass, then their count at idx[ncells]
    void* gacc = nullptr;     // vec4 per cell: the particles' part of the gradient
    size_t cap = 0;           // cells the compact vectors hold
    int hist = 0;             // correction pairs they hold
    void* vec = nullptr;      // vstar, x, g, xold, gold, q, then s[hist], y[hist]
    double* red = nullptr;    // device reductions
    double* hred = nullptr;   // their page-locked host copy
};

struct rd_adjoint_data {
    bool recorded = false;
    uint64_t version = 0;  // handle version the record belongs to
    double dt = 0.0;
    int steps = 0, every = 0;
    size_t state_bytes = 0, grid_bytes = 0, split_bytes = 0;
    size_t nckpt = 0, nseg = 0;         // capacities (states)
    void* ckpt = nullptr;               // nckpt states
    // two segment stores, so that the recomputation of one segment runs
    // beside the reverse kernels of the next (a second stream)
    void* sstore[2] = {nullptr, nullptr};    // nseg + 1 states
    void* gstore[2] = {nullptr, nullptr};    // nseg grids (m, p) of those states
    uint32_t* sperm[2] = {nullptr, nullptr}; // nseg sorted permutations of those states
    int4* swork[2] = {nullptr, nullptr};     // nseg work lists
    uint32_t* snwork[2] = {nullptr, nullptr};// nseg (front, back) work-item counts
    void* ssplit[2] = {nullptr, nullptr};    // nseg plastic splits (U, s, V per sorted slot)
    int tail_store = 0;                 // the store the record's last segment is in
    cudaStream_t stream2 = nullptr;     // the reverse kernels
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr, ev_rec[2] = {nullptr, nullptr}, ev_rev[2] = {nullptr, nullptr};
    int occ_g2p = 1, occ_p2g = 1;       // resident CTAs per SM of the reverse kernels
    bool tail_valid = false;            // the store holds the last segment of the record
    // the reverse sweep captured as one CUDA graph, for one start assignment
    // of the ping-pong buffers and one record shape
    cudaGraphExec_t sweep = nullptr;
    int sweep_key = -1, sweep_end = 0, sweep_steps = 0, sweep_every = 0, sweep_wp = 0, sweep_mult = 0;
    double sweep_dt = 0.0;
    uint64_t sweep_launches = 0;
    // the record (forward with checkpoints) captured the same way; the host
    // state it starts from is part of the key, the one it ends in is replayed
    cudaGraphExec_t record = nullptr;
    int rec_key = -1, rec_end = 0, rec_steps = 0, rec_every = 0, rec_wp = 0, rec_mult = 0;
    double rec_dt = 0.0;
    uint64_t rec_launches = 0;
    void* final_state = nullptr;
    // adjoints in slot order, 25 n reals each (x 3n | v 3n | B 9n | F 9n | J_P n):
    // [0], [1] the states either side of the step being reversed, [2] the
    // partials of the first reverse kernel (and staging at both ends)
    void* adj[3] = {nullptr, nullptr, nullptr};
    void* agrid = nullptr;
    double* pacc = nullptr;             // 4 per particle slot
    double* acc = nullptr;              // 4 per scene
};

struct rd_handle {
    rd_params prm{};                    // scene 0's (precision, device, flags for all)
    uint64_t version = 0;               // bumped by every public call that changes the state
    rd_adjoint_data adj;
    rd_implicit_data imp;
    std::vector<rd_scene_info> scenes;  // one, or a batch
    void* d_scenes = nullptr;           // DevParams<T> per scene (batches)
    uint32_t* d_sblock = nullptr;       // first block of each scene, then the total
    uint32_t* d_spoff = nullptr;        // first particle of each scene, then the total
    void* h_scenes = nullptr;           // pinned staging of the table
    bool table_valid = false;
    double table_dt = 0.0, table_fs = 0.0;
    size_t max_scene_cells = 0;
    std::vector<rd_graph> graphs;
    bool use_graphs = true;
    bool capturing = false;  // inside a larger capture: no step-pair graphs
    std::vector<rd_collider> cols;  // box colliders (single scene)
    int col_mode = RD_COLLIDE_REFERENCE;
    double col_mu = 0.5;
    void* d_col = nullptr;          // Collider<T>[RD_MAX_COLLIDERS]
    TileMaps<1> smaps[2] = {};      // TMA maps of grid[0], grid[1] (single scene; kernel parameters)
    TileMaps<kBatchMaps>* bmaps = nullptr;  // [2]: the same per scene of a batch (the first kBatchMaps)
    int wp = 0;         // particles per work item (<= WorkP)
    int grid_mult = 0;  // persistent CTAs per SM of the step kernels (0: occupancy)
    int scatter = RD_SCATTER_LANE_PAIRS;     // lane layout of the fused kernel's P2G scatter
    std::vector<rd_tune_trial> tune_trials;  // the points the last rd_autotune timed
    cudaStream_t stream = nullptr;
    // the step's grid clear runs on `side` while the sort runs on `stream`
    // (forked and joined with the two events, so a captured step graph holds
    // the two branches)
    cudaStream_t side = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
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
    uint32_t* slot_of = nullptr;  // slot of each particle id (rd_get_particles)
    uint32_t* counts = nullptr;
    uint32_t* bcount = nullptr;   // particles per block
    uint8_t* gmark[2] = {nullptr, nullptr};  // blocks of grid[0] / grid[1] holding data
    uint32_t* cursor = nullptr;
    int4* work = nullptr;
    // item counters: front [0..1] and back [2..3] of the current sort's list
    // and the next's (by nb), then the fused kernel's claim counters [4..5]
    // (by grid buffer, h->g)
    uint32_t* nwork2 = nullptr;
    int nb = 0;                  // nwork2[nb] belongs to the last sort
    uint32_t* tile_sums = nullptr;
    uint32_t* tile_list = nullptr;  // non-empty tiles of the current sort, their count last
    size_t work_cap = 0;
    void* grid[2] = {nullptr, nullptr};  // (m, p) of this step / the next (fused); (m, v) in stage mode
    int g = 0;                           // current grid buffer
    bool fgrid_valid = false;            // grid[g] holds P2G(x) for rd_step with fgrid_dt
    bool in_order = false;               // planes in the current sort's slot order (perm the identity)
    bool clean_grids = false;            // both grid buffers zero and unmarked (cleared during an upload)
    void* stress = nullptr;              // P F^T of each particle by slot (3 vec4), from an upload
    bool stress_valid = false;           // stress holds the current state's
    bool slot_of_valid = false;          // slot_of holds the current state's (single scene)
    bool after_upload = false;           // the next step is the first after rd_set_particles
    double fgrid_dt = 0.0;
    void* gforce = nullptr;
    uint32_t* flags = nullptr;
    float4* xyzs = nullptr;
    uint32_t* rgba = nullptr;             // colour stream, original order
    unsigned long long* zid = nullptr;    // splat depth / id per pixel (allocated on first use)
    uint32_t* img = nullptr;              // splat image staging for host output
    size_t img_pixels = 0;
    void* io = nullptr;  // device SoA staging for set/get (36 reals per particle)
    void* grid_io = nullptr;  // device staging for rd_get_grid to host (7 reals per cell)
    bool keys_valid = false;
    bool sorted = false;
    int grid_mode = GRID_NONE;
    double last_dt = 0.0;
    uint64_t launches = 0, graph_replays = 0;
    uint64_t io_direct = 0, io_staged = 0;  // particle bytes set / got in place in host memory, through staging
    void* split_out = nullptr;  // the fused kernel keeps each particle's plastic split here (adjoint segments)
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

template <typename T>
DevParams<T> params_of(const rd_params& p, const int NB[3], int nkeys, int n, double dt, T fscale) {
    DevParams<T> P{};
    P.M[0] = p.max_i; P.M[1] = p.max_j; P.M[2] = p.max_k;
    P.NB[0] = NB[0]; P.NB[1] = NB[1]; P.NB[2] = NB[2];
    P.nkeys = nkeys;
    P.n = n;
    const T hh = (T)p.h;
    P.h = hh;
    P.dinv = reference_dinv<T>(hh);
    int he = 0;
    P.hinv_pow2 = std::frexp((double)hh, &he) == 0.5 ? (T)std::ldexp(1.0, 1 - he) : T(0);
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
    // the stress without an SVD (stress_direct): FP32 only, and while the
    // clamp keeps every |s_i^2 - 1| <= 0.1, where its series converges fast
    const double elo = (double)P.lo * (double)P.lo - 1.0 + 1e-5, ehi = (double)P.hi * (double)P.hi - 1.0 - 1e-5;
    const bool direct = sizeof(T) == 4 && elo >= -0.1 && ehi <= 0.1 && elo < ehi;
    P.elo = direct ? (T)elo : T(1);
    P.ehi = direct ? (T)ehi : T(-1);
    for (int a = 0; a < 3; ++a) P.g[a] = (T)p.gravity[a];
    volatile T xl = T(3) * hh;
    P.xlo = xl;
    volatile T x0 = (T)(p.max_i - 3) * hh, x1 = (T)(p.max_j - 3) * hh, x2 = (T)(p.max_k - 3) * hh;
    P.xhi[0] = x0; P.xhi[1] = x1; P.xhi[2] = x2;
    P.fscale = fscale;
    P.bc = p.bc;
    P.bc_width = p.bc_width;
    P.lagged = p.lagged_b;
    P.block_base = 0;
    P.goff = 0;
    return P;
}

// Parameters of scene 0 (the whole handle for a single scene); n is the
// particle count of all scenes, the stride of the particle planes.
template <typename T> DevParams<T> make_params(const rd_handle* h, double dt, T fscale) {
    DevParams<T> P = params_of<T>(h->prm, h->NB, h->nkeys, h->n, dt, fscale);
    P.ncol = (int)h->cols.size();
    P.col_mode = h->col_mode;
    P.mu = (T)h->col_mu;
    return P;
}

inline bool batched(const rd_handle* h) { return h->scenes.size() > 1; }

template <typename T> DevParams<T> scene_params(const rd_handle* h, int s, double dt, T fscale) {
    const rd_scene_info& sc = h->scenes[s];
    DevParams<T> P = params_of<T>(sc.prm, sc.NB, sc.nblocks * kCellsPerBlock, h->n, dt, fscale);
    P.block_base = sc.block_base;
    P.goff = sc.goff;
    if (!batched(h)) {  // colliders act on single-scene handles only
        P.ncol = (int)h->cols.size();
        P.col_mode = h->col_mode;
        P.mu = (T)h->col_mu;
    }
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
    D.nwork_back = h->nwork2 + 2 + h->nb;
    D.claim = h->nwork2 + 4 + h->g;
    D.claim_next = h->nwork2 + 4 + (h->g ^ 1);
    D.work_cap = (uint32_t)h->work_cap;
    D.grid = h->grid[h->g];
    D.grid_next = h->grid[h->g ^ 1];
    D.gforce = h->gforce;
    D.flags = h->flags;
    D.split_out = h->split_out;
    D.bcount = h->bcount;
    D.gmark = h->gmark[h->g];
    D.gmark_next = h->gmark[h->g ^ 1];
    D.scenes = h->d_scenes;
    D.sblock = h->d_sblock;
    D.spoff = h->d_spoff;
    D.nscenes = (int)h->scenes.size();
    D.colliders = h->d_col;
    return D;
}

inline unsigned blocks_for(size_t n, unsigned t) { return (unsigned)std::max<size_t>(1, (n + t - 1) / t); }

rd_status launched(rd_handle* h, const char* what, int count = 1) {
    h->launches += (uint64_t)count;
    return check_cuda(h, cudaGetLastError(), what);
}

constexpr size_t kEventPairs = 4096;

// Uploads the per-scene parameter table of a batch for (dt, fscale) unless it
// holds them already.
template <typename T> rd_status ensure_table(rd_handle* h, double dt, T fscale) {
    if (!batched(h)) return RD_OK;
    if (h->table_valid && h->table_dt == dt && h->table_fs == (double)fscale) return RD_OK;
    // the pinned staging may still be the source of the previous upload
    RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    DevParams<T>* hp = static_cast<DevParams<T>*>(h->h_scenes);
    for (size_t s = 0; s < h->scenes.size(); ++s) hp[s] = scene_params<T>(h, (int)s, dt, fscale);
    RD_TRY(check_cuda(h, cudaMemcpyAsync(h->d_scenes, hp, h->scenes.size() * sizeof(DevParams<T>),
                                         cudaMemcpyHostToDevice, h->stream),
                      "scene table"));
    h->table_valid = true;
    h->table_dt = dt;
    h->table_fs = (double)fscale;
    return RD_OK;
}

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

template <typename T> int work_size(const rd_handle* h) {
    return h->wp > 0 ? std::min(h->wp, WorkP<T>::value) : WorkP<T>::value;
}

// Sort by block key: histogram (unless the last fused G2P already counted),
// scan + work items, scatter into perm (unless the caller places the
// particles by the scan's cursors itself: scatter false).
template <typename T> rd_status sort_particles(rd_handle* h, bool scatter = true) {
    if (h->n == 0) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->nwork2, 0, 4 * sizeof(uint32_t), h->stream), "memset nwork"));
        h->sorted = true;
        return RD_OK;
    }
    DevParams<T> P = make_params<T>(h, 0.0, T(0));
    h->in_order = false;  // a new permutation
    if (!h->keys_valid) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->counts, 0, sizeof(uint32_t) * h->nkeys, h->stream), "memset counts"));
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->bcount, 0, sizeof(uint32_t) * h->nblocks, h->stream), "memset counts"));
        long t = tmark_begin(h, RD_KERNEL_KEYS);
        const DevBufs D = bufs<T>(h);
        const vec4<T>* pl = static_cast<const vec4<T>*>(h->pl[h->cur]);
        if (batched(h)) {
            RD_TRY(ensure_table<T>(h, h->table_valid ? h->table_dt : 0.0, T(h->table_valid ? h->table_fs : 0.0)));
            k_keys<T, true><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, D, pl, h->keys[h->cur]);
        } else {
            k_keys<T, false><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, D, pl, h->keys[h->cur]);
        }
        tmark_end(h, t);
        RD_TRY(launched(h, "k_keys"));
    }
    const int ntiles = (h->nkeys + kScanTile - 1) / kScanTile;
    // this sort fills nwork2[nb ^ 1] (cleared by the previous sort or at
    // creation) and clears nwork2[nb] for the next one
    uint32_t* nw = h->nwork2 + (h->nb ^ 1);
    uint32_t* nw_next = h->nwork2 + h->nb;
    uint32_t* nw_back = h->nwork2 + 2 + (h->nb ^ 1);
    uint32_t* nw_next_back = h->nwork2 + 2 + h->nb;
    long t = tmark_begin(h, RD_KERNEL_SCAN);
    if (ntiles <= kTileSumsInPrefix) {  // small grids: the prefix kernel sums the tiles itself
        k_tile_prefix<<<1, 1024, 0, h->stream>>>(h->tile_sums, ntiles, nw_next, (uint32_t)h->n, h->flags,
                                                 h->tile_list, h->bcount, h->nblocks, nw_next_back);
    } else {
        k_tile_sums<<<blocks_for((size_t)ntiles * 32, 256), 256, 0, h->stream>>>(h->bcount, h->nblocks, ntiles,
                                                                                 h->tile_sums);
        RD_TRY(launched(h, "k_tile_sums"));
        k_tile_prefix<<<1, 1024, 0, h->stream>>>(h->tile_sums, ntiles, nw_next, (uint32_t)h->n, h->flags,
                                                 h->tile_list, nullptr, 0, nw_next_back);
    }
    const unsigned scan_grid = (unsigned)std::min<size_t>((size_t)ntiles, (size_t)h->sms * 2);
    k_scan<<<scan_grid, kScanThreads, 0, h->stream>>>(h->counts, h->cursor, h->bcount, h->tile_sums, h->tile_list,
                                                      ntiles, h->nkeys, h->work, nw, (uint32_t)h->work_cap,
                                                      (uint32_t)work_size<T>(h), h->flags, h->d_sblock,
                                                      (int)h->scenes.size(), nw_back);
    tmark_end(h, t);
    RD_TRY(launched(h, "k_scan", 2));
    h->nb ^= 1;
    if (scatter) {
        t = tmark_begin(h, RD_KERNEL_SCATTER);
        k_scatter<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(h->n, h->keys[h->cur], h->cursor, h->perm);
        tmark_end(h, t);
        RD_TRY(launched(h, "k_scatter"));
    }
    h->keys_valid = false;  // counts consumed
    h->sorted = true;
    return RD_OK;
}

// The k_g2p2g instantiation for this handle: batch or single scene, with or
// without the full F_P, and the order of the F update.
template <typename T> using SingleFused = void (*)(DevParams<T>, DevBufs, const FusedMaps<false>);
template <typename T> using BatchFused = void (*)(DevParams<T>, DevBufs, const FusedMaps<true>);
// Scatter layouts a handle can use: both for FP32 with the lagged-B order and
// J_P only (the instantiations the record-pairs layout is compiled for), else
// the lane-pairs layout alone.
int scatter_layouts(const rd_handle* h) {
    return h->prm.precision == RD_FP32 && h->prm.lagged_b && !h->prm.track_fp ? 2 : 1;
}
template <typename T> BatchFused<T> batch_fused_kernel(const rd_handle* h) {
    if constexpr (sizeof(T) == 4) {
        if (h->scatter == RD_SCATTER_RECORD_PAIRS && scatter_layouts(h) > 1) return k_g2p2g<T, false, true, true, true>;
    }
    return h->prm.lagged_b ? k_g2p2g<T, false, true, true> : k_g2p2g<T, false, true, false>;
}
template <typename T> SingleFused<T> single_fused_kernel(const rd_handle* h) {
    const bool lag = h->prm.lagged_b != 0;
    if constexpr (sizeof(T) == 4) {
        if (h->scatter == RD_SCATTER_RECORD_PAIRS && scatter_layouts(h) > 1) return k_g2p2g<T, false, false, true, true>;
    }
    if (h->prm.track_fp) return lag ? k_g2p2g<T, true, false, true> : k_g2p2g<T, true, false, false>;
    return lag ? k_g2p2g<T, false, false, true> : k_g2p2g<T, false, false, false>;
}
template <typename T> const void* fused_kernel(const rd_handle* h) {
    return batched(h) ? (const void*)batch_fused_kernel<T>(h) : (const void*)single_fused_kernel<T>(h);
}

template <typename T> unsigned persistent_grid(const rd_handle* h, int occ) {
    const size_t max_items = (size_t)h->n / work_size<T>(h) + (size_t)std::min<int64_t>(h->nblocks, h->n) + 1;
    const int per_sm = h->grid_mult > 0 ? std::min(h->grid_mult, occ) : occ;
    return (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)h->sms * per_sm));
}

// Zeroes the marked node blocks of grid buffer `which` (k_grid_clear), on
// `st` (the handle's stream by default).
template <typename T> rd_status clear_grid(rd_handle* h, int which, cudaStream_t st = nullptr) {
    if (!st) st = h->stream;
    const DevParams<T> P = make_params<T>(h, 0.0, T(0));
    DevBufs D = bufs<T>(h);
    const unsigned nb = (unsigned)std::min<size_t>(blocks_for((size_t)h->nblocks, 256), (size_t)h->sms * 16);
    vec4<T>* grid = static_cast<vec4<T>*>(h->grid[which]);
    if (batched(h))
        k_grid_clear<T, true><<<nb, 256, 0, st>>>(P, D, grid, h->gmark[which], h->nblocks);
    else
        k_grid_clear<T, false><<<nb, 256, 0, st>>>(P, D, grid, h->gmark[which], h->nblocks);
    return launched(h, "k_grid_clear");
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
    const bool batch = batched(h);
    if (batch) RD_TRY(ensure_table<T>(h, dt, (T)dt));
    // a steady step clears the next grid buffer (the one the previous step
    // read; nothing in the sort touches it) on the side stream while the sort
    // runs; per-kernel timing keeps every launch on the handle's stream
    const bool rebuild = !(h->fgrid_valid && h->fgrid_dt == dt);
    const bool fork = !rebuild && !h->sorted && !h->timing && h->side;
    if (fork) {
        RD_TRY(check_cuda(h, cudaEventRecord(h->ev_fork, h->stream), "fork"));
        RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->side, h->ev_fork, 0), "fork"));
        RD_TRY(clear_grid<T>(h, h->g ^ 1, h->side));
        RD_TRY(check_cuda(h, cudaEventRecord(h->ev_join, h->side), "join"));
    }
    if (!h->sorted) RD_TRY(sort_particles<T>(h));
    DevParams<T> P = make_params<T>(h, dt, (T)dt);
    long t;
    if (rebuild) {  // P2G of the current state
        if (!h->clean_grids) {
            t = tmark_begin(h, RD_KERNEL_GRID_CLEAR);
            RD_TRY(clear_grid<T>(h, h->g));
            tmark_end(h, t);
        }
        DevBufs D = bufs<T>(h);
        // particles not yet in sorted order (an upload): k_p2g, which reads
        // them all through the permutation, also writes them to the other
        // plane buffer in order, so the fused kernel reads them sequentially.
        // Not in the adjoint's stored segments, whose plane buffers are the
        // store's slots.
        const bool reorder = !h->split_out && !h->prm.track_fp && !h->in_order;
        if (reorder) {
            D.reorder_out = h->pl[h->cur ^ 1];
            D.perm_reset = h->perm;
        }
        if (h->stress_valid) D.stress = h->stress;
        t = tmark_begin(h, RD_KERNEL_P2G);
        const unsigned pg = persistent_grid<T>(h, h->occ_p2g);
        if (batch)
            k_p2g<T, true, true, true><<<pg, kP2GThreads<T>, sizeof(P2GShared<T>), h->stream>>>(P, D);
        else
            k_p2g<T, true, true, false><<<pg, kP2GThreads<T>, sizeof(P2GShared<T>), h->stream>>>(P, D);
        tmark_end(h, t);
        RD_TRY(launched(h, "k_p2g"));
        if (reorder) h->cur ^= 1;  // the ordered copy is the state now; perm is the identity
    }
    if (fork) {
        RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->stream, h->ev_join, 0), "join"));
    } else if (!h->clean_grids) {
        t = tmark_begin(h, RD_KERNEL_GRID_CLEAR);
        RD_TRY(clear_grid<T>(h, h->g ^ 1));
        tmark_end(h, t);
    }
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    DevBufs D = bufs<T>(h);
    // the first step after an upload keeps slot_of current, so that a download
    // right after it (a caller moving the state in and out every step) needs
    // no k_slot_of_id; steady steps do not pay for the scattered stores
    const bool keep_slots = !batch && h->after_upload;
    if (keep_slots) D.slot_of = h->slot_of;
    h->after_upload = false;
    t = tmark_begin(h, RD_KERNEL_G2P2G);
    const unsigned fg = persistent_grid<T>(h, h->occ_g2p);
    if (batch)
        batch_fused_kernel<T>(h)<<<fg, kFusedThreads, fused_smem_bytes<T>(), h->stream>>>(P, D, h->bmaps[h->g]);
    else
        single_fused_kernel<T>(h)<<<fg, kFusedThreads, fused_smem_bytes<T>(), h->stream>>>(P, D, h->smaps[h->g]);
    tmark_end(h, t);
    RD_TRY(launched(h, "k_g2p2g"));
    h->slot_of_valid = keep_slots;
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
    if (batched(h)) return fail(h, RD_NOT_SUPPORTED, "the stage calls drive a single scene; batches step with rd_step");
    const size_t nc = h->ncells;
    const unsigned cb = blocks_for(nc, 256);
    DevParams<T> P = make_params<T>(h, dt, T(1));
    h->fgrid_valid = false;
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    switch (stage) {
        case RD_STAGE_RASTERIZE: {
            if (!h->sorted) RD_TRY(sort_particles<T>(h));
            RD_TRY(check_cuda(h, cudaMemsetAsync(h->grid[h->g], 0, nc * sizeof(vec4<T>), h->stream), "memset grid"));
            RD_TRY(check_cuda(h, cudaMemsetAsync(h->gforce, 0, nc * sizeof(vec4<T>), h->stream), "memset force"));
            if (h->n > 0) {
                DevBufs D = bufs<T>(h);
                k_p2g<T, true, false, false><<<persistent_grid<T>(h, h->occ_p2g), kP2GThreads<T>, sizeof(P2GShared<T>), h->stream>>>(P, D);
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
                k_p2g<T, false, true, false><<<persistent_grid<T>(h, h->occ_p2g), kP2GThreads<T>, sizeof(P2GShared<T>), h->stream>>>(P, D);
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
            if (h->cols.empty()) return RD_OK;  // empty collider list: bodyCollision is the identity
            if (h->grid_mode != GRID_V) return fail(h, RD_INVALID_ARG, "collision stage needs a grid");
            k_grid_collide<T><<<cb, 256, 0, h->stream>>>(P, static_cast<vec4<T>*>(h->grid[h->g]),
                                                          static_cast<const Collider<T>*>(h->d_col));
            return launched(h, "k_grid_collide");
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
            k_volumes<T, false><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(
                P, bufs<T>(h), static_cast<vec4<T>*>(h->pl[h->cur]), static_cast<const vec4<T>*>(h->grid[h->g]));
            return launched(h, "k_volumes");
        default:
            return fail(h, RD_INVALID_ARG, "unknown stage id");
    }
}

// True when the kernels can read and write [p, p + bytes) in place: the range
// lies inside one page-locked host allocation mapped at the same address on
// the device (cudaHostAlloc / cudaHostRegister under unified addressing).
// The pack and unpack kernels then move the particle state over the
// CPU-GPU link themselves, with no staging copy through device memory; on a
// Grace-Blackwell node that is faster than copying in and packing apart.
bool host_in_place(const void* p, size_t bytes) {
    using PtrAttr = CUresult (*)(void*, CUpointer_attribute, CUdeviceptr);
    static PtrAttr attr = nullptr;
    static std::once_flag once;
    std::call_once(once, [] {
        cudaDriverEntryPointQueryResult q{};
        void* fn = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuPointerGetAttribute", &fn, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            attr = reinterpret_cast<PtrAttr>(fn);
    });
    cudaPointerAttributes a{};
    if (cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();  // an unknown pointer is not an error here
        return false;
    }
    if (a.type != cudaMemoryTypeHost || a.devicePointer != p || !attr) return false;
    CUdeviceptr start = 0;
    size_t size = 0;
    if (attr(&start, CU_POINTER_ATTRIBUTE_RANGE_START_ADDR, (CUdeviceptr)p) != CUDA_SUCCESS ||
        attr(&size, CU_POINTER_ATTRIBUTE_RANGE_SIZE, (CUdeviceptr)p) != CUDA_SUCCESS)
        return false;
    return (uintptr_t)p >= (uintptr_t)start && (uintptr_t)p + bytes <= (uintptr_t)start + size;
}

template <typename T> rd_status set_particles_impl(rd_handle* h, int scene, const rd_particles* in, int where) {
    rd_scene_info& sc = h->scenes[scene];
    const size_t n = (size_t)sc.n;
    if (!in->x || !in->v || !in->mass) return fail(h, RD_INVALID_ARG, "x, v and mass are required");
    T* io = static_cast<T*>(h->io);
    // io layout: x 3n | v 3n | B 9n | FE 9n | FP 9n | Jp n | mass n | vol n
    T* d[8] = {io, io + 3 * n, io + 6 * n, io + 15 * n, io + 24 * n, io + 33 * n, io + 34 * n, io + 35 * n};
    const void* src[8] = {in->x, in->v, in->B, in->FE, in->FP, in->Jp, in->mass, in->volume};
    const size_t cnt[8] = {3 * n, 3 * n, 9 * n, 9 * n, 9 * n, n, n, n};
    const T* ptr[8];
    bool from_host = n > 0;  // every array page-locked host memory read in place (the link is the bound)
    for (int k = 0; k < 8; ++k) {
        if (!src[k] || n == 0) { ptr[k] = nullptr; continue; }
        const bool in_place = host_in_place(src[k], cnt[k] * sizeof(T));
        if (where == RD_HOST && !in_place) {
            RD_TRY(check_cuda(h, cudaMemcpyAsync(d[k], src[k], cnt[k] * sizeof(T), cudaMemcpyHostToDevice, h->stream),
                              "upload"));
            ptr[k] = d[k];
            h->io_staged += cnt[k] * sizeof(T);
        } else {
            ptr[k] = static_cast<const T*>(src[k]);
            if (where == RD_HOST) h->io_direct += cnt[k] * sizeof(T);
        }
        from_host = from_host && in_place;
    }
    // a single scene's first sort reads its keys and histogram from the pack
    const bool keys = !batched(h) && n > 0;
    if (keys) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->counts, 0, sizeof(uint32_t) * h->nkeys, h->stream), "memset counts"));
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->bcount, 0, sizeof(uint32_t) * h->nblocks, h->stream), "memset counts"));
    }
    // A single scene after its first step, read in place from page-locked
    // host memory: the upload sorts the particles on the way in - keys from
    // the positions, the scan, then every particle to its sorted slot - so the
    // next step's P2G reads them in order.  It replaces the step's scatter,
    // its permuted-read P2G and its reordering copy, and its scattered stores
    // and the first P2G's stress run while the link is the bound.  From device
    // memory (or the staging buffer) nothing hides them, and the one-pass
    // route (k_pack, coalesced) costs less, as it does on a first upload.
    if (keys && from_host && h->last_dt > 0.0 && !h->split_out) {
        const DevParams<T> P = make_params<T>(h, 0.0, T(0));
        const unsigned nb = blocks_for(n, kIoThreads);
        k_pack_keys<T><<<nb, kIoThreads, 0, h->stream>>>((int)n, ptr[0], ptr[0] == d[0] ? nullptr : d[0], P,
                                                         h->keys[h->cur], h->counts, h->bcount, h->flags);
        RD_TRY(launched(h, "k_pack_keys"));
        h->keys_valid = true;
        h->sorted = false;
        RD_TRY(sort_particles<T>(h, false));
        // both grid buffers cleared on the second stream while the link is busy
        const bool side = h->side && !h->timing;
        if (side) {
            RD_TRY(check_cuda(h, cudaEventRecord(h->ev_fork, h->stream), "fork"));
            RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->side, h->ev_fork, 0), "fork"));
        }
        RD_TRY(clear_grid<T>(h, 0, side ? h->side : h->stream));
        RD_TRY(clear_grid<T>(h, 1, side ? h->side : h->stream));
        if (side) RD_TRY(check_cuda(h, cudaEventRecord(h->ev_join, h->side), "join"));
        if (!h->stress) {  // on the first such upload: the first P2G's stress, 3 vec4 a particle
            const cudaError_t e = cudaMalloc(&h->stress, 3 * n * sizeof(vec4<T>));
            if (e != cudaSuccess) {
                cudaGetLastError();
                h->stress = nullptr;  // the P2G computes it then
            }
        }
        k_pack_place<T><<<nb, kIoThreads, 0, h->stream>>>(
            (int)n, d[0], ptr[1], ptr[2], ptr[3], ptr[4], ptr[5], ptr[6], ptr[7], static_cast<vec4<T>*>(h->pl[h->cur]),
            h->prm.track_fp, h->keys[h->cur], h->cursor, h->perm, h->flags, P, static_cast<vec4<T>*>(h->stress),
            h->slot_of);
        RD_TRY(launched(h, "k_pack_place"));
        if (side) RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->stream, h->ev_join, 0), "join"));
        sc.set = true;
        h->keys_valid = false;
        h->sorted = true;
        h->in_order = true;
        h->fgrid_valid = false;
        h->clean_grids = true;
        h->stress_valid = h->stress != nullptr;
        h->slot_of_valid = true;
        h->after_upload = true;
        h->grid_mode = GRID_NONE;
        return RD_OK;
    }
    if (n > 0) {
        k_pack<T><<<blocks_for(n, kIoThreads), kIoThreads, 0, h->stream>>>(
            (int)n, (int)sc.poff, h->n, ptr[0], ptr[1], ptr[2], ptr[3], ptr[4], ptr[5], ptr[6], ptr[7],
            static_cast<vec4<T>*>(h->pl[h->cur]), h->prm.track_fp, make_params<T>(h, 0.0, T(0)),
            keys ? h->keys[h->cur] : nullptr, h->counts, h->bcount, h->flags);
        RD_TRY(launched(h, "k_pack"));
    }
    sc.set = true;
    h->after_upload = true;
    h->keys_valid = keys;
    h->sorted = false;
    h->fgrid_valid = false;
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    h->grid_mode = GRID_NONE;
    return RD_OK;
}

template <typename T> rd_status get_particles_impl(rd_handle* h, int scene, rd_particles* out, int where) {
    const rd_scene_info& sc = h->scenes[scene];
    const size_t n = (size_t)sc.n;
    if (n == 0) return RD_OK;
    T* io = static_cast<T*>(h->io);
    T* d[8] = {io, io + 3 * n, io + 6 * n, io + 15 * n, io + 24 * n, io + 33 * n, io + 34 * n, io + 35 * n};
    void* dst[8] = {out->x, out->v, out->B, out->FE, out->FP, out->Jp, out->mass, out->volume};
    const size_t cnt[8] = {3 * n, 3 * n, 9 * n, 9 * n, 9 * n, n, n, n};
    T* tgt[8];
    bool staged[8];
    for (int k = 0; k < 8; ++k) {
        staged[k] = dst[k] && where == RD_HOST && !host_in_place(dst[k], cnt[k] * sizeof(T));
        tgt[k] = dst[k] ? (staged[k] ? d[k] : static_cast<T*>(dst[k])) : nullptr;
        if (dst[k] && where == RD_HOST) (staged[k] ? h->io_staged : h->io_direct) += cnt[k] * sizeof(T);
    }
    const vec4<T>* pl = static_cast<const vec4<T>*>(h->pl[h->cur]);
    if (batched(h) || !h->slot_of_valid) {
        k_slot_of_id<T><<<blocks_for(n, 256), 256, 0, h->stream>>>((int)n, (int)sc.poff, h->n, pl, h->slot_of);
        RD_TRY(launched(h, "k_slot_of_id"));
        h->slot_of_valid = !batched(h);
    }
    k_unpack<T><<<blocks_for(n, kIoThreads), kIoThreads, 0, h->stream>>>((int)n, (int)sc.poff, h->n, pl, h->slot_of,
                                                                         tgt[0], tgt[1], tgt[2], tgt[3], tgt[4],
                                                                         tgt[5], tgt[6], tgt[7], h->prm.track_fp);
    RD_TRY(launched(h, "k_unpack"));
    if (where == RD_HOST) {
        for (int k = 0; k < 8; ++k)
            if (staged[k])
                RD_TRY(check_cuda(h, cudaMemcpyAsync(dst[k], d[k], cnt[k] * sizeof(T), cudaMemcpyDeviceToHost, h->stream),
                                  "download"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    }
    return RD_OK;
}

template <typename T>
rd_status get_grid_impl(rd_handle* h, int scene, void* mass, void* vel, void* force, int where) {
    const rd_scene_info& sc = h->scenes[scene];
    const size_t nc = sc.ncells;
    if (h->grid_mode == GRID_NONE) return fail(h, RD_INVALID_ARG, "no grid computed yet");
    if (force && batched(h)) return fail(h, RD_NOT_SUPPORTED, "grid forces exist in stage mode only");
    const bool host = where == RD_HOST;
    if (host && !h->grid_io) {  // allocated on first use only: a debugging / parity path
        RD_TRY(check_cuda(h, cudaMalloc(&h->grid_io, 7 * h->max_scene_cells * sizeof(T)), "grid export buffer"));
    }
    T* scratch = static_cast<T*>(h->grid_io);
    T* m_d = host ? scratch : static_cast<T*>(mass);
    T* v_d = host ? scratch + nc : static_cast<T*>(vel);
    DevParams<T> P = scene_params<T>(h, scene, h->last_dt, T(1));
    const unsigned cb = blocks_for(nc, 256);
    if (h->grid_mode == GRID_FUSED)  // the grid the last step's G2P read
        k_grid_export<T, true><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g ^ 1]) + sc.goff,
                                                          mass ? m_d : nullptr, vel ? v_d : nullptr,
                                                          static_cast<const Collider<T>*>(h->d_col));
    else
        k_grid_export<T, false><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g]) + sc.goff,
                                                           mass ? m_d : nullptr, vel ? v_d : nullptr,
                                                           static_cast<const Collider<T>*>(h->d_col));
    RD_TRY(launched(h, "k_grid_export"));
    T* f_d = nullptr;
    if (force) {
        f_d = host ? scratch + 4 * nc : static_cast<T*>(force);
        if (h->grid_mode == GRID_FUSED) {
            RD_TRY(check_cuda(h, cudaMemsetAsync(f_d, 0, 3 * nc * sizeof(T), h->stream), "force"));
        } else {
            k_grid_export<T, false><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->gforce), nullptr, f_d,
                                                               nullptr);
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
    if (!batched(h)) {
        RD_TRY(stage_impl<T>(h, RD_STAGE_RASTERIZE, 0.0));
        return stage_impl<T>(h, RD_STAGE_VOLUMES, 0.0);
    }
    // a batch: the rasterized mass of every scene, then V_p = m_p / rho_p
    RD_TRY(ensure_table<T>(h, h->table_valid ? h->table_dt : 0.0, T(h->table_valid ? h->table_fs : 0.0)));
    if (!h->sorted) RD_TRY(sort_particles<T>(h));
    h->fgrid_valid = false;
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    RD_TRY(clear_grid<T>(h, h->g));
    const DevParams<T> P = make_params<T>(h, 0.0, T(1));
    const DevBufs D = bufs<T>(h);
    k_p2g<T, true, false, true><<<persistent_grid<T>(h, h->occ_p2g), kP2GThreads<T>, sizeof(P2GShared<T>), h->stream>>>(P, D);
    RD_TRY(launched(h, "k_p2g<rasterize>"));
    k_volumes<T, true><<<blocks_for(h->n, 256), 256, 0, h->stream>>>(P, D, static_cast<vec4<T>*>(h->pl[h->cur]),
                                                                      static_cast<const vec4<T>*>(h->grid[h->g]));
    RD_TRY(launched(h, "k_volumes"));
    h->grid_mode = GRID_MV;
    return RD_OK;
}

template <typename T> rd_status occupancy(rd_handle* h) {
    int o = 0;
    const int sm = (int)sizeof(P2GShared<T>);
    const void* p2g[] = {(const void*)k_p2g<T, true, true, false>, (const void*)k_p2g<T, true, false, false>,
                         (const void*)k_p2g<T, false, true, false>, (const void*)k_p2g<T, true, true, true>,
                         (const void*)k_p2g<T, true, false, true>};
    for (const void* f : p2g)
        RD_TRY(check_cuda(h, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, sm), "smem attr"));
    RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_p2g<T, true, true, false>, kP2GThreads<T>, sm), "occ"));
    h->occ_p2g = std::max(1, o);
    const int fsm = (int)fused_smem_bytes<T>();
    // every scatter layout the handle can switch to: the smallest occupancy
    const int layout = h->scatter;
    int occ = 0;
    for (int l = 0; l < scatter_layouts(h); ++l) {
        h->scatter = l;
        const void* used = (const void*)fused_kernel<T>(h);
        rd_status st = check_cuda(h, cudaFuncSetAttribute(used, cudaFuncAttributeMaxDynamicSharedMemorySize, fsm),
                                  "smem attr");
        if (st == RD_OK)
            st = check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, used, kFusedThreads, fsm), "occ");
        if (st != RD_OK) {
            h->scatter = layout;
            return st;
        }
        occ = l == 0 ? o : std::min(occ, o);
    }
    h->scatter = layout;
    h->occ_g2p = std::max(1, occ);
    return RD_OK;
}

void drop_graphs(rd_handle* h) {
    for (rd_graph& g : h->graphs)
        if (g.exec) cudaGraphExecDestroy(g.exec);
    h->graphs.clear();
    if (h->adj.sweep) cudaGraphExecDestroy(h->adj.sweep);
    h->adj.sweep = nullptr;
    h->adj.sweep_key = -1;
    if (h->adj.record) cudaGraphExecDestroy(h->adj.record);
    h->adj.record = nullptr;
    h->adj.rec_key = -1;
}

void release(rd_handle* h) {
    for (cudaEvent_t e : h->ev)
        if (e) cudaEventDestroy(e);
    {
        rd_implicit_data& m = h->imp;
        void* ip[] = {m.idx, m.gacc, m.vec, m.red};
        for (void* p : ip)
            if (p) cudaFree(p);
        if (m.hred) cudaFreeHost(m.hred);
        m = rd_implicit_data{};
    }
    h->ev.clear();
    drop_graphs(h);
    rd_adjoint_data& a = h->adj;
    for (int b = 0; b < 2; ++b) {
        void* sp[] = {a.sstore[b], a.gstore[b], a.sperm[b], a.swork[b], a.snwork[b], a.ssplit[b]};
        for (void* p : sp)
            if (p) cudaFree(p);
    }
    cudaEvent_t evs[] = {a.ev_fork, a.ev_join, a.ev_rec[0], a.ev_rec[1], a.ev_rev[0], a.ev_rev[1]};
    for (cudaEvent_t e : evs)
        if (e) cudaEventDestroy(e);
    if (a.stream2) cudaStreamDestroy(a.stream2);
    void* aptrs[] = {a.ckpt, a.final_state, a.adj[0], a.adj[1], a.adj[2],
                     a.agrid, a.pacc, a.acc};
    for (void* p : aptrs)
        if (p) cudaFree(p);
    void* ptrs[] = {h->pl[0], h->pl[1], h->keys[0], h->keys[1], h->perm, h->slot_of, h->counts, h->bcount, h->gmark[0],
                    h->gmark[1], h->cursor, h->work,
                    h->nwork2, h->tile_sums, h->tile_list, h->grid[0], h->grid[1], h->gforce, h->flags, h->xyzs, h->io, h->grid_io,
                    h->d_col, h->rgba, h->zid, h->img, h->stress,
                    h->d_scenes, h->d_sblock, h->d_spoff};
    for (void* p : ptrs)
        if (p) cudaFree(p);
    if (h->h_scenes) cudaFreeHost(h->h_scenes);
    delete[] h->bmaps;
    h->bmaps = nullptr;
    if (h->ev_fork) cudaEventDestroy(h->ev_fork);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    if (h->side) cudaStreamDestroy(h->side);
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

}  // extern "C"

namespace {

// At least 8 nodes per axis: the stencil needs them, and the fused kernel's
// TMA box (kTile nodes per axis) then never exceeds a grid axis.
static_assert(kTile <= 8, "tile copies assume grids of at least kTile nodes per axis");
bool valid_scene(const rd_params& p) {
    return p.max_i >= 8 && p.max_j >= 8 && p.max_k >= 8 && p.num_particles >= 0 && p.h > 0 &&
           (p.precision == RD_FP32 || p.precision == RD_FP64) && p.bc_width >= 0 &&
           (int64_t)p.max_i * p.max_j * p.max_k <= (int64_t)1 << 30;
}

// Creates a handle over nscenes scenes: the particles of scene s occupy
// [poff_s, poff_s + n_s) of the shared particle planes (in every step's
// sorted order too, since the block keys of scene s precede those of s + 1),
// its grid nodes [goff_s, goff_s + cells_s) of each grid buffer.
// Tensor maps of both grid buffers for the fused kernel's tile copies: per
// scene (the first kBatchMaps of a batch), its grid region as a 4-D tensor
// (channel, z, y, x) of the element type, box 4 x kTile^3; nodes outside the
// region read as zero.  They are passed by value as the kernel's
// __grid_constant__ parameter (TileMaps), so no map is read from memory the
// host writes.  The encoder is the driver's cuTensorMapEncodeTiled, fetched
// through the runtime.
rd_status encode_tile_maps(rd_handle* h) {
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    static std::mutex mu;
    {
        std::lock_guard<std::mutex> lock(mu);
        if (!encode) {
            cudaDriverEntryPointQueryResult q{};
            void* fn = nullptr;
            if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) !=
                    cudaSuccess ||
                q != cudaDriverEntryPointSuccess || !fn)
                return fail(h, RD_CUDA_ERROR, "cuTensorMapEncodeTiled is not available");
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(fn);
        }
    }
    const bool batch = batched(h);
    if (batch) {
        h->bmaps = new (std::nothrow) TileMaps<kBatchMaps>[2]();
        if (!h->bmaps) return fail(h, RD_OOM, "tensor maps");
    }
    const size_t ns = std::min<size_t>(h->scenes.size(), kBatchMaps);
    const cuuint64_t es = (cuuint64_t)h->esize;
    for (size_t k = 0; k < 2 * ns; ++k) {
        const int b = (int)(k / ns);
        const size_t s = k % ns;
        const rd_scene_info& sc = h->scenes[s];
        const cuuint64_t M0 = (cuuint64_t)sc.prm.max_i, M1 = (cuuint64_t)sc.prm.max_j, M2 = (cuuint64_t)sc.prm.max_k;
        const cuuint64_t dims[4] = {4, M2, M1, M0};
        const cuuint64_t strides[3] = {4 * es, 4 * es * M2, 4 * es * M2 * M1};
        const cuuint32_t box[4] = {4, (cuuint32_t)kTile, (cuuint32_t)kTile, (cuuint32_t)kTile};
        const cuuint32_t estr[4] = {1, 1, 1, 1};
        void* base = static_cast<char*>(h->grid[b]) + sc.goff * 4 * es;
        const CUresult r = encode(batch ? &h->bmaps[b].m[s] : &h->smaps[b].m[0],
                                  es == 8 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT64 : CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 4, base,
                                  dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                  CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                                  CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        if (r != CUDA_SUCCESS) return fail(h, RD_CUDA_ERROR, "tensor map of a grid tile");
    }
    return RD_OK;
}

rd_status create_impl(const rd_params* params, int nscenes, rd_handle** out) {
    if (!params || !out || nscenes < 1) return RD_INVALID_ARG;
    *out = nullptr;
    const rd_params& p = params[0];
    int64_t ntot = 0, cells = 0, blocks = 0;
    for (int s = 0; s < nscenes; ++s) {
        const rd_params& q = params[s];
        if (!valid_scene(q)) return RD_INVALID_ARG;
        if (q.precision != p.precision || q.device != p.device || q.lagged_b != p.lagged_b || q.track_fp != p.track_fp)
            return RD_INVALID_ARG;
        ntot += q.num_particles;
        cells += (int64_t)q.max_i * q.max_j * q.max_k;
        blocks += (int64_t)((q.max_i + kBlk - 1) / kBlk) * ((q.max_j + kBlk - 1) / kBlk) * ((q.max_k + kBlk - 1) / kBlk);
    }
    if (nscenes > 1 && p.track_fp) return RD_NOT_SUPPORTED;
    if (ntot >= ((int64_t)1 << 30) || blocks * kCellsPerBlock >= ((int64_t)1 << 31)) return RD_TOO_LARGE;
    rd_handle* h = new (std::nothrow) rd_handle;
    if (!h) return RD_OOM;
    h->prm = p;
    h->scenes.resize(nscenes);
    {
        uint32_t poff = 0, bbase = 0;
        size_t goff = 0;
        for (int s = 0; s < nscenes; ++s) {
            rd_scene_info& sc = h->scenes[s];
            sc.prm = params[s];
            sc.n = params[s].num_particles;
            sc.poff = poff;
            sc.ncells = (size_t)sc.prm.max_i * sc.prm.max_j * sc.prm.max_k;
            sc.goff = goff;
            sc.NB[0] = (sc.prm.max_i + kBlk - 1) / kBlk;
            sc.NB[1] = (sc.prm.max_j + kBlk - 1) / kBlk;
            sc.NB[2] = (sc.prm.max_k + kBlk - 1) / kBlk;
            sc.nblocks = sc.NB[0] * sc.NB[1] * sc.NB[2];
            sc.block_base = bbase;
            poff += (uint32_t)sc.n;
            goff += sc.ncells;
            bbase += (uint32_t)sc.nblocks;
            h->max_scene_cells = std::max(h->max_scene_cells, sc.ncells);
        }
    }
    h->n = (int)ntot;
    h->esize = p.precision == RD_FP64 ? 8 : 4;
    h->planes = p.track_fp ? kPlanesFP : kPlanes;
    h->ncells = (size_t)cells;
    for (int a = 0; a < 3; ++a) h->NB[a] = h->scenes[0].NB[a];
    h->nblocks = (int)blocks;
    h->nkeys = (int)blocks * kCellsPerBlock;
    auto bail = [&](rd_status st) { release(h); delete h; return st; };
    if (cudaSetDevice(p.device) != cudaSuccess) return bail(RD_CUDA_ERROR);
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, p.device) != cudaSuccess) return bail(RD_CUDA_ERROR);
    h->sms = prop.multiProcessorCount;
    if (cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking) != cudaSuccess) return bail(RD_CUDA_ERROR);
    if (cudaStreamCreateWithFlags(&h->side, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_fork, cudaEventDisableTiming) != cudaSuccess ||
        cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming) != cudaSuccess)
        return bail(RD_CUDA_ERROR);
    const size_t n = std::max<size_t>(1, (size_t)h->n);
    const size_t v4 = 4 * h->esize;
    const size_t wp = p.precision == RD_FP64 ? WorkP<double>::value : WorkP<float>::value;
    // items: at most n / wp + one partial item per occupied block; autotuned
    // item sizes go down to wp / 4
    h->work_cap = 4 * (n / wp) + std::min<size_t>((size_t)h->nblocks, n) + 2;
    const size_t psize = p.precision == RD_FP64 ? sizeof(DevParams<double>) : sizeof(DevParams<float>);
    const bool batch = nscenes > 1;
    struct { void** ptr; size_t bytes; bool need; } allocs[] = {
        {&h->pl[0], (size_t)h->planes * n * v4, true},
        {&h->pl[1], (size_t)h->planes * n * v4, true},
        {(void**)&h->keys[0], n * 4, true},
        {(void**)&h->keys[1], n * 4, true},
        {(void**)&h->perm, n * 4, true},
        {(void**)&h->slot_of, n * 4, true},
        {(void**)&h->counts, (size_t)h->nkeys * 4, true},
        {(void**)&h->bcount, (size_t)h->nblocks * 4, true},
        {(void**)&h->gmark[0], (size_t)h->nblocks, true},
        {(void**)&h->gmark[1], (size_t)h->nblocks, true},
        {(void**)&h->cursor, (size_t)h->nkeys * 4, true},
        {(void**)&h->work, h->work_cap * sizeof(int4), true},
        {(void**)&h->nwork2, 6 * sizeof(uint32_t), true},
        {(void**)&h->tile_sums, (size_t)((h->nkeys + kScanTile - 1) / kScanTile + 1) * 4, true},
        {(void**)&h->tile_list, (size_t)((h->nkeys + kScanTile - 1) / kScanTile + 1) * 4, true},
        {&h->grid[0], h->ncells * v4, true},
        {&h->grid[1], h->ncells * v4, true},
        {&h->gforce, h->ncells * v4, !batch},  // stage mode only
        {(void**)&h->flags, 4, true},
        {(void**)&h->xyzs, n * sizeof(float4), true},
        {(void**)&h->rgba, n * sizeof(uint32_t), true},
        {&h->io, align_up(36 * n * h->esize, 256), true},
        {&h->d_scenes, nscenes * psize, batch},
        {(void**)&h->d_sblock, (nscenes + 1) * sizeof(uint32_t), batch},
        {(void**)&h->d_spoff, (nscenes + 1) * sizeof(uint32_t), batch},
        {&h->d_col, RD_MAX_COLLIDERS * sizeof(Collider<double>), !batch},
    };
    for (auto& a : allocs) {
        if (!a.need) continue;
        cudaError_t e = cudaMalloc(a.ptr, a.bytes);
        if (e != cudaSuccess) {
            cudaGetLastError();
            return bail(e == cudaErrorMemoryAllocation ? RD_OOM : RD_CUDA_ERROR);
        }
    }
    if (batch) {
        if (cudaMallocHost(&h->h_scenes, nscenes * psize) != cudaSuccess) return bail(RD_OOM);
        std::vector<uint32_t> sb(nscenes + 1), sp(nscenes + 1);
        for (int s = 0; s < nscenes; ++s) { sb[s] = h->scenes[s].block_base; sp[s] = h->scenes[s].poff; }
        sb[nscenes] = (uint32_t)blocks;
        sp[nscenes] = (uint32_t)ntot;
        // in the handle's stream (a plain cudaMemcpy from pageable memory may
        // return before its data lands, and the handle's streams do not wait
        // for the legacy stream); the creation's final synchronisation covers it
        if (cudaMemcpyAsync(h->d_sblock, sb.data(), sb.size() * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
            cudaMemcpyAsync(h->d_spoff, sp.data(), sp.size() * 4, cudaMemcpyHostToDevice, h->stream) != cudaSuccess ||
            cudaStreamSynchronize(h->stream) != cudaSuccess)
            return bail(RD_CUDA_ERROR);
    }
    cudaMemsetAsync(h->counts, 0, (size_t)h->nkeys * 4, h->stream);
    cudaMemsetAsync(h->bcount, 0, (size_t)h->nblocks * 4, h->stream);
    // both grid buffers start zero and unmarked; from then on only marked
    // blocks are written and cleared
    cudaMemsetAsync(h->grid[0], 0, h->ncells * v4, h->stream);
    cudaMemsetAsync(h->grid[1], 0, h->ncells * v4, h->stream);
    cudaMemsetAsync(h->gmark[0], 0, (size_t)h->nblocks, h->stream);
    cudaMemsetAsync(h->gmark[1], 0, (size_t)h->nblocks, h->stream);
    cudaMemsetAsync(h->perm, 0, n * 4, h->stream);  // every entry is a valid index from the start
    cudaMemsetAsync(h->flags, 0, 4, h->stream);
    cudaMemsetAsync(h->nwork2, 0, 6 * sizeof(uint32_t), h->stream);
    cudaMemsetAsync(h->rgba, 0xff, n * sizeof(uint32_t), h->stream);  // white
    rd_status st = encode_tile_maps(h);
    if (st == RD_OK) st = p.precision == RD_FP64 ? occupancy<double>(h) : occupancy<float>(h);
    if (st != RD_OK) return bail(st);
    if (cudaStreamSynchronize(h->stream) != cudaSuccess) return bail(RD_CUDA_ERROR);
    *out = h;
    return RD_OK;
}

// Replays (capturing first if needed) two steady steps as one CUDA graph.
// Steady: the keys of the current positions are counted, the grid holds
// their P2G for this dt, and the scene table (batches) is current, so the two
// steps are exactly scan, scatter, grid clear and k_g2p2g twice, and leave the
// host-side state as they found it.
template <typename T> rd_status graph_two_steps(rd_handle* h, double dt) {
    const int key = h->cur | (h->g << 1) | (h->nb << 2);
    for (rd_graph& g : h->graphs)
        if (g.key == key && g.dt == dt) {
            RD_TRY(check_cuda(h, cudaGraphLaunch(g.exec, h->stream), "graph launch"));
            h->launches += g.launches;
            ++h->graph_replays;
            return RD_OK;
        }
    if (h->graphs.size() >= 8) drop_graphs(h);
    const uint64_t l0 = h->launches;
    RD_TRY(check_cuda(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture"));
    rd_status s1 = step_fused<T>(h, dt);
    rd_status s2 = s1 == RD_OK ? step_fused<T>(h, dt) : s1;
    cudaGraph_t graph = nullptr;
    const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
    if (s2 != RD_OK || e != cudaSuccess) {
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        h->use_graphs = false;  // eager steps from here on
        return s2 != RD_OK ? s2 : check_cuda(h, e, "end capture");
    }
    rd_graph g;
    g.key = key;
    g.dt = dt;
    g.launches = h->launches - l0;
    const cudaError_t ie = cudaGraphInstantiate(&g.exec, graph, 0);
    cudaGraphDestroy(graph);
    RD_TRY(check_cuda(h, ie, "graph instantiate"));
    h->graphs.push_back(g);
    ++h->graph_replays;
    return check_cuda(h, cudaGraphLaunch(g.exec, h->stream), "graph launch");
}

bool steady(const rd_handle* h, double dt) {
    // the table's force scale is dt in the arithmetic type (ensure_table(h, dt, (T)dt))
    const double fs = h->prm.precision == RD_FP64 ? dt : (double)(float)dt;
    return h->use_graphs && !h->timing && !h->capturing && h->n > 0 && h->keys_valid && !h->sorted && h->fgrid_valid &&
           h->fgrid_dt == dt && h->grid_mode == GRID_FUSED &&
           (!batched(h) || (h->table_valid && h->table_dt == dt && h->table_fs == fs));
}

template <typename T> rd_status steps_impl(rd_handle* h, double dt, int nsteps) {
    NvtxRange range("rd_step");
    for (int s = 0; s < nsteps;) {
        if (nsteps - s >= 2 && steady(h, dt)) {
            RD_TRY(graph_two_steps<T>(h, dt));
            s += 2;
        } else {
            RD_TRY(step_fused<T>(h, dt));
            s += 1;
        }
    }
    return RD_OK;
}

// Tuning cache: a text file of "key<TAB>particles_per_item ctas_per_sm
// scatter ms_per_step" lines; the last line with a key counts.
bool tune_key_ok(const char* key) {
    if (!key || !*key) return false;
    for (const char* c = key; *c; ++c)
        if (*c == '\t' || *c == '\n' || *c == '\r') return false;
    return true;
}

bool tune_cache_find(const char* path, const char* key, rd_tune_result* out) {
    FILE* f = std::fopen(path, "r");
    if (!f) return false;
    const size_t klen = std::strlen(key);
    bool found = false;
    std::string line;
    char buf[512];
    while (std::fgets(buf, sizeof buf, f)) {
        line += buf;
        if (line.back() != '\n' && !std::feof(f)) continue;  // a line longer than the buffer: read on
        if (line.size() > klen && line.compare(0, klen, key) == 0 && line[klen] == '\t') {
            int a = 0, b = 0, c = 0;
            double ms = 0.0;
            char tail = 0;
            const int got = std::sscanf(line.c_str() + klen + 1, "%d %d %d %lf %c", &a, &b, &c, &ms, &tail);
            if (got == 4 && a >= 0 && b >= 0 && (c == RD_SCATTER_LANE_PAIRS || c == RD_SCATTER_RECORD_PAIRS) &&
                std::isfinite(ms)) {
                *out = rd_tune_result{a, b, ms, 0, c, 1};
                found = true;
            }
        }
        line.clear();
    }
    std::fclose(f);
    return found;
}

// Device architecture and SM count, precision, step options, scene count,
// particle count, grid nodes and the largest grid of any scene.
std::string tune_key_of(const rd_handle* h) {
    int major = 0, minor = 0;
    cudaDeviceGetAttribute(&major, cudaDevAttrComputeCapabilityMajor, h->prm.device);
    cudaDeviceGetAttribute(&minor, cudaDevAttrComputeCapabilityMinor, h->prm.device);
    int64_t particles = 0, nodes = 0;
    int gmax[3] = {0, 0, 0};
    const size_t nsc = std::max<size_t>(1, h->scenes.size());
    for (size_t s = 0; s < nsc; ++s) {
        const rd_params& p = h->scenes.empty() ? h->prm : h->scenes[s].prm;
        particles += p.num_particles;
        nodes += (int64_t)p.max_i * p.max_j * p.max_k;
        gmax[0] = std::max(gmax[0], p.max_i);
        gmax[1] = std::max(gmax[1], p.max_j);
        gmax[2] = std::max(gmax[2], p.max_k);
    }
    char buf[256];
    std::snprintf(buf, sizeof buf, "sm%d%d sms%d %s lagged%d trackfp%d scenes%zu particles%lld nodes%lld grid%dx%dx%d",
                  major, minor, h->sms, h->prm.precision == RD_FP64 ? "fp64" : "fp32", h->prm.lagged_b ? 1 : 0,
                  h->prm.track_fp ? 1 : 0, nsc, (long long)particles, (long long)nodes, gmax[0], gmax[1], gmax[2]);
    return buf;
}

// Whether a cached point fits this handle.
template <typename T> bool tune_point_ok(const rd_handle* h, const rd_tune_result& r) {
    const int wmax = WorkP<T>::value;
    return (r.particles_per_item == 0 || (r.particles_per_item >= wmax / 4 && r.particles_per_item <= wmax)) &&
           r.ctas_per_sm <= h->occ_g2p && r.scatter < scatter_layouts(h);
}

// Times the step under each candidate work-item size, persistent grid (CTAs
// per SM) and scatter layout from the same saved state, keeps the fastest and
// puts the state back as it was (the next step re-sorts and rebuilds the grid).
template <typename T> rd_status autotune_impl(rd_handle* h, double dt, int steps, const char* cache_path,
                                              rd_tune_result* res) {
    NvtxRange range("rd_autotune");
    const int wps_f[] = {64, 128, 192, 256}, wps_d[] = {32, 64, 96, 128};
    const int* wps = sizeof(T) == 4 ? wps_f : wps_d;
    rd_tune_result best{WorkP<T>::value, 0, 0.0, 0, RD_SCATTER_LANE_PAIRS, 0};
    h->tune_trials.clear();
    if (h->n == 0) { *res = best; return RD_OK; }
    const std::string key = tune_key_of(h);
    if (cache_path) {
        rd_tune_result hit;
        if (tune_cache_find(cache_path, key.c_str(), &hit) && tune_point_ok<T>(h, hit)) {
            h->wp = hit.particles_per_item;
            h->grid_mult = hit.ctas_per_sm;
            h->scatter = hit.scatter;
            drop_graphs(h);
            *res = hit;
            return RD_OK;
        }
    }
    const size_t bytes = (size_t)h->planes * h->n * 4 * h->esize;
    void* saved = nullptr;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    auto cleanup = [&](rd_status st) {
        cudaStreamSynchronize(h->stream);
        if (saved) cudaFree(saved);
        if (e0) cudaEventDestroy(e0);
        if (e1) cudaEventDestroy(e1);
        return st;
    };
    auto restore = [&]() {
        h->keys_valid = false;
        h->sorted = false;
        h->fgrid_valid = false;
        h->clean_grids = false;
        h->stress_valid = false;
        h->slot_of_valid = false;
        h->grid_mode = GRID_NONE;
        return check_cuda(h, cudaMemcpyAsync(h->pl[h->cur], saved, bytes, cudaMemcpyDeviceToDevice, h->stream),
                          "restore state");
    };
    rd_status st = check_cuda(h, cudaMalloc(&saved, bytes), "autotune state");
    if (st == RD_OK) st = check_cuda(h, cudaEventCreate(&e0), "event");
    if (st == RD_OK) st = check_cuda(h, cudaEventCreate(&e1), "event");
    if (st == RD_OK)
        st = check_cuda(h, cudaMemcpyAsync(saved, h->pl[h->cur], bytes, cudaMemcpyDeviceToDevice, h->stream), "save");
    const int old_wp = h->wp, old_mult = h->grid_mult, old_scatter = h->scatter;
    float best_ms = 0.f;
    for (int l = 0; l < scatter_layouts(h) && st == RD_OK; ++l)
        for (int a = 0; a < 4 && st == RD_OK; ++a)
            for (int c = 1; c <= h->occ_g2p && st == RD_OK; ++c) {
                h->wp = wps[a];
                h->grid_mult = c;
                h->scatter = l;
                drop_graphs(h);
                if ((st = restore()) != RD_OK) break;
                // two eager steps (sort, P2G), then one captured pair, untimed
                if ((st = steps_impl<T>(h, dt, 2)) != RD_OK) break;
                if ((st = steps_impl<T>(h, dt, 2)) != RD_OK) break;
                if ((st = check_cuda(h, cudaEventRecord(e0, h->stream), "event")) != RD_OK) break;
                if ((st = steps_impl<T>(h, dt, steps)) != RD_OK) break;
                if ((st = check_cuda(h, cudaEventRecord(e1, h->stream), "event")) != RD_OK) break;
                if ((st = check_cuda(h, cudaEventSynchronize(e1), "event sync")) != RD_OK) break;
                float ms = 0.f;
                if ((st = check_cuda(h, cudaEventElapsedTime(&ms, e0, e1), "event time")) != RD_OK) break;
                ++best.trials;
                h->tune_trials.push_back(rd_tune_trial{wps[a], c, l, (double)ms / steps});
                if (best.trials == 1 || ms < best_ms) {
                    best_ms = ms;
                    best.particles_per_item = wps[a];
                    best.ctas_per_sm = c;
                    best.scatter = l;
                }
            }
    if (st != RD_OK) {
        h->wp = old_wp;
        h->grid_mult = old_mult;
        h->scatter = old_scatter;
        drop_graphs(h);
        if (saved) restore();
        return cleanup(st);
    }
    h->wp = best.particles_per_item;
    h->grid_mult = best.ctas_per_sm;
    h->scatter = best.scatter;
    best.ms_per_step = best_ms / steps;
    drop_graphs(h);
    st = restore();
    *res = best;
    st = cleanup(st);
    if (st == RD_OK && cache_path && rd_tune_cache_put(cache_path, key.c_str(), &best) != RD_OK)
        st = fail(h, RD_INVALID_ARG, "tuning cache: could not append to the file");
    return st;
}


// ---------------------------------------------------------------- implicit
rd_implicit_opts implicit_defaults() {
    rd_implicit_opts o;
    o.max_iters = 50;
    o.history = 8;
    o.grad_tol = 1e-2;
    o.step_tol = 1e-2;
    o.mu0 = 1.0;
    o.lambda0 = 1.0;
    o.xi = 10.0;
    o.hardening = RD_HARDENING_REFERENCE;
    o.ls_max_iters = 200;
    return o;
}

bool implicit_opts_ok(const rd_implicit_opts& o) {
    return o.max_iters >= 0 && o.history >= 1 && o.history <= 32 && o.grad_tol >= 0 && o.step_tol >= 0 &&
           std::isfinite(o.mu0) && std::isfinite(o.lambda0) && std::isfinite(o.xi) &&
           (o.hardening == RD_HARDENING_REFERENCE || o.hardening == RD_HARDENING_INTENDED) && o.ls_max_iters >= 1;
}

// The solver's view of one call: the cells with mass, the compact vectors and
// the device reductions; every helper runs on the handle's stream.
template <typename T> struct Implicit {
    rd_handle* h;
    DevParams<T> P;
    ImpParams<T> Q;
    int nused = 0, n3 = 0;
    T *vstar = nullptr, *x = nullptr, *g = nullptr, *xold = nullptr, *gold = nullptr, *q = nullptr;
    T* s(int i) const { return static_cast<T*>(h->imp.vec) + (size_t)(6 + i) * 3 * h->imp.cap; }
    T* y(int i) const { return static_cast<T*>(h->imp.vec) + (size_t)(6 + h->imp.hist + i) * 3 * h->imp.cap; }
    int evaluations = 0;
    vec4<T>* grid() const { return static_cast<vec4<T>*>(h->grid[h->g]); }

    unsigned blocks(size_t n) const { return (unsigned)std::min<size_t>(blocks_for(n, 256), (size_t)h->sms * 8); }

    // Finds the cells with mass and sizes the buffers.
    rd_status setup(int hist) {
        rd_implicit_data& m = h->imp;
        const size_t nc = h->ncells;
        if (!m.idx) {
            RD_TRY(check_cuda(h, cudaMalloc(&m.idx, (nc + 1) * sizeof(uint32_t)), "implicit cell list"));
            RD_TRY(check_cuda(h, cudaMalloc(&m.gacc, nc * sizeof(vec4<T>)), "implicit gradient"));
            RD_TRY(check_cuda(h, cudaMalloc(&m.red, 4 * sizeof(double)), "implicit reductions"));
            RD_TRY(check_cuda(h, cudaMallocHost(&m.hred, 4 * sizeof(double)), "implicit reductions"));
        }
        // zero everywhere: particles that moved since the rasterize may reach cells without mass
        RD_TRY(check_cuda(h, cudaMemsetAsync(m.gacc, 0, nc * sizeof(vec4<T>), h->stream), "implicit gradient"));
        RD_TRY(check_cuda(h, cudaMemsetAsync(m.idx + nc, 0, sizeof(uint32_t), h->stream), "implicit count"));
        k_imp_used<T><<<blocks_for(nc, 256), 256, 0, h->stream>>>(grid(), nc, m.idx, m.idx + nc);
        RD_TRY(launched(h, "k_imp_used"));
        uint32_t cnt = 0;
        RD_TRY(check_cuda(h, cudaMemcpyAsync(&cnt, m.idx + nc, sizeof cnt, cudaMemcpyDeviceToHost, h->stream), "count"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "count"));
        nused = (int)cnt;
        n3 = 3 * nused;
        if ((size_t)nused > m.cap || hist > m.hist) {
            if (m.vec) cudaFree(m.vec);
            m.vec = nullptr;
            m.cap = std::max<size_t>({(size_t)nused + nused / 4, m.cap, 1});
            m.hist = std::max(hist, m.hist);
            RD_TRY(check_cuda(h, cudaMalloc(&m.vec, (size_t)(6 + 2 * m.hist) * 3 * m.cap * sizeof(T)),
                              "implicit vectors"));
        }
        T* base = static_cast<T*>(m.vec);
        const size_t stride = 3 * m.cap;
        vstar = base; x = base + stride; g = base + 2 * stride; xold = base + 3 * stride;
        gold = base + 4 * stride; q = base + 5 * stride;
        return RD_OK;
    }

    rd_status fetch(int k, double* out) {
        RD_TRY(check_cuda(h, cudaMemcpyAsync(h->imp.hred, h->imp.red, k * sizeof(double), cudaMemcpyDeviceToHost,
                                             h->stream), "reduction"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "reduction"));
        for (int i = 0; i < k; ++i) out[i] = h->imp.hred[i];
        return RD_OK;
    }

    // E at the trial point xp + a d (d null: xp), written into the grid; with
    // gout, the gradient there too.
    rd_status energy(const T* xp, T a, const T* d, T* gout, double* e) {
        ++evaluations;
        k_imp_put<T><<<blocks_for(nused, 256), 256, 0, h->stream>>>(grid(), h->imp.idx, nused, xp, a, d);
        RD_TRY(launched(h, "k_imp_put"));
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->imp.red, 0, sizeof(double), h->stream), "reduction"));
        const vec4<T>* pl = static_cast<const vec4<T>*>(h->pl[h->cur]);
        vec4<T>* gacc = static_cast<vec4<T>*>(h->imp.gacc);
        if (h->n > 0) {
            if (gout)
                k_imp_particles<T, true><<<blocks_for(h->n, kThreads), kThreads, 0, h->stream>>>(P, Q, pl, grid(), gacc,
                                                                                               h->imp.red);
            else
                k_imp_particles<T, false><<<blocks_for(h->n, kThreads), kThreads, 0, h->stream>>>(P, Q, pl, grid(), gacc,
                                                                                                h->imp.red);
            RD_TRY(launched(h, "k_imp_particles"));
        }
        if (gout)
            k_imp_cells<T, true><<<blocks_for(nused, 256), 256, 0, h->stream>>>(grid(), h->imp.idx, nused, vstar, xp, a,
                                                                               d, gacc, gout, h->imp.red);
        else
            k_imp_cells<T, false><<<blocks_for(nused, 256), 256, 0, h->stream>>>(grid(), h->imp.idx, nused, vstar, xp,
                                                                                a, d, gacc, gout, h->imp.red);
        RD_TRY(launched(h, "k_imp_cells"));
        return fetch(1, e);
    }

    // (a . b, b . b)
    rd_status dot(const T* a, const T* b, double out[2]) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->imp.red, 0, 2 * sizeof(double), h->stream), "reduction"));
        k_imp_dot<T><<<blocks(n3), 256, 0, h->stream>>>(a, b, n3, h->imp.red);
        RD_TRY(launched(h, "k_imp_dot"));
        return fetch(2, out);
    }
    rd_status axpy(T* yv, double a, const T* xv) {
        k_imp_axpy<T><<<blocks(n3), 256, 0, h->stream>>>(yv, (T)a, xv, n3);
        return launched(h, "k_imp_axpy");
    }
    rd_status sub(T* z, const T* a, const T* b) {
        k_imp_sub<T><<<blocks(n3), 256, 0, h->stream>>>(z, a, b, n3);
        return launched(h, "k_imp_sub");
    }
    rd_status copy(T* dst, const T* src) {
        return check_cuda(h, cudaMemcpyAsync(dst, src, (size_t)n3 * sizeof(T), cudaMemcpyDeviceToDevice, h->stream),
                          "copy");
    }
    rd_status absmax(const T* v, double* out) {
        RD_TRY(check_cuda(h, cudaMemsetAsync(h->imp.red, 0, sizeof(double), h->stream), "reduction"));
        k_imp_absmax<T><<<blocks(n3), 256, 0, h->stream>>>(
            v, n3, reinterpret_cast<unsigned long long*>(h->imp.red));
        RD_TRY(launched(h, "k_imp_absmax"));
        return fetch(1, out);
    }
};

template <typename T> rd_status implicit_begin(rd_handle* h, double dt, const rd_implicit_opts& o, Implicit<T>& I) {
    if (batched(h)) return fail(h, RD_NOT_SUPPORTED, "implicit integration drives a single scene");
    if (h->grid_mode != GRID_V)
        return fail(h, RD_INVALID_ARG, "implicit integration needs the stage-mode grid (run the rasterize stage)");
    I.h = h;
    I.P = make_params<T>(h, dt, T(1));
    I.Q = ImpParams<T>{(T)dt, (T)o.mu0, (T)o.lambda0, (T)o.xi, o.hardening == RD_HARDENING_INTENDED ? 1 : 0};
    return I.setup(o.history);
}

// timeIntegration (material_point_method.cpp:212-233): L-BFGS over the
// velocities of the cells with mass (Nocedal & Wright, Numerical
// Optimization, 7.2, as the vendored minimiser implements it: two-loop
// recursion with the scaling s.y / y.y, backtracking Armijo line search,
// steepest descent with a step of min(1, 1 / |g|_inf) whenever the direction
// is not a descent direction).
template <typename T> rd_status time_integration_impl(rd_handle* h, double dt, const rd_implicit_opts& o,
                                                      rd_implicit_result* res) {
    NvtxRange range("rd_time_integration");
    Implicit<T> I;
    RD_TRY(implicit_begin<T>(h, dt, o, I));
    rd_implicit_result r{};
    r.unknowns = I.n3;
    if (I.nused == 0) {
        *res = r;
        return RD_OK;
    }
    k_imp_gather<T><<<blocks_for(I.nused, 256), 256, 0, h->stream>>>(I.grid(), h->imp.idx, I.nused, I.vstar);
    RD_TRY(launched(h, "k_imp_gather"));
    RD_TRY(I.copy(I.x, I.vstar));
    double fx = 0.0;
    RD_TRY(I.energy(I.x, T(0), nullptr, I.g, &fx));
    r.energy_start = fx;
    const int M = o.history;
    std::vector<double> rho(M), alpha(M);
    int npairs = 0, head = 0;  // ring of correction pairs: the newest at (head - 1) mod M
    double gamma = 1.0, alpha_init = 1.0;
    int k = 0;
    r.converged = 0;
    for (; k < o.max_iters; ++k) {
        RD_TRY(I.copy(I.xold, I.x));
        RD_TRY(I.copy(I.gold, I.g));
        RD_TRY(I.copy(I.q, I.g));
        // first loop, newest pair first
        for (int j = npairs - 1; j >= 0; --j) {
            const int c = (head - npairs + j + 2 * M) % M;
            double sy[2], sq[2];
            RD_TRY(I.dot(I.y(c), I.s(c), sy));  // y . s
            rho[j] = 1.0 / sy[0];
            RD_TRY(I.dot(I.q, I.s(c), sq));  // q . s
            alpha[j] = rho[j] * sq[0];
            RD_TRY(I.axpy(I.q, -alpha[j], I.y(c)));
        }
        k_imp_scale<T><<<I.blocks(I.n3), 256, 0, h->stream>>>(I.q, (T)gamma, I.n3);
        RD_TRY(launched(h, "k_imp_scale"));
        for (int j = 0; j < npairs; ++j) {
            const int c = (head - npairs + j + 2 * M) % M;
            double yq[2];
            RD_TRY(I.dot(I.q, I.y(c), yq));
            const double beta = rho[j] * yq[0];
            RD_TRY(I.axpy(I.q, alpha[j] - beta, I.s(c)));
        }
        double qg[2];
        RD_TRY(I.dot(I.g, I.q, qg));  // (g . q, q . q)
        double dir = qg[0];
        if (!(dir > 0.0)) {  // not a descent direction: steepest descent
            RD_TRY(I.copy(I.q, I.g));
            npairs = 0;
            double gmax = 0.0;
            RD_TRY(I.absmax(I.g, &gmax));
            alpha_init = gmax > 0.0 ? std::min(1.0, 1.0 / gmax) : 1.0;
            RD_TRY(I.dot(I.g, I.q, qg));
            dir = qg[0];
        }
        // backtracking along -q from x: f(x - a q) <= f(x) - 1e-4 a (g . q)
        double a = alpha_init, fa = 0.0;
        int ls = 0;
        for (; ls < o.ls_max_iters; ++ls) {
            RD_TRY(I.energy(I.x, (T)(-a), I.q, nullptr, &fa));
            if (fa <= fx - 1e-4 * a * dir) break;
            a *= 0.7;
        }
        if (ls >= o.ls_max_iters) {
            r.converged = -1;
            break;
        }
        RD_TRY(I.axpy(I.x, -a, I.q));
        const double step = a * std::sqrt(qg[1]);
        double gn[2];
        RD_TRY(I.dot(I.g, I.g, gn));
        if (std::sqrt(gn[0]) < o.grad_tol || step < o.step_tol) {  // the gradient before the step, as the reference tests it
            r.converged = 1;
            fx = fa;
            ++k;
            break;
        }
        RD_TRY(I.energy(I.x, T(0), nullptr, I.g, &fx));
        const int c = head;
        RD_TRY(I.sub(I.s(c), I.x, I.xold));
        RD_TRY(I.sub(I.y(c), I.g, I.gold));
        head = (head + 1) % M;
        npairs = std::min(npairs + 1, M);
        double ys[2];
        RD_TRY(I.dot(I.s(c), I.y(c), ys));  // (s . y, y . y)
        if (!(std::abs(ys[1]) > 0.0)) {
            ++k;
            break;
        }
        gamma = ys[0] / ys[1];
        alpha_init = 1.0;
    }
    // the result into the grid, and the energy and gradient there
    RD_TRY(I.energy(I.x, T(0), nullptr, I.g, &fx));
    double gn[2];
    RD_TRY(I.dot(I.g, I.g, gn));
    r.iterations = k;
    r.evaluations = I.evaluations;
    r.energy = fx;
    r.grad_norm = std::sqrt(gn[0]);
    *res = r;
    return RD_OK;
}

template <typename T> rd_status implicit_energy_impl(rd_handle* h, double dt, const rd_implicit_opts& o,
                                                     const void* vel, void* grad, int where, double* energy) {
    Implicit<T> I;
    RD_TRY(implicit_begin<T>(h, dt, o, I));
    const size_t nc = h->ncells;
    // the field in, as the compact trial point (the grid gets it back afterwards)
    const T* dv = static_cast<const T*>(vel);
    T* dense = nullptr;
    rd_status st = check_cuda(h, cudaMalloc(&dense, nc * 3 * sizeof(T)), "implicit field");
    if (st != RD_OK) return st;
    auto done = [&](rd_status s2) {
        cudaStreamSynchronize(h->stream);
        cudaFree(dense);
        return s2;
    };
    if (cudaMemcpyAsync(dense, dv, nc * 3 * sizeof(T), where == RD_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                        h->stream) != cudaSuccess)
        return done(check_cuda(h, cudaGetLastError(), "implicit field"));
    if (I.nused > 0) {
        k_imp_gather<T><<<blocks_for(I.nused, 256), 256, 0, h->stream>>>(I.grid(), h->imp.idx, I.nused, I.vstar);
        if ((st = launched(h, "k_imp_gather")) != RD_OK) return done(st);
        k_imp_take<T><<<blocks_for(I.nused, 256), 256, 0, h->stream>>>(dense, h->imp.idx, I.nused, I.x);
        if ((st = launched(h, "k_imp_take")) != RD_OK) return done(st);
    }
    double e = 0.0;
    st = I.nused > 0 ? I.energy(I.x, T(0), nullptr, grad ? I.g : nullptr, &e) : RD_OK;
    if (st == RD_OK && grad) {
        if ((st = check_cuda(h, cudaMemsetAsync(dense, 0, nc * 3 * sizeof(T), h->stream), "gradient")) == RD_OK &&
            I.nused > 0) {
            k_imp_spread<T><<<blocks_for(I.nused, 256), 256, 0, h->stream>>>(dense, h->imp.idx, I.nused, I.g);
            st = launched(h, "k_imp_spread");
        }
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(grad, dense, nc * 3 * sizeof(T),
                                               where == RD_HOST ? cudaMemcpyDeviceToHost : cudaMemcpyDeviceToDevice,
                                               h->stream), "gradient out");
    }
    // the grid's own velocities back
    if (st == RD_OK && I.nused > 0) {
        k_imp_put<T><<<blocks_for(I.nused, 256), 256, 0, h->stream>>>(I.grid(), h->imp.idx, I.nused, I.vstar, T(0),
                                                                     nullptr);
        st = launched(h, "k_imp_put");
    }
    *energy = e;
    return done(st);
}

// ---------------------------------------------------------------- adjoint
template <typename T> rd_status adj_occupancy(rd_handle* h) {
    const int sg = (int)sizeof(AdjG2PShared<T>), sp = (int)sizeof(AdjP2GShared<T>);
    const void* g2p[] = {(const void*)k_adj_g2p<T, false>, (const void*)k_adj_g2p<T, true>};
    const void* p2g[] = {(const void*)k_adj_p2g<T, false>, (const void*)k_adj_p2g<T, true>};
    for (const void* f : g2p)
        RD_TRY(check_cuda(h, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, sg), "smem attr"));
    for (const void* f : p2g)
        RD_TRY(check_cuda(h, cudaFuncSetAttribute(f, cudaFuncAttributeMaxDynamicSharedMemorySize, sp), "smem attr"));
    int o = 0;
    RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_adj_g2p<T, false>, kAdjThreads, sg), "occ"));
    h->adj.occ_g2p = std::max(1, o);
    RD_TRY(check_cuda(h, cudaOccupancyMaxActiveBlocksPerMultiprocessor(&o, k_adj_p2g<T, false>, kAdjThreads, sp), "occ"));
    h->adj.occ_p2g = std::max(1, o);
    return RD_OK;
}

rd_status adj_alloc(rd_handle* h, int steps, int every) {
    rd_adjoint_data& a = h->adj;
    const size_t n = std::max<size_t>(1, (size_t)h->n);
    a.state_bytes = (size_t)h->planes * n * 4 * h->esize;
    a.grid_bytes = h->ncells * 4 * h->esize;
    a.split_bytes = (size_t)kSplitPlanes * n * 4 * h->esize;
    const size_t nckpt = (size_t)((steps + every - 1) / every), nseg = (size_t)every;
    auto grow = [&](void** ptr, size_t bytes) -> rd_status {
        drop_graphs(h);  // a captured sweep holds the old pointers
        if (*ptr) cudaFree(*ptr);
        *ptr = nullptr;
        return check_cuda(h, cudaMalloc(ptr, bytes), "adjoint buffers");
    };
    if (a.nckpt < nckpt) {
        RD_TRY(grow(&a.ckpt, nckpt * a.state_bytes));
        a.nckpt = nckpt;
    }
    if (a.nseg < nseg) {
        for (int b = 0; b < 2; ++b) {
            RD_TRY(grow(&a.sstore[b], (nseg + 1) * a.state_bytes));  // slot len: the state after the segment
            RD_TRY(grow(&a.gstore[b], nseg * a.grid_bytes));
            RD_TRY(grow((void**)&a.sperm[b], nseg * n * sizeof(uint32_t)));
            RD_TRY(grow((void**)&a.swork[b], nseg * h->work_cap * sizeof(int4)));
            RD_TRY(grow((void**)&a.snwork[b], 2 * nseg * sizeof(uint32_t)));
            RD_TRY(grow(&a.ssplit[b], nseg * a.split_bytes));
        }
        a.nseg = nseg;
    }
    if (!a.final_state) {
        RD_TRY(check_cuda(h, cudaStreamCreateWithFlags(&a.stream2, cudaStreamNonBlocking), "adjoint stream"));
        cudaEvent_t* evs[] = {&a.ev_fork, &a.ev_join, &a.ev_rec[0], &a.ev_rec[1], &a.ev_rev[0], &a.ev_rev[1]};
        for (cudaEvent_t* e : evs)
            RD_TRY(check_cuda(h, cudaEventCreateWithFlags(e, cudaEventDisableTiming), "adjoint events"));
        RD_TRY(check_cuda(h, cudaMalloc(&a.final_state, a.state_bytes), "adjoint buffers"));
        for (int k = 0; k < 3; ++k)
            RD_TRY(check_cuda(h, cudaMalloc(&a.adj[k], (size_t)kAdjPlanes * 4 * n * h->esize), "adjoint buffers"));
        RD_TRY(check_cuda(h, cudaMalloc(&a.agrid, a.grid_bytes), "adjoint buffers"));
        RD_TRY(check_cuda(h, cudaMalloc((void**)&a.pacc, kAccPerScene * n * sizeof(double)), "adjoint buffers"));
        RD_TRY(check_cuda(h, cudaMalloc((void**)&a.acc, kAccPerScene * h->scenes.size() * sizeof(double)),
                          "adjoint buffers"));
        RD_TRY(h->prm.precision == RD_FP64 ? adj_occupancy<double>(h) : adj_occupancy<float>(h));
    }
    return RD_OK;
}

inline char* at(void* base, size_t i, size_t bytes) { return static_cast<char*>(base) + i * bytes; }

// `len` forward steps with the segment store as the particle buffers: step j
// reads its state from slot j and writes the next one to slot j + 1 (slot 0
// must hold the first state), sorts into slot j of the sort store, and its
// grid is copied to slot j of the grid store.  The handle's own particle and
// sort buffers are left alone; slot len ends up holding the state after the
// segment.
template <typename T> rd_status stored_segment(rd_handle* h, double dt, int len, int b) {
    rd_adjoint_data& a = h->adj;
    const size_t n = (size_t)h->n;
    void* const pl0 = h->pl[0];
    void* const pl1 = h->pl[1];
    uint32_t* const perm0 = h->perm;
    int4* const work0 = h->work;
    rd_status st = RD_OK;
    for (int j = 0; j < len && st == RD_OK; ++j) {
        h->pl[h->cur] = at(a.sstore[b], (size_t)j, a.state_bytes);
        h->pl[h->cur ^ 1] = at(a.sstore[b], (size_t)j + 1, a.state_bytes);
        h->perm = a.sperm[b] + (size_t)j * n;
        h->work = a.swork[b] + (size_t)j * h->work_cap;
        h->split_out = at(a.ssplit[b], (size_t)j, a.split_bytes);
        st = step_fused<T>(h, dt);
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(at(a.gstore[b], (size_t)j, a.grid_bytes), h->grid[h->g ^ 1], a.grid_bytes,
                                               cudaMemcpyDeviceToDevice, h->stream),
                            "segment grid");
        // the step's list counts, front and back
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(a.snwork[b] + 2 * j, h->nwork2 + h->nb, sizeof(uint32_t),
                                               cudaMemcpyDeviceToDevice, h->stream),
                            "segment sort");
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(a.snwork[b] + 2 * j + 1, h->nwork2 + 2 + h->nb, sizeof(uint32_t),
                                               cudaMemcpyDeviceToDevice, h->stream),
                            "segment sort");
    }
    h->pl[0] = pl0;
    h->pl[1] = pl1;
    h->perm = perm0;
    h->work = work0;
    h->split_out = nullptr;
    return st;
}

// Copies `src` into slot 0 of the segment store as a fresh state (no sort, no grid).
rd_status begin_segment(rd_handle* h, const void* src, int b) {
    rd_adjoint_data& a = h->adj;
    RD_TRY(check_cuda(h, cudaMemcpyAsync(a.sstore[b], src, a.state_bytes, cudaMemcpyDeviceToDevice, h->stream),
                      "segment start"));
    h->keys_valid = false;
    h->sorted = false;
    h->fgrid_valid = false;
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    h->grid_mode = GRID_NONE;
    return RD_OK;
}

// The record: checkpoints every `every` steps, the last segment straight into
// the segment store, the final state kept.  Enqueues work only.
template <typename T> rd_status record_body(rd_handle* h, double dt, int steps, int every) {
    rd_adjoint_data& a = h->adj;
    a.tail_valid = false;
    for (int s = 0; s < steps; s += every) {
        RD_TRY(check_cuda(h, cudaMemcpyAsync(at(a.ckpt, (size_t)(s / every), a.state_bytes), h->pl[h->cur],
                                             a.state_bytes, cudaMemcpyDeviceToDevice, h->stream),
                          "checkpoint"));
        const int len = std::min(every, steps - s);
        if (s + every >= steps && h->n > 0) {  // the last segment goes straight into its store
            const int b = (s / every) & 1;
            a.tail_store = b;
            RD_TRY(begin_segment(h, h->pl[h->cur], b));
            RD_TRY(stored_segment<T>(h, dt, len, b));
            // the handle holds the final state again
            RD_TRY(check_cuda(h, cudaMemcpyAsync(h->pl[h->cur], at(a.sstore[b], (size_t)len, a.state_bytes), a.state_bytes,
                                                 cudaMemcpyDeviceToDevice, h->stream),
                              "final state"));
            h->keys_valid = false;
            h->sorted = false;
            h->fgrid_valid = false;
            h->clean_grids = false;
            h->stress_valid = false;
            h->slot_of_valid = false;
            h->grid_mode = GRID_NONE;
            a.tail_valid = true;
        } else {
            RD_TRY(steps_impl<T>(h, dt, len));
        }
    }
    return check_cuda(h, cudaMemcpyAsync(a.final_state, h->pl[h->cur], a.state_bytes, cudaMemcpyDeviceToDevice,
                                         h->stream),
                      "final state");
}

// Host-side step state (buffer assignment and validity flags) packed in an int.
int host_state(const rd_handle* h, double dt) {
    return h->cur | (h->g << 1) | (h->nb << 2) | (h->keys_valid << 3) | (h->sorted << 4) |
           ((h->fgrid_valid && h->fgrid_dt == dt) << 5) | (h->grid_mode << 6);
}
void set_host_state(rd_handle* h, int s, double dt) {
    h->cur = s & 1;
    h->g = (s >> 1) & 1;
    h->nb = (s >> 2) & 1;
    h->keys_valid = (s >> 3) & 1;
    h->sorted = (s >> 4) & 1;
    h->fgrid_valid = (s >> 5) & 1;
    h->fgrid_dt = dt;
    h->grid_mode = (s >> 6) & 3;
    h->last_dt = dt;
}

template <typename T> rd_status adjoint_record_impl(rd_handle* h, double dt, int steps, int every) {
    NvtxRange range("rd_adjoint_record");
    RD_TRY(adj_alloc(h, steps, every));
    rd_adjoint_data& a = h->adj;
    a.recorded = false;
    if (batched(h)) RD_TRY(ensure_table<T>(h, dt, (T)dt));  // no synchronisation inside a capture
    if (!h->use_graphs || h->timing || h->n == 0) {
        RD_TRY(record_body<T>(h, dt, steps, every));
    } else {
        const int key = host_state(h, dt);
        const bool hit = a.record && a.rec_key == key && a.rec_dt == dt && a.rec_steps == steps &&
                         a.rec_every == every && a.rec_wp == h->wp && a.rec_mult == h->grid_mult;
        if (!hit) {
            if (a.record) cudaGraphExecDestroy(a.record);
            a.record = nullptr;
            const uint64_t l0 = h->launches;
            RD_TRY(check_cuda(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture"));
            h->capturing = true;
            const rd_status st = record_body<T>(h, dt, steps, every);
            h->capturing = false;
            cudaGraph_t graph = nullptr;
            const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
            if (st != RD_OK || e != cudaSuccess) {
                if (graph) cudaGraphDestroy(graph);
                cudaGetLastError();
                return st != RD_OK ? st : check_cuda(h, e, "end capture");
            }
            const cudaError_t ie = cudaGraphInstantiate(&a.record, graph, 0);
            cudaGraphDestroy(graph);
            RD_TRY(check_cuda(h, ie, "graph instantiate"));
            a.rec_key = key;
            a.rec_end = host_state(h, dt);
            a.rec_dt = dt;
            a.rec_steps = steps;
            a.rec_every = every;
            a.rec_wp = h->wp;
            a.rec_mult = h->grid_mult;
            a.rec_launches = h->launches - l0;
        } else {
            set_host_state(h, a.rec_end, dt);
            h->launches += a.rec_launches;
            a.tail_valid = h->n > 0;
            a.tail_store = (((steps + every - 1) / every) - 1) & 1;
        }
        RD_TRY(check_cuda(h, cudaGraphLaunch(a.record, h->stream), "graph launch"));
    }
    a.recorded = true;
    a.dt = dt;
    a.steps = steps;
    a.every = every;
    a.version = h->version;
    return RD_OK;
}

template <typename T> AdjState<T> adj_view(rd_handle* h, int k) {
    return AdjState<T>{static_cast<vec4<T>*>(h->adj.adj[k]), (size_t)h->n};
}

// Puts the handle's state back to `src` (a stored state) for the next step.
rd_status load_state(rd_handle* h, const void* src, size_t bytes) {
    RD_TRY(check_cuda(h, cudaMemcpyAsync(h->pl[h->cur], src, bytes, cudaMemcpyDeviceToDevice, h->stream), "restore"));
    h->keys_valid = false;
    h->sorted = false;
    h->fgrid_valid = false;
    h->clean_grids = false;
    h->stress_valid = false;
    h->slot_of_valid = false;
    h->grid_mode = GRID_NONE;
    return RD_OK;
}

// The reverse sweep over all segments, last to first; nxt is the adjoint
// buffer holding the adjoint of the final state on entry.  Ends with the
// final state back in the handle.  Enqueues work only (capturable).
// Segment k uses store k & 1: the handle's stream recomputes a segment into
// its store while the second stream runs the reverse kernels of the segment
// after it from the other store; events order each store's reuse.
template <typename T> rd_status adjoint_sweep(rd_handle* h, int nxt) {
    rd_adjoint_data& a = h->adj;
    const size_t n = (size_t)h->n;
    const double dt = a.dt;
    const bool batch = batched(h);
    const int nseg = (a.steps + a.every - 1) / a.every;
    const bool two = !h->timing && a.stream2;  // per-kernel event timing runs on the handle's stream only
    cudaStream_t rs = two ? a.stream2 : h->stream;
    if (two) {  // the reverse stream follows everything queued so far (and joins a capture)
        RD_TRY(check_cuda(h, cudaEventRecord(a.ev_fork, h->stream), "event"));
        RD_TRY(check_cuda(h, cudaStreamWaitEvent(rs, a.ev_fork, 0), "event"));
    }
    for (int seg = nseg - 1; seg >= 0 && n; --seg) {
        const int c = seg * a.every, len = std::min(a.every, a.steps - c);
        const int b = (seg == nseg - 1 && a.tail_valid) ? a.tail_store : (seg & 1);
        if (!(seg == nseg - 1 && a.tail_valid)) {  // recompute the segment into store b
            if (two && seg + 2 <= nseg - 1)        // once the reverse of segment seg + 2 is done with it
                RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->stream, a.ev_rev[b], 0), "event"));
            RD_TRY(begin_segment(h, at(a.ckpt, (size_t)seg, a.state_bytes), b));
            RD_TRY(stored_segment<T>(h, dt, len, b));
        }
        if (two) {
            RD_TRY(check_cuda(h, cudaEventRecord(a.ev_rec[b], h->stream), "event"));
            RD_TRY(check_cuda(h, cudaStreamWaitEvent(rs, a.ev_rec[b], 0), "event"));
        }
        // slot len holds the state after the segment, in this pass's slot
        // order: bring the adjoint of that state into the same order
        const vec4<T>* after = reinterpret_cast<const vec4<T>*>(at(a.sstore[b], (size_t)len, a.state_bytes));
        const unsigned nb256 = blocks_for(n, 256);
        if (seg == nseg - 1) {  // dL/dx, dL/dv of the final state (staged in adj[2] by id)
            const T* gx = static_cast<const T*>(a.adj[2]);  // staged by particle id (adjoint_backward_impl)
            k_adj_seed<T><<<nb256, 256, 0, rs>>>((int)n, after, gx, gx + 3 * n, adj_view<T>(h, nxt));
            RD_TRY(launched(h, "k_adj_seed"));
        } else {  // from the order of the next segment's checkpoint
            const vec4<T>* ck = reinterpret_cast<const vec4<T>*>(at(a.ckpt, (size_t)seg + 1, a.state_bytes));
            k_adj_to_id<T><<<nb256, 256, 0, rs>>>((int)n, ck, adj_view<T>(h, nxt), adj_view<T>(h, 2));
            k_adj_from_id<T><<<nb256, 256, 0, rs>>>((int)n, after, adj_view<T>(h, 2), adj_view<T>(h, nxt));
            RD_TRY(launched(h, "k_adj_remap", 2));
        }
        const DevParams<T> P = make_params<T>(h, dt, (T)dt);
        const size_t max_items = n / WorkP<T>::value + std::min<size_t>((size_t)h->nblocks, n) + 1;
        const unsigned gg = (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)h->sms * a.occ_g2p));
        const unsigned gp = (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)h->sms * a.occ_p2g));
        const size_t sg = sizeof(AdjG2PShared<T>), sp = sizeof(AdjP2GShared<T>);
        for (int j = len - 1; j >= 0; --j) {
            const int cur = nxt ^ 1;
            const vec4<T>* st = reinterpret_cast<const vec4<T>*>(at(a.sstore[b], (size_t)j, a.state_bytes));
            const vec4<T>* gr = reinterpret_cast<const vec4<T>*>(at(a.gstore[b], (size_t)j, a.grid_bytes));
            const vec4<T>* spl = reinterpret_cast<const vec4<T>*>(at(a.ssplit[b], (size_t)j, a.split_bytes));
            // the split of step j - 1 is F of state j (none kept for a segment's first step)
            const vec4<T>* spl_prev =
                j > 0 ? reinterpret_cast<const vec4<T>*>(at(a.ssplit[b], (size_t)j - 1, a.split_bytes)) : nullptr;
            vec4<T>* ag = static_cast<vec4<T>*>(a.agrid);
            DevBufs D = bufs<T>(h);
            D.perm = a.sperm[b] + (size_t)j * n;
            D.work = a.swork[b] + (size_t)j * h->work_cap;
            D.nwork = a.snwork[b] + 2 * j;
            D.nwork_back = a.snwork[b] + 2 * j + 1;
            RD_TRY(check_cuda(h, cudaMemsetAsync(a.agrid, 0, a.grid_bytes, rs), "adjoint grid"));
            const AdjState<T> An = adj_view<T>(h, nxt), Ap = adj_view<T>(h, 2), Ac = adj_view<T>(h, cur);
            long t = tmark_begin(h, RD_KERNEL_ADJ_G2P);
            if (batch)
                k_adj_g2p<T, true><<<gg, kAdjThreads, sg, rs>>>(P, D, st, gr, ag, An, Ap, a.pacc, spl);
            else
                k_adj_g2p<T, false><<<gg, kAdjThreads, sg, rs>>>(P, D, st, gr, ag, An, Ap, a.pacc, spl);
            tmark_end(h, t);
            t = tmark_begin(h, RD_KERNEL_ADJ_P2G);
            if (batch)
                k_adj_p2g<T, true><<<gp, kAdjThreads, sp, rs>>>(P, D, st, gr, ag, Ap, Ac, a.pacc, spl_prev);
            else
                k_adj_p2g<T, false><<<gp, kAdjThreads, sp, rs>>>(P, D, st, gr, ag, Ap, Ac, a.pacc, spl_prev);
            tmark_end(h, t);
            RD_TRY(launched(h, "adjoint step", 2));
            nxt = cur;
        }
        if (two) RD_TRY(check_cuda(h, cudaEventRecord(a.ev_rev[b], rs), "event"));
    }
    if (two) {  // the handle's stream waits for the reverse kernels
        RD_TRY(check_cuda(h, cudaEventRecord(a.ev_join, rs), "event"));
        RD_TRY(check_cuda(h, cudaStreamWaitEvent(h->stream, a.ev_join, 0), "event"));
    }
    return load_state(h, a.final_state, a.state_bytes);
}

// adjoint_sweep through a cached CUDA graph (captured on first use).  The
// ping-pong assignment the sweep ends in is part of the cache entry.
template <typename T> rd_status sweep_graph(rd_handle* h) {
    rd_adjoint_data& a = h->adj;
    const int key = (h->cur | (h->g << 1) | (h->nb << 2)) + (a.tail_valid ? 8 : 0);
    const bool hit = a.sweep && a.sweep_key == key && a.sweep_dt == a.dt && a.sweep_steps == a.steps &&
                     a.sweep_every == a.every && a.sweep_wp == h->wp && a.sweep_mult == h->grid_mult;
    if (!hit) {
        if (a.sweep) cudaGraphExecDestroy(a.sweep);
        a.sweep = nullptr;
        const uint64_t l0 = h->launches;
        RD_TRY(check_cuda(h, cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal), "begin capture"));
        const rd_status st = adjoint_sweep<T>(h, 1);
        cudaGraph_t graph = nullptr;
        const cudaError_t e = cudaStreamEndCapture(h->stream, &graph);
        if (st != RD_OK || e != cudaSuccess) {
            if (graph) cudaGraphDestroy(graph);
            cudaGetLastError();
            return st != RD_OK ? st : check_cuda(h, e, "end capture");
        }
        const cudaError_t ie = cudaGraphInstantiate(&a.sweep, graph, 0);
        cudaGraphDestroy(graph);
        RD_TRY(check_cuda(h, ie, "graph instantiate"));
        a.sweep_key = key;
        a.sweep_end = h->cur | (h->g << 1) | (h->nb << 2);
        a.sweep_dt = a.dt;
        a.sweep_steps = a.steps;
        a.sweep_every = a.every;
        a.sweep_wp = h->wp;
        a.sweep_mult = h->grid_mult;
        a.sweep_launches = h->launches - l0;
    } else {
        // the host-side state the sweep leaves behind
        h->cur = a.sweep_end & 1;
        h->g = (a.sweep_end >> 1) & 1;
        h->nb = (a.sweep_end >> 2) & 1;
        h->launches += a.sweep_launches;
        h->keys_valid = false;
        h->sorted = false;
        h->fgrid_valid = false;
        h->clean_grids = false;
        h->stress_valid = false;
        h->slot_of_valid = false;
        h->grid_mode = GRID_NONE;
        h->last_dt = a.dt;
    }
    return check_cuda(h, cudaGraphLaunch(a.sweep, h->stream), "graph launch");
}

template <typename T>
rd_status adjoint_backward_impl(rd_handle* h, const void* grad_x, const void* grad_v, int where, rd_grads* out) {
    NvtxRange range("rd_adjoint_backward");
    rd_adjoint_data& a = h->adj;
    const size_t n = (size_t)h->n;
    const bool batch = batched(h);
    const cudaMemcpyKind kin = where == RD_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice;
    int nxt = 1;
    if (n) {  // dL/dx, dL/dv of the final state by particle id (n x 3 each), staged in the
              // scratch adjoint for the sweep's seed
        T* sx = static_cast<T*>(a.adj[2]);
        T* sv = sx + 3 * n;
        if (grad_x) RD_TRY(check_cuda(h, cudaMemcpyAsync(sx, grad_x, 3 * n * sizeof(T), kin, h->stream), "adjoint seed"));
        else RD_TRY(check_cuda(h, cudaMemsetAsync(sx, 0, 3 * n * sizeof(T), h->stream), "adjoint seed"));
        if (grad_v) RD_TRY(check_cuda(h, cudaMemcpyAsync(sv, grad_v, 3 * n * sizeof(T), kin, h->stream), "adjoint seed"));
        else RD_TRY(check_cuda(h, cudaMemsetAsync(sv, 0, 3 * n * sizeof(T), h->stream), "adjoint seed"));
    }
    RD_TRY(check_cuda(h, cudaMemsetAsync(a.pacc, 0, kAccPerScene * std::max<size_t>(n, 1) * sizeof(double), h->stream),
                      "adjoint acc"));
    if (n) {
        if (h->use_graphs && !h->timing)
            RD_TRY(sweep_graph<T>(h));
        else
            RD_TRY(adjoint_sweep<T>(h, 1));
        // the store now holds the first segment unless there was only one
        a.tail_valid = a.tail_valid && a.steps <= a.every;
    }
    nxt = 1 ^ (a.steps & 1);  // the buffer the sweep left the start state's adjoint in
    k_reduce_acc<<<(unsigned)h->scenes.size(), 256, 0, h->stream>>>(a.pacc, batch ? h->d_spoff : nullptr,
                                                                   (int)h->scenes.size(), h->n, a.acc);
    RD_TRY(launched(h, "k_reduce_acc"));
    if (out && out->v0 && n) {  // dL/dv of the start state (checkpoint 0) in particle id order
        T* dst = where == RD_HOST ? static_cast<T*>(a.adj[2]) : static_cast<T*>(out->v0);
        k_adj_out<T><<<blocks_for(n, 256), 256, 0, h->stream>>>((int)n, static_cast<const vec4<T>*>(a.ckpt),
                                                                 adj_view<T>(h, nxt), dst);
        RD_TRY(launched(h, "k_adj_out"));
        if (where == RD_HOST)
            RD_TRY(check_cuda(h, cudaMemcpyAsync(out->v0, dst, 3 * n * sizeof(T), cudaMemcpyDeviceToHost, h->stream),
                              "v0 gradient"));
    }
    std::vector<double> acc(kAccPerScene * h->scenes.size());
    RD_TRY(check_cuda(h, cudaMemcpyAsync(acc.data(), a.acc, acc.size() * sizeof(double), cudaMemcpyDeviceToHost,
                                         h->stream),
                      "parameter gradients"));
    if (!n) RD_TRY(load_state(h, a.final_state, a.state_bytes));
    RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    if (out) {
        for (size_t s = 0; s < h->scenes.size(); ++s) {
            const double E = h->scenes[s].prm.E, nu = h->scenes[s].prm.nu;
            const double mub = acc[kAccPerScene * s], lamb = acc[kAccPerScene * s + 1];
            const double den = (1.0 + nu) * (1.0 - 2.0 * nu);
            // mu0 = E / (2 (1 + nu)), lambda0 = E nu / ((1 + nu)(1 - 2 nu))
            if (out->E) out->E[s] = mub / (2.0 * (1.0 + nu)) + lamb * nu / den;
            if (out->nu) out->nu[s] = -mub * E / (2.0 * (1.0 + nu) * (1.0 + nu)) + lamb * E * (1.0 + 2.0 * nu * nu) / (den * den);
            if (out->theta_c) out->theta_c[s] = acc[kAccPerScene * s + 2];
            if (out->theta_s) out->theta_s[s] = acc[kAccPerScene * s + 3];
        }
    }
    return RD_OK;
}

// World-from-box rotation of a unit quaternion (w, x, y, z), row-major
// (glm::mat3_cast); translation, half extents and velocity as they are.
template <typename T> Collider<T> device_collider(const rd_collider& c) {
    double w = c.rotation[0], x = c.rotation[1], y = c.rotation[2], z = c.rotation[3];
    const double nn = std::sqrt(w * w + x * x + y * y + z * z);
    if (nn > 0) { w /= nn; x /= nn; y /= nn; z /= nn; }
    const double R[9] = {1 - 2 * (y * y + z * z), 2 * (x * y - w * z),     2 * (x * z + w * y),
                         2 * (x * y + w * z),     1 - 2 * (x * x + z * z), 2 * (y * z - w * x),
                         2 * (x * z - w * y),     2 * (y * z + w * x),     1 - 2 * (x * x + y * y)};
    Collider<T> d{};
    for (int e = 0; e < 9; ++e) d.R[e] = (T)R[e];
    for (int a = 0; a < 3; ++a) {
        d.t[a] = (T)c.translation[a];
        d.s[a] = (T)c.scale[a];
        d.v[a] = (T)c.velocity[a];
    }
    return d;
}

template <typename T> rd_status upload_colliders(rd_handle* h) {
    std::vector<Collider<T>> d(h->cols.size());
    for (size_t k = 0; k < d.size(); ++k) d[k] = device_collider<T>(h->cols[k]);
    // the previous set may still be read by queued steps
    RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    // in stream order with the steps that read them (a plain cudaMemcpy from
    // pageable memory may return before its data lands)
    if (!d.empty()) {
        RD_TRY(check_cuda(h, cudaMemcpyAsync(h->d_col, d.data(), d.size() * sizeof(Collider<T>), cudaMemcpyHostToDevice,
                                             h->stream),
                          "colliders"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    }
    return RD_OK;
}

// MeshCollider::move on the device, in stream order with the steps.
template <typename T> __global__ void k_move_colliders(Collider<T>* cols, int n, T dt) {
    const int k = threadIdx.x;
    if (k >= n) return;
#pragma unroll
    for (int a = 0; a < 3; ++a) cols[k].t[a] += dt * cols[k].v[a];
}

template <typename T> rd_status move_colliders_impl(rd_handle* h, double dt) {
    for (rd_collider& c : h->cols)
        for (int a = 0; a < 3; ++a) c.translation[a] += dt * c.velocity[a];
    if (h->cols.empty()) return RD_OK;
    k_move_colliders<T><<<1, RD_MAX_COLLIDERS, 0, h->stream>>>(static_cast<Collider<T>*>(h->d_col),
                                                               (int)h->cols.size(), (T)dt);
    return launched(h, "k_move_colliders");
}

template <typename T> rd_status initialize_impl(rd_handle* h, const rd_init_spec& sp, int32_t* need_more) {
    const int n = h->n;
    InitSpec S{};
    const float hh = (float)h->prm.h;
    for (int a = 0; a < 3; ++a) { S.origin[a] = (float)sp.origin[a]; S.vel[a] = (float)sp.velocity[a]; }
    S.width = (float)sp.radius;
    S.mass = (float)sp.mass;
    S.h = hh;
    S.seed = sp.seed;
    // glm::ivec3(particlesOrigin / h), int(width / h), in float as the reference
    volatile float ox = S.origin[0] / hh, oy = S.origin[1] / hh, oz = S.origin[2] / hh, wc = S.width / hh;
    S.cx = (int)ox; S.cy = (int)oy; S.cz = (int)oz; S.wic = (int)wc;
    if (S.wic < 0 || S.wic > 4096) return fail(h, RD_INVALID_ARG, "radius out of range");
    vec4<T>* pl = static_cast<vec4<T>*>(h->pl[h->cur]);
    int more = 0;
    int* d_more = nullptr;
    uint32_t* chunk = nullptr;
    auto cleanup = [&](rd_status st) {
        if (d_more) cudaFree(d_more);
        if (chunk) cudaFree(chunk);
        return st;
    };
    rd_status st = RD_OK;
    if (n > 0) {
        k_init_defaults<T><<<blocks_for(n, 256), 256, 0, h->stream>>>(S, n, pl);
        st = launched(h, "k_init_defaults");
    }
    if (st == RD_OK && sp.mode == RD_INIT_REFERENCE) {
        st = check_cuda(h, cudaMalloc((void**)&d_more, sizeof(int)), "init");
        if (st == RD_OK) {
            k_init_reference<T><<<1, 32, 0, h->stream>>>(S, n, pl, d_more);
            st = launched(h, "k_init_reference");
        }
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(&more, d_more, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "init");
    } else if (st == RD_OK) {
        const uint64_t side = 2 * (uint64_t)S.wic;
        const uint64_t ncand = side * side * side * 8;
        if (ncand >= ((uint64_t)1 << 31)) return cleanup(fail(h, RD_TOO_LARGE, "too many candidate points"));
        const unsigned nchunks = (unsigned)std::max<uint64_t>(1, (ncand + 1023) / 1024);
        st = check_cuda(h, cudaMalloc((void**)&chunk, (nchunks + 3) * sizeof(uint32_t)), "init");
        if (st == RD_OK) {
            uint32_t* scratch = chunk + nchunks + 1;  // item counter and flags of k_tile_prefix, unused here
            k_init_count<<<nchunks, 1024, 0, h->stream>>>(S, (uint32_t)ncand, chunk);
            k_tile_prefix<<<1, 1024, 0, h->stream>>>(chunk, (int)nchunks, scratch, 0u, scratch + 1, nullptr);
            k_init_place<T><<<nchunks, 1024, 0, h->stream>>>(S, (uint32_t)ncand, chunk, n, pl);
            st = launched(h, "k_init", 3);
        }
        uint32_t kept = 0;
        if (st == RD_OK)
            st = check_cuda(h, cudaMemcpyAsync(&kept, chunk + nchunks, sizeof(uint32_t), cudaMemcpyDeviceToHost,
                                               h->stream),
                            "init");
        if (st == RD_OK) st = check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
        more = (int)std::max<int64_t>(0, (int64_t)kept - n);
    }
    if (st == RD_OK) st = check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
    if (st == RD_OK) {
        if (need_more) *need_more = more;
        h->scenes[0].set = true;
        h->keys_valid = false;
        h->sorted = false;
        h->fgrid_valid = false;
        h->clean_grids = false;
        h->stress_valid = false;
        h->slot_of_valid = false;
        h->grid_mode = GRID_NONE;
    }
    return cleanup(st);
}

template <typename T> rd_status diagnostics_impl(rd_handle* h, int scene, rd_diagnostics* out) {
    const rd_scene_info& sc = h->scenes[scene];
    double* acc = nullptr;
    RD_TRY(check_cuda(h, cudaMalloc((void**)&acc, 20 * sizeof(double)), "diagnostics"));
    auto done = [&](rd_status st) { cudaFree(acc); return st; };
    rd_status st = check_cuda(h, cudaMemsetAsync(acc, 0, 20 * sizeof(double), h->stream), "diagnostics");
    if (st == RD_OK && sc.n > 0) {
        k_diag_particles<T><<<blocks_for(sc.n, 256), 256, 0, h->stream>>>(
            (int)sc.poff, sc.n, h->n, static_cast<const vec4<T>*>(h->pl[h->cur]), h->prm.track_fp, acc);
        st = launched(h, "k_diag_particles");
    }
    if (st == RD_OK && h->grid_mode != GRID_NONE) {
        const DevParams<T> P = scene_params<T>(h, scene, h->last_dt, T(1));
        const Collider<T>* cols = static_cast<const Collider<T>*>(h->d_col);
        const unsigned cb = blocks_for(sc.ncells, 256);
        if (h->grid_mode == GRID_FUSED)
            k_diag_grid<T, true><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g ^ 1]) + sc.goff,
                                                            cols, acc + 15);
        else
            k_diag_grid<T, false><<<cb, 256, 0, h->stream>>>(P, static_cast<const vec4<T>*>(h->grid[h->g]) + sc.goff,
                                                             cols, acc + 15);
        st = launched(h, "k_diag_grid");
    }
    double a[20];
    if (st == RD_OK) st = check_cuda(h, cudaMemcpyAsync(a, acc, sizeof a, cudaMemcpyDeviceToHost, h->stream), "d2h");
    if (st == RD_OK) st = check_cuda(h, cudaStreamSynchronize(h->stream), "sync");
    if (st != RD_OK) return done(st);
    std::memset(out, 0, sizeof(*out));
    out->particle_mass = a[0];
    for (int k = 0; k < 3; ++k) { out->particle_momentum[k] = a[1 + k]; out->grid_momentum[k] = a[16 + k]; }
    out->average_particle_density = a[5] > 0 ? a[4] / a[5] : 0.0;
    for (int e = 0; e < 9; ++e) out->average_deformation_gradient[e] = sc.n > 0 ? a[6 + e] / sc.n : 0.0;
    out->grid_mass = a[15];
    out->used_cells = (int64_t)a[19];
    return done(RD_OK);
}

bool all_set(const rd_handle* h) {
    for (const rd_scene_info& sc : h->scenes)
        if (!sc.set && sc.n > 0) return false;
    return true;
}

}  // namespace

extern "C" {

rd_status rd_create(const rd_params* params, rd_handle** out) { return create_impl(params, 1, out); }

rd_status rd_batch_create(const rd_params* scenes, int32_t nscenes, rd_handle** out) {
    return create_impl(scenes, nscenes, out);
}

rd_status rd_batch_num_scenes(rd_handle* h, int32_t* nscenes) {
    if (!h || !nscenes) return RD_INVALID_ARG;
    *nscenes = (int32_t)h->scenes.size();
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

rd_status rd_batch_set_particles(rd_handle* h, int32_t scene, const rd_particles* in, int where) {
    if (!h || !in || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (scene < 0 || scene >= (int32_t)h->scenes.size()) return fail(h, RD_INVALID_ARG, "no such scene");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, set_particles_impl, h, scene, in, where);
}

rd_status rd_batch_get_particles(rd_handle* h, int32_t scene, rd_particles* out, int where) {
    if (!h || !out || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (scene < 0 || scene >= (int32_t)h->scenes.size()) return fail(h, RD_INVALID_ARG, "no such scene");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_particles_impl, h, scene, out, where);
}

rd_status rd_batch_get_grid(rd_handle* h, int32_t scene, void* mass, void* velocity, int where) {
    if (!h || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (scene < 0 || scene >= (int32_t)h->scenes.size()) return fail(h, RD_INVALID_ARG, "no such scene");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_grid_impl, h, scene, mass, velocity, nullptr, where);
}

rd_status rd_batch_step(rd_handle* h, double dt, int32_t nsteps) { return rd_step(h, dt, nsteps); }

rd_status rd_set_particles(rd_handle* h, const rd_particles* in, int where) {
    if (!h || !in || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (batched(h)) return fail(h, RD_INVALID_ARG, "a batch takes its particles per scene (rd_batch_set_particles)");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, set_particles_impl, h, 0, in, where);
}

rd_status rd_get_particles(rd_handle* h, rd_particles* out, int where) {
    if (!h || !out || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (batched(h)) return fail(h, RD_INVALID_ARG, "a batch returns its particles per scene (rd_batch_get_particles)");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_particles_impl, h, 0, out, where);
}

rd_status rd_init_volumes(rd_handle* h) {
    if (!h) return RD_INVALID_ARG;
    if (!all_set(h)) return fail(h, RD_INVALID_ARG, "every scene needs its particles first");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, init_volumes_impl, h);
}

rd_status rd_step(rd_handle* h, double dt, int32_t nsteps) {
    if (!h || nsteps < 0 || !std::isfinite(dt)) return RD_INVALID_ARG;
    if (!all_set(h)) return fail(h, RD_INVALID_ARG, "every scene needs its particles first");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, steps_impl, h, dt, nsteps);
}

rd_status rd_autotune(rd_handle* h, double dt, int32_t steps, const char* cache_path, rd_tune_result* result) {
    if (!h || !result || steps < 1 || !std::isfinite(dt)) return RD_INVALID_ARG;
    if (!all_set(h)) return fail(h, RD_INVALID_ARG, "every scene needs its particles first");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, autotune_impl, h, dt, steps, cache_path, result);
}

rd_status rd_tune_trials(rd_handle* h, rd_tune_trial* out, int32_t cap, int32_t* count) {
    if (!h || !count || cap < 0 || (cap > 0 && !out)) return RD_INVALID_ARG;
    const int32_t n = (int32_t)std::min<size_t>((size_t)cap, h->tune_trials.size());
    for (int32_t i = 0; i < n; ++i) out[i] = h->tune_trials[i];
    *count = (int32_t)h->tune_trials.size();
    return RD_OK;
}

rd_status rd_tune_key(rd_handle* h, char* buf, size_t len) {
    if (!h || !buf || len == 0) return RD_INVALID_ARG;
    const std::string k = tune_key_of(h);
    if (k.size() + 1 > len) return RD_TOO_LARGE;
    std::memcpy(buf, k.c_str(), k.size() + 1);
    return RD_OK;
}

rd_status rd_tune_cache_get(const char* path, const char* key, rd_tune_result* out, int32_t* found) {
    if (!path || !out || !found || !tune_key_ok(key)) return RD_INVALID_ARG;
    *found = tune_cache_find(path, key, out) ? 1 : 0;
    return RD_OK;
}

rd_status rd_tune_cache_put(const char* path, const char* key, const rd_tune_result* r) {
    if (!path || !r || !tune_key_ok(key) || r->particles_per_item < 0 || r->ctas_per_sm < 0 ||
        (r->scatter != RD_SCATTER_LANE_PAIRS && r->scatter != RD_SCATTER_RECORD_PAIRS) ||
        !std::isfinite(r->ms_per_step))
        return RD_INVALID_ARG;
    FILE* f = std::fopen(path, "a");
    if (!f) return RD_INVALID_ARG;
    const int ok = std::fprintf(f, "%s\t%d %d %d %.9g\n", key, r->particles_per_item, r->ctas_per_sm, r->scatter,
                                r->ms_per_step);
    return (std::fclose(f) == 0 && ok > 0) ? RD_OK : RD_INVALID_ARG;
}

rd_status rd_set_tuning(rd_handle* h, int32_t particles_per_item, int32_t ctas_per_sm, int32_t scatter) {
    if (!h || particles_per_item < 0 || ctas_per_sm < 0 ||
        (scatter != RD_SCATTER_LANE_PAIRS && scatter != RD_SCATTER_RECORD_PAIRS))
        return RD_INVALID_ARG;
    const int wmax = h->prm.precision == RD_FP64 ? WorkP<double>::value : WorkP<float>::value;
    if (particles_per_item != 0 && (particles_per_item < wmax / 4 || particles_per_item > wmax))
        return fail(h, RD_INVALID_ARG, "particles per item out of range");
    cudaSetDevice(h->prm.device);
    h->wp = particles_per_item;
    h->grid_mult = ctas_per_sm;
    h->scatter = scatter < scatter_layouts(h) ? scatter : RD_SCATTER_LANE_PAIRS;
    drop_graphs(h);
    return RD_OK;
}

rd_status rd_get_tuning(rd_handle* h, int32_t* particles_per_item, int32_t* ctas_per_sm, int32_t* scatter) {
    if (!h || !particles_per_item || !ctas_per_sm || !scatter) return RD_INVALID_ARG;
    const int wmax = h->prm.precision == RD_FP64 ? WorkP<double>::value : WorkP<float>::value;
    *particles_per_item = h->wp > 0 ? std::min(h->wp, wmax) : wmax;
    *ctas_per_sm = h->grid_mult > 0 ? std::min(h->grid_mult, h->occ_g2p) : h->occ_g2p;
    *scatter = h->scatter;
    return RD_OK;
}

rd_status rd_initialize_particles(rd_handle* h, const rd_init_spec* spec, int32_t* need_more) {
    if (!h || !spec || !(spec->radius >= 0) || !std::isfinite(spec->mass) ||
        (spec->mode != RD_INIT_REFERENCE && spec->mode != RD_INIT_PARALLEL))
        return RD_INVALID_ARG;
    if (batched(h)) return fail(h, RD_NOT_SUPPORTED, "the initialiser fills single-scene handles");
    cudaSetDevice(h->prm.device);
    ++h->version;
    return RD_DISPATCH(h, initialize_impl, h, *spec, need_more);
}

rd_status rd_set_colliders(rd_handle* h, const rd_collider* colliders, int32_t count, int32_t mode, double friction) {
    if (!h || count < 0 || count > RD_MAX_COLLIDERS || (count && !colliders) || !std::isfinite(friction) ||
        (mode != RD_COLLIDE_REFERENCE && mode != RD_COLLIDE_COULOMB))
        return RD_INVALID_ARG;
    if (batched(h)) return fail(h, RD_NOT_SUPPORTED, "colliders act on single-scene handles");
    cudaSetDevice(h->prm.device);
    ++h->version;
    h->cols.assign(colliders, colliders + count);
    h->col_mode = mode;
    h->col_mu = friction;
    drop_graphs(h);  // the collider count and rule are launch parameters
    return RD_DISPATCH(h, upload_colliders, h);
}

rd_status rd_move_colliders(rd_handle* h, double dt) {
    if (!h || !std::isfinite(dt)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    ++h->version;
    return RD_DISPATCH(h, move_colliders_impl, h, dt);
}

rd_status rd_adjoint_record(rd_handle* h, double dt, int32_t steps, int32_t checkpoint_every) {
    if (!h || steps < 1 || checkpoint_every < 1 || !std::isfinite(dt)) return RD_INVALID_ARG;
    if (!h->cols.empty()) return fail(h, RD_NOT_SUPPORTED, "the adjoint has no collider backward");
    if (!h->prm.lagged_b) return fail(h, RD_NOT_SUPPORTED, "the adjoint follows the reference's lagged-B step");
    if (!all_set(h)) return fail(h, RD_INVALID_ARG, "every scene needs its particles first");
    cudaSetDevice(h->prm.device);
    ++h->version;
    return RD_DISPATCH(h, adjoint_record_impl, h, dt, steps, checkpoint_every);
}

void rd_default_implicit_opts(rd_implicit_opts* opts) {
    if (opts) *opts = implicit_defaults();
}

rd_status rd_time_integration(rd_handle* h, double dt, const rd_implicit_opts* opts, rd_implicit_result* result) {
    if (!h || !result || !std::isfinite(dt)) return RD_INVALID_ARG;
    const rd_implicit_opts o = opts ? *opts : implicit_defaults();
    if (!implicit_opts_ok(o)) return fail(h, RD_INVALID_ARG, "implicit options out of range");
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, time_integration_impl, h, dt, o, result);
}

rd_status rd_implicit_energy(rd_handle* h, double dt, const rd_implicit_opts* opts, const void* vel, void* grad,
                             int where, double* energy) {
    if (!h || !vel || !energy || !std::isfinite(dt) || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    const rd_implicit_opts o = opts ? *opts : implicit_defaults();
    if (!implicit_opts_ok(o)) return fail(h, RD_INVALID_ARG, "implicit options out of range");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, implicit_energy_impl, h, dt, o, vel, grad, where, energy);
}

rd_status rd_adjoint_backward(rd_handle* h, const void* grad_x, const void* grad_v, int where, rd_grads* grads) {
    if (!h || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (!h->adj.recorded || h->adj.version != h->version)
        return fail(h, RD_INVALID_ARG, "no adjoint record of the current state (rd_adjoint_record)");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, adjoint_backward_impl, h, grad_x, grad_v, where, grads);
}

rd_status rd_set_graphs(rd_handle* h, int enable) {
    if (!h) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    h->use_graphs = enable != 0;
    if (!enable) drop_graphs(h);
    return RD_OK;
}

rd_status rd_stage(rd_handle* h, int32_t stage, double dt) {
    if (!h || !std::isfinite(dt)) return RD_INVALID_ARG;
    ++h->version;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, stage_impl, h, stage, dt);
}

rd_status rd_get_grid(rd_handle* h, void* mass, void* velocity, void* force, int where) {
    if (!h || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    if (batched(h)) return fail(h, RD_INVALID_ARG, "a batch exports its grids per scene (rd_batch_get_grid)");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, get_grid_impl, h, 0, mass, velocity, force, where);
}

rd_status rd_device_xyzs(rd_handle* h, float** xyzs) {
    if (!h || !xyzs) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, xyzs_impl, h, xyzs);
}

rd_status rd_set_colors(rd_handle* h, const uint8_t* rgba, int where) {
    if (!h || !rgba || (where != RD_HOST && where != RD_DEVICE)) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    if (h->n == 0) return RD_OK;
    return check_cuda(h, cudaMemcpyAsync(h->rgba, rgba, (size_t)h->n * 4,
                                         where == RD_HOST ? cudaMemcpyHostToDevice : cudaMemcpyDeviceToDevice,
                                         h->stream),
                      "colors");
}

rd_status rd_device_colors(rd_handle* h, uint8_t** rgba) {
    if (!h || !rgba) return RD_INVALID_ARG;
    *rgba = reinterpret_cast<uint8_t*>(h->rgba);
    return RD_OK;
}

rd_status rd_splat(rd_handle* h, const rd_view* view, void* image, int where) {
    if (!h || !view || !image || (where != RD_HOST && where != RD_DEVICE) || view->width < 1 || view->height < 1 ||
        (int64_t)view->width * view->height > ((int64_t)1 << 28) || view->max_radius < 0)
        return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    const size_t npix = (size_t)view->width * view->height;
    if (h->img_pixels < npix) {  // the splat buffers follow the largest image asked for
        if (h->zid) cudaFree(h->zid);
        if (h->img) cudaFree(h->img);
        h->zid = nullptr;
        h->img = nullptr;
        h->img_pixels = 0;
        RD_TRY(check_cuda(h, cudaMalloc((void**)&h->zid, npix * sizeof(unsigned long long)), "splat buffers"));
        RD_TRY(check_cuda(h, cudaMalloc((void**)&h->img, npix * sizeof(uint32_t)), "splat buffers"));
        h->img_pixels = npix;
    }
    float* unused = nullptr;
    RD_TRY(rd_device_xyzs(h, &unused));
    ViewDev V{};
    for (int e = 0; e < 16; ++e) V.vp[e] = view->view_projection[e];
    for (int a = 0; a < 3; ++a) { V.right[a] = view->camera_right[a]; V.up[a] = view->camera_up[a]; }
    V.width = view->width;
    V.height = view->height;
    V.background = view->background;
    V.max_radius = view->max_radius > 0 ? view->max_radius : 32;
    uint32_t* out = where == RD_DEVICE ? static_cast<uint32_t*>(image) : h->img;
    k_splat_clear<<<blocks_for(npix, 256), 256, 0, h->stream>>>(h->zid, (int)npix);
    if (h->n > 0) k_splat<<<blocks_for(h->n, 256), 256, 0, h->stream>>>(V, h->n, h->xyzs, h->zid);
    k_splat_resolve<<<blocks_for(npix, 256), 256, 0, h->stream>>>(V, h->n, h->xyzs, h->rgba, h->zid, out);
    RD_TRY(launched(h, "k_splat", h->n > 0 ? 3 : 2));
    if (where == RD_HOST) {
        RD_TRY(check_cuda(h, cudaMemcpyAsync(image, out, npix * 4, cudaMemcpyDeviceToHost, h->stream), "image"));
        RD_TRY(check_cuda(h, cudaStreamSynchronize(h->stream), "sync"));
    }
    return RD_OK;
}

rd_status rd_get_diagnostics(rd_handle* h, int32_t scene, rd_diagnostics* out) {
    if (!h || !out) return RD_INVALID_ARG;
    if (scene < 0 || scene >= (int32_t)h->scenes.size()) return fail(h, RD_INVALID_ARG, "no such scene");
    cudaSetDevice(h->prm.device);
    return RD_DISPATCH(h, diagnostics_impl, h, scene, out);
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

rd_status rd_debug_bounds_violations(uint64_t* count, int32_t* checked) {
    if (!count || !checked) return RD_INVALID_ARG;
#ifdef RD_BOUNDS_CHECK
    unsigned long long v = 0;
    if (cudaMemcpyFromSymbol(&v, rd::rd_bounds_count, sizeof v) != cudaSuccess) return RD_CUDA_ERROR;
    *count = (uint64_t)v;
    *checked = 1;
#else
    *count = 0;
    *checked = 0;
#endif
    return RD_OK;
}

rd_status rd_debug_wait_timeout(rd_handle* h, int32_t tries, int32_t* gave_up) {
    if (!h || !gave_up || tries < 1 || tries > kTileWaitTries) return RD_INVALID_ARG;
    cudaSetDevice(h->prm.device);
    int* d = nullptr;
    RD_TRY(check_cuda(h, cudaMalloc((void**)&d, sizeof(int)), "probe"));
    rd_status st = check_cuda(h, cudaMemsetAsync(d, 0, sizeof(int), h->stream), "probe");
    if (st == RD_OK) {
        k_wait_probe<<<1, 64, 0, h->stream>>>(tries, h->flags, d);
        st = launched(h, "k_wait_probe");
    }
    int g = 0;
    if (st == RD_OK) st = check_cuda(h, cudaMemcpyAsync(&g, d, sizeof(int), cudaMemcpyDeviceToHost, h->stream), "probe");
    if (st == RD_OK) st = check_cuda(h, cudaStreamSynchronize(h->stream), "probe");
    cudaFree(d);
    *gave_up = g;
    return st;
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

rd_status rd_graph_replays(rd_handle* h, uint64_t* count) {
    if (!h || !count) return RD_INVALID_ARG;
    *count = h->graph_replays;
    return RD_OK;
}

rd_status rd_io_bytes(rd_handle* h, uint64_t* in_place, uint64_t* staged) {
    if (!h || !in_place || !staged) return RD_INVALID_ARG;
    *in_place = h->io_direct;
    *staged = h->io_staged;
    return RD_OK;
}

rd_status rd_host_alloc(size_t bytes, void** out) {
    if (!out) return RD_INVALID_ARG;
    *out = nullptr;
    if (bytes == 0) return RD_OK;
    if (cudaHostAlloc(out, bytes, cudaHostAllocDefault) != cudaSuccess) {
        cudaGetLastError();
        *out = nullptr;
        return RD_OOM;
    }
    return RD_OK;
}

rd_status rd_host_free(void* p) {
    if (p && cudaFreeHost(p) != cudaSuccess) {
        cudaGetLastError();
        return RD_CUDA_ERROR;
    }
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
    uint32_t bcount[kNaMaxKeys / kCellsPerBlock];
    uint32_t cursor[kNaMaxKeys];
    uint32_t tile_sums[kNaMaxTiles + 1];
    uint32_t tile_list[kNaMaxTiles + 1];
    uint32_t nwork[2];
    uint32_t flags;
};

// Block key and histogram of particles given as device arrays (x: n x 3).
__global__ void __launch_bounds__(256) k_na_keys(DevParams<float> P, const float* __restrict__ x,
                                                 uint32_t* __restrict__ keys, uint32_t* __restrict__ counts,
                                                 uint32_t* __restrict__ bcount, uint32_t* flags) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P.n) return;
    const int b[3] = {base_of(x[3 * i], P.h), base_of(x[3 * i + 1], P.h), base_of(x[3 * i + 2], P.h)};
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    const uint32_t key = sort_key(P, b);
    keys[i] = key;
    count_key(counts, bcount, key);
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
        p2g_tasks<float, true, kBlk>(S, sorted_total(S));
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
    // an error left pending by earlier, unrelated work stays where it is (peeked,
    // not consumed) and nothing is queued, so the errors checked below are this
    // call's own
    if (cudaPeekAtLastError() != cudaSuccess) return RD_CUDA_ERROR;
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
        cudaMemsetAsync(sc->bcount, 0, (size_t)hp.nblocks * sizeof(uint32_t), st) != cudaSuccess ||
        cudaMemsetAsync(sc->nwork, 0, 2 * sizeof(uint32_t) + sizeof(uint32_t), st) != cudaSuccess)
        return RD_CUDA_ERROR;
    if (n > 0) {
        const int ntiles = (hp.nkeys + kScanTile - 1) / kScanTile;
        const uint32_t work_cap = (uint32_t)kNaMaxWork;
        k_na_keys<<<blocks_for(n, 256), 256, 0, st>>>(P, static_cast<const float*>(in->x), sc->keys, sc->counts,
                                                      sc->bcount, &sc->flags);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
        k_tile_sums<<<blocks_for((size_t)ntiles * 32, 256), 256, 0, st>>>(sc->bcount, hp.nblocks, ntiles, sc->tile_sums);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
        k_tile_prefix<<<1, 1024, 0, st>>>(sc->tile_sums, ntiles, &sc->nwork[1], (uint32_t)n, &sc->flags,
                                          sc->tile_list);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
        const unsigned scan_grid = (unsigned)std::min<size_t>((size_t)ntiles, (size_t)nd.sms * 2);
        k_scan<<<scan_grid, kScanThreads, 0, st>>>(sc->counts, sc->cursor, sc->bcount, sc->tile_sums, sc->tile_list,
                                                   ntiles, hp.nkeys, sc->work, &sc->nwork[0], work_cap,
                                                   (uint32_t)WorkP<float>::value, &sc->flags, nullptr, 1);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
        k_scatter<<<blocks_for(n, 256), 256, 0, st>>>(n, sc->keys, sc->cursor, sc->perm);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
        const size_t max_items = (size_t)n / WorkP<float>::value + (size_t)std::min<int64_t>(nblocks, n) + 1;
        const unsigned grid = (unsigned)std::max<size_t>(1, std::min<size_t>(max_items, (size_t)nd.sms * nd.occ));
        k_na_p2g<<<grid, kThreads, sizeof(P2GTile<float, kBlk>), st>>>(
            P, static_cast<const float*>(in->x), static_cast<const float*>(in->v), static_cast<const float*>(in->B),
            static_cast<const float*>(in->mass), sc->perm, sc->work, &sc->nwork[0], work_cap,
            reinterpret_cast<float4*>(grid_out), &sc->flags);
        if (cudaGetLastError() != cudaSuccess) return RD_CUDA_ERROR;
    }
    return RD_OK;
}

extern "C" rd_status rd_rasterize_noalloc_flags(uint32_t* flags) {
    if (!flags) return RD_INVALID_ARG;
    *flags = 0;
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return RD_CUDA_ERROR;
    NaScratch* sc = nullptr;
    {
        std::lock_guard<std::mutex> lock(g_na_mutex);
        sc = g_na[dev].scratch;
    }
    if (!sc) return RD_OK;  // no rasterize has run on this device
    return cudaMemcpy(flags, &sc->flags, sizeof(uint32_t), cudaMemcpyDeviceToHost) == cudaSuccess ? RD_OK
                                                                                               : RD_CUDA_ERROR;
}
