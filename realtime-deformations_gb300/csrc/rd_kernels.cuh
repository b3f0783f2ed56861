// sm_103a kernels of the MPM step.  One step of rd_step is
//   k_keys (only when positions changed outside a step and the upload did not
//   count them) -> k_tile_sums -> k_tile_prefix -> k_scan -> k_scatter
//   -> k_grid_clear -> k_g2p2g (k_p2g first when the grid must be rebuilt)
// and the stage kernels serve rd_stage, which runs the reference's seven
// stages one by one (material_point_method.cpp:94-350).
#pragma once
#include <cuda.h>  // CUtensorMap (TileMaps)

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
    int nkeys;     // blocks x 64 cells
    int n;         // particles
    T h, dinv, dt;
    T hinv_pow2;   // 1 / h when h is a power of two (x / h == x * hinv_pow2 exactly), else 0
    T mu0, lambda0, xi;
    T lo, hi;      // singular value clamp
    T elo, ehi;    // eigenvalues of F^T F - I for stress_direct (elo >= ehi: not used)
    T g[3];
    T xlo, xhi[3]; // position clamp (material_point_method.cpp:381-388)
    T fscale;      // force scale in P2G: dt when fused with the momentum, 1 alone
    int bc, bc_width;
    int lagged;
    // Place of this scene in a batch (zero for a single scene): its first
    // 4x4x4 block among all scenes' blocks, and its first grid node.
    uint32_t block_base;
    unsigned long long goff;
    // box colliders applied in the grid update (single scene): count, rule, mu
    int ncol, col_mode;
    T mu;
};

struct DevBufs {
    const void* pin;   // particle planes read
    void* pout;        // particle planes written (fused G2P: sorted order)
    const uint32_t* perm;
    uint32_t* keys_out;
    uint32_t* counts;
    const int4* work;
    // items from the front of `work` (nwork) and, when nwork_back is set, from
    // its back (work_item)
    const uint32_t* nwork;
    const uint32_t* nwork_back;
    uint32_t work_cap;
    // fused kernel: the counter its CTAs claim work items from (zero at the
    // launch) and the next launch's, which this launch zeroes
    uint32_t* claim;
    uint32_t* claim_next;
    void* grid;        // vec4 per cell
    void* grid_next;   // vec4 per cell: P2G of the next step (fused kernel)
    void* gforce;      // vec4 per cell (stage mode forces)
    uint32_t* flags;
    // fused kernel, adjoint segments: U, singular values and V of each
    // particle's plastic split, 6 vec4 planes by sorted slot (null: not kept)
    void* split_out;
    // k_p2g of a step whose particles are not in sorted order (after an
    // upload): the particles copied to these planes at their sorted
    // positions, and perm_reset[s] = s, so the fused kernel then reads them
    // in order (null: no copy)
    void* reorder_out;
    uint32_t* perm_reset;
    // k_p2g with the force: P F^T of each particle, computed during an upload
    // (3 vec4 planes by slot, row-major, the last 3 entries unused), read
    // instead of computed (null: computed)
    const void* stress;
    // fused kernel, single scene: slot_of[id] = the sorted slot each particle
    // is written to, for the next download (null: not kept)
    uint32_t* slot_of;
    uint32_t* bcount;  // particles per 4x4x4 block (the block sums of counts)
    uint8_t* gmark;       // blocks of grid that hold data (set by every writer)
    uint8_t* gmark_next;  // the same for grid_next
    // batches: DevParams<T> per scene, first block and first particle of each
    // scene (nscenes + 1 entries, ascending)
    const void* scenes;
    const uint32_t* sblock;
    const uint32_t* spoff;
    int nscenes;
    const void* colliders;  // Collider<T>[ncol]
};

// The work list: `nf` items from the front of D.work and `nb` from its back,
// the back ones stored from index work_cap - 1 downwards (work_item maps a
// claim 0 .. work_items - 1 to its entry).  Without a back counter all items
// are at the front.
__device__ __forceinline__ void work_counts(const DevBufs& D, uint32_t& nf, uint32_t& nb) {
    nf = min(*D.nwork, D.work_cap);
    nb = D.nwork_back ? min(*D.nwork_back, D.work_cap - nf) : 0u;
}
__device__ __forceinline__ int4 work_item(const DevBufs& D, uint32_t nf, uint32_t c) {
    return D.work[c < nf ? c : D.work_cap - 1u - (c - nf)];
}

// A box collider on the device: R (world from box, row-major), centre t, half
// extents s, velocity v.
template <typename T> struct Collider {
    T R[9], t[3], s[3], v[3];
};

// MeshCollider::sdf (material_point_method.hpp:80-88): with p = R^T (x - t)
// and q = |p| - s, the reference returns |max(q_x, q_y, q_z, 0)| +
// min(max(q_x, q_y, q_z), 0), i.e. max_i q_i.
template <typename T>
__device__ __forceinline__ T box_sdf(const Collider<T>& c, T x0, T x1, T x2) {
    const T d0 = x0 - c.t[0], d1 = x1 - c.t[1], d2 = x2 - c.t[2];
    const T q0 = abs_(c.R[0] * d0 + c.R[3] * d1 + c.R[6] * d2) - c.s[0];
    const T q1 = abs_(c.R[1] * d0 + c.R[4] * d1 + c.R[7] * d2) - c.s[1];
    const T q2 = abs_(c.R[2] * d0 + c.R[5] * d1 + c.R[8] * d2) - c.s[2];
    const T qm = q0 > q1 ? (q0 > q2 ? q0 : q2) : (q1 > q2 ? q1 : q2);
    return abs_(qm > T(0) ? qm : T(0)) + (qm < T(0) ? qm : T(0));
}

// bodyCollision (material_point_method.cpp:264-300) for a grid node at x with
// velocity v, over the colliders in order.
template <typename T>
__device__ __forceinline__ void collide_node(const DevParams<T>& P, const Collider<T>* __restrict__ cols, T x0, T x1,
                                             T x2, T v[3]) {
    for (int k = 0; k < P.ncol; ++k) {
        const Collider<T>& c = cols[k];
        if (box_sdf(c, x0, x1, x2) > T(0)) continue;
        T n[3];
        if (P.col_mode == 0) {  // gradient(phi, pos, 3): central differences, delta 0.001
            const T dl = T(0.001f);
            n[0] = (box_sdf(c, x0 + dl, x1, x2) - box_sdf(c, x0 - dl, x1, x2)) / (T(2) * dl);
            n[1] = (box_sdf(c, x0, x1 + dl, x2) - box_sdf(c, x0, x1 - dl, x2)) / (T(2) * dl);
            n[2] = (box_sdf(c, x0, x1, x2 + dl) - box_sdf(c, x0, x1, x2 - dl)) / (T(2) * dl);
        } else {  // outward normal of the face of largest q
            const T d0 = x0 - c.t[0], d1 = x1 - c.t[1], d2 = x2 - c.t[2];
            T p[3], q[3];
#pragma unroll
            for (int a = 0; a < 3; ++a) {
                p[a] = c.R[a] * d0 + c.R[3 + a] * d1 + c.R[6 + a] * d2;
                q[a] = abs_(p[a]) - c.s[a];
            }
            const int f = q[0] > q[1] ? (q[0] > q[2] ? 0 : 2) : (q[1] > q[2] ? 1 : 2);
            const T sg = p[f] < T(0) ? T(-1) : T(1);
#pragma unroll
            for (int a = 0; a < 3; ++a) n[a] = sg * c.R[3 * a + f];
        }
        const T r0 = v[0] - c.v[0], r1 = v[1] - c.v[1], r2 = v[2] - c.v[2];
        const T vn = r0 * n[0] + r1 * n[1] + r2 * n[2];
        if (vn >= T(0)) continue;
        const T t0 = r0 - n[0] * vn, t1 = r1 - n[1] * vn, t2 = r2 - n[2] * vn;
        const T len = P.col_mode == 0 ? T(3) : sqrt_(t0 * t0 + t1 * t1 + t2 * t2);
        T f = T(0);
        if (len > -P.mu * vn && len > T(0)) f = T(1) + P.mu * vn / len;
        v[0] = t0 * f + c.v[0];
        v[1] = t1 * f + c.v[1];
        v[2] = t2 * f + c.v[2];
    }
}

// The scene holding item v of a batch: the last s with starts[s] <= v.
__device__ __forceinline__ int scene_of(const uint32_t* __restrict__ starts, int nscenes, uint32_t v) {
    int lo = 0, hi = nscenes - 1;
    while (lo < hi) {
        const int mid = (lo + hi + 1) >> 1;
        if (__ldg(starts + mid) <= v) lo = mid; else hi = mid - 1;
    }
    return lo;
}

// Copies scene s's parameters into shared memory (all threads; the caller
// synchronises before use).
template <typename T>
__device__ __forceinline__ void copy_scene(DevParams<T>& dst, const void* table, int s) {
    static_assert(sizeof(DevParams<T>) % 4 == 0, "DevParams is copied as words");
    const uint32_t* src = reinterpret_cast<const uint32_t*>(static_cast<const DevParams<T>*>(table) + s);
    uint32_t* d = reinterpret_cast<uint32_t*>(&dst);
    for (int k = threadIdx.x; k < (int)(sizeof(DevParams<T>) / 4); k += blockDim.x) d[k] = __ldg(src + k);
}

__device__ __forceinline__ void raise_flag(uint32_t* flags, uint32_t f) {
    if ((__ldcg(flags) & f) == 0) atomicOr(flags, f);
}

// Sort key of base cell b: the cell's 4x4x4 block (linearised x-major like
// the grid) times 64 plus the cell's index within the block, so a block's
// particles are contiguous and, inside the block, grouped by cell.  b is
// clamped into the grid first; the caller flags out-of-range particles.
constexpr int kCellsPerBlock = kBlk * kBlk * kBlk;
template <typename T>
__device__ __forceinline__ uint32_t sort_key(const DevParams<T>& P, const int b[3]) {
    int k[3], c[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const int v = b[a] < 0 ? 0 : (b[a] > P.M[a] - 1 ? P.M[a] - 1 : b[a]);
        k[a] = v / kBlk;
        c[a] = v - k[a] * kBlk;
    }
    const uint32_t blk = P.block_base + ((uint32_t)k[0] * P.NB[1] + k[1]) * P.NB[2] + k[2];
    return blk * kCellsPerBlock + (uint32_t)((c[0] * kBlk + c[1]) * kBlk + c[2]);
}

template <typename T>
__device__ __forceinline__ bool stencil_in_grid(const DevParams<T>& P, const int b[3]) {
    return b[0] >= 1 && b[1] >= 1 && b[2] >= 1 && b[0] + 2 < P.M[0] && b[1] + 2 < P.M[1] && b[2] + 2 < P.M[2];
}

// One atomic per distinct key, and one per distinct block, among the active
// lanes of the warp.
__device__ __forceinline__ void count_key(uint32_t* counts, uint32_t* bcount, uint32_t key) {
    const uint32_t active = __activemask();
    const uint32_t peers = __match_any_sync(active, key);
    const int lane = (int)(threadIdx.x & 31);
    if (lane == __ffs(peers) - 1) atomicAdd(counts + key, (uint32_t)__popc(peers));
    const uint32_t bpeers = __match_any_sync(active, key / 64u);
    if (lane == __ffs(bpeers) - 1) atomicAdd(bcount + key / 64u, (uint32_t)__popc(bpeers));
}

// ---------------------------------------------------------------- sorting
template <typename T, bool BATCH>
__global__ void __launch_bounds__(256) k_keys(DevParams<T> P0, DevBufs D, const vec4<T>* __restrict__ pl,
                                              uint32_t* __restrict__ keys) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P0.n) return;
    uint32_t* counts = D.counts;
    uint32_t* flags = D.flags;
    DevParams<T> P;
    if (BATCH) P = static_cast<const DevParams<T>*>(D.scenes)[scene_of(D.spoff, D.nscenes, (uint32_t)i)];
    else P = P0;
    const vec4<T> x = ld_stream(pl + i);
    const int b[3] = {base_of(x.x, P.h), base_of(x.y, P.h), base_of(x.z, P.h)};
    if (!stencil_in_grid(P, b)) raise_flag(flags, 1u);
    const uint32_t key = sort_key(P, b);
    keys[i] = key;
    count_key(counts, D.bcount, key);
}

// Exclusive scan of the per-cell counts into the scatter cursor (the first
// sorted slot of each cell), emission of the work items and reset of the
// counts for the next histogram, over kScanTile-key tiles on all SMs:
// k_tile_sums adds up each tile from the block counts, k_tile_prefix turns
// the tile sums into their exclusive prefix and lists the non-empty tiles (one
// CTA), and k_scan, a persistent grid over that list, scans one tile (64 whole
// blocks) per CTA trip from its prefix; empty tiles cost no CTA and only
// occupied blocks read or write their cells, so empty grid space costs 4 bytes
// per block.  A block of c particles becomes ceil(c / wp) work items of nearly
// equal size; the items are appended to the list through an atomic counter
// (their order does not matter) and the counter of the next sort is cleared
// here.
constexpr int kScanThreads = 1024;
constexpr int kScanPer = 4;                                 // consecutive keys per thread
constexpr int kScanTile = kScanThreads * kScanPer;          // keys per CTA
constexpr int kBlocksPerTile = kScanTile / kCellsPerBlock;  // 64
constexpr int kThreadsPerBlockKeys = kCellsPerBlock / kScanPer;  // 16

__device__ __forceinline__ uint4 ld4_or_zero(const uint32_t* p, int k0, int nkeys) {
    if (k0 + kScanPer <= nkeys) return *reinterpret_cast<const uint4*>(p + k0);
    uint4 r = make_uint4(0u, 0u, 0u, 0u);
    if (k0 < nkeys) r.x = p[k0];
    if (k0 + 1 < nkeys) r.y = p[k0 + 1];
    if (k0 + 2 < nkeys) r.z = p[k0 + 2];
    return r;
}
__device__ __forceinline__ void st4(uint32_t* p, int k0, int nkeys, uint4 v) {
    if (k0 + kScanPer <= nkeys) { *reinterpret_cast<uint4*>(p + k0) = v; return; }
    if (k0 < nkeys) p[k0] = v.x;
    if (k0 + 1 < nkeys) p[k0 + 1] = v.y;
    if (k0 + 2 < nkeys) p[k0 + 2] = v.z;
}

// Particles per tile from the block counts: a warp per tile of 64 blocks.
__global__ void __launch_bounds__(256) k_tile_sums(const uint32_t* __restrict__ bcount, int nblocks, int ntiles,
                                                   uint32_t* __restrict__ tile_sums) {
    const int t = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5), lane = threadIdx.x & 31;
    if (t >= ntiles) return;
    const int b0 = t * kBlocksPerTile + 2 * lane;
    uint32_t sum = 0;
    if (b0 < nblocks) sum += bcount[b0];
    if (b0 + 1 < nblocks) sum += bcount[b0 + 1];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
    if (lane == 0) tile_sums[t] = sum;
}

// In place: sums[t] -> sum of sums[0 .. t-1] for t < ntiles, sums[ntiles] =
// the total (which must be the particle count); also clears the item counter
// of the next sort.  With `list` given, the indices of the non-empty tiles
// go to list[0 ..) in ascending order and their number to list[ntiles].  One
// CTA of 1024 threads; each thread takes kPrefixPer consecutive tiles per
// trip, loaded together, so the trips (and their barriers) are few.  With
// `bcount` given (grids of at most kTileSumsInPrefix tiles) the CTA first
// sums the block counts into the tiles itself, a warp per tile, which saves
// the k_tile_sums launch of small scenes.
constexpr int kPrefixPer = 8;
constexpr int kTileSumsInPrefix = 128;

__global__ void __launch_bounds__(1024) k_tile_prefix(uint32_t* __restrict__ sums, int ntiles,
                                                      uint32_t* __restrict__ nwork_next_sort, uint32_t n_expected,
                                                      uint32_t* flags, uint32_t* __restrict__ list,
                                                      const uint32_t* __restrict__ bcount = nullptr,
                                                      int nblocks = 0,
                                                      uint32_t* __restrict__ nwork_next_back = nullptr) {
    __shared__ uint2 s_w[32];   // per warp: (particles, non-empty tiles)
    __shared__ uint2 s_carry;   // totals of the previous trips
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    if (tid == 0) {
        s_carry = make_uint2(0u, 0u);
        *nwork_next_sort = 0u;
        if (nwork_next_back) *nwork_next_back = 0u;
    }
    if (bcount) {
        for (int t = wid; t < ntiles; t += 32) {
            const int b0 = t * kBlocksPerTile + 2 * lane;
            uint32_t sum = 0;
            if (b0 < nblocks) sum += bcount[b0];
            if (b0 + 1 < nblocks) sum += bcount[b0 + 1];
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) sum += __shfl_xor_sync(0xffffffffu, sum, o);
            if (lane == 0) sums[t] = sum;
        }
    }
    __syncthreads();
    for (int base = 0; base < ntiles; base += 1024 * kPrefixPer) {
        const int t0 = base + tid * kPrefixPer;
        uint32_t v[kPrefixPer];
        uint32_t s = 0u, o = 0u;
#pragma unroll
        for (int j = 0; j < kPrefixPer; ++j) v[j] = t0 + j < ntiles ? sums[t0 + j] : 0u;
#pragma unroll
        for (int j = 0; j < kPrefixPer; ++j) { s += v[j]; o += v[j] != 0u; }
        uint32_t xs = s, xo = o;
#pragma unroll
        for (int d = 1; d < 32; d <<= 1) {
            const uint32_t ys = __shfl_up_sync(0xffffffffu, xs, d), yo = __shfl_up_sync(0xffffffffu, xo, d);
            if (lane >= d) { xs += ys; xo += yo; }
        }
        if (lane == 31) s_w[wid] = make_uint2(xs, xo);
        __syncthreads();
        if (wid == 0) {
            uint2 w = s_w[lane];
#pragma unroll
            for (int d = 1; d < 32; d <<= 1) {
                const uint32_t ys = __shfl_up_sync(0xffffffffu, w.x, d), yo = __shfl_up_sync(0xffffffffu, w.y, d);
                if (lane >= d) { w.x += ys; w.y += yo; }
            }
            s_w[lane] = w;  // inclusive over warps
        }
        __syncthreads();
        const uint2 c = s_carry;
        const uint2 wp = wid ? s_w[wid - 1] : make_uint2(0u, 0u);
        uint32_t es = c.x + wp.x + xs - s, eo = c.y + wp.y + xo - o;
#pragma unroll
        for (int j = 0; j < kPrefixPer; ++j) {
            if (t0 + j < ntiles) {
                sums[t0 + j] = es;
                if (list && v[j]) list[eo++] = (uint32_t)(t0 + j);
                es += v[j];
            }
        }
        __syncthreads();  // s_carry and s_w read by every thread
        if (tid == 0) s_carry = make_uint2(c.x + s_w[31].x, c.y + s_w[31].y);
        __syncthreads();
    }
    if (tid == 0) {
        sums[ntiles] = s_carry.x;
        if (list) list[ntiles] = s_carry.y;
        if (s_carry.x != n_expected) atomicOr(flags, 4u);
    }
}

__global__ void __launch_bounds__(kScanThreads) k_scan(uint32_t* __restrict__ counts, uint32_t* __restrict__ cursor,
                                                       uint32_t* __restrict__ bcount,
                                                       const uint32_t* __restrict__ tile_pre,
                                                       const uint32_t* __restrict__ tile_list, int ntiles, int nkeys,
                                                       int4* __restrict__ work, uint32_t* __restrict__ nwork,
                                                       uint32_t work_cap, uint32_t wp, uint32_t* flags,
                                                       const uint32_t* __restrict__ sblock, int nscenes,
                                                       uint32_t* __restrict__ nwork_back = nullptr) {
    __shared__ uint32_t s_w[32];
    __shared__ uint32_t s_blk[kBlocksPerTile];  // particles per block of this tile
    const int tid = threadIdx.x, lane = tid & 31, wid = tid >> 5;
    const uint32_t nocc = tile_list[ntiles];
    for (uint32_t it = blockIdx.x; it < nocc; it += gridDim.x) {
        const int t = (int)tile_list[it];
        const uint32_t s_off = tile_pre[t];
        const int k0 = t * kScanTile + tid * kScanPer;
        // the cell counts of an empty block are zero and its cursor is never read:
        // only occupied blocks touch their 64 cells
        const int gblk = k0 / kCellsPerBlock;
        const uint32_t bsum = gblk * kCellsPerBlock < nkeys ? bcount[gblk] : 0u;
        const uint4 c = bsum ? ld4_or_zero(counts, k0, nkeys) : make_uint4(0u, 0u, 0u, 0u);
        const uint32_t tc = c.x + c.y + c.z + c.w;
        if ((tid & (kThreadsPerBlockKeys - 1)) == 0) s_blk[tid / kThreadsPerBlockKeys] = bsum;
        uint32_t ic = tc;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const uint32_t y = __shfl_up_sync(0xffffffffu, ic, o);
            if (lane >= o) ic += y;
        }
        __syncthreads();
        if (lane == 31) s_w[wid] = ic;
        __syncthreads();
        if (wid == 0) {
            uint32_t wc = s_w[lane];
#pragma unroll
            for (int o = 1; o < 32; o <<= 1) {
                const uint32_t y = __shfl_up_sync(0xffffffffu, wc, o);
                if (lane >= o) wc += y;
            }
            s_w[lane] = wc;  // inclusive prefix over warps
        }
        __syncthreads();
        const uint32_t st0 = s_off + (wid ? s_w[wid - 1] : 0u) + ic - tc;
        if (bsum) {
            st4(cursor, k0, nkeys, make_uint4(st0, st0 + c.x, st0 + c.x + c.y, st0 + c.x + c.y + c.z));
            st4(counts, k0, nkeys, make_uint4(0u, 0u, 0u, 0u));
        }
        // the first thread of each block emits the block's work items and clears
        // the block count for the next histogram
        if ((tid & (kThreadsPerBlockKeys - 1)) == 0) {
            const int b = tid / kThreadsPerBlockKeys;
            const uint32_t bc = s_blk[b];
            if (bc) bcount[gblk] = 0u;
            const uint32_t ni = (bc + wp - 1) / wp;
            if (ni) {
                const uint32_t blk = (uint32_t)(t * kBlocksPerTile + b);
                const int scene = nscenes > 1 ? scene_of(sblock, nscenes, blk) : 0;
                // with a back counter, items of more than half the work-item
                // size fill the list from the front and smaller ones from the
                // back, so a kernel claiming items in list order takes the
                // large ones first and ends on small ones
                const bool back = nwork_back && 2u * (bc / ni) <= wp;
                uint32_t oi = atomicAdd(back ? nwork_back : nwork, ni);
                uint32_t st = st0;
                for (uint32_t j = 0; j < ni; ++j, ++oi) {
                    const uint32_t cnt = bc / ni + (j < bc % ni ? 1u : 0u);
                    if (oi < work_cap) work[back ? work_cap - 1u - oi : oi] = make_int4((int)blk, (int)st, (int)cnt, scene);
                    else atomicOr(flags, 4u);
                    st += cnt;
                }
            }
        }
        __syncthreads();  // s_blk and s_w are refilled by the next tile
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

// Weights and offsets of the stencil of x; rel = base - 1 - org must lie in
// [0, rmax] for the stencil to fit the tile with origin org.
template <typename T>
__device__ __forceinline__ bool make_stencil(const DevParams<T>& P, const T x[3], const int org[3], Stencil<T>& S,
                                             int rmax = kTile - 4) {
    bool ok = true;
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        const T t = P.hinv_pow2 != T(0) ? x[a] * P.hinv_pow2 : div_rn(x[a], P.h);
        S.b[a] = (int)t;
        bspline4(t, S.b[a], S.w[a]);
#pragma unroll
        for (int o = 0; o < 4; ++o) S.d[a][o] = (T)(S.b[a] - 1 + o) * P.h - x[a];
        S.rel[a] = S.b[a] - 1 - org[a];
        ok = ok && S.rel[a] >= 0 && S.rel[a] <= rmax;
    }
    return ok;
}

// P F^T of the fixed-corotated stress with the reference's hardening
// (material_point_method.cpp:239-248): P = 2 mu (F - R) + lambda (J - 1) J F^-T,
// so P F^T = 2 mu (F - R) F^T + lambda (J - 1) J I.  With F = U S V^T and the
// reference's proper rotation R = U D V^T (D = I, or diag(.., -1) on the
// smallest singular value when det F < 0), (F - R) F^T = U (S - D) S U^T.
// F stays within a few 1e-3 of a rotation, so s - 1 (svd3_near) and J - 1
// are formed without cancellation from G = F - I (exact in floating point):
// J - 1 = tr G + (sum of the principal 2x2 minors of G) + det G.
template <typename T>
__device__ __forceinline__ void stress_PFt_svd(const DevParams<T>& P, const T F[9], T Jp, const T U[9], const T s[3],
                                               const T sm1[3], T out[9]) {
    T G[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) G[e] = F[e];
    G[0] -= T(1); G[4] -= T(1); G[8] -= T(1);
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
        const T sm = (J < T(0) && c == kmin) ? (s[c] + T(1)) : sm1[c];  // s - d
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

// The 9 entries of P F^T as 3 vec4 planes of n elements (the stress of the
// first P2G after an upload, computed while the upload is bound by the link).
template <typename T>
__device__ __forceinline__ void store_stress(vec4<T>* __restrict__ st, size_t n, size_t i, const T G[9]) {
    st[i] = mk4<T>(G[0], G[1], G[2], G[3]);
    st[n + i] = mk4<T>(G[4], G[5], G[6], G[7]);
    st[2 * n + i] = mk4<T>(G[8], T(0), T(0), T(0));
}
template <typename T>
__device__ __forceinline__ void load_stress(const vec4<T>* __restrict__ st, size_t n, size_t i, T G[9]) {
    const vec4<T> a = st[i], b = st[n + i], c = st[2 * n + i];
    G[0] = a.x; G[1] = a.y; G[2] = a.z; G[3] = a.w;
    G[4] = b.x; G[5] = b.y; G[6] = b.z; G[7] = b.w;
    G[8] = c.x;
}

template <typename T>
__device__ __forceinline__ void stress_PFt(const DevParams<T>& P, const T F[9], T Jp, T out[9]) {
    T U[9], s[3], sm1[3], V[9];
    svd3_near(F, U, s, sm1, V);
    stress_PFt_svd(P, F, Jp, U, s, sm1, out);
}

// The clamped split of F_E* = U S V^T that updateDeformationGradient makes,
// kept for the stress of the next P2G: sc = clamp(S), sc - 1 without
// cancellation, and the sign of det F_E*.
template <typename T> struct Split {
    T U[9], sc[3], scm1[3], sgn;
};

// updateDeformationGradient (material_point_method.cpp:306-330) for one
// particle: F_E* = (I + dt B D^-1) F_E = U S V^T, F_E <- U clamp(S) V^T, and
// det F_P *= prod over clamped i of S_i / clamp(S_i) (the reference's
// F_P <- F_E^-1 Fhat with Fhat = F_E* F_P); with the full F_P,
// F_P <- V (S / clamp(S)) V^T F_P.  s_i - 1 for an unclamped value comes
// from svd3_near without cancellation.
template <typename T>
__device__ __forceinline__ void f_star(const DevParams<T>& P, const T Bm[9], const T F[9], T Fs[9]) {
    T A[9];
    const T ddt = P.dinv * P.dt;
#pragma unroll
    for (int e = 0; e < 9; ++e) A[e] = Bm[e] * ddt;
    A[0] += T(1); A[4] += T(1); A[8] += T(1);
    matmul3(Fs, A, F);
}

// The split of a given F_E* (Fs), as update_F makes it.
template <typename T, bool TRACK_FP>
__device__ __forceinline__ void update_F_star(const DevParams<T>& P, const T Fs[9], T F[9], T& Jp, T FP[9],
                                              Split<T>& sp, T* s_out = nullptr, T* sm1_out = nullptr,
                                              T* V_out = nullptr) {
    T s[3], sm1[3], V[9];
    svd3_near(Fs, sp.U, s, sm1, V);
    if (s_out) {
#pragma unroll
        for (int c = 0; c < 3; ++c) { s_out[c] = s[c]; sm1_out[c] = sm1[c]; }
#pragma unroll
        for (int e = 0; e < 9; ++e) V_out[e] = V[e];
    }
    T ratio = T(1);
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        if (s[c] < P.lo) {
            sp.sc[c] = P.lo; sp.scm1[c] = P.lo - T(1); ratio *= s[c] / P.lo;
        } else if (s[c] > P.hi) {
            sp.sc[c] = P.hi; sp.scm1[c] = P.hi - T(1); ratio *= s[c] / P.hi;
        } else {
            sp.sc[c] = s[c];
            sp.scm1[c] = sm1[c];
        }
    }
    sp.sgn = det3(Fs) < T(0) ? T(-1) : T(1);
    if (!(s[0] < P.lo || s[0] > P.hi || s[1] < P.lo || s[1] > P.hi || s[2] < P.lo || s[2] > P.hi)) {
        // nothing clamped: U S V^T is F* itself
#pragma unroll
        for (int e = 0; e < 9; ++e) F[e] = Fs[e];
    } else {
#pragma unroll
        for (int r = 0; r < 3; ++r)
#pragma unroll
            for (int c = 0; c < 3; ++c)
                F[3 * r + c] = sp.U[3 * r] * sp.sc[0] * V[3 * c] + sp.U[3 * r + 1] * sp.sc[1] * V[3 * c + 1] +
                               sp.U[3 * r + 2] * sp.sc[2] * V[3 * c + 2];
    }
    Jp = Jp * ratio;
    if (TRACK_FP) {
        T r[3], Mv[9], out[9];
#pragma unroll
        for (int c = 0; c < 3; ++c) r[c] = s[c] / sp.sc[c];
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

template <typename T, bool TRACK_FP>
__device__ __forceinline__ void update_F(const DevParams<T>& P, const T Bm[9], T F[9], T& Jp, T FP[9],
                                         Split<T>& sp, T* s_out = nullptr, T* sm1_out = nullptr,
                                         T* V_out = nullptr) {
    T Fs[9];
    f_star(P, Bm, F, Fs);
    update_F_star<T, TRACK_FP>(P, Fs, F, Jp, FP, sp, s_out, sm1_out, V_out);
}

// scale * P F^T of F = U sc V^T (the split just made), as stress_PFt computes
// it from an SVD of F: U diag(2 mu (sc - d) sc) U^T + lambda (J - 1) J I with
// J = sgn prod sc and J - 1 expanded in sc - 1 so nothing cancels.  The
// matrix is symmetric; its entries 00 01 02 11 12 22 go to out, each formed
// as sum_k (U_rk U_ck) dg_k so that the rounding is symmetric too.
template <typename T>
__device__ __forceinline__ void stress_from_split(const DevParams<T>& P, const Split<T>& sp, T Jp, T scale,
                                                  T out[6]) {
    const T e0 = sp.scm1[0], e1 = sp.scm1[1], e2 = sp.scm1[2];
    const T pm1 = (e0 + e1 + e2) + (e0 * e1 + e0 * e2 + e1 * e2) + e0 * e1 * e2;  // prod sc - 1
    const T J = sp.sgn > T(0) ? T(1) + pm1 : -(T(1) + pm1);
    const T jm1 = sp.sgn > T(0) ? pm1 : J - T(1);
    const T hard = exp_(P.xi * (T(1) - Jp));
    const T mu = P.mu0 * hard, lam = P.lambda0 * hard;
    int kmin = 0;
#pragma unroll
    for (int c = 1; c < 3; ++c) kmin = sp.sc[c] < sp.sc[kmin] ? c : kmin;
    T dg[3];
#pragma unroll
    for (int c = 0; c < 3; ++c) {
        const T sm = (J < T(0) && c == kmin) ? (sp.sc[c] + T(1)) : sp.scm1[c];
        dg[c] = T(2) * mu * sm * sp.sc[c];
    }
    const T iso = lam * jm1 * J;
    int k = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = r; c < 3; ++c, ++k)
            out[k] = scale * ((sp.U[3 * r] * sp.U[3 * c]) * dg[0] + (sp.U[3 * r + 1] * sp.U[3 * c + 1]) * dg[1] +
                              (sp.U[3 * r + 2] * sp.U[3 * c + 2]) * dg[2] + (r == c ? iso : T(0)));
}

// Index into the 6 entries of a symmetric 3x3 matrix (00 01 02 11 12 22).
__host__ __device__ constexpr int sym6(int r, int c) {
    return r <= c ? (r == 0 ? c : (r == 1 ? 2 + c : 5)) : (c == 0 ? r : (c == 1 ? 2 + r : 5));
}

// ---------------------------------------------------------------- stress without an SVD
// S = F^T F - I as 6 entries (sym6), formed from G = F - I as svd3_near forms
// it, and det F - 1 expanded in G (trace, principal 2x2 minors,
// determinant), so neither cancels when F is near the identity.
template <typename T>
__device__ __forceinline__ void strain_of(const T F[9], T S[6], T& jm1) {
    T G[9];
#pragma unroll
    for (int e = 0; e < 9; ++e) G[e] = F[e];
    G[0] -= T(1); G[4] -= T(1); G[8] -= T(1);
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int c = r; c < 3; ++c)
            S[sym6(r, c)] = (G[3 * r + c] + G[3 * c + r]) + (G[r] * G[c] + G[3 + r] * G[3 + c] + G[6 + r] * G[6 + c]);
    jm1 = (G[0] + G[4] + G[8]) + ((G[0] * G[4] - G[1] * G[3]) + (G[0] * G[8] - G[2] * G[6]) +
                                  (G[4] * G[8] - G[5] * G[7])) + det3(G);
}

// Sylvester's criterion: the symmetric matrix is positive definite when its
// leading principal minors are positive (false for NaN).
template <typename T>
__device__ __forceinline__ bool pos_def(T m00, T m01, T m02, T m11, T m12, T m22) {
    const T d2 = m00 * m11 - m01 * m01;
    const T d3 = m00 * (m11 * m22 - m12 * m12) - m01 * (m01 * m22 - m12 * m02) + m02 * (m01 * m12 - m11 * m02);
    return m00 > T(0) && d2 > T(0) && d3 > T(0);
}

// Whether an F_E* with strain S and det - 1 jm1 (strain_of) is clamped
// nowhere: every eigenvalue e_i = s_i^2 - 1 of S inside (P.elo, P.ehi), that
// is S - elo I and ehi I - S positive definite, and det F_E* > 0.  The host
// sets elo = lo^2 - 1 and ehi = hi^2 - 1 moved inwards by 1e-5, far more than
// the rounding of this test or of the singular values svd3_near finds, so a
// particle accepted here is one that update_F would leave unclamped too.
template <typename T>
__device__ __forceinline__ bool inside_clamp(const DevParams<T>& P, const T S[6], T jm1) {
    const T a = P.elo, b = P.ehi;
    return jm1 > T(-1) && pos_def(S[0] - a, S[1], S[2], S[3] - a, S[4], S[5] - a) &&
           pos_def(b - S[0], -S[1], -S[2], b - S[3], -S[4], b - S[5]);
}

// scale * P F^T for an F that inside_clamp accepted (so F_E = F_E*, J_P and
// F_P unchanged), without an SVD.  The polar factor is R = F (I + S)^(-1/2),
// so F - R = F Q with Q = I - (I + S)^(-1/2) = sum_k q_k S^k,
// q_k = (-1)^(k+1) C(2k, k) / 4^k (the binomial series, exact binary
// fractions), and 2 mu (F - R) F^T = 2 mu F Q F^T; with F = U S V^T this is
// the U diag(2 mu (s - 1) s) U^T of stress_from_split.  The series is summed
// through the Cayley-Hamilton theorem: S^3 = I1 S^2 - I2 S + I3 I with the
// invariants of S, so S^k = a_k I + b_k S + c_k S^2 with scalar recurrences
// and Q = alpha I + beta S + gamma S^2.  Seven terms: the host uses this
// only while |e_i| <= 0.1, where the first term left out, q_8 e^8, is below
// 4e-8 of Q's eigenvalue (about e / 2).  The isotropic part lambda (J - 1) J uses J - 1 from strain_of.
template <typename T>
__device__ __forceinline__ void stress_direct(const DevParams<T>& P, const T F[9], const T S[6], T jm1, T Jp,
                                              T scale, T out[6]) {
    const T I1 = S[0] + S[3] + S[5];
    const T c00 = S[3] * S[5] - S[4] * S[4], c11 = S[0] * S[5] - S[2] * S[2], c22 = S[0] * S[3] - S[1] * S[1];
    const T I2 = c00 + c11 + c22;
    const T I3 = S[0] * c00 - S[1] * (S[1] * S[5] - S[4] * S[2]) + S[2] * (S[1] * S[4] - S[3] * S[2]);
    constexpr T q[8] = {T(0), T(1) / T(2), T(-3) / T(8), T(5) / T(16), T(-35) / T(128), T(63) / T(256),
                        T(-231) / T(1024), T(429) / T(2048)};
    // S^2 is (a, b, c) = (0, 0, 1); S^1 and S^2 give beta = q1, gamma = q2
    T a = T(0), b = T(0), c = T(1);
    T al = T(0), be = q[1], ga = q[2];
#pragma unroll
    for (int k = 3; k <= 7; ++k) {
        const T an = c * I3, bn = a - c * I2, cn = b + c * I1;
        a = an; b = bn; c = cn;
        al += q[k] * a; be += q[k] * b; ga += q[k] * c;
    }
    T Q[9];
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = r; cc < 3; ++cc) {
            const T s2 = S[sym6(r, 0)] * S[sym6(0, cc)] + S[sym6(r, 1)] * S[sym6(1, cc)] +
                         S[sym6(r, 2)] * S[sym6(2, cc)];
            const T v = be * S[sym6(r, cc)] + ga * s2 + (r == cc ? al : T(0));
            Q[3 * r + cc] = v;
            Q[3 * cc + r] = v;
        }
    T FQ[9];
    matmul3(FQ, F, Q);
    const T hard = exp_(P.xi * (T(1) - Jp));
    const T mu2 = T(2) * (P.mu0 * hard), lam = P.lambda0 * hard;
    const T iso = lam * jm1 * (T(1) + jm1);
    int k = 0;
#pragma unroll
    for (int r = 0; r < 3; ++r)
#pragma unroll
        for (int cc = r; cc < 3; ++cc, ++k)
            out[k] = scale * (mu2 * (FQ[3 * r] * F[3 * cc] + FQ[3 * r + 1] * F[3 * cc + 1] +
                                     FQ[3 * r + 2] * F[3 * cc + 2]) + (r == cc ? iso : T(0)));
}

template <typename T>
__device__ __forceinline__ T clampx(T x, T lo, T hi) { return x < lo ? lo : (hi < x ? hi : x); }

template <typename T>
__device__ __forceinline__ bool wall_node(const DevParams<T>& P, int i, int j, int k) {
    const int w = P.bc_width;
    return i < w || j < w || k < w || i >= P.M[0] - w || j >= P.M[1] - w || k >= P.M[2] - w;
}

template <typename T>
__device__ __forceinline__ void tile_origin(const DevParams<T>& P, int gkey, int org[3]) {
    const int key = gkey - (int)P.block_base;
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

// ---------------------------------------------------------------- grid marks
// Every kernel that adds to a grid buffer marks the 4x4x4 node blocks it may
// have written (one byte per block, indexed like the sort blocks), so that
// k_grid_clear zeroes only those blocks before the buffer is filled again.

// Marks the blocks within one block of block key (a tile of P2G nodes
// spans at most the neighbouring blocks).
template <typename T>
__device__ __forceinline__ void mark_around_block(const DevParams<T>& P, uint8_t* marks, int bx, int by, int bz) {
    const int t = threadIdx.x;
    if (t >= 27) return;
    const int nx = bx + t / 9 - 1, ny = by + (t / 3) % 3 - 1, nz = bz + t % 3 - 1;
    if (nx < 0 || ny < 0 || nz < 0 || nx >= P.NB[0] || ny >= P.NB[1] || nz >= P.NB[2]) return;
    marks[P.block_base + (nx * P.NB[1] + ny) * P.NB[2] + nz] = 1;
}
template <typename T>
__device__ __forceinline__ void mark_around(const DevParams<T>& P, uint8_t* marks, int gkey) {
    const int key = gkey - (int)P.block_base;
    mark_around_block(P, marks, key / (P.NB[1] * P.NB[2]), (key / P.NB[2]) % P.NB[1], key % P.NB[2]);
}

// Marks the blocks holding nodes b - 1 .. b + 2 (one particle's stencil).
template <typename T>
__device__ __forceinline__ void mark_stencil(const DevParams<T>& P, uint8_t* marks, const int b[3]) {
    int lo[3], hi[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) {
        lo[a] = max(b[a] - 1, 0) / kBlk;
        hi[a] = min(b[a] + 2, P.M[a] - 1) / kBlk;
    }
    for (int x = lo[0]; x <= hi[0]; ++x)
        for (int y = lo[1]; y <= hi[1]; ++y)
            for (int z = lo[2]; z <= hi[2]; ++z) marks[P.block_base + (x * P.NB[1] + y) * P.NB[2] + z] = 1;
}

// Zeroes the node blocks marked in marks and clears the marks: a warp looks
// at 32 blocks, each lane finds its block's scene and grid geometry, then the
// warp zeroes the marked blocks one after the other (two nodes a lane).
template <typename T, bool BATCH>
__global__ void __launch_bounds__(256) k_grid_clear(DevParams<T> P0, DevBufs D, vec4<T>* __restrict__ grid0,
                                                    uint8_t* __restrict__ marks, int nblocks) {
    const int lane = threadIdx.x & 31;
    const int warp = (int)((blockIdx.x * blockDim.x + threadIdx.x) >> 5);
    const int nwarps = (int)((gridDim.x * blockDim.x) >> 5);
    for (int b0 = warp * 32; b0 < nblocks; b0 += nwarps * 32) {
        const int mine = b0 + lane;
        const bool m = mine < nblocks && marks[mine] != 0;
        int key = 0, nb1 = 1, nb2 = 1, m0 = 0, m1 = 0, m2 = 0;
        unsigned long long goff = 0;
        if (m) {
            const DevParams<T>* sp = &P0;
            if (BATCH)
                sp = static_cast<const DevParams<T>*>(D.scenes) + scene_of(D.sblock, D.nscenes, (uint32_t)mine);
            key = mine - (int)sp->block_base;
            nb1 = sp->NB[1]; nb2 = sp->NB[2];
            m0 = sp->M[0]; m1 = sp->M[1]; m2 = sp->M[2];
            goff = sp->goff;
        }
        uint32_t todo = __ballot_sync(0xffffffffu, m);
        while (todo) {
            const int l = __ffs(todo) - 1;
            todo &= todo - 1;
            const int k = __shfl_sync(0xffffffffu, key, l);
            const int NB1 = __shfl_sync(0xffffffffu, nb1, l), NB2 = __shfl_sync(0xffffffffu, nb2, l);
            const int M0 = __shfl_sync(0xffffffffu, m0, l), M1 = __shfl_sync(0xffffffffu, m1, l);
            const int M2 = __shfl_sync(0xffffffffu, m2, l);
            const unsigned long long go = __shfl_sync(0xffffffffu, goff, l);
            const int bz = k % NB2, by = (k / NB2) % NB1, bx = k / (NB1 * NB2);
            vec4<T>* grid = grid0 + go;
#pragma unroll
            for (int q = 0; q < 2; ++q) {
                const int node = lane + 32 * q;  // 0..63: x = node / 16, y = (node / 4) % 4, z = node % 4
                const int gx = bx * kBlk + node / 16, gy = by * kBlk + (node / 4) % 4, gz = bz * kBlk + node % 4;
                if (gx < M0 && gy < M1 && gz < M2)
                    grid[((size_t)gx * M1 + gy) * M2 + gz] = mk4<T>(T(0), T(0), T(0), T(0));
            }
        }
        if (m) marks[mine] = 0;
    }
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
template <> struct WorkP<float> { static constexpr int value = 256; };
template <> struct WorkP<double> { static constexpr int value = 128; };

constexpr int kRecV4 = 7;

// Shared memory of the P2G phase for a cell space of CA^3 base cells and a
// (CA + 3)^3-node tile.
template <typename T, int CA> struct P2GTile {
    static constexpr int TS = CA + 3;
    static constexpr int TC = TS * TS * TS;
    static constexpr int NC = CA * CA * CA;
    alignas(16) T tile[4 * TC];
    vec4<T> rec[WorkP<T>::value * kRecV4];
    int cnt[NC];
    int off[NC];
    uint16_t order[WorkP<T>::value];
    uint8_t cellof[WorkP<T>::value];
    uint8_t scell[WorkP<T>::value];  // cell of each sorted slot
};

// Zeroes the four channel planes of a P2G tile with 16-byte stores.
template <typename T, int CA>
__device__ __forceinline__ void zero_tile(P2GTile<T, CA>& S) {
    static_assert((4 * P2GTile<T, CA>::TC * sizeof(T)) % 16 == 0, "16-byte stores");
    float4* t = reinterpret_cast<float4*>(S.tile);
    for (int c = threadIdx.x; c < (int)(4 * P2GTile<T, CA>::TC * sizeof(T) / 16); c += blockDim.x)
        t[c] = make_float4(0.f, 0.f, 0.f, 0.f);
}

template <typename T> __device__ __forceinline__ T pick4(const vec4<T>& v, int i) {
    return i == 0 ? v.x : (i == 1 ? v.y : (i == 2 ? v.z : v.w));
}

// The record of one particle: node base - 1 + o receives w_o (m, q' + h A o),
// q' = m v + A e with e = (base - 1) h - x.  r[0], r[1]: the x and y weights
// at offsets 0..3; r[2]: the z weights in the order 0, 2, 1, 3, so that the two
// z nodes of a scatter lane (oz and oz + 2) are adjacent; r[3] = (q', m);
// r[4..6]: h A.
template <typename T, bool MOM>
__device__ __forceinline__ void write_record(vec4<T>* r, const Stencil<T>& St, const T x[3], const T A[9],
                                             const T mv[3], T m, T h) {
    T e3[3];
#pragma unroll
    for (int a = 0; a < 3; ++a) e3[a] = (T)(St.b[a] - 1) * h - x[a];
    T qp[3];
#pragma unroll
    for (int r = 0; r < 3; ++r) qp[r] = mv[r] + (A[3 * r] * e3[0] + A[3 * r + 1] * e3[1] + A[3 * r + 2] * e3[2]);
    r[0] = mk4<T>(St.w[0][0], St.w[0][1], St.w[0][2], St.w[0][3]);
    r[1] = mk4<T>(St.w[1][0], St.w[1][1], St.w[1][2], St.w[1][3]);
    r[2] = mk4<T>(St.w[2][0], St.w[2][2], St.w[2][1], St.w[2][3]);  // z pairs (0, 2), (1, 3)
    r[3] = mk4<T>(qp[0], qp[1], qp[2], MOM ? m : T(0));
    r[4] = mk4<T>(h * A[0], h * A[3], h * A[6], h * A[1]);
    r[5] = mk4<T>(h * A[4], h * A[7], h * A[2], h * A[5]);
    r[6] = mk4<T>(h * A[8], T(0), T(0), T(0));
}

// Counting sort of the records by cell: S.cnt holds the counts on entry and
// again on exit, S.off the offsets, S.order the record index per slot.
// Called by every thread of the block.
template <typename T, int CA>
__device__ __forceinline__ void sort_records(P2GTile<T, CA>& S, int count) {
    constexpr int NC = P2GTile<T, CA>::NC;
    constexpr int PER = (NC + 31) / 32;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int l = threadIdx.x;
        int loc[PER];
        int tot = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int c = l * PER + k;
            loc[k] = c < NC ? S.cnt[c] : 0;
            tot += loc[k];
        }
        int x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (l >= o) x += y;
        }
        int run = x - tot;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int c = l * PER + k;
            if (c < NC) { S.off[c] = run; S.cnt[c] = run; }
            run += loc[k];
        }
    }
    __syncthreads();
    for (int j = threadIdx.x; j < count; j += blockDim.x) {
        const int c = S.cellof[j];
        if (c != 0xff) {
            const int k = atomicAdd(&S.cnt[c], 1);
            S.order[k] = (uint16_t)j;
            S.scell[k] = (uint8_t)c;
        }
    }
    __syncthreads();
    for (int c = threadIdx.x; c < NC; c += blockDim.x) S.cnt[c] -= S.off[c];
    __syncthreads();
}

// Phase 2, warp-cooperative: the warps of the block split the cell-sorted
// records into contiguous runs; within a warp every lane owns two of the 64
// stencil nodes (ox = l / 8, oy = (l / 2) % 4, oz = l % 2 and l % 2 + 2) and
// all lanes walk the run together, so each record is read by broadcast and
// contributes to all 64 nodes at once.  A lane keeps (m, q) of its two nodes
// in registers while consecutive records share a base cell and adds them to
// the shared tile when the cell changes.
template <typename T, int CA>
__device__ __forceinline__ void p2g_flush_lane(P2GTile<T, CA>& S, int c, int ox, int oy, int oz0, const T am[2],
                                               const T aq[2][3], bool mom) {
    constexpr int TS = P2GTile<T, CA>::TS;
    constexpr int TC = P2GTile<T, CA>::TC;
    const int cz = c % CA, cy = (c / CA) % CA, cx = c / (CA * CA);
#pragma unroll
    for (int k = 0; k < 2; ++k) {
        const int node = ((cx + ox) * TS + (cy + oy)) * TS + (cz + oz0 + 2 * k);
        if (!RD_IN_BOUNDS(node, TC) || !RD_IN_BOUNDS(c, (P2GTile<T, CA>::NC))) continue;
        if (mom) atomicAdd(&S.tile[node], am[k]);
        atomicAdd(&S.tile[TC + node], aq[k][0]);
        atomicAdd(&S.tile[2 * TC + node], aq[k][1]);
        atomicAdd(&S.tile[3 * TC + node], aq[k][2]);
    }
}

// Counting sort of the records by cell when every record already holds its
// rank among its cell's records (the value its count atomic returned): one
// scan of the counts into S.off, then each thread places its own record
// (cell 0xff: none).  S.cnt keeps the counts.  Called by every thread.
template <typename T, int CA>
__device__ __forceinline__ void sort_ranked(P2GTile<T, CA>& S, int j, int cell, int rank) {
    constexpr int NC = P2GTile<T, CA>::NC;
    constexpr int PER = (NC + 31) / 32;
    __syncthreads();
    if (threadIdx.x < 32) {
        const int l = threadIdx.x;
        int loc[PER];
        int tot = 0;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int c = l * PER + k;
            loc[k] = c < NC ? S.cnt[c] : 0;
            tot += loc[k];
        }
        int x = tot;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const int y = __shfl_up_sync(0xffffffffu, x, o);
            if (l >= o) x += y;
        }
        int run = x - tot;
#pragma unroll
        for (int k = 0; k < PER; ++k) {
            const int c = l * PER + k;
            if (c < NC) S.off[c] = run;
            run += loc[k];
        }
    }
    __syncthreads();
    if (cell != 0xff && RD_IN_BOUNDS(cell, NC)) {
        const int k = S.off[cell] + rank;
        if (RD_IN_BOUNDS(k, WorkP<T>::value)) {
            S.order[k] = (uint16_t)j;
            S.scell[k] = (uint8_t)cell;
        }
    }
    __syncthreads();
}

// Sorted slots holding a record after sort_records / sort_ranked (records of
// cell 0xff are not placed).
template <typename T, int CA> __device__ __forceinline__ int sorted_total(const P2GTile<T, CA>& S) {
    return S.off[P2GTile<T, CA>::NC - 1] + S.cnt[P2GTile<T, CA>::NC - 1];
}

// total: the slots 0 .. total - 1 of S.order / S.scell hold the records, the
// records of one cell contiguous.
template <typename T, bool MOM, int CA>
__device__ __forceinline__ void p2g_tasks(P2GTile<T, CA>& S, int total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int ox = lane >> 3, oy = (lane >> 1) & 3, oz0 = lane & 1;
    const T fx = (T)ox, fy = (T)oy, fz = (T)oz0;
    // a warp's share of the slots (total <= WorkP, so 32-bit products)
    const int k0 = (int)((unsigned)(total * warp) / (unsigned)nwarps);
    const int k1 = (int)((unsigned)(total * (warp + 1)) / (unsigned)nwarps);
    const T* recs = reinterpret_cast<const T*>(S.rec);
    int cur = -1;
    if constexpr (sizeof(T) == 4) {
        // FP32: the lane's two nodes (z offsets oz0 and oz0 + 2) as float2
        // pairs, two FMAs per instruction
        const float2 fzz = make_float2(fz, fz + 2.f);
        float2 am2 = make_float2(0.f, 0.f), qx2 = am2, qy2 = am2, qz2 = am2;
        for (int k = k0; k < k1; ++k) {
            const int j = S.order[k];
            const int c = S.scell[k];
            if (c != cur) {
                if (cur >= 0) {
                    const T am[2] = {am2.x, am2.y};
                    const T aq[2][3] = {{qx2.x, qy2.x, qz2.x}, {qx2.y, qy2.y, qz2.y}};
                    p2g_flush_lane<T, CA>(S, cur, ox, oy, oz0, am, aq, MOM);
                }
                cur = c;
                am2 = qx2 = qy2 = qz2 = make_float2(0.f, 0.f);
            }
            const T* rs = recs + j * (4 * kRecV4);
            const float wxy = rs[ox] * rs[4 + oy];
            const float2 w = __fmul2_rn(make_float2(wxy, wxy), *reinterpret_cast<const float2*>(rs + 8 + 2 * oz0));
            const vec4<T>* r = &S.rec[j * kRecV4];
            const vec4<T> qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
            // q' + h A o: the x and y offsets are common to both nodes
            const float cx = qm.x + a4.x * fx + a4.w * fy;
            const float cy = qm.y + a4.y * fx + b4.x * fy;
            const float cz = qm.z + a4.z * fx + b4.y * fy;
            const float2 px = __ffma2_rn(make_float2(b4.z, b4.z), fzz, make_float2(cx, cx));
            const float2 py = __ffma2_rn(make_float2(b4.w, b4.w), fzz, make_float2(cy, cy));
            const float2 pz = __ffma2_rn(make_float2(c4.x, c4.x), fzz, make_float2(cz, cz));
            if (MOM) am2 = __ffma2_rn(w, make_float2(qm.w, qm.w), am2);
            qx2 = __ffma2_rn(w, px, qx2);
            qy2 = __ffma2_rn(w, py, qy2);
            qz2 = __ffma2_rn(w, pz, qz2);
        }
        if (cur >= 0) {
            const T am[2] = {am2.x, am2.y};
            const T aq[2][3] = {{qx2.x, qy2.x, qz2.x}, {qx2.y, qy2.y, qz2.y}};
            p2g_flush_lane<T, CA>(S, cur, ox, oy, oz0, am, aq, MOM);
        }
    } else {
        T am[2] = {T(0), T(0)}, aq[2][3] = {{T(0), T(0), T(0)}, {T(0), T(0), T(0)}};
        for (int k = k0; k < k1; ++k) {
            const int j = S.order[k];
            const int c = S.scell[k];
            if (c != cur) {
                if (cur >= 0) p2g_flush_lane<T, CA>(S, cur, ox, oy, oz0, am, aq, MOM);
                cur = c;
                am[0] = am[1] = T(0);
                aq[0][0] = aq[0][1] = aq[0][2] = aq[1][0] = aq[1][1] = aq[1][2] = T(0);
            }
            const T* rs = recs + j * (4 * kRecV4);
            const T wxy = rs[ox] * rs[4 + oy];
            const T w0 = wxy * rs[8 + 2 * oz0], w1 = wxy * rs[9 + 2 * oz0];
            const vec4<T>* r = &S.rec[j * kRecV4];
            const vec4<T> qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
            // q' + h A o; h A columns x (a4.x, a4.y, a4.z), y (a4.w, b4.x, b4.y), z (b4.z, b4.w, c4.x)
            const T q0x = qm.x + a4.x * fx + a4.w * fy + b4.z * fz;
            const T q0y = qm.y + a4.y * fx + b4.x * fy + b4.w * fz;
            const T q0z = qm.z + a4.z * fx + b4.y * fy + c4.x * fz;
            const T q1x = q0x + T(2) * b4.z, q1y = q0y + T(2) * b4.w, q1z = q0z + T(2) * c4.x;
            if (MOM) { am[0] += w0 * qm.w; am[1] += w1 * qm.w; }
            aq[0][0] += w0 * q0x; aq[0][1] += w0 * q0y; aq[0][2] += w0 * q0z;
            aq[1][0] += w1 * q1x; aq[1][1] += w1 * q1y; aq[1][2] += w1 * q1z;
        }
        if (cur >= 0) p2g_flush_lane<T, CA>(S, cur, ox, oy, oz0, am, aq, MOM);
    }
}

// p2g_tasks by runs: a warp takes its share of the sorted slots as runs of
// one cell, each run's end known from the cell's offset and count (S.off,
// S.cnt after sort_ranked), so the loop over a run carries no per-record cell
// load or test; a lane accumulates while the run lasts and flushes once.
template <typename T, bool MOM, int CA>
__device__ __forceinline__ void p2g_runs(P2GTile<T, CA>& S, int total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int ox = lane >> 3, oy = (lane >> 1) & 3, oz0 = lane & 1;
    const T fx = (T)ox, fy = (T)oy, fz = (T)oz0;
    // a warp's share of the slots (total <= WorkP, so 32-bit products)
    const int k0 = (int)((unsigned)(total * warp) / (unsigned)nwarps);
    const int k1 = (int)((unsigned)(total * (warp + 1)) / (unsigned)nwarps);
    const T* recs = reinterpret_cast<const T*>(S.rec);
    int k = k0;
    if constexpr (sizeof(T) == 4) {
        const float2 fzz = make_float2(fz, fz + 2.f);
        while (k < k1) {
            const int c = S.scell[k];
            if (!RD_IN_BOUNDS(c, (P2GTile<T, CA>::NC))) break;
            const int e = min(S.off[c] + S.cnt[c], k1);
            float2 am2 = make_float2(0.f, 0.f), qx2 = am2, qy2 = am2, qz2 = am2;
#pragma unroll 1
            for (; k < e; ++k) {
                const int j = S.order[k];
                if (!RD_IN_BOUNDS(j, WorkP<T>::value)) continue;
                const T* rs = recs + j * (4 * kRecV4);
                const float wxy = rs[ox] * rs[4 + oy];
                const float2 w = __fmul2_rn(make_float2(wxy, wxy), *reinterpret_cast<const float2*>(rs + 8 + 2 * oz0));
                const vec4<T>* r = &S.rec[j * kRecV4];
                const vec4<T> qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
                const float cx = qm.x + a4.x * fx + a4.w * fy;
                const float cy = qm.y + a4.y * fx + b4.x * fy;
                const float cz = qm.z + a4.z * fx + b4.y * fy;
                const float2 px = __ffma2_rn(make_float2(b4.z, b4.z), fzz, make_float2(cx, cx));
                const float2 py = __ffma2_rn(make_float2(b4.w, b4.w), fzz, make_float2(cy, cy));
                const float2 pz = __ffma2_rn(make_float2(c4.x, c4.x), fzz, make_float2(cz, cz));
                if (MOM) am2 = __ffma2_rn(w, make_float2(qm.w, qm.w), am2);
                qx2 = __ffma2_rn(w, px, qx2);
                qy2 = __ffma2_rn(w, py, qy2);
                qz2 = __ffma2_rn(w, pz, qz2);
            }
            const T am[2] = {am2.x, am2.y};
            const T aq[2][3] = {{qx2.x, qy2.x, qz2.x}, {qx2.y, qy2.y, qz2.y}};
            p2g_flush_lane<T, CA>(S, c, ox, oy, oz0, am, aq, MOM);
        }
    } else {
        while (k < k1) {
            const int c = S.scell[k];
            if (!RD_IN_BOUNDS(c, (P2GTile<T, CA>::NC))) break;
            const int e = min(S.off[c] + S.cnt[c], k1);
            T am[2] = {T(0), T(0)}, aq[2][3] = {{T(0), T(0), T(0)}, {T(0), T(0), T(0)}};
            for (; k < e; ++k) {
                const int j = S.order[k];
                if (!RD_IN_BOUNDS(j, WorkP<T>::value)) continue;
                const T* rs = recs + j * (4 * kRecV4);
                const T wxy = rs[ox] * rs[4 + oy];
                const T w0 = wxy * rs[8 + 2 * oz0], w1 = wxy * rs[9 + 2 * oz0];
                const vec4<T>* r = &S.rec[j * kRecV4];
                const vec4<T> qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
                const T q0x = qm.x + a4.x * fx + a4.w * fy + b4.z * fz;
                const T q0y = qm.y + a4.y * fx + b4.x * fy + b4.w * fz;
                const T q0z = qm.z + a4.z * fx + b4.y * fy + c4.x * fz;
                const T q1x = q0x + T(2) * b4.z, q1y = q0y + T(2) * b4.w, q1z = q0z + T(2) * c4.x;
                if (MOM) { am[0] += w0 * qm.w; am[1] += w1 * qm.w; }
                aq[0][0] += w0 * q0x; aq[0][1] += w0 * q0y; aq[0][2] += w0 * q0z;
                aq[1][0] += w1 * q1x; aq[1][1] += w1 * q1y; aq[1][2] += w1 * q1z;
            }
            p2g_flush_lane<T, CA>(S, c, ox, oy, oz0, am, aq, MOM);
        }
    }
}

// p2g_runs for FP32 with the two half-warps on two records of the same run at
// once: a lane owns the four nodes of one z column (ox, oy) of the 4 x 4 x 4
// stencil, so 16 lanes cover a record and each warp instruction serves two
// records.  A lane keeps two node pairs as float2: its own pair S0 and the
// pair S1 that its partner lane (lane ^ 16, the same column in the other
// half) owns - half 0 owns z offsets {0, 2}, half 1 {1, 3} - so at the end of
// a run each lane sends S1 to its partner with one shuffle per value, adds
// what it receives to S0 and flushes its two nodes, as p2g_runs does.  A run
// of odd length gives the last record to half 0; half 1 adds zero weight.
template <bool MOM, int CA>
__device__ __forceinline__ void p2g_runs_pairs(P2GTile<float, CA>& S, int total) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarps = blockDim.x >> 5;
    const int hw = lane >> 4, col = lane & 15;
    const int ox = col >> 2, oy = col & 3;
    const float fx = (float)ox, fy = (float)oy;
    // z offsets of the pairs: record z weights are stored in the order 0, 2, 1, 3
    const float2 fz0 = hw ? make_float2(1.f, 3.f) : make_float2(0.f, 2.f);
    const float2 fz1 = hw ? make_float2(0.f, 2.f) : make_float2(1.f, 3.f);
    const int wz0 = 8 + 2 * hw, wz1 = 10 - 2 * hw;
    // a warp's share of the slots (total <= WorkP, so 32-bit products)
    const int k0 = (int)((unsigned)(total * warp) / (unsigned)nwarps);
    const int k1 = (int)((unsigned)(total * (warp + 1)) / (unsigned)nwarps);
    const float* recs = reinterpret_cast<const float*>(S.rec);
    int k = k0;
    while (k < k1) {
        const int c = S.scell[k];
        if (!RD_IN_BOUNDS(c, (P2GTile<float, CA>::NC))) break;
        const int e = min(S.off[c] + S.cnt[c], k1);
        float2 m0 = make_float2(0.f, 0.f), x0 = m0, y0 = m0, z0 = m0, m1 = m0, x1 = m0, y1 = m0, z1 = m0;
        for (int kb = k; kb < e; kb += 2) {
            const bool mine = kb + hw < e;
            const int kk = S.order[mine ? kb + hw : kb];
            if (!RD_IN_BOUNDS(kk, WorkP<float>::value)) continue;
            const float* rs = recs + kk * (4 * kRecV4);
            const float wxy = mine ? rs[ox] * rs[4 + oy] : 0.f;
            const float2 w0 = __fmul2_rn(make_float2(wxy, wxy), *reinterpret_cast<const float2*>(rs + wz0));
            const float2 w1 = __fmul2_rn(make_float2(wxy, wxy), *reinterpret_cast<const float2*>(rs + wz1));
            const float4* r = &S.rec[kk * kRecV4];
            const float4 qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
            const float cx = qm.x + a4.x * fx + a4.w * fy;
            const float cy = qm.y + a4.y * fx + b4.x * fy;
            const float cz = qm.z + a4.z * fx + b4.y * fy;
            if (MOM) {
                m0 = __ffma2_rn(w0, make_float2(qm.w, qm.w), m0);
                m1 = __ffma2_rn(w1, make_float2(qm.w, qm.w), m1);
            }
            x0 = __ffma2_rn(w0, __ffma2_rn(make_float2(b4.z, b4.z), fz0, make_float2(cx, cx)), x0);
            y0 = __ffma2_rn(w0, __ffma2_rn(make_float2(b4.w, b4.w), fz0, make_float2(cy, cy)), y0);
            z0 = __ffma2_rn(w0, __ffma2_rn(make_float2(c4.x, c4.x), fz0, make_float2(cz, cz)), z0);
            x1 = __ffma2_rn(w1, __ffma2_rn(make_float2(b4.z, b4.z), fz1, make_float2(cx, cx)), x1);
            y1 = __ffma2_rn(w1, __ffma2_rn(make_float2(b4.w, b4.w), fz1, make_float2(cy, cy)), y1);
            z1 = __ffma2_rn(w1, __ffma2_rn(make_float2(c4.x, c4.x), fz1, make_float2(cz, cz)), z1);
        }
        k = e;
        // the partner's pair S1 comes over, this lane's S1 goes to the partner
        m0.x += __shfl_xor_sync(0xffffffffu, m1.x, 16); m0.y += __shfl_xor_sync(0xffffffffu, m1.y, 16);
        x0.x += __shfl_xor_sync(0xffffffffu, x1.x, 16); x0.y += __shfl_xor_sync(0xffffffffu, x1.y, 16);
        y0.x += __shfl_xor_sync(0xffffffffu, y1.x, 16); y0.y += __shfl_xor_sync(0xffffffffu, y1.y, 16);
        z0.x += __shfl_xor_sync(0xffffffffu, z1.x, 16); z0.y += __shfl_xor_sync(0xffffffffu, z1.y, 16);
        const float am[2] = {m0.x, m0.y};
        const float aq[2][3] = {{x0.x, y0.x, z0.x}, {x0.y, y0.y, z0.y}};
        p2g_flush_lane<float, CA>(S, c, ox, oy, hw, am, aq, MOM);
    }
}

// Adds the tile (origin org) to the grid: one vector reduction per node that
// received anything.
template <typename T, int CA>
__device__ __forceinline__ void p2g_flush(const DevParams<T>& P, const P2GTile<T, CA>& S, const int org[3],
                                          vec4<T>* __restrict__ grid, int x0 = 0,
                                          int x1 = P2GTile<T, CA>::TS - 1) {
    constexpr int TS = P2GTile<T, CA>::TS;
    constexpr int TC = P2GTile<T, CA>::TC;
    // only the x layers x0..x1 of the tile can hold anything
    for (int c = x0 * TS * TS + (int)threadIdx.x; c < (x1 + 1) * TS * TS; c += blockDim.x) {
        const int ix = c / (TS * TS), iy = (c / TS) % TS, iz = c % TS;
        const int gx = org[0] + ix, gy = org[1] + iy, gz = org[2] + iz;
        if (gx < 0 || gy < 0 || gz < 0 || gx >= P.M[0] || gy >= P.M[1] || gz >= P.M[2]) continue;
        const vec4<T> v = mk4<T>(S.tile[c], S.tile[TC + c], S.tile[2 * TC + c], S.tile[3 * TC + c]);
        const size_t lin = ((size_t)gx * P.M[1] + gy) * P.M[2] + gz;
        if (!RD_IN_BOUNDS(lin, (size_t)P.M[0] * P.M[1] * P.M[2])) continue;
        if (v.x != T(0) || v.y != T(0) || v.z != T(0) || v.w != T(0)) red_add4(grid + lin, v);
    }
}

// Direct scatter of one record to the grid, for a particle outside its
// block's cell space (moved more than one cell in a step).
template <typename T>
__device__ void p2g_direct(const DevParams<T>& P, const vec4<T>* r, const int b[3], vec4<T>* __restrict__ grid) {
    const vec4<T> wx4 = r[0], wy4 = r[1], wz4 = r[2], qm = r[3], a4 = r[4], b4 = r[5], c4 = r[6];
    const T wx[4] = {wx4.x, wx4.y, wx4.z, wx4.w}, wy[4] = {wy4.x, wy4.y, wy4.z, wy4.w},
            wz[4] = {wz4.x, wz4.z, wz4.y, wz4.w};
    for (int ox = 0; ox < 4; ++ox)
        for (int oy = 0; oy < 4; ++oy)
            for (int oz = 0; oz < 4; ++oz) {
                const int gx = b[0] - 1 + ox, gy = b[1] - 1 + oy, gz = b[2] - 1 + oz;
                if (gx < 0 || gy < 0 || gz < 0 || gx >= P.M[0] || gy >= P.M[1] || gz >= P.M[2]) continue;
                const T w = (wx[ox] * wy[oy]) * wz[oz];
                const T fo[3] = {(T)ox, (T)oy, (T)oz};
                const T q0 = qm.x + a4.x * fo[0] + a4.w * fo[1] + b4.z * fo[2];
                const T q1 = qm.y + a4.y * fo[0] + b4.x * fo[1] + b4.w * fo[2];
                const T q2 = qm.z + a4.z * fo[0] + b4.y * fo[1] + c4.x * fo[2];
                red_add4(grid + ((size_t)gx * P.M[1] + gy) * P.M[2] + gz, mk4<T>(w * qm.w, w * q0, w * q1, w * q2));
            }
}

// One work item of k_p2g; P is the item's scene.
template <typename T, bool MOM, bool FORCE>
__device__ __forceinline__ void p2g_item(const DevParams<T>& P, const DevBufs& D, P2GTile<T, kBlk>& S,
                                         const int4 it) {
    const vec4<T>* __restrict__ pl = static_cast<const vec4<T>*>(D.pin);
    vec4<T>* __restrict__ grid = static_cast<vec4<T>*>(MOM ? D.grid : D.gforce) + P.goff;
    const size_t n = (size_t)P.n;
    zero_tile(S);
    for (int c = threadIdx.x; c < P2GTile<T, kBlk>::NC; c += blockDim.x) S.cnt[c] = 0;
    int org[3];
    tile_origin(P, it.x, org);
    const int count = min(it.z, min(WorkP<T>::value, P.n - it.y));
    __syncthreads();
    bool stray = false;  // a record outside the cell space, or one whose cell is not its key's
    // phase 1: a record per particle
    for (int j = threadIdx.x; j < count; j += blockDim.x) {
        if (!RD_IN_BOUNDS(it.y + j, n) || !RD_IN_BOUNDS(D.perm[it.y + j], n)) {
            S.cellof[j] = 0xff;
            S.scell[j] = 0;
            stray = true;
            continue;
        }
        Particle<T> p;
        load_particle(pl, n, D.perm[it.y + j], p);
        if (D.reorder_out) {  // the particle to its sorted position
            store_particle(static_cast<vec4<T>*>(D.reorder_out), n, (size_t)(it.y + j), p);
            D.perm_reset[it.y + j] = (uint32_t)(it.y + j);
        }
        Stencil<T> St;
        if (!make_stencil(P, p.x, org, St)) {
            raise_flag(D.flags, 4u);
            S.cellof[j] = 0xff;
            stray = true;
            continue;
        }
        if (!stencil_in_grid(P, St.b)) {
            raise_flag(D.flags, 1u);
            // a base cell past the grid's end was clamped in its sort key, so
            // its record's cell need not be its key's: sort the records
            stray = stray || St.b[0] > P.M[0] - 1 || St.b[1] > P.M[1] - 1 || St.b[2] > P.M[2] - 1;
        }
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
            if (D.stress) load_stress(static_cast<const vec4<T>*>(D.stress), n, D.perm[it.y + j], G);
            else stress_PFt(P, p.F, p.Jp, G);
            const T sc = P.fscale * (p.vol * P.dinv);
#pragma unroll
            for (int e = 0; e < 9; ++e) A[e] -= sc * G[e];
        }
        write_record<T, MOM>(&S.rec[j * kRecV4], St, p.x, A, mv, p.m, P.h);
        const int cell = (St.rel[0] * kBlk + St.rel[1]) * kBlk + St.rel[2];
        S.cellof[j] = (uint8_t)cell;
        S.order[j] = (uint16_t)j;
        S.scell[j] = (uint8_t)cell;
    }
    // The item is a run of the global sort by cell key and nothing has moved
    // since, so its records are grouped by cell already, in item order: the
    // slot after each cell's last record is its run's end (p2g_runs reads
    // off + cnt, so off = 0 and cnt = end).  Only a particle outside the cell
    // space or with a clamped key (flagged above) needs the record sort.
    int total = count;
    if (__syncthreads_or(stray)) {
        for (int j = threadIdx.x; j < count; j += blockDim.x)
            if (S.cellof[j] != 0xff) atomicAdd(&S.cnt[S.cellof[j]], 1);
        sort_records<T, kBlk>(S, count);
        total = sorted_total(S);
    } else {
        for (int j = threadIdx.x; j < count; j += blockDim.x) {
            const int c = S.scell[j];
            if (j + 1 == count || S.scell[j + 1] != c) {
                S.off[c] = 0;
                S.cnt[c] = j + 1;
            }
        }
        __syncthreads();
    }
    p2g_runs<T, MOM, kBlk>(S, total);
    __syncthreads();
    p2g_flush<T, kBlk>(P, S, org, grid);
    if (MOM) mark_around(P, D.gmark, it.x);
    __syncthreads();
}

// k_p2g runs one particle per thread, three CTAs per SM in FP32: a work
// item's particle loads (through the sort permutation, scattered when the
// state was just uploaded) are all in flight at once.
template <typename T> constexpr int kP2GThreads = WorkP<T>::value;

template <typename T> struct P2GShared {
    P2GTile<T, kBlk> t;
    DevParams<T> par;  // the item's scene (batches)
};

// BATCH: the work items belong to different scenes (D.scenes); otherwise all
// to the scene P0.
template <typename T, bool MOM, bool FORCE, bool BATCH>
__global__ void __launch_bounds__(kP2GThreads<T>, sizeof(T) == 4 ? 3 : 1) k_p2g(DevParams<T> P0, DevBufs D) {
    extern __shared__ __align__(32) unsigned char smem_raw[];
    P2GShared<T>& S = *reinterpret_cast<P2GShared<T>*>(smem_raw);
    uint32_t nf, nb;
    work_counts(D, nf, nb);
    const uint32_t nw = nf + nb;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = work_item(D, nf, wi);
        if constexpr (BATCH) {
            copy_scene(S.par, D.scenes, it.w);
            __syncthreads();
            p2g_item<T, MOM, FORCE>(S.par, D, S.t, it);
        } else {
            p2g_item<T, MOM, FORCE>(P0, D, S.t, it);
        }
    }
}

// ---------------------------------------------------------------- fused G2P2G
// One step for one work item per loop trip: gridVelocitiesUpdate,
// updateDeformationGradient, updateParticleVelocities and
// updateParticlePositions of this step (material_point_method.cpp:256-262,
// 306-350), then rasterizeParticlesToGrid + computeExplicitGridForces of the
// next step (:94-129,235-254) into the other grid buffer.
//   * The 7^3 tile of grid n arrives as (m, p = m v + dt f) and becomes
//     v = p / m + dt g (zero where m = 0 and on sticky walls) in shared memory.
//   * A thread per particle: G2P, the plastic split, advection; the particle
//     is written at its sorted slot of the other plane buffer and its next
//     block key is counted; then its P2G record at x_{n+1}, whose stress comes
//     from the split just made (no second SVD).
//   * The records are scattered into a 9^3 tile of grid n+1 around the block
//     (base cells within one cell of the block, 6^3 cell space); a particle
//     that moved further goes straight to the grid.
// The force of the next step uses this step's dt: rd_step recomputes the grid
// with k_p2g when dt changes.
constexpr int kFusedThreads = 256;
// Three resident CTAs per SM in FP32 (at most 85 registers a thread): the
// scatter loop is latency-bound and the kernel runs 10% faster with 24 warps
// per SM than with 16, more than the spills of the per-particle phase cost.
constexpr int kFusedMinBlocks = 3;
static_assert(WorkP<float>::value <= kFusedThreads && WorkP<double>::value <= kFusedThreads,
              "k_g2p2g runs at most one particle per thread");
template <typename T> struct FusedShared {
    alignas(128) vec4<T> graw[kTileCells];  // (m, p) tile of this step's grid, copied by TMA
    vec4<T> gv[kTileCells];  // grid velocity of this step, (vx, vy, vz, 0)
    P2GTile<T, kBlk + 2> p;
    DevParams<T> par;        // the item's scene (batches)
    uint64_t tbar;           // mbarrier of the tile copy
    int org[3];              // tile origin of the item whose tile is (being) copied
    uint32_t wi_next;        // the work item this CTA claimed next
    uint32_t wi_ahead;       // thread 0: the one claimed after it
    int2 next_span;          // first sorted slot and particle count of the next item
};
// Dynamic shared memory of k_g2p2g: the struct plus room to align it to the
// 128 bytes a TMA destination needs.
template <typename T> constexpr size_t fused_smem_bytes() { return sizeof(FusedShared<T>) + 128; }

// Polls of a tile copy's mbarrier before the kernel gives up (RD_FLAG_WAIT_TIMEOUT).
constexpr int kTileWaitTries = 1 << 16;
// After giving up, the CTA stays resident until the copy it issued has landed
// (a bulk copy cannot be cancelled, and it writes this CTA's shared memory):
// up to this many rounds of kTileWaitTries / 64 polls, each followed by a
// 64 us sleep - a second or more in all - before it leaves regardless.
constexpr int kTileDrainRounds = 16384;

// The tile-copy wait on an mbarrier that no copy and no thread arrives at:
// it must give up after `tries` polls and report it.
__global__ void k_wait_probe(int tries, uint32_t* flags, int* gave_up) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) mbar_init(&bar);
    __syncthreads();
    const bool arrived = mbar_wait(&bar, 0u, tries);
    if (__syncthreads_or(!arrived)) {
        if (threadIdx.x == 0) {
            raise_flag(flags, 8u);
            *gave_up = 1;
        }
    }
}

// Tensor maps of a launch's grid tiles, passed by value as the fused
// kernel's __grid_constant__ parameter, so a copy reads a map that is
// constant for the launch and never one in memory the host rewrites: one for
// a single scene, one per scene for the first kBatchMaps scenes of a batch
// (the tiles of later scenes are loaded by the threads themselves).
constexpr int kBatchMaps = 128;
template <int N> struct TileMaps {
    CUtensorMap m[N];
};
template <bool BATCH> using FusedMaps = TileMaps<BATCH ? kBatchMaps : 1>;

// One thread (always thread 0): the grid tile of work item `it` (the kTile^3
// nodes from its tile origin) into S.graw by TMA with `map`, the tensor map
// of the item's scene region of this step's grid.
// The origin also goes to S.org, where the item reads it (one set of
// divisions per item instead of one per thread).
template <typename T>
__device__ __forceinline__ void issue_tile(const DevParams<T>& P, const CUtensorMap* map, FusedShared<T>& S,
                                           int4 it) {
    int org[3];
    tile_origin(P, it.x, org);
    S.org[0] = org[0]; S.org[1] = org[1]; S.org[2] = org[2];
    tma_load_4d(S.graw, map, &S.tbar, (uint32_t)(kTileCells * sizeof(vec4<T>)), org[2], org[1], org[0]);
}

// All threads: the grid tile of work item `it` (scene P, the kTile^3 nodes
// from its tile origin; nodes outside the scene's grid as zero) into S.graw
// with plain loads, for a batch scene without a tensor map; the caller
// synchronises before use.
template <typename T>
__device__ __forceinline__ void load_tile(const DevParams<T>& P, const DevBufs& D, FusedShared<T>& S, int4 it) {
    int org[3];
    tile_origin(P, it.x, org);
    if (threadIdx.x == 0) { S.org[0] = org[0]; S.org[1] = org[1]; S.org[2] = org[2]; }
    const vec4<T>* g = static_cast<const vec4<T>*>(D.grid) + P.goff;
    for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
        size_t lin;
        S.graw[c] = cell_of_tile(P, org, c, lin) ? g[lin] : mk4<T>(T(0), T(0), T(0), T(0));
    }
}

// G2P of one particle from the velocity tile (updateParticleVelocities,
// material_point_method.cpp:332-342): v_p = sum w v_i and
// B_p = sum w v_i (x_i - x_p)^T, evaluated separably: with w = wx wy wz and
// (x_i - x_p) = (dx[ox], dy[oy], dz[oz]), the z sums of each (ox, oy) column
// are formed first (sum wz v and sum wz dz v), then weighted by wy, wy dy and
// by wx, wx dx.
template <typename T>
__device__ __forceinline__ void g2p_gather(const vec4<T>* __restrict__ gv, const Stencil<T>& St, T vp[3], T Bp[9]) {
    T wzd[4], wyd[4];
#pragma unroll
    for (int o = 0; o < 4; ++o) { wzd[o] = St.w[2][o] * St.d[2][o]; wyd[o] = St.w[1][o] * St.d[1][o]; }
#pragma unroll
    for (int r = 0; r < 3; ++r) vp[r] = T(0);
#pragma unroll
    for (int e = 0; e < 9; ++e) Bp[e] = T(0);
#pragma unroll
    for (int ox = 0; ox < 4; ++ox) {
        T sx[3] = {T(0), T(0), T(0)}, sy[3] = {T(0), T(0), T(0)}, sz[3] = {T(0), T(0), T(0)};
#pragma unroll
        for (int oy = 0; oy < 4; ++oy) {
            T col[3] = {T(0), T(0), T(0)}, colz[3] = {T(0), T(0), T(0)};
            const int rowc = ((St.rel[0] + ox) * kTile + (St.rel[1] + oy)) * kTile + St.rel[2];
            if constexpr (sizeof(T) == 4) {
                // (sum wz v, sum wz dz v) of each velocity component as one pair
                float2 c0 = make_float2(0.f, 0.f), c1 = c0, c2 = c0;
#pragma unroll
                for (int oz = 0; oz < 4; ++oz) {
                    const vec4<T> v = RD_IN_BOUNDS(rowc + oz, kTileCells) ? gv[rowc + oz] : mk4<T>(T(0), T(0), T(0), T(0));
                    const float2 wz2 = make_float2(St.w[2][oz], wzd[oz]);
                    c0 = __ffma2_rn(wz2, make_float2(v.x, v.x), c0);
                    c1 = __ffma2_rn(wz2, make_float2(v.y, v.y), c1);
                    c2 = __ffma2_rn(wz2, make_float2(v.z, v.z), c2);
                }
                col[0] = c0.x; colz[0] = c0.y; col[1] = c1.x; colz[1] = c1.y; col[2] = c2.x; colz[2] = c2.y;
            } else {
#pragma unroll
                for (int oz = 0; oz < 4; ++oz) {
                    const vec4<T> v = RD_IN_BOUNDS(rowc + oz, kTileCells) ? gv[rowc + oz] : mk4<T>(T(0), T(0), T(0), T(0));
                    col[0] += St.w[2][oz] * v.x; col[1] += St.w[2][oz] * v.y; col[2] += St.w[2][oz] * v.z;
                    colz[0] += wzd[oz] * v.x; colz[1] += wzd[oz] * v.y; colz[2] += wzd[oz] * v.z;
                }
            }
#pragma unroll
            for (int r = 0; r < 3; ++r) {
                sx[r] += St.w[1][oy] * col[r];
                sy[r] += wyd[oy] * col[r];
                sz[r] += St.w[1][oy] * colz[r];
            }
        }
        const T wx = St.w[0][ox], wxd = St.w[0][ox] * St.d[0][ox];
#pragma unroll
        for (int r = 0; r < 3; ++r) {
            vp[r] += wx * sx[r];
            Bp[3 * r + 0] += wxd * sx[r];
            Bp[3 * r + 1] += wx * sy[r];
            Bp[3 * r + 2] += wx * sz[r];
        }
    }
}

// updateDeformationGradient of one particle with velocity gradient Bm (the
// lagged B, or the one just gathered): F_E, J_P (and F_P) updated and
// stored (planes 5-6 and the F_P planes), the finite check of those, and
// the scaled stress sc P F^T of the next P2G as 6 symmetric entries.
// FP32, when the split is not kept for the adjoint: a warp whose particles
// are all clamped nowhere (inside_clamp) takes F_E = F_E* and the stress from
// stress_direct, with no SVD; any other warp runs the SVD for all its
// particles, so the two paths never run one after the other in a warp.
template <typename T, bool TRACK_FP>
__device__ __forceinline__ void split_particle(const DevParams<T>& P, Particle<T>& p, T FP[9], const T Bm[9],
                                               vec4<T>* __restrict__ pout, size_t n, size_t s, T G6[6],
                                               bool& finite, void* split_out) {
    T Fs[9];
    f_star(P, Bm, p.F, Fs);
    const T scale = P.fscale * (p.vol * P.dinv);
    bool direct = false;
    if constexpr (sizeof(T) == 4) {
        if (!split_out && P.elo < P.ehi) {
            T S6[6], jm1;
            strain_of(Fs, S6, jm1);
            direct = __all_sync(__activemask(), inside_clamp(P, S6, jm1));
            if (direct) {
                stress_direct(P, Fs, S6, jm1, p.Jp, scale, G6);
#pragma unroll
                for (int e = 0; e < 9; ++e) p.F[e] = Fs[e];
            }
        }
    }
    if (!direct) {
        Split<T> sp;
        T sv[3], svm1[3], V[9];
        update_F_star<T, TRACK_FP>(P, Fs, p.F, p.Jp, FP, sp, sv, svm1, V);
        if (split_out) store_split(static_cast<vec4<T>*>(split_out), n, s, sp.U, sv, svm1, V);
        stress_from_split(P, sp, p.Jp, scale, G6);
    }
    store_particle_back(pout, n, s, p);
    if (TRACK_FP) store_fp(pout, n, s, FP);
    // a NaN or infinity anywhere makes the sum non-finite (the values are far
    // from overflowing)
    T sum = p.Jp;
#pragma unroll
    for (int e = 0; e < 9; ++e) sum += p.F[e];
    finite = isfinite(sum);
}

// One work item of k_g2p2g; P is the item's scene.  LAGGED: the F update
// uses the B of the previous G2P (the reference's order), else the B just
// gathered.  The item's grid tile is in S.graw; once it is converted,
// thread 0 copies the next item's tile (nit) in by TMA while this item runs,
// with maps[0] for a single scene or maps[scene] for a batch scene that has a
// map (the next item's scene parameters from the batch's table).  The next
// item was claimed one item ago (S.wi_ahead); this item's flush claims the
// one after it and reads the next item's permutation entries into pf.  BATCH: P is the item's scene copied to shared memory, and
// the item ends on a barrier.
template <typename T, bool TRACK_FP, bool LAGGED, bool PAIRS, bool BATCH>
__device__ __forceinline__ void g2p2g_item(const DevParams<T>& P, const DevBufs& D, FusedShared<T>& S,
                                           const int4 it, uint32_t nf, uint32_t nw, const CUtensorMap* maps,
                                           uint32_t& pf, bool& pf_ok) {
    static_assert(!PAIRS || sizeof(T) == 4, "the record-pairs scatter is FP32");
    constexpr int CA = kBlk + 2;
    const vec4<T>* __restrict__ pin = static_cast<const vec4<T>*>(D.pin);
    vec4<T>* __restrict__ pout = static_cast<vec4<T>*>(D.pout);
    vec4<T>* __restrict__ gnext = static_cast<vec4<T>*>(D.grid_next) + P.goff;
    const size_t n = (size_t)P.n;
    {
        // the origin thread 0 stored when it copied this tile (published by
        // the barrier after the tile wait); it writes the next item's only
        // after the barrier that follows the tile conversion
        const int org[3] = {S.org[0], S.org[1], S.org[2]};
        const int porg[3] = {org[0] - 1, org[1] - 1, org[2] - 1};
        const int count = min(it.z, min(WorkP<T>::value, P.n - it.y));
        // one particle per thread (WorkP == blockDim): start its loads before
        // the tile is staged so the two latencies overlap
        // (the permutation entry was read during the previous item's flush
        // when this CTA had one)
        const int j = threadIdx.x;
        const uint32_t src = pf_ok ? pf : (j < count ? D.perm[it.y + j] : 0u);
        const bool mine = j < count && RD_IN_BOUNDS(it.y + j, n) && RD_IN_BOUNDS(src, n);
        Particle<T> p;
        T FP[9];
        if (mine) {
            load_particle(pin, n, src, p);
            if (TRACK_FP) load_fp(pin, n, src, FP);
        }
        // thread 0 holds the next item's index, claimed during the previous
        // item's flush: its work item is read now, the load passing while the
        // tile is converted
        uint32_t wn = 0u;
        int4 nit = make_int4(0, 0, 0, 0);
        if (threadIdx.x == 0) {
            wn = S.wi_ahead;
            if (wn < nw) nit = work_item(D, nf, wn);
        }
        // the (m, p) tile arrived by TMA (nodes outside the grid read as
        // zero): the grid update, walls and colliders into velocities
        // a tile clear of the sticky walls (most of them) skips the per-node test
        const int bw = P.bc_width;
        const bool walls = P.bc == 1 && (org[0] < bw || org[1] < bw || org[2] < bw || org[0] + kTile > P.M[0] - bw ||
                                         org[1] + kTile > P.M[1] - bw || org[2] + kTile > P.M[2] - bw);
        for (int c = threadIdx.x; c < kTileCells; c += blockDim.x) {
            T v0 = T(0), v1 = T(0), v2 = T(0);
            const vec4<T> g4 = S.graw[c];
            if (g4.x != T(0)) {
                const T im = rcp_fast(g4.x);
                v0 = g4.y * im + P.dt * P.g[0];
                v1 = g4.z * im + P.dt * P.g[1];
                v2 = g4.w * im + P.dt * P.g[2];
                const int ix = c / (kTile * kTile), iy = (c / kTile) % kTile, iz = c % kTile;
                if (walls && wall_node(P, org[0] + ix, org[1] + iy, org[2] + iz)) v0 = v1 = v2 = T(0);
                if (P.ncol) {
                    T vv[3] = {v0, v1, v2};
                    collide_node(P, static_cast<const Collider<T>*>(D.colliders), (T)(org[0] + ix) * P.h,
                                 (T)(org[1] + iy) * P.h, (T)(org[2] + iz) * P.h, vv);
                    v0 = vv[0]; v1 = vv[1]; v2 = vv[2];
                }
            }
            S.gv[c] = mk4<T>(v0, v1, v2, T(0));
        }
        zero_tile(S.p);
        for (int c = threadIdx.x; c < P2GTile<T, CA>::NC; c += blockDim.x) S.p.cnt[c] = 0;
        __syncthreads();
        // S.graw is free again: copy the next item's tile while this one runs
        // (the later barriers of this item publish S.wi_next)
        if (threadIdx.x == 0) {
            S.wi_next = wn;
            S.next_span = make_int2(nit.y, wn < nw ? max(0, min(nit.z, min(WorkP<T>::value, P.n - nit.y))) : 0);
            if (wn < nw) {
                if constexpr (BATCH) {
                    if (nit.w < kBatchMaps)
                        issue_tile(static_cast<const DevParams<T>*>(D.scenes)[nit.w], maps + nit.w, S, nit);
                } else {
                    issue_tile(P, maps, S, nit);
                }
            }
        }
        int rcell = 0xff, rrank = 0;  // this thread's record: cell and rank within it
        if (mine) {
            const int s = it.y + j;
            // the plastic split first: the stress of the next P2G (6 entries)
            // and the F_E / J_P / F_P planes are final after it, so none of the
            // split is live across the gather
            T G6[6];
            bool finite = true;
            // the stress, m, V, the id and x wait in this thread's record slot
            // (written only after the gather), holding no registers across it
            vec4<T>* stash = &S.p.rec[j * kRecV4 + 4];
            if constexpr (LAGGED) {
                split_particle<T, TRACK_FP>(P, p, FP, p.B, pout, n, s, G6, finite, D.split_out);
                stash[0] = mk4<T>(G6[0], G6[1], G6[2], G6[3]);
                stash[1] = mk4<T>(G6[4], G6[5], p.m, p.vol);
                stash[2] = mk4<T>(id_to_real<T>(p.id), p.x[0], p.x[1], p.x[2]);
            }
            Stencil<T> St;
            const bool ok = make_stencil(P, p.x, org, St);
            if (!ok) raise_flag(D.flags, 4u);
            T vp[3] = {T(0), T(0), T(0)};
            T Bp[9];
#pragma unroll
            for (int e = 0; e < 9; ++e) Bp[e] = T(0);
            if (ok) g2p_gather(S.gv, St, vp, Bp);
            if constexpr (LAGGED) {
                const vec4<T> a = stash[0], b = stash[1], c = stash[2];
                G6[0] = a.x; G6[1] = a.y; G6[2] = a.z; G6[3] = a.w; G6[4] = b.x; G6[5] = b.y;
                p.m = b.z; p.vol = b.w; p.id = real_to_id<T>(c.x);
                p.x[0] = c.y; p.x[1] = c.z; p.x[2] = c.w;
            }
            if constexpr (!LAGGED) split_particle<T, TRACK_FP>(P, p, FP, Bp, pout, n, s, G6, finite, D.split_out);
#pragma unroll
            for (int a = 0; a < 3; ++a) p.v[a] = vp[a];
#pragma unroll
            for (int e = 0; e < 9; ++e) p.B[e] = Bp[e];
#pragma unroll
            for (int a = 0; a < 3; ++a) p.x[a] = clampx(p.x[a] + p.v[a] * P.dt, P.xlo, P.xhi[a]);
            store_particle_front(pout, n, s, p);
            if (D.slot_of && p.id < (uint32_t)n) D.slot_of[p.id] = (uint32_t)s;
            {
                T sum = (p.x[0] + p.x[1]) + (p.x[2] + p.v[0]) + (p.v[1] + p.v[2]);
#pragma unroll
                for (int e = 0; e < 9; ++e) sum += p.B[e];
                finite = finite && isfinite(sum);
            }
            if (!finite) raise_flag(D.flags, 2u);
            // next step's P2G record
            Stencil<T> S2;
            const bool in_space = make_stencil(P, p.x, porg, S2, CA - 1);
            const uint32_t key = sort_key(P, S2.b);
            D.keys_out[s] = key;
            count_key(D.counts, D.bcount, key);
            if (!stencil_in_grid(P, S2.b)) raise_flag(D.flags, 1u);
            T A[9], mv[3];
#pragma unroll
            for (int r = 0; r < 3; ++r)
#pragma unroll
                for (int c = 0; c < 3; ++c) A[3 * r + c] = p.m * (p.B[3 * r + c] * P.dinv) - G6[sym6(r, c)];
#pragma unroll
            for (int a = 0; a < 3; ++a) mv[a] = p.m * p.v[a];
            vec4<T>* rec = &S.p.rec[j * kRecV4];
            write_record<T, true>(rec, S2, p.x, A, mv, p.m, P.h);
            if (in_space && RD_IN_BOUNDS((S2.rel[0] * CA + S2.rel[1]) * CA + S2.rel[2], (P2GTile<T, CA>::NC))) {
                rcell = (S2.rel[0] * CA + S2.rel[1]) * CA + S2.rel[2];
                S.p.cellof[j] = (uint8_t)rcell;
                rrank = atomicAdd(&S.p.cnt[rcell], 1);
            } else {
                S.p.cellof[j] = 0xff;
                p2g_direct(P, rec, S2.b, gnext);
                mark_stencil(P, D.gmark_next, S2.b);
            }
        }
        sort_ranked<T, CA>(S.p, j, rcell, rrank);
        const int total = sorted_total(S.p);
        if constexpr (PAIRS) p2g_runs_pairs<true, CA>(S.p, total);
        else p2g_runs<T, true, CA>(S.p, total);
        // the records are sorted by cell, x-major: the first and the last give
        // the x layers of the tile the scatter touched (cell x .. x + 3)
        const int x0 = total > 0 ? S.p.scell[0] / (CA * CA) : 0;
        const int x1 = total > 0 ? S.p.scell[total - 1] / (CA * CA) + 3 : -1;
        __syncthreads();
        // thread 0 claims the item after the next one; the atomic's round trip
        // passes during the flush
        uint32_t claim = nw;
        if (threadIdx.x == 0 && S.wi_next < nw) claim = atomicAdd(D.claim, 1u);
        // each thread reads its particle's permutation entry for the next item
        {
            const int2 sp = S.next_span;
            pf = j < sp.y ? D.perm[sp.x + j] : 0u;
            pf_ok = true;
        }
        p2g_flush<T, CA>(P, S.p, porg, gnext, x0, x1);
        mark_around_block(P, D.gmark_next, (org[0] + 1) / kBlk, (org[1] + 1) / kBlk, (org[2] + 1) / kBlk);
        if (threadIdx.x == 0) S.wi_ahead = claim;
        // a single scene: the next item's first barrier (after its tile wait)
        // separates this flush from the next item's writes to shared memory; a
        // batch copies the next scene's parameters before that barrier
        if (BATCH) __syncthreads();
    }
}

// BATCH: the work items belong to different scenes (D.scenes); otherwise all
// to the scene P0.  Tiles come by TMA with the maps of `maps` (TileMaps),
// except in batch scenes past the first kBatchMaps, whose items load their
// tiles with plain loads.  PAIRS: the scatter's lane layout p2g_runs_pairs
// (FP32) instead of p2g_runs; the autotuner picks one.
template <typename T, bool TRACK_FP, bool BATCH, bool LAGGED, bool PAIRS = false>
__global__ void __launch_bounds__(kFusedThreads, sizeof(T) == 4 ? kFusedMinBlocks : 1)
    k_g2p2g(DevParams<T> P0, DevBufs D, const __grid_constant__ FusedMaps<BATCH> maps) {
    extern __shared__ __align__(128) unsigned char smem_fused[];
    FusedShared<T>& S =
        *reinterpret_cast<FusedShared<T>*>(smem_fused + ((128u - (smem_addr(smem_fused) & 127u)) & 127u));
    const DevParams<T>* scenes = static_cast<const DevParams<T>*>(D.scenes);
    uint32_t nf, nb;
    work_counts(D, nf, nb);
    const uint32_t nw = nf + nb;
    // items are claimed one at a time from D.claim, so CTAs that drew small
    // items take more of them (each CTA holds the next item and the one after
    // it); the next launch's counter is this launch's predecessor's,
    // finished, and is zeroed here
    if (blockIdx.x == 0 && threadIdx.x == 0) *D.claim_next = 0u;
    if (threadIdx.x == 0) {
        mbar_init(&S.tbar);
        const uint32_t w0 = atomicAdd(D.claim, 1u);
        S.wi_next = w0;
        S.wi_ahead = w0 < nw ? atomicAdd(D.claim, 1u) : nw;
        if (w0 < nw) {
            const int4 it0 = work_item(D, nf, w0);
            if constexpr (BATCH) {
                if (it0.w < kBatchMaps) issue_tile(scenes[it0.w], &maps.m[it0.w], S, it0);
            } else {
                issue_tile(P0, &maps.m[0], S, it0);
            }
        }
    }
    __syncthreads();
    // the k-th TMA tile of this CTA completes phase k & 1 of the mbarrier; the
    // next item's copy is issued inside g2p2g_item once this tile is
    // converted, and the item after it claimed
    uint32_t parity = 0u;
    uint32_t pf = 0u;    // this thread's permutation entry of the next item
    bool pf_ok = false;  // (read during the previous item's flush)
    for (uint32_t wi = S.wi_next; wi < nw; wi = S.wi_next) {
        const int4 it = work_item(D, nf, wi);
        bool arrived = true;
        if constexpr (BATCH) {
            copy_scene(S.par, D.scenes, it.w);
            if (it.w >= kBatchMaps) load_tile(scenes[it.w], D, S, it);
        }
        if (!BATCH || it.w < kBatchMaps) {
            arrived = mbar_wait(&S.tbar, parity, kTileWaitTries);
            parity ^= 1u;
        }
        // every thread decides together (this barrier also publishes S.par
        // and a loaded tile)
        if (__syncthreads_or(!arrived)) {
            if (threadIdx.x == 0) {
                raise_flag(D.flags, 8u);
                // the copy in flight (this item's) lands in this CTA's shared
                // memory: wait for it before the CTA exits, bounded
                for (int r = 0; r < kTileDrainRounds; ++r) {
                    if (mbar_wait(&S.tbar, parity ^ 1u, kTileWaitTries / 64)) break;
                    __nanosleep(64000);
                }
            }
            return;
        }
        if constexpr (BATCH)
            g2p2g_item<T, TRACK_FP, LAGGED, PAIRS, true>(S.par, D, S, it, nf, nw, &maps.m[0], pf, pf_ok);
        else
            g2p2g_item<T, TRACK_FP, LAGGED, PAIRS, false>(P0, D, S, it, nf, nw, &maps.m[0], pf, pf_ok);
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

// gridBasedCollisions as its own stage (grid holds (m, v)), in place.
template <typename T>
__global__ void k_grid_collide(DevParams<T> P, vec4<T>* __restrict__ grid, const Collider<T>* __restrict__ cols) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nc = (size_t)P.M[0] * P.M[1] * P.M[2];
    if (c >= nc) return;
    vec4<T> g = grid[c];
    if (g.x == T(0)) return;
    const int k = (int)(c % P.M[2]), j = (int)((c / P.M[2]) % P.M[1]), i = (int)(c / ((size_t)P.M[1] * P.M[2]));
    T vv[3] = {g.y, g.z, g.w};
    collide_node(P, cols, (T)i * P.h, (T)j * P.h, (T)k * P.h, vv);
    g.y = vv[0]; g.z = vv[1]; g.w = vv[2];
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
    Split<T> sp;
    update_F<T, TRACK_FP>(P, p.B, p.F, p.Jp, FP, sp);
    store_particle(pl, n, i, p);
    if (TRACK_FP) store_fp(pl, n, i, FP);
}

// updateParticleVelocities as its own stage (grid holds (m, v)), in place.
template <typename T>
__global__ void __launch_bounds__(kThreads) k_g2p_stage(DevParams<T> P, DevBufs D) {
    __shared__ T sv[3 * kTileCells];
    vec4<T>* __restrict__ pl = static_cast<vec4<T>*>(D.pout);
    const vec4<T>* __restrict__ grid = static_cast<const vec4<T>*>(D.grid);
    uint32_t nf, nb;
    work_counts(D, nf, nb);
    const uint32_t nw = nf + nb;
    const size_t n = (size_t)P.n;
    for (uint32_t wi = blockIdx.x; wi < nw; wi += gridDim.x) {
        const int4 it = work_item(D, nf, wi);
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
template <typename T, bool BATCH>
__global__ void k_volumes(DevParams<T> P0, DevBufs D, vec4<T>* __restrict__ pl, const vec4<T>* __restrict__ grid0) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= P0.n) return;
    uint32_t* flags = D.flags;
    DevParams<T> P;
    if (BATCH) P = static_cast<const DevParams<T>*>(D.scenes)[scene_of(D.spoff, D.nscenes, (uint32_t)i)];
    else P = P0;
    const vec4<T>* __restrict__ grid = grid0 + P.goff;
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
// fused mode (m, p) -> v = p / m + dt g (+ walls) as k_g2p2g stages it.
template <typename T, bool FUSED>
__global__ void k_grid_export(DevParams<T> P, const vec4<T>* __restrict__ grid, T* __restrict__ mass,
                              T* __restrict__ vel, const Collider<T>* __restrict__ cols) {
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
            if (P.ncol) {
                T vv[3] = {v0, v1, v2};
                collide_node(P, cols, (T)i * P.h, (T)j * P.h, (T)k * P.h, vv);
                v0 = vv[0]; v1 = vv[1]; v2 = vv[2];
            }
        }
    }
    if (mass) mass[c] = g.x;
    if (vel) { vel[3 * c] = v0; vel[3 * c + 1] = v1; vel[3 * c + 2] = v2; }
}

// ---------------------------------------------------------------- diagnostics
// Block sums of k values per thread into acc (double atomics, one per block and value).
template <int K>
__device__ __forceinline__ void block_sum_to(double (&v)[K], double* __restrict__ acc) {
    __shared__ double part[K][8];
#pragma unroll
    for (int k = 0; k < K; ++k) {
        double x = v[k];
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0) part[k][threadIdx.x >> 5] = x;
    }
    __syncthreads();
    if (threadIdx.x < K) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += part[threadIdx.x][w];
        if (t != 0.0) atomicAdd(acc + threadIdx.x, t);
    }
}

// particleMomentum, mass, averageParticleDensity, averageDeformationGradient
// (material_point_method.cpp:361-367,410-421,437-443) over particles [off, off + cnt):
// acc = mass | momentum 3 | sum m / V | count V > 0 | sum F_E F_P 9.
template <typename T>
__global__ void __launch_bounds__(256) k_diag_particles(int off, int cnt, int ntot, const vec4<T>* __restrict__ pl,
                                                        int track_fp, double* __restrict__ acc) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double v[15];
#pragma unroll
    for (int k = 0; k < 15; ++k) v[k] = 0.0;
    if (i < cnt) {
        Particle<T> p;
        load_particle(pl, (size_t)ntot, (size_t)(off + i), p);
        v[0] = (double)p.m;
#pragma unroll
        for (int a = 0; a < 3; ++a) v[1 + a] = (double)p.m * (double)p.v[a];
        if (p.vol > T(0)) { v[4] = (double)p.m / (double)p.vol; v[5] = 1.0; }
        T FP[9];
        if (track_fp) {
            load_fp(pl, (size_t)ntot, (size_t)(off + i), FP);
        } else {
            const T c = cbrt(p.Jp);
#pragma unroll
            for (int e = 0; e < 9; ++e) FP[e] = (e % 4 == 0) ? c : T(0);
        }
        T F[9];
        matmul3(F, p.F, FP);
#pragma unroll
        for (int e = 0; e < 9; ++e) v[6 + e] = (double)F[e];
    }
    block_sum_to<15>(v, acc);
}

// gridMass, gridMomentum (material_point_method.cpp:352-359,370-376) and the
// used-cell count over a scene's grid, its velocities as G2P reads them (in
// fused mode v = p / m + dt g, then walls and colliders): acc = mass |
// momentum 3 | count.
template <typename T, bool FUSED>
__global__ void __launch_bounds__(256) k_diag_grid(DevParams<T> P, const vec4<T>* __restrict__ grid,
                                                   const Collider<T>* __restrict__ cols, double* __restrict__ acc) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    const size_t nc = (size_t)P.M[0] * P.M[1] * P.M[2];
    double v[5] = {0.0, 0.0, 0.0, 0.0, 0.0};
    if (c < nc) {
        const vec4<T> g = grid[c];
        if (g.x != T(0)) {
            T vv[3] = {g.y, g.z, g.w};
            if (FUSED) {
                const int k = (int)(c % P.M[2]), j = (int)((c / P.M[2]) % P.M[1]),
                          i = (int)(c / ((size_t)P.M[1] * P.M[2]));
                vv[0] = g.y / g.x + P.dt * P.g[0];
                vv[1] = g.z / g.x + P.dt * P.g[1];
                vv[2] = g.w / g.x + P.dt * P.g[2];
                if (P.bc == 1 && wall_node(P, i, j, k)) vv[0] = vv[1] = vv[2] = T(0);
                if (P.ncol) collide_node(P, cols, (T)i * P.h, (T)j * P.h, (T)k * P.h, vv);
            }
            v[0] = (double)g.x;
#pragma unroll
            for (int a = 0; a < 3; ++a) v[1 + a] = (double)g.x * (double)vv[a];
            v[4] = 1.0;
        }
    }
    block_sum_to<5>(v, acc);
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
