// lbm_step_vec.cu -- physics-mode step with four cells per thread (phys_cells4_update of
// lbm_cell4.cuh): one aligned vector load and store per population plane and thread,
// warp shuffles for the +-x shifted directions.  Requires nx % 4 == 0.
//
// Algorithmic traffic per cell update: 9 loads + 9 stores of the stored type (72 B FP32,
// 36 B FP16/BF16, 144 B FP64) plus the 2-byte flag word.
#include <algorithm>

#include "lbm_cell4.cuh"
#include "lbm_cell_tiled.cuh"
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbm {

constexpr int VEC_TPB = 128;  // 512 cells of a row per block

template <class ST, bool MACRO, class IDX>
__global__ void __launch_bounds__(VEC_TPB) k_phys_step_v4(const typename ST::T* __restrict__ A,
                                                          typename ST::T* __restrict__ B, uint16_t* __restrict__ flags,
                                                          lbm_lattice_info* __restrict__ info, typename ST::R omega,
                                                          int nx, int ny, float* __restrict__ macro) {
    const int x0 = (blockIdx.x * VEC_TPB + threadIdx.x) * 4;
    phys_cells4_update<ST, MACRO, 4, IDX>(A, B, flags, info, omega, x0, blockIdx.y, nx, nx, ny, x0 < nx, macro);
}

// 32-bit element offsets are exact when every offset (9 planes, 3 macro planes) stays below 2^32
static inline bool idx32_ok(const lbm_handle* h) { return (size_t)9 * h->N < ((size_t)1 << 32); }

// two cells per thread: one 32-bit access per plane for FP16 / BF16 (threads that walk
// several rows, amortising the column set-up, measured slower: register spills at 48
// registers, or lower occupancy at 64)
template <class ST, bool MACRO, class IDX, bool SR>
__global__ void __launch_bounds__(VEC_TPB, 10) k_phys_step_v2(const typename ST::T* __restrict__ A,
                                                              typename ST::T* __restrict__ B,
                                                              uint16_t* __restrict__ flags,
                                                              lbm_lattice_info* __restrict__ info,
                                                              typename ST::R omega, int nx, int ny,
                                                              float* __restrict__ macro, uint32_t seed) {
    const int x0 = (blockIdx.x * VEC_TPB + threadIdx.x) * 2;
    phys_cells4_update<ST, MACRO, 2, IDX, SR>(A, B, flags, info, omega, x0, blockIdx.y, nx, nx, ny, x0 < nx, macro,
                                              seed);
}

template <class ST, bool MACRO, bool SR>
static cudaError_t phys_step_v2_s(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    using R = typename ST::R;
    const R omega = sizeof(R) == 8 ? (R)h->omega_d : (R)h->omega;
    const dim3 grid((unsigned)((h->nx / 2 + VEC_TPB - 1) / VEC_TPB), (unsigned)h->ny);
    const uint32_t seed = SR ? sr_seed(h->steps, h->p.seed) : 0u;
    if (idx32_ok(h))
        k_phys_step_v2<ST, MACRO, uint32_t, SR><<<grid, VEC_TPB, 0, s>>>(
            (const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1], h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro, seed);
    else
        k_phys_step_v2<ST, MACRO, size_t, SR><<<grid, VEC_TPB, 0, s>>>(
            (const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1], h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro, seed);
    return cudaGetLastError();
}

// stochastic rounding exists for 16-bit storage only (validated at create)
template <class ST, bool MACRO>
static cudaError_t phys_step_v2_t(lbm_handle* h, cudaStream_t s) {
    constexpr bool SIXTEEN = ST::dtype == LBM_DTYPE_F16 || ST::dtype == LBM_DTYPE_BF16;
    if (SIXTEEN && h->p.rounding == LBM_ROUNDING_STOCHASTIC) return phys_step_v2_s<ST, MACRO, SIXTEEN>(h, s);
    return phys_step_v2_s<ST, MACRO, false>(h, s);
}

cudaError_t launch_phys_step_vec2(lbm_handle* h, bool write_macro, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return write_macro ? phys_step_v2_t<StoreF32, true>(h, s) : phys_step_v2_t<StoreF32, false>(h, s);
        case LBM_DTYPE_F64: return write_macro ? phys_step_v2_t<StoreF64, true>(h, s) : phys_step_v2_t<StoreF64, false>(h, s);
        case LBM_DTYPE_F16: return write_macro ? phys_step_v2_t<StoreF16, true>(h, s) : phys_step_v2_t<StoreF16, false>(h, s);
        default: return write_macro ? phys_step_v2_t<StoreBF16, true>(h, s) : phys_step_v2_t<StoreBF16, false>(h, s);
    }
}

template <class ST, bool MACRO>
static cudaError_t phys_step_v4_t(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    using R = typename ST::R;
    const R omega = sizeof(R) == 8 ? (R)h->omega_d : (R)h->omega;
    const dim3 grid((unsigned)((h->nx / 4 + VEC_TPB - 1) / VEC_TPB), (unsigned)h->ny);
    if (idx32_ok(h))
        k_phys_step_v4<ST, MACRO, uint32_t><<<grid, VEC_TPB, 0, s>>>((const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1],
                                                                    h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro);
    else
        k_phys_step_v4<ST, MACRO, size_t><<<grid, VEC_TPB, 0, s>>>((const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1],
                                                                  h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro);
    return cudaGetLastError();
}

// tiled 16-bit layout: one warp per 64-cell tile, the warps of a block on consecutive tiles
// of row blockIdx.y (SR: stochastic rounding of the stores, seed from the step counter)
template <class ST, bool MACRO, bool SR>
__global__ void __launch_bounds__(VEC_TPB, 10) k_phys_step_tiled(const typename ST::T* __restrict__ A,
                                                                 typename ST::T* __restrict__ B,
                                                                 uint16_t* __restrict__ flags,
                                                                 lbm_lattice_info* __restrict__ info, float omega,
                                                                 int nx, int ny, float* __restrict__ macro,
                                                                 uint32_t seed) {
    const int tx = (int)((blockIdx.x * VEC_TPB + threadIdx.x) >> 5);
    if (tx >= nx / POP_TILE) return;  // whole warps
    phys_tile_update<ST, MACRO, SR>(A, B, flags, info, omega, tx, (int)blockIdx.y, nx, ny, macro, seed);
}

bool tiled_layout_eligible(const lbm_params& p) {
    return p.mode == LBM_MODE_PHYSICS && (p.dtype == LBM_DTYPE_F16 || p.dtype == LBM_DTYPE_BF16) &&
           p.collision == LBM_COLLISION_BGK && p.nx % POP_TILE == 0 && (size_t)9 * p.nx * p.ny < ((size_t)1 << 32);
}

template <class ST, bool MACRO, bool SR>
static cudaError_t phys_step_tiled_t(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    const dim3 grid((unsigned)((h->nx / POP_TILE * 32 + VEC_TPB - 1) / VEC_TPB), (unsigned)h->ny);
    k_phys_step_tiled<ST, MACRO, SR><<<grid, VEC_TPB, 0, s>>>((const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1],
                                                                h->d_flags, h->d_info, h->omega, h->nx, h->ny,
                                                                h->d_macro, sr_seed(h->steps, h->p.seed));
    return cudaGetLastError();
}

template <class ST>
static cudaError_t phys_step_tiled_r(lbm_handle* h, bool write_macro, cudaStream_t s) {
    if (h->p.rounding == LBM_ROUNDING_STOCHASTIC)
        return write_macro ? phys_step_tiled_t<ST, true, true>(h, s) : phys_step_tiled_t<ST, false, true>(h, s);
    return write_macro ? phys_step_tiled_t<ST, true, false>(h, s) : phys_step_tiled_t<ST, false, false>(h, s);
}

cudaError_t launch_phys_step_tiled(lbm_handle* h, bool write_macro, cudaStream_t s) {
    if (h->p.dtype == LBM_DTYPE_F16) return phys_step_tiled_r<StoreF16>(h, write_macro, s);
    return phys_step_tiled_r<StoreBF16>(h, write_macro, s);
}

bool vec_step_supported(const lbm_handle* h) { return h->p.mode == LBM_MODE_PHYSICS && (h->nx % 4) == 0; }

cudaError_t launch_phys_step_vec(lbm_handle* h, bool write_macro, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return write_macro ? phys_step_v4_t<StoreF32, true>(h, s) : phys_step_v4_t<StoreF32, false>(h, s);
        case LBM_DTYPE_F64: return write_macro ? phys_step_v4_t<StoreF64, true>(h, s) : phys_step_v4_t<StoreF64, false>(h, s);
        case LBM_DTYPE_F16: return write_macro ? phys_step_v4_t<StoreF16, true>(h, s) : phys_step_v4_t<StoreF16, false>(h, s);
        default: return write_macro ? phys_step_v4_t<StoreBF16, true>(h, s) : phys_step_v4_t<StoreBF16, false>(h, s);
    }
}

// ---- the tiled layout fed from a ring of row strips in shared memory ------------------------
//
// A block walks down a strip of RING_TILES consecutive tiles (RING_TILES * 64 cells) over a
// range of rows.  In the tiled layout the strip's tiles of one row are one contiguous run of
// RING_TILES * 1152 bytes, so a producer warp copies each row with one cp.async.bulk into a
// slot of a ring of RING_SLOTS rows, with a second one for the strip's flag words; six of its
// lanes copy the pairs of the neighbour tiles that the strip's edge lanes pull from (cells 62,
// 63 of the left tile's e_x = +1 planes, cells 0, 1 of the right tile's e_x = -1 planes; the row
// wraps) with 4-byte cp.async.  All complete on the slot's "full" mbarrier.  Consumer warp w
// updates tile w of the strip in row y from the slots of rows y - 1, y and y + 1 with
// phys_tile_finish (the tiled kernel's collision and stores, so the results are the same bit for
// bit; the extra populations of cells next to a solid and of outflow cells come from the slots
// too), then arrives on the "empty" mbarrier of row y - 1's slot, which the producer waits for
// before reusing the slot.  No block barrier in the loop: warps drift apart by up to
// RING_SLOTS - 3 rows, and the bytes in flight are set by the ring depth, not by registers.
//
// Measured on GB300 at 8192^2 FP16 it runs below the tiled kernel on the 5 %-solid channel
// (129 against 158 GLUPS): a strip moves at the pace of its slowest warp, and a tile next to a
// solid takes the general per-cell rules.  Without solids the two run alike (161 and 162).  It
// is kept as LBM_KERNEL_RING; LBM_KERNEL_AUTO takes the tiled kernel.
//
// Every wait is bounded (1 s).  A consumer warp that gives up records LBM_ERR_TIMEOUT in the
// handle's status word and leaves; the producer that gives up records it, waits (bounded again)
// for the copies it started and leaves.
#ifndef LBM_RING_SLOTS
#define LBM_RING_SLOTS 5
#endif
constexpr int RING_TILES = 8;                     // tiles (consumer warps) per strip
constexpr int RING_TPB = 32 * (RING_TILES + 1);   // + the producer warp
constexpr unsigned long long RING_WAIT_NS = 1000000000ull;

template <int NSLOT>
struct RingLayout {
    static constexpr int TILE_BYTES = 9 * POP_TILE * 2;             // one tile of 16-bit populations
    static constexpr int HALO_OFF = RING_TILES * TILE_BYTES;         // 3 left pairs, then 3 right
    static constexpr int FLAG_OFF = HALO_OFF + 32;
    static constexpr int SLOT_BYTES = FLAG_OFF + RING_TILES * POP_TILE * 2;
    static constexpr int FULL_OFF = NSLOT * SLOT_BYTES;              // NSLOT "full" mbarriers
    static constexpr int EMPTY_OFF = FULL_OFF + 8 * NSLOT;           // NSLOT "empty" mbarriers
    static constexpr int SMEM = EMPTY_OFF + 8 * NSLOT;
    static_assert(SLOT_BYTES % 16 == 0 && HALO_OFF % 16 == 0 && FLAG_OFF % 16 == 0, "bulk copies need 16-byte offsets");
    static_assert(NSLOT >= 4, "a consumer holds three rows while the next one loads");
    // resident blocks per SM the kernel is compiled for (shared memory allows this many)
    static constexpr int MIN_BLOCKS = NSLOT <= 5 ? 4 : (NSLOT <= 7 ? 3 : 2);
};

// the halo pair of direction j among the three with the same e_x (1, 5, 8 and 3, 6, 7)
__host__ __device__ constexpr int halo_rank(int j) { return (j == 1 || j == 3) ? 0 : ((j == 5 || j == 6) ? 1 : 2); }

__device__ __forceinline__ unsigned ring_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }
__device__ __forceinline__ bool ring_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ bool ring_wait(unsigned bar, unsigned parity) {
    if (ring_try(bar, parity)) return true;
    unsigned long long t0, t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t0));
    while (!ring_try(bar, parity)) {
        asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
        if (t - t0 > RING_WAIT_NS) return false;
    }
    return true;
}
__device__ __forceinline__ void ring_copy(unsigned dst, const void* src, unsigned bytes, unsigned bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(dst),
                 "l"(src), "r"(bytes), "r"(bar)
                 : "memory");
}

// two consecutive / one stored 16-bit value(s) from shared memory, in stored units
template <class ST>
struct RingLd;
template <>
struct RingLd<StoreF16> {
    __device__ __forceinline__ static void pair(const unsigned char* p, float (&r)[2]) {
        const unsigned q = *reinterpret_cast<const unsigned*>(p);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q));
        r[0] = a.x; r[1] = a.y;
    }
    __device__ __forceinline__ static float one(const unsigned char* p) { return __half2float(*reinterpret_cast<const __half*>(p)); }
};
template <>
struct RingLd<StoreBF16> {
    __device__ __forceinline__ static void pair(const unsigned char* p, float (&r)[2]) {
        const unsigned q = *reinterpret_cast<const unsigned*>(p);
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q));
        r[0] = a.x; r[1] = a.y;
    }
    __device__ __forceinline__ static float one(const unsigned char* p) {
        return __bfloat162float(*reinterpret_cast<const __nv_bfloat16*>(p));
    }
};

// the general per-cell rules' extra populations (TileSrcGlobal's values) from the staged rows:
// `off` is the byte offset of the lane's first cell in plane 0 of its tile
template <class ST>
struct TileSrcRing {
    const unsigned char *top, *mid, *bot;  // slots of rows y - 1, y, y + 1
    int off;
    __device__ __forceinline__ float col(int j, int dy, int k) const {
        const unsigned char* r = dy < 0 ? top : (dy > 0 ? bot : mid);
        return RingLd<ST>::one(r + off + j * POP_TILE * 2 + 2 * k);
    }
};

template <class ST, bool MACRO, bool SR, int NSLOT>
__global__ void __launch_bounds__(RING_TPB, RingLayout<NSLOT>::MIN_BLOCKS) k_phys_step_ring(const typename ST::T* __restrict__ A,
                                                             typename ST::T* __restrict__ B,
                                                             uint16_t* __restrict__ flags,
                                                             lbm_lattice_info* __restrict__ info, float omega, int nx,
                                                             int ny, int rows_per_block, float* __restrict__ macro,
                                                             uint32_t seed, int* __restrict__ status) {
    using L = RingLayout<NSLOT>;
    constexpr int TS = 9 * POP_TILE;  // elements per tile
    extern __shared__ __align__(128) unsigned char ring[];
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    const int tpr = nx / POP_TILE;
    const int tx0 = blockIdx.x * RING_TILES;
    const int nt = min(RING_TILES, tpr - tx0);       // tiles of this strip
    const int y0 = blockIdx.y * rows_per_block;
    const int rows = min(rows_per_block, ny - y0);   // >= 1 by the launch
    const int nload = rows + 2;                      // rows y0 - 1 .. y0 + rows, wrapped
    const unsigned full0 = ring_u32(ring + L::FULL_OFF), empty0 = ring_u32(ring + L::EMPTY_OFF);
    if (threadIdx.x == 0) {
        for (int s = 0; s < NSLOT; ++s) {
            asm volatile("mbarrier.init.shared::cta.b64 [%0], 7;" ::"r"(full0 + 8 * s) : "memory");  // lane 0 + 6 halo lanes
            asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(empty0 + 8 * s), "r"(nt) : "memory");
        }
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();

    if (warp == RING_TILES) {  // producer warp
        const unsigned long long NP = 9ull * (unsigned long long)nx * (unsigned long long)ny;
        const unsigned long long NC = (unsigned long long)nx * (unsigned long long)ny;
        const int txl = tx0 == 0 ? tpr - 1 : tx0 - 1;      // tile left of the strip (wraps)
        const int txr = tx0 + nt == tpr ? 0 : tx0 + nt;   // tile right of the strip (wraps)
        const unsigned row_bytes = (unsigned)nt * L::TILE_BYTES, flag_bytes = (unsigned)nt * POP_TILE * 2;
        // lanes 1..6: the halo pair of direction hj (1, 5, 8 from the left tile: cells 62, 63;
        // 3, 6, 7 from the right tile: cells 0, 1)
        const int hj = lane == 1 ? 1 : lane == 2 ? 5 : lane == 3 ? 8 : lane == 4 ? 3 : lane == 5 ? 6 : 7;
        const bool halo_lane = lane >= 1 && lane <= 6;
        bool ok = true;
        int k = 0;
        for (; k < nload; ++k) {
            const int s = k % NSLOT;
            // the slot's previous row (load k - NSLOT) must be released by every consumer warp
            if (k >= NSLOT) {
                if (lane == 0) ok = ring_wait(empty0 + 8 * s, (unsigned)(k / NSLOT - 1) & 1u);
                ok = __shfl_sync(0xffffffffu, ok, 0);
                if (!ok) break;
            }
            int yy = y0 - 1 + k;
            yy = yy < 0 ? yy + ny : (yy >= ny ? yy - ny : yy);
            const size_t row = (size_t)yy * tpr;  // first tile of row yy
            const unsigned dst = ring_u32(ring + s * L::SLOT_BYTES), bar = full0 + 8 * s;
            if (lane == 0) {
                // bounds-checked build: the copies' last elements inside their buffers, else
                // none is started and the slot's phase completes with no bytes (stale contents)
                const bool in = in_bounds((row + tx0 + nt) * TS - 1, NP, BS_BULK_COPY) &&
                                in_bounds((size_t)yy * nx + (size_t)(tx0 + nt) * POP_TILE - 1, NC, BS_BULK_COPY);
                asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
                asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(bar),
                             "r"(in ? row_bytes + flag_bytes : 0u)
                             : "memory");
                if (in) {
                    ring_copy(dst, A + (row + tx0) * TS, row_bytes, bar);
                    ring_copy(dst + L::FLAG_OFF, flags + (size_t)yy * nx + (size_t)tx0 * POP_TILE, flag_bytes, bar);
                }
            } else if (halo_lane) {
                // one 4-byte cp.async per lane, its completion counted on the same mbarrier
                const size_t src = EX(hj) == 1 ? (row + txl) * TS + hj * POP_TILE + (POP_TILE - 2)
                                               : (row + txr) * TS + hj * POP_TILE;
                if (in_bounds(src + 1, NP, BS_BULK_COPY))
                    asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(dst + L::HALO_OFF + 4 * (lane - 1)),
                                 "l"(A + src)
                                 : "memory");
                asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(bar) : "memory");
            }
        }
        if (lane == 0) {
            if (!ok) atomicExch(status, LBM_ERR_TIMEOUT);
            // leave only when the copies started have landed (the consumers may be gone)
            for (int kk = max(0, k - NSLOT); kk < k; ++kk)
                ring_wait(full0 + 8 * (kk % NSLOT), (unsigned)(kk / NSLOT) & 1u);
        }
        return;
    }
    if (warp >= nt) return;  // a strip narrower than RING_TILES tiles

    const int w = warp;
    for (int i = 0; i < rows; ++i) {
        // rows y - 1, y, y + 1 are loads i, i + 1, i + 2 (the first two were waited for earlier)
        bool ok = true;
        if (i == 0) ok = ring_wait(full0, 0u) && ring_wait(full0 + 8 * (1 % NSLOT), 0u);
        ok = ok && ring_wait(full0 + 8 * ((i + 2) % NSLOT), (unsigned)((i + 2) / NSLOT) & 1u);
        if (!__all_sync(0xffffffffu, ok)) {
            if (lane == 0) atomicExch(status, LBM_ERR_TIMEOUT);
            return;
        }
        const unsigned char* top = ring + (i % NSLOT) * L::SLOT_BYTES;
        const unsigned char* mid = ring + ((i + 1) % NSLOT) * L::SLOT_BYTES;
        const unsigned char* bot = ring + ((i + 2) % NSLOT) * L::SLOT_BYTES;
        float d[9][2];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const unsigned char* src = EY(j) == 1 ? top : (EY(j) == -1 ? bot : mid);  // source row y - e_y
            const unsigned char* plane = src + w * L::TILE_BYTES + j * POP_TILE * 2;
            float v[2];
            RingLd<ST>::pair(plane + 4 * lane, v);
            if (EX(j) == 0) {
                d[j][0] = v[0];
                d[j][1] = v[1];
            } else if (EX(j) == 1) {  // source x - 1: lane 0 takes cell 63 of the tile to the left
                float prev = __shfl_up_sync(0xffffffffu, v[1], 1);
                if (lane == 0)
                    prev = RingLd<ST>::one(w > 0 ? plane - L::TILE_BYTES + 2 * (POP_TILE - 1)
                                                 : src + L::HALO_OFF + 4 * halo_rank(j) + 2);
                d[j][0] = prev;
                d[j][1] = v[0];
            } else {  // source x + 1: lane 31 takes cell 0 of the tile to the right
                float next = __shfl_down_sync(0xffffffffu, v[0], 1);
                if (lane == 31)
                    next = RingLd<ST>::one(w < nt - 1 ? plane + L::TILE_BYTES : src + L::HALO_OFF + 12 + 4 * halo_rank(j));
                d[j][0] = v[1];
                d[j][1] = next;
            }
        }
        const unsigned fq = *reinterpret_cast<const unsigned*>(mid + L::FLAG_OFF + w * (POP_TILE * 2) + 4 * lane);
        const TileSrcRing<ST> src{top, mid, bot, w * L::TILE_BYTES + 4 * lane};
        phys_tile_finish<ST, MACRO, SR>(d, fq, src, B, flags, info, omega, tx0 + w, y0 + i, nx, ny, macro, seed);
        // every read of row y - 1's slot is done: release it to the producer
        __syncwarp();
        if (lane == 0) asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(empty0 + 8 * (i % NSLOT)) : "memory");
    }
}

template <class ST, bool MACRO, bool SR>
static cudaError_t phys_step_ring_t(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    constexpr int NSLOT = LBM_RING_SLOTS;
    using L = RingLayout<NSLOT>;
    struct Setup {
        int blocks_per_sm, sms;
    };
    static PerDevice<Setup> per_device;
    Setup su{};
    cudaError_t e = per_device.get(
        h->device,
        [&](Setup& v) {
            cudaError_t r = cudaFuncSetAttribute(k_phys_step_ring<ST, MACRO, SR, NSLOT>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM);
            if (r == cudaSuccess)
                r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v.blocks_per_sm, k_phys_step_ring<ST, MACRO, SR, NSLOT>,
                                                                  RING_TPB, L::SMEM);
            if (r == cudaSuccess) r = cudaDeviceGetAttribute(&v.sms, cudaDevAttrMultiProcessorCount, h->device);
            if (v.blocks_per_sm < 1) v.blocks_per_sm = 1;
            return r;
        },
        &su);
    if (e != cudaSuccess) return e;
    // one wave: strips x row segments <= the resident blocks, each segment as long as possible
    // (a segment reads two rows beyond its own)
    const int tpr = h->nx / POP_TILE;
    const int nstrip = (tpr + RING_TILES - 1) / RING_TILES;
    const long resident = (long)su.blocks_per_sm * su.sms;
    int nseg = (int)std::min<long>(h->ny, std::max<long>(1, resident / nstrip));
    const int rows = (h->ny + nseg - 1) / nseg;
    nseg = (h->ny + rows - 1) / rows;
    k_phys_step_ring<ST, MACRO, SR, NSLOT><<<dim3((unsigned)nstrip, (unsigned)nseg), RING_TPB, L::SMEM, s>>>(
        (const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1], h->d_flags, h->d_info, h->omega, h->nx, h->ny, rows,
        h->d_macro, sr_seed(h->steps, h->p.seed), h->d_status);
    return cudaGetLastError();
}

template <class ST>
static cudaError_t phys_step_ring_r(lbm_handle* h, bool write_macro, cudaStream_t s) {
    if (h->p.rounding == LBM_ROUNDING_STOCHASTIC)
        return write_macro ? phys_step_ring_t<ST, true, true>(h, s) : phys_step_ring_t<ST, false, true>(h, s);
    return write_macro ? phys_step_ring_t<ST, true, false>(h, s) : phys_step_ring_t<ST, false, false>(h, s);
}

cudaError_t launch_phys_step_ring(lbm_handle* h, bool write_macro, cudaStream_t s) {
    if (h->p.dtype == LBM_DTYPE_F16) return phys_step_ring_r<StoreF16>(h, write_macro, s);
    return phys_step_ring_r<StoreBF16>(h, write_macro, s);
}

#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_vec(BoundsRecord* out) { return bounds_take_local(out); }
#endif

}  // namespace lbm
