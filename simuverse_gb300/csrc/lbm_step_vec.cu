// lbm_step_vec.cu -- physics-mode step with four cells per thread (phys_cells4_update of
// lbm_cell4.cuh): one aligned vector load and store per population plane and thread,
// warp shuffles for the +-x shifted directions.  Requires nx % 4 == 0.
//
// Algorithmic traffic per cell update: 9 loads + 9 stores of the stored type (72 B FP32,
// 36 B FP16/BF16, 144 B FP64) plus the 2-byte flag word.
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

#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_vec(BoundsRecord* out) { return bounds_take_local(out); }
#endif

}  // namespace lbm
