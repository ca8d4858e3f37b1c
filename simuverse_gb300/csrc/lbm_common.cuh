// lbm_common.cuh -- D2Q9 constants, per-cell flag layout and population storage formats
// shared by the step kernels.
//
// Lattice (simuverse/src/fluid/mod.rs:22-52): direction j has vector (EX(j), EY(j)) with y
// growing downwards, inverse INV(j).  Reference-mode weights and clamp maxima are the
// truncated literals of mod.rs:40-48; physics mode uses the exact 4/9, 1/9, 1/36.
#pragma once

#include <cuda_bf16.h>
#include <cuda_fp16.h>
#include <cuda_runtime.h>
#include <stdint.h>

#include "../../include/lbm.h"
#include "lbm_internal.h"

namespace lbm {

__host__ __device__ constexpr int EX(int j) {
    return (j == 1 || j == 5 || j == 8) ? 1 : ((j == 3 || j == 6 || j == 7) ? -1 : 0);
}
__host__ __device__ constexpr int EY(int j) {
    return (j == 4 || j == 7 || j == 8) ? 1 : ((j == 2 || j == 5 || j == 6) ? -1 : 0);
}
__host__ __device__ constexpr int INV(int j) {
    return j == 0 ? 0 : j == 1 ? 3 : j == 2 ? 4 : j == 3 ? 1 : j == 4 ? 2 : j == 5 ? 7 : j == 6 ? 8 : j == 7 ? 5 : 6;
}
// mod.rs:40-48 (truncated literals, reference mode)
__host__ __device__ constexpr float REF_W(int j) { return j == 0 ? 0.444444f : (j <= 4 ? 0.111111f : 0.0277777f); }
__host__ __device__ constexpr float REF_MAX(int j) { return j == 0 ? 0.6f : (j <= 4 ? 0.2222f : 0.1111f); }
// exact weights (physics mode)
template <class R>
__host__ __device__ constexpr R PW(int j) {
    return j == 0 ? R(4) / R(9) : (j <= 4 ? R(1) / R(9) : R(1) / R(36));
}

// Per-cell flags (uint16), rebuilt from the info records whenever the mask changes:
//   bits 0-3  material code (0 = unknown code, treated as plain fluid)
//   bits 4-12 one bit per direction k = 0..8:
//     reference mode, fluid cell: the post-collision population k is handed to the wall
//       cell c+e_k (boundary.wgsl:28-31 moved into the owning fluid cell);
//     reference mode, solid cell: slot k is zeroed (wall-to-wall slot, see lbm_kernels.cu);
//     physics mode, fluid cell: the pull source of direction k is solid (bounce-back).
//   bit 13    physics mode: some bounce-back source is a moving wall
//   bit 14    physics mode: plain fluid (bulk, ghost or code 0, no solid pull source), the
//             cells the step kernels' warp-uniform fast path takes
constexpr unsigned FL_MAT_MASK = 15u;
constexpr int FL_DIR_SHIFT = 4;
constexpr unsigned FL_MOVING = 1u << 13;
constexpr unsigned FL_PLAIN = 1u << 14;
__host__ __device__ constexpr unsigned plain_bit(unsigned fl) {
    return ((fl & FL_MAT_MASK) == LBM_BULK || (fl & FL_MAT_MASK) == LBM_GHOST || (fl & FL_MAT_MASK) == 0u) &&
                   !(fl & (0x1FFu << FL_DIR_SHIFT))
               ? FL_PLAIN
               : 0u;
}

__host__ __device__ constexpr bool is_solid(int m) { return m == LBM_BOUNDARY || m == LBM_OBSTACLE; }

// Population layouts.  SoA (the reference's, d2q9_fn.wgsl:13-17): direction j of cell c at
// j * N + c.  Tiled (16-bit storage with the two-cell kernel, nx % POP_TILE == 0): rows are
// cut into tiles of POP_TILE cells and a tile keeps its nine planes together, direction j of
// cell c at (c / POP_TILE) * 9 * POP_TILE + j * POP_TILE + c % POP_TILE.  Both use 9 N elements.
constexpr int POP_TILE = 64;
__host__ __device__ __forceinline__ size_t pop_index(bool tiled, size_t N, int j, size_t c) {
    return tiled ? (c / POP_TILE) * (9 * POP_TILE) + (size_t)j * POP_TILE + (c % POP_TILE) : (size_t)j * N + c;
}

// ---- bounds-checked builds (-DLBM_BOUNDS_CHECK) ------------------------------------
// A bounds-checked build of the library compares every population, flag and info index of
// the step kernels with the extent of its buffer before the access.  An index outside it is
// counted in g_bounds together with the first offending index, its extent and the access
// site; the access is skipped (a load gives 0): nothing traps and the context stays usable.
// lbm_bounds_report reads and clears the records.  In normal builds in_bounds is the constant
// true and the checks compile away.
enum BoundsSite : int {
    BS_REF_FLAGS = 1, BS_REF_PULL, BS_REF_INFO, BS_REF_STORE, BS_REF_WALL, BS_REF_MACRO,
    BS_CELL_FLAGS = 11, BS_CELL_PULL, BS_CELL_INFO, BS_CELL_STORE, BS_CELL_MACRO,
    BS_TILE_FLAGS = 21, BS_TILE_PULL, BS_TILE_INFO, BS_TILE_STORE, BS_TILE_MACRO,
    BS_BULK_COPY = 31, BS_BULK_PULL, BS_BULK_INFO, BS_BULK_STORE, BS_BULK_MACRO,
    BS_SELFTEST = 99
};
#ifdef LBM_BOUNDS_CHECK
static __device__ BoundsRecord g_bounds;  // one per translation unit
#endif
__device__ __forceinline__ bool in_bounds(unsigned long long idx, unsigned long long limit, int site) {
#ifdef LBM_BOUNDS_CHECK
    if (idx < limit) return true;
    if (atomicAdd(&g_bounds.count, 1ull) == 0ull) {
        g_bounds.index = idx;
        g_bounds.limit = limit;
        g_bounds.site = site;
    }
    return false;
#else
    (void)idx;
    (void)limit;
    (void)site;
    return true;
#endif
}
#ifdef LBM_BOUNDS_CHECK
// the records of the calling translation unit on the current device, cleared after reading
static inline cudaError_t bounds_take_local(BoundsRecord* out) {
    cudaError_t e = cudaMemcpyFromSymbol(out, g_bounds, sizeof(BoundsRecord));
    if (e != cudaSuccess) return e;
    const BoundsRecord zero = {0, 0, 0, 0, 0};
    return cudaMemcpyToSymbol(g_bounds, &zero, sizeof(BoundsRecord));
}
#endif

// round-to-nearest add and multiply that the compiler may not contract into an FMA
__device__ __forceinline__ float add_rn(float a, float b) { return __fadd_rn(a, b); }
__device__ __forceinline__ double add_rn(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ float mul_rn(float a, float b) { return __fmul_rn(a, b); }
__device__ __forceinline__ double mul_rn(double a, double b) { return __dmul_rn(a, b); }
// correctly rounded reciprocal
__device__ __forceinline__ float recip_rn(float a) { return __frcp_rn(a); }
__device__ __forceinline__ double recip_rn(double a) { return __drcp_rn(a); }

// ---- stochastic rounding of 16-bit stores (LBM_ROUNDING_STOCHASTIC) ---------------
// A value v between two neighbouring stored values lo < v < hi is stored as hi with
// probability (v - lo) / (hi - lo), so the rounding error has zero mean: a field that changes
// by less than the stored spacing from one cell or step to the next (the pressure gradient of
// an open channel) is kept on average instead of being rounded away, the stagnation of
// round-to-nearest (Connolly, Higham & Mary, SIAM J. Sci. Comput. 43 (2021) A566).  The store
// adds a uniform random integer below the stored precision to the FP32 bit pattern (the
// significand bits that the conversion drops: SR_DROP) and converts rounding toward zero; the
// pattern's low 31 bits are the magnitude, so both signs round alike.  Where the 16-bit image
// is subnormal (FP16 stored magnitudes below 2^-14) more bits are dropped and the rounding
// keeps a bias toward zero of at most that spacing.
//
// Random bits: one hash per thread and step, sr_hash(cell ^ seed), the "lowbias32" integer
// hash of C. Wellons' hash-prospector (2018); the value j of a thread takes the top SR_DROP
// bits of hash * sr_mul(j) (odd multipliers, so every value's bits are uniform).  The host
// derives seed from the step counter (sr_seed): runs are reproducible.
__host__ __device__ __forceinline__ uint32_t sr_hash(uint32_t x) {
    x ^= x >> 16;
    x *= 0x7feb352du;
    x ^= x >> 15;
    x *= 0x846ca68bu;
    x ^= x >> 16;
    return x;
}
__host__ __device__ constexpr uint32_t sr_mul(int i) {
    return (((0x9E3779B9u * (uint32_t)(i + 1)) ^ ((0x9E3779B9u * (uint32_t)(i + 1)) >> 15)) * 0x2C1B3C6Du) | 1u;
}
// seed of step `step` of a handle whose channel seed is `seed` (splitmix64 finaliser)
inline uint32_t sr_seed(uint64_t step, uint64_t seed) {
    uint64_t z = step + 0x9E3779B97F4A7C15ull * (seed + 1);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
    return (uint32_t)((z ^ (z >> 31)) >> 32);
}
// v with `r`'s top DROP bits added to its pattern (the conversion that follows truncates)
template <int DROP>
__device__ __forceinline__ float sr_dither(float v, uint32_t r) {
    return __uint_as_float(__float_as_uint(v) + (r >> (32 - DROP)));
}
// two FP32 values to packed 16-bit (element 0 in the low half), rounding toward zero
__device__ __forceinline__ unsigned pack_half2_rz(float a0, float a1) {
    unsigned d;
    asm("cvt.rz.f16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(a1), "f"(a0));
    return d;
}
__device__ __forceinline__ unsigned pack_bf162_rz(float a0, float a1) {
    unsigned d;
    asm("cvt.rz.bf16x2.f32 %0, %1, %2;" : "=r"(d) : "f"(a1), "f"(a0));
    return d;
}

// ---- population storage formats ------------------------------------------------
// R: arithmetic type; T: stored type.  Physics-mode storage holds d = f - w (shifted
// deviation); FP16 additionally scales by 2^10 so that small deviations stay normal.
struct StoreF32 {
    using T = float;
    using R = float;
    static constexpr int dtype = LBM_DTYPE_F32;
    static constexpr float UNIT = 1.0f;
    __device__ __forceinline__ static R ld(const T* p) { return __ldg(p); }
    __device__ __forceinline__ static void st(T* p, R v) { *p = v; }
    __device__ __forceinline__ static R ldu(const T* p) { return __ldg(p); }
    __device__ __forceinline__ static void stu(T* p, R v) { *p = v; }
    __device__ __forceinline__ static void stu_sr(T* p, R v, uint32_t) { *p = v; }  // no rounding
    __host__ __device__ static R to_r(T v) { return v; }
    __host__ __device__ static T from_r(R v) { return v; }
};
struct StoreF64 {
    using T = double;
    using R = double;
    static constexpr int dtype = LBM_DTYPE_F64;
    static constexpr double UNIT = 1.0;
    __device__ __forceinline__ static R ld(const T* p) { return __ldg(p); }
    __device__ __forceinline__ static void st(T* p, R v) { *p = v; }
    __device__ __forceinline__ static R ldu(const T* p) { return __ldg(p); }
    __device__ __forceinline__ static void stu(T* p, R v) { *p = v; }
    __device__ __forceinline__ static void stu_sr(T* p, R v, uint32_t) { *p = v; }  // no rounding
    __host__ __device__ static R to_r(T v) { return v; }
    __host__ __device__ static T from_r(R v) { return v; }
};
constexpr float F16_SCALE = 1024.0f;
constexpr float F16_INV_SCALE = 1.0f / 1024.0f;
struct StoreF16 {
    using T = __half;
    using R = float;
    static constexpr int dtype = LBM_DTYPE_F16;
    // the step kernels compute in stored units (deviations times 2^10): UNIT is the stored
    // value of a unit density, ldu / stu move stored values without rescaling
    static constexpr float UNIT = F16_SCALE;
    __device__ __forceinline__ static R ld(const T* p) { return __half2float(__ldg(p)) * F16_INV_SCALE; }
    __device__ __forceinline__ static void st(T* p, R v) { *p = __float2half_rn(v * F16_SCALE); }
    __device__ __forceinline__ static R ldu(const T* p) { return __half2float(__ldg(p)); }
    __device__ __forceinline__ static void stu(T* p, R v) { *p = __float2half_rn(v); }
    static constexpr int SR_DROP = 13;  // FP32 significand bits below FP16's
    __device__ __forceinline__ static void stu_sr(T* p, R v, uint32_t r) {
        *p = __float2half_rz(sr_dither<SR_DROP>(v, r));
    }
    __host__ __device__ static R to_r(T v) { return __half2float(v) * F16_INV_SCALE; }
    __host__ __device__ static T from_r(R v) { return __float2half_rn(v * F16_SCALE); }
};
struct StoreBF16 {
    using T = __nv_bfloat16;
    using R = float;
    static constexpr int dtype = LBM_DTYPE_BF16;
    static constexpr float UNIT = 1.0f;
    __device__ __forceinline__ static R ld(const T* p) { return __bfloat162float(__ldg(p)); }
    __device__ __forceinline__ static void st(T* p, R v) { *p = __float2bfloat16_rn(v); }
    __device__ __forceinline__ static R ldu(const T* p) { return __bfloat162float(__ldg(p)); }
    __device__ __forceinline__ static void stu(T* p, R v) { *p = __float2bfloat16_rn(v); }
    static constexpr int SR_DROP = 16;  // FP32 significand bits below BF16's
    __device__ __forceinline__ static void stu_sr(T* p, R v, uint32_t r) {
        *p = __float2bfloat16_rz(sr_dither<SR_DROP>(v, r));
    }
    __host__ __device__ static R to_r(T v) { return __bfloat162float(v); }
    __host__ __device__ static T from_r(R v) { return __float2bfloat16_rn(v); }
};

}  // namespace lbm
