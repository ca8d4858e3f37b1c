// lbm_cell4.cuh -- the physics-mode update of CPT (2 or 4) consecutive cells of one row by
// one thread, shared by the single-lattice kernel (lbm_step_vec.cu) and the batched persistent
// kernel (lbm_batch.cu).
//
// Populations are loaded and stored in stored units (ST::ldu / ST::stu; FP16 keeps its 2^10
// scale through the collision, which takes ST::UNIT as the unit density).
// Cells x0..x0+CPT-1 (x0 a multiple of CPT) of row y; rows are `pitch` elements apart
// (pitch % CPT == 0, pitch >= nx) and cells x >= nx are padding, never read by a fluid
// cell.  Every population plane is read and written with one aligned vector access per
// thread.  The pull of a direction with e_x = +1 needs x0-1..x0+2: the thread's own
// vector shifted by one, the missing element coming from the left neighbour lane by a
// warp shuffle (lane 0 loads it, wrapping to nx-1 at x0 = 0); e_x = -1 is the mirror
// image (the last active lane of the row loads its right halo, wrapping to 0).  All 32
// lanes of the warp must call this function for the same row (the shuffles use the full
// mask); lanes with x0 >= nx pass active = false.  Bounce-back and moving-wall
// corrections read the cell's own opposite population with a scalar load, only in cells
// next to a solid.  The collision is phys_collide of lbm_cell.cuh.
#pragma once

#include "lbm_cell.cuh"
#include "lbm_common.cuh"

namespace lbm {

template <class ST>
struct Vec4;

template <>
struct Vec4<StoreF32> {
    __device__ __forceinline__ static void ld(const float* p, float (&r)[4]) {
        const float4 q = __ldg(reinterpret_cast<const float4*>(p));
        r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
    }
    __device__ __forceinline__ static void st(float* p, const float (&r)[4]) {
        *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
    }
};

template <>
struct Vec4<StoreF64> {
    __device__ __forceinline__ static void ld(const double* p, double (&r)[4]) {
        const double2 a = __ldg(reinterpret_cast<const double2*>(p));
        const double2 b = __ldg(reinterpret_cast<const double2*>(p + 2));
        r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
    }
    __device__ __forceinline__ static void st(double* p, const double (&r)[4]) {
        reinterpret_cast<double2*>(p)[0] = make_double2(r[0], r[1]);
        reinterpret_cast<double2*>(p)[1] = make_double2(r[2], r[3]);
    }
};

template <>
struct Vec4<StoreF16> {
    __device__ __forceinline__ static void ld(const __half* p, float (&r)[4]) {
        const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
        r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
    }
    __device__ __forceinline__ static void st(__half* p, const float (&r)[4]) {
        const __half2 a = __floats2half2_rn(r[0], r[1]);
        const __half2 b = __floats2half2_rn(r[2], r[3]);
        uint2 q;
        q.x = *reinterpret_cast<const unsigned*>(&a);
        q.y = *reinterpret_cast<const unsigned*>(&b);
        *reinterpret_cast<uint2*>(p) = q;
    }
};

template <>
struct Vec4<StoreBF16> {
    __device__ __forceinline__ static void ld(const __nv_bfloat16* p, float (&r)[4]) {
        const uint2 q = __ldg(reinterpret_cast<const uint2*>(p));
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.x));
        const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.y));
        r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
    }
    __device__ __forceinline__ static void st(__nv_bfloat16* p, const float (&r)[4]) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(r[0], r[1]);
        const __nv_bfloat162 b = __floats2bfloat162_rn(r[2], r[3]);
        uint2 q;
        q.x = *reinterpret_cast<const unsigned*>(&a);
        q.y = *reinterpret_cast<const unsigned*>(&b);
        *reinterpret_cast<uint2*>(p) = q;
    }
};

template <class ST>
struct Vec2;
template <>
struct Vec2<StoreF32> {
    __device__ __forceinline__ static void ld(const float* p, float (&r)[2]) {
        const float2 q = __ldg(reinterpret_cast<const float2*>(p));
        r[0] = q.x; r[1] = q.y;
    }
    __device__ __forceinline__ static void st(float* p, const float (&r)[2]) {
        *reinterpret_cast<float2*>(p) = make_float2(r[0], r[1]);
    }
    __device__ __forceinline__ static void st_sr(float* p, const float (&r)[2], uint32_t, uint32_t) { st(p, r); }
};
template <>
struct Vec2<StoreF64> {
    __device__ __forceinline__ static void ld(const double* p, double (&r)[2]) {
        const double2 q = __ldg(reinterpret_cast<const double2*>(p));
        r[0] = q.x; r[1] = q.y;
    }
    __device__ __forceinline__ static void st(double* p, const double (&r)[2]) {
        *reinterpret_cast<double2*>(p) = make_double2(r[0], r[1]);
    }
    __device__ __forceinline__ static void st_sr(double* p, const double (&r)[2], uint32_t, uint32_t) { st(p, r); }
};
template <>
struct Vec2<StoreF16> {
    __device__ __forceinline__ static void ld(const __half* p, float (&r)[2]) {
        const unsigned q = __ldg(reinterpret_cast<const unsigned*>(p));
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q));
        r[0] = a.x; r[1] = a.y;
    }
    __device__ __forceinline__ static void st(__half* p, const float (&r)[2]) {
        const __half2 a = __floats2half2_rn(r[0], r[1]);
        *reinterpret_cast<unsigned*>(p) = *reinterpret_cast<const unsigned*>(&a);
    }
    // stochastic rounding with random words q0, q1 (lbm_common.cuh)
    __device__ __forceinline__ static void st_sr(__half* p, const float (&r)[2], uint32_t q0, uint32_t q1) {
        *reinterpret_cast<unsigned*>(p) = pack_half2_rz(sr_dither<StoreF16::SR_DROP>(r[0], q0),
                                                        sr_dither<StoreF16::SR_DROP>(r[1], q1));
    }
};
template <>
struct Vec2<StoreBF16> {
    __device__ __forceinline__ static void ld(const __nv_bfloat16* p, float (&r)[2]) {
        const unsigned q = __ldg(reinterpret_cast<const unsigned*>(p));
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q));
        r[0] = a.x; r[1] = a.y;
    }
    __device__ __forceinline__ static void st(__nv_bfloat16* p, const float (&r)[2]) {
        const __nv_bfloat162 a = __floats2bfloat162_rn(r[0], r[1]);
        *reinterpret_cast<unsigned*>(p) = *reinterpret_cast<const unsigned*>(&a);
    }
    __device__ __forceinline__ static void st_sr(__nv_bfloat16* p, const float (&r)[2], uint32_t q0, uint32_t q1) {
        *reinterpret_cast<unsigned*>(p) = pack_bf162_rz(sr_dither<StoreBF16::SR_DROP>(r[0], q0),
                                                        sr_dither<StoreBF16::SR_DROP>(r[1], q1));
    }
};

template <class ST, int CPT>
struct VecN;
template <class ST>
struct VecN<ST, 4> : Vec4<ST> {};
template <class ST>
struct VecN<ST, 2> : Vec2<ST> {};

// IDX: the integer type of element offsets (uint32_t when 9 * pitch * ny < 2^32, which saves
// the 64-bit address arithmetic of every plane access; size_t otherwise)
// SR: stochastic rounding of the stores with the step's `seed` (two cells per thread only)
template <class ST, bool MACRO, int CPT = 4, class IDX = size_t, bool SR = false>
__device__ __forceinline__ void phys_cells4_update(const typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                                                   uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                   typename ST::R omega, int x0, int y, int nx, int pitch, int ny,
                                                   bool active, float* __restrict__ macro, uint32_t seed = 0) {
    static_assert(!SR || CPT == 2, "stochastic rounding runs on the two-cell form");
    using R = typename ST::R;
    using T = typename ST::T;
    const int lane = threadIdx.x & 31;
    const IDX N = (IDX)pitch * (IDX)ny;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const IDX r0 = (IDX)y * (IDX)pitch, rm = (IDX)ym * (IDX)pitch, rp = (IDX)yp * (IDX)pitch;
    const int xl = x0 == 0 ? nx - 1 : x0 - 1;
    const int xr = x0 + CPT >= nx ? 0 : x0 + CPT;
    const bool own_left = lane == 0;
    const bool own_right = lane == 31 || x0 + CPT >= nx;

    unsigned fl[CPT];
#pragma unroll
    for (int k = 0; k < CPT; ++k) fl[k] = LBM_BOUNDARY;
    if (active) {
        if (CPT == 4) {
            const uint2 q = *reinterpret_cast<const uint2*>(flags + (r0 + (IDX)x0));
            fl[0] = q.x & 0xffffu; fl[1] = q.x >> 16; fl[CPT > 2 ? 2 : 0] = q.y & 0xffffu; fl[CPT > 3 ? 3 : 0] = q.y >> 16;
        } else {
            const unsigned q = *reinterpret_cast<const unsigned*>(flags + (r0 + (IDX)x0));
            fl[0] = q & 0xffffu; fl[1] = q >> 16;
        }
    }

    R d[9][CPT];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const IDX row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
        const T* Aj = A + ((IDX)j * N + row);
        R v[CPT];
#pragma unroll
        for (int k = 0; k < CPT; ++k) v[k] = R(0);
        if (active) VecN<ST, CPT>::ld(Aj + (IDX)x0, v);
        if (EX(j) == 0) {
#pragma unroll
            for (int k = 0; k < CPT; ++k) d[j][k] = v[k];
        } else if (EX(j) == 1) {  // source x - 1
            R prev = __shfl_up_sync(0xffffffffu, v[CPT - 1], 1);
            if (own_left && active) prev = ST::ldu(Aj + xl);
            d[j][0] = prev;
#pragma unroll
            for (int k = 1; k < CPT; ++k) d[j][k] = v[k - 1];
        } else {  // source x + 1
            R next = __shfl_down_sync(0xffffffffu, v[0], 1);
            if (own_right && active) next = ST::ldu(Aj + xr);
#pragma unroll
            for (int k = 0; k < CPT - 1; ++k) d[j][k] = v[k + 1];
            d[j][CPT - 1] = next;
            if (x0 + CPT > nx && active) {  // row end inside this group: cell nx-1 wraps to 0
                const int k = nx - 1 - x0;
                d[j][k < 0 ? 0 : k] = ST::ldu(Aj);
            }
        }
    }
    // warp-uniform fast path: every cell of the warp is plain fluid (bulk, ghost or unknown
    // material, no solid pull source) -- no boundary rule to test per cell
    bool plain = true;
#pragma unroll
    for (int k = 0; k < CPT; ++k) plain = plain && (fl[k] & FL_PLAIN) && x0 + k < nx;
    const bool fast = __all_sync(0xffffffffu, !active || plain);
    if (!active) return;

    R mr[CPT], mu[CPT], mv[CPT];
    if (fast) {
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            R dk[9], o[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) dk[j] = d[j][k];
            if constexpr (ST::dtype == LBM_DTYPE_F16 || ST::dtype == LBM_DTYPE_BF16)
                bgk_plain_fast(dk, omega, R(ST::UNIT), o, mr[k], mu[k], mv[k]);
            else
                phys_collide<R, LBM_COLLISION_BGK, true>(dk, LBM_BULK, fl[k], (size_t)(r0 + (IDX)(x0 + k)), flags, info,
                                                         omega, o, mr[k], mu[k], mv[k], R(ST::UNIT));
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j][k] = o[j];
        }
    } else {
#pragma unroll
    for (int k = 0; k < CPT; ++k) {
        const unsigned f = fl[k];
        const int m = (int)(f & FL_MAT_MASK);
        const int x = x0 + k;
        const IDX c = r0 + (IDX)x;
        R dk[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) dk[j] = d[j][k];
        if (is_solid(m) || x >= nx) {
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j][k] = R(0);
            mr[k] = R(0); mu[k] = R(0); mv[k] = R(0);
            continue;
        }
        if (m == LBM_OUTLET) {  // zero-gradient: e_x = -1 populations come from the own column
            dk[3] = ST::ldu(A + (3 * N + r0 + (IDX)x));
            dk[6] = ST::ldu(A + (6 * N + rp + (IDX)x));
            dk[7] = ST::ldu(A + (7 * N + rm + (IDX)x));
        }
        if (f & (0xFFu << (FL_DIR_SHIFT + 1))) {  // some pull source is solid: bounce back
#pragma unroll
            for (int j = 1; j < 9; ++j) {
                if (f & (1u << (FL_DIR_SHIFT + j))) {
                    R v = ST::ldu(A + (c + (IDX)INV(j) * N));
                    if (f & FL_MOVING) {
                        int sx = x - EX(j);
                        if (m == LBM_OUTLET && EX(j) == -1) sx = x;
                        sx = sx < 0 ? nx - 1 : (sx >= nx ? 0 : sx);
                        const IDX srow = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
                        const lbm_lattice_info si = info[srow + sx];
                        const R uw = R(EX(j)) * R(si.vx) + R(EY(j)) * R(si.vy);
                        if (uw != R(0)) v = add_rn(v, mul_rn(R(6) * PW<R>(j) * R(ST::UNIT), uw));
                    }
                    dk[j] = v;
                }
            }
        }
        R o[9];
        phys_collide<R>(dk, m, f, (size_t)c, flags, info, omega, o, mr[k], mu[k], mv[k], R(ST::UNIT));
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j][k] = o[j];
    }
    }
    if constexpr (SR) {
        const uint32_t q = sr_hash((uint32_t)(r0 + (IDX)x0) ^ seed);
#pragma unroll
        for (int j = 0; j < 9; ++j)
            Vec2<ST>::st_sr(B + ((IDX)j * N + r0 + (IDX)x0), d[j], q * sr_mul(2 * j), q * sr_mul(2 * j + 1));
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) VecN<ST, CPT>::st(B + ((IDX)j * N + r0 + (IDX)x0), d[j]);
    }
    if (MACRO) {
#pragma unroll
        for (int k = 0; k < CPT; ++k) {
            macro[r0 + (IDX)(x0 + k)] = (float)mr[k];
            macro[N + r0 + (IDX)(x0 + k)] = (float)mu[k];
            macro[2 * N + r0 + (IDX)(x0 + k)] = (float)mv[k];
        }
    }
}

}  // namespace lbm
