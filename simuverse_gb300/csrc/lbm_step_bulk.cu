// lbm_step_bulk.cu -- physics-mode step fed by bulk asynchronous copies into shared memory.
//
// A tile is TW = 512 consecutive cells of one row.  For each tile, thread 0 starts one
// cp.async.bulk per population plane -- plane j's source row is y - e_y(j), columns
// [x0 - H, x0 + TW + H) with H = 16 bytes of elements, so every copy starts and ends on
// a 16-byte boundary -- plus the tile's flag words; they all complete on the stage's
// mbarrier.  Halo elements beyond the row ends (x = -1 -> nx-1, x = nx -> 0) are patched
// with plain loads.  Blocks are persistent and double-buffered: while a block computes
// tile i from one stage, the copies of its tile i+1 fill the other, so bytes stay in
// flight independently of register occupancy.  Each thread reads its four cells of every
// plane as one aligned vector from shared memory, builds the +-x shifted vectors with
// warp shuffles (lanes 0 / 31 read their halo element), collides (phys_collide) and
// writes each plane with one aligned vector store.
//
// Every mbarrier wait is bounded (1 s): a block that gives up records LBM_ERR_TIMEOUT in
// the handle's status word, waits (bounded again) for the copies it started, and returns.
//
// Requirement: nx % 8 == 0 (16-byte aligned rows and flag segments).  Algorithmic traffic
// per cell update: 9 loads + 9 stores of the stored type.
#include <algorithm>

#include "lbm_cell.cuh"
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbm {

namespace {

__device__ __forceinline__ unsigned smem_u32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long* bar, unsigned count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(unsigned long long* bar, unsigned bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)), "r"(bytes) : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(unsigned long long* bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    return ok != 0;
}

__device__ __forceinline__ void bulk_g2s(void* dst, const void* src, unsigned bytes, unsigned long long* bar) {
    asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                     smem_u32(dst)),
                 "l"(src), "r"(bytes), "r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// bounded wait on phase `parity`; false after ~limit_ns
__device__ __forceinline__ bool mbar_wait_bounded(unsigned long long* bar, unsigned parity,
                                                  unsigned long long limit_ns) {
    if (mbar_try_wait(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!mbar_try_wait(bar, parity)) {
        if (now_ns() - t0 > limit_ns) return false;
    }
    return true;
}

template <class T>
struct SmemVec4;
template <>
struct SmemVec4<float> {
    __device__ __forceinline__ static void ld(const float* p, float (&r)[4]) {
        const float4 q = *reinterpret_cast<const float4*>(p);
        r[0] = q.x; r[1] = q.y; r[2] = q.z; r[3] = q.w;
    }
};
template <>
struct SmemVec4<double> {
    __device__ __forceinline__ static void ld(const double* p, double (&r)[4]) {
        const double2 a = reinterpret_cast<const double2*>(p)[0];
        const double2 b = reinterpret_cast<const double2*>(p)[1];
        r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
    }
};
template <>
struct SmemVec4<__half> {
    __device__ __forceinline__ static void ld(const __half* p, float (&r)[4]) {
        const uint2 q = *reinterpret_cast<const uint2*>(p);
        const float2 a = __half22float2(*reinterpret_cast<const __half2*>(&q.x));
        const float2 b = __half22float2(*reinterpret_cast<const __half2*>(&q.y));
        r[0] = a.x * F16_INV_SCALE; r[1] = a.y * F16_INV_SCALE; r[2] = b.x * F16_INV_SCALE; r[3] = b.y * F16_INV_SCALE;
    }
};
template <>
struct SmemVec4<__nv_bfloat16> {
    __device__ __forceinline__ static void ld(const __nv_bfloat16* p, float (&r)[4]) {
        const uint2 q = *reinterpret_cast<const uint2*>(p);
        const float2 a = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.x));
        const float2 b = __bfloat1622float2(*reinterpret_cast<const __nv_bfloat162*>(&q.y));
        r[0] = a.x; r[1] = a.y; r[2] = b.x; r[3] = b.y;
    }
};

template <class ST>
__device__ __forceinline__ void vec4_store(typename ST::T* p, const typename ST::R (&r)[4]);
template <>
__device__ __forceinline__ void vec4_store<StoreF32>(float* p, const float (&r)[4]) {
    *reinterpret_cast<float4*>(p) = make_float4(r[0], r[1], r[2], r[3]);
}
template <>
__device__ __forceinline__ void vec4_store<StoreF64>(double* p, const double (&r)[4]) {
    reinterpret_cast<double2*>(p)[0] = make_double2(r[0], r[1]);
    reinterpret_cast<double2*>(p)[1] = make_double2(r[2], r[3]);
}
template <>
__device__ __forceinline__ void vec4_store<StoreF16>(__half* p, const float (&r)[4]) {
    const __half2 a = __floats2half2_rn(r[0] * F16_SCALE, r[1] * F16_SCALE);
    const __half2 b = __floats2half2_rn(r[2] * F16_SCALE, r[3] * F16_SCALE);
    uint2 q;
    q.x = *reinterpret_cast<const unsigned*>(&a);
    q.y = *reinterpret_cast<const unsigned*>(&b);
    *reinterpret_cast<uint2*>(p) = q;
}
template <>
__device__ __forceinline__ void vec4_store<StoreBF16>(__nv_bfloat16* p, const float (&r)[4]) {
    const __nv_bfloat162 a = __floats2bfloat162_rn(r[0], r[1]);
    const __nv_bfloat162 b = __floats2bfloat162_rn(r[2], r[3]);
    uint2 q;
    q.x = *reinterpret_cast<const unsigned*>(&a);
    q.y = *reinterpret_cast<const unsigned*>(&b);
    *reinterpret_cast<uint2*>(p) = q;
}

}  // namespace

constexpr int BULK_TPB = 128;           // threads per block
constexpr int BULK_TW = 4 * BULK_TPB;   // cells per tile (one row segment)
constexpr int BULK_STAGES = 2;          // tiles in flight per block
constexpr unsigned long long BULK_WAIT_NS = 1000000000ull;

template <class ST>
struct BulkLayout {
    using T = typename ST::T;
    static constexpr int H = 16 / (int)sizeof(T);  // halo elements (16 bytes)
    static constexpr int ROW = BULK_TW + 2 * H;    // elements per plane segment
    static constexpr int PLANE_BYTES = ROW * (int)sizeof(T);
    static constexpr int FLAG_BYTES = BULK_TW * 2;
    static constexpr int STAGE_BYTES = 9 * PLANE_BYTES + FLAG_BYTES;
    static constexpr int SMEM = BULK_STAGES * STAGE_BYTES + 16 * BULK_STAGES;
};

struct TileGeom {
    int y, x0, tw;
};

__device__ __forceinline__ TileGeom tile_geom(int t, int tiles_per_row, int nx) {
    TileGeom g;
    g.y = t / tiles_per_row;
    g.x0 = (t - g.y * tiles_per_row) * BULK_TW;
    g.tw = min(BULK_TW, nx - g.x0);
    return g;
}

// thread 0: start the copies of tile g into a stage; threads 0..8 / 16..24 patch the halo
// elements beyond the row ends (called by all threads)
template <class ST>
__device__ __forceinline__ void bulk_issue(const typename ST::T* __restrict__ A, const uint16_t* __restrict__ flags,
                                           typename ST::T* sp, uint16_t* sfl, unsigned long long* bar, TileGeom g,
                                           int nx, int ny) {
    using L = BulkLayout<ST>;
    const int tid = threadIdx.x;
    const size_t N = (size_t)nx * ny;
    const int ym = g.y == 0 ? ny - 1 : g.y - 1, yp = g.y == ny - 1 ? 0 : g.y + 1;
    const size_t r0 = (size_t)g.y * nx, rm = (size_t)ym * nx, rp = (size_t)yp * nx;
    const int c0 = max(g.x0 - L::H, 0), c1 = min(g.x0 + g.tw + L::H, nx);
    if (tid == 0) {
        const unsigned seg_bytes = (unsigned)(c1 - c0) * (unsigned)sizeof(typename ST::T);
        const int sofs = c0 - (g.x0 - L::H);
        // bounds-checked build: every copy's last element inside its buffer, else none is
        // started and the stage's phase completes with no bytes (its contents are stale)
        bool ok = in_bounds(r0 + (size_t)g.x0 + (size_t)g.tw - 1, N, BS_BULK_COPY);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const size_t row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
            ok = in_bounds((size_t)j * N + row + (size_t)c1 - 1, 9 * N, BS_BULK_COPY) && ok;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // earlier generic reads of this stage
        mbar_arrive_expect_tx(bar, ok ? 9 * seg_bytes + (unsigned)g.tw * 2u : 0u);
        if (ok) {
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const size_t row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
                bulk_g2s(sp + j * L::ROW + sofs, A + (size_t)j * N + row + c0, seg_bytes, bar);
            }
            bulk_g2s(sfl, flags + r0 + g.x0, (unsigned)g.tw * 2u, bar);
        }
    }
    if (tid < 9 && g.x0 == 0) {  // x = -1 wraps to nx - 1
        const int j = tid;
        const size_t row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
        const size_t i = (size_t)j * N + row + (nx - 1);
        if (in_bounds(i, 9 * N, BS_BULK_PULL)) sp[j * L::ROW + L::H - 1] = A[i];
    }
    if (tid >= 16 && tid < 25 && g.x0 + g.tw == nx) {  // x = nx wraps to 0
        const int j = tid - 16;
        const size_t row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
        const size_t i = (size_t)j * N + row;
        if (in_bounds(i, 9 * N, BS_BULK_PULL)) sp[j * L::ROW + L::H + g.tw] = A[i];
    }
}

template <class ST, bool MACRO>
__global__ void __launch_bounds__(BULK_TPB) k_phys_step_bulk(const typename ST::T* __restrict__ A,
                                                             typename ST::T* __restrict__ B,
                                                             uint16_t* __restrict__ flags,
                                                             lbm_lattice_info* __restrict__ info, typename ST::R omega,
                                                             int nx, int ny, float* __restrict__ macro,
                                                             int* __restrict__ status) {
    using T = typename ST::T;
    using R = typename ST::R;
    using L = BulkLayout<ST>;
    extern __shared__ __align__(128) unsigned char smem_raw[];
    unsigned long long* bars = reinterpret_cast<unsigned long long*>(smem_raw + BULK_STAGES * L::STAGE_BYTES);
    auto stage_planes = [&](int st) { return reinterpret_cast<T*>(smem_raw + st * L::STAGE_BYTES); };
    auto stage_flags = [&](int st) {
        return reinterpret_cast<uint16_t*>(smem_raw + st * L::STAGE_BYTES + 9 * L::PLANE_BYTES);
    };

    __shared__ int s_ok;
    const int tid = threadIdx.x, lane = tid & 31;
    const int tiles_per_row = (nx + BULK_TW - 1) / BULK_TW;
    const int ntiles = tiles_per_row * ny;
    const size_t N = (size_t)nx * ny;

    if (tid == 0) {
        for (int st = 0; st < BULK_STAGES; ++st) mbar_init(&bars[st], 1);
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    __syncthreads();
    // prologue: fill every stage
    for (int st = 0; st < BULK_STAGES; ++st) {
        const int t = blockIdx.x + st * gridDim.x;
        if (t < ntiles)
            bulk_issue<ST>(A, flags, stage_planes(st), stage_flags(st), &bars[st], tile_geom(t, tiles_per_row, nx), nx, ny);
    }
    __syncthreads();

    int it = 0;
    for (int t = blockIdx.x; t < ntiles; t += gridDim.x, ++it) {
        const int st = it % BULK_STAGES;
        const unsigned parity = (unsigned)(it / BULK_STAGES) & 1u;
        const TileGeom g = tile_geom(t, tiles_per_row, nx);
        // thread 0 waits with a time limit and the block follows its outcome, so the block
        // leaves together (no thread is left behind at a __syncthreads)
        if (tid == 0) s_ok = mbar_wait_bounded(&bars[st], parity, BULK_WAIT_NS) ? 1 : 0;
        __syncthreads();
        if (!s_ok) {
            if (tid == 0) {
                atomicExch(status, LBM_ERR_TIMEOUT);
                for (int k = 1; k < BULK_STAGES; ++k)  // let copies already started land before leaving
                    mbar_wait_bounded(&bars[(it + k) % BULK_STAGES], (unsigned)((it + k) / BULK_STAGES) & 1u,
                                      BULK_WAIT_NS);
            }
            return;
        }
        mbar_wait_bounded(&bars[st], parity, BULK_WAIT_NS);  // phase already complete: acquire it
        const T* sp = stage_planes(st);
        const uint16_t* sfl = stage_flags(st);
        const int ym = g.y == 0 ? ny - 1 : g.y - 1, yp = g.y == ny - 1 ? 0 : g.y + 1;
        const size_t r0 = (size_t)g.y * nx, rm = (size_t)ym * nx, rp = (size_t)yp * nx;
        const int xl = 4 * tid;
        const bool active = xl < g.tw;
        R d[9][4];
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const T* s = sp + j * L::ROW + L::H + xl;
            R v[4] = {R(0), R(0), R(0), R(0)};
            if (active) SmemVec4<T>::ld(s, v);
            if (EX(j) == 0) {
#pragma unroll
                for (int k = 0; k < 4; ++k) d[j][k] = v[k];
            } else if (EX(j) == 1) {
                R prev = __shfl_up_sync(0xffffffffu, v[3], 1);
                if (lane == 0 && active) prev = ST::to_r(s[-1]);
                d[j][0] = prev; d[j][1] = v[0]; d[j][2] = v[1]; d[j][3] = v[2];
            } else {
                R next = __shfl_down_sync(0xffffffffu, v[0], 1);
                if ((lane == 31 || xl + 4 >= g.tw) && active) next = ST::to_r(s[4]);
                d[j][0] = v[1]; d[j][1] = v[2]; d[j][2] = v[3]; d[j][3] = next;
            }
        }
        if (active) {
            R mr[4], mu[4], mv[4];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const unsigned f = sfl[xl + k];
                const int m = (int)(f & FL_MAT_MASK);
                const int x = g.x0 + xl + k;
                const size_t c = r0 + x;
                if (is_solid(m)) {
#pragma unroll
                    for (int j = 0; j < 9; ++j) d[j][k] = R(0);
                    mr[k] = R(0); mu[k] = R(0); mv[k] = R(0);
                    continue;
                }
                R dk[9];
#pragma unroll
                for (int j = 0; j < 9; ++j) dk[j] = d[j][k];
                if (m == LBM_OUTLET) {  // zero-gradient: e_x = -1 populations come from the own column
                    dk[3] = ST::to_r(sp[3 * L::ROW + L::H + xl + k]);
                    dk[6] = ST::to_r(sp[6 * L::ROW + L::H + xl + k]);
                    dk[7] = ST::to_r(sp[7 * L::ROW + L::H + xl + k]);
                }
                if (f & (0xFFu << (FL_DIR_SHIFT + 1))) {  // some pull source is solid: bounce back
#pragma unroll
                    for (int j = 1; j < 9; ++j) {
                        if (f & (1u << (FL_DIR_SHIFT + j))) {
                            const size_t ib = c + (size_t)INV(j) * N;
                            R v = in_bounds(ib, 9 * N, BS_BULK_PULL) ? ST::ld(A + ib) : R(0);
                            if (f & FL_MOVING) {
                                int sx = x - EX(j);
                                if (m == LBM_OUTLET && EX(j) == -1) sx = x;
                                sx = sx < 0 ? nx - 1 : (sx >= nx ? 0 : sx);
                                const size_t srow = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
                                lbm_lattice_info si = {0, 0, 0.0f, 0.0f};
                                if (in_bounds(srow + sx, N, BS_BULK_INFO)) si = info[srow + sx];
                                const R uw = R(EX(j)) * R(si.vx) + R(EY(j)) * R(si.vy);
                                if (uw != R(0)) v = add_rn(v, mul_rn(R(6) * PW<R>(j), uw));
                            }
                            dk[j] = v;
                        }
                    }
                }
                R o[9];
                phys_collide<R>(dk, m, f, c, flags, info, omega, o, mr[k], mu[k], mv[k]);
#pragma unroll
                for (int j = 0; j < 9; ++j) d[j][k] = o[j];
            }
            const size_t cs = r0 + g.x0 + xl;
#pragma unroll
            for (int j = 0; j < 9; ++j)
                if (in_bounds((size_t)j * N + cs + 3, 9 * N, BS_BULK_STORE)) vec4_store<ST>(B + (size_t)j * N + cs, d[j]);
            if (MACRO && in_bounds(2 * N + cs + 3, 3 * N, BS_BULK_MACRO)) {
                *reinterpret_cast<float4*>(macro + cs) =
                    make_float4((float)mr[0], (float)mr[1], (float)mr[2], (float)mr[3]);
                *reinterpret_cast<float4*>(macro + N + cs) =
                    make_float4((float)mu[0], (float)mu[1], (float)mu[2], (float)mu[3]);
                *reinterpret_cast<float4*>(macro + 2 * N + cs) =
                    make_float4((float)mv[0], (float)mv[1], (float)mv[2], (float)mv[3]);
            }
        }
        __syncthreads();  // every thread is done with this stage
        const int tn = t + BULK_STAGES * gridDim.x;
        if (tn < ntiles)
            bulk_issue<ST>(A, flags, stage_planes(st), stage_flags(st), &bars[st], tile_geom(tn, tiles_per_row, nx), nx,
                           ny);
    }
}

template <class ST, bool MACRO>
static cudaError_t bulk_t(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    using R = typename ST::R;
    using L = BulkLayout<ST>;
    // per device (the handle's device is current): the shared-memory attribute, resident
    // blocks per SM and the SM count
    struct Setup {
        int blocks_per_sm, sms;
    };
    static PerDevice<Setup> per_device;
    Setup su{};
    cudaError_t e = per_device.get(
        h->device,
        [&](Setup& v) {
            cudaError_t r = cudaFuncSetAttribute(k_phys_step_bulk<ST, MACRO>,
                                                 cudaFuncAttributeMaxDynamicSharedMemorySize, L::SMEM);
            if (r == cudaSuccess)
                r = cudaOccupancyMaxActiveBlocksPerMultiprocessor(&v.blocks_per_sm, k_phys_step_bulk<ST, MACRO>,
                                                                  BULK_TPB, L::SMEM);
            if (r == cudaSuccess) r = cudaDeviceGetAttribute(&v.sms, cudaDevAttrMultiProcessorCount, h->device);
            if (v.blocks_per_sm < 1) v.blocks_per_sm = 1;
            return r;
        },
        &su);
    if (e != cudaSuccess) return e;
    const int blocks_per_sm = su.blocks_per_sm, sms = su.sms;
    const R omega = sizeof(R) == 8 ? (R)h->omega_d : (R)h->omega;
    const long ntiles = (long)((h->nx + BULK_TW - 1) / BULK_TW) * h->ny;
    const long grid = std::min<long>(ntiles, (long)blocks_per_sm * sms);
    k_phys_step_bulk<ST, MACRO><<<(unsigned)grid, BULK_TPB, L::SMEM, s>>>((const T*)h->buf[h->cur],
                                                                          (T*)h->buf[h->cur ^ 1], h->d_flags,
                                                                          h->d_info, omega, h->nx, h->ny, h->d_macro,
                                                                          h->d_status);
    return cudaGetLastError();
}

bool bulk_step_supported(const lbm_handle* h) { return h->p.mode == LBM_MODE_PHYSICS && h->nx % 8 == 0; }

cudaError_t launch_phys_step_bulk(lbm_handle* h, bool write_macro, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return write_macro ? bulk_t<StoreF32, true>(h, s) : bulk_t<StoreF32, false>(h, s);
        case LBM_DTYPE_F64: return write_macro ? bulk_t<StoreF64, true>(h, s) : bulk_t<StoreF64, false>(h, s);
        case LBM_DTYPE_F16: return write_macro ? bulk_t<StoreF16, true>(h, s) : bulk_t<StoreF16, false>(h, s);
        default: return write_macro ? bulk_t<StoreBF16, true>(h, s) : bulk_t<StoreBF16, false>(h, s);
    }
}

#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_bulk(BoundsRecord* out) { return bounds_take_local(out); }
#endif

}  // namespace lbm
