// lbm_batch.cu -- the batched form: hundreds of independent lattices of uneven size
// (lid-driven cavities and channels) advanced together.
//
// Storage.  Every domain's rows are padded to a multiple of 4 cells (pitch) so the
// four-cells-per-thread update (lbm_cell4.cuh) applies; padding cells are solid and never
// read by a fluid cell.  Populations of all domains live in two pooled FP32 buffers
// (planes of domain d at pop_off[d] + j * pitch * ny), flags / info / macro in pooled
// arrays at cell_off[d].
//
// Work.  Domains are cut into tiles of (cells_per_thread * tx) x ty cells, or (linear tiles)
// into runs of tx * ty consecutive cells of the padded rows, which leave no partly filled
// tile at a domain's right edge; a tile list covers them all (one cell per thread, or four
// with vector accesses).
// Method 0: one cooperative persistent launch runs every step: blocks take tiles
// round-robin, then meet at a grid barrier before the next step.  The barrier spins with
// a time limit: a block that waits longer sets an error word (LBM_ERR_TIMEOUT), every
// waiting block sees it and leaves, and the host reads the status -- no trap, the context
// stays usable.  The launch (with the barrier reset) is captured once into a CUDA graph
// per (steps, parity) and replayed.  Method 1: one tile-list launch per step.  Method 2:
// one launch per domain per step (the plain loop a caller would write).
//
// Autotuning.  lbm_batch_tune times a few steps of each candidate (tx, ty, blocks per SM)
// and keeps the fastest; results are cached per shape class (total cells, domain count).
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <map>
#include <random>
#include <string>
#include <tuple>
#include <type_traits>
#include <vector>

#include "lbm_cell4.cuh"
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbm {

struct BatchDomain {
    size_t pop_off;   // element offset of plane 0 in the population pools
    size_t cell_off;  // cell offset in the flags / info pools (macro: 3 * cell_off)
    int nx, ny, pitch, scene;
    float omega, speed;
    float inv_pitch;  // 1 / pitch (row of a linear tile's cell)
};

struct BarrierState {
    unsigned int count;
    int error;
    int where_step;
    int where_block;
};

__device__ __forceinline__ unsigned long long global_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

__device__ __forceinline__ unsigned ld_acquire_u32(const unsigned* p) {
    unsigned v;
    asm volatile("ld.acquire.gpu.global.u32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

__device__ __forceinline__ int ld_relaxed_i32(const int* p) {
    int v;
    asm volatile("ld.relaxed.gpu.global.s32 %0, [%1];" : "=r"(v) : "l"(p) : "memory");
    return v;
}

// Grid barrier with a time limit; returns false when the batch is in error.
__device__ bool grid_barrier(BarrierState* bar, unsigned target, unsigned long long timeout_ns, int step) {
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0 && threadIdx.y == 0) {
        __threadfence();
        atomicAdd(&bar->count, 1u);
        const unsigned long long t0 = global_ns();
        int ok = 1;
        while (ld_acquire_u32(&bar->count) < target) {
            if (ld_relaxed_i32(&bar->error) != 0) { ok = 0; break; }
            if (global_ns() - t0 > timeout_ns) {
                if (atomicCAS(&bar->error, 0, LBM_ERR_TIMEOUT) == 0) {
                    bar->where_step = step;
                    bar->where_block = blockIdx.x;
                }
                ok = 0;
                break;
            }
            __nanosleep(100);
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// one tile = (cells_per_thread * blockDim.x) x blockDim.y cells of one domain, or (CPT == 0,
// linear tiles) blockDim.x * blockDim.y consecutive cells from cell tl.y of the padded rows
template <int CPT>
__device__ __forceinline__ void tile_update(const BatchDomain* __restrict__ doms, int4 tl, const float* __restrict__ A0,
                                            float* __restrict__ B0, uint16_t* __restrict__ flags,
                                            lbm_lattice_info* __restrict__ info, float* __restrict__ macro,
                                            bool write_macro) {
    const BatchDomain dm = doms[tl.x];
    if (CPT == 0) {
        // cells below 2^24 are exact in FP32, and the quotient's error is far below one row;
        // the two corrections make the row exact
        const int c = tl.y + (int)(threadIdx.y * blockDim.x + threadIdx.x);
        int y = (int)(((float)c + 0.5f) * dm.inv_pitch);
        int x = c - y * dm.pitch;
        if (x < 0) { --y; x += dm.pitch; }
        if (x >= dm.pitch) { ++y; x -= dm.pitch; }
        if (y >= dm.ny || x >= dm.nx) return;  // past the domain's end, or a padding column
        // pool base pointers and the domain's 32-bit offsets (not per-domain pointers: fewer
        // registers; lbm_batch_create keeps the pools below 2^32 elements)
        if (write_macro)
            phys_cell_update<StoreF32, true, LBM_COLLISION_BGK, false, uint32_t>(
                A0, B0, flags, info, dm.omega, x, y, dm.nx, dm.pitch, dm.ny, macro, 0u, (uint32_t)dm.pop_off,
                (uint32_t)dm.cell_off);
        else
            phys_cell_update<StoreF32, false, LBM_COLLISION_BGK, false, uint32_t>(
                A0, B0, flags, info, dm.omega, x, y, dm.nx, dm.pitch, dm.ny, macro, 0u, (uint32_t)dm.pop_off,
                (uint32_t)dm.cell_off);
        return;
    }
    const int y = tl.z + (int)threadIdx.y;
    if (y >= dm.ny) return;  // warp-uniform: a warp spans one row
    if (CPT == 1) {
        const int x = tl.y + (int)threadIdx.x;
        if (x >= dm.nx) return;
        if (write_macro)
            phys_cell_update<StoreF32, true, LBM_COLLISION_BGK, false, uint32_t>(
                A0, B0, flags, info, dm.omega, x, y, dm.nx, dm.pitch, dm.ny, macro, 0u, (uint32_t)dm.pop_off,
                (uint32_t)dm.cell_off);
        else
            phys_cell_update<StoreF32, false, LBM_COLLISION_BGK, false, uint32_t>(
                A0, B0, flags, info, dm.omega, x, y, dm.nx, dm.pitch, dm.ny, macro, 0u, (uint32_t)dm.pop_off,
                (uint32_t)dm.cell_off);
    } else {
        const int x0 = tl.y + (int)threadIdx.x * 4;
        const bool active = x0 < dm.nx;
        const float* A = A0 + dm.pop_off;
        float* B = B0 + dm.pop_off;
        if (write_macro)
            phys_cells4_update<StoreF32, true>(A, B, flags + dm.cell_off, info + dm.cell_off, dm.omega, x0, y, dm.nx,
                                               dm.pitch, dm.ny, active, macro + 3 * dm.cell_off);
        else
            phys_cells4_update<StoreF32, false>(A, B, flags + dm.cell_off, info + dm.cell_off, dm.omega, x0, y, dm.nx,
                                                dm.pitch, dm.ny, active, macro + 3 * dm.cell_off);
    }
}

// Kernel form KF: the tile form (KF % 10: 0 linear tiles, 1 one cell per thread, 4 four cells)
// and the register budget of the one-cell forms: 40 registers (6 blocks of 256 threads per SM,
// a few bytes of spills) for KF < 10, 32 registers (8 blocks: full occupancy, more spills) for
// KF >= 10; the autotuner times both.  Four cells per thread take their natural 128+.
constexpr int batch_min_blocks(int kf) { return kf >= 10 ? 8 : (kf == 4 ? 1 : 6); }

// method 0: all steps in one cooperative launch
template <int KF>
__global__ void __launch_bounds__(256, batch_min_blocks(KF)) k_batch_persistent(const BatchDomain* __restrict__ doms,
                                                          const int4* __restrict__ tiles, int ntiles, float* pool0,
                                                          float* pool1, uint16_t* flags, lbm_lattice_info* info,
                                                          float* macro, int nsteps, int cur0, BarrierState* bar,
                                                          unsigned long long timeout_ns, int skip_block, int skip_step) {
    for (int s = 0; s < nsteps; ++s) {
        const bool odd = ((cur0 + s) & 1) != 0;
        const float* A = odd ? pool1 : pool0;
        float* B = odd ? pool0 : pool1;
        const bool mac = (s == nsteps - 1);
        for (int t = blockIdx.x; t < ntiles; t += gridDim.x)
            tile_update<KF % 10>(doms, tiles[t], A, B, flags, info, macro, mac);
        if ((int)blockIdx.x == skip_block && s == skip_step) return;  // injected missing arrival (tests)
        if (!grid_barrier(bar, (unsigned)(s + 1) * gridDim.x, timeout_ns, s)) return;
    }
}
// method 1: one step over the tile list, one tile per block
template <int KF>
__global__ void __launch_bounds__(256, batch_min_blocks(KF)) k_batch_tiles(const BatchDomain* __restrict__ doms, const int4* __restrict__ tiles,
                                                     const float* A, float* B, uint16_t* flags, lbm_lattice_info* info,
                                                     float* macro, int write_macro) {
    tile_update<KF % 10>(doms, tiles[blockIdx.x], A, B, flags, info, macro, write_macro != 0);
}

// method 2: one domain per launch (the single-lattice one-cell kernel's layout)
__global__ void __launch_bounds__(128, 12) k_batch_domain(BatchDomain dm, const float* A0, float* B0, uint16_t* flags,
                                                          lbm_lattice_info* info, float* macro, int write_macro) {
    const int x = blockIdx.x * 128 + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= dm.nx) return;
    const float* A = A0 + dm.pop_off;
    float* B = B0 + dm.pop_off;
    if (write_macro)
        phys_cell_update<StoreF32, true>(A, B, flags + dm.cell_off, info + dm.cell_off, dm.omega, x, y, dm.nx, dm.pitch,
                                         dm.ny, macro + 3 * dm.cell_off);
    else
        phys_cell_update<StoreF32, false>(A, B, flags + dm.cell_off, info + dm.cell_off, dm.omega, x, y, dm.nx,
                                          dm.pitch, dm.ny, macro + 3 * dm.cell_off);
}

// masks of the batch: cavity = solid ring with the row y = 0 moving at `speed`; channel =
// walls y = 0, ny-1, parabolic Zou-He inlet (peak `speed`) at x = 0, outflow at x = nx-1.
// Padding cells x >= nx are solid.
__global__ void k_batch_info(const BatchDomain* __restrict__ doms, int ndom, lbm_lattice_info* __restrict__ info) {
    const int d = blockIdx.y;
    if (d >= ndom) return;
    const BatchDomain dm = doms[d];
    const size_t n = (size_t)dm.pitch * dm.ny;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % dm.pitch), y = (int)(c / dm.pitch);
        lbm_lattice_info r;
        r.material = LBM_BULK;
        r.block_iter = -1;
        r.vx = 0.0f;
        r.vy = 0.0f;
        if (x >= dm.nx) {
            r.material = LBM_BOUNDARY;
        } else if (dm.scene == LBM_SCENE_CAVITY) {
            if (x == 0 || x == dm.nx - 1 || y == 0 || y == dm.ny - 1) r.material = LBM_BOUNDARY;
            if (y == 0 && x >= 1 && x <= dm.nx - 2) r.vx = dm.speed;
        } else {
            if (y == 0 || y == dm.ny - 1) {
                r.material = LBM_BOUNDARY;
            } else if (x == 0) {
                r.material = LBM_INLET;
                const double H = (double)(dm.ny - 2), s = (double)y - 0.5;
                r.vx = (float)(4.0 * (double)dm.speed * s * (H - s) / (H * H));
            } else if (x == dm.nx - 1) {
                r.material = LBM_OUTLET;
            }
        }
        info[dm.cell_off + c] = r;
    }
}

__global__ void k_batch_flags(const BatchDomain* __restrict__ doms, int ndom, const lbm_lattice_info* __restrict__ info,
                              uint16_t* __restrict__ flags) {
    const int d = blockIdx.y;
    if (d >= ndom) return;
    const BatchDomain dm = doms[d];
    const size_t n = (size_t)dm.pitch * dm.ny;
    const lbm_lattice_info* in = info + dm.cell_off;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < n; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % dm.pitch), y = (int)(c / dm.pitch);
        const int code = in[c].material;
        unsigned fl = (code >= 0 && code <= 15) ? (unsigned)code : 0u;
        if (!is_solid(code) && x < dm.nx) {
            for (int j = 1; j < 9; ++j) {
                int sx = x - EX(j), sy = y - EY(j);
                if (code == LBM_OUTLET && EX(j) == -1) sx = x;
                sx = sx < 0 ? dm.nx - 1 : (sx >= dm.nx ? 0 : sx);
                sy = sy < 0 ? dm.ny - 1 : (sy >= dm.ny ? 0 : sy);
                const lbm_lattice_info s = in[(size_t)sy * dm.pitch + sx];
                if (is_solid(s.material)) {
                    fl |= 1u << (FL_DIR_SHIFT + j);
                    if (s.vx != 0.0f || s.vy != 0.0f) fl |= FL_MOVING;
                }
            }
            fl |= plain_bit(fl);
        }
        flags[dm.cell_off + c] = (uint16_t)fl;
    }
}

#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_batch(BoundsRecord* out) { return bounds_take_local(out); }
#endif

}  // namespace lbm

// =====================================================================================
// host side
// =====================================================================================
namespace {

int bfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lbm::set_error(code, buf);
}

#define B_CK(call)                                                                                      \
    do {                                                                                                \
        cudaError_t e_ = (call);                                                                        \
        if (e_ != cudaSuccess) return bfail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));   \
    } while (0)

#define B_TRY(expr)            \
    do {                       \
        int r_ = (expr);       \
        if (r_ < 0) return r_; \
    } while (0)

struct TuneKey {
    long cells_class;
    int ndom;
    bool operator<(const TuneKey& o) const { return std::tie(cells_class, ndom) < std::tie(o.cells_class, o.ndom); }
};
std::map<TuneKey, lbm_batch_config> g_tune_cache;

}  // namespace

struct lbm_batch {
    std::vector<lbm_domain_desc> desc;
    std::vector<lbm::BatchDomain> doms;
    lbm::BatchDomain* d_doms = nullptr;
    int4* d_tiles = nullptr;
    int ntiles = 0;
    float* pool[2] = {nullptr, nullptr};
    uint16_t* d_flags = nullptr;
    lbm_lattice_info* d_info = nullptr;
    float* d_macro = nullptr;
    double* d_part = nullptr;
    lbm::BarrierState* d_bar = nullptr;
    size_t pop_elems = 0, cells = 0, live_cells = 0;
    int cur = 0;
    cudaStream_t stream = nullptr, own_stream = nullptr;
    int device = 0, sms = 0;
    lbm_batch_config cfg;
    unsigned long long timeout_ns = 1000000000ull;
    // cached graph of the persistent launch
    cudaGraphExec_t graph = nullptr;
    int graph_steps = -1, graph_cur = -1, graph_grid = -1;
    uint64_t launches = 0, steps = 0;
};

namespace {

void free_graph(lbm_batch* b) {
    if (b->graph) cudaGraphExecDestroy(b->graph);
    b->graph = nullptr;
    b->graph_steps = b->graph_cur = b->graph_grid = -1;
}

int build_tiles(lbm_batch* b) {
    const int tw = b->cfg.cells_per_thread * b->cfg.tile_threads_x, th = b->cfg.tile_rows;
    std::vector<int4> tiles;
    for (size_t d = 0; d < b->doms.size(); ++d) {
        const lbm::BatchDomain& dm = b->doms[d];
        if (b->cfg.linear) {
            const int run = b->cfg.tile_threads_x * b->cfg.tile_rows, n = dm.pitch * dm.ny;
            for (int c0 = 0; c0 < n; c0 += run) tiles.push_back(make_int4((int)d, c0, 0, 1));
            continue;
        }
        for (int y0 = 0; y0 < dm.ny; y0 += th)
            for (int x0 = 0; x0 < dm.pitch; x0 += tw) tiles.push_back(make_int4((int)d, x0, y0, 0));
    }
    if (b->d_tiles) cudaFree(b->d_tiles);
    b->d_tiles = nullptr;
    B_CK(cudaMalloc((void**)&b->d_tiles, tiles.size() * sizeof(int4)));
    B_CK(cudaMemcpy(b->d_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice));
    b->ntiles = (int)tiles.size();
    free_graph(b);
    return LBM_OK;
}

// the kernels' form KF (k_batch_persistent): tile form + 10 for the 32-register budget
int tile_form(const lbm_batch* b) {
    const int f = b->cfg.linear ? 0 : b->cfg.cells_per_thread;
    return f != 4 && b->cfg.full_occupancy ? f + 10 : f;
}

// calls fn(std::integral_constant<int, KF>) for the configured form
template <class F>
int with_form(const lbm_batch* b, F&& fn) {
    switch (tile_form(b)) {
        case 0: return fn(std::integral_constant<int, 0>{});
        case 1: return fn(std::integral_constant<int, 1>{});
        case 10: return fn(std::integral_constant<int, 10>{});
        case 11: return fn(std::integral_constant<int, 11>{});
        default: return fn(std::integral_constant<int, 4>{});
    }
}

int persistent_grid(lbm_batch* b, int* grid) {
    int per_sm = 0;
    const int threads = b->cfg.tile_threads_x * b->cfg.tile_rows;
    B_TRY(with_form(b, [&](auto kf) {
        B_CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, lbm::k_batch_persistent<decltype(kf)::value>,
                                                           threads, 0));
        return LBM_OK;
    }));
    if (per_sm < 1) return bfail(LBM_ERR_ARG, "persistent kernel does not fit %d threads per block", threads);
    const int want = b->cfg.blocks_per_sm > 0 ? b->cfg.blocks_per_sm : per_sm;
    *grid = std::min(want, per_sm) * b->sms;
    return LBM_OK;
}

int launch_persistent(lbm_batch* b, int nsteps, int skip_block, int skip_step, cudaStream_t s) {
    int grid = 0;
    B_TRY(persistent_grid(b, &grid));
    B_CK(cudaMemsetAsync(b->d_bar, 0, sizeof(lbm::BarrierState), s));
    cudaLaunchConfig_t lc;
    std::memset(&lc, 0, sizeof(lc));
    lc.gridDim = dim3((unsigned)grid);
    lc.blockDim = dim3((unsigned)b->cfg.tile_threads_x, (unsigned)b->cfg.tile_rows);
    lc.stream = s;
    cudaLaunchAttribute attr[1];
    attr[0].id = cudaLaunchAttributeCooperative;
    attr[0].val.cooperative = 1;
    lc.attrs = attr;
    lc.numAttrs = 1;
    B_TRY(with_form(b, [&](auto kf) {
        B_CK(cudaLaunchKernelEx(&lc, lbm::k_batch_persistent<decltype(kf)::value>, (const lbm::BatchDomain*)b->d_doms,
                                (const int4*)b->d_tiles, b->ntiles, b->pool[0], b->pool[1], b->d_flags, b->d_info,
                                b->d_macro, nsteps, b->cur, b->d_bar, b->timeout_ns, skip_block, skip_step));
        return LBM_OK;
    }));
    return LBM_OK;
}

int run_persistent_graph(lbm_batch* b, int nsteps) {
    int grid = 0;
    B_TRY(persistent_grid(b, &grid));
    if (!b->graph || b->graph_steps != nsteps || b->graph_cur != b->cur || b->graph_grid != grid) {
        free_graph(b);
        cudaStream_t cs;
        B_CK(cudaStreamCreateWithFlags(&cs, cudaStreamNonBlocking));
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamBeginCapture(cs, cudaStreamCaptureModeThreadLocal);
        int r = LBM_OK;
        if (e == cudaSuccess) r = launch_persistent(b, nsteps, -1, -1, cs);
        cudaError_t e2 = cudaStreamEndCapture(cs, &g);
        if (e == cudaSuccess && r == LBM_OK && e2 == cudaSuccess) e = cudaGraphInstantiate(&b->graph, g, 0);
        if (g) cudaGraphDestroy(g);
        cudaStreamDestroy(cs);
        if (r != LBM_OK) return r;
        if (e != cudaSuccess || e2 != cudaSuccess)
            return bfail(LBM_ERR_CUDA, "graph capture of the persistent launch: %s",
                         cudaGetErrorString(e != cudaSuccess ? e : e2));
        b->graph_steps = nsteps;
        b->graph_cur = b->cur;
        b->graph_grid = grid;
    }
    B_CK(cudaGraphLaunch(b->graph, b->stream));
    return LBM_OK;
}

int run_steps(lbm_batch* b, int nsteps, int method) {
    if (nsteps == 0) return LBM_OK;
    if (method == LBM_BATCH_PERSISTENT) {
        B_TRY(run_persistent_graph(b, nsteps));
        b->launches += 1;
    } else if (method == LBM_BATCH_TILE_LAUNCHES) {
        const dim3 block((unsigned)b->cfg.tile_threads_x, (unsigned)b->cfg.tile_rows);
        for (int s = 0; s < nsteps; ++s) {
            const float* A = b->pool[(b->cur + s) & 1];
            float* B = b->pool[(b->cur + s + 1) & 1];
            B_TRY(with_form(b, [&](auto kf) {
                lbm::k_batch_tiles<decltype(kf)::value><<<(unsigned)b->ntiles, block, 0, b->stream>>>(
                    b->d_doms, b->d_tiles, A, B, b->d_flags, b->d_info, b->d_macro, s == nsteps - 1);
                return LBM_OK;
            }));
            B_CK(cudaGetLastError());
        }
        b->launches += nsteps;
    } else {
        for (int s = 0; s < nsteps; ++s) {
            const float* A = b->pool[(b->cur + s) & 1];
            float* B = b->pool[(b->cur + s + 1) & 1];
            for (const lbm::BatchDomain& dm : b->doms) {
                const dim3 grid((unsigned)((dm.nx + 127) / 128), (unsigned)dm.ny);
                lbm::k_batch_domain<<<grid, 128, 0, b->stream>>>(dm, A, B, b->d_flags, b->d_info, b->d_macro,
                                                                 s == nsteps - 1);
            }
            B_CK(cudaGetLastError());
        }
        b->launches += (uint64_t)nsteps * b->doms.size();
    }
    b->cur = (b->cur + nsteps) & 1;
    b->steps += nsteps;
    return LBM_OK;
}

int check_batch(const lbm_batch* b) {
    if (!b) return bfail(LBM_ERR_ARG, "null batch");
    return LBM_OK;
}

int read_status(lbm_batch* b) {
    lbm::BarrierState st;
    B_CK(cudaMemcpyAsync(&st, b->d_bar, sizeof(st), cudaMemcpyDeviceToHost, b->stream));
    B_CK(cudaStreamSynchronize(b->stream));
    if (st.error != 0)
        return bfail(st.error, "persistent batch kernel: grid barrier timed out at step %d (block %d)", st.where_step,
                     st.where_block);
    return LBM_OK;
}

double unit53(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

}  // namespace

extern "C" {

int lbm_batch_generate(int32_t n, uint64_t seed, lbm_domain_desc* out) {
    if (n < 1 || !out) return bfail(LBM_ERR_ARG, "need n >= 1 and an output array");
    std::mt19937_64 g(seed);
    const double l0 = std::log(64.0), l1 = std::log(1024.0);
    for (int i = 0; i < n; ++i) {
        // nx log-uniform in [64, 1024], ny = nx * aspect; redrawn until ny is in range too
        int nx = 0, ny = 0;
        do {
            const double side = std::exp(l0 + (l1 - l0) * unit53(g));
            const double aspect = 0.5 + 1.5 * unit53(g);
            nx = (int)std::lround(side);
            ny = (int)std::lround(side * aspect);
        } while (ny < 64 || ny > 1024);
        const double tau = 0.55 + 0.45 * unit53(g);
        const double speed = 0.02 + 0.08 * unit53(g);
        const double kind = unit53(g);
        lbm_domain_desc& d = out[i];
        std::memset(&d, 0, sizeof(d));
        d.nx = nx;
        d.ny = ny;
        d.scene = kind < 0.5 ? LBM_SCENE_CAVITY : LBM_SCENE_CHANNEL;
        d.tau = (float)tau;
        d.speed = (float)speed;
    }
    return LBM_OK;
}

int lbm_batch_create(int32_t n, const lbm_domain_desc* desc, lbm_batch** out) {
    if (!out || !desc || n < 1) return bfail(LBM_ERR_ARG, "need n >= 1 domains");
    *out = nullptr;
    size_t cells = 0, live = 0, pop = 0;
    std::vector<lbm::BatchDomain> doms((size_t)n);
    for (int i = 0; i < n; ++i) {
        const lbm_domain_desc& d = desc[i];
        if (d.nx < 4 || d.ny < 4 || d.nx > 65535 || d.ny > 65535)
            return bfail(LBM_ERR_ARG, "domain %d: size %dx%d outside [4, 65535]", i, d.nx, d.ny);
        if (d.scene != LBM_SCENE_CAVITY && d.scene != LBM_SCENE_CHANNEL)
            return bfail(LBM_ERR_ARG, "domain %d: scene must be cavity or channel", i);
        if (!(d.tau > 0.5f) || !std::isfinite(d.tau)) return bfail(LBM_ERR_ARG, "domain %d: tau must exceed 0.5", i);
        if (!(std::fabs(d.speed) < 0.3f)) return bfail(LBM_ERR_ARG, "domain %d: |speed| must stay below 0.3", i);
        lbm::BatchDomain& dm = doms[(size_t)i];
        dm.nx = d.nx;
        dm.ny = d.ny;
        dm.pitch = (d.nx + 3) & ~3;
        dm.inv_pitch = 1.0f / (float)dm.pitch;
        dm.scene = d.scene;
        dm.omega = 1.0f / d.tau;
        dm.speed = d.speed;
        dm.cell_off = cells;
        dm.pop_off = pop;
        const size_t nc = (size_t)dm.pitch * dm.ny;
        cells += (nc + 31) & ~(size_t)31;  // 128-byte aligned starts
        pop += 9 * ((nc + 31) & ~(size_t)31);
        live += (size_t)d.nx * d.ny;
    }
    if (cells > ((size_t)1 << 31)) return bfail(LBM_ERR_ARG, "batch of %zu cells exceeds 2^31", cells);
    // the one-cell updates address the pools with 32-bit element offsets
    if (pop >= ((size_t)1 << 32))
        return bfail(LBM_ERR_ARG, "batch of %zu population elements reaches 2^32 (at most ~477 M padded cells)", pop);
    lbm_batch* b = new (std::nothrow) lbm_batch();
    if (!b) return bfail(LBM_ERR_NOMEM, "out of host memory");
    b->desc.assign(desc, desc + n);
    b->doms = doms;
    b->cells = cells;
    b->live_cells = live;
    b->pop_elems = pop;
    b->cfg.tile_threads_x = 128;
    b->cfg.tile_rows = 2;
    b->cfg.cells_per_thread = 1;
    b->cfg.linear = 0;
    b->cfg.full_occupancy = 0;
    b->cfg.blocks_per_sm = 0;
    b->cfg.method = LBM_BATCH_PERSISTENT;
    b->cfg.ms_per_step = 0.0f;
    cudaError_t e = cudaGetDevice(&b->device);
    if (e == cudaSuccess) e = cudaDeviceGetAttribute(&b->sms, cudaDevAttrMultiProcessorCount, b->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&b->own_stream, cudaStreamNonBlocking);
    b->stream = b->own_stream;
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->pool[0], pop * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->pool[1], pop * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_flags, cells * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_info, cells * sizeof(lbm_lattice_info));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_macro, 3 * cells * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_part, (size_t)lbm::RED_BLOCKS * 6 * sizeof(double) + 64 * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_bar, sizeof(lbm::BarrierState));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b->d_doms, doms.size() * sizeof(lbm::BatchDomain));
    if (e == cudaSuccess)
        e = cudaMemcpy(b->d_doms, doms.data(), doms.size() * sizeof(lbm::BatchDomain), cudaMemcpyHostToDevice);
    // equilibrium at rest: all deviations zero
    if (e == cudaSuccess) e = cudaMemset(b->pool[0], 0, pop * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(b->pool[1], 0, pop * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(b->d_macro, 0, 3 * cells * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(b->d_info, 0, cells * sizeof(lbm_lattice_info));
    if (e == cudaSuccess) e = cudaMemset(b->d_flags, 0, cells * sizeof(uint16_t));
    if (e == cudaSuccess) e = cudaMemset(b->d_bar, 0, sizeof(lbm::BarrierState));
    if (e == cudaSuccess) {
        lbm::k_batch_info<<<dim3(64, (unsigned)n), 256>>>(b->d_doms, n, b->d_info);
        lbm::k_batch_flags<<<dim3(64, (unsigned)n), 256>>>(b->d_doms, n, b->d_info, b->d_flags);
        e = cudaGetLastError();
    }
    if (e == cudaSuccess) e = cudaDeviceSynchronize();
    int r = e == cudaSuccess ? build_tiles(b) : bfail(LBM_ERR_CUDA, "batch set-up: %s", cudaGetErrorString(e));
    if (r != LBM_OK) {
        lbm_batch_destroy(b);
        return r;
    }
    *out = b;
    return LBM_OK;
}

int lbm_batch_destroy(lbm_batch* b) {
    if (!b) return LBM_OK;
    cudaSetDevice(b->device);
    if (b->stream) cudaStreamSynchronize(b->stream);
    free_graph(b);
    cudaFree(b->pool[0]);
    cudaFree(b->pool[1]);
    cudaFree(b->d_flags);
    cudaFree(b->d_info);
    cudaFree(b->d_macro);
    cudaFree(b->d_part);
    cudaFree(b->d_bar);
    cudaFree(b->d_doms);
    cudaFree(b->d_tiles);
    if (b->own_stream) cudaStreamDestroy(b->own_stream);
    delete b;
    return LBM_OK;
}

int lbm_batch_set_stream(lbm_batch* b, void* s) {
    B_TRY(check_batch(b));
    B_CK(cudaStreamSynchronize(b->stream));
    b->stream = s ? (cudaStream_t)s : b->own_stream;
    return LBM_OK;
}

int lbm_batch_info(const lbm_batch* b, int32_t* ndomains, uint64_t* cells) {
    B_TRY(check_batch(b));
    if (ndomains) *ndomains = (int32_t)b->doms.size();
    if (cells) *cells = b->live_cells;
    return LBM_OK;
}

int lbm_batch_set_config(lbm_batch* b, const lbm_batch_config* cfg) {
    B_TRY(check_batch(b));
    if (!cfg) return bfail(LBM_ERR_ARG, "null config");
    const int tx = cfg->tile_threads_x, ty = cfg->tile_rows;
    if (tx < 32 || tx % 32 != 0 || ty < 1 || tx * ty > 256)
        return bfail(LBM_ERR_ARG, "tile of %d x %d threads: tx must be a multiple of 32 and tx*ty <= 256", tx, ty);
    if (cfg->blocks_per_sm < 0 || cfg->blocks_per_sm > 32) return bfail(LBM_ERR_ARG, "blocks_per_sm out of range");
    if (cfg->method < LBM_BATCH_PERSISTENT || cfg->method > LBM_BATCH_DOMAIN_LOOP) return bfail(LBM_ERR_ARG, "unknown method");
    if (cfg->cells_per_thread != 1 && cfg->cells_per_thread != 4) return bfail(LBM_ERR_ARG, "cells_per_thread must be 1 or 4");
    if (cfg->linear != 0 && cfg->linear != 1) return bfail(LBM_ERR_ARG, "linear must be 0 or 1");
    if (cfg->full_occupancy != 0 && cfg->full_occupancy != 1) return bfail(LBM_ERR_ARG, "full_occupancy must be 0 or 1");
    if (cfg->linear) {
        if (cfg->cells_per_thread != 1) return bfail(LBM_ERR_ARG, "linear tiles take one cell per thread");
        for (const lbm::BatchDomain& dm : b->doms)
            if ((size_t)dm.pitch * dm.ny >= ((size_t)1 << 24))
                return bfail(LBM_ERR_ARG, "linear tiles need domains below 2^24 cells");
    }
    B_CK(cudaStreamSynchronize(b->stream));
    const bool retile = tx != b->cfg.tile_threads_x || ty != b->cfg.tile_rows ||
                        cfg->cells_per_thread != b->cfg.cells_per_thread || cfg->linear != b->cfg.linear;
    b->cfg = *cfg;
    if (retile) B_TRY(build_tiles(b));
    free_graph(b);
    return LBM_OK;
}

int lbm_batch_get_config(const lbm_batch* b, lbm_batch_config* cfg) {
    B_TRY(check_batch(b));
    if (!cfg) return bfail(LBM_ERR_ARG, "null config");
    *cfg = b->cfg;
    return LBM_OK;
}

int lbm_batch_step(lbm_batch* b, int32_t nsteps) {
    LbmRange range_("lbm_batch_step");
    B_TRY(check_batch(b));
    if (nsteps < 0) return bfail(LBM_ERR_ARG, "negative step count");
    B_CK(cudaSetDevice(b->device));
    return run_steps(b, nsteps, b->cfg.method);
}

int lbm_batch_status(lbm_batch* b) {
    B_TRY(check_batch(b));
    B_CK(cudaSetDevice(b->device));
    return read_status(b);
}

int lbm_batch_inject_missing_arrival(lbm_batch* b, int32_t nsteps, int32_t block, int32_t step, uint64_t timeout_ns) {
    B_TRY(check_batch(b));
    if (nsteps < 1 || block < 0 || step < 0 || step >= nsteps) return bfail(LBM_ERR_ARG, "bad injection point");
    B_CK(cudaSetDevice(b->device));
    const unsigned long long keep = b->timeout_ns;
    b->timeout_ns = timeout_ns ? timeout_ns : keep;
    const int r = launch_persistent(b, nsteps, block, step, b->stream);
    b->timeout_ns = keep;
    B_TRY(r);
    b->launches += 1;
    return read_status(b);
}

int lbm_batch_tune(lbm_batch* b, int32_t trial_steps, lbm_batch_config* best_out) {
    LbmRange range_("lbm_batch_tune");
    B_TRY(check_batch(b));
    if (trial_steps < 1) return bfail(LBM_ERR_ARG, "trial_steps must be >= 1");
    B_CK(cudaSetDevice(b->device));
    const TuneKey key{(long)std::lround(std::log2((double)b->live_cells + 1.0) * 4.0), (int)b->doms.size()};
    auto it = g_tune_cache.find(key);
    if (it != g_tune_cache.end()) {
        B_TRY(lbm_batch_set_config(b, &it->second));
        if (best_out) *best_out = it->second;
        return LBM_OK;
    }
    const int cpts[] = {0, 1, 4, 10, 11};  // 0: linear tiles; + 10: the 32-register budget
    const int txs[] = {32, 64, 128, 256};
    const int tys[] = {1, 2, 4};
    const int bps[] = {0, 2, 4, 6, 8, 12, 16};
    lbm_batch_config best = b->cfg;
    best.method = LBM_BATCH_PERSISTENT;
    float best_ms = 1e30f;
    cudaEvent_t e0, e1;
    B_CK(cudaEventCreate(&e0));
    B_CK(cudaEventCreate(&e1));
    for (int cpt : cpts)
    for (int tx : txs)
        for (int ty : tys) {
            if (tx * ty > 256) continue;
            for (int bp : bps) {
                lbm_batch_config c = b->cfg;
                if (cpt % 10 == 0 && ty != 1) continue;  // a linear run depends on tx * ty only
                c.cells_per_thread = cpt % 10 == 0 ? 1 : cpt % 10;
                c.linear = cpt % 10 == 0 ? 1 : 0;
                c.full_occupancy = cpt >= 10 ? 1 : 0;
                c.tile_threads_x = tx;
                c.tile_rows = ty;
                c.blocks_per_sm = bp;
                c.method = LBM_BATCH_PERSISTENT;
                if (lbm_batch_set_config(b, &c) != LBM_OK) continue;
                int grid = 0;
                if (persistent_grid(b, &grid) != LBM_OK) continue;
                if (bp > 0 && grid != bp * b->sms) continue;  // over the occupancy limit: same as a smaller bp
                if (run_steps(b, 2, LBM_BATCH_PERSISTENT) != LBM_OK) continue;  // warm-up (and graph capture)
                B_CK(cudaEventRecord(e0, b->stream));
                B_TRY(run_steps(b, trial_steps, LBM_BATCH_PERSISTENT));
                B_CK(cudaEventRecord(e1, b->stream));
                B_CK(cudaEventSynchronize(e1));
                B_TRY(read_status(b));
                float ms = 0.0f;
                B_CK(cudaEventElapsedTime(&ms, e0, e1));
                ms /= (float)trial_steps;
                if (ms < best_ms) {
                    best_ms = ms;
                    best = c;
                    best.ms_per_step = ms;
                }
            }
        }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    B_TRY(lbm_batch_set_config(b, &best));
    g_tune_cache[key] = best;
    if (best_out) *best_out = best;
    return LBM_OK;
}

int lbm_batch_read_macro(lbm_batch* b, int32_t i, float* rho, float* ux, float* uy) {
    B_TRY(check_batch(b));
    if (i < 0 || i >= (int)b->doms.size()) return bfail(LBM_ERR_ARG, "domain %d out of range", i);
    B_CK(cudaSetDevice(b->device));
    const lbm::BatchDomain& dm = b->doms[(size_t)i];
    const size_t n = (size_t)dm.pitch * dm.ny;
    float* dst[3] = {rho, ux, uy};
    for (int k = 0; k < 3; ++k)
        if (dst[k])
            B_CK(cudaMemcpy2DAsync(dst[k], (size_t)dm.nx * sizeof(float), b->d_macro + 3 * dm.cell_off + k * n,
                                   (size_t)dm.pitch * sizeof(float), (size_t)dm.nx * sizeof(float), (size_t)dm.ny,
                                   cudaMemcpyDeviceToHost, b->stream));
    B_CK(cudaStreamSynchronize(b->stream));
    return LBM_OK;
}

int lbm_batch_read_populations(lbm_batch* b, int32_t i, float* f) {
    B_TRY(check_batch(b));
    if (i < 0 || i >= (int)b->doms.size() || !f) return bfail(LBM_ERR_ARG, "bad domain index or output");
    B_CK(cudaSetDevice(b->device));
    const lbm::BatchDomain& dm = b->doms[(size_t)i];
    const size_t n = (size_t)dm.pitch * dm.ny, plane = (size_t)dm.nx * dm.ny;
    for (int j = 0; j < 9; ++j)
        B_CK(cudaMemcpy2DAsync(f + j * plane, (size_t)dm.nx * sizeof(float), b->pool[b->cur] + dm.pop_off + j * n,
                               (size_t)dm.pitch * sizeof(float), (size_t)dm.nx * sizeof(float), (size_t)dm.ny,
                               cudaMemcpyDeviceToHost, b->stream));
    B_CK(cudaStreamSynchronize(b->stream));
    for (int j = 0; j < 9; ++j) {
        const float w = lbm::PW<float>(j);
        for (size_t c = 0; c < plane; ++c) f[j * plane + c] += w;
    }
    return LBM_OK;
}

int lbm_batch_read_info(lbm_batch* b, int32_t i, lbm_lattice_info* info) {
    B_TRY(check_batch(b));
    if (i < 0 || i >= (int)b->doms.size() || !info) return bfail(LBM_ERR_ARG, "bad domain index or output");
    B_CK(cudaSetDevice(b->device));
    const lbm::BatchDomain& dm = b->doms[(size_t)i];
    B_CK(cudaMemcpy2DAsync(info, (size_t)dm.nx * sizeof(lbm_lattice_info), b->d_info + dm.cell_off,
                           (size_t)dm.pitch * sizeof(lbm_lattice_info), (size_t)dm.nx * sizeof(lbm_lattice_info),
                           (size_t)dm.ny, cudaMemcpyDeviceToHost, b->stream));
    B_CK(cudaStreamSynchronize(b->stream));
    return LBM_OK;
}

int lbm_batch_conservation(lbm_batch* b, int32_t i, double out[3]) {
    B_TRY(check_batch(b));
    if (i < 0 || i >= (int)b->doms.size() || !out) return bfail(LBM_ERR_ARG, "bad domain index or output");
    B_CK(cudaSetDevice(b->device));
    const lbm::BatchDomain& dm = b->doms[(size_t)i];
    double* d_out = b->d_part + (size_t)lbm::RED_BLOCKS * 6;
    B_CK(lbm::launch_conservation_f32_phys(b->pool[b->cur] + dm.pop_off, b->d_flags + dm.cell_off,
                                           (size_t)dm.pitch * dm.ny, b->d_part, d_out, b->stream));
    B_CK(cudaMemcpyAsync(out, d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, b->stream));
    B_CK(cudaStreamSynchronize(b->stream));
    return LBM_OK;
}

int lbm_batch_counters(const lbm_batch* b, uint64_t* steps, uint64_t* launches) {
    B_TRY(check_batch(b));
    if (steps) *steps = b->steps;
    if (launches) *launches = b->launches;
    return LBM_OK;
}

}  // extern "C"
