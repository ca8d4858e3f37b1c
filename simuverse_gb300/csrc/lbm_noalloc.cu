// lbm_noalloc.cu -- FP64 mass / momentum sums over caller-owned device buffers, with no
// allocation by the library.
//
// Who needs it.  lbm_conservation works on a handle, and a handle allocates its device
// buffers when it is created.  Some callers cannot allocate at all: a host application
// whose own runtime owns every device buffer (the simulation state lives in buffers it
// allocated itself and only lends out), a process whose device memory is already claimed
// by another allocator's pool, or a real-time loop that must not pay for cudaMalloc's
// implicit device synchronisation.  For them, lbm_conservation_noalloc takes the
// population and info buffers they already hold and writes the three sums into an output
// buffer they also hold.  The library itself calls no cudaMalloc, cudaFree or other
// allocating routine on this path.
//
// Scratch.  The per-block partial sums live in g_noalloc_partials, a file-scope
// __device__ array of NOALLOC_BLOCKS x 3 doubles (29,184 bytes) that every GPU loading the
// library keeps until the process exits.  Host code cannot use the array's name as a
// device address (on the host it names a stand-in object), so the first call on each
// device resolves the address with cudaGetSymbolAddress, with that device current, and
// caches it; make that first call before any stream capture.  The cached address belongs to
// the device's primary context (the CUDA runtime's): calls must run with that context
// current, and a cudaDeviceReset, which destroys it, invalidates the cache.  Each call overwrites all
// NOALLOC_BLOCKS partial triples before the final pass reads them, so nothing has to be
// cleared between calls.  All calls share the one array: two calls whose kernels overlap
// on the GPU (for example on two streams) race on it and may return wrong sums.
//
// Results.  The reduction uses the same fixed grid, the same per-thread assignment and
// the same summation order as lbm_conservation, so for the same populations the sums are
// bit-identical.
#include <mutex>

#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace {

constexpr int NOALLOC_BLOCKS = lbm::RED_BLOCKS;  // 1216 partial triples
constexpr int NOALLOC_TPB = lbm::RED_TPB;
constexpr int NOALLOC_MAX_DEVICES = 64;
constexpr size_t NOALLOC_MAX_CELLS = (size_t)1 << 30;  // the library's lattice limit

static __device__ __align__(256) double g_noalloc_partials[NOALLOC_BLOCKS * 3];

std::mutex g_setup_mutex;
double* g_partials_addr[NOALLOC_MAX_DEVICES] = {};

template <int K>
__device__ __forceinline__ void noalloc_block_sum(double (&v)[K], double* smem) {
#pragma unroll
    for (int k = 0; k < K; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) smem[k * 32 + warp] = v[k];
    __syncthreads();
    if (warp == 0) {
        const int nw = blockDim.x >> 5;
#pragma unroll
        for (int k = 0; k < K; ++k) {
            v[k] = lane < nw ? smem[k * 32 + lane] : 0.0;
#pragma unroll
            for (int o = 16; o > 0; o >>= 1) v[k] += __shfl_down_sync(0xffffffffu, v[k], o);
        }
    }
}

// per-block partials: physics mode skips solid cells and counts 1 per fluid cell (the
// stored values are f - w); reference mode sums every slot of every cell (walls hold the
// populations in transit)
template <class ST, int MODE>
__global__ void __launch_bounds__(NOALLOC_TPB) k_noalloc_partials(const typename ST::T* __restrict__ A,
                                                                  const lbm_lattice_info* __restrict__ info, size_t N,
                                                                  double* __restrict__ part) {
    __shared__ double smem[3 * 32];
    double v[3] = {0.0, 0.0, 0.0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += stride) {
        if (MODE == LBM_MODE_PHYSICS) {
            if (lbm::is_solid(info[c].material)) continue;
            v[0] += 1.0;
        }
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const double f = (double)ST::to_r(A[c + (size_t)j * N]);
            v[0] += f;
            v[1] += (double)lbm::EX(j) * f;
            v[2] += (double)lbm::EY(j) * f;
        }
    }
    noalloc_block_sum<3>(v, smem);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 3 + 0] = v[0];
        part[blockIdx.x * 3 + 1] = v[1];
        part[blockIdx.x * 3 + 2] = v[2];
    }
}

__global__ void __launch_bounds__(NOALLOC_TPB) k_noalloc_final(const double* __restrict__ part, int nparts,
                                                               double* __restrict__ out) {
    __shared__ double smem[3 * 32];
    double v[3] = {0.0, 0.0, 0.0};
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < 3; ++k) v[k] += part[b * 3 + k];
    noalloc_block_sum<3>(v, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < 3; ++k) out[k] = v[k];
}

// once per device, with that device current: the device address of the scratch array
int partials_address(double** out) {
    int dev = -1;
    cudaError_t e = cudaGetDevice(&dev);
    if (e != cudaSuccess) return lbm::set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
    if (dev < 0 || dev >= NOALLOC_MAX_DEVICES)
        return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: device ordinal beyond 63");
    std::lock_guard<std::mutex> lock(g_setup_mutex);
    if (!g_partials_addr[dev]) {
        double* p = nullptr;
        e = cudaGetSymbolAddress((void**)&p, g_noalloc_partials);
        if (e != cudaSuccess || !p)
            return lbm::set_error(LBM_ERR_CUDA, "lbm_conservation_noalloc: cudaGetSymbolAddress of the scratch failed");
        g_partials_addr[dev] = p;
    }
    *out = g_partials_addr[dev];
    return LBM_OK;
}

template <class ST>
cudaError_t launch_noalloc(const void* pops, int mode, const lbm_lattice_info* info, size_t N, double* part,
                           double* out, cudaStream_t s) {
    const auto* A = (const typename ST::T*)pops;
    if (mode == LBM_MODE_PHYSICS)
        k_noalloc_partials<ST, LBM_MODE_PHYSICS><<<NOALLOC_BLOCKS, NOALLOC_TPB, 0, s>>>(A, info, N, part);
    else
        k_noalloc_partials<ST, LBM_MODE_REFERENCE><<<NOALLOC_BLOCKS, NOALLOC_TPB, 0, s>>>(A, info, N, part);
    k_noalloc_final<<<1, NOALLOC_TPB, 0, s>>>(part, NOALLOC_BLOCKS, out);
    return cudaGetLastError();
}

}  // namespace

extern "C" int lbm_conservation_noalloc(const void* d_populations, int32_t dtype, int32_t mode,
                                        const lbm_lattice_info* d_info, int32_t nx, int32_t ny, double* d_out,
                                        void* cuda_stream) {
    if (!d_populations || !d_out) return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: null buffer");
    if (mode != LBM_MODE_REFERENCE && mode != LBM_MODE_PHYSICS)
        return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: unknown mode");
    if (dtype < LBM_DTYPE_F32 || dtype > LBM_DTYPE_BF16 || (mode == LBM_MODE_REFERENCE && dtype != LBM_DTYPE_F32))
        return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: dtype not valid for this mode");
    if (mode == LBM_MODE_PHYSICS && !d_info)
        return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: physics mode needs the info records");
    if (nx < 1 || ny < 1) return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: empty lattice");
    const size_t N = (size_t)nx * (size_t)ny;
    if (N > NOALLOC_MAX_CELLS)
        return lbm::set_error(LBM_ERR_ARG, "lbm_conservation_noalloc: lattice larger than 2^30 cells");
    double* part = nullptr;
    const int r = partials_address(&part);
    if (r != LBM_OK) return r;
    cudaStream_t s = (cudaStream_t)cuda_stream;
    cudaError_t e;
    switch (dtype) {
        case LBM_DTYPE_F32: e = launch_noalloc<lbm::StoreF32>(d_populations, mode, d_info, N, part, d_out, s); break;
        case LBM_DTYPE_F64: e = launch_noalloc<lbm::StoreF64>(d_populations, mode, d_info, N, part, d_out, s); break;
        case LBM_DTYPE_F16: e = launch_noalloc<lbm::StoreF16>(d_populations, mode, d_info, N, part, d_out, s); break;
        default: e = launch_noalloc<lbm::StoreBF16>(d_populations, mode, d_info, N, part, d_out, s); break;
    }
    if (e != cudaSuccess) return lbm::set_error(LBM_ERR_CUDA, cudaGetErrorString(e));
    return LBM_OK;
}
