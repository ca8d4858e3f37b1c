// lbm_internal.h -- handle layout and kernel launchers shared by the C ABI (lbm_api.cpp)
// and the kernels (lbm_kernels.cu).  Not installed; the public surface is include/lbm.h.
#pragma once

#include <cuda_runtime.h>
#include <stddef.h>
#include <stdint.h>

#include <mutex>
#include <string>
#include <vector>

#include "../../include/lbm.h"

// NVTX ranges around the entry points, visible in Nsight tools (header-only NVTX 3; no ranges
// where the toolkit lacks it).  One object per call: LbmRange r("lbm_step");
#if __has_include(<nvtx3/nvToolsExt.h>)
#include <nvtx3/nvToolsExt.h>
struct LbmRange {
    explicit LbmRange(const char* name) { nvtxRangePushA(name); }
    ~LbmRange() { nvtxRangePop(); }
    LbmRange(const LbmRange&) = delete;
    LbmRange& operator=(const LbmRange&) = delete;
};
#else
struct LbmRange {
    explicit LbmRange(const char*) {}
};
#endif

struct lbm_handle {
    lbm_params p;
    int nx = 0, ny = 0;
    size_t N = 0;
    int fluid_ty = 0;  // d2q9_node.rs:53-57: 1 for the cavity, else 0
    bool tiled = false;  // populations in the tiled layout (pop_index), 16-bit storage only
    float tau = 0.6f, omega = 1.0f / 0.6f;
    double omega_d = 1.0 / (double)0.6f;  // 1 / tau in FP64, for FP64 storage
    void* buf[2] = {nullptr, nullptr};  // ping-pong population buffers (9*N each)
    int cur = 0;                        // buffer holding the state the next step reads
    uint16_t* d_flags = nullptr;
    lbm_lattice_info* d_info = nullptr;
    std::vector<lbm_lattice_info> host_info;  // D2Q9Node::lattice_info_data
    std::vector<double> scene_disks;  // the channel's disk list while its upload may still read it
    bool host_info_lazy = false;  // host_info not built yet: the scene mask was built on the device
    float* d_macro = nullptr;                 // rho, ux, uy planes
    double* d_part = nullptr;                 // reduction partials
    unsigned long long* d_count = nullptr;
    int* d_status = nullptr;  // kernel status word (LBM_ERR_TIMEOUT from a bounded wait)
    cudaStream_t stream = nullptr;
    cudaStream_t own_stream = nullptr;
    uint64_t steps = 0;
    uint64_t launches = 0;
    bool stepped_since_init = false;  // macro_tex holds (0,0,0,1) right after init
    float pre_x = 0.0f, pre_y = 0.0f;  // FluidSimulator::pre_pos
    int device = 0;
    // device copy of host_info for batched edits (lbm_apply_edits); uploaded on first use
    lbm_lattice_info* d_host_info = nullptr;
    bool host_mirror_valid = false;
    void* d_edits = nullptr;  // edit lists of lbm_apply_edits
    size_t edits_cap = 0;
};

namespace lbm {

// Launch set-up that belongs to one device: function attributes are set per device context
// and SM counts may differ between devices.  PerDevice<T> keeps one T per device ordinal,
// filled once by the caller's set-up under a mutex (thread-safe, each device on its own).
constexpr int MAX_DEVICES = 64;
template <class T>
struct PerDevice {
    std::mutex mu;
    T val[MAX_DEVICES] = {};
    bool ready[MAX_DEVICES] = {};
    // the device's value, running setup(T&) -> cudaError_t the first time; an error leaves
    // the device not set up (the next call tries again)
    template <class F>
    cudaError_t get(int dev, F setup, T* out) {
        if (dev < 0 || dev >= MAX_DEVICES) return cudaErrorInvalidDevice;
        std::lock_guard<std::mutex> lock(mu);
        if (!ready[dev]) {
            T v{};
            const cudaError_t e = setup(v);
            if (e != cudaSuccess) return e;
            val[dev] = v;
            ready[dev] = true;
        }
        *out = val[dev];
        return cudaSuccess;
    }
    // the device's value if it was set up, without setting it up
    bool peek(int dev, T* out) {
        if (dev < 0 || dev >= MAX_DEVICES) return false;
        std::lock_guard<std::mutex> lock(mu);
        if (!ready[dev]) return false;
        *out = val[dev];
        return true;
    }
};

// bounds-checked builds (LBM_BOUNDS_CHECK, see in_bounds in lbm_common.cuh): the number of
// out-of-range indices and the first one's index, extent and access site.  Each translation
// unit with step kernels keeps its own record on every device; bounds_take_* reads and
// clears it on the current device (lbm_bounds_report adds them up).
struct BoundsRecord {
    unsigned long long count, index, limit;
    int site, pad;
};
#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_kernels(BoundsRecord* out);  // lbm_kernels.cu: k_ref_step, k_phys_step
cudaError_t bounds_take_vec(BoundsRecord* out);      // lbm_step_vec.cu: k_phys_step_tiled
cudaError_t bounds_take_bulk(BoundsRecord* out);     // lbm_step_bulk.cu: k_phys_step_bulk
cudaError_t bounds_take_batch(BoundsRecord* out);    // lbm_batch.cu: the batched one-cell update
// one thread evaluates one index equal to its extent (no memory access): the record must show it
cudaError_t bounds_selftest(cudaStream_t s);
#endif

constexpr int TPB = 128;          // threads per block along x for the step kernels
constexpr int RED_BLOCKS = 1216;  // 8 x 152 SMs; fixed so FP64 sums have a fixed order
constexpr int RED_TPB = 256;

// records msg as the calling thread's lbm_last_error() and returns code
int set_error(int code, const char* msg);

inline size_t dtype_size(int dtype) { return dtype == LBM_DTYPE_F64 ? 8 : (dtype == LBM_DTYPE_F32 ? 4 : 2); }

// Kernel launchers (lbm_kernels.cu).  All return cudaGetLastError() of the launch.
cudaError_t launch_build_flags(const lbm_handle* h, cudaStream_t s);
// physics-mode scene mask on the device: base pattern of p's scene, then the disks
// (cx, cy, r triples in device memory) as obstacles
cudaError_t launch_build_scene(lbm_handle* h, cudaStream_t s);  // walls, inlet, outlet, lid
// the channel's disks into the info records; clear_state: also the solid-cell state in the
// populations and macro planes of an initialised lattice
cudaError_t launch_raster_disks(lbm_handle* h, const double* d_disks, int ndisks, bool clear_state, cudaStream_t s);
cudaError_t launch_ref_init(lbm_handle* h, cudaStream_t s);
cudaError_t launch_phys_init(lbm_handle* h, const float* d_rho, const float* d_ux, const float* d_uy,
                             cudaStream_t s);
cudaError_t launch_step(lbm_handle* h, bool write_macro, cudaStream_t s);
// four-cells-per-thread physics step (lbm_step_vec.cu)
bool vec_step_supported(const lbm_handle* h);
cudaError_t launch_phys_step_vec(lbm_handle* h, bool write_macro, cudaStream_t s);
cudaError_t launch_phys_step_vec2(lbm_handle* h, bool write_macro, cudaStream_t s);
cudaError_t launch_phys_step_tiled(lbm_handle* h, bool write_macro, cudaStream_t s);
cudaError_t launch_phys_step_ring(lbm_handle* h, bool write_macro, cudaStream_t s);
// the tiled layout applies: physics mode, 16-bit storage, BGK, nx % POP_TILE == 0, 9 N < 2^32
bool tiled_layout_eligible(const lbm_params& p);
// bulk-copy fed physics step (lbm_step_bulk.cu)
bool bulk_step_supported(const lbm_handle* h);
cudaError_t launch_phys_step_bulk(lbm_handle* h, bool write_macro, cudaStream_t s);
cudaError_t launch_conservation(lbm_handle* h, double* d_out3, cudaStream_t s);
cudaError_t launch_count_nonfinite(lbm_handle* h, cudaStream_t s);
cudaError_t launch_conservation_f32_phys(const float* A, const uint16_t* flags, size_t N, double* part, double* out,
                                         cudaStream_t s);
cudaError_t launch_macro_error(lbm_handle* h, lbm_handle* ref, double* d_out4, cudaStream_t s);
// batched interactive edits (lbm_kernels.cu): obstacles[j] = (x, y, seq), forces[k] =
// (cell, seq, vx bits, vy bits); sequence numbers give the order of the edits
struct EditObstacle {
    int32_t x, y, seq, pad;
};
struct EditForce {
    uint32_t cell;
    int32_t seq;
    float vx, vy;
};
cudaError_t launch_edits(lbm_handle* h, const EditObstacle* d_obst, int nobst, const EditForce* d_force, int nforce,
                         int row0, int row1, cudaStream_t s);
cudaError_t launch_macro_rgba16f(lbm_handle* h, uint16_t* d_rgba, cudaStream_t s);
cudaError_t launch_to_absolute(lbm_handle* h, const void* state, void* dst, int dst_dtype, cudaStream_t s);
cudaError_t launch_from_absolute(lbm_handle* h, const void* src, int src_dtype, void* state, cudaStream_t s);

}  // namespace lbm
