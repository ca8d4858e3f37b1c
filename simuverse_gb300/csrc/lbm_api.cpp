// lbm_api.cpp -- the C ABI of include/lbm.h: handle lifetime, masks, interactive edits,
// read-back, diagnostics and checkpoints.  Host logic mirrors simuverse's fluid module:
//   D2Q9Node::new                simuverse/src/fluid/d2q9_node.rs:31-209
//   init_lattice_material        simuverse/src/fluid/lattice.rs:26-98
//   D2Q9Node::add_obstacle       simuverse/src/fluid/d2q9_node.rs:215-245
//   D2Q9Node::reset_lattice_info simuverse/src/fluid/d2q9_node.rs:247-261
//   D2Q9Node::add_external_force simuverse/src/fluid/d2q9_node.rs:263-300
//   FluidSimulator::on_click / touch_move / update_uniforms
//                                simuverse/src/fluid/fluid_simulator.rs:137-193
// Built with -ffp-contract=off so that the float geometry of the masks and force strokes
// rounds as the Rust code does.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <string>
#include <vector>

#include "lbm_internal.h"

namespace {

thread_local std::string g_err;

int fail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define LBM_CK(call)                                                                                 \
    do {                                                                                             \
        cudaError_t e_ = (call);                                                                     \
        if (e_ != cudaSuccess) return fail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

#define LBM_TRY(expr)          \
    do {                       \
        int r_ = (expr);       \
        if (r_ < 0) return r_; \
    } while (0)

// Lattice memory.  A lattice's device buffers come from one stream-ordered pool per device
// that the library owns (cudaMallocFromPoolAsync on the lattice's stream).  lbm_destroy gives
// them back with cudaFreeAsync, and the pool keeps up to `retain` bytes of returned memory
// reserved, so the next lattice of a similar size is served from it without a device
// allocation (cudaMalloc of the 1.7 GB of a 4096^2 FP32 lattice takes about 0.5 ms).
std::mutex g_pool_mu;
uint64_t g_retain = 0;       // bytes a pool keeps; 0 until set: the default of each device
bool g_retain_set = false;
lbm::PerDevice<cudaMemPool_t> g_pools;

uint64_t default_retain(int dev) {
    size_t total = 0;
    cudaDeviceProp prop;
    if (cudaGetDeviceProperties(&prop, dev) == cudaSuccess) total = prop.totalGlobalMem;
    return std::min<uint64_t>((uint64_t)total / 8, (uint64_t)16 << 30);
}

cudaError_t device_pool(int dev, cudaMemPool_t* out) {
    return g_pools.get(
        dev,
        [&](cudaMemPool_t& pool) {
            cudaMemPoolProps props;
            std::memset(&props, 0, sizeof(props));
            props.allocType = cudaMemAllocationTypePinned;
            props.location.type = cudaMemLocationTypeDevice;
            props.location.id = dev;
            cudaError_t e = cudaMemPoolCreate(&pool, &props);
            if (e != cudaSuccess) return e;
            uint64_t keep;
            {
                std::lock_guard<std::mutex> lock(g_pool_mu);
                keep = g_retain_set ? g_retain : default_retain(dev);
            }
            e = cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep);
            if (e != cudaSuccess) cudaMemPoolDestroy(pool);
            return e;
        },
        out);
}

// bytes of device memory on the current device, ordered on stream s
template <class T>
cudaError_t pool_alloc(T** p, size_t bytes, cudaStream_t s) {
    *p = nullptr;
    int dev = 0;
    cudaError_t e = cudaGetDevice(&dev);
    cudaMemPool_t pool = nullptr;
    if (e == cudaSuccess) e = device_pool(dev, &pool);
    if (e == cudaSuccess) e = cudaMallocFromPoolAsync((void**)p, bytes, pool, s);
    return e;
}

void pool_free(void* p, cudaStream_t s) {
    if (p) cudaFreeAsync(p, s);
}

constexpr float OBSTACLE_RADIUS = 28.0f;  // fluid/mod.rs:1

bool sd_sphere(float px, float py, float r) {  // fluid/mod.rs:57-59 (glam Vec2::length)
    const float d = std::sqrt(px * px + py * py);
    return d <= r;
}

lbm_lattice_info make_info(int material, float vx = 0.0f, float vy = 0.0f, int block_iter = -1) {
    lbm_lattice_info r;
    r.material = material;
    r.block_iter = block_iter;
    r.vx = vx;
    r.vy = vy;
    return r;
}

// lattice.rs:26-98 (nz = 1)
void mask_reference(int nx, int ny, int scene, float lid, float inlet, std::vector<lbm_lattice_info>& out) {
    out.resize((size_t)nx * ny);
    const float s0x = (float)nx / 7.0f - OBSTACLE_RADIUS, s0y = (float)ny / 2.0f;
    const float s1x = (float)nx / 5.0f, s1y = (float)ny / 4.0f;
    const float s2x = (float)nx / 5.0f, s2y = (float)ny * 0.75f;
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            int m = LBM_BULK;
            float vx = 0.0f;
            if (scene == LBM_SCENE_CUSTOM) {
                if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) m = LBM_BOUNDARY;
            } else if (scene == LBM_SCENE_CAVITY) {
                if (x == 0 || x == nx - 1 || y == ny - 1) m = LBM_BOUNDARY;
                else if (y == 0) m = LBM_GHOST;
                else if (y == 1) { m = LBM_EXTERNAL_FORCE; vx = lid; }
            } else {  // Poiseuille
                if (y == 0 || y == ny - 1) m = LBM_BOUNDARY;
                else if (x == 0 || x == nx - 1) m = LBM_GHOST;
                else if (x == 1) { m = LBM_INLET; vx = inlet; }
                else if (x == nx - 2) m = LBM_OUTLET;
                else {
                    const float px = (float)x, py = (float)y;
                    if (sd_sphere(px - s0x, py - s0y, OBSTACLE_RADIUS) || sd_sphere(px - s1x, py - s1y, OBSTACLE_RADIUS) ||
                        sd_sphere(px - s2x, py - s2y, OBSTACLE_RADIUS))
                        m = LBM_OBSTACLE;
                }
            }
            out[(size_t)y * nx + x] = make_info(m, vx);
        }
}

// physics-mode lid-driven cavity: solid box, row y = 0 (screen top) moves with lid_vx
void mask_phys_cavity(int nx, int ny, float lid, std::vector<lbm_lattice_info>& out) {
    out.resize((size_t)nx * ny);
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            const bool wall = x == 0 || x == nx - 1 || y == 0 || y == ny - 1;
            const float vx = (y == 0 && x >= 1 && x <= nx - 2) ? lid : 0.0f;
            out[(size_t)y * nx + x] = make_info(wall ? LBM_BOUNDARY : LBM_BULK, vx);
        }
}

double unit53(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

// Channel: walls y = 0 and y = ny-1, Zou-He inlet x = 0 with the parabolic profile of a
// channel whose walls sit half-way between rows, outflow x = nx-1, and non-overlapping
// disks (radius U[rmin, rmax], gap >= 2 cells) placed by rejection sampling until the
// solid fraction is reached.
//
// The cells of disk (cx, cy, r): lattice points of its bounding box inside [1, nx-2] x
// [1, ny-2] with (x - cx)^2 + (y - cy)^2 <= r^2, evaluated as rounded FP64 products and sum
// (the device rasteriser k_raster_disks evaluates the same expression).
template <class F>
void disk_cells(int nx, int ny, double cx, double cy, double r, F&& visit) {
    const int x0 = (int)std::floor(cx - r), x1 = (int)std::ceil(cx + r);
    const int y0 = (int)std::floor(cy - r), y1 = (int)std::ceil(cy + r);
    for (int y = y0; y <= y1; ++y)
        for (int x = x0; x <= x1; ++x) {
            if (x < 1 || x > nx - 2 || y < 1 || y > ny - 2) continue;
            const double dx = (double)x - cx, dy = (double)y - cy;
            if (dx * dx + dy * dy <= r * r) visit((size_t)y * nx + x);
        }
}

// Number of cells disk_cells visits, one row at a time.  On a row the test holds on one run of
// x around cx: the rounded (x - cx)^2 does not decrease as |x - cx| grows, since rounding is
// monotone.  So the run's ends are found from sqrt(r^2 - dy^2) and corrected by evaluating
// the exact test, and the count equals the cell-by-cell loop's.
long disk_cell_count(int nx, int ny, double cx, double cy, double r) {
    const int bx0 = std::max((int)std::floor(cx - r), 1), bx1 = std::min((int)std::ceil(cx + r), nx - 2);
    const int by0 = std::max((int)std::floor(cy - r), 1), by1 = std::min((int)std::ceil(cy + r), ny - 2);
    const int xf = (int)std::floor(cx);  // the lattice points nearest cx are xf and xf + 1
    long n = 0;
    for (int y = by0; y <= by1; ++y) {
        const double dy = (double)y - cy;
        auto in = [&](int x) {
            const double dx = (double)x - cx;
            return dx * dx + dy * dy <= r * r;
        };
        // the run, if any, holds the row's point nearest cx
        const int xm = in(xf) ? xf : xf + 1;
        if (!in(xm)) continue;
        const double w = std::sqrt(std::max(0.0, r * r - dy * dy));
        int hi = std::max(xm, (int)std::floor(cx + w)), lo = std::min(xm, (int)std::ceil(cx - w));
        if (in(hi)) { while (in(hi + 1)) ++hi; } else { while (!in(hi)) --hi; }
        if (in(lo)) { while (in(lo - 1)) --lo; } else { while (!in(lo)) ++lo; }
        lo = std::max(lo, bx0);
        hi = std::min(hi, bx1);
        if (hi >= lo) n += hi - lo + 1;
    }
    return n;
}

// The disk list (cx, cy, r per disk).  Accepted disks keep a gap of 2 cells, so no cell
// belongs to two disks and every disk cell is a bulk cell of the base pattern: the solid
// count is the sum of the disks' cell counts.  A candidate is tested only against the disks
// in its own and the eight neighbouring squares of a grid whose side is at least the largest
// centre distance that can overlap (2 rmax + 2); the test itself is the plain pairwise one, so
// the accepted list, and the generator's draws, do not depend on the grid.
std::vector<double> channel_disks(int nx, int ny, uint64_t seed, float frac, float rmin, float rmax) {
    const long target = (long)std::ceil((double)frac * (double)nx * (double)ny);
    const double xlo = nx / 16 > 2 ? (double)(nx / 16) : 2.0;
    const double xhi = (double)(nx - 1) - (nx / 8 > 2 ? (double)(nx / 8) : 2.0);
    const double ylo = 2.0, yhi = (double)(ny - 3);
    const double side = std::max({2.0 * (double)rmax + 2.0, (double)nx / 128.0, (double)ny / 128.0, 1.0});
    const int gx = (int)((double)nx / side) + 1, gy = (int)((double)ny / side) + 1;
    std::vector<std::vector<int>> grid((size_t)gx * gy);
    auto square = [&](double v, int n) { return std::min(std::max((int)std::floor(v / side), 0), n - 1); };
    std::mt19937_64 g(seed);
    std::vector<double> disks;
    long solid = 0, attempts = 0;
    while (solid < target && attempts < 200000) {
        ++attempts;
        const double r = (double)rmin + ((double)rmax - (double)rmin) * unit53(g);
        const double u2 = unit53(g), u3 = unit53(g);
        if (xhi - xlo < 2.0 * r || yhi - ylo < 2.0 * r) continue;
        const double cx = xlo + r + (xhi - xlo - 2.0 * r) * u2;
        const double cy = ylo + r + (yhi - ylo - 2.0 * r) * u3;
        const int sx = square(cx, gx), sy = square(cy, gy);
        bool ok = true;
        for (int qy = std::max(sy - 1, 0); ok && qy <= std::min(sy + 1, gy - 1); ++qy)
            for (int qx = std::max(sx - 1, 0); ok && qx <= std::min(sx + 1, gx - 1); ++qx)
                for (int k : grid[(size_t)qy * gx + qx]) {
                    const double dx = cx - disks[3 * k], dy = cy - disks[3 * k + 1], md = r + disks[3 * k + 2] + 2.0;
                    if (dx * dx + dy * dy < md * md) { ok = false; break; }
                }
        if (!ok) continue;
        grid[(size_t)sy * gx + sx].push_back((int)(disks.size() / 3));
        disks.push_back(cx); disks.push_back(cy); disks.push_back(r);
        solid += disk_cell_count(nx, ny, cx, cy, r);
    }
    return disks;
}

// inlet x velocity of row y (FP64 products in source order, rounded once to FP32); the device
// builder k_build_scene evaluates the same expression
float channel_inlet_vx(int y, int ny, float u_max) {
    const double H = (double)(ny - 2);
    const double s = (double)y - 0.5;
    return (float)(4.0 * (double)u_max * s * (H - s) / (H * H));
}

int mask_phys_channel(int nx, int ny, float u_max, uint64_t seed, float frac, float rmin, float rmax,
                      std::vector<lbm_lattice_info>& out) {
    out.resize((size_t)nx * ny);
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            lbm_lattice_info r = make_info(LBM_BULK);
            if (y == 0 || y == ny - 1) r.material = LBM_BOUNDARY;
            else if (x == 0) {
                r.material = LBM_INLET;
                r.vx = channel_inlet_vx(y, ny, u_max);
            } else if (x == nx - 1) r.material = LBM_OUTLET;
            out[(size_t)y * nx + x] = r;
        }
    const std::vector<double> disks = channel_disks(nx, ny, seed, frac, rmin, rmax);
    for (size_t k = 0; k < disks.size(); k += 3)
        disk_cells(nx, ny, disks[k], disks[k + 1], disks[k + 2], [&](size_t c) { out[c].material = LBM_OBSTACLE; });
    return (int)(disks.size() / 3);
}

void build_scene_mask(const lbm_params& p, std::vector<lbm_lattice_info>& out) {
    if (p.mode == LBM_MODE_REFERENCE) {
        mask_reference(p.nx, p.ny, p.scene, p.lid_speed, p.inlet_speed, out);
        return;
    }
    switch (p.scene) {
        case LBM_SCENE_CAVITY: mask_phys_cavity(p.nx, p.ny, p.lid_speed, out); break;
        case LBM_SCENE_CHANNEL:
            mask_phys_channel(p.nx, p.ny, p.inlet_speed, p.seed, p.solid_fraction, p.disk_rmin, p.disk_rmax, out);
            break;
        case LBM_SCENE_PERIODIC: out.assign((size_t)p.nx * p.ny, make_info(LBM_BULK)); break;
        default: mask_reference(p.nx, p.ny, p.scene, p.lid_speed, p.inlet_speed, out); break;
    }
}

// Physics-mode scenes are built on the device (no upload of the info records); the host copy
// is then built from the same parameters when a host-side path first needs it.
bool device_scene(const lbm_params& p) {
    return p.mode == LBM_MODE_PHYSICS &&
           (p.scene == LBM_SCENE_CAVITY || p.scene == LBM_SCENE_CHANNEL || p.scene == LBM_SCENE_PERIODIC);
}

// d2q9_node.rs:222-241: cells of rows [y-28, y+28) within radius 28 of (x+0.5, y+0.5)
void obstacle_disc(int nx, int x, int y, lbm_lattice_info* info) {
    const int r = (int)OBSTACLE_RADIUS;
    const int min_y = y - r, max_y = min_y + 2 * r;
    const float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
    for (int yy = min_y; yy < max_y; ++yy)
        for (int xx = 0; xx < nx; ++xx)
            if (sd_sphere((float)xx + 0.5f - cx, (float)yy + 0.5f - cy, OBSTACLE_RADIUS))
                info[(size_t)yy * nx + xx] = make_info(LBM_OBSTACLE);
}

// d2q9_node.rs:269-299: the record and the cells (in stroke order) of a force stroke
lbm_lattice_info force_stroke(int nx, int ny, int pixel_size, float pos_x, float pos_y, float pre_x, float pre_y,
                              std::vector<size_t>& cells) {
    const float ddx = pos_x - pre_x, ddy = pos_y - pre_y;
    const float dis = std::sqrt(ddx * ddx + ddy * ddy);
    float force = 0.1f * (dis / 20.0f);
    if (force > 0.12f) force = 0.12f;
    const float ridian = std::atan2(pos_y - pre_y, pos_x - pre_x);
    const float vx = force * std::cos(ridian);
    const float vy = force * std::sin(ridian);
    const float c = std::ceil(dis / (float)(pixel_size - 1));
    const float step = dis / c;
    const int count = (int)c;
    const unsigned ps = (unsigned)pixel_size;
    for (int i = 0; i < count; ++i) {
        const float d = step * (float)i;
        const float p_x = std::round(pre_x + d * std::cos(ridian));
        const float p_y = std::round(pre_y + d * std::sin(ridian));
        const unsigned ux = p_x <= 0.0f ? 0u : (unsigned)p_x;  // Rust `as u32` saturates
        const unsigned uy = p_y <= 0.0f ? 0u : (unsigned)p_y;
        const unsigned x = ux / ps, y = uy / ps;
        if (x < 1 || (long)x >= (long)nx - 2 || y < 1 || (long)y >= (long)ny - 2) continue;
        cells.push_back((size_t)y * nx + x);
    }
    return make_info(LBM_EXTERNAL_FORCE, vx, vy, 90);
}

int validate_params(const lbm_params& p) {
    if (p.nx < 4 || p.ny < 4 || p.nx > 65535 || p.ny > 65535)
        return fail(LBM_ERR_ARG, "lattice %dx%d outside [4, 65535]", p.nx, p.ny);
    if ((size_t)p.nx * (size_t)p.ny > ((size_t)1 << 30))
        return fail(LBM_ERR_ARG, "lattice of %zu cells exceeds 2^30", (size_t)p.nx * p.ny);
    if (p.mode != LBM_MODE_REFERENCE && p.mode != LBM_MODE_PHYSICS) return fail(LBM_ERR_ARG, "unknown mode %d", p.mode);
    if (p.dtype < LBM_DTYPE_F32 || p.dtype > LBM_DTYPE_BF16) return fail(LBM_ERR_ARG, "unknown dtype %d", p.dtype);
    if (p.mode == LBM_MODE_REFERENCE && p.dtype != LBM_DTYPE_F32)
        return fail(LBM_ERR_ARG, "reference mode stores FP32 populations only");
    if (p.scene < 0 || p.scene > LBM_SCENE_PERIODIC) return fail(LBM_ERR_ARG, "unknown scene %d", p.scene);
    if (p.mode == LBM_MODE_REFERENCE && p.scene > LBM_SCENE_CUSTOM)
        return fail(LBM_ERR_ARG, "scene %d exists in physics mode only", p.scene);
    if (!(p.tau > 0.0f) || !std::isfinite(p.tau)) return fail(LBM_ERR_ARG, "tau must be positive and finite");
    if (p.pixel_size < 1) return fail(LBM_ERR_ARG, "pixel_size must be >= 1");
    if (p.kernel < LBM_KERNEL_AUTO || p.kernel > LBM_KERNEL_RING) return fail(LBM_ERR_ARG, "unknown kernel %d", p.kernel);
    if ((p.kernel == LBM_KERNEL_TILED || p.kernel == LBM_KERNEL_RING) && !lbm::tiled_layout_eligible(p))
        return fail(LBM_ERR_ARG, "the tiled kernels need physics mode, FP16 or BF16 storage, BGK and nx %% 64 == 0");
    if (p.collision < LBM_COLLISION_BGK || p.collision > LBM_COLLISION_KBC)
        return fail(LBM_ERR_ARG, "unknown collision %d", p.collision);
    if (p.collision != LBM_COLLISION_BGK && p.mode != LBM_MODE_PHYSICS)
        return fail(LBM_ERR_ARG, "reference mode is BGK only");
    if (p.rounding != LBM_ROUNDING_NEAREST && p.rounding != LBM_ROUNDING_STOCHASTIC)
        return fail(LBM_ERR_ARG, "unknown rounding %d", p.rounding);
    if (p.arith != LBM_ARITH_EXACT && p.arith != LBM_ARITH_FAST) return fail(LBM_ERR_ARG, "unknown arith %d", p.arith);
    if (p.rounding == LBM_ROUNDING_STOCHASTIC) {
        if (p.mode != LBM_MODE_PHYSICS || (p.dtype != LBM_DTYPE_F16 && p.dtype != LBM_DTYPE_BF16))
            return fail(LBM_ERR_ARG, "stochastic rounding applies to physics-mode FP16 / BF16 storage");
        if (p.kernel != LBM_KERNEL_AUTO && p.kernel != LBM_KERNEL_TILED && p.kernel != LBM_KERNEL_RING &&
            p.kernel != LBM_KERNEL_VEC2 && p.kernel != LBM_KERNEL_CELL)
            return fail(LBM_ERR_ARG, "stochastic rounding runs on the tiled, two-cell and one-cell kernels");
    }
    if (p.kernel == LBM_KERNEL_VEC2 && (p.mode != LBM_MODE_PHYSICS || p.nx % 2 != 0))
        return fail(LBM_ERR_ARG, "the two-cell kernel needs physics mode and nx %% 2 == 0");
    if (p.kernel == LBM_KERNEL_VEC4 && (p.mode != LBM_MODE_PHYSICS || p.nx % 4 != 0))
        return fail(LBM_ERR_ARG, "the four-cell kernel needs physics mode and nx %% 4 == 0");
    if (p.kernel == LBM_KERNEL_BULK && (p.mode != LBM_MODE_PHYSICS || p.nx % 8 != 0))
        return fail(LBM_ERR_ARG, "the bulk-copy kernel needs physics mode and nx %% 8 == 0");
    if (p.scene == LBM_SCENE_CHANNEL && !(p.disk_rmin >= 0.0f && p.disk_rmax >= p.disk_rmin && std::isfinite(p.disk_rmax) && p.solid_fraction >= 0.0f &&
                                         p.solid_fraction < 0.5f))
        return fail(LBM_ERR_ARG, "channel disk parameters out of range");
    return LBM_OK;
}

int use_device(const lbm_handle* h) {
    LBM_CK(cudaSetDevice(h->device));
    return LBM_OK;
}

// the host copy of the info records (built from the parameters on first use when the scene
// mask was built on the device; until then the device records equal the parameters' mask)
void ensure_host_info(lbm_handle* h) {
    if (!h->host_info_lazy) return;
    build_scene_mask(h->p, h->host_info);
    h->host_info_lazy = false;
}

// the physics-mode scene mask built on the device: the host samples the channel's disk list
// only (a few thousand numbers) and uploads that instead of the records
// Physics-mode scenes built on the device, with the initial state.  The base pattern (walls,
// inlet, outlet, lid) and the initialisation are launched first, so the GPU runs them while the
// host draws the channel's disk list; rasterising the disks then marks their cells solid and
// gives them the state the initialisation gives a solid cell (disk cells are bulk cells of the
// base pattern), which is the state of initialising the finished scene.  The disk list stays
// in the handle until the caller's sync: its copy to the device reads it.
int init_state(lbm_handle* h);

int scene_and_state_on_device(lbm_handle* h) {
    LBM_CK(lbm::launch_build_scene(h, h->stream));
    ++h->launches;
    LBM_TRY(init_state(h));
    h->scene_disks.clear();
    if (h->p.scene == LBM_SCENE_CHANNEL)
        h->scene_disks = channel_disks(h->nx, h->ny, h->p.seed, h->p.solid_fraction, h->p.disk_rmin, h->p.disk_rmax);
    const int nd = (int)(h->scene_disks.size() / 3);
    if (nd > 0) {
        double* d_disks = nullptr;
        LBM_CK(pool_alloc(&d_disks, h->scene_disks.size() * sizeof(double), h->stream));
        cudaError_t e = cudaMemcpyAsync(d_disks, h->scene_disks.data(), h->scene_disks.size() * sizeof(double),
                                        cudaMemcpyHostToDevice, h->stream);
        if (e == cudaSuccess) e = lbm::launch_raster_disks(h, d_disks, nd, true, h->stream);
        pool_free(d_disks, h->stream);  // ordered after the kernel that reads it
        if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "scene mask on the device: %s", cudaGetErrorString(e));
        ++h->launches;
    }
    h->host_info.clear();
    h->host_info_lazy = true;
    return LBM_OK;
}

int upload_info_rows(lbm_handle* h, int y0, int y1) {
    ensure_host_info(h);
    const size_t off = (size_t)y0 * h->nx, cnt = (size_t)(y1 - y0) * h->nx;
    LBM_CK(cudaMemcpyAsync(h->d_info + off, h->host_info.data() + off, cnt * sizeof(lbm_lattice_info),
                           cudaMemcpyHostToDevice, h->stream));
    if (h->host_mirror_valid)  // the uploaded rows are rows of the host copy
        LBM_CK(cudaMemcpyAsync(h->d_host_info + off, h->d_info + off, cnt * sizeof(lbm_lattice_info),
                               cudaMemcpyDeviceToDevice, h->stream));
    return LBM_OK;
}

int rebuild_flags(lbm_handle* h) {
    LBM_CK(lbm::launch_build_flags(h, h->stream));
    ++h->launches;
    return LBM_OK;
}

int init_state(lbm_handle* h) {
    if (h->p.mode == LBM_MODE_REFERENCE) {
        LBM_CK(lbm::launch_ref_init(h, h->stream));
    } else {
        LBM_CK(lbm::launch_phys_init(h, nullptr, nullptr, nullptr, h->stream));
    }
    ++h->launches;
    h->cur = 0;
    h->stepped_since_init = false;
    return LBM_OK;
}

int sync(lbm_handle* h) {
    LBM_CK(cudaStreamSynchronize(h->stream));
    return LBM_OK;
}

// the lattice's buffers back to the pool (ordered on the lattice's own stream: the caller has
// waited for the stream the lattice ran on)
void free_all(lbm_handle* h) {
    cudaStream_t s = h->own_stream;
    pool_free(h->buf[0], s);
    pool_free(h->buf[1], s);
    pool_free(h->d_flags, s);
    pool_free(h->d_info, s);
    pool_free(h->d_macro, s);
    pool_free(h->d_part, s);
    pool_free(h->d_count, s);
    pool_free(h->d_status, s);
    pool_free(h->d_host_info, s);
    pool_free(h->d_edits, s);
    if (s) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
}

int check_handle(const lbm_handle* h) {
    if (!h) return fail(LBM_ERR_ARG, "null handle");
    return LBM_OK;
}

}  // namespace

namespace lbm {
int set_error(int code, const char* msg) {
    g_err = msg;
    return code;
}
}  // namespace lbm

extern "C" {

int lbm_abi_version(void) { return LBM_ABI_VERSION; }

int lbm_memory_set_retain(uint64_t bytes) {
    {
        std::lock_guard<std::mutex> lock(g_pool_mu);
        g_retain = bytes;
        g_retain_set = true;
    }
    int n = 0;
    LBM_CK(cudaGetDeviceCount(&n));
    for (int d = 0; d < n && d < lbm::MAX_DEVICES; ++d) {
        cudaMemPool_t pool = nullptr;
        if (!g_pools.peek(d, &pool)) continue;  // created later with the new value
        LBM_CK(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &bytes));
    }
    return LBM_OK;
}

int lbm_memory_trim(void) {
    int dev = 0;
    LBM_CK(cudaGetDevice(&dev));
    cudaMemPool_t pool = nullptr;
    if (!g_pools.peek(dev, &pool)) return LBM_OK;
    LBM_CK(cudaDeviceSynchronize());  // frees still in flight return their memory first
    LBM_CK(cudaMemPoolTrimTo(pool, 0));
    return LBM_OK;
}

int lbm_memory_stats(uint64_t* reserved, uint64_t* used) {
    if (!reserved || !used) return fail(LBM_ERR_ARG, "null argument");
    *reserved = 0;
    *used = 0;
    int dev = 0;
    LBM_CK(cudaGetDevice(&dev));
    cudaMemPool_t pool = nullptr;
    if (!g_pools.peek(dev, &pool)) return LBM_OK;
    LBM_CK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, reserved));
    LBM_CK(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, used));
    return LBM_OK;
}

const char* lbm_last_error(void) { return g_err.c_str(); }

void lbm_params_default(lbm_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->nx = 600;  // 1200x750 canvas at lattice_pixel_size 2 (app_handler.rs:57-58, d2q9_node.rs:38-43)
    p->ny = 375;
    p->mode = LBM_MODE_REFERENCE;
    p->dtype = LBM_DTYPE_F32;
    p->scene = LBM_SCENE_POISEUILLE;
    p->tau = 3.0f * 0.02f + 0.5f;  // setting_obj.rs:32 viscosity 0.02
    p->lid_speed = 0.13f;
    p->inlet_speed = 0.12f;
    p->solid_fraction = 0.05f;
    p->disk_rmin = 8.0f;
    p->disk_rmax = 32.0f;
    p->seed = 0;
    p->pixel_size = 2;
    p->macro_every_step = 0;
}

int lbm_create(const lbm_params* pin, lbm_handle** out) {
    LbmRange range_("lbm_create");
    if (!pin || !out) return fail(LBM_ERR_ARG, "null argument");
    *out = nullptr;
    const lbm_params& p = *pin;
    LBM_TRY(validate_params(p));

    lbm_handle* h = new (std::nothrow) lbm_handle();
    if (!h) return fail(LBM_ERR_NOMEM, "out of host memory");
    h->p = p;
    h->nx = p.nx;
    h->ny = p.ny;
    h->N = (size_t)p.nx * p.ny;
    h->fluid_ty = (p.scene == LBM_SCENE_CAVITY) ? 1 : 0;
    h->tiled = (p.kernel == LBM_KERNEL_TILED || p.kernel == LBM_KERNEL_RING || p.kernel == LBM_KERNEL_AUTO) &&
               lbm::tiled_layout_eligible(p);
    h->tau = p.tau;
    h->omega = 1.0f / p.tau;
    h->omega_d = 1.0 / (double)p.tau;
    cudaError_t e = cudaGetDevice(&h->device);
    const size_t pop_bytes = 9 * h->N * lbm::dtype_size(p.dtype);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&h->own_stream, cudaStreamNonBlocking);
    h->stream = h->own_stream;
    const cudaStream_t s = h->own_stream;
    if (e == cudaSuccess) e = pool_alloc(&h->buf[0], pop_bytes, s);
    if (e == cudaSuccess) e = pool_alloc(&h->buf[1], pop_bytes, s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_flags, h->N * sizeof(uint16_t), s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_info, h->N * sizeof(lbm_lattice_info), s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_macro, 3 * h->N * sizeof(float), s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_part, (size_t)lbm::RED_BLOCKS * 6 * sizeof(double) + 64 * sizeof(double), s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_count, sizeof(unsigned long long), s);
    if (e == cudaSuccess) e = pool_alloc(&h->d_status, sizeof(int), s);
    if (e == cudaSuccess) e = cudaMemsetAsync(h->d_status, 0, sizeof(int), s);
    if (e != cudaSuccess) {
        free_all(h);
        delete h;
        return fail(LBM_ERR_CUDA, "allocation for a %dx%d lattice failed: %s", p.nx, p.ny, cudaGetErrorString(e));
    }
    int r = LBM_OK;
    if (device_scene(p)) {
        r = scene_and_state_on_device(h);  // also initialises the state
    } else {
        build_scene_mask(p, h->host_info);
        r = upload_info_rows(h, 0, h->ny);
        if (r == LBM_OK) r = init_state(h);
    }
    if (r == LBM_OK) r = rebuild_flags(h);
    const int rs = sync(h);                  // also after a failed launch: the copy reads the list
    h->scene_disks = std::vector<double>();
    if (r == LBM_OK) r = rs;
    if (r != LBM_OK) {
        free_all(h);
        delete h;
        return r;
    }
    *out = h;
    return LBM_OK;
}

int lbm_destroy(lbm_handle* h) {
    if (!h) return LBM_OK;
    cudaSetDevice(h->device);
    if (h->stream) cudaStreamSynchronize(h->stream);
    free_all(h);
    delete h;
    return LBM_OK;
}

int lbm_set_stream(lbm_handle* h, void* s) {
    LBM_TRY(check_handle(h));
    LBM_TRY(use_device(h));
    LBM_CK(cudaStreamSynchronize(h->stream));
    h->stream = s ? (cudaStream_t)s : h->own_stream;
    return LBM_OK;
}

int lbm_get_size(const lbm_handle* h, int32_t* nx, int32_t* ny) {
    LBM_TRY(check_handle(h));
    if (nx) *nx = h->nx;
    if (ny) *ny = h->ny;
    return LBM_OK;
}

int lbm_get_params(const lbm_handle* h, lbm_params* out) {
    LBM_TRY(check_handle(h));
    if (!out) return fail(LBM_ERR_ARG, "null output");
    *out = h->p;
    out->tau = h->tau;
    return LBM_OK;
}

int lbm_step(lbm_handle* h, int32_t nsteps) {
    LbmRange range_("lbm_step");
    LBM_TRY(check_handle(h));
    if (nsteps < 0) return fail(LBM_ERR_ARG, "negative step count");
    LBM_TRY(use_device(h));
    for (int32_t s = 0; s < nsteps; ++s) {
        const bool macro = h->p.macro_every_step || s == nsteps - 1;
        LBM_CK(lbm::launch_step(h, macro, h->stream));
        h->cur ^= 1;
        ++h->steps;
        ++h->launches;
    }
    if (nsteps > 0) h->stepped_since_init = true;
    return LBM_OK;
}

int lbm_compute(lbm_handle* h) { return lbm_step(h, 2); }

int lbm_reset(lbm_handle* h) {
    LbmRange range_("lbm_reset");
    LBM_TRY(check_handle(h));
    LBM_TRY(use_device(h));
    // reference: only the Poiseuille scene rebuilds its mask (d2q9_node.rs:248-255)
    int r = LBM_OK;
    if (device_scene(h->p)) {
        r = scene_and_state_on_device(h);  // the host copy follows lazily, as after create
        h->host_mirror_valid = false;      // the device copy of the host copy is stale
    } else {
        if (h->p.mode == LBM_MODE_PHYSICS || h->p.scene == LBM_SCENE_POISEUILLE) {
            build_scene_mask(h->p, h->host_info);
            h->host_info_lazy = false;
            r = upload_info_rows(h, 0, h->ny);
        }
        if (r == LBM_OK) r = init_state(h);
    }
    if (r == LBM_OK) r = rebuild_flags(h);
    h->pre_x = h->pre_y = 0.0f;  // fluid_simulator.rs:214
    const int rs = sync(h);      // also before the disk list is released on a failed launch
    h->scene_disks = std::vector<double>();
    return r != LBM_OK ? r : rs;
}

int lbm_set_tau(lbm_handle* h, float tau) {
    LBM_TRY(check_handle(h));
    if (!(tau > 0.0f) || !std::isfinite(tau)) return fail(LBM_ERR_ARG, "tau must be positive and finite");
    h->tau = tau;
    h->omega = 1.0f / tau;  // mod.rs:35
    h->omega_d = 1.0 / (double)tau;
    return LBM_OK;
}

int lbm_update_viscosity(lbm_handle* h, float viscosity) {
    const float tau = 3.0f * viscosity + 0.5f;  // fluid_simulator.rs:177
    return lbm_set_tau(h, tau);
}

int lbm_add_obstacle(lbm_handle* h, int32_t x, int32_t y) {
    LBM_TRY(check_handle(h));
    const int r = (int)OBSTACLE_RADIUS;
    const int min_y = y - r, max_y = min_y + 2 * r;
    if (x < 0 || x >= h->nx || min_y < 0 || max_y > h->ny)
        return fail(LBM_ERR_ARG, "obstacle rows [%d, %d) or column %d outside the lattice", min_y, max_y, x);
    LBM_TRY(use_device(h));
    ensure_host_info(h);
    obstacle_disc(h->nx, x, y, h->host_info.data());
    // the reference uploads whole rows from its host copy (d2q9_node.rs:243-244)
    LBM_TRY(upload_info_rows(h, min_y, max_y));
    LBM_TRY(rebuild_flags(h));
    return sync(h);
}

int lbm_on_click(lbm_handle* h, float px, float py) {
    LBM_TRY(check_handle(h));
    if (px <= 0.0f || py <= 0.0f) return LBM_IGNORED;
    const unsigned ps = (unsigned)h->p.pixel_size;
    const unsigned x = (unsigned)px / ps, y = (unsigned)py / ps;
    const unsigned half = (unsigned)OBSTACLE_RADIUS;
    if (x < half || (long)x >= (long)h->nx - (long)(half + 2) || y < half || (long)y >= (long)h->ny - (long)(half + 2))
        return LBM_IGNORED;
    return lbm_add_obstacle(h, (int32_t)x, (int32_t)y);
}

int lbm_touch_begin(lbm_handle* h) {
    LBM_TRY(check_handle(h));
    h->pre_x = h->pre_y = 0.0f;
    return LBM_OK;
}

int lbm_touch_move(lbm_handle* h, float px, float py) {
    LBM_TRY(check_handle(h));
    if (px <= 0.0f || py <= 0.0f) {
        h->pre_x = h->pre_y = 0.0f;
        return LBM_IGNORED;
    }
    const float dx = px - h->pre_x, dy = py - h->pre_y;
    const float dis = std::sqrt(dx * dx + dy * dy);
    if ((h->pre_x == 0.0f && h->pre_y == 0.0f) || dis > 300.0f) {
        h->pre_x = px;
        h->pre_y = py;
        return LBM_IGNORED;
    }
    const int r = lbm_add_external_force(h, px, py, h->pre_x, h->pre_y);
    h->pre_x = px;
    h->pre_y = py;
    return r;
}

int lbm_add_external_force(lbm_handle* h, float pos_x, float pos_y, float pre_x, float pre_y) {
    LBM_TRY(check_handle(h));
    if (h->p.pixel_size < 2)
        return fail(LBM_ERR_ARG, "force strokes need pixel_size >= 2 (the reference divides by pixel_size - 1)");
    LBM_TRY(use_device(h));
    std::vector<size_t> cells;
    const lbm_lattice_info rec = force_stroke(h->nx, h->ny, h->p.pixel_size, pos_x, pos_y, pre_x, pre_y, cells);
    // queue.write_buffer of one record per cell; the host copy is not updated, as in the reference
    for (size_t k = 0; k < cells.size(); ++k) {
        if (k > 0 && cells[k] == cells[k - 1]) continue;
        LBM_CK(cudaMemcpyAsync(h->d_info + cells[k], &rec, sizeof(rec), cudaMemcpyHostToDevice, h->stream));
    }
    LBM_TRY(rebuild_flags(h));
    return sync(h);
}

int lbm_apply_edits(lbm_handle* h, const lbm_edit* edits, int32_t n, int32_t* applied) {
    LbmRange range_("lbm_apply_edits");
    LBM_TRY(check_handle(h));
    if (n < 0 || (n > 0 && !edits)) return fail(LBM_ERR_ARG, "bad edit list");
    ensure_host_info(h);
    // resolve the list on the host exactly as the single calls would (guards, touch state,
    // stroke geometry), then let two kernels write the device mask
    float pre_x = h->pre_x, pre_y = h->pre_y;
    std::vector<lbm::EditObstacle> obs;
    std::vector<lbm::EditForce> forces;
    int32_t count = 0;
    const int r = (int)OBSTACLE_RADIUS;
    auto stroke = [&](float px, float py, float qx, float qy, int seq) {
        std::vector<size_t> cells;
        const lbm_lattice_info rec = force_stroke(h->nx, h->ny, h->p.pixel_size, px, py, qx, qy, cells);
        for (size_t c : cells) forces.push_back({(uint32_t)c, seq, rec.vx, rec.vy});
        ++count;
    };
    for (int32_t i = 0; i < n; ++i) {
        const lbm_edit& e = edits[i];
        switch (e.kind) {
            case LBM_EDIT_OBSTACLE: {
                const int x = (int)e.a, y = (int)e.b;
                if ((float)x != e.a || (float)y != e.b || x < 0 || x >= h->nx || y - r < 0 || y + r > h->ny)
                    return fail(LBM_ERR_ARG, "edit %d: obstacle at (%g, %g) outside the lattice", i, e.a, e.b);
                obs.push_back({x, y, i, 0});
                ++count;
                break;
            }
            case LBM_EDIT_CLICK: {  // lbm_on_click
                if (e.a <= 0.0f || e.b <= 0.0f) break;
                const unsigned ps = (unsigned)h->p.pixel_size;
                const unsigned x = (unsigned)e.a / ps, y = (unsigned)e.b / ps;
                const unsigned half = (unsigned)OBSTACLE_RADIUS;
                if (x < half || (long)x >= (long)h->nx - (long)(half + 2) || y < half ||
                    (long)y >= (long)h->ny - (long)(half + 2))
                    break;
                obs.push_back({(int)x, (int)y, i, 0});
                ++count;
                break;
            }
            case LBM_EDIT_FORCE:
                if (h->p.pixel_size < 2) return fail(LBM_ERR_ARG, "edit %d: force strokes need pixel_size >= 2", i);
                stroke(e.a, e.b, e.c, e.d, i);
                break;
            case LBM_EDIT_TOUCH_BEGIN: pre_x = pre_y = 0.0f; break;
            case LBM_EDIT_TOUCH_MOVE: {  // lbm_touch_move
                if (e.a <= 0.0f || e.b <= 0.0f) {
                    pre_x = pre_y = 0.0f;
                    break;
                }
                const float dx = e.a - pre_x, dy = e.b - pre_y;
                const float dis = std::sqrt(dx * dx + dy * dy);
                if (!((pre_x == 0.0f && pre_y == 0.0f) || dis > 300.0f)) {
                    if (h->p.pixel_size < 2)
                        return fail(LBM_ERR_ARG, "edit %d: force strokes need pixel_size >= 2", i);
                    stroke(e.a, e.b, pre_x, pre_y, i);
                }
                pre_x = e.a;
                pre_y = e.b;
                break;
            }
            default: return fail(LBM_ERR_ARG, "edit %d: unknown kind %d", i, e.kind);
        }
    }
    LBM_TRY(use_device(h));
    // a cell written by several strokes keeps the last one
    if (forces.size() > 1) {
        std::vector<size_t> order(forces.size());
        for (size_t k = 0; k < order.size(); ++k) order[k] = k;
        std::stable_sort(order.begin(), order.end(),
                         [&](size_t a, size_t b) { return forces[a].cell < forces[b].cell; });
        std::vector<lbm::EditForce> last;
        for (size_t k = 0; k < order.size(); ++k)
            if (k + 1 == order.size() || forces[order[k + 1]].cell != forces[order[k]].cell)
                last.push_back(forces[order[k]]);
        forces.swap(last);
    }
    if (!h->host_mirror_valid && !obs.empty()) {
        if (!h->d_host_info) LBM_CK(pool_alloc(&h->d_host_info, h->N * sizeof(lbm_lattice_info), h->stream));
        LBM_CK(cudaMemcpyAsync(h->d_host_info, h->host_info.data(), h->N * sizeof(lbm_lattice_info),
                               cudaMemcpyHostToDevice, h->stream));
        h->host_mirror_valid = true;
    }
    const size_t bytes = obs.size() * sizeof(lbm::EditObstacle) + forces.size() * sizeof(lbm::EditForce);
    if (bytes > 0) {
        if (bytes > h->edits_cap) {
            pool_free(h->d_edits, h->stream);  // after the kernels that read the old list
            h->d_edits = nullptr;
            h->edits_cap = 0;
            const size_t cap = std::max(bytes, (size_t)4096);
            LBM_CK(pool_alloc(&h->d_edits, cap, h->stream));
            h->edits_cap = cap;
        }
        std::vector<unsigned char> stage(bytes);
        std::memcpy(stage.data(), obs.data(), obs.size() * sizeof(lbm::EditObstacle));
        std::memcpy(stage.data() + obs.size() * sizeof(lbm::EditObstacle), forces.data(),
                    forces.size() * sizeof(lbm::EditForce));
        LBM_CK(cudaMemcpyAsync(h->d_edits, stage.data(), bytes, cudaMemcpyHostToDevice, h->stream));
        int row0 = h->ny, row1 = 0;
        for (const auto& o : obs) {
            row0 = std::min(row0, o.y - r);
            row1 = std::max(row1, o.y + r);
            obstacle_disc(h->nx, o.x, o.y, h->host_info.data());  // D2Q9Node::lattice_info_data
        }
        const auto* d_obs = (const lbm::EditObstacle*)h->d_edits;
        const auto* d_forces = (const lbm::EditForce*)((const unsigned char*)h->d_edits +
                                                        obs.size() * sizeof(lbm::EditObstacle));
        LBM_CK(lbm::launch_edits(h, d_obs, (int)obs.size(), d_forces, (int)forces.size(), row0, row1, h->stream));
        h->launches += (obs.empty() ? 0 : 1) + (forces.empty() ? 0 : 1);
        LBM_TRY(rebuild_flags(h));
    }
    h->pre_x = pre_x;
    h->pre_y = pre_y;
    if (applied) *applied = count;
    return LBM_OK;
}

int lbm_build_mask(const lbm_params* p, lbm_lattice_info* out) {
    if (!p || !out) return fail(LBM_ERR_ARG, "null argument");
    LBM_TRY(validate_params(*p));
    std::vector<lbm_lattice_info> m;
    build_scene_mask(*p, m);
    std::memcpy(out, m.data(), m.size() * sizeof(lbm_lattice_info));
    return LBM_OK;
}

int lbm_scene_disks(const lbm_params* p, double* out, int32_t cap, int32_t* n) {
    if (!p || !n || cap < 0 || (cap > 0 && !out)) return fail(LBM_ERR_ARG, "bad argument");
    LBM_TRY(validate_params(*p));
    *n = 0;
    if (p->mode != LBM_MODE_PHYSICS || p->scene != LBM_SCENE_CHANNEL) return LBM_OK;
    const std::vector<double> d = channel_disks(p->nx, p->ny, p->seed, p->solid_fraction, p->disk_rmin, p->disk_rmax);
    const int32_t nd = (int32_t)(d.size() / 3);
    if (cap > 0 && nd > 0) std::memcpy(out, d.data(), (size_t)std::min(nd, cap) * 3 * sizeof(double));
    *n = nd;
    return LBM_OK;
}

int lbm_mask_add_obstacle(int32_t nx, int32_t ny, lbm_lattice_info* info, int32_t x, int32_t y) {
    if (!info) return fail(LBM_ERR_ARG, "null info");
    const int r = (int)OBSTACLE_RADIUS;
    if (nx < 1 || x < 0 || x >= nx || y - r < 0 || y + r > ny)
        return fail(LBM_ERR_ARG, "obstacle rows [%d, %d) or column %d outside the lattice", y - r, y + r, x);
    obstacle_disc(nx, x, y, info);
    return LBM_OK;
}

int lbm_mask_force_stroke(int32_t nx, int32_t ny, int32_t pixel_size, lbm_lattice_info* info, float pos_x, float pos_y,
                          float pre_x, float pre_y) {
    if (!info) return fail(LBM_ERR_ARG, "null info");
    if (pixel_size < 2) return fail(LBM_ERR_ARG, "force strokes need pixel_size >= 2");
    std::vector<size_t> cells;
    const lbm_lattice_info rec = force_stroke(nx, ny, pixel_size, pos_x, pos_y, pre_x, pre_y, cells);
    for (size_t c : cells) info[c] = rec;
    return (int)cells.size();
}

int lbm_set_info(lbm_handle* h, const lbm_lattice_info* info) {
    LBM_TRY(check_handle(h));
    if (!info) return fail(LBM_ERR_ARG, "null info");
    LBM_TRY(use_device(h));
    h->host_info.assign(info, info + h->N);
    h->host_info_lazy = false;
    LBM_TRY(upload_info_rows(h, 0, h->ny));
    LBM_TRY(rebuild_flags(h));
    return sync(h);
}

int lbm_get_info(lbm_handle* h, lbm_lattice_info* out) {
    LBM_TRY(check_handle(h));
    if (!out) return fail(LBM_ERR_ARG, "null output");
    LBM_TRY(use_device(h));
    LBM_CK(cudaMemcpyAsync(out, h->d_info, h->N * sizeof(lbm_lattice_info), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int lbm_read_macro(lbm_handle* h, float* rho, float* ux, float* uy) {
    LbmRange range_("lbm_read_macro");
    LBM_TRY(check_handle(h));
    LBM_TRY(use_device(h));
    float* dst[3] = {rho, ux, uy};
    for (int k = 0; k < 3; ++k)
        if (dst[k])
            LBM_CK(cudaMemcpyAsync(dst[k], h->d_macro + k * h->N, h->N * sizeof(float), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int lbm_read_macro_rgba16f(lbm_handle* h, uint16_t* rgba) {
    LBM_TRY(check_handle(h));
    if (!rgba) return fail(LBM_ERR_ARG, "null output");
    LBM_TRY(use_device(h));
    uint16_t* d = nullptr;
    LBM_CK(pool_alloc(&d, 4 * h->N * sizeof(uint16_t), h->stream));
    cudaError_t e = lbm::launch_macro_rgba16f(h, d, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(rgba, d, 4 * h->N * sizeof(uint16_t), cudaMemcpyDeviceToHost, h->stream);
    pool_free(d, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "rgba16f read-back: %s", cudaGetErrorString(e));
    ++h->launches;
    return LBM_OK;
}

int lbm_read_populations(lbm_handle* h, void* dst, int32_t dd) {
    LBM_TRY(check_handle(h));
    if (!dst) return fail(LBM_ERR_ARG, "null output");
    if (dd != LBM_DTYPE_F32 && dd != LBM_DTYPE_F64) return fail(LBM_ERR_ARG, "read dtype must be F32 or F64");
    LBM_TRY(use_device(h));
    const size_t bytes = 9 * h->N * lbm::dtype_size(dd);
    if (h->p.mode == LBM_MODE_REFERENCE && dd == LBM_DTYPE_F32) {
        LBM_CK(cudaMemcpyAsync(dst, h->buf[h->cur], bytes, cudaMemcpyDeviceToHost, h->stream));
        return sync(h);
    }
    void* tmp = nullptr;
    LBM_CK(pool_alloc(&tmp, bytes, h->stream));
    cudaError_t e = lbm::launch_to_absolute(h, h->buf[h->cur], tmp, dd, h->stream);
    if (e == cudaSuccess) e = cudaMemcpyAsync(dst, tmp, bytes, cudaMemcpyDeviceToHost, h->stream);
    pool_free(tmp, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "population read-back: %s", cudaGetErrorString(e));
    ++h->launches;
    return LBM_OK;
}

int lbm_write_populations(lbm_handle* h, const void* src, int32_t sd) {
    LBM_TRY(check_handle(h));
    if (!src) return fail(LBM_ERR_ARG, "null input");
    if (sd != LBM_DTYPE_F32 && sd != LBM_DTYPE_F64) return fail(LBM_ERR_ARG, "write dtype must be F32 or F64");
    LBM_TRY(use_device(h));
    const size_t bytes = 9 * h->N * lbm::dtype_size(sd);
    void* tmp = nullptr;
    LBM_CK(pool_alloc(&tmp, bytes, h->stream));
    cudaError_t e = cudaMemcpyAsync(tmp, src, bytes, cudaMemcpyHostToDevice, h->stream);
    if (e == cudaSuccess) e = lbm::launch_from_absolute(h, tmp, sd, h->buf[h->cur], h->stream);
    pool_free(tmp, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "population upload: %s", cudaGetErrorString(e));
    ++h->launches;
    return LBM_OK;
}

int lbm_init_equilibrium(lbm_handle* h, const float* rho, const float* ux, const float* uy) {
    LBM_TRY(check_handle(h));
    if (h->p.mode != LBM_MODE_PHYSICS) return fail(LBM_ERR_STATE, "equilibrium initialisation is a physics-mode call");
    LBM_TRY(use_device(h));
    float* d = nullptr;
    const size_t plane = h->N * sizeof(float);
    LBM_CK(pool_alloc(&d, 3 * plane, h->stream));
    const float* src[3] = {rho, ux, uy};
    const float* dp[3] = {nullptr, nullptr, nullptr};
    cudaError_t e = cudaSuccess;
    for (int k = 0; k < 3 && e == cudaSuccess; ++k)
        if (src[k]) {
            e = cudaMemcpyAsync(d + k * h->N, src[k], plane, cudaMemcpyHostToDevice, h->stream);
            dp[k] = d + k * h->N;
        }
    if (e == cudaSuccess) e = lbm::launch_phys_init(h, dp[0], dp[1], dp[2], h->stream);
    pool_free(d, h->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
    if (e != cudaSuccess) return fail(LBM_ERR_CUDA, "equilibrium initialisation: %s", cudaGetErrorString(e));
    ++h->launches;
    h->cur = 0;
    h->stepped_since_init = false;
    return LBM_OK;
}

int lbm_conservation(lbm_handle* h, double out[3]) {
    LbmRange range_("lbm_conservation");
    LBM_TRY(check_handle(h));
    if (!out) return fail(LBM_ERR_ARG, "null output");
    LBM_TRY(use_device(h));
    double* d_out = h->d_part + (size_t)lbm::RED_BLOCKS * 6;
    LBM_CK(lbm::launch_conservation(h, d_out, h->stream));
    h->launches += 2;
    LBM_CK(cudaMemcpyAsync(out, d_out, 3 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

int lbm_check_finite(lbm_handle* h, uint64_t* count) {
    LBM_TRY(check_handle(h));
    LBM_TRY(use_device(h));
    LBM_CK(lbm::launch_count_nonfinite(h, h->stream));
    ++h->launches;
    unsigned long long n = 0;
    LBM_CK(cudaMemcpyAsync(&n, h->d_count, sizeof(n), cudaMemcpyDeviceToHost, h->stream));
    LBM_TRY(sync(h));
    if (count) *count = n;
    if (n) return fail(LBM_ERR_NAN, "%llu non-finite populations", n);
    return LBM_OK;
}

int lbm_macro_error(lbm_handle* h, lbm_handle* ref, double out[4]) {
    LBM_TRY(check_handle(h));
    LBM_TRY(check_handle(ref));
    if (!out) return fail(LBM_ERR_ARG, "null output");
    if (h->nx != ref->nx || h->ny != ref->ny) return fail(LBM_ERR_ARG, "lattice sizes differ");
    if (h->device != ref->device) return fail(LBM_ERR_ARG, "handles live on different devices");
    LBM_TRY(use_device(h));
    LBM_CK(cudaStreamSynchronize(ref->stream));
    double* d_out = h->d_part + (size_t)lbm::RED_BLOCKS * 6 + 8;
    LBM_CK(lbm::launch_macro_error(h, ref, d_out, h->stream));
    h->launches += 2;
    LBM_CK(cudaMemcpyAsync(out, d_out, 4 * sizeof(double), cudaMemcpyDeviceToHost, h->stream));
    return sync(h);
}

// ---------------------------------------------------------------------------------
// checkpoints
// ---------------------------------------------------------------------------------
struct ckpt_header {
    char magic[8];
    uint32_t version;
    int32_t nx, ny, mode, dtype, scene, fluid_ty, cur;
    float tau, pre_x, pre_y;
    int32_t stepped;
    int32_t layout;  // 1: tiled 16-bit populations (zero in checkpoints written before it existed)
    uint64_t steps;
};

int lbm_save(lbm_handle* h, const char* path) {
    LBM_TRY(check_handle(h));
    if (!path) return fail(LBM_ERR_ARG, "null path");
    LBM_TRY(use_device(h));
    LBM_TRY(sync(h));
    const size_t pop_bytes = 9 * h->N * lbm::dtype_size(h->p.dtype);
    std::vector<char> state(2 * pop_bytes);
    std::vector<lbm_lattice_info> info(h->N);
    std::vector<float> macro(3 * h->N);
    LBM_CK(cudaMemcpy(state.data(), h->buf[0], pop_bytes, cudaMemcpyDeviceToHost));
    LBM_CK(cudaMemcpy(state.data() + pop_bytes, h->buf[1], pop_bytes, cudaMemcpyDeviceToHost));
    LBM_CK(cudaMemcpy(info.data(), h->d_info, h->N * sizeof(lbm_lattice_info), cudaMemcpyDeviceToHost));
    LBM_CK(cudaMemcpy(macro.data(), h->d_macro, 3 * h->N * sizeof(float), cudaMemcpyDeviceToHost));
    ckpt_header hd;
    std::memset(&hd, 0, sizeof(hd));
    std::memcpy(hd.magic, "LBMCKPT1", 8);
    hd.version = 1;
    hd.nx = h->nx; hd.ny = h->ny; hd.mode = h->p.mode; hd.dtype = h->p.dtype; hd.scene = h->p.scene;
    hd.fluid_ty = h->fluid_ty; hd.cur = h->cur; hd.tau = h->tau; hd.pre_x = h->pre_x; hd.pre_y = h->pre_y;
    hd.stepped = h->stepped_since_init ? 1 : 0;
    hd.layout = h->tiled ? 1 : 0;
    hd.steps = h->steps;
    FILE* f = std::fopen(path, "wb");
    if (!f) return fail(LBM_ERR_IO, "cannot open %s for writing", path);
    bool ok = std::fwrite(&hd, sizeof(hd), 1, f) == 1;
    ok = ok && std::fwrite(state.data(), 1, state.size(), f) == state.size();
    ok = ok && std::fwrite(info.data(), sizeof(lbm_lattice_info), h->N, f) == h->N;
    ensure_host_info(h);
    ok = ok && std::fwrite(h->host_info.data(), sizeof(lbm_lattice_info), h->N, f) == h->N;
    ok = ok && std::fwrite(macro.data(), sizeof(float), 3 * h->N, f) == 3 * h->N;
    ok = (std::fclose(f) == 0) && ok;
    if (!ok) return fail(LBM_ERR_IO, "short write to %s", path);
    return LBM_OK;
}

int lbm_load(lbm_handle* h, const char* path) {
    LBM_TRY(check_handle(h));
    if (!path) return fail(LBM_ERR_ARG, "null path");
    LBM_TRY(use_device(h));
    FILE* f = std::fopen(path, "rb");
    if (!f) return fail(LBM_ERR_IO, "cannot open %s", path);
    ckpt_header hd;
    if (std::fread(&hd, sizeof(hd), 1, f) != 1 || std::memcmp(hd.magic, "LBMCKPT1", 8) != 0 || hd.version != 1) {
        std::fclose(f);
        return fail(LBM_ERR_IO, "%s is not a checkpoint of this library", path);
    }
    if (hd.nx != h->nx || hd.ny != h->ny || hd.mode != h->p.mode || hd.dtype != h->p.dtype) {
        std::fclose(f);
        return fail(LBM_ERR_ARG, "checkpoint %dx%d mode %d dtype %d does not match the handle", hd.nx, hd.ny, hd.mode, hd.dtype);
    }
    if ((hd.layout != 0) != h->tiled) {
        std::fclose(f);
        return fail(LBM_ERR_ARG, "checkpoint population layout (%s) does not match the handle's", hd.layout ? "tiled" : "SoA");
    }
    const size_t pop_bytes = 9 * h->N * lbm::dtype_size(h->p.dtype);
    std::vector<char> state(2 * pop_bytes);
    std::vector<lbm_lattice_info> info(h->N), hinfo(h->N);
    std::vector<float> macro(3 * h->N);
    bool ok = std::fread(state.data(), 1, state.size(), f) == state.size();
    ok = ok && std::fread(info.data(), sizeof(lbm_lattice_info), h->N, f) == h->N;
    ok = ok && std::fread(hinfo.data(), sizeof(lbm_lattice_info), h->N, f) == h->N;
    ok = ok && std::fread(macro.data(), sizeof(float), 3 * h->N, f) == 3 * h->N;
    std::fclose(f);
    if (!ok) return fail(LBM_ERR_IO, "truncated checkpoint %s", path);
    LBM_TRY(sync(h));
    LBM_CK(cudaMemcpy(h->buf[0], state.data(), pop_bytes, cudaMemcpyHostToDevice));
    LBM_CK(cudaMemcpy(h->buf[1], state.data() + pop_bytes, pop_bytes, cudaMemcpyHostToDevice));
    LBM_CK(cudaMemcpy(h->d_info, info.data(), h->N * sizeof(lbm_lattice_info), cudaMemcpyHostToDevice));
    LBM_CK(cudaMemcpy(h->d_macro, macro.data(), 3 * h->N * sizeof(float), cudaMemcpyHostToDevice));
    h->host_info = hinfo;
    h->host_info_lazy = false;
    h->host_mirror_valid = false;
    h->cur = hd.cur & 1;
    h->tau = hd.tau;
    h->omega = 1.0f / hd.tau;
    h->omega_d = 1.0 / (double)hd.tau;
    h->pre_x = hd.pre_x;
    h->pre_y = hd.pre_y;
    h->stepped_since_init = hd.stepped != 0;
    h->steps = hd.steps;
    h->p.scene = hd.scene;
    h->fluid_ty = hd.fluid_ty;
    LBM_TRY(rebuild_flags(h));
    return sync(h);
}

int lbm_status(lbm_handle* h) {
    LBM_TRY(check_handle(h));
    LBM_TRY(use_device(h));
    int st = 0;
    LBM_CK(cudaMemcpyAsync(&st, h->d_status, sizeof(int), cudaMemcpyDeviceToHost, h->stream));
    LBM_TRY(sync(h));
    if (st != 0) return fail(st, "a step kernel gave up on a bounded wait (status %d)", st);
    return LBM_OK;
}

int lbm_steps_done(const lbm_handle* h, uint64_t* steps) {
    LBM_TRY(check_handle(h));
    if (steps) *steps = h->steps;
    return LBM_OK;
}

int lbm_kernel_launches(const lbm_handle* h, uint64_t* launches) {
    LBM_TRY(check_handle(h));
    if (launches) *launches = h->launches;
    return LBM_OK;
}

int lbm_device_macro(lbm_handle* h, float** rho, float** ux, float** uy) {
    LBM_TRY(check_handle(h));
    if (rho) *rho = h->d_macro;
    if (ux) *ux = h->d_macro + h->N;
    if (uy) *uy = h->d_macro + 2 * h->N;
    return LBM_OK;
}

int lbm_bounds_report(uint64_t* count, uint64_t* first_index, uint64_t* first_limit, int32_t* first_site) {
#ifdef LBM_BOUNDS_CHECK
    lbm::BoundsRecord total{};
    cudaError_t (*takes[])(lbm::BoundsRecord*) = {lbm::bounds_take_kernels, lbm::bounds_take_vec,
                                                 lbm::bounds_take_bulk, lbm::bounds_take_batch};
    for (auto take : takes) {
        lbm::BoundsRecord r{};
        LBM_CK(take(&r));
        if (r.count && !total.count) {
            total.index = r.index;
            total.limit = r.limit;
            total.site = r.site;
        }
        total.count += r.count;
    }
    if (count) *count = total.count;
    if (first_index) *first_index = total.index;
    if (first_limit) *first_limit = total.limit;
    if (first_site) *first_site = total.site;
    return LBM_OK;
#else
    (void)count;
    (void)first_index;
    (void)first_limit;
    (void)first_site;
    return fail(LBM_ERR_STATE, "not a bounds-checked build: load liblbm_bounds.so");
#endif
}

int lbm_bounds_selftest(void) {
#ifdef LBM_BOUNDS_CHECK
    LBM_CK(lbm::bounds_selftest(nullptr));
    LBM_CK(cudaDeviceSynchronize());
    return LBM_OK;
#else
    return fail(LBM_ERR_STATE, "not a bounds-checked build: load liblbm_bounds.so");
#endif
}

int lbm_device_populations(lbm_handle* h, void** d_state, int32_t* tiled) {
    LBM_TRY(check_handle(h));
    if (d_state) *d_state = h->buf[h->cur];
    if (tiled) *tiled = h->tiled ? 1 : 0;
    return LBM_OK;
}

}  // extern "C"
