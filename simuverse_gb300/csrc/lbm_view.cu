// lbm_view.cu -- the consumers of the macro field that simuverse runs after each step:
// tracer particles with their splat canvas, the canvas presentation (colour mapping and
// trail fade), the curl field and the colour mapping of the field itself.  All work stays
// on the device: the kernels read the lattice's macro planes (rho, ux, uy) in place and
// write device buffers; there is no texture or graphics interop.
//
// What each kernel restates (paths inside the simuverse project):
//   k_particles_move / k_particles_splat  assets/wgsl/lbm/particle_update.wgsl:55-87 with
//       func/bilinear_interpolate_3f.wgsl:1-13 and the src_3f clamp (particle_update.wgsl:15-21)
//   k_present_canvas   assets/wgsl/present.wgsl:15-54 (particle colour, alpha fade)
//   k_curl             assets/wgsl/lbm/curl_update.wgsl:12-33
//   k_colorize         assets/wgsl/lbm/present.wgsl:18-40 (curl hue) and
//                      assets/wgsl/lbm/blend_img.wgsl:11-16 (velocity angle hue)
//   hsv2rgb            assets/wgsl/func/color_space_convert.wgsl:2-8
//   particle layout    simuverse/src/lib.rs:248-316 (get_particles_data, init_trajectory_particles)
//
// The macro field the reference samples is an rgba16float texture (macro_tex), so every
// field value is rounded to FP16 before use (h16).  Arithmetic is FP32 with explicit
// round-to-nearest operations and no contraction, so the CPU restatement reproduces the
// particle positions and the canvas bit for bit; atan2 and the colours agree to rounding.
//
// Splat conflicts.  Several particles can write the same canvas pixel in one update; the
// reference's dispatch leaves the winner to the hardware.  In deterministic mode the
// particle with the highest index wins: the move kernel takes a 64-bit atomicMax of
// (update epoch << 32 | index + 1) on every pixel it covers and the splat kernel writes
// the pixels a particle won.  Fast mode writes directly, as the reference does.
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <random>
#include <vector>

#include "lbm_common.cuh"
#include "lbm_internal.h"

struct lbm_particles {
    lbm_particle_params p;
    int num_x = 0, num_y = 0, count = 0;
    int nx = 0, ny = 0, fluid_ty = 0;
    float lattice_pixel = 1.0f;
    float* d_state = nullptr;  // 6 planes of count floats: pos x, pos y, initial x, initial y, life, fade
    float* d_vel = nullptr;    // 2 planes: velocity of the splat of the last update
    uint8_t* d_splat = nullptr;
    unsigned long long* d_winner = nullptr;  // canvas pixels (deterministic mode)
    float* d_canvas = nullptr;               // canvas pixels x (alpha, vx, vy), the reference's Pixel
    float* d_rgba = nullptr;                 // canvas pixels x RGBA of the last present
    uint32_t epoch = 0;
    uint64_t launches = 0, updates = 0;
    int device = 0;
};

namespace view {

using lbm::add_rn;
using lbm::mul_rn;

__device__ __forceinline__ float h16(float v) { return __half2float(__float2half_rn(v)); }
__device__ __forceinline__ float sub_rn(float a, float b) { return __fsub_rn(a, b); }

struct Field {
    const float* rho;
    const float* ux;
    const float* uy;
    int nx, ny;
    int zero;  // no step since initialisation: macro_tex still holds zeros
};

__device__ __forceinline__ float3 texel(const Field& f, int u, int v) {
    u = u < 0 ? 0 : (u > f.nx - 1 ? f.nx - 1 : u);
    v = v < 0 ? 0 : (v > f.ny - 1 ? f.ny - 1 : v);
    if (f.zero) return make_float3(0.0f, 0.0f, 0.0f);
    const size_t c = (size_t)v * f.nx + u;
    return make_float3(h16(__ldg(f.ux + c)), h16(__ldg(f.uy + c)), h16(__ldg(f.rho + c)));
}

// bilinear_interpolate_3f.wgsl:1-13: weights ((1-fx)(1-fy), (1-fx)fy, fx(1-fy), fx fy) on
// (minX, minY), (minX, minY+1), (minX+1, minY), (minX+1, minY+1), summed in that order
__device__ __forceinline__ float2 bilinear_velocity(const Field& f, float x, float y) {
    const int mx = __float2int_rz(floorf(x)), my = __float2int_rz(floorf(y));
    const float fx = sub_rn(x, (float)mx), fy = sub_rn(y, (float)my);
    const float gx = sub_rn(1.0f, fx), gy = sub_rn(1.0f, fy);
    const float w00 = mul_rn(gx, gy), w01 = mul_rn(gx, fy), w10 = mul_rn(fx, gy), w11 = mul_rn(fx, fy);
    const float3 a = texel(f, mx, my), b = texel(f, mx, my + 1), c = texel(f, mx + 1, my), d = texel(f, mx + 1, my + 1);
    float2 r;
    r.x = add_rn(add_rn(add_rn(mul_rn(a.x, w00), mul_rn(b.x, w01)), mul_rn(c.x, w10)), mul_rn(d.x, w11));
    r.y = add_rn(add_rn(add_rn(mul_rn(a.y, w00), mul_rn(b.y, w01)), mul_rn(c.y, w10)), mul_rn(d.y, w11));
    return r;
}

struct ParticleConsts {
    float life_time, speed_factor, lattice_pixel;
    int point_size, canvas_w, canvas_h, poiseuille, deterministic;
};

// particle_update.wgsl:55-87 for particle k; update_canvas (:30-53) splats a point_size
// square at the new position with (fade, velocity)
__global__ void k_particles_move(float* __restrict__ st, int count, float* __restrict__ vel,
                                 uint8_t* __restrict__ splat, unsigned long long* __restrict__ winner,
                                 float* __restrict__ canvas, ParticleConsts pc, Field f, unsigned long long epoch) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count) return;
    const size_t n = (size_t)count;
    float px = st[k], py = st[n + k], life = st[4 * n + k], fade = st[5 * n + k];
    bool draw = false;
    float2 v = make_float2(0.0f, 0.0f);
    if (life <= 0.1f) {
        fade = 0.0f;
        px = st[2 * n + k];
        py = st[3 * n + k];
        life = pc.life_time;
    } else {
        life = sub_rn(life, 1.0f);
        if (fade < 1.0f) fade = fade < 0.95f ? add_rn(fade, 0.1f) : 1.0f;
        const float gx = sub_rn(__fdiv_rn(px, pc.lattice_pixel), 0.5f);
        const float gy = sub_rn(__fdiv_rn(py, pc.lattice_pixel), 0.5f);
        v = bilinear_velocity(f, gx, gy);
        px = add_rn(px, mul_rn(v.x, pc.speed_factor));
        py = add_rn(py, mul_rn(v.y, pc.speed_factor));
        const float speed = add_rn(fabsf(v.x), fabsf(v.y));
        draw = !((!pc.poiseuille && speed < 0.0f) || (pc.poiseuille && speed < 0.015f));
    }
    st[k] = px;
    st[n + k] = py;
    st[4 * n + k] = life;
    st[5 * n + k] = fade;
    splat[k] = draw ? 1 : 0;
    vel[k] = v.x;
    vel[n + k] = v.y;
    if (!draw) return;
    const int x0 = __float2int_rz(px) - pc.point_size / 2, y0 = __float2int_rz(py) - pc.point_size / 2;
    const unsigned long long key = epoch | (unsigned long long)(k + 1);
    for (int dx = 0; dx < pc.point_size; ++dx)
        for (int dy = 0; dy < pc.point_size; ++dy) {
            const int cx = x0 + dx, cy = y0 + dy;
            if (cx < 0 || cx >= pc.canvas_w || cy < 0 || cy >= pc.canvas_h) continue;
            const size_t idx = (size_t)cx + (size_t)pc.canvas_w * cy;
            if (pc.deterministic) {
                atomicMax(winner + idx, key);
            } else {
                canvas[3 * idx] = fade;
                canvas[3 * idx + 1] = v.x;
                canvas[3 * idx + 2] = v.y;
            }
        }
}

// deterministic mode: write the pixels particle k won in this update
__global__ void k_particles_splat(const float* __restrict__ st, int count, const float* __restrict__ vel,
                                  const uint8_t* __restrict__ splat, const unsigned long long* __restrict__ winner,
                                  float* __restrict__ canvas, ParticleConsts pc, unsigned long long epoch) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= count || !splat[k]) return;
    const size_t n = (size_t)count;
    const float px = st[k], py = st[n + k], fade = st[5 * n + k], vx = vel[k], vy = vel[n + k];
    const int x0 = __float2int_rz(px) - pc.point_size / 2, y0 = __float2int_rz(py) - pc.point_size / 2;
    const unsigned long long key = epoch | (unsigned long long)(k + 1);
    for (int dx = 0; dx < pc.point_size; ++dx)
        for (int dy = 0; dy < pc.point_size; ++dy) {
            const int cx = x0 + dx, cy = y0 + dy;
            if (cx < 0 || cx >= pc.canvas_w || cy < 0 || cy >= pc.canvas_h) continue;
            const size_t idx = (size_t)cx + (size_t)pc.canvas_w * cy;
            if (winner[idx] != key) continue;
            canvas[3 * idx] = fade;
            canvas[3 * idx + 1] = vx;
            canvas[3 * idx + 2] = vy;
        }
}

// color_space_convert.wgsl:2-8: K = (1, 2/3, 1/3, 3); p = |fract(h + K.xyz) * 6 - K.w|;
// rgb = v * mix(K.x, clamp(p - K.x, 0, 1), s), mix(a, b, t) = a (1 - t) + b t
__device__ __forceinline__ float3 hsv2rgb(float h, float s, float v) {
    const float K[3] = {1.0f, 2.0f / 3.0f, 1.0f / 3.0f};
    float o[3];
#pragma unroll
    for (int i = 0; i < 3; ++i) {
        const float t = add_rn(h, K[i]);
        const float fr = sub_rn(t, floorf(t));
        const float p = fabsf(sub_rn(mul_rn(fr, 6.0f), 3.0f));
        const float c = fminf(fmaxf(sub_rn(p, 1.0f), 0.0f), 1.0f);
        o[i] = mul_rn(v, add_rn(mul_rn(1.0f, sub_rn(1.0f, s)), mul_rn(c, s)));
    }
    return make_float3(o[0], o[1], o[2]);
}

struct PresentConsts {
    int npix, color_ty, speed_ty;
    float fade_out_factor;
    float r, g, b;
};

// present.wgsl:15-54 for one canvas pixel: colour from the stored splat, then the trail
// fade of the stored alpha
__global__ void k_present_canvas(float* __restrict__ canvas, float4* __restrict__ rgba, PresentConsts c) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= c.npix) return;
    const float a = canvas[3 * (size_t)i], vx = canvas[3 * (size_t)i + 1], vy = canvas[3 * (size_t)i + 2];
    if (!(a > 0.001f)) {
        rgba[i] = make_float4(0.0f, 0.0f, 0.0f, 0.0f);
        return;
    }
    float3 col;
    if (c.color_ty == 1) {
        const float velocity = __fsqrt_rn(add_rn(mul_rn(vx, vx), mul_rn(vy, vy)));
        const float speed = c.speed_ty == 0 ? velocity : fminf(__fdiv_rn(velocity, 0.25f), 1.15f);
        col = hsv2rgb(add_rn(0.05f, mul_rn(speed, 0.75f)), 0.9f, 1.0f);
    } else if (c.color_ty == 0) {
        const float angle = __fdiv_rn(atan2f(vy, vx), mul_rn(2.0f, 3.1415926535f));
        col = hsv2rgb(angle, 0.9f, 1.0f);
    } else {
        col = make_float3(c.r, c.g, c.b);
    }
    rgba[i] = make_float4(col.x, col.y, col.z, a);
    canvas[3 * (size_t)i] = a >= 0.2f ? mul_rn(a, c.fade_out_factor) : mul_rn(a, 0.5f);
}

// curl_update.wgsl:12-33: right/bottom neighbours are clamped to the lattice size (an index
// one past the edge) and left/top to 0; a texel load one past the edge returns the edge
// texel (bounds-restricted load).  curl = R.y - L.y + T.x - B.x, stored as
// curl * 3.5 + 0.5 in an rgba16float texel
__device__ __forceinline__ float texel1(const Field& f, const float* plane, int u, int v) {
    u = u < 0 ? 0 : (u > f.nx - 1 ? f.nx - 1 : u);
    v = v < 0 ? 0 : (v > f.ny - 1 ? f.ny - 1 : v);
    return f.zero ? 0.0f : h16(__ldg(plane + (size_t)v * f.nx + u));
}

__global__ void k_curl(Field f, float* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= f.nx) return;
    const float Ry = texel1(f, f.uy, x + 1 > f.nx ? f.nx : x + 1, y), Ly = texel1(f, f.uy, x - 1 < 0 ? 0 : x - 1, y);
    const float Tx = texel1(f, f.ux, x, y - 1 < 0 ? 0 : y - 1), Bx = texel1(f, f.ux, x, y + 1 > f.ny ? f.ny : y + 1);
    const float curl = sub_rn(add_rn(sub_rn(Ry, Ly), Tx), Bx);
    out[(size_t)y * f.nx + x] = h16(add_rn(mul_rn(curl, 3.5f), 0.5f));
}

// the same for four consecutive cells x0..x0+3 per thread (nx % 4 == 0, so x0 + 3 < nx): one
// 16-byte load per row and plane, the left / right neighbours of the row y by scalar loads
__global__ void k_curl4(Field f, float* __restrict__ out) {
    const int x0 = 4 * (blockIdx.x * blockDim.x + threadIdx.x), y = blockIdx.y;
    if (x0 >= f.nx) return;
    float4 r;
    if (f.zero) {
        const float c = h16(0.5f);  // curl 0 stored as 0 * 3.5 + 0.5
        r = make_float4(c, c, c, c);
    } else {
        const int yt = y - 1 < 0 ? 0 : y - 1, yb = y + 1 > f.ny - 1 ? f.ny - 1 : y + 1;  // clamped rows
        const float4 T = __ldg(reinterpret_cast<const float4*>(f.ux + (size_t)yt * f.nx + x0));
        const float4 Bv = __ldg(reinterpret_cast<const float4*>(f.ux + (size_t)yb * f.nx + x0));
        const float* uyr = f.uy + (size_t)y * f.nx;
        const float4 M = __ldg(reinterpret_cast<const float4*>(uyr + x0));
        const float l = __ldg(uyr + (x0 > 0 ? x0 - 1 : 0));
        const float rr = __ldg(uyr + (x0 + 4 < f.nx ? x0 + 4 : f.nx - 1));
        const float uy[6] = {h16(l), h16(M.x), h16(M.y), h16(M.z), h16(M.w), h16(rr)};
        const float tx[4] = {h16(T.x), h16(T.y), h16(T.z), h16(T.w)};
        const float bx[4] = {h16(Bv.x), h16(Bv.y), h16(Bv.z), h16(Bv.w)};
        float o[4];
#pragma unroll
        for (int k = 0; k < 4; ++k) {
            // left neighbour of x0 + k is uy[k] (clamped at x = 0 by the load above), right is uy[k + 2]
            const float curl = sub_rn(add_rn(sub_rn(uy[k + 2], uy[k]), tx[k]), bx[k]);
            o[k] = h16(add_rn(mul_rn(curl, 3.5f), 0.5f));
        }
        r = make_float4(o[0], o[1], o[2], o[3]);
    }
    *reinterpret_cast<float4*>(out + (size_t)y * f.nx + x0) = r;
}

// The field colour map: canvas pixel (px, py) samples each plane at uv = ((px + 0.5) / cw,
// (py + 0.5) / ch), as the full-screen triangle of bufferless.vs.wgsl interpolates it, with
// linear filtering and clamp-to-edge addressing and exact FP32 weights:
//   h(row) = t[row][xa] bx + t[row][xb] ax,   value = h(ya) by + h(yb) ay
// (every product and sum rounded on its own).  A thread owns one canvas column and COLOR_ROWS
// consecutive pixels of it, so the column's weights and texel columns are computed once, and
// the horizontal terms h of a texel row are kept while consecutive pixel rows sample it (a
// canvas larger than the lattice samples each texel row for several pixel rows).  The rows'
// weights are computed once per block.
constexpr int COLOR_ROWS = 8;
constexpr int COLOR_TPB = 128;

template <int MODE>
__global__ void __launch_bounds__(COLOR_TPB) k_colorize(Field f, const float* __restrict__ curl, int cw, int ch,
                                                        float4* __restrict__ rgba) {
    __shared__ float s_ay[COLOR_ROWS], s_by[COLOR_ROWS];
    __shared__ int s_ya[COLOR_ROWS], s_yb[COLOR_ROWS];
    const int py0 = blockIdx.y * COLOR_ROWS;
    if (threadIdx.x < COLOR_ROWS) {
        const int py = py0 + (int)threadIdx.x;
        const float v = __fdiv_rn(add_rn((float)py, 0.5f), (float)ch);
        const float ty = sub_rn(mul_rn(v, (float)f.ny), 0.5f);
        const float fy0 = floorf(ty);
        const float ay = sub_rn(ty, fy0);
        const int y0 = (int)fy0;
        s_ay[threadIdx.x] = ay;
        s_by[threadIdx.x] = sub_rn(1.0f, ay);
        s_ya[threadIdx.x] = y0 < 0 ? 0 : (y0 > f.ny - 1 ? f.ny - 1 : y0);
        s_yb[threadIdx.x] = y0 + 1 < 0 ? 0 : (y0 + 1 > f.ny - 1 ? f.ny - 1 : y0 + 1);
    }
    __syncthreads();
    const int px = blockIdx.x * COLOR_TPB + threadIdx.x;
    if (px >= cw) return;
    const float u = __fdiv_rn(add_rn((float)px, 0.5f), (float)cw);
    const float tx = sub_rn(mul_rn(u, (float)f.nx), 0.5f);
    const float fx0 = floorf(tx);
    const float ax = sub_rn(tx, fx0), bx = sub_rn(1.0f, ax);
    const int x0 = (int)fx0;
    const int xa = x0 < 0 ? 0 : (x0 > f.nx - 1 ? f.nx - 1 : x0), xb = x0 + 1 < 0 ? 0 : (x0 + 1 > f.nx - 1 ? f.nx - 1 : x0 + 1);
    // horizontal terms of texel row y: ux, uy, rho (rounded to FP16 as macro_tex holds them), curl
    constexpr int NP = MODE == LBM_COLOR_CURL ? 4 : 2;
    auto row_terms = [&](int y, float* h) {
        const size_t ra = (size_t)y * f.nx + xa, rb = (size_t)y * f.nx + xb;
        const float* planes[3] = {f.ux, f.uy, f.rho};
#pragma unroll
        for (int k = 0; k < (NP < 3 ? NP : 3); ++k)
            h[k] = f.zero ? 0.0f
                          : add_rn(mul_rn(h16(__ldg(planes[k] + ra)), bx), mul_rn(h16(__ldg(planes[k] + rb)), ax));
        if (NP == 4) h[3] = curl ? add_rn(mul_rn(__ldg(curl + ra), bx), mul_rn(__ldg(curl + rb), ax)) : 0.0f;
    };
    int r0 = -1, r1 = -1;  // texel rows whose terms h0, h1 hold
    float h0[NP], h1[NP];
#pragma unroll 1
    for (int k = 0; k < COLOR_ROWS; ++k) {
        const int py = py0 + k;
        if (py >= ch) break;
        const int ya = s_ya[k], yb = s_yb[k];
        const float ay = s_ay[k], by = s_by[k];
        float ha[NP], hb[NP];
        // warp-uniform branches: every thread of the block is on the same pixel row
        if (ya == r0) {
#pragma unroll
            for (int q = 0; q < NP; ++q) ha[q] = h0[q];
        } else if (ya == r1) {
#pragma unroll
            for (int q = 0; q < NP; ++q) ha[q] = h1[q];
        } else {
            row_terms(ya, ha);
        }
        if (yb == ya) {
#pragma unroll
            for (int q = 0; q < NP; ++q) hb[q] = ha[q];
        } else if (yb == r1) {
#pragma unroll
            for (int q = 0; q < NP; ++q) hb[q] = h1[q];
        } else if (yb == r0) {
#pragma unroll
            for (int q = 0; q < NP; ++q) hb[q] = h0[q];
        } else {
            row_terms(yb, hb);
        }
        r0 = ya;
        r1 = yb;
#pragma unroll
        for (int q = 0; q < NP; ++q) {
            h0[q] = ha[q];
            h1[q] = hb[q];
        }
        float m[NP];
#pragma unroll
        for (int q = 0; q < NP; ++q) m[q] = add_rn(mul_rn(ha[q], by), mul_rn(hb[q], ay));
        float4 out;
        if (MODE == LBM_COLOR_CURL) {
            const float speed = add_rn(fabsf(m[0]), fabsf(m[1]));
            const float3 col = hsv2rgb(m[NP - 1], add_rn(0.6f, mul_rn(speed, 1.4f)), add_rn(0.6f, mul_rn(m[2 % NP], 0.33f)));
            out = make_float4(col.x, col.y, col.z, m[2 % NP]);
        } else {  // blend_img.wgsl: hue from atan2(ux, uy) with PI = 3.1415926
            const float angle = __fdiv_rn(add_rn(atan2f(m[0], m[1]), 3.1415926f), mul_rn(2.0f, 3.1415926f));
            const float3 col = hsv2rgb(angle, 0.75f, 1.0f);
            out = make_float4(col.x, col.y, col.z, 1.0f);
        }
        rgba[(size_t)py * cw + px] = out;
    }
}

}  // namespace view

namespace {

int vfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lbm::set_error(code, buf);
}

#define V_CK(call)                                                                                    \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return vfail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
    } while (0)

view::Field field_of(const lbm_handle* h) {
    view::Field f;
    f.rho = h->d_macro;
    f.ux = h->d_macro + h->N;
    f.uy = h->d_macro + 2 * h->N;
    f.nx = h->nx;
    f.ny = h->ny;
    f.zero = h->stepped_since_init ? 0 : 1;
    return f;
}

double unit53(std::mt19937_64& g) { return (double)(g() >> 11) * (1.0 / 9007199254740992.0); }

// uniform on [lo, hi] from one 53-bit draw
float uniform_incl(std::mt19937_64& g, float lo, float hi) { return (float)((double)lo + ((double)hi - (double)lo) * unit53(g)); }

void free_particles(lbm_particles* ps) {
    cudaFree(ps->d_state);
    cudaFree(ps->d_vel);
    cudaFree(ps->d_splat);
    cudaFree(ps->d_winner);
    cudaFree(ps->d_canvas);
    cudaFree(ps->d_rgba);
}

int check_pair(const lbm_particles* ps, const lbm_handle* h) {
    if (!ps || !h) return vfail(LBM_ERR_ARG, "null argument");
    if (h->nx != ps->nx || h->ny != ps->ny)
        return vfail(LBM_ERR_ARG, "lattice %dx%d does not match the particles' %dx%d", h->nx, h->ny, ps->nx, ps->ny);
    return LBM_OK;
}

}  // namespace

extern "C" {

void lbm_particle_params_default(lbm_particle_params* p) {
    if (!p) return;
    std::memset(p, 0, sizeof(*p));
    p->count = 10000;
    p->life_time = 60.0f;
    p->point_size = 2;
    p->speed_factor = 4.15f;     // setting_obj.rs:49-53 (fluid simulator)
    p->fade_out_factor = 0.96f;  // setting_obj.rs:48
    p->color_ty = 1;
    p->color[0] = p->color[1] = p->color[2] = p->color[3] = 1.0f;
    p->seed = 0;
    p->deterministic = 1;
}

int lbm_particles_grid(int32_t canvas_w, int32_t canvas_h, int32_t count, int32_t* num_x, int32_t* num_y) {
    if (canvas_w < 1 || canvas_h < 1 || count < 1 || !num_x || !num_y)
        return vfail(LBM_ERR_ARG, "canvas and count must be positive");
    // lib.rs:253-262: x = ceil(sqrt(count * ratio)), height = ceil(x / ratio)
    const float ratio = (float)canvas_w / (float)canvas_h;
    const float x = std::ceil(std::sqrt((float)count * ratio));
    *num_x = (int32_t)x;
    *num_y = (int32_t)std::ceil(x * (1.0f / ratio));
    return LBM_OK;
}

int lbm_particles_init_state(const lbm_particle_params* p, int32_t num_x, int32_t num_y, float* out) {
    if (!p || !out || num_x < 2 || num_y < 2) return vfail(LBM_ERR_ARG, "particle grid must be at least 2 x 2");
    // lib.rs:286-316: a jittered grid in canvas pixels; particle (x, y) of the grid is entry
    // x * num_y + y.  Draw order per particle: jitter x, jitter y, then (life_time <= 1)
    // the initial x, else the life.  rand::rng() is replaced by mt19937_64(seed).
    std::mt19937_64 g(p->seed);
    const float step_x = (float)p->canvas_w / (float)(num_x - 1), step_y = (float)p->canvas_h / (float)(num_y - 1);
    const float life_hi = p->life_time <= 0.0f ? 1.0f : p->life_time;
    size_t k = 0;
    for (int x = 0; x < num_x; ++x) {
        const float pixel_x = step_x * (float)x;
        for (int y = 0; y < num_y; ++y, ++k) {
            float* o = out + 6 * k;
            o[0] = pixel_x + uniform_incl(g, -step_x, step_x);
            o[1] = step_y * (float)y + uniform_incl(g, -step_y, step_y);
            if (p->life_time <= 1.0f) {
                o[2] = (float)((double)step_x * unit53(g));
                o[3] = o[1];
                o[4] = 0.0f;
            } else {
                o[2] = o[0];
                o[3] = o[1];
                o[4] = uniform_incl(g, 0.0f, life_hi);
            }
            o[5] = 0.0f;
        }
    }
    return LBM_OK;
}

int lbm_particles_create(lbm_handle* h, const lbm_particle_params* p, lbm_particles** out) {
    if (!h || !p || !out) return vfail(LBM_ERR_ARG, "null argument");
    *out = nullptr;
    if (p->canvas_w / h->p.pixel_size != h->nx || p->canvas_h / h->p.pixel_size != h->ny)
        return vfail(LBM_ERR_ARG, "canvas %dx%d at %d pixels per cell is not the %dx%d lattice (d2q9_node.rs:38-42)",
                     p->canvas_w, p->canvas_h, h->p.pixel_size, h->nx, h->ny);
    if (p->point_size < 1 || p->point_size > 64) return vfail(LBM_ERR_ARG, "point_size must be in [1, 64]");
    if (!std::isfinite(p->speed_factor) || !std::isfinite(p->life_time) || !std::isfinite(p->fade_out_factor))
        return vfail(LBM_ERR_ARG, "non-finite particle parameter");
    int nxp = 0, nyp = 0;
    int r = lbm_particles_grid(p->canvas_w, p->canvas_h, p->count, &nxp, &nyp);
    if (r < 0) return r;
    if (nxp < 2 || nyp < 2 || (int64_t)nxp * nyp > (1 << 30)) return vfail(LBM_ERR_ARG, "particle grid %dx%d out of range", nxp, nyp);
    std::vector<float> aos((size_t)6 * nxp * nyp);
    r = lbm_particles_init_state(p, nxp, nyp, aos.data());
    if (r < 0) return r;
    lbm_particles* ps = new (std::nothrow) lbm_particles();
    if (!ps) return vfail(LBM_ERR_NOMEM, "out of host memory");
    ps->p = *p;
    ps->num_x = nxp;
    ps->num_y = nyp;
    ps->count = nxp * nyp;
    ps->nx = h->nx;
    ps->ny = h->ny;
    ps->fluid_ty = h->fluid_ty;
    ps->lattice_pixel = (float)h->p.pixel_size;
    ps->device = h->device;
    const size_t n = (size_t)ps->count, npix = (size_t)p->canvas_w * p->canvas_h;
    cudaError_t e = cudaSetDevice(h->device);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_state, 6 * n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_vel, 2 * n * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_splat, n);
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_winner, npix * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_canvas, 3 * npix * sizeof(float));
    if (e == cudaSuccess) e = cudaMalloc((void**)&ps->d_rgba, 4 * npix * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(ps->d_winner, 0, npix * sizeof(unsigned long long));
    if (e == cudaSuccess) e = cudaMemset(ps->d_canvas, 0, 3 * npix * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(ps->d_rgba, 0, 4 * npix * sizeof(float));
    if (e == cudaSuccess) {
        std::vector<float> soa(6 * n);
        for (size_t k = 0; k < n; ++k)
            for (int q = 0; q < 6; ++q) soa[q * n + k] = aos[6 * k + q];
        e = cudaMemcpy(ps->d_state, soa.data(), soa.size() * sizeof(float), cudaMemcpyHostToDevice);
    }
    if (e != cudaSuccess) {
        free_particles(ps);
        delete ps;
        return vfail(LBM_ERR_CUDA, "particle allocation: %s", cudaGetErrorString(e));
    }
    *out = ps;
    return LBM_OK;
}

int lbm_particles_destroy(lbm_particles* ps) {
    if (!ps) return LBM_OK;
    cudaSetDevice(ps->device);
    cudaDeviceSynchronize();
    free_particles(ps);
    delete ps;
    return LBM_OK;
}

int lbm_particles_info(const lbm_particles* ps, int32_t* num_x, int32_t* num_y) {
    if (!ps || !num_x || !num_y) return vfail(LBM_ERR_ARG, "null argument");
    *num_x = ps->num_x;
    *num_y = ps->num_y;
    return LBM_OK;
}

int lbm_particles_update(lbm_particles* ps, lbm_handle* h) {
    LbmRange range_("lbm_particles_update");
    int r = check_pair(ps, h);
    if (r < 0) return r;
    V_CK(cudaSetDevice(ps->device));
    if (++ps->epoch == 0) {  // 2^32 updates: restart the keys from a clean winner map
        V_CK(cudaMemsetAsync(ps->d_winner, 0, (size_t)ps->p.canvas_w * ps->p.canvas_h * sizeof(unsigned long long),
                             h->stream));
        ps->epoch = 1;
    }
    view::ParticleConsts pc;
    pc.life_time = ps->p.life_time;
    pc.speed_factor = ps->p.speed_factor;
    pc.lattice_pixel = ps->lattice_pixel;
    pc.point_size = ps->p.point_size;
    pc.canvas_w = ps->p.canvas_w;
    pc.canvas_h = ps->p.canvas_h;
    pc.poiseuille = h->fluid_ty == 0 ? 1 : 0;
    pc.deterministic = ps->p.deterministic ? 1 : 0;
    const unsigned long long epoch = (unsigned long long)ps->epoch << 32;
    const int blocks = (ps->count + 255) / 256;
    view::k_particles_move<<<blocks, 256, 0, h->stream>>>(ps->d_state, ps->count, ps->d_vel, ps->d_splat, ps->d_winner,
                                                         ps->d_canvas, pc, field_of(h), epoch);
    V_CK(cudaGetLastError());
    ++ps->launches;
    if (pc.deterministic) {
        view::k_particles_splat<<<blocks, 256, 0, h->stream>>>(ps->d_state, ps->count, ps->d_vel, ps->d_splat,
                                                              ps->d_winner, ps->d_canvas, pc, epoch);
        V_CK(cudaGetLastError());
        ++ps->launches;
    }
    ++ps->updates;
    return LBM_OK;
}

int lbm_particles_present(lbm_particles* ps, lbm_handle* h, float** d_rgba) {
    LbmRange range_("lbm_particles_present");
    int r = check_pair(ps, h);
    if (r < 0) return r;
    V_CK(cudaSetDevice(ps->device));
    view::PresentConsts c;
    c.npix = ps->p.canvas_w * ps->p.canvas_h;
    c.color_ty = ps->p.color_ty;
    c.speed_ty = 1;  // d2q9_node.rs:74: lattice speeds
    c.fade_out_factor = ps->p.fade_out_factor;
    c.r = ps->p.color[0];
    c.g = ps->p.color[1];
    c.b = ps->p.color[2];
    view::k_present_canvas<<<(c.npix + 255) / 256, 256, 0, h->stream>>>(ps->d_canvas,
                                                                        reinterpret_cast<float4*>(ps->d_rgba), c);
    V_CK(cudaGetLastError());
    ++ps->launches;
    if (d_rgba) *d_rgba = ps->d_rgba;
    return LBM_OK;
}

int lbm_particles_read(lbm_particles* ps, float* out) {
    if (!ps || !out) return vfail(LBM_ERR_ARG, "null argument");
    V_CK(cudaSetDevice(ps->device));
    const size_t n = (size_t)ps->count;
    std::vector<float> soa(6 * n);
    V_CK(cudaDeviceSynchronize());
    V_CK(cudaMemcpy(soa.data(), ps->d_state, soa.size() * sizeof(float), cudaMemcpyDeviceToHost));
    for (size_t k = 0; k < n; ++k)
        for (int q = 0; q < 6; ++q) out[6 * k + q] = soa[q * n + k];
    return LBM_OK;
}

int lbm_particles_write(lbm_particles* ps, const float* in) {
    if (!ps || !in) return vfail(LBM_ERR_ARG, "null argument");
    V_CK(cudaSetDevice(ps->device));
    const size_t n = (size_t)ps->count;
    std::vector<float> soa(6 * n);
    for (size_t k = 0; k < n; ++k)
        for (int q = 0; q < 6; ++q) soa[q * n + k] = in[6 * k + q];
    V_CK(cudaDeviceSynchronize());
    V_CK(cudaMemcpy(ps->d_state, soa.data(), soa.size() * sizeof(float), cudaMemcpyHostToDevice));
    return LBM_OK;
}

int lbm_particles_read_canvas(lbm_particles* ps, float* canvas, float* rgba) {
    if (!ps || (!canvas && !rgba)) return vfail(LBM_ERR_ARG, "null argument");
    V_CK(cudaSetDevice(ps->device));
    V_CK(cudaDeviceSynchronize());
    const size_t npix = (size_t)ps->p.canvas_w * ps->p.canvas_h;
    if (canvas) V_CK(cudaMemcpy(canvas, ps->d_canvas, 3 * npix * sizeof(float), cudaMemcpyDeviceToHost));
    if (rgba) V_CK(cudaMemcpy(rgba, ps->d_rgba, 4 * npix * sizeof(float), cudaMemcpyDeviceToHost));
    return LBM_OK;
}

int lbm_particles_counters(const lbm_particles* ps, uint64_t* updates, uint64_t* launches) {
    if (!ps || !updates || !launches) return vfail(LBM_ERR_ARG, "null argument");
    *updates = ps->updates;
    *launches = ps->launches;
    return LBM_OK;
}

int lbm_curl(lbm_handle* h, float* d_out) {
    LbmRange range_("lbm_curl");
    if (!h || !d_out) return vfail(LBM_ERR_ARG, "null argument");
    V_CK(cudaSetDevice(h->device));
    if (h->nx % 4 == 0 && ((uintptr_t)d_out & 15) == 0) {
        const dim3 grid((unsigned)((h->nx / 4 + 127) / 128), (unsigned)h->ny);
        view::k_curl4<<<grid, 128, 0, h->stream>>>(field_of(h), d_out);
    } else {
        const dim3 grid((unsigned)((h->nx + 127) / 128), (unsigned)h->ny);
        view::k_curl<<<grid, 128, 0, h->stream>>>(field_of(h), d_out);
    }
    V_CK(cudaGetLastError());
    ++h->launches;
    return LBM_OK;
}

int lbm_colorize(lbm_handle* h, int32_t mode, const float* d_curl, int32_t canvas_w, int32_t canvas_h, float* d_rgba) {
    LbmRange range_("lbm_colorize");
    if (!h || !d_rgba) return vfail(LBM_ERR_ARG, "null argument");
    if (mode != LBM_COLOR_CURL && mode != LBM_COLOR_ANGLE) return vfail(LBM_ERR_ARG, "unknown colour mode %d", mode);
    if (canvas_w < 1 || canvas_h < 1 || canvas_h > 65535) return vfail(LBM_ERR_ARG, "canvas size out of range");
    V_CK(cudaSetDevice(h->device));
    const dim3 grid((unsigned)((canvas_w + view::COLOR_TPB - 1) / view::COLOR_TPB),
                    (unsigned)((canvas_h + view::COLOR_ROWS - 1) / view::COLOR_ROWS));
    if (mode == LBM_COLOR_CURL)
        view::k_colorize<LBM_COLOR_CURL><<<grid, view::COLOR_TPB, 0, h->stream>>>(
            field_of(h), d_curl, canvas_w, canvas_h, reinterpret_cast<float4*>(d_rgba));
    else
        view::k_colorize<LBM_COLOR_ANGLE><<<grid, view::COLOR_TPB, 0, h->stream>>>(
            field_of(h), d_curl, canvas_w, canvas_h, reinterpret_cast<float4*>(d_rgba));
    V_CK(cudaGetLastError());
    ++h->launches;
    return LBM_OK;
}

}  // extern "C"
