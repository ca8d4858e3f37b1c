// lbm_closure.cu -- the learned closure of a 4x-coarsened lattice: coarse-graining, the
// BF16 convolutional correction (forward, backward, inference), its training with Adam,
// and the conservation projection.  No counterpart in the reference.
//
// Features and outputs.  For a coarse cell with deviations d (= f - w), density rho and
// velocity u, the input features are s_in * f_neq, f_neq = d - deq(rho, u), or (inputs
// LBM_CLOSURE_INPUT_EQ) s_in * deq(rho, u), which depends on the macroscopic fields only
// (9 channels either way).
// The network output y (9 channels, output units) becomes the correction
//   delta = P(y) / s_out,   P(y)_i = y_i - w_i (sum_k y_k + 3 e_i . sum_k e_k y_k),
// which satisfies sum_i delta_i = 0 and sum_i e_i delta_i = 0 exactly (up to rounding):
// the correction changes neither the density nor the momentum of any cell.
//
// Training pairs.  For a coarse state C (the coarse-grained fine state, stepped k coarse
// steps) and the target C* (the coarse-grained fine state k*factor fine steps later), the
// features are taken from C and the target is s_out * P(C* - C).  The loss is the mean
// squared difference of P(y) and the target over the interior of each crop (3 cells in
// from every edge: the network's receptive field is 7 x 7).
//
// Parameters.  Master copies are FP32 in a padded layout (W1[9][16][32], b1[32], W2[9][32][32],
// b2[32], W3[9][32][16], b3[16]; padded entries stay 0), converted to BF16 conv layouts
// after every update.  The logical parameter vector of the API is W1[9][9][32], b1[32],
// W2[9][32][32], b2[32], W3[9][32][9], b3[9] (14,473 values), [tap][cin][cout].
#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <random>
#include <type_traits>
#include <vector>

#include "lbm_closure_kernels.cuh"
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbm {
namespace closure {

// padded parameter layout
constexpr int OW1 = 0, NW1 = 9 * 16 * 32;
constexpr int OB1 = OW1 + NW1, NB1 = 32;
constexpr int OW2 = OB1 + NB1, NW2 = 9 * 32 * 32;
constexpr int OB2 = OW2 + NW2, NB2 = 32;
constexpr int OW3 = OB2 + NB2, NW3 = 9 * 32 * 16;
constexpr int OB3 = OW3 + NW3, NB3 = 16;
constexpr int NPARAM = OB3 + NB3;  // 18512
constexpr int NLOGICAL = 9 * 9 * 32 + 32 + 9 * 32 * 32 + 32 + 9 * 32 * 9 + 9;  // 14473
constexpr int DW_BLOCKS = 304;  // 2 x 152 SMs

__device__ __forceinline__ void project9(float (&v)[9]) {
    float s = 0.0f, sx = 0.0f, sy = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        s += v[i];
        sx += (float)EX(i) * v[i];
        sy += (float)EY(i) * v[i];
    }
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] -= PW<float>(i) * (s + 3.0f * ((float)EX(i) * sx + (float)EY(i) * sy));
}

// transpose of project9: g_k - sum_i w_i g_i - 3 e_k . sum_i w_i e_i g_i
__device__ __forceinline__ void project9_t(float (&g)[9]) {
    float a = 0.0f, ax = 0.0f, ay = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        a += PW<float>(i) * g[i];
        ax += PW<float>(i) * (float)EX(i) * g[i];
        ay += PW<float>(i) * (float)EY(i) * g[i];
    }
#pragma unroll
    for (int k = 0; k < 9; ++k) g[k] -= a + 3.0f * ((float)EX(k) * ax + (float)EY(k) * ay);
}

__device__ __forceinline__ void load_dev(const float* __restrict__ d, size_t N, size_t c, float (&v)[9]) {
#pragma unroll
    for (int i = 0; i < 9; ++i) v[i] = d[c + (size_t)i * N];
}

// equilibrium deviation deq_i(rho, u) for the deviations d of one cell; returns f_neq in v
__device__ __forceinline__ void non_equilibrium(float (&v)[9]) {
    float drho = 0.0f, jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        drho += v[i];
        jx += (float)EX(i) * v[i];
        jy += (float)EY(i) * v[i];
    }
    const float rho = 1.0f + drho, ux = jx / rho, uy = jy / rho;
    const float usq = 1.5f * (ux * ux + uy * uy);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float eu = (float)EX(i) * ux + (float)EY(i) * uy;
        v[i] -= PW<float>(i) * (drho + rho * (3.0f * eu + 4.5f * eu * eu - usq));
    }
}

// features of an H x W window at (ox, oy) of an nx x ny periodic coarse field: s_in * f_neq
// (inputs LBM_CLOSURE_INPUT_NEQ) or s_in * deq(rho, u) (LBM_CLOSURE_INPUT_EQ)
__global__ void k_features(const float* __restrict__ d, int nx, int ny, int ox, int oy, int H, int W, float s_in,
                           int inputs, __nv_bfloat16* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const int gx = (ox + x) % nx, gy = (oy + y) % ny;
    float v[9];
    load_dev(d, (size_t)nx * ny, (size_t)gy * nx + gx, v);
    if (inputs == LBM_CLOSURE_INPUT_EQ) {
        float n[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) n[i] = v[i];
        non_equilibrium(n);
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] -= n[i];
    } else {
        non_equilibrium(v);
    }
    unsigned* o = reinterpret_cast<unsigned*>(out + ((size_t)y * W + x) * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = pack_bf16x2(s_in * v[2 * k], s_in * v[2 * k + 1]);
    o[4] = pack_bf16x2(s_in * v[8], 0.0f);
    o[5] = o[6] = o[7] = 0u;
}

// target of an H x W window at (ox, oy): s_out * (target - pred) (LBM_CLOSURE_TARGET_POPULATIONS),
// s_out * (deq(rho*, u*) - deq(rho, u)) (LBM_CLOSURE_TARGET_EQUILIBRIUM) or the momentum
// difference alone, s_out * 3 w_i e_i . (j* - j) (LBM_CLOSURE_TARGET_MOMENTUM); projected cell by
// cell with P when the projection is LBM_CLOSURE_PROJECT_CELL
__global__ void k_target(const float* __restrict__ dt, const float* __restrict__ dp, int nx, int ny, int ox, int oy,
                         int H, int W, float s_out, int target, int project_cell, __nv_bfloat16* __restrict__ out) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = blockIdx.y;
    if (x >= W) return;
    const size_t N = (size_t)nx * ny, c = (size_t)((oy + y) % ny) * nx + (ox + x) % nx;
    float v[9];
    if (target == LBM_CLOSURE_TARGET_MOMENTUM) {
        float jx = 0.0f, jy = 0.0f;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float df = dt[c + i * N] - dp[c + i * N];
            jx += (float)EX(i) * df;
            jy += (float)EY(i) * df;
        }
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = 3.0f * PW<float>(i) * ((float)EX(i) * jx + (float)EY(i) * jy);
    } else if (target == LBM_CLOSURE_TARGET_EQUILIBRIUM) {
        float a[9], b[9], na[9], nb[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            a[i] = na[i] = dt[c + i * N];
            b[i] = nb[i] = dp[c + i * N];
        }
        non_equilibrium(na);
        non_equilibrium(nb);
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = (a[i] - na[i]) - (b[i] - nb[i]);
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = dt[c + i * N] - dp[c + i * N];
    }
    if (project_cell) project9(v);
    unsigned* o = reinterpret_cast<unsigned*>(out + ((size_t)y * W + x) * 16);
#pragma unroll
    for (int k = 0; k < 4; ++k) o[k] = pack_bf16x2(s_out * v[2 * k], s_out * v[2 * k + 1]);
    o[4] = pack_bf16x2(s_out * v[8], 0.0f);
    o[5] = o[6] = o[7] = 0u;
}

// FP64 partial sums over the field of (sum_i y_i, sum_i e_x y_i, sum_i e_y y_i), one triple
// per block, grid-stride over cells in a fixed order
__global__ void k_ysums(const float* __restrict__ y, size_t N, double* __restrict__ part) {
    __shared__ double red[3][32];
    double m = 0.0, jx = 0.0, jy = 0.0;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += (size_t)gridDim.x * blockDim.x) {
        float s = 0.0f, sx = 0.0f, sy = 0.0f;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float v = y[c * 16 + i];
            s += v;
            sx += (float)EX(i) * v;
            sy += (float)EY(i) * v;
        }
        m += s;
        jx += sx;
        jy += sy;
    }
    for (int o = 16; o > 0; o >>= 1) {
        m += __shfl_down_sync(0xffffffffu, m, o);
        jx += __shfl_down_sync(0xffffffffu, jx, o);
        jy += __shfl_down_sync(0xffffffffu, jy, o);
    }
    if ((threadIdx.x & 31) == 0) {
        red[0][threadIdx.x >> 5] = m;
        red[1][threadIdx.x >> 5] = jx;
        red[2][threadIdx.x >> 5] = jy;
    }
    __syncthreads();
    if (threadIdx.x < 3) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[threadIdx.x][w];
        part[3 * blockIdx.x + threadIdx.x] = t;
    }
}

// means[k] = sum of the partials of component k / N, in block order
__global__ void k_ymeans(const double* __restrict__ part, int nblocks, double inv_n, double* __restrict__ means) {
    if (blockIdx.x != 0 || threadIdx.x >= 3) return;
    double t = 0.0;
    for (int b = 0; b < nblocks; ++b) t += part[3 * b + threadIdx.x];
    means[threadIdx.x] = t * inv_n;
}

// the correction delta of a full nx x ny field (y: [ny][nx][16] f32): P(y) / s_out cell by
// cell (means == nullptr), or (y_i - w_i (m + 3 e_i . j)) / s_out with (m, j) the field means
// of the network output's density and momentum, so that the field's total mass and momentum
// do not change.  accumulate: d += delta (the populations); else d = delta (9 planes)
__global__ void k_apply(const float* __restrict__ y, float* __restrict__ d, int nx, int ny, float inv_s_out,
                        const double* __restrict__ means, int accumulate) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (x >= nx) return;
    const size_t N = (size_t)nx * ny, c = (size_t)r * nx + x;
    float v[9];
    const float4* yp = reinterpret_cast<const float4*>(y + c * 16);
    const float4 a = yp[0], b = yp[1];
    v[0] = a.x; v[1] = a.y; v[2] = a.z; v[3] = a.w; v[4] = b.x; v[5] = b.y; v[6] = b.z; v[7] = b.w;
    v[8] = y[c * 16 + 8];
    if (means) {
        const float m = (float)means[0], jx = (float)means[1], jy = (float)means[2];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] -= PW<float>(i) * (m + 3.0f * ((float)EX(i) * jx + (float)EY(i) * jy));
    } else {
        project9(v);
    }
    if (accumulate) {
#pragma unroll
        for (int i = 0; i < 9; ++i) d[c + i * N] += inv_s_out * v[i];
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) d[c + i * N] = inv_s_out * v[i];
    }
}

// The stress target's correction, a momentum change in flux form: dj(x) = -1/2 sum_i e_i
// z_i(x - e_i) / s_out over the periodic field, z = P(y) as 9 planes of nx * ny floats, added
// to the cell's populations as 3 w_i e_i . dj.  No cell's density changes; the lattice's total
// momentum does not either (a lattice divergence sums to zero).  accumulate: d += delta, else
// d = delta (9 planes)
__global__ void k_apply_stress(const float* __restrict__ z, float* __restrict__ d, int nx, int ny, float inv_s_out,
                               int accumulate) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, r = blockIdx.y;
    if (x >= nx) return;
    const size_t N = (size_t)nx * ny, c = (size_t)r * nx + x;
    float jx = 0.0f, jy = 0.0f;
#pragma unroll
    for (int i = 1; i < 9; ++i) {  // population i of the source cell x - e_i
        const int sx = x - EX(i) < 0 ? nx - 1 : (x - EX(i) >= nx ? 0 : x - EX(i));
        const int sy = r - EY(i) < 0 ? ny - 1 : (r - EY(i) >= ny ? 0 : r - EY(i));
        const float v = z[(size_t)i * N + (size_t)sy * nx + sx];
        jx += (float)EX(i) * v;
        jy += (float)EY(i) * v;
    }
    jx *= -0.5f * inv_s_out;
    jy *= -0.5f * inv_s_out;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float delta = 3.0f * PW<float>(i) * ((float)EX(i) * jx + (float)EY(i) * jy);
        if (accumulate)
            d[c + i * N] += delta;
        else
            d[c + i * N] = delta;
    }
}

// P(y) of every cell of a field (y: [N][16] f32) into 9 planes of N floats
__global__ void k_project_planes(const float* __restrict__ y, size_t N, float* __restrict__ z) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    float v[9];
#pragma unroll
    for (int k = 0; k < 9; ++k) v[k] = y[c * 16 + k];
    project9(v);
#pragma unroll
    for (int k = 0; k < 9; ++k) z[(size_t)k * N + c] = v[k];
}

// loss over the interior [3, H-3) x [3, W-3) of every image and the output gradient
// g = P^T(2 (P(y) - T) / count) (zero outside the interior), or without P when project_cell
// is 0; per-block FP64 loss partials
__global__ void k_loss(const float* __restrict__ y, const __nv_bfloat16* __restrict__ T, int nimg, int H, int W,
                       float inv_count, int project_cell, __nv_bfloat16* __restrict__ g, double* __restrict__ part) {
    __shared__ double red[32];
    const size_t total = (size_t)nimg * H * W;
    double acc = 0.0;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % W), r = (int)((c / W) % H);
        unsigned* go = reinterpret_cast<unsigned*>(g + c * 16);
        if (x < 3 || x >= W - 3 || r < 3 || r >= H - 3) {
#pragma unroll
            for (int k = 0; k < 8; ++k) go[k] = 0u;
            continue;
        }
        float v[9];
#pragma unroll
        for (int i = 0; i < 9; ++i) v[i] = y[c * 16 + i];
        if (project_cell) project9(v);
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float e = v[i] - __bfloat162float(T[c * 16 + i]);
            acc += (double)e * (double)e;
            v[i] = 2.0f * e * inv_count;
        }
        if (project_cell) project9_t(v);
#pragma unroll
        for (int k = 0; k < 4; ++k) go[k] = pack_bf16x2(v[2 * k], v[2 * k + 1]);
        go[4] = pack_bf16x2(v[8], 0.0f);
        go[5] = go[6] = go[7] = 0u;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double s = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) s += red[w];
        part[blockIdx.x] = s;
    }
}

// Stress target (LBM_CLOSURE_TARGET_STRESS).  Each application changes a cell's momentum by the
// lattice divergence of the projected outputs, -1/2 sum_i e_i P(y)_i(x - e_i) / s_out
// (k_apply_stress); over a pair's window of n coarse steps with an application every k steps the
// model is m(x) = -factor sum_i e_i P(y)_i(x - e_i) in output units, factor = n / (2 k).
// Pass 1: over the cells [4, H-4) x [4, W-4) of every image the residual r = m - T_j, T_j =
// sum_i e_i T_i the stored momentum target, into res (zero elsewhere), FP64 loss partials.
__global__ void k_stress_residual(const float* __restrict__ z, const __nv_bfloat16* __restrict__ T, int nimg, int H,
                                  int W, float factor, float2* __restrict__ res, double* __restrict__ part) {
    // z: P(y) of every cell as 9 planes (k_project_planes), so each cell is projected once
    __shared__ double red[32];
    const size_t total = (size_t)nimg * H * W;
    double acc = 0.0;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % W), r = (int)((c / W) % H);
        if (x < 4 || x >= W - 4 || r < 4 || r >= H - 4) {
            res[c] = make_float2(0.0f, 0.0f);
            continue;
        }
        float mx = 0.0f, my = 0.0f;
#pragma unroll
        for (int i = 1; i < 9; ++i) {  // P(y) of the source cell x - e_i, its population i
            const long src = (long)c - (long)EY(i) * W - EX(i);
            const float v = z[(size_t)i * total + (size_t)src];
            mx += (float)EX(i) * v;
            my += (float)EY(i) * v;
        }
        float tx = 0.0f, ty = 0.0f;
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const float t = __bfloat162float(T[c * 16 + i]);
            tx += (float)EX(i) * t;
            ty += (float)EY(i) * t;
        }
        const float rx = -factor * mx - tx, ry = -factor * my - ty;
        res[c] = make_float2(rx, ry);
        acc += (double)rx * rx + (double)ry * ry;
    }
    for (int o = 16; o > 0; o >>= 1) acc += __shfl_down_sync(0xffffffffu, acc, o);
    if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = acc;
    __syncthreads();
    if (threadIdx.x == 0) {
        double t = 0.0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t += red[w];
        part[blockIdx.x] = t;
    }
}

// pass 2: the output gradient g(x) = P^T(h), h_i = -factor * 2 inv_count * e_i . r(x + e_i)
// (r zero outside its cells and outside the image), BF16 into g (16 channels)
__global__ void k_stress_grad(const float2* __restrict__ res, int nimg, int H, int W, float factor, float inv_count,
                              __nv_bfloat16* __restrict__ g) {
    const size_t total = (size_t)nimg * H * W;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < total; c += (size_t)gridDim.x * blockDim.x) {
        const int x = (int)(c % W), r = (int)((c / W) % H);
        float h[9];
        h[0] = 0.0f;
#pragma unroll
        for (int i = 1; i < 9; ++i) {
            const int xx = x + EX(i), rr = r + EY(i);
            float2 q = make_float2(0.0f, 0.0f);
            if (xx >= 0 && xx < W && rr >= 0 && rr < H) q = res[(long)c + (long)EY(i) * W + EX(i)];
            h[i] = -factor * 2.0f * inv_count * ((float)EX(i) * q.x + (float)EY(i) * q.y);
        }
        project9_t(h);
        unsigned* go = reinterpret_cast<unsigned*>(g + c * 16);
#pragma unroll
        for (int k = 0; k < 4; ++k) go[k] = pack_bf16x2(h[2 * k], h[2 * k + 1]);
        go[4] = pack_bf16x2(h[8], 0.0f);
        go[5] = go[6] = go[7] = 0u;
    }
}

__global__ void __launch_bounds__(256) k_sum_partials(const double* __restrict__ part, int n, double scale,
                                                      double* __restrict__ out) {
    // 256 threads: strided partial sums, then a fixed tree (deterministic)
    __shared__ double s[256];
    double a = 0.0;
    for (int i = threadIdx.x; i < n; i += 256) a += part[i];
    s[threadIdx.x] = a;
    __syncthreads();
    for (int w = 128; w > 0; w >>= 1) {
        if ((int)threadIdx.x < w) s[threadIdx.x] += s[threadIdx.x + w];
        __syncthreads();
    }
    if (threadIdx.x == 0) out[0] = s[0] * scale;
}

// coarse cell = block average of factor x factor fine cells: rho and momentum averaged,
// populations rebuilt as equilibrium(rho, u) + neq_scale * (average fine f_neq)
__global__ void k_coarsen(const float* __restrict__ df, int nxf, int nyf, int F, float neq_scale,
                          float* __restrict__ dc) {
    const int xc = blockIdx.x * blockDim.x + threadIdx.x, yc = blockIdx.y;
    const int nxc = nxf / F, nyc = nyf / F;
    if (xc >= nxc) return;
    const size_t Nf = (size_t)nxf * nyf, Nc = (size_t)nxc * nyc;
    float neq[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
    float drho = 0.0f, jx = 0.0f, jy = 0.0f;
    for (int dy = 0; dy < F; ++dy)
        for (int dx = 0; dx < F; ++dx) {
            float v[9];
            load_dev(df, Nf, (size_t)(yc * F + dy) * nxf + (xc * F + dx), v);
            float r = 0.0f, a = 0.0f, b = 0.0f;
#pragma unroll
            for (int i = 0; i < 9; ++i) {
                r += v[i];
                a += (float)EX(i) * v[i];
                b += (float)EY(i) * v[i];
            }
            drho += r;
            jx += a;
            jy += b;
            non_equilibrium(v);
#pragma unroll
            for (int i = 0; i < 9; ++i) neq[i] += v[i];
        }
    const float inv = 1.0f / (float)(F * F);
    drho *= inv;
    jx *= inv;
    jy *= inv;
    const float rho = 1.0f + drho, ux = jx / rho, uy = jy / rho;
    const float usq = 1.5f * (ux * ux + uy * uy);
    const size_t c = (size_t)yc * nxc + xc;
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const float eu = (float)EX(i) * ux + (float)EY(i) * uy;
        dc[c + (size_t)i * Nc] = PW<float>(i) * (drho + rho * (3.0f * eu + 4.5f * eu * eu - usq)) + neq_scale * inv * neq[i];
    }
}

__global__ void k_adam(float* __restrict__ p, const float* __restrict__ g, float* __restrict__ m, float* __restrict__ v,
                       const float* __restrict__ mask, int n, float lr, float b1, float b2, float eps, float c1,
                       float c2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] * mask[i];
    const float mi = b1 * m[i] + (1.0f - b1) * gi;
    const float vi = b2 * v[i] + (1.0f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    p[i] = (p[i] - lr * (mi / c1) / (sqrtf(vi / c2) + eps)) * mask[i];
}

// BF16 conv layouts from the FP32 master parameters (forward: [tap][cout][cin];
// backward of layers 3 and 2: taps flipped, channel roles swapped)
__global__ void k_pack(const float* __restrict__ p, __nv_bfloat16* __restrict__ f1, __nv_bfloat16* __restrict__ f2,
                       __nv_bfloat16* __restrict__ f3, __nv_bfloat16* __restrict__ b3, __nv_bfloat16* __restrict__ b2) {
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < 9 * 32 * 16) {  // f1 [tap][co 32][ci 16] <- W1[tap][ci][co]
        const int ci = i % 16, co = (i / 16) % 32, t = i / 512;
        f1[i] = __float2bfloat16_rn(p[OW1 + (t * 16 + ci) * 32 + co]);
    }
    if (i < 9 * 32 * 32) {  // f2 [tap][co][ci] <- W2[tap][ci][co];  b2 [tap'][co'][ci'] <- W2[8-tap'][co'][ci']
        const int ci = i % 32, co = (i / 32) % 32, t = i / 1024;
        f2[i] = __float2bfloat16_rn(p[OW2 + (t * 32 + ci) * 32 + co]);
        b2[i] = __float2bfloat16_rn(p[OW2 + ((8 - t) * 32 + co) * 32 + ci]);
    }
    if (i < 9 * 16 * 32) {  // f3 [tap][co 16][ci 32] <- W3[tap][ci][co]
        const int ci = i % 32, co = (i / 32) % 16, t = i / 512;
        f3[i] = __float2bfloat16_rn(p[OW3 + (t * 32 + ci) * 16 + co]);
    }
    if (i < 9 * 32 * 16) {  // b3 [tap'][co' 32][ci' 16] <- W3[8-tap'][ci = co'][co = ci']
        const int ci = i % 16, co = (i / 16) % 32, t = i / 512;
        b3[i] = __float2bfloat16_rn(p[OW3 + ((8 - t) * 32 + co) * 16 + ci]);
    }
}

#include "lbm_closure_tc.cuh"

}  // namespace closure
}  // namespace lbm

// =====================================================================================
// host side
// =====================================================================================
using lbm::closure::NPARAM;
namespace cl = lbm::closure;

struct lbm_closure {
    int nx = 0, ny = 0;
    float s_in = 1000.0f, s_out = 1000.0f;
    int inputs = LBM_CLOSURE_INPUT_NEQ;
    int target = LBM_CLOSURE_TARGET_POPULATIONS;
    int projection = LBM_CLOSURE_PROJECT_CELL;
    int kernel = LBM_CLOSURE_KERNEL_FUSED;  // inference: one tcgen05 kernel, or the three layer kernels
    float stress_factor = 0.5f;             // stress target: window / (2 x application interval)
    float* bres = nullptr;                  // stress target: residuals of a batch (2 floats per cell)
    float* bz = nullptr;                    // stress target: P(y) of a batch (9 planes)
    float* zp = nullptr;                    // stress target: P(y) of the field, 9 planes
    int* d_status = nullptr;                // LBM_ERR_TIMEOUT from a bounded wait of the fused kernel
    double* dmeans = nullptr;  // reduction partials (RED_BLOCKS x 3) and the 3 field means
    int device = 0;
    cudaStream_t stream = nullptr;
    float *p = nullptr, *g = nullptr, *m = nullptr, *v = nullptr, *mask = nullptr;
    __nv_bfloat16 *wf1 = nullptr, *wf2 = nullptr, *wf3 = nullptr, *wb3 = nullptr, *wb2 = nullptr;
    // full-field inference buffers
    __nv_bfloat16 *x0 = nullptr, *x1 = nullptr, *x2 = nullptr;
    float* y = nullptr;
    // training
    int cap = 0, npairs = 0, crop = 0, batch = 0;
    __nv_bfloat16 *dsx = nullptr, *dst = nullptr;          // dataset features / targets [cap][crop][crop][16]
    __nv_bfloat16 *bx0 = nullptr, *bt = nullptr, *bx1 = nullptr, *bx2 = nullptr, *bg3 = nullptr, *bg2 = nullptr,
                  *bg1 = nullptr;
    float* by = nullptr;
    float* dwpart = nullptr;
    double* lpart = nullptr;
    double* dloss = nullptr;
    uint64_t adam_t = 0;
    uint64_t launches = 0;
};

namespace {

int cfail(int code, const char* fmt, ...) {
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    return lbm::set_error(code, buf);
}

#define C_CK(call)                                                                                    \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return cfail(LBM_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_));  \
    } while (0)
#define C_TRY(expr)            \
    do {                       \
        int r_ = (expr);       \
        if (r_ < 0) return r_; \
    } while (0)

template <class T>
cudaError_t dalloc(T** p, size_t n) {
    return cudaMalloc((void**)p, n * sizeof(T));
}

// logical <-> padded parameter index maps
void logical_to_padded(std::vector<int>& map) {
    map.clear();
    for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < 9; ++ci)
            for (int co = 0; co < 32; ++co) map.push_back(cl::OW1 + (t * 16 + ci) * 32 + co);
    for (int co = 0; co < 32; ++co) map.push_back(cl::OB1 + co);
    for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < 32; ++ci)
            for (int co = 0; co < 32; ++co) map.push_back(cl::OW2 + (t * 32 + ci) * 32 + co);
    for (int co = 0; co < 32; ++co) map.push_back(cl::OB2 + co);
    for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < 32; ++ci)
            for (int co = 0; co < 9; ++co) map.push_back(cl::OW3 + (t * 32 + ci) * 16 + co);
    for (int co = 0; co < 9; ++co) map.push_back(cl::OB3 + co);
}

int pack(lbm_closure* c) {
    cl::k_pack<<<(9 * 32 * 32 + 255) / 256, 256, 0, c->stream>>>(c->p, c->wf1, c->wf2, c->wf3, c->wb3, c->wb2);
    C_CK(cudaGetLastError());
    ++c->launches;
    return LBM_OK;
}

// one 3x3 convolution of nimg images: the training path's (zero padding) on the tcgen05 tensor
// cores with the FUSED kernels, else on the mma.sync layer kernel
template <int CIN, int COUT, int EPI, bool PER>
int conv(lbm_closure* c, const __nv_bfloat16* in, void* out, const __nv_bfloat16* w, const float* bias,
         const __nv_bfloat16* mask, int nimg, int H, int W) {
    if (!PER && c->kernel == LBM_CLOSURE_KERNEL_FUSED) {
        using L = cl::tc::ConvTcLayout<CIN, COUT>;
        static lbm::PerDevice<bool> attr_tc;  // the attribute is set per device (c's device is current)
        bool done_tc = false;
        C_CK(attr_tc.get(
            c->device,
            [](bool& v) {
                v = true;
                return cudaFuncSetAttribute(cl::tc::k_conv_tc<CIN, COUT, EPI>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            L::SMEM);
            },
            &done_tc));
        const dim3 grid((unsigned)((W + 127) / 128), (unsigned)((H + cl::tc::CONV_TC_ROWS - 1) / cl::tc::CONV_TC_ROWS),
                        (unsigned)nimg);
        cl::tc::k_conv_tc<CIN, COUT, EPI><<<grid, cl::tc::CONV_TC_THREADS, L::SMEM, c->stream>>>(in, out, w, bias, mask, H,
                                                                                              W, c->d_status);
        C_CK(cudaGetLastError());
        ++c->launches;
        return LBM_OK;
    }
    constexpr size_t smem = cl::conv_smem_bytes<CIN, COUT>();
    static lbm::PerDevice<bool> attr;  // the attribute is set per device (c's device is current)
    bool done = false;
    C_CK(attr.get(
        c->device,
        [](bool& v) {
            v = true;
            return cudaFuncSetAttribute(cl::k_conv3x3<CIN, COUT, EPI, PER>,
                                        cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        },
        &done));
    const dim3 grid((unsigned)((W + cl::CONV_CELLS - 1) / cl::CONV_CELLS), (unsigned)((H + cl::CONV_ROWS - 1) / cl::CONV_ROWS),
                    (unsigned)nimg);
    cl::k_conv3x3<CIN, COUT, EPI, PER><<<grid, 32 * cl::CONV_WARPS, smem, c->stream>>>(in, out, w, bias, mask, H, W);
    C_CK(cudaGetLastError());
    ++c->launches;
    return LBM_OK;
}

// forward of the whole network on nimg images of H x W (training crops: zero padding;
// inference: periodic)
template <bool PER>
int forward(lbm_closure* c, const __nv_bfloat16* x0, __nv_bfloat16* x1, __nv_bfloat16* x2, float* y, int nimg, int H,
            int W) {
    C_TRY((conv<16, 32, cl::EPI_BIAS_RELU, PER>(c, x0, x1, c->wf1, c->p + cl::OB1, nullptr, nimg, H, W)));
    C_TRY((conv<32, 32, cl::EPI_BIAS_RELU, PER>(c, x1, x2, c->wf2, c->p + cl::OB2, nullptr, nimg, H, W)));
    C_TRY((conv<32, 16, cl::EPI_BIAS_F32, PER>(c, x2, y, c->wf3, c->p + cl::OB3, nullptr, nimg, H, W)));
    return LBM_OK;
}

// weight and bias gradients of one layer: on the tcgen05 tensor cores (FUSED kernels, crops a
// multiple of 64 wide), else on the CUDA cores; both write per-block partial sums that
// k_dweight_final adds in block order
template <int CIN, int COUT, class GT>
int dweight(lbm_closure* c, const __nv_bfloat16* x, const GT* gr, int nimg, int H, int W, float* out) {
    constexpr int threads = 9 * (CIN / 4) * (COUT / 8);
    constexpr int len = 9 * CIN * COUT + COUT;
    int blocks = cl::DW_BLOCKS;
    if (std::is_same<GT, __nv_bfloat16>::value && c->kernel == LBM_CLOSURE_KERNEL_FUSED && W % cl::tc::DW_TILE == 0) {
        using L = cl::tc::DwLayout<CIN, COUT>;
        static lbm::PerDevice<int> sms;  // the attribute is set per device (c's device is current)
        int nsm = 0;
        C_CK(sms.get(
            c->device,
            [&](int& v) {
                cudaError_t e = cudaDeviceGetAttribute(&v, cudaDevAttrMultiProcessorCount, c->device);
                if (e == cudaSuccess)
                    e = cudaFuncSetAttribute(cl::tc::k_dweight_tc<CIN, COUT>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             L::SMEM);
                return e;
            },
            &nsm));
        const int ntiles = nimg * H * (W / cl::tc::DW_TILE);
        blocks = std::min(std::min(nsm, cl::DW_BLOCKS), ntiles);
        cl::tc::k_dweight_tc<CIN, COUT><<<blocks, cl::tc::DW_THREADS, L::SMEM, c->stream>>>(
            x, reinterpret_cast<const __nv_bfloat16*>(gr), nimg, H, W, c->dwpart, c->d_status);
    } else {
        cl::k_dweight<CIN, COUT, GT, false><<<cl::DW_BLOCKS, threads, 0, c->stream>>>(x, gr, nimg, H, W, 0, H, 0, W,
                                                                                       c->dwpart);
    }
    C_CK(cudaGetLastError());
    cl::k_dweight_final<<<(len + 31) / 32, 256, 0, c->stream>>>(c->dwpart, blocks, len, 1.0f, out);
    C_CK(cudaGetLastError());
    c->launches += 2;
    return LBM_OK;
}

// the mean loss of the network outputs c->by against the targets c->bt (nimg crops) into
// c->dloss (device) and the output gradient into c->bg3
int batch_loss(lbm_closure* c, int nimg) {
    const int S = c->crop;
    if (c->target == LBM_CLOSURE_TARGET_STRESS) {
        const double count = (double)nimg * (S - 8) * (S - 8) * 2.0;
        const size_t cells = (size_t)nimg * S * S;
        cl::k_project_planes<<<(unsigned)((cells + 255) / 256), 256, 0, c->stream>>>(c->by, cells, c->bz);
        C_CK(cudaGetLastError());
        cl::k_stress_residual<<<lbm::RED_BLOCKS, 256, 0, c->stream>>>(c->bz, c->bt, nimg, S, S, c->stress_factor,
                                                                        reinterpret_cast<float2*>(c->bres), c->lpart);
        C_CK(cudaGetLastError());
        cl::k_stress_grad<<<lbm::RED_BLOCKS, 256, 0, c->stream>>>(reinterpret_cast<const float2*>(c->bres), nimg, S, S,
                                                                    c->stress_factor, (float)(1.0 / count), c->bg3);
        C_CK(cudaGetLastError());
        cl::k_sum_partials<<<1, 256, 0, c->stream>>>(c->lpart, lbm::RED_BLOCKS, 1.0 / count, c->dloss);
        C_CK(cudaGetLastError());
        c->launches += 4;
        return LBM_OK;
    }
    const double count = (double)nimg * (S - 6) * (S - 6) * 9.0;
    cl::k_loss<<<lbm::RED_BLOCKS, 256, 0, c->stream>>>(c->by, c->bt, nimg, S, S, (float)(1.0 / count),
                                                         c->projection == LBM_CLOSURE_PROJECT_CELL, c->bg3, c->lpart);
    C_CK(cudaGetLastError());
    cl::k_sum_partials<<<1, 256, 0, c->stream>>>(c->lpart, lbm::RED_BLOCKS, 1.0 / count, c->dloss);
    C_CK(cudaGetLastError());
    c->launches += 2;
    return LBM_OK;
}

// gradient of the mean loss of the batch in c->bx0 / c->bt (nimg crops) into c->g;
// loss into c->dloss (device)
int loss_and_grad(lbm_closure* c, int nimg) {
    const int S = c->crop;
    C_TRY(forward<false>(c, c->bx0, c->bx1, c->bx2, c->by, nimg, S, S));
    C_TRY(batch_loss(c, nimg));
    // layer 3: dW3, db3 from x2 and g3; g2 = conv_bwd3(g3) masked by x2 > 0; and so on down
    C_TRY((dweight<32, 16, __nv_bfloat16>(c, c->bx2, c->bg3, nimg, S, S, c->g + cl::OW3)));
    C_TRY((conv<16, 32, cl::EPI_MASK, false>(c, c->bg3, c->bg2, c->wb3, nullptr, c->bx2, nimg, S, S)));
    C_TRY((dweight<32, 32, __nv_bfloat16>(c, c->bx1, c->bg2, nimg, S, S, c->g + cl::OW2)));
    C_TRY((conv<32, 32, cl::EPI_MASK, false>(c, c->bg2, c->bg1, c->wb2, nullptr, c->bx1, nimg, S, S)));
    C_TRY((dweight<16, 32, __nv_bfloat16>(c, c->bx0, c->bg1, nimg, S, S, c->g + cl::OW1)));
    return LBM_OK;
}

int check_closure(const lbm_closure* c) {
    if (!c) return cfail(LBM_ERR_ARG, "null closure");
    return LBM_OK;
}

int check_coarse(const lbm_closure* c, const lbm_handle* h) {
    if (!h) return cfail(LBM_ERR_ARG, "null handle");
    if (h->p.mode != LBM_MODE_PHYSICS || h->p.dtype != LBM_DTYPE_F32)
        return cfail(LBM_ERR_ARG, "the closure works on physics-mode FP32 lattices");
    if (c && (h->nx != c->nx || h->ny != c->ny))
        return cfail(LBM_ERR_ARG, "lattice %dx%d does not match the closure's %dx%d", h->nx, h->ny, c->nx, c->ny);
    return LBM_OK;
}

}  // namespace

extern "C" {

int lbm_closure_destroy(lbm_closure* c);

int lbm_closure_param_count(void) { return cl::NLOGICAL; }

int lbm_closure_create(int32_t nx, int32_t ny, uint64_t seed, lbm_closure** out) {
    if (!out) return cfail(LBM_ERR_ARG, "null output");
    *out = nullptr;
    if (nx < 16 || ny < 3 || nx % 16 != 0 || nx > 65535 || ny > 65535)
        return cfail(LBM_ERR_ARG, "closure lattice %dx%d: nx must be a multiple of 16", nx, ny);
    lbm_closure* c = new (std::nothrow) lbm_closure();
    if (!c) return cfail(LBM_ERR_NOMEM, "out of host memory");
    c->nx = nx;
    c->ny = ny;
    const size_t N = (size_t)nx * ny;
    cudaError_t e = cudaGetDevice(&c->device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = dalloc(&c->p, NPARAM);
    if (e == cudaSuccess) e = dalloc(&c->g, NPARAM);
    if (e == cudaSuccess) e = dalloc(&c->m, NPARAM);
    if (e == cudaSuccess) e = dalloc(&c->v, NPARAM);
    if (e == cudaSuccess) e = dalloc(&c->mask, NPARAM);
    if (e == cudaSuccess) e = dalloc(&c->wf1, 9 * 32 * 16);
    if (e == cudaSuccess) e = dalloc(&c->wf2, 9 * 32 * 32);
    if (e == cudaSuccess) e = dalloc(&c->wf3, 9 * 16 * 32);
    if (e == cudaSuccess) e = dalloc(&c->wb3, 9 * 32 * 16);
    if (e == cudaSuccess) e = dalloc(&c->wb2, 9 * 32 * 32);
    if (e == cudaSuccess) e = dalloc(&c->x0, N * 16);
    if (e == cudaSuccess) e = dalloc(&c->x1, N * 32);
    if (e == cudaSuccess) e = dalloc(&c->x2, N * 32);
    if (e == cudaSuccess) e = dalloc(&c->y, N * 16);
    if (e == cudaSuccess) e = dalloc(&c->lpart, lbm::RED_BLOCKS);
    if (e == cudaSuccess) e = dalloc(&c->dmeans, (size_t)lbm::RED_BLOCKS * 3 + 3);
    if (e == cudaSuccess) e = dalloc(&c->dloss, 8);
    if (e == cudaSuccess) e = dalloc(&c->dwpart, (size_t)cl::DW_BLOCKS * (9 * 32 * 32 + 32));
    if (e == cudaSuccess) e = dalloc(&c->d_status, 1);
    if (e == cudaSuccess) e = dalloc(&c->zp, N * 9);
    if (e == cudaSuccess) e = cudaMemset(c->d_status, 0, sizeof(int));
    if (e != cudaSuccess) {
        lbm_closure_destroy(c);
        return cfail(LBM_ERR_CUDA, "closure allocation: %s", cudaGetErrorString(e));
    }
    // He-normal initialisation (seeded); the last layer starts small so the initial
    // correction is close to zero
    std::mt19937_64 rng(seed);
    std::normal_distribution<float> nd(0.0f, 1.0f);
    std::vector<float> hp(NPARAM, 0.0f), hm(NPARAM, 0.0f);
    std::vector<int> map;
    logical_to_padded(map);
    for (int k = 0; k < cl::NLOGICAL; ++k) hm[map[k]] = 1.0f;
    for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < 9; ++ci)
            for (int co = 0; co < 32; ++co) hp[cl::OW1 + (t * 16 + ci) * 32 + co] = nd(rng) * std::sqrt(2.0f / 81.0f);
    for (int k = 0; k < cl::NW2; ++k) hp[cl::OW2 + k] = nd(rng) * std::sqrt(2.0f / 288.0f);
    for (int t = 0; t < 9; ++t)
        for (int ci = 0; ci < 32; ++ci)
            for (int co = 0; co < 9; ++co) hp[cl::OW3 + (t * 32 + ci) * 16 + co] = nd(rng) * 0.1f * std::sqrt(1.0f / 288.0f);
    e = cudaMemcpy(c->p, hp.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemcpy(c->mask, hm.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice);
    if (e == cudaSuccess) e = cudaMemset(c->m, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(c->v, 0, NPARAM * sizeof(float));
    if (e == cudaSuccess) e = cudaMemset(c->g, 0, NPARAM * sizeof(float));
    int r = e == cudaSuccess ? pack(c) : cfail(LBM_ERR_CUDA, "closure init: %s", cudaGetErrorString(e));
    if (r == LBM_OK && cudaStreamSynchronize(c->stream) != cudaSuccess) r = cfail(LBM_ERR_CUDA, "closure init sync");
    if (r != LBM_OK) {
        lbm_closure_destroy(c);
        return r;
    }
    *out = c;
    return LBM_OK;
}

int lbm_closure_destroy(lbm_closure* c) {
    if (!c) return LBM_OK;
    cudaSetDevice(c->device);
    if (c->stream) cudaStreamSynchronize(c->stream);
    void* bufs[] = {c->p,  c->g,  c->m,   c->v,   c->mask, c->wf1, c->wf2, c->wf3, c->wb3, c->wb2, c->x0,
                    c->x1, c->x2, c->y,   c->dsx, c->dst,  c->bx0, c->bt,  c->bx1, c->bx2, c->bg3, c->bg2,
                    c->bg1, c->by, c->dwpart, c->lpart, c->dloss, c->dmeans, c->d_status, c->bres, c->bz, c->zp};
    for (void* b : bufs) cudaFree(b);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
    return LBM_OK;
}

int lbm_closure_set_scales(lbm_closure* c, float s_in, float s_out) {
    C_TRY(check_closure(c));
    if (!(s_in > 0.0f) || !(s_out > 0.0f)) return cfail(LBM_ERR_ARG, "scales must be positive");
    c->s_in = s_in;
    c->s_out = s_out;
    return LBM_OK;
}

int lbm_closure_set_form(lbm_closure* c, int32_t inputs, int32_t target, int32_t projection) {
    C_TRY(check_closure(c));
    if (inputs != LBM_CLOSURE_INPUT_NEQ && inputs != LBM_CLOSURE_INPUT_EQ)
        return cfail(LBM_ERR_ARG, "unknown closure input mode %d", inputs);
    if (target != LBM_CLOSURE_TARGET_POPULATIONS && target != LBM_CLOSURE_TARGET_EQUILIBRIUM &&
        target != LBM_CLOSURE_TARGET_MOMENTUM && target != LBM_CLOSURE_TARGET_STRESS)
        return cfail(LBM_ERR_ARG, "unknown closure target %d", target);
    if (target == LBM_CLOSURE_TARGET_STRESS && projection != LBM_CLOSURE_PROJECT_CELL)
        return cfail(LBM_ERR_ARG, "the stress target acts through the per-cell projection");
    if (projection != LBM_CLOSURE_PROJECT_CELL && projection != LBM_CLOSURE_PROJECT_DOMAIN)
        return cfail(LBM_ERR_ARG, "unknown closure projection %d", projection);
    if (target == LBM_CLOSURE_TARGET_MOMENTUM && projection == LBM_CLOSURE_PROJECT_CELL)
        return cfail(LBM_ERR_ARG, "the per-cell projection removes a momentum target entirely");
    c->inputs = inputs;
    c->target = target;
    c->projection = projection;
    return LBM_OK;
}

int lbm_closure_set_stress_factor(lbm_closure* c, float factor) {
    C_TRY(check_closure(c));
    if (!(factor > 0.0f) || !std::isfinite(factor)) return cfail(LBM_ERR_ARG, "the stress factor must be positive");
    c->stress_factor = factor;
    return LBM_OK;
}

int lbm_closure_get_params(lbm_closure* c, float* out) {
    C_TRY(check_closure(c));
    if (!out) return cfail(LBM_ERR_ARG, "null output");
    std::vector<float> hp(NPARAM);
    C_CK(cudaStreamSynchronize(c->stream));
    C_CK(cudaMemcpy(hp.data(), c->p, NPARAM * sizeof(float), cudaMemcpyDeviceToHost));
    std::vector<int> map;
    logical_to_padded(map);
    for (int k = 0; k < cl::NLOGICAL; ++k) out[k] = hp[map[k]];
    return LBM_OK;
}

int lbm_closure_set_params(lbm_closure* c, const float* in) {
    C_TRY(check_closure(c));
    if (!in) return cfail(LBM_ERR_ARG, "null input");
    std::vector<float> hp(NPARAM, 0.0f);
    std::vector<int> map;
    logical_to_padded(map);
    for (int k = 0; k < cl::NLOGICAL; ++k) hp[map[k]] = in[k];
    C_CK(cudaStreamSynchronize(c->stream));
    C_CK(cudaMemcpy(c->p, hp.data(), NPARAM * sizeof(float), cudaMemcpyHostToDevice));
    C_TRY(pack(c));
    C_CK(cudaStreamSynchronize(c->stream));
    return LBM_OK;
}

int lbm_coarsen(lbm_handle* fine, lbm_handle* coarse, int32_t factor, float neq_scale) {
    LbmRange range_("lbm_coarsen");
    if (!fine || !coarse) return cfail(LBM_ERR_ARG, "null handle");
    C_TRY(check_coarse(nullptr, fine));
    C_TRY(check_coarse(nullptr, coarse));
    if (factor < 1 || fine->nx != coarse->nx * factor || fine->ny != coarse->ny * factor)
        return cfail(LBM_ERR_ARG, "fine %dx%d is not %d x coarse %dx%d", fine->nx, fine->ny, factor, coarse->nx,
                     coarse->ny);
    C_CK(cudaSetDevice(coarse->device));
    C_CK(cudaStreamSynchronize(fine->stream));
    const dim3 grid((unsigned)((coarse->nx + 127) / 128), (unsigned)coarse->ny);
    cl::k_coarsen<<<grid, 128, 0, coarse->stream>>>((const float*)fine->buf[fine->cur], fine->nx, fine->ny, factor,
                                                    neq_scale, (float*)coarse->buf[coarse->cur]);
    C_CK(cudaGetLastError());
    coarse->launches += 1;
    C_CK(cudaStreamSynchronize(coarse->stream));
    return LBM_OK;
}

}  // extern "C"

namespace {

// features, forward and the projected correction of the whole lattice h on h's stream:
// added to h's populations (accumulate) or written to the 9 planes at out
int correction(lbm_closure* c, lbm_handle* h, float* out, int accumulate) {
    cudaStream_t s = h->stream;
    cudaStream_t keep = c->stream;
    c->stream = s;  // run on the lattice's stream
    const dim3 g1((unsigned)((c->nx + 127) / 128), (unsigned)c->ny);
    cudaError_t e = cudaSuccess;
    int r = LBM_OK;
    if (c->kernel == LBM_CLOSURE_KERNEL_FUSED) {
        // features and the three layers in one tcgen05 kernel (its shared-memory attribute is
        // set per device)
        static lbm::PerDevice<bool> attr;
        bool done = false;
        e = attr.get(
            c->device,
            [](bool& v) {
                v = true;
                return cudaFuncSetAttribute(cl::tc::k_closure_fused, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                            cl::tc::SMEM_BYTES);
            },
            &done);
        // applying a per-cell projected correction needs no field reduction: the kernel adds it
        // itself and writes the corrected state into the lattice's other buffer
        const bool in_kernel = accumulate && out == (float*)h->buf[h->cur] &&
                               c->projection == LBM_CLOSURE_PROJECT_CELL && c->target != LBM_CLOSURE_TARGET_STRESS;
        if (e == cudaSuccess) {
            const dim3 grid((unsigned)((c->nx + cl::tc::OUT_W - 1) / cl::tc::OUT_W),
                            (unsigned)((c->ny + cl::tc::TC_ROWS - 1) / cl::tc::TC_ROWS));
            cl::tc::k_closure_fused<<<grid, cl::tc::TC_THREADS, cl::tc::SMEM_BYTES, s>>>(
                (const float*)h->buf[h->cur], c->nx, c->ny, c->s_in, c->inputs, c->wf1, c->wf2, c->wf3, c->p + cl::OB1,
                c->p + cl::OB2, c->p + cl::OB3, c->y, in_kernel ? (float*)h->buf[h->cur ^ 1] : nullptr,
                1.0f / c->s_out, c->target == LBM_CLOSURE_TARGET_STRESS ? c->zp : nullptr, c->d_status);
            e = cudaGetLastError();
            ++c->launches;
        }
        if (e != cudaSuccess) {
            r = cfail(LBM_ERR_CUDA, "fused closure kernel: %s", cudaGetErrorString(e));
        } else if (in_kernel) {
            h->cur ^= 1;  // the corrected state is the one the next step reads
            c->stream = keep;
            return LBM_OK;
        }
    } else {
        cl::k_features<<<g1, 128, 0, s>>>((const float*)h->buf[h->cur], c->nx, c->ny, 0, 0, c->ny, c->nx, c->s_in,
                                          c->inputs, c->x0);
        e = cudaGetLastError();
        r = e == cudaSuccess ? forward<true>(c, c->x0, c->x1, c->x2, c->y, 1, c->ny, c->nx)
                             : cfail(LBM_ERR_CUDA, "features: %s", cudaGetErrorString(e));
    }
    const double* means = nullptr;
    if (r == LBM_OK && c->projection == LBM_CLOSURE_PROJECT_DOMAIN) {
        const size_t N = (size_t)c->nx * c->ny;
        cl::k_ysums<<<lbm::RED_BLOCKS, 256, 0, s>>>(c->y, N, c->dmeans);
        cl::k_ymeans<<<1, 32, 0, s>>>(c->dmeans, lbm::RED_BLOCKS, 1.0 / (double)N, c->dmeans + 3 * lbm::RED_BLOCKS);
        means = c->dmeans + 3 * lbm::RED_BLOCKS;
        c->launches += 2;
        e = cudaGetLastError();
        if (e != cudaSuccess) r = cfail(LBM_ERR_CUDA, "field means: %s", cudaGetErrorString(e));
    }
    if (r == LBM_OK && c->target == LBM_CLOSURE_TARGET_STRESS) {
        if (c->kernel != LBM_CLOSURE_KERNEL_FUSED) {  // the fused kernel writes the planes itself
            const size_t N = (size_t)c->nx * c->ny;
            cl::k_project_planes<<<(unsigned)((N + 255) / 256), 256, 0, s>>>(c->y, N, c->zp);
            ++c->launches;
        }
        cl::k_apply_stress<<<g1, 128, 0, s>>>(c->zp, out, c->nx, c->ny, 1.0f / c->s_out, accumulate);
        e = cudaGetLastError();
        if (e != cudaSuccess) r = cfail(LBM_ERR_CUDA, "apply: %s", cudaGetErrorString(e));
    } else if (r == LBM_OK) {
        cl::k_apply<<<g1, 128, 0, s>>>(c->y, out, c->nx, c->ny, 1.0f / c->s_out, means, accumulate);
        e = cudaGetLastError();
        if (e != cudaSuccess) r = cfail(LBM_ERR_CUDA, "apply: %s", cudaGetErrorString(e));
    }
    c->stream = keep;
    c->launches += 2;
    return r;
}

}  // namespace

extern "C" {

int lbm_closure_apply(lbm_closure* c, lbm_handle* h) {
    LbmRange range_("lbm_closure_apply");
    C_TRY(check_closure(c));
    C_TRY(check_coarse(c, h));
    C_CK(cudaSetDevice(c->device));
    const int r = correction(c, h, (float*)h->buf[h->cur], 1);
    if (c->kernel == LBM_CLOSURE_KERNEL_FUSED)  // one kernel, plus the field means and the apply pass
        h->launches += c->projection == LBM_CLOSURE_PROJECT_DOMAIN ? 4 : (c->target == LBM_CLOSURE_TARGET_STRESS ? 2 : 1);
    else
        h->launches += 4 + (c->projection == LBM_CLOSURE_PROJECT_DOMAIN ? 3 : (c->target == LBM_CLOSURE_TARGET_STRESS ? 2 : 1));
    return r;
}

int lbm_closure_set_kernel(lbm_closure* c, int32_t kernel) {
    C_TRY(check_closure(c));
    if (kernel != LBM_CLOSURE_KERNEL_FUSED && kernel != LBM_CLOSURE_KERNEL_LAYERS)
        return cfail(LBM_ERR_ARG, "unknown closure kernel %d", kernel);
    c->kernel = kernel;
    return LBM_OK;
}

int lbm_closure_status(lbm_closure* c) {
    C_TRY(check_closure(c));
    C_CK(cudaSetDevice(c->device));
    C_CK(cudaDeviceSynchronize());
    int st = 0;
    C_CK(cudaMemcpy(&st, c->d_status, sizeof(int), cudaMemcpyDeviceToHost));
    if (st != 0) return cfail(st, "the fused closure kernel gave up on a bounded wait");
    return LBM_OK;
}

int lbm_closure_reserve(lbm_closure* c, int32_t max_pairs, int32_t crop, int32_t batch) {
    C_TRY(check_closure(c));
    if (max_pairs < 1 || crop < 16 || crop % 16 != 0 || batch < 1 || batch > max_pairs)
        return cfail(LBM_ERR_ARG, "need max_pairs >= batch >= 1 and crop a multiple of 16");
    C_CK(cudaSetDevice(c->device));
    C_CK(cudaStreamSynchronize(c->stream));
    __nv_bfloat16** bufs[] = {&c->dsx, &c->dst, &c->bx0, &c->bt, &c->bx1, &c->bx2, &c->bg3, &c->bg2, &c->bg1};
    for (auto b : bufs) {
        cudaFree(*b);
        *b = nullptr;
    }
    cudaFree(c->by);
    c->by = nullptr;
    cudaFree(c->bres);
    c->bres = nullptr;
    cudaFree(c->bz);
    c->bz = nullptr;
    const size_t cs = (size_t)crop * crop;
    C_CK(dalloc(&c->dsx, (size_t)max_pairs * cs * 16));
    C_CK(dalloc(&c->dst, (size_t)max_pairs * cs * 16));
    C_CK(dalloc(&c->bx0, (size_t)batch * cs * 16));
    C_CK(dalloc(&c->bt, (size_t)batch * cs * 16));
    C_CK(dalloc(&c->bx1, (size_t)batch * cs * 32));
    C_CK(dalloc(&c->bx2, (size_t)batch * cs * 32));
    C_CK(dalloc(&c->bg3, (size_t)batch * cs * 16));
    C_CK(dalloc(&c->bg2, (size_t)batch * cs * 32));
    C_CK(dalloc(&c->bg1, (size_t)batch * cs * 32));
    C_CK(dalloc(&c->by, (size_t)batch * cs * 16));
    C_CK(dalloc(&c->bres, (size_t)batch * cs * 2));
    C_CK(dalloc(&c->bz, (size_t)batch * cs * 9));
    c->cap = max_pairs;
    c->crop = crop;
    c->batch = batch;
    c->npairs = 0;
    return LBM_OK;
}

int lbm_closure_add_pair(lbm_closure* c, lbm_handle* pred, lbm_handle* target, int32_t ox, int32_t oy) {
    LbmRange range_("lbm_closure_add_pair");
    C_TRY(check_closure(c));
    C_TRY(check_coarse(nullptr, pred));
    C_TRY(check_coarse(nullptr, target));
    if (pred->nx != target->nx || pred->ny != target->ny) return cfail(LBM_ERR_ARG, "pred and target sizes differ");
    if (c->npairs >= c->cap) return cfail(LBM_ERR_STATE, "dataset full (%d pairs)", c->cap);
    if (c->crop > pred->nx || c->crop > pred->ny) return cfail(LBM_ERR_ARG, "crop larger than the lattice");
    C_CK(cudaSetDevice(c->device));
    C_CK(cudaStreamSynchronize(pred->stream));
    C_CK(cudaStreamSynchronize(target->stream));
    const int S = c->crop;
    const size_t off = (size_t)c->npairs * S * S * 16;
    const dim3 g((unsigned)((S + 127) / 128), (unsigned)S);
    const int x = ((ox % pred->nx) + pred->nx) % pred->nx, y = ((oy % pred->ny) + pred->ny) % pred->ny;
    cl::k_features<<<g, 128, 0, c->stream>>>((const float*)pred->buf[pred->cur], pred->nx, pred->ny, x, y, S, S,
                                             c->s_in, c->inputs, c->dsx + off);
    cl::k_target<<<g, 128, 0, c->stream>>>((const float*)target->buf[target->cur], (const float*)pred->buf[pred->cur],
                                           pred->nx, pred->ny, x, y, S, S, c->s_out,
                                           c->target == LBM_CLOSURE_TARGET_STRESS ? LBM_CLOSURE_TARGET_MOMENTUM
                                                                                  : c->target,
                                           c->projection == LBM_CLOSURE_PROJECT_CELL &&
                                               c->target != LBM_CLOSURE_TARGET_STRESS,
                                           c->dst + off);
    C_CK(cudaGetLastError());
    c->launches += 2;
    ++c->npairs;
    return LBM_OK;
}

int lbm_closure_pairs(const lbm_closure* c, int32_t* n) {
    C_TRY(check_closure(c));
    if (n) *n = c->npairs;
    return LBM_OK;
}

// Adam on random batches of stored pairs; loss_out (may be NULL) receives the mean loss of
// the last iteration
int lbm_closure_train(lbm_closure* c, int32_t iters, float lr, uint64_t seed, double* loss_out) {
    LbmRange range_("lbm_closure_train");
    C_TRY(check_closure(c));
    if (c->npairs < 1) return cfail(LBM_ERR_STATE, "no training pairs");
    if (iters < 0 || !(lr > 0.0f)) return cfail(LBM_ERR_ARG, "bad iteration count or learning rate");
    C_CK(cudaSetDevice(c->device));
    std::mt19937_64 rng(seed);
    const int S = c->crop, B = std::min(c->batch, c->npairs);
    const size_t img = (size_t)S * S * 16;
    for (int it = 0; it < iters; ++it) {
        for (int b = 0; b < B; ++b) {
            const int k = (int)(rng() % (uint64_t)c->npairs);
            C_CK(cudaMemcpyAsync(c->bx0 + b * img, c->dsx + k * img, img * 2, cudaMemcpyDeviceToDevice, c->stream));
            C_CK(cudaMemcpyAsync(c->bt + b * img, c->dst + k * img, img * 2, cudaMemcpyDeviceToDevice, c->stream));
        }
        C_TRY(loss_and_grad(c, B));
        ++c->adam_t;
        const float b1 = 0.9f, b2 = 0.999f;
        const float c1 = 1.0f - std::pow(b1, (float)c->adam_t), c2 = 1.0f - std::pow(b2, (float)c->adam_t);
        cl::k_adam<<<(NPARAM + 255) / 256, 256, 0, c->stream>>>(c->p, c->g, c->m, c->v, c->mask, NPARAM, lr, b1, b2,
                                                                 1e-8f, c1, c2);
        C_CK(cudaGetLastError());
        C_TRY(pack(c));
        c->launches += 1;
    }
    if (loss_out) {
        C_CK(cudaMemcpyAsync(loss_out, c->dloss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    }
    C_CK(cudaStreamSynchronize(c->stream));
    return LBM_OK;
}

// mean loss over stored pairs [begin, end) without updating the parameters
int lbm_closure_eval(lbm_closure* c, int32_t begin, int32_t end, double* loss_out) {
    C_TRY(check_closure(c));
    if (begin < 0 || end > c->npairs || begin >= end || !loss_out) return cfail(LBM_ERR_ARG, "bad pair range");
    C_CK(cudaSetDevice(c->device));
    const int S = c->crop;
    const size_t img = (size_t)S * S * 16;
    double total = 0.0;
    int n = 0;
    for (int k0 = begin; k0 < end; k0 += c->batch) {
        const int B = std::min(c->batch, end - k0);
        C_CK(cudaMemcpyAsync(c->bx0, c->dsx + k0 * img, B * img * 2, cudaMemcpyDeviceToDevice, c->stream));
        C_CK(cudaMemcpyAsync(c->bt, c->dst + k0 * img, B * img * 2, cudaMemcpyDeviceToDevice, c->stream));
        C_TRY(forward<false>(c, c->bx0, c->bx1, c->bx2, c->by, B, S, S));
        C_TRY(batch_loss(c, B));
        double l = 0.0;
        C_CK(cudaMemcpyAsync(&l, c->dloss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
        C_CK(cudaStreamSynchronize(c->stream));
        total += l * B;
        n += B;
    }
    *loss_out = total / n;
    return LBM_OK;
}

// forward + backward on host-provided crops (for gradient checks): feats and targets are
// [nimg][size][size][9] floats in feature / output units; grads receives the logical
// gradient vector (lbm_closure_param_count() floats), loss the mean loss
int lbm_closure_loss_grad(lbm_closure* c, int32_t nimg, int32_t size, const float* feats, const float* targets,
                          double* loss, float* grads) {
    C_TRY(check_closure(c));
    if (!feats || !targets || nimg < 1 || size != c->crop || nimg > c->batch)
        return cfail(LBM_ERR_ARG, "crops must match the reserved crop size and batch");
    C_CK(cudaSetDevice(c->device));
    const size_t cells = (size_t)nimg * size * size;
    std::vector<__nv_bfloat16> hx(cells * 16), ht(cells * 16);
    for (size_t i = 0; i < cells; ++i)
        for (int k = 0; k < 16; ++k) {
            hx[i * 16 + k] = __float2bfloat16_rn(k < 9 ? feats[i * 9 + k] : 0.0f);
            ht[i * 16 + k] = __float2bfloat16_rn(k < 9 ? targets[i * 9 + k] : 0.0f);
        }
    C_CK(cudaMemcpyAsync(c->bx0, hx.data(), cells * 32, cudaMemcpyHostToDevice, c->stream));
    C_CK(cudaMemcpyAsync(c->bt, ht.data(), cells * 32, cudaMemcpyHostToDevice, c->stream));
    C_TRY(loss_and_grad(c, nimg));
    std::vector<float> hg(NPARAM);
    C_CK(cudaMemcpyAsync(hg.data(), c->g, NPARAM * sizeof(float), cudaMemcpyDeviceToHost, c->stream));
    if (loss) C_CK(cudaMemcpyAsync(loss, c->dloss, sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    C_CK(cudaStreamSynchronize(c->stream));
    if (grads) {
        std::vector<int> map;
        logical_to_padded(map);
        for (int k = 0; k < cl::NLOGICAL; ++k) grads[k] = hg[map[k]];
    }
    return LBM_OK;
}

// the correction delta (9 planes of nx * ny floats) the closure would add to the whole
// lattice h, without applying it (inspection and tests)
int lbm_closure_predict(lbm_closure* c, lbm_handle* h, float* delta_out) {
    LbmRange range_("lbm_closure_predict");
    C_TRY(check_closure(c));
    C_TRY(check_coarse(c, h));
    if (!delta_out) return cfail(LBM_ERR_ARG, "null output");
    C_CK(cudaSetDevice(c->device));
    const size_t N = (size_t)c->nx * c->ny;
    float* d = nullptr;
    C_CK(cudaMalloc((void**)&d, 9 * N * sizeof(float)));
    int r = correction(c, h, d, 0);
    if (r == LBM_OK) {
        cudaError_t e = cudaMemcpyAsync(delta_out, d, 9 * N * sizeof(float), cudaMemcpyDeviceToHost, h->stream);
        if (e == cudaSuccess) e = cudaStreamSynchronize(h->stream);
        if (e != cudaSuccess) r = cfail(LBM_ERR_CUDA, "predict: %s", cudaGetErrorString(e));
    }
    cudaStreamSynchronize(h->stream);
    cudaFree(d);
    return r;
}

int lbm_closure_counters(const lbm_closure* c, uint64_t* launches, uint64_t* adam_steps) {
    C_TRY(check_closure(c));
    if (launches) *launches = c->launches;
    if (adam_steps) *adam_steps = c->adam_t;
    return LBM_OK;
}

}  // extern "C"
