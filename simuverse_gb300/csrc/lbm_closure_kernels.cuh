// lbm_closure_kernels.cuh -- kernels of the learned closure for a coarsened lattice.
//
// Network: x0 (9 features, stored as 16 channels) -> conv3x3 16->32 + bias, ReLU -> x1
//          -> conv3x3 32->32 + bias, ReLU -> x2 -> conv3x3 32->9 (stored as 16) + bias -> y.
// Activations are BF16 in NHWC order ([image][row][column][channel]); accumulation is FP32.
// The convolutions are implicit GEMMs on the tensor cores with mma.sync.m16n8k16 (BF16 in,
// FP32 accumulate), fragments loaded with ldmatrix: a warp owns 16 consecutive cells of one
// row (GEMM rows) times all output channels (GEMM columns); K runs over the 9 taps x input
// channels.  The block stages the 3
// input rows it needs (64 + 2 cells each) and all weights in shared memory with a padded
// per-cell stride of (C/2 + 4) words, which makes every fragment load bank-conflict free.
//
// Weight layout for the conv kernel: BF16 [tap][cout][cin] (cin contiguous), tap = 3 (dy+1) +
// (dx+1).  The input-gradient pass of a layer is the same kernel run on the output gradient
// with the taps flipped (tap -> 8 - tap) and the channel roles swapped.
#pragma once

#include <cuda_bf16.h>
#include <stdint.h>

#include "lbm_common.cuh"

namespace lbm {
namespace closure {

constexpr int CONV_WARPS = 4;
constexpr int CONV_CELLS = 16 * CONV_WARPS;  // cells of one row per block
constexpr int CONV_ROWS = 8;                 // output rows per block (weights staged once)

enum { EPI_BIAS_RELU = 0, EPI_BIAS_F32 = 1, EPI_MASK = 2 };

__device__ __forceinline__ void mma_bf16_16816(float (&d)[4], unsigned a0, unsigned a1, unsigned a2, unsigned a3,
                                               unsigned b0, unsigned b1) {
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a0), "r"(a1), "r"(a2), "r"(a3), "r"(b0), "r"(b1));
}

// four 8x8 b16 matrices from shared memory, one row address per thread (threads 8i .. 8i+7
// address the rows of matrix i); thread t receives row t/4, columns 2(t%4), 2(t%4)+1 of each
__device__ __forceinline__ void ldsm_x4(unsigned (&r)[4], const unsigned* row) {
    const unsigned a = (unsigned)__cvta_generic_to_shared(row);
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(a));
}

// 16-byte global -> shared copy that bypasses the registers (cp.async); with full == false the
// destination is zero-filled and nothing is read
__device__ __forceinline__ void cp_async16(unsigned* dst, const void* src, bool full) {
    const unsigned d = (unsigned)__cvta_generic_to_shared(dst);
    const int n = full ? 16 : 0;
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;" ::"r"(d), "l"(src), "r"(n) : "memory");
}
__device__ __forceinline__ void cp_async_wait_all() {
    asm volatile("cp.async.commit_group;\n\tcp.async.wait_group 0;" ::: "memory");
}

__device__ __forceinline__ unsigned pack_bf16x2(float lo, float hi) {
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);
    return *reinterpret_cast<const unsigned*>(&v);
}

template <int C>
struct SmemStride {
    static constexpr int WORDS = C / 2 + 4;  // 32-bit words per cell (padding breaks bank conflicts)
};

// One 3x3 convolution.  in: [nimg][H][W][CIN] bf16, out: [nimg][H][W][COUT] (bf16, or f32
// for EPI_BIAS_F32), wk: [9][COUT][CIN] bf16, bias: [COUT] f32 (unused for EPI_MASK),
// mask: [nimg][H][W][COUT] bf16 (EPI_MASK only: out = acc where mask > 0, else 0).
// PERIODIC: coordinates wrap; otherwise cells outside the image read as zero.
// A block computes CONV_ROWS rows of 64 cells: it stages the weights and the CONV_ROWS + 2
// input rows once, then each warp runs its 16 cells down the rows.
// Requires W % 16 == 0.  Grid: (ceil(W / 64), ceil(H / CONV_ROWS), nimg), 128 threads.
template <int CIN, int COUT, int EPI, bool PERIODIC>
__global__ void __launch_bounds__(32 * CONV_WARPS) k_conv3x3(const __nv_bfloat16* __restrict__ in,
                                                             void* __restrict__ out,
                                                             const __nv_bfloat16* __restrict__ wk,
                                                             const float* __restrict__ bias,
                                                             const __nv_bfloat16* __restrict__ mask, int H, int W) {
    constexpr int CS = SmemStride<CIN>::WORDS;
    constexpr int ROWC = CONV_CELLS + 2;
    constexpr int SR = CONV_ROWS + 2;  // staged input rows
    constexpr int NT = COUT / 8;
    extern __shared__ __align__(16) unsigned csm[];
    unsigned* sin = csm;                     // [SR][ROWC][CS]
    unsigned* sw = csm + SR * ROWC * CS;     // [9][COUT][CS]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    const int img = blockIdx.z, y0 = blockIdx.y * CONV_ROWS, xs = blockIdx.x * CONV_CELLS;
    const size_t img_off = (size_t)img * H * W;

    // stage the input rows y0-1..y0+CONV_ROWS, columns xs-1 .. xs+64 (16-byte vectors)
    constexpr int VPC = CIN / 8;  // 16-byte vectors per cell
    for (int i = tid; i < SR * ROWC * VPC; i += 32 * CONV_WARPS) {
        const int v = i % VPC, cell = (i / VPC) % ROWC, r = i / (VPC * ROWC);
        int gy = y0 + r - 1, gx = xs + cell - 1;
        bool ok = true;
        if (PERIODIC) {  // staged rows run from -1 to H + CONV_ROWS, which may exceed 2 H
            gy = ((gy % H) + H) % H;
            gx = gx < 0 ? gx + W : (gx >= W ? gx - W : gx);
        } else {
            ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
        }
        // asynchronous 16-byte copy; a cell outside the image is filled with zeros (source size 0)
        const __nv_bfloat16* src = ok ? in + (img_off + (size_t)gy * W + gx) * CIN + v * 8 : in;
        cp_async16(sin + (r * ROWC + cell) * CS + v * 4, src, ok);
    }
    // stage the weights
    for (int i = tid; i < 9 * COUT * VPC; i += 32 * CONV_WARPS) {
        const int v = i % VPC, row = i / VPC;  // row = tap * COUT + co
        cp_async16(sw + row * CS + v * 4, wk + (size_t)row * CIN + v * 8, true);
    }
    cp_async_wait_all();
    __syncthreads();

    const int x0 = xs + warp * 16;
    if (x0 >= W) return;
    const int g = lane >> 2, c = lane & 3;
    // ldmatrix row addresses: A (cells x channels): matrix m = lane / 8 holds cells 8 (m % 2) ..
    // +7 and channels 8 (m / 2) .. +7 of the 16 x 16 k-chunk; B (out x in channels): matrices
    // (n-tile 2p, k lo), (2p, k hi), (2p + 1, k lo), (2p + 1, k hi)
    const int mi = lane >> 3, rr = lane & 7;
    const int a_cell = warp * 16 + rr + 8 * (mi & 1), a_k = 4 * (mi >> 1);
    const int b_row = rr + 8 * (mi >> 1), b_k = 4 * (mi & 1);
    // two output rows at a time: the weight fragments serve both, and the two accumulator
    // sets are independent chains of mma
#pragma unroll 1
    for (int r = 0; r < CONV_ROWS; r += 2) {
        if (y0 + r >= H) break;
        float acc[2][NT][4];
#pragma unroll
        for (int q = 0; q < 2; ++q)
#pragma unroll
            for (int n = 0; n < NT; ++n) acc[q][n][0] = acc[q][n][1] = acc[q][n][2] = acc[q][n][3] = 0.0f;
#pragma unroll
        for (int tap = 0; tap < 9; ++tap) {
            const int dy = tap / 3, dx = tap % 3;  // staged row / column offsets (0..2)
            const unsigned* ra = sin + ((r + dy) * ROWC + a_cell + dx) * CS + a_k;
            const unsigned* rw = sw + (tap * COUT + b_row) * CS + b_k;
#pragma unroll
            for (int kc = 0; kc < CIN / 16; ++kc) {
                unsigned a0[4], a1[4];
                ldsm_x4(a0, ra + kc * 8);
                ldsm_x4(a1, ra + ROWC * CS + kc * 8);  // the next row (staged rows r + 1 + dy)
#pragma unroll
                for (int p = 0; p < NT / 2; ++p) {
                    unsigned b[4];
                    ldsm_x4(b, rw + 16 * p * CS + kc * 8);
                    mma_bf16_16816(acc[0][2 * p], a0[0], a0[1], a0[2], a0[3], b[0], b[1]);
                    mma_bf16_16816(acc[0][2 * p + 1], a0[0], a0[1], a0[2], a0[3], b[2], b[3]);
                    mma_bf16_16816(acc[1][2 * p], a1[0], a1[1], a1[2], a1[3], b[0], b[1]);
                    mma_bf16_16816(acc[1][2 * p + 1], a1[0], a1[1], a1[2], a1[3], b[2], b[3]);
                }
            }
        }
        // epilogue: thread holds rows g, g+8 (cells x0+g, x0+g+8) and columns n*8 + 2c, +1
#pragma unroll
        for (int q = 0; q < 2; ++q) {
            const int y = y0 + r + q;
            if (y >= H) break;
            const size_t cell0 = img_off + (size_t)y * W + x0 + g;
#pragma unroll
            for (int n = 0; n < NT; ++n) {
                const int ch = n * 8 + 2 * c;
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const size_t cell = cell0 + 8 * h;
                    float v0 = acc[q][n][2 * h], v1 = acc[q][n][2 * h + 1];
                    if (EPI == EPI_BIAS_RELU) {
                        v0 = fmaxf(v0 + bias[ch], 0.0f);
                        v1 = fmaxf(v1 + bias[ch + 1], 0.0f);
                        reinterpret_cast<unsigned*>(out)[(cell * COUT + ch) / 2] = pack_bf16x2(v0, v1);
                    } else if (EPI == EPI_BIAS_F32) {
                        *reinterpret_cast<float2*>(reinterpret_cast<float*>(out) + cell * COUT + ch) =
                            make_float2(v0 + bias[ch], v1 + bias[ch + 1]);
                    } else {
                        const __nv_bfloat162 mk = *reinterpret_cast<const __nv_bfloat162*>(mask + cell * COUT + ch);
                        v0 = __bfloat162float(mk.x) > 0.0f ? v0 : 0.0f;
                        v1 = __bfloat162float(mk.y) > 0.0f ? v1 : 0.0f;
                        reinterpret_cast<unsigned*>(out)[(cell * COUT + ch) / 2] = pack_bf16x2(v0, v1);
                    }
                }
            }
        }
    }
}

template <int CIN, int COUT>
constexpr size_t conv_smem_bytes() {
    return (size_t)((CONV_ROWS + 2) * (CONV_CELLS + 2) + 9 * COUT) * SmemStride<CIN>::WORDS * 4;
}

// Weight gradients of one layer, FP32 on the CUDA cores:
//   dW[tap][ci][co] = sum_cells x[cell + off(tap)][ci] * g[cell][co],  db[co] = sum_cells g[cell][co]
// over the cells of rows [r0, r1) and columns [c0, c1) of every image (the region the loss
// covers; inputs outside the image read as zero, or wrap when PERIODIC).  Each thread owns a
// 4 (ci) x 8 (co) block of one tap.  Blocks loop over 64-cell row segments and write one
// partial each; k_dweight_final sums the partials in a fixed order (deterministic).
// blockDim = 9 * (CIN / 4) * (COUT / 8).  GT: gradient element type (bf16 or f32).
template <int CIN, int COUT, class GT, bool PERIODIC>
__global__ void k_dweight(const __nv_bfloat16* __restrict__ x, const GT* __restrict__ gr, int nimg, int H, int W,
                          int r0, int r1, int c0, int c1, float* __restrict__ partials) {
    constexpr int SEG = 64;
    constexpr int CB = CIN / 4, OB = COUT / 8;
    __shared__ float sx[3][SEG + 2][CIN + 1];
    __shared__ float sg[SEG][COUT + 1];
    const int tid = threadIdx.x;
    const int tap = tid / (CB * OB), cb = (tid / OB) % CB, ob = tid % OB;
    const int dy = tap / 3 - 1, dx = tap % 3 - 1;
    float acc[4][8];
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[i][j] = 0.0f;
    float bacc[8];
#pragma unroll
    for (int j = 0; j < 8; ++j) bacc[j] = 0.0f;
    const int segs_per_row = (c1 - c0 + SEG - 1) / SEG;
    const long nseg = (long)nimg * (r1 - r0) * segs_per_row;
    for (long s = blockIdx.x; s < nseg; s += gridDim.x) {
        const int img = (int)(s / ((long)(r1 - r0) * segs_per_row));
        const int rem = (int)(s % ((long)(r1 - r0) * segs_per_row));
        const int y = r0 + rem / segs_per_row;
        const int xs = c0 + (rem % segs_per_row) * SEG;
        const int n = min(SEG, c1 - xs);
        __syncthreads();
        for (int i = tid; i < 3 * (SEG + 2) * CIN; i += blockDim.x) {
            const int ci = i % CIN, cell = (i / CIN) % (SEG + 2), r = i / (CIN * (SEG + 2));
            int gy = y + r - 1, gx = xs + cell - 1;
            float v = 0.0f;
            if (PERIODIC) {
                gy = gy < 0 ? gy + H : (gy >= H ? gy - H : gy);
                gx = gx < 0 ? gx + W : (gx >= W ? gx - W : gx);
                v = __bfloat162float(x[(((size_t)img * H + gy) * W + gx) * CIN + ci]);
            } else if (gy >= 0 && gy < H && gx >= 0 && gx < W) {
                v = __bfloat162float(x[(((size_t)img * H + gy) * W + gx) * CIN + ci]);
            }
            sx[r][cell][ci] = v;
        }
        for (int i = tid; i < SEG * COUT; i += blockDim.x) {
            const int co = i % COUT, cell = i / COUT;
            float v = 0.0f;
            if (cell < n) v = static_cast<float>(gr[(((size_t)img * H + y) * W + xs + cell) * COUT + co]);
            sg[cell][co] = v;
        }
        __syncthreads();
        for (int cell = 0; cell < n; ++cell) {
            float xv[4], gv[8];
#pragma unroll
            for (int i = 0; i < 4; ++i) xv[i] = sx[dy + 1][cell + dx + 1][cb * 4 + i];
#pragma unroll
            for (int j = 0; j < 8; ++j) gv[j] = sg[cell][ob * 8 + j];
#pragma unroll
            for (int i = 0; i < 4; ++i)
#pragma unroll
                for (int j = 0; j < 8; ++j) acc[i][j] = fmaf(xv[i], gv[j], acc[i][j]);
            if (tap == 4 && cb == 0)
#pragma unroll
                for (int j = 0; j < 8; ++j) bacc[j] += gv[j];
        }
    }
    float* p = partials + (size_t)blockIdx.x * (9 * CIN * COUT + COUT);
#pragma unroll
    for (int i = 0; i < 4; ++i)
#pragma unroll
        for (int j = 0; j < 8; ++j) p[(tap * CIN + cb * 4 + i) * COUT + ob * 8 + j] = acc[i][j];
    if (tap == 4 && cb == 0)
#pragma unroll
        for (int j = 0; j < 8; ++j) p[9 * CIN * COUT + ob * 8 + j] = bacc[j];
}

// out[k] = scale * sum_b partials[b][k]: 8 threads per output each add a fixed range of the
// blocks in order, then the 8 sums are added in order (deterministic).  256 threads, 32 outputs
// per block.
__global__ void __launch_bounds__(256) k_dweight_final(const float* __restrict__ partials, int nblocks, int len,
                                                       float scale, float* __restrict__ out) {
    __shared__ double s[8][32];
    const int kk = threadIdx.x & 31, seg = threadIdx.x >> 5;
    const int k = blockIdx.x * 32 + kk;
    double a = 0.0;
    if (k < len) {
        const int per = (nblocks + 7) / 8, b0 = seg * per, b1 = min(nblocks, b0 + per);
        for (int b = b0; b < b1; ++b) a += (double)partials[(size_t)b * len + k];
    }
    s[seg][kk] = a;
    __syncthreads();
    if (seg == 0 && k < len) {
        double t = 0.0;
#pragma unroll
        for (int j = 0; j < 8; ++j) t += s[j][kk];
        out[k] = (float)(t * (double)scale);
    }
}

}  // namespace closure
}  // namespace lbm
