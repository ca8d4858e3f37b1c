// lbm_closure_tc.cuh -- the closure network's inference as one fused kernel on the 5th-generation
// tensor cores (tcgen05.mma, accumulators in tensor memory).  Included by lbm_closure.cu inside
// namespace lbm::closure, after the per-cell helpers (load_dev, non_equilibrium, pack_bf16x2).
//
// y = conv3(relu(conv2(relu(conv1(x0))))) of the whole periodic field, with x0 = the features of
// the lattice's populations computed on the fly: the activations never leave shared memory and
// tensor memory.
//
// Tiling.  A CTA owns a strip of OUT_W = 124 output columns and TC_ROWS = 32 output rows and walks
// down its rows.  A row of every activation -- input features (16 channels), layer-1 and layer-2
// outputs (32 channels, BF16) -- holds POS = 130 positions, position p being column x0 - 3 + p
// (wrapped): one MMA row block of 128 positions plus the two positions a 3-wide stencil reads
// beyond them.  Output position p of a layer is MMA row p - 1; each layer loses one position per
// side, so layer 3 is valid at positions 3..126 = the strip's 124 columns.
//
// Rows stacked along N.  A layer reads each of its input rows r once: for each column shift dx
// (and 16-channel chunk) one MMA multiplies the 128 positions starting at dx by the weights of
// all three row taps dy side by side (N = 3 x cout), contributing to output rows r + 1 - dy.
// Output row o accumulates in tensor-memory slot o % 3 (cout columns each); the weights are
// stored in the row-tap order [2, 1, 0, 2, 1], so the order a row r needs -- slot k receives
// tap (r + 1 - k) mod 3 -- is three consecutive blocks starting at (1 - r) mod 3.  A row is
// complete after its last contributing input row; the epilogue reads it, zeroes the slot with
// tcgen05.st for row o + 3, and writes the BF16 activations (bias, ReLU) to the next layer's
// input, double-buffered in shared memory.  Per input row: layer 1 3 MMAs of M128 N96 K16,
// layer 2 6 of M128 N96 K16, layer 3 6 of M128 N48 K16.
//
// Operands.  Shared-memory matrices in the canonical K-major layout without swizzle: core
// matrices of 8 rows x 16 bytes (8 BF16 channels); an activation row stores its channel groups as
// planes of POS x 16 bytes, so the descriptor's leading (K-direction) byte offset is POS * 16 and
// its stride (8-row) offset 128; weights [dx][channel group][row-tap block 5][cout][8] with leading
// offset 5 * cout * 16.  The descriptor encoding and the accumulator lane layout (warp w reads
// TMEM lanes 32 (w % 4) .. + 31 = MMA rows with tcgen05.ld 32x32b) were checked against a host
// product before use.  The CTA's two warpgroups split every epilogue by accumulator columns.
//
// Schedule.  Step a issues one batch: layer 1 on input row a, layer 2 on layer-1 row a - 2,
// layer 3 on layer-2 row a - 4 (rows finished in earlier steps), committed to one mbarrier.
// While the batch runs the block loads the populations of input row a + 1; after it, the
// epilogues finish layer-1 row a - 1, layer-2 row a - 3 and layer-3 row a - 5 (the output row,
// to global memory) and store the features of row a + 1.  Generic shared-memory writes are fenced
// to the async proxy before the next batch.  Thread 0 waits on the mbarrier with a 1 s limit
// and the block follows its outcome; a timed-out wait records LBM_ERR_TIMEOUT, waits (bounded)
// for the MMAs in flight, frees the tensor memory and leaves.
#pragma once

namespace tc {

constexpr int POS = 130;           // ring-row positions: columns x0 - 3 .. x0 + 126
constexpr int OUT_W = 124;         // output columns per strip (positions 3 .. 126)
constexpr int TC_ROWS = 32;        // output rows per CTA
constexpr int TC_THREADS = 256;  // two warpgroups: each epilogue is split between them by columns
constexpr int PLANE = POS * 16;    // bytes of one 8-channel group of a ring row
constexpr int IN_ROW = 2 * PLANE;  // 16 input channels
constexpr int H_ROW = 4 * PLANE;   // 32 hidden channels
constexpr int OFF_IN = 0;                        // input rows, double-buffered
constexpr int OFF_L1 = OFF_IN + 2 * IN_ROW;      // layer-1 rows, double-buffered
constexpr int OFF_L2 = OFF_L1 + 2 * H_ROW;       // layer-2 rows, double-buffered
constexpr int OFF_W1 = OFF_L2 + 2 * H_ROW;       // [dx 3][group 2][block 5][cout 32] x 16 B
constexpr int OFF_W2 = OFF_W1 + 3 * 2 * 5 * 32 * 16;  // [3][4][5][32]
constexpr int OFF_W3 = OFF_W2 + 3 * 4 * 5 * 32 * 16;  // [3][4][5][16]
constexpr int OFF_BIAS = OFF_W3 + 3 * 4 * 5 * 16 * 16;
constexpr int OFF_BAR = OFF_BIAS + 80 * 4;
constexpr int OFF_TSLOT = OFF_BAR + 8;
constexpr int SMEM_BYTES = ((OFF_TSLOT + 4 + 127) / 128) * 128;
// accumulators: layer 1 columns 0-95 (3 row slots of 32), layer 2 96-191, layer 3 192-239
constexpr int TM_L1 = 0, TM_L2 = 96, TM_L3 = 192;
constexpr int TMEM_COLS = 256;
constexpr unsigned long long WAIT_NS = 1000000000ull;

static_assert(OFF_L1 % 16 == 0 && OFF_L2 % 16 == 0 && OFF_W1 % 16 == 0 && OFF_W2 % 16 == 0 && OFF_W3 % 16 == 0,
              "operands must start on 16-byte boundaries");
static_assert(OFF_BAR % 8 == 0, "mbarriers are 8-byte aligned");
static_assert(2 * SMEM_BYTES <= 227 * 1024, "two CTAs per SM");

__device__ __forceinline__ unsigned su32(const void* p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start address, leading (K) and stride (8-row) byte offsets,
// descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t sdesc(unsigned addr, unsigned lbo, unsigned sbo) {
    return (uint64_t)((addr & 0x3FFFFu) >> 4) | ((uint64_t)((lbo >> 4) & 0x3FFFu) << 16) |
           ((uint64_t)((sbo >> 4) & 0x3FFFu) << 32) | ((uint64_t)1 << 46);
}
// instruction descriptor of kind::f16: FP32 accumulator, BF16 A and B, both K-major, M x N
__host__ __device__ constexpr uint32_t idesc_bf16(int M, int N) {
    return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma(unsigned dtmem, uint64_t a, uint64_t b, uint32_t id, unsigned accumulate) {
    asm volatile(
        "{\n\t.reg .pred p;\n\tsetp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(dtmem),
        "l"(a), "l"(b), "r"(id), "r"(accumulate)
        : "memory");
}
__device__ __forceinline__ void commit(unsigned bar) {
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar) : "memory");
}
__device__ __forceinline__ void fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void fence_async_smem() { asm volatile("fence.proxy.async.shared::cta;" ::: "memory"); }

__device__ __forceinline__ bool bar_try(unsigned bar, unsigned parity) {
    unsigned ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\tmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(bar), "r"(parity)
        : "memory");
    return ok != 0;
}
__device__ __forceinline__ unsigned long long now_ns() {
    unsigned long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}
__device__ __forceinline__ bool bar_wait_bounded(unsigned bar, unsigned parity) {
    if (bar_try(bar, parity)) return true;
    const unsigned long long t0 = now_ns();
    while (!bar_try(bar, parity))
        if (now_ns() - t0 > WAIT_NS) return false;
    return true;
}

// 16 / 8 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld16(unsigned taddr, float (&v)[16]) {
    unsigned r[16];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 16; ++j) v[j] = __uint_as_float(r[j]);
}

// zeros into 16 / 8 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_zero16(unsigned taddr) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x16.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(
                     taddr),
                 "r"(0u)
                 : "memory");
}
__device__ __forceinline__ void tmem_zero8(unsigned taddr) {
    asm volatile("tcgen05.st.sync.aligned.32x32b.x8.b32 [%0], {%1,%1,%1,%1,%1,%1,%1,%1};" ::"r"(taddr), "r"(0u)
                 : "memory");
}
__device__ __forceinline__ void tmem_wait_st() { asm volatile("tcgen05.wait::st.sync.aligned;" ::: "memory"); }
__device__ __forceinline__ void tmem_ld8(unsigned taddr, float (&v)[8]) {
    unsigned r[8];
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x8.b32 {%0,%1,%2,%3,%4,%5,%6,%7}, [%8];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7])
                 : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 8; ++j) v[j] = __uint_as_float(r[j]);
}

// 16 hidden activations, channels 16 h .. 16 h + 15 (bias + ReLU, BF16), into ring row `row` at
// position p: channel groups 2 h and 2 h + 1
__device__ __forceinline__ void store_hidden16(unsigned char* row, int p, int h, const float (&v16)[16],
                                               const float* bias) {
#pragma unroll
    for (int gg = 0; gg < 2; ++gg) {
        const int g = 2 * h + gg;
        const float* vv = v16 + 8 * gg;
        const float* bb = bias + 8 * g;
        uint4 q;
        q.x = pack_bf16x2(fmaxf(vv[0] + bb[0], 0.0f), fmaxf(vv[1] + bb[1], 0.0f));
        q.y = pack_bf16x2(fmaxf(vv[2] + bb[2], 0.0f), fmaxf(vv[3] + bb[3], 0.0f));
        q.z = pack_bf16x2(fmaxf(vv[4] + bb[4], 0.0f), fmaxf(vv[5] + bb[5], 0.0f));
        q.w = pack_bf16x2(fmaxf(vv[6] + bb[6], 0.0f), fmaxf(vv[7] + bb[7], 0.0f));
        *reinterpret_cast<uint4*>(row + g * PLANE + p * 16) = q;
    }
}

// the MMAs of one input row r of a layer: per column shift dx and 16-channel chunk kc, the 128
// positions starting at dx times the three row taps' weights side by side (N = 3 x COUT), into
// the three accumulator slots; the weight blocks start at (1 - r) mod 3 of the stored order
template <int KC, int COUT>
__device__ __forceinline__ void issue_row(unsigned dtmem, unsigned in_row, int r, unsigned wts) {
    constexpr uint32_t ID = idesc_bf16(128, 3 * COUT);
    constexpr unsigned LBO_W = 5 * COUT * 16;
    const int s0 = ((1 - r) % 3 + 3) % 3;
#pragma unroll
    for (int dx = 0; dx < 3; ++dx)
#pragma unroll
        for (int kc = 0; kc < KC; ++kc) {
            const uint64_t a = sdesc(in_row + (unsigned)(dx * 16 + 2 * kc * PLANE), PLANE, 128);
            const uint64_t b = sdesc(wts + (unsigned)(((dx * 2 * KC + 2 * kc) * 5 + s0) * COUT * 16), LBO_W, 128);
            mma(dtmem, a, b, ID, 1u);
        }
}

// Inference of the whole network on an nx x ny periodic lattice.  d: the lattice's populations
// (FP32 deviations, 9 planes); w1 [9][32][16], w2 [9][32][32], w3 [9][16][32] BF16 (tap, cout,
// cin); b1 [32], b2 [32], b3 [16] FP32.  With d_next == nullptr the outputs go to y ([nx * ny][16]
// FP32, 9 used); otherwise the correction is applied here: d_next = d + inv_s_out * P(y) cell by
// cell (P removes a cell's density and momentum), d_next being a buffer other than d (the CTAs
// read each other's halo rows of d).  With zp != nullptr (and d_next == nullptr) the outputs go
// projected, P(y), to 9 planes of nx * ny floats instead of y.
// Grid (ceil(nx / OUT_W), ceil(ny / TC_ROWS)), TC_THREADS threads, SMEM_BYTES dynamic shared memory.
__global__ void __launch_bounds__(TC_THREADS, 2)
    k_closure_fused(const float* __restrict__ d, int nx, int ny, float s_in, int inputs,
                    const __nv_bfloat16* __restrict__ w1, const __nv_bfloat16* __restrict__ w2,
                    const __nv_bfloat16* __restrict__ w3, const float* __restrict__ b1, const float* __restrict__ b2,
                    const float* __restrict__ b3, float* __restrict__ y, float* __restrict__ d_next, float inv_s_out,
                    float* __restrict__ zp, int* __restrict__ status) {
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5;
    const int x0 = blockIdx.x * OUT_W, ys = blockIdx.y * TC_ROWS;
    const size_t N = (size_t)nx * ny;
    unsigned char* ring_in = sm + OFF_IN;
    unsigned char* ring_l1 = sm + OFF_L1;
    unsigned char* ring_l2 = sm + OFF_L2;
    float* bias = reinterpret_cast<float*>(sm + OFF_BIAS);  // b1 [0, 32), b2 [32, 64), b3 [64, 80)
    const unsigned bar = su32(sm + OFF_BAR);
    unsigned* tslot = reinterpret_cast<unsigned*>(sm + OFF_TSLOT);

    // activation rows to zero (positions no layer writes stay finite); weights to the operand
    // layout, row-tap block i holding tap dy = (2 - i) mod 3
    for (int i = tid; i < OFF_W1 / 16; i += TC_THREADS) reinterpret_cast<uint4*>(sm)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 3 * 2 * 5 * 32; i += TC_THREADS) {  // (dx, group, block, cout)
        const int n = i % 32, blk = (i / 32) % 5, g = (i / 160) % 2, dx = i / 320;
        const int t = 3 * ((2 - blk + 3) % 3) + dx;
        *reinterpret_cast<uint4*>(sm + OFF_W1 + i * 16) = *reinterpret_cast<const uint4*>(w1 + (t * 32 + n) * 16 + g * 8);
    }
    for (int i = tid; i < 3 * 4 * 5 * 32; i += TC_THREADS) {
        const int n = i % 32, blk = (i / 32) % 5, g = (i / 160) % 4, dx = i / 640;
        const int t = 3 * ((2 - blk + 3) % 3) + dx;
        *reinterpret_cast<uint4*>(sm + OFF_W2 + i * 16) = *reinterpret_cast<const uint4*>(w2 + (t * 32 + n) * 32 + g * 8);
    }
    for (int i = tid; i < 3 * 4 * 5 * 16; i += TC_THREADS) {
        const int n = i % 16, blk = (i / 16) % 5, g = (i / 80) % 4, dx = i / 320;
        const int t = 3 * ((2 - blk + 3) % 3) + dx;
        *reinterpret_cast<uint4*>(sm + OFF_W3 + i * 16) = *reinterpret_cast<const uint4*>(w3 + (t * 16 + n) * 32 + g * 8);
    }
    if (tid < 32) {
        bias[tid] = b1[tid];
        bias[32 + tid] = b2[tid];
        if (tid < 16) bias[64 + tid] = b3[tid];
    }
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    // warp w reads TMEM lanes 32 (w % 4) .. + 31 (MMA rows = positions - 1); warpgroup h = w / 4
    // takes half of every accumulator row's columns
    const int lane_q = warp & 3, half = warp >> 2;
    const int mrow = lane_q * 32 + (tid & 31);  // this thread's MMA row
    const unsigned lane_off = (unsigned)(lane_q * 32) << 16;
    // every accumulator slot starts at zero (each warpgroup its half of the columns)
#pragma unroll
    for (int k = 0; k < 6; ++k) tmem_zero16(tmem + lane_off + 32 * k + 16 * half);  // layers 1 and 2
#pragma unroll
    for (int k = 0; k < 3; ++k) tmem_zero8(tmem + lane_off + TM_L3 + 16 * k + 8 * half);
    tmem_wait_st();
    unsigned parity = 0u;
    bool alive = true;

    // the populations of input row a (lattice row ys - 3 + a, wrapped) at this thread's positions
    // tid and tid + TC_THREADS (< POS), loaded ahead of their use
    constexpr int NP = (POS + TC_THREADS - 1) / TC_THREADS;
    float pre[NP][9];
    auto load_row = [&](int a) {
        const int gy = ((ys - 3 + a) % ny + ny) % ny;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const int p = tid + k * TC_THREADS;
            if (p < POS) load_dev(d, N, (size_t)gy * nx + ((x0 - 3 + p) % nx + nx) % nx, pre[k]);
        }
    };
    // features of the prefetched row into input buffer a % 2
    auto store_features = [&](int a) {
        unsigned char* row = ring_in + (a % 2) * IN_ROW;
#pragma unroll
        for (int k = 0; k < NP; ++k) {
            const int p = tid + k * TC_THREADS;
            if (p >= POS) continue;
            float v[9];
#pragma unroll
            for (int i = 0; i < 9; ++i) v[i] = pre[k][i];
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
            *reinterpret_cast<uint4*>(row + p * 16) =
                make_uint4(pack_bf16x2(s_in * v[0], s_in * v[1]), pack_bf16x2(s_in * v[2], s_in * v[3]),
                           pack_bf16x2(s_in * v[4], s_in * v[5]), pack_bf16x2(s_in * v[6], s_in * v[7]));
            *reinterpret_cast<uint4*>(row + PLANE + p * 16) = make_uint4(pack_bf16x2(s_in * v[8], 0.0f), 0u, 0u, 0u);
        }
    };
    const auto slot = [](int row) { return ((row % 3) + 3) % 3; };

    // Local rows: input a = lattice row ys - 3 + a (0 .. TC_ROWS + 5); layer-1 rows 1 .. TC_ROWS + 4,
    // layer-2 rows 2 .. TC_ROWS + 3 and layer-3 rows 3 .. TC_ROWS + 2 (= output row ys + e - 3) are
    // the complete ones that the next layer uses; the partial rows at the ends are discarded.
    // Step a: layer-1 MMAs on input row a, layer-2 MMAs on layer-1 row a - 2, layer-3 MMAs on
    // layer-2 row a - 4; then layer-1 row a - 1, layer-2 row a - 3 and layer-3 row a - 5 are
    // complete, read out and their slots zeroed.  A buffer written in step a (layer-1 row a - 1,
    // layer-2 row a - 3, input row a + 1) was last read by the batch of step a - 1.
    load_row(0);
    store_features(0);
    fence_async_smem();
    __syncthreads();
    constexpr int STEPS = TC_ROWS + 8;
    for (int a = 0; a < STEPS; ++a) {
        const bool m1 = a <= TC_ROWS + 5;               // layer-1 MMAs on input row a
        const bool m2 = a >= 3 && a <= TC_ROWS + 6;     // layer-2 MMAs on layer-1 row a - 2
        const bool m3 = a >= 6;                         // layer-3 MMAs on layer-2 row a - 4
        if (tid == 0) {
            fence_after();
            if (m1) issue_row<1, 32>(tmem + TM_L1, su32(ring_in + (a % 2) * IN_ROW), a, su32(sm + OFF_W1));
            if (m2) issue_row<2, 32>(tmem + TM_L2, su32(ring_l1 + ((a - 2) % 2) * H_ROW), a - 2, su32(sm + OFF_W2));
            if (m3) issue_row<2, 16>(tmem + TM_L3, su32(ring_l2 + ((a - 4) % 2) * H_ROW), a - 4, su32(sm + OFF_W3));
            commit(bar);
        }
        const bool next = a + 1 <= TC_ROWS + 5;
        if (next) load_row(a + 1);
        if (tid == 0) s_ok = bar_wait_bounded(bar, parity) ? 1 : 0;
        __syncthreads();
        if (!s_ok) {
            alive = false;
            break;
        }
        bar_try(bar, parity);  // complete: acquire the phase in every thread
        parity ^= 1u;
        fence_after();
        if (m1) {  // layer-1 row a - 1 complete (rows 1 .. TC_ROWS + 4 are used)
            const unsigned t = tmem + lane_off + TM_L1 + 32 * slot(a - 1) + 16 * half;
            if (a - 1 >= 1) {
                float v[16];
                tmem_ld16(t, v);
                store_hidden16(ring_l1 + ((a - 1) % 2) * H_ROW, mrow + 1, half, v, bias);
            }
            tmem_zero16(t);
        }
        if (m2) {  // layer-2 row a - 3 complete (rows 2 .. TC_ROWS + 3 are used)
            const unsigned t = tmem + lane_off + TM_L2 + 32 * slot(a - 3) + 16 * half;
            if (a - 3 >= 2) {
                float v[16];
                tmem_ld16(t, v);
                store_hidden16(ring_l2 + ((a - 3) % 2) * H_ROW, mrow + 1, half, v, bias + 32);
            }
            tmem_zero16(t);
        }
        if (m3) {  // layer-3 row a - 5 complete: output row ys + a - 8 (rows 3 .. TC_ROWS + 2)
            const int p = mrow + 1, oy = ys + a - 8, ox = x0 - 3 + p;
            const bool valid = a - 5 >= 3 && p >= 3 && p < 3 + OUT_W && ox < nx && oy < ny;
            const unsigned t0 = tmem + lane_off + TM_L3 + 16 * slot(a - 5);
            if (d_next == nullptr && zp == nullptr) {  // the outputs, split between the warpgroups
                const unsigned t = t0 + 8 * half;
                if (a - 5 >= 3) {
                    float v[8];
                    tmem_ld8(t, v);
                    if (valid) {
                        const float* bb = bias + 64 + 8 * half;
                        float4* o = reinterpret_cast<float4*>(y + ((size_t)oy * nx + ox) * 16 + 8 * half);
                        o[0] = make_float4(v[0] + bb[0], v[1] + bb[1], v[2] + bb[2], v[3] + bb[3]);
                        o[1] = make_float4(v[4] + bb[4], v[5] + bb[5], v[6] + bb[6], v[7] + bb[7]);
                    }
                }
                tmem_zero8(t);
            } else if (half == 0) {  // the projected outputs: added to the populations, or as planes
                if (a - 5 >= 3) {
                    float v[16];
                    tmem_ld16(t0, v);
                    if (valid) {
                        float q[9];
#pragma unroll
                        for (int i = 0; i < 9; ++i) q[i] = v[i] + bias[64 + i];
                        project9(q);
                        const size_t c = (size_t)oy * nx + ox;
                        if (d_next != nullptr) {
#pragma unroll
                            for (int i = 0; i < 9; ++i)
                                d_next[c + (size_t)i * N] = d[c + (size_t)i * N] + inv_s_out * q[i];
                        } else {
#pragma unroll
                            for (int i = 0; i < 9; ++i) zp[c + (size_t)i * N] = q[i];
                        }
                    }
                }
                tmem_zero16(t0);
            }
        }
        tmem_wait_st();
        if (next) store_features(a + 1);
        fence_before();
        fence_async_smem();
        __syncthreads();
    }
    if (!alive) {  // a wait ran out: record it and let the MMAs in flight finish before freeing
        if (tid == 0) {
            atomicExch(status, LBM_ERR_TIMEOUT);
            bar_wait_bounded(bar, parity);
        }
        fence_before();
        __syncthreads();
    }
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
    }
}

// ------------------------------------------------------------------------------------------
// Weight gradients of one layer on the tensor cores (training):
//   dW[tap][ci][co] = sum_cells x[cell + off(tap)][ci] g[cell][co],   db[co] = sum_cells g[cell][co]
// over every cell of nimg images of H x W (W % 64 == 0; inputs outside an image read as zero),
// as GEMMs with the cells as the K dimension: for each row tap dy, A = the three column-shifted
// copies of the input row y + dy - 1 stacked along M (row dx * CIN + ci, a row of ones whose
// product is db, zero rows up to 128), B = the output gradients of row y (N = COUT), D in
// tensor memory (columns dy * COUT), accumulated over all the CTA's tiles.  A tile is 64 cells
// of one image row (K = 64: 4 MMAs of K16 per row tap).
//
// Sliding rows.  The tiles are numbered down the rows of each 64-column strip of each image, and
// a CTA takes a contiguous range of them, so consecutive tiles are consecutive rows of a strip:
// the transposed copies of an input row live in one of four slots (row r in slot (r + 1) % 4)
// and serve the three tiles that read it.  A tile transposes one new input row (the row below),
// or three where its strip starts, while the MMAs of the previous tile may still read theirs.
// (A ring one tile deeper -- five slots, three gradient buffers -- measured no faster: the
// per-tile work on the SM, not the wait for the MMAs, sets the pace.)
//
// Staging.  The input rows and the tile's 64 gradient cells are copied as they are stored (NHWC,
// channels contiguous) into shared memory with cp.async, through a ring of three raw buffers (the
// copies of the next two tiles are in flight while a tile is transposed); ldmatrix.trans turns
// each 8-cell x 8-channel block into the canonical K-major core matrix (8 rows = channels, 16
// bytes = 8 cells): thread t of the warp receives exactly the 4 bytes at offset 4t of the core
// matrix, so the stores are contiguous.  Operand layout [k chunk][row][8]: the descriptor's
// leading (K) offset is rows * 16, its stride (8-row) offset 128, as in the inference kernel.
// Gradients are double-buffered.  Before a slot or gradient buffer is rewritten, thread 0 waits
// (1 s limit) for the commit of the MMAs that read it: the tile two back, or the previous tile
// where a strip starts.  Each CTA
// writes its partial sums in the CUDA-core kernel's layout, so k_dweight_final reduces them the
// same way.
constexpr int DW_TILE = 64;
constexpr int DW_THREADS = 256;
constexpr int DW_TMEM_COLS = 128;

template <int CIN, int COUT>
struct DwLayout {
    static constexpr int SROWS = 128;               // rows of a slot: 3 CIN shifted rows, ones, zeros
    static constexpr int SLOT = 8 * SROWS * 16;     // [k chunk 8][128 rows][16 B]
    static constexpr int NSLOT = 4;                 // input-row slots: 3 read + 1 being filled
    static constexpr int NB = 2;                    // gradient buffers (and mbarriers)
    static constexpr int XSTR = CIN * 2 + 16;       // padded: ldmatrix rows 8 cells apart hit distinct banks
    static constexpr int GSTR = COUT * 2 + 16;
    static constexpr int RAW_X = 3 * (DW_TILE + 2) * XSTR;
    static constexpr int RAW = ((RAW_X + DW_TILE * GSTR + 127) / 128) * 128;
    static constexpr int NRAW = 3;                  // raw ring depth
    static constexpr int B_BYTES = COUT * DW_TILE * 2;
    static constexpr int OFF_SLOT = NRAW * RAW;
    static constexpr int OFF_B = OFF_SLOT + NSLOT * SLOT;
    static constexpr int OFF_BAR = OFF_B + NB * B_BYTES;
    static constexpr int OFF_TSLOT = OFF_BAR + 8 * NB;
    static constexpr int SMEM = OFF_TSLOT + 16;
    static_assert(3 * CIN + 1 <= SROWS, "three shifted rows and the ones row fit a slot");
    static_assert(3 * COUT <= DW_TMEM_COLS, "accumulators fit the allocation");
    static_assert(OFF_SLOT % 128 == 0 && OFF_B % 128 == 0 && OFF_BAR % 8 == 0, "alignment");
    static_assert(SMEM <= 227 * 1024, "one CTA per SM");
};

__device__ __forceinline__ void ldsm_x4_trans(unsigned (&r)[4], unsigned addr) {
    asm volatile("ldmatrix.sync.aligned.m8n8.x4.trans.shared.b16 {%0,%1,%2,%3}, [%4];"
                 : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3])
                 : "r"(addr));
}

template <int CIN, int COUT>
__global__ void __launch_bounds__(DW_THREADS, 1)
    k_dweight_tc(const __nv_bfloat16* __restrict__ x, const __nv_bfloat16* __restrict__ g, int nimg, int H, int W,
                 float* __restrict__ partials, int* __restrict__ status) {
    using L = DwLayout<CIN, COUT>;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const unsigned bar0 = su32(sm + L::OFF_BAR);  // one mbarrier per gradient buffer, 8 bytes apart
    unsigned* tslot = reinterpret_cast<unsigned*>(sm + L::OFF_TSLOT);
    const int tiles_x = W / DW_TILE, ntiles = nimg * tiles_x * H;
    // this CTA's tiles: a contiguous range of t = (img * tiles_x + strip) * H + y
    const int G = (int)gridDim.x;
    const int t_begin = (int)(((long long)ntiles * blockIdx.x) / G), t_end = (int)(((long long)ntiles * (blockIdx.x + 1)) / G);

    // rows of the slots that no tile writes: the ones row (db) and the zero rows
    for (int i = tid; i < L::NSLOT * 8 * (L::SROWS - 3 * CIN); i += DW_THREADS) {
        const int per = 8 * (L::SROWS - 3 * CIN);
        const int sl = i / per, rem = i % per, kc = rem / (L::SROWS - 3 * CIN), m = 3 * CIN + rem % (L::SROWS - 3 * CIN);
        const unsigned v = m == 3 * CIN ? 0x3F803F80u : 0u;  // BF16 1.0 pairs
        *reinterpret_cast<uint4*>(sm + L::OFF_SLOT + sl * L::SLOT + (kc * L::SROWS + m) * 16) = make_uint4(v, v, v, v);
    }
    if (tid == 0) {
        for (int k = 0; k < L::NB; ++k) asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar0 + 8 * k) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(DW_TMEM_COLS)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }

    // raw copies of tile t into raw buffer b: the input rows it needs first (rows y - 1 .. y + 1
    // into raw rows 0 .. 2 where its strip starts in this CTA, else row y + 1 into raw row 2) and
    // its 64 gradient cells.  Thread tid copies the 16-byte chunks tid, tid + 256, ... of the
    // buffer, the same in every tile.
    constexpr int XC = CIN / 8, GC = COUT / 8;
    constexpr int NXCH = 3 * (DW_TILE + 2) * XC, NGCH = DW_TILE * GC;
    constexpr int NCOPY = (NXCH + NGCH + DW_THREADS - 1) / DW_THREADS;
    int crow[NCOPY], ccol[NCOPY];  // input chunk: raw row, column (-1: a gradient chunk; -2: none)
    unsigned coff[NCOPY], soff[NCOPY];  // channel offset within the cell / smem byte offset
#pragma unroll
    for (int k = 0; k < NCOPY; ++k) {
        const int q = tid + k * DW_THREADS;
        if (q < NXCH) {
            const int cc = q % XC, col = (q / XC) % (DW_TILE + 2), r = q / (XC * (DW_TILE + 2));
            crow[k] = r;
            ccol[k] = col;
            coff[k] = (unsigned)(cc * 8);
            soff[k] = (unsigned)((r * (DW_TILE + 2) + col) * L::XSTR + cc * 16);
        } else if (q < NXCH + NGCH) {
            const int qq = q - NXCH, cc = qq % GC, cell = qq / GC;
            crow[k] = -1;
            ccol[k] = cell;
            coff[k] = (unsigned)(cc * 8);
            soff[k] = (unsigned)(L::RAW_X + cell * L::GSTR + cc * 16);
        } else {
            crow[k] = -2;
            ccol[k] = 0;
            coff[k] = 0;
            soff[k] = 0;
        }
    }
    auto starts = [&](int t) { return t == t_begin || t % H == 0; };  // a strip starts: three new rows
    auto stage = [&](int t, int b) {
        const int y = t % H, strip = t / H, img = strip / tiles_x, x0 = (strip % tiles_x) * DW_TILE;
        const int first = starts(t) ? 0 : 2;
        unsigned char* raw = sm + b * L::RAW;
        const size_t rowx = ((size_t)img * H + y) * W;  // cell index of (img, y, 0)
#pragma unroll
        for (int k = 0; k < NCOPY; ++k) {
            if (crow[k] >= first) {
                const int gy = y + crow[k] - 1, gx = x0 + ccol[k] - 1;
                const bool in = gy >= 0 && gy < H && gx >= 0 && gx < W;
                const __nv_bfloat16* src =
                    in ? x + (size_t)((long long)rowx + (long long)(crow[k] - 1) * W + gx) * CIN + coff[k] : x;
                cp_async16(reinterpret_cast<unsigned*>(raw + soff[k]), src, in);
            } else if (crow[k] == -1) {
                cp_async16(reinterpret_cast<unsigned*>(raw + soff[k]), g + (rowx + x0 + ccol[k]) * COUT + coff[k], true);
            }
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    // operands of tile t from raw buffer rb: each new input row r (raw row r - y + 1) into slot
    // (r + 1) % 4 as three column-shifted copies (slot row dx * CIN + ci holds the cells shifted
    // by dx - 1), and the gradients into gradient buffer gb.  One ldmatrix.x4.trans covers 4
    // consecutive k chunks of one 8-row group; the lane's part of the source address is a
    // constant, the rest is warp-uniform.
    constexpr int OPR = 3 * XC * 2, OPB = GC * 2;  // ops per input row, per gradient row
    const unsigned lane_src_x = (unsigned)(((lane >> 3) * 8 + (lane & 7)) * L::XSTR);
    const unsigned lane_src_g = (unsigned)(((lane >> 3) * 8 + (lane & 7)) * L::GSTR);
    auto transpose = [&](int t, int rb, int gb) {
        const int y = t % H;
        const int first = starts(t) ? 0 : 2, nops = (3 - first) * OPR + OPB;
        const unsigned rx = su32(sm + rb * L::RAW);
        unsigned char* S = sm + L::OFF_SLOT + 4 * lane;
        unsigned char* Bm = sm + L::OFF_B + gb * L::B_BYTES + 4 * lane;
        for (int op = warp; op < nops; op += DW_THREADS / 32) {
            unsigned r[4];
            unsigned char* dst;
            unsigned stride;
            if (op < (3 - first) * OPR) {
                const int rr = first + op / OPR, o = op % OPR;  // raw row, op within the row
                const int kh = o & 1, cg = (o >> 1) % XC, dx = (o >> 1) / XC;
                ldsm_x4_trans(r, rx + lane_src_x + (unsigned)((rr * (DW_TILE + 2) + kh * 32 + dx) * L::XSTR + cg * 16));
                const int slot = (y + rr) % L::NSLOT;  // input row y + rr - 1
                dst = S + slot * L::SLOT + ((kh * 4) * L::SROWS + dx * CIN + cg * 8) * 16;
                stride = L::SROWS * 16;
            } else {
                const int q = op - (3 - first) * OPR, kh = q & 1, ng = q >> 1;
                ldsm_x4_trans(r, rx + L::RAW_X + lane_src_g + (unsigned)((kh * 32) * L::GSTR + ng * 16));
                dst = Bm + ((kh * 4) * COUT + ng * 8) * 16;
                stride = COUT * 16;
            }
#pragma unroll
            for (int q4 = 0; q4 < 4; ++q4) *reinterpret_cast<unsigned*>(dst + q4 * stride) = r[q4];
        }
    };

    fence_async_smem();
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    constexpr uint32_t ID = idesc_bf16(128, COUT);
    // operand descriptors of slot 0 and gradient buffer 0 at k chunk 0 (shared memory is below
    // 256 KB, so adding an offset / 16 to the start address field never carries out of it)
    const uint64_t a_desc0 = sdesc(su32(sm + L::OFF_SLOT), L::SROWS * 16, 128);
    const uint64_t b_desc0 = sdesc(su32(sm + L::OFF_B), COUT * 16, 128);
    bool alive = true;
    int i = 0, last = -1;
    // the copies of the first two tiles (an empty group when there is no second tile, so that
    // one group per tile is always outstanding)
    if (t_begin < t_end) stage(t_begin, 0);
    if (t_begin + 1 < t_end) stage(t_begin + 1, 1);
    else asm volatile("cp.async.commit_group;" ::: "memory");
    for (int t = t_begin; t < t_end; ++t, ++i) {
        const int b = i % L::NB;
        asm volatile("cp.async.wait_group 1;" ::: "memory");  // tile i's copies (tile i + 1's may run)
        if (tid == 0) {
            // the slot this tile fills and gradient buffer b were last read by tile i - NB; where a
            // strip starts, three slots are refilled: wait for the previous tile (and so all)
            bool ok = i < L::NB || bar_wait_bounded(bar0 + 8 * b, ((i - L::NB) / L::NB) & 1);
            if (ok && starts(t) && i >= 1) ok = bar_wait_bounded(bar0 + 8 * ((i - 1) % L::NB), ((i - 1) / L::NB) & 1);
            s_ok = ok ? 1 : 0;
        }
        __syncthreads();
        if (!s_ok) {
            alive = false;
            break;
        }
        transpose(t, i % L::NRAW, b);
        // raw buffer (i + 2) % 3 was last read by the transposes of tile i - 1
        if (t + 2 < t_end) stage(t + 2, (i + 2) % L::NRAW);
        else asm volatile("cp.async.commit_group;" ::: "memory");
        fence_async_smem();
        fence_before();
        __syncthreads();
        if (tid == 0) {
            fence_after();
            const int y = t % H;
            // descriptors differ only in their start address field (address / 16, low bits)
#pragma unroll
            for (int dy = 0; dy < 3; ++dy) {
                const uint64_t ad0 = a_desc0 + (uint64_t)((((y + dy) % L::NSLOT) * L::SLOT) >> 4);  // input row y + dy - 1
#pragma unroll
                for (int ks = 0; ks < DW_TILE / 16; ++ks)
                    mma(tmem + (unsigned)(dy * COUT), ad0 + (uint64_t)((2 * ks * L::SROWS * 16) >> 4),
                        b_desc0 + (uint64_t)((b * L::B_BYTES + 2 * ks * COUT * 16) >> 4), ID, (i > 0 || ks > 0) ? 1u : 0u);
            }
            commit(bar0 + 8 * b);
        }
        last = i;
    }
    // the last commit covers every MMA of the CTA
    if (tid == 0) s_ok = (last < 0 || bar_wait_bounded(bar0 + 8 * (last % L::NB), (last / L::NB) & 1)) ? 1 : 0;
    __syncthreads();
    if (!s_ok) alive = false;
    if (alive && last >= 0) {
        fence_after();
        // accumulator rows: row tap dy's tile, row dx * CIN + ci = tap (3 dy + dx), channel ci;
        // row 3 CIN of every tile is db (read from dy = 1)
        const int lane_q = warp & 3, half = warp >> 2;
        float* p = partials + (size_t)blockIdx.x * (9 * CIN * COUT + COUT);
        for (int dy = half; dy < 3; dy += 2) {
            const int m = lane_q * 32 + lane;
#pragma unroll
            for (int c0 = 0; c0 < COUT; c0 += 16) {
                float v[16];
                tmem_ld16(tmem + ((unsigned)(lane_q * 32) << 16) + (unsigned)(dy * COUT + c0), v);
                float* o = m < 3 * CIN ? p + (size_t)(dy * 3 * CIN + m) * COUT + c0
                                       : (m == 3 * CIN && dy == 1 ? p + 9 * CIN * COUT + c0 : nullptr);
                if (o != nullptr)
#pragma unroll
                    for (int j = 0; j < 16; ++j) o[j] = v[j];
            }
        }
    } else if (last < 0) {  // no tile: zero partials
        float* p = partials + (size_t)blockIdx.x * (9 * CIN * COUT + COUT);
        for (int k = tid; k < 9 * CIN * COUT + COUT; k += DW_THREADS) p[k] = 0.0f;
    }
    if (!alive) {  // a wait ran out: record it and let the MMAs in flight finish before freeing
        if (tid == 0) {
            atomicExch(status, LBM_ERR_TIMEOUT);
            if (last >= 0) bar_wait_bounded(bar0 + 8 * (last % L::NB), (last / L::NB) & 1);
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(DW_TMEM_COLS)
                     : "memory");
    }
}

// ------------------------------------------------------------------------------------------
// One 3x3 convolution of the training path on the tcgen05 tensor cores, the same operation as
// k_conv3x3 (non-periodic: cells outside an image read as zero): in [nimg][H][W][CIN] BF16,
// wk [9][COUT][CIN] BF16 (tap = 3 (dy + 1) + (dx + 1)), bias [COUT] FP32; out [nimg][H][W][COUT]
// BF16 with bias and ReLU (EPI_BIAS_RELU), FP32 with bias (EPI_BIAS_F32), or BF16 where the mask
// activation is positive (EPI_MASK, the input gradient of a ReLU layer).
//
// The inference kernel's schedule for one layer: a CTA owns 128 output columns (positions
// x0 .. x0 + 127 = MMA rows) and CONV_TC_ROWS output rows and walks its input rows y0 - 1 ..
// y0 + CONV_TC_ROWS.  Each input row (130 positions, x0 - 1 .. x0 + 128) is read once: per column
// shift dx and 16-channel chunk one MMA multiplies the 128 positions starting at dx by the three
// row taps' weights side by side (N = 3 COUT), the row-tap blocks stored in the order [2, 1, 0, 2,
// 1] so that output row o always lands in accumulator slot o mod 3.  After input row r the output
// row r - 1 is complete: its slot is read, the epilogue written to global memory and the slot
// zeroed.  Input rows are double-buffered and copied with cp.async while the MMAs of the row
// before run; thread 0 waits (1 s limit) for each row's commit, and a wait that runs out records
// LBM_ERR_TIMEOUT, waits (bounded) for the MMAs in flight and frees the tensor memory.
constexpr int CONV_TC_ROWS = 8;
constexpr int CONV_TC_THREADS = 256;
constexpr int CONV_TC_TMEM = 128;

template <int CIN, int COUT>
struct ConvTcLayout {
    static constexpr int GIN = CIN / 8;                       // 8-channel groups of an input row
    static constexpr int IN_ROW = GIN * PLANE;                // [group][130 positions][16 B]
    static constexpr int OFF_W = 2 * IN_ROW;                  // [dx 3][group][block 5][cout][16 B]
    static constexpr int W_BYTES = 3 * GIN * 5 * COUT * 16;
    static constexpr int OFF_BIAS = OFF_W + W_BYTES;
    static constexpr int OFF_BAR = OFF_BIAS + COUT * 4;
    static constexpr int OFF_TSLOT = OFF_BAR + 8;
    static constexpr int SMEM = ((OFF_TSLOT + 4 + 127) / 128) * 128;
    static_assert(CIN % 16 == 0 && (COUT == 16 || COUT == 32), "channel counts of the closure layers");
    static_assert(3 * COUT <= CONV_TC_TMEM, "accumulator slots fit the allocation");
    static_assert(OFF_W % 16 == 0 && OFF_BAR % 8 == 0, "alignment");
};

template <int CIN, int COUT, int EPI>
__global__ void __launch_bounds__(CONV_TC_THREADS, 4)
    k_conv_tc(const __nv_bfloat16* __restrict__ in, void* __restrict__ out, const __nv_bfloat16* __restrict__ wk,
              const float* __restrict__ bias, const __nv_bfloat16* __restrict__ mask, int H, int W,
              int* __restrict__ status) {
    using L = ConvTcLayout<CIN, COUT>;
    constexpr int KC = CIN / 16;
    extern __shared__ __align__(128) unsigned char sm[];
    __shared__ int s_ok;
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    const int img = blockIdx.z, y0 = blockIdx.y * CONV_TC_ROWS, x0 = blockIdx.x * 128;
    const size_t img_off = (size_t)img * H * W;
    unsigned char* ring = sm;
    float* sbias = reinterpret_cast<float*>(sm + L::OFF_BIAS);
    const unsigned bar = su32(sm + L::OFF_BAR);
    unsigned* tslot = reinterpret_cast<unsigned*>(sm + L::OFF_TSLOT);

    // weights to the operand layout, row-tap block i holding tap dy = (2 - i) mod 3
    for (int i = tid; i < 3 * L::GIN * 5 * COUT; i += CONV_TC_THREADS) {  // (dx, group, block, cout)
        const int n = i % COUT, blk = (i / COUT) % 5, g = (i / (5 * COUT)) % L::GIN, dx = i / (5 * COUT * L::GIN);
        const int t = 3 * ((2 - blk + 3) % 3) + dx;
        *reinterpret_cast<uint4*>(sm + L::OFF_W + i * 16) =
            *reinterpret_cast<const uint4*>(wk + ((size_t)t * COUT + n) * CIN + g * 8);
    }
    if (EPI != EPI_MASK && tid < COUT) sbias[tid] = bias[tid];
    if (tid == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
    }
    if (warp == 0) {
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(su32(tslot)),
                     "r"(CONV_TC_TMEM)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    // input row gy (zero outside the image) into ring buffer b: group g, position p = column x0 - 1 + p
    auto stage = [&](int gy, int b) {
        unsigned char* row = ring + b * L::IN_ROW;
        for (int i = tid; i < L::GIN * POS; i += CONV_TC_THREADS) {
            const int p = i % POS, g = i / POS, gx = x0 - 1 + p;
            const bool ok = gy >= 0 && gy < H && gx >= 0 && gx < W;
            const __nv_bfloat16* src = ok ? in + (img_off + (size_t)gy * W + gx) * CIN + g * 8 : in;
            cp_async16(reinterpret_cast<unsigned*>(row + g * PLANE + p * 16), src, ok);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
    };
    stage(y0 - 1, 0);
    fence_before();
    __syncthreads();
    fence_after();
    const unsigned tmem = *tslot;
    const int lane_q = warp & 3, half = warp >> 2;
    const unsigned lane_off = (unsigned)(lane_q * 32) << 16;
    constexpr int HC = COUT / 2;  // accumulator columns per warpgroup
    // every slot starts at zero (each warpgroup its half of the columns)
#pragma unroll
    for (int k = 0; k < 3; ++k) {
        if constexpr (HC == 16) tmem_zero16(tmem + lane_off + k * COUT + half * HC);
        else tmem_zero8(tmem + lane_off + k * COUT + half * HC);
    }
    tmem_wait_st();
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    fence_async_smem();
    fence_before();
    __syncthreads();
    unsigned parity = 0u;
    bool alive = true;
    const int nrows = min(CONV_TC_ROWS, H - y0);  // output rows of this CTA
    for (int a = 0; a < nrows + 2; ++a) {  // input row y0 - 1 + a
        const int gy = y0 - 1 + a;
        if (tid == 0) {
            fence_after();
            issue_row<KC, COUT>(tmem, su32(ring + (a & 1) * L::IN_ROW), gy, su32(sm + L::OFF_W));
            commit(bar);
        }
        if (a + 1 < nrows + 2) stage(gy + 1, (a + 1) & 1);  // its buffer was read by row a - 1's MMAs
        if (tid == 0) s_ok = bar_wait_bounded(bar, parity) ? 1 : 0;
        __syncthreads();
        if (!s_ok) {
            alive = false;
            break;
        }
        bar_try(bar, parity);  // complete: acquire the phase in every thread
        parity ^= 1u;
        fence_after();
        // output row gy - 1 is complete; rows before y0 only had to be cleared
        const int go = gy - 1;
        const int slot = ((go % 3) + 3) % 3;
        const unsigned t = tmem + lane_off + slot * COUT + half * HC;
        const int p = lane_q * 32 + lane, gx = x0 + p;
        if (go >= y0) {
            float v[HC];
            if constexpr (HC == 16) tmem_ld16(t, v);
            else tmem_ld8(t, v);
            if (gx < W) {
                const size_t cell = img_off + (size_t)go * W + gx;
                const int c0 = half * HC;
                if (EPI == EPI_BIAS_F32) {
                    float4* o = reinterpret_cast<float4*>(reinterpret_cast<float*>(out) + cell * COUT + c0);
#pragma unroll
                    for (int q = 0; q < HC / 4; ++q)
                        o[q] = make_float4(v[4 * q] + sbias[c0 + 4 * q], v[4 * q + 1] + sbias[c0 + 4 * q + 1],
                                           v[4 * q + 2] + sbias[c0 + 4 * q + 2], v[4 * q + 3] + sbias[c0 + 4 * q + 3]);
                } else {
                    unsigned w[HC / 2];
                    if (EPI == EPI_BIAS_RELU) {
#pragma unroll
                        for (int q = 0; q < HC / 2; ++q)
                            w[q] = pack_bf16x2(fmaxf(v[2 * q] + sbias[c0 + 2 * q], 0.0f),
                                               fmaxf(v[2 * q + 1] + sbias[c0 + 2 * q + 1], 0.0f));
                    } else {  // EPI_MASK
                        const uint4* mk = reinterpret_cast<const uint4*>(mask + cell * COUT + c0);
#pragma unroll
                        for (int q4 = 0; q4 < HC / 8; ++q4) {
                            const uint4 mm = mk[q4];
                            const unsigned mw[4] = {mm.x, mm.y, mm.z, mm.w};
#pragma unroll
                            for (int q = 0; q < 4; ++q) {
                                const __nv_bfloat162 m2 = *reinterpret_cast<const __nv_bfloat162*>(&mw[q]);
                                const int k = 8 * q4 + 2 * q;
                                w[4 * q4 + q] = pack_bf16x2(__bfloat162float(m2.x) > 0.0f ? v[k] : 0.0f,
                                                            __bfloat162float(m2.y) > 0.0f ? v[k + 1] : 0.0f);
                            }
                        }
                    }
                    uint4* o = reinterpret_cast<uint4*>(reinterpret_cast<__nv_bfloat16*>(out) + cell * COUT + c0);
#pragma unroll
                    for (int q = 0; q < HC / 8; ++q) o[q] = make_uint4(w[4 * q], w[4 * q + 1], w[4 * q + 2], w[4 * q + 3]);
                }
            }
        }
        if constexpr (HC == 16) tmem_zero16(t);
        else tmem_zero8(t);
        tmem_wait_st();
        asm volatile("cp.async.wait_group 0;" ::: "memory");  // input row a + 1 landed
        fence_async_smem();
        fence_before();
        __syncthreads();
    }
    if (!alive) {  // a wait ran out: record it and let the MMAs in flight finish before freeing
        if (tid == 0) {
            atomicExch(status, LBM_ERR_TIMEOUT);
            bar_wait_bounded(bar, parity);
        }
    }
    asm volatile("cp.async.wait_group 0;" ::: "memory");
    fence_before();
    __syncthreads();
    if (warp == 0) {
        fence_after();
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(CONV_TC_TMEM)
                     : "memory");
    }
}

}  // namespace tc
