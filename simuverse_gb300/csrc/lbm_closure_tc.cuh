// lbm_closure_tc.cuh -- the closure network's inference as one fused kernel on the 5th-generation
// tensor cores (tcgen05.mma, accumulators in tensor memory).  Included by lbm_closure.cu inside
// namespace lbm::closure, after the per-cell helpers (load_dev, non_equilibrium, pack_bf16x2).
//
// y = conv3(relu(conv2(relu(conv1(x0))))) of the whole periodic field, with x0 = the features of
// the lattice's populations computed on the fly: the activations never leave shared memory and
// tensor memory.
//
// Tiling.  A CTA owns a strip of OUT_W = 124 output columns and TC_ROWS = 32 output rows.  It walks
// down the rows with three ring buffers of three rows each in shared memory: input features
// (16 channels), layer-1 and layer-2 activations (32 channels, BF16).  Every ring row holds
// POS = 130 positions, position p being column x0 - 3 + p (wrapped): one MMA row block of 128
// positions plus the two positions its 3-wide stencil reads beyond them.  Output position p of a
// layer is MMA row p - 1, its A operand for tap (dy, dx) the 128 positions starting at dx of ring
// row (r - 1 + dy); each layer loses one position per side, so layer 3 is valid at positions
// 3..126 = the strip's 124 columns.  Per row: layer 1 (9 MMAs of M128 N32 K16), layer 2 (18 MMAs
// M128 N32 K16), layer 3 (18 MMAs M128 N16 K16).
//
// Operands.  Shared-memory matrices in the canonical K-major layout without swizzle: core
// matrices of 8 rows x 16 bytes (8 BF16 channels); a ring row stores its channel groups as planes
// of POS x 16 bytes, so the descriptor's leading (K-direction) byte offset is POS * 16 and its
// stride (8-row) offset 128; weights [tap][channel group][cout][8] with leading offset cout * 16.
// The descriptor encoding and the accumulator lane layout (thread t of the warpgroup reads TMEM
// lane t = MMA row t with tcgen05.ld 32x32b) were checked against a host product before use.
//
// Schedule.  Step a issues one batch of MMAs: layer-1 row a - 1, layer-2 row a - 3 and layer-3
// row a - 5, which depend only on rows finished in earlier steps, committed to one mbarrier.
// While the batch runs the block loads the populations of the next input row; after it, the
// epilogues (bias, ReLU, BF16) write the new layer rows over the ring rows that the batch was the
// last to read, the output row of layer 3 to global memory, and the next row's features.
// Generic shared-memory writes are fenced to the async proxy before the next batch.  Thread 0
// waits on the mbarrier with a 1 s limit and the block follows its outcome; a timed-out wait
// records LBM_ERR_TIMEOUT, waits (bounded) for the MMAs in flight, frees the tensor memory and
// leaves.
#pragma once

namespace tc {

constexpr int POS = 130;           // ring-row positions: columns x0 - 3 .. x0 + 126
constexpr int OUT_W = 124;         // output columns per strip (positions 3 .. 126)
constexpr int TC_ROWS = 32;        // output rows per CTA
constexpr int TC_THREADS = 128;
constexpr int PLANE = POS * 16;    // bytes of one 8-channel group of a ring row
constexpr int IN_ROW = 2 * PLANE;  // 16 input channels
constexpr int H_ROW = 4 * PLANE;   // 32 hidden channels
constexpr int OFF_IN = 0;
constexpr int OFF_L1 = OFF_IN + 3 * IN_ROW;
constexpr int OFF_L2 = OFF_L1 + 3 * H_ROW;
constexpr int OFF_W1 = OFF_L2 + 3 * H_ROW;
constexpr int OFF_W2 = OFF_W1 + 9 * 2 * 32 * 16;
constexpr int OFF_W3 = OFF_W2 + 9 * 4 * 32 * 16;
constexpr int OFF_BIAS = OFF_W3 + 9 * 4 * 16 * 16;
constexpr int OFF_BAR = OFF_BIAS + 80 * 4;
constexpr int OFF_TSLOT = OFF_BAR + 8;
constexpr int SMEM_BYTES = ((OFF_TSLOT + 4 + 127) / 128) * 128;
constexpr int TMEM_COLS = 128;  // layer 1: columns 0-31, layer 2: 32-63, layer 3: 64-79
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

// 32 / 16 consecutive accumulator columns of this thread's lane
__device__ __forceinline__ void tmem_ld32(unsigned taddr, float (&v)[32]) {
    unsigned r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
        "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]), "=r"(r[8]),
          "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]), "=r"(r[16]),
          "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]), "=r"(r[24]),
          "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
    for (int j = 0; j < 32; ++j) v[j] = __uint_as_float(r[j]);
}
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

// 32 hidden activations (bias + ReLU, BF16) into ring row `row` at position p: 4 channel groups
__device__ __forceinline__ void store_hidden(unsigned char* row, int p, const float (&v)[32], const float* bias) {
#pragma unroll
    for (int g = 0; g < 4; ++g) {
        uint4 q;
        q.x = pack_bf16x2(fmaxf(v[8 * g + 0] + bias[8 * g + 0], 0.0f), fmaxf(v[8 * g + 1] + bias[8 * g + 1], 0.0f));
        q.y = pack_bf16x2(fmaxf(v[8 * g + 2] + bias[8 * g + 2], 0.0f), fmaxf(v[8 * g + 3] + bias[8 * g + 3], 0.0f));
        q.z = pack_bf16x2(fmaxf(v[8 * g + 4] + bias[8 * g + 4], 0.0f), fmaxf(v[8 * g + 5] + bias[8 * g + 5], 0.0f));
        q.w = pack_bf16x2(fmaxf(v[8 * g + 6] + bias[8 * g + 6], 0.0f), fmaxf(v[8 * g + 7] + bias[8 * g + 7], 0.0f));
        *reinterpret_cast<uint4*>(row + g * PLANE + p * 16) = q;
    }
}

// one layer row: 9 taps x KC channel chunks of 16; A from ring rows (r - 1 + dy), B from the
// layer's weights [tap][group][cout][8] (cout rows of 16 bytes per group)
template <int KC, int COUT>
__device__ __forceinline__ void issue_layer(unsigned dtmem, unsigned ring, int ring_row_bytes, int r, unsigned wts) {
    constexpr uint32_t ID = idesc_bf16(128, COUT);
#pragma unroll
    for (int tap = 0; tap < 9; ++tap) {
        const int dy = tap / 3, dx = tap % 3;
        const unsigned arow = ring + (unsigned)(((r - 1 + dy) % 3) * ring_row_bytes) + (unsigned)(dx * 16);
#pragma unroll
        for (int kc = 0; kc < KC; ++kc) {
            const uint64_t a = sdesc(arow + (unsigned)(2 * kc * PLANE), PLANE, 128);
            const uint64_t b = sdesc(wts + (unsigned)((tap * 2 * KC + 2 * kc) * COUT * 16), COUT * 16, 128);
            mma(dtmem, a, b, ID, (tap | kc) != 0 ? 1u : 0u);
        }
    }
}

// Inference of the whole network on an nx x ny periodic lattice.  d: the lattice's populations
// (FP32 deviations, 9 planes); w1 [9][32][16], w2 [9][32][32], w3 [9][16][32] BF16 (tap, cout,
// cin); b1 [32], b2 [32], b3 [16] FP32; y: [nx * ny][16] FP32 outputs (9 used).
// Grid (ceil(nx / OUT_W), ceil(ny / TC_ROWS)), TC_THREADS threads, SMEM_BYTES dynamic shared memory.
__global__ void __launch_bounds__(TC_THREADS, 2)
    k_closure_fused(const float* __restrict__ d, int nx, int ny, float s_in, int inputs,
                    const __nv_bfloat16* __restrict__ w1, const __nv_bfloat16* __restrict__ w2,
                    const __nv_bfloat16* __restrict__ w3, const float* __restrict__ b1, const float* __restrict__ b2,
                    const float* __restrict__ b3, float* __restrict__ y, int* __restrict__ status) {
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

    // rings to zero (positions no layer writes stay finite), weights to the operand layout
    for (int i = tid; i < OFF_W1 / 16; i += TC_THREADS) reinterpret_cast<uint4*>(sm)[i] = make_uint4(0, 0, 0, 0);
    for (int i = tid; i < 9 * 2 * 32; i += TC_THREADS) {  // (tap, group, cout)
        const int n = i % 32, g = (i / 32) % 2, t = i / 64;
        *reinterpret_cast<uint4*>(sm + OFF_W1 + i * 16) = *reinterpret_cast<const uint4*>(w1 + (t * 32 + n) * 16 + g * 8);
    }
    for (int i = tid; i < 9 * 4 * 32; i += TC_THREADS) {
        const int n = i % 32, g = (i / 32) % 4, t = i / 128;
        *reinterpret_cast<uint4*>(sm + OFF_W2 + i * 16) = *reinterpret_cast<const uint4*>(w2 + (t * 32 + n) * 32 + g * 8);
    }
    for (int i = tid; i < 9 * 4 * 16; i += TC_THREADS) {
        const int n = i % 16, g = (i / 16) % 4, t = i / 64;
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
    const unsigned lane_off = (unsigned)(warp * 32) << 16;
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
    // features of the prefetched row into input ring row a
    auto store_features = [&](int a) {
        unsigned char* row = ring_in + (a % 3) * IN_ROW;
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

    // Local rows: input a = lattice row ys - 3 + a (0 .. TC_ROWS + 5), layer-1 b (1 .. TC_ROWS + 4)
    // from input rows b - 1 .. b + 1, layer-2 c (2 .. TC_ROWS + 3), layer-3 e (3 .. TC_ROWS + 2)
    // = output row ys + e - 3.  Step a computes layer-1 row a - 1, layer-2 row a - 3, layer-3 row
    // a - 5 in one batch and stores input row a + 1.  Ring row k % 3 of a layer is overwritten by
    // row k only after the batch that read row k - 3 for the last time has completed.
    load_row(0);
    store_features(0);
    fence_async_smem();
    __syncthreads();
    constexpr int STEPS = TC_ROWS + 8;
    for (int a = 0; a < STEPS; ++a) {
        const bool l1 = a >= 2 && a <= TC_ROWS + 5;
        const bool l2 = a >= 5 && a <= TC_ROWS + 6;
        const bool l3 = a >= 8;
        const bool any = l1 || l2 || l3;
        if (tid == 0 && any) {
            fence_after();
            if (l1) issue_layer<1, 32>(tmem, su32(ring_in), IN_ROW, a - 1, su32(sm + OFF_W1));
            if (l2) issue_layer<2, 32>(tmem + 32, su32(ring_l1), H_ROW, a - 3, su32(sm + OFF_W2));
            if (l3) issue_layer<2, 16>(tmem + 64, su32(ring_l2), H_ROW, a - 5, su32(sm + OFF_W3));
            commit(bar);
        }
        const bool next = a + 1 <= TC_ROWS + 5;
        if (next) load_row(a + 1);
        if (any) {
            if (tid == 0) s_ok = bar_wait_bounded(bar, parity) ? 1 : 0;
            __syncthreads();
            if (!s_ok) {
                alive = false;
                break;
            }
            bar_try(bar, parity);  // complete: acquire the phase in every thread
            parity ^= 1u;
            fence_after();
            if (l1) {
                float v[32];
                tmem_ld32(tmem + lane_off, v);
                store_hidden(ring_l1 + ((a - 1) % 3) * H_ROW, tid + 1, v, bias);
            }
            if (l2) {
                float v[32];
                tmem_ld32(tmem + lane_off + 32, v);
                store_hidden(ring_l2 + ((a - 3) % 3) * H_ROW, tid + 1, v, bias + 32);
            }
            if (l3) {
                float v[16];
                tmem_ld16(tmem + lane_off + 64, v);
                const int p = tid + 1, oy = ys + a - 8, ox = x0 - 3 + p;
                if (p >= 3 && p < 3 + OUT_W && ox < nx && oy < ny) {
                    float4* o = reinterpret_cast<float4*>(y + ((size_t)oy * nx + ox) * 16);
#pragma unroll
                    for (int q = 0; q < 4; ++q)
                        o[q] = make_float4(v[4 * q] + bias[64 + 4 * q], v[4 * q + 1] + bias[65 + 4 * q],
                                           v[4 * q + 2] + bias[66 + 4 * q], v[4 * q + 3] + bias[67 + 4 * q]);
                }
            }
        }
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

}  // namespace tc
