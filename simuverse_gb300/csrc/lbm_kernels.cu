// lbm_kernels.cu -- sm_103a kernels of the D2Q9 step and its helpers.
//
// One fused pass per time step replaces the reference's two dispatches
// (collide_stream.wgsl then boundary.wgsl, d2q9_node.rs:302-312):
//   * pull streaming from the ping-pong buffer A (layout_and_fn.wgsl:38-51),
//   * moments, forcing and BGK collision (collide_stream.wgsl:43-87),
//   * the bounce-back of boundary.wgsl:3-35, folded into the owning fluid cell: a fluid
//     cell strictly inside the outer ring whose neighbour c+e_i is solid writes its
//     post-collision population i into the wall slot (c+e_i, inv(i)) and a zero into its
//     own slot (c, i), which is exactly what the boundary dispatch leaves behind.  Each wall
//     slot has one writer, so the pass is race-free.  Wall-to-wall slots (both cells solid)
//     are never read by a fluid cell; the reference's boundary dispatch races on them, and
//     this kernel sets them to zero, one of the outcomes that race can produce.
//   * the macro field (rho, ux, uy) when requested (collide_stream.wgsl:36,74).
//
// Reference mode reproduces the WGSL arithmetic operation by operation with explicit
// round-to-nearest intrinsics (no multiply-add contraction), so it agrees bit for bit with
// a CPU restatement compiled with contraction off.  Physics mode is a standard BGK step
// with exact weights, stored as deviations f - w.
#include "lbm_cell.cuh"
#include "lbm_common.cuh"
#include "lbm_internal.h"

namespace lbm {

// ------------------------------------------------------------------------------------
// flags
// ------------------------------------------------------------------------------------
__global__ void k_build_flags(const lbm_lattice_info* __restrict__ info, uint16_t* __restrict__ flags, int nx,
                              int ny, int mode) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    const size_t c = (size_t)y * nx + x;
    const int code = info[c].material;
    unsigned fl = (code >= 0 && code <= 15) ? (unsigned)code : 0u;
    auto inside = [&](int xx, int yy) { return xx > 0 && yy > 0 && xx < nx - 1 && yy < ny - 1; };
    if (mode == LBM_MODE_REFERENCE) {
        if (is_solid(code)) {
#pragma unroll
            for (int k = 0; k < 9; ++k) {
                const int px = x + EX(k), py = y + EY(k);
                if (px < 0 || py < 0 || px >= nx || py >= ny) continue;
                if (is_solid(info[(size_t)py * nx + px].material) && (inside(x, y) || inside(px, py)))
                    fl |= 1u << (FL_DIR_SHIFT + k);
            }
        } else if (inside(x, y)) {
#pragma unroll
            for (int k = 1; k < 9; ++k) {
                if (is_solid(info[(size_t)(y + EY(k)) * nx + (x + EX(k))].material)) fl |= 1u << (FL_DIR_SHIFT + k);
            }
        }
    } else {
        if (!is_solid(code)) {
#pragma unroll
            for (int j = 1; j < 9; ++j) {
                int sx = x - EX(j), sy = y - EY(j);
                if (code == LBM_OUTLET && EX(j) == -1) sx = x;
                sx = sx < 0 ? nx - 1 : (sx >= nx ? 0 : sx);
                sy = sy < 0 ? ny - 1 : (sy >= ny ? 0 : sy);
                const lbm_lattice_info s = info[(size_t)sy * nx + sx];
                if (is_solid(s.material)) {
                    fl |= 1u << (FL_DIR_SHIFT + j);
                    if (s.vx != 0.0f || s.vy != 0.0f) fl |= FL_MOVING;
                }
            }
        }
        fl |= plain_bit(fl);
    }
    flags[c] = (uint16_t)fl;
}

// ------------------------------------------------------------------------------------
// physics-mode scene masks on the device.  The expressions are the host builder's
// (mask_phys_cavity, mask_phys_channel, disk_cells in lbm_api.cpp) with every FP64 product,
// sum and quotient rounded separately, so the records are bit-identical to the host copy.
// ------------------------------------------------------------------------------------
__global__ void k_build_scene(lbm_lattice_info* __restrict__ info, int nx, int ny, int scene, float lid, float u_max) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    lbm_lattice_info r;
    r.material = LBM_BULK;
    r.block_iter = -1;
    r.vx = 0.0f;
    r.vy = 0.0f;
    if (scene == LBM_SCENE_CAVITY) {
        if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) r.material = LBM_BOUNDARY;
        if (y == 0 && x >= 1 && x <= nx - 2) r.vx = lid;
    } else if (scene == LBM_SCENE_CHANNEL) {
        if (y == 0 || y == ny - 1) {
            r.material = LBM_BOUNDARY;
        } else if (x == 0) {
            r.material = LBM_INLET;
            const double H = (double)(ny - 2), s = (double)y - 0.5;
            r.vx = (float)__ddiv_rn(__dmul_rn(__dmul_rn(__dmul_rn(4.0, (double)u_max), s), __dsub_rn(H, s)),
                                    __dmul_rn(H, H));
        } else if (x == nx - 1) {
            r.material = LBM_OUTLET;
        }
    }
    info[(size_t)y * nx + x] = r;
}

// one block per disk: the lattice points of its bounding box inside [1, nx-2] x [1, ny-2]
// with (x - cx)^2 + (y - cy)^2 <= r^2 become obstacles
// A disk's cells become obstacles.  With A non-null the lattice was initialised before the
// disks were drawn (lbm_create, lbm_reset): each disk cell also gets the state the
// initialisation gives a solid cell -- zero populations in both buffers (all-zero bits in every
// storage format, at pop_index of the handle's layout) and a zero macro value.
__global__ void k_raster_disks(lbm_lattice_info* __restrict__ info, int nx, int ny, const double* __restrict__ disks,
                               unsigned char* __restrict__ A, unsigned char* __restrict__ B, int elem_bytes,
                               bool tiled, float* __restrict__ macro) {
    const double cx = disks[3 * blockIdx.x], cy = disks[3 * blockIdx.x + 1], r = disks[3 * blockIdx.x + 2];
    const int x0 = (int)floor(__dsub_rn(cx, r)), x1 = (int)ceil(__dadd_rn(cx, r));
    const int y0 = (int)floor(__dsub_rn(cy, r)), y1 = (int)ceil(__dadd_rn(cy, r));
    const int w = x1 - x0 + 1, n = w * (y1 - y0 + 1);
    const double r2 = __dmul_rn(r, r);
    const size_t N = (size_t)nx * ny;
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        const int x = x0 + i % w, y = y0 + i / w;
        if (x < 1 || x > nx - 2 || y < 1 || y > ny - 2) continue;
        const double dx = __dsub_rn((double)x, cx), dy = __dsub_rn((double)y, cy);
        if (__dadd_rn(__dmul_rn(dx, dx), __dmul_rn(dy, dy)) > r2) continue;
        const size_t c = (size_t)y * nx + x;
        info[c].material = LBM_OBSTACLE;
        if (A) {
#pragma unroll
            for (int j = 0; j < 9; ++j) {
                const size_t b = pop_index(tiled, N, j, c) * (size_t)elem_bytes;
                if (elem_bytes == 2) {
                    *reinterpret_cast<uint16_t*>(A + b) = 0; *reinterpret_cast<uint16_t*>(B + b) = 0;
                } else if (elem_bytes == 4) {
                    *reinterpret_cast<uint32_t*>(A + b) = 0u; *reinterpret_cast<uint32_t*>(B + b) = 0u;
                } else {
                    *reinterpret_cast<uint64_t*>(A + b) = 0ull; *reinterpret_cast<uint64_t*>(B + b) = 0ull;
                }
            }
            macro[c] = 0.0f; macro[c + N] = 0.0f; macro[c + 2 * N] = 0.0f;
        }
    }
}

cudaError_t launch_build_scene(lbm_handle* h, cudaStream_t s) {
    const dim3 grid((unsigned)((h->nx + 255) / 256), (unsigned)h->ny);
    k_build_scene<<<grid, 256, 0, s>>>(h->d_info, h->nx, h->ny, h->p.scene, h->p.lid_speed, h->p.inlet_speed);
    return cudaGetLastError();
}

cudaError_t launch_raster_disks(lbm_handle* h, const double* d_disks, int ndisks, bool clear_state, cudaStream_t s) {
    if (ndisks <= 0) return cudaSuccess;
    k_raster_disks<<<(unsigned)ndisks, 256, 0, s>>>(
        h->d_info, h->nx, h->ny, d_disks, clear_state ? (unsigned char*)h->buf[h->cur] : nullptr,
        clear_state ? (unsigned char*)h->buf[h->cur ^ 1] : nullptr, (int)dtype_size(h->p.dtype), h->tiled, h->d_macro);
    return cudaGetLastError();
}

// ------------------------------------------------------------------------------------
// initialisation
// ------------------------------------------------------------------------------------
// init.wgsl:19-63
__global__ void k_ref_init(float* __restrict__ A, float* __restrict__ B, lbm_lattice_info* __restrict__ info,
                           uint16_t* __restrict__ flags, int nx, int ny, int fluid_ty, float* __restrict__ macro) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    const size_t N = (size_t)nx * ny;
    const size_t c = (size_t)y * nx + x;
    lbm_lattice_info in = info[c];
    if (is_solid(in.material)) {
#pragma unroll
        for (int i = 0; i < 9; ++i) { A[c + i * N] = 0.0f; B[c + i * N] = 0.0f; }
    } else if (fluid_ty == 0) {
#pragma unroll
        for (int i = 0; i < 9; ++i) { A[c + i * N] = REF_W(i); B[c + i * N] = 0.0f; }
        const float temp = __fmul_rn(REF_W(3), 0.5f);
        A[c + 1 * N] = __fadd_rn(REF_W(1), temp);
        A[c + 3 * N] = temp;
        B[c + 1 * N] = __fadd_rn(REF_W(1), temp);
        B[c + 3 * N] = temp;
    } else {
#pragma unroll
        for (int i = 0; i < 9; ++i) { A[c + i * N] = REF_W(i); B[c + i * N] = 0.0f; }
    }
    if ((in.material == LBM_INLET || in.material == LBM_EXTERNAL_FORCE) && in.block_iter > 0) {
        in.block_iter = 0;
        in.material = LBM_BULK;
        in.vx = 0.0f;
        in.vy = 0.0f;
        info[c] = in;
        flags[c] = (uint16_t)((flags[c] & ~FL_MAT_MASK) | LBM_BULK);
    }
    macro[c] = 0.0f;
    macro[c + N] = 0.0f;
    macro[c + 2 * N] = 0.0f;
}

template <class ST>
__global__ void k_phys_init(typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                            const lbm_lattice_info* __restrict__ info, const float* __restrict__ rho_in,
                            const float* __restrict__ ux_in, const float* __restrict__ uy_in, int nx, int ny,
                            float* __restrict__ macro, bool tiled) {
    using R = typename ST::R;
    const int x = blockIdx.x * blockDim.x + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    const size_t N = (size_t)nx * ny;
    const size_t c = (size_t)y * nx + x;
    if (is_solid(info[c].material)) {
#pragma unroll
        for (int i = 0; i < 9; ++i) {
            const size_t k = pop_index(tiled, N, i, c);
            ST::st(A + k, R(0));
            ST::st(B + k, R(0));
        }
        macro[c] = 0.0f; macro[c + N] = 0.0f; macro[c + 2 * N] = 0.0f;
        return;
    }
    const R rho = rho_in ? R(rho_in[c]) : R(1);
    const R ux = ux_in ? R(ux_in[c]) : R(0);
    const R uy = uy_in ? R(uy_in[c]) : R(0);
    const R drho = rho - R(1);
    const R usq = R(1.5) * (ux * ux + uy * uy);
#pragma unroll
    for (int i = 0; i < 9; ++i) {
        const R eu = R(EX(i)) * ux + R(EY(i)) * uy;
        const R d = PW<R>(i) * (drho + rho * (R(3) * eu + R(4.5) * (eu * eu) - usq));
        ST::st(A + pop_index(tiled, N, i, c), d);
    }
    // B's fluid cells are left as they are: every step writes all of them before anything reads
    // B (a step reads only the current buffer), and its solid cells, which no step writes, are
    // cleared above
    macro[c] = (float)rho; macro[c + N] = (float)ux; macro[c + 2 * N] = (float)uy;
}

// ------------------------------------------------------------------------------------
// reference-mode step: collide_stream.wgsl:25-88 + boundary.wgsl:3-35, one pass
//
// FAST = false (LBM_ARITH_EXACT): every WGSL operation rounded on its own, bit-identical to
// the oracle.  FAST = true (LBM_ARITH_FAST): the same rules -- truncated weights and maxima,
// rho clamp, forcing rows, population clamp, wall-cell storage -- with the moments summed as
// a tree, one correctly rounded reciprocal of rho instead of the IEEE divisions, the
// equilibrium of each opposite pair (j, inv j) split into the part even in e,
// rho w (1 - 1.5 u.u + 4.5 (e.u)^2), and the odd part 3 rho w (e.u), and multiply-adds left
// to the compiler: about half the instructions, so the step runs at memory speed.
// ------------------------------------------------------------------------------------
// resident blocks of TPB threads per SM the reference-mode step is compiled for (16: 32
// registers, full occupancy; both arithmetic forms fit without spills with 32-bit indices)
#ifndef LBM_REF_MIN_BLOCKS
#define LBM_REF_MIN_BLOCKS 16
#endif
template <bool MACRO, class IDX, bool FAST>
__global__ void __launch_bounds__(TPB, LBM_REF_MIN_BLOCKS) k_ref_step(const float* __restrict__ A, float* __restrict__ B,
                                                  uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                  float omega, int nx, int ny, float* __restrict__ macro) {
    const int x = blockIdx.x * TPB + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    const IDX N = (IDX)nx * (IDX)ny;
    const IDX c = (IDX)y * (IDX)nx + (IDX)x;
    // extents for the bounds-checked build: cells, population elements, macro elements
    const unsigned long long NC = (unsigned long long)N, NP = 9ull * NC, NM = 3ull * NC;
    const unsigned fl = in_bounds(c, NC, BS_REF_FLAGS) ? flags[c] : 0u;
    const int m = (int)(fl & FL_MAT_MASK);
    if (is_solid(m)) {  // collide_stream.wgsl:34-38
        if (MACRO && in_bounds(c + 2 * N, NM, BS_REF_MACRO)) {
            macro[c] = 0.0f; macro[c + N] = 0.0f; macro[c + 2 * N] = 0.0f;
        }
#pragma unroll
        for (int k = 0; k < 9; ++k)
            if ((fl & (1u << (FL_DIR_SHIFT + k))) && in_bounds(c + (IDX)k * N, NP, BS_REF_STORE))
                B[c + (IDX)k * N] = 0.0f;
        return;
    }
    // warp-uniform: no cell of the (active part of the) warp pushes into a wall slot or forces
    const bool plain = !(fl & (0x1FFu << FL_DIR_SHIFT)) && m != LBM_INLET && m != LBM_EXTERNAL_FORCE;
    const bool fast = __all_sync(__activemask(), plain);
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const IDX r0 = (IDX)y * (IDX)nx, rm = (IDX)ym * (IDX)nx, rp = (IDX)yp * (IDX)nx;
    float f[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {  // source uv - e(j), wrapped
        const int sx = EX(j) == 1 ? xm : (EX(j) == -1 ? xp : x);
        const IDX row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
        const IDX i = row + (IDX)sx + (IDX)j * N;
        f[j] = in_bounds(i, NP, BS_REF_PULL) ? __ldg(A + i) : 0.0f;
    }
    // collide_stream.wgsl:40-48
    float rho = 0.0f, vx = 0.0f, vy = 0.0f, inv = 0.0f;
    if constexpr (FAST) {
        rho = f[0] + (((f[1] + f[3]) + (f[2] + f[4])) + ((f[5] + f[7]) + (f[6] + f[8])));
        const float jx = (f[1] - f[3]) + ((f[5] - f[7]) + (f[8] - f[6]));
        const float jy = (f[4] - f[2]) + ((f[7] - f[5]) + (f[8] - f[6]));
        rho = fminf(fmaxf(rho, 0.8f), 1.2f);
        inv = __frcp_rn(rho);
        vx = jx * inv;
        vy = jy * inv;
    } else {
        // the terms e * f with e = 0 add a zero and those with e = +-1 add or subtract f
        // exactly, so they are written as such (populations are finite and clamped to
        // [0, max], so the values are those of the literal expressions; only the sign of an
        // exact zero may differ)
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            rho = __fadd_rn(rho, f[j]);
            if (EX(j) == 1) vx = __fadd_rn(vx, f[j]);
            if (EX(j) == -1) vx = __fsub_rn(vx, f[j]);
            if (EY(j) == 1) vy = __fadd_rn(vy, f[j]);
            if (EY(j) == -1) vy = __fsub_rn(vy, f[j]);
        }
        rho = fminf(fmaxf(rho, 0.8f), 1.2f);
        vx = __fdiv_rn(vx, rho);
        vy = __fdiv_rn(vy, rho);
    }
    float fx = 0.0f, fy = 0.0f;  // the forcing term F_j = 3 w_j (e_j . f) is 0 unless a force acts
    if (!fast && (m == LBM_INLET || m == LBM_EXTERNAL_FORCE) && in_bounds(c, NC, BS_REF_INFO)) {
        // collide_stream.wgsl:55-71
        lbm_lattice_info in = info[c];
        if (in.block_iter > 0) {
            in.block_iter = in.block_iter - 1;
            if (in.block_iter == 0) {
                in.material = LBM_BULK;
                flags[c] = (uint16_t)((fl & ~FL_MAT_MASK) | LBM_BULK);
            }
            info[c] = in;
        }
        fx = in.vx;
        fy = in.vy;
        if constexpr (FAST) {
            vx = (0.5f * fx) * inv;
            vy = (0.5f * fy) * inv;
        } else {
            vx = __fdiv_rn(__fmul_rn(fx, 0.5f), rho);
            vy = __fdiv_rn(__fmul_rn(fy, 0.5f), rho);
        }
    }
    if (MACRO && in_bounds(c + 2 * N, NM, BS_REF_MACRO)) { macro[c] = rho; macro[c + N] = vx; macro[c + 2 * N] = vy; }
    float t[9];
    if constexpr (FAST) {
        // t_j = (1 - omega) f_j + omega feq_j, feq of the pair (j, k = inv j) = sym +- asy
        const float usqr = 1.5f * (vx * vx + vy * vy);
        const float base = 1.0f - usqr, om1 = 1.0f - omega;
        const float ow0 = omega * (rho * REF_W(0)), ow1 = omega * (rho * REF_W(1)), ow5 = omega * (rho * REF_W(5));
        t[0] = om1 * f[0] + ow0 * base;
        auto pair = [&](int j, int k, float eu, float ow) {
            const float sym = ow * (base + (4.5f * eu) * eu);
            const float asy = (3.0f * ow) * eu;
            t[j] = om1 * f[j] + (sym + asy);
            t[k] = om1 * f[k] + (sym - asy);
        };
        pair(1, 3, vx, ow1);
        pair(4, 2, vy, ow1);
        pair(8, 6, vx + vy, ow5);
        pair(5, 7, vx - vy, ow5);
    } else {
        const float usqr = __fmul_rn(1.5f, __fadd_rn(__fmul_rn(vx, vx), __fmul_rn(vy, vy)));
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            // e . u with e_x, e_y in {-1, 0, 1}: the same value as the literal products and sum
            const float ex = EX(j) == 1 ? vx : (EX(j) == -1 ? -vx : 0.0f);
            const float ey = EY(j) == 1 ? vy : (EY(j) == -1 ? -vy : 0.0f);
            const float eu = (EX(j) == 0) ? ey : ((EY(j) == 0) ? ex : __fadd_rn(ex, ey));
            const float feq = __fmul_rn(
                __fmul_rn(rho, REF_W(j)),
                __fsub_rn(__fadd_rn(__fadd_rn(1.0f, __fmul_rn(3.0f, eu)), __fmul_rn(4.5f, __fmul_rn(eu, eu))), usqr));
            t[j] = __fsub_rn(f[j], __fmul_rn(omega, __fsub_rn(f[j], feq)));
        }
    }
    if (fast) {
        // no cell of the warp forces or pushes into a wall slot: clamp (collide_stream.wgsl:79-83)
        // and store, one warp-uniform branch for all nine directions (with `fast` tested per
        // direction inside the general loop below the exact form ran 14 % slower at 8192^2)
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            float v = t[j];
            if (v > REF_MAX(j)) v = REF_MAX(j);
            else if (v < 0.0f) v = 0.0f;
            const IDX own = c + (IDX)j * N;
            if (in_bounds(own, NP, BS_REF_STORE)) B[own] = v;
        }
        return;
    }
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        float v = t[j];
        // + F_j (+-0 when no force acts: the value is unchanged)
        if constexpr (FAST)
            v = v + (3.0f * REF_W(j)) * ((float)EX(j) * fx + (float)EY(j) * fy);
        else
            v = __fadd_rn(v, __fmul_rn(__fmul_rn(REF_W(j), 3.0f),
                                       __fadd_rn(__fmul_rn((float)EX(j), fx), __fmul_rn((float)EY(j), fy))));
        if (v > REF_MAX(j)) v = REF_MAX(j);  // collide_stream.wgsl:79-83
        else if (v < 0.0f) v = 0.0f;
        const IDX own = c + (IDX)j * N;
        if (fl & (1u << (FL_DIR_SHIFT + j))) {
            const IDX wall = c + (IDX)(EY(j) * nx + EX(j)) + (IDX)INV(j) * N;
            if (in_bounds(wall, NP, BS_REF_WALL)) B[wall] = v;
            if (in_bounds(own, NP, BS_REF_STORE)) B[own] = 0.0f;
        } else if (in_bounds(own, NP, BS_REF_STORE)) {
            B[own] = v;
        }
    }
}

// ------------------------------------------------------------------------------------
// physics-mode step (cell update in lbm_cell.cuh)
// ------------------------------------------------------------------------------------
// BGK and regularised fit 32 registers (full occupancy); MRT and KBC get 48
// (SR: stochastic rounding of 16-bit stores, seed from the step counter)
template <class ST, bool MACRO, int COLL, bool SR>
__global__ void __launch_bounds__(TPB, (COLL == LBM_COLLISION_MRT || COLL == LBM_COLLISION_KBC) ? 10 : 16) k_phys_step(const typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                                                   uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                   typename ST::R omega, int nx, int ny, float* __restrict__ macro,
                                                   uint32_t seed) {
    const int x = blockIdx.x * TPB + threadIdx.x;
    const int y = blockIdx.y;
    if (x >= nx) return;
    phys_cell_update<ST, MACRO, COLL, SR>(A, B, flags, info, omega, x, y, nx, nx, ny, macro, seed);
}

// ------------------------------------------------------------------------------------
// FP64 reductions (fixed grid, fixed order -> deterministic)
// ------------------------------------------------------------------------------------
template <int K>
__device__ __forceinline__ void block_reduce_sum(double (&v)[K], double* smem /* K * 32 */) {
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

template <class ST, int MODE>
__global__ void __launch_bounds__(RED_TPB) k_conservation(const typename ST::T* __restrict__ A,
                                                          const uint16_t* __restrict__ flags, size_t N,
                                                          double* __restrict__ part, bool tiled = false) {
    __shared__ double smem[3 * 32];
    double v[3] = {0.0, 0.0, 0.0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += stride) {
        const bool solid = is_solid((int)(flags[c] & FL_MAT_MASK));
        if (MODE == LBM_MODE_PHYSICS && solid) continue;
        if (MODE == LBM_MODE_PHYSICS) v[0] += 1.0;
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const double f = (double)ST::to_r(A[pop_index(tiled, N, j, c)]);
            v[0] += f;
            v[1] += (double)EX(j) * f;
            v[2] += (double)EY(j) * f;
        }
    }
    block_reduce_sum<3>(v, smem);
    if (threadIdx.x == 0) {
        part[blockIdx.x * 3 + 0] = v[0];
        part[blockIdx.x * 3 + 1] = v[1];
        part[blockIdx.x * 3 + 2] = v[2];
    }
}

template <int K>
__global__ void __launch_bounds__(RED_TPB) k_final_sum(const double* __restrict__ part, int nparts,
                                                       double* __restrict__ out) {
    __shared__ double smem[K * 32];
    double v[K];
#pragma unroll
    for (int k = 0; k < K; ++k) v[k] = 0.0;
    for (int b = threadIdx.x; b < nparts; b += blockDim.x)
#pragma unroll
        for (int k = 0; k < K; ++k) v[k] += part[b * K + k];
    block_reduce_sum<K>(v, smem);
    if (threadIdx.x == 0)
#pragma unroll
        for (int k = 0; k < K; ++k) out[k] = v[k];
}

template <class ST>
__global__ void k_count_nonfinite(const typename ST::T* __restrict__ A, size_t total, unsigned long long* count) {
    unsigned long long local = 0;
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < total; i += stride) {
        const double v = (double)ST::to_r(A[i]);
        if (!isfinite(v)) ++local;
    }
    for (int o = 16; o > 0; o >>= 1) local += __shfl_down_sync(0xffffffffu, local, o);
    if ((threadIdx.x & 31) == 0 && local) atomicAdd(count, local);
}

// sums over non-solid cells of h: |drho|^2, |rho_ref|^2, |du|^2, |u_ref|^2, then maxima
__global__ void __launch_bounds__(RED_TPB) k_macro_error(const float* __restrict__ m, const float* __restrict__ mref,
                                                         const uint16_t* __restrict__ flags, size_t N,
                                                         double* __restrict__ part) {
    __shared__ double smem[6 * 32];
    double v[6] = {0, 0, 0, 0, 0, 0};
    const size_t stride = (size_t)gridDim.x * blockDim.x;
    for (size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x; c < N; c += stride) {
        if (is_solid((int)(flags[c] & FL_MAT_MASK))) continue;
        const double r = m[c], rr = mref[c];
        const double ux = m[c + N], uy = m[c + 2 * N], rux = mref[c + N], ruy = mref[c + 2 * N];
        const double dr = r - rr, dux = ux - rux, duy = uy - ruy;
        v[0] += dr * dr;
        v[1] += rr * rr;
        v[2] += dux * dux + duy * duy;
        v[3] += rux * rux + ruy * ruy;
        v[4] = fmax(v[4], sqrt(dux * dux + duy * duy));
        v[5] = fmax(v[5], fabs(dr));
    }
    // sums
    double s[4] = {v[0], v[1], v[2], v[3]};
    block_reduce_sum<4>(s, smem);
    __syncthreads();
    // maxima
    double mx[2] = {v[4], v[5]};
#pragma unroll
    for (int k = 0; k < 2; ++k)
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) mx[k] = fmax(mx[k], __shfl_down_sync(0xffffffffu, mx[k], o));
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    if (lane == 0) { smem[warp] = mx[0]; smem[32 + warp] = mx[1]; }
    __syncthreads();
    if (threadIdx.x == 0) {
        double a = 0, b = 0;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) { a = fmax(a, smem[w]); b = fmax(b, smem[32 + w]); }
        part[blockIdx.x * 6 + 0] = s[0];
        part[blockIdx.x * 6 + 1] = s[1];
        part[blockIdx.x * 6 + 2] = s[2];
        part[blockIdx.x * 6 + 3] = s[3];
        part[blockIdx.x * 6 + 4] = a;
        part[blockIdx.x * 6 + 5] = b;
    }
}

__global__ void k_macro_error_final(const double* __restrict__ part, int nparts, double* __restrict__ out) {
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    double s[4] = {0, 0, 0, 0}, a = 0, b = 0;
    for (int i = 0; i < nparts; ++i) {
        for (int k = 0; k < 4; ++k) s[k] += part[i * 6 + k];
        a = fmax(a, part[i * 6 + 4]);
        b = fmax(b, part[i * 6 + 5]);
    }
    out[0] = s[1] > 0 ? sqrt(s[0] / s[1]) : sqrt(s[0]);
    out[1] = s[3] > 0 ? sqrt(s[2] / s[3]) : sqrt(s[2]);
    out[2] = a;
    out[3] = b;
}

// ------------------------------------------------------------------------------------
// conversions
// ------------------------------------------------------------------------------------
__global__ void k_macro_rgba16f(const float* __restrict__ macro, const uint16_t* __restrict__ flags, size_t N,
                                int stepped, ushort4* __restrict__ out) {
    const size_t c = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (c >= N) return;
    const bool solid = is_solid((int)(flags[c] & FL_MAT_MASK));
    ushort4 o;
    o.x = __half_as_ushort(__float2half_rn(macro[c + N]));
    o.y = __half_as_ushort(__float2half_rn(macro[c + 2 * N]));
    o.z = __half_as_ushort(__float2half_rn(macro[c]));
    o.w = __half_as_ushort(__float2half_rn((stepped && solid) ? 0.0f : 1.0f));
    out[c] = o;
}

// dst / src: SoA host-order arrays (direction j of cell c at j * N + c) whatever the state's layout
template <class ST, class D>
__global__ void k_to_absolute(const typename ST::T* __restrict__ s, D* __restrict__ dst, size_t N, int mode,
                              bool tiled) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * N) return;
    const int j = (int)(i / N);
    using R = typename ST::R;
    const R v = ST::to_r(s[pop_index(tiled, N, j, i - (size_t)j * N)]);
    if (mode == LBM_MODE_REFERENCE) dst[i] = (D)v;
    else dst[i] = (D)PW<D>(j) + (D)v;
}

template <class ST, class D>
__global__ void k_from_absolute(const D* __restrict__ src, typename ST::T* __restrict__ s, size_t N, int mode,
                                bool tiled) {
    const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= 9 * N) return;
    const int j = (int)(i / N);
    using R = typename ST::R;
    const size_t k = pop_index(tiled, N, j, i - (size_t)j * N);
    if (mode == LBM_MODE_REFERENCE) s[k] = ST::from_r((R)src[i]);
    else s[k] = ST::from_r((R)(src[i] - PW<D>(j)));
}

// ------------------------------------------------------------------------------------
// batched interactive edits: the result of applying, in sequence order, obstacle discs
// (d2q9_node.rs:215-245: the disc goes into the host copy of the mask and rows [y-28, y+28)
// of that copy overwrite the device mask) and force-stroke cells (d2q9_node.rs:263-300: one
// record per cell written to the device mask only).  For a cell of an obstacle row, the last
// obstacle whose rows hold it decides its value: the obstacle record if a disc of that or an
// earlier obstacle covers it, else the host copy; a force cell keeps its record unless a
// later obstacle's rows hold it.
// ------------------------------------------------------------------------------------
__device__ __forceinline__ bool in_obstacle_disc(int x, int y, int ox, int oy) {
    // fluid/mod.rs:57-59 with the cell centres of d2q9_node.rs:222-229
    const float px = __fsub_rn(__fadd_rn((float)x, 0.5f), __fadd_rn((float)ox, 0.5f));
    const float py = __fsub_rn(__fadd_rn((float)y, 0.5f), __fadd_rn((float)oy, 0.5f));
    return __fsqrt_rn(__fadd_rn(__fmul_rn(px, px), __fmul_rn(py, py))) <= 28.0f;
}

__global__ void k_edit_obstacles(lbm_lattice_info* __restrict__ info, lbm_lattice_info* __restrict__ host_copy,
                                 const EditObstacle* __restrict__ ob, int nobst, int nx, int row0) {
    const int x = blockIdx.x * blockDim.x + threadIdx.x, y = row0 + (int)blockIdx.y;
    if (x >= nx) return;
    int last = -1;
    bool cover_any = false, cover_last = false;
    for (int j = 0; j < nobst; ++j) {
        const EditObstacle o = ob[j];
        const bool row = y >= o.y - 28 && y < o.y + 28;
        const bool disc = row && in_obstacle_disc(x, y, o.x, o.y);
        cover_any |= disc;
        if (row) {
            last = j;
            cover_last = cover_any;
        }
    }
    if (last < 0) return;
    const size_t c = (size_t)y * nx + x;
    lbm_lattice_info obst;
    obst.material = LBM_OBSTACLE;
    obst.block_iter = -1;
    obst.vx = 0.0f;
    obst.vy = 0.0f;
    const lbm_lattice_info orig = host_copy[c];
    info[c] = cover_last ? obst : orig;
    if (cover_any) host_copy[c] = obst;
}

__global__ void k_edit_forces(lbm_lattice_info* __restrict__ info, const EditObstacle* __restrict__ ob, int nobst,
                              const EditForce* __restrict__ fc, int nforce, int nx) {
    const int k = blockIdx.x * blockDim.x + threadIdx.x;
    if (k >= nforce) return;
    const EditForce f = fc[k];
    const int y = (int)(f.cell / (uint32_t)nx);
    for (int j = 0; j < nobst; ++j)
        if (ob[j].seq > f.seq && y >= ob[j].y - 28 && y < ob[j].y + 28) return;
    lbm_lattice_info r;
    r.material = LBM_EXTERNAL_FORCE;
    r.block_iter = 90;
    r.vx = f.vx;
    r.vy = f.vy;
    info[f.cell] = r;
}

// ------------------------------------------------------------------------------------
// launchers
// ------------------------------------------------------------------------------------
static inline dim3 cell_grid(const lbm_handle* h) { return dim3((unsigned)((h->nx + TPB - 1) / TPB), (unsigned)h->ny); }

cudaError_t launch_edits(lbm_handle* h, const EditObstacle* d_obst, int nobst, const EditForce* d_force, int nforce,
                         int row0, int row1, cudaStream_t s) {
    if (nobst > 0 && row1 > row0) {
        k_edit_obstacles<<<dim3((unsigned)((h->nx + TPB - 1) / TPB), (unsigned)(row1 - row0)), TPB, 0, s>>>(
            h->d_info, h->d_host_info, d_obst, nobst, h->nx, row0);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    if (nforce > 0) {
        k_edit_forces<<<(nforce + 127) / 128, 128, 0, s>>>(h->d_info, d_obst, nobst, d_force, nforce, h->nx);
        cudaError_t e = cudaGetLastError();
        if (e != cudaSuccess) return e;
    }
    return cudaSuccess;
}

cudaError_t launch_build_flags(const lbm_handle* h, cudaStream_t s) {
    k_build_flags<<<cell_grid(h), TPB, 0, s>>>(h->d_info, h->d_flags, h->nx, h->ny, h->p.mode);
    return cudaGetLastError();
}

cudaError_t launch_ref_init(lbm_handle* h, cudaStream_t s) {
    k_ref_init<<<cell_grid(h), TPB, 0, s>>>((float*)h->buf[0], (float*)h->buf[1], h->d_info, h->d_flags, h->nx, h->ny,
                                             h->fluid_ty, h->d_macro);
    return cudaGetLastError();
}

template <class ST>
static cudaError_t phys_init_t(lbm_handle* h, const float* r, const float* ux, const float* uy, cudaStream_t s) {
    k_phys_init<ST><<<cell_grid(h), TPB, 0, s>>>((typename ST::T*)h->buf[0], (typename ST::T*)h->buf[1], h->d_info, r, ux,
                                                 uy, h->nx, h->ny, h->d_macro, h->tiled);
    return cudaGetLastError();
}

cudaError_t launch_phys_init(lbm_handle* h, const float* r, const float* ux, const float* uy, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return phys_init_t<StoreF32>(h, r, ux, uy, s);
        case LBM_DTYPE_F64: return phys_init_t<StoreF64>(h, r, ux, uy, s);
        case LBM_DTYPE_F16: return phys_init_t<StoreF16>(h, r, ux, uy, s);
        default: return phys_init_t<StoreBF16>(h, r, ux, uy, s);
    }
}

template <class ST, bool MACRO, int COLL>
static cudaError_t phys_step_c(lbm_handle* h, cudaStream_t s) {
    using T = typename ST::T;
    using R = typename ST::R;
    const R omega = sizeof(R) == 8 ? (R)h->omega_d : (R)h->omega;
    // stochastic rounding exists for 16-bit storage only (validated at create)
    constexpr bool SIXTEEN = ST::dtype == LBM_DTYPE_F16 || ST::dtype == LBM_DTYPE_BF16;
    if (SIXTEEN && h->p.rounding == LBM_ROUNDING_STOCHASTIC)
        k_phys_step<ST, MACRO, COLL, SIXTEEN><<<cell_grid(h), TPB, 0, s>>>(
            (const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1], h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro,
            sr_seed(h->steps, h->p.seed));
    else
        k_phys_step<ST, MACRO, COLL, false><<<cell_grid(h), TPB, 0, s>>>(
            (const T*)h->buf[h->cur], (T*)h->buf[h->cur ^ 1], h->d_flags, h->d_info, omega, h->nx, h->ny, h->d_macro, 0u);
    return cudaGetLastError();
}

// the collision is a compile-time choice so that each rule gets its own register budget
template <class ST, bool MACRO>
static cudaError_t phys_step_t(lbm_handle* h, cudaStream_t s) {
    switch (h->p.collision) {
        case LBM_COLLISION_REGULARIZED: return phys_step_c<ST, MACRO, LBM_COLLISION_REGULARIZED>(h, s);
        case LBM_COLLISION_MRT: return phys_step_c<ST, MACRO, LBM_COLLISION_MRT>(h, s);
        case LBM_COLLISION_KBC: return phys_step_c<ST, MACRO, LBM_COLLISION_KBC>(h, s);
        default: return phys_step_c<ST, MACRO, LBM_COLLISION_BGK>(h, s);
    }
}

template <bool MACRO, class IDX, bool FAST>
static cudaError_t ref_step_t(lbm_handle* h, cudaStream_t s) {
    k_ref_step<MACRO, IDX, FAST><<<cell_grid(h), TPB, 0, s>>>((const float*)h->buf[h->cur], (float*)h->buf[h->cur ^ 1],
                                                              h->d_flags, h->d_info, h->omega, h->nx, h->ny, h->d_macro);
    return cudaGetLastError();
}

cudaError_t launch_step(lbm_handle* h, bool write_macro, cudaStream_t s) {
    if (h->p.mode == LBM_MODE_REFERENCE) {
        const bool idx32 = (size_t)9 * h->N < ((size_t)1 << 32);
        if (h->p.arith == LBM_ARITH_FAST)
            return idx32 ? (write_macro ? ref_step_t<true, uint32_t, true>(h, s) : ref_step_t<false, uint32_t, true>(h, s))
                         : (write_macro ? ref_step_t<true, size_t, true>(h, s) : ref_step_t<false, size_t, true>(h, s));
        return idx32 ? (write_macro ? ref_step_t<true, uint32_t, false>(h, s) : ref_step_t<false, uint32_t, false>(h, s))
                     : (write_macro ? ref_step_t<true, size_t, false>(h, s) : ref_step_t<false, size_t, false>(h, s));
    }
    // auto = the fastest variant measured on GB300: one cell per thread for FP32 and FP64
    // (94.9 % of the HBM copy bandwidth at 4096^2 FP32, against 70.9 % for VEC4 and 68.6 % for
    // BULK), two cells per thread for 16-bit storage (130 against 112 GLUPS at 8192^2 FP16)
    if (h->p.collision != LBM_COLLISION_BGK) {  // the vector kernels implement BGK only
        switch (h->p.dtype) {
            case LBM_DTYPE_F32: return write_macro ? phys_step_t<StoreF32, true>(h, s) : phys_step_t<StoreF32, false>(h, s);
            case LBM_DTYPE_F64: return write_macro ? phys_step_t<StoreF64, true>(h, s) : phys_step_t<StoreF64, false>(h, s);
            case LBM_DTYPE_F16: return write_macro ? phys_step_t<StoreF16, true>(h, s) : phys_step_t<StoreF16, false>(h, s);
            default: return write_macro ? phys_step_t<StoreBF16, true>(h, s) : phys_step_t<StoreBF16, false>(h, s);
        }
    }
    if (h->tiled)
        return h->p.kernel == LBM_KERNEL_RING ? launch_phys_step_ring(h, write_macro, s)
                                              : launch_phys_step_tiled(h, write_macro, s);
    if (h->p.kernel == LBM_KERNEL_BULK) return launch_phys_step_bulk(h, write_macro, s);
    if (h->p.kernel == LBM_KERNEL_VEC4) return launch_phys_step_vec(h, write_macro, s);
    if (h->p.kernel == LBM_KERNEL_VEC2) return launch_phys_step_vec2(h, write_macro, s);
    if (h->p.kernel == LBM_KERNEL_AUTO && (h->p.dtype == LBM_DTYPE_F16 || h->p.dtype == LBM_DTYPE_BF16) &&
        h->nx % 2 == 0)
        return launch_phys_step_vec2(h, write_macro, s);
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return write_macro ? phys_step_t<StoreF32, true>(h, s) : phys_step_t<StoreF32, false>(h, s);
        case LBM_DTYPE_F64: return write_macro ? phys_step_t<StoreF64, true>(h, s) : phys_step_t<StoreF64, false>(h, s);
        case LBM_DTYPE_F16: return write_macro ? phys_step_t<StoreF16, true>(h, s) : phys_step_t<StoreF16, false>(h, s);
        default: return write_macro ? phys_step_t<StoreBF16, true>(h, s) : phys_step_t<StoreBF16, false>(h, s);
    }
}

template <class ST>
static cudaError_t conservation_t(lbm_handle* h, double* out, cudaStream_t s) {
    const auto* A = (const typename ST::T*)h->buf[h->cur];
    if (h->p.mode == LBM_MODE_REFERENCE)
        k_conservation<ST, LBM_MODE_REFERENCE><<<RED_BLOCKS, RED_TPB, 0, s>>>(A, h->d_flags, h->N, h->d_part, h->tiled);
    else
        k_conservation<ST, LBM_MODE_PHYSICS><<<RED_BLOCKS, RED_TPB, 0, s>>>(A, h->d_flags, h->N, h->d_part, h->tiled);
    k_final_sum<3><<<1, RED_TPB, 0, s>>>(h->d_part, RED_BLOCKS, out);
    return cudaGetLastError();
}

cudaError_t launch_conservation(lbm_handle* h, double* out, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return conservation_t<StoreF32>(h, out, s);
        case LBM_DTYPE_F64: return conservation_t<StoreF64>(h, out, s);
        case LBM_DTYPE_F16: return conservation_t<StoreF16>(h, out, s);
        default: return conservation_t<StoreBF16>(h, out, s);
    }
}

cudaError_t launch_conservation_f32_phys(const float* A, const uint16_t* flags, size_t N, double* part, double* out,
                                         cudaStream_t s) {
    k_conservation<StoreF32, LBM_MODE_PHYSICS><<<RED_BLOCKS, RED_TPB, 0, s>>>(A, flags, N, part);
    k_final_sum<3><<<1, RED_TPB, 0, s>>>(part, RED_BLOCKS, out);
    return cudaGetLastError();
}

cudaError_t launch_count_nonfinite(lbm_handle* h, cudaStream_t s) {
    cudaError_t e = cudaMemsetAsync(h->d_count, 0, sizeof(unsigned long long), s);
    if (e != cudaSuccess) return e;
    const size_t total = 9 * h->N;
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: k_count_nonfinite<StoreF32><<<RED_BLOCKS, RED_TPB, 0, s>>>((const float*)h->buf[h->cur], total, h->d_count); break;
        case LBM_DTYPE_F64: k_count_nonfinite<StoreF64><<<RED_BLOCKS, RED_TPB, 0, s>>>((const double*)h->buf[h->cur], total, h->d_count); break;
        case LBM_DTYPE_F16: k_count_nonfinite<StoreF16><<<RED_BLOCKS, RED_TPB, 0, s>>>((const __half*)h->buf[h->cur], total, h->d_count); break;
        default: k_count_nonfinite<StoreBF16><<<RED_BLOCKS, RED_TPB, 0, s>>>((const __nv_bfloat16*)h->buf[h->cur], total, h->d_count); break;
    }
    return cudaGetLastError();
}

cudaError_t launch_macro_error(lbm_handle* h, lbm_handle* ref, double* out, cudaStream_t s) {
    k_macro_error<<<RED_BLOCKS, RED_TPB, 0, s>>>(h->d_macro, ref->d_macro, h->d_flags, h->N, h->d_part);
    k_macro_error_final<<<1, 32, 0, s>>>(h->d_part, RED_BLOCKS, out);
    return cudaGetLastError();
}

cudaError_t launch_macro_rgba16f(lbm_handle* h, uint16_t* d_rgba, cudaStream_t s) {
    const unsigned blocks = (unsigned)((h->N + 255) / 256);
    k_macro_rgba16f<<<blocks, 256, 0, s>>>(h->d_macro, h->d_flags, h->N, h->stepped_since_init ? 1 : 0, (ushort4*)d_rgba);
    return cudaGetLastError();
}

template <class ST>
static cudaError_t to_abs_t(lbm_handle* h, const void* state, void* dst, int dd, cudaStream_t s) {
    const unsigned blocks = (unsigned)((9 * h->N + 255) / 256);
    if (dd == LBM_DTYPE_F64)
        k_to_absolute<ST, double><<<blocks, 256, 0, s>>>((const typename ST::T*)state, (double*)dst, h->N, h->p.mode,
                                                         h->tiled);
    else
        k_to_absolute<ST, float><<<blocks, 256, 0, s>>>((const typename ST::T*)state, (float*)dst, h->N, h->p.mode,
                                                        h->tiled);
    return cudaGetLastError();
}

cudaError_t launch_to_absolute(lbm_handle* h, const void* state, void* dst, int dd, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return to_abs_t<StoreF32>(h, state, dst, dd, s);
        case LBM_DTYPE_F64: return to_abs_t<StoreF64>(h, state, dst, dd, s);
        case LBM_DTYPE_F16: return to_abs_t<StoreF16>(h, state, dst, dd, s);
        default: return to_abs_t<StoreBF16>(h, state, dst, dd, s);
    }
}

template <class ST>
static cudaError_t from_abs_t(lbm_handle* h, const void* src, int sd, void* state, cudaStream_t s) {
    const unsigned blocks = (unsigned)((9 * h->N + 255) / 256);
    if (sd == LBM_DTYPE_F64)
        k_from_absolute<ST, double><<<blocks, 256, 0, s>>>((const double*)src, (typename ST::T*)state, h->N, h->p.mode,
                                                           h->tiled);
    else
        k_from_absolute<ST, float><<<blocks, 256, 0, s>>>((const float*)src, (typename ST::T*)state, h->N, h->p.mode,
                                                          h->tiled);
    return cudaGetLastError();
}

cudaError_t launch_from_absolute(lbm_handle* h, const void* src, int sd, void* state, cudaStream_t s) {
    switch (h->p.dtype) {
        case LBM_DTYPE_F32: return from_abs_t<StoreF32>(h, src, sd, state, s);
        case LBM_DTYPE_F64: return from_abs_t<StoreF64>(h, src, sd, state, s);
        case LBM_DTYPE_F16: return from_abs_t<StoreF16>(h, src, sd, state, s);
        default: return from_abs_t<StoreBF16>(h, src, sd, state, s);
    }
}

#ifdef LBM_BOUNDS_CHECK
cudaError_t bounds_take_kernels(BoundsRecord* out) { return bounds_take_local(out); }

__global__ void k_bounds_selftest() {
    if (threadIdx.x == 0 && blockIdx.x == 0) (void)in_bounds(7ull, 7ull, BS_SELFTEST);
}

cudaError_t bounds_selftest(cudaStream_t s) {
    k_bounds_selftest<<<1, 32, 0, s>>>();
    return cudaGetLastError();
}
#endif

}  // namespace lbm
