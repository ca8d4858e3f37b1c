// lbm_cell.cuh -- the physics-mode update of one cell, shared by the single-lattice step
// kernel (lbm_kernels.cu) and the batched persistent kernel (lbm_batch.cu).
//
// Pull streaming with half-way bounce-back (a moving wall adds 6 w_j (e_j . u_w), wall
// density 1), Zou-He velocity inlet on a west face, zero-gradient outflow on an east face
// anchored at rho = 1, Guo forcing with the reference's block_iter countdown
// (collide_stream.wgsl:55-62), BGK with exact weights.  Populations are stored as
// deviations d = f - w; the rest population is computed from mass conservation so that
// sum_j o_j equals the pulled density deviation exactly up to rounding.
#pragma once

#include "lbm_common.cuh"

namespace lbm {

// Boundary rules on the pulled populations d (Zou-He inlet, anchored outflow), moments,
// Guo forcing with countdown, BGK.  o receives the post-collision deviations; rho, ux, uy
// the macroscopic values of the cell.
template <class R>
__device__ __forceinline__ void phys_collide(R (&d)[9], int m, unsigned fl, size_t c, uint16_t* __restrict__ flags,
                                             lbm_lattice_info* __restrict__ info, R omega, R (&o)[9], R& rho_out,
                                             R& ux_out, R& uy_out) {
    const bool outlet = (m == LBM_OUTLET);
    if (m == LBM_INLET) {  // Zou-He velocity inlet, west face: unknowns 1, 5, 8
        const lbm_lattice_info in = info[c];
        const R ux = R(in.vx), uy = R(in.vy);
        const R S = d[0] + d[2] + d[4] + R(2) * (d[3] + d[6] + d[7]);
        const R rho = (R(1) + S) / (R(1) - ux);
        const R rux = rho * ux, ruy = rho * uy;
        d[1] = d[3] + (R(2) / R(3)) * rux;
        d[5] = d[7] + R(0.5) * (d[4] - d[2]) + rux / R(6) - R(0.5) * ruy;
        d[8] = d[6] + R(0.5) * (d[2] - d[4]) + rux / R(6) + R(0.5) * ruy;
    }
    if (outlet) {  // zero-gradient outflow anchored at rho = 1: f_j <- f_j / rho
        const R dr = d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7] + d[8];
        const R inv = R(1) / (R(1) + dr);
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j] = (d[j] - PW<R>(j) * dr) * inv;
    }
    const R drho = d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7] + d[8];
    R jx = (d[1] - d[3]) + (d[5] - d[6]) + (d[8] - d[7]);
    R jy = (d[4] - d[2]) + (d[7] - d[5]) + (d[8] - d[6]);
    const R rho = R(1) + drho;
    R Fx = R(0), Fy = R(0);
    const bool forced = (m == LBM_EXTERNAL_FORCE);
    if (forced) {  // Guo forcing with the reference's block_iter countdown
        lbm_lattice_info in = info[c];
        if (in.block_iter > 0) {
            in.block_iter = in.block_iter - 1;
            if (in.block_iter == 0) {
                in.material = LBM_BULK;
                flags[c] = (uint16_t)((fl & ~FL_MAT_MASK) | LBM_BULK);
            }
            info[c] = in;
        }
        Fx = R(in.vx);
        Fy = R(in.vy);
        jx = jx + R(0.5) * Fx;
        jy = jy + R(0.5) * Fy;
    }
    const R ux = jx / rho, uy = jy / rho;
    const R usq = R(1.5) * (ux * ux + uy * uy);
    const R gf = R(1) - R(0.5) * omega;
#pragma unroll
    for (int j = 1; j < 9; ++j) {
        const R ex = R(EX(j)), ey = R(EY(j));
        const R eu = ex * ux + ey * uy;
        const R deq = PW<R>(j) * (drho + rho * (R(3) * eu + R(4.5) * (eu * eu) - usq));
        R out = d[j] - omega * (d[j] - deq);
        if (forced) {
            const R eF = ex * Fx + ey * Fy;
            const R uF = ux * Fx + uy * Fy;
            out = out + gf * PW<R>(j) * (R(3) * (eF - uF) + R(9) * eu * eF);
        }
        o[j] = out;
    }
    o[0] = drho - (((o[1] + o[3]) + (o[2] + o[4])) + ((o[5] + o[7]) + (o[6] + o[8])));
    rho_out = rho;
    ux_out = ux;
    uy_out = uy;
}

template <class ST, bool MACRO>
__device__ __forceinline__ void phys_cell_update(const typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                                                 uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                 typename ST::R omega, int x, int y, int nx, int ny,
                                                 float* __restrict__ macro) {
    using R = typename ST::R;
    const size_t N = (size_t)nx * ny;
    const size_t c = (size_t)y * nx + x;
    const unsigned fl = flags[c];
    const int m = (int)(fl & FL_MAT_MASK);
    if (is_solid(m)) {
        if (MACRO) { macro[c] = 0.0f; macro[c + N] = 0.0f; macro[c + 2 * N] = 0.0f; }
        return;
    }
    const bool outlet = (m == LBM_OUTLET);
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const size_t r0 = (size_t)y * nx, rm = (size_t)ym * nx, rp = (size_t)yp * nx;
    R d[9];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const int sx = EX(j) == 1 ? xm : (EX(j) == -1 ? (outlet ? x : xp) : x);
        const size_t row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
        if (fl & (1u << (FL_DIR_SHIFT + j))) {
            R v = ST::ld(A + c + (size_t)INV(j) * N);  // half-way bounce-back
            if (fl & FL_MOVING) {
                const lbm_lattice_info si = info[row + sx];
                const R uw = R(EX(j)) * R(si.vx) + R(EY(j)) * R(si.vy);
                // rounded product, not an FMA: a contracted wall term leaves a
                // systematic mass drift of ~1e-12 per step in FP32
                if (uw != R(0)) v = add_rn(v, mul_rn(R(6) * PW<R>(j), uw));
            }
            d[j] = v;
        } else {
            d[j] = ST::ld(A + row + sx + (size_t)j * N);
        }
    }
    R o[9], rho, ux, uy;
    phys_collide<R>(d, m, fl, c, flags, info, omega, o, rho, ux, uy);
    if (MACRO) { macro[c] = (float)rho; macro[c + N] = (float)ux; macro[c + 2 * N] = (float)uy; }
#pragma unroll
    for (int j = 0; j < 9; ++j) ST::st(B + c + (size_t)j * N, o[j]);
}

}  // namespace lbm
