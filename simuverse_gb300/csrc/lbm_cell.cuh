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

// MRT relaxation rates of the non-hydrodynamic moments (energy, energy square, energy flux)
constexpr double MRT_S_E = 1.1, MRT_S_EPS = 1.0, MRT_S_Q = 1.2;

// Boundary rules on the pulled populations d (Zou-He inlet, anchored outflow), moments,
// Guo forcing with countdown, BGK.  o receives the post-collision deviations; rho, ux, uy
// the macroscopic values of the cell.
template <class R, int COLL = LBM_COLLISION_BGK, bool PLAIN = false>
__device__ __forceinline__ void phys_collide(R (&d)[9], int m, unsigned fl, size_t c, uint16_t* __restrict__ flags,
                                             lbm_lattice_info* __restrict__ info, R omega, R (&o)[9], R& rho_out,
                                             R& ux_out, R& uy_out, const R U = R(1)) {
    // PLAIN: the caller knows the cell is plain fluid (no inlet, outlet or forcing rule)
    const bool outlet = !PLAIN && (m == LBM_OUTLET);
    if (!PLAIN && m == LBM_INLET) {  // Zou-He velocity inlet, west face: unknowns 1, 5, 8
        const lbm_lattice_info in = info[c];
        const R ux = R(in.vx), uy = R(in.vy);
        const R S = d[0] + d[2] + d[4] + R(2) * (d[3] + d[6] + d[7]);
        const R rho = (U + S) / (R(1) - ux);
        const R rux = rho * ux, ruy = rho * uy;
        d[1] = d[3] + (R(2) / R(3)) * rux;
        d[5] = d[7] + R(0.5) * (d[4] - d[2]) + rux / R(6) - R(0.5) * ruy;
        d[8] = d[6] + R(0.5) * (d[2] - d[4]) + rux / R(6) + R(0.5) * ruy;
    }
    if (outlet) {  // zero-gradient outflow anchored at rho = 1: f_j <- f_j / rho
        const R dr = d[0] + d[1] + d[2] + d[3] + d[4] + d[5] + d[6] + d[7] + d[8];
        const R inv = U / (U + dr);
#pragma unroll
        for (int j = 0; j < 9; ++j) d[j] = (d[j] - PW<R>(j) * dr) * inv;
    }
    const R drho = d[0] + (((d[1] + d[3]) + (d[2] + d[4])) + ((d[5] + d[7]) + (d[6] + d[8])));
    R jx = (d[1] - d[3]) + ((d[5] - d[7]) + (d[8] - d[6]));
    R jy = (d[4] - d[2]) + ((d[7] - d[5]) + (d[8] - d[6]));
    const R rho = U + drho;
    R Fx = R(0), Fy = R(0);
    const bool forced = !PLAIN && (m == LBM_EXTERNAL_FORCE);
    if (forced) {  // Guo forcing with the reference's block_iter countdown
        lbm_lattice_info in = info[c];
        if (in.block_iter > 0) {
            in.block_iter = in.block_iter - 1;
            if (in.block_iter == 0) {
                in.material = LBM_BULK;
                const unsigned nf = (fl & ~FL_MAT_MASK) | LBM_BULK;
                flags[c] = (uint16_t)(nf | plain_bit(nf));
            }
            info[c] = in;
        }
        Fx = R(in.vx) * U;
        Fy = R(in.vy) * U;
        jx = jx + R(0.5) * Fx;
        jy = jy + R(0.5) * Fy;
    }
    const R inv_rho = recip_rn(rho);
    const R ux = jx * inv_rho, uy = jy * inv_rho;
    const R usq = R(1.5) * (ux * ux + uy * uy);
    // BGK on opposite pairs (j, inv j): the equilibrium deviation splits into an even part
    // w (drho + rho (4.5 (e.u)^2 - 1.5 u.u)) shared by the pair and an odd part 3 w rho e.u
    const R om = omega, om1 = R(1) - omega;
    const R r1 = rho * (R(3) * PW<R>(1)), r5 = rho * (R(3) * PW<R>(5));
    if (COLL == LBM_COLLISION_KBC) {
        // entropic KBC (Karlin, Bosch & Chikatamarla 2014) on the natural moments: f = k + s + h
        // with the shear part s from N = Pxx - Pyy and Pxy (s = N/4 on the x axis, -N/4 on the
        // y axis, sigma lambda Pxy / 4 on the diagonals); f' = f - beta (2 ds + gamma dh),
        // beta = omega / 2 (BGK's shear viscosity), gamma = 1/beta - (2 - 1/beta) <ds|dh> / <dh|dh>
        // with <x|y> = sum x_i y_i / feq_i, i.e. the stabiliser that keeps the entropy
        // production right; gamma = 2 is BGK.
        R q[9];
        {
            const R e1 = ux, e2 = uy, e3 = ux + uy, e4 = ux - uy;
            const R s1 = PW<R>(1) * (drho + rho * (R(4.5) * e1 * e1 - usq)), a1 = r1 * e1;
            const R s2 = PW<R>(1) * (drho + rho * (R(4.5) * e2 * e2 - usq)), a2 = r1 * e2;
            const R s3 = PW<R>(5) * (drho + rho * (R(4.5) * e3 * e3 - usq)), a3 = r5 * e3;
            const R s4 = PW<R>(5) * (drho + rho * (R(4.5) * e4 * e4 - usq)), a4 = r5 * e4;
            q[1] = s1 + a1; q[3] = s1 - a1;
            q[4] = s2 + a2; q[2] = s2 - a2;
            q[8] = s3 + a3; q[6] = s3 - a3;
            q[5] = s4 + a4; q[7] = s4 - a4;
            q[0] = PW<R>(0) * (drho - rho * usq);
        }
        R n[9];
#pragma unroll
        for (int j = 0; j < 9; ++j) n[j] = d[j] - q[j];
        const R dN = (n[1] + n[3]) - (n[2] + n[4]);
        const R dP = (n[8] + n[6]) - (n[5] + n[7]);
        R ds[9];
        ds[0] = R(0);
        ds[1] = ds[3] = R(0.25) * dN;
        ds[2] = ds[4] = R(-0.25) * dN;
        ds[8] = ds[6] = R(0.25) * dP;
        ds[5] = ds[7] = R(-0.25) * dP;
        R sh = R(0), hh = R(0);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const R dh = n[j] - ds[j];
            const R inv_feq = recip_rn(PW<R>(j) * U + q[j]);
            sh += ds[j] * dh * inv_feq;
            hh += dh * dh * inv_feq;
        }
        const R beta = R(0.5) * om, ib = R(1) / beta;
        const R gamma = hh > R(1e-30) ? ib - (R(2) - ib) * (sh / hh) : R(2);
#pragma unroll
        for (int j = 1; j < 9; ++j) o[j] = d[j] - beta * (R(2) * ds[j] + gamma * (n[j] - ds[j]));
    } else if (COLL == LBM_COLLISION_MRT) {
        // multiple relaxation times on the orthogonal D2Q9 moments of Lallemand & Luo
        // (2000): energy e, energy square eps, energy fluxes qx, qy relax at fixed rates,
        // the stresses pxx, pxy at omega (same shear viscosity as BGK); density and
        // momentum are untouched.  Moments of the deviations d; rest-state moments removed.
        const R a = d[1] + d[3] + d[2] + d[4];    // axis populations
        const R g = d[5] + d[6] + d[7] + d[8];    // diagonal populations
        const R me = R(-4) * d[0] - a + R(2) * g;
        const R meps = R(4) * d[0] - R(2) * a + g;
        const R qx = R(-2) * (d[1] - d[3]) + ((d[5] - d[7]) + (d[8] - d[6]));
        const R qy = R(-2) * (d[4] - d[2]) + ((d[7] - d[5]) + (d[8] - d[6]));
        const R pxx = (d[1] + d[3]) - (d[2] + d[4]);
        const R pxy = (d[8] + d[6]) - (d[5] + d[7]);
        const R jxx = jx * ux, jyy = jy * uy;  // j^2 / rho split by component
        const R eeq = R(-2) * drho + R(3) * (jxx + jyy);
        const R epseq = drho - R(3) * (jxx + jyy);
        const R de = R(MRT_S_E) * (eeq - me);       // delta m = -s (m - m_eq)
        const R deps = R(MRT_S_EPS) * (epseq - meps);
        const R dqx = R(MRT_S_Q) * (-jx - qx);
        const R dqy = R(MRT_S_Q) * (-jy - qy);
        const R dpxx = om * ((jxx - jyy) - pxx);
        const R dpxy = om * (jx * uy - pxy);
        // back to populations: f += M^T D^-1 delta m (row norms 36, 36, 12, 12, 4, 4)
        const R ce = de * (R(1) / R(36)), cp = deps * (R(1) / R(36));
        const R cqx = dqx * (R(1) / R(12)), cqy = dqy * (R(1) / R(12));
        const R cxx = dpxx * R(0.25), cxy = dpxy * R(0.25);
        const R axis = -ce - R(2) * cp;   // common part of the axis populations
        const R diag = R(2) * ce + cp;    // common part of the diagonal populations
        o[1] = d[1] + axis - R(2) * cqx + cxx;
        o[3] = d[3] + axis + R(2) * cqx + cxx;
        o[4] = d[4] + axis - R(2) * cqy - cxx;
        o[2] = d[2] + axis + R(2) * cqy - cxx;
        o[8] = d[8] + diag + cqx + cqy + cxy;
        o[6] = d[6] + diag - cqx - cqy + cxy;
        o[5] = d[5] + diag + cqx - cqy - cxy;
        o[7] = d[7] + diag - cqx + cqy - cxy;
    } else if (COLL == LBM_COLLISION_REGULARIZED) {
        // regularised BGK: the non-equilibrium part is replaced by its projection on the
        // second-order Hermite moments before relaxation (same viscosity; the non-
        // hydrodynamic moments are reset every step)
        R q[9];
        {
            const R e1 = ux, e2 = uy, e3 = ux + uy, e4 = ux - uy;
            const R s1 = PW<R>(1) * (drho + rho * (R(4.5) * e1 * e1 - usq)), a1 = r1 * e1;
            const R s2 = PW<R>(1) * (drho + rho * (R(4.5) * e2 * e2 - usq)), a2 = r1 * e2;
            const R s3 = PW<R>(5) * (drho + rho * (R(4.5) * e3 * e3 - usq)), a3 = r5 * e3;
            const R s4 = PW<R>(5) * (drho + rho * (R(4.5) * e4 * e4 - usq)), a4 = r5 * e4;
            q[1] = s1 + a1; q[3] = s1 - a1;
            q[4] = s2 + a2; q[2] = s2 - a2;
            q[8] = s3 + a3; q[6] = s3 - a3;
            q[5] = s4 + a4; q[7] = s4 - a4;
        }
        R n[9];
#pragma unroll
        for (int j = 1; j < 9; ++j) n[j] = d[j] - q[j];
        const R pd = (n[5] + n[6]) + (n[7] + n[8]);
        const R pxx = (n[1] + n[3]) + pd, pyy = (n[2] + n[4]) + pd;
        const R pxy = (n[8] + n[6]) - (n[5] + n[7]);
        const R k1 = om1 * R(4.5) * PW<R>(1), k5 = om1 * R(4.5) * PW<R>(5);
        const R third = R(1) / R(3);
        const R ax = k1 * (R(2) * third * pxx - third * pyy);  // e = (+-1, 0)
        const R ay = k1 * (R(2) * third * pyy - third * pxx);  // e = (0, +-1)
        const R dg = k5 * (R(2) * third * (pxx + pyy));
        o[1] = q[1] + ax; o[3] = q[3] + ax;
        o[2] = q[2] + ay; o[4] = q[4] + ay;
        o[8] = q[8] + (dg + k5 * R(2) * pxy); o[6] = q[6] + (dg + k5 * R(2) * pxy);
        o[5] = q[5] + (dg - k5 * R(2) * pxy); o[7] = q[7] + (dg - k5 * R(2) * pxy);
    } else {
    {  // 1 / 3: e = (+-1, 0)
        const R eu = ux;
        const R sym = om * (PW<R>(1) * (drho + rho * (R(4.5) * eu * eu - usq)));
        const R asy = om * (r1 * eu);
        o[1] = om1 * d[1] + (sym + asy);
        o[3] = om1 * d[3] + (sym - asy);
    }
    {  // 4 / 2: e = (0, +-1)
        const R eu = uy;
        const R sym = om * (PW<R>(1) * (drho + rho * (R(4.5) * eu * eu - usq)));
        const R asy = om * (r1 * eu);
        o[4] = om1 * d[4] + (sym + asy);
        o[2] = om1 * d[2] + (sym - asy);
    }
    {  // 8 / 6: e = +-(1, 1)
        const R eu = ux + uy;
        const R sym = om * (PW<R>(5) * (drho + rho * (R(4.5) * eu * eu - usq)));
        const R asy = om * (r5 * eu);
        o[8] = om1 * d[8] + (sym + asy);
        o[6] = om1 * d[6] + (sym - asy);
    }
    {  // 5 / 7: e = +-(1, -1)
        const R eu = ux - uy;
        const R sym = om * (PW<R>(5) * (drho + rho * (R(4.5) * eu * eu - usq)));
        const R asy = om * (r5 * eu);
        o[5] = om1 * d[5] + (sym + asy);
        o[7] = om1 * d[7] + (sym - asy);
    }
    }
    if (forced) {
        const R gf = R(1) - R(0.5) * omega;
        const R uF = ux * Fx + uy * Fy;
#pragma unroll
        for (int j = 1; j < 9; ++j) {
            const R eF = (EX(j) == 0 ? R(0) : R(EX(j)) * Fx) + (EY(j) == 0 ? R(0) : R(EY(j)) * Fy);
            const R eu = (EX(j) == 0 ? R(0) : R(EX(j)) * ux) + (EY(j) == 0 ? R(0) : R(EY(j)) * uy);
            o[j] = o[j] + gf * PW<R>(j) * (R(3) * (eF - uF) + R(9) * eu * eF);
        }
    }
    // rest population from mass conservation: sum_j o_j = drho by construction (the BGK
    // value in exact arithmetic; removes the bias of the rounded weights' moments)
    o[0] = drho - (((o[1] + o[3]) + (o[2] + o[4])) + ((o[5] + o[7]) + (o[6] + o[8])));
    rho_out = rho * (R(1) / U);
    ux_out = ux;
    uy_out = uy;
}

// BGK of a plain fluid cell for 16-bit storage, whose rounding (2^-9 to 2^-12 relative) dwarfs
// the last bits of the arithmetic: the reciprocal of the density is the hardware approximation,
// omega is folded into the weights and the rest population takes its own BGK update instead of
// the mass balance.  U is the stored unit density (see phys_collide).
__device__ __forceinline__ void bgk_plain_fast(const float (&d)[9], float omega, float U, float (&o)[9],
                                               float& rho_out, float& ux_out, float& uy_out) {
    const float s13 = d[1] + d[3], s24 = d[2] + d[4], s57 = d[5] + d[7], s68 = d[6] + d[8];
    const float drho = d[0] + ((s13 + s24) + (s57 + s68));
    const float d86 = d[8] - d[6], d57 = d[5] - d[7];
    const float jx = (d[1] - d[3]) + (d57 + d86);
    const float jy = (d[4] - d[2]) + (d86 - d57);
    const float rho = U + drho;
    const float inv = __fdividef(1.0f, rho);
    const float ux = jx * inv, uy = jy * inv;
    const float uxx = ux * ux, uyy = uy * uy;
    // t0 = drho - 1.5 rho u.u is the isotropic part of every equilibrium deviation; the pair
    // (j, inv j) shares w_j (t0 + 4.5 rho (e_j.u)^2) and differs by -+ 3 w_j rho e_j.u
    const float t0 = drho - rho * (1.5f * (uxx + uyy));
    const float om1 = 1.0f - omega;
    const float w1 = omega * PW<float>(1), w5 = omega * PW<float>(5);
    const float a1 = w1 * t0, a5 = w5 * t0;
    const float r1 = rho * (3.0f * w1), r5 = rho * (3.0f * w5);
    const float q1 = rho * (4.5f * w1), q5 = rho * (4.5f * w5);
    {
        const float sym = q1 * uxx + a1;
        o[1] = om1 * d[1] + (r1 * ux + sym);
        o[3] = om1 * d[3] + (sym - r1 * ux);
    }
    {
        const float sym = q1 * uyy + a1;
        o[4] = om1 * d[4] + (r1 * uy + sym);
        o[2] = om1 * d[2] + (sym - r1 * uy);
    }
    {
        const float eu = ux + uy;
        const float sym = q5 * (eu * eu) + a5;
        o[8] = om1 * d[8] + (r5 * eu + sym);
        o[6] = om1 * d[6] + (sym - r5 * eu);
    }
    {
        const float eu = ux - uy;
        const float sym = q5 * (eu * eu) + a5;
        o[5] = om1 * d[5] + (r5 * eu + sym);
        o[7] = om1 * d[7] + (sym - r5 * eu);
    }
    o[0] = om1 * d[0] + (omega * PW<float>(0)) * t0;
    rho_out = rho * (1.0f / U);
    ux_out = ux;
    uy_out = uy;
}

// One cell (x, y) of a lattice of nx x ny cells whose rows are `pitch` elements apart
// (pitch >= nx; the single-lattice kernel passes pitch = nx).
// SR: stochastic rounding of the stores with the step's `seed` (lbm_common.cuh).  A lattice
// inside a pool (the batched form) passes the pool's base pointers and its element offsets:
// populations at pop_off, flags and info at cell_off, macro planes at 3 * cell_off; OFF is
// their integer type (32-bit when the pool allows, which keeps the pointers out of registers).
template <class ST, bool MACRO, int COLL = LBM_COLLISION_BGK, bool SR = false, class OFF = size_t>
__device__ __forceinline__ void phys_cell_update(const typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                                                 uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                 typename ST::R omega, int x, int y, int nx, int pitch, int ny,
                                                 float* __restrict__ macro, uint32_t seed = 0, OFF pop_off = 0,
                                                 OFF cell_off = 0) {
    using R = typename ST::R;
    const OFF N = (OFF)pitch * (OFF)ny;
    const unsigned c = (unsigned)y * (unsigned)pitch + (unsigned)x;  // cells < 2^31
    const OFF cc = cell_off + (OFF)c, mc = (OFF)3 * cell_off + (OFF)c;
    // ends of this lattice's ranges for the bounds-checked build (phys_collide's info and flag
    // accesses use cc, checked here)
    const unsigned long long end_c = (unsigned long long)cell_off + (unsigned long long)N;
    const unsigned long long end_p = (unsigned long long)pop_off + 9ull * (unsigned long long)N;
    const unsigned long long end_m = 3ull * (unsigned long long)cell_off + 3ull * (unsigned long long)N;
    const unsigned fl = in_bounds(cc, end_c, BS_CELL_FLAGS) ? flags[cc] : 0u;
    const int m = (int)(fl & FL_MAT_MASK);
    if (is_solid(m)) {
        if (MACRO && in_bounds(mc + 2 * N, end_m, BS_CELL_MACRO)) {
            macro[mc] = 0.0f; macro[mc + N] = 0.0f; macro[mc + 2 * N] = 0.0f;
        }
        return;
    }
    const bool outlet = (m == LBM_OUTLET);
    const int xm = x == 0 ? nx - 1 : x - 1, xp = x == nx - 1 ? 0 : x + 1;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const unsigned r0 = (unsigned)y * pitch, rm = (unsigned)ym * pitch, rp = (unsigned)yp * pitch;
    R d[9];
    if (!(fl & (0x1FEu << FL_DIR_SHIFT))) {  // no solid neighbour: plain pull
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const int sx = EX(j) == 1 ? xm : (EX(j) == -1 ? (outlet ? x : xp) : x);
            const unsigned row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
            const OFF i = pop_off + (OFF)j * N + (OFF)(row + (unsigned)sx);
            d[j] = in_bounds(i, end_p, BS_CELL_PULL) ? ST::ldu(A + i) : R(0);
        }
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const int sx = EX(j) == 1 ? xm : (EX(j) == -1 ? (outlet ? x : xp) : x);
            const unsigned row = EY(j) == 1 ? rm : (EY(j) == -1 ? rp : r0);
            if (fl & (1u << (FL_DIR_SHIFT + j))) {
                const OFF ib = pop_off + (OFF)INV(j) * N + (OFF)c;  // half-way bounce-back
                R v = in_bounds(ib, end_p, BS_CELL_PULL) ? ST::ldu(A + ib) : R(0);
                const OFF is = cell_off + (OFF)(row + sx);
                if ((fl & FL_MOVING) && in_bounds(is, end_c, BS_CELL_INFO)) {
                    const lbm_lattice_info si = info[is];
                    const R uw = R(EX(j)) * R(si.vx) + R(EY(j)) * R(si.vy);
                    // rounded product, not an FMA: a contracted wall term leaves a
                    // systematic mass drift of ~1e-12 per step in FP32
                    if (uw != R(0)) v = add_rn(v, mul_rn(R(6) * PW<R>(j) * R(ST::UNIT), uw));
                }
                d[j] = v;
            } else {
                const OFF i = pop_off + (OFF)j * N + (OFF)(row + (unsigned)sx);
                d[j] = in_bounds(i, end_p, BS_CELL_PULL) ? ST::ldu(A + i) : R(0);
            }
        }
    }
    R o[9], rho, ux, uy;
    phys_collide<R, COLL>(d, m, fl, (size_t)cc, flags, info, omega, o, rho, ux, uy, R(ST::UNIT));
    if (MACRO && in_bounds(mc + 2 * N, end_m, BS_CELL_MACRO)) {
        macro[mc] = (float)rho; macro[mc + N] = (float)ux; macro[mc + 2 * N] = (float)uy;
    }
    if (SR) {
        const uint32_t q = sr_hash(c ^ seed);
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const OFF i = pop_off + (OFF)j * N + (OFF)c;
            if (in_bounds(i, end_p, BS_CELL_STORE)) ST::stu_sr(B + i, o[j], q * sr_mul(j));
        }
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j) {
            const OFF i = pop_off + (OFF)j * N + (OFF)c;
            if (in_bounds(i, end_p, BS_CELL_STORE)) ST::stu(B + i, o[j]);
        }
    }
}

}  // namespace lbm
