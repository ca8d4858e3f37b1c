// lbm_cell_tiled.cuh -- the physics-mode step for 16-bit storage in the tiled population
// layout (pop_index in lbm_common.cuh): rows are cut into tiles of 64 cells and a tile keeps
// its nine 64-element planes together, so the nine loads (and stores) of a thread differ only
// by compile-time offsets from one base address per row.
//
// One warp updates one tile (lane l: cells 2l and 2l + 1 of the tile).  The pull of a direction
// with e_x = +1 takes the left neighbour lane's second cell by a warp shuffle (lane 0 loads the
// last cell of the previous tile, wrapping to the last tile of the row), e_x = -1 the mirror
// image.  Cells next to a solid, inlet, outlet and forcing cells take the general per-cell
// rules of phys_collide; when every cell of the warp is plain fluid the collision is
// bgk_plain_fast with no per-cell test.
#pragma once

#include "lbm_cell.cuh"
#include "lbm_cell4.cuh"
#include "lbm_common.cuh"

namespace lbm {

// Where the general per-cell rules read the extra populations of a lane's own column: the
// bounce-back source (population j of the cell itself) and the outflow's e_x = -1 populations
// (rows y - 1, y, y + 1).  TileSrcGlobal reads the current population buffer; the kernel that
// stages rows in shared memory passes a source over its staged rows (the same values).
template <class ST>
struct TileSrcGlobal {
    const typename ST::T* A;
    uint32_t N;
    int nx, x0, y, ym, yp;  // x0: the lane's first cell
    // population j of cell (x0 + k, row y + dy), dy in {-1, 0, 1} (wrapped)
    __device__ __forceinline__ float col(int j, int dy, int k) const {
        const int yy = dy < 0 ? ym : (dy > 0 ? yp : y);
        const size_t i = pop_index(true, N, j, (size_t)yy * nx + x0 + k);
        return in_bounds(i, 9ull * N, BS_TILE_PULL) ? ST::ldu(A + i) : 0.0f;
    }
};

// The collision and the stores of one tile row for a warp (lane l: cells 2l and 2l + 1 of tile
// tx in row y), given the pulled populations d (stored units) and the two cells' flag words fq.
// Shared by the kernel that pulls from global memory (phys_tile_update) and the one that pulls
// from rows staged in shared memory (k_phys_step_ring); cells next to a solid and outflow cells
// read their extra populations through src (SRC::col), inlet and forcing cells their records
// from info.
// SR: stochastic rounding of the stores with the step's `seed` (lbm_common.cuh)
template <class ST, bool MACRO, bool SR, class SRC>
__device__ __forceinline__ void phys_tile_finish(float (&d)[9][2], unsigned fq, const SRC& src,
                                                 typename ST::T* __restrict__ B, uint16_t* __restrict__ flags,
                                                 lbm_lattice_info* __restrict__ info, float omega, int tx, int y,
                                                 int nx, int ny, float* __restrict__ macro, uint32_t seed) {
    using T = typename ST::T;
    using R = float;
    constexpr int W = POP_TILE, TS = 9 * POP_TILE;
    const int lane = threadIdx.x & 31;
    const int tpr = nx / W;
    const uint32_t N = (uint32_t)nx * (uint32_t)ny;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    const int x0 = tx * W + 2 * lane;
    const uint32_t o0 = ((uint32_t)y * tpr + tx) * TS + 2 * lane;
    const uint32_t c0 = (uint32_t)y * nx + x0;
    const unsigned long long NC = N, NP = 9ull * N, NM = 3ull * N;
    unsigned fl[2];
    fl[0] = fq & 0xffffu;
    fl[1] = fq >> 16;
    const bool fast = __all_sync(0xffffffffu, (fq & (FL_PLAIN | FL_PLAIN << 16)) == (FL_PLAIN | FL_PLAIN << 16));

    R mr[2], mu[2], mv[2];
    if (fast) {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            R dk[9], o[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) dk[j] = d[j][k];
            bgk_plain_fast(dk, omega, R(ST::UNIT), o, mr[k], mu[k], mv[k]);
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j][k] = o[j];
        }
    } else {
#pragma unroll
        for (int k = 0; k < 2; ++k) {
            const unsigned f = fl[k];
            const int m = (int)(f & FL_MAT_MASK);
            const int x = x0 + k;
            const uint32_t c = c0 + k;
            R dk[9];
#pragma unroll
            for (int j = 0; j < 9; ++j) dk[j] = d[j][k];
            if (is_solid(m)) {
#pragma unroll
                for (int j = 0; j < 9; ++j) d[j][k] = R(0);
                mr[k] = R(0); mu[k] = R(0); mv[k] = R(0);
                continue;
            }
            if (m == LBM_OUTLET) {  // zero-gradient: e_x = -1 populations come from the own column
                dk[3] = src.col(3, 0, k);
                dk[6] = src.col(6, 1, k);
                dk[7] = src.col(7, -1, k);
            }
            if (f & (0xFFu << (FL_DIR_SHIFT + 1))) {  // some pull source is solid: bounce back
#pragma unroll
                for (int j = 1; j < 9; ++j) {
                    if (f & (1u << (FL_DIR_SHIFT + j))) {
                        R v = src.col(INV(j), 0, k);  // half-way bounce-back: the cell's own population
                        if (f & FL_MOVING) {
                            int sx = x - EX(j);
                            if (m == LBM_OUTLET && EX(j) == -1) sx = x;
                            sx = sx < 0 ? nx - 1 : (sx >= nx ? 0 : sx);
                            const int sy = EY(j) == 1 ? ym : (EY(j) == -1 ? yp : y);
                            const size_t is = (size_t)sy * nx + sx;
                            lbm_lattice_info si = {0, 0, 0.0f, 0.0f};
                            if (in_bounds(is, NC, BS_TILE_INFO)) si = info[is];
                            const R uw = R(EX(j)) * R(si.vx) + R(EY(j)) * R(si.vy);
                            if (uw != R(0)) v = add_rn(v, mul_rn(R(6) * PW<R>(j) * R(ST::UNIT), uw));
                        }
                        dk[j] = v;
                    }
                }
            }
            R o[9];
            phys_collide<R>(dk, m, f, (size_t)c, flags, info, omega, o, mr[k], mu[k], mv[k], R(ST::UNIT));
#pragma unroll
            for (int j = 0; j < 9; ++j) d[j][k] = o[j];
        }
    }
    T* Q0 = B + o0;
    if (SR) {
        const uint32_t q = sr_hash(c0 ^ seed);
#pragma unroll
        for (int j = 0; j < 9; ++j)
            if (in_bounds(o0 + (unsigned long long)(j * W) + 1ull, NP, BS_TILE_STORE))
                Vec2<ST>::st_sr(Q0 + j * W, d[j], q * sr_mul(2 * j), q * sr_mul(2 * j + 1));
    } else {
#pragma unroll
        for (int j = 0; j < 9; ++j)
            if (in_bounds(o0 + (unsigned long long)(j * W) + 1ull, NP, BS_TILE_STORE)) Vec2<ST>::st(Q0 + j * W, d[j]);
    }
    if (MACRO && in_bounds(2ull * N + c0 + 1ull, NM, BS_TILE_MACRO)) {
        *reinterpret_cast<float2*>(macro + c0) = make_float2(mr[0], mr[1]);
        *reinterpret_cast<float2*>(macro + N + c0) = make_float2(mu[0], mu[1]);
        *reinterpret_cast<float2*>(macro + 2 * N + c0) = make_float2(mv[0], mv[1]);
    }
}

// One warp's tile row, pulled from global memory.
// SR: stochastic rounding of the stores with the step's `seed` (lbm_common.cuh)
template <class ST, bool MACRO, bool SR = false>
__device__ __forceinline__ void phys_tile_update(const typename ST::T* __restrict__ A, typename ST::T* __restrict__ B,
                                                 uint16_t* __restrict__ flags, lbm_lattice_info* __restrict__ info,
                                                 float omega, int tx, int y, int nx, int ny, float* __restrict__ macro,
                                                 uint32_t seed = 0) {
    using T = typename ST::T;
    using R = float;
    constexpr int W = POP_TILE, TS = 9 * POP_TILE;  // cells per tile, elements per tile
    const int lane = threadIdx.x & 31;
    const int tpr = nx / W;  // tiles per row
    const uint32_t N = (uint32_t)nx * (uint32_t)ny;
    const int ym = y == 0 ? ny - 1 : y - 1, yp = y == ny - 1 ? 0 : y + 1;
    // element distance from a thread's own cell to the halo cell: lane 0 reads the last cell of
    // the tile to the left (wrapping to the row's last tile), lane 31 the first cell of the tile
    // to the right (wrapping to the row's first tile); the same in every row and plane
    const int dl = (tx == 0 ? (tpr - 1) * TS : -TS) + (W - 1);
    const int dr = (tx == tpr - 1 ? -(tpr - 1) * TS : TS) - (W - 2);
    const int x0 = tx * W + 2 * lane;
    // element offset of this thread's first cell in the tiles of rows ym, y, yp
    const uint32_t o0 = ((uint32_t)y * tpr + tx) * TS + 2 * lane;
    const uint32_t om = ((uint32_t)ym * tpr + tx) * TS + 2 * lane;
    const uint32_t op = ((uint32_t)yp * tpr + tx) * TS + 2 * lane;
    const uint32_t c0 = (uint32_t)y * nx + x0;  // cell index (flags, info, macro)

    // extents for the bounds-checked build: cells, population elements
    const unsigned long long NC = N, NP = 9ull * N;
    const unsigned fq = in_bounds(c0 + 1ull, NC, BS_TILE_FLAGS) ? *reinterpret_cast<const unsigned*>(flags + c0) : 0u;

    const T* Pm = A + om;  // every plane of a tile is a compile-time offset from these
    const T* P0 = A + o0;
    const T* Pp = A + op;
    R d[9][2];
#pragma unroll
    for (int j = 0; j < 9; ++j) {
        const T* Pr = EY(j) == 1 ? Pm : (EY(j) == -1 ? Pp : P0);
        const long long pr = (long long)(Pr - A) + j * W;  // element index of the pair (checked build)
        R v[2] = {R(0), R(0)};
        if (in_bounds((unsigned long long)pr + 1ull, NP, BS_TILE_PULL)) Vec2<ST>::ld(Pr + j * W, v);
        if (EX(j) == 0) {
            d[j][0] = v[0];
            d[j][1] = v[1];
        } else if (EX(j) == 1) {  // source x - 1
            R prev = __shfl_up_sync(0xffffffffu, v[1], 1);
            if (lane == 0) prev = in_bounds((unsigned long long)(pr + dl), NP, BS_TILE_PULL) ? ST::ldu(Pr + dl + j * W) : R(0);
            d[j][0] = prev;
            d[j][1] = v[0];
        } else {  // source x + 1
            R next = __shfl_down_sync(0xffffffffu, v[0], 1);
            if (lane == 31) next = in_bounds((unsigned long long)(pr + dr), NP, BS_TILE_PULL) ? ST::ldu(Pr + dr + j * W) : R(0);
            d[j][0] = v[1];
            d[j][1] = next;
        }
    }

    const TileSrcGlobal<ST> src{A, N, nx, x0, y, ym, yp};
    phys_tile_finish<ST, MACRO, SR>(d, fq, src, B, flags, info, omega, tx, y, nx, ny, macro, seed);
}

}  // namespace lbm
