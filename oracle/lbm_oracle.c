/*
 * lbm_oracle.c -- TEST INFRASTRUCTURE, NOT PRODUCT CODE (see lbm_oracle.h).
 *
 * CPU restatement of simuverse's D2Q9 lattice-Boltzmann path.  Only tests/, the smoke
 * check and bench.py's CPU-baseline leg use it.  Parity status: UNPINNED (no reference
 * outputs can be produced on these machines; see lbm_oracle.h).
 *
 * Build: gcc -O3 -fopenmp -ffp-contract=off -fPIC -shared (oracle/build.py).  Contraction
 * must stay off so that every float operation rounds the way the WGSL expression reads.
 */
#include "lbm_oracle.h"

#include <math.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

/* simuverse/src/fluid/mod.rs:39-52 -- e, truncated weight, clamp maximum, inverse */
static const float REF_EX[9] = {0.0f, 1.0f, 0.0f, -1.0f, 0.0f, 1.0f, -1.0f, -1.0f, 1.0f};
static const float REF_EY[9] = {0.0f, 0.0f, -1.0f, 0.0f, 1.0f, -1.0f, -1.0f, 1.0f, 1.0f};
static const float REF_W[9] = {0.444444f, 0.111111f, 0.111111f, 0.111111f, 0.111111f,
                               0.0277777f, 0.0277777f, 0.0277777f, 0.0277777f};
static const float REF_MAX[9] = {0.6f, 0.2222f, 0.2222f, 0.2222f, 0.2222f,
                                 0.1111f, 0.1111f, 0.1111f, 0.1111f};
static const int IEX[9] = {0, 1, 0, -1, 0, 1, -1, -1, 1};
static const int IEY[9] = {0, 0, -1, 0, 1, -1, -1, 1, 1};
static const int INV[9] = {0, 3, 4, 1, 2, 7, 8, 5, 6};

#define OBSTACLE_RADIUS 28.0f /* fluid/mod.rs:1 */

enum { M_BULK = 1, M_BOUNDARY = 2, M_INLET = 3, M_OBSTACLE = 4, M_OUTLET = 5, M_FORCE = 6, M_GHOST = 7 };

static int is_solid(int m) { return m == M_BOUNDARY || m == M_OBSTACLE; }    /* d2q9_fn.wgsl:19,22 */
static int is_accelerate(int m) { return m == M_INLET || m == M_FORCE; }      /* d2q9_fn.wgsl:24 */

int lo_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

void lo_set_num_threads(int n) {
#ifdef _OPENMP
    if (n > 0) omp_set_num_threads(n);
#else
    (void)n;
#endif
}

/* fluid/mod.rs:57-59 with glam's Vec2::length (x*x + y*y, then sqrt) */
static int is_sd_sphere(float px, float py, float r) {
    float d = sqrtf(px * px + py * py);
    return d <= r;
}

/* ------------------------------------------------------------------------- */
/* lattice.rs:26-98                                                          */
/* ------------------------------------------------------------------------- */
void lo_mask_reference(int nx, int ny, int scene, float lid_vx, float inlet_vx, lo_info* info) {
    const float s0x = (float)nx / 7.0f - OBSTACLE_RADIUS, s0y = (float)ny / 2.0f;
    const float s1x = (float)nx / 5.0f, s1y = (float)ny / 4.0f;
    const float s2x = (float)nx / 5.0f, s2y = (float)ny * 0.75f;
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            int material = M_BULK;
            float vx = 0.0f;
            if (scene == 2) { /* Custom */
                if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) material = M_BOUNDARY;
            } else if (scene == 1) { /* LidDrivenCavity */
                if (x == 0 || x == nx - 1 || y == ny - 1) {
                    material = M_BOUNDARY;
                } else if (y == 0) {
                    material = M_GHOST;
                } else if (y == 1) {
                    material = M_FORCE;
                    vx = lid_vx;
                }
            } else { /* Poiseuille */
                if (y == 0 || y == ny - 1) {
                    material = M_BOUNDARY;
                } else if (x == 0 || x == nx - 1) {
                    material = M_GHOST;
                } else if (x == 1) {
                    material = M_INLET;
                    vx = inlet_vx;
                } else if (x == nx - 2) {
                    material = M_OUTLET;
                } else {
                    float px = (float)x, py = (float)y;
                    if (is_sd_sphere(px - s0x, py - s0y, OBSTACLE_RADIUS) ||
                        is_sd_sphere(px - s1x, py - s1y, OBSTACLE_RADIUS) ||
                        is_sd_sphere(px - s2x, py - s2y, OBSTACLE_RADIUS))
                        material = M_OBSTACLE;
                }
            }
            lo_info* c = &info[(size_t)y * nx + x];
            c->material = material;
            c->block_iter = -1;
            c->vx = vx;
            c->vy = 0.0f;
        }
    }
}

/* ------------------------------------------------------------------------- */
/* init.wgsl:19-63                                                           */
/* ------------------------------------------------------------------------- */
void lo_ref_init(int nx, int ny, int fluid_ty, lo_info* info, float* A, float* B) {
    const size_t N = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            size_t c = (size_t)y * nx + x;
            lo_info in = info[c];
            if (is_solid(in.material)) {
                for (int i = 0; i < 9; ++i) { A[c + i * N] = 0.0f; B[c + i * N] = 0.0f; }
            } else if (fluid_ty == 0) {
                for (int i = 0; i < 9; ++i) { A[c + i * N] = REF_W[i]; B[c + i * N] = 0.0f; }
                float temp = REF_W[3] * 0.5f;
                A[c + 1 * N] = REF_W[1] + temp;
                A[c + 3 * N] = temp;
                B[c + 1 * N] = REF_W[1] + temp;
                B[c + 3 * N] = temp;
            } else {
                for (int i = 0; i < 9; ++i) { A[c + i * N] = REF_W[i]; B[c + i * N] = 0.0f; }
            }
            if (is_accelerate(in.material) && in.block_iter > 0) {
                in.block_iter = 0;
                in.material = M_BULK;
                in.vx = 0.0f;
                in.vy = 0.0f;
                info[c] = in;
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* collide_stream.wgsl:25-88 then boundary.wgsl:3-35                         */
/* ------------------------------------------------------------------------- */
static inline int wrap(int v, int n) { return v < 0 ? n - 1 : (v >= n ? 0 : v); } /* layout_and_fn.wgsl:40-49 */

void lo_ref_step(int nx, int ny, float omega, lo_info* info, const float* A, float* B,
                 float* macro4, float* scratch) {
    const size_t N = (size_t)nx * ny;
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            const size_t c = (size_t)y * nx + x;
            lo_info in = info[c];
            if (is_solid(in.material)) {
                if (macro4) { macro4[4 * c + 0] = 0.0f; macro4[4 * c + 1] = 0.0f; macro4[4 * c + 2] = 0.0f; macro4[4 * c + 3] = 0.0f; }
                continue;
            }
            float f[9];
            float vx = 0.0f, vy = 0.0f, rho = 0.0f;
            for (int i = 0; i < 9; ++i) {
                /* streaming_in: uv + e(inv(i)), wrapped (layout_and_fn.wgsl:38-51) */
                int sx = wrap(x + IEX[INV[i]], nx), sy = wrap(y + IEY[INV[i]], ny);
                f[i] = A[(size_t)sy * nx + sx + i * N];
                rho = rho + f[i];
                vx = vx + REF_EX[i] * f[i];
                vy = vy + REF_EY[i] * f[i];
            }
            /* WGSL clamp(e, lo, hi) = min(max(e, lo), hi) */
            rho = fminf(fmaxf(rho, 0.8f), 1.2f);
            vx = vx / rho;
            vy = vy / rho;
            float F[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
            if (is_accelerate(in.material)) {
                if (in.block_iter > 0) {
                    in.block_iter = in.block_iter - 1;
                    if (in.block_iter == 0) in.material = M_BULK;
                }
                info[c] = in;
                float fx = in.vx, fy = in.vy;
                vx = fx * 0.5f / rho;
                vy = fy * 0.5f / rho;
                for (int i = 0; i < 9; ++i) F[i] = REF_W[i] * 3.0f * (REF_EX[i] * fx + REF_EY[i] * fy);
            }
            if (macro4) { macro4[4 * c + 0] = vx; macro4[4 * c + 1] = vy; macro4[4 * c + 2] = rho; macro4[4 * c + 3] = 1.0f; }
            float usqr = 1.5f * (vx * vx + vy * vy);
            for (int i = 0; i < 9; ++i) {
                float eu = REF_EX[i] * vx + REF_EY[i] * vy;
                float feq = rho * REF_W[i] * (1.0f + 3.0f * eu + 4.5f * (eu * eu) - usqr);
                float t = f[i] - omega * (f[i] - feq) + F[i];
                if (t > REF_MAX[i]) t = REF_MAX[i];
                else if (t < 0.0f) t = 0.0f;
                B[c + i * N] = t;
            }
        }
    }
    /* boundary pass, phase 1: read every value that a wall cell pulls */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            const size_t c = (size_t)y * nx + x;
            if (!is_solid(info[c].material)) continue;
            for (int i = 0; i < 9; ++i) {
                int nxp = x - IEX[i], nyp = y - IEY[i];
                if (nxp <= 0 || nyp <= 0 || nxp >= nx - 1 || nyp >= ny - 1) continue;
                scratch[c * 9 + i] = B[(size_t)nyp * nx + nxp + i * N];
            }
        }
    }
    /* phase 2: stream_cell[uv, inv(i)] = val */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            const size_t c = (size_t)y * nx + x;
            if (!is_solid(info[c].material)) continue;
            for (int i = 0; i < 9; ++i) {
                int nxp = x - IEX[i], nyp = y - IEY[i];
                if (nxp <= 0 || nyp <= 0 || nxp >= nx - 1 || nyp >= ny - 1) continue;
                B[c + INV[i] * N] = scratch[c * 9 + i];
            }
        }
    }
    /* phase 3: stream_cell[new_uv, i] = 0 */
#pragma omp parallel for schedule(static)
    for (int y = 0; y < ny; ++y) {
        for (int x = 0; x < nx; ++x) {
            const size_t c = (size_t)y * nx + x;
            if (!is_solid(info[c].material)) continue;
            for (int i = 0; i < 9; ++i) {
                int nxp = x - IEX[i], nyp = y - IEY[i];
                if (nxp <= 0 || nyp <= 0 || nxp >= nx - 1 || nyp >= ny - 1) continue;
                B[(size_t)nyp * nx + nxp + i * N] = 0.0f;
            }
        }
    }
}

/* ------------------------------------------------------------------------- */
/* interactive edits: d2q9_node.rs:215-300, fluid_simulator.rs:137-152       */
/* ------------------------------------------------------------------------- */
int lo_add_obstacle(int nx, int ny, lo_info* host_info, lo_info* dev_info, int x, int y) {
    const int r = (int)OBSTACLE_RADIUS;
    int min_y = y - r, max_y = min_y + r * 2;
    if (min_y < 0 || max_y > ny || x < 0 || x >= nx) return -1;
    const float cx = (float)x + 0.5f, cy = (float)y + 0.5f;
    for (int yy = min_y; yy < max_y; ++yy) {
        for (int xx = 0; xx < nx; ++xx) {
            size_t idx = (size_t)yy * nx + xx;
            if (is_sd_sphere((float)xx + 0.5f - cx, (float)yy + 0.5f - cy, OBSTACLE_RADIUS)) {
                host_info[idx].material = M_OBSTACLE;
                host_info[idx].block_iter = -1;
                host_info[idx].vx = 0.0f;
                host_info[idx].vy = 0.0f;
            }
            dev_info[idx] = host_info[idx];
        }
    }
    return 0;
}

int lo_on_click(int nx, int ny, int pixel_size, lo_info* host_info, lo_info* dev_info, float px, float py) {
    if (px <= 0.0f || py <= 0.0f) return 1;
    unsigned x = (unsigned)px / (unsigned)pixel_size;
    unsigned y = (unsigned)py / (unsigned)pixel_size;
    unsigned half = (unsigned)OBSTACLE_RADIUS;
    if (x < half || (long)x >= (long)nx - (long)(half + 2) || y < half || (long)y >= (long)ny - (long)(half + 2)) return 1;
    return lo_add_obstacle(nx, ny, host_info, dev_info, (int)x, (int)y);
}

void lo_add_external_force(int nx, int ny, int pixel_size, lo_info* dev_info,
                           float pos_x, float pos_y, float pre_x, float pre_y) {
    float ddx = pos_x - pre_x, ddy = pos_y - pre_y;
    float dis = sqrtf(ddx * ddx + ddy * ddy);
    float force = 0.1f * (dis / 20.0f);
    if (force > 0.12f) force = 0.12f;
    float ridian = atan2f(pos_y - pre_y, pos_x - pre_x);
    float vx = force * cosf(ridian);
    float vy = force * sinf(ridian);
    float c = ceilf(dis / (float)(pixel_size - 1));
    float step = dis / c;
    int count = (int)c;
    for (int i = 0; i < count; ++i) {
        float d = step * (float)i;
        float p_x = roundf(pre_x + d * cosf(ridian));
        float p_y = roundf(pre_y + d * sinf(ridian));
        /* Rust `as u32` saturates: negative -> 0 */
        unsigned ux = p_x <= 0.0f ? 0u : (unsigned)p_x;
        unsigned uy = p_y <= 0.0f ? 0u : (unsigned)p_y;
        unsigned x = ux / (unsigned)pixel_size, y = uy / (unsigned)pixel_size;
        if (x < 1 || (long)x >= (long)nx - 2 || y < 1 || (long)y >= (long)ny - 2) continue;
        lo_info* t = &dev_info[(size_t)y * nx + x];
        t->material = M_FORCE;
        t->block_iter = 90;
        t->vx = vx;
        t->vy = vy;
    }
}

/* ------------------------------------------------------------------------- */
/* physics mode                                                              */
/* ------------------------------------------------------------------------- */
void lo_mask_physics_cavity(int nx, int ny, float lid_vx, lo_info* info) {
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            lo_info* c = &info[(size_t)y * nx + x];
            c->block_iter = -1;
            c->vx = 0.0f;
            c->vy = 0.0f;
            c->material = M_BULK;
            if (x == 0 || x == nx - 1 || y == 0 || y == ny - 1) c->material = M_BOUNDARY;
            if (y == 0 && x >= 1 && x <= nx - 2) c->vx = lid_vx;
        }
}

/* mt19937_64 (Matsumoto & Nishimura 2000; parameters as in ISO C++ std::mt19937_64) */
typedef struct { uint64_t mt[312]; int mti; } mt64;
static void mt64_seed(mt64* s, uint64_t seed) {
    s->mt[0] = seed;
    for (int i = 1; i < 312; ++i)
        s->mt[i] = 6364136223846793005ULL * (s->mt[i - 1] ^ (s->mt[i - 1] >> 62)) + (uint64_t)i;
    s->mti = 312;
}
static uint64_t mt64_next(mt64* s) {
    static const uint64_t MAG[2] = {0ULL, 0xB5026F5AA96619E9ULL};
    const uint64_t UM = 0xFFFFFFFF80000000ULL, LM = 0x7FFFFFFFULL;
    if (s->mti >= 312) {
        int i;
        for (i = 0; i < 312 - 156; ++i) {
            uint64_t x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
            s->mt[i] = s->mt[i + 156] ^ (x >> 1) ^ MAG[x & 1ULL];
        }
        for (; i < 311; ++i) {
            uint64_t x = (s->mt[i] & UM) | (s->mt[i + 1] & LM);
            s->mt[i] = s->mt[i + (156 - 312)] ^ (x >> 1) ^ MAG[x & 1ULL];
        }
        uint64_t x = (s->mt[311] & UM) | (s->mt[0] & LM);
        s->mt[311] = s->mt[155] ^ (x >> 1) ^ MAG[x & 1ULL];
        s->mti = 0;
    }
    uint64_t x = s->mt[s->mti++];
    x ^= (x >> 29) & 0x5555555555555555ULL;
    x ^= (x << 17) & 0x71D67FFFEDA60000ULL;
    x ^= (x << 37) & 0xFFF7EEE000000000ULL;
    x ^= (x >> 43);
    return x;
}
static double mt64_unit(mt64* s) { return (double)(mt64_next(s) >> 11) * (1.0 / 9007199254740992.0); }

int lo_mask_physics_channel(int nx, int ny, float u_max, uint64_t seed, float solid_fraction,
                            float rmin, float rmax, lo_info* info) {
    const double H = (double)(ny - 2);
    for (int y = 0; y < ny; ++y)
        for (int x = 0; x < nx; ++x) {
            lo_info* c = &info[(size_t)y * nx + x];
            c->block_iter = -1;
            c->vx = 0.0f;
            c->vy = 0.0f;
            if (y == 0 || y == ny - 1) {
                c->material = M_BOUNDARY;
            } else if (x == 0) {
                c->material = M_INLET;
                double s = (double)y - 0.5; /* walls sit half-way between rows 0|1 and ny-2|ny-1 */
                c->vx = (float)(4.0 * (double)u_max * s * (H - s) / (H * H));
            } else if (x == nx - 1) {
                c->material = M_OUTLET;
            } else {
                c->material = M_BULK;
            }
        }
    /* seeded non-overlapping disks by rejection sampling */
    const long target = (long)ceil((double)solid_fraction * (double)nx * (double)ny);
    const double xlo = nx / 16 > 2 ? (double)(nx / 16) : 2.0;
    const double xhi = (double)(nx - 1) - (nx / 8 > 2 ? (double)(nx / 8) : 2.0);
    const double ylo = 2.0, yhi = (double)(ny - 3);
    mt64 rng;
    mt64_seed(&rng, seed);
    int cap = 4096, nd = 0;
    double* disks = (double*)malloc(sizeof(double) * 3 * cap);
    long solid = 0;
    long attempts = 0, max_attempts = 200000;
    while (solid < target && attempts < max_attempts) {
        ++attempts;
        double r = (double)rmin + ((double)rmax - (double)rmin) * mt64_unit(&rng);
        double u2 = mt64_unit(&rng), u3 = mt64_unit(&rng);
        if (xhi - xlo < 2.0 * r || yhi - ylo < 2.0 * r) continue;
        double cx = xlo + r + (xhi - xlo - 2.0 * r) * u2;
        double cy = ylo + r + (yhi - ylo - 2.0 * r) * u3;
        int ok = 1;
        for (int k = 0; k < nd; ++k) {
            double dx = cx - disks[3 * k], dy = cy - disks[3 * k + 1];
            double md = r + disks[3 * k + 2] + 2.0;
            if (dx * dx + dy * dy < md * md) { ok = 0; break; }
        }
        if (!ok) continue;
        if (nd == cap) { cap *= 2; disks = (double*)realloc(disks, sizeof(double) * 3 * cap); }
        disks[3 * nd] = cx; disks[3 * nd + 1] = cy; disks[3 * nd + 2] = r; ++nd;
        int x0 = (int)floor(cx - r), x1 = (int)ceil(cx + r), y0 = (int)floor(cy - r), y1 = (int)ceil(cy + r);
        for (int y = y0; y <= y1; ++y)
            for (int x = x0; x <= x1; ++x) {
                if (x < 1 || x > nx - 2 || y < 1 || y > ny - 2) continue;
                double dx = (double)x - cx, dy = (double)y - cy;
                if (dx * dx + dy * dy <= r * r) {
                    lo_info* c = &info[(size_t)y * nx + x];
                    if (c->material != M_OBSTACLE) { c->material = M_OBSTACLE; ++solid; }
                }
            }
    }
    free(disks);
    return nd;
}

/* generic physics step, instantiated for float and double */
#define LO_REAL float
#define LO_SFX f32
#include "lbm_oracle_phys.inc"
#undef LO_REAL
#undef LO_SFX
#define LO_REAL double
#define LO_SFX f64
#include "lbm_oracle_phys.inc"
#undef LO_REAL
#undef LO_SFX

/* ------------------------------------------------------------------------- */
/* consumers of the macro field: particles, canvas, curl, colour maps        */
/* ------------------------------------------------------------------------- */
#include "lbm_oracle_view.inc"
