/* A plain C99 caller of liblbm.so through include/lbm.h only: what a host application written in
 * another language binds (no Python, no torch).  It builds a physics-mode moving-lid cavity and
 * a reference-mode Poiseuille lattice driven the way simuverse's FluidSimulator drives it
 * (frames of two steps, a click, a force stroke, a viscosity change), checks the statuses, mass
 * conservation and the read-back fields, and the argument errors.  Prints "ok" and returns 0, or
 * names the first failed check and returns 1.  Run by tests/test_gpu_abi.py. */
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "lbm.h"

#define CHECK(cond, ...)                           \
    do {                                           \
        if (!(cond)) {                             \
            fprintf(stderr, "FAILED %s: ", #cond); \
            fprintf(stderr, __VA_ARGS__);          \
            fprintf(stderr, " (%s)\n", lbm_last_error()); \
            return 1;                              \
        }                                          \
    } while (0)

static int cavity(void) {
    lbm_params p;
    lbm_params_default(&p);
    p.nx = 200;
    p.ny = 150;
    p.mode = LBM_MODE_PHYSICS;
    p.scene = LBM_SCENE_CAVITY;
    p.tau = 0.6f;
    p.lid_speed = 0.1f;
    lbm_handle* h = NULL;
    CHECK(lbm_create(&p, &h) == LBM_OK && h != NULL, "create cavity");
    int32_t nx = 0, ny = 0;
    CHECK(lbm_get_size(h, &nx, &ny) == LBM_OK && nx == 200 && ny == 150, "size %d x %d", nx, ny);
    double m0[3], m1[3];
    CHECK(lbm_conservation(h, m0) == LBM_OK, "conservation");
    CHECK(lbm_step(h, 500) == LBM_OK, "step");
    CHECK(lbm_conservation(h, m1) == LBM_OK, "conservation");
    CHECK(fabs(m1[0] - m0[0]) <= 1e-10 * m0[0], "mass %.17g -> %.17g", m0[0], m1[0]);
    uint64_t done = 0;
    CHECK(lbm_steps_done(h, &done) == LBM_OK && done == 500, "steps done %llu", (unsigned long long)done);
    const size_t n = (size_t)nx * ny;
    float* rho = (float*)malloc(n * sizeof(float));
    float* ux = (float*)malloc(n * sizeof(float));
    float* uy = (float*)malloc(n * sizeof(float));
    CHECK(rho && ux && uy, "host memory");
    CHECK(lbm_read_macro(h, rho, ux, uy) == LBM_OK, "read macro");
    double umax = 0.0;
    for (size_t c = 0; c < n; ++c) {
        CHECK(isfinite(rho[c]) && isfinite(ux[c]) && isfinite(uy[c]), "finite at %zu", c);
        const double u = sqrt((double)ux[c] * ux[c] + (double)uy[c] * uy[c]);
        if (u > umax) umax = u;
    }
    /* the lid drives the flow: the largest speed is near the lid speed, not above it */
    CHECK(umax > 0.02 && umax < 0.12, "max speed %g", umax);
    uint64_t bad = 1;
    CHECK(lbm_check_finite(h, &bad) == LBM_OK && bad == 0, "non-finite %llu", (unsigned long long)bad);
    free(rho);
    free(ux);
    free(uy);
    CHECK(lbm_destroy(h) == LBM_OK, "destroy");
    return 0;
}

static int poiseuille(void) {
    lbm_params p;
    lbm_params_default(&p); /* the reference UI's lattice: 600 x 375, Poiseuille, reference rules */
    lbm_handle* h = NULL;
    CHECK(lbm_create(&p, &h) == LBM_OK, "create poiseuille");
    for (int frame = 0; frame < 20; ++frame) CHECK(lbm_compute(h) == LBM_OK, "compute frame %d", frame);
    CHECK(lbm_on_click(h, 600.0f, 300.0f) == LBM_OK, "click");
    CHECK(lbm_touch_begin(h) == LBM_OK, "touch begin");
    /* the first point of a stroke only records the position (a status above zero) */
    CHECK(lbm_touch_move(h, 300.0f, 200.0f) == LBM_IGNORED, "touch move: first point");
    CHECK(lbm_touch_move(h, 340.0f, 210.0f) == LBM_OK, "touch move");
    CHECK(lbm_update_viscosity(h, 0.03f) == LBM_OK, "viscosity");
    for (int frame = 0; frame < 20; ++frame) CHECK(lbm_compute(h) == LBM_OK, "compute frame %d", frame);
    uint64_t done = 0;
    CHECK(lbm_steps_done(h, &done) == LBM_OK && done == 80, "steps done %llu", (unsigned long long)done);
    const size_t n = (size_t)p.nx * p.ny;
    uint16_t* tex = (uint16_t*)malloc(4 * n * sizeof(uint16_t));
    CHECK(tex != NULL, "host memory");
    CHECK(lbm_read_macro_rgba16f(h, tex) == LBM_OK, "rgba16f");
    size_t moving = 0;
    for (size_t c = 0; c < n; ++c)
        if ((tex[4 * c] & 0x7fff) != 0) ++moving; /* ux is not +-0 */
    CHECK(moving > n / 4, "moving cells %zu of %zu", moving, n);
    free(tex);
    CHECK(lbm_reset(h) == LBM_OK, "reset");
    CHECK(lbm_destroy(h) == LBM_OK, "destroy");
    return 0;
}

static int errors(void) {
    lbm_params p;
    lbm_params_default(&p);
    p.nx = 2;
    lbm_handle* h = (lbm_handle*)&p; /* must be cleared on failure */
    CHECK(lbm_create(&p, &h) == LBM_ERR_ARG && h == NULL, "small lattice accepted");
    CHECK(strlen(lbm_last_error()) > 0, "no message");
    CHECK(lbm_step(NULL, 1) == LBM_ERR_ARG, "null handle");
    CHECK(lbm_destroy(NULL) == LBM_OK, "destroy null");
    CHECK(lbm_create(NULL, &h) == LBM_ERR_ARG, "null params");
    uint64_t reserved = 0, used = 0;
    CHECK(lbm_memory_stats(&reserved, &used) == LBM_OK && used <= reserved, "pool stats %llu %llu",
          (unsigned long long)reserved, (unsigned long long)used);
    CHECK(lbm_memory_trim() == LBM_OK, "trim");
    return 0;
}

int main(void) {
    CHECK(lbm_abi_version() == LBM_ABI_VERSION, "ABI version %d", lbm_abi_version());
    if (cavity() || poiseuille() || errors()) return 1;
    printf("ok\n");
    return 0;
}
