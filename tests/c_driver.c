/* Minimal C driver of libps3d_gpu.so: the calls a Fortran or C host makes
 * through the C ABI of include/ps3d_gpu.h, in plain C99.
 *
 *   c_driver [n] [steps] [checkpoint-path]
 *
 * Builds the Beltrami vorticity (beltrami.f90:162-181; k = l = 2, m = 1) on
 * an n^3 grid of the box (2 pi, 2 pi, pi) with lower z = -pi/2, sets it up
 * (setup_fields, utils.f90:136-184), advances `steps` steps of the FP64 form,
 * prints the energy series and writes a checkpoint.  Without a CUDA device it
 * reports PS3D_ERR_NO_DEVICE and exits 0.
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "ps3d_gpu.h"

static const double PI = 3.14159265358979323846;

static int check(ps3d_gpu_ctx *ctx, int rc, const char *what)
{
    if (rc != PS3D_OK) {
        fprintf(stderr, "%s: %s (%s)\n", what, ps3d_gpu_strerror(rc), ctx ? ps3d_gpu_last_error(ctx) : "");
        return 1;
    }
    return 0;
}

int main(int argc, char **argv)
{
    const int n = argc > 1 ? atoi(argv[1]) : 32;
    const int steps = argc > 2 ? atoi(argv[2]) : 2;
    const char *ckpt = argc > 3 ? argv[3] : NULL;
    ps3d_gpu_config cfg;
    memset(&cfg, 0, sizeof(cfg));
    cfg.nx = cfg.ny = cfg.nz = n;
    cfg.nnu = 3;
    cfg.lower[0] = 0.0;
    cfg.lower[1] = 0.0;
    cfg.lower[2] = -0.5 * PI;
    cfg.extent[0] = 2.0 * PI;
    cfg.extent[1] = 2.0 * PI;
    cfg.extent[2] = PI;
    cfg.prediss = 30.0;
    cfg.pretype = PS3D_PRE_VORCH;
    cfg.length_scale = PS3D_KOLMOGOROV;
    cfg.filtering = PS3D_HOU_LI;
    cfg.stepper = PS3D_IMPL_DIFF_RK4;
    cfg.cflmax = 0.5;
    cfg.alpha = 0.1;
    cfg.time_limit = 1.0e30;
    cfg.roll_mean_win_size = 1000;
    cfg.precision = PS3D_PRECISION_FP64;
    cfg.device = 0;
    cfg.buoy_roll_mean_win_size = 1000;

    ps3d_gpu_ctx *ctx = NULL;
    int rc = ps3d_gpu_create(&cfg, &ctx);
    if (rc == PS3D_ERR_NO_DEVICE) {
        printf("c_driver: %s\n", ps3d_gpu_strerror(rc));
        return 0;
    }
    if (check(ctx, rc, "create")) return 1;

    /* Beltrami vorticity, reference host layout (0:nz, 0:ny-1, 0:nx-1) */
    const size_t nz1 = (size_t)n + 1, nf = nz1 * (size_t)n * (size_t)n;
    double *vor = malloc(3 * nf * sizeof(double));
    if (!vor) return 1;
    const double k = 2.0, l = 2.0, m = 1.0, alpha = sqrt(k * k + l * l + m * m), f = alpha / (k * k + l * l);
    for (int ix = 0; ix < n; ++ix)
        for (int iy = 0; iy < n; ++iy)
            for (int iz = 0; iz <= n; ++iz) {
                const double x = cfg.lower[0] + cfg.extent[0] / n * ix;
                const double y = cfg.lower[1] + cfg.extent[1] / n * iy;
                const double z = cfg.lower[2] + cfg.extent[2] / n * iz;
                const size_t i = (size_t)iz + nz1 * ((size_t)iy + (size_t)n * (size_t)ix);
                const double s = sin(k * x + l * y), c = cos(k * x + l * y);
                vor[i] = f * (k * m * sin(m * z) - l * alpha * cos(m * z)) * s;
                vor[nf + i] = f * (l * m * sin(m * z) + k * alpha * cos(m * z)) * s;
                vor[2 * nf + i] = alpha * cos(m * z) * c;
            }
    double te = 0.0, en = 0.0, t = 0.0;
    rc = ps3d_gpu_setup_fields(ctx, vor, NULL, &te, &en);
    free(vor);
    if (check(ctx, rc, "setup_fields")) return 1;
    printf("c_driver: %d^3, te %.12f, en %.12f\n", n, te, en);
    for (int s = 0; s < steps; ++s) {
        ps3d_gpu_diag d;
        if (check(ctx, ps3d_gpu_advance(ctx, &t, 1, &d), "advance")) return 1;
        printf("c_driver: t %.6f dt %.6f ke %.12f en %.12f hel %.12f\n", t, d.dt, d.ke, d.en, d.hel);
    }
    if (ckpt && check(ctx, ps3d_gpu_save_state(ctx, ckpt, t), "save_state")) return 1;
    return check(ctx, ps3d_gpu_destroy(ctx), "destroy");
}
