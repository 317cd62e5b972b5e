/*
 * ref_harness.c -- builds the UNMODIFIED reference functions (Limit-sticky9.c) into a shared
 * library for parity checks.  TEST INFRASTRUCTURE ONLY: the output goes to oracle/_ref/,
 * which is git-ignored.  The reference source is included from where it lies (its path is
 * passed by oracle/Makefile as LS9_SOURCE); nothing of it is copied into this repository.
 *
 * The reference's main() is renamed so that the file can be linked as a library, and its
 * three entry points are re-exported under ls9_* names so they do not clash with the
 * drop-in symbols of libpn.so when both are loaded into one process.
 *
 * ls9_rk_step restates the body of the reference's integration loop
 * (Limit-sticky9.c:844-893) around the reference's own force(), with the same arithmetic
 * order, so that trajectories can be generated from the reference code.
 */
#define main ls9_reference_main
#include LS9_SOURCE
#undef main

#include <string.h>

void ls9_force(double (*x)[3], double (*v)[3], double *m, double eps, double (*a)[3], int n) {
    force(x, v, m, eps, a, (double *)0, n);
}

void ls9_initial_energy(double (*x)[3], double (*v)[3], double *m, int n, double *init_ene,
                        double eps) {
    initial_energy(x, v, m, n, init_ene, eps);
}

void ls9_energy(double t, double (*x)[3], double (*v)[3], double *m, int n, double init_ene,
                double eps) {
    energy(t, x, v, m, n, init_ene, eps);
}

/* One integration step on x, v (in place).  scratch: 11*3*n doubles. */
void ls9_rk_step(double (*x)[3], double (*v)[3], double *m, double eps, double dt, int n,
                 double *scratch) {
    size_t s3 = (size_t)3 * (size_t)n;
    double *hx = scratch, *hv = scratch + 4 * s3;
    double (*x1)[3] = (double (*)[3])(scratch + 8 * s3);
    double (*v1)[3] = (double (*)[3])(scratch + 9 * s3);
    double (*a)[3] = (double (*)[3])(scratch + 10 * s3);
    double *xf = &x[0][0], *vf = &v[0][0], *x1f = &x1[0][0], *v1f = &v1[0][0], *af = &a[0][0];
    memcpy(hx, xf, s3 * sizeof(double));
    memcpy(hv, vf, s3 * sizeof(double));
    force(x, v, m, eps, a, (double *)0, n);
    for (size_t q = 0; q < s3; q++) {
        x1f[q] = xf[q] + 0.5 * vf[q] * dt;
        v1f[q] = vf[q] + 0.5 * af[q] * dt;
        hx[s3 + q] = x1f[q];
        hv[s3 + q] = v1f[q];
    }
    force(x1, v1, m, eps, a, (double *)0, n);
    for (size_t q = 0; q < s3; q++) {
        x1f[q] = xf[q] + 0.5 * v1f[q] * dt;
        v1f[q] = vf[q] + 0.5 * af[q] * dt;
        hx[2 * s3 + q] = x1f[q];
        hv[2 * s3 + q] = v1f[q];
    }
    force(x1, v1, m, eps, a, (double *)0, n);
    for (size_t q = 0; q < s3; q++) {
        x1f[q] = xf[q] + v1f[q] * dt;
        v1f[q] = vf[q] + af[q] * dt;
        hx[3 * s3 + q] = x1f[q];
        hv[3 * s3 + q] = v1f[q];
    }
    for (size_t q = 0; q < s3; q++) {
        xf[q] = (hx[q] + hx[3 * s3 + q] + 2.0 * (hx[s3 + q] + hx[2 * s3 + q])) / 6.0;
        vf[q] = (hv[q] + hv[3 * s3 + q] + 2.0 * (hv[s3 + q] + hv[2 * s3 + q])) / 6.0;
    }
}
