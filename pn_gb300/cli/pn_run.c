/*
 * pn_run.c -- command-line driver equivalent to the reference's main (Limit-sticky9.c:740-920)
 * on the device-resident API.
 *
 * Defaults are the reference's run parameters: eps = 0.001 (:770), dt = 1/131072 (:771),
 * n = 10001 (:772), endtime = 10 (:774), deouttime = 0.005 (:775), input Init10k-sphere.dat
 * (:779), output Sphere-r10-1PN.dat (:777), masses m0 = 100/n and m_i = 1/(n-1) (:813-816),
 * the BH at the origin at rest (:786-792).  As the reference, it prints "Init", "start", the
 * initial energies, the energies and DE at every snapshot time, writes the initial state, a
 * snapshot at every snapshot time and the final state in the reference's "%lf %lf %lf \n"
 * format, and prints the final time.
 *
 * Additions: --precision fp64|mixed, --inv-c2 (1/c^2), --lossless (snapshots with %.17g),
 * --checkpoint FILE (binary checkpoint at every snapshot time), --resume FILE.
 *
 *   pn_run [--input F] [--output F] [-n N] [--eps E] [--dt DT] [--endtime T] [--deouttime D]
 *          [--precision fp64|mixed] [--inv-c2 X] [--lossless] [--checkpoint F] [--resume F]
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include "../../include/pn.h"

static int write_snap(const char *path, int n, const double *x, const double *v, int lossless) {
    if (!lossless) return pn_write_snapshot(path, n, x, v, 1);
    FILE *fp = fopen(path, "a");
    if (!fp) return PN_ERR_IO;
    for (int i = 0; i < n; i++) fprintf(fp, "%.17g %.17g %.17g\n", x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    for (int i = 0; i < n; i++) fprintf(fp, "%.17g %.17g %.17g\n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return fclose(fp) == 0 ? PN_OK : PN_ERR_IO;
}

static void print_energy(double t, const pn_energy_t *e, int with_de, double init_ene) {
    printf("time = %g\n", t);
    printf("pot = %22.15e kin = %22.15e \n pot_pn = %22.15e \n  total= %22.15e ratio = %e\n", e->pot_n,
           e->kin_n, e->pot_pn, e->total, e->kin_n / e->pot_n);
    if (with_de) printf(" DE = %e %g\n", (init_ene - e->total) / e->total, t);
}

static int die(const char *what, int rc) {
    fprintf(stderr, "pn_run: %s: %s (%s)\n", what, pn_strerror(rc), pn_last_error_message());
    return 1;
}

int main(int argc, char **argv) {
    const char *input = "Init10k-sphere.dat", *output = "Sphere-r10-1PN.dat";
    const char *ckpt = NULL, *resume = NULL;
    int n = 10001, lossless = 0;
    double endtime = 10.0, deouttime = 0.005;
    pn_params p;
    pn_params_default(&p);
    for (int a = 1; a < argc; a++) {
        const char *k = argv[a];
        const char *val = a + 1 < argc ? argv[a + 1] : NULL;
        if (!strcmp(k, "--lossless")) { lossless = 1; continue; }
        if (!val) { fprintf(stderr, "pn_run: %s needs a value\n", k); return 2; }
        if (!strcmp(k, "--input")) input = val;
        else if (!strcmp(k, "--output")) output = val;
        else if (!strcmp(k, "-n")) n = atoi(val);
        else if (!strcmp(k, "--eps")) p.eps = atof(val);
        else if (!strcmp(k, "--dt")) p.dt = atof(val);
        else if (!strcmp(k, "--endtime")) endtime = atof(val);
        else if (!strcmp(k, "--deouttime")) deouttime = atof(val);
        else if (!strcmp(k, "--inv-c2")) p.inv_c2 = atof(val);
        else if (!strcmp(k, "--precision")) p.precision = !strcmp(val, "mixed") ? PN_PREC_MIXED : PN_PREC_FP64;
        else if (!strcmp(k, "--checkpoint")) ckpt = val;
        else if (!strcmp(k, "--resume")) resume = val;
        else { fprintf(stderr, "pn_run: unknown option %s\n", k); return 2; }
        a++;
    }
    if (n < 2 || n > PN_NMAX) { fprintf(stderr, "pn_run: n out of range\n"); return 2; }
    double *x = calloc((size_t)3 * n, sizeof(double)), *v = calloc((size_t)3 * n, sizeof(double));
    double *m = calloc((size_t)n, sizeof(double));
    if (!x || !v || !m) return 1;
    pn_ctx *ctx = NULL;
    int rc = pn_create(&ctx, n, &p);
    if (rc) return die("pn_create", rc);
    double time = 0.0, eouttime, init_ene;
    pn_energy_t e;
    if (resume) {
        rc = pn_load_checkpoint(ctx, resume, &eouttime, &init_ene);
        if (rc) return die("resume", rc);
        time = pn_time(ctx);
    } else {
        printf("Init \n");                                   /* :794 */
        rc = pn_read_init(input, n - 1, x + 3, v + 3);       /* :795-811, BH row 0 stays 0 */
        if (rc) { perror("data_input"); return 1; }
        m[0] = 100.0 / (double)n;                            /* :813-816 */
        for (int i = 1; i < n; i++) m[i] = 1.0 / (double)(n - 1);
        printf("start \n");
        remove(output);
        rc = write_snap(output, n, x, v, lossless);          /* :820-826 */
        if (rc) return die("snapshot", rc);
        rc = pn_set_state(ctx, n, x, v, m);
        if (rc) return die("pn_set_state", rc);
        eouttime = time + deouttime;                          /* :828 */
    }
    /* An energy owed for the current state (initial_energy at :837, or energy at a snapshot,
     * :896) is taken from the force sweep that starts the next steps at that same state
     * (pn_steps_energy_async) and printed when those steps are done; a snapshot's state is
     * copied out while those steps run (pn_snapshot_begin/end) and written to the file before
     * the energy line is printed.  Printed lines and their order are the reference's.  A run
     * that ends on a snapshot, or that writes checkpoints, uses a separate energy sweep. */
    enum { OWE_NONE, OWE_INITIAL, OWE_SNAPSHOT } owed = resume ? OWE_NONE : OWE_INITIAL;
    double owed_time = 0.0;
    int snap_pending = 0;
    if (owed == OWE_INITIAL && !(time < endtime)) {
        rc = pn_energy(ctx, &e);
        if (rc) return die("pn_energy", rc);
        print_energy(0.0, &e, 0, 0.0);
        init_ene = e.total;
        owed = OWE_NONE;
    }
    /* the reference steps until time >= endtime, with a snapshot whenever time >= eouttime
     * (:841-908); steps between snapshots run back to back on the GPU */
    while (time < endtime) {
        int k = 0;
        double t = time;
        while (t < endtime) {
            t += p.dt;
            k++;
            if (t >= eouttime) break;
        }
        rc = owed != OWE_NONE ? pn_steps_energy_async(ctx, k) : pn_steps(ctx, k);
        if (rc) return die("pn_steps", rc);
        if (snap_pending) {  /* the previous snapshot, written while these steps run */
            rc = pn_snapshot_end(ctx, x, v);
            if (!rc) rc = write_snap(output, n, x, v, lossless);
            if (rc) return die("snapshot", rc);
            snap_pending = 0;
        }
        if (owed != OWE_NONE) {
            rc = pn_energy_result(ctx, &e);
            if (rc) return die("pn_steps_energy", rc);
            if (owed == OWE_INITIAL) {
                print_energy(0.0, &e, 0, 0.0);
                init_ene = e.total;
            } else {
                print_energy(owed_time, &e, 1, init_ene);
            }
            owed = OWE_NONE;
        } else {
            rc = pn_sync(ctx);
            if (rc) return die("pn_steps", rc);
        }
        time = t;
        if (time >= eouttime) {                               /* :895-906 */
            eouttime += deouttime;
            if (ckpt || !(time < endtime)) {
                rc = pn_get_state(ctx, x, v);
                if (!rc) rc = write_snap(output, n, x, v, lossless);
                if (rc) return die("snapshot", rc);
                rc = pn_energy(ctx, &e);
                if (rc) return die("pn_energy", rc);
                print_energy(time, &e, 1, init_ene);
                if (ckpt) {
                    rc = pn_save_checkpoint(ctx, ckpt, eouttime, init_ene);
                    if (rc) return die("checkpoint", rc);
                }
            } else {
                rc = pn_snapshot_begin(ctx);
                if (rc) return die("snapshot", rc);
                snap_pending = 1;
                owed = OWE_SNAPSHOT;
                owed_time = time;
            }
            fflush(stdout);
        }
    }
    rc = pn_get_state(ctx, x, v);                             /* :910-916 */
    if (!rc) rc = write_snap(output, n, x, v, lossless);
    if (rc) return die("final snapshot", rc);
    printf("%lf \n", time);                                   /* :919 */
    pn_destroy(ctx);
    free(x);
    free(v);
    free(m);
    return 0;
}
