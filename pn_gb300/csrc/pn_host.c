/*
 * pn_host.c -- host-side utilities of libpn: initial-condition generators and the
 * reference's text formats.  Plain C, no CUDA.
 *
 *   pn_read_init / pn_write_init   input file, Limit-sticky9.c:779-811 (fscanf "%f %f %f")
 *   pn_write_snapshot              snapshot block, Limit-sticky9.c:820-826, 899-905, 910-916
 *   pn_ic_uniform_sphere           cold uniform ball (the reference's Init10k-sphere.dat is a
 *                                  cold sphere of this kind)
 *   pn_ic_plummer                  Plummer sphere, Aarseth, Henon & Wielen (1974, A&A 37, 183)
 */
#include <math.h>
#include <stdio.h>
#include <stdlib.h>

#include "../../include/pn.h"

/* splitmix64 (Steele, Lea & Flood 2014): a small, portable, seedable generator. */
static uint64_t sm64_next(uint64_t *s) {
    uint64_t z = (*s += 0x9E3779B97F4A7C15ULL);
    z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ULL;
    z = (z ^ (z >> 27)) * 0x94D049BB133111EBULL;
    return z ^ (z >> 31);
}

/* Uniform double in [0, 1) with 53 random bits. */
static double u01(uint64_t *s) { return (double)(sm64_next(s) >> 11) * (1.0 / 9007199254740992.0); }

/* Isotropic direction scaled to length r (uniform z in [-1,1], uniform azimuth). */
static void iso(uint64_t *s, double r, double out[3]) {
    double z = (1.0 - 2.0 * u01(s)) * r;
    double ph = 2.0 * 3.14159265358979323846 * u01(s);
    double rho = sqrt(r * r - z * z > 0.0 ? r * r - z * z : 0.0);
    out[0] = rho * cos(ph);
    out[1] = rho * sin(ph);
    out[2] = z;
}

int pn_ic_uniform_sphere(int nstars, double radius, uint64_t seed, double *x, double *v) {
    if (nstars < 0 || (nstars > 0 && (!x || !v)) || !(radius > 0.0)) return PN_ERR_INVALID;
    uint64_t s = seed;
    for (int i = 0; i < nstars; i++) {
        double r = radius * cbrt(u01(&s));
        iso(&s, r, x + 3 * i);
        v[3 * i] = v[3 * i + 1] = v[3 * i + 2] = 0.0;
    }
    return PN_OK;
}

int pn_ic_plummer(int nstars, uint64_t seed, double *x, double *v) {
    if (nstars < 0 || (nstars > 0 && (!x || !v))) return PN_ERR_INVALID;
    uint64_t s = seed;
    const double pi = 3.14159265358979323846;
    const double rscale = 3.0 * pi / 16.0;    /* a = 1 model -> Henon length unit */
    const double vscale = 1.0 / sqrt(rscale); /* velocity unit follows from G = M = 1 */
    for (int i = 0; i < nstars; i++) {
        /* radius from the cumulative mass M(r) = r^3 (1 + r^2)^(-3/2); the outer 0.1 % of
         * the mass is cut (X1 <= 0.999), as is customary for this sampler. */
        double X1;
        do {
            X1 = u01(&s);
        } while (X1 <= 1e-12 || X1 > 0.999);
        double r = 1.0 / sqrt(pow(X1, -2.0 / 3.0) - 1.0);
        iso(&s, r, x + 3 * i);
        /* speed: q = v / v_esc drawn from g(q) = q^2 (1 - q^2)^(7/2) by rejection
         * (max g < 0.1), v_esc = sqrt(2) (1 + r^2)^(-1/4). */
        double q;
        for (;;) {
            double X4 = u01(&s), X5 = u01(&s);
            if (0.1 * X5 < X4 * X4 * pow(1.0 - X4 * X4, 3.5)) {
                q = X4;
                break;
            }
        }
        double ve = sqrt(2.0) * pow(1.0 + r * r, -0.25);
        iso(&s, q * ve, v + 3 * i);
        for (int k = 0; k < 3; k++) {
            x[3 * i + k] *= rscale;
            v[3 * i + k] *= vscale;
        }
    }
    /* centre-of-mass frame (equal masses) */
    if (nstars > 0) {
        double cx[3] = {0, 0, 0}, cv[3] = {0, 0, 0};
        for (int i = 0; i < nstars; i++)
            for (int k = 0; k < 3; k++) {
                cx[k] += x[3 * i + k];
                cv[k] += v[3 * i + k];
            }
        for (int k = 0; k < 3; k++) {
            cx[k] /= nstars;
            cv[k] /= nstars;
        }
        for (int i = 0; i < nstars; i++)
            for (int k = 0; k < 3; k++) {
                x[3 * i + k] -= cx[k];
                v[3 * i + k] -= cv[k];
            }
    }
    return PN_OK;
}

int pn_read_init(const char *path, int nstars, double *x, double *v) {
    if (!path || nstars < 0 || (nstars > 0 && (!x || !v))) return PN_ERR_INVALID;
    FILE *fp = fopen(path, "r");
    if (!fp) return PN_ERR_IO;
    int rc = PN_OK;
    for (int pass = 0; pass < 2 && rc == PN_OK; pass++) {
        double *dst = pass == 0 ? x : v;
        for (int i = 0; i < nstars; i++) {
            float a, b, c; /* parsed as float and widened, Limit-sticky9.c:766, 796-808 */
            if (fscanf(fp, "%f %f %f \n", &a, &b, &c) != 3) {
                rc = PN_ERR_IO;
                break;
            }
            dst[3 * i] = a;
            dst[3 * i + 1] = b;
            dst[3 * i + 2] = c;
        }
    }
    fclose(fp);
    return rc;
}

int pn_write_init(const char *path, int nstars, const double *x, const double *v) {
    if (!path || nstars < 0 || (nstars > 0 && (!x || !v))) return PN_ERR_INVALID;
    FILE *fp = fopen(path, "w");
    if (!fp) return PN_ERR_IO;
    /* 9 significant digits: every float value read back by "%f" is reproduced exactly */
    for (int pass = 0; pass < 2; pass++) {
        const double *src = pass == 0 ? x : v;
        for (int i = 0; i < nstars; i++)
            fprintf(fp, "%.9g %.9g %.9g\n", (double)(float)src[3 * i],
                    (double)(float)src[3 * i + 1], (double)(float)src[3 * i + 2]);
    }
    return fclose(fp) == 0 ? PN_OK : PN_ERR_IO;
}

int pn_write_snapshot(const char *path, int n, const double *x, const double *v, int append) {
    if (!path || n < 0 || (n > 0 && (!x || !v))) return PN_ERR_INVALID;
    FILE *fp = fopen(path, append ? "a" : "w");
    if (!fp) return PN_ERR_IO;
    for (int i = 0; i < n; i++) fprintf(fp, "%lf %lf %lf \n", x[3 * i], x[3 * i + 1], x[3 * i + 2]);
    for (int i = 0; i < n; i++) fprintf(fp, "%lf %lf %lf \n", v[3 * i], v[3 * i + 1], v[3 * i + 2]);
    return fclose(fp) == 0 ? PN_OK : PN_ERR_IO;
}
