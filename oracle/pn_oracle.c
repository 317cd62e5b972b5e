/*
 * pn_oracle.c -- CPU restatement of the Limit-sticky9 direct-summation force path.
 *
 * TEST INFRASTRUCTURE ONLY.  This file is the checker that the CUDA library is compared
 * against; it is never linked into, called by, or used as a fallback for the product library
 * (pn_gb300/libpn.so).  Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg
 * load it.
 *
 * What it restates (file:line in the reference project, Limit-sticky9.c):
 *   orc_force            force()            Limit-sticky9.c:21-424
 *   orc_energy           energy() / initial_energy() arithmetic
 *                                           Limit-sticky9.c:427-564 and 566-714
 *   orc_rk_step          one step of the main loop's Runge-Kutta scheme
 *                                           Limit-sticky9.c:841-893
 *
 * Bit-exactness.  Every expression keeps the reference's association order and its
 * operand order, so that with gcc -O2 -ffp-contract=off the results are bit-identical to the
 * reference functions compiled with the same flags (checked by tests/test_oracle.py against
 * oracle/_ref and against committed golden vectors).  Values the reference recomputes
 * unchanged inside inner loops (e.g. the i-particle's BH distance) are computed once here:
 * that does not change a single bit.  The layout is AoS double[n][3], index 0 = the BH,
 * exactly as the reference's arrays.
 *
 * Differences from the reference that do not touch arithmetic:
 *   - scratch (the reference's 6.5 MB stack array ac[NMAX][3] and the energy's pot arrays)
 *     is heap-allocated, so the oracle runs on any thread;
 *   - energy components are returned instead of printed;
 *   - inv_c2 is not supported here: the oracle is the reference, c = 1 (G = c = 1 units).
 */
#include <stdlib.h>
#include <string.h>
#include <tgmath.h>

/* The arithmetic type.  The default build uses double, as the reference.  Built with
 * -DORC_LONG_DOUBLE the same algorithm runs in long double (x86-64: 64-bit significand) and
 * exports orcld_* entry points: the reference's formulas evaluated with ~11 more bits, i.e.
 * the exact value the reference's own double rounding is measured against. */
#ifdef ORC_LONG_DOUBLE
typedef long double real;
#define ORC(name) orcld_##name
#else
typedef double real;
#define ORC(name) orc_##name
#endif

/* Limit-sticky9.c:15-19: rsqrt(r2) = 1.0/sqrt(r2), correctly rounded sqrt then division. */
static real orc_rsqrt(real r2) { return 1.0 / sqrt(r2); }

/* ((a0*b0 + a1*b1) + a2*b2): the reference's inline 3-term dot product order. */
static real dot3(const real *a, const real *b) {
    return a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
}

/* Softened BH distance of particle p: returns r1be = rsqrt(|x_p - x_0|^2 + eps2) and the
 * unsoftened square in *r2_out.  The sign convention of the difference does not matter for
 * the squares (x0-xp is the exact negation of xp-x0). */
static real bh_rinv(const real *x, int p, real eps2, real *r2_out) {
    real d[3];
    for (int k = 0; k < 3; k++) d[k] = x[3 * p + k] - x[k];
    real r2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
    if (r2_out) *r2_out = r2;
    return orc_rsqrt(r2 + eps2);
}

/* ---------------------------------------------------------------------------------------
 * Newtonian star-star (and BH) accelerations, Limit-sticky9.c:36-51.
 * a_i = sum_{j=0..n-1} m_j dx (|dx|^2+eps2)^(-3/2), self pair included (it adds 0).
 * ------------------------------------------------------------------------------------- */
static void newton_all(int n, const real *x, const real *m, real eps2, real *a) {
    for (int i = 0; i < n; i++) {
        const real *xi = x + 3 * i;
        real acc[3] = {0.0, 0.0, 0.0};
        for (int j = 0; j < n; j++) {
            const real *xj = x + 3 * j;
            real dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
            real r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2] + eps2;
            real rinv = orc_rsqrt(r2);
            real mrinv = m[j] * rinv;
            real mr3inv = mrinv * rinv * rinv;
            for (int k = 0; k < 3; k++) acc[k] += mr3inv * dx[k];
        }
        for (int k = 0; k < 3; k++) a[3 * i + k] = acc[k];
    }
}

/* 1PN correction to the BH from each star, Limit-sticky9.c:54-97.  Note the unsoftened r2
 * in the 1.5 (v.dx)^2 / r2 term (a star exactly on the BH gives 0/0, as in the reference). */
static void bh_1pn_single(int n, const real *x, const real *v, const real *m,
                          real eps2, real a1[3]) {
    a1[0] = a1[1] = a1[2] = 0.0;
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dx[3];
        for (int k = 0; k < 3; k++) dx[k] = x[3 * i + k] - x[k];
        real r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2];
        real reinv = orc_rsqrt(r2 + eps2);
        real mrinv = m[i] * reinv;
        real mr3inv = mrinv * reinv * reinv;
        real vv = dot3(vi, vi);
        real vd = vi[0] * dx[0] + vi[1] * dx[1] + vi[2] * dx[2];
        for (int k = 0; k < 3; k++)
            a1[k] += mr3inv * dx[k] * (5.0 * m[0] * reinv - 2.0 * vv + 1.5 * vd * vd / r2)
                     + 3.0 * mr3inv * vi[k] * vd;
    }
}

/* The BH's three-body "cross" term a1c, Limit-sticky9.c:99-207: the single sum (:101-115),
 * the (i,j) pair sum over stars (:116-174) and the reference's self-pair removal
 * (:176-207), which keeps the reference's sign and its 1.25*eps factor verbatim. */
static void bh_cross(int n, const real *x, const real *v, const real *m, real eps,
                     real eps2, real a1c[3]) {
    a1c[0] = a1c[1] = a1c[2] = 0.0;
    /* :101-115 */
    for (int i = 1; i < n; i++) {
        real dxb[3];
        for (int k = 0; k < 3; k++) dxb[k] = x[3 * i + k] - x[k];
        real r1be = bh_rinv(x, i, eps2, NULL);
        real mr1b3e = m[i] * r1be * r1be * r1be;
        for (int k = 0; k < 3; k++) a1c[k] += 4.0 * mr1b3e * r1be * m[i] * dxb[k];
    }
    /* :116-174 */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3], r1b2;
        for (int k = 0; k < 3; k++) dxb[k] = x[3 * i + k] - x[k];
        real r1be = bh_rinv(x, i, eps2, &r1b2);
        real mr1b3e = m[i] * r1be * r1be * r1be;
        for (int j = 1; j < n; j++) {
            const real *vj = v + 3 * j;
            real dxc[3], dxbc[3];
            for (int k = 0; k < 3; k++) {
                dxc[k] = x[3 * j + k] - x[k];
                dxbc[k] = x[3 * j + k] - x[3 * i + k];
            }
            real r1c2 = dxc[0] * dxc[0] + dxc[1] * dxc[1] + dxc[2] * dxc[2];
            real r1ce = orc_rsqrt(r1c2 + eps2);
            real rbc2e = dxbc[0] * dxbc[0] + dxbc[1] * dxbc[1] + dxbc[2] * dxbc[2] + eps2;
            real rbce = orc_rsqrt(rbc2e);
            real vivj = dot3(vi, vj);
            real vidxb = dot3(vi, dxb);
            real vjdxb = dot3(vj, dxb);
            real radial = 4.0 * r1ce + 1.25 * rbce - 0.25 * r1c2 / rbc2e * rbce
                            + 0.25 * r1b2 / rbc2e * rbce;
            for (int k = 0; k < 3; k++)
                a1c[k] += mr1b3e * m[j] * dxb[k] * radial
                          - 3.5 * (rbce * rbce * rbce) * r1be * m[i] * m[j] * dxbc[k]
                          - mr1b3e * m[j] / m[0]
                                * (4.0 * vivj * dxb[k] - 3.0 * vidxb * vj[k]
                                   - 4.0 * vjdxb * vi[k]);
        }
    }
    /* :176-207 (dxb = x0 - xi here, opposite to the pair loop) */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3];
        for (int k = 0; k < 3; k++) dxb[k] = x[k] - x[3 * i + k];
        real r1be = bh_rinv(x, i, eps2, NULL);
        real mr1b3e = m[i] * r1be * r1be * r1be;
        real vivi = dot3(vi, vi);
        real vidxb = dot3(vi, dxb);
        for (int k = 0; k < 3; k++)
            a1c[k] -= mr1b3e * m[i] * dxb[k] * (4.0 * r1be + 1.25 * eps)
                      - mr1b3e * m[i] / m[0] * (4.0 * vivi * dxb[k] - 7.0 * vidxb * vi[k]);
    }
}

/* Per-star 1PN terms from the BH alone: a_{a-BH} (Limit-sticky9.c:213-238) and the direct
 * part of aa_cross (:249-274).  Added into a[i] in the reference's order. */
static void star_bh_terms(int n, const real *x, const real *v, const real *m,
                          real eps2, real *a) {
    /* :215-238, dxb = x0 - xi */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3];
        for (int k = 0; k < 3; k++) dxb[k] = x[k] - x[3 * i + k];
        real r1be = bh_rinv(x, i, eps2, NULL);
        real mrinv = m[0] * r1be;
        real mr3inv = mrinv * r1be * r1be;
        real vivi = dot3(vi, vi);
        real vidxb = dot3(vi, dxb);
        for (int k = 0; k < 3; k++)
            a[3 * i + k] += mr3inv * dxb[k] * (4.0 * mrinv - vivi)
                            + 4.0 * mr3inv * vidxb * vi[k];
    }
    /* :249-274, dxb = xi - x0 */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3];
        for (int k = 0; k < 3; k++) dxb[k] = x[3 * i + k] - x[k];
        real r1be = bh_rinv(x, i, eps2, NULL);
        real mr3inv = m[0] * r1be * r1be * r1be;
        real vivi = dot3(vi, vi);
        real vidxb = dot3(vi, dxb);
        for (int k = 0; k < 3; k++)
            a[3 * i + k] += 5.0 * mr3inv * m[i] * r1be * dxb[k]
                            - m[i] * r1be * r1be * r1be
                                  * (4.0 * vivi * dxb[k] - 7.0 * vidxb * vi[k]);
    }
}

/* The stars' three-body cross term ac[i] (Limit-sticky9.c:276-382), summed over j >= 1 with
 * the self pair included, then added to a[i] (:386-390) and followed by the exact self-pair
 * removal (:392-422). */
static void star_cross(int n, const real *x, const real *v, const real *m, real eps,
                       real eps2, real *a) {
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3], r1b2;
        for (int k = 0; k < 3; k++) dxb[k] = x[k] - x[3 * i + k];
        real r1be = bh_rinv(x, i, eps2, &r1b2);
        real vivi = dot3(vi, vi);
        real ac[3] = {0.0, 0.0, 0.0};
        for (int j = 1; j < n; j++) {
            const real *vj = v + 3 * j;
            real dxc[3], dxbc[3], dvbc[3];
            for (int k = 0; k < 3; k++) {
                dxc[k] = x[k] - x[3 * j + k];
                dxbc[k] = x[3 * j + k] - x[3 * i + k];
                dvbc[k] = vj[k] - vi[k];
            }
            real r1c2 = dxc[0] * dxc[0] + dxc[1] * dxc[1] + dxc[2] * dxc[2];
            real r1ce = orc_rsqrt(r1c2 + eps2);
            real rbc2 = dxbc[0] * dxbc[0] + dxbc[1] * dxbc[1] + dxbc[2] * dxbc[2];
            real rbc2e = rbc2 + eps2;
            real rbce = orc_rsqrt(rbc2e);
            real mr3inv = m[j] * rbce * rbce * rbce;
            real vivj = dot3(vi, vj);
            real vjdxb = dot3(vj, dxb);
            real vidxb = dot3(vi, dxb);
            real vjdxbc = dot3(vj, dxbc);
            real dv2 = dot3(dvbc, dvbc);
            real w_b = m[j] * r1be * r1be * r1be * m[0]
                         * (4.0 * rbce + 1.25 * r1ce + 0.25 * (r1b2 - rbc2) * r1ce * r1ce * r1ce);
            real w_bc = mr3inv * m[0]
                          * (4.0 * r1be + 1.25 * r1ce + 0.25 * (-r1b2 + rbc2) * r1ce * r1ce * r1ce);
            real w_c = 3.5 * m[j] * m[0] * r1ce * r1ce * r1ce * (rbce - r1be);
            real mb3 = m[j] * r1be * r1be * r1be;
            real w_v = mr3inv * (vivi - 2.0 * dv2 + 1.5 * vjdxbc * vjdxbc / rbc2e);
            real w_dv = mr3inv
                          * (dxbc[0] * (4.0 * vi[0] - 3.0 * vj[0])
                             + dxbc[1] * (4.0 * vi[1] - 3.0 * vj[1])
                             + dxbc[2] * (4.0 * vi[2] - 3.0 * vj[2]));
            for (int k = 0; k < 3; k++)
                ac[k] += w_b * dxb[k] + w_bc * dxbc[k] - w_c * dxc[k]
                         - mb3 * (4.0 * vivj * dxb[k] - 3.0 * vjdxb * vi[k] - 4.0 * vidxb * vj[k])
                         + w_v * dxbc[k] + w_dv * dvbc[k];
        }
        for (int k = 0; k < 3; k++) a[3 * i + k] += ac[k];
    }
    /* :392-422 */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dxb[3], r1b2;
        for (int k = 0; k < 3; k++) dxb[k] = x[k] - x[3 * i + k];
        real r1be = bh_rinv(x, i, eps2, &r1b2);
        real mr3inv = m[i] * r1be * r1be * r1be;
        real vivi = dot3(vi, vi);
        real vidxb = dot3(vi, dxb);
        for (int k = 0; k < 3; k++)
            a[3 * i + k] -= mr3inv * m[0] * dxb[k]
                                * (4.0 / eps + 1.25 * r1be + 0.25 * r1b2 * r1be * r1be * r1be)
                            - 3.5 * mr3inv * m[0] * (1.0 / eps - r1be) * dxb[k]
                            - mr3inv * (4.0 * vivi * dxb[k] - 7.0 * vidxb * vi[k]);
    }
}

/* force(), Limit-sticky9.c:21-424, in the reference's order of accumulation into a. */
void ORC(force)(int n, const real *x, const real *v, const real *m, real eps,
               real *a) {
    real eps2 = eps * eps;
    real a1[3], a1c[3];
    newton_all(n, x, m, eps2, a);                       /* :36-51   */
    bh_1pn_single(n, x, v, m, eps2, a1);                /* :54-95   */
    for (int k = 0; k < 3; k++) a[k] += a1[k];          /* :97      */
    bh_cross(n, x, v, m, eps, eps2, a1c);               /* :99-207  */
    for (int k = 0; k < 3; k++) a[k] += a1c[k];         /* :209-211 */
    star_bh_terms(n, x, v, m, eps2, a);                 /* :213-274 */
    star_cross(n, x, v, m, eps, eps2, a);               /* :276-422 */
}

/* The Newtonian part alone (:36-51), for tests that isolate the pair kernel. */
void ORC(force_newton)(int n, const real *x, const real *m, real eps, real *a) {
    newton_all(n, x, m, eps * eps, a);
}

/* energy() / initial_energy() arithmetic, Limit-sticky9.c:445-556 (identical to :583-699).
 * out[0] = pot_n, out[1] = kin_n, out[2] = pot_pn, out[3] = total (ene).  Returns total. */
real ORC(energy)(int n, const real *x, const real *v, const real *m, real eps,
                  real out[4]) {
    real eps2 = eps * eps;
    real kin_n = 0.0, pot_n = 0.0, pot_pn = 0.0;
    real *pot = (real *)malloc(sizeof(real) * (size_t)(n > 0 ? n : 1));
    real *pot_pn2 = (real *)malloc(sizeof(real) * (size_t)(n > 0 ? n : 1));
    /* :452-456 */
    for (int i = 0; i < n; i++) kin_n += m[i] * dot3(v + 3 * i, v + 3 * i);
    kin_n *= 0.5;
    /* :458-480 */
    for (int i = 0; i < n; i++) {
        const real *xi = x + 3 * i;
        real p = 0.0;
        for (int j = 0; j < n; j++) {
            const real *xj = x + 3 * j;
            real dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
            real r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2] + eps2;
            real rinv = orc_rsqrt(r2);
            p -= rinv * m[j];
        }
        p += m[i] / sqrt(eps2);
        pot[i] = p * m[i];
    }
    for (int i = 0; i < n; i++) pot_n += pot[i];
    pot_n *= 0.5;
    /* :484-502 */
    const real *v0 = v;
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real dx[3];
        for (int k = 0; k < 3; k++) dx[k] = x[3 * i + k] - x[k];
        real r1ainv = orc_rsqrt(dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2] + eps2);
        real mr1ainv = m[0] * r1ainv;
        real vi2 = dot3(vi, vi);
        real v0vi = dot3(v0, vi);
        real dxv0 = dot3(dx, v0);
        real dxvi = dot3(dx, vi);
        pot_pn += 0.375 * m[i] * vi2 * vi2 + 1.5 * mr1ainv * m[i] * vi2
                  + 0.5 * mr1ainv * mr1ainv * m[i]
                  + 0.5 * mr1ainv * m[i] * (3.0 * vi2 - 7.0 * v0vi - dxv0 * dxvi * r1ainv * r1ainv);
    }
    /* :504-537 */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real r1ainv = bh_rinv(x, i, eps2, NULL);
        real vi2 = dot3(vi, vi);
        real s = 0.0;
        for (int j = 1; j < n; j++) {
            const real *vj = v + 3 * j;
            real dxab[3];
            for (int k = 0; k < 3; k++) dxab[k] = x[3 * j + k] - x[3 * i + k];
            real r1binv = bh_rinv(x, j, eps2, NULL);
            real rab2e = dxab[0] * dxab[0] + dxab[1] * dxab[1] + dxab[2] * dxab[2] + eps2;
            real rabinv = orc_rsqrt(rab2e);
            real vivj = dot3(vi, vj);
            real dvi = dot3(dxab, vi);
            real dvj = dot3(dxab, vj);
            s += 0.25 * rabinv * m[i] * m[j] * (6.0 * vi2 - 7.0 * vivj - dvi * dvj / rab2e)
                 + m[0] * m[i] * m[j] * r1ainv * rabinv
                 + 0.5 * m[0] * m[i] * m[j] * r1ainv * r1binv;
        }
        pot_pn2[i] = s;
    }
    /* :539-550 */
    for (int i = 1; i < n; i++) {
        const real *vi = v + 3 * i;
        real r1ainv = bh_rinv(x, i, eps2, NULL);
        real vi2 = dot3(vi, vi);
        pot_pn2[i] -= 0.25 * m[i] * m[i] / eps * (-vi2)
                      + m[0] * m[i] * m[i] * (r1ainv / eps + 0.5 * r1ainv * r1ainv);
    }
    /* :552-556 */
    real ene = kin_n + pot_n + pot_pn;
    for (int i = 1; i < n; i++) ene += pot_pn2[i];
    free(pot);
    free(pot_pn2);
    if (out) {
        out[0] = pot_n;
        out[1] = kin_n;
        out[2] = pot_pn;
        out[3] = ene;
    }
    return ene;
}

/* One step of the main loop's integrator, Limit-sticky9.c:844-893: three force() calls,
 * three stage updates and the state-averaging combine (x <- (h0 + h3 + 2 (h1 + h2)) / 6,
 * likewise v).  x, v are updated in place.  scratch must hold 11*3*n doubles. */
void ORC(rk_step)(int n, real *x, real *v, const real *m, real eps, real dt,
                 real *scratch) {
    size_t s3 = (size_t)3 * (size_t)n;
    real *hx = scratch;            /* 4 snapshots of x */
    real *hv = scratch + 4 * s3;   /* 4 snapshots of v */
    real *x1 = scratch + 8 * s3;
    real *v1 = scratch + 9 * s3;
    real *a = scratch + 10 * s3;
    memcpy(hx, x, s3 * sizeof(real));                        /* :844-849 */
    memcpy(hv, v, s3 * sizeof(real));
    ORC(force)(n, x, v, m, eps, a);                             /* :851 */
    for (size_t q = 0; q < s3; q++) {                          /* :853-860 */
        x1[q] = x[q] + 0.5 * v[q] * dt;
        v1[q] = v[q] + 0.5 * a[q] * dt;
        hx[s3 + q] = x1[q];
        hv[s3 + q] = v1[q];
    }
    ORC(force)(n, x1, v1, m, eps, a);                           /* :862 */
    for (size_t q = 0; q < s3; q++) {                          /* :864-871 */
        x1[q] = x[q] + 0.5 * v1[q] * dt;
        v1[q] = v[q] + 0.5 * a[q] * dt;
        hx[2 * s3 + q] = x1[q];
        hv[2 * s3 + q] = v1[q];
    }
    ORC(force)(n, x1, v1, m, eps, a);                           /* :873 */
    for (size_t q = 0; q < s3; q++) {                          /* :875-882 */
        x1[q] = x[q] + v1[q] * dt;
        v1[q] = v[q] + a[q] * dt;
        hx[3 * s3 + q] = x1[q];
        hv[3 * s3 + q] = v1[q];
    }
    for (size_t q = 0; q < s3; q++) {                          /* :884-891 */
        x[q] = (hx[q] + hx[3 * s3 + q] + 2.0 * (hx[s3 + q] + hx[2 * s3 + q])) / 6.0;
        v[q] = (hv[q] + hv[3 * s3 + q] + 2.0 * (hv[s3 + q] + hv[2 * s3 + q])) / 6.0;
    }
}

/* nsteps steps of orc_rk_step; allocates its own scratch.  Returns 0, or -1 on OOM. */
int ORC(run)(int n, real *x, real *v, const real *m, real eps, real dt, int nsteps) {
    real *scratch = (real *)malloc(sizeof(real) * 33 * (size_t)(n > 0 ? n : 1));
    if (!scratch) return -1;
    for (int s = 0; s < nsteps; s++) ORC(rk_step)(n, x, v, m, eps, dt, scratch);
    free(scratch);
    return 0;
}

/* Force on a subset of i-particles (rows) only, same arithmetic as orc_force for those rows.
 * Lets tests and the CPU baseline work on a bounded sample of a large N.  rows[] holds
 * particle indices; a_out is [nrows][3].  a1c_out (optional, [nrows][3]) receives each row's
 * share of the BH's three-body sum (Limit-sticky9.c:118-174 for that i), so that a sample
 * row costs what one row of a full force() call costs.  Row 0 (the BH) is rejected (-1). */
int ORC(force_rows)(int n, const real *x, const real *v, const real *m, real eps,
                   const int *rows, int nrows, real *a_out, real *a1c_out) {
    real eps2 = eps * eps;
    for (int r = 0; r < nrows; r++) {
        int i = rows[r];
        if (i <= 0 || i >= n) return -1;
        const real *xi = x + 3 * i;
        const real *vi = v + 3 * i;
        real acc[3] = {0.0, 0.0, 0.0};
        /* :39-51 */
        for (int j = 0; j < n; j++) {
            const real *xj = x + 3 * j;
            real dx[3] = {xj[0] - xi[0], xj[1] - xi[1], xj[2] - xi[2]};
            real r2 = dx[0] * dx[0] + dx[1] * dx[1] + dx[2] * dx[2] + eps2;
            real rinv = orc_rsqrt(r2);
            real mrinv = m[j] * rinv;
            real mr3inv = mrinv * rinv * rinv;
            for (int k = 0; k < 3; k++) acc[k] += mr3inv * dx[k];
        }
        /* :215-238 */
        {
            real dxb[3];
            for (int k = 0; k < 3; k++) dxb[k] = x[k] - xi[k];
            real r1be = bh_rinv(x, i, eps2, NULL);
            real mrinv = m[0] * r1be;
            real mr3inv = mrinv * r1be * r1be;
            real vivi = dot3(vi, vi);
            real vidxb = dot3(vi, dxb);
            for (int k = 0; k < 3; k++)
                acc[k] += mr3inv * dxb[k] * (4.0 * mrinv - vivi) + 4.0 * mr3inv * vidxb * vi[k];
        }
        /* :249-274 */
        {
            real dxb[3];
            for (int k = 0; k < 3; k++) dxb[k] = xi[k] - x[k];
            real r1be = bh_rinv(x, i, eps2, NULL);
            real mr3inv = m[0] * r1be * r1be * r1be;
            real vivi = dot3(vi, vi);
            real vidxb = dot3(vi, dxb);
            for (int k = 0; k < 3; k++)
                acc[k] += 5.0 * mr3inv * m[i] * r1be * dxb[k]
                          - m[i] * r1be * r1be * r1be * (4.0 * vivi * dxb[k] - 7.0 * vidxb * vi[k]);
        }
        /* :276-390 for this i */
        {
            real dxb[3], r1b2;
            for (int k = 0; k < 3; k++) dxb[k] = x[k] - xi[k];
            real r1be = bh_rinv(x, i, eps2, &r1b2);
            real vivi = dot3(vi, vi);
            real ac[3] = {0.0, 0.0, 0.0};
            for (int j = 1; j < n; j++) {
                const real *vj = v + 3 * j;
                real dxc[3], dxbc[3], dvbc[3];
                for (int k = 0; k < 3; k++) {
                    dxc[k] = x[k] - x[3 * j + k];
                    dxbc[k] = x[3 * j + k] - xi[k];
                    dvbc[k] = vj[k] - vi[k];
                }
                real r1c2 = dxc[0] * dxc[0] + dxc[1] * dxc[1] + dxc[2] * dxc[2];
                real r1ce = orc_rsqrt(r1c2 + eps2);
                real rbc2 = dxbc[0] * dxbc[0] + dxbc[1] * dxbc[1] + dxbc[2] * dxbc[2];
                real rbc2e = rbc2 + eps2;
                real rbce = orc_rsqrt(rbc2e);
                real mr3inv = m[j] * rbce * rbce * rbce;
                real vivj = dot3(vi, vj);
                real vjdxb = dot3(vj, dxb);
                real vidxb = dot3(vi, dxb);
                real vjdxbc = dot3(vj, dxbc);
                real dv2 = dot3(dvbc, dvbc);
                real w_b = m[j] * r1be * r1be * r1be * m[0]
                             * (4.0 * rbce + 1.25 * r1ce + 0.25 * (r1b2 - rbc2) * r1ce * r1ce * r1ce);
                real w_bc = mr3inv * m[0]
                              * (4.0 * r1be + 1.25 * r1ce + 0.25 * (-r1b2 + rbc2) * r1ce * r1ce * r1ce);
                real w_c = 3.5 * m[j] * m[0] * r1ce * r1ce * r1ce * (rbce - r1be);
                real mb3 = m[j] * r1be * r1be * r1be;
                real w_v = mr3inv * (vivi - 2.0 * dv2 + 1.5 * vjdxbc * vjdxbc / rbc2e);
                real w_dv = mr3inv
                              * (dxbc[0] * (4.0 * vi[0] - 3.0 * vj[0])
                                 + dxbc[1] * (4.0 * vi[1] - 3.0 * vj[1])
                                 + dxbc[2] * (4.0 * vi[2] - 3.0 * vj[2]));
                for (int k = 0; k < 3; k++)
                    ac[k] += w_b * dxb[k] + w_bc * dxbc[k] - w_c * dxc[k]
                             - mb3 * (4.0 * vivj * dxb[k] - 3.0 * vjdxb * vi[k] - 4.0 * vidxb * vj[k])
                             + w_v * dxbc[k] + w_dv * dvbc[k];
            }
            for (int k = 0; k < 3; k++) acc[k] += ac[k];
            /* :392-422 */
            real mr3inv = m[i] * r1be * r1be * r1be;
            real vidxb = dot3(vi, dxb);
            for (int k = 0; k < 3; k++)
                acc[k] -= mr3inv * m[0] * dxb[k]
                              * (4.0 / eps + 1.25 * r1be + 0.25 * r1b2 * r1be * r1be * r1be)
                          - 3.5 * mr3inv * m[0] * (1.0 / eps - r1be) * dxb[k]
                          - mr3inv * (4.0 * vivi * dxb[k] - 7.0 * vidxb * vi[k]);
        }
        for (int k = 0; k < 3; k++) a_out[3 * r + k] = acc[k];
        if (a1c_out) {
            /* :118-174 for this i */
            real dxb[3], r1b2, s1c[3] = {0.0, 0.0, 0.0};
            for (int k = 0; k < 3; k++) dxb[k] = xi[k] - x[k];
            real r1be = bh_rinv(x, i, eps2, &r1b2);
            real mr1b3e = m[i] * r1be * r1be * r1be;
            for (int j = 1; j < n; j++) {
                const real *vj = v + 3 * j;
                real dxc[3], dxbc[3];
                for (int k = 0; k < 3; k++) {
                    dxc[k] = x[3 * j + k] - x[k];
                    dxbc[k] = x[3 * j + k] - xi[k];
                }
                real r1c2 = dxc[0] * dxc[0] + dxc[1] * dxc[1] + dxc[2] * dxc[2];
                real r1ce = orc_rsqrt(r1c2 + eps2);
                real rbc2e = dxbc[0] * dxbc[0] + dxbc[1] * dxbc[1] + dxbc[2] * dxbc[2] + eps2;
                real rbce = orc_rsqrt(rbc2e);
                real vivj = dot3(vi, vj);
                real vidxb = dot3(vi, dxb);
                real vjdxb = dot3(vj, dxb);
                real radial = 4.0 * r1ce + 1.25 * rbce - 0.25 * r1c2 / rbc2e * rbce
                                + 0.25 * r1b2 / rbc2e * rbce;
                for (int k = 0; k < 3; k++)
                    s1c[k] += mr1b3e * m[j] * dxb[k] * radial
                              - 3.5 * (rbce * rbce * rbce) * r1be * m[i] * m[j] * dxbc[k]
                              - mr1b3e * m[j] / m[0]
                                    * (4.0 * vivj * dxb[k] - 3.0 * vidxb * vj[k] - 4.0 * vjdxb * vi[k]);
            }
            for (int k = 0; k < 3; k++) a1c_out[3 * r + k] = s1c[k];
        }
    }
    return 0;
}

#ifdef ORC_LONG_DOUBLE
/* double-array interface of the long-double build (ctypes passes double arrays) */
static long double *ld_copy(const double *src, size_t cnt) {
    long double *d = (long double *)malloc(sizeof(long double) * (cnt ? cnt : 1));
    for (size_t q = 0; q < cnt; q++) d[q] = src[q];
    return d;
}

void orcld_force_d(int n, const double *x, const double *v, const double *m, double eps,
                   double *a) {
    size_t c3 = (size_t)3 * (size_t)n;
    long double *X = ld_copy(x, c3), *V = ld_copy(v, c3), *M = ld_copy(m, (size_t)n);
    long double *A = (long double *)malloc(sizeof(long double) * (c3 ? c3 : 1));
    orcld_force(n, X, V, M, (long double)eps, A);
    for (size_t q = 0; q < c3; q++) a[q] = (double)A[q];
    free(X); free(V); free(M); free(A);
}

double orcld_energy_d(int n, const double *x, const double *v, const double *m, double eps,
                      double out[4]) {
    size_t c3 = (size_t)3 * (size_t)n;
    long double *X = ld_copy(x, c3), *V = ld_copy(v, c3), *M = ld_copy(m, (size_t)n);
    long double o[4];
    long double e = orcld_energy(n, X, V, M, (long double)eps, o);
    if (out)
        for (int q = 0; q < 4; q++) out[q] = (double)o[q];
    free(X); free(V); free(M);
    return (double)e;
}
#endif
