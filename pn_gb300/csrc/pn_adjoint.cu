// pn_adjoint.cu -- discrete adjoint of the force path and of the integration scheme.
//
// Force VJP.  For an adjoint abar (one 3-vector per particle) of the accelerations, the
// gradients xbar, vbar of abar . a(x, v, m) and dL/dm0 are computed in four launches:
//   k_prep            (forward, O(N)) pack and global sums of the evaluation state
//   k_finish_vjp      (O(N)) per star: the adjoint of the closed forms of the finishing kernel
//                     (generated from the same formulas, pn_finish_vjp_gen.cuh): adjoints of
//                     the star's pair sums (the "adjoint state" Gbar, Phibar, S0bar, Ubar, Wbar),
//                     of its own s, v, of the global sums and of m0
//   k_pair_vjp        (O(N^2)) one symmetric sweep: for star p against every star q, the pair
//                     term's derivative with p as the accumulating particle (adjoint state of p)
//                     and with p as the source particle (adjoint state of q streamed with q's
//                     data), i.e. the pairwise tidal-tensor contraction with the adjoint state
//                     plus the hand-differentiated 1PN pair terms
//   k_vjp_assemble    (O(N)) chain rule through R = (|s|^2+eps^2)^(-1/2), the per-particle
//                     pack constants and the global sums; xbar_0 = -sum_p sbar_p; dL/dm0
// The forward pair sums the VJP needs are those of the forward evaluation (stored by
// k_finish's sums_out), so the O(N^2) forward sweep is not repeated.
//
// Trajectory adjoint.  pn_adj_forward runs nsteps integration steps and keeps the state every
// K steps (checkpoints).  pn_adj_backward walks the segments backwards: each segment is
// recomputed from its checkpoint, storing its stage states and pair sums, and then its steps are
// reversed stage by stage (the adjoint of Limit-sticky9.c:853-891 is linear algebra on the
// stage adjoints, with one force VJP per stage).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "pn_ctx.h"
#include "pn_finish_vjp_gen.cuh"

using namespace pn;

namespace pn {

enum VjpSlot : int { V_SX = 0, V_SY, V_SZ, V_VX, V_VY, V_VZ, V_QE, V_MU3, V_C1, V_C3, V_K35, NV_VJP };
enum GbarSlot : int { GB_A1 = 0, GB_B3X, GB_B3Y, GB_B3Z, GB_C, GB_PX, GB_PY, GB_PZ, GB_M0, NGBAR };

// Threads per block of the O(N) adjoint kernels: their per-star FP64 work is heavy, so small
// blocks spread a system of a few thousand stars over every SM.
constexpr int VJP_ON_NT = 64;

// ------------------------------------------------------------------ per-star adjoint
struct FinVjpArgs {
    const double *spos, *v, *m, *sums, *glob;
    long long vsp, vsk;
    const double *abar;  // [p*asp + k*ask]
    long long asp, ask;
    int nstar, npad, nfill, f32;
    double eps, eps2, ic2;
    void *apack;         // adjoint state per star (FP64: 5 double2 groups; FP32: 3 float4)
    double *sdir, *vdir; // [3][npad]
    double *part, *gbar;
    unsigned *ticket;
};

__device__ __forceinline__ void block_sum_n(double *v, int nv, double *scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
    for (int q = 0; q < nv; ++q)
        for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
    if (lane == 0)
        for (int q = 0; q < nv; ++q) scratch[warp * nv + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0)
        for (int q = 0; q < nv; ++q) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += scratch[w * nv + q];
            v[q] = s;
        }
    __syncthreads();
}

__device__ __forceinline__ bool last_of(unsigned *ticket) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) am_last = atomicAdd(ticket, 1u) == gridDim.x - 1;
    __syncthreads();
    return am_last;
}

__global__ void __launch_bounds__(256) k_finish_vjp(const FinVjpArgs a) {
    __shared__ double red[32 * NGBAR];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double g[NGBAR];
    for (int q = 0; q < NGBAR; ++q) g[q] = 0.0;
    if (i < a.nfill) {
        double Gb[3] = {0, 0, 0}, Wb[3] = {0, 0, 0}, Phib = 0, S0b = 0, Ub = 0, v[3] = {0, 0, 0};
        if (i < a.nstar) {
            const int p = i + 1;
            const double s[3] = {a.spos[i], a.spos[a.npad + i], a.spos[2 * a.npad + i]};
            double ab[3], bb[3], G[3];
            for (int k = 0; k < 3; ++k) {
                v[k] = a.v[p * a.vsp + k * a.vsk];
                ab[k] = a.abar[p * a.asp + k * a.ask];
                bb[k] = a.abar[k * a.ask];
                G[k] = a.sums[(size_t)(A_GX + k) * a.npad + i];
            }
            const double Phi = a.sums[(size_t)A_PHI * a.npad + i];
            const double S0 = a.sums[(size_t)A_S0 * a.npad + i];
            const double U = a.sums[(size_t)A_U * a.npad + i];
            double sb[3], vb[3], gBb[3], gPb[3], m0b, gAb, gCb;
            finish_vjp_gen(s[0], s[1], s[2], v[0], v[1], v[2], G[0], G[1], G[2], a.glob[G_B3X],
                           a.glob[G_B3Y], a.glob[G_B3Z], a.glob[G_PX], a.glob[G_PY], a.glob[G_PZ],
                           ab[0], ab[1], ab[2], bb[0], bb[1], bb[2], Phi, S0, U, a.m[p], a.m[0],
                           a.eps, a.eps2, a.ic2, a.glob[G_A1], a.glob[G_C], sb, vb, Gb, Wb, gBb, gPb,
                           Phib, S0b, Ub, m0b, gAb, gCb);
            for (int k = 0; k < 3; ++k) {
                a.sdir[(size_t)k * a.npad + i] = sb[k];
                a.vdir[(size_t)k * a.npad + i] = vb[k];
            }
            g[GB_A1] = gAb;
            g[GB_C] = gCb;
            g[GB_M0] = m0b;
            for (int k = 0; k < 3; ++k) {
                g[GB_B3X + k] = gBb[k];
                g[GB_PX + k] = gPb[k];
            }
        }
        // |v|^2 and Wbar . v from the values the sweep itself reads (FP32 in mixed mode)
        if (a.f32) {
            const float vf[3] = {(float)v[0], (float)v[1], (float)v[2]};
            const float wf[3] = {(float)Wb[0], (float)Wb[1], (float)Wb[2]};
            const float vi2 = fmaf(vf[2], vf[2], fmaf(vf[1], vf[1], vf[0] * vf[0]));
            const float cw = fmaf(wf[2], vf[2], fmaf(wf[1], vf[1], wf[0] * vf[0]));
            float4 *ap = static_cast<float4 *>(a.apack);
            ap[i] = make_float4((float)Gb[0], (float)Gb[1], (float)Gb[2], (float)Phib);
            ap[a.npad + i] = make_float4(wf[0], wf[1], wf[2], (float)S0b);
            ap[2 * a.npad + i] = make_float4((float)Ub, vi2, cw, 0.f);
        } else {
            const double vi2 = fma(v[2], v[2], fma(v[1], v[1], v[0] * v[0]));
            const double cw = fma(Wb[2], v[2], fma(Wb[1], v[1], Wb[0] * v[0]));
            double2 *ap = static_cast<double2 *>(a.apack);
            ap[i] = make_double2(Gb[0], Gb[1]);
            ap[a.npad + i] = make_double2(Gb[2], Phib);
            ap[2 * a.npad + i] = make_double2(S0b, Ub);
            ap[3 * a.npad + i] = make_double2(Wb[0], Wb[1]);
            ap[4 * a.npad + i] = make_double2(Wb[2], vi2);
            ap[5 * a.npad + i] = make_double2(cw, 0.0);
        }
    }
    block_sum_n(g, NGBAR, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < NGBAR; ++q) a.part[(size_t)blockIdx.x * NGBAR + q] = g[q];
    if (last_of(a.ticket)) {
        double t[NGBAR];
        for (int q = 0; q < NGBAR; ++q) t[q] = 0.0;
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            for (int q = 0; q < NGBAR; ++q) t[q] += __ldcg(&a.part[(size_t)b * NGBAR + q]);
        block_sum_n(t, NGBAR, red);
        if (threadIdx.x == 0) {
            for (int q = 0; q < NGBAR; ++q) a.gbar[q] = t[q];
            // the BH's Newtonian acceleration is B3 itself (Limit-sticky9.c:36-51, row 0)
            for (int k = 0; k < 3; ++k) a.gbar[GB_B3X + k] += a.abar[k * a.ask];
            *a.ticket = 0u;
        }
    }
}

// ------------------------------------------------------------------ the O(N^2) adjoint sweep
struct PairVjpArgs {
    const void *pack;    // forward pack (prep), [NGF][npad]
    const void *apack;   // adjoint state, [NGA][npad]
    const TileOrigin *torg;
    const double *spos;
    double *out;         // [gsplit][NV_VJP][npad]
    int *err;
    int nstar, npad, tj, ntiles, gsplit;
    double eps2;
};

template <typename T> struct VjpState {
    T ex, ey, ez, lx, ly, lz;  // position (FP32: hi/lo relative to the tile origin)
    T vx, vy, vz, m, mu3, c3, k35, qe;
    T nvi2, c1v;               // -|v|^2 and c1 - 2 |v|^2 (the pair term's |v_i|^2 - 2 |dv|^2, split)
    T Gx, Gy, Gz, Phi, S0, U, Wx, Wy, Wz;  // adjoint state
    T cW;                                  // Wbar . v
};

// Sums of one row p of the factored sweep.  Both roles share the two vector sums; the terms of
// role 1 that carry a factor of row p only (Gbar_p, Wbar_p, v_p) are summed as scalars and
// multiplied in once per row (vjp_row_out).
enum VjpRowSum : int {
    Y_SX = 0, Y_SY, Y_SZ, Y_VX, Y_VY, Y_VZ,
    Y_A,    // sum mQ^3 wdv           (role 1: times -4 v_p into sbar)
    Y_B,    // sum cd                 (role 1: times -Wbar_p into sbar)
    Y_SG,   // sum mQ^3 wd            (role 1: times -2 v_p into vbar)
    Y_SCV,  // sum cv                 (role 1: times -Wbar_p into vbar)
    Y_QE,   // sum c3 mQ^3 wd         (role 1: qebar = -this)
    Y_S0,   // sum m_q Q^3            (role 1: times -Gbar_p into sbar)
    Y_SG2,  // sum m_p Q^3 wd'        (role 2: times -4 v_p into vbar; c1bar)
    Y_SB2,  // sum beta'              (role 2: times v_p into sbar)
    Y_MU3, Y_C3, Y_K35,
    NY
};

// One (p, q) pair, both roles, d = s_q - s_p.  Role 1: p accumulates the derivative of its own
// pair term (adjoint state of p); role 2: p is the source in q's pair term (adjoint state of q,
// streamed with q's data).  The algebra: with F = Gbar.(mQ^3 d) + Phibar mQ + S0bar mQ^3 +
// Ubar mu3 Q + Wbar.(cd d + cv dv) for one ordered pair (i, j),
//   dF/dd  = mQ^3 [Gbar + 2 c3 wd d + 3 Q^2 vdj wd v_j + wdv (4 v_i - 3 v_j)] + cd Wbar - LQ Q^3 d
//   dF/dv_i = mQ^3 wd (4 v_j - 2 v_i) + 4 mQ^3 wdv d - cv Wbar
//   dF/dv_j = mQ^3 wd (4 (v_i - v_j) - 3 Q^2 vdj d) ... + cv Wbar   (role 2, with d -> -d)
// LQ = 3 m Q^2 (gd + S0bar + br wd + k4 wdv) + Phibar m + Ubar mu3 + wd (3 mQ^3 vdj^2 Q + k35).
// The self pair (q = p, d = 0) contributes only Ubar_p / eps to mu3bar; it is skipped here
// (Q = 0) and that term is added per row, so no 1/eps^3 term has to cancel in the sums.
// The intermediates of the two pair terms of one unordered pair {p, q}: F(p, q) with p's adjoint
// state (role 1 of row p, role 2 of row q) and F(q, p) with q's adjoint state (role 2 of row p,
// role 1 of row q).  d = s_q - s_p.
template <typename T> struct VjpTerms {
    T Q, rp, rq;               // inverse distance (0 for the self pair); rhoe - qe_p, rhoe - qe_q
    T mQ3, ga, h, cd, cv, be;  // F(p, q): m_q Q^3, mQ^3 wd, mQ^3 wdv, cd, cv, beta
    T mQ3b, ga2, h2, cd2, cv2, be2;  // F(q, p), the same quantities
    T wd, wq;                  // Wbar_p . d, Wbar_q . d
    T cS, cSv, cV, cVd;        // coefficients of the shared vector sums
};

template <typename T>
__device__ __forceinline__ VjpTerms<T> vjp_terms(const VjpState<T> &P, const VjpState<T> &Qj, T dx, T dy, T dz,
                                                 T eps2, bool self) {
    VjpTerms<T> r;
    const T rhoe = pn_fma(dz, dz, pn_fma(dy, dy, pn_fma(dx, dx, eps2)));
    T Q = pn_rsqrt<T>(rhoe);
    if (self) Q = T(0);
    const T Q2 = Q * Q, Q3 = Q2 * Q;
    const T vdp = pn_fma(P.vz, dz, pn_fma(P.vy, dy, P.vx * dx));     // v_p . d
    const T vdq = pn_fma(Qj.vz, dz, pn_fma(Qj.vy, dy, Qj.vx * dx));  // v_q . d
    const T vpq = pn_fma(P.vz, Qj.vz, pn_fma(P.vy, Qj.vy, P.vx * Qj.vx));
    // |v_i|^2 - 2 |dv|^2 = -|v_i|^2 - 2 |v_j|^2 + 4 v_i.v_j: the -2 |v_j|^2 lives in c1v
    const T Q2x3 = T(3) * Q2;
    // ---- F(p, q): (i, j) = (p, q), adjoint state of p
    const T mQ3 = Qj.m * Q3;
    const T gd = pn_fma(P.Gz, dz, pn_fma(P.Gy, dy, P.Gx * dx));
    const T wd = pn_fma(P.Wz, dz, pn_fma(P.Wy, dy, P.Wx * dx));
    const T wdv = pn_fma(P.Wz, Qj.vz, pn_fma(P.Wy, Qj.vy, pn_fma(P.Wx, Qj.vx, -P.cW)));
    const T tQ2 = (vdq * vdq) * Q2;
    const T rp = rhoe - P.qe;
    T br = pn_fma(rp, Qj.c3, Qj.c1v) + pn_fma(T(4), vpq, P.nvi2);
    br = pn_fma(tQ2, T(1.5), br);
    const T k4 = pn_fma(T(4), vdp, T(-3) * vdq);
    const T cd = pn_fma(mQ3, br, Qj.k35 * Q);
    const T cv = mQ3 * k4;
    const T in = pn_fma(k4, wdv, pn_fma(br, wd, gd + P.S0));
    // LQ = 3 m Q^2 (in + wd t Q^2) + m Phibar + Ubar mu3 + wd k35   (3 mQ^3 t Q = 3 m Q^2 . t Q^2)
    const T LQ = pn_fma(Qj.m * Q2x3, pn_fma(wd, tQ2, in), pn_fma(Qj.m, P.Phi, pn_fma(wd, Qj.k35, P.U * Qj.mu3)));
    const T ga = mQ3 * wd;
    const T h = mQ3 * wdv;
    const T al = pn_fma(T(2) * Qj.c3, ga, -LQ * Q3);
    const T be = T(3) * pn_fma(Q2 * vdq, ga, -h);
    // ---- F(q, p): (i, j) = (q, p), adjoint state of q; d' = -d, dv' = v_p - v_q
    const T mQ3b = P.m * Q3;
    const T gq = pn_fma(Qj.Gz, dz, pn_fma(Qj.Gy, dy, Qj.Gx * dx));  // -gd'
    const T wq = pn_fma(Qj.Wz, dz, pn_fma(Qj.Wy, dy, Qj.Wx * dx));  // -wd'
    const T wdv2 = pn_fma(Qj.Wz, P.vz, pn_fma(Qj.Wy, P.vy, pn_fma(Qj.Wx, P.vx, -Qj.cW)));
    const T t2Q2 = (vdp * vdp) * Q2;
    const T rq = rhoe - Qj.qe;
    T br2 = pn_fma(rq, P.c3, P.c1v) + pn_fma(T(4), vpq, Qj.nvi2);
    br2 = pn_fma(t2Q2, T(1.5), br2);
    const T k42 = pn_fma(T(3), vdp, T(-4) * vdq);
    const T cd2 = pn_fma(mQ3b, br2, P.k35 * Q);
    const T cv2 = mQ3b * k42;
    const T in2 = pn_fma(k42, wdv2, pn_fma(-br2, wq, Qj.S0 - gq));
    const T LQ2 = pn_fma(P.m * Q2x3, pn_fma(-wq, t2Q2, in2),
                         pn_fma(P.m, Qj.Phi, pn_fma(-wq, P.k35, Qj.U * P.mu3)));
    const T ga2 = -mQ3b * wq;
    const T h2 = mQ3b * wdv2;
    const T al2 = pn_fma(T(2) * P.c3, ga2, -LQ2 * Q3);
    const T be2 = T(-3) * pn_fma(Q2 * vdp, ga2, h2);
    r.Q = Q; r.rp = rp; r.rq = rq;
    r.mQ3 = mQ3; r.ga = ga; r.h = h; r.cd = cd; r.cv = cv; r.be = be;
    r.mQ3b = mQ3b; r.ga2 = ga2; r.h2 = h2; r.cd2 = cd2; r.cv2 = cv2; r.be2 = be2;
    r.wd = wd; r.wq = wq;
    r.cS = -(al + al2);
    r.cSv = pn_fma(T(4), h2, -be);
    r.cV = T(4) * (ga + ga2);
    r.cVd = pn_fma(T(4), h, -be2);
    return r;
}

// Row p's sums from the pair terms: role 1 (F(p, q)) and role 2 (F(q, p)), shared vector sums.
template <typename T>
__device__ __forceinline__ void vjp_acc_p(T *y, const VjpTerms<T> &r, const VjpState<T> &Qj, T dx, T dy, T dz) {
    y[Y_A] += r.h;
    y[Y_B] += r.cd;
    y[Y_SG] += r.ga;
    y[Y_SCV] += r.cv;
    y[Y_QE] = pn_fma(Qj.c3, r.ga, y[Y_QE]);
    y[Y_S0] += r.mQ3;
    y[Y_SG2] += r.ga2;
    y[Y_SB2] += r.be2;
    y[Y_MU3] = pn_fma(Qj.U, r.Q, y[Y_MU3]);
    y[Y_C3] = pn_fma(r.ga2, r.rq, y[Y_C3]);
    y[Y_K35] = pn_fma(-r.Q, r.wq, y[Y_K35]);
    y[Y_SX] = pn_fma(r.cd2, Qj.Wx, pn_fma(r.mQ3b, Qj.Gx, pn_fma(r.cSv, Qj.vx, pn_fma(r.cS, dx, y[Y_SX]))));
    y[Y_SY] = pn_fma(r.cd2, Qj.Wy, pn_fma(r.mQ3b, Qj.Gy, pn_fma(r.cSv, Qj.vy, pn_fma(r.cS, dy, y[Y_SY]))));
    y[Y_SZ] = pn_fma(r.cd2, Qj.Wz, pn_fma(r.mQ3b, Qj.Gz, pn_fma(r.cSv, Qj.vz, pn_fma(r.cS, dz, y[Y_SZ]))));
    y[Y_VX] = pn_fma(r.cv2, Qj.Wx, pn_fma(r.cVd, dx, pn_fma(r.cV, Qj.vx, y[Y_VX])));
    y[Y_VY] = pn_fma(r.cv2, Qj.Wy, pn_fma(r.cVd, dy, pn_fma(r.cV, Qj.vy, y[Y_VY])));
    y[Y_VZ] = pn_fma(r.cv2, Qj.Wz, pn_fma(r.cVd, dz, pn_fma(r.cV, Qj.vz, y[Y_VZ])));
}

// Row q's sums from the same terms: the roles exchange (F(q, p) is q's role 1, F(p, q) its
// role 2) and d -> -d; the shared coefficients swap too (q's cSv is p's cVd and vice versa).
template <typename T>
__device__ __forceinline__ void vjp_acc_q(T *z, const VjpTerms<T> &r, const VjpState<T> &P, T dx, T dy, T dz) {
    z[Y_A] += r.h2;
    z[Y_B] += r.cd2;
    z[Y_SG] += r.ga2;
    z[Y_SCV] += r.cv2;
    z[Y_QE] = pn_fma(P.c3, r.ga2, z[Y_QE]);
    z[Y_S0] += r.mQ3b;
    z[Y_SG2] += r.ga;
    z[Y_SB2] += r.be;
    z[Y_MU3] = pn_fma(P.U, r.Q, z[Y_MU3]);
    z[Y_C3] = pn_fma(r.ga, r.rp, z[Y_C3]);
    z[Y_K35] = pn_fma(r.Q, r.wd, z[Y_K35]);
    z[Y_SX] = pn_fma(r.cd, P.Wx, pn_fma(r.mQ3, P.Gx, pn_fma(r.cVd, P.vx, pn_fma(-r.cS, dx, z[Y_SX]))));
    z[Y_SY] = pn_fma(r.cd, P.Wy, pn_fma(r.mQ3, P.Gy, pn_fma(r.cVd, P.vy, pn_fma(-r.cS, dy, z[Y_SY]))));
    z[Y_SZ] = pn_fma(r.cd, P.Wz, pn_fma(r.mQ3, P.Gz, pn_fma(r.cVd, P.vz, pn_fma(-r.cS, dz, z[Y_SZ]))));
    z[Y_VX] = pn_fma(r.cv, P.Wx, pn_fma(-r.cSv, dx, pn_fma(r.cV, P.vx, z[Y_VX])));
    z[Y_VY] = pn_fma(r.cv, P.Wy, pn_fma(-r.cSv, dy, pn_fma(r.cV, P.vy, z[Y_VY])));
    z[Y_VZ] = pn_fma(r.cv, P.Wz, pn_fma(-r.cSv, dz, pn_fma(r.cV, P.vz, z[Y_VZ])));
}

// One (p, q) pair, both roles, into row p's sums (the ordered sweep).  The algebra: with
// F = Gbar.(mQ^3 d) + Phibar mQ + S0bar mQ^3 + Ubar mu3 Q + Wbar.(cd d + cv dv) for one ordered
// pair (i, j),
//   dF/dd  = mQ^3 [Gbar + 2 c3 wd d + 3 Q^2 vdj wd v_j + wdv (4 v_i - 3 v_j)] + cd Wbar - LQ Q^3 d
//   dF/dv_i = mQ^3 wd (4 v_j - 2 v_i) + 4 mQ^3 wdv d - cv Wbar
//   dF/dv_j = mQ^3 wd (4 (v_i - v_j) - 3 Q^2 vdj d) ... + cv Wbar   (role 2, with d -> -d)
// LQ = 3 m Q^2 (gd + S0bar + br wd + k4 wdv) + Phibar m + Ubar mu3 + wd (3 mQ^3 vdj^2 Q + k35).
// The self pair (q = p, d = 0) contributes only Ubar_p / eps to mu3bar; it is skipped here
// (Q = 0) and that term is added per row, so no 1/eps^3 term has to cancel in the sums.
template <typename T>
__device__ __forceinline__ void vjp_pair(T *y, const VjpState<T> &P, const VjpState<T> &Qj, T dx, T dy,
                                         T dz, T eps2, bool self) {
    const VjpTerms<T> r = vjp_terms<T>(P, Qj, dx, dy, dz, eps2, self);
    vjp_acc_p<T>(y, r, Qj, dx, dy, dz);
}

// The row's outputs (NV_VJP slots) from its sums, in FP64.  qself = 1/eps for the split whose
// j-range holds p itself (the self pair's mu3 term), else 0.
template <typename T>
__device__ __forceinline__ void vjp_row_out(double *o, const double *Y, const VjpState<T> &P, double qself) {
    const double vp[3] = {(double)P.vx, (double)P.vy, (double)P.vz};
    const double Gp[3] = {(double)P.Gx, (double)P.Gy, (double)P.Gz};
    const double Wp[3] = {(double)P.Wx, (double)P.Wy, (double)P.Wz};
    for (int k = 0; k < 3; ++k) {
        o[V_SX + k] = Y[Y_SX + k] - Gp[k] * Y[Y_S0] - 4.0 * vp[k] * Y[Y_A] - Wp[k] * Y[Y_B] + vp[k] * Y[Y_SB2];
        o[V_VX + k] = Y[Y_VX + k] - 2.0 * vp[k] * Y[Y_SG] - Wp[k] * Y[Y_SCV] - 4.0 * vp[k] * Y[Y_SG2];
    }
    o[V_QE] = -Y[Y_QE];
    o[V_MU3] = Y[Y_MU3] + (double)P.U * qself;  // the self pair's Ubar_p mu3_p Q
    o[V_C1] = Y[Y_SG2];
    o[V_C3] = Y[Y_C3];
    o[V_K35] = Y[Y_K35];
}

template <typename T> struct VjpPack;
template <> struct VjpPack<float> { using V = float4; static constexpr int NGF = 4, NGA = 3; };
template <> struct VjpPack<double> { using V = double2; static constexpr int NGF = 6, NGA = 6; };

template <typename T>
__device__ __forceinline__ void vjp_load(VjpState<T> &S, const typename VjpPack<T>::V *f, const typename VjpPack<T>::V *ad,
                                         int stride, int j) {
    if constexpr (sizeof(T) == 4) {
        const float4 g0 = f[j], g1 = f[stride + j], g2 = f[2 * stride + j], g3 = f[3 * stride + j];
        S.ex = g0.x; S.ey = g0.y; S.ez = g0.z; S.m = g0.w;
        S.lx = g1.x; S.ly = g1.y; S.lz = g1.z; S.mu3 = g1.w;
        S.vx = g2.x; S.vy = g2.y; S.vz = g2.z; S.qe = g2.w;
        S.c3 = g3.y; S.k35 = g3.z;
        const float4 a0 = ad[j], a1 = ad[stride + j], a2 = ad[2 * stride + j];
        S.Gx = a0.x; S.Gy = a0.y; S.Gz = a0.z; S.Phi = a0.w;
        S.Wx = a1.x; S.Wy = a1.y; S.Wz = a1.z; S.S0 = a1.w;
        S.U = a2.x; S.cW = a2.z;
        S.nvi2 = -a2.y;
        S.c1v = fmaf(-2.f, a2.y, g3.x);
    } else {
        const double2 g0 = f[j], g1 = f[stride + j], g2 = f[2 * stride + j], g3 = f[3 * stride + j],
                      g4 = f[4 * stride + j], g5 = f[5 * stride + j];
        S.ex = g0.x; S.ey = g0.y; S.ez = g1.x; S.m = g1.y;
        S.lx = S.ly = S.lz = 0.0;
        S.vx = g2.x; S.vy = g2.y; S.vz = g3.x; S.mu3 = g3.y;
        S.c3 = g4.y; S.k35 = g5.x; S.qe = g5.y;
        const double2 a0 = ad[j], a1 = ad[stride + j], a2 = ad[2 * stride + j], a3 = ad[3 * stride + j],
                      a4 = ad[4 * stride + j], a5 = ad[5 * stride + j];
        S.Gx = a0.x; S.Gy = a0.y; S.Gz = a1.x; S.Phi = a1.y;
        S.S0 = a2.x; S.U = a2.y;
        S.Wx = a3.x; S.Wy = a3.y; S.Wz = a4.x;
        S.nvi2 = -a4.y;
        S.c1v = fma(-2.0, a4.y, g4.x);
        S.cW = a5.x;
    }
}

constexpr int VJP_NT = 128;

// One thread per star p, tiles of tj stars q staged by the TMA engine (double buffered), the
// j-range split over gridDim.y; FP32 sums are Kahan-folded per tile.
template <typename T>
__global__ void __launch_bounds__(VJP_NT) k_pair_vjp(const PairVjpArgs a) {
    using V = typename VjpPack<T>::V;
    constexpr int NGF = VjpPack<T>::NGF, NGA = VjpPack<T>::NGA, NG = NGF + NGA;
    constexpr bool F32 = sizeof(T) == 4;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    V *buf = reinterpret_cast<V *>(smem + 128);
    const int tid = threadIdx.x;
    const int i = blockIdx.x * VJP_NT + tid;
    const int split = blockIdx.y;
    const int t0 = (int)(((long long)a.ntiles * split) / a.gsplit);
    const int t1 = (int)(((long long)a.ntiles * (split + 1)) / a.gsplit);
    const int tj = a.tj;
    const V *pf = static_cast<const V *>(a.pack);
    const V *pa = static_cast<const V *>(a.apack);
    const bool valid = i < a.nstar;
    VjpState<T> P{};
    double sx = 0, sy = 0, sz = 0;
    if (valid) {
        vjp_load<T>(P, pf, pa, a.npad, i);
        sx = a.spos[i];
        sy = a.spos[a.npad + i];
        sz = a.spos[2 * a.npad + i];
        P.ex = (T)sx; P.ey = (T)sy; P.ez = (T)sz;
        P.lx = P.ly = P.lz = T(0);
    }
    T run[NY], cmp[NY];
    for (int q = 0; q < NY; ++q) run[q] = cmp[q] = T(0);
    if (tid == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    const uint32_t gbytes = (uint32_t)tj * (uint32_t)sizeof(V);
    auto issue = [&](int t, int stage) {
        mbar_arrive_expect_tx(&bars[stage], (uint32_t)NG * gbytes);
        for (int g = 0; g < NGF; ++g)
            bulk_g2s(buf + (size_t)(stage * NG + g) * tj, pf + (size_t)g * a.npad + (size_t)t * tj, gbytes, &bars[stage]);
        for (int g = 0; g < NGA; ++g)
            bulk_g2s(buf + (size_t)(stage * NG + NGF + g) * tj, pa + (size_t)g * a.npad + (size_t)t * tj, gbytes,
                     &bars[stage]);
    };
    if (tid == 0 && t0 < t1) issue(t0, 0);
    for (int t = t0; t < t1; ++t) {
        const int it = t - t0, stage = it & 1;
        const uint32_t phase = (uint32_t)(it >> 1) & 1u;
        const bool next = t + 1 < t1;
        if (tid == 0 && next) issue(t + 1, stage ^ 1);
        const bool ok = mbar_wait_bounded(&bars[stage], phase);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(a.err, DEVERR_TIMEOUT);
                mbar_wait_bounded(&bars[stage], phase);
                if (next) mbar_wait_bounded(&bars[stage ^ 1], (uint32_t)((it + 1) >> 1) & 1u);
            }
            return;
        }
        if constexpr (F32) {
            const TileOrigin o = a.torg[t];
            const double rx = sx - o.x, ry = sy - o.y, rz = sz - o.z;
            P.ex = (float)rx; P.ey = (float)ry; P.ez = (float)rz;
            P.lx = (float)(rx - (double)P.ex); P.ly = (float)(ry - (double)P.ey); P.lz = (float)(rz - (double)P.ez);
        }
        const V *bf = buf + (size_t)stage * NG * tj;
        const V *ba = bf + (size_t)NGF * tj;
        T tacc[NY];
        for (int q = 0; q < NY; ++q) tacc[q] = T(0);
        const int jself = i - t * tj;  // the tile index of p itself, if this tile holds it
        for (int j = 0; j < tj; ++j) {
            VjpState<T> Qj;
            vjp_load<T>(Qj, bf, ba, tj, j);
            T dx, dy, dz;
            if constexpr (F32) {
                dx = (Qj.ex - P.ex) + (Qj.lx - P.lx);
                dy = (Qj.ey - P.ey) + (Qj.ly - P.ly);
                dz = (Qj.ez - P.ez) + (Qj.lz - P.lz);
            } else {
                dx = Qj.ex - P.ex;
                dy = Qj.ey - P.ey;
                dz = Qj.ez - P.ez;
            }
            vjp_pair<T>(F32 ? tacc : run, P, Qj, dx, dy, dz, (T)a.eps2, j == jself);
        }
        if constexpr (F32)
            for (int q = 0; q < NY; ++q) kahan_add(run[q], cmp[q], tacc[q]);
        __syncthreads();
    }
    if (valid) {
        double Y[NY], o[NV_VJP];
        for (int q = 0; q < NY; ++q) Y[q] = F32 ? (double)run[q] - (double)cmp[q] : (double)run[q];
        // the self-pair term belongs to one split only
        const int tself = i / tj;
        const bool has_self = tself >= t0 && tself < t1;
        vjp_row_out<T>(o, Y, P, has_self ? 1.0 / sqrt(a.eps2) : 0.0);
        for (int q = 0; q < NV_VJP; ++q) a.out[((size_t)split * NV_VJP + q) * a.npad + i] = o[q];
    }
}

// ------------------------------------------------------------------ the symmetric adjoint sweep
// Each unordered pair {p, q} is visited once: the intermediates of its two pair terms serve both
// rows (vjp_acc_p, vjp_acc_q), about 94 operations per ordered pair instead of 154.
//
// Work item = a pair of 128-star tiles (I, J), I <= J (the pack's tiles), one CTA of four warps.
// Tile J is staged in shared memory; warp w holds the rows p of stars I*128 + 32w + lane in
// registers.  For each 32-star sub-tile k of J, lane l visits q = 32k + (l + s) mod 32 at step s,
// so the 32 lanes meet 32 different q, and the running sums of row q travel with q: after each
// step every lane passes its q-sums to lane l - 1 (one shuffle per sum).  After 32 steps lane l
// holds the warp's sums for q = 32k + l; the four warps' sums are added in a fixed order in
// shared memory.  The CTA writes row p's sums from tile J to part[J][.][p] and row q's sums from
// tile I to part[I][.][q]: every (tile, star) slot of part is written by exactly one CTA, and
// k_vjp_sym_rows adds a star's slots in tile order in FP64 (deterministic).  A diagonal item
// (I = J) visits every pair of its tile in both orders, so its sums are halved; the self pair is
// skipped (its mu3 term is added per row, as in the ordered sweep).
constexpr int SYM_T = 128;

// Rows per lane: FP32 lanes hold two rows p against the same q (the q data read from shared
// memory and the 17 shuffles of q's sums then serve two pairs), FP64 lanes one (register-bound).
template <typename T> __host__ __device__ constexpr int sym_rows() { return sizeof(T) == 4 ? 2 : 1; }
template <typename T> __host__ __device__ constexpr int sym_threads() { return SYM_T / sym_rows<T>(); }
template <typename T> __host__ __device__ constexpr int sym_min_blocks() { return sizeof(T) == 4 ? 6 : 2; }

template <typename T>
constexpr size_t sym_smem_bytes() {
    return (size_t)(VjpPack<T>::NGF + VjpPack<T>::NGA) * SYM_T * sizeof(typename VjpPack<T>::V) +
           (size_t)(sym_threads<T>() / 32) * NY * SYM_T * sizeof(T);
}

template <typename T>
__global__ void __launch_bounds__(sym_threads<T>(), (sym_min_blocks<T>()))
    k_pair_vjp_sym(const PairVjpArgs a, T *part) {
    using V = typename VjpPack<T>::V;
    constexpr int NGF = VjpPack<T>::NGF, NGA = VjpPack<T>::NGA;
    constexpr int R = sym_rows<T>(), NTH = sym_threads<T>(), NW = NTH / 32;
    constexpr bool F32 = sizeof(T) == 4;
    extern __shared__ __align__(128) unsigned char smem[];
    V *qd = reinterpret_cast<V *>(smem);                                          // [NGF + NGA][SYM_T]
    T *qp = reinterpret_cast<T *>(smem + (size_t)(NGF + NGA) * SYM_T * sizeof(V));  // [NW][NY][SYM_T]
    const int tid = threadIdx.x, lane = tid & 31, warp = tid >> 5;
    // work item u -> tile pair (I, J), I <= J, u = J (J + 1) / 2 + I
    const long long u = blockIdx.x;
    int J = (int)((sqrt(8.0 * (double)u + 1.0) - 1.0) * 0.5);
    while ((long long)J * (J + 1) / 2 > u) --J;
    while ((long long)(J + 1) * (J + 2) / 2 <= u) ++J;
    const int I = (int)(u - (long long)J * (J + 1) / 2);
    const bool diag = I == J;
    const V *pf = static_cast<const V *>(a.pack);
    const V *pa = static_cast<const V *>(a.apack);
    const int q0 = J * SYM_T;
    for (int e = tid; e < SYM_T; e += NTH) {
#pragma unroll
        for (int g = 0; g < NGF; ++g) qd[g * SYM_T + e] = pf[(size_t)g * a.npad + q0 + e];
#pragma unroll
        for (int g = 0; g < NGA; ++g) qd[(NGF + g) * SYM_T + e] = pa[(size_t)g * a.npad + q0 + e];
    }
    // lane's rows: local star 32 (R warp + r) + lane of tile I
    VjpState<T> P[R];
    T y[R][NY];
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int p = I * SYM_T + 32 * (R * warp + r) + lane;
        vjp_load<T>(P[r], pf, pa, a.npad, p);
        if constexpr (F32) {  // p relative to tile J's origin, as an FP32 hi/lo pair
            const TileOrigin o = a.torg[J];
            const double rx = a.spos[p] - o.x, ry = a.spos[a.npad + p] - o.y, rz = a.spos[2 * a.npad + p] - o.z;
            P[r].ex = (float)rx; P[r].ey = (float)ry; P[r].ez = (float)rz;
            P[r].lx = (float)(rx - (double)P[r].ex);
            P[r].ly = (float)(ry - (double)P[r].ey);
            P[r].lz = (float)(rz - (double)P[r].ez);
        }
#pragma unroll
        for (int c = 0; c < NY; ++c) y[r][c] = T(0);
    }
    __syncthreads();
    const T eps2 = (T)a.eps2;
    const V *qa = qd + NGF * SYM_T;
    const int from = (lane + 1) & 31;
    T z[NY];
    for (int k = 0; k < SYM_T / 32; ++k) {
#pragma unroll
        for (int c = 0; c < NY; ++c) z[c] = T(0);
#pragma unroll 1
        for (int st = 0; st < 32; ++st) {
            const int qi = k * 32 + ((lane + st) & 31);
            VjpState<T> Qj;
            vjp_load<T>(Qj, qd, qa, SYM_T, qi);
#pragma unroll
            for (int r = 0; r < R; ++r) {
                T dx, dy, dz;
                if constexpr (F32) {
                    dx = (Qj.ex - P[r].ex) + (Qj.lx - P[r].lx);
                    dy = (Qj.ey - P[r].ey) + (Qj.ly - P[r].ly);
                    dz = (Qj.ez - P[r].ez) + (Qj.lz - P[r].lz);
                } else {
                    dx = Qj.ex - P[r].ex;
                    dy = Qj.ey - P[r].ey;
                    dz = Qj.ez - P[r].ez;
                }
                const VjpTerms<T> t = vjp_terms<T>(P[r], Qj, dx, dy, dz, eps2, diag && k == R * warp + r && st == 0);
                vjp_acc_p<T>(y[r], t, Qj, dx, dy, dz);
                vjp_acc_q<T>(z, t, P[r], dx, dy, dz);
            }
#pragma unroll
            for (int c = 0; c < NY; ++c) z[c] = __shfl_sync(0xffffffffu, z[c], from);
        }
#pragma unroll
        for (int c = 0; c < NY; ++c) qp[(warp * NY + c) * SYM_T + k * 32 + lane] = z[c];
    }
    __syncthreads();
    // rows q of tile J: the warps' sums added in a fixed order; one thread per star q
    for (int e = tid; e < SYM_T; e += NTH) {
#pragma unroll
        for (int c = 0; c < NY; ++c) {
            T zq = qp[c * SYM_T + e];
#pragma unroll
            for (int w = 1; w < NW; ++w) zq += qp[(w * NY + c) * SYM_T + e];
            if (diag)
                qp[c * SYM_T + e] = zq;  // this thread alone reads and writes star e's slots
            else
                part[((size_t)I * NY + c) * a.npad + q0 + e] = zq;  // row q, its pairs with tile I
        }
    }
    if (diag) __syncthreads();  // uniform over the CTA
#pragma unroll
    for (int r = 0; r < R; ++r) {
        const int pl = 32 * (R * warp + r) + lane;
        const int p = I * SYM_T + pl;
#pragma unroll
        for (int c = 0; c < NY; ++c) {
            if (diag)  // every pair of the tile was visited in both orders: half of each
                part[((size_t)I * NY + c) * a.npad + p] = T(0.5) * (y[r][c] + qp[c * SYM_T + pl]);
            else
                part[((size_t)J * NY + c) * a.npad + p] = y[r][c];  // row p, its pairs with tile J
        }
    }
}

// Per (star, sum): the star's slots over every tile, added in tile order.  Each thread takes 16
// bytes of consecutive stars (4 in FP32, 2 in FP64) with one vector load per tile.  FP32 slots
// are added with Kahan compensation in FP32 (the ordered sweep's numerics): converting each to
// FP64 and adding there would put ~2 x tiles x N operations on GB300's 1/64-rate FP64 pipe, which
// measured 148 us per VJP at N = 16,384 against ~20 us for the compensated FP32 sum.
template <typename T> struct SymVec;
template <> struct SymVec<float> { using V = float4; static constexpr int W = 4; };
template <> struct SymVec<double> { using V = double2; static constexpr int W = 2; };

template <typename T>
__global__ void __launch_bounds__(256) k_vjp_sym_reduce(const T *part, double *Y, int nt, int nstar, int npad) {
    using V = typename SymVec<T>::V;
    constexpr int W = SymVec<T>::W;
    const int i = (blockIdx.x * blockDim.x + threadIdx.x) * W;  // first star of this thread
    const int c = blockIdx.y;
    if (i >= nstar) return;
    const V *src = reinterpret_cast<const V *>(part + (size_t)c * npad + i);
    const size_t stride = (size_t)NY * npad / W;  // one tile, in vectors
    double t[W];
    if constexpr (W == 4) {
        float sum[4] = {0.f, 0.f, 0.f, 0.f}, cmp[4] = {0.f, 0.f, 0.f, 0.f};
#pragma unroll 8
        for (int b = 0; b < nt; ++b) {
            const V x = src[(size_t)b * stride];
            kahan_add(sum[0], cmp[0], x.x);
            kahan_add(sum[1], cmp[1], x.y);
            kahan_add(sum[2], cmp[2], x.z);
            kahan_add(sum[3], cmp[3], x.w);
        }
#pragma unroll
        for (int e = 0; e < 4; ++e) t[e] = (double)sum[e] - (double)cmp[e];
    } else {
        t[0] = t[1] = 0.0;
#pragma unroll 8
        for (int b = 0; b < nt; ++b) {
            const V x = src[(size_t)b * stride];
            t[0] += (double)x.x;
            t[1] += (double)x.y;
        }
    }
#pragma unroll
    for (int e = 0; e < W; ++e)
        if (i + e < nstar) Y[(size_t)c * npad + i + e] = t[e];
}

// Per star: the row outputs (split 0 of out) from its summed slots.
template <typename T>
__global__ void __launch_bounds__(128) k_vjp_sym_rows(const PairVjpArgs a, const double *Ysum) {
    using V = typename VjpPack<T>::V;
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= a.nstar) return;
    double Y[NY];
    for (int c = 0; c < NY; ++c) Y[c] = Ysum[(size_t)c * a.npad + i];
    VjpState<T> P;
    vjp_load<T>(P, static_cast<const V *>(a.pack), static_cast<const V *>(a.apack), a.npad, i);
    double o[NV_VJP];
    vjp_row_out<T>(o, Y, P, 1.0 / sqrt(a.eps2));
    for (int c = 0; c < NV_VJP; ++c) a.out[(size_t)c * a.npad + i] = o[c];
}

// ------------------------------------------------------------------ assembly
struct AssembleArgs {
    const double *spos, *m, *vjp, *sdir, *vdir, *gbar;
    int nstar, npad, gsplit;
    double eps2;
    double *xbar, *vbar;  // outputs [p*osp + k*osk] (accumulated into when accumulate != 0)
    long long osp, osk;
    int accumulate;
    int m0_accumulate;
    double *part, *m0bar;  // m0bar[0] += dL/dm0 (when m0_accumulate) or = (otherwise)
    unsigned *ticket;
};

__global__ void __launch_bounds__(256) k_vjp_assemble(const AssembleArgs a) {
    __shared__ double red[32 * 4];
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    double r[4] = {0, 0, 0, 0};  // -sum sbar (3), m0 partial
    if (i < a.nstar) {
        const int p = i + 1;
        const double s[3] = {a.spos[i], a.spos[a.npad + i], a.spos[2 * a.npad + i]};
        double S[NV_VJP];
        for (int q = 0; q < NV_VJP; ++q) {
            double t = 0.0;
            for (int g = 0; g < a.gsplit; ++g) t += a.vjp[((size_t)g * NV_VJP + q) * a.npad + i];
            S[q] = t;
        }
        const double mp = a.m[p], m0 = a.m[0];
        const double q2 = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
        const double R = 1.0 / sqrt(q2 + a.eps2), R2 = R * R, R3 = R2 * R;
        const double *G = a.gbar;
        const double B3s = G[GB_B3X] * s[0] + G[GB_B3Y] * s[1] + G[GB_B3Z] * s[2];
        // R enters c1 = 1.25 m0 R, c3 = 0.25 m0 R^3, k35 = 3.5 m0 m R^3, mu3 = m R^3 (pack) and
        // A1 = sum m R, B3 = sum m R^3 s, C = sum m R^3 q (global sums)
        const double Rb = 1.25 * m0 * S[V_C1] + 0.75 * m0 * R2 * S[V_C3] + 10.5 * m0 * mp * R2 * S[V_K35] +
                          3.0 * mp * R2 * S[V_MU3] + mp * G[GB_A1] + 3.0 * mp * R2 * B3s +
                          3.0 * mp * R2 * q2 * G[GB_C];
        const double qb = S[V_QE] + G[GB_C] * mp * R3;
        double sb[3], vb[3];
        for (int k = 0; k < 3; ++k) {
            sb[k] = a.sdir[(size_t)k * a.npad + i] + S[V_SX + k] - Rb * R3 * s[k] + 2.0 * qb * s[k] +
                    G[GB_B3X + k] * mp * R3;
            vb[k] = a.vdir[(size_t)k * a.npad + i] + S[V_VX + k] + mp * G[GB_PX + k];
            double *xo = &a.xbar[p * a.osp + k * a.osk];
            double *vo = &a.vbar[p * a.osp + k * a.osk];
            *xo = a.accumulate ? *xo + sb[k] : sb[k];
            *vo = a.accumulate ? *vo + vb[k] : vb[k];
            r[k] = -sb[k];
        }
        r[3] = 1.25 * R * S[V_C1] + 0.25 * R3 * S[V_C3] + 3.5 * mp * R3 * S[V_K35];
    }
    block_sum_n(r, 4, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) a.part[(size_t)blockIdx.x * 4 + q] = r[q];
    if (last_of(a.ticket)) {
        double t[4] = {0, 0, 0, 0};
        for (int b = threadIdx.x; b < (int)gridDim.x; b += blockDim.x)
            for (int q = 0; q < 4; ++q) t[q] += __ldcg(&a.part[(size_t)b * 4 + q]);
        block_sum_n(t, 4, red);
        if (threadIdx.x == 0) {
            for (int k = 0; k < 3; ++k) {
                double *xo = &a.xbar[k * a.osk];
                double *vo = &a.vbar[k * a.osk];
                *xo = a.accumulate ? *xo + t[k] : t[k];  // x_0 enters through s_p = x_p - x_0
                if (!a.accumulate) *vo = 0.0;             // the force ignores the BH velocity
            }
            const double m0b = t[3] + a.gbar[GB_M0];
            a.m0bar[0] = a.m0_accumulate ? a.m0bar[0] + m0b : m0b;
            *a.ticket = 0u;
        }
    }
}

// ------------------------------------------------------------------ integrator adjoint (elementwise)
// Reverse of one step (Limit-sticky9.c:853-891): called with which = 0..4.
//   0: from (Xb, Vb): xb = Xb/6, vb = Vb/6; x3b = Xb/6, x1b = x2b = Xb/3; v3b = Vb/6, v1b = v2b = Vb/3;
//      then x3 = x + h v2, v3 = v + h a2: xb += x3b, v2b += h x3b, vb += v3b, ab = h v3b
//   1: after the VJP at (x2, v2): xb += x2b, v1b += h/2 x2b, vb += v2b, ab = h/2 v2b
//   2: after the VJP at (x1, v1): xb += x1b, vb += h/2 x1b + v1b, ab = h/2 v1b
// The VJP outputs (xF, vF) are added to (x2b, v2b), (x1b, v1b), (xb, vb) respectively.
struct StageAdjArgs {
    double *Xb, *Vb;   // in: step-output adjoints; out (which 3): step-input adjoints
    double *xb, *vb, *x1b, *v1b, *x2b, *v2b, *ab;
    const double *xF, *vF;
    double h;
    int n;
    long long ld;
    int which;
};

__global__ void k_stage_adj(const StageAdjArgs a) {
    const int p = blockIdx.x * blockDim.x + threadIdx.x;
    if (p >= a.n) return;
    for (int k = 0; k < 3; ++k) {
        const size_t o = (size_t)k * a.ld + p;
        const double h = a.h;
        if (a.which == 0) {
            const double X = a.Xb[o], Vv = a.Vb[o];
            const double x3b = X / 6.0, v3b = Vv / 6.0;
            a.xb[o] = X / 6.0 + x3b;
            a.x1b[o] = X / 3.0;
            a.x2b[o] = X / 3.0;
            a.v1b[o] = Vv / 3.0;
            a.v2b[o] = Vv / 3.0 + h * x3b;
            a.vb[o] = Vv / 6.0 + v3b;
            a.ab[o] = h * v3b;
        } else if (a.which == 1) {  // VJP at (x2, v2) done: add it, then reverse x2, v2
            const double x2b = a.x2b[o] + a.xF[o], v2b = a.v2b[o] + a.vF[o];
            a.xb[o] += x2b;
            a.v1b[o] += 0.5 * h * x2b;
            a.vb[o] += v2b;
            a.ab[o] = 0.5 * h * v2b;
        } else if (a.which == 2) {  // VJP at (x1, v1) done: add it, then reverse x1, v1
            const double x1b = a.x1b[o] + a.xF[o], v1b = a.v1b[o] + a.vF[o];
            a.xb[o] += x1b;
            a.vb[o] += 0.5 * h * x1b + v1b;
            a.ab[o] = 0.5 * h * v1b;
        } else {  // VJP at (x, v) done: the step-input adjoints
            a.Xb[o] = a.xb[o] + a.xF[o];
            a.Vb[o] = a.vb[o] + a.vF[o];
        }
    }
}

}  // namespace pn

// ------------------------------------------------------------------ host side
struct AdjointWork {
    int npad = 0;
    long long ld = 0;
    double *sums = nullptr;  // [9][npad]
    void *apack = nullptr;   // [6][npad] x 16 B
    double *sdir = nullptr, *vdir = nullptr, *vjp = nullptr, *gbar = nullptr, *part = nullptr;
    int vjp_splits = 0;
    int g_best = 1, g_nstar = -1, g_f32 = -1;  // split count of the ordered VJP sweep for this size
    void *sympart = nullptr;  // [tiles][NY][npad] partial sums of the symmetric sweep
    double *symsum = nullptr; // [NY][npad] their sums over the tiles
    size_t sym_bytes = 0;
    double *m0bar = nullptr;
    unsigned *tickets = nullptr;
    double *work = nullptr;  // [12][3][ld]: Xb Vb xb vb x1b v1b x2b v2b ab xF vF spare
    // trajectory
    int nsteps = 0, K = 0, nck = 0;
    double *ckpt = nullptr;        // [nck][6][ld]  (x, v at steps 0, K, 2K, ...)
    double *seg[2] = {};           // [K][3][6][ld] evaluation states of a segment's stages (2 buffers)
    double *segsums[2] = {};       // [K][3][9][npad]
    int holds[2] = {-1, -1};       // segment whose stages each buffer holds (-1: none)
    // the VJP's own copies of the evaluation buffers (pack, tile origins, BH-relative positions,
    // global sums), so that a segment's recomputation (which uses the context's) can run on the
    // second stream while the previous segment is reversed
    void *vpack = nullptr;
    TileOrigin *vtorg = nullptr;
    double *vspos = nullptr, *vpart = nullptr, *vglob = nullptr;
    cudaStream_t s2 = nullptr;     // recomputation stream (default priority)
    cudaStream_t s1 = nullptr;     // reversal stream (highest priority: the critical path)
    cudaEvent_t ev_rec[2] = {}, ev_done[2] = {}, ev_sync = nullptr;
    double time0 = 0.0;
};

namespace pn {

void free_adjoint(pn_ctx *c) {
    AdjointWork *w = c->adj;
    if (!w) return;
    if (w->s2) cudaStreamSynchronize(w->s2);
    if (w->s1) cudaStreamSynchronize(w->s1);
    void *b[] = {w->sums, w->apack, w->sdir, w->vdir, w->vjp, w->gbar, w->part, w->m0bar, w->tickets,
                 w->work, w->ckpt, w->seg[0], w->seg[1], w->segsums[0], w->segsums[1], w->sympart, w->symsum,
                 w->vpack, w->vtorg, w->vspos, w->vpart, w->vglob};
    for (void *p : b)
        if (p) cudaFree(p);
    for (int q = 0; q < 2; ++q) {
        if (w->ev_rec[q]) cudaEventDestroy(w->ev_rec[q]);
        if (w->ev_done[q]) cudaEventDestroy(w->ev_done[q]);
    }
    if (w->ev_sync) cudaEventDestroy(w->ev_sync);
    if (w->s2) cudaStreamDestroy(w->s2);
    if (w->s1) cudaStreamDestroy(w->s1);
    delete w;
    c->adj = nullptr;
}

}  // namespace pn

static int adj_ensure(pn_ctx *c) {
    if (c->adj) return PN_OK;
    AdjointWork *w = new AdjointWork();
    c->adj = w;
    w->npad = c->npad;
    w->ld = c->ld;
    const size_t np = (size_t)c->npad, ld = (size_t)c->ld;
    auto mal = [&](void **p, size_t bytes) {
        if (cudaMalloc(p, bytes) != cudaSuccess) {
            cudaGetLastError();
            return false;
        }
        return true;
    };
    const bool ok = mal((void **)&w->sums, 9 * np * 8) && mal(&w->apack, 6 * np * 16) &&
                    mal((void **)&w->sdir, 3 * np * 8) && mal((void **)&w->vdir, 3 * np * 8) &&
                    mal((void **)&w->gbar, 16 * 8) && mal((void **)&w->part, (np / VJP_ON_NT + 2) * 16 * 8) &&
                    mal((void **)&w->m0bar, 2 * 8) && mal((void **)&w->tickets, 4 * sizeof(unsigned)) &&
                    mal((void **)&w->work, 12 * 3 * ld * 8) && mal(&w->vpack, 6 * np * 16) &&
                    mal((void **)&w->vtorg, (np / 32 + 1) * sizeof(TileOrigin)) &&
                    mal((void **)&w->vspos, 3 * np * 8) && mal((void **)&w->vpart, (np / 256 + 2) * 8 * 2 * 8) &&
                    mal((void **)&w->vglob, 16 * 8);
    if (!ok) {
        free_adjoint(c);
        return set_err(PN_ERR_NOMEM, "adjoint buffers");
    }
    int prio_low = 0, prio_high = 0;
    bool ev_ok = cudaDeviceGetStreamPriorityRange(&prio_low, &prio_high) == cudaSuccess &&
                 cudaStreamCreateWithFlags(&w->s2, cudaStreamNonBlocking) == cudaSuccess &&
                 cudaStreamCreateWithPriority(&w->s1, cudaStreamNonBlocking, prio_high) == cudaSuccess &&
                 cudaEventCreateWithFlags(&w->ev_sync, cudaEventDisableTiming) == cudaSuccess;
    for (int q = 0; q < 2 && ev_ok; ++q)
        ev_ok = cudaEventCreateWithFlags(&w->ev_rec[q], cudaEventDisableTiming) == cudaSuccess &&
                cudaEventCreateWithFlags(&w->ev_done[q], cudaEventDisableTiming) == cudaSuccess;
    if (!ev_ok) {
        cudaGetLastError();
        free_adjoint(c);
        return set_err(PN_ERR_CUDA, "adjoint streams");
    }
    CU(cudaMemset(w->vpack, 0, 6 * np * 16));
    CU(cudaMemset(w->tickets, 0, 4 * sizeof(unsigned)));
    CU(cudaMemset(w->apack, 0, 6 * np * 16));
    CU(cudaMemset(w->work, 0, 12 * 3 * ld * 8));
    return PN_OK;
}

// Tile of the pack and of the ordered adjoint sweep.  The symmetric sweep's tiles are SYM_T
// stars: in mixed precision they must be the pack's tiles (the FP32 positions are relative to
// each tile's origin); the FP64 pack holds BH-relative positions and has no tile origins.
static int vjp_tj(const pn_ctx *c) { return is_f32(c) ? SYM_T : 64; }
// Largest per-tile partial-sum array of the symmetric sweep (larger systems take the ordered one).
constexpr size_t kSymPartMax = (size_t)6 << 30;

// VJP of one force evaluation at (x, v) (SoA, leading dim ld), whose pair sums are in `sums`
// ([9][npad]).  abar: SoA [3][ld].  Writes (accumulate=0) or adds (1) xbar, vbar (SoA) and
// m0bar.
static int vjp_eval(pn_ctx *c, const double *x, const double *v, const double *sums, const double *abar,
                    double *xbar, double *vbar, double *m0bar, int m0_accumulate, cudaStream_t s) {
    const int accumulate = 0;
    AdjointWork *w = c->adj;
    const int nstar = c->n - 1;
    const bool f32 = is_f32(c);
    const int tj = vjp_tj(c);
    const double eps2 = c->p.eps * c->p.eps;
    const long long ld = c->ld;
    // prep: pack (forward data), global sums of this state
    PrepArgs pa{};
    pa.x = x; pa.v = v; pa.m = c->st.m; pa.sp = 1; pa.sk = ld;
    pa.nstar = nstar; pa.npad = c->npad; pa.nfill = (int)round_up(nstar > 0 ? nstar : 1, 256);
    pa.tj = tj; pa.f32 = f32; pa.eps2 = eps2;
    pa.pack = w->vpack; pa.torg = w->vtorg; pa.spos = w->vspos;
    pa.part = w->vpart; pa.glob = w->vglob; pa.ticket = &w->tickets[2];
    CU(launch_prep(pa, s));
    // per-star adjoint
    FinVjpArgs fa{};
    fa.spos = w->vspos; fa.v = v; fa.m = c->st.m; fa.sums = sums; fa.glob = w->vglob;
    fa.vsp = 1; fa.vsk = ld; fa.abar = abar; fa.asp = 1; fa.ask = ld;
    fa.nstar = nstar; fa.npad = c->npad; fa.nfill = pa.nfill; fa.f32 = f32;
    fa.eps = c->p.eps; fa.eps2 = eps2; fa.ic2 = c->p.inv_c2;
    fa.apack = w->apack; fa.sdir = w->sdir; fa.vdir = w->vdir; fa.part = w->part; fa.gbar = w->gbar;
    fa.ticket = &w->tickets[0];
    const int nbf = (pa.nfill + VJP_ON_NT - 1) / VJP_ON_NT;
    k_finish_vjp<<<nbf, VJP_ON_NT, 0, s>>>(fa);
    CU(cudaGetLastError());
    // O(N^2) sweep: the symmetric form (each unordered pair once) unless its per-tile partial
    // sums would take more than kSymPartMax bytes, or PN_VJP_SWEEP=ordered asks for the ordered one
    const int ntiles = nstar > 0 ? (nstar + tj - 1) / tj : 0;
    const int nt_sym = nstar > 0 ? (nstar + SYM_T - 1) / SYM_T : 0;
    const size_t tsize = f32 ? sizeof(float) : sizeof(double);
    const size_t sym_bytes = (size_t)nt_sym * NY * c->npad * tsize;
    const char *sweep_env = getenv("PN_VJP_SWEEP");
    const bool ordered = sweep_env && !strcmp(sweep_env, "ordered");
    const bool sym = nstar > 0 && !ordered && sym_bytes <= kSymPartMax && (!f32 || tj == SYM_T);
    int g = 1;
    if (sym) {
        if (sym_bytes > w->sym_bytes) {
            if (w->sympart) cudaFree(w->sympart);
            w->sympart = nullptr;
            w->sym_bytes = 0;
            if (cudaMalloc(&w->sympart, sym_bytes) != cudaSuccess) {
                cudaGetLastError();
                return set_err(PN_ERR_NOMEM, "vjp tile partials: %zu bytes", sym_bytes);
            }
            w->sym_bytes = sym_bytes;
        }
        if (!w->symsum) {
            if (cudaMalloc(&w->symsum, (size_t)NY * c->npad * sizeof(double)) != cudaSuccess) {
                cudaGetLastError();
                return set_err(PN_ERR_NOMEM, "vjp row sums");
            }
        }
    } else {
        const int nib = (nstar + VJP_NT - 1) / VJP_NT;
        // j-range splits: the count whose CTAs fill the resident slots in the fewest tile-times,
        // waves x tiles per CTA (a wave of small systems leaves SMs idle otherwise)
        if (w->g_nstar != nstar || w->g_f32 != (int)f32) {
            int per = 0;
            const size_t smem = 128 + 2 * (size_t)(f32 ? VjpPack<float>::NGF + VjpPack<float>::NGA
                                                        : VjpPack<double>::NGF + VjpPack<double>::NGA) * tj * 16;
            CU(f32 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pair_vjp<float>, VJP_NT, smem)
                   : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, k_pair_vjp<double>, VJP_NT, smem));
            const long long slots = (long long)c->sms * (per > 0 ? per : 1);
            int best = 1;
            long long best_cost = -1;
            for (int gc = 1; gc <= 64 && gc <= (ntiles > 0 ? ntiles : 1); ++gc) {
                const long long waves = ((long long)nib * gc + slots - 1) / slots;
                const long long cost = waves * ((ntiles + gc - 1) / gc);
                if (best_cost < 0 || cost < best_cost) {
                    best_cost = cost;
                    best = gc;
                }
            }
            w->g_best = best;
            w->g_nstar = nstar;
            w->g_f32 = (int)f32;
        }
        g = w->g_best;
    }
    if (g > w->vjp_splits) {
        if (w->vjp) cudaFree(w->vjp);
        w->vjp = nullptr;
        if (cudaMalloc(&w->vjp, (size_t)g * NV_VJP * c->npad * sizeof(double)) != cudaSuccess) {
            cudaGetLastError();
            w->vjp_splits = 0;
            return set_err(PN_ERR_NOMEM, "vjp partials");
        }
        w->vjp_splits = g;
    }
    if (nstar > 0) {
        PairVjpArgs qa{};
        qa.pack = w->vpack; qa.apack = w->apack; qa.torg = w->vtorg; qa.spos = w->vspos; qa.out = w->vjp;
        qa.err = c->err; qa.nstar = nstar; qa.npad = c->npad; qa.tj = tj; qa.ntiles = ntiles; qa.gsplit = g;
        qa.eps2 = eps2;
        if (sym) {
            const unsigned items = (unsigned)((long long)nt_sym * (nt_sym + 1) / 2);
            const unsigned nbr = (unsigned)((nstar + 127) / 128);
            const unsigned nbsum = (unsigned)((nstar + 4 * 256 - 1) / (4 * 256));  // FP32: 4 stars per thread
            if (f32) {
                const size_t smem = sym_smem_bytes<float>();
                static size_t configured = 0;
                if (smem > 48 * 1024 && smem > configured) {
                    CU(cudaFuncSetAttribute(k_pair_vjp_sym<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    configured = smem;
                }
                k_pair_vjp_sym<float><<<items, sym_threads<float>(), smem, s>>>(qa, static_cast<float *>(w->sympart));
                CU(cudaGetLastError());
                k_vjp_sym_reduce<float><<<dim3(nbsum, NY), 256, 0, s>>>(static_cast<const float *>(w->sympart),
                                                                       w->symsum, nt_sym, nstar, c->npad);
                CU(cudaGetLastError());
                k_vjp_sym_rows<float><<<nbr, 128, 0, s>>>(qa, w->symsum);
            } else {
                const size_t smem = sym_smem_bytes<double>();
                static size_t configured = 0;
                if (smem > 48 * 1024 && smem > configured) {
                    CU(cudaFuncSetAttribute(k_pair_vjp_sym<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    configured = smem;
                }
                k_pair_vjp_sym<double><<<items, sym_threads<double>(), smem, s>>>(qa, static_cast<double *>(w->sympart));
                CU(cudaGetLastError());
                k_vjp_sym_reduce<double><<<dim3(2 * nbsum, NY), 256, 0, s>>>(static_cast<const double *>(w->sympart),
                                                                        w->symsum, nt_sym, nstar, c->npad);
                CU(cudaGetLastError());
                k_vjp_sym_rows<double><<<nbr, 128, 0, s>>>(qa, w->symsum);
            }
            CU(cudaGetLastError());
        } else {
            const int nib = (nstar + VJP_NT - 1) / VJP_NT;
            dim3 grid((unsigned)nib, (unsigned)g);
            if (f32) {
                const size_t smem = 128 + 2 * (size_t)(VjpPack<float>::NGF + VjpPack<float>::NGA) * tj * 16;
                static size_t configured = 0;
                if (smem > 48 * 1024 && smem > configured) {
                    CU(cudaFuncSetAttribute(k_pair_vjp<float>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    configured = smem;
                }
                k_pair_vjp<float><<<grid, VJP_NT, smem, s>>>(qa);
            } else {
                const size_t smem = 128 + 2 * (size_t)(VjpPack<double>::NGF + VjpPack<double>::NGA) * tj * 16;
                static size_t configured = 0;
                if (smem > 48 * 1024 && smem > configured) {
                    CU(cudaFuncSetAttribute(k_pair_vjp<double>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
                    configured = smem;
                }
                k_pair_vjp<double><<<grid, VJP_NT, smem, s>>>(qa);
            }
            CU(cudaGetLastError());
        }
    }
    AssembleArgs aa{};
    aa.spos = w->vspos; aa.m = c->st.m; aa.vjp = w->vjp; aa.sdir = w->sdir; aa.vdir = w->vdir; aa.gbar = w->gbar;
    aa.nstar = nstar; aa.npad = c->npad; aa.gsplit = nstar > 0 ? g : 0; aa.eps2 = eps2;
    aa.xbar = xbar; aa.vbar = vbar; aa.osp = 1; aa.osk = ld; aa.accumulate = accumulate;
    aa.m0_accumulate = m0_accumulate;
    aa.part = w->part; aa.m0bar = m0bar; aa.ticket = &w->tickets[1];
    const int nba = nstar > 0 ? (nstar + VJP_ON_NT - 1) / VJP_ON_NT : 1;
    k_vjp_assemble<<<nba, VJP_ON_NT, 0, s>>>(aa);
    CU(cudaGetLastError());
    return PN_OK;
}

static void to_soa(const double *aos, double *h, int n, size_t ld) {
    for (int p = 0; p < n; ++p)
        for (int k = 0; k < 3; ++k) h[k * ld + p] = aos[3 * p + k];
}
static void from_soa(const double *h, double *aos, int n, size_t ld) {
    for (int p = 0; p < n; ++p)
        for (int k = 0; k < 3; ++k) aos[3 * p + k] = h[k * ld + p];
}

extern "C" int pn_force_vjp(pn_ctx *c, const double *abar, double *xbar, double *vbar, double *m0bar) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_force_vjp: no state");
    if (!abar || !xbar || !vbar || !m0bar) return set_err(PN_ERR_INVALID, "pn_force_vjp");
    int rc = adj_ensure(c);
    if (rc) return rc;
    AdjointWork *w = c->adj;
    const size_t ld = (size_t)c->ld;
    cudaStream_t s = c->stream;
    // forward evaluation (its pair sums feed the VJP)
    rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, c->ld, nullptr, 3, 1, 0, s, false, -1, w->sums);
    if (rc) return rc;
    std::vector<double> h(3 * ld, 0.0);
    to_soa(abar, h.data(), c->n, ld);
    double *d_ab = w->work + 8 * 3 * ld, *d_xF = w->work + 9 * 3 * ld, *d_vF = w->work + 10 * 3 * ld;
    CU(cudaMemcpyAsync(d_ab, h.data(), 3 * ld * 8, cudaMemcpyHostToDevice, s));
    rc = vjp_eval(c, c->st.x, c->st.v, w->sums, d_ab, d_xF, d_vF, w->m0bar, 0, s);
    if (rc) return rc;
    std::vector<double> hx(3 * ld), hv(3 * ld);
    CU(cudaMemcpyAsync(hx.data(), d_xF, 3 * ld * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(hv.data(), d_vF, 3 * ld * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(m0bar, w->m0bar, 8, cudaMemcpyDeviceToHost, s));
    rc = check_device_err(c);
    if (rc) return rc;
    from_soa(hx.data(), xbar, c->n, ld);
    from_soa(hv.data(), vbar, c->n, ld);
    return PN_OK;
}

// `steps` integration steps from the context's current state on stream s, keeping every stage's
// evaluation state and pair sums in segment buffer `buf` (the same evaluations as pn_steps).
static int record_segment(pn_ctx *c, int steps, int buf, cudaStream_t s) {
    AdjointWork *w = c->adj;
    const size_t ld = (size_t)c->ld, np = (size_t)c->npad;
    const long long LD = c->ld;
    for (int t = 0; t < steps; ++t) {
        double *S0 = w->seg[buf] + ((size_t)t * 3 + 0) * 6 * ld;
        double *S1 = w->seg[buf] + ((size_t)t * 3 + 1) * 6 * ld;
        double *S2 = w->seg[buf] + ((size_t)t * 3 + 2) * 6 * ld;
        double *ss = w->segsums[buf] + (size_t)t * 3 * 9 * np;
        CU(cudaMemcpyAsync(S0, c->st.x, 6 * ld * 8, cudaMemcpyDeviceToDevice, s));
        int rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, LD, nullptr, 3, 1, 1, s, false, -1, ss);
        if (rc) return rc;
        CU(cudaMemcpyAsync(S1, c->st.xs, 3 * ld * 8, cudaMemcpyDeviceToDevice, s));
        CU(cudaMemcpyAsync(S1 + 3 * ld, c->st.vs, 3 * ld * 8, cudaMemcpyDeviceToDevice, s));
        rc = eval_force(c, c->st.xs, c->st.vs, c->st.m, 1, LD, nullptr, 3, 1, 2, s, false, -1, ss + 9 * np);
        if (rc) return rc;
        CU(cudaMemcpyAsync(S2, c->st.xs, 3 * ld * 8, cudaMemcpyDeviceToDevice, s));
        CU(cudaMemcpyAsync(S2 + 3 * ld, c->st.vs, 3 * ld * 8, cudaMemcpyDeviceToDevice, s));
        rc = eval_force(c, c->st.xs, c->st.vs, c->st.m, 1, LD, nullptr, 3, 1, 3, s, false, -1, ss + 18 * np);
        if (rc) return rc;
        c->time += c->p.dt;
    }
    return PN_OK;
}

extern "C" int pn_adj_forward(pn_ctx *c, int nsteps, int checkpoint_every) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_adj_forward: no state");
    if (nsteps < 1 || checkpoint_every < 1) return set_err(PN_ERR_INVALID, "pn_adj_forward");
    int rc = adj_ensure(c);
    if (rc) return rc;
    AdjointWork *w = c->adj;
    const size_t ld = (size_t)c->ld, np = (size_t)c->npad;
    const int K = checkpoint_every;
    const int nck = (nsteps + K - 1) / K;
    if (w->nsteps != nsteps || w->K != K) {
        CU(cudaStreamSynchronize(w->s2));
        void *old[] = {w->ckpt, w->seg[0], w->seg[1], w->segsums[0], w->segsums[1]};
        for (void *p : old)
            if (p) cudaFree(p);
        w->ckpt = w->seg[0] = w->seg[1] = w->segsums[0] = w->segsums[1] = nullptr;
        // a second segment buffer only when there is a segment to recompute while another is reversed
        const int nbuf = nck > 1 ? 2 : 1;
        bool ok = cudaMalloc(&w->ckpt, (size_t)nck * 6 * ld * 8) == cudaSuccess;
        for (int q = 0; q < nbuf && ok; ++q)
            ok = cudaMalloc(&w->seg[q], (size_t)K * 3 * 6 * ld * 8) == cudaSuccess &&
                 cudaMalloc(&w->segsums[q], (size_t)K * 3 * 9 * np * 8) == cudaSuccess;
        if (!ok) {
            cudaGetLastError();
            return set_err(PN_ERR_NOMEM, "checkpoints");
        }
        w->nsteps = nsteps;
        w->K = K;
        w->nck = nck;
    }
    w->time0 = c->time;
    w->holds[0] = w->holds[1] = -1;
    for (int k = 0; k < nck; ++k) {
        CU(cudaMemcpyAsync(w->ckpt + (size_t)k * 6 * ld, c->st.x, 6 * ld * 8, cudaMemcpyDeviceToDevice, c->stream));
        const int steps = (k + 1) * K <= nsteps ? K : nsteps - k * K;
        // the last segment keeps its stages now, so the backward pass need not recompute it
        rc = k == nck - 1 ? record_segment(c, steps, k & 1, c->stream) : pn_steps(c, steps);
        if (rc) return rc;
    }
    w->holds[(nck - 1) & 1] = nck - 1;
    return check_device_err(c);
}

extern "C" int pn_adj_backward(pn_ctx *c, const double *xbar_T, const double *vbar_T, double *xbar_0,
                               double *vbar_0, double *m0bar) {
    if (!c || !c->adj || !c->adj->ckpt) return set_err(PN_ERR_STATE, "pn_adj_backward: no forward run");
    if (!xbar_T || !vbar_T || !xbar_0 || !vbar_0 || !m0bar) return set_err(PN_ERR_INVALID, "pn_adj_backward");
    AdjointWork *w = c->adj;
    const size_t ld = (size_t)c->ld, np = (size_t)c->npad;
    const long long LD = c->ld;
    cudaStream_t s = c->stream;
    const double h = c->p.dt;
    double *Xb = w->work, *Vb = w->work + 3 * ld, *xb = w->work + 2 * 3 * ld, *vb = w->work + 3 * 3 * ld;
    double *x1b = w->work + 4 * 3 * ld, *v1b = w->work + 5 * 3 * ld, *x2b = w->work + 6 * 3 * ld;
    double *v2b = w->work + 7 * 3 * ld, *ab = w->work + 8 * 3 * ld, *xF = w->work + 9 * 3 * ld;
    double *vF = w->work + 10 * 3 * ld;
    std::vector<double> hb(6 * ld, 0.0);
    to_soa(xbar_T, hb.data(), c->n, ld);
    to_soa(vbar_T, hb.data() + 3 * ld, c->n, ld);
    CU(cudaMemcpyAsync(Xb, hb.data(), 6 * ld * 8, cudaMemcpyHostToDevice, s));  // Xb, Vb adjacent
    CU(cudaMemsetAsync(w->m0bar + 1, 0, 8, s));
    // the context's state arrays are the recompute workspace; the final state is restored last
    std::vector<double> final_state(6 * ld);
    CU(cudaMemcpyAsync(final_state.data(), c->st.x, 6 * ld * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaStreamSynchronize(s));
    const int nthreads = 256, nblk = (c->n + nthreads - 1) / nthreads;
    StageAdjArgs sa{};
    sa.Xb = Xb; sa.Vb = Vb; sa.xb = xb; sa.vb = vb; sa.x1b = x1b; sa.v1b = v1b; sa.x2b = x2b; sa.v2b = v2b;
    sa.ab = ab; sa.xF = xF; sa.vF = vF; sa.h = h; sa.n = c->n; sa.ld = LD;
    const double time_final = c->time;
    // Two streams: the context's (s) reverses segment k while w->s2 recomputes segment k - 1 from
    // its checkpoint into the other segment buffer (the recomputation uses the context's state and
    // evaluation buffers, the reversal the VJP's own), so the O(N) kernels of each fill the
    // other's gaps.  ev_rec[b]: buffer b holds its segment; ev_done[b]: its reversal is done.
    cudaStream_t s2 = w->s2;
    cudaStream_t s0 = s;  // the context's stream: host copies before and after
    s = w->s1;            // the reversal, at the highest stream priority
    auto segsteps = [&](int k) { return (k + 1) * w->K <= w->nsteps ? w->K : w->nsteps - k * w->K; };
    bool done_valid[2] = {false, false};
    auto recompute = [&](int k) -> int {
        const int b = k & 1;
        if (done_valid[b]) CU(cudaStreamWaitEvent(s2, w->ev_done[b], 0));
        CU(cudaMemcpyAsync(c->st.x, w->ckpt + (size_t)k * 6 * ld, 6 * ld * 8, cudaMemcpyDeviceToDevice, s2));
        int rc = record_segment(c, segsteps(k), b, s2);
        if (rc) return rc;
        CU(cudaEventRecord(w->ev_rec[b], s2));
        w->holds[b] = k;
        return PN_OK;
    };
    CU(cudaEventRecord(w->ev_sync, s0));  // everything queued so far (the forward pass, Xb) first
    CU(cudaStreamWaitEvent(s2, w->ev_sync, 0));
    CU(cudaStreamWaitEvent(s, w->ev_sync, 0));
    const int klast = w->nck - 1;
    if (w->holds[klast & 1] == klast) {
        CU(cudaEventRecord(w->ev_rec[klast & 1], s));  // recorded by the forward pass on s
    } else {
        int rc = recompute(klast);
        if (rc) return rc;
    }
    for (int k = klast; k >= 0; --k) {
        const int b = k & 1;
        if (k >= 1) {  // queue the next segment's recomputation first, so that it overlaps
            int rc = recompute(k - 1);
            if (rc) return rc;
        }
        CU(cudaStreamWaitEvent(s, w->ev_rec[b], 0));
        const int steps = segsteps(k);
        // reverse the segment's steps
        for (int t = steps - 1; t >= 0; --t) {
            const double *S0 = w->seg[b] + ((size_t)t * 3 + 0) * 6 * ld;
            const double *S1 = w->seg[b] + ((size_t)t * 3 + 1) * 6 * ld;
            const double *S2 = w->seg[b] + ((size_t)t * 3 + 2) * 6 * ld;
            const double *ss = w->segsums[b] + (size_t)t * 3 * 9 * np;
            // stage 3 evaluated a2 = F(x2, v2); stage 2 a1 = F(x1, v1); stage 1 a0 = F(x, v)
            sa.which = 0;
            k_stage_adj<<<nblk, nthreads, 0, s>>>(sa);
            int rc = vjp_eval(c, S2, S2 + 3 * ld, ss + 18 * np, ab, xF, vF, w->m0bar + 1, 1, s);
            if (rc) return rc;
            sa.which = 1;
            k_stage_adj<<<nblk, nthreads, 0, s>>>(sa);
            rc = vjp_eval(c, S1, S1 + 3 * ld, ss + 9 * np, ab, xF, vF, w->m0bar + 1, 1, s);
            if (rc) return rc;
            sa.which = 2;
            k_stage_adj<<<nblk, nthreads, 0, s>>>(sa);
            rc = vjp_eval(c, S0, S0 + 3 * ld, ss, ab, xF, vF, w->m0bar + 1, 1, s);
            if (rc) return rc;
            sa.which = 3;
            k_stage_adj<<<nblk, nthreads, 0, s>>>(sa);
            CU(cudaGetLastError());
        }
        CU(cudaEventRecord(w->ev_done[b], s));
        done_valid[b] = true;
    }
    CU(cudaEventRecord(w->ev_sync, s2));  // the context's state is restored after the last recompute
    CU(cudaStreamWaitEvent(s0, w->ev_sync, 0));
    CU(cudaEventRecord(w->ev_rec[0], s));  // and after the last reversal
    CU(cudaStreamWaitEvent(s0, w->ev_rec[0], 0));
    s = s0;
    CU(cudaMemcpyAsync(hb.data(), Xb, 6 * ld * 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(m0bar, w->m0bar + 1, 8, cudaMemcpyDeviceToHost, s));
    CU(cudaMemcpyAsync(c->st.x, final_state.data(), 6 * ld * 8, cudaMemcpyHostToDevice, s));
    c->time = time_final;
    int rc = check_device_err(c);
    if (rc) return rc;
    from_soa(hb.data(), xbar_0, c->n, ld);
    from_soa(hb.data() + 3 * ld, vbar_0, c->n, ld);
    return PN_OK;
}
