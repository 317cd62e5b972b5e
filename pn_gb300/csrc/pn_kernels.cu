// pn_kernels.cu -- the O(N) kernels of libpn's force path (FP64 throughout).
//
//   k_prep          per-star quantities, the j-particle pack, the global sums
//   k_finish        per-star accelerations (Limit-sticky9.c:36-51 BH column, :213-274,
//                   the closed-form parts of :276-422), the BH's acceleration (:36-51 BH row,
//                   :54-211), and optionally one stage of the integration step (:853-891)
//   k_energy_finish the energies (:445-556) from the energy pair sweep
//
// Reductions over particles are two-level and deterministic: each CTA writes its partial,
// and the last CTA to finish (atomic ticket) sums all partials in block order and resets
// the ticket, so results do not depend on scheduling.
#include <cstdio>

#include "pn_kernels.h"

namespace pn {

// ------------------------------------------------------------------ small helpers
__device__ __forceinline__ double ld_x(const double *p, long long sp, long long sk, int i, int k) {
    return p[(long long)i * sp + (long long)k * sk];
}

// Double-double accumulation (TwoSum, Knuth TAOCP vol. 2 4.2.2) for the compensated sums.
struct DD {
    double hi, lo;
};
__device__ __forceinline__ DD dd_add(DD a, DD b) {
    double s = a.hi + b.hi;
    double bb = s - a.hi;
    double e = (a.hi - (s - bb)) + (b.hi - bb);
    e += a.lo + b.lo;
    double t = s + e;
    return DD{t, e - (t - s)};
}

// Block-wide reduction of NV doubles (fixed order: warp butterfly, then warps in order).
// Result valid in thread 0.  'scratch' holds >= 32*NV doubles.
template <int NV>
__device__ __forceinline__ void block_sum(double (&v)[NV], double *scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) v[q] += __shfl_xor_sync(0xffffffffu, v[q], off);
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) scratch[warp * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            double s = 0.0;
            for (int w = 0; w < nw; ++w) s += scratch[w * NV + q];
            v[q] = s;
        }
    }
    __syncthreads();
}

template <int NV>
__device__ __forceinline__ void block_sum_dd(DD (&v)[NV], DD *scratch) {
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = blockDim.x >> 5;
#pragma unroll
    for (int q = 0; q < NV; ++q)
#pragma unroll
        for (int off = 16; off > 0; off >>= 1) {
            DD o{__shfl_xor_sync(0xffffffffu, v[q].hi, off), __shfl_xor_sync(0xffffffffu, v[q].lo, off)};
            v[q] = dd_add(v[q], o);
        }
    if (lane == 0)
#pragma unroll
        for (int q = 0; q < NV; ++q) scratch[warp * NV + q] = v[q];
    __syncthreads();
    if (threadIdx.x == 0) {
#pragma unroll
        for (int q = 0; q < NV; ++q) {
            DD s{0.0, 0.0};
            for (int w = 0; w < nw; ++w) s = dd_add(s, scratch[w * NV + q]);
            v[q] = s;
        }
    }
    __syncthreads();
}

// Last-CTA election after each CTA published its partial.
__device__ __forceinline__ bool last_block(unsigned *ticket, int nblk) {
    __shared__ bool am_last;
    __threadfence();
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned t = atomicAdd(ticket, 1u);
        am_last = (t == (unsigned)nblk - 1u);
    }
    __syncthreads();
    return am_last;
}

// ------------------------------------------------------------------ prep
// Per star j (particle p = j + 1): s = x_p - x_0, q = |s|^2, R = 1/sqrt(q + eps^2) (the
// reference's rsqrt, Limit-sticky9.c:15-19), and the pack entries; global sums
// A1 = sum m R, B3 = sum m R^3 s, C = sum m R^3 q, P = sum m v.
__device__ __forceinline__ void prep_body(const PrepArgs &a, int blk, int nblk) {
    __shared__ double red[32 * NGLOB];
    const int j = blk * blockDim.x + threadIdx.x;
    const double eps2 = a.eps2;
    const double x0 = ld_x(a.x, a.sp, a.sk, 0, 0), y0 = ld_x(a.x, a.sp, a.sk, 0, 1),
                 z0 = ld_x(a.x, a.sp, a.sk, 0, 2);
    const double m0 = a.m[0];
    double g[NGLOB];
#pragma unroll
    for (int q = 0; q < NGLOB; ++q) g[q] = 0.0;

    if (j < a.nfill) {
        const bool real = j < a.nstar;
        double s[3] = {0, 0, 0}, vv[3] = {0, 0, 0}, mj = 0, R = 0, q = 0;
        if (real) {
            const int p = j + 1;
            s[0] = ld_x(a.x, a.sp, a.sk, p, 0) - x0;
            s[1] = ld_x(a.x, a.sp, a.sk, p, 1) - y0;
            s[2] = ld_x(a.x, a.sp, a.sk, p, 2) - z0;
            vv[0] = ld_x(a.v, a.sp, a.sk, p, 0);
            vv[1] = ld_x(a.v, a.sp, a.sk, p, 1);
            vv[2] = ld_x(a.v, a.sp, a.sk, p, 2);
            mj = a.m[p];
            q = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
            R = 1.0 / sqrt(q + eps2);
        }
        const double R3 = R * R * R;
        const double mu3 = mj * R3;
        const double c1 = 1.25 * m0 * R, c3 = 0.25 * m0 * R3, k35 = 3.5 * m0 * mu3;
        const double qe = real ? q + eps2 : 0.0;
        a.spos[j] = s[0];
        a.spos[a.npad + j] = s[1];
        a.spos[2 * a.npad + j] = s[2];
        if (a.f32) {
            // position relative to the tile origin (the tile's first star) as an FP32 hi/lo pair
            double o[3] = {0, 0, 0};
            const int jt = (j / a.tj) * a.tj;
            if (real) {
                const int pt = jt + 1;
                o[0] = ld_x(a.x, a.sp, a.sk, pt, 0) - x0;
                o[1] = ld_x(a.x, a.sp, a.sk, pt, 1) - y0;
                o[2] = ld_x(a.x, a.sp, a.sk, pt, 2) - z0;
            }
            float hi[3], lo[3];
            for (int k = 0; k < 3; ++k) {
                const double r = real ? s[k] - o[k] : 0.0;
                hi[k] = (float)r;
                lo[k] = (float)(r - (double)hi[k]);
            }
            if (a.pack) {  // the scalar sweep's pack (not needed when only the packed sweep runs)
                float4 *pk = static_cast<float4 *>(a.pack);
                pk[j] = make_float4(hi[0], hi[1], hi[2], (float)mj);
                pk[a.npad + j] = make_float4(lo[0], lo[1], lo[2], (float)mu3);
                pk[2 * a.npad + j] = make_float4((float)vv[0], (float)vv[1], (float)vv[2], (float)qe);
                pk[3 * a.npad + j] = make_float4((float)c1, (float)c3, (float)k35, 0.f);
            }
            if (a.pack2) {  // paired layout: star j is lane (j & 1) of pair j / 2; scaled
                const int lane = j & 1;
                const size_t prow = (size_t)a.npad / 2;
                float *p2 = reinterpret_cast<float *>(a.pack2 + j / 2);
                const double K = X2_K, v2 = vv[0] * vv[0] + vv[1] * vv[1] + vv[2] * vv[2];
                const float vals[7][2] = {{hi[0], hi[1]},
                                          {hi[2], (float)(mj / (K * K * K))},
                                          {lo[0], lo[1]},
                                          {lo[2], (float)(mu3 / K)},
                                          {(float)(X2_SQRT3 * vv[0]), (float)(X2_SQRT3 * vv[1])},
                                          {(float)(X2_SQRT3 * vv[2]), (float)(c1 - 2.0 * v2)},
                                          {(float)c3, (float)(k35 / K)}};
                for (int g = 0; g < 7; ++g) {
                    p2[g * prow * 4 + lane] = vals[g][0];
                    p2[g * prow * 4 + 2 + lane] = vals[g][1];
                }
                a.ipack[j] = make_float4((float)vv[0], (float)vv[1], (float)vv[2], (float)qe);
            }
            if (j % a.tj == 0 && real) {
                TileOrigin o{s[0], s[1], s[2], 0.0};
                o.hx = (float)s[0]; o.lx = (float)(s[0] - (double)o.hx);
                o.hy = (float)s[1]; o.ly = (float)(s[1] - (double)o.hy);
                o.hz = (float)s[2]; o.lz = (float)(s[2] - (double)o.hz);
                o.pad0 = o.pad1 = 0.f;
                a.torg[j / a.tj] = o;
            }
        } else {
            double2 *pk = static_cast<double2 *>(a.pack);
            pk[j] = make_double2(s[0], s[1]);
            pk[a.npad + j] = make_double2(s[2], mj);
            pk[2 * a.npad + j] = make_double2(vv[0], vv[1]);
            pk[3 * a.npad + j] = make_double2(vv[2], mu3);
            pk[4 * a.npad + j] = make_double2(c1, c3);
            pk[5 * a.npad + j] = make_double2(k35, qe);
        }
        if (real) {
            g[G_A1] = mj * R;
            g[G_B3X] = mu3 * s[0];
            g[G_B3Y] = mu3 * s[1];
            g[G_B3Z] = mu3 * s[2];
            g[G_C] = mu3 * q;
            g[G_PX] = mj * vv[0];
            g[G_PY] = mj * vv[1];
            g[G_PZ] = mj * vv[2];
        }
    }
    block_sum<NGLOB>(g, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < NGLOB; ++q) a.part[(size_t)blk * NGLOB + q] = g[q];
    if (last_block(a.ticket, nblk)) {
        double t[NGLOB];
        for (int q = 0; q < NGLOB; ++q) t[q] = 0.0;
        for (int b = threadIdx.x; b < nblk; b += blockDim.x)
            for (int q = 0; q < NGLOB; ++q) t[q] += __ldcg(&a.part[(size_t)b * NGLOB + q]);
        block_sum<NGLOB>(t, red);
        if (threadIdx.x == 0) {
            for (int q = 0; q < NGLOB; ++q) a.glob[q] = t[q];
            *a.ticket = 0u;
        }
    }
}

// ------------------------------------------------------------------ finish
// Stage updates of the integration step (Limit-sticky9.c:853-891) without FMA contraction,
// so the state arithmetic is rounded exactly as the reference's.
__device__ __forceinline__ void stage_update(const FinishArgs &a, int p, const double acc3[3]) {
    const double dt = a.dt;
    for (int k = 0; k < 3; ++k) {
        const size_t o = (size_t)k * a.ld + p;
        const double x = a.st.x[o], v = a.st.v[o];
        if (a.stage >= STAGE_RK4_1) {
            // classic fourth-order Runge-Kutta (optional integrator; hx, hv accumulate
            // k1 + 2 k2 + 2 k3 of the position and velocity slopes)
            if (a.stage == STAGE_RK4_1) {
                a.st.xs[o] = x + 0.5 * dt * v;
                a.st.vs[o] = v + 0.5 * dt * acc3[k];
                a.st.hx[o] = v;
                a.st.hv[o] = acc3[k];
            } else if (a.stage == STAGE_RK4_4) {
                const double vprev = a.st.vs[o];
                a.st.x[o] = x + (dt / 6.0) * (a.st.hx[o] + vprev);
                a.st.v[o] = v + (dt / 6.0) * (a.st.hv[o] + acc3[k]);
            } else {
                const double vprev = a.st.vs[o];
                const double f = a.stage == STAGE_RK4_2 ? 0.5 * dt : dt;
                a.st.xs[o] = x + f * vprev;
                a.st.vs[o] = v + f * acc3[k];
                a.st.hx[o] += 2.0 * vprev;
                a.st.hv[o] += 2.0 * acc3[k];
            }
        } else if (a.stage == 1) {  // :853-860
            const double x1 = __dadd_rn(x, __dmul_rn(__dmul_rn(0.5, v), dt));
            const double v1 = __dadd_rn(v, __dmul_rn(__dmul_rn(0.5, acc3[k]), dt));
            a.st.xs[o] = x1;
            a.st.vs[o] = v1;
            a.st.hx[o] = x1;
            a.st.hv[o] = v1;
        } else if (a.stage == 2) {  // :864-871
            const double vprev = a.st.vs[o];
            const double x1 = __dadd_rn(x, __dmul_rn(__dmul_rn(0.5, vprev), dt));
            const double v1 = __dadd_rn(v, __dmul_rn(__dmul_rn(0.5, acc3[k]), dt));
            a.st.xs[o] = x1;
            a.st.vs[o] = v1;
            a.st.hx[o] = __dadd_rn(a.st.hx[o], x1);
            a.st.hv[o] = __dadd_rn(a.st.hv[o], v1);
        } else {  // :875-891
            const double vprev = a.st.vs[o];
            const double x3 = __dadd_rn(x, __dmul_rn(vprev, dt));
            const double v3 = __dadd_rn(v, __dmul_rn(acc3[k], dt));
            a.st.x[o] = __ddiv_rn(__dadd_rn(__dadd_rn(x, x3), __dmul_rn(2.0, a.st.hx[o])), 6.0);
            a.st.v[o] = __ddiv_rn(__dadd_rn(__dadd_rn(v, v3), __dmul_rn(2.0, a.st.hv[o])), 6.0);
        }
    }
}

__device__ __forceinline__ void finish_body(const FinishArgs &a, int blk, int nblk) {
    __shared__ double red[32 * 3];
    const int i = blk * blockDim.x + threadIdx.x;
    const double m0 = a.m[0];
    const double eps = a.eps, eps2 = a.eps2, ic2 = a.inv_c2;
    const double *G = a.glob;
    double bh[3] = {0.0, 0.0, 0.0};
    bool bad = false;

    if (i < a.nstar) {
        const int p = i + 1;
        const double s[3] = {a.spos[i], a.spos[a.npad + i], a.spos[2 * a.npad + i]};
        const double q = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
        const double R = 1.0 / sqrt(q + eps2);
        const double R3 = R * R * R;
        const double mi = a.m[p];
        // the force slots only (a fused-energy sweep has one more, read by the energy kernel)
        const int nk = a.nacc < NACC_MAX ? a.nacc : NACC_MAX;
        double S[NACC_MAX];
        for (int k = 0; k < nk; ++k) {
            double t = 0.0;
            for (int g = 0; g < a.gsplit; ++g) t += a.acc[((size_t)g * a.nacc + k) * a.npad + i];
            S[k] = t;
        }
        if (a.sums_out)
            for (int k = 0; k < nk; ++k) a.sums_out[(size_t)k * a.npad + i] = S[k];
        const double Gv[3] = {S[A_GX], S[A_GY], S[A_GZ]};
        double acc3[3];
        for (int k = 0; k < 3; ++k) acc3[k] = Gv[k] - m0 * R3 * s[k];  // Newton incl. BH column
        if (a.pn1) {
            const double v[3] = {ld_x(a.v, a.vsp, a.vsk, p, 0), ld_x(a.v, a.vsp, a.vsk, p, 1),
                                 ld_x(a.v, a.vsp, a.vsk, p, 2)};
            const double P[3] = {G[G_PX], G[G_PY], G[G_PZ]};
            const double B3[3] = {G[G_B3X], G[G_B3Y], G[G_B3Z]};
            const double A1 = G[G_A1], C = G[G_C];
            const double Phi = S[A_PHI], S0 = S[A_S0], U = S[A_U];
            const double W[3] = {S[A_WX], S[A_WY], S[A_WZ]};
            const double vi2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
            const double vis = v[0] * s[0] + v[1] * s[1] + v[2] * s[2];
            const double viP = v[0] * P[0] + v[1] * P[1] + v[2] * P[2];
            const double Ps = P[0] * s[0] + P[1] * s[1] + P[2] * s[2];
            const double sB3 = s[0] * B3[0] + s[1] * B3[1] + s[2] * B3[2];
            const double sG = s[0] * Gv[0] + s[1] * Gv[1] + s[2] * Gv[2];
            // star i: :215-238 (a_BH), :249-274 (ac direct), :276-382 summed over j (t1..t4, W),
            // minus the self-pair removal :392-422
            const double cs = -m0 * R3 * (4.0 * m0 * R - vi2)        // a_BH, s part
                              + 5.0 * m0 * R3 * mi * R - 4.0 * mi * R3 * vi2   // ac direct
                              - m0 * R3 * (4.0 * Phi + 1.25 * A1 - 0.25 * C + 0.5 * sB3)  // t1
                              + 3.5 * m0 * U                             // t3 (s U part)
                              + 4.0 * R3 * viP                           // t4
                              + mi * R3 * m0 * (4.0 / eps + 1.25 * R + 0.25 * q * R3)    // -rem
                              - 3.5 * mi * R3 * m0 * (1.0 / eps - R) - 4.0 * mi * R3 * vi2;
            const double cv = -4.0 * m0 * R3 * vis + 7.0 * mi * R3 * vis - 3.0 * R3 * Ps
                              + 7.0 * mi * R3 * vis;
            const double cg = 4.0 * m0 * R;                              // t2
            for (int k = 0; k < 3; ++k) {
                const double pn = cs * s[k] + cv * v[k] + cg * Gv[k] - 3.5 * m0 * R * B3[k]
                                  - 4.0 * R3 * vis * P[k] + W[k];
                acc3[k] += ic2 * pn;
            }
            // this star's share of the BH's 1PN acceleration: :58-95 (a1), :101-115 (single),
            // :118-174 summed over j, minus :179-207 (removal, with its 1.25*eps)
            const double T = -2.0 * sG - (Phi - eps2 * S0);
            const double mR3 = mi * R3;
            const double bs = mR3 * (5.0 * m0 * R - 2.0 * vi2 + 1.5 * vis * vis / q)  // a1
                              + 4.0 * mR3 * R * mi                                  // single
                              + mR3 * (4.0 * A1 + 1.25 * Phi + 0.25 * T)           // pair
                              - (mR3 / m0) * 4.0 * viP
                              + mR3 * mi * (4.0 * R + 1.25 * eps)                   // -removal
                              - (mR3 * mi / m0) * 4.0 * vi2;
            const double bv = 3.0 * mR3 * vis + (mR3 / m0) * 4.0 * Ps + (mR3 * mi / m0) * 7.0 * vis;
            for (int k = 0; k < 3; ++k)
                bh[k] = bs * s[k] + bv * v[k] - 3.5 * R * mi * Gv[k] + (mR3 / m0) * 3.0 * vis * P[k];
        }
        for (int k = 0; k < 3; ++k) {
            if (!isfinite(acc3[k])) bad = true;
            if (a.a) a.a[(long long)p * a.asp + (long long)k * a.ask] = acc3[k];
        }
        if (a.stage) stage_update(a, p, acc3);
    }
    if (bad) atomicOr(a.err, DEVERR_NONFINITE);
    block_sum<3>(bh, red);
    if (threadIdx.x == 0)
        for (int k = 0; k < 3; ++k) a.part[(size_t)blk * 3 + k] = bh[k];
    if (last_block(a.ticket, nblk)) {
        double t[3] = {0.0, 0.0, 0.0};
        for (int b = threadIdx.x; b < nblk; b += blockDim.x)
            for (int k = 0; k < 3; ++k) t[k] += __ldcg(&a.part[(size_t)b * 3 + k]);
        block_sum<3>(t, red);
        if (threadIdx.x == 0) {
            double acc3[3];
            bool b0 = false;
            for (int k = 0; k < 3; ++k) {
                // BH: Newtonian pull of the stars (:36-51, row 0) plus the 1PN sum
                acc3[k] = G[G_B3X + k] + (a.pn1 ? ic2 * t[k] : 0.0);
                if (!isfinite(acc3[k])) b0 = true;
                if (a.a) a.a[(long long)k * a.ask] = acc3[k];
            }
            if (b0) atomicOr(a.err, DEVERR_NONFINITE);
            if (a.stage) stage_update(a, 0, acc3);
            *a.ticket = 0u;
        }
    }
}

// ------------------------------------------------------------------ energy
// Per star (Limit-sticky9.c:452-556): kinetic, Newtonian potential row, O(N) 1PN term and the
// pairwise 1PN energy with its self-pair removal; compensated (double-double) sums.
__device__ __forceinline__ void energy_body(const EnergyArgs &a, int blk, int nblk) {
    __shared__ DD red[32 * 4];
    const int i = blk * blockDim.x + threadIdx.x;
    const double m0 = a.m[0], eps = a.eps, eps2 = a.eps2;
    const double v0[3] = {ld_x(a.v, a.sp, a.sk, 0, 0), ld_x(a.v, a.sp, a.sk, 0, 1),
                          ld_x(a.v, a.sp, a.sk, 0, 2)};
    const double A1 = a.glob[G_A1];
    DD e[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};  // kin, pot, pot_pn, pn2
    if (i < a.nstar) {
        const int p = i + 1;
        const double s[3] = {a.spos[i], a.spos[a.npad + i], a.spos[2 * a.npad + i]};
        const double v[3] = {ld_x(a.v, a.sp, a.sk, p, 0), ld_x(a.v, a.sp, a.sk, p, 1),
                             ld_x(a.v, a.sp, a.sk, p, 2)};
        const double mi = a.m[p];
        double Phi = 0.0, Psi = 0.0;
        for (int g = 0; g < a.gsplit; ++g) {
            Phi += a.acc[((size_t)g * a.nacc + a.sphi) * a.npad + i];
            Psi += a.acc[((size_t)g * a.nacc + a.spsi) * a.npad + i];
        }
        const double q = s[0] * s[0] + s[1] * s[1] + s[2] * s[2];
        const double R = 1.0 / sqrt(q + eps2);
        const double vi2 = v[0] * v[0] + v[1] * v[1] + v[2] * v[2];
        const double v0vi = v0[0] * v[0] + v0[1] * v[1] + v0[2] * v[2];
        const double sv0 = s[0] * v0[0] + s[1] * v0[1] + s[2] * v0[2];
        const double svi = s[0] * v[0] + s[1] * v[1] + s[2] * v[2];
        const double mR = m0 * R;
        e[0].hi = mi * vi2;
        e[1].hi = (-(mR + Phi) + mi / sqrt(eps2)) * mi;
        e[2].hi = 0.375 * mi * vi2 * vi2 + 1.5 * mR * mi * vi2 + 0.5 * mR * mR * mi
                  + 0.5 * mR * mi * (3.0 * vi2 - 7.0 * v0vi - sv0 * svi * R * R);
        e[3].hi = 0.25 * mi * (6.0 * vi2 * Phi - Psi) + m0 * mi * R * Phi + 0.5 * m0 * mi * R * A1
                  - (0.25 * mi * mi / eps * (-vi2) + m0 * mi * mi * (R / eps + 0.5 * R * R));
    }
    block_sum_dd<4>(e, red);
    if (threadIdx.x == 0)
        for (int q = 0; q < 4; ++q) {
            a.part[((size_t)blk * 4 + q) * 2] = e[q].hi;
            a.part[((size_t)blk * 4 + q) * 2 + 1] = e[q].lo;
        }
    if (last_block(a.ticket, nblk)) {
        DD t[4] = {{0, 0}, {0, 0}, {0, 0}, {0, 0}};
        for (int b = threadIdx.x; b < nblk; b += blockDim.x)
            for (int q = 0; q < 4; ++q)
                t[q] = dd_add(t[q], DD{__ldcg(&a.part[((size_t)b * 4 + q) * 2]),
                                       __ldcg(&a.part[((size_t)b * 4 + q) * 2 + 1])});
        block_sum_dd<4>(t, red);
        if (threadIdx.x == 0) {
            const double kin0 = m0 * (v0[0] * v0[0] + v0[1] * v0[1] + v0[2] * v0[2]);
            const double kin = 0.5 * ((t[0].hi + t[0].lo) + kin0);
            const double pot = 0.5 * ((t[1].hi + t[1].lo) - m0 * A1);
            const double potpn = a.inv_c2 * (t[2].hi + t[2].lo);
            const double pn2 = a.inv_c2 * (t[3].hi + t[3].lo);
            a.out[0] = pot;
            a.out[1] = kin;
            a.out[2] = potpn;
            a.out[3] = kin + pot + potpn + pn2;
            *a.ticket = 0u;
        }
    }
}

// ------------------------------------------------------------------ kernels
// One system: the block index is the block within the system.
__global__ void __launch_bounds__(256) k_prep(const PrepArgs a) { prep_body(a, blockIdx.x, gridDim.x); }
__global__ void __launch_bounds__(256) k_finish(const FinishArgs a) { finish_body(a, blockIdx.x, gridDim.x); }
__global__ void __launch_bounds__(256) k_energy_finish(const EnergyArgs a) {
    energy_body(a, blockIdx.x, gridDim.x);
}

// An ensemble in one launch: blockmap[b] = (cluster, block within the cluster, blocks of the
// cluster); each cluster's arguments come from a device table.
__global__ void __launch_bounds__(256) k_prep_ens(const PrepArgs *tab, const int4 *blockmap) {
    const int4 bm = blockmap[blockIdx.x];
    const PrepArgs a = tab[bm.x];
    prep_body(a, bm.y, bm.z);
}
__global__ void __launch_bounds__(256) k_finish_ens(const FinishArgs *tab, const int4 *blockmap) {
    const int4 bm = blockmap[blockIdx.x];
    const FinishArgs a = tab[bm.x];
    finish_body(a, bm.y, bm.z);
}
__global__ void __launch_bounds__(256) k_energy_ens(const EnergyArgs *tab, const int4 *blockmap) {
    const int4 bm = blockmap[blockIdx.x];
    const EnergyArgs a = tab[bm.x];
    energy_body(a, bm.y, bm.z);
}

// ------------------------------------------------------------------ launchers
cudaError_t launch_prep_ens(const PrepArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s) {
    k_prep_ens<<<nblocks, 256, 0, s>>>(tab, blockmap);
    return cudaGetLastError();
}
cudaError_t launch_finish_ens(const FinishArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s) {
    k_finish_ens<<<nblocks, 256, 0, s>>>(tab, blockmap);
    return cudaGetLastError();
}
cudaError_t launch_energy_ens(const EnergyArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s) {
    k_energy_ens<<<nblocks, 256, 0, s>>>(tab, blockmap);
    return cudaGetLastError();
}

cudaError_t launch_prep(const PrepArgs &a, cudaStream_t s) {
    const int nb = (a.nfill + 255) / 256;
    k_prep<<<nb, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_finish(const FinishArgs &a, cudaStream_t s) {
    const int nb = a.nstar > 0 ? (a.nstar + 255) / 256 : 1;
    k_finish<<<nb, 256, 0, s>>>(a);
    return cudaGetLastError();
}

cudaError_t launch_energy_finish(const EnergyArgs &a, cudaStream_t s) {
    const int nb = a.nstar > 0 ? (a.nstar + 255) / 256 : 1;
    k_energy_finish<<<nb, 256, 0, s>>>(a);
    return cudaGetLastError();
}

}  // namespace pn
