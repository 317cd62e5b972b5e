// pn_pair2.cuh -- the FP32 pair sweep on packed FP32x2 instructions (sm_100+ f32x2 PTX).
//
// Same sweeps and the same arithmetic per pair as k_pair<float, MODE> (pn_pair.cuh), but every
// instruction works on TWO j-stars at once: lane 0 of an f32x2 register holds star 2k of the
// tile, lane 1 star 2k+1, while the i-particle's values are broadcast to both lanes once per
// tile.  A pair then costs about half the issue slots (the FMA pipe still does the same work),
// which lifts the sweep from issue-bound to FMA-pipe-bound.  The MUFU rsqrt has no paired form
// and runs once per lane.
//
// j-data come from the "paired" pack (written by k_prep in mixed precision): for star pair k
// of a tile, 7 float4 groups, group-major over pairs ([g][npad/2]):
//   P0 (hx hx' hy hy')  P1 (hz hz' mK mK')  P2 (lx lx' ly ly')  P3 (lz lz' mu3K mu3K')
//   P4 (wx wx' wy wy')  P5 (wz wz' c1v c1v')  P6 (c3 c3' k35K k35K')
// (primed = odd star), so one 128-bit shared load yields two f32x2 operands.  The entries are
// scaled (pn_device.cuh, X2_K): mK = m / K^3, mu3K = mu3 / K, k35K = k35 / K, w = sqrt(3) v,
// c1v = c1 - 2 |v|^2.  With the sweep's Q' = K Q these fold every constant factor of the pair
// expressions into data: 50 FP32 operations per force pair instead of 56, and
//   br = (rhoe - qe) c3 + c1 + |v_i|^2 - 2 |dv|^2 + 1.5 vdj^2 Q^2
//      = (rhoe - qe) c3 + c1v + (vi* . w_j - |v_i|^2) + (w_j . d)^2 Q'^2      (vi* = 4 v_i / sqrt(3))
//   sum_j cv dv = sum_j ct w_j - 0.75 vi* sum_j ct,  ct = mQ^3 (vi* . d - w_j . d) = cv / sqrt(3)
// (the last term is applied once per tile).  3 K^2 = 1.5 (1 + 1.3e-7): the vdj^2 term carries
// that relative bias, a 1PN sub-term far below the FP32 rounding of the sums.
#pragma once

#include "pn_pair.cuh"

namespace pn {

typedef unsigned long long f2;  // two FP32 values in one 64-bit register pair

__device__ __forceinline__ f2 f2_pack(float lo, float hi) {
    f2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r) : "f"(lo), "f"(hi));
    return r;
}
__device__ __forceinline__ void f2_unpack(f2 v, float &lo, float &hi) {
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(v));
}
__device__ __forceinline__ f2 f2_bcast(float v) { return f2_pack(v, v); }
__device__ __forceinline__ f2 add2(f2 a, f2 b) {
    f2 r;
    asm("add.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 sub2(f2 a, f2 b) {
    f2 r;
    asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 mul2(f2 a, f2 b) {
    f2 r;
    asm("mul.rn.f32x2 %0, %1, %2;" : "=l"(r) : "l"(a), "l"(b));
    return r;
}
__device__ __forceinline__ f2 fma2(f2 a, f2 b, f2 c) {
    f2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r) : "l"(a), "l"(b), "l"(c));
    return r;
}
// One 128-bit shared-memory load of a pack group: two f32x2 operands.  A plain C++ load, so the
// compiler can schedule it among the arithmetic (an asm volatile load issued 6 % more
// instructions and ran 2 % slower); it cannot move above the tile's arrival, which the
// mbarrier wait (an asm with a memory clobber) orders before it.
__device__ __forceinline__ void lds2(const void *p, f2 &a, f2 &b) {
    const ulonglong2 u = *static_cast<const ulonglong2 *>(p);
    a = u.x;
    b = u.y;
}
// K times the inverse square root of both lanes: MUFU rsqrt each, refined by one Newton-Raphson
// step y' = y (1.5 - 0.5 x y^2) whose two constants are scaled by K (exact in FP32).
__device__ __forceinline__ f2 rsqrt2k(f2 x) {
    float a, b;
    f2_unpack(x, a, b);
    float ya, yb;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(ya) : "f"(a));
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(yb) : "f"(b));
    const f2 y = f2_pack(ya, yb);
    constexpr float K = (float)X2_K;
    const f2 nxh = mul2(x, f2_bcast(-0.5f * K));
    const f2 r = fma2(nxh, mul2(y, y), f2_bcast(1.5f * K));
    return mul2(y, r);
}
__device__ __forceinline__ float f2_sum(f2 v) {
    float a, b;
    f2_unpack(v, a, b);
    return a + b;
}

struct I2 {  // one i-particle, broadcast to both lanes
    f2 ex, ey, ez, lx, ly, lz;  // hi/lo of s_i - o_tile (refreshed per tile)
    f2 vx, vy, vz;              // force: 4 v_i / sqrt(3); energy: v_i / sqrt(3)
    f2 nvi2, qe;                // -|v_i|^2, |s_i|^2 + eps^2
};


template <int MODE>
__device__ __forceinline__ void pair2_accumulate(f2 *acc, const I2 &I, f2 jx, f2 jy, f2 jz, f2 jlx, f2 jly,
                                                 f2 jlz, f2 jm, f2 jwx, f2 jwy, f2 jwz, f2 jmu3, f2 jc1,
                                                 f2 jc3, f2 jk35, f2 eps2) {
    const f2 dx = add2(sub2(jx, I.ex), sub2(jlx, I.lx));
    const f2 dy = add2(sub2(jy, I.ey), sub2(jly, I.ly));
    const f2 dz = add2(sub2(jz, I.ez), sub2(jlz, I.lz));
    const f2 rhoe = fma2(dz, dz, fma2(dy, dy, fma2(dx, dx, eps2)));
    const f2 Q = rsqrt2k(rhoe);   // K Q
    const f2 Q2 = mul2(Q, Q);     // K^2 Q^2
    const f2 mQ = mul2(jm, Q);    // m Q / K^2
    if constexpr (MODE == MODE_NEWTON) {
        const f2 mQ3 = mul2(mQ, Q2);  // m Q^3
        acc[A_GX] = fma2(mQ3, dx, acc[A_GX]);
        acc[A_GY] = fma2(mQ3, dy, acc[A_GY]);
        acc[A_GZ] = fma2(mQ3, dz, acc[A_GZ]);
    } else if constexpr (mode_has_force(MODE)) {
        constexpr int A_CT = ModeInfo<MODE>::NACC;  // per-tile sum of ct (folded into W per tile)
        const f2 mQ3 = mul2(mQ, Q2);
        acc[A_GX] = fma2(mQ3, dx, acc[A_GX]);
        acc[A_GY] = fma2(mQ3, dy, acc[A_GY]);
        acc[A_GZ] = fma2(mQ3, dz, acc[A_GZ]);
        acc[A_PHI] = add2(acc[A_PHI], mQ);
        acc[A_S0] = add2(acc[A_S0], mQ3);
        acc[A_U] = fma2(jmu3, Q, acc[A_U]);
        const f2 vivj = fma2(I.vz, jwz, fma2(I.vy, jwy, fma2(I.vx, jwx, I.nvi2)));  // 4 vi.vj - vi^2
        const f2 vdj = fma2(jwz, dz, fma2(jwy, dy, mul2(jwx, dx)));                // sqrt(3) vj.d
        const f2 vdi = fma2(I.vz, dz, fma2(I.vy, dy, mul2(I.vx, dx)));             // 4/sqrt(3) vi.d
        f2 br = fma2(sub2(rhoe, I.qe), jc3, jc1);
        br = add2(br, vivj);
        br = fma2(mul2(vdj, vdj), Q2, br);
        const f2 cd = fma2(mQ3, br, mul2(jk35, Q));
        const f2 ct = mul2(mQ3, sub2(vdi, vdj));
        acc[A_WX] = fma2(cd, dx, fma2(ct, jwx, acc[A_WX]));
        acc[A_WY] = fma2(cd, dy, fma2(ct, jwy, acc[A_WY]));
        acc[A_WZ] = fma2(cd, dz, fma2(ct, jwz, acc[A_WZ]));
        acc[A_CT] = add2(acc[A_CT], ct);
        if constexpr (MODE == MODE_FORCE_ENERGY) {
            // sum mQ' (7K^2 vivj + vdi vdj Q'^2) = 4 Psi - 7 |v_i|^2 Phi with the scaled operands
            // above; Psi = sum/4 + 1.75 |v_i|^2 Phi is formed in FP64 when the sums are written
            constexpr float c7 = (float)(7.0 * X2_K * X2_K);
            acc[A_PSI] = fma2(mQ, fma2(f2_bcast(c7), vivj, mul2(mul2(vdi, vdj), Q2)), acc[A_PSI]);
        }
    } else {  // MODE_ENERGY: sum m Q K^2 (7 vi.vj + vdi vdj Q^2) / K^2
        acc[E_PHI] = add2(acc[E_PHI], mQ);
        const f2 vivj = fma2(I.vz, jwz, fma2(I.vy, jwy, mul2(I.vx, jwx)));
        const f2 vdj = fma2(jwz, dz, fma2(jwy, dy, mul2(jwx, dx)));
        const f2 vdi = fma2(I.vz, dz, fma2(I.vy, dy, mul2(I.vx, dx)));
        constexpr float c7 = (float)(7.0 * X2_K * X2_K);
        acc[E_PSI] = fma2(mQ, fma2(f2_bcast(c7), vivj, mul2(mul2(vdi, vdj), Q2)), acc[E_PSI]);
    }
}

template <int MODE> struct Mode2 {
    static constexpr int NG = MODE == MODE_NEWTON ? 4 : (mode_has_force(MODE) ? 7 : 6);
    static constexpr int NTACC = ModeInfo<MODE>::NACC + (mode_has_force(MODE) ? 1 : 0);  // + ct
    static constexpr int PHI = mode_has_force(MODE) ? (int)A_PHI : (MODE == MODE_ENERGY ? (int)E_PHI : -1);
};

// Kahan running sums of the per-i tile partials, kept in shared memory (they are touched once
// per tile), [2 (sum, compensation)][NACC][IPT][PAIR_NT] floats after the two mbarriers; the
// tile buffers follow at a fixed offset, so the ensemble kernel's per-cluster tile sizes need no
// runtime layout.
template <int MODE, int IPT>
__host__ __device__ constexpr size_t pair2_kahan_bytes() {
    return (size_t)2 * ModeInfo<MODE>::NACC * IPT * PAIR_NT * sizeof(float);
}
template <int MODE, int IPT>
inline size_t pair2_smem_bytes(int tj) {
    return 128 + pair2_kahan_bytes<MODE, IPT>() + 2 * (size_t)Mode2<MODE>::NG * (size_t)(tj / 2) * 16;
}

// Resident CTAs per SM the register budget is sized for: 4 at IPT = 1 (<= 128 registers); at
// IPT = 2 either 2 (no register cap, ~196) or 3 (<= 168 registers), both offered to the tuner
// (PairCfg::x2 = 1 or 2).
template <int IPT, int OCC>
constexpr int pair2_min_blocks() {
    return IPT == 1 ? 4 : OCC;
}

// One work item of the paired sweep: the i-block at ibase (128 * IPT stars) against j-range
// `split`.  As pair_block (pn_pair.cuh): TMA double-buffered tiles, bounded waits, per-i Kahan
// folding of each tile's sums, FP64 partial sums out.  a.pack is the paired pack, a.ipack the
// i-side float4 (v.xyz, qe) array.
template <int MODE, int IPT>
__device__ __forceinline__ bool pair2_block(const PairArgs &a, int ibase, int split, uint64_t *bars,
                                            float *kahan, float4 *buf, uint32_t &seq) {
    constexpr int NT = PAIR_NT;
    constexpr int NG = Mode2<MODE>::NG;
    constexpr int NACC = ModeInfo<MODE>::NACC;
    constexpr int NTACC = Mode2<MODE>::NTACC;
    const int tid = threadIdx.x;
    const int t0 = (int)(((long long)a.ntiles * split) / a.gsplit);
    const int t1 = (int)(((long long)a.ntiles * (split + 1)) / a.gsplit);
    const int tj = a.tj, tp = tj / 2;  // stars and star pairs per tile
    const int prow = a.npad / 2;       // row stride of the paired pack, in float4
    const float4 *pack = static_cast<const float4 *>(a.pack);
    const f2 eps2 = f2_bcast((float)a.eps2);

    I2 I[IPT];
    // the i position (BH-relative) as an FP32 pair, split once; per tile, s_i - o_t is formed
    // from it and the tile origin's FP32 pair by an exact difference (two_diff), with no FP64
    // arithmetic in the tile loop
    float shx[IPT], shy[IPT], shz[IPT], slx[IPT], sly[IPT], slz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + tid + k * NT;
        const bool valid = i < a.nstar;
        const double sx = valid ? a.spos[i] : 0.0;
        const double sy = valid ? a.spos[a.npad + i] : 0.0;
        const double sz = valid ? a.spos[2 * a.npad + i] : 0.0;
        shx[k] = (float)sx; slx[k] = (float)(sx - (double)shx[k]);
        shy[k] = (float)sy; sly[k] = (float)(sy - (double)shy[k]);
        shz[k] = (float)sz; slz[k] = (float)(sz - (double)shz[k]);
        float vx = 0.f, vy = 0.f, vz = 0.f, qe = 0.f;
        if (MODE != MODE_NEWTON && valid) {
            const float4 g = a.ipack[i];
            vx = g.x; vy = g.y; vz = g.z; qe = g.w;
        }
        constexpr float vs = (float)(mode_has_force(MODE) ? 4.0 / X2_SQRT3 : 1.0 / X2_SQRT3);
        I[k].vx = f2_bcast(vs * vx);
        I[k].vy = f2_bcast(vs * vy);
        I[k].vz = f2_bcast(vs * vz);
        I[k].qe = f2_bcast(qe);
        I[k].nvi2 = f2_bcast(-fmaf(vz, vz, fmaf(vy, vy, vx * vx)));
    }
    // Kahan state of (slot q, i k) of this thread at kahan[q][k][tid] (sum) and
    // kahan[NACC + q][k][tid] (compensation)
    auto ksum = [&](int q, int k) -> float & { return kahan[(q * IPT + k) * NT + tid]; };
    auto kcmp = [&](int q, int k) -> float & { return kahan[((NACC + q) * IPT + k) * NT + tid]; };
#pragma unroll
    for (int k = 0; k < IPT; ++k)
#pragma unroll
        for (int q = 0; q < NACC; ++q) ksum(q, k) = kcmp(q, k) = 0.f;

    const uint32_t gbytes = (uint32_t)tp * 16u;
    auto issue = [&](int t, int stage) {
        mbar_arrive_expect_tx(&bars[stage], (uint32_t)NG * gbytes);
#pragma unroll
        for (int g = 0; g < NG; ++g)
            bulk_g2s(buf + (size_t)(stage * NG + g) * tp, pack + (size_t)g * prow + (size_t)t * tp, gbytes,
                     &bars[stage]);
    };
    if (tid == 0 && t0 < t1) issue(t0, (int)(seq & 1u));

    for (int t = t0; t < t1; ++t) {
        const uint32_t it = seq + (uint32_t)(t - t0);
        const int stage = (int)(it & 1u);
        const uint32_t phase = (it >> 1) & 1u;
        const bool next = (t + 1 < t1);
        if (tid == 0 && next) issue(t + 1, stage ^ 1);
        const bool ok = mbar_wait_bounded(&bars[stage], phase);
        if (__syncthreads_or(!ok)) {
            if (tid == 0) {
                atomicOr(a.err, DEVERR_TIMEOUT);
                mbar_wait_bounded(&bars[stage], phase);
                if (next) mbar_wait_bounded(&bars[stage ^ 1], ((it + 1) >> 1) & 1u);
            }
            return false;
        }
        {
            // s_i - o_t = (sh - oh) + (sl - ol): the hi difference exactly (two_diff), its error
            // and the lo difference in the lo part
            const TileOrigin &o = a.torg[t];
            const float ohx = o.hx, ohy = o.hy, ohz = o.hz, olx = o.lx, oly = o.ly, olz = o.lz;
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                float ex, ey, ez;
                const float hx = two_diff(shx[k], ohx, ex);
                const float hy = two_diff(shy[k], ohy, ey);
                const float hz = two_diff(shz[k], ohz, ez);
                I[k].ex = f2_bcast(hx);
                I[k].ey = f2_bcast(hy);
                I[k].ez = f2_bcast(hz);
                I[k].lx = f2_bcast(ex + (slx[k] - olx));
                I[k].ly = f2_bcast(ey + (sly[k] - oly));
                I[k].lz = f2_bcast(ez + (slz[k] - olz));
            }
        }
        const float4 *b = buf + (size_t)stage * NG * tp;
        f2 tacc[IPT][NTACC];
#pragma unroll
        for (int k = 0; k < IPT; ++k)
#pragma unroll
            for (int q = 0; q < NTACC; ++q) tacc[k][q] = 0ull;  // +0.0f in both lanes

#pragma unroll 2
        for (int jp = 0; jp < tp; ++jp) {
            f2 jx, jy, jz, jm, jlx, jly, jlz, jmu3, jvx = 0, jvy = 0, jvz = 0, jc1 = 0, jc3 = 0, jk35 = 0;  // scaled
            lds2(b + jp, jx, jy);
            lds2(b + tp + jp, jz, jm);
            lds2(b + 2 * tp + jp, jlx, jly);
            lds2(b + 3 * tp + jp, jlz, jmu3);
            if constexpr (MODE != MODE_NEWTON) {
                lds2(b + 4 * tp + jp, jvx, jvy);
                lds2(b + 5 * tp + jp, jvz, jc1);
            }
            if constexpr (mode_has_force(MODE)) lds2(b + 6 * tp + jp, jc3, jk35);
#pragma unroll
            for (int k = 0; k < IPT; ++k)
                pair2_accumulate<MODE>(tacc[k], I[k], jx, jy, jz, jlx, jly, jlz, jm, jvx, jvy, jvz, jmu3, jc1,
                                       jc3, jk35, eps2);
        }
#pragma unroll
        for (int k = 0; k < IPT; ++k) {
            float ts[NACC];
#pragma unroll
            for (int q = 0; q < NACC; ++q) ts[q] = f2_sum(tacc[k][q]);
            if constexpr (mode_has_force(MODE)) {  // sum ct dv = sum ct w_j - 0.75 vi* sum ct
                const float c = -0.75f * f2_sum(tacc[k][NACC]);
                float wx, wy, wz, u;
                f2_unpack(I[k].vx, wx, u);
                f2_unpack(I[k].vy, wy, u);
                f2_unpack(I[k].vz, wz, u);
                ts[A_WX] = fmaf(c, wx, ts[A_WX]);
                ts[A_WY] = fmaf(c, wy, ts[A_WY]);
                ts[A_WZ] = fmaf(c, wz, ts[A_WZ]);
            }
#pragma unroll
            for (int q = 0; q < NACC; ++q) {
                float sum = ksum(q, k), comp = kcmp(q, k);
                kahan_add(sum, comp, ts[q]);
                ksum(q, k) = sum;
                kcmp(q, k) = comp;
            }
        }
        __syncthreads();
    }
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + tid + k * NT;
        if (i < a.nstar) {
            double val[NACC];
#pragma unroll
            for (int q = 0; q < NACC; ++q)
                val[q] = ((double)ksum(q, k) - (double)kcmp(q, k)) * (q == Mode2<MODE>::PHI ? X2_K * X2_K : 1.0);
            if constexpr (MODE == MODE_FORCE_ENERGY) {
                float nvi2, u;
                f2_unpack(I[k].nvi2, nvi2, u);
                val[A_PSI] = 0.25 * val[A_PSI] - 1.75 * (double)nvi2 * val[A_PHI];
            }
#pragma unroll
            for (int q = 0; q < NACC; ++q) a.out[((size_t)split * NACC + q) * a.npad + i] = val[q];
        }
    }
    seq += (uint32_t)(t1 - t0 > 0 ? t1 - t0 : 0);
    return true;
}

template <int MODE, int IPT, int OCC>
__global__ void __launch_bounds__(PAIR_NT, (pair2_min_blocks<IPT, OCC>())) k_pair2(const PairArgs a) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float *kahan = reinterpret_cast<float *>(smem + 128);
    float4 *buf = reinterpret_cast<float4 *>(smem + 128 + pair2_kahan_bytes<MODE, IPT>());
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t seq = 0;
    pair2_block<MODE, IPT>(a, blockIdx.x * (PAIR_NT * IPT), blockIdx.y, bars, kahan, buf, seq);
}

// Ensemble form: one persistent launch over the work items of every cluster, as k_pair_ens
// (pn_pair.cuh), each item swept in the packed form on its cluster's paired pack (the table's
// pack2).  The counter only grows, so every CTA leaves after at most nitems + 1 fetches.
template <int MODE, int IPT>
__global__ void __launch_bounds__(PAIR_NT, (pair2_min_blocks<IPT, 3>()))
    k_pair2_ens(const PairArgs *tab, const int4 *items, int nitems, unsigned *counter) {
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    float *kahan = reinterpret_cast<float *>(smem + 128);
    float4 *buf = reinterpret_cast<float4 *>(smem + 128 + pair2_kahan_bytes<MODE, IPT>());
    __shared__ int cur;
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t seq = 0;
    for (;;) {
        if (threadIdx.x == 0) cur = (int)atomicAdd(counter, 1u);
        __syncthreads();
        const int w = cur;
        __syncthreads();  // everyone has read cur before thread 0 fetches the next item
        if (w >= nitems) break;
        const int4 it = items[w];
        PairArgs a = tab[it.x];
        a.pack = a.pack2;
        if (!pair2_block<MODE, IPT>(a, it.y, it.z, bars, kahan, buf, seq)) break;
    }
}

}  // namespace pn
