// pn_device.cuh -- device-side building blocks shared by the libpn kernels (sm_103a).
//
//  * bulk-copy (TMA, non-tensor) + mbarrier helpers with bounded waits;
//  * the j-particle "pack" layouts streamed through shared memory;
//  * the per-pair arithmetic of the three pair-sweep modes.
//
// The pair arithmetic is the reference's force (Limit-sticky9.c:36-51 Newtonian, :116-174 and
// :276-382 the two three-body cross sums) and energy (:462-474, :508-537) sweeps, rewritten
// so that one rsqrt per (i,j) pair suffices.  Every BH-distance factor of the reference's pair
// expressions (r1be, r1ce, r1b2, r1c2) depends on one particle only, so it is precomputed per
// particle; the factors that depend on the pair distance (rbce, rbc2e) become per-i sums:
//
//   G_i   = sum_j m_j Q^3 d                     (Newtonian star-star acceleration)
//   Phi_i = sum_j m_j Q                         (star-star potential)
//   S0_i  = sum_j m_j Q^3
//   U_i   = sum_j mu3_j Q                       (mu3_j = m_j R_j^3)
//   W_i   = sum_j cd_ij d + cv_ij dv            (the velocity- and R_j-weighted cross terms)
//   Psi_i = sum_j m_j Q (7 v_i.v_j + (d.v_i)(d.v_j) Q^2)     (energy only)
//
// with d = x_j - x_i, Q = (|d|^2 + eps^2)^(-1/2), R_j = (|x_j - x_0|^2 + eps^2)^(-1/2) and
//   cd_ij = m_j Q^3 [c1_j + c3_j (|d|^2+eps^2 - qe_i) + |v_i|^2 - 2|dv|^2 + 1.5 (v_j.d)^2 Q^2]
//           + k35_j Q
//   cv_ij = m_j Q^3 (4 v_i.d - 3 v_j.d)
// (c1_j = 1.25 m_0 R_j, c3_j = 0.25 m_0 R_j^3, k35_j = 3.5 m_0 mu3_j, qe_i = |x_i-x_0|^2+eps^2).
// The rest of each reference term is a product of per-particle quantities and global sums
// and is evaluated in FP64 by the finishing kernel.  All sums include the j = i self pair,
// as the reference's loops do; the reference's own self-pair removals are applied afterwards.
#pragma once

#include <cstdint>
#include <cuda_runtime.h>

namespace pn {

// ------------------------------------------------------------------ modes and pack layouts
enum PairMode : int {
    MODE_NEWTON = 0,  // G only (inv_c2 == 0)
    MODE_FORCE = 1,   // G, Phi, S0, U, W
    MODE_ENERGY = 2,  // Phi, Psi
    MODE_FORCE_ENERGY = 3  // MODE_FORCE plus Psi: a force evaluation and the energy of its state
};
__host__ __device__ constexpr bool mode_has_force(int mode) { return mode == MODE_FORCE || mode == MODE_FORCE_ENERGY; }

template <int MODE> struct ModeInfo;
template <> struct ModeInfo<MODE_NEWTON> { static constexpr int NACC = 3; static constexpr int NG32 = 2; static constexpr int NG64 = 2; };
template <> struct ModeInfo<MODE_FORCE>  { static constexpr int NACC = 9; static constexpr int NG32 = 4; static constexpr int NG64 = 6; };
template <> struct ModeInfo<MODE_ENERGY> { static constexpr int NACC = 2; static constexpr int NG32 = 3; static constexpr int NG64 = 4; };
template <> struct ModeInfo<MODE_FORCE_ENERGY> { static constexpr int NACC = 10; static constexpr int NG32 = 4; static constexpr int NG64 = 6; };

// Accumulator slots (FP64 output arrays acc[split][slot][i]).
enum AccSlot : int { A_GX = 0, A_GY, A_GZ, A_PHI, A_S0, A_U, A_WX, A_WY, A_WZ, A_PSI };
enum AccSlotE : int { E_PHI = 0, E_PSI = 1 };

// FP32 pack: NG32 float4 groups per star, group-major ([g][padded star]):
//   g0 = hi.xyz, m     g1 = lo.xyz, mu3     g2 = v.xyz, qe     g3 = c1, c3, k35, 0
// where hi + lo is the position relative to the j-tile's FP64 origin split into two FP32
// numbers (hi = fl32(s - o), lo = fl32((s - o) - hi)); the pair difference
// d = (hi_j - hi_i) + (lo_j - lo_i) is then accurate to ~2^-24 |d| + 2^-48 |s - o|, however
// the particles are ordered.
// FP64 pack: NG64 double2 groups per star, group-major:
//   g0 = s.x s.y   g1 = s.z m   g2 = v.x v.y   g3 = v.z mu3   g4 = c1 c3   g5 = k35 qe
// (s = x - x_0, the BH-relative position; qe = |s|^2 + eps^2.)
// Padding stars (index >= nstar) have zero mass and zero weights: they add exactly 0.

// Operand scalings of the packed FP32x2 sweep (pn_pair2.cuh), chosen so that constant factors
// of the pair expressions fold into per-star pack entries and per-i registers instead of
// costing an instruction per pair:
//   the sweep's inverse distance is Q' = K Q: Newton's step y (1.5 - 0.5 x y^2) with both
//   constants times K, exact in FP32 because K has a 22-bit mantissa (K ~ 1/sqrt(2), so
//   Q'^2 ~ Q^2 / 2 carries the 1/2 of the vdj^2 term);
//   j velocities are stored times sqrt(3), the i velocity times 4/sqrt(3) (force sweep; the
//   cv weight 4 vdi - 3 vdj then becomes sqrt(3) (vdi* - vdj')), or times 1/sqrt(3) (energy);
//   masses are stored as m / K^3 and mu3, k35 as mu3 / K, k35 / K; c1 as c1 - 2 |v|^2.
// The sweep's Phi sum comes out as Phi / K^2 and is scaled back in FP64.
constexpr double X2_K = 2965821.0 / 4194304.0;
constexpr double X2_SQRT3 = 1.7320508075688772935;

// Origin of one j-tile (BH-relative): FP64, and the same split into an FP32 pair
// (h = fl32(x), l = fl32(x - h)) for sweeps that form (s_i - o) without FP64 arithmetic.
struct __align__(32) TileOrigin {
    double x, y, z, w;
    float hx, hy, hz, lx, ly, lz, pad0, pad1;
};

// Exact FP32 difference a - b as s + err (Knuth's TwoSum; no multiplications, so nothing is
// contracted into an FMA).
__device__ __forceinline__ float two_diff(float a, float b, float &err) {
    const float s = a - b;
    const float bb = s - a;
    err = (a - (s - bb)) - (b + bb);
    return s;
}

// ------------------------------------------------------------------ device error word bits
enum DevErr : int { DEVERR_TIMEOUT = 1, DEVERR_NONFINITE = 2 };

// ------------------------------------------------------------------ PTX helpers
__device__ __forceinline__ uint32_t smem_u32(const void *p) {
    return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

__device__ __forceinline__ void mbar_init(uint64_t *bar, uint32_t count) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count));
}

__device__ __forceinline__ void fence_mbar_init() {
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

__device__ __forceinline__ void mbar_arrive_expect_tx(uint64_t *bar, uint32_t bytes) {
    asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(smem_u32(bar)),
                 "r"(bytes)
                 : "memory");
}

// 1-D bulk copy global -> shared (the TMA engine, no tensor map).  dst, src 16-byte aligned,
// bytes a multiple of 16; completion is signalled on *bar as transaction bytes.
__device__ __forceinline__ void bulk_g2s(void *dst, const void *src, uint32_t bytes, uint64_t *bar) {
    asm volatile(
        "cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];"
        ::"r"(smem_u32(dst)), "l"(src), "r"(bytes), "r"(smem_u32(bar))
        : "memory");
}

__device__ __forceinline__ bool mbar_try_wait(uint64_t *bar, uint32_t phase) {
    uint32_t ok;
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n\t"
        "selp.u32 %0, 1, 0, p;\n\t}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(phase)
        : "memory");
    return ok != 0;
}

// Bounded wait: gives up after ~limit_cycles SM clocks (about a second) and reports false.
__device__ __forceinline__ bool mbar_wait_bounded(uint64_t *bar, uint32_t phase,
                                                  long long limit_cycles = 2000000000LL) {
    if (mbar_try_wait(bar, phase)) return true;
    long long t0 = clock64();
    while (!mbar_try_wait(bar, phase)) {
        if (clock64() - t0 > limit_cycles) return false;
    }
    return true;
}

// MUFU reciprocal square root (rsqrt.approx, flush-to-zero) refined by one Newton-Raphson
// step y' = y + (y/2)(1 - x y^2) (Newton's method on f(y) = 1/y^2 - x).
__device__ __forceinline__ float rsqrt_mufu_nr(float x) {
    float y;
    asm("rsqrt.approx.ftz.f32 %0, %1;" : "=f"(y) : "f"(x));
    float h = x * y;
    float r = fmaf(-h, y, 1.0f);
    return fmaf(0.5f * y, r, y);
}

// Kahan (compensated) addition of a tile partial into (sum, comp).
__device__ __forceinline__ void kahan_add(float &sum, float &comp, float x) {
    float y = x - comp;
    float t = sum + y;
    comp = (t - sum) - y;
    sum = t;
}

// ------------------------------------------------------------------ per-pair arithmetic
// i-particle state held in registers.
template <typename T> struct IState {
    T ex, ey, ez;   // FP32: hi part of s_i - o_tile (refreshed per tile); FP64: s_i
    T lx, ly, lz;   // FP32: lo part (FP64: unused, 0)
    T vx, vy, vz;
    T vi2;          // |v_i|^2
    T qe;           // |s_i|^2 + eps^2
};

// One (i, j) pair into the running sums acc[NACC].
//   jx..jz: position (FP32: hi part relative to the tile origin; FP64: BH-relative)
//   jlx..jlz: FP32 lo part (FP64: 0)
//   jm: mass, jv*: velocity, jmu3 = m R^3, jc1 = 1.25 m0 R, jc3 = 0.25 m0 R^3, jk35 = 3.5 m0 mu3

template <typename T> __device__ __forceinline__ T pn_rsqrt(T x);
template <> __device__ __forceinline__ float pn_rsqrt<float>(float x) { return rsqrt_mufu_nr(x); }
template <> __device__ __forceinline__ double pn_rsqrt<double>(double x) { return rsqrt(x); }

template <typename T> __device__ __forceinline__ T pn_fma(T a, T b, T c);
template <> __device__ __forceinline__ float pn_fma<float>(float a, float b, float c) { return fmaf(a, b, c); }
template <> __device__ __forceinline__ double pn_fma<double>(double a, double b, double c) { return fma(a, b, c); }

template <int MODE, typename T>
__device__ __forceinline__ void pair_accumulate(T *acc, const IState<T> &I, T jx, T jy, T jz,
                                                T jlx, T jly, T jlz, T jm, T jvx, T jvy, T jvz,
                                                T jmu3, T jc1, T jc3, T jk35, T eps2) {
    T dx, dy, dz;
    if constexpr (sizeof(T) == 4) {
        dx = (jx - I.ex) + (jlx - I.lx);
        dy = (jy - I.ey) + (jly - I.ly);
        dz = (jz - I.ez) + (jlz - I.lz);
    } else {
        dx = jx - I.ex;
        dy = jy - I.ey;
        dz = jz - I.ez;
    }
    const T rhoe = pn_fma(dz, dz, pn_fma(dy, dy, pn_fma(dx, dx, eps2)));
    const T Q = pn_rsqrt<T>(rhoe);
    const T Q2 = Q * Q;
    const T mQ = jm * Q;
    if constexpr (MODE == MODE_NEWTON) {
        const T mQ3 = mQ * Q2;
        acc[A_GX] = pn_fma(mQ3, dx, acc[A_GX]);
        acc[A_GY] = pn_fma(mQ3, dy, acc[A_GY]);
        acc[A_GZ] = pn_fma(mQ3, dz, acc[A_GZ]);
    } else if constexpr (mode_has_force(MODE)) {
        const T mQ3 = mQ * Q2;
        acc[A_GX] = pn_fma(mQ3, dx, acc[A_GX]);
        acc[A_GY] = pn_fma(mQ3, dy, acc[A_GY]);
        acc[A_GZ] = pn_fma(mQ3, dz, acc[A_GZ]);
        acc[A_PHI] += mQ;
        acc[A_S0] += mQ3;
        acc[A_U] = pn_fma(jmu3, Q, acc[A_U]);
        const T dvx = jvx - I.vx, dvy = jvy - I.vy, dvz = jvz - I.vz;
        const T dv2 = pn_fma(dvz, dvz, pn_fma(dvy, dvy, dvx * dvx));
        const T vdj = pn_fma(jvz, dz, pn_fma(jvy, dy, jvx * dx));
        const T vdi = pn_fma(I.vz, dz, pn_fma(I.vy, dy, I.vx * dx));
        T br = pn_fma(rhoe - I.qe, jc3, jc1);
        br += pn_fma(T(-2), dv2, I.vi2);
        br = pn_fma(T(1.5), (vdj * vdj) * Q2, br);
        const T cd = pn_fma(mQ3, br, jk35 * Q);
        const T cv = mQ3 * pn_fma(T(4), vdi, T(-3) * vdj);
        acc[A_WX] = pn_fma(cd, dx, pn_fma(cv, dvx, acc[A_WX]));
        acc[A_WY] = pn_fma(cd, dy, pn_fma(cv, dvy, acc[A_WY]));
        acc[A_WZ] = pn_fma(cd, dz, pn_fma(cv, dvz, acc[A_WZ]));
        if constexpr (MODE == MODE_FORCE_ENERGY) {  // Psi, as MODE_ENERGY's
            const T vivj = pn_fma(I.vz, jvz, pn_fma(I.vy, jvy, I.vx * jvx));
            acc[A_PSI] = pn_fma(mQ, pn_fma(T(7), vivj, (vdi * vdj) * Q2), acc[A_PSI]);
        }
    } else {  // MODE_ENERGY
        acc[E_PHI] += mQ;
        const T vivj = pn_fma(I.vz, jvz, pn_fma(I.vy, jvy, I.vx * jvx));
        const T vdj = pn_fma(jvz, dz, pn_fma(jvy, dy, jvx * dx));
        const T vdi = pn_fma(I.vz, dz, pn_fma(I.vy, dy, I.vx * dx));
        acc[E_PSI] = pn_fma(mQ, pn_fma(T(7), vivj, (vdi * vdj) * Q2), acc[E_PSI]);
    }
}

}  // namespace pn
