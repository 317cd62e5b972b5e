// pn_pair.cuh -- the O(N^2) pair-sweep kernel of libpn.
//
// One kernel template serves the three sweeps of the reference's force path:
//   MODE_NEWTON  Limit-sticky9.c:36-51 (star-star part; the BH row/column is O(N))
//   MODE_FORCE   :36-51 + the pairwise parts of :116-174 and :276-382 (see pn_device.cuh)
//   MODE_ENERGY  the pairwise parts of :462-474 and :508-537
//   MODE_FORCE_ENERGY  MODE_FORCE and MODE_ENERGY's Psi in one sweep (the energy of the state
//                the force is evaluated at, Limit-sticky9.c:895-898 then :837)
// in FP64 (T = double: parity with the reference) or mixed precision (T = float: pair terms
// in FP32, positions relative to a per-tile FP64 origin held as FP32 hi/lo pairs, per-i
// Kahan folding of each tile's partial sums).
//
// Work decomposition.  A CTA of NT = 128 threads owns BI = 128 * IPT / JS i-particles
// (IPT per thread, held in registers; JS consecutive lanes share the same i-set and split each
// tile's j-range, their partial sums are combined by warp shuffles at the end).  blockIdx.y
// selects one of gsplit contiguous j-tile ranges; each range writes its own FP64 partial
// sums acc[split][slot][i], summed in a fixed order by the finishing kernel (deterministic).
//
// j-tiles of tj stars are streamed global -> shared memory by the TMA engine (one
// cp.async.bulk per pack group per tile, completion on an mbarrier), double buffered: the
// copy of tile t+1 is in flight while tile t is computed.  Waits are bounded; a CTA whose
// copy does not arrive within ~1 s sets DEVERR_TIMEOUT, waits (bounded) for its own copies
// and returns.
#pragma once

#include "pn_device.cuh"

namespace pn {

template <typename T> struct PackVec;
template <> struct PackVec<float> { using V = float4; };
template <> struct PackVec<double> { using V = double2; };

struct PairArgs {
    const void *pack;     // [NG][npad] of PackVec<T>::V
    const TileOrigin *torg;  // FP32 only: per-tile FP64 origin (BH-relative), one per tile of tj
    const void *pack2;       // FP32 only: the paired pack of the f32x2 sweep (pn_pair2.cuh)
    const float4 *ipack;     // FP32 only: per star (v.xyz, qe), the f32x2 sweep's i-side data
    const double *spos;   // [3][npad] BH-relative FP64 positions
    double *out;          // [gsplit][NACC][npad]
    int *err;             // device error word
    int nstar;            // stars (particles 1..n-1)
    int npad;             // padded star count (multiple of 256)
    int tj;               // stars per tile (32, 64, 128 or 256)
    int ntiles;           // ceil(nstar / tj)
    int gsplit;           // j-range splits (gridDim.y)
    double eps2;
};

constexpr int PAIR_NT = 128;

inline size_t pair_smem_bytes(int ng, int tj, size_t vec_bytes) {
    return 128 + 2 * (size_t)ng * (size_t)tj * vec_bytes;
}

// Register budget: the FP32 force sweep with 2 i per thread is capped at 128 registers so
// that 4 CTAs (16 warps) stay resident per SM.
template <typename T, int MODE, int IPT>
constexpr int pair_min_blocks() {
    return (sizeof(T) == 4 && IPT == 2) ? 4 : 1;
}

// One work item: the i-block starting at ibase against j-range `split` of a.gsplit.  bars/buf
// are the CTA's two mbarriers and double-buffered tile storage; seq counts the tiles this CTA
// has consumed before (it selects the stage and the mbarrier phase), so a CTA can run several
// items back to back.  Returns false when a bounded wait gave up (the CTA must then stop).
template <typename T, int MODE, int IPT, int JS>
__device__ __forceinline__ bool pair_block(const PairArgs &a, int ibase, int split, uint64_t *bars,
                                           typename PackVec<T>::V *buf, uint32_t &seq) {
    constexpr int NT = PAIR_NT;
    constexpr bool F32 = sizeof(T) == 4;
    constexpr int NG = F32 ? ModeInfo<MODE>::NG32 : ModeInfo<MODE>::NG64;
    constexpr int NACC = ModeInfo<MODE>::NACC;
    constexpr int NI = NT / JS;  // distinct i-lanes per CTA
    using V = typename PackVec<T>::V;
    static_assert(32 % JS == 0, "JS must divide the warp");

    const int tid = threadIdx.x;
    const int sub = tid % JS;
    const int grp = tid / JS;
    const int t0 = (int)(((long long)a.ntiles * split) / a.gsplit);
    const int t1 = (int)(((long long)a.ntiles * (split + 1)) / a.gsplit);
    const int tj = a.tj;
    const V *pack = static_cast<const V *>(a.pack);
    const T eps2 = (T)a.eps2;

    // ---- i-particles into registers
    IState<T> I[IPT];
    double sx[IPT], sy[IPT], sz[IPT];
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + grp + k * NI;
        const bool valid = i < a.nstar;
        sx[k] = valid ? a.spos[i] : 0.0;
        sy[k] = valid ? a.spos[a.npad + i] : 0.0;
        sz[k] = valid ? a.spos[2 * a.npad + i] : 0.0;
        I[k].ex = (T)sx[k];
        I[k].ey = (T)sy[k];
        I[k].ez = (T)sz[k];
        I[k].lx = I[k].ly = I[k].lz = T(0);
        I[k].vx = I[k].vy = I[k].vz = I[k].vi2 = I[k].qe = T(0);
        if constexpr (MODE != MODE_NEWTON) {
            if (valid) {
                if constexpr (F32) {
                    const float4 g2 = reinterpret_cast<const float4 *>(pack)[2 * a.npad + i];
                    I[k].vx = g2.x; I[k].vy = g2.y; I[k].vz = g2.z;
                    I[k].qe = g2.w;
                } else {
                    const double2 g2 = reinterpret_cast<const double2 *>(pack)[2 * a.npad + i];
                    const double2 g3 = reinterpret_cast<const double2 *>(pack)[3 * a.npad + i];
                    I[k].vx = g2.x; I[k].vy = g2.y; I[k].vz = g3.x;
                    if constexpr (mode_has_force(MODE))
                        I[k].qe = reinterpret_cast<const double2 *>(pack)[5 * a.npad + i].y;
                }
                I[k].vi2 = pn_fma(I[k].vz, I[k].vz, pn_fma(I[k].vy, I[k].vy, I[k].vx * I[k].vx));
            }
        }
    }

    // ---- running sums: FP32 mode keeps Kahan (sum, comp) pairs; FP64 mode sums directly
    T run[IPT][NACC];
    T cmp[IPT][NACC];
#pragma unroll
    for (int k = 0; k < IPT; ++k)
#pragma unroll
        for (int q = 0; q < NACC; ++q) run[k][q] = cmp[k][q] = T(0);

    const uint32_t gbytes = (uint32_t)tj * (uint32_t)sizeof(V);
    auto issue = [&](int t, int stage) {
        mbar_arrive_expect_tx(&bars[stage], (uint32_t)NG * gbytes);
#pragma unroll
        for (int g = 0; g < NG; ++g)
            bulk_g2s(buf + (size_t)(stage * NG + g) * tj, pack + (size_t)g * a.npad + (size_t)t * tj,
                     gbytes, &bars[stage]);
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
            // A copy did not arrive: record it, let this CTA's copies drain (bounded), leave.
            if (tid == 0) {
                atomicOr(a.err, DEVERR_TIMEOUT);
                mbar_wait_bounded(&bars[stage], phase);
                if (next) mbar_wait_bounded(&bars[stage ^ 1], ((it + 1) >> 1) & 1u);
            }
            return false;
        }
        if constexpr (F32) {
            const TileOrigin o = a.torg[t];
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                const double rx = sx[k] - o.x, ry = sy[k] - o.y, rz = sz[k] - o.z;
                I[k].ex = (float)rx;
                I[k].ey = (float)ry;
                I[k].ez = (float)rz;
                I[k].lx = (float)(rx - (double)I[k].ex);
                I[k].ly = (float)(ry - (double)I[k].ey);
                I[k].lz = (float)(rz - (double)I[k].ez);
            }
        }
        const V *b = buf + (size_t)stage * NG * tj;
        T tacc[IPT][NACC];
#pragma unroll
        for (int k = 0; k < IPT; ++k)
#pragma unroll
            for (int q = 0; q < NACC; ++q) tacc[k][q] = T(0);

#pragma unroll 2
        for (int j = sub; j < tj; j += JS) {
            T jx, jy, jz, jm, jlx = 0, jly = 0, jlz = 0, jvx = 0, jvy = 0, jvz = 0, jmu3 = 0,
              jc1 = 0, jc3 = 0, jk35 = 0;
            if constexpr (F32) {
                const float4 g0 = b[j], g1 = b[tj + j];
                jx = g0.x; jy = g0.y; jz = g0.z; jm = g0.w;
                jlx = g1.x; jly = g1.y; jlz = g1.z; jmu3 = g1.w;
                if constexpr (MODE != MODE_NEWTON) {
                    const float4 g2 = b[2 * tj + j];
                    jvx = g2.x; jvy = g2.y; jvz = g2.z;
                }
                if constexpr (mode_has_force(MODE)) {
                    const float4 g3 = b[3 * tj + j];
                    jc1 = g3.x; jc3 = g3.y; jk35 = g3.z;
                }
            } else {
                const double2 g0 = b[j], g1 = b[tj + j];
                jx = g0.x; jy = g0.y; jz = g1.x; jm = g1.y;
                if constexpr (MODE != MODE_NEWTON) {
                    const double2 g2 = b[2 * tj + j], g3 = b[3 * tj + j];
                    jvx = g2.x; jvy = g2.y; jvz = g3.x; jmu3 = g3.y;
                }
                if constexpr (mode_has_force(MODE)) {
                    const double2 g4 = b[4 * tj + j], g5 = b[5 * tj + j];
                    jc1 = g4.x; jc3 = g4.y; jk35 = g5.x;
                }
            }
#pragma unroll
            for (int k = 0; k < IPT; ++k) {
                if constexpr (F32)
                    pair_accumulate<MODE, T>(tacc[k], I[k], jx, jy, jz, jlx, jly, jlz, jm, jvx, jvy,
                                             jvz, jmu3, jc1, jc3, jk35, eps2);
                else
                    pair_accumulate<MODE, T>(run[k], I[k], jx, jy, jz, jlx, jly, jlz, jm, jvx, jvy,
                                             jvz, jmu3, jc1, jc3, jk35, eps2);
            }
        }
        if constexpr (F32) {
#pragma unroll
            for (int k = 0; k < IPT; ++k)
#pragma unroll
                for (int q = 0; q < NACC; ++q) kahan_add(run[k][q], cmp[k][q], tacc[k][q]);
        }
        __syncthreads();  // every thread is done with this stage before it is refilled
    }

    // ---- combine the JS lanes sharing an i-set, write FP64 partial sums
#pragma unroll
    for (int k = 0; k < IPT; ++k) {
        const int i = ibase + grp + k * NI;
#pragma unroll
        for (int q = 0; q < NACC; ++q) {
            double val = F32 ? (double)run[k][q] - (double)cmp[k][q] : (double)run[k][q];
#pragma unroll
            for (int off = JS / 2; off > 0; off >>= 1) val += __shfl_xor_sync(0xffffffffu, val, off);
            if (sub == 0 && i < a.nstar)
                a.out[((size_t)split * NACC + q) * a.npad + i] = val;
        }
    }
    seq += (uint32_t)(t1 - t0 > 0 ? t1 - t0 : 0);
    return true;
}

template <typename T, int MODE, int IPT, int JS>
__global__ void __launch_bounds__(PAIR_NT, (pair_min_blocks<T, MODE, IPT>())) k_pair(const PairArgs a) {
    using V = typename PackVec<T>::V;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    V *buf = reinterpret_cast<V *>(smem + 128);
    if (threadIdx.x == 0) {
        mbar_init(&bars[0], 1);
        mbar_init(&bars[1], 1);
        fence_mbar_init();
    }
    __syncthreads();
    uint32_t seq = 0;
    pair_block<T, MODE, IPT, JS>(a, blockIdx.x * (PAIR_NT / JS * IPT), blockIdx.y, bars, buf, seq);
}

// Ensemble sweep: one persistent launch over the work items of every cluster.
// items[w] = (cluster, first i of the block, j-range split, 0), ordered by decreasing cost;
// tab[cluster] holds that cluster's arguments (pointers offset to its slots, its tile size,
// split count and softening).  Each CTA takes the next item from *counter until the list is
// exhausted: the counter only grows, so every CTA leaves after at most nitems + 1 fetches.
// The counter is zeroed before each launch.
template <typename T, int MODE, int IPT, int JS>
__global__ void __launch_bounds__(PAIR_NT, (pair_min_blocks<T, MODE, IPT>()))
    k_pair_ens(const PairArgs *tab, const int4 *items, int nitems, unsigned *counter) {
    using V = typename PackVec<T>::V;
    extern __shared__ __align__(128) unsigned char smem[];
    uint64_t *bars = reinterpret_cast<uint64_t *>(smem);
    V *buf = reinterpret_cast<V *>(smem + 128);
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
        const PairArgs a = tab[it.x];
        if (!pair_block<T, MODE, IPT, JS>(a, it.y, it.z, bars, buf, seq)) break;
    }
}

}  // namespace pn
