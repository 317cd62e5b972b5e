// pn_pair_f32.cu -- instantiations and launcher of the float pair-sweep kernel (see pn_pair.cuh).
#include "pn_internal.h"
#include "pn_pair2.cuh"

namespace pn {

// the packed f32x2 sweep (pn_pair2.cuh) on the paired pack
template <int MODE, int IPT, int OCC>
static cudaError_t launch_two(const PairCfg &c, const PairArgs &a0, cudaStream_t s) {
    PairArgs a = a0;
    a.pack = a0.pack2;
    const size_t smem = pair2_smem_bytes<MODE, IPT>(c.tj);
    auto fn = k_pair2<MODE, IPT, OCC>;
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const int bi = PAIR_NT * IPT;
    dim3 grid((unsigned)((a.nstar + bi - 1) / bi), (unsigned)c.gsplit);
    fn<<<grid, PAIR_NT, smem, s>>>(a);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_two_mode(const PairCfg &c, const PairArgs &a, cudaStream_t s) {
    if (c.js != 1 || !a.pack2 || !a.ipack) return cudaErrorInvalidValue;
    if (c.ipt == 1) return launch_two<MODE, 1, 4>(c, a, s);
    if (c.ipt == 2) {
        if constexpr (mode_has_force(MODE)) {  // 3 or 4 CTAs per SM (x2 = 2, 3): the force sweeps only
            if (c.x2 == 2) return launch_two<MODE, 2, 3>(c, a, s);
            if (c.x2 == 3) return launch_two<MODE, 2, 4>(c, a, s);
        }
        return launch_two<MODE, 2, 2>(c, a, s);
    }
    return cudaErrorInvalidValue;
}

template <int MODE, int IPT, int JS>
static cudaError_t launch_one(const PairCfg &c, const PairArgs &a, cudaStream_t s) {
    constexpr bool F32 = sizeof(float) == 4;
    const int ng = F32 ? ModeInfo<MODE>::NG32 : ModeInfo<MODE>::NG64;
    const size_t smem = pair_smem_bytes(ng, c.tj, sizeof(float4));
    auto fn = k_pair<float, MODE, IPT, JS>;
    static size_t configured = 0;  // largest dynamic smem size enabled so far
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    const int bi = PAIR_NT * IPT / JS;
    dim3 grid((unsigned)((a.nstar + bi - 1) / bi), (unsigned)c.gsplit);
    fn<<<grid, PAIR_NT, smem, s>>>(a);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_mode(const PairCfg &c, const PairArgs &a, cudaStream_t s) {
    if (c.js == 1) {
        if (c.ipt == 1) return launch_one<MODE, 1, 1>(c, a, s);
        if (c.ipt == 2) return launch_one<MODE, 2, 1>(c, a, s);
        if (c.ipt == 4) return launch_one<MODE, 4, 1>(c, a, s);
    } else if (c.ipt == 1) {
        if (c.js == 2) return launch_one<MODE, 1, 2>(c, a, s);
        if (c.js == 4) return launch_one<MODE, 1, 4>(c, a, s);
        if (c.js == 8) return launch_one<MODE, 1, 8>(c, a, s);
    }
    return cudaErrorInvalidValue;
}

cudaError_t launch_pair_f32(int mode, const PairCfg &c, const PairArgs &a, cudaStream_t s) {
    if (a.nstar <= 0) return cudaSuccess;
    if (c.x2) {
        switch (mode) {
            case MODE_NEWTON: return launch_two_mode<MODE_NEWTON>(c, a, s);
            case MODE_FORCE: return launch_two_mode<MODE_FORCE>(c, a, s);
            case MODE_ENERGY: return launch_two_mode<MODE_ENERGY>(c, a, s);
            case MODE_FORCE_ENERGY: return launch_two_mode<MODE_FORCE_ENERGY>(c, a, s);
            default: return cudaErrorInvalidValue;
        }
    }
    if (mode == MODE_FORCE_ENERGY) {  // instantiated for the block shapes with one i-set per lane
        PairCfg k = c;
        if (k.js != 1 || (k.ipt != 1 && k.ipt != 2)) { k.js = 1; k.ipt = 1; }
        return k.ipt == 2 ? launch_one<MODE_FORCE_ENERGY, 2, 1>(k, a, s) : launch_one<MODE_FORCE_ENERGY, 1, 1>(k, a, s);
    }
    switch (mode) {
        case MODE_NEWTON: return launch_mode<MODE_NEWTON>(c, a, s);
        case MODE_FORCE: return launch_mode<MODE_FORCE>(c, a, s);
        case MODE_ENERGY: return launch_mode<MODE_ENERGY>(c, a, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pn

namespace pn {

template <int MODE, int IPT, int JS>
static cudaError_t launch_ens_one(int tjmax, int grid, const PairArgs *tab, const int4 *items,
                                  int nitems, unsigned *counter, cudaStream_t s) {
    constexpr bool F32 = sizeof(float) == 4;
    const int ng = F32 ? ModeInfo<MODE>::NG32 : ModeInfo<MODE>::NG64;
    const size_t smem = pair_smem_bytes(ng, tjmax, sizeof(float4));
    auto fn = k_pair_ens<float, MODE, IPT, JS>;
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    if (grid <= 0) {  // persistent: as many CTAs as fit on the GPU at once
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, PAIR_NT, smem);
        grid = sms * (per > 0 ? per : 1);
    }
    fn<<<grid, PAIR_NT, smem, s>>>(tab, items, nitems, counter);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_ens_mode(int ipt, int js, int tjmax, int grid, const PairArgs *tab,
                                   const int4 *items, int nitems, unsigned *counter, cudaStream_t s) {
    if (js == 1) {
        if (ipt == 1) return launch_ens_one<MODE, 1, 1>(tjmax, grid, tab, items, nitems, counter, s);
        if (ipt == 2) return launch_ens_one<MODE, 2, 1>(tjmax, grid, tab, items, nitems, counter, s);
    } else if (ipt == 1 && js == 4) {
        return launch_ens_one<MODE, 1, 4>(tjmax, grid, tab, items, nitems, counter, s);
    }
    return cudaErrorInvalidValue;
}

template <int MODE, int IPT>
static cudaError_t launch_ens_two(int tjmax, int grid, const PairArgs *tab, const int4 *items, int nitems,
                                  unsigned *counter, cudaStream_t s) {
    const size_t smem = pair2_smem_bytes<MODE, IPT>(tjmax);
    auto fn = k_pair2_ens<MODE, IPT>;
    static size_t configured = 0;
    if (smem > 48 * 1024 && smem > configured) {
        cudaError_t e = cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem);
        if (e != cudaSuccess) return e;
        configured = smem;
    }
    if (grid <= 0) {  // persistent: as many CTAs as fit on the GPU at once
        int dev = 0, sms = 0, per = 0;
        cudaGetDevice(&dev);
        cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
        cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per, fn, PAIR_NT, smem);
        grid = sms * (per > 0 ? per : 1);
    }
    fn<<<grid, PAIR_NT, smem, s>>>(tab, items, nitems, counter);
    return cudaGetLastError();
}

template <int MODE>
static cudaError_t launch_ens_two_mode(int ipt, int tjmax, int grid, const PairArgs *tab, const int4 *items,
                                       int nitems, unsigned *counter, cudaStream_t s) {
    if (ipt == 1) return launch_ens_two<MODE, 1>(tjmax, grid, tab, items, nitems, counter, s);
    if (ipt == 2) return launch_ens_two<MODE, 2>(tjmax, grid, tab, items, nitems, counter, s);
    return cudaErrorInvalidValue;
}

cudaError_t launch_pair2_ens_f32(int mode, int ipt, int tjmax, int grid, const PairArgs *tab,
                                 const int4 *items, int nitems, unsigned *counter, cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    switch (mode) {
        case MODE_NEWTON: return launch_ens_two_mode<MODE_NEWTON>(ipt, tjmax, grid, tab, items, nitems, counter, s);
        case MODE_FORCE: return launch_ens_two_mode<MODE_FORCE>(ipt, tjmax, grid, tab, items, nitems, counter, s);
        case MODE_ENERGY: return launch_ens_two_mode<MODE_ENERGY>(ipt, tjmax, grid, tab, items, nitems, counter, s);
        default: return cudaErrorInvalidValue;
    }
}

cudaError_t launch_pair_ens_f32(int mode, int ipt, int js, int tjmax, int grid, const PairArgs *tab,
                                 const int4 *items, int nitems, unsigned *counter, cudaStream_t s) {
    if (nitems <= 0) return cudaSuccess;
    switch (mode) {
        case MODE_NEWTON: return launch_ens_mode<MODE_NEWTON>(ipt, js, tjmax, grid, tab, items, nitems, counter, s);
        case MODE_FORCE: return launch_ens_mode<MODE_FORCE>(ipt, js, tjmax, grid, tab, items, nitems, counter, s);
        case MODE_ENERGY: return launch_ens_mode<MODE_ENERGY>(ipt, js, tjmax, grid, tab, items, nitems, counter, s);
        default: return cudaErrorInvalidValue;
    }
}

}  // namespace pn
