// pn_internal.h -- host-side declarations shared by libpn's translation units.
#pragma once

#include <cuda_runtime.h>

#include "pn_pair.cuh"

namespace pn {

struct PairCfg {
    int ipt = 2;     // i-particles per thread
    int js = 1;      // lanes sharing one i-set
    int tj = 128;    // stars per j-tile
    int gsplit = 1;  // j-range splits across CTAs
    int x2 = 0;      // FP32 only: the packed f32x2 sweep (pn_pair2.cuh; js = 1, ipt 1 or 2);
                     // 2 / 3 = the same sized for 3 / 4 CTAs per SM (ipt 2, force sweeps)
};

// Launches k_pair for the given precision/mode/shape (returns cudaErrorInvalidValue for an
// unsupported (ipt, js) combination).  Implemented in pn_pair_f32.cu / pn_pair_f64.cu.
cudaError_t launch_pair_f32(int mode, const PairCfg &c, const PairArgs &a, cudaStream_t s);
cudaError_t launch_pair_f64(int mode, const PairCfg &c, const PairArgs &a, cudaStream_t s);
bool pair_shape_supported(int ipt, int js);

// Persistent ensemble sweep (k_pair_ens): (ipt, js) in {(1,1), (2,1), (1,4)}; tjmax = the
// largest tile size among the clusters; grid <= 0 = one wave of resident CTAs.
cudaError_t launch_pair_ens_f32(int mode, int ipt, int js, int tjmax, int grid, const PairArgs *tab,
                                const int4 *items, int nitems, unsigned *counter, cudaStream_t s);
cudaError_t launch_pair_ens_f64(int mode, int ipt, int js, int tjmax, int grid, const PairArgs *tab,
                                const int4 *items, int nitems, unsigned *counter, cudaStream_t s);
// the packed FP32x2 form of the ensemble sweep (tab[c].pack2 / ipack set; js = 1, ipt 1 or 2)
cudaError_t launch_pair2_ens_f32(int mode, int ipt, int tjmax, int grid, const PairArgs *tab,
                                 const int4 *items, int nitems, unsigned *counter, cudaStream_t s);
inline bool ens_shape_supported(int ipt, int js) {
    return (js == 1 && (ipt == 1 || ipt == 2)) || (ipt == 1 && js == 4);
}

inline int pair_ng(bool f32, int mode) {
    if (f32) return mode == MODE_NEWTON ? ModeInfo<MODE_NEWTON>::NG32
                  : mode_has_force(mode) ? ModeInfo<MODE_FORCE>::NG32
                                         : ModeInfo<MODE_ENERGY>::NG32;
    return mode == MODE_NEWTON ? ModeInfo<MODE_NEWTON>::NG64
         : mode_has_force(mode) ? ModeInfo<MODE_FORCE>::NG64
                                : ModeInfo<MODE_ENERGY>::NG64;
}

inline int pair_nacc(int mode) {
    return mode == MODE_NEWTON ? ModeInfo<MODE_NEWTON>::NACC
         : mode == MODE_FORCE  ? ModeInfo<MODE_FORCE>::NACC
         : mode == MODE_FORCE_ENERGY ? ModeInfo<MODE_FORCE_ENERGY>::NACC
                               : ModeInfo<MODE_ENERGY>::NACC;
}

inline int pair_block_i(const PairCfg &c) { return PAIR_NT * c.ipt / c.js; }

}  // namespace pn
