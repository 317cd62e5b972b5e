// pn_kernels.h -- argument blocks and launchers of libpn's O(N) kernels.
#pragma once

#include "pn_internal.h"

namespace pn {

// Stage codes of the optional classic fourth-order Runge-Kutta integrator (the reference's own
// scheme, Limit-sticky9.c:844-893, uses stages 1..3).
enum RK4Stage : int { STAGE_RK4_1 = 11, STAGE_RK4_2 = 12, STAGE_RK4_3 = 13, STAGE_RK4_4 = 14 };

// Global per-evaluation sums (FP64) written by k_prep.
enum GlobSlot : int { G_A1 = 0, G_B3X, G_B3Y, G_B3Z, G_C, G_PX, G_PY, G_PZ, NGLOB };
constexpr int NACC_MAX = 9;

// Device state of one system, SoA [3][ld] doubles each (index 0 = BH).
struct DevState {
    double *x, *v;    // step-start state (the reference's x, v; hx[0], hv[0])
    double *xs, *vs;  // stage state (the reference's x1, v1)
    double *hx, *hv;  // hx[1] + hx[2] (and hv), accumulated in the reference's order
    double *m;        // [ld]
    long long ld;     // leading dimension
};

struct PrepArgs {
    const double *x, *v, *m;  // particle p, component k at [p*sp + k*sk]
    long long sp, sk;
    int nstar, npad, tj;  // npad: row stride of pack/spos
    int nfill;            // entries written: round_up(nstar, 256) <= npad
    int f32;
    double eps2;
    void *pack;
    TileOrigin *torg;
    double *spos;
    double *part, *glob;
    unsigned *ticket;
    float4 *pack2;  // optional (FP32): paired pack [7][npad/2] of the f32x2 sweep
    float4 *ipack;  // optional (FP32): [npad] (v.xyz, qe)
};

struct FinishArgs {
    const double *v, *m;  // evaluation-state velocities (strided as in PrepArgs) and masses
    long long vsp, vsk;
    const double *spos, *acc, *glob;
    int nstar, npad, nacc, gsplit;
    int pn1;              // 1PN terms on (pair sweep in MODE_FORCE)
    double eps, eps2, inv_c2, dt;
    double *a;            // output acceleration (may be null), [p*asp + k*ask]
    long long asp, ask;
    int stage;            // 0: none; 1..3: the reference's stages; STAGE_RK4_1..4: classic RK4
    double *sums_out;     // optional [nacc][npad]: the per-star pair sums (adjoint reuse)
    DevState st;
    long long ld;
    double *part;
    unsigned *ticket;
    int *err;
};

struct EnergyArgs {
    const double *v, *m;
    long long sp, sk;
    const double *spos, *acc, *glob;
    int nstar, npad, gsplit;
    int nacc, sphi, spsi;  // pair-sum layout: slots per split and the Phi, Psi slots
    double eps, eps2, inv_c2;
    double *part, *out;  // out[4] = pot_n, kin_n, pot_pn, total
    unsigned *ticket;
};

cudaError_t launch_prep(const PrepArgs &a, cudaStream_t s);
cudaError_t launch_finish(const FinishArgs &a, cudaStream_t s);
cudaError_t launch_energy_finish(const EnergyArgs &a, cudaStream_t s);
// Ensemble forms: one launch over every cluster's blocks (blockmap[b] = cluster, block within
// the cluster, the cluster's block count, 0), per-cluster arguments from device tables.
cudaError_t launch_prep_ens(const PrepArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s);
cudaError_t launch_finish_ens(const FinishArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s);
cudaError_t launch_energy_ens(const EnergyArgs *tab, const int4 *blockmap, int nblocks, cudaStream_t s);

}  // namespace pn
