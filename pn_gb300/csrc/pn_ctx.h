// pn_ctx.h -- the device-resident context (private to libpn) and the helpers its
// translation units share.
#pragma once

#include "../../include/pn.h"
#include "pn_kernels.h"

struct AdjointWork;  // pn_adjoint.cu

struct pn_ctx {
    int dev = 0;
    int sms = 0;       // SM count of dev (launch-shape heuristics)
    int nmax = 0, n = 0;
    int npad = 0;      // padded star capacity (multiple of 256)
    long long ld = 0;  // state leading dimension
    pn_params p{};

    cudaStream_t stream = nullptr;
    pn::DevState st{};
    double *state_buf = nullptr;  // backing store of st
    double *a_aos = nullptr;      // [ld][3] device acceleration (AoS), for pn_force / drop-ins
    double *in_aos = nullptr;     // [2][ld][3] + [ld] device AoS x, v, m staging (drop-ins)
    double *spos = nullptr;
    void *pack = nullptr;
    float4 *pack2 = nullptr;      // paired pack of the f32x2 sweep [7][npad/2]
    float4 *ipack = nullptr;      // [npad] (v.xyz, qe)
    pn::TileOrigin *torg = nullptr;
    double *acc = nullptr;
    int acc_splits = 0;
    double *part = nullptr;  // partial sums (prep / finish / energy share one buffer region each)
    double *glob = nullptr;  // [NGLOB]
    double *eout = nullptr;  // [4]
    unsigned *tickets = nullptr;  // [4]
    int *err = nullptr;
    double *h_eout = nullptr;     // pinned
    int *h_err = nullptr;         // pinned
    double time = 0.0;
    bool have_state = false;
    cudaGraphExec_t step_exec = nullptr;
    bool step_valid = false;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr, ev2 = nullptr;
    cudaEvent_t evp[8] = {};      // around the pair launches of a captured step (3, or 4 for RK4)
    void *flush = nullptr;        // L2 flush buffer (benchmarks only)
    size_t flush_bytes = 0;
    pn_stats stats{};
    pn::PairCfg cfg_force{}, cfg_energy{};
    bool cfg_set = false;
    AdjointWork *adj = nullptr;  // buffers of the adjoint (created on first use)
    // asynchronous snapshots (created on first use): device copy of x, v, its pinned host image,
    // the copy stream and the events ordering them against the context's stream
    double *snap_dev = nullptr, *snap_host = nullptr;
    cudaStream_t snap_stream = nullptr;
    cudaEvent_t snap_taken = nullptr, snap_done = nullptr;
    bool snap_pending = false;
    int snap_n = 0;
};

namespace pn {
int set_err(int code, const char *fmt, ...);
long long round_up(long long a, long long b);
bool is_f32(const pn_ctx *c);
int force_mode(const pn_ctx *c);
void refresh_cfg(pn_ctx *c);
int ensure_acc(pn_ctx *c, int splits);
int check_device_err(pn_ctx *c);
// One force evaluation; see pn_api.cu.  sums_out (optional) receives the per-star pair sums.
int eval_force(pn_ctx *c, const double *x, const double *v, const double *m, long long sp,
               long long sk, double *a_out, long long asp, long long ask, int stage,
               cudaStream_t s, bool timed, int tslot = -1, double *sums_out = nullptr,
               bool with_energy = false);
void free_adjoint(pn_ctx *c);
}  // namespace pn

#define CU(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess)                                                               \
            return pn::set_err(PN_ERR_CUDA, "%s: %s (%s:%d)", #call, cudaGetErrorString(e_), \
                               __FILE__, __LINE__);                                          \
    } while (0)
