// pn_api.cu -- libpn host runtime and C ABI (include/pn.h).
//
// A pn_ctx owns the device-resident state of one system and the work buffers of its force
// evaluations.  One force evaluation is three kernels on the context's stream:
//   k_prep   (O(N): per-star quantities, j-pack, global sums)
//   k_pair   (O(N^2): the TMA-streamed pair sweep, FP64 or mixed)
//   k_finish (O(N): accelerations of stars and BH, optionally fused with an integration stage)
// An integration step (Limit-sticky9.c:844-893) is three evaluations whose k_finish performs
// stage 1, 2 and 3 (the last one also the state-averaging combine); it is captured once in a
// CUDA graph and replayed.
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <mutex>
#include <vector>

#include "pn_ctx.h"
#include "pn_tune.h"

using namespace pn;

// ------------------------------------------------------------------ errors
static thread_local int g_last_error = PN_OK;
static thread_local char g_last_msg[256] = "";

int pn::set_err(int code, const char *fmt, ...) {
    g_last_error = code;
    if (fmt) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(g_last_msg, sizeof g_last_msg, fmt, ap);
        va_end(ap);
    }
    return code;
}


extern "C" const char *pn_strerror(int s) {
    switch (s) {
        case PN_OK: return "ok";
        case PN_ERR_INVALID: return "invalid argument";
        case PN_ERR_CUDA: return "CUDA error";
        case PN_ERR_NOMEM: return "out of memory";
        case PN_ERR_NONFINITE: return "non-finite force or energy";
        case PN_ERR_IO: return "I/O error";
        case PN_ERR_TIMEOUT: return "bounded in-kernel wait timed out";
        case PN_ERR_UNSUPPORTED: return "unsupported configuration or no GPU";
        case PN_ERR_STATE: return "call out of order";
        default: return "unknown status";
    }
}

extern "C" int pn_last_error(void) { return g_last_error; }
extern "C" const char *pn_last_error_message(void) { return g_last_msg; }

extern "C" int pn_device_count(void) {
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess) {
        cudaGetLastError();
        return 0;
    }
    return n;
}

extern "C" const char *pn_version(void) { return "pn-gb300 0.1 (sm_103a)"; }

// ------------------------------------------------------------------ context
// struct pn_ctx: pn_ctx.h


long long pn::round_up(long long a, long long b) { return (a + b - 1) / b * b; }

extern "C" void pn_params_default(pn_params *p) {
    if (!p) return;
    std::memset(p, 0, sizeof *p);
    p->eps = 0.001;               // Limit-sticky9.c:770
    p->dt = 1.0 / 131072.0;       // Limit-sticky9.c:771
    p->inv_c2 = 1.0;              // the reference's implicit c = 1
    p->precision = PN_PREC_FP64;
}

bool pn::is_f32(const pn_ctx *c) { return c->p.precision == PN_PREC_MIXED; }
int pn::force_mode(const pn_ctx *c) { return c->p.inv_c2 != 0.0 ? MODE_FORCE : MODE_NEWTON; }

// Launch shape of the pair sweep: explicit parameters win; otherwise a heuristic sized for
// GB300 (152 SMs): enough CTAs for several waves, split along j when there are few i-blocks.
static PairCfg choose_cfg(const pn_ctx *c, int mode, int nstar) {
    PairCfg k;
    const bool f32 = is_f32(c);
    // defaults from a shape sweep on GB300 (N = 2k..256k); pn_autotune refines them
    if (f32) {
        k.ipt = (mode == MODE_NEWTON || nstar >= 131072) ? 4 : (nstar >= 4096 ? 2 : 1);
        k.tj = nstar >= 4096 ? 256 : 128;
        k.js = 1;
    } else {
        k.ipt = 1;
        k.tj = 128;
        k.js = nstar >= 32768 ? 4 : 2;
    }
    if (c->p.i_per_thread > 0) k.ipt = c->p.i_per_thread;
    if (c->p.j_split > 0) k.js = c->p.j_split;
    if (c->p.tile_j > 0) k.tj = c->p.tile_j;
    if (!pair_shape_supported(k.ipt, k.js)) { k.ipt = 1; k.js = 1; }
    const bool explicit_shape = c->p.i_per_thread > 0 || c->p.j_split > 0 || c->p.tile_j > 0 ||
                                c->p.grid_split > 0;
    // the packed f32x2 sweep: JS = 1 and 1 or 2 i per thread; explicit choice or tuned
    const bool x2_ok = f32 && k.js == 1 && k.ipt <= 2;
    const int pv = c->p.pair_variant;
    PairCfg tuned;
    if (!explicit_shape && pv == PN_PAIR_AUTO && nstar > 0 &&
        tune_lookup(c->p.precision, mode, nstar, &tuned)) {
        const int ntiles_t = (nstar + tuned.tj - 1) / tuned.tj;
        if (tuned.gsplit > ntiles_t) tuned.gsplit = ntiles_t;
        return tuned;
    }
    if ((pv == PN_PAIR_F32X2 || pv == PN_PAIR_F32X2_OCC3 || pv == PN_PAIR_F32X2_OCC4) && f32) {
        if (k.ipt > 2) k.ipt = 2;
        if (k.js != 1) k.js = 1;
        const bool occ = k.ipt == 2 && mode_has_force(mode);
        k.x2 = (occ && pv == PN_PAIR_F32X2_OCC3) ? 2 : (occ && pv == PN_PAIR_F32X2_OCC4) ? 3 : 1;
    } else if (pv == PN_PAIR_AUTO && f32 && !explicit_shape) {
        // untuned default of the mixed sweep: the packed f32x2 form, 2 i per thread for
        // N >= 4096 (fastest in the tuner's measurements at N = 2^18: 111 ms vs 125 ms)
        k.ipt = nstar >= 4096 ? 2 : 1;
        k.js = 1;
        k.x2 = 1;
    } else {
        k.x2 = 0;  // scalar sweep: FP64, PN_PAIR_SCALAR, or an explicit shape without the variant
    }
    (void)x2_ok;
    const int bi = pair_block_i(k);
    const int nib = (nstar + bi - 1) / bi;
    const int ntiles = (nstar + k.tj - 1) / k.tj;
    // j-splits for about 8 waves of 4 CTAs per SM, keeping >= 4 tiles per split
    int g = c->p.grid_split > 0 ? c->p.grid_split : (8 * c->sms * 4 + nib - 1) / (nib > 0 ? nib : 1);
    if (c->p.grid_split <= 0) {
        if (g > (nstar >= 65536 ? 8 : 32)) g = nstar >= 65536 ? 8 : 32;
        if (g > ntiles / 4) g = ntiles / 4;
    }
    if (g > ntiles) g = ntiles;
    if (g < 1) g = 1;
    k.gsplit = g;
    return k;
}

bool pn::pair_shape_supported(int ipt, int js) {
    if (js == 1) return ipt == 1 || ipt == 2 || ipt == 4;
    return ipt == 1 && (js == 2 || js == 4 || js == 8);
}

int pn::ensure_acc(pn_ctx *c, int splits) {
    if (splits <= c->acc_splits) return PN_OK;
    if (c->acc) cudaFree(c->acc);
    c->acc = nullptr;
    c->acc_splits = 0;
    // room for the widest sweep: the force sweep with the fused energy sum
    size_t bytes = (size_t)splits * pair_nacc(MODE_FORCE_ENERGY) * (size_t)c->npad * sizeof(double);
    if (cudaMalloc(&c->acc, bytes) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PN_ERR_NOMEM, "acc: %zu bytes", bytes);
    }
    c->acc_splits = splits;
    return PN_OK;
}

static void free_ctx(pn_ctx *c) {
    if (!c) return;
    free_adjoint(c);
    if (c->step_exec) cudaGraphExecDestroy(c->step_exec);
    void *bufs[] = {c->state_buf, c->a_aos, c->in_aos, c->spos, c->pack, c->pack2, c->ipack, c->torg, c->acc,
                    c->part, c->glob, c->eout, c->tickets, c->err};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (c->h_eout) cudaFreeHost(c->h_eout);
    if (c->h_err) cudaFreeHost(c->h_err);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev2) cudaEventDestroy(c->ev2);
    for (cudaEvent_t e : c->evp)
        if (e) cudaEventDestroy(e);
    if (c->flush) cudaFree(c->flush);
    if (c->snap_stream) cudaStreamSynchronize(c->snap_stream);
    if (c->snap_dev) cudaFree(c->snap_dev);
    if (c->snap_host) cudaFreeHost(c->snap_host);
    if (c->snap_taken) cudaEventDestroy(c->snap_taken);
    if (c->snap_done) cudaEventDestroy(c->snap_done);
    if (c->snap_stream) cudaStreamDestroy(c->snap_stream);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

static int validate_params(const pn_params *p) {
    if (!p) return PN_ERR_INVALID;
    if (!(p->eps > 0.0) || !(p->dt == p->dt) || !(p->inv_c2 >= 0.0)) return PN_ERR_INVALID;
    if (p->precision != PN_PREC_FP64 && p->precision != PN_PREC_MIXED) return PN_ERR_INVALID;
    if (p->tile_j && p->tile_j != 32 && p->tile_j != 64 && p->tile_j != 128 && p->tile_j != 256)
        return PN_ERR_INVALID;
    if (p->i_per_thread < 0 || p->j_split < 0 || p->grid_split < 0 || p->grid_split > 64)
        return PN_ERR_INVALID;
    if (p->pair_variant < PN_PAIR_AUTO || p->pair_variant > PN_PAIR_F32X2_OCC4) return PN_ERR_INVALID;
    if (p->integrator != PN_INT_REFERENCE && p->integrator != PN_INT_RK4) return PN_ERR_INVALID;
    if ((p->i_per_thread || p->j_split) &&
        !pair_shape_supported(p->i_per_thread ? p->i_per_thread : 1, p->j_split ? p->j_split : 1))
        return PN_ERR_INVALID;
    return PN_OK;
}

extern "C" int pn_create(pn_ctx **out, int nmax, const pn_params *p) {
    if (!out || nmax < 1) return set_err(PN_ERR_INVALID, "pn_create: nmax=%d", nmax);
    *out = nullptr;
    pn_params pp;
    if (p) pp = *p; else pn_params_default(&pp);
    if (validate_params(&pp) != PN_OK) return set_err(PN_ERR_INVALID, "pn_create: bad params");
    if (pn_device_count() < 1) return set_err(PN_ERR_UNSUPPORTED, "no CUDA device");
    pn_ctx *c = new pn_ctx();
    c->p = pp;
    c->nmax = nmax;
    c->npad = (int)round_up(nmax > 1 ? nmax - 1 : 1, 256);
    c->ld = round_up(nmax, 256);
    cudaGetDevice(&c->dev);
    if (cudaDeviceGetAttribute(&c->sms, cudaDevAttrMultiProcessorCount, c->dev) != cudaSuccess || c->sms < 1) {
        cudaGetLastError();
        const int dev = c->dev;
        delete c;
        return set_err(PN_ERR_CUDA, "pn_create: SM count of device %d", dev);
    }
    auto fail = [&](const char *what) {
        cudaGetLastError();
        free_ctx(c);
        return set_err(PN_ERR_NOMEM, "pn_create: %s", what);
    };
    if (cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking) != cudaSuccess) return fail("stream");
    const size_t ld = (size_t)c->ld, np = (size_t)c->npad;
    if (cudaMalloc(&c->state_buf, (6 * 3 * ld + ld) * sizeof(double)) != cudaSuccess) return fail("state");
    double *b = c->state_buf;
    c->st.x = b; c->st.v = b + 3 * ld; c->st.xs = b + 6 * ld; c->st.vs = b + 9 * ld;
    c->st.hx = b + 12 * ld; c->st.hv = b + 15 * ld; c->st.m = b + 18 * ld; c->st.ld = c->ld;
    if (cudaMalloc(&c->a_aos, 3 * ld * sizeof(double)) != cudaSuccess) return fail("a");
    if (cudaMalloc(&c->in_aos, 7 * ld * sizeof(double)) != cudaSuccess) return fail("in");
    if (cudaMalloc(&c->spos, 3 * np * sizeof(double)) != cudaSuccess) return fail("spos");
    if (cudaMalloc(&c->pack, 6 * np * 16) != cudaSuccess) return fail("pack");
    if (cudaMalloc(&c->pack2, 7 * (np / 2) * 16) != cudaSuccess) return fail("pack2");
    if (cudaMalloc(&c->ipack, np * 16) != cudaSuccess) return fail("ipack");
    if (cudaMemset(c->pack2, 0, 7 * (np / 2) * 16) != cudaSuccess) return fail("memset");
    if (cudaMalloc(&c->torg, (np / 32 + 1) * sizeof(TileOrigin)) != cudaSuccess) return fail("torg");
    const size_t nblk = np / 256 + 2;
    if (cudaMalloc(&c->part, nblk * 8 * 2 * sizeof(double)) != cudaSuccess) return fail("part");
    if (cudaMalloc(&c->glob, 16 * sizeof(double)) != cudaSuccess) return fail("glob");
    if (cudaMalloc(&c->eout, 4 * sizeof(double)) != cudaSuccess) return fail("eout");
    if (cudaMalloc(&c->tickets, 4 * sizeof(unsigned)) != cudaSuccess) return fail("tickets");
    if (cudaMalloc(&c->err, sizeof(int)) != cudaSuccess) return fail("err");
    if (cudaMallocHost(&c->h_eout, 4 * sizeof(double)) != cudaSuccess) return fail("h_eout");
    if (cudaMallocHost(&c->h_err, sizeof(int)) != cudaSuccess) return fail("h_err");
    if (cudaMemset(c->state_buf, 0, (6 * 3 * ld + ld) * sizeof(double)) != cudaSuccess) return fail("memset");
    if (cudaMemset(c->pack, 0, 6 * np * 16) != cudaSuccess) return fail("memset");
    if (cudaMemset(c->tickets, 0, 4 * sizeof(unsigned)) != cudaSuccess) return fail("memset");
    if (cudaMemset(c->err, 0, sizeof(int)) != cudaSuccess) return fail("memset");
    if (cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess ||
        cudaEventCreate(&c->ev2) != cudaSuccess)
        return fail("events");
    for (cudaEvent_t &e : c->evp)
        if (cudaEventCreate(&e) != cudaSuccess) return fail("events");
    if (cudaDeviceSynchronize() != cudaSuccess) return fail("sync");
    *out = c;
    return set_err(PN_OK, nullptr);
}

extern "C" int pn_destroy(pn_ctx *c) {
    if (!c) return PN_ERR_INVALID;
    cudaStreamSynchronize(c->stream);
    free_ctx(c);
    return PN_OK;
}

extern "C" int pn_set_params(pn_ctx *c, const pn_params *p) {
    if (!c || validate_params(p) != PN_OK) return set_err(PN_ERR_INVALID, "pn_set_params");
    c->p = *p;
    c->cfg_set = false;
    c->step_valid = false;
    return PN_OK;
}

void pn::refresh_cfg(pn_ctx *c) {
    if (c->cfg_set) return;
    const int nstar = c->n - 1;
    c->cfg_force = choose_cfg(c, force_mode(c), nstar);
    c->cfg_energy = choose_cfg(c, MODE_ENERGY, nstar);
    c->cfg_set = true;
}

// One force evaluation.  x, v, m: particle p component k at [p*sp + k*sk] (device).
// a_out: optional device output (AoS when asp=3, ask=1).  stage: fused integration stage.
// with_energy: the same sweep also accumulates the energy's Psi, and the energies of the state
// (x, v) are written to c->eout (the sweep's Phi is the energy's Phi).
int pn::eval_force(pn_ctx *c, const double *x, const double *v, const double *m, long long sp,
                   long long sk, double *a_out, long long asp, long long ask, int stage,
                   cudaStream_t s, bool timed, int tslot, double *sums_out, bool with_energy) {
    const int n = c->n;
    const int nstar = n - 1;
    refresh_cfg(c);
    const int mode = with_energy ? (int)MODE_FORCE_ENERGY : force_mode(c);
    const PairCfg &k = c->cfg_force;
    int rc = ensure_acc(c, k.gsplit);
    if (rc) return rc;
    const double eps2 = c->p.eps * c->p.eps;

    PrepArgs pa{};
    pa.x = x; pa.v = v; pa.m = m; pa.sp = sp; pa.sk = sk;
    pa.nstar = nstar; pa.npad = c->npad; pa.nfill = (int)round_up(nstar > 0 ? nstar : 1, 256);
    pa.tj = k.tj; pa.f32 = is_f32(c); pa.eps2 = eps2;
    pa.pack = c->pack; pa.torg = c->torg; pa.spos = c->spos;
    if (pa.f32) {
        pa.pack2 = c->pack2;
        pa.ipack = c->ipack;
        if (k.x2) pa.pack = nullptr;  // the packed sweep reads the paired pack only
    }
    pa.part = c->part; pa.glob = c->glob; pa.ticket = &c->tickets[0];
    CU(launch_prep(pa, s));

    PairArgs qa{};
    qa.pack = c->pack; qa.torg = c->torg; qa.spos = c->spos; qa.pack2 = c->pack2; qa.ipack = c->ipack; qa.out = c->acc; qa.err = c->err;
    qa.nstar = nstar; qa.npad = c->npad; qa.tj = k.tj; qa.ntiles = (nstar + k.tj - 1) / k.tj;
    qa.gsplit = k.gsplit; qa.eps2 = eps2;
    if (timed) CU(cudaEventRecord(c->ev0, s));
    // external event nodes, so that the events are really recorded when a captured step replays
    // (the flag is valid only while the stream is being captured)
    if (tslot >= 0) {
        cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
        CU(cudaStreamIsCapturing(s, &cs));
        if (cs != cudaStreamCaptureStatusActive) tslot = -1;
    }
    if (tslot >= 0) CU(cudaEventRecordWithFlags(c->evp[2 * tslot], s, cudaEventRecordExternal));
    if (nstar > 0) {
        if (is_f32(c)) CU(launch_pair_f32(mode, k, qa, s));
        else CU(launch_pair_f64(mode, k, qa, s));
    }
    if (tslot >= 0) CU(cudaEventRecordWithFlags(c->evp[2 * tslot + 1], s, cudaEventRecordExternal));
    if (timed) CU(cudaEventRecord(c->ev1, s));
    if (with_energy) {
        EnergyArgs ea{};
        ea.v = v; ea.m = m; ea.sp = sp; ea.sk = sk;
        ea.spos = c->spos; ea.acc = c->acc; ea.glob = c->glob;
        ea.nstar = nstar; ea.npad = c->npad; ea.gsplit = k.gsplit;
        ea.nacc = pair_nacc(mode); ea.sphi = A_PHI; ea.spsi = A_PSI;
        ea.eps = c->p.eps; ea.eps2 = eps2; ea.inv_c2 = c->p.inv_c2;
        ea.part = c->part + (size_t)(c->npad / 256 + 2) * 8;
        ea.out = c->eout; ea.ticket = &c->tickets[2];
        CU(launch_energy_finish(ea, s));
    }

    FinishArgs fa{};
    fa.v = v; fa.m = m; fa.vsp = sp; fa.vsk = sk;
    fa.spos = c->spos; fa.acc = c->acc; fa.glob = c->glob;
    fa.nstar = nstar; fa.npad = c->npad; fa.nacc = pair_nacc(mode); fa.gsplit = k.gsplit;
    fa.pn1 = mode_has_force(mode) && c->p.inv_c2 != 0.0;
    fa.eps = c->p.eps; fa.eps2 = eps2; fa.inv_c2 = c->p.inv_c2; fa.dt = c->p.dt;
    fa.a = a_out; fa.asp = asp; fa.ask = ask;
    fa.stage = stage; fa.st = c->st; fa.ld = c->ld; fa.sums_out = sums_out;
    fa.part = c->part + (size_t)(c->npad / 256 + 2) * 8;
    fa.ticket = &c->tickets[1]; fa.err = c->err;
    CU(launch_finish(fa, s));
    if (timed) CU(cudaEventRecord(c->ev2, s));
    c->stats.tile_j = k.tj; c->stats.i_per_thread = k.ipt; c->stats.j_split = k.js;
    c->stats.grid_split = k.gsplit; c->stats.threads = PAIR_NT;
    c->stats.pair_variant = k.x2 == 3   ? PN_PAIR_F32X2_OCC4
                            : k.x2 == 2 ? PN_PAIR_F32X2_OCC3
                            : k.x2      ? PN_PAIR_F32X2
                                        : PN_PAIR_SCALAR;
    c->stats.interactions = (double)nstar * (double)nstar;
    return PN_OK;
}

int pn::check_device_err(pn_ctx *c) {
    CU(cudaMemcpyAsync(c->h_err, c->err, sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    CU(cudaStreamSynchronize(c->stream));
    int e = *c->h_err;
    if (e) {
        CU(cudaMemsetAsync(c->err, 0, sizeof(int), c->stream));
        CU(cudaStreamSynchronize(c->stream));
        if (e & DEVERR_TIMEOUT) return set_err(PN_ERR_TIMEOUT, "in-kernel wait timed out");
        return set_err(PN_ERR_NONFINITE, "non-finite acceleration");
    }
    return set_err(PN_OK, nullptr);
}

extern "C" int pn_set_state(pn_ctx *c, int n, const double *x, const double *v, const double *m) {
    if (!c || n < 1 || n > c->nmax || !x || !v || !m)
        return set_err(PN_ERR_INVALID, "pn_set_state: n=%d nmax=%d", n, c ? c->nmax : 0);
    if (!(m[0] > 0.0)) return set_err(PN_ERR_INVALID, "pn_set_state: BH mass must be > 0");
    // host AoS -> device AoS staging -> SoA state (transpose on the host: O(N), once)
    const size_t ld = (size_t)c->ld;
    double *h = nullptr;
    if (cudaMallocHost(&h, (6 * ld + ld) * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PN_ERR_NOMEM, "pinned staging");
    }
    std::memset(h, 0, (6 * ld + ld) * sizeof(double));
    for (int p = 0; p < n; ++p)
        for (int k = 0; k < 3; ++k) {
            h[k * ld + p] = x[3 * p + k];
            h[3 * ld + k * ld + p] = v[3 * p + k];
        }
    for (int p = 0; p < n; ++p) h[6 * ld + p] = m[p];
    cudaError_t e1 = cudaMemcpyAsync(c->st.x, h, 3 * ld * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    cudaError_t e2 = cudaMemcpyAsync(c->st.v, h + 3 * ld, 3 * ld * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    cudaError_t e3 = cudaMemcpyAsync(c->st.m, h + 6 * ld, ld * sizeof(double), cudaMemcpyHostToDevice, c->stream);
    cudaError_t e4 = cudaStreamSynchronize(c->stream);
    cudaFreeHost(h);
    if (e1 || e2 || e3 || e4) return set_err(PN_ERR_CUDA, "pn_set_state: copy failed");
    if (n != c->n) { c->cfg_set = false; c->step_valid = false; }
    c->n = n;
    c->time = 0.0;
    c->have_state = true;
    return set_err(PN_OK, nullptr);
}

extern "C" int pn_get_state(pn_ctx *c, double *x, double *v) {
    if (!c || !c->have_state || (!x && !v)) return set_err(PN_ERR_STATE, "pn_get_state");
    const size_t ld = (size_t)c->ld;
    double *h = nullptr;
    if (cudaMallocHost(&h, 6 * ld * sizeof(double)) != cudaSuccess) {
        cudaGetLastError();
        return set_err(PN_ERR_NOMEM, "pinned staging");
    }
    cudaError_t e1 = cudaMemcpyAsync(h, c->st.x, 6 * ld * sizeof(double), cudaMemcpyDeviceToHost, c->stream);
    cudaError_t e2 = cudaStreamSynchronize(c->stream);
    if (!e1 && !e2)
        for (int p = 0; p < c->n; ++p)
            for (int k = 0; k < 3; ++k) {
                if (x) x[3 * p + k] = h[k * ld + p];
                if (v) v[3 * p + k] = h[3 * ld + k * ld + p];
            }
    cudaFreeHost(h);
    if (e1 || e2) return set_err(PN_ERR_CUDA, "pn_get_state: copy failed");
    return set_err(PN_OK, nullptr);
}

extern "C" int pn_force(pn_ctx *c, double *a) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_force: no state");
    if (!a) return set_err(PN_ERR_INVALID, "pn_force: a");
    int rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, c->ld, c->a_aos, 3, 1, 0, c->stream, true);
    if (rc) return rc;
    CU(cudaMemcpyAsync(a, c->a_aos, 3 * (size_t)c->n * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    rc = check_device_err(c);
    if (rc) return rc;
    float ms = 0.f;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev1) == cudaSuccess) c->stats.pair_ms = ms;
    if (cudaEventElapsedTime(&ms, c->ev0, c->ev2) == cudaSuccess) c->stats.total_ms = ms;
    return PN_OK;
}

extern "C" int pn_force_device(pn_ctx *c, int n, const double *d_x, const double *d_v,
                               const double *d_m, double *d_a, void *stream) {
    if (!c || n < 1 || n > c->nmax || !d_x || !d_v || !d_m || !d_a)
        return set_err(PN_ERR_INVALID, "pn_force_device");
    cudaStream_t s = stream ? (cudaStream_t)stream : c->stream;
    if (n != c->n) { c->cfg_set = false; c->step_valid = false; }
    c->n = n;
    return eval_force(c, d_x, d_v, d_m, 3, 1, d_a, 3, 1, 0, s, false);
}

// Enqueue one integration step (three evaluations with fused stage updates).
static int step_evaluations(const pn_ctx *c) { return c->p.integrator == PN_INT_RK4 ? 4 : 3; }

// energy_first: the first evaluation (at the step's starting state) also yields the energies of
// that state in c->eout.
static int enqueue_step(pn_ctx *c, cudaStream_t s, bool energy_first = false) {
    const long long ld = c->ld;
    if (c->p.integrator == PN_INT_RK4) {  // classic RK4: evaluations at y, y2, y3, y4
        int rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, ld, nullptr, 3, 1, STAGE_RK4_1, s, false, 0,
                            nullptr, energy_first);
        for (int k = 1; k < 4 && !rc; ++k)
            rc = eval_force(c, c->st.xs, c->st.vs, c->st.m, 1, ld, nullptr, 3, 1, STAGE_RK4_1 + k, s, false, k);
        return rc;
    }
    int rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, ld, nullptr, 3, 1, 1, s, false, 0, nullptr,
                        energy_first);
    if (!rc) rc = eval_force(c, c->st.xs, c->st.vs, c->st.m, 1, ld, nullptr, 3, 1, 2, s, false, 1);
    if (!rc) rc = eval_force(c, c->st.xs, c->st.vs, c->st.m, 1, ld, nullptr, 3, 1, 3, s, false, 2);
    return rc;
}

static int build_step_graph(pn_ctx *c) {
    if (c->step_valid) return PN_OK;
    if (c->step_exec) { cudaGraphExecDestroy(c->step_exec); c->step_exec = nullptr; }
    refresh_cfg(c);
    int rc = ensure_acc(c, c->cfg_force.gsplit);  // allocate before capture
    if (rc) return rc;
    cudaGraph_t g = nullptr;
    CU(cudaStreamBeginCapture(c->stream, cudaStreamCaptureModeThreadLocal));
    rc = enqueue_step(c, c->stream);
    cudaError_t ec = cudaStreamEndCapture(c->stream, &g);
    if (rc) { if (g) cudaGraphDestroy(g); return rc; }
    if (ec != cudaSuccess) return set_err(PN_ERR_CUDA, "graph capture: %s", cudaGetErrorString(ec));
    cudaError_t ei = cudaGraphInstantiate(&c->step_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return set_err(PN_ERR_CUDA, "graph instantiate: %s", cudaGetErrorString(ei));
    c->step_valid = true;
    return PN_OK;
}

extern "C" int pn_steps(pn_ctx *c, int nsteps) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_steps: no state");
    if (nsteps < 0) return set_err(PN_ERR_INVALID, "pn_steps: nsteps");
    static const bool no_graph = getenv("PN_NO_GRAPH") != nullptr;
    if (no_graph) {
        for (int s = 0; s < nsteps; ++s) {
            int rc = enqueue_step(c, c->stream);
            if (rc) return rc;
            c->time += c->p.dt;
        }
        return PN_OK;
    }
    int rc = build_step_graph(c);
    if (rc) return rc;
    for (int s = 0; s < nsteps; ++s) {
        CU(cudaGraphLaunch(c->step_exec, c->stream));
        c->time += c->p.dt;  // Limit-sticky9.c:893
    }
    return PN_OK;
}

static int read_energy(pn_ctx *c, pn_energy_t *e) {
    CU(cudaMemcpyAsync(c->h_eout, c->eout, 4 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    int rc = check_device_err(c);
    if (rc) return rc;
    e->pot_n = c->h_eout[0];
    e->kin_n = c->h_eout[1];
    e->pot_pn = c->h_eout[2];
    e->total = c->h_eout[3];
    for (int q = 0; q < 4; ++q)
        if (!std::isfinite(c->h_eout[q])) return set_err(PN_ERR_NONFINITE, "non-finite energy");
    return PN_OK;
}

extern "C" int pn_steps_energy_async(pn_ctx *c, int nsteps) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_steps_energy: no state");
    if (nsteps < 1) return set_err(PN_ERR_INVALID, "pn_steps_energy: nsteps");
    int rc = build_step_graph(c);  // before the first launch (allocations, shapes)
    if (rc) return rc;
    rc = enqueue_step(c, c->stream, true);
    if (rc) return rc;
    c->time += c->p.dt;
    for (int s = 1; s < nsteps; ++s) {
        CU(cudaGraphLaunch(c->step_exec, c->stream));
        c->time += c->p.dt;
    }
    return PN_OK;
}

extern "C" int pn_energy_result(pn_ctx *c, pn_energy_t *e) {
    if (!c || !e) return set_err(PN_ERR_INVALID, "pn_energy_result");
    return read_energy(c, e);
}

extern "C" int pn_steps_energy(pn_ctx *c, int nsteps, pn_energy_t *e) {
    if (!e) return set_err(PN_ERR_INVALID, "pn_steps_energy: e");
    int rc = pn_steps_energy_async(c, nsteps);
    return rc ? rc : read_energy(c, e);
}

// ------------------------------------------------------------------ asynchronous snapshots
extern "C" int pn_snapshot_begin(pn_ctx *c) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_snapshot_begin: no state");
    if (c->snap_pending) return set_err(PN_ERR_STATE, "pn_snapshot_begin: previous snapshot not ended");
    const size_t bytes = 6 * (size_t)c->ld * sizeof(double);  // x and v are adjacent in the state
    if (!c->snap_dev) {
        if (cudaMalloc(&c->snap_dev, bytes) != cudaSuccess || cudaMallocHost(&c->snap_host, bytes) != cudaSuccess) {
            cudaGetLastError();
            return set_err(PN_ERR_NOMEM, "snapshot buffers");
        }
        CU(cudaStreamCreateWithFlags(&c->snap_stream, cudaStreamNonBlocking));
        CU(cudaEventCreateWithFlags(&c->snap_taken, cudaEventDisableTiming));
        CU(cudaEventCreateWithFlags(&c->snap_done, cudaEventDisableTiming));
    }
    // the device copy is ordered on the context's stream (before any later step); the transfer
    // to the host runs on the copy stream, concurrently with those steps
    CU(cudaMemcpyAsync(c->snap_dev, c->st.x, bytes, cudaMemcpyDeviceToDevice, c->stream));
    CU(cudaEventRecord(c->snap_taken, c->stream));
    CU(cudaStreamWaitEvent(c->snap_stream, c->snap_taken, 0));
    CU(cudaMemcpyAsync(c->snap_host, c->snap_dev, bytes, cudaMemcpyDeviceToHost, c->snap_stream));
    CU(cudaEventRecord(c->snap_done, c->snap_stream));
    c->snap_pending = true;
    c->snap_n = c->n;
    return PN_OK;
}

extern "C" int pn_snapshot_end(pn_ctx *c, double *x, double *v) {
    if (!c || !c->snap_pending) return set_err(PN_ERR_STATE, "pn_snapshot_end: no snapshot begun");
    c->snap_pending = false;
    CU(cudaEventSynchronize(c->snap_done));
    const size_t ld = (size_t)c->ld;
    for (int p = 0; p < c->snap_n; ++p)
        for (int k = 0; k < 3; ++k) {
            if (x) x[3 * p + k] = c->snap_host[k * ld + p];
            if (v) v[3 * p + k] = c->snap_host[3 * ld + k * ld + p];
        }
    return set_err(PN_OK, nullptr);
}

extern "C" int pn_sync(pn_ctx *c) {
    if (!c) return PN_ERR_INVALID;
    return check_device_err(c);
}

extern "C" double pn_time(pn_ctx *c) { return c ? c->time : 0.0; }

extern "C" int pn_get_stats(pn_ctx *c, pn_stats *s) {
    if (!c || !s) return PN_ERR_INVALID;
    *s = c->stats;
    return PN_OK;
}

// ------------------------------------------------------------------ binary checkpoints
static const char kCkptMagic[8] = {'P', 'N', 'C', 'K', '0', '0', '0', '1'};

extern "C" int pn_save_checkpoint(pn_ctx *c, const char *path, double eouttime, double init_ene) {
    if (!c || !c->have_state || !path) return set_err(PN_ERR_STATE, "pn_save_checkpoint");
    const int n = c->n;
    std::vector<double> x(3 * (size_t)n), v(3 * (size_t)n), m((size_t)n);
    int rc = pn_get_state(c, x.data(), v.data());
    if (rc) return rc;
    CU(cudaMemcpy(m.data(), c->st.m, (size_t)n * sizeof(double), cudaMemcpyDeviceToHost));
    FILE *f = fopen(path, "wb");
    if (!f) return set_err(PN_ERR_IO, "cannot open %s", path);
    const int32_t n32 = n;
    const double hdr[3] = {c->time, eouttime, init_ene};
    bool ok = fwrite(kCkptMagic, 1, 8, f) == 8 && fwrite(&n32, 4, 1, f) == 1 && fwrite(hdr, 8, 3, f) == 3 &&
              fwrite(&c->p, sizeof(pn_params), 1, f) == 1 && fwrite(x.data(), 8, x.size(), f) == x.size() &&
              fwrite(v.data(), 8, v.size(), f) == v.size() && fwrite(m.data(), 8, m.size(), f) == m.size();
    ok = (fclose(f) == 0) && ok;
    return ok ? set_err(PN_OK, nullptr) : set_err(PN_ERR_IO, "write %s", path);
}

extern "C" int pn_load_checkpoint(pn_ctx *c, const char *path, double *eouttime, double *init_ene) {
    if (!c || !path) return set_err(PN_ERR_INVALID, "pn_load_checkpoint");
    FILE *f = fopen(path, "rb");
    if (!f) return set_err(PN_ERR_IO, "cannot open %s", path);
    char magic[8];
    int32_t n32 = 0;
    double hdr[3];
    pn_params p{};
    bool ok = fread(magic, 1, 8, f) == 8 && std::memcmp(magic, kCkptMagic, 8) == 0 && fread(&n32, 4, 1, f) == 1 &&
              fread(hdr, 8, 3, f) == 3 && fread(&p, sizeof(pn_params), 1, f) == 1;
    if (!ok || n32 < 1 || n32 > c->nmax) {
        fclose(f);
        return set_err(PN_ERR_IO, "%s: not a checkpoint or n out of range", path);
    }
    const size_t n = (size_t)n32;
    std::vector<double> x(3 * n), v(3 * n), m(n);
    ok = fread(x.data(), 8, x.size(), f) == x.size() && fread(v.data(), 8, v.size(), f) == v.size() &&
         fread(m.data(), 8, m.size(), f) == m.size();
    fclose(f);
    if (!ok) return set_err(PN_ERR_IO, "%s: truncated", path);
    int rc = pn_set_params(c, &p);
    if (rc) return rc;
    rc = pn_set_state(c, n32, x.data(), v.data(), m.data());
    if (rc) return rc;
    c->time = hdr[0];
    if (eouttime) *eouttime = hdr[1];
    if (init_ene) *init_ene = hdr[2];
    return PN_OK;
}

static int eval_energy(pn_ctx *c, const double *x, const double *v, const double *m, long long sp,
                       long long sk, pn_energy_t *e) {
    const int nstar = c->n - 1;
    refresh_cfg(c);
    const PairCfg &k = c->cfg_energy;
    int rc = ensure_acc(c, k.gsplit);
    if (rc) return rc;
    const double eps2 = c->p.eps * c->p.eps;
    cudaStream_t s = c->stream;
    PrepArgs pa{};
    pa.x = x; pa.v = v; pa.m = m; pa.sp = sp; pa.sk = sk;
    pa.nstar = nstar; pa.npad = c->npad; pa.nfill = (int)round_up(nstar > 0 ? nstar : 1, 256);
    pa.tj = k.tj; pa.f32 = is_f32(c); pa.eps2 = eps2;
    pa.pack = c->pack; pa.torg = c->torg; pa.spos = c->spos;
    if (pa.f32) { pa.pack2 = c->pack2; pa.ipack = c->ipack; }
    pa.part = c->part; pa.glob = c->glob; pa.ticket = &c->tickets[0];
    CU(launch_prep(pa, s));
    PairArgs qa{};
    qa.pack = c->pack; qa.torg = c->torg; qa.spos = c->spos; qa.pack2 = c->pack2; qa.ipack = c->ipack; qa.out = c->acc; qa.err = c->err;
    qa.nstar = nstar; qa.npad = c->npad; qa.tj = k.tj; qa.ntiles = (nstar + k.tj - 1) / k.tj;
    qa.gsplit = k.gsplit; qa.eps2 = eps2;
    if (nstar > 0) {
        if (is_f32(c)) CU(launch_pair_f32(MODE_ENERGY, k, qa, s));
        else CU(launch_pair_f64(MODE_ENERGY, k, qa, s));
    }
    EnergyArgs ea{};
    ea.v = v; ea.m = m; ea.sp = sp; ea.sk = sk;
    ea.spos = c->spos; ea.acc = c->acc; ea.glob = c->glob;
    ea.nstar = nstar; ea.npad = c->npad; ea.gsplit = k.gsplit;
    ea.nacc = pair_nacc(MODE_ENERGY); ea.sphi = E_PHI; ea.spsi = E_PSI;
    ea.eps = c->p.eps; ea.eps2 = eps2; ea.inv_c2 = c->p.inv_c2;
    ea.part = c->part + (size_t)(c->npad / 256 + 2) * 8;
    ea.out = c->eout; ea.ticket = &c->tickets[2];
    CU(launch_energy_finish(ea, s));
    return read_energy(c, e);
}

extern "C" int pn_energy(pn_ctx *c, pn_energy_t *e) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_energy: no state");
    if (!e) return set_err(PN_ERR_INVALID, "pn_energy");
    return eval_energy(c, c->st.x, c->st.v, c->st.m, 1, c->ld, e);
}

// ------------------------------------------------------------------ drop-in entry points
// One implicit context (capacity PN_NMAX, Limit-sticky9.c:13), created at first use.  Like the
// reference these functions are not thread-safe.
static pn_ctx *g_drop = nullptr;
static double *g_drop_h = nullptr;  // pinned host staging [7][PN_NMAX]
static int g_drop_prec = -1;
static double g_drop_ic2 = 1.0;

extern "C" int pn_dropin_configure(int precision, double inv_c2) {
    if ((precision != PN_PREC_FP64 && precision != PN_PREC_MIXED) || !(inv_c2 >= 0.0))
        return set_err(PN_ERR_INVALID, "pn_dropin_configure");
    g_drop_prec = precision;
    g_drop_ic2 = inv_c2;
    if (g_drop) {
        pn_params p = g_drop->p;
        p.precision = precision;
        p.inv_c2 = inv_c2;
        return pn_set_params(g_drop, &p);
    }
    return PN_OK;
}

extern "C" void pn_dropin_release(void) {
    if (g_drop) pn_destroy(g_drop);
    if (g_drop_h) cudaFreeHost(g_drop_h);
    g_drop = nullptr;
    g_drop_h = nullptr;
}

[[noreturn]] static void drop_fatal(const char *where) {
    fprintf(stderr, "libpn %s: %s (%s)\n", where, pn_strerror(g_last_error), g_last_msg);
    abort();
}

static pn_ctx *drop_ctx(double eps) {
    if (!g_drop) {
        if (g_drop_prec < 0) {
            const char *e = getenv("PN_PRECISION");
            g_drop_prec = (e && (!strcmp(e, "mixed") || !strcmp(e, "MIXED"))) ? PN_PREC_MIXED : PN_PREC_FP64;
        }
        pn_params p;
        pn_params_default(&p);
        p.eps = eps;
        p.precision = g_drop_prec;
        p.inv_c2 = g_drop_ic2;
        const int rc = pn_create(&g_drop, PN_NMAX, &p);
        if (rc == PN_ERR_UNSUPPORTED) return nullptr;  // no GPU: reported, not fatal
        if (rc != PN_OK) drop_fatal("context");
        if (cudaMallocHost(&g_drop_h, 7 * (size_t)PN_NMAX * sizeof(double)) != cudaSuccess) {
            set_err(PN_ERR_NOMEM, "pinned staging");
            drop_fatal("context");
        }
        atexit(pn_dropin_release);
    }
    if (g_drop->p.eps != eps) {
        pn_params p = g_drop->p;
        p.eps = eps;
        pn_set_params(g_drop, &p);
    }
    return g_drop;
}

// Copies x, v, m (host AoS) to the device AoS staging buffers of the implicit context.
static int drop_upload(pn_ctx *c, const double *x, const double *v, const double *m, int n) {
    const size_t ld = (size_t)c->ld;
    std::memcpy(g_drop_h, x, 3 * (size_t)n * sizeof(double));
    std::memcpy(g_drop_h + 3 * ld, v, 3 * (size_t)n * sizeof(double));
    std::memcpy(g_drop_h + 6 * ld, m, (size_t)n * sizeof(double));
    CU(cudaMemcpyAsync(c->in_aos, g_drop_h, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->in_aos + 3 * ld, g_drop_h + 3 * ld, 3 * (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    CU(cudaMemcpyAsync(c->in_aos + 6 * ld, g_drop_h + 6 * ld, (size_t)n * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    if (n != c->n) { c->cfg_set = false; c->step_valid = false; }
    c->n = n;
    return PN_OK;
}

extern "C" void force(double (*x)[3], double (*v)[3], double *m, double eps, double (*a)[3],
                      double *pot, int n) {
    (void)pot;  // unused by the reference too (Limit-sticky9.c:23)
    if (n < 1 || n > PN_NMAX || !x || !v || !m || !a || !(eps > 0.0) || !(m[0] > 0.0)) {
        set_err(PN_ERR_INVALID, "force: n=%d", n);
        return;
    }
    pn_ctx *c = drop_ctx(eps);
    if (!c) return;
    const size_t ld = (size_t)c->ld;
    if (drop_upload(c, &x[0][0], &v[0][0], m, n)) drop_fatal("force");
    int rc = eval_force(c, c->in_aos, c->in_aos + 3 * ld, c->in_aos + 6 * ld, 3, 1, c->a_aos, 3, 1, 0,
                        c->stream, false);
    if (rc) drop_fatal("force");
    if (cudaMemcpyAsync(g_drop_h, c->a_aos, 3 * (size_t)n * sizeof(double), cudaMemcpyDeviceToHost,
                        c->stream) != cudaSuccess) {
        set_err(PN_ERR_CUDA, "force: copy back");
        drop_fatal("force");
    }
    rc = check_device_err(c);  // sets the last error (PN_OK or PN_ERR_NONFINITE)
    if (rc == PN_ERR_CUDA || rc == PN_ERR_TIMEOUT) drop_fatal("force");
    std::memcpy(&a[0][0], g_drop_h, 3 * (size_t)n * sizeof(double));
}

static int drop_energy(double x[][3], double v[][3], double m[], int n, double eps, pn_energy_t *e) {
    if (n < 1 || n > PN_NMAX || !x || !v || !m || !(eps > 0.0) || !(m[0] > 0.0))
        return set_err(PN_ERR_INVALID, "energy: n=%d", n);
    pn_ctx *c = drop_ctx(eps);
    if (!c) return g_last_error;
    const size_t ld = (size_t)c->ld;
    if (drop_upload(c, &x[0][0], &v[0][0], m, n)) drop_fatal("energy");
    int rc = eval_energy(c, c->in_aos, c->in_aos + 3 * ld, c->in_aos + 6 * ld, 3, 1, e);
    if (rc == PN_ERR_CUDA || rc == PN_ERR_TIMEOUT) drop_fatal("energy");
    return rc;
}

extern "C" void energy(double t, double x[][3], double v[][3], double m[], int n, double init_ene,
                       double eps) {
    pn_energy_t e{};
    const int rc = drop_energy(x, v, m, n, eps, &e);
    if (rc == PN_ERR_INVALID || rc == PN_ERR_UNSUPPORTED) return;
    const double DE = (init_ene - e.total) / e.total;  // Limit-sticky9.c:558
    printf("time = %g\n", t);                          // :560-563, same format
    printf("pot = %22.15e kin = %22.15e \n pot_pn = %22.15e \n  total= %22.15e ratio = %e\n",
           e.pot_n, e.kin_n, e.pot_pn, e.total, e.kin_n / e.pot_n);
    printf(" DE = %e %g\n", DE, t);
    fflush(stdout);
}

extern "C" void initial_energy(double x[][3], double v[][3], double m[], int n, double *init_ene,
                               double eps) {
    pn_energy_t e{};
    const int rc = drop_energy(x, v, m, n, eps, &e);
    if (rc == PN_ERR_INVALID || rc == PN_ERR_UNSUPPORTED) return;
    printf("time = %g\n", 0.0);  // :701-703, same format
    printf("pot = %22.15e kin = %22.15e \n pot_pn = %22.15e \n  total= %22.15e ratio = %e\n",
           e.pot_n, e.kin_n, e.pot_pn, e.total, e.kin_n / e.pot_n);
    fflush(stdout);
    if (init_ene) *init_ene = e.total;  // :705
}

// Limit-sticky9.c:716-738 (not called by the reference main; kept for link compatibility).
extern "C" void push_velocity(double v[][3], double a[][3], double dt, int n) {
    for (int j = 0; j < n; j++)
        for (int k = 0; k < 3; k++) v[j][k] += dt * a[j][k];
}

extern "C" void push_position(double x[][3], double v[][3], double dt, int n) {
    for (int j = 0; j < n; j++)
        for (int k = 0; k < 3; k++) x[j][k] += dt * v[j][k];
}

// ------------------------------------------------------------------ self-test of bounded waits
// A CTA waits on an mbarrier that nothing ever completes; the wait gives up after its limit,
// the kernel records DEVERR_TIMEOUT and returns, and the host reads PN_ERR_TIMEOUT.  This
// exercises the same bounded-wait path as the pair kernel's tile pipeline, with no fault.
static __global__ void k_selftest_wait(int *err, long long limit_cycles) {
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
    }
    __syncthreads();
    const bool ok = mbar_wait_bounded(&bar, 0u, limit_cycles);
    if (!ok && threadIdx.x == 0) atomicOr(err, DEVERR_TIMEOUT);
}

extern "C" int pn_selftest_wait_timeout(pn_ctx *c, double seconds) {
    if (!c || !(seconds > 0.0) || seconds > 5.0) return set_err(PN_ERR_INVALID, "selftest");
    int khz = 0;
    CU(cudaDeviceGetAttribute(&khz, cudaDevAttrClockRate, c->dev));
    const long long limit = (long long)(seconds * (double)khz * 1e3);
    k_selftest_wait<<<1, 32, 0, c->stream>>>(c->err, limit);
    CU(cudaGetLastError());
    return check_device_err(c);
}

// ------------------------------------------------------------------ benchmark support
extern "C" int pn_bench_steps(pn_ctx *c, int nsteps, int flush_l2, double *step_ms, double *pair_ms) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_bench_steps: no state");
    if (nsteps < 0 || (nsteps > 0 && (!step_ms || !pair_ms)))
        return set_err(PN_ERR_INVALID, "pn_bench_steps");
    int rc = build_step_graph(c);
    if (rc) return rc;
    if (flush_l2 && !c->flush) {
        int l2 = 0;
        CU(cudaDeviceGetAttribute(&l2, cudaDevAttrL2CacheSize, c->dev));
        c->flush_bytes = 2 * (size_t)(l2 > 0 ? l2 : (128 << 20));  // twice the L2
        if (cudaMalloc(&c->flush, c->flush_bytes) != cudaSuccess) {
            cudaGetLastError();
            c->flush = nullptr;
            return set_err(PN_ERR_NOMEM, "flush buffer");
        }
    }
    for (int k = 0; k < nsteps; ++k) {
        if (flush_l2) CU(cudaMemsetAsync(c->flush, k & 0xff, c->flush_bytes, c->stream));
        CU(cudaEventRecord(c->ev0, c->stream));
        CU(cudaGraphLaunch(c->step_exec, c->stream));
        CU(cudaEventRecord(c->ev1, c->stream));
        CU(cudaStreamSynchronize(c->stream));
        c->time += c->p.dt;
        float ms = 0.f;
        CU(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
        step_ms[k] = ms;
        double pm = 0.0;
        for (int q = 0; q < step_evaluations(c); ++q) {
            CU(cudaEventElapsedTime(&ms, c->evp[2 * q], c->evp[2 * q + 1]));
            pm += ms;
        }
        pair_ms[k] = pm;
    }
    return check_device_err(c);
}

// Arithmetic work of one pair interaction in each sweep, counting an FMA as 2 flops, the MUFU
// rsqrt as 1 and every other add/multiply as 1 (the operations written in pn_device.cuh).
extern "C" double pn_flops_per_pair(int mode, int precision, int pair_variant) {
    const bool f32 = precision == PN_PREC_MIXED;
    if (f32 && pair_variant >= PN_PAIR_F32X2 && pair_variant <= PN_PAIR_F32X2_OCC4) {
        // the packed sweep (operands pre-scaled): FORCE 50 FP32 operations of which 24 FMA,
        // NEWTON 22 (7 FMA), ENERGY 32 (12 FMA); FMA = 2 flops, the MUFU rsqrt = 1
        switch (mode) {
            case MODE_NEWTON: return 30.0;
            case MODE_FORCE: return 75.0;
            case MODE_ENERGY: return 45.0;
            default: return 0.0;
        }
    }
    switch (mode) {
        // FP32 counts include the hi/lo difference (9 vs 3) and the Newton step of the MUFU
        // rsqrt (7 vs 1 for FP64, whose rsqrt counts as one operation)
        case MODE_NEWTON: return f32 ? 31.0 : 19.0;
        case MODE_FORCE: return f32 ? 82.0 : 70.0;
        case MODE_ENERGY: return f32 ? 46.0 : 34.0;
        default: return 0.0;
    }
}

// Peak FMA throughput probe: each thread runs 8 independent FMA chains (no memory traffic),
// 16 iterations unrolled per loop trip so that loop overhead stays below 1 %.
template <typename T> __device__ __forceinline__ T probe_fma(T x, T a, T b);
template <> __device__ __forceinline__ float probe_fma<float>(float x, float a, float b) { return fmaf(x, a, b); }
template <> __device__ __forceinline__ double probe_fma<double>(double x, double a, double b) { return fma(x, a, b); }

// packed FP32x2: both lanes of a 64-bit register pair in one fma.rn.f32x2
struct F2 { unsigned long long v; };
template <> __device__ __forceinline__ F2 probe_fma<F2>(F2 x, F2 a, F2 b) {
    F2 r;
    asm("fma.rn.f32x2 %0, %1, %2, %3;" : "=l"(r.v) : "l"(x.v), "l"(a.v), "l"(b.v));
    return r;
}
static __device__ __forceinline__ F2 f2_of(float lo, float hi) {
    F2 r;
    asm("mov.b64 %0, {%1, %2};" : "=l"(r.v) : "f"(lo), "f"(hi));
    return r;
}
static __global__ void k_fma2_probe(float *out, int iters, float a, float b) {
    F2 r[8];
    const F2 a2 = f2_of(a, a), b2 = f2_of(b, b);
#pragma unroll
    for (int q = 0; q < 8; ++q) r[q] = f2_of((float)(threadIdx.x + q), (float)(threadIdx.x - q));
    for (int it = 0; it < iters; it += 16)
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int q = 0; q < 8; ++q) r[q] = probe_fma<F2>(r[q], a2, b2);
    float s = 0.f;
#pragma unroll
    for (int q = 0; q < 8; ++q) {
        float lo, hi;
        asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(r[q].v));
        s += lo + hi;
    }
    if (s == 123456.0f) out[threadIdx.x] = s;  // keeps the chains live
}

template <typename T>
static __global__ void k_fma_probe(T *out, int iters, T a, T b) {
    T r[8];
#pragma unroll
    for (int q = 0; q < 8; ++q) r[q] = (T)(threadIdx.x + q);
    for (int it = 0; it < iters; it += 16)
#pragma unroll
        for (int u = 0; u < 16; ++u)
#pragma unroll
            for (int q = 0; q < 8; ++q) r[q] = probe_fma<T>(r[q], a, b);
    T s = 0;
#pragma unroll
    for (int q = 0; q < 8; ++q) s += r[q];
    if (s == (T)123456.0) out[threadIdx.x] = s;  // keeps the chains live
}

extern "C" int pn_probe_fma_peak(int precision, double *tflops) {
    if (!tflops) return set_err(PN_ERR_INVALID, "probe");
    if (precision < PN_PREC_FP64 || precision > PN_PROBE_F32X2) return set_err(PN_ERR_INVALID, "probe: precision");
    if (pn_device_count() < 1) return set_err(PN_ERR_UNSUPPORTED, "no CUDA device");
    int dev = 0, sms = 0;
    CU(cudaGetDevice(&dev));
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    void *out = nullptr;
    CU(cudaMalloc(&out, 1024 * sizeof(double)));
    cudaEvent_t e0, e1;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    const int threads = 256, blocks = sms * 8;
    const int iters = precision == PN_PREC_FP64 ? 1000 : 20000;
    float best = 1e30f;
    for (int rep = 0; rep < 4; ++rep) {
        cudaEventRecord(e0);
        if (precision == PN_PREC_MIXED)
            k_fma_probe<float><<<blocks, threads>>>((float *)out, iters, 0.9999f, 1e-4f);
        else if (precision == PN_PROBE_F32X2)
            k_fma2_probe<<<blocks, threads>>>((float *)out, iters / 2, 0.9999f, 1e-4f);
        else
            k_fma_probe<double><<<blocks, threads>>>((double *)out, iters, 0.9999, 1e-4);
        cudaEventRecord(e1);
        cudaEventSynchronize(e1);
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;
    }
    cudaError_t e = cudaGetLastError();
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (e != cudaSuccess) return set_err(PN_ERR_CUDA, "probe: %s", cudaGetErrorString(e));
    // the packed probe runs iters / 2 instructions of two lanes each: the same flops
    const double flops = 2.0 * 8.0 * (double)iters * threads * (double)blocks;
    *tflops = flops / (best * 1e-3) / 1e12;
    return PN_OK;
}

// ------------------------------------------------------------------ autotuning
// Times every candidate launch shape of the force sweep (and, with sweeps & 2, the energy
// sweep) on the context's current state and keeps the fastest for this precision and size
// class.  The state is not modified (the sweeps only write work buffers).
extern "C" int pn_autotune(pn_ctx *c, int sweeps, double *best_ms) {
    if (!c || !c->have_state) return set_err(PN_ERR_STATE, "pn_autotune: no state");
    const int nstar = c->n - 1;
    if (nstar < 1) return PN_OK;
    int sms = 0;
    CU(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, c->dev));
    const bool f32 = is_f32(c);
    const double eps2 = c->p.eps * c->p.eps;
    const int modes[2] = {force_mode(c), MODE_ENERGY};
    for (int which = 0; which < 2; ++which) {
        if (!(sweeps & (1 << which))) continue;
        const int mode = modes[which];
        std::vector<PairCfg> cands = tune_candidates(f32, mode, nstar, sms);
        PairCfg best{};
        float best_t = 1e30f;
        for (const PairCfg &k : cands) {
            int rc = ensure_acc(c, k.gsplit);
            if (rc) return rc;
            PrepArgs pa{};
            pa.x = c->st.x; pa.v = c->st.v; pa.m = c->st.m; pa.sp = 1; pa.sk = c->ld;
            pa.nstar = nstar; pa.npad = c->npad; pa.nfill = (int)round_up(nstar, 256);
            pa.tj = k.tj; pa.f32 = f32; pa.eps2 = eps2;
            pa.pack = c->pack; pa.torg = c->torg; pa.spos = c->spos;
    if (pa.f32) { pa.pack2 = c->pack2; pa.ipack = c->ipack; }
            pa.part = c->part; pa.glob = c->glob; pa.ticket = &c->tickets[0];
            CU(launch_prep(pa, c->stream));
            PairArgs qa{};
            qa.pack = c->pack; qa.torg = c->torg; qa.spos = c->spos; qa.pack2 = c->pack2; qa.ipack = c->ipack; qa.out = c->acc; qa.err = c->err;
            qa.nstar = nstar; qa.npad = c->npad; qa.tj = k.tj; qa.ntiles = (nstar + k.tj - 1) / k.tj;
            qa.gsplit = k.gsplit; qa.eps2 = eps2;
            float t = 1e30f;
            if (which == 0) {
                // the force sweep: time the whole evaluation (prep, pair sweep, finish), so that
                // the finishing kernel's reads of the j-range partial sums (72 B per star and
                // split) count against the shapes with many splits
                c->cfg_force = k;
                c->cfg_energy = k;
                c->cfg_set = true;
                for (int rep = 0; rep < 3; ++rep) {  // first evaluation warms up; best of two
                    CU(cudaEventRecord(c->ev0, c->stream));
                    rc = eval_force(c, c->st.x, c->st.v, c->st.m, 1, c->ld, nullptr, 3, 1, 0, c->stream, false);
                    if (rc) return rc;
                    CU(cudaEventRecord(c->ev1, c->stream));
                    CU(cudaEventSynchronize(c->ev1));
                    float ms = 0.f;
                    CU(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
                    if (rep > 0 && ms < t) t = ms;
                }
            } else {
                for (int rep = 0; rep < 2; ++rep) {  // first launch warms up
                    CU(cudaEventRecord(c->ev0, c->stream));
                    cudaError_t e = f32 ? launch_pair_f32(mode, k, qa, c->stream)
                                        : launch_pair_f64(mode, k, qa, c->stream);
                    if (e != cudaSuccess) return set_err(PN_ERR_CUDA, "autotune: %s", cudaGetErrorString(e));
                    CU(cudaEventRecord(c->ev1, c->stream));
                    CU(cudaEventSynchronize(c->ev1));
                    float ms = 0.f;
                    CU(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
                    if (rep > 0) t = ms;
                }
            }
            if (getenv("PN_TUNE_VERBOSE"))
                fprintf(stderr, "pn_autotune mode %d: ipt %d js %d tj %d gsplit %d x2 %d: %.3f ms\n", mode,
                        k.ipt, k.js, k.tj, k.gsplit, k.x2, t);
            if (t < best_t) {
                best_t = t;
                best = k;
            }
        }
        int rc = check_device_err(c);
        if (rc) return rc;
        tune_store(c->p.precision, mode, nstar, best, best_t);
        if (best_ms) best_ms[which] = best_t;
    }
    c->cfg_set = false;
    c->step_valid = false;
    return PN_OK;
}

extern "C" void pn_autotune_clear(void) { tune_clear(); }
