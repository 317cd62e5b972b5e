// pn_ensemble.cu -- many independent clusters (BH + stars each) advanced together.
//
// Layout.  All clusters' particles are concatenated (cluster c occupies particles
// [p0_c, p0_c + n_c), SoA [3][LD] state arrays as for one system).  Star slots are padded per
// cluster to a multiple of 256 (cluster c owns slots [s0_c, s0_c + slots_c)), so every 256-slot
// block and every j-tile belongs to exactly one cluster, and tile origins index as for one
// system.  The pack, the BH-relative positions and the pair sums of all clusters share one
// set of arrays with row stride S (the total slot count).
//
// One force evaluation of the whole ensemble is three launches:
//   k_prep_ens    every cluster's 256-slot blocks (per-cluster reductions by per-cluster
//                 last-block tickets)
//   k_pair_ens    ONE persistent launch over the (cluster, i-block, j-range) work items of all
//                 clusters, biggest first, fetched from a global counter
//   k_finish_ens  every cluster's blocks, with the fused integration stage
// An integration step is three evaluations and is captured in one CUDA graph.
//
// Launch shapes: the persistent kernel has one (i per thread, lanes per i-set) for the
// launch; the j-tile size and the number of j-range splits are chosen per size class
// (floor(log2 N)) by pn_ens_autotune.
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>

#include "../../include/pn.h"
#include "pn_kernels.h"

using namespace pn;

extern "C" int pn_device_count(void);

namespace {

thread_local int g_ens_err = PN_OK;

int fail(int code, const char *what, cudaError_t e = cudaSuccess) {
    g_ens_err = code;
    if (e != cudaSuccess) fprintf(stderr, "libpn ensemble: %s: %s\n", what, cudaGetErrorString(e));
    return code;
}

#define ECU(call)                                                       \
    do {                                                                \
        cudaError_t e_ = (call);                                        \
        if (e_ != cudaSuccess) return fail(PN_ERR_CUDA, #call, e_);     \
    } while (0)

inline long long rup(long long a, long long b) { return (a + b - 1) / b * b; }

int size_class(int nstar) {
    int c = 0;
    while ((1 << (c + 1)) <= nstar) ++c;
    return c;
}

struct ClassShape {
    int tj = 128;
    int tiles_per_item = 32;  // j-range of one work item, in tiles
};

}  // namespace

struct pn_ens {
    int nc = 0;
    std::vector<int> n, p0, s0, slots, blk0, nblk;
    std::vector<double> eps;
    int P = 0, S = 0, LD = 0, B = 0;  // particles, star slots, state leading dim, 256-blocks
    pn_params p{};
    int ipt = 2, js = 1;
    int x2 = 0;  // mixed precision: the packed FP32x2 sweep (js = 1)
    ClassShape cls[32];
    cudaStream_t stream = nullptr;
    double *state = nullptr;
    DevState st{};
    double *a_aos = nullptr;
    double *spos = nullptr, *acc = nullptr, *ppart = nullptr, *fpart = nullptr, *glob = nullptr,
           *eout = nullptr;
    int acc_splits = 0;
    void *pack = nullptr;
    float4 *pack2 = nullptr, *ipack = nullptr;  // mixed precision: paired pack [7][S/2], i-data [S]
    TileOrigin *torg = nullptr;
    unsigned *tickets = nullptr, *counter = nullptr;
    int *err = nullptr;
    int4 *blockmap = nullptr, *items = nullptr;
    int nitems = 0;
    PrepArgs *t_prep = nullptr;    // [2][nc]: evaluation at (x, v) / at (xs, vs)
    FinishArgs *t_fin = nullptr;   // [4][nc]: stage 0 (a out), 1, 2, 3
    EnergyArgs *t_en = nullptr;    // [nc]
    PairArgs *t_pair = nullptr;    // [2][nc]: force / energy sweep
    cudaGraphExec_t step_exec = nullptr;
    bool step_valid = false;
    bool have_state = false;
    double time = 0.0;
    cudaEvent_t e0 = nullptr, e1 = nullptr;
};

static bool ens_f32(const pn_ens *e) { return e->p.precision == PN_PREC_MIXED; }
static int ens_mode(const pn_ens *e) { return e->p.inv_c2 != 0.0 ? MODE_FORCE : MODE_NEWTON; }

static void ens_free(pn_ens *e) {
    if (!e) return;
    if (e->step_exec) cudaGraphExecDestroy(e->step_exec);
    void *bufs[] = {e->state, e->a_aos, e->spos, e->acc, e->ppart, e->fpart, e->glob, e->eout,
                    e->pack, e->pack2, e->ipack, e->torg, e->tickets, e->counter, e->err, e->blockmap, e->items,
                    e->t_prep, e->t_fin, e->t_en, e->t_pair};
    for (void *b : bufs)
        if (b) cudaFree(b);
    if (e->e0) cudaEventDestroy(e->e0);
    if (e->e1) cudaEventDestroy(e->e1);
    if (e->stream) cudaStreamDestroy(e->stream);
    delete e;
}

// Per-cluster j-range splits of the current shapes.
static int cluster_gsplit(const pn_ens *e, int c) {
    const int nstar = e->n[c] - 1;
    const ClassShape &k = e->cls[size_class(nstar > 0 ? nstar : 1)];
    const int ntiles = (nstar + k.tj - 1) / k.tj;
    int g = (ntiles + k.tiles_per_item - 1) / k.tiles_per_item;
    if (g < 1) g = 1;
    if (g > ntiles) g = ntiles;
    if (g > 64) g = 64;
    return g;
}

// Rebuilds the argument tables and the work-item list from the current shapes.
static int ens_build_tables(pn_ens *e) {
    const bool f32 = ens_f32(e);
    const int mode = ens_mode(e);
    const int nc = e->nc;
    int gmax = 1;
    for (int c = 0; c < nc; ++c) gmax = std::max(gmax, cluster_gsplit(e, c));
    if (gmax > e->acc_splits) {
        if (e->acc) cudaFree(e->acc);
        e->acc = nullptr;
        ECU(cudaMalloc(&e->acc, (size_t)gmax * NACC_MAX * e->S * sizeof(double)));
        e->acc_splits = gmax;
    }
    std::vector<PrepArgs> tp(2 * nc);
    std::vector<FinishArgs> tf(4 * nc);
    std::vector<EnergyArgs> te(nc);
    std::vector<PairArgs> tq(2 * nc);
    std::vector<int4> items;
    const int bi = PAIR_NT * e->ipt / e->js;
    const long long ld = e->LD;
    for (int c = 0; c < nc; ++c) {
        const int nstar = e->n[c] - 1;
        const ClassShape &k = e->cls[size_class(nstar > 0 ? nstar : 1)];
        const int g = cluster_gsplit(e, c);
        const double eps = e->eps[c], eps2 = eps * eps;
        const size_t so = (size_t)e->s0[c];
        DevState sc = e->st;  // pointers offset to this cluster's first particle
        sc.x += e->p0[c]; sc.v += e->p0[c]; sc.xs += e->p0[c]; sc.vs += e->p0[c];
        sc.hx += e->p0[c]; sc.hv += e->p0[c]; sc.m += e->p0[c];
        for (int ev = 0; ev < 2; ++ev) {
            PrepArgs &pa = tp[ev * nc + c];
            pa = PrepArgs{};
            pa.x = ev ? sc.xs : sc.x;
            pa.v = ev ? sc.vs : sc.v;
            pa.m = sc.m;
            pa.sp = 1;
            pa.sk = ld;
            pa.nstar = nstar;
            pa.npad = e->S;
            pa.nfill = e->slots[c];
            pa.tj = k.tj;
            pa.f32 = f32;
            pa.eps2 = eps2;
            pa.pack = static_cast<char *>(e->pack) + so * 16;
            if (e->pack2) {  // slot offsets are multiples of 256, so so / 2 is a whole pair row
                pa.pack2 = e->pack2 + so / 2;
                pa.ipack = e->ipack + so;
            }
            pa.torg = e->torg + so / 32;  // tile origins at 32-slot granularity (tj >= 32)
            pa.spos = e->spos + so;
            pa.part = e->ppart + (size_t)e->blk0[c] * NGLOB;
            pa.glob = e->glob + (size_t)c * 16;
            pa.ticket = &e->tickets[c * 4 + 0];
        }
        for (int pm = 0; pm < 2; ++pm) {
            PairArgs &qa = tq[pm * nc + c];
            qa = PairArgs{};
            qa.pack = static_cast<char *>(e->pack) + so * 16;
            if (e->pack2) {
                qa.pack2 = e->pack2 + so / 2;
                qa.ipack = e->ipack + so;
            }
            qa.torg = e->torg + so / 32;
            qa.spos = e->spos + so;
            qa.out = e->acc + so;
            qa.err = e->err;
            qa.nstar = nstar;
            qa.npad = e->S;
            qa.tj = k.tj;
            qa.ntiles = (nstar + k.tj - 1) / k.tj;
            qa.gsplit = g;
            qa.eps2 = eps2;
        }
        for (int stg = 0; stg < 4; ++stg) {
            FinishArgs &fa = tf[stg * nc + c];
            fa = FinishArgs{};
            const bool at_x = stg <= 1;  // stage 0 (force) and stage 1 evaluate at (x, v)
            fa.v = at_x ? sc.v : sc.vs;
            fa.m = sc.m;
            fa.vsp = 1;
            fa.vsk = ld;
            fa.spos = e->spos + so;
            fa.acc = e->acc + so;
            fa.glob = e->glob + (size_t)c * 16;
            fa.nstar = nstar;
            fa.npad = e->S;
            fa.nacc = pair_nacc(mode);
            fa.gsplit = g;
            fa.pn1 = mode == MODE_FORCE;
            fa.eps = eps;
            fa.eps2 = eps2;
            fa.inv_c2 = e->p.inv_c2;
            fa.dt = e->p.dt;
            fa.a = stg == 0 ? e->a_aos + 3 * (size_t)e->p0[c] : nullptr;
            fa.asp = 3;
            fa.ask = 1;
            fa.stage = stg;
            fa.st = sc;
            fa.ld = ld;
            fa.part = e->fpart + (size_t)e->blk0[c] * 8;
            fa.ticket = &e->tickets[c * 4 + 1];
            fa.err = e->err;
        }
        EnergyArgs &ea = te[c];
        ea = EnergyArgs{};
        ea.v = sc.v;
        ea.m = sc.m;
        ea.sp = 1;
        ea.sk = ld;
        ea.spos = e->spos + so;
        ea.acc = e->acc + so;
        ea.glob = e->glob + (size_t)c * 16;
        ea.nstar = nstar;
        ea.npad = e->S;
        ea.gsplit = g;
        ea.nacc = pair_nacc(MODE_ENERGY);
        ea.sphi = E_PHI;
        ea.spsi = E_PSI;
        ea.eps = eps;
        ea.eps2 = eps2;
        ea.inv_c2 = e->p.inv_c2;
        ea.part = e->fpart + (size_t)e->blk0[c] * 8;
        ea.out = e->eout + (size_t)c * 4;
        ea.ticket = &e->tickets[c * 4 + 2];
        const int nib = nstar > 0 ? (nstar + bi - 1) / bi : 0;
        for (int ib = 0; ib < nib; ++ib)
            for (int s = 0; s < g; ++s) items.push_back(make_int4(c, ib * bi, s, 0));
    }
    // biggest items first: cost ~ i-block x tiles of its j-range
    auto cost = [&](const int4 &w) {
        const int nstar = e->n[w.x] - 1;
        const int tjc = e->cls[size_class(nstar)].tj;
        const int nt = (nstar + tjc - 1) / tjc;
        const int g = cluster_gsplit(e, w.x);
        const int t0 = (int)((long long)nt * w.z / g), t1 = (int)((long long)nt * (w.z + 1) / g);
        return (long long)(t1 - t0) * tjc * std::min(bi, nstar - w.y);
    };
    std::stable_sort(items.begin(), items.end(),
                     [&](const int4 &a, const int4 &b) { return cost(a) > cost(b); });
    if (e->items) cudaFree(e->items);
    e->items = nullptr;
    e->nitems = (int)items.size();
    ECU(cudaMalloc(&e->items, std::max<size_t>(1, items.size()) * sizeof(int4)));
    ECU(cudaMemcpy(e->items, items.data(), items.size() * sizeof(int4), cudaMemcpyHostToDevice));
    ECU(cudaMemcpy(e->t_prep, tp.data(), tp.size() * sizeof(PrepArgs), cudaMemcpyHostToDevice));
    ECU(cudaMemcpy(e->t_fin, tf.data(), tf.size() * sizeof(FinishArgs), cudaMemcpyHostToDevice));
    ECU(cudaMemcpy(e->t_en, te.data(), te.size() * sizeof(EnergyArgs), cudaMemcpyHostToDevice));
    ECU(cudaMemcpy(e->t_pair, tq.data(), tq.size() * sizeof(PairArgs), cudaMemcpyHostToDevice));
    e->step_valid = false;
    return PN_OK;
}

static int ens_tjmax(const pn_ens *e) {
    int t = 32;
    for (int c = 0; c < e->nc; ++c) t = std::max(t, e->cls[size_class(std::max(1, e->n[c] - 1))].tj);
    return t;
}

static int ens_pair_launch(pn_ens *e, int mode, const PairArgs *tab, cudaStream_t s) {
    ECU(cudaMemsetAsync(e->counter, 0, sizeof(unsigned), s));
    cudaError_t r;
    if (ens_f32(e) && e->x2 && e->js == 1 && e->pack2)
        r = launch_pair2_ens_f32(mode, e->ipt, ens_tjmax(e), 0, tab, e->items, e->nitems, e->counter, s);
    else
        r = ens_f32(e) ? launch_pair_ens_f32(mode, e->ipt, e->js, ens_tjmax(e), 0, tab,
                                             e->items, e->nitems, e->counter, s)
                       : launch_pair_ens_f64(mode, e->ipt, e->js, ens_tjmax(e), 0, tab,
                                             e->items, e->nitems, e->counter, s);
    if (r != cudaSuccess) return fail(PN_ERR_CUDA, "pair_ens", r);
    return PN_OK;
}

// One evaluation of every cluster: ev = 0 at (x, v), 1 at (xs, vs); stage as in k_finish.
static int ens_eval(pn_ens *e, int ev, int stage, cudaStream_t s) {
    ECU(launch_prep_ens(e->t_prep + (size_t)ev * e->nc, e->blockmap, e->B, s));
    int rc = ens_pair_launch(e, ens_mode(e), e->t_pair, s);
    if (rc) return rc;
    ECU(launch_finish_ens(e->t_fin + (size_t)stage * e->nc, e->blockmap, e->B, s));
    return PN_OK;
}

static int ens_check(pn_ens *e) {
    int h = 0;
    ECU(cudaMemcpyAsync(&h, e->err, sizeof(int), cudaMemcpyDeviceToHost, e->stream));
    ECU(cudaStreamSynchronize(e->stream));
    if (h) {
        ECU(cudaMemsetAsync(e->err, 0, sizeof(int), e->stream));
        ECU(cudaStreamSynchronize(e->stream));
        return fail((h & DEVERR_TIMEOUT) ? PN_ERR_TIMEOUT : PN_ERR_NONFINITE, "device check");
    }
    g_ens_err = PN_OK;
    return PN_OK;
}

extern "C" int pn_ens_create(pn_ens **out, int nclusters, const int *n, const double *eps,
                             const pn_params *p) {
    if (!out || nclusters < 1 || !n || !eps) return fail(PN_ERR_INVALID, "pn_ens_create");
    *out = nullptr;
    if (pn_device_count() < 1) return fail(PN_ERR_UNSUPPORTED, "no CUDA device");
    pn_ens *e = new pn_ens();
    if (p) e->p = *p; else pn_params_default(&e->p);
    if (e->p.precision != PN_PREC_FP64 && e->p.precision != PN_PREC_MIXED) {
        ens_free(e);
        return fail(PN_ERR_INVALID, "precision");
    }
    e->nc = nclusters;
    e->n.assign(n, n + nclusters);
    e->eps.assign(eps, eps + nclusters);
    int P = 0, S = 0, B = 0;
    for (int c = 0; c < nclusters; ++c) {
        if (n[c] < 1 || !(eps[c] > 0.0)) {
            ens_free(e);
            return fail(PN_ERR_INVALID, "cluster size or eps");
        }
        e->p0.push_back(P);
        e->s0.push_back(S);
        e->blk0.push_back(B);
        const int slots = (int)std::max<long long>(256, rup(n[c] - 1, 256));
        e->slots.push_back(slots);
        e->nblk.push_back(slots / 256);
        P += n[c];
        S += slots;
        B += slots / 256;
    }
    e->P = P;
    e->S = S;
    e->B = B;
    e->LD = (int)rup(P, 256);
    if (ens_f32(e)) { e->ipt = 2; e->js = 1; e->x2 = 1; } else { e->ipt = 1; e->js = 4; }
    for (int k = 0; k < 32; ++k) {
        e->cls[k].tj = ens_f32(e) ? (k >= 12 ? 256 : 128) : 128;
        e->cls[k].tiles_per_item = 32;
    }
    auto bad = [&](const char *w) {
        cudaGetLastError();
        ens_free(e);
        return fail(PN_ERR_NOMEM, w);
    };
    const size_t ld = (size_t)e->LD;
    if (cudaStreamCreateWithFlags(&e->stream, cudaStreamNonBlocking)) return bad("stream");
    if (cudaMalloc(&e->state, (19 * ld) * sizeof(double))) return bad("state");
    double *b = e->state;
    e->st.x = b; e->st.v = b + 3 * ld; e->st.xs = b + 6 * ld; e->st.vs = b + 9 * ld;
    e->st.hx = b + 12 * ld; e->st.hv = b + 15 * ld; e->st.m = b + 18 * ld; e->st.ld = e->LD;
    if (cudaMalloc(&e->a_aos, 3 * ld * sizeof(double))) return bad("a");
    if (cudaMalloc(&e->spos, 3 * (size_t)S * sizeof(double))) return bad("spos");
    if (cudaMalloc(&e->pack, 6 * (size_t)S * 16)) return bad("pack");
    if (ens_f32(e)) {
        if (cudaMalloc(&e->pack2, 7 * ((size_t)S / 2) * 16) || cudaMalloc(&e->ipack, (size_t)S * 16) ||
            cudaMemset(e->pack2, 0, 7 * ((size_t)S / 2) * 16) || cudaMemset(e->ipack, 0, (size_t)S * 16))
            return bad("pack2");
    }
    if (cudaMalloc(&e->torg, ((size_t)S / 32 + 1) * sizeof(TileOrigin))) return bad("torg");
    if (cudaMalloc(&e->ppart, (size_t)B * NGLOB * sizeof(double))) return bad("ppart");
    if (cudaMalloc(&e->fpart, (size_t)B * 8 * sizeof(double))) return bad("fpart");
    if (cudaMalloc(&e->glob, (size_t)nclusters * 16 * sizeof(double))) return bad("glob");
    if (cudaMalloc(&e->eout, (size_t)nclusters * 4 * sizeof(double))) return bad("eout");
    if (cudaMalloc(&e->tickets, (size_t)nclusters * 4 * sizeof(unsigned))) return bad("tickets");
    if (cudaMalloc(&e->counter, sizeof(unsigned))) return bad("counter");
    if (cudaMalloc(&e->err, sizeof(int))) return bad("err");
    if (cudaMalloc(&e->blockmap, (size_t)B * sizeof(int4))) return bad("blockmap");
    if (cudaMalloc(&e->t_prep, 2 * (size_t)nclusters * sizeof(PrepArgs))) return bad("tables");
    if (cudaMalloc(&e->t_fin, 4 * (size_t)nclusters * sizeof(FinishArgs))) return bad("tables");
    if (cudaMalloc(&e->t_en, (size_t)nclusters * sizeof(EnergyArgs))) return bad("tables");
    if (cudaMalloc(&e->t_pair, 2 * (size_t)nclusters * sizeof(PairArgs))) return bad("tables");
    if (cudaMemset(e->state, 0, 19 * ld * sizeof(double)) || cudaMemset(e->pack, 0, 6 * (size_t)S * 16) ||
        cudaMemset(e->tickets, 0, (size_t)nclusters * 4 * sizeof(unsigned)) || cudaMemset(e->err, 0, sizeof(int)))
        return bad("memset");
    if (cudaEventCreate(&e->e0) || cudaEventCreate(&e->e1)) return bad("events");
    std::vector<int4> bm(B);
    for (int c = 0; c < nclusters; ++c)
        for (int k = 0; k < e->nblk[c]; ++k) bm[e->blk0[c] + k] = make_int4(c, k, e->nblk[c], 0);
    if (cudaMemcpy(e->blockmap, bm.data(), (size_t)B * sizeof(int4), cudaMemcpyHostToDevice)) return bad("blockmap");
    int rc = ens_build_tables(e);
    if (rc) {
        ens_free(e);
        return rc;
    }
    *out = e;
    return PN_OK;
}

extern "C" int pn_ens_destroy(pn_ens *e) {
    if (!e) return PN_ERR_INVALID;
    cudaStreamSynchronize(e->stream);
    ens_free(e);
    return PN_OK;
}

extern "C" int pn_ens_set_state(pn_ens *e, const double *x, const double *v, const double *m) {
    if (!e || !x || !v || !m) return fail(PN_ERR_INVALID, "pn_ens_set_state");
    for (int c = 0; c < e->nc; ++c)
        if (!(m[e->p0[c]] > 0.0)) return fail(PN_ERR_INVALID, "BH mass must be > 0");
    const size_t ld = (size_t)e->LD;
    std::vector<double> h(7 * ld, 0.0);
    for (int p = 0; p < e->P; ++p) {
        for (int k = 0; k < 3; ++k) {
            h[k * ld + p] = x[3 * p + k];
            h[3 * ld + k * ld + p] = v[3 * p + k];
        }
        h[6 * ld + p] = m[p];
    }
    ECU(cudaMemcpyAsync(e->st.x, h.data(), 3 * ld * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    ECU(cudaMemcpyAsync(e->st.v, h.data() + 3 * ld, 3 * ld * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    ECU(cudaMemcpyAsync(e->st.m, h.data() + 6 * ld, ld * sizeof(double), cudaMemcpyHostToDevice, e->stream));
    ECU(cudaStreamSynchronize(e->stream));
    e->have_state = true;
    e->time = 0.0;
    return PN_OK;
}

extern "C" int pn_ens_get_state(pn_ens *e, double *x, double *v) {
    if (!e || !e->have_state) return fail(PN_ERR_STATE, "pn_ens_get_state");
    const size_t ld = (size_t)e->LD;
    std::vector<double> h(6 * ld);
    ECU(cudaMemcpyAsync(h.data(), e->st.x, 6 * ld * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    ECU(cudaStreamSynchronize(e->stream));
    for (int p = 0; p < e->P; ++p)
        for (int k = 0; k < 3; ++k) {
            if (x) x[3 * p + k] = h[k * ld + p];
            if (v) v[3 * p + k] = h[3 * ld + k * ld + p];
        }
    return PN_OK;
}

extern "C" int pn_ens_force(pn_ens *e, double *a) {
    if (!e || !e->have_state || !a) return fail(PN_ERR_STATE, "pn_ens_force");
    int rc = ens_eval(e, 0, 0, e->stream);
    if (rc) return rc;
    ECU(cudaMemcpyAsync(a, e->a_aos, 3 * (size_t)e->P * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    return ens_check(e);
}

static int ens_build_graph(pn_ens *e) {
    if (e->step_valid) return PN_OK;
    if (e->step_exec) {
        cudaGraphExecDestroy(e->step_exec);
        e->step_exec = nullptr;
    }
    cudaGraph_t g = nullptr;
    ECU(cudaStreamBeginCapture(e->stream, cudaStreamCaptureModeThreadLocal));
    int rc = ens_eval(e, 0, 1, e->stream);
    if (!rc) rc = ens_eval(e, 1, 2, e->stream);
    if (!rc) rc = ens_eval(e, 1, 3, e->stream);
    cudaError_t ec = cudaStreamEndCapture(e->stream, &g);
    if (rc) {
        if (g) cudaGraphDestroy(g);
        return rc;
    }
    if (ec != cudaSuccess) return fail(PN_ERR_CUDA, "capture", ec);
    cudaError_t ei = cudaGraphInstantiate(&e->step_exec, g, 0);
    cudaGraphDestroy(g);
    if (ei != cudaSuccess) return fail(PN_ERR_CUDA, "instantiate", ei);
    e->step_valid = true;
    return PN_OK;
}

extern "C" int pn_ens_steps(pn_ens *e, int nsteps) {
    if (!e || !e->have_state || nsteps < 0) return fail(PN_ERR_STATE, "pn_ens_steps");
    int rc = ens_build_graph(e);
    if (rc) return rc;
    for (int s = 0; s < nsteps; ++s) {
        ECU(cudaGraphLaunch(e->step_exec, e->stream));
        e->time += e->p.dt;
    }
    return PN_OK;
}

extern "C" int pn_ens_sync(pn_ens *e) {
    if (!e) return PN_ERR_INVALID;
    return ens_check(e);
}

extern "C" int pn_ens_bench_steps(pn_ens *e, int nsteps, double *step_ms) {
    if (!e || !e->have_state || nsteps < 0 || (nsteps && !step_ms)) return fail(PN_ERR_INVALID, "bench");
    int rc = ens_build_graph(e);
    if (rc) return rc;
    for (int s = 0; s < nsteps; ++s) {
        ECU(cudaEventRecord(e->e0, e->stream));
        ECU(cudaGraphLaunch(e->step_exec, e->stream));
        ECU(cudaEventRecord(e->e1, e->stream));
        ECU(cudaEventSynchronize(e->e1));
        float ms = 0.f;
        ECU(cudaEventElapsedTime(&ms, e->e0, e->e1));
        step_ms[s] = ms;
        e->time += e->p.dt;
    }
    return ens_check(e);
}

extern "C" int pn_ens_energy(pn_ens *e, double *out) {
    if (!e || !e->have_state || !out) return fail(PN_ERR_STATE, "pn_ens_energy");
    ECU(launch_prep_ens(e->t_prep, e->blockmap, e->B, e->stream));
    int rc = ens_pair_launch(e, MODE_ENERGY, e->t_pair + e->nc, e->stream);
    if (rc) return rc;
    ECU(launch_energy_ens(e->t_en, e->blockmap, e->B, e->stream));
    ECU(cudaMemcpyAsync(out, e->eout, (size_t)e->nc * 4 * sizeof(double), cudaMemcpyDeviceToHost, e->stream));
    return ens_check(e);
}

extern "C" double pn_ens_time(pn_ens *e) { return e ? e->time : 0.0; }
extern "C" int pn_ens_last_error(void) { return g_ens_err; }

extern "C" int pn_ens_set_shape(pn_ens *e, int ipt, int js, int size_class_, int tile_j, int tiles_per_item) {
    if (!e) return fail(PN_ERR_INVALID, "pn_ens_set_shape");
    if (ipt > 0 || js > 0) {
        if (!ens_shape_supported(ipt, js)) return fail(PN_ERR_INVALID, "shape");
        e->ipt = ipt;
        e->js = js;
        e->x2 = 0;  // an explicit shape selects the scalar sweep
    }
    if (size_class_ >= 0) {
        if (size_class_ > 31 || (tile_j != 32 && tile_j != 64 && tile_j != 128 && tile_j != 256) ||
            tiles_per_item < 1)
            return fail(PN_ERR_INVALID, "class shape");
        e->cls[size_class_].tj = tile_j;
        e->cls[size_class_].tiles_per_item = tiles_per_item;
    }
    return ens_build_tables(e);
}

// Chooses, per size class present, the j-tile size and work-item length (in tiles) that make
// that class's share of the persistent sweep fastest, then the (i per thread, lanes per i-set)
// of the launch.  Each candidate is timed on the live state with the class's items alone.
extern "C" int pn_ens_autotune(pn_ens *e) {
    if (!e || !e->have_state) return fail(PN_ERR_STATE, "pn_ens_autotune");
    const int mode = ens_mode(e);
    const bool f32 = ens_f32(e);
    std::vector<int> classes;
    for (int c = 0; c < e->nc; ++c) {
        int k = size_class(std::max(1, e->n[c] - 1));
        if (std::find(classes.begin(), classes.end(), k) == classes.end()) classes.push_back(k);
    }
    const int tjs32[] = {64, 128, 256}, tjs64[] = {64, 128, 256};
    const int tpis[] = {8, 16, 32, 64};
    auto time_sweep = [&](float *ms) -> int {
        ECU(launch_prep_ens(e->t_prep, e->blockmap, e->B, e->stream));
        ECU(cudaEventRecord(e->e0, e->stream));
        int rc = ens_pair_launch(e, mode, e->t_pair, e->stream);
        if (rc) return rc;
        ECU(cudaEventRecord(e->e1, e->stream));
        ECU(cudaEventSynchronize(e->e1));
        ECU(cudaEventElapsedTime(ms, e->e0, e->e1));
        return PN_OK;
    };
    // per class: the other classes keep their shape; only this class's items are timed by
    // restricting the item list to it
    for (int k : classes) {
        ClassShape best = e->cls[k];
        float best_ms = 1e30f;
        for (int q = 0; q < 3; ++q)
            for (int tpi : tpis) {
                e->cls[k].tj = f32 ? tjs32[q] : tjs64[q];
                e->cls[k].tiles_per_item = tpi;
                int rc = ens_build_tables(e);
                if (rc) return rc;
                // keep only class-k items
                std::vector<int4> all(e->nitems), mine;
                ECU(cudaMemcpy(all.data(), e->items, (size_t)e->nitems * sizeof(int4), cudaMemcpyDeviceToHost));
                for (auto &w : all)
                    if (size_class(std::max(1, e->n[w.x] - 1)) == k) mine.push_back(w);
                ECU(cudaMemcpy(e->items, mine.data(), mine.size() * sizeof(int4), cudaMemcpyHostToDevice));
                const int saved = e->nitems;
                e->nitems = (int)mine.size();
                float ms = 0.f, ms2 = 0.f;
                rc = time_sweep(&ms);
                if (!rc) rc = time_sweep(&ms2);
                e->nitems = saved;
                if (rc) return rc;
                ms = std::min(ms, ms2);
                if (ms < best_ms) {
                    best_ms = ms;
                    best = e->cls[k];
                }
            }
        e->cls[k] = best;
    }
    // launch-wide (ipt, js, packed)
    const int shapes[5][3] = {{1, 1, 0}, {2, 1, 0}, {1, 4, 0}, {1, 1, 1}, {2, 1, 1}};
    int bi = e->ipt, bj = e->js, bx = e->x2;
    float best_ms = 1e30f;
    for (auto &sh : shapes) {
        if (sh[2] && !(f32 && e->pack2)) continue;
        e->ipt = sh[0];
        e->js = sh[1];
        e->x2 = sh[2];
        int rc = ens_build_tables(e);
        if (rc) return rc;
        float ms = 0.f, ms2 = 0.f;
        rc = time_sweep(&ms);
        if (!rc) rc = time_sweep(&ms2);
        if (rc) return rc;
        ms = std::min(ms, ms2);
        if (ms < best_ms) {
            best_ms = ms;
            bi = sh[0];
            bj = sh[1];
            bx = sh[2];
        }
    }
    e->ipt = bi;
    e->js = bj;
    e->x2 = bx;
    int rc = ens_build_tables(e);
    if (rc) return rc;
    return ens_check(e);
}

extern "C" int pn_ens_get_shape(pn_ens *e, int size_class_, int *ipt, int *js, int *tile_j,
                                int *tiles_per_item) {
    if (!e || size_class_ < 0 || size_class_ > 31) return fail(PN_ERR_INVALID, "pn_ens_get_shape");
    if (ipt) *ipt = e->ipt;
    if (js) *js = e->js;
    if (tile_j) *tile_j = e->cls[size_class_].tj;
    if (tiles_per_item) *tiles_per_item = e->cls[size_class_].tiles_per_item;
    return PN_OK;
}
