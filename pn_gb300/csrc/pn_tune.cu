// pn_tune.cu -- launch-shape autotuner of the pair sweep.
//
// A shape is (i per thread, lanes per i-set, j-tile size, j-range splits).  The tuner times a
// candidate list on real data (CUDA events; the force sweep as a whole evaluation, so that the
// cost of reading back many j-range partial sums counts, the energy sweep as its pair launch;
// one warm-up per shape) and keeps the fastest per key (precision, sweep mode, size class =
// floor(log2 N)).
// Results live in a process-wide table; with PN_TUNE_CACHE=<file> they are also read from and
// appended to a text file ("prec mode class ipt js tj gsplit x2 ms" per line), so a tuned
// shape is reused by later runs.  x2 = 1 selects the packed f32x2 sweep (pn_pair2.cuh).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <mutex>
#include <vector>

#include "pn_tune.h"

namespace pn {

namespace {
struct Entry {
    int prec, mode, cls;
    PairCfg cfg;
    double ms;
};
std::mutex g_mu;
std::vector<Entry> g_table;
bool g_loaded = false;

int size_class(int nstar) {
    int c = 0;
    while ((1 << (c + 1)) <= nstar) ++c;
    return c;
}

void load_file_locked() {
    if (g_loaded) return;
    g_loaded = true;
    const char *path = getenv("PN_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "r");
    if (!f) return;
    Entry e{};
    while (fscanf(f, "%d %d %d %d %d %d %d %d %lf", &e.prec, &e.mode, &e.cls, &e.cfg.ipt, &e.cfg.js,
                  &e.cfg.tj, &e.cfg.gsplit, &e.cfg.x2, &e.ms) == 9) {
        if (pair_shape_supported(e.cfg.ipt, e.cfg.js) && e.cfg.gsplit >= 1 && e.cfg.gsplit <= 64 &&
            (e.cfg.tj == 32 || e.cfg.tj == 64 || e.cfg.tj == 128 || e.cfg.tj == 256) &&
            (e.cfg.x2 == 0 || (e.cfg.x2 == 1 && e.cfg.js == 1 && e.cfg.ipt <= 2 && e.prec == 1) ||
             ((e.cfg.x2 == 2 || e.cfg.x2 == 3) && e.cfg.js == 1 && e.cfg.ipt == 2 && e.prec == 1)))
            g_table.push_back(e);
    }
    fclose(f);
}

void append_file_locked(const Entry &e) {
    const char *path = getenv("PN_TUNE_CACHE");
    if (!path) return;
    FILE *f = fopen(path, "a");
    if (!f) return;
    fprintf(f, "%d %d %d %d %d %d %d %d %.6f\n", e.prec, e.mode, e.cls, e.cfg.ipt, e.cfg.js, e.cfg.tj,
            e.cfg.gsplit, e.cfg.x2, e.ms);
    fclose(f);
}
}  // namespace

bool tune_lookup(int prec, int mode, int nstar, PairCfg *out) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_file_locked();
    const int cls = size_class(nstar);
    for (auto it = g_table.rbegin(); it != g_table.rend(); ++it)
        if (it->prec == prec && it->mode == mode && it->cls == cls) {
            *out = it->cfg;
            return true;
        }
    return false;
}

void tune_store(int prec, int mode, int nstar, const PairCfg &cfg, double ms) {
    std::lock_guard<std::mutex> lk(g_mu);
    load_file_locked();
    Entry e{prec, mode, size_class(nstar), cfg, ms};
    g_table.push_back(e);
    append_file_locked(e);
}

void tune_clear() {
    std::lock_guard<std::mutex> lk(g_mu);
    g_table.clear();
    g_loaded = true;  // do not re-read the file after an explicit clear
}

std::vector<PairCfg> tune_candidates(bool f32, int mode, int nstar, int sms) {
    // Large systems: only the shapes that can win there (several i per thread, long tiles);
    // small systems: every shape, including lanes splitting j within a warp.
    std::vector<PairCfg> out;
    const bool big = nstar >= 65536;
    const int shapes_big32[][2] = {{1, 1}, {2, 1}, {4, 1}};
    const int shapes_big64[][2] = {{1, 1}, {1, 2}, {1, 4}};  // FP64: lanes splitting j win
    const int shapes_all[][2] = {{1, 1}, {2, 1}, {4, 1}, {1, 2}, {1, 4}, {1, 8}};
    const int nsh = big ? 3 : 6;
    const int tjs32[] = {64, 128, 256}, tjs64[] = {32, 64, 128};
    const int gs[] = {1, 2, 4, 8, 16, 32};
    for (int s = 0; s < nsh; ++s) {
        const int (*tab)[2] = big ? (f32 ? shapes_big32 : shapes_big64) : shapes_all;
        const int ipt = tab[s][0];
        const int js = tab[s][1];
        if (!f32 && ipt == 4) continue;  // FP64 pair terms: register-bound at 4 i per thread
        for (int q = big ? 1 : 0; q < 3; ++q) {
            PairCfg c;
            c.ipt = ipt;
            c.js = js;
            c.tj = f32 ? tjs32[q] : tjs64[q];
            const int ntiles = (nstar + c.tj - 1) / c.tj;
            for (int g : gs) {
                if (g > 1 && g > ntiles / 4) break;  // keep >= 4 tiles per j-range
                // large systems: at most 8 j-range splits; more saved < 0.3 % of the sweep (ncu
                // launch list at N = 2^18) and cost 72 B per star and split of partial sums
                if (big && g > 8) break;
                c.gsplit = g;
                c.x2 = 0;
                // large mixed-precision systems: the packed sweep only (the scalar one measured
                // 15-20 % slower there at every shape)
                if (!(f32 && big)) out.push_back(c);
                if (f32 && js == 1 && ipt <= 2) {  // the packed f32x2 sweep of the same shape
                    c.x2 = 1;
                    out.push_back(c);
                    if (ipt == 2 && mode != MODE_ENERGY) {  // ... sized for 3 and 4 CTAs per SM
                        c.x2 = 2;
                        out.push_back(c);
                        c.x2 = 3;
                        out.push_back(c);
                    }
                }
            }
        }
    }
    (void)sms;
    return out;
}

}  // namespace pn
