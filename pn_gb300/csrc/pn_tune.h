// pn_tune.h -- the pair-sweep launch-shape table (see pn_tune.cu).
#pragma once

#include <vector>

#include "pn_internal.h"

namespace pn {

bool tune_lookup(int prec, int mode, int nstar, PairCfg *out);
void tune_store(int prec, int mode, int nstar, const PairCfg &cfg, double ms);
void tune_clear();
std::vector<PairCfg> tune_candidates(bool f32, int mode, int nstar, int sms);

}  // namespace pn
