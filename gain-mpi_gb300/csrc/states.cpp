// Host-side state selection: the rules of BaseClasses/States.cpp, over a plain state table,
// and the block-pair plan that feeds the batched engine.
#include <algorithm>
#include <cmath>
#include <cstdlib>
#include <map>
#include <tuple>
#include <vector>

#include "gain_internal.h"

namespace {

bool isym_do(const gain_filters* f, int g) { return f->gns[g] >= 1e-15; }   // TroveInput.cpp:300-304

// States.cpp:46-49
bool filter_lower(const gain_filters* f, double energy, int g) {
    return (energy - f->zpe) <= f->erange_lower[1] && (energy - f->zpe) >= f->erange_lower[0] && isym_do(f, g);
}
// States.cpp:50-53
bool filter_upper(const gain_filters* f, double energy, int g) {
    return (energy - f->zpe) <= f->erange_upper[1] && (energy - f->zpe) >= f->erange_upper[0] && isym_do(f, g);
}

// the conditions of States.cpp:54-76 that depend on the two states' blocks only
bool block_pair_ok(const gain_filters* f, int jI, int gI, int jF, int gF) {
    return f->gns[gI] > 0.0 && f->gns[gF] > 0.0 && (jF != f->maxJ || jI != f->maxJ) &&
           f->isym_pairs[gI] == f->isym_pairs[gF] && f->igamma_pair[gI] == gF && std::abs(jF - jI) <= 1 &&
           jI + jF >= 1;
}

bool valid_filters(const gain_filters* f) {
    return f && f->nsym > 0 && f->gns && f->isym_pairs && f->igamma_pair && f->sym_degen;
}

bool valid_state(const gain_filters* f, const gain_state* s) {
    return s && s->gamma >= 0 && s->gamma < f->nsym;
}

}  // namespace

extern "C" {

int gain_filter_lower(const gain_filters* f, const gain_state* I) {
    if (!valid_filters(f) || !valid_state(f, I)) return 0;
    return filter_lower(f, I->energy, I->gamma);
}

int gain_filter_intensity(const gain_filters* f, const gain_state* I, const gain_state* F) {
    if (!valid_filters(f) || !valid_state(f, I) || !valid_state(f, F)) return 0;
    const double nu = F->energy - I->energy;
    return f->gns[I->gamma] > 0.0 && f->gns[F->gamma] > 0.0 && nu >= f->freq_window[0] &&
           nu <= f->freq_window[1] && filter_lower(f, I->energy, I->gamma) &&
           filter_upper(f, F->energy, F->gamma) && (F->J != f->maxJ || I->J != f->maxJ) &&
           f->isym_pairs[I->gamma] == f->isym_pairs[F->gamma] && f->igamma_pair[I->gamma] == F->gamma &&
           std::abs(F->J - I->J) <= 1 && I->J + F->J >= 1;
}

int gain_degeneracy_filter(const gain_filters* f, int gammaI, int gammaF, int idegI, int idegF) {
    if (!valid_filters(f) || gammaI < 0 || gammaI >= f->nsym || gammaF < 0 || gammaF >= f->nsym) return 0;
    if (f->sym_degen[gammaI] == 1 || f->sym_degen[gammaF] == 1) return 1;
    if (!f->reduced) return 1;
    if (f->symmetry_type == 1) return 1;
    if (f->symmetry_type == 2) return idegI == 1 && idegF == 0;
    if (f->symmetry_type == 3) {
        if (gammaI == 3 && gammaF == 4 && idegI == 1 && idegF == 0) return 1;
        if (gammaI == 4 && gammaF == 3 && idegI == 2 && idegF == 0) return 1;
        if (gammaI == 2 && gammaF == 2 && idegI == 1 && idegF == 0) return 1;
    }
    return 0;
}

gain_status gain_transition_details(const gain_filters* f, const gain_state* st, int n, int* num_initial,
                                    long long* num_trans, int* max_trans) {
    gain::clear_error();
    if (!valid_filters(f) || (n > 0 && !st) || n < 0 || !num_initial || !num_trans || !max_trans)
        return gain::set_error(GAIN_ERR_INVALID_ARG, "gain_transition_details: bad argument");
    for (int i = 0; i < n; ++i)
        if (!valid_state(f, &st[i])) return gain::set_error(GAIN_ERR_INVALID_ARG, "state %d has a bad Gamma", i);
    int ninit = 0, mx = 0;
    long long total = 0;
    for (int i = 0; i < n; ++i) {
        if (!filter_lower(f, st[i].energy, st[i].gamma)) continue;
        int per = 0;
        for (int j = 0; j < n; ++j)
            if (gain_filter_intensity(f, &st[i], &st[j])) ++per;
        total += per;
        mx = std::max(mx, per);
        ++ninit;
    }
    *num_initial = ninit;
    *num_trans = total;
    *max_trans = mx;
    return GAIN_OK;
}

gain_status gain_plan_pairs(const gain_filters* f, const gain_state* st, int n, int* n_pairs, int* pairs,
                            int* offs, long long* n_levels, int* levels) {
    gain::clear_error();
    if (!valid_filters(f) || (n > 0 && !st) || n < 0 || !n_pairs || !n_levels)
        return gain::set_error(GAIN_ERR_INVALID_ARG, "gain_plan_pairs: bad argument");
    // per block: lower-eligible and upper-eligible levels, in energy (table) order
    std::map<std::pair<int, int>, std::vector<int>> low, up;
    std::map<std::pair<int, int>, int> Jof;
    for (int i = 0; i < n; ++i) {
        const gain_state& s = st[i];
        if (!valid_state(f, &s)) return gain::set_error(GAIN_ERR_INVALID_ARG, "state %d has a bad Gamma", i);
        const auto key = std::make_pair(s.jind, s.gamma);
        Jof[key] = s.J;
        if (filter_lower(f, s.energy, s.gamma)) low[key].push_back(s.ilevel);
        if (filter_upper(f, s.energy, s.gamma)) up[key].push_back(s.ilevel);
    }
    std::vector<std::tuple<int, int, int, int>> plan;
    long long total = 0;
    for (auto& lk : low)
        for (auto& uk : up) {
            const int jI = Jof[lk.first], jF = Jof[uk.first];
            if (lk.second.empty() || uk.second.empty()) continue;
            if (!block_pair_ok(f, jI, lk.first.second, jF, uk.first.second)) continue;
            plan.emplace_back(lk.first.first, lk.first.second, uk.first.first, uk.first.second);
            total += (long long)lk.second.size() + (long long)uk.second.size();
        }
    *n_pairs = (int)plan.size();
    *n_levels = total;
    if (!pairs) return GAIN_OK;
    if (!offs || !levels) return gain::set_error(GAIN_ERR_INVALID_ARG, "gain_plan_pairs: NULL output arrays");
    long long pos = 0;
    for (size_t p = 0; p < plan.size(); ++p) {
        int a, b, c, d;
        std::tie(a, b, c, d) = plan[p];
        pairs[4 * p] = a;
        pairs[4 * p + 1] = b;
        pairs[4 * p + 2] = c;
        pairs[4 * p + 3] = d;
        const auto& L = low[{a, b}];
        const auto& U = up[{c, d}];
        offs[2 * p] = (int)pos;
        for (int l : L) levels[pos++] = l;
        offs[2 * p + 1] = (int)pos;
        for (int u : U) levels[pos++] = u;
    }
    offs[2 * plan.size()] = (int)pos;
    return GAIN_OK;
}

}  // extern "C"
