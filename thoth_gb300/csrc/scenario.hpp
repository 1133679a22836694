// scenario.hpp — bumped and rolled variants of a book for the bump-and-revalue Greeks
// (greeks.cu) and the American exercise Greeks (american_host.cu): the reference's bump
// definitions (pricer.hpp:20-30, constants.hpp:36, pricer_mcl_greeks.cpp:43-299,
// heston_volatility.hpp Shifted). Host code.
#pragma once

#include "thoth_gpu.h"

#include <algorithm>
#include <cmath>
#include <string>
#include <vector>

namespace thoth_scenario {

constexpr double SPOT_BUMP = 0.01;   // delta: S -> S (1 + 0.01), one-sided
constexpr double GAMMA_BUMP = 0.10;  // gamma: S -> S (1 +/- 0.10), central
constexpr double VOL_BUMP = 0.01;    // vega: one vol point
constexpr double RATE_BUMP = 0.0001; // rho: one basis point
constexpr double PARAM_BUMP = 0.01;  // vega_<param>: additive on the Heston parameter

// one priced variant of the caller's book; it owns every array it changes and
// points at the caller's arrays for the rest
struct Scenario {
    ThothBookDesc d{};
    std::vector<ThothAsset> assets;
    std::vector<ThothProduct> products;
    std::vector<std::vector<double>> carry, lev_step, lev_vals;
    std::vector<std::vector<int64_t>> lev_off;
    std::vector<std::vector<int32_t>> mon, obs;
    std::vector<int32_t> days;
    std::vector<double> t;
    std::vector<double> premium;
    ThothBookResult r{};

    explicit Scenario(const ThothBookDesc& base)
        : d(base), assets(base.assets, base.assets + base.n_assets),
          products(base.products, base.products + base.n_products)
    {
        relink();
    }
    Scenario(const Scenario&) = delete;
    void relink()
    {
        d.assets = assets.data();
        d.products = products.data();
    }
};

inline bool is_heston(const ThothAsset& a) { return a.model == THOTH_MODEL_HESTON || a.model == THOTH_MODEL_LSV; }

// every asset's vol level one point up: GBM sigma + 0.01; Heston / LSV v0 and
// theta -> (sqrt(v) + 0.01)^2 (heston_volatility.hpp, Shifted); leverage kept
inline void vol_shift(Scenario& s, double h)
{
    for (ThothAsset& a : s.assets) {
        if (a.model == THOTH_MODEL_GBM) {
            a.vol += h;
        } else {
            const double sv0 = std::sqrt(a.v0) + h, sth = std::sqrt(a.theta) + h;
            a.v0 = sv0 * sv0;
            a.theta = sth * sth;
        }
    }
}

// every curve one basis point up: the carry to each date and each zero rate
inline void rate_shift(Scenario& s, double h)
{
    const int nd = s.d.n_dates;
    s.carry.resize(s.assets.size());
    for (size_t a = 0; a < s.assets.size(); a++) {
        s.carry[a].assign(s.assets[a].carry, s.assets[a].carry + nd);
        for (double& c : s.carry[a]) c += h;
        s.assets[a].carry = s.carry[a].data();
    }
    for (ThothProduct& p : s.products) p.zero_rate += h;
}

// today rolled one calendar day forward (the theta reprice). With date 1 one
// day after today, date 1 becomes today: every date index moves down by one and
// observations on today drop out; otherwise today+1 is the new date 0 in front
// of the same future dates. Carries are re-based to the new today, flat before
// the first date; zero rates are kept (flat curves). Needs days.
inline bool roll_one_day(Scenario& s, const ThothBookDesc& b, std::string& why)
{
    if (!b.days) {
        why = "theta needs the calendar days of the dates";
        return false;
    }
    const int nd = b.n_dates;
    const bool drop = nd >= 3 && b.days[1] == b.days[0] + 1;
    if (!drop && b.days[1] < b.days[0] + 2) {
        why = "date 1 must lie at least one day after today";
        return false;
    }
    const int sh = drop ? 1 : 0; // old index = new index + sh (new index >= 1)
    const int nn = nd - sh;
    s.days.resize(nn);
    s.t.resize(nn);
    for (int i = 0; i < nn; i++) {
        s.days[i] = i == 0 ? 0 : b.days[i + sh] - b.days[0] - 1;
        s.t[i] = s.days[i] / 365.0;
    }
    s.d.n_dates = nn;
    s.d.days = s.days.data();
    s.d.t = s.t.data();
    const double t1 = 1.0 / 365.0;
    s.carry.resize(s.assets.size());
    s.lev_step.resize(s.assets.size());
    s.lev_off.resize(s.assets.size());
    s.lev_vals.resize(s.assets.size());
    for (size_t a = 0; a < s.assets.size(); a++) {
        ThothAsset& A = s.assets[a];
        const double c1 = A.carry[1]; // carry to today + 1: date 1's (flat before date 1)
        std::vector<double>& c = s.carry[a];
        c.resize(nn);
        for (int i = 0; i < nn; i++) {
            const int o = i == 0 ? (drop ? 1 : 0) : i + sh;
            const double T = b.t[o];
            c[i] = i == 0 ? c1 : (A.carry[o] * T - c1 * t1) / s.t[i];
        }
        A.carry = c.data();
        if (A.model == THOTH_MODEL_LSV && A.lev_points > 0) {
            s.lev_step[a].assign(A.lev_ln_step + sh, A.lev_ln_step + nd);
            s.lev_off[a].assign(A.lev_offset + sh, A.lev_offset + nd);
            s.lev_vals[a].assign(A.lev_values + (size_t)sh * A.lev_points, A.lev_values + (size_t)nd * A.lev_points);
            A.lev_ln_step = s.lev_step[a].data();
            A.lev_offset = s.lev_off[a].data();
            A.lev_values = s.lev_vals[a].data();
        }
    }
    s.mon.resize(s.products.size());
    s.obs.resize(s.products.size());
    for (size_t p = 0; p < s.products.size(); p++) {
        ThothProduct& P = s.products[p];
        P.maturity = std::max(P.maturity - sh, 0);
        if (P.n_monitor > 0 && P.monitor) {
            for (int k = 0; k < P.n_monitor; k++)
                if (P.monitor[k] - sh >= 0) s.mon[p].push_back(P.monitor[k] - sh);
            P.n_monitor = (int32_t)s.mon[p].size();
            P.monitor = s.mon[p].data();
        }
        if (P.n_obs > 0 && P.obs) {
            for (int k = 0; k < P.n_obs; k++)
                if (P.obs[k] - sh > 0) s.obs[p].push_back(P.obs[k] - sh);
            P.n_obs = (int32_t)s.obs[p].size();
            P.obs = s.obs[p].empty() ? nullptr : s.obs[p].data();
        }
        if (P.total_year_fraction > 0) P.total_year_fraction = std::max(P.total_year_fraction - t1, 0.0);
    }
    return true;
}

} // namespace thoth_scenario
