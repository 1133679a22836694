// american_host.cu — thoth_gpu_price_american[_book]: Longstaff-Schwartz exercise of the
// American vanillas of a book and their Greeks, the steps of PricerMCL::PriceAmerican
// (pricer_mcl_american.cpp:137-261):
// - fit each contract's policy on the base paths and value it on them;
// - value the frozen policies on the paths of each bumped scenario;
// - refit on the book rolled one day for theta (the reference's theta is a full reprice,
//   pricer_mcl_greeks.cpp:220-276).
// A scenario is simulated once per asset that carries contracts, with that asset's spot stored
// on the device, and every contract on the asset is fitted or valued on the same stored paths
// (thoth_lsm_passes, thoth_gpu.cu; kernels in american.cu). Host code.
#include "thoth_gpu.h"
#include "american.cuh"
#include "scenario.hpp"

#include <cmath>
#include <cstring>
#include <map>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

using namespace thoth_scenario;

thread_local std::string g_aerr;

int afail(int code, const std::string& m)
{
    g_aerr = m;
    return code;
}

struct Contract {
    int product = 0, asset = 0, call = 0;
    double strike = 0, norm = 0;
    int min_itm = 50;
    std::vector<double> z; // zero rate of the premium currency at each date of the base book
};

// Vanilla::Intrinsic (vanilla.cpp:79-82): max(phi (S - K), 0)
double intrinsic(double s, const Contract& c)
{
    const double v = c.call ? s - c.strike : c.strike - s;
    return v < 0.0 ? 0.0 : v;
}

// The pass of contract c on book b with zero rates z per date of b. Discounting as the
// reference's fit and apply steps: a cashflow rolls back from date t+1 to t by
// exp(r_t tau_t - r_{t+1} tau_{t+1}); an exercise at t is worth exp(-r_t (tau_t - tau_0)) today.
LsmPass make_pass(const ThothBookDesc& b, const Contract& c, const std::vector<double>& z, const LsmPass* policy)
{
    const int M = b.products[c.product].maturity + 1;
    LsmPass io;
    io.asset = c.asset;
    io.M = M;
    io.call = c.call;
    io.strike = c.strike;
    io.norm = c.norm;
    io.min_itm = c.min_itm;
    io.fit = policy == nullptr;
    io.df.assign(M, 1.0);
    io.disc.assign(M, 1.0);
    for (int t = 0; t < M; t++) {
        io.disc[t] = std::exp(-z[t] * (b.t[t] - b.t[0]));
        if (t + 1 < M) io.df[t] = std::exp(z[t] * b.t[t] - z[t + 1] * b.t[t + 1]);
    }
    if (policy) {
        io.beta = policy->beta;
        io.fit_at = policy->fit_at;
    }
    return io;
}

struct Valued {
    double value = 0, trust = 0, euro = 0;
};

// ApplyAmericanPolicy's result from a finished pass: max(mean, intrinsic at the spot of
// date 0), and the standard error
Valued value_of(const LsmPass& io, const Contract& c)
{
    Valued v;
    const double n = (double)io.paths;
    const double mean = io.sum / n;
    v.trust = io.paths > 1 ? std::sqrt((io.sum2 / n - mean * mean) / (n - 1.0)) : 0.0;
    v.value = std::max(mean, intrinsic(io.s0, c));
    v.euro = io.euro / n;
    return v;
}

// Price contracts `which` (indices into cs) on book b, zero rates zs[i] per date of b: fit
// (policies null) or value the frozen policies. One simulation per asset. A contract whose
// maturity is today is worth 0, as in the reference's fit and apply steps.
int run_all(const ThothBookDesc& b, const std::vector<Contract>& cs, const std::vector<int>& which,
            const std::vector<std::vector<double>>& zs, const std::vector<LsmPass>* policies,
            std::vector<Valued>& out, std::vector<LsmPass>* keep, double& ms)
{
    std::map<int, std::vector<int>> by_asset;
    for (int i : which) {
        out[i] = Valued{};
        if (b.products[cs[i].product].maturity + 1 >= 2) by_asset[cs[i].asset].push_back(i);
    }
    for (auto& kv : by_asset) {
        std::vector<LsmPass> passes;
        passes.reserve(kv.second.size());
        for (int i : kv.second) passes.push_back(make_pass(b, cs[i], zs[i], policies ? &(*policies)[i] : nullptr));
        for (size_t k = 0; k < passes.size(); k++)
            if (!passes[k].fit && (int)passes[k].fit_at.size() != passes[k].M)
                return afail(THOTH_GPU_E_INVALID, "frozen policy on another exercise grid");
        const int rc = thoth_lsm_passes(&b, kv.first, passes.data(), (int)passes.size());
        if (rc) return afail(rc, thoth_gpu_last_error());
        for (size_t k = 0; k < passes.size(); k++) {
            const int i = kv.second[k];
            out[i] = value_of(passes[k], cs[i]);
            ms += passes[k].sim_ms + passes[k].lsm_ms;
            if (keep) (*keep)[i] = std::move(passes[k]);
        }
    }
    return THOTH_GPU_OK;
}

int price_american_book(const ThothBookDesc* book, ThothAmerican* am, int n)
{
    g_aerr.clear();
    if (!book || !am || n < 1) return afail(THOTH_GPU_E_INVALID, "null argument");
    if (book->n_dates < 1 || !book->t || book->n_assets < 1 || !book->assets || book->n_products < 1 ||
        !book->products)
        return afail(THOTH_GPU_E_INVALID, "bad descriptor");
    const int nd = book->n_dates;
    std::vector<Contract> cs(n);
    for (int i = 0; i < n; i++) {
        if (am[i].product < 0 || am[i].product >= book->n_products)
            return afail(THOTH_GPU_E_INVALID, "product out of range");
        const ThothProduct& P = book->products[am[i].product];
        if (P.kind != THOTH_PRODUCT_VANILLA)
            return afail(THOTH_GPU_E_UNSUPPORTED, "American exercise is for vanilla products");
        if (P.quanto != 0.0) return afail(THOTH_GPU_E_UNSUPPORTED, "American exercise of a quanto product");
        if (P.asset < 0 || P.asset >= book->n_assets) return afail(THOTH_GPU_E_INVALID, "asset out of range");
        if (P.maturity < 0 || P.maturity >= nd) return afail(THOTH_GPU_E_INVALID, "maturity out of range");
        if (P.option_type != THOTH_CALL && P.option_type != THOTH_PUT)
            return afail(THOTH_GPU_E_INVALID, "bad option type");
        Contract& c = cs[i];
        c.product = am[i].product;
        c.asset = P.asset;
        c.call = P.option_type == THOTH_CALL;
        c.strike = P.strike;
        // Vanilla::LsmBasisNorm (vanilla.hpp:38-41): the strike, else the paths' spot at date 0
        // (stored in single precision)
        c.norm = P.strike > 0 ? P.strike : (double)(float)book->assets[P.asset].spot;
        c.min_itm = am[i].min_itm > 0 ? am[i].min_itm : 50;
        c.z.resize(nd);
        for (int k = 0; k < nd; k++) c.z[k] = am[i].zero_rates ? am[i].zero_rates[k] : P.zero_rate;
        const double nan = std::nan("");
        am[i].premium = am[i].trust = am[i].european = nan;
        am[i].delta = am[i].gamma = am[i].vega = am[i].rho = am[i].theta = nan;
        am[i].fitted_dates = 0;
        am[i].device_ms = am[i].exercise_ms = 0;
    }
    std::vector<std::vector<double>> zbase(n);
    for (int i = 0; i < n; i++) zbase[i] = cs[i].z;
    double ms = 0;
    const double nan = std::nan("");

    // base: fit every policy and value it on the same paths
    std::vector<int> all(n);
    for (int i = 0; i < n; i++) all[i] = i;
    std::vector<Valued> base(n);
    std::vector<LsmPass> pol(n);
    int rc = run_all(*book, cs, all, zbase, nullptr, base, &pol, ms);
    if (rc) return rc;
    double fit_ms = 0;
    for (int i = 0; i < n; i++) fit_ms += pol[i].lsm_ms;
    for (int i = 0; i < n; i++) {
        const int M = book->products[cs[i].product].maturity + 1;
        am[i].premium = base[i].value;
        am[i].trust = base[i].trust;
        am[i].european = base[i].euro;
        am[i].exercise_ms = fit_ms;
        if (M >= 2)
            for (int t = 0; t < M; t++) am[i].fitted_dates += pol[i].fit_at[t] ? 1 : 0;
        if (am[i].beta)
            for (int t = 0; t < nd; t++)
                for (int k = 0; k < 3; k++)
                    am[i].beta[3 * t + k] =
                        (M >= 2 && t < M && pol[i].fit_at[t]) ? pol[i].beta[3 * (size_t)t + k] : nan;
    }
    auto wants = [&](int flag) {
        std::vector<int> w;
        for (int i = 0; i < n; i++)
            if (am[i].flags & flag) w.push_back(i);
        return w;
    };
    std::vector<Valued> sc(n);

    // delta and gamma: the frozen policies on the paths of each bumped asset
    const std::vector<int> wd = wants(THOTH_BUMP_DELTA), wg = wants(THOTH_BUMP_GAMMA);
    auto spot_bump = [&](int a, double h, const std::vector<int>& on, std::vector<Valued>& v) -> int {
        Scenario s(*book);
        s.assets[a].spot *= 1.0 + h;
        return run_all(s.d, cs, on, zbase, &pol, v, nullptr, ms);
    };
    for (int a = 0; a < book->n_assets; a++) {
        std::vector<int> d_on, g_on;
        for (int i : wd)
            if (cs[i].asset == a) d_on.push_back(i);
        for (int i : wg)
            if (cs[i].asset == a) g_on.push_back(i);
        const double S = book->assets[a].spot;
        if (!d_on.empty()) {
            if ((rc = spot_bump(a, SPOT_BUMP, d_on, sc))) return rc;
            for (int i : d_on) am[i].delta = (sc[i].value - base[i].value) / (SPOT_BUMP * S);
        }
        if (!g_on.empty()) {
            std::vector<Valued> dn(n);
            if ((rc = spot_bump(a, GAMMA_BUMP, g_on, sc))) return rc;
            if ((rc = spot_bump(a, -GAMMA_BUMP, g_on, dn))) return rc;
            for (int i : g_on)
                am[i].gamma = (sc[i].value - 2.0 * base[i].value + dn[i].value) / ((GAMMA_BUMP * S) * (GAMMA_BUMP * S));
        }
    }
    const std::vector<int> wv = wants(THOTH_BUMP_VEGA);
    if (!wv.empty()) {
        Scenario s(*book);
        vol_shift(s, VOL_BUMP);
        if ((rc = run_all(s.d, cs, wv, zbase, &pol, sc, nullptr, ms))) return rc;
        for (int i : wv) am[i].vega = sc[i].value - base[i].value;
    }
    const std::vector<int> wr = wants(THOTH_BUMP_RHO);
    if (!wr.empty()) {
        // the rho scenario drifts and discounts at the bumped curve (pricer_mcl_american.cpp:218-226)
        Scenario s(*book);
        rate_shift(s, RATE_BUMP);
        std::vector<std::vector<double>> zr(zbase);
        for (auto& z : zr)
            for (double& x : z) x += RATE_BUMP;
        if ((rc = run_all(s.d, cs, wr, zr, &pol, sc, nullptr, ms))) return rc;
        for (int i : wr) am[i].rho = (sc[i].value - base[i].value) / RATE_BUMP * 0.01;
    }
    const std::vector<int> wt = wants(THOTH_BUMP_THETA);
    if (!wt.empty()) {
        Scenario s(*book);
        std::string why;
        if (!roll_one_day(s, *book, why)) {
            g_aerr = "theta: " + why;
        } else {
            // the same calendar dates keep their zero rates
            const int sh = s.d.n_dates < nd ? 1 : 0;
            std::vector<std::vector<double>> zt(n);
            for (int i : wt) {
                zt[i].resize(s.d.n_dates);
                for (int k = 0; k < s.d.n_dates; k++) zt[i][k] = cs[i].z[k == 0 ? sh : k + sh];
            }
            if ((rc = run_all(s.d, cs, wt, zt, nullptr, sc, nullptr, ms))) return rc;
            for (int i : wt) am[i].theta = sc[i].value - base[i].value;
        }
    }
    for (int i = 0; i < n; i++) am[i].device_ms = ms;
    return THOTH_GPU_OK;
}

} // namespace

extern "C" {

int thoth_gpu_price_american_book(const ThothBookDesc* book, ThothAmerican* am, int32_t n)
{
    try {
        return price_american_book(book, am, n);
    } catch (const std::bad_alloc&) {
        return afail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return afail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

int thoth_gpu_price_american(const ThothBookDesc* book, ThothAmerican* am)
{
    return thoth_gpu_price_american_book(book, am, 1);
}

const char* thoth_gpu_american_last_error(void) { return g_aerr.c_str(); }

} // extern "C"
