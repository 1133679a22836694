// american_host.cu — thoth_gpu_price_american: Longstaff-Schwartz exercise of one vanilla of a
// book and its Greeks, the steps of PricerMCL::PriceAmerican (pricer_mcl_american.cpp:137-261):
// fit the policy on the base paths, value it on them, value the frozen policy on the paths of
// each bumped scenario, and refit on the book rolled one day for theta (the reference's theta
// is a full reprice, pricer_mcl_greeks.cpp:220-276). Each pass simulates the book into device
// memory and runs one exercise kernel (american.cu) through thoth_lsm_pass. Host code.
#include "thoth_gpu.h"
#include "american.cuh"
#include "scenario.hpp"

#include <cmath>
#include <cstring>
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
};

// Vanilla::Intrinsic (vanilla.cpp:79-82): max(phi (S - K), 0)
double intrinsic(double s, const Contract& c)
{
    const double v = c.call ? s - c.strike : c.strike - s;
    return v < 0.0 ? 0.0 : v;
}

// One pass on book b (its dates and the contract's maturity there) with zero rates z per
// date. Discounting as the reference's fit and apply steps: a cashflow rolls back from
// date t+1 to t by exp(r_t tau_t - r_{t+1} tau_{t+1}); an exercise at t is worth
// exp(-r_t (tau_t - tau_0)) today.
int run_pass(const ThothBookDesc& b, const Contract& c, const std::vector<double>& z, bool fit,
             const LsmPass* policy, double& value, double& trust, double* euro, LsmPass* keep, double& ms)
{
    const int M = b.products[c.product].maturity + 1;
    if (M < 2) { // maturity today: the reference's fit and apply steps return 0
        value = trust = 0.0;
        if (euro) *euro = 0.0;
        return THOTH_GPU_OK;
    }
    LsmPass io;
    io.asset = c.asset;
    io.M = M;
    io.call = c.call;
    io.strike = c.strike;
    io.norm = c.norm;
    io.min_itm = c.min_itm;
    io.fit = fit;
    io.df.assign(M, 1.0);
    io.disc.assign(M, 1.0);
    for (int t = 0; t < M; t++) {
        io.disc[t] = std::exp(-z[t] * (b.t[t] - b.t[0]));
        if (t + 1 < M) io.df[t] = std::exp(z[t] * b.t[t] - z[t + 1] * b.t[t + 1]);
    }
    if (!fit) {
        io.beta = policy->beta;
        io.fit_at = policy->fit_at;
        if ((int)io.fit_at.size() != M) return afail(THOTH_GPU_E_INVALID, "frozen policy on another exercise grid");
    }
    const int rc = thoth_lsm_pass(&b, io);
    if (rc) return afail(rc, thoth_gpu_last_error());
    const double n = (double)io.paths;
    const double mean = io.sum / n;
    trust = io.paths > 1 ? std::sqrt((io.sum2 / n - mean * mean) / (n - 1.0)) : 0.0;
    value = std::max(mean, intrinsic(io.s0, c));
    if (euro) *euro = io.euro / n;
    ms += io.sim_ms + io.lsm_ms;
    if (keep) *keep = std::move(io);
    return THOTH_GPU_OK;
}

int price_american(const ThothBookDesc* book, ThothAmerican* am)
{
    g_aerr.clear();
    if (!book || !am) return afail(THOTH_GPU_E_INVALID, "null argument");
    if (book->n_dates < 1 || !book->t || book->n_assets < 1 || !book->assets || book->n_products < 1 ||
        !book->products)
        return afail(THOTH_GPU_E_INVALID, "bad descriptor");
    if (am->product < 0 || am->product >= book->n_products) return afail(THOTH_GPU_E_INVALID, "product out of range");
    const ThothProduct& P = book->products[am->product];
    if (P.kind != THOTH_PRODUCT_VANILLA)
        return afail(THOTH_GPU_E_UNSUPPORTED, "American exercise is for vanilla products");
    if (P.quanto != 0.0) return afail(THOTH_GPU_E_UNSUPPORTED, "American exercise of a quanto product");
    if (P.asset < 0 || P.asset >= book->n_assets) return afail(THOTH_GPU_E_INVALID, "asset out of range");
    if (P.maturity < 0 || P.maturity >= book->n_dates) return afail(THOTH_GPU_E_INVALID, "maturity out of range");
    if (P.option_type != THOTH_CALL && P.option_type != THOTH_PUT) return afail(THOTH_GPU_E_INVALID, "bad option type");
    const int nd = book->n_dates;
    Contract c;
    c.product = am->product;
    c.asset = P.asset;
    c.call = P.option_type == THOTH_CALL;
    c.strike = P.strike;
    // Vanilla::LsmBasisNorm (vanilla.hpp:38-41): the strike, else the paths' spot at date 0
    // (stored in single precision)
    c.norm = P.strike > 0 ? P.strike : (double)(float)book->assets[P.asset].spot;
    c.min_itm = am->min_itm > 0 ? am->min_itm : 50;
    std::vector<double> z(nd);
    for (int i = 0; i < nd; i++) z[i] = am->zero_rates ? am->zero_rates[i] : P.zero_rate;

    const double nan = std::nan("");
    am->premium = am->trust = am->european = nan;
    am->delta = am->gamma = am->vega = am->rho = am->theta = nan;
    am->fitted_dates = 0;
    am->device_ms = am->exercise_ms = 0;
    double ms = 0;

    LsmPass base;
    double A0, t0, eu;
    int rc = run_pass(*book, c, z, true, nullptr, A0, t0, &eu, &base, ms);
    if (rc) return rc;
    am->premium = A0;
    am->trust = t0;
    am->european = eu;
    am->exercise_ms = base.lsm_ms;
    const int M = P.maturity + 1;
    if (am->beta)
        for (int t = 0; t < nd; t++)
            for (int k = 0; k < 3; k++)
                am->beta[3 * t + k] = (M >= 2 && t < M && base.fit_at[t]) ? base.beta[3 * (size_t)t + k] : nan;
    if (M >= 2)
        for (int t = 0; t < M; t++) am->fitted_dates += base.fit_at[t] ? 1 : 0;

    const int f = am->flags;
    const double S = book->assets[c.asset].spot;
    double tr;
    // frozen policy on the paths of a bumped copy of the book
    auto frozen = [&](Scenario& s, const std::vector<double>& zs, double& v) -> int {
        if (M < 2) {
            v = 0.0;
            return THOTH_GPU_OK;
        }
        return run_pass(s.d, c, zs, false, &base, v, tr, nullptr, nullptr, ms);
    };
    auto spot_bump = [&](double h, double& v) -> int {
        Scenario s(*book);
        s.assets[c.asset].spot *= 1.0 + h;
        return frozen(s, z, v);
    };
    if (f & (THOTH_BUMP_DELTA | THOTH_BUMP_GAMMA)) {
        double up = 0;
        if (f & THOTH_BUMP_DELTA) {
            if ((rc = spot_bump(SPOT_BUMP, up))) return rc;
            am->delta = (up - A0) / (SPOT_BUMP * S);
        }
        if (f & THOTH_BUMP_GAMMA) {
            double gu, gd;
            if ((rc = spot_bump(GAMMA_BUMP, gu))) return rc;
            if ((rc = spot_bump(-GAMMA_BUMP, gd))) return rc;
            am->gamma = (gu - 2.0 * A0 + gd) / ((GAMMA_BUMP * S) * (GAMMA_BUMP * S));
        }
    }
    if (f & THOTH_BUMP_VEGA) {
        Scenario s(*book);
        vol_shift(s, VOL_BUMP);
        double v;
        if ((rc = frozen(s, z, v))) return rc;
        am->vega = v - A0;
    }
    if (f & THOTH_BUMP_RHO) {
        // the rho scenario drifts and discounts at the bumped curve (pricer_mcl_american.cpp:218-226)
        Scenario s(*book);
        rate_shift(s, RATE_BUMP);
        std::vector<double> zr(z);
        for (double& x : zr) x += RATE_BUMP;
        double v;
        if ((rc = frozen(s, zr, v))) return rc;
        am->rho = (v - A0) / RATE_BUMP * 0.01;
    }
    if (f & THOTH_BUMP_THETA) {
        Scenario s(*book);
        std::string why;
        if (!roll_one_day(s, *book, why)) {
            g_aerr = "theta: " + why;
        } else {
            // the same calendar dates keep their zero rates
            const int sh = s.d.n_dates < nd ? 1 : 0;
            std::vector<double> zt(s.d.n_dates);
            for (int i = 0; i < s.d.n_dates; i++) zt[i] = z[i == 0 ? sh : i + sh];
            double v, tt;
            if ((rc = run_pass(s.d, c, zt, true, nullptr, v, tt, nullptr, nullptr, ms))) return rc;
            am->theta = v - A0;
        }
    }
    am->device_ms = ms;
    return THOTH_GPU_OK;
}

} // namespace

extern "C" {

int thoth_gpu_price_american(const ThothBookDesc* book, ThothAmerican* am)
{
    try {
        return price_american(book, am);
    } catch (const std::bad_alloc&) {
        return afail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return afail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

const char* thoth_gpu_american_last_error(void) { return g_aerr.c_str(); }

} // extern "C"
