// greeks.cu — bump-and-revalue Greeks on common random numbers, the reference's
// definitions (pricer_mcl_greeks.cpp:43-299, pricer.cpp:144-193, bump sizes
// pricer.hpp:20-30 and constants.hpp:36): every bumped scenario of the book is
// priced in one batch (one CUDA graph) on the same Sobol paths as the base, and
// the Greeks are the reference's finite differences, per contract and for the
// book. Host code only, a client of the C ABI.
#include "thoth_gpu.h"
#include "scenario.hpp"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <stdexcept>
#include <string>
#include <vector>

namespace {

using namespace thoth_scenario;

thread_local std::string g_gerr;

int gfail(int code, const std::string& m)
{
    g_gerr = m;
    return code;
}

int bump_greeks(const ThothBookDesc* book, ThothBumpGreeks* out)
{
    g_gerr.clear();
    if (!book || !out) return gfail(THOTH_GPU_E_INVALID, "null argument");
    if (book->n_assets < 1 || !book->assets || book->n_products < 1 || !book->products || book->n_dates < 2 ||
        !book->t)
        return gfail(THOTH_GPU_E_INVALID, "bad descriptor");
    for (int a = 0; a < book->n_assets; a++)
        if (!book->assets[a].carry) return gfail(THOTH_GPU_E_INVALID, "asset carry is null");
    const int np = book->n_products, na = book->n_assets;
    const int f = out->flags;
    const double nan = std::nan("");
    // scenarios: base, then the requested bumps
    std::vector<Scenario*> sc;
    struct Guard {
        std::vector<Scenario*>& v;
        ~Guard()
        {
            for (Scenario* s : v) delete s;
        }
    } guard{sc};
    auto add = [&]() {
        sc.push_back(new Scenario(*book));
        return sc.back();
    };
    add(); // base
    std::vector<int> i_delta(na, -1), i_gup(na, -1), i_gdn(na, -1);
    int i_vega = -1, i_rho = -1, i_theta = -1, i_param[5] = {-1, -1, -1, -1, -1};
    std::string theta_why;
    for (int a = 0; a < na; a++) {
        const double s0 = book->assets[a].spot;
        if (f & THOTH_BUMP_DELTA) {
            i_delta[a] = (int)sc.size();
            add()->assets[a].spot = s0 * (1 + SPOT_BUMP);
        }
        if (f & THOTH_BUMP_GAMMA) {
            i_gup[a] = (int)sc.size();
            add()->assets[a].spot = s0 * (1 + GAMMA_BUMP);
            i_gdn[a] = (int)sc.size();
            add()->assets[a].spot = s0 * (1 - GAMMA_BUMP);
        }
    }
    if (f & THOTH_BUMP_VEGA) {
        i_vega = (int)sc.size();
        vol_shift(*add(), VOL_BUMP);
    }
    if (f & THOTH_BUMP_RHO) {
        i_rho = (int)sc.size();
        rate_shift(*add(), RATE_BUMP);
    }
    if (f & THOTH_BUMP_THETA) {
        Scenario* s = add();
        if (roll_one_day(*s, *book, theta_why)) {
            i_theta = (int)sc.size() - 1;
        } else {
            delete s;
            sc.pop_back();
        }
    }
    bool any_heston = false;
    for (int a = 0; a < na; a++) any_heston |= is_heston(book->assets[a]);
    if ((f & THOTH_BUMP_PARAMS) && any_heston) {
        for (int k = 0; k < 5; k++) {
            i_param[k] = (int)sc.size();
            Scenario* s = add();
            for (ThothAsset& A : s->assets) {
                if (!is_heston(A)) continue;
                double* v[5] = {&A.v0, &A.kappa, &A.theta, &A.xi, &A.rho};
                *v[k] += PARAM_BUMP;
            }
        }
    }
    // one batch, one graph, the same Sobol paths for every scenario
    const int n = (int)sc.size();
    std::vector<ThothBookDesc> descs(n);
    std::vector<ThothBookResult> res(n);
    for (int k = 0; k < n; k++) {
        sc[k]->relink();
        descs[k] = sc[k]->d;
        descs[k].greeks = 0;
        sc[k]->premium.assign(np, nan);
        std::memset(&res[k], 0, sizeof(ThothBookResult));
        res[k].premium = sc[k]->premium.data();
    }
    const int rc = thoth_gpu_price_batch(descs.data(), n, res.data());
    if (rc) return gfail(rc, std::string("bumped scenarios: ") + thoth_gpu_last_error());
    const std::vector<double>& p0 = sc[0]->premium;
    const double b0 = res[0].book_premium;
    auto fill = [&](double* dst, double& bdst, auto per_product, auto per_book) {
        if (dst)
            for (int p = 0; p < np; p++) dst[p] = per_product(p);
        bdst = per_book();
    };
    auto prem = [&](int k, int p) { return sc[k]->premium[p]; };
    if (out->premium)
        for (int p = 0; p < np; p++) out->premium[p] = p0[p];
    out->book_premium = b0;
    // delta / gamma: summed over the per-underlying spot bumps
    fill(out->delta, out->book_delta,
         [&](int p) {
             if (!(f & THOTH_BUMP_DELTA)) return nan;
             double s = 0;
             for (int a = 0; a < na; a++) s += (prem(i_delta[a], p) - p0[p]) / (SPOT_BUMP * book->assets[a].spot);
             return s;
         },
         [&]() {
             if (!(f & THOTH_BUMP_DELTA)) return nan;
             double s = 0;
             for (int a = 0; a < na; a++) s += (res[i_delta[a]].book_premium - b0) / (SPOT_BUMP * book->assets[a].spot);
             return s;
         });
    fill(out->gamma, out->book_gamma,
         [&](int p) {
             if (!(f & THOTH_BUMP_GAMMA)) return nan;
             double s = 0;
             for (int a = 0; a < na; a++) {
                 const double h = GAMMA_BUMP * book->assets[a].spot;
                 s += (prem(i_gup[a], p) - 2 * p0[p] + prem(i_gdn[a], p)) / (h * h);
             }
             return s;
         },
         [&]() {
             if (!(f & THOTH_BUMP_GAMMA)) return nan;
             double s = 0;
             for (int a = 0; a < na; a++) {
                 const double h = GAMMA_BUMP * book->assets[a].spot;
                 s += (res[i_gup[a]].book_premium - 2 * b0 + res[i_gdn[a]].book_premium) / (h * h);
             }
             return s;
         });
    // vega per vol point, rho per 1 % rate move, theta per day
    fill(out->vega, out->book_vega, [&](int p) { return i_vega < 0 ? nan : (prem(i_vega, p) - p0[p]) / VOL_BUMP * 0.01; },
         [&]() { return i_vega < 0 ? nan : (res[i_vega].book_premium - b0) / VOL_BUMP * 0.01; });
    fill(out->rho, out->book_rho, [&](int p) { return i_rho < 0 ? nan : (prem(i_rho, p) - p0[p]) / RATE_BUMP * 0.01; },
         [&]() { return i_rho < 0 ? nan : (res[i_rho].book_premium - b0) / RATE_BUMP * 0.01; });
    fill(out->theta, out->book_theta, [&](int p) { return i_theta < 0 ? nan : prem(i_theta, p) - p0[p]; },
         [&]() { return i_theta < 0 ? nan : res[i_theta].book_premium - b0; });
    // vega_<param>, per unit of the parameter
    for (int k = 0; k < 5; k++) {
        double* dst = out->vega_param ? out->vega_param + (size_t)k * np : nullptr;
        fill(dst, out->book_vega_param[k],
             [&](int p) { return i_param[k] < 0 ? nan : (prem(i_param[k], p) - p0[p]) / PARAM_BUMP; },
             [&]() { return i_param[k] < 0 ? nan : (res[i_param[k]].book_premium - b0) / PARAM_BUMP; });
    }
    out->n_scenarios = n;
    out->device_ms = res[0].device_ms;
    if ((f & THOTH_BUMP_THETA) && i_theta < 0) return gfail(THOTH_GPU_OK, theta_why); // theta NaN, rest valid
    return THOTH_GPU_OK;
}

} // namespace

extern "C" {

int thoth_gpu_bump_greeks(const ThothBookDesc* book, ThothBumpGreeks* out)
{
    try {
        return bump_greeks(book, out);
    } catch (const std::bad_alloc&) {
        return gfail(THOTH_GPU_E_NOMEM, "out of host memory");
    } catch (const std::exception& e) {
        return gfail(THOTH_GPU_E_INVALID, std::string("host error: ") + e.what());
    }
}

const char* thoth_gpu_bump_greeks_last_error(void) { return g_gerr.c_str(); }

} // extern "C"
