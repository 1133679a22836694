// Exercises the C++ drop-in (gpu:: namespace) the way PricerMCL's GPU gate calls
// it (pricer_mcl_gpu_gate.cpp:109-126): one GBM contract, a two-contract book, an American put
// with its delta, and a leverage calibration.
// Prints "premium trust" lines; exits non-zero on any error.
#include "mcl_gpu.hpp"

#include <algorithm>
#include <cmath>
#include <cstdio>
#include <stdexcept>
#include <vector>

int main()
{
    try
    {
        if ( !gpu::Available() )
        {
            std::printf( "unavailable %s\n", gpu::DeviceInfo().c_str() );
            return 2;
        }
        const double F = 100.0 * std::exp( 0.02 ), df = std::exp( -0.03 );
        const gpu::GbmResult g = gpu::PriceEuropeanGbm( F, 100.0, 1.0, 0.25, df, true, 1L << 18, 0UL );
        std::printf( "gbm %.10f %.10f\n", g.premium, g.trust );

        const double t[2] = { 0.0, 1.0 }, carry[2] = { 0.02, 0.02 };
        ThothAsset a{};
        a.model = THOTH_MODEL_GBM;
        a.spot = 100.0;
        a.carry = carry;
        a.vol = 0.25;
        ThothProduct p[2]{};
        for ( int k = 0; k < 2; k++ )
        {
            p[k].kind = THOTH_PRODUCT_VANILLA;
            p[k].option_type = k == 0 ? THOTH_CALL : THOTH_PUT;
            p[k].maturity = 1;
            p[k].strike = 100.0;
            p[k].zero_rate = 0.03;
            p[k].fx = 1.0;
        }
        ThothBookDesc d{};
        d.n_dates = 2;
        d.t = t;
        d.n_assets = 1;
        d.assets = &a;
        d.n_products = 2;
        d.products = p;
        d.paths = 1L << 18;
        d.use_sobol = 1;
        const gpu::BookResult b = gpu::PriceBook( d );
        std::printf( "book %.10f %.10f %.10f %.10f\n", b.contract_premium[0], b.contract_premium[1], b.premium, b.trust );
        // an American put with its delta on a 13-date grid (at most 30 days a step)
        int32_t days[14];
        double t13[14], carry13[14];
        for ( int k = 0; k < 14; k++ )
        {
            days[k] = k < 13 ? 30 * k : 365;
            t13[k] = days[k] / 365.0;
            carry13[k] = 0.08;
        }
        ThothAsset a13 = a;
        a13.vol = 0.30;
        a13.carry = carry13;
        ThothProduct put{};
        put.kind = THOTH_PRODUCT_VANILLA;
        put.option_type = THOTH_PUT;
        put.maturity = 13;
        put.strike = 100.0;
        put.zero_rate = 0.08;
        put.fx = 1.0;
        ThothBookDesc am = d;
        am.n_dates = 14;
        am.days = days;
        am.t = t13;
        am.assets = &a13;
        am.n_products = 1;
        am.products = &put;
        am.paths = 1L << 16;
        std::vector<ThothAmerican> c( 1 );
        c[0].product = 0;
        c[0].flags = THOTH_BUMP_DELTA;
        gpu::PriceAmericanBook( am, c );
        std::printf( "american %.10f %.10f %.10f\n", c[0].premium, c[0].european, c[0].delta );
        // leverage layers for a flat 25 % local vol on a Heston base at 20 %, 30 daily dates
        const int nd = 31, np = 201;
        std::vector<int32_t> cd( nd );
        std::vector<double> cc( nd, 0.02 ), step( nd, 0.01 ), lv( (size_t)nd * np, 0.25 );
        std::vector<int64_t> off( nd, (int64_t)std::floor( std::log( 100.0 ) / 0.01 ) - np / 2 );
        for ( int k = 0; k < nd; k++ )
        {
            cd[k] = k;
        }
        ThothLeverageCalib lc{};
        lc.n_dates = nd;
        lc.points = np;
        lc.days = cd.data();
        lc.carry = cc.data();
        lc.spot = 100.0;
        lc.v0 = lc.theta = 0.04;
        lc.kappa = 1.5;
        lc.xi = 0.3;
        lc.rho = -0.5;
        lc.ln_step = step.data();
        lc.offset = off.data();
        lc.local_vol = lv.data();
        lc.particles = 4096;
        lc.seed = 20260708;
        const std::vector<double> lev = gpu::CalibrateLeverage( lc );
        double lo = lev[0], hi = lev[0];
        for ( double x : lev )
        {
            lo = std::min( lo, x );
            hi = std::max( hi, x );
        }
        std::printf( "calib %.10f %.10f\n", lo, hi );
        // the error path reaches the caller as the reference's ERR exception
        d.paths = 1;
        try
        {
            gpu::PriceBook( d );
            std::printf( "no error raised\n" );
            return 1;
        }
        catch ( const std::runtime_error& e )
        {
            std::printf( "error ok: %s\n", e.what() );
        }
        return 0;
    }
    catch ( const std::exception& e )
    {
        std::printf( "%s\n", e.what() );
        return 1;
    }
}
