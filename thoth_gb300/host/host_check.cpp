// Exercises the C++ drop-in (gpu:: namespace) the way PricerMCL's GPU gate calls
// it (pricer_mcl_gpu_gate.cpp:109-126): one GBM contract, then a two-contract book.
// Prints "premium trust" lines; exits non-zero on any error.
#include "mcl_gpu.hpp"

#include <cmath>
#include <cstdio>
#include <stdexcept>

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
