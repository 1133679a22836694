// C++ host side of the GPU boundary over the C ABI (see mcl_gpu.hpp).
#include "mcl_gpu.hpp"

#include <algorithm>
#include <stdexcept>

namespace gpu
{
namespace
{
[[noreturn]] void Err( const std::string& what, int code )
{
    throw std::runtime_error( "ERR> gpu " + what + " failed (" + std::to_string( code ) + "): " +
                              thoth_gpu_last_error() );
}
} // namespace

bool Available()
{
    return thoth_gpu_available() == 1;
}

std::string DeviceInfo()
{
    char buf[256];
    if ( thoth_gpu_device_info( buf, sizeof buf ) != THOTH_GPU_OK )
    {
        return "CUDA device query failed";
    }
    return buf;
}

GbmResult PriceEuropeanGbm( double Forward, double Strike, double T, double Vol, double Df, bool IsCall,
                            long Paths, unsigned long Seed )
{
    ThothGbmResult r{ 0.0, 0.0 };
    const int rc = thoth_gpu_price_european_gbm( Forward, Strike, T, Vol, Df, IsCall ? 1 : 0, (int64_t)Paths,
                                                 (uint64_t)Seed, &r );
    if ( rc != THOTH_GPU_OK )
    {
        Err( "PriceEuropeanGbm", rc );
    }
    return GbmResult{ r.premium, r.trust };
}

BookResult PriceBook( const ThothBookDesc& Book )
{
    BookResult out;
    const size_t n = Book.n_products > 0 ? (size_t)Book.n_products : 0;
    out.contract_premium.assign( n, 0.0 );
    out.contract_trust.assign( n, 0.0 );
    out.delta.assign( n, 0.0 );
    out.delta_trust.assign( n, 0.0 );
    out.vega.assign( n, 0.0 );
    out.vega_trust.assign( n, 0.0 );
    ThothBookResult r{};
    r.premium = out.contract_premium.data();
    r.trust = out.contract_trust.data();
    r.delta = out.delta.data();
    r.delta_trust = out.delta_trust.data();
    r.vega = out.vega.data();
    r.vega_trust = out.vega_trust.data();
    const int rc = thoth_gpu_price_book( &Book, &r );
    if ( rc != THOTH_GPU_OK )
    {
        Err( "PriceBook", rc );
    }
    out.premium = r.book_premium;
    out.trust = r.book_trust;
    out.device_ms = r.device_ms;
    return out;
}

void PriceAmericanBook( const ThothBookDesc& Book, std::vector<ThothAmerican>& Contracts )
{
    if ( Contracts.empty() )
    {
        return;
    }
    const int rc = thoth_gpu_price_american_book( &Book, Contracts.data(), (int32_t)Contracts.size() );
    if ( rc != THOTH_GPU_OK )
    {
        throw std::runtime_error( "ERR> gpu PriceAmericanBook failed (" + std::to_string( rc ) +
                                  "): " + thoth_gpu_american_last_error() );
    }
}

std::vector<double> CalibrateLeverage( const ThothLeverageCalib& Calib )
{
    ThothLeverageCalib c = Calib;
    std::vector<double> lev( (size_t)std::max( c.n_dates, 0 ) * (size_t)std::max( c.points, 0 ) );
    c.leverage = lev.data();
    const int rc = thoth_gpu_calibrate_leverage( &c );
    if ( rc != THOTH_GPU_OK )
    {
        Err( "CalibrateLeverage", rc );
    }
    return lev;
}

} // namespace gpu
