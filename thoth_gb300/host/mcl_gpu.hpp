#pragma once
// Drop-in replacement for the reference's pricer/src/tasks/mcl_gpu.hpp:16-48:
// the same namespace, names, argument meaning and return types, implemented over
// the C ABI of libthoth_gpu.so (include/thoth_gpu.h). A C++23 host that compiled
// against the reference header compiles against this one unchanged, and gains
// gpu::PriceBook for whole-book pricing (one sweep for every contract).
#include <string>
#include <vector>

#include "thoth_gpu.h"

namespace gpu
{

//! true iff a usable sm_103 device is present (reference: mcl_gpu.cu:77-82)
bool Available();

//! one-line device description (reference: mcl_gpu.cu:84-98)
std::string DeviceInfo();

//! reference gpu::GbmResult (mcl_gpu.hpp:34-38)
struct GbmResult
{
    double premium;
    double trust;
};

//! European vanilla under GBM in the forward measure (reference: mcl_gpu.hpp:40-46).
//! Errors are reported the reference host's way: a std::runtime_error("ERR> gpu ...")
//! (helpers/misc.hpp:30-31 ERR), never a silent zero.
GbmResult PriceEuropeanGbm( double Forward, double Strike, double T, double Vol, double Df, bool IsCall,
                            long Paths, unsigned long Seed );

//! whole-book result: per contract premium/trust (+ pathwise Greeks) and the book
struct BookResult
{
    double premium = 0, trust = 0;
    std::vector<double> contract_premium, contract_trust, delta, delta_trust, vega, vega_trust;
    double device_ms = 0;
};

//! price every product of a flat book descriptor in one GPU sweep
BookResult PriceBook( const ThothBookDesc& Book );

//! the American vanillas of a book by Longstaff-Schwartz (reference: PricerMCL::PriceAmerican,
//! pricer_mcl_american.cpp:137-261): each entry's product and flags (and optionally min_itm,
//! zero_rates, beta) in, its premium, trust and Greeks out
void PriceAmericanBook( const ThothBookDesc& Book, std::vector<ThothAmerican>& Contracts );

//! leverage layers [n_dates][points] by the reference's particle method
//! (Single::CalibrateLeverage, single.cpp:390-473); Calib.leverage is not used
std::vector<double> CalibrateLeverage( const ThothLeverageCalib& Calib );

} // namespace gpu
