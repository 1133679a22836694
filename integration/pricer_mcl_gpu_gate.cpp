//! pricer_mcl_gpu_gate.cpp — the GPU gate of PricerMCL for the GB300 Monte-Carlo engine.
//!
//! Replaces the reference's pricer/src/tasks/pricer_mcl_gpu_gate.cpp (its lines 46-126:
//! GpuGbmParamsFor, PricerMCL::BookIsGpuSupported, PricerMCL::PriceContract) in the
//! pricer's build, with the same two members and the same call sites
//! (pricer_mcl.cpp:175 decides _use_gpu once in PreCheck; PriceBook -> PriceBookByContract
//! -> PriceContract per contract and per bump-and-revalue scenario). What changes:
//!
//!  * the gate is widened from "single-asset European vanilla under flat GBM" to every
//!    book the engine prices on the device: European vanillas, barriers (discrete or
//!    continuous with the Broadie-Glasserman-Kou shift of barrier.cpp:122-173) and
//!    variance swaps (fresh or seasoned, continuous or discrete observation), on equity
//!    names under flat Black-Scholes, Heston (no jumps) or LSV, in the pricer's currency
//!    and on deterministic curves. Baskets, composites, quanto and cross-currency
//!    contracts, Bates jumps, local-vol (SABR) surfaces, discrete dividends, Hull-White
//!    rates, American exercise and books with two or more correlated Black-Scholes names
//!    keep the CPU engine (all or nothing, as before);
//!  * the book is priced in ONE engine call (thoth_gpu_price_book) on the pricer's own
//!    diffusion grid (InitDates) and Sobol / bridge configuration, so the GPU paths are the
//!    CPU engine's paths (pricer_mcl.cpp:387-455). PriceContract prices the whole book the
//!    first time it meets a scenario and reads every other contract of that scenario from
//!    the same call: the scenario is identified by the bytes of its descriptor, so a bump
//!    (spot, vol, rate, today) is a new descriptor and a new call;
//!  * LSV leverage layers come from the name's own calibration on the same grid
//!    (Single::CalibrateLeverage), as Single::BuildLeverageNode gets them.
//!
//! Everything crosses into the engine through the C ABI of include/thoth_gpu.h; the
//! device side is the GB300 engine (libthoth_gpu.so).
#include "thoth.hpp"
#include "pricer_mcl.hpp"
#include "barrier.hpp"
#include "cancellation.hpp"
#include "contract.hpp"
#include "currency.hpp"
#include "enums.hpp"
#include "equity.hpp"
#include "mcl_gpu.hpp"
#include "single.hpp"
#include "vanilla.hpp"
#include "variance.hpp"
#include "yield_curve.hpp"

#include "thoth_gpu.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <functional>
#include <map>
#include <mutex>
#include <string>
#include <vector>

namespace
{

//! every array behind one ThothBookDesc, and the contracts in product order
struct GpuBook
{
    vector<int32_t> days;
    vector<double> t;
    vector<ThothAsset> assets;
    vector<vector<double>> carry, lev_ln_step, lev_values;
    vector<vector<int64_t>> lev_offset;
    vector<ThothProduct> products;
    vector<vector<int32_t>> index_lists; //!< barrier monitors, variance observations
    vector<Contract*> contracts;         //!< product k prices contracts[k]
    ThothBookDesc desc{};
    string key; //!< the scenario: every input byte of the descriptor
};

void Append( string& key, const void* p, size_t n )
{
    key.append( static_cast<const char*>( p ), n );
}

template <class T>
void AppendVec( string& key, const vector<T>& v )
{
    const size_t n = v.size();
    Append( key, &n, sizeof n );
    if ( n )
    {
        Append( key, v.data(), n * sizeof( T ) );
    }
}

//! the single names of the book the engine can diffuse, or "" with the reason why not
string AssetFor( Single* s, const set<date>& Dates, const date& Today, const Currency* BookCcy,
                 GpuBook& B, std::map<Single*, int>& index )
{
    if ( index.count( s ) )
    {
        return "";
    }
    if ( s->IsForex() || !dynamic_cast<Equity*>( s ) )
    {
        return "underlying '" + s->GetName() + "' is not an equity";
    }
    if ( s->FutureDividendPv( Today ) != 0 )
    {
        return "underlying '" + s->GetName() + "' pays discrete dividends";
    }
    Currency* ccy = s->GetCurrency();
    if ( ccy != BookCcy || ccy->GetRateModel() )
    {
        return "underlying '" + s->GetName() + "' is not on the book's deterministic curve";
    }
    Volatility* vol = s->GetVolatility();
    ThothAsset a{};
    a.spot = s->GetDiffusionSpot( *Dates.rbegin() );
    //! the DriftNode's value at each diffusion date: the currency's zero rate less the
    //! name's dividend + repo yield (drift_node.cpp:20-27, equity.cpp:149-154, 215-230)
    vector<double> carry;
    for ( const date& d : Dates )
    {
        carry.push_back( ccy->GetRate()->GetCurveValue( d ) - s->DividendRepoYield( d ) );
    }
    if ( vol->IsStochastic() )
    {
        const StochasticVolParams h = vol->StochasticParams();
        if ( h.has_jumps() )
        {
            return "underlying '" + s->GetName() + "' carries Bates jumps";
        }
        a.model = THOTH_MODEL_HESTON;
        a.v0 = h.v0;
        a.kappa = h.kappa;
        a.theta = h.theta;
        a.xi = h.xi;
        a.rho = h.rho;
        if ( vol->IsLsv() )
        {
            //! one layer per diffusion date, on the name's own grid (single.cpp:400-473)
            const LeverageSurface lev = s->CalibrateLeverage( vector<date>( Dates.begin(), Dates.end() ) );
            if ( lev.Layers() != Dates.size() )
            {
                return "leverage of '" + s->GetName() + "' does not have one layer per date";
            }
            size_t points = 0;
            for ( size_t k = 0; k < lev.Layers(); k++ )
            {
                points = std::max( points, lev.Levels( k ).size() );
            }
            vector<double> step( lev.Layers() ), values( lev.Layers() * points );
            vector<int64_t> offset( lev.Layers() );
            for ( size_t k = 0; k < lev.Layers(); k++ )
            {
                const vector<double>& L = lev.Levels( k );
                if ( L.size() != points )
                {
                    return "leverage layers of '" + s->GetName() + "' differ in size";
                }
                step[k] = lev.LnStep( k );
                offset[k] = lev.Offset( k );
                std::copy( L.begin(), L.end(), values.begin() + k * points );
            }
            a.model = THOTH_MODEL_LSV;
            a.lev_points = (int32_t)points;
            B.lev_ln_step.push_back( std::move( step ) );
            B.lev_offset.push_back( std::move( offset ) );
            B.lev_values.push_back( std::move( values ) );
        }
    }
    else if ( vol->_is_local )
    {
        return "underlying '" + s->GetName() + "' has a local-vol surface";
    }
    else
    {
        //! the constant BS vol node (bs_volatility.cpp:37-49): vol + vega shift, day-weighted
        a.model = THOTH_MODEL_GBM;
        a.vol = s->GetImplicitVol( s->GetSpot(), *Dates.rbegin() );
    }
    index[s] = (int)B.assets.size();
    B.carry.push_back( std::move( carry ) );
    B.assets.push_back( a );
    return "";
}

//! ThothBookDesc of the whole book on the pricer's diffusion grid, or "" with the reason why not
string DescribeBook( Book* TheBook, const SingleSet& Singles, const date& Today, const set<date>& Dates,
                     const Currency* BookCcy, const MclConfiguration* Mcl, GpuBook& B,
                     std::function<double( Contract* )> FxToBook )
{
    if ( Dates.size() < 2 || *Dates.begin() != Today )
    {
        return "the diffusion grid must start today and hold a later date";
    }
    vector<date> dl( Dates.begin(), Dates.end() );
    auto index_of = [&]( const date& d ) -> int
    {
        auto it = std::lower_bound( dl.begin(), dl.end(), d );
        return ( it == dl.end() || *it != d ) ? -1 : (int)( it - dl.begin() );
    };
    for ( const date& d : dl )
    {
        B.days.push_back( (int32_t)( d - Today ).days() );
        B.t.push_back( YearFraction( Today, d ) );
    }
    //! the assets in the pricer's name order: the Sobol factors are every name's spot noise,
    //! then the stochastic names' variance noises, each in that order (pricer_mcl.cpp:414-431),
    //! and the engine lays its factors out the same way from the asset order
    std::map<Single*, int> asset_of;
    for ( Single* s : Singles )
    {
        if ( string why = AssetFor( s, Dates, Today, BookCcy, B, asset_of ); !why.empty() )
        {
            return why;
        }
    }
    for ( Contract* c : TheBook->GetContractSet() )
    {
        if ( c->IsAmerican() )
        {
            return "contract '" + c->GetName() + "' is American";
        }
        Underlying* u = c->GetUnderlying();
        if ( !u->IsMono() )
        {
            return "contract '" + c->GetName() + "' is on a multi-asset underlying";
        }
        Single* s = *u->GetSingleSet().begin();
        if ( c->GetPremiumCurrency() != s->GetCurrency() )
        {
            return "contract '" + c->GetName() + "' settles in another currency (quanto)";
        }
        if ( !asset_of.count( s ) )
        {
            return "contract '" + c->GetName() + "' is on a name outside the pricer's set";
        }
        ThothProduct p{};
        p.asset = asset_of[s];
        p.fx = FxToBook( c );
        const date mat = c->GetMaturityDate();
        p.maturity = index_of( mat );
        if ( p.maturity < 0 )
        {
            return "maturity of '" + c->GetName() + "' is not a diffusion date";
        }
        //! flat-to-maturity discounting of the premium currency (contract_node.cpp:16-51)
        const double tm = B.t[p.maturity];
        const double df = c->GetPremiumCurrency()->GetDiscountRate()->GetDiscountFactor( mat );
        p.zero_rate = tm > 0 ? -std::log( df ) / tm : 0.0;
        vector<int32_t> list;
        if ( auto* v = dynamic_cast<Vanilla*>( c ) )
        {
            p.kind = THOTH_PRODUCT_VANILLA;
            p.strike = v->GetStrike();
            p.option_type = v->GetType() == OptionType::Call ? THOTH_CALL : THOTH_PUT;
        }
        else if ( auto* br = dynamic_cast<Barrier*>( c ) )
        {
            p.kind = THOTH_PRODUCT_BARRIER;
            p.strike = br->_strike;
            p.option_type = br->_type == OptionType::Call ? THOTH_CALL : THOTH_PUT;
            p.barrier_up = br->IsUp() ? 1 : 0;
            p.barrier_in = br->IsIn() ? 1 : 0;
            double H = br->Level();
            if ( br->IsDiscrete() )
            {
                for ( const date& d : br->GetMonitoringDates() )
                {
                    list.push_back( index_of( d ) );
                }
            }
            else
            {
                //! every diffusion date up to maturity and the BGK shift of barrier.cpp:147-165
                for ( int i = 0; i <= p.maturity; i++ )
                {
                    list.push_back( i );
                }
                const size_t steps = list.size() > 1 ? list.size() - 1 : 1;
                const double dt = YearFraction( Today, mat ) / (double)steps;
                const double vol = u->GetImplicitVol( br->_strike, mat );
                H *= std::exp( ( p.barrier_up ? -1.0 : 1.0 ) * 0.5826 * vol * std::sqrt( dt ) );
            }
            if ( std::find( list.begin(), list.end(), -1 ) != list.end() )
            {
                return "a monitoring date of '" + c->GetName() + "' is not a diffusion date";
            }
            p.barrier_level = H;
        }
        else if ( auto* vs = dynamic_cast<Variance*>( c ) )
        {
            p.kind = THOTH_PRODUCT_VARIANCE;
            p.notional = vs->GetNotional();
            p.strike_variance = vs->GetVolatilityStrike() * vs->GetVolatilityStrike();
            if ( vs->IsSeasoned() )
            {
                p.past_variance = vs->PastSumSquaredReturns();
                p.total_year_fraction = vs->GetTotalYearFraction();
            }
            if ( vs->IsDiscretelyObserved() )
            {
                for ( const date& d : vs->GetObservationDates() )
                {
                    list.push_back( index_of( d ) );
                }
                if ( std::find( list.begin(), list.end(), -1 ) != list.end() )
                {
                    return "an observation date of '" + c->GetName() + "' is not a diffusion date";
                }
            }
        }
        else
        {
            return "contract '" + c->GetName() + "' is of a kind the GPU engine does not price";
        }
        B.index_lists.push_back( std::move( list ) );
        B.products.push_back( p );
        B.contracts.push_back( c );
    }
    if ( B.products.empty() )
    {
        return "empty book";
    }
    if ( B.assets.size() > THOTH_MAX_ASSETS )
    {
        return "more underlyings than the GPU engine diffuses in one book";
    }
    //! the reference correlates the GBM names' noises through its Cholesky factor
    //! (pricer_mcl.cpp:246-314) and leaves Heston / LSV names on their own: with one GBM
    //! name at most there is nothing to correlate, so no factor crosses the boundary
    if ( std::count_if( B.assets.begin(), B.assets.end(),
                        []( const ThothAsset& a ) { return a.model == THOTH_MODEL_GBM; } ) > 1 )
    {
        return "several Black-Scholes names (their correlation stays with the CPU engine)";
    }
    //! pointers into the owned arrays (stable from here on)
    size_t lev = 0;
    for ( size_t a = 0; a < B.assets.size(); a++ )
    {
        B.assets[a].carry = B.carry[a].data();
        if ( B.assets[a].model == THOTH_MODEL_LSV )
        {
            B.assets[a].lev_ln_step = B.lev_ln_step[lev].data();
            B.assets[a].lev_offset = B.lev_offset[lev].data();
            B.assets[a].lev_values = B.lev_values[lev].data();
            lev++;
        }
    }
    for ( size_t k = 0; k < B.products.size(); k++ )
    {
        ThothProduct& p = B.products[k];
        const vector<int32_t>& l = B.index_lists[k];
        if ( p.kind == THOTH_PRODUCT_BARRIER )
        {
            p.n_monitor = (int32_t)l.size();
            p.monitor = l.data();
        }
        else if ( p.kind == THOTH_PRODUCT_VARIANCE && !l.empty() )
        {
            p.n_obs = (int32_t)l.size();
            p.obs = l.data();
        }
    }
    ThothBookDesc& d = B.desc;
    d.n_dates = (int32_t)B.t.size();
    d.days = B.days.data();
    d.t = B.t.data();
    d.n_assets = (int32_t)B.assets.size();
    d.assets = B.assets.data();
    d.cholesky = nullptr; //!< one GBM name at most (checked above): every name on its own noise
    d.n_products = (int32_t)B.products.size();
    d.products = B.products.data();
    d.paths = Mcl->_paths;
    d.use_sobol = Mcl->_use_sobol ? 1 : 0;
    d.sobol_skip = (int64_t)Mcl->_sobol_skip;
    d.seed = (uint64_t)Mcl->_seed;
    d.greeks = 0;
    //! the scenario key: grid, model inputs, products, path configuration
    string& key = B.key;
    AppendVec( key, B.t );
    for ( size_t a = 0; a < B.assets.size(); a++ )
    {
        const ThothAsset& x = B.assets[a];
        const double sc[7] = { x.spot, x.vol, x.v0, x.kappa, x.theta, x.xi, x.rho };
        Append( key, &x.model, sizeof x.model );
        Append( key, sc, sizeof sc );
        AppendVec( key, B.carry[a] );
    }
    for ( size_t k = 0; k < B.lev_values.size(); k++ )
    {
        AppendVec( key, B.lev_ln_step[k] );
        AppendVec( key, B.lev_offset[k] );
        AppendVec( key, B.lev_values[k] );
    }
    for ( size_t k = 0; k < B.products.size(); k++ )
    {
        const ThothProduct& p = B.products[k];
        const double sc[8] = { p.strike, p.zero_rate, p.fx, p.barrier_level, p.notional, p.strike_variance,
                               p.total_year_fraction, p.past_variance };
        const int32_t ic[6] = { p.kind, p.option_type, p.asset, p.maturity, p.barrier_up, p.barrier_in };
        Append( key, sc, sizeof sc );
        Append( key, ic, sizeof ic );
        AppendVec( key, B.index_lists[k] );
    }
    const int64_t cfg[4] = { d.paths, d.use_sobol, d.sobol_skip, (int64_t)d.seed };
    Append( key, cfg, sizeof cfg );
    return "";
}

//! the last whole-book result of each pricer: the scenario key and every contract's premium
struct Priced
{
    string key;
    std::map<string, std::pair<double, double>> by_contract; //!< premium, trust
};
std::mutex g_priced_mutex;
std::map<const void*, Priced> g_priced;

} // namespace

//! GPU-priceable iff a device is present and the engine prices every contract of the book
//! (DescribeBook above). All-or-nothing: a mixed book runs on the CPU so the result is
//! never a half-GPU/half-CPU patchwork.
bool PricerMCL::BookIsGpuSupported()
{
    if ( !gpu::Available() )
    {
        return false;
    }
    _book->Reset( _today, _correlation );
    _diffusion_dates.clear();
    InitDates();
    GpuBook B;
    const string why = DescribeBook( _book, _single_set, _today, _diffusion_dates, _currency, _mcl, B,
                                     [this]( Contract* c ) { return FxToBook( c ); } );
    if ( !why.empty() )
    {
        LOG( "GPU", "book '" + _name + "' stays on the CPU engine: " + why );
    }
    return why.empty();
}

//! price one contract on the GPU: the whole book is priced in one engine call the first time
//! a scenario is met, and every other contract of that scenario is read from that call.
void PricerMCL::PriceContract( Contract* Ctr )
{
    cancellation::CancellationPoint();
    _diffusion_dates.clear();
    InitDates();
    GpuBook B;
    const string why = DescribeBook( _book, _single_set, _today, _diffusion_dates, _currency, _mcl, B,
                                     [this]( Contract* c ) { return FxToBook( c ); } );
    if ( !why.empty() )
    {
        //! BookIsGpuSupported guarantees every contract is supported in GPU mode
        ERR( "gpu pricing '" + _name + "': " + why );
    }
    std::lock_guard<std::mutex> lock( g_priced_mutex );
    Priced& memo = g_priced[this];
    if ( memo.key != B.key )
    {
        const size_t n = B.products.size();
        vector<double> premium( n ), trust( n );
        ThothBookResult r{};
        r.premium = premium.data();
        r.trust = trust.data();
        const int rc = thoth_gpu_price_book( &B.desc, &r );
        if ( rc != THOTH_GPU_OK )
        {
            memo.key.clear();
            if ( rc == THOTH_GPU_E_CANCELLED )
            {
                cancellation::CancellationPoint();
            }
            ERR( "gpu pricing '" + _name + "' failed (" + std::to_string( rc ) + "): " + thoth_gpu_last_error() );
        }
        memo.by_contract.clear();
        for ( size_t k = 0; k < n; k++ )
        {
            memo.by_contract[B.contracts[k]->GetName()] = { premium[k], trust[k] };
        }
        memo.key = B.key;
    }
    const auto& v = memo.by_contract.at( Ctr->GetName() );
    Result( Ctr ).premium = v.first;
    Result( Ctr ).premium_trust = v.second;
}
