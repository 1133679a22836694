//! ref_harness.cpp — TEST INFRASTRUCTURE ONLY (parity oracle, never shipped).
//!
//! Drives the reference's own, unmodified Monte-Carlo node classes (compiled
//! from GValas/Thoth's sources by oracle/Makefile into oracle/_ref/) on a book
//! described by the C-ABI descriptor of include/thoth_gpu.h. The node graph is
//! wired the way the reference's graph builders wire it:
//!   * noises, Brownians, Sobol factor order  pricer/src/tasks/pricer_mcl.cpp:327-455
//!   * GBM / Heston / LSV spot nodes           pricer/src/marketdata/single.cpp:65-153
//!   * correlation of GBM Brownians            pricer/src/tasks/pricer_mcl.cpp:246-314
//!   * contract / flow / quanto nodes          pricer/src/contracts/contract.cpp:63-116,
//!                                             vanilla.cpp:92-104, barrier.cpp:122-173
//!   * path loop and read-out                  pricer/src/tasks/pricer_mcl.cpp:598-709
//! Rates and carries are fed through small table nodes defined here (the
//! reference's curve classes need the YAML object layer, which is not built).
//! Used only by tests/ and by the fixture generator under tests/golden/.

#include "thoth.hpp"
#include "node_collector.hpp"
#include "path_generator.hpp"
#include "sobol_generator.hpp"
#include "distributions.hpp"
#include "rng.hpp"
#include "maths.hpp"
#include "finance.hpp"

#include "thoth_gpu.h"

#include <cstdint>
#include <cstring>

namespace
{

//! per-date constant table (path-independent: never scheduled per path)
class TableNode : public MonteCarloNode
{
  public:
    explicit TableNode( const string& Name ) : MonteCarloNode( Name ) {}
    void Fill( const double* v, size_t n )
    {
        for ( size_t i = 0; i < n && i < _value_list.size(); i++ )
        {
            _value_list[i] = v[i];
        }
    }
    void FillConstant( double v )
    {
        for ( double& x : _value_list )
        {
            x = v;
        }
    }
    bool IsConstant( size_t ) override { return true; }
    void ComputeValue( size_t ) override {}
    void GetDateDependencies( size_t, vector<MonteCarloNode*>&, vector<size_t>& ) override {}
};

string AssetName( int a )
{
    char b[16];
    std::snprintf( b, sizeof b, "a%03d", a );
    return b;
}
string ProductName( int p )
{
    char b[16];
    std::snprintf( b, sizeof b, "p%04d", p );
    return b;
}

struct Harness
{
    NodeCollector nc;
    Rng rng;
    std::unique_ptr<PathGenerator> pg;
    MonteCarloNode* book = nullptr;
    vector<MonteCarloNode*> contracts;
    vector<MonteCarloNode*> spot_nodes;
};

//! build the node graph of one book; returns false on an unsupported descriptor
bool Build( const ThothBookDesc* d, Harness& h )
{
    if ( !d->days || d->n_dates < 2 )
    {
        return false;
    }
    set<date> dates;
    for ( int i = 0; i < d->n_dates; i++ )
    {
        dates.insert( date( d->days[i] ) );
    }
    if ( (int)dates.size() != d->n_dates )
    {
        return false;
    }
    NodeCollector& nc = h.nc;
    nc.SetDiffusionDates( dates );
    const int na = d->n_assets;

    //! noises (pricer_mcl.cpp:327-382)
    for ( int a = 0; a < na; a++ )
    {
        const ThothAsset& A = d->assets[a];
        NoiseNode* n = nc.NewNode<NoiseNode>( AssetName( a ) + node_name::WHITE_NOISE );
        n->SetRandomGenerator( &h.rng );
        if ( A.model == THOTH_MODEL_GBM )
        {
            BrownianNode* b = nc.NewBrownianNode( AssetName( a ) + node_name::BROWNIAN );
            b->SetNoiseNode( n );
        }
        else
        {
            NoiseNode* vn = nc.NewNode<NoiseNode>( AssetName( a ) + node_name::VOL_WHITE_NOISE );
            vn->SetRandomGenerator( &h.rng );
        }
    }

    //! Sobol + bridge wiring: spot noises first, then variance noises (pricer_mcl.cpp:387-455)
    h.rng.Seed( d->seed );
    vector<string> factor_noise;
    for ( int a = 0; a < na; a++ )
    {
        factor_noise.push_back( AssetName( a ) + node_name::WHITE_NOISE );
    }
    for ( int a = 0; a < na; a++ )
    {
        if ( d->assets[a].model != THOTH_MODEL_GBM )
        {
            factor_noise.push_back( AssetName( a ) + node_name::VOL_WHITE_NOISE );
        }
    }
    if ( d->use_sobol )
    {
        vector<double> times;
        for ( int i = 0; i < d->n_dates; i++ )
        {
            times.push_back( YearFraction( date( d->days[0] ), date( d->days[i] ) ) );
        }
        h.pg = std::make_unique<PathGenerator>( times, (int)factor_noise.size(), true, &h.rng,
                                                (uint64_t)d->sobol_skip );
        for ( size_t f = 0; f < factor_noise.size(); f++ )
        {
            nc.GetTypedNode<NoiseNode>( factor_noise[f] )->SetNoiseBuffer( h.pg->Buffer( (int)f ) );
        }
    }

    //! correlated Brownians for GBM assets (pricer_mcl.cpp:246-314)
    if ( na > 1 && d->cholesky )
    {
        for ( int u = 0; u < na; u++ )
        {
            BrownianNode* B = nc.GetBrownianNode( AssetName( u ) + node_name::BROWNIAN );
            if ( !B )
            {
                continue;
            }
            CorrelatedNoiseNode* cn = nc.NewNode<CorrelatedNoiseNode>( AssetName( u ) + node_name::NOISE );
            for ( int v = 0; v < na; v++ )
            {
                const double l = d->cholesky[u * na + v];
                if ( l != 0 )
                {
                    ConstantNode* c = nc.NewNode<ConstantNode>( AssetName( u ) + "#" + AssetName( v ) + node_name::CHOLESKY );
                    c->SetConstantValue( l );
                    cn->PushNoiseNode( nc.GetNode( AssetName( v ) + node_name::WHITE_NOISE ) );
                    cn->PushCholeskyNode( c );
                }
            }
            B->SetNoiseNode( cn );
        }
    }

    //! spot nodes (single.cpp:65-153)
    const size_t nd = (size_t)d->n_dates;
    for ( int a = 0; a < na; a++ )
    {
        const ThothAsset& A = d->assets[a];
        TableNode* drift = nc.NewNode<TableNode>( AssetName( a ) + node_name::DRIFT );
        drift->Fill( A.carry, nd );
        if ( A.model == THOTH_MODEL_GBM )
        {
            SpotDiffusionNode* S = nc.NewNode<SpotDiffusionNode>( AssetName( a ) + node_name::SPOT );
            ConstantNode* vol = nc.NewNode<ConstantNode>( AssetName( a ) + node_name::VOL );
            vol->SetConstantValue( A.vol );
            S->SetBrownianNode( nc.GetNode( AssetName( a ) + node_name::BROWNIAN ) );
            S->SetDriftNode( drift );
            S->SetSpot( A.spot );
            S->SetLocalVolNode( vol );
            h.spot_nodes.push_back( S );
        }
        else
        {
            HestonVarianceNode* V = nc.NewNode<HestonVarianceNode>( AssetName( a ) + node_name::VARIANCE );
            V->SetParameters( A.v0, A.kappa, A.theta, A.xi );
            V->SetNoiseNode( nc.GetNode( AssetName( a ) + node_name::VOL_WHITE_NOISE ) );
            HestonSpotNode* S = nc.NewNode<HestonSpotNode>( AssetName( a ) + node_name::SPOT );
            S->SetParameters( A.kappa, A.theta, A.xi, A.rho );
            S->SetVarianceNode( V );
            S->SetDriftNode( drift );
            S->SetNoiseNode( nc.GetNode( AssetName( a ) + node_name::WHITE_NOISE ) );
            if ( A.model == THOTH_MODEL_LSV )
            {
                //! one leverage layer per diffusion date (single.cpp:479-500)
                LocalVolatilityNode* L = nc.NewNode<LocalVolatilityNode>( AssetName( a ) + node_name::LEVERAGE );
                L->SetSpotNode( S );
                for ( size_t i = 0; i < nd; i++ )
                {
                    L->PushLnStep( A.lev_ln_step[i] );
                    L->PushOffset( (long)A.lev_offset[i] );
                    la_vector* v = la_vector_alloc( (size_t)A.lev_points );
                    for ( int k = 0; k < A.lev_points; k++ )
                    {
                        la_vector_set( v, (size_t)k, A.lev_values[i * (size_t)A.lev_points + k] );
                    }
                    L->PushVolVector( v );
                }
                S->SetLeverageNode( L );
            }
            S->SetSpot( A.spot );
            h.spot_nodes.push_back( S );
        }
    }

    //! products (contract.cpp:63-116 and the flow builders)
    BookNode* book = nc.NewNode<BookNode>( "book" );
    for ( int p = 0; p < d->n_products; p++ )
    {
        const ThothProduct& P = d->products[p];
        const string pn = ProductName( p );
        auto quanto_of = [&]( int a ) -> MonteCarloNode*
        {
            MonteCarloNode* s = h.spot_nodes[(size_t)a];
            if ( P.quanto == 0 )
            {
                return s;
            }
            //! QuantoAdjustmentNode reads exp(-v*w*c*t): feed v = quanto, w = c = 1
            QuantoAdjustmentNode* q = nc.NewNode<QuantoAdjustmentNode>( pn + "#" + AssetName( a ) + "#quanto" );
            const string qn = pn + "#" + AssetName( a );
            ConstantNode* v = nc.NewNode<ConstantNode>( qn + "#qv" );
            ConstantNode* w = nc.NewNode<ConstantNode>( qn + "#qw" );
            ConstantNode* c = nc.NewNode<ConstantNode>( qn + "#qc" );
            v->SetConstantValue( P.quanto );
            w->SetConstantValue( 1.0 );
            c->SetConstantValue( 1.0 );
            q->SetUdlSpotNode( s );
            q->SetUdlVolNode( v );
            q->SetFxVolNode( w );
            q->SetUdlFxCorrelNode( c );
            return q;
        };
        const OptionType type = ( P.option_type == THOTH_CALL ) ? OptionType::Call : OptionType::Put;
        MonteCarloNode* flow = nullptr;
        if ( P.kind == THOTH_PRODUCT_VANILLA || P.kind == THOTH_PRODUCT_BASKET )
        {
            MonteCarloNode* udl;
            if ( P.kind == THOTH_PRODUCT_BASKET )
            {
                AbsoluteBasketNode* b = nc.NewNode<AbsoluteBasketNode>( pn + "#basket" );
                for ( int k = 0; k < P.n_components; k++ )
                {
                    b->PushUnderlying( quanto_of( P.components[k] ) );
                    b->PushWeight( P.weights[k] );
                }
                udl = b;
            }
            else
            {
                udl = quanto_of( P.asset );
            }
            VanillaFlowNode* f = nc.NewNode<VanillaFlowNode>( pn + node_name::FLOW );
            f->SetFloor( 0 );
            f->SetType( type );
            f->SetStrike( P.strike );
            f->SetSpotNode( udl );
            f->SetFlowDateIndex( (size_t)P.maturity );
            flow = f;
        }
        else if ( P.kind == THOTH_PRODUCT_BARRIER )
        {
            BarrierFlowNode* f = nc.NewNode<BarrierFlowNode>( pn + node_name::FLOW );
            f->SetFloor( 0 );
            f->SetType( type );
            f->SetStrike( P.strike );
            f->SetSpotNode( quanto_of( P.asset ) );
            f->SetFlowDateIndex( (size_t)P.maturity );
            f->SetBarrierLevel( P.barrier_level );
            f->SetIsUp( P.barrier_up != 0 );
            f->SetIsIn( P.barrier_in != 0 );
            vector<size_t> mon;
            for ( int k = 0; k < P.n_monitor; k++ )
            {
                mon.push_back( (size_t)P.monitor[k] );
            }
            f->SetMonitorIndexList( mon );
            flow = f;
        }
        else if ( P.kind == THOTH_PRODUCT_VARIANCE )
        {
            VarianceFlowNode* f = nc.NewNode<VarianceFlowNode>( pn + node_name::FLOW );
            f->SetSpotNode( quanto_of( P.asset ) );
            f->SetFlowDateIndex( (size_t)P.maturity );
            f->SetNotional( P.notional );
            f->SetStrikeVariance( P.strike_variance );
            f->SetTotalYearFraction( P.total_year_fraction );
            f->SetPastVariance( P.past_variance );
            vector<size_t> obs;
            for ( int k = 0; k < P.n_obs; k++ )
            {
                obs.push_back( (size_t)P.obs[k] );
            }
            f->SetObservationDateIndices( obs );
            flow = f;
        }
        else
        {
            return false;
        }
        ContractNode* c = nc.NewNode<ContractNode>( pn );
        TableNode* rate = nc.NewNode<TableNode>( pn + node_name::RATE );
        rate->FillConstant( P.zero_rate );
        c->PushFlowNode( flow, (size_t)P.maturity );
        c->SetRateCurveNode( rate );
        book->PushContractNode( c );
        if ( P.fx != 1.0 )
        {
            ConstantNode* fx = nc.NewNode<ConstantNode>( pn + node_name::FX );
            fx->SetConstantValue( P.fx );
            book->PushForexNode( fx );
        }
        else
        {
            book->PushForexNode( nullptr );
        }
        h.contracts.push_back( c );
    }
    h.book = book;
    nc.SortNodes( vector<MonteCarloNode*>{ book } );
    return true;
}

} // namespace

extern "C" {

//! Sobol integer coordinates through the reference generator (Skip + Next)
int ref_sobol_points( int dims, int64_t skip, int64_t n, uint32_t* out )
{
    SobolGenerator g( (unsigned)dims );
    if ( skip > 0 )
    {
        g.Skip( (uint64_t)skip );
    }
    vector<double> p;
    const int D = (int)g.Dimension();
    for ( int64_t i = 0; i < n; i++ )
    {
        g.Next( p );
        for ( int d = 0; d < D; d++ )
        {
            out[i * D + d] = (uint32_t)( p[(size_t)d] * 4294967296.0 );
        }
    }
    return D;
}

int ref_normal_cdf_inv( const double* p, int64_t n, double* out )
{
    for ( int64_t i = 0; i < n; i++ )
    {
        out[i] = NormalCdfInv( p[i] );
    }
    return 0;
}

//! normalised bridge increments, layout [path][factor][N] (index 1..N of Buffer)
int ref_bridge_increments( const double* t, int n_dates, int factors, int64_t skip, int64_t n_paths,
                           uint64_t seed, double* out )
{
    vector<double> times( t, t + n_dates );
    Rng rng( seed );
    PathGenerator g( times, factors, true, &rng, (uint64_t)skip );
    const int N = n_dates - 1;
    for ( int64_t p = 0; p < n_paths; p++ )
    {
        g.NextPath();
        for ( int f = 0; f < factors; f++ )
        {
            const vector<double>& b = *g.Buffer( f );
            for ( int i = 1; i <= N; i++ )
            {
                out[( p * factors + f ) * N + ( i - 1 )] = b[(size_t)i];
            }
        }
    }
    return 0;
}

//! price a book through the reference node graph. per_path (optional) receives
//! the discounted contract values of the first n_per_path paths, [path][product].
int ref_price_book( const ThothBookDesc* d, ThothBookResult* r, double* per_path, int64_t n_per_path )
{
    try
    {
        Harness h;
        if ( !Build( d, h ) )
        {
            return THOTH_GPU_E_UNSUPPORTED;
        }
        for ( int64_t i = 0; i < d->paths; i++ )
        {
            if ( h.pg )
            {
                h.pg->NextPath();
            }
            h.nc.PriceNodes();
            if ( per_path && i < n_per_path )
            {
                for ( size_t p = 0; p < h.contracts.size(); p++ )
                {
                    per_path[i * (int64_t)h.contracts.size() + (int64_t)p] = h.contracts[p]->GetValue( 0 );
                }
            }
        }
        r->book_premium = h.book->GetIndicatorValue( 0 );
        r->book_trust = h.book->GetIndicatorTrust( 0 );
        for ( size_t p = 0; p < h.contracts.size(); p++ )
        {
            if ( r->premium )
            {
                r->premium[p] = h.contracts[p]->GetIndicatorValue( 0 );
            }
            if ( r->trust )
            {
                r->trust[p] = h.contracts[p]->GetIndicatorTrust( 0 );
            }
        }
        return THOTH_GPU_OK;
    }
    catch ( const std::exception& e )
    {
        std::fprintf( stderr, "ref_price_book: %s\n", e.what() );
        return THOTH_GPU_E_INVALID;
    }
}

//! the reference's own LeastSquares (helpers/maths.cpp:419-470) on X [n][p] row-major;
//! returns 0 where it returns an empty vector (singular normal matrix)
int ref_least_squares( const double* X, int64_t n, int p, const double* y, double* beta )
{
    la_matrix* A = la_matrix_alloc( (size_t)n, (size_t)p );
    la_vector* v = la_vector_alloc( (size_t)n );
    for ( int64_t k = 0; k < n; k++ )
    {
        for ( int j = 0; j < p; j++ )
        {
            la_matrix_set( A, (size_t)k, (size_t)j, X[k * p + j] );
        }
        la_vector_set( v, (size_t)k, y[k] );
    }
    vector<double> b = LeastSquares( A, v );
    la_matrix_free( A );
    la_vector_free( v );
    for ( size_t j = 0; j < b.size(); j++ )
    {
        beta[j] = b[j];
    }
    return b.empty() ? 0 : 1;
}

//! Longstaff-Schwartz fit and frozen apply on date-major paths S[M][n] (the engine's
//! single-precision spots): the loops of PricerMCL::FitAmericanPolicy and
//! ApplyAmericanPolicy (tasks/pricer_mcl_american.cpp:263-447), restated here because
//! that file needs the whole pricer, around the reference's own LeastSquares and
//! payoff_vanilla. Sums in path order, as the reference. fit = 0 applies beta / has_fit.
int ref_lsm( const float* S, int64_t n, int M, const double* tau, const double* rates, double strike, int is_call,
             double norm, int min_itm, int fit, double* beta, int* has_fit, double* premium, double* trust )
{
    const OptionType ty = is_call ? OptionType::Call : OptionType::Put;
    auto intrinsic = [&]( double s ) { return payoff_vanilla( s, strike, ty, false, 0, true, 0 ); };
    auto at = [&]( int64_t p, int t ) { return (double)S[(int64_t)t * n + p]; };
    if ( M < 2 )
    {
        *premium = 0;
        *trust = 0;
        return 0;
    }
    if ( fit )
    {
        for ( int t = 0; t < M; t++ )
        {
            has_fit[t] = 0;
            beta[3 * t] = beta[3 * t + 1] = beta[3 * t + 2] = 0;
        }
        vector<double> cf( (size_t)n );
        for ( int64_t p = 0; p < n; p++ )
        {
            cf[p] = intrinsic( at( p, M - 1 ) );
        }
        for ( int t = M - 2; t >= 1; t-- )
        {
            double df = exp( rates[t] * tau[t] - rates[t + 1] * tau[t + 1] );
            for ( int64_t p = 0; p < n; p++ )
            {
                cf[p] *= df;
            }
            vector<int64_t> itm;
            for ( int64_t p = 0; p < n; p++ )
            {
                if ( intrinsic( at( p, t ) ) > 0 )
                {
                    itm.push_back( p );
                }
            }
            if ( itm.size() < (size_t)min_itm )
            {
                continue;
            }
            la_matrix* X = la_matrix_alloc( itm.size(), 3 );
            la_vector* y = la_vector_alloc( itm.size() );
            for ( size_t k = 0; k < itm.size(); k++ )
            {
                double m = at( itm[k], t ) / norm;
                la_matrix_set( X, k, 0, 1.0 );
                la_matrix_set( X, k, 1, m );
                la_matrix_set( X, k, 2, m * m );
                la_vector_set( y, k, cf[itm[k]] );
            }
            vector<double> b = LeastSquares( X, y );
            la_matrix_free( X );
            la_vector_free( y );
            if ( b.empty() )
            {
                continue;
            }
            beta[3 * t] = b[0];
            beta[3 * t + 1] = b[1];
            beta[3 * t + 2] = b[2];
            has_fit[t] = 1;
            for ( int64_t p : itm )
            {
                double s = at( p, t );
                double m = s / norm;
                double c = b[0] + b[1] * m + b[2] * m * m;
                double iv = intrinsic( s );
                if ( iv >= c )
                {
                    cf[p] = iv;
                }
            }
        }
    }
    double sum = 0, sum2 = 0;
    for ( int64_t p = 0; p < n; p++ )
    {
        double value = 0;
        for ( int t = 1; t < M; t++ )
        {
            double s = at( p, t );
            double iv = intrinsic( s );
            if ( t == M - 1 )
            {
                value = iv * exp( -rates[t] * ( tau[t] - tau[0] ) );
                break;
            }
            if ( iv > 0 && has_fit[t] )
            {
                double m = s / norm;
                double c = beta[3 * t] + beta[3 * t + 1] * m + beta[3 * t + 2] * m * m;
                if ( iv >= c )
                {
                    value = iv * exp( -rates[t] * ( tau[t] - tau[0] ) );
                    break;
                }
            }
        }
        sum += value;
        sum2 += value * value;
    }
    double mean = sum / n;
    *trust = sqrt( ( sum2 / n - mean * mean ) / ( n - 1 ) );
    *premium = std::max( mean, intrinsic( at( 0, 0 ) ) );
    return 0;
}

//! raw draws and Gaussians of the reference's own Rng (helpers/rng.hpp): n draws after
//! skipping `skip`, as Gaussian() would consume them
int ref_rng_draws( uint64_t seed, uint64_t skip, int64_t n, uint64_t* raw, double* gauss )
{
    Rng a( seed ), b( seed );
    for ( uint64_t i = 0; i < skip; i++ )
    {
        a();
        b();
    }
    for ( int64_t i = 0; i < n; i++ )
    {
        raw[i] = a();
        gauss[i] = b.Gaussian();
    }
    return 0;
}

} // extern "C"
