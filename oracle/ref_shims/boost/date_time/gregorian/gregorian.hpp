// Minimal stand-in for boost::gregorian used ONLY to compile the reference's
// Monte-Carlo node sources into the parity oracle (oracle/_ref). A date is a
// day count from an arbitrary epoch; only the operations those sources use
// (ordering, day differences, day offsets, printing) are provided.
#pragma once
#include <string>

namespace boost
{
namespace gregorian
{
class date_duration
{
  public:
    explicit date_duration( long n = 0 ) : _n( n ) {}
    long days() const { return _n; }

  private:
    long _n;
};
using days = date_duration;
class date
{
  public:
    date() : _d( 0 ) {}
    explicit date( long d ) : _d( d ) {}
    long day_number() const { return _d; }
    bool operator<( const date& o ) const { return _d < o._d; }
    bool operator>( const date& o ) const { return _d > o._d; }
    bool operator<=( const date& o ) const { return _d <= o._d; }
    bool operator>=( const date& o ) const { return _d >= o._d; }
    bool operator==( const date& o ) const { return _d == o._d; }
    bool operator!=( const date& o ) const { return _d != o._d; }
    date_duration operator-( const date& o ) const { return date_duration( _d - o._d ); }
    date operator+( const date_duration& n ) const { return date( _d + n.days() ); }
    date operator-( const date_duration& n ) const { return date( _d - n.days() ); }
    date& operator+=( const date_duration& n )
    {
        _d += n.days();
        return *this;
    }

  private:
    long _d;
};
inline std::string to_simple_string( const date& d ) { return "D" + std::to_string( d.day_number() ); }
inline std::string to_iso_extended_string( const date& d ) { return to_simple_string( d ); }
inline date from_simple_string( const std::string& s ) { return date( std::stol( s ) ); }
} // namespace gregorian
} // namespace boost
