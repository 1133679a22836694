// Stand-in for the Boost.Math policy header: only the names that the
// reference's distributions.cpp spells out. GammaCdf is not on the Monte-Carlo
// path and is never called by the oracle.
#pragma once
namespace boost { namespace math { namespace policies {
enum error_policy_type { ignore_error = 0 };
template <error_policy_type> struct overflow_error {};
template <error_policy_type> struct domain_error {};
template <error_policy_type> struct pole_error {};
template <class... T> struct policy {};
} } }
