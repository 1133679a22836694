// Stand-in for Boost.Math's Gauss-Kronrod quadrature. The reference's Heston
// characteristic-function price is NOT used from the oracle build (the FP64
// closed-form oracle is re-derived in oracle/closed_forms.c); this stub returns
// NaN so any accidental use is visible.
#pragma once
#include <limits>
namespace boost { namespace math { namespace quadrature {
template <class T, unsigned N> struct gauss_kronrod
{
    template <class F> static T integrate( F, T, T, unsigned = 0, T = 0, T* = nullptr, T* = nullptr )
    {
        return std::numeric_limits<T>::quiet_NaN();
    }
};
} } }
