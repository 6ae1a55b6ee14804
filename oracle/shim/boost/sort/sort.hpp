// Stand-in for the Boost.Sort header used by the reference tree solvers.
//
// Boost is not installed here.  The reference calls
// boost::sort::spreadsort::integer_sort(first, last, rightshift, lessthan),
// an unstable radix sort whose tie order is undefined.  This stand-in sorts
// with std::stable_sort on the same comparator, which fixes the tie order to
// "input order" -- the order the GPU radix sort also produces.
#pragma once
#include <algorithm>

namespace boost { namespace sort { namespace spreadsort {
template <class It, class Shift, class Less>
inline void integer_sort(It first, It last, Shift, Less less)
{
    std::stable_sort(first, last, less);
}
}}}
