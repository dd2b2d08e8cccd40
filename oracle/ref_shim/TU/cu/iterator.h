// Stand-in for TU/cu/iterator.h: declarations of the iterator helpers that
// GuidedFilter2::convolve names (never instantiated by the oracle harness).
#pragma once
namespace TU
{
namespace cu
{
template <class... A> int stride(A...);
template <class... A> int make_range_iterator(A...);
template <class... A> int make_map_iterator(A...);
template <class... A> int make_assignment_iterator(A...);
}  // namespace cu
}  // namespace TU
