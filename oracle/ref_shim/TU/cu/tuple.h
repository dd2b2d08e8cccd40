// Stand-in for TU/cu/tuple.h: the guided-filter functors only need
// thrust::tuple / thrust::get, mapped here onto std::tuple.
#pragma once
#include <tuple>
namespace thrust
{
using std::get;
using std::tuple;
}  // namespace thrust
