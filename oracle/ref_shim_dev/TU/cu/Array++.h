// Stand-in for TU/cu/Array++.h: the array types the filter classes name.
// FIRFilter2<> is instantiated as a class (its LobeSizeMax sizes the constant
// lobes), so its Array2 member needs a complete type.
#pragma once
#include <cstddef>
namespace TU
{
template <class T>
class Array;
namespace cu
{
template <class T>
class Array2
{
};
template <class T>
class Array3
{
};
}  // namespace cu
}  // namespace TU
