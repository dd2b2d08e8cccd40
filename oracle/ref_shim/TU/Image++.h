// Stand-in for TULibs' TU/Image++.h, as included by
// Testprog/filterTest/filterImageGold.h (oracle fixtures only).
#pragma once
#include "TU/shim_array.h"
namespace TU
{
template <class T>
class Image : public Array2<Array<T>>
{
};
}  // namespace TU
