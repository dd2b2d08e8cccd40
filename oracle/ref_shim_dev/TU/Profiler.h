// Stand-in for TULibs' TU/Profiler.h: BoxFilter2 derives from Profiler<CLOCK>.
#pragma once
namespace TU
{
template <class CLOCK>
class Profiler
{
};
}  // namespace TU
