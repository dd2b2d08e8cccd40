// Stand-in prelude for compiling the reference's host code with g++ (test
// infrastructure for the oracle fixtures only).  CUDA qualifiers become
// no-ops; <math.h>/<stdlib.h> bring the float overloads of exp/abs into the
// global namespace, as the CUDA headers do in the reference's own build.
#pragma once
#include <sys/types.h>
#include <cmath>
#include <cstdlib>
#include <math.h>
#include <stdlib.h>
#include <cstddef>
#include <iostream>
#include <iterator>
#include <stdexcept>
#include <string>
#include <tuple>
#include <utility>
#include <vector>
#define __host__
#define __device__
#define __forceinline__ inline
using std::cerr;
