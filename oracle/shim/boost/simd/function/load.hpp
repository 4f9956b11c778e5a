// Stand-in header: everything lives in boost/simd/pack.hpp (test infrastructure only).
#pragma once
#include "../pack.hpp"
