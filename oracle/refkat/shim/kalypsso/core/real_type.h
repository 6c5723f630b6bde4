// Stub of kalypsso-core's real_type.h, written for the known-answer bridge only: just enough for
// the reference's models/*.h to compile unmodified on the host in FP64.
#pragma once
#include <cmath>
namespace kalypsso
{
using real_t = double;
}
#define KALYPSSO_NUM(x) static_cast<kalypsso::real_t>(x)
#define ZERO_F KALYPSSO_NUM(0.0)
#define HALF_F KALYPSSO_NUM(0.5)
#define ONE_THIRD_F KALYPSSO_NUM(1.0 / 3.0)
#define ONE_F KALYPSSO_NUM(1.0)
#define ONE_FOURTH_F KALYPSSO_NUM(0.25)
#define COPYSIGN(a, b) std::copysign((a), (b))
#define KALYPSSO_STATIC_MATH_CONSTANT(name, value) static constexpr kalypsso::real_t name = value
