// Stub of kalypsso-core's base header for the functor bridge: the assertion macro.
#pragma once
#include <cassert>
#define assertm(exp, msg) assert(((void)(msg), (exp)))
