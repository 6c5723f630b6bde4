// Stub of kalypsso-core's block index helpers for the functor bridge (test infrastructure); they live
// with the containers in kalypsso_data_container.h, which other core headers also provide.
#pragma once
#include <kalypsso/core/kalypsso_data_container.h>
