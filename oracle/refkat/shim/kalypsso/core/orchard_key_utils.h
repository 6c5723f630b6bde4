// Stub: orchard keys live in orchard_key_base.h.
#pragma once
#include <kalypsso/core/orchard_key_base.h>
