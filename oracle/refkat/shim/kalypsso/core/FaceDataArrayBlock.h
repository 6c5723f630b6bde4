// Stub: the face-centred container lives with the other containers in kalypsso_data_container.h.
#pragma once
#include <kalypsso/core/kalypsso_data_container.h>
