// Stub of kalypsso-core's mesh helpers: nothing of it is used by the bridged functors beyond the
// include.
#pragma once
